// Gmsh *.msh 2.2 (ASCII) reader: the gmsh branch of fbem_mesh%read_from_file
// (lib/fbem/src/mesh.f90:104-494), host side, so the meshes the reference's
// input decks name (`mesh_file_mode = 2 "file.msh"`) can be read without the
// Fortran front end. Sections are located by name as the reference does
// (fbem_search_section_gmsh), and the same inputs are refused:
//   $MeshFormat    required; its line has 3 words, the first "2.2"
//   $PhysicalNames required; "dim id name" lines, ids > 0 and unique (the
//                  reference's parts)
//   $Elements      ids > 0 and unique; the first tag is the part, which must
//                  be a declared physical id; the type is a gmsh code (or the
//                  reference's name) of a known element; its nodes follow the
//                  tags, in gmsh order (the reference keeps that order)
//   $Nodes         ids > 0 and unique; at most 4 words (id and up to three
//                  coordinates)
// element nodes must name declared nodes, and every part holds elements of
// one dimension (at least one element).
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct Msh {
  std::vector<int32_t> part_id;
  std::vector<int32_t> part_dim;
  std::vector<std::string> part_name;
  std::vector<int32_t> node_id;
  std::vector<double> x;  // [n_nodes][3]
  std::vector<int32_t> el_id, el_type, el_part, el_off, el_nodes;  // el_off: [n_el + 1] into el_nodes
};

thread_local std::string g_msh_err;

// gmsh type code -> number of nodes (the types fbem_mesh%read_from_file names)
int gmsh_nodes(int type) {
  switch (type) {
    case 15: return 1;   // point1
    case 1: return 2;    // line2
    case 8: return 3;    // line3
    case 26: return 4;   // line4
    case 2: return 3;    // tri3
    case 9: return 6;    // tri6
    case 3: return 4;    // quad4
    case 16: return 8;   // quad8
    case 10: return 9;   // quad9
    case 4: return 4;    // tet4
    case 11: return 10;  // tet10
    case 5: return 8;    // hex8
    case 17: return 20;  // hex20
    case 12: return 27;  // hex27
    default: return 0;
  }
}
// dimension of an element of a known gmsh type
int gmsh_dim(int type) {
  switch (type) {
    case 15: return 0;
    case 1: case 8: case 26: return 1;
    case 2: case 9: case 3: case 16: case 10: return 2;
    default: return 3;
  }
}
int type_by_name(const std::string& s) {
  static const std::map<std::string, int> names = {
      {"point1", 15}, {"line2", 1}, {"line3", 8}, {"line4", 26}, {"tri3", 2},   {"tri6", 9},   {"quad4", 3},
      {"quad8", 16},  {"quad9", 10}, {"tet4", 4},  {"tet10", 11}, {"hex8", 5}, {"hex20", 17}, {"hex27", 12}};
  auto it = names.find(s);
  if (it != names.end()) return it->second;
  char* end = nullptr;
  const long v = std::strtol(s.c_str(), &end, 10);
  return (end && *end == 0 && gmsh_nodes((int)v) > 0) ? (int)v : 0;
}

std::vector<std::string> words(const std::string& line) {
  std::vector<std::string> w;
  std::istringstream is(line);
  std::string t;
  while (is >> t) w.push_back(t);
  return w;
}

// the line index after "$<name>", or -1
long find_section(const std::vector<std::string>& lines, const std::string& name) {
  const std::string key = "$" + name;
  for (size_t i = 0; i < lines.size(); ++i) {
    std::string t = lines[i];
    while (!t.empty() && std::isspace((unsigned char)t.back())) t.pop_back();
    size_t a = 0;
    while (a < t.size() && std::isspace((unsigned char)t[a])) ++a;
    if (t.compare(a, std::string::npos, key) == 0) return (long)i + 1;
  }
  return -1;
}

bool fail(const std::string& m) {
  g_msh_err = m;
  return false;
}

bool parse(const std::vector<std::string>& L, Msh& m) {
  long s = find_section(L, "MeshFormat");
  if (s < 0 || s >= (long)L.size()) return fail("The section $MeshFormat is required.");
  {
    const auto w = words(L[s]);
    if (w.size() != 3) return fail("This line in $MeshFormat must have 3 numbers.");
    if (w[0] != "2.2") return fail("only gmsh *.msh file version 2.2 can be read");
    if (w[1] != "0") return fail("only the ASCII *.msh format can be read");
  }
  // parts
  s = find_section(L, "PhysicalNames");
  if (s < 0 || s >= (long)L.size()) return fail("The section PhysicalNames is required.");
  const long np = std::strtol(L[s].c_str(), nullptr, 10);
  if (np <= 0) return fail("the number of parts must be >0");
  std::map<int, int> part_iid;
  for (long i = 0; i < np; ++i) {
    if (s + 1 + i >= (long)L.size()) return fail("PhysicalNames ends early");
    const auto w = words(L[s + 1 + i]);
    if (w.size() < 3) return fail("invalid line in PhysicalNames");
    const int dim = std::atoi(w[0].c_str()), id = std::atoi(w[1].c_str());
    std::string name = L[s + 1 + i].substr(L[s + 1 + i].find(w[2]));
    while (!name.empty() && std::isspace((unsigned char)name.back())) name.pop_back();
    if (name.size() >= 2 && name.front() == '"' && name.back() == '"') name = name.substr(1, name.size() - 2);
    if (id <= 0) return fail("part " + std::to_string(id) + ": identifiers must be >0");
    if (part_iid.count(id)) return fail("part " + std::to_string(id) + " is repeated");
    part_iid[id] = (int)m.part_id.size();
    m.part_id.push_back(id);
    m.part_dim.push_back(dim);
    m.part_name.push_back(name);
  }
  // elements
  s = find_section(L, "Elements");
  if (s < 0 || s >= (long)L.size()) return fail("The section Elements is required.");
  const long ne = std::strtol(L[s].c_str(), nullptr, 10);
  if (ne <= 0) return fail("the number of elements must be >0");
  std::map<int, int> el_seen;
  m.el_off.push_back(0);
  for (long i = 0; i < ne; ++i) {
    if (s + 1 + i >= (long)L.size()) return fail("Elements ends early");
    const auto w = words(L[s + 1 + i]);
    if (w.size() < 3) return fail("invalid line in Elements");
    const int id = std::atoi(w[0].c_str());
    const int type = type_by_name(w[1]);
    const int ntags = std::atoi(w[2].c_str());
    if (id <= 0) return fail("element " + std::to_string(id) + ": identifiers must be >0");
    if (el_seen.count(id)) return fail("element " + std::to_string(id) + " is repeated");
    el_seen[id] = (int)i;
    if (ntags < 1 || (long)w.size() < 3 + ntags) return fail("element " + std::to_string(id) + ": missing tags");
    const int part = std::atoi(w[3].c_str());
    if (!part_iid.count(part))
      return fail("element " + std::to_string(id) + " is assigned to the invalid part " + std::to_string(part));
    if (type == 0) return fail("element " + std::to_string(id) + ": unrecognized type of element");
    const int nn = gmsh_nodes(type);
    if ((long)w.size() < 3 + ntags + nn) return fail("element " + std::to_string(id) + ": missing nodes");
    m.el_id.push_back(id);
    m.el_type.push_back(type);
    m.el_part.push_back(part);
    for (int k = 0; k < nn; ++k) m.el_nodes.push_back(std::atoi(w[3 + ntags + k].c_str()));
    m.el_off.push_back((int32_t)m.el_nodes.size());
  }
  // nodes
  s = find_section(L, "Nodes");
  if (s < 0 || s >= (long)L.size()) return fail("The section Nodes is required.");
  const long nn = std::strtol(L[s].c_str(), nullptr, 10);
  if (nn <= 0) return fail("the number of nodes must be >0");
  std::map<int, int> node_seen;
  for (long i = 0; i < nn; ++i) {
    if (s + 1 + i >= (long)L.size()) return fail("Nodes ends early");
    const auto w = words(L[s + 1 + i]);
    if (w.empty() || w.size() > 4) return fail("invalid number of arguments in the list of nodes");
    const int id = std::atoi(w[0].c_str());
    if (id <= 0) return fail("node " + std::to_string(id) + ": identifiers must be >0");
    if (node_seen.count(id)) return fail("node " + std::to_string(id) + " is repeated");
    node_seen[id] = (int)i;
    m.node_id.push_back(id);
    for (int c = 0; c < 3; ++c) {
      double v = 0.0;
      if (c + 1 < (int)w.size()) {
        std::string t = w[c + 1];
        for (char& ch : t)
          if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'E';  // Fortran exponent letters
        v = std::strtod(t.c_str(), nullptr);
      }
      m.x.push_back(v);
    }
  }
  for (int32_t v : m.el_nodes)
    if (!node_seen.count(v)) return fail("an element refers to the undeclared node " + std::to_string(v));
  // each part holds elements of one dimension (mesh.f90:364-372); the
  // reference reads the dimension of a part's first element, so a part
  // without elements is refused too
  for (size_t i = 0; i < m.part_id.size(); ++i) {
    int dim = -1;
    for (size_t e = 0; e < m.el_id.size(); ++e) {
      if (m.el_part[e] != m.part_id[i]) continue;
      const int d = gmsh_dim(m.el_type[e]);
      if (dim < 0) dim = d;
      else if (d != dim)
        return fail("part " + std::to_string(m.part_id[i]) + " contain elements of different dimensions");
    }
    if (dim < 0) return fail("part " + std::to_string(m.part_id[i]) + " contains no elements");
  }
  return true;
}

}  // namespace

extern "C" {

// Read a *.msh 2.2 file; *out receives a handle for the accessors below.
// Returns 0, or -1 with the reason in mfbem_msh_error().
int mfbem_msh_read(const char* path, void** out) {
  g_msh_err.clear();
  if (!path || !out) {
    g_msh_err = "null argument";
    return -1;
  }
  *out = nullptr;
  std::ifstream f(path);
  if (!f) {
    g_msh_err = std::string("cannot open ") + path;
    return -1;
  }
  std::vector<std::string> lines;
  std::string line;
  while (std::getline(f, line)) lines.push_back(line);
  Msh* m = new Msh();
  if (!parse(lines, *m)) {
    delete m;
    return -1;
  }
  *out = m;
  return 0;
}
const char* mfbem_msh_error(void) { return g_msh_err.c_str(); }
// counts[0..3] = parts, nodes, elements, element-node entries
int mfbem_msh_sizes(void* h, int32_t* counts) {
  const Msh* m = (const Msh*)h;
  if (!m || !counts) return -1;
  counts[0] = (int32_t)m->part_id.size();
  counts[1] = (int32_t)m->node_id.size();
  counts[2] = (int32_t)m->el_id.size();
  counts[3] = (int32_t)m->el_nodes.size();
  return 0;
}
// parts: id, dimension, name (names: n_parts x name_len bytes, NUL-padded)
int mfbem_msh_parts(void* h, int32_t* id, int32_t* dim, char* names, int32_t name_len) {
  const Msh* m = (const Msh*)h;
  if (!m) return -1;
  for (size_t i = 0; i < m->part_id.size(); ++i) {
    if (id) id[i] = m->part_id[i];
    if (dim) dim[i] = m->part_dim[i];
    if (names && name_len > 0) {
      char* d = names + i * (size_t)name_len;
      std::memset(d, 0, (size_t)name_len);
      std::strncpy(d, m->part_name[i].c_str(), (size_t)name_len - 1);
    }
  }
  return 0;
}
// nodes in file order: id, x [n_nodes][3]
int mfbem_msh_nodes(void* h, int32_t* id, double* x) {
  const Msh* m = (const Msh*)h;
  if (!m) return -1;
  if (id) std::copy(m->node_id.begin(), m->node_id.end(), id);
  if (x) std::copy(m->x.begin(), m->x.end(), x);
  return 0;
}
// elements in file order: id, gmsh type, part (physical id), offsets
// [n_elements + 1] into nodes (node ids, gmsh order)
int mfbem_msh_elements(void* h, int32_t* id, int32_t* type, int32_t* part, int32_t* offsets, int32_t* nodes) {
  const Msh* m = (const Msh*)h;
  if (!m) return -1;
  if (id) std::copy(m->el_id.begin(), m->el_id.end(), id);
  if (type) std::copy(m->el_type.begin(), m->el_type.end(), type);
  if (part) std::copy(m->el_part.begin(), m->el_part.end(), part);
  if (offsets) std::copy(m->el_off.begin(), m->el_off.end(), offsets);
  if (nodes) std::copy(m->el_nodes.begin(), m->el_nodes.end(), nodes);
  return 0;
}
void mfbem_msh_free(void* h) { delete (Msh*)h; }

}  // extern "C"

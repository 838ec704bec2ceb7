// Caller-side mesh preparation: what MultiFEBE's Fortran host computes before it
// calls the region builders, for one BE region of continuous quad8 elements:
//   - element data (src/build_data_of_be_elements.f90:52-96): csize, n_phi,
//     bounding ball;
//   - node normals / boundary tangents (src/build_data_at_geometrical_nodes.f90:177-222);
//   - mesh-boundary nodes and default formulations
//     (lib/fbem/src/data_structures.f90:1433-1495, src/assign_default_bem_formulation.f90:76-93);
//   - MCA collocation points (src/build_data_at_collocation_points.f90:125-147,174-223);
//   - DOF numbering (src/build_auxiliary_variables_mechanics_static.f90:60-207).
// The results are the inputs of mfbem_mesh_upload; none of it runs per frequency.
#include "mfbem_host.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

using namespace mfb;

namespace {

// fbem_qs_phijac_ngp_2d, quadrilateral branch (quasisingular_integration.f90:812-975)
int phijac_ngp_q8(const double* x, double error_height, bool* achieve) {
  double eh = error_height;
  if (eh <= 0.0) eh = 1e-6;
  else if (eh < 1e-12) eh = 1e-12;
  double integral[8] = {0, 0, 0, 0, 0, 0, 0, 0}, old[8];
  bool cont = true;
  *achieve = true;
  int j = 1;
  while (cont) {
    for (int l = 0; l < 8; ++l) { old[l] = integral[l]; integral[l] = 0.0; }
    for (int k1 = 1; k1 <= j; ++k1)
      for (int k2 = 1; k2 <= j; ++k2) {
        double x1 = gl11x(k1, j), x2 = gl11x(k2, j);
        double d1[8], d2[8], phi[8];
        dphi_q8<double>(x1, x2, d1, d2);
        double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
        for (int l = 0; l < 8; ++l)
          for (int c = 0; c < 3; ++c) { T1[c] += d1[l] * x[3 * l + c]; T2[c] += d2[l] * x[3 * l + c]; }
        double N[3];
        cross3(T1, T2, N);
        double jw = norm3(N) * gl11w(k1, j) * gl11w(k2, j);
        phi_q8<double>(x1, x2, phi);
        for (int l = 0; l < 8; ++l) integral[l] += (phi[l] + 1.0) * jw;
      }
    if (j == 1) {
      j = j + 1;
    } else {
      cont = false;
      for (int l = 0; l < 8; ++l)
        if (std::fabs((old[l] - integral[l]) / integral[l]) > eh) { cont = true; j = j + 1; break; }
      if (j == 33) { cont = false; *achieve = false; }
    }
  }
  return j - 1;
}

// fbem_geometry_element_ball, quadrilateral branch (geometry.f90:3904-4235)
void ball_q8(const double* x, int glp, double c[3], double* radius) {
  double esize = 0.0, xm[3] = {0, 0, 0};
  for (int k1 = 1; k1 <= glp; ++k1)
    for (int k2 = 1; k2 <= glp; ++k2) {
      double xp[3], T1[3], T2[3], phi[8], N[3];
      geom_q8(x, gl11x(k1, glp), gl11x(k2, glp), xp, T1, T2, phi);
      cross3(T1, T2, N);
      double jw = norm3(N) * gl11w(k1, glp) * gl11w(k2, glp);
      esize = esize + jw;
      for (int q = 0; q < 3; ++q) xm[q] = xm[q] + xp[q] * jw;
    }
  for (int q = 0; q < 3; ++q) c[q] = xm[q] / esize;
  double r = 0.0;
  for (int k = 0; k < 8; ++k) {
    double v[3] = {x[3 * k] - c[0], x[3 * k + 1] - c[1], x[3 * k + 2] - c[2]};
    double t = norm3(v);
    if (r < t) r = t;
  }
  for (int k1 = 1; k1 <= glp; ++k1)
    for (int k2 = 1; k2 <= glp; ++k2) {
      double phi[8];
      phi_q8<double>(gl11x(k1, glp), gl11x(k2, glp), phi);
      double xp[3] = {0, 0, 0};
      for (int k = 0; k < 8; ++k)
        for (int q = 0; q < 3; ++q) xp[q] = xp[q] + phi[k] * x[3 * k + q];
      double v[3] = {xp[0] - c[0], xp[1] - c[1], xp[2] - c[2]};
      double t = norm3(v);
      if (r < t) r = t;
    }
  *radius = r;
}

}  // namespace

struct mfbem_prep {
  mfbem_mesh_desc desc;
  int nn, ne;
  std::vector<double> x_gn, csize, bball, n_gn, tbp_gn, cvalue, xi_mca, x_mca, X;
  std::vector<int32_t> element_node, n_phi, reversion, row, col, ctype, sbie, gln;
  std::vector<int32_t> dof, order;
  // HBIE formulations (mfbem_prep_set_formulation) and crack-like boundaries
  // (mfbem_prep_set_crack)
  mfbem_dual_desc dual;
  bool has_dual = false;
  std::vector<int32_t> form, hbie, dualv, common;
  std::vector<double> alpha, delta, xi_hbie, x_hbie, n_hbie;
  std::vector<int32_t> crack_el, crack_node, ctype2, dof2;
  std::vector<double> cvalue2;
};

namespace {

// MCA collocation points of the mesh-boundary nodes: xi moved from the edge by
// 0.05 (assign_default_bem_formulation.f90:39,85-92), or by the quadratic
// default 0.22540333 for a 'dual_bm_mixed' node
// (read_bem_formulation_selected_nodes.f90:273-294).
void mca_points(mfbem_prep* P) {
  for (int e = 0; e < P->ne; ++e)
    for (int k = 0; k < 8; ++k) {
      const int s = P->element_node[8 * e + k] - 1;
      if (!P->sbie[s]) continue;
      const double dl = (!P->form.empty() && P->form[s] == 3) ? 0.22540333 : 0.05;
      double x1 = q8xi(k, 0), x2 = q8xi(k, 1);
      if (on_quad_edge(x1, x2)) { x1 = x1 * (1.0 - dl); x2 = x2 * (1.0 - dl); }
      P->xi_mca[16 * (size_t)e + 2 * k] = x1;
      P->xi_mca[16 * (size_t)e + 2 * k + 1] = x2;
      double phi[8];
      phi_q8<double>(x1, x2, phi);
      double xp[3] = {0, 0, 0};
      for (int q = 0; q < 8; ++q)
        for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[q] * P->x_gn[24 * (size_t)e + 3 * q + c];
      for (int c = 0; c < 3; ++c) P->x_mca[24 * (size_t)e + 3 * k + c] = xp[c];
    }
}

// DOF numbering, src/build_auxiliary_variables_mechanics_static.f90:60-207:
// nodes in order of first appearance over the elements; an ordinary node
// takes rows r, r+1, r+2 (col = row of the unknown of each direction); a
// crack-like node r..r+5 with row(k,1) = r + 2(k-1) (SBIE), row(k,2) =
// row(k,1) + 1 (HBIE) and face 2's unknown in column row(k,1) + 1.
void number_dofs(mfbem_prep* P) {
  const int nn = P->nn, ne = P->ne;
  const bool ck = !P->crack_node.empty();
  P->row.assign(3 * (size_t)nn, 0);
  P->col.assign(6 * (size_t)nn, 0);
  P->dof.assign(3 * (size_t)nn, -1);
  P->dof2.assign(3 * (size_t)nn, -1);
  P->order.clear();
  std::vector<char> used(nn, 0);
  int r = 1;
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      const int s = P->element_node[8 * e + k] - 1;
      if (used[s]) continue;
      used[s] = 1;
      P->order.push_back(s);
      const int w = (ck && P->crack_node[s]) ? 2 : 1;
      for (int c = 0; c < 3; ++c) {
        const int rc = r + w * c;
        P->row[3 * (size_t)s + c] = rc;
        if (P->ctype[3 * (size_t)s + c] == 0) P->col[6 * (size_t)s + 3 + c] = rc;
        else P->col[6 * (size_t)s + c] = rc;
        P->dof[3 * (size_t)s + c] = rc - 1;
        if (w == 2) P->dof2[3 * (size_t)s + c] = rc;
      }
      r += 3 * w;
    }
  P->desc.n_dof = r - 1;
  P->desc.row = P->row.data();
  P->desc.col = P->col.data();
}

// The dual descriptor from the formulation codes and the crack-like
// boundaries: HBIE points of every node with an HBIE, xi moved from the
// element edge by delta (fbem_move_xi1xi2_from_edge; quadratic default
// 0.22540333, assign_default_bem_formulation.f90:42) and the unit normal
// there (src/build_data_at_collocation_points.f90:148-160,368-376).
void rebuild_dual(mfbem_prep* P) {
  const int nn = P->nn, ne = P->ne;
  if (P->form.empty()) P->form.assign(nn, 0);
  if (P->alpha.empty()) P->alpha.assign(nn, 1.0);
  if (P->delta.empty()) P->delta.assign(nn, 0.0);
  const bool ck = !P->crack_node.empty();
  P->hbie.assign(nn, 0);
  P->dualv.assign(nn, 0);
  P->common.assign(nn, 0);
  for (int s = 0; s < nn; ++s) {
    if (ck && P->crack_node[s]) {
      P->hbie[s] = 1;
      P->dualv[s] = 2;
      P->common[s] = 1;
      continue;
    }
    P->hbie[s] = P->form[s] != 0;
    P->dualv[s] = P->form[s] >= 2;
    P->common[s] = P->form[s] == 2;
  }
  P->xi_hbie.assign(16 * (size_t)ne, 0.0);
  P->x_hbie.assign(24 * (size_t)ne, 0.0);
  P->n_hbie.assign(24 * (size_t)ne, 0.0);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      const int s = P->element_node[8 * e + k] - 1;
      if (!P->hbie[s]) continue;
      const double dl = P->delta[s] > 0.0 ? P->delta[s] : 0.22540333;
      double x1 = q8xi(k, 0), x2 = q8xi(k, 1);
      if (on_quad_edge(x1, x2)) { x1 = x1 * (1.0 - dl); x2 = x2 * (1.0 - dl); }
      const double* x = &P->x_gn[24 * (size_t)e];
      double xp[3], T1[3], T2[3], phi[8], N[3];
      geom_q8(x, x1, x2, xp, T1, T2, phi);
      cross3(T1, T2, N);
      const double jn = norm3(N);
      P->xi_hbie[16 * (size_t)e + 2 * k] = x1;
      P->xi_hbie[16 * (size_t)e + 2 * k + 1] = x2;
      for (int c = 0; c < 3; ++c) {
        P->x_hbie[24 * (size_t)e + 3 * k + c] = xp[c];
        P->n_hbie[24 * (size_t)e + 3 * k + c] = N[c] / jn;
      }
    }
  mfbem_dual_desc& d = P->dual;
  d.hbie = P->hbie.data();
  d.dual = P->dualv.data();
  d.dual_is_common = P->common.data();
  d.alpha = P->alpha.data();
  d.xi_i_hbie = P->xi_hbie.data();
  d.x_i_hbie = P->x_hbie.data();
  d.n_i_hbie = P->n_hbie.data();
  d.crack_el = ck ? P->crack_el.data() : nullptr;
  d.ctype2 = ck ? P->ctype2.data() : nullptr;
  d.cvalue2 = ck ? P->cvalue2.data() : nullptr;
  P->has_dual = true;
}

}  // namespace

extern "C" mfbem_prep* mfbem_prep_create(int32_t nn, const double* X, int32_t ne, const int32_t* conn,
                                         const int32_t* ctype, const double* cvalue, double qsi_re, int32_t ns_max,
                                         int32_t n_ps, const int32_t* ps_gln, double geo_tol) {
  host_gauss_tables();
  mfbem_prep* P = new mfbem_prep();
  P->nn = nn;
  P->ne = ne;
  P->X.assign(X, X + 3 * (size_t)nn);
  P->x_gn.resize(24 * (size_t)ne);
  P->element_node.resize(8 * (size_t)ne);
  P->csize.resize(ne);
  P->n_phi.resize(ne);
  P->bball.resize(4 * (size_t)ne);
  P->reversion.assign(ne, 0);
  P->n_gn.resize(24 * (size_t)ne);
  P->tbp_gn.resize(24 * (size_t)ne);
  P->xi_mca.assign(16 * (size_t)ne, 0.0);
  P->x_mca.assign(24 * (size_t)ne, 0.0);
  for (int e = 0; e < ne; ++e) {
    double* x = &P->x_gn[24 * (size_t)e];
    for (int k = 0; k < 8; ++k) {
      int s = conn[8 * e + k];
      P->element_node[8 * e + k] = s + 1;
      for (int c = 0; c < 3; ++c) x[3 * k + c] = X[3 * (size_t)s + c];
    }
    P->csize[e] = clen_q8(x, 1e-9);
    bool ok;
    int n1 = phijac_ngp_q8(x, qsi_re, &ok);
    int n2 = phijac_ngp_q8(x, qsi_re, &ok);
    P->n_phi[e] = std::max(n1, n2);
    ball_q8(x, P->n_phi[e], &P->bball[4 * e], &P->bball[4 * e + 3]);
    // fbem_unormal3d and fbem_utangents_at_boundary at the nodes (geometry.f90:1044-1092, 657-914)
    for (int k = 0; k < 8; ++k) {
      double d1[8], d2[8];
      dphi_q8<double>(q8xi(k, 0), q8xi(k, 1), d1, d2);
      double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0}, N[3];
      for (int i = 0; i < 8; ++i)
        for (int c = 0; c < 3; ++c) { T1[c] = T1[c] + d1[i] * x[3 * i + c]; T2[c] = T2[c] + d2[i] * x[3 * i + c]; }
      cross3(T1, T2, N);
      double t = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
      double n1_ = norm3(T1), n2_ = norm3(T2);
      for (int c = 0; c < 3; ++c) {
        P->n_gn[24 * (size_t)e + 3 * k + c] = N[c] / t;
        // tbp: node 1 +t1, 2 +t2, 3 -t1, 4 -t2, 5 +t1, 6 +t2, 7 -t1, 8 -t2
        static const int which[8] = {1, 2, 1, 2, 1, 2, 1, 2};
        static const double sgn[8] = {1, 1, -1, -1, 1, 1, -1, -1};
        double tv = (which[k] == 1 ? T1[c] / n1_ : T2[c] / n2_);
        P->tbp_gn[24 * (size_t)e + 3 * k + c] = sgn[k] * tv;
      }
    }
  }
  // mesh-boundary nodes: edges with a single element
  std::map<std::pair<int, int>, int> ecount;
  for (int e = 0; e < ne; ++e)
    for (int ke = 0; ke < 4; ++ke) {
      int a = conn[8 * e + q8edge(ke, 0)], b = conn[8 * e + q8edge(ke, 1)];
      ecount[{std::min(a, b), std::max(a, b)}]++;
    }
  std::vector<char> inb(nn, 0);
  for (int e = 0; e < ne; ++e)
    for (int ke = 0; ke < 4; ++ke) {
      int a = conn[8 * e + q8edge(ke, 0)], b = conn[8 * e + q8edge(ke, 1)];
      if (ecount[{std::min(a, b), std::max(a, b)}] == 1)
        for (int q = 0; q < 3; ++q) inb[conn[8 * e + q8edge(ke, q)]] = 1;
    }
  P->sbie.assign(nn, 0);
  for (int s = 0; s < nn; ++s) P->sbie[s] = inb[s] ? 1 : 0;
  mca_points(P);
  P->ctype.assign(ctype, ctype + 3 * (size_t)nn);
  P->cvalue.assign(cvalue, cvalue + 6 * (size_t)nn);
  number_dofs(P);
  P->gln.assign(ps_gln, ps_gln + n_ps);
  mfbem_mesh_desc& d = P->desc;
  d.n_nodes = nn;
  d.n_elements = ne;
  d.x_gn = P->x_gn.data();
  d.element_node = P->element_node.data();
  d.csize = P->csize.data();
  d.n_phi = P->n_phi.data();
  d.bball = P->bball.data();
  d.reversion = P->reversion.data();
  d.n_gn = P->n_gn.data();
  d.tbp_gn = P->tbp_gn.data();
  d.ctype = P->ctype.data();
  d.cvalue = P->cvalue.data();
  d.sbie = P->sbie.data();
  d.xi_i_sbie_mca = P->xi_mca.data();
  d.x_i_sbie_mca = P->x_mca.data();
  d.qsi_relative_error = qsi_re;
  d.qsi_ns_max = ns_max;
  d.n_precalsets = n_ps;
  d.precalset_gln = P->gln.data();
  d.geometric_tolerance = geo_tol;
  return P;
}

// BEM formulation per node, as src/read_bem_formulation_selected_nodes.f90:
// 70-295 sets it for an ordinary boundary of continuous elements: form 0 SBIE
// (the default of assign_default_bem_formulation.f90), 1 'hbie', 2
// 'dual_bm_same', 3 'dual_bm_mixed' (both with weight alpha); delta moves the
// HBIE point of each element node into the element (the quadratic default
// 0.22540333 when delta <= 0). Returns -1 for a code out of range.
extern "C" int mfbem_prep_set_formulation(mfbem_prep* P, const int32_t* form, const double* alpha,
                                          const double* delta) {
  const int nn = P->nn;
  for (int s = 0; s < nn; ++s)
    if (form[s] < 0 || form[s] > 3) return -1;
  P->form.assign(form, form + nn);
  P->alpha.assign(nn, 1.0);
  P->delta.assign(nn, 0.0);
  for (int s = 0; s < nn; ++s) {
    if (alpha) P->alpha[s] = alpha[s];
    if (delta) P->delta[s] = delta[s];
  }
  mca_points(P);
  rebuild_dual(P);
  return 0;
}

// Crack-like boundary (dual BEM): crack_el [ne] marks its elements, ctype2 /
// cvalue2 [nn][3] the conditions of face 2 (read for its nodes). Renumbers
// the DOF (six per crack node) and sets its nodes' formulation
// (src/assign_default_bem_formulation.f90:94-128; delta of their points as
// given to mfbem_prep_set_formulation, else the quadratic default).
// Returns -1 if a node of a crack-like element also belongs to an ordinary
// one, -2 for a ctype2 other than 0 / 1.
extern "C" int mfbem_prep_set_crack(mfbem_prep* P, const int32_t* crack_el, const int32_t* ctype2,
                                    const double* cvalue2) {
  const int nn = P->nn, ne = P->ne;
  std::vector<int32_t> cn(nn, 0), on(nn, 0);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) (crack_el[e] ? cn : on)[P->element_node[8 * e + k] - 1] = 1;
  for (int s = 0; s < nn; ++s) {
    if (cn[s] && on[s]) return -1;
    if (cn[s])
      for (int c = 0; c < 3; ++c)
        if (ctype2[3 * s + c] != 0 && ctype2[3 * s + c] != 1) return -2;
  }
  P->crack_el.assign(ne, 0);
  for (int e = 0; e < ne; ++e) P->crack_el[e] = crack_el[e] ? 1 : 0;
  P->crack_node = cn;
  P->ctype2.assign(ctype2, ctype2 + 3 * (size_t)nn);
  P->cvalue2.assign(cvalue2, cvalue2 + 6 * (size_t)nn);
  number_dofs(P);
  rebuild_dual(P);
  return 0;
}
extern "C" const mfbem_dual_desc* mfbem_prep_dual(const mfbem_prep* p) { return p->has_dual ? &p->dual : nullptr; }

extern "C" const mfbem_mesh_desc* mfbem_prep_desc(const mfbem_prep* p) { return &p->desc; }
extern "C" void mfbem_prep_free(mfbem_prep* p) { delete p; }
extern "C" void mfbem_prep_dof(const mfbem_prep* p, int32_t* dof, int32_t* order) {
  for (size_t i = 0; i < p->dof.size(); ++i) dof[i] = p->dof[i];
  for (size_t i = 0; i < p->order.size(); ++i) order[i] = p->order[i];
}
extern "C" void mfbem_prep_dof2(const mfbem_prep* p, int32_t* dof2) {
  for (size_t i = 0; i < p->dof2.size(); ++i) dof2[i] = p->dof2[i];
}

// element far-field order (phijac_ngp) for callers outside this file
int mfb::host_phijac_ngp_q8(const double* x, double error_height) {
  bool ok;
  return phijac_ngp_q8(x, error_height, &ok);
}

// Device-resident mesh snapshot and work lists, shared by the kernels
// (mfbem_kernels.cu) and the C-ABI layer (mfbem_abi.cpp).
//
// HBM layout (all arrays structure-of-arrays, 0-based):
//   elements   ex[ne][8][3], cl, gln_far, ball[ne][4], rev, edof[ne][8]
//              (DOF index of direction 1 of each element node = row base;
//              rev bit 0: reversed, bit 1: element of a crack-like boundary,
//              whose nodes interleave both faces: face f, direction c at
//              edof + 2 c + f)
//   DOFs       dct[ndof] (0 u known / 1 t known), dcv[ndof] complex value
//   colloc.    points sorted by DOF-order node ("dnode"): cpx[ncp][3], cp_dn,
//              cp_kind (0 nodal SBIE / 1 SBIE-MCA), cp_elem, cp_kn, cp_xi[2];
//              dn_cp[ndn+1] = range of points of each dnode (its 3 rows)
//   datasets   px/pn[ne][ptot][3], pphi[ne][ptot][8]: x, unit normal and
//              phi*J*w at the Gauss points of every precalculated rule
//   pair class cls[ncp][ne]: rule index, CLS_ADP or CLS_SING
//   lists      per collocation point, in element order: regular pairs
//              (e | rule << 24) with exclusive point offsets, adaptive pairs
//              with their subdivision leaves, singular pairs with their polar
//              layout and static line integrals
#pragma once
#include <cstdint>

namespace mfb {

enum : uint8_t { CLS_ADP = 254, CLS_SING = 255 };

constexpr int LEAF_D = 16;  // xs[4][2], telles1 {a,b,c,d}, telles2 {a,b,c,d}
constexpr int SING_D = 56;  // xi_i[2], x_i[3], phi_i[8], hli[9], th[8][2], thp[8][2], pad
constexpr int SING_I = 28;  // nsub, st[8], ngp_theta[8], off[9] (combo offsets), total, pad
constexpr int FT_D = 10;    // cp (solid-angle part) and sum_b[3][3] of the free term
// HBIE singular pairs: n_i[3], psi_i[8][3], then the edge line integrals
// lli[3][3], mli1, mli2[3], mli3[3][3], mli4[3], mli5[3][3][3]
constexpr int HSING_X = 80;
constexpr int HX_N = 0, HX_PSI = 3, HX_LLI = 27, HX_M1 = 36, HX_M2 = 37, HX_M3 = 40, HX_M4 = 49, HX_M5 = 52;

struct DMesh {
  int ne, ndn, ncp, ndof, nps, ptot, ns_max;
  int ps_gln[16], ps_off[16];
  int ps_gln_max;
  // elements
  const double* ex;
  const double* cl;
  const int* gln_far;
  const double* ball;
  const int* rev;
  const int* edof;
  // dofs
  const int* dct;
  const double* dcv;
  // collocation points
  const double* cpx;
  const int* cp_dn;
  const int* cp_kind;
  const int* cp_elem;
  const int* cp_kn;
  const double* cp_xi;
  const int* dn_cp;
  // free-term inputs: incidences of SBIE collocation nodes (element, local node)
  const int* inc_start;  // [ncp+1]
  const int* inc_el;     // element*8 + local
  const double* n_gn;    // [ne][8][3]
  const double* tbp_gn;  // [ne][8][3]
  double geo_tol;
  // datasets
  double* px;
  double* pn;
  double* pphi;
  // classes and lists
  uint8_t* cls;
  int* reg_start;        // [ncp+1]
  int* reg_pair;         // e | rule<<24
  long long* reg_pt;     // [nreg+1] exclusive prefix of points
  int* adp_start;        // [ncp+1]
  int* adp_e;
  int* adp_leaf;         // [nadp+1]
  double* leaf;          // [nleaf][LEAF_D]
  int* leaf_gln;
  int* leaf_pair;        // adaptive pair index of each leaf
  long long* leaf_pt;    // [nleaf+1]
  int* sing_start;       // [ncp+1]
  int* sing_e;
  double* sing_d;        // [nsing][SING_D]
  int* sing_i;           // [nsing][SING_I]
  long long* sing_pt;    // [nsing+1]
  // frequency-independent geometry of every singular / adaptive-leaf
  // quadrature point, component-major [component][point] (null: recompute)
  double* sing_geo;      // 22 components: x - x_i (3), unit normal (3), phi*jw (8), (phi - phi_i)*jw (8)
  double* leaf_geo;      // 14 components: x - x_i (3), unit normal (3), phi*jw (8)
  int* adp_cp;           // collocation point of each adaptive pair
  long long nsing_pts, nleaf_pts;
  double* ft;            // [ncp][FT_D]
  int* ft_ok;            // [ncp] 1 ok, 0 invalid configuration
  long long nreg, nadp, nleaf, nsing;
  // half-space region with a traction-free surface x[hs_ax] = hs_x (free
  // terms of collocation points on it doubled); hs_ax = -1: full space
  int hs_ax;
  double hs_x;
  // quasi-singular estimate order of the pair classification (5: SBIE, 7:
  // HBIE and the shared SBIE/HBIE classification of shbie_auto) and of the
  // adaptive subdivision (5 SBIE, 7 HBIE)
  int fcls, fadp;
  // HBIE view: collocation points carry the unit normal n_i and the Burton &
  // Miller weight alpha (cp_kind 2: HBIE alone, 3: Burton & Miller); the
  // singular pairs keep their HSING_X extras
  int hbie;
  const double* cp_n;
  const double* cp_alpha;
  double* hsing_x;
  // rows of each dnode's equations in a region with crack-like boundaries
  // (null: 3 dn + il): (row base << 1) | s, rows base + (il << s); a crack
  // node's SBIE rows are r, r+2, r+4 and its HBIE rows r+1, r+3, r+5
  // (build_auxiliary_variables_mechanics_static.f90:146-207)
  const int* dn_rb;
};

#ifdef __CUDACC__
__device__ __forceinline__ size_t dn_row(const DMesh& m, int dn, int il) {
  if (!m.dn_rb) return 3 * (size_t)dn + il;
  const int v = m.dn_rb[dn];
  return (size_t)(v >> 1) + ((size_t)il << (v & 1));
}
#endif

}  // namespace mfb

// CPU FP64 restatement of MultiFEBE's 3D collocation-BEM hot path (staela / harela).
//
// TEST INFRASTRUCTURE ONLY. This code is the oracle the GPU product is checked
// against; nothing under multifebe_gb300/ may include, link or call it. It follows
// the reference's Fortran control flow, constants and thresholds one to one (the
// file:line citations in orc_*.cpp name the routine each function restates), runs
// on the host cores with OpenMP, and is also the timed "reference-equivalent CPU
// path" when the Fortran reference cannot be built.
//
// Parity anchoring: the reference ships no golden vectors for this path. The
// oracle is pinned against (a) the reference's own quadrature tables
// (lib/fbem/src/resources_quad_rules/gl11.rc, gl01.rc) read in place, (b) the
// closed-form KAT of docs/examples/ME-ST-EL-002 (confined cube, exact linear
// field) and (c) rigid-body / static-limit identities of the method.
#pragma once
#include <complex>
#include <vector>
#include <cstdint>

namespace orc {

typedef std::complex<double> cplx;
typedef _Float128 quad;

// lib/fbem/src/numerical.f90:74-93
constexpr double c_pi = 3.14159265358979323846264338328;
constexpr double c_2pi = 6.28318530717958623199592693709;
constexpr double c_pi_2 = 1.57079632679489661923132169164;
constexpr double c_pi_4 = 0.78539816339744830961566084582;
constexpr double c_1_4pi = 0.07957747154594767280411105048;
constexpr double c_sqrt2 = 1.41421356237309504880168872421;
// lib/fbem/src/shape_functions.f90:280
constexpr double check_xi_tolerance = 0.5e-12;

// ---------------------------------------------------------------- quadrature
struct GaussTables {
  // Fortran layout gl11_xi(point, rule): index [(rule-1)*32 + point-1]
  double gl11_xi[32 * 32], gl11_w[32 * 32];
  double gl01_xi[32 * 32], gl01_w[32 * 32];
};
const GaussTables& gauss();
inline double gl11_xi(int k, int n) { return gauss().gl11_xi[(n - 1) * 32 + k - 1]; }
inline double gl11_w(int k, int n) { return gauss().gl11_w[(n - 1) * 32 + k - 1]; }
inline double gl01_xi(int k, int n) { return gauss().gl01_xi[(n - 1) * 32 + k - 1]; }
inline double gl01_w(int k, int n) { return gauss().gl01_w[(n - 1) * 32 + k - 1]; }

// ---------------------------------------------------------- shape functions
void phi_quad8(const double xi[2], double phi[8]);
void dphi_quad8(const double xi[2], double d1[8], double d2[8]);
void phi_quad8_q(const quad xi[2], quad phi[8]);
void dphi_quad8_q(const quad xi[2], quad d1[8], quad d2[8]);
void phi_quad4(const double xi[2], double phi[4]);
void dphi_quad4(const double xi[2], double d1[4], double d2[4]);
void phi_line3(double xi, double phi[3]);
void dphi_line3(double xi, double dphi[3]);
void phi_line3_q(quad xi, quad phi[3]);
void dphi_line3_q(quad xi, quad dphi[3]);
extern const double quad8_xi_nodes[8][2];
extern const int quad8_edge_node[4][3];

// ---------------------------------------------------------- quasi-singular
struct QsParams {
  double re;
  double dmin[3][8], dmax[3][8], alpha0[3][8], alpha1[3][8], beta1[3][8];
  double t_dmin[3][8], t_dmax[3][8], t_alpha0[3][8], t_alpha1[3][8], t_beta1[3][8];
};
void qs_calculate_parameters(double relative_error, QsParams& p);
// rn is ignored (3D only); dim = 1 (line) or 2 (quad); f = integrand 1/r^f
int qs_n_estimation_standard(int dim, int f, const QsParams& p, double d, const double* barxi);
int qs_n_estimation_telles(int dim, int f, const QsParams& p, double d, const double* barxi);
int qs_phijac_ngp_2d_quad8(const double x[8][3], double error_height, bool* achieve);

// ---------------------------------------------------------- telles
struct Telles { double c[4]; };
double telles_barr_any(double d);
Telles telles11(double bar_xi, double bar_r);
inline void telles_xi_jac(const Telles& t, double g, double& xi, double& jac) {
  xi = t.c[0] * (g * g * g) + t.c[1] * (g * g) + t.c[2] * g + t.c[3];
  jac = 3.0 * t.c[0] * (g * g) + 2.0 * t.c[1] * g + t.c[2];
}

// ---------------------------------------------------------- geometry
double length3d_line3(const double x[3][3], double tol);
double characteristic_length_quad8(const double x[8][3], double tol);
double characteristic_length_line3(const double x[3][3], double tol);
void element_ball_quad8(const double x[8][3], int glp, double centre[3], double* radius);
// method: 1 nodes, 2 minimisation, 3 sampling
void nearest_element_point_quad8(const double x[8][3], double cl, const double xi_[3],
                                 double barxi[2], double* rmin, double* d, int* method);
void nearest_element_point_line3(const double x[3][3], double cl, const double xi_[3],
                                 double* barxi, double* rmin, double* d, int* method);
void subdivision_coords_quad8(const double x[8][3], const double xi_s[4][2], double x_s[8][3]);
void subdivision_coords_line3(const double x[3][3], const double xi_s[2], double x_s[3][3]);

// ---------------------------------------------------------- polar
void polar_setup_quad(const double xi_i[2], int* nsubtri, int subtri[8], double theta[8][2],
                      double thetap[8][2]);
void polar_angular_quad(const double xi_i[2], int subtri, double thetap, double* theta,
                        double* rhoij);
bool check_xi1xi2_edge_quad(const double xi[2]);

// ---------------------------------------------------------- numerical
void zexp_decomposed(int nz, const cplx* z, cplx E[][2]);  // E[k][kz], k=0..6

}  // namespace orc

// Oracle (test infrastructure only): quadrature tables, shape functions,
// quasi-singular order estimation, Telles transformation and the decomposed
// exponential. Each function cites the reference routine it restates.
#include "orc.h"
#include <cmath>
#include <mutex>

namespace orc {

// --------------------------------------------------------------------------
// Gauss-Legendre rules 1..32 on [-1,1] and [0,1].
// The reference stores them as DATA tables (lib/fbem/src/quad_rules.f90:81-140,
// resources_quad_rules/gl11.rc, gl01.rc). Here they are recomputed from the
// Legendre recurrence by Newton iteration in binary128 and rounded once to
// binary64; tests/test_oracle_tables.py compares both tables point by point.
// --------------------------------------------------------------------------
static void legendre_q(int n, quad x, quad* p, quad* dp) {
  quad p0 = 1, p1 = x;
  if (n == 0) { *p = 1; *dp = 0; return; }
  for (int k = 2; k <= n; ++k) {
    quad pk = ((quad)(2 * k - 1) * x * p1 - (quad)(k - 1) * p0) / (quad)k;
    p0 = p1;
    p1 = pk;
  }
  *p = p1;
  *dp = (quad)n * (x * p1 - p0) / (x * x - (quad)1);
}

static GaussTables* build_gauss() {
  GaussTables* t = new GaussTables();
  for (int i = 0; i < 32 * 32; ++i) t->gl11_xi[i] = t->gl11_w[i] = t->gl01_xi[i] = t->gl01_w[i] = 0;
  for (int n = 1; n <= 32; ++n) {
    quad xs[32], ws[32];
    if (n == 1) {
      xs[0] = 0; ws[0] = 2;
    } else {
      for (int k = 1; k <= n; ++k) {
        // k-th largest root
        quad x = (quad)std::cos(c_pi * ((double)k - 0.25) / ((double)n + 0.5));
        for (int it = 0; it < 100; ++it) {
          quad p, dp;
          legendre_q(n, x, &p, &dp);
          quad dx = p / dp;
          x -= dx;
          double adx = (double)(dx < 0 ? -dx : dx);
          if (adx < 1e-33) break;
        }
        quad p, dp;
        legendre_q(n, x, &p, &dp);
        // ascending order as in the reference tables
        xs[n - k] = x;
        ws[n - k] = (quad)2 / (((quad)1 - x * x) * dp * dp);
      }
      if (n % 2 == 1) xs[n / 2] = 0;
    }
    for (int k = 0; k < n; ++k) {
      t->gl11_xi[(n - 1) * 32 + k] = (double)xs[k];
      t->gl11_w[(n - 1) * 32 + k] = (double)ws[k];
      t->gl01_xi[(n - 1) * 32 + k] = (double)(((quad)1 + xs[k]) / (quad)2);
      t->gl01_w[(n - 1) * 32 + k] = (double)(ws[k] / (quad)2);
    }
  }
  return t;
}

const GaussTables& gauss() {
  static GaussTables* g = nullptr;
  static std::once_flag once;
  std::call_once(once, [] { g = build_gauss(); });
  return *g;
}

// --------------------------------------------------------------------------
// quad8 / quad4 / line3 shape functions (delta = 0, continuous elements).
// Restates resources_shape_functions/phi_quad8.rc, dphidxi1_quad8.rc,
// dphidxi2_quad8.rc, phi_quad4.rc, dphidxi{1,2}_quad4.rc, phi_line3.rc,
// dphidxi_line3.rc. Node order: 1(-1,-1) 2(1,-1) 3(1,1) 4(-1,1) 5(0,-1) 6(1,0)
// 7(0,1) 8(-1,0) (resources_shape_functions/xi_quad8.rc).
// --------------------------------------------------------------------------
const double quad8_xi_nodes[8][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1},
                                     {0, -1},  {1, 0},  {0, 1}, {-1, 0}};
// shape_functions.f90:841-880 (quad8 edges: vertices then the mid node)
const int quad8_edge_node[4][3] = {{0, 1, 4}, {1, 2, 5}, {2, 3, 6}, {3, 0, 7}};

template <typename T>
static inline void phi8(const T xi[2], T phi[8]) {
  const T one = 1, q = 0.25, h = 0.5, two = 2;
  T a1 = xi[0], a2 = xi[1];
  T a3 = q * (one + a1), a4 = q * (one - a1);
  T a5 = one + a2, a6 = one - a2;
  T a7 = one - a1 * a1, a8 = one - a2 * a2;
  phi[0] = a4 * a6 * (-a1 - a5);
  phi[1] = a3 * a6 * (a1 - a5);
  phi[2] = a3 * a5 * (a1 - a6);
  phi[3] = a4 * a5 * (-a1 - a6);
  phi[4] = h * a6 * a7;
  phi[5] = two * a3 * a8;
  phi[6] = h * a5 * a7;
  phi[7] = two * a4 * a8;
}
template <typename T>
static inline void dphi8(const T xi[2], T d1[8], T d2[8]) {
  const T one = 1, q = 0.25, h = 0.5, two = 2;
  // d/dxi1
  {
    T a3 = xi[1] + one, a4 = xi[1] - one;
    T a5 = xi[1] + two * xi[0], a6 = xi[1] - two * xi[0];
    T a7 = -q, a8 = -xi[0];
    d1[0] = a7 * a4 * a5;
    d1[1] = -a7 * a4 * a6;
    d1[2] = -a7 * a3 * a5;
    d1[3] = a7 * a3 * a6;
    d1[4] = -a8 * a4;
    d1[5] = h * (-one) * a3 * a4;
    d1[6] = a8 * a3;
    d1[7] = -d1[5];
  }
  // d/dxi2
  {
    T a3 = xi[0] + one, a4 = xi[0] - one;
    T a5 = two * xi[1] + xi[0], a6 = two * xi[1] - xi[0];
    T a7 = -q, a8 = -xi[1];
    d2[0] = a7 * a4 * a5;
    d2[1] = -a7 * a3 * a6;
    d2[2] = -a7 * a3 * a5;
    d2[3] = a7 * a4 * a6;
    d2[4] = -h * (-one) * a3 * a4;
    d2[5] = a8 * a3;
    d2[6] = -d2[4];
    d2[7] = -a8 * a4;
  }
}
void phi_quad8(const double xi[2], double phi[8]) { phi8<double>(xi, phi); }
void dphi_quad8(const double xi[2], double d1[8], double d2[8]) { dphi8<double>(xi, d1, d2); }
void phi_quad8_q(const quad xi[2], quad phi[8]) { phi8<quad>(xi, phi); }
void dphi_quad8_q(const quad xi[2], quad d1[8], quad d2[8]) { dphi8<quad>(xi, d1, d2); }

void phi_quad4(const double xi[2], double phi[4]) {
  double a3 = 0.25 * (1.0 + xi[0]), a4 = 0.25 * (1.0 - xi[0]);
  double a5 = 1.0 + xi[1], a6 = 1.0 - xi[1];
  phi[0] = a4 * a6;
  phi[1] = a3 * a6;
  phi[2] = a3 * a5;
  phi[3] = a4 * a5;
}
void dphi_quad4(const double xi[2], double d1[4], double d2[4]) {
  d1[0] = -0.25 * (1.0 - xi[1]);
  d1[1] = 0.25 * (1.0 - xi[1]);
  d1[2] = 0.25 * (1.0 + xi[1]);
  d1[3] = -0.25 * (1.0 + xi[1]);
  d2[0] = -0.25 * (1.0 - xi[0]);
  d2[1] = -0.25 * (1.0 + xi[0]);
  d2[2] = 0.25 * (1.0 + xi[0]);
  d2[3] = 0.25 * (1.0 - xi[0]);
}
template <typename T>
static inline void phil3(T xi, T phi[3]) {
  const T h = 0.5, one = 1;
  T a2 = h * xi, a3 = xi - one, a4 = xi + one;
  phi[0] = a2 * a3;
  phi[1] = a2 * a4;
  phi[2] = -a3 * a4;
}
template <typename T>
static inline void dphil3(T xi, T d[3]) {
  const T h = 0.5, two = 2;
  d[0] = xi - h;
  d[1] = xi + h;
  d[2] = -two * xi;
}
void phi_line3(double xi, double phi[3]) { phil3<double>(xi, phi); }
void dphi_line3(double xi, double d[3]) { dphil3<double>(xi, d); }
void phi_line3_q(quad xi, quad phi[3]) { phil3<quad>(xi, phi); }
void dphi_line3_q(quad xi, quad d[3]) { dphil3<quad>(xi, d); }

// --------------------------------------------------------------------------
// Quasi-singular integration order estimator.
// Calibration coefficients: lib/fbem/src/quasisingular_integration.f90:181-287.
// They are the reference's fitted constants and must be identical here.
// --------------------------------------------------------------------------
// [curve][coef] as in the Fortran (curve,coefficient) arrays
static const double d1rn_alpha0[3][6] = {
    {2.443943976922257e-1, -7.845125775746743e-2, 3.895326800087784e-2, 8.783124822346978e-4,
     -1.719172638314362e-3, -1.575912106080523e-3},
    {1.855869272054077e-1, -8.441784317192081e-2, 3.992519918023225e-2, 1.003034542932314e-3,
     -2.012460287158036e-3, -1.596684136739970e-3},
    {1.964994120809251e-1, -7.533682025056084e-2, 6.300967117113785e-2, 1.453521059340246e-3,
     -1.653933461489553e-3, -2.613368441217468e-3}};
static const double d1rn_alpha1[3][6] = {
    {-8.421216556191472e-1, -8.778262996280104e-2, 1.679496012553309e-2, 6.522695414940627e-4,
     -2.649807213627071e-3, -8.472009602597869e-4},
    {-8.012899104725332e-1, -7.060561516342915e-2, 5.713299243166406e-3, -1.952251227204736e-4,
     -1.984455335909311e-3, -6.680823196695776e-4},
    {-5.891778953073477e-1, -4.515354064860566e-2, 5.728946548799128e-3, 1.106131193536092e-6,
     -1.179100966502172e-3, -5.355782068751523e-4}};
static const double d1rn_beta1[3][6] = {
    {-2.693032219216048e-2, -6.138311391493901e-2, 2.273921394673689e-2, 9.789745450155518e-4,
     -2.030377872751224e-3, -9.059289455187508e-4},
    {-2.353515879579821e-1, -5.141856801187955e-2, 1.693100431819354e-2, -1.491381226735667e-5,
     -1.330369292483563e-3, -1.264704521827383e-3},
    {-9.828561879516765e-2, -3.074365737570111e-2, 1.306905121742232e-2, 6.065437465834727e-5,
     -7.853234287066991e-4, -1.025889829482388e-3}};
static const double lnr_alpha0[3][3] = {
    {2.511371433253553e-1, -8.318131267946077e-2, -1.973643360180158e-3},
    {1.588915580092415e-1, -9.469173675969373e-2, -2.500979779162619e-3},
    {1.303338290205561e-1, -9.041069352366727e-2, -2.302123487272636e-3}};
static const double lnr_alpha1[3][3] = {
    {-8.301769338383449e-1, -7.458331284021328e-2, -1.992535165956408e-3},
    {-8.575272011921337e-1, -6.866562987114574e-2, -1.735469217262563e-3},
    {-5.785210418300009e-1, -3.107089548772586e-2, -4.204818399993008e-4}};
static const double lnr_beta1[3][3] = {
    {-1.114783338380396e-1, -6.169581618278328e-2, -1.873698813959166e-3},
    {-3.918234478283774e-1, -6.478096580939043e-2, -1.657459305149584e-3},
    {-1.933844506192423e-1, -3.303326826061181e-2, -6.497990057394490e-4}};
static const double t_lnr_alpha0[3][3] = {
    {2.5834148732821033e-01, -8.8865167808209675e-02, -2.3640194116454241e-03},
    {5.1283007739426911e-01, -1.1479138136155583e-02, 1.7167160355773211e-03},
    {4.1061632629507161e-01, -3.0669024691563598e-02, 5.1920314153891956e-04}};
static const double t_lnr_alpha1[3][3] = {
    {-9.1721308433764848e-01, -6.2837979237008845e-02, -1.1580362636310136e-03},
    {-1.0632414684959128e+00, -1.1633428696469847e-01, -4.4173578665990879e-03},
    {-1.1740312565911180e+00, -1.3946434974037192e-01, -5.4264705520737193e-03}};
static const double t_lnr_beta1[3][3] = {
    {-4.9431525769444484e-01, -6.5628053690049357e-02, -1.2683068366630545e-03},
    {-9.1742055835524161e-01, -1.4448614058834844e-01, -5.5849846784841173e-03},
    {-1.1668939380105636e+00, -1.7686541251294283e-01, -6.9562836980345301e-03}};
static const double t_d1rn_alpha0[3][6] = {
    {2.9379042486857926e-01, -7.6518438657183094e-02, 3.0011332045426935e-02, 5.8900790667561719e-04,
     -1.7642732320416377e-03, -1.3634192833061319e-03},
    {1.1155167367380846e-01, -9.0043220465500617e-02, 3.9605615471752335e-02, 1.0669688965738889e-03,
     -2.2428131063082419e-03, -1.6030309471606837e-03},
    {9.5587534756324991e-02, -8.5841370957250140e-02, 5.9724590614136340e-02, 1.4101322853742803e-03,
     -2.0424217927592597e-03, -2.4264102214015559e-03}};
static const double t_d1rn_alpha1[3][6] = {
    {-9.8339088502232042e-01, -8.6761356304300027e-02, 2.6028760963988956e-02, 7.7677507397256337e-04,
     -2.3619290417702245e-03, -1.2891431252005461e-03},
    {-6.5856321275500784e-01, -4.7354561095619759e-02, 1.9423558756522371e-03, -2.9087437598165618e-04,
     -1.1859755938049318e-03, -4.5988734937654318e-04},
    {-2.4634605754204883e-01, 1.0051411705899942e-02, -1.1994978255365170e-02, -1.0022065157916291e-03,
     7.9639034155470554e-04, -1.8103634920482468e-04}};
static const double t_d1rn_beta1[3][6] = {
    {-4.5453529921363467e-01, -7.3941529478921839e-02, 3.7672240427426076e-02, 9.8276802658567980e-04,
     -1.8897770518175436e-03, -1.8079562352345093e-03},
    {-2.6610069546799336e-01, -3.6048387668689889e-02, 1.3288129149913631e-02, -1.8099231920766130e-04,
     -7.6015457149682889e-04, -1.2247286683263207e-03},
    {7.5605400079843565e-02, 2.4021121564322980e-02, -9.3693044556669332e-03, -1.3532246088221670e-03,
     1.3564674989692248e-03, -7.4467072775070487e-04}};

// numerical.f90:675-697
static inline double poly1q(const double c[3], double x) { return c[0] + c[1] * x + c[2] * (x * x); }
static inline double poly2q(const double c[6], double x, double y) {
  return c[0] + c[1] * x + c[2] * y + c[3] * x * y + c[4] * (x * x) + c[5] * (y * y);
}

// quasisingular_integration.f90:318-398. log10(30.) and log10(2.) are default
// (single precision) REAL literals in the Fortran; reproduced as float.
void qs_calculate_parameters(double relative_error, QsParams& p) {
  double l = std::log10(std::fabs(relative_error));
  if (l > -3.0) l = -3.0;
  if (l < -15.0) l = -15.0;
  p.re = std::pow(10.0, l);
  const double l30 = (double)std::log10(30.0f), l2 = (double)std::log10(2.0f);
  for (int c = 0; c < 3; ++c) {
    p.alpha0[c][0] = poly1q(lnr_alpha0[c], l);
    p.alpha1[c][0] = poly1q(lnr_alpha1[c], l);
    p.beta1[c][0] = poly1q(lnr_beta1[c], l);
    p.dmin[c][0] = std::pow(10.0, (l30 - p.alpha0[c][0]) / (p.alpha1[c][0] - l30 * p.beta1[c][0]));
    p.dmax[c][0] = std::pow(10.0, (l2 - p.alpha0[c][0]) / (p.alpha1[c][0] - l2 * p.beta1[c][0]));
  }
  for (int i = 1; i <= 7; ++i)
    for (int c = 0; c < 3; ++c) {
      p.alpha0[c][i] = poly2q(d1rn_alpha0[c], l, (double)i);
      p.alpha1[c][i] = poly2q(d1rn_alpha1[c], l, (double)i);
      p.beta1[c][i] = poly2q(d1rn_beta1[c], l, (double)i);
      p.dmin[c][i] = std::pow(10.0, (l30 - p.alpha0[c][i]) / (p.alpha1[c][i] - l30 * p.beta1[c][i]));
      p.dmax[c][i] = std::pow(10.0, (l2 - p.alpha0[c][i]) / (p.alpha1[c][i] - l2 * p.beta1[c][i]));
    }
  for (int c = 0; c < 3; ++c) {
    p.t_alpha0[c][0] = poly1q(t_lnr_alpha0[c], l);
    p.t_alpha1[c][0] = poly1q(t_lnr_alpha1[c], l);
    p.t_beta1[c][0] = poly1q(t_lnr_beta1[c], l);
    p.t_dmin[c][0] = std::pow(10.0, (l30 - p.t_alpha0[c][0]) / (p.t_alpha1[c][0] - l30 * p.t_beta1[c][0]));
    p.t_dmax[c][0] = std::pow(10.0, (l2 - p.t_alpha0[c][0]) / (p.t_alpha1[c][0] - l2 * p.t_beta1[c][0]));
    if (p.t_dmin[c][0] < 1e-6) p.t_dmin[c][0] = 1e-6;
    if (p.t_dmin[c][0] > p.t_dmax[c][0]) p.t_dmin[c][0] = 1e-6;
  }
  for (int i = 1; i <= 7; ++i)
    for (int c = 0; c < 3; ++c) {
      p.t_alpha0[c][i] = poly2q(t_d1rn_alpha0[c], l, (double)i);
      p.t_alpha1[c][i] = poly2q(t_d1rn_alpha1[c], l, (double)i);
      p.t_beta1[c][i] = poly2q(t_d1rn_beta1[c], l, (double)i);
      p.t_dmin[c][i] = std::pow(10.0, (l30 - p.t_alpha0[c][i]) / (p.t_alpha1[c][i] - l30 * p.t_beta1[c][i]));
      p.t_dmax[c][i] = std::pow(10.0, (l2 - p.t_alpha0[c][i]) / (p.t_alpha1[c][i] - l2 * p.t_beta1[c][i]));
      if (p.t_dmin[c][i] < 1e-6) p.t_dmin[c][i] = 1e-6;
      if (p.t_dmin[c][i] > p.t_dmax[c][i]) p.t_dmin[c][i] = 1e-6;
    }
}

static inline double ncurve(double a0, double a1, double b1, double l) {
  return std::pow(10.0, (a0 + a1 * l) / (1.0 + b1 * l));
}

// Shared body of quasisingular_integration.f90:402-554 (standard) and
// 558-711 (telles); only the curve set for d<=2 differs. The optional r,q
// orientation arguments are never passed on this path.
static int qs_estimate(int dim, int f, const QsParams& p, double d, const double* barxi, bool tel) {
  const double(*dmin)[8] = tel ? p.t_dmin : p.dmin;
  const double(*dmax)[8] = tel ? p.t_dmax : p.dmax;
  const double(*a0)[8] = tel ? p.t_alpha0 : p.alpha0;
  const double(*a1)[8] = tel ? p.t_alpha1 : p.alpha1;
  const double(*b1)[8] = tel ? p.t_beta1 : p.beta1;
  int res;
  if (d <= 2.0) {
    double l = std::log10(d);
    double N1 = 0, N2 = 0;
    if (dim == 1) {
      if (std::fabs(barxi[0]) < 1.0) {
        if (d <= dmin[0][f]) return 0;
        N1 = (d >= dmax[0][f]) ? 2.0 : ncurve(a0[0][f], a1[0][f], b1[0][f], l);
        if (d <= dmin[1][f]) return 0;
        N2 = (d >= dmax[1][f]) ? 2.0 : ncurve(a0[1][f], a1[1][f], b1[1][f], l);
        res = (int)std::ceil(barxi[0] * barxi[0] * (N2 - N1) + N1);
      } else {
        if (d <= dmin[1][f]) return 0;
        N2 = (d >= dmax[1][f]) ? 2.0 : ncurve(a0[1][f], a1[1][f], b1[1][f], l);
        res = (int)std::ceil(N2);
      }
    } else {
      if (d <= dmin[0][f]) return 0;
      N1 = (d >= dmax[0][f]) ? 2.0 : ncurve(a0[0][f], a1[0][f], b1[0][f], l);
      if (d <= dmin[1][f]) return 0;
      N2 = (d >= dmax[1][f]) ? 2.0 : ncurve(a0[1][f], a1[1][f], b1[1][f], l);
      res = (int)std::ceil((barxi[0] * barxi[0]) * (barxi[1] * barxi[1]) * (N2 - N1) + N1);
    }
  } else {
    // both variants use the standard curve 3 for d>2
    if (d >= p.dmax[2][f]) {
      res = 2;
    } else {
      double l = std::log10(d);
      res = (int)std::lround(ncurve(p.alpha0[2][f], p.alpha1[2][f], p.beta1[2][f], l));
    }
  }
  if (res > 30) res = 0;
  return res;
}
int qs_n_estimation_standard(int dim, int f, const QsParams& p, double d, const double* barxi) {
  return qs_estimate(dim, f, p, d, barxi, false);
}
int qs_n_estimation_telles(int dim, int f, const QsParams& p, double d, const double* barxi) {
  return qs_estimate(dim, f, p, d, barxi, true);
}

// quasisingular_integration.f90:812-975 (quadrilateral branch, rn=3)
int qs_phijac_ngp_2d_quad8(const double x[8][3], double error_height, bool* achieve) {
  double eh = error_height;
  if (eh <= 0.0) eh = 1e-6;
  else if (eh < 1e-12) eh = 1e-12;
  bool cont = true;
  *achieve = true;
  double integral[8] = {0}, old[8];
  int j = 1;
  while (cont) {
    for (int l = 0; l < 8; ++l) { old[l] = integral[l]; integral[l] = 0.0; }
    for (int k1 = 1; k1 <= j; ++k1) {
      for (int k2 = 1; k2 <= j; ++k2) {
        double xi[2] = {gl11_xi(k1, j), gl11_xi(k2, j)};
        double d1[8], d2[8];
        dphi_quad8(xi, d1, d2);
        double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
        for (int l = 0; l < 8; ++l)
          for (int c = 0; c < 3; ++c) { T1[c] += d1[l] * x[l][c]; T2[c] += d2[l] * x[l][c]; }
        double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2],
                       T1[0] * T2[1] - T1[1] * T2[0]};
        double jac = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        double jw = jac * gl11_w(k1, j) * gl11_w(k2, j);
        double phi[8];
        phi_quad8(xi, phi);
        for (int l = 0; l < 8; ++l) integral[l] += (phi[l] + 1.0) * jw;
      }
    }
    if (j == 1) {
      j = j + 1;
    } else {
      cont = false;
      for (int l = 0; l < 8; ++l) {
        if (std::fabs((old[l] - integral[l]) / integral[l]) > eh) { cont = true; j = j + 1; break; }
      }
      if (j == 33) { cont = false; *achieve = false; }
    }
  }
  return j - 1;
}

// --------------------------------------------------------------------------
// Telles cubic transformation, telles_transformation.f90:77-162,221-233
// --------------------------------------------------------------------------
double telles_barr_any(double d) {
  double r = (d < 3.0) ? d / (0.89039 * d + 0.32883) : 1.0;
  if (r > 1.0) r = 1.0;
  return r;
}
Telles telles11(double bx, double br) {
  double w = bx / (1.0 + 2.0 * br);
  double p = 1.0 / (3.0 * (1.0 + 2.0 * br)) * (3.0 - 2.0 * br - 3.0 * w * bx);
  double q = w / 2.0 * ((3.0 - 2.0 * br) / (1.0 + 2.0 * br) - 2.0 * (w * w) - 1.0);
  double R2 = std::sqrt(q * q + p * p * p);
  double R31 = -q + R2, R32 = -q - R2;
  const double d13 = 1.0 / 3.0;
  R31 = (R31 >= 0.0) ? std::pow(R31, d13) : -std::pow(std::fabs(R31), d13);
  R32 = (R32 >= 0.0) ? std::pow(R32, d13) : -std::pow(std::fabs(R32), d13);
  double bg = R31 + R32 + w;
  double Q = 1.0 + 3.0 * (bg * bg);
  Telles t;
  t.c[0] = (1.0 - br) / Q;
  t.c[1] = -3.0 * bg * t.c[0];
  t.c[2] = (br + 3.0 * (bg * bg)) / Q;
  t.c[3] = -t.c[1];
  return t;
}

// --------------------------------------------------------------------------
// E_n decomposition of exp(z), numerical.f90:1258-1331
// --------------------------------------------------------------------------
void zexp_decomposed(int nz, const cplx* z, cplx E[][2]) {
  for (int kz = 0; kz < nz; ++kz) {
    cplx zk = z[kz];
    double absz = std::abs(zk);
    if (absz <= 1.0) {
      int n;
      if (absz <= 1e-6) n = 1;
      else n = (int)std::lround(std::pow(10.0, 1.176 + 0.175 * std::log10(absz)));
      cplx term[22];
      term[0] = cplx(1.0, 0.0);
      term[1] = zk;
      double fact = 1.0;
      cplx zp = zk;
      for (int k = 2; k <= n + 6; ++k) {
        fact = fact * (double)k;
        zp = zp * zk;
        term[k] = zp / fact;
      }
      cplx e6(0.0, 0.0);
      for (int k = n + 6; k >= 6; --k) e6 = e6 + term[k];
      E[6][kz] = e6;
      E[5][kz] = E[6][kz] + term[5];
      E[4][kz] = E[5][kz] + term[4];
      E[3][kz] = E[4][kz] + term[3];
      E[2][kz] = E[3][kz] + term[2];
      E[1][kz] = E[2][kz] + term[1];
      E[0][kz] = E[1][kz] + term[0];
    } else {
      cplx ez = std::exp(zk);
      cplx z2 = zk * zk, z3 = z2 * zk, z4 = z3 * zk, z5 = z4 * zk;
      E[0][kz] = ez;
      E[1][kz] = ez - 1.0;
      E[2][kz] = E[1][kz] - zk;
      E[3][kz] = E[2][kz] - 0.5 * z2;
      E[4][kz] = E[3][kz] - (1.0 / 6.0) * z3;
      E[5][kz] = E[4][kz] - (1.0 / 24.0) * z4;
      E[6][kz] = E[5][kz] - (1.0 / 120.0) * z5;
    }
  }
}

}  // namespace orc

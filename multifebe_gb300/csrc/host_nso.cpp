// Nodal-solution export (*.nso) of the mechanics problems, host side: the
// boundary-node records of src/export_solution_mechanics_harmonic_nso.f90 and
// src/export_solution_mechanics_static_nso.f90 for an ordinary boundary of a
// BE region, written with the Fortran edit descriptors the reference's export
// settings select (src/read_export.f90:61-70,163-171,212-214): integer
// columns Iw, real columns Ew.dEe (sci_*) or ENw.dEe (eng_*, the default
// en18.8e2). So a parity run can produce the reference's output files
// without the Fortran front end.
//
// Formatting follows the Fortran standard's rules for output editing: E
// editing prints 0.d1...dd with the exponent chosen so that the first digit
// is nonzero (scale factor 0), EN editing a significand in [1, 1000) and an
// exponent divisible by three; the exponent field has e digits after its
// sign; fields are right-justified in w characters (w asterisks when the
// value does not fit). Decimal rounding is the C library's (correctly
// rounded, nearest).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

thread_local std::string g_nso_err;

std::string stars(int w) { return std::string((size_t)std::max(w, 0), '*'); }

std::string rjust(const std::string& s, int w) {
  if ((int)s.size() > w) return stars(w);
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

// digits (without point) and decimal exponent x of |v| rounded to `sig`
// significant digits: |v| ~ 0.D1D2... x 10^x
void sig_digits(double a, int sig, std::string& digits, int& x) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*e", sig - 1, a);  // d.ddd...e+XX
  const char* p = buf;
  digits.clear();
  for (; *p && *p != 'e'; ++p)
    if (*p >= '0' && *p <= '9') digits.push_back(*p);
  x = std::atoi(p + 1) + 1;
}

std::string exp_field(int x, int e) {
  char b[32];
  std::snprintf(b, sizeof b, "%c%0*d", x < 0 ? '-' : '+', e, std::abs(x));
  if ((int)std::strlen(b) > e + 1) return "";  // exponent does not fit
  return b;
}

}  // namespace

extern "C" {

// One value v under the edit descriptor kind 'I' (w), 'E' (Ew.dEe) or 'N'
// (ENw.dEe), written NUL-terminated to out (at least w + 1 bytes).
int mfbem_fortran_format(char kind, int32_t w, int32_t d, int32_t e, double v, char* out) {
  if (!out || w <= 0 || w > 200 || d < 0 || d > 60 || e < 1 || e > 6) return -1;
  std::string s;
  if (kind == 'I') {
    char b[64];
    std::snprintf(b, sizeof b, "%lld", (long long)v);
    s = rjust(b, w);
  } else if (kind == 'E' || kind == 'N') {
    const bool neg = std::signbit(v) && v != 0.0;
    const double a = std::fabs(v);
    std::string mant;
    int x = 0;
    if (!std::isfinite(v)) {
      s = rjust(std::isnan(v) ? "NaN" : (neg ? "-Infinity" : "Infinity"), w);
    } else if (kind == 'E') {
      std::string dig;
      if (a == 0.0) {
        dig = std::string((size_t)std::max(d, 1), '0');
        x = 0;
      } else {
        sig_digits(a, std::max(d, 1), dig, x);
      }
      mant = "0." + dig.substr(0, (size_t)d);
      const std::string ef = exp_field(x, e);
      s = ef.empty() ? stars(w) : rjust(std::string(neg ? "-" : "") + mant + "E" + ef, w);
    } else {
      // EN: significand in [1, 1000), exponent a multiple of 3
      std::string dig;
      int ip = 1;  // digits before the point
      if (a == 0.0) {
        dig = std::string((size_t)(d + 1), '0');
        x = 1;
      } else {
        // the rounding can carry into a new decade: settle the exponent first
        int xe = (int)std::floor(std::log10(a)) + 1;  // a ~ 0.D x 10^xe
        for (int pass = 0; pass < 3; ++pass) {
          const int t = ((xe - 1) % 3 + 3) % 3;  // (xe - 1) mod 3
          sig_digits(a, t + 1 + d, dig, x);
          if (x == xe) break;
          xe = x;
        }
        ip = ((x - 1) % 3 + 3) % 3 + 1;
      }
      const int xs = x - ip;  // exponent of the significand
      mant = dig.substr(0, (size_t)ip) + "." + dig.substr((size_t)ip, (size_t)d);
      const std::string ef = exp_field(xs, e);
      s = ef.empty() ? stars(w) : rjust(std::string(neg ? "-" : "") + mant + "E" + ef, w);
    }
  } else {
    return -1;
  }
  std::memcpy(out, s.c_str(), s.size() + 1);
  return 0;
}

// Boundary-node records of one ordinary boundary of a BE region (3D,
// elastic or viscoelastic): per record C1 step / frequency index, C2 0 or
// the frequency, C3-C5 region id, class (1, BE) and type (2, viscoelastic),
// C6-C8 boundary id, class (1, ordinary) and face (1), C9 node id, C10-C12
// coordinates, then u1 u2 u3 t1 t2 t3 (harmonic: each as two columns,
// cartesian re / im (complex_notation 2) or polar |z| / arg z (1), followed by
// the incident field, zero here). values: [n][6] doubles (static) or [n][6]
// complex as re / im pairs (harmonic). Integer columns I(int_w), real columns
// the descriptor (kind, w, d, e). header: text written first (NULL: none).
// append: add to the file instead of replacing it. Returns 0 or -1 (reason
// in mfbem_nso_error()).
int mfbem_nso_write(const char* path, int32_t append, const char* header, int32_t harmonic, int32_t kf, double omega,
                    int32_t region_id, int32_t n, const int32_t* node_id, const int32_t* boundary_id, const double* x,
                    const double* values, int32_t int_w, char kind, int32_t w, int32_t d, int32_t e,
                    int32_t complex_notation) {
  g_nso_err.clear();
  if (!path || n < 0 || (n > 0 && (!node_id || !boundary_id || !x || !values)) || int_w <= 0 ||
      (harmonic && complex_notation != 1 && complex_notation != 2)) {
    g_nso_err = "invalid argument";
    return -1;
  }
  FILE* f = std::fopen(path, append ? "a" : "w");
  if (!f) {
    g_nso_err = std::string("cannot open ") + path;
    return -1;
  }
  if (header) std::fputs(header, f);
  char b[256];
  auto I = [&](double v) {
    mfbem_fortran_format('I', int_w, 0, 1, v, b);
    std::fputs(b, f);
  };
  auto R = [&](double v) -> bool {
    if (mfbem_fortran_format(kind, w, d, e, v, b)) return false;
    std::fputs(b, f);
    return true;
  };
  for (int r = 0; r < n; ++r) {
    I(harmonic ? kf : 0);
    if (!R(harmonic ? omega : 0.0)) {
      std::fclose(f);
      g_nso_err = "invalid real edit descriptor";
      return -1;
    }
    I(region_id);
    I(1);
    I(2);
    I(boundary_id[r]);
    I(1);
    I(1);
    I(node_id[r]);
    for (int c = 0; c < 3; ++c) R(x[3 * (size_t)r + c]);
    if (harmonic) {
      for (int k = 0; k < 6; ++k) {
        const double re = values[12 * (size_t)r + 2 * k], im = values[12 * (size_t)r + 2 * k + 1];
        if (complex_notation == 2) {
          R(re);
          R(im);
        } else {
          R(std::hypot(re, im));
          R(std::atan2(im, re));
        }
      }
      for (int k = 0; k < 12; ++k) R(0.0);
    } else {
      for (int k = 0; k < 6; ++k) R(values[6 * (size_t)r + k]);
    }
    std::fputc('\n', f);
  }
  std::fclose(f);
  return 0;
}

const char* mfbem_nso_error(void) { return g_nso_err.c_str(); }

}  // extern "C"

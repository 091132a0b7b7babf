// Host-side mesh preparation (see tmc_prep.h).  Compiled with
// -ffp-contract=off so the derived metrics and stencil weights are the
// IEEE results of the reference's expression order.
#include "tmc_prep.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace tmc {

// ----------------------------------------------------------------------------
// Space-filling curve
// ----------------------------------------------------------------------------
uint64_t hilbert_key(double x, double y, double z) {
  const int b = 20;
  const double scale = (double)((1u << b) - 1);
  uint32_t X[3];
  const double c[3] = {x, y, z};
  for (int i = 0; i < 3; ++i) {
    double t = (std::min(1.0, std::max(-1.0, c[i])) + 1.0) * 0.5;
    X[i] = (uint32_t)std::llround(t * scale);
  }
  // Skilling, "Programming the Hilbert curve" (AIP Conf. Proc. 707, 2004):
  // axes -> transposed Hilbert index.
  const uint32_t M = 1u << (b - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t key = 0;
  for (int j = b - 1; j >= 0; --j)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> j) & 1u);
  return key;
}

// 3-D Morton (Z-order) index of a point of [-1,1]^3: the bits of the three
// 20-bit coordinates interleaved, most significant first.
uint64_t morton_key(double x, double y, double z) {
  const int b = 20;
  const double scale = (double)((1u << b) - 1);
  const double c[3] = {x, y, z};
  uint32_t X[3];
  for (int i = 0; i < 3; ++i) {
    const double t = (std::min(1.0, std::max(-1.0, c[i])) + 1.0) * 0.5;
    X[i] = (uint32_t)std::llround(t * scale);
  }
  uint64_t key = 0;
  for (int j = b - 1; j >= 0; --j)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> j) & 1u);
  return key;
}

namespace {

// element order: 0 the caller's, 1 Hilbert curve, 2 Morton curve of the
// unit-sphere positions
std::vector<int32_t> sfc_order(int n, const double* x, const double* y, const double* z, int mode) {
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  if (mode == 0) return order;
  std::vector<uint64_t> key(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double r = std::sqrt(x[i] * x[i] + y[i] * y[i] + z[i] * z[i]);
    key[i] = mode == 2 ? morton_key(x[i] / r, y[i] / r, z[i] / r) : hilbert_key(x[i] / r, y[i] / r, z[i] / r);
  }
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
  return order;
}

// ----------------------------------------------------------------------------
// poly_fit_run (src/utils/poly_fit_mod.F90:119-609) with math_inv_matrix /
// gaussian_elimination (src/utils/math_mod.F90:52-133) and the geometry of
// src/utils/sphere_geometry_mod.F90:186-252, in the reference's arithmetic
// order.  Indices here are 0-based in the ORIGINAL numbering.
// ----------------------------------------------------------------------------
struct Fit {
  // n-by-n matrices are column-major with leading dimension n
  static void gauss(int n, double* A, int* ipiv) {
    auto a = [&](int i, int j) -> double& { return A[(j - 1) * n + (i - 1)]; };
    double c[kMaxFit + 1];
    int k = 1;
    for (int i = 1; i <= n; ++i) ipiv[i] = i;
    for (int i = 1; i <= n; ++i) {
      double c1 = 0.0;
      for (int j = 1; j <= n; ++j) c1 = std::fmax(c1, std::fabs(a(i, j)));
      c[i] = c1;
    }
    for (int j = 1; j <= n - 1; ++j) {
      double best = 0.0;
      for (int i = j; i <= n; ++i) {
        double v = std::fabs(a(ipiv[i], j)) / c[ipiv[i]];
        if (v > best) {
          best = v;
          k = i;
        }
      }
      std::swap(ipiv[j], ipiv[k]);
      for (int i = j + 1; i <= n; ++i) {
        double pj = a(ipiv[i], j) / a(ipiv[j], j);
        a(ipiv[i], j) = pj;
        for (int q = j + 1; q <= n; ++q) a(ipiv[i], q) = a(ipiv[i], q) - pj * a(ipiv[j], q);
      }
    }
  }
  static void inverse(int n, double* A, double* B) {
    double C[kMaxFit * kMaxFit];
    int ipiv[kMaxFit + 1];
    auto a = [&](int i, int j) -> double& { return A[(j - 1) * n + (i - 1)]; };
    auto cc = [&](int i, int j) -> double& { return C[(j - 1) * n + (i - 1)]; };
    auto bb = [&](int i, int j) -> double& { return B[(j - 1) * n + (i - 1)]; };
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) cc(i, j) = (i == j) ? 1.0 : 0.0;
    gauss(n, A, ipiv);
    for (int i = 1; i <= n - 1; ++i)
      for (int j = i + 1; j <= n; ++j)
        for (int k = 1; k <= n; ++k) cc(ipiv[j], k) = cc(ipiv[j], k) - a(ipiv[j], i) * cc(ipiv[i], k);
    for (int i = 1; i <= n; ++i) {
      bb(n, i) = cc(ipiv[n], i) / a(ipiv[n], n);
      for (int j = n - 1; j >= 1; --j) {
        bb(j, i) = cc(ipiv[j], i);
        for (int k = j + 1; k <= n; ++k) bb(j, i) = bb(j, i) - a(ipiv[j], k) * bb(k, i);
        bb(j, i) = bb(j, i) / a(ipiv[j], j);
      }
    }
  }
  static double dot3(const double* a, const double* b) {
    double s = 0.0;
    s = s + a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
  }
  static void cross3(const double* x, const double* y, double* r) {
    r[0] = x[1] * y[2] - x[2] * y[1];
    r[1] = x[2] * y[0] - x[0] * y[2];
    r[2] = x[0] * y[1] - x[1] * y[0];
  }
  static void normalize(double* x) {
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = s + x[i] * x[i];
    double n = std::sqrt(s);
    if (n != 0)
      for (int i = 0; i < 3; ++i) x[i] = x[i] / n;
  }
  static double sphere_angle(const double* a, const double* b, const double* c) {
    double nab[3], nac[3], d1[3], d2[3], t[3];
    cross3(a, b, nab);
    normalize(nab);
    cross3(a, c, nac);
    normalize(nac);
    double r = std::acos(std::fmax(std::fmin(dot3(nab, nac), 1.0), -1.0));
    for (int i = 0; i < 3; ++i) {
      d1[i] = b[i] - a[i];
      d2[i] = c[i] - a[i];
    }
    cross3(d1, d2, t);
    if (dot3(t, a) < 0.0) r = -r;
    return r;
  }
  static double arc_length(const double* a, const double* b) {
    return std::acos(std::fmax(std::fmin(dot3(a, b), 1.0), -1.0));
  }

  // Projected coordinates of fit points fit[0..nf-1] (poly_fit_mod.F90:187-207).
  static void project(const int32_t* fit, int nf, const double* X, const double* Y, const double* Z,
                      double radius, double* xp, double* yp, double* theta) {
    double xc[kFitLd][3];
    for (int i = 0; i < nf; ++i) {
      xc[i][0] = X[fit[i]] / radius;
      xc[i][1] = Y[fit[i]] / radius;
      xc[i][2] = Z[fit[i]] / radius;
    }
    xp[0] = 0.0;
    yp[0] = 0.0;
    for (int i = 1; i < nf; ++i) {
      theta[i] = sphere_angle(xc[0], xc[1], xc[i]);
      double d = radius * arc_length(xc[0], xc[i]);
      xp[i] = std::cos(theta[i]) * d;
      yp[i] = std::sin(theta[i]) * d;
    }
  }

  // B(1:n,1:m) of the unweighted least-squares fit (poly_fit_mod.F90:209-230);
  // B is returned column-major with leading dimension kMaxFit.
  static void lsq(int m, int n, const double* xp, const double* yp, double* B) {
    double P[kMaxFit * kMaxFit], PTP[kMaxFit * kMaxFit], A[kMaxFit * kMaxFit], Ai[kMaxFit * kMaxFit];
    auto p = [&](int i, int j) -> double& { return P[(j - 1) * kMaxFit + (i - 1)]; };
    std::memset(P, 0, sizeof(P));
    for (int i = 1; i <= m; ++i) {
      double x = xp[i], y = yp[i];
      p(i, 1) = x;
      p(i, 2) = y;
      p(i, 3) = x * x;
      p(i, 4) = x * y;
      p(i, 5) = y * y;
      if (n >= 9) {
        p(i, 6) = x * x * x;
        p(i, 7) = y * (x * x);
        p(i, 8) = x * (y * y);
        p(i, 9) = y * y * y;
      }
      if (n >= 14) {
        p(i, 10) = (x * x) * (x * x);
        p(i, 11) = y * (x * x * x);
        p(i, 12) = (x * x) * (y * y);
        p(i, 13) = x * (y * y * y);
        p(i, 14) = (y * y) * (y * y);
      }
    }
    // P^T W^T W P with W = I: sum over fit points in order
    for (int i = 1; i <= n; ++i)
      for (int j = 1; j <= n; ++j) {
        double s = 0.0;
        for (int k = 1; k <= m; ++k) s = s + p(k, i) * p(k, j);
        PTP[(j - 1) * kMaxFit + (i - 1)] = s;
      }
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) A[(j - 1) * n + (i - 1)] = PTP[(j - 1) * kMaxFit + (i - 1)];
    inverse(n, A, Ai);
    std::memset(B, 0, sizeof(double) * kMaxFit * kMaxFit);
    for (int i = 1; i <= n; ++i)
      for (int j = 1; j <= m; ++j) {
        double s = 0.0;
        for (int k = 1; k <= n; ++k) s = s + Ai[(k - 1) * n + (i - 1)] * p(j, k);
        B[(j - 1) * kMaxFit + (i - 1)] = s;
      }
  }
};

inline double bm(const double* B, int i, int j) { return B[(j - 1) * kMaxFit + (i - 1)]; }

struct FitTables {
  std::vector<int32_t> nfit2c, nfit4c, nfit2v, nfit4v;  // counts (incl. centre)
  std::vector<int32_t> fit2c, fit4c, fit2v, fit4v;      // [n][kFitLd], 0-based original
  std::vector<double> d2c, d3c, d4c, d2v, d4v;          // [ne][2][kFitLd]
};

void poly_fit(const tmc_mesh_desc& d, int nc, int ne, int nv, int me, int vd, double radius,
              const std::vector<double>& Xc, const std::vector<double>& Yc, const std::vector<double>& Zc,
              const std::vector<double>& Xv, const std::vector<double>& Yv, const std::vector<double>& Zv,
              const std::vector<int32_t>& vov, bool do_cells, bool do_vertices, FitTables& F) {
  auto eoc = [&](int i, int c) { return d.edgesOnCell[(size_t)c * me + i] - 1; };
  auto coc = [&](int i, int c) { return d.cellsOnCell[(size_t)c * me + i] - 1; };
  auto voc = [&](int i, int c) { return d.verticesOnCell[(size_t)c * me + i] - 1; };
  auto coe = [&](int i, int e) { return d.cellsOnEdge[(size_t)e * 2 + i] - 1; };
  auto voe = [&](int i, int e) { return d.verticesOnEdge[(size_t)e * 2 + i] - 1; };
  auto cov = [&](int i, int v) { return d.cellsOnVertex[(size_t)v * vd + i] - 1; };
  auto eov = [&](int i, int v) { return d.edgesOnVertex[(size_t)v * vd + i] - 1; };
  auto nEoC = [&](int c) { return d.nEdgesOnCell[c]; };
  auto D = [&](std::vector<double>& a, int j, int s, int e) -> double& {
    return a[((size_t)e * 2 + s) * kFitLd + j];
  };

  if (do_cells) {
    F.nfit2c.assign(nc, 0);
    F.nfit4c.assign(nc, 0);
    F.fit2c.assign((size_t)nc * kFitLd, -1);
    F.fit4c.assign((size_t)nc * kFitLd, -1);
    F.d2c.assign((size_t)ne * 2 * kFitLd, 0.0);
    F.d3c.assign((size_t)ne * 2 * kFitLd, 0.0);
    F.d4c.assign((size_t)ne * 2 * kFitLd, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int c = 0; c < nc; ++c) {
      int32_t* f2 = &F.fit2c[(size_t)c * kFitLd];
      int32_t* f4 = &F.fit4c[(size_t)c * kFitLd];
      int n = nEoC(c);
      f2[0] = c;
      f4[0] = c;
      for (int i = 0; i < n; ++i) f2[i + 1] = f4[i + 1] = coc(i, c);
      int n2 = n + 1, n4 = n + 1;
      for (int i = 1; i <= n; ++i) {
        int fi = f4[i];
        for (int j = 0; j < nEoC(fi); ++j) {
          int g = coc(j, fi);
          bool rec = false;
          for (int k = 0; k < n4; ++k)
            if (f4[k] == g) {
              rec = true;
              break;
            }
          if (!rec && n4 < kFitLd) f4[n4++] = g;
        }
      }
      F.nfit2c[c] = n2;
      F.nfit4c[c] = n4;
      double xp[kFitLd], yp[kFitLd], th[kFitLd], B[kMaxFit * kMaxFit];
      // 2nd order
      Fit::project(f2, n2, Xc.data(), Yc.data(), Zc.data(), radius, xp, yp, th);
      Fit::lsq(n2 - 1, 5, xp, yp, B);
      for (int i = 1; i <= n; ++i) {
        int e = eoc(i - 1, c);
        int s = (c == coe(0, e)) ? 0 : 1;
        double ct = std::cos(th[i]), st = std::sin(th[i]);
        for (int j = 1; j <= n2 - 1; ++j) {
          double a = 2.0 * bm(B, 3, j) * (ct * ct);
          double b = bm(B, 4, j) * ct * st;
          double cc = 2.0 * bm(B, 5, j) * (st * st);
          D(F.d2c, j, s, e) = a + 2.0 * b + cc;
        }
      }
      // 3rd order on the 2-ring stencil; d3fdxdy2 is never set in the
      // reference (poly_fit_mod.F90:310-314) and is taken as 0 here.
      Fit::project(f4, n4, Xc.data(), Yc.data(), Zc.data(), radius, xp, yp, th);
      Fit::lsq(n4 - 1, 9, xp, yp, B);
      for (int i = 1; i <= n; ++i) {
        int e = eoc(i - 1, c);
        int s = (c == coe(0, e)) ? 0 : 1;
        double ct = std::cos(th[i]), st = std::sin(th[i]);
        for (int j = 1; j <= n4 - 1; ++j) {
          double a = 6.0 * bm(B, 6, j) * (ct * ct * ct);
          double b = 2.0 * bm(B, 8, j) * ct * (st * st);
          double e3 = 6.0 * bm(B, 9, j) * (st * st * st);
          D(F.d3c, j, s, e) = a + 3.0 * b + 3.0 * 0.0 + e3;
        }
      }
      // 4th order
      Fit::lsq(n4 - 1, 14, xp, yp, B);
      for (int i = 1; i <= n; ++i) {
        int e = eoc(i - 1, c);
        int s = (c == coe(0, e)) ? 0 : 1;
        double ct = std::cos(th[i]), st = std::sin(th[i]);
        for (int j = 1; j <= n4 - 1; ++j) {
          double a = 24.0 * bm(B, 10, j) * ((ct * ct) * (ct * ct));
          double b = 6.0 * bm(B, 11, j) * (ct * ct * ct) * st;
          double cc = 4.0 * bm(B, 12, j) * (ct * ct) * (st * st);
          double dd = 6.0 * bm(B, 13, j) * ct * (st * st * st);
          double ee = 24.0 * bm(B, 14, j) * ((st * st) * (st * st));
          D(F.d4c, j, s, e) = a + 4.0 * b + 6.0 * cc + 4.0 * dd + ee;
        }
      }
    }
  }

  if (do_vertices) {
    F.nfit2v.assign(nv, 0);
    F.nfit4v.assign(nv, 0);
    F.fit2v.assign((size_t)nv * kFitLd, -1);
    F.fit4v.assign((size_t)nv * kFitLd, -1);
    F.d2v.assign((size_t)ne * 2 * kFitLd, 0.0);
    F.d4v.assign((size_t)ne * 2 * kFitLd, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int v = 0; v < nv; ++v) {
      int32_t* f2 = &F.fit2v[(size_t)v * kFitLd];
      int32_t* f4 = &F.fit4v[(size_t)v * kFitLd];
      f2[0] = v;
      for (int i = 0; i < vd; ++i) f2[i + 1] = vov[(size_t)v * vd + i];
      int n2 = vd + 1;
      auto add = [&](int32_t* f, int& nf, int g) {
        for (int k = 0; k < nf; ++k)
          if (f[k] == g) return;
        if (nf < kFitLd) f[nf++] = g;
      };
      for (int i = 0; i < vd; ++i) {
        int hc = cov(i, v);
        for (int j = 0; j < nEoC(hc); ++j) add(f2, n2, voc(j, hc));
      }
      int n4 = n2;
      for (int k = 0; k < kFitLd; ++k) f4[k] = f2[k];
      for (int q = 0; q < vd; ++q) {
        int hv = vov[(size_t)v * vd + q];
        for (int i = 0; i < vd; ++i) {
          int hc = cov(i, hv);
          for (int j = 0; j < nEoC(hc); ++j) add(f4, n4, voc(j, hc));
        }
      }
      F.nfit2v[v] = n2;
      F.nfit4v[v] = n4;
      double xp[kFitLd], yp[kFitLd], th[kFitLd], B[kMaxFit * kMaxFit];
      Fit::project(f2, n2, Xv.data(), Yv.data(), Zv.data(), radius, xp, yp, th);
      Fit::lsq(n2 - 1, 5, xp, yp, B);
      for (int i = 1; i <= vd; ++i) {
        int e = eov(i - 1, v);
        int s = (v == voe(0, e)) ? 0 : 1;
        double ct = std::cos(th[i]), st = std::sin(th[i]);
        for (int j = 1; j <= n2 - 1; ++j) {
          double a = 2.0 * bm(B, 3, j) * (ct * ct);
          double b = bm(B, 4, j) * ct * st;
          double cc = 2.0 * bm(B, 5, j) * (st * st);
          D(F.d2v, j, s, e) = a + 2.0 * b + cc;
        }
      }
      Fit::project(f4, n4, Xv.data(), Yv.data(), Zv.data(), radius, xp, yp, th);
      Fit::lsq(n4 - 1, 14, xp, yp, B);
      for (int i = 1; i <= vd; ++i) {
        int e = eov(i - 1, v);
        int s = (v == voe(0, e)) ? 0 : 1;
        double ct = std::cos(th[i]), st = std::sin(th[i]);
        for (int j = 1; j <= n4 - 1; ++j) {
          double a = 24.0 * bm(B, 10, j) * ((ct * ct) * (ct * ct));
          double b = 6.0 * bm(B, 11, j) * (ct * ct * ct) * st;
          double cc = 4.0 * bm(B, 12, j) * (ct * ct) * (st * st);
          double dd = 6.0 * bm(B, 13, j) * ct * (st * st * st);
          double ee = 24.0 * bm(B, 14, j) * ((st * st) * (st * st));
          D(F.d4v, j, s, e) = a + 4.0 * b + 6.0 * cc + 4.0 * dd + ee;
        }
      }
    }
  }
}

// Compact one (fit counts, fit lists, deriv weights) family into a Stencil.
void compact(const std::vector<int32_t>& nfit, const std::vector<int32_t>& fit, const std::vector<double>& der,
             const std::vector<int32_t>& side_centre /*[ne][2] original*/, const std::vector<int32_t>& o2n,
             const std::vector<int32_t>& edge_n2o, int ne, Stencil& S) {
  int width = 0;
  for (int e = 0; e < ne; ++e)
    for (int s = 0; s < 2; ++s) width = std::max(width, nfit[side_centre[(size_t)e * 2 + s]] - 1);
  S.width = width;
  S.count.assign((size_t)2 * ne, 0);
  S.idx.assign((size_t)width * 2 * ne, 0);
  S.w.assign((size_t)width * 2 * ne, 0.0);
#pragma omp parallel for schedule(static)
  for (int en = 0; en < ne; ++en) {
    int eo = edge_n2o[en];
    for (int s = 0; s < 2; ++s) {
      int ctr = side_centre[(size_t)eo * 2 + s];
      int n = nfit[ctr] - 1;
      S.count[(size_t)s * ne + en] = (uint8_t)n;
      for (int j = 1; j <= n; ++j) {
        size_t k = ((size_t)(j - 1) * 2 + s) * ne + en;
        S.idx[k] = o2n[fit[(size_t)ctr * kFitLd + j]];
        S.w[k] = der[((size_t)eo * 2 + s) * kFitLd + j];
      }
    }
  }
}

// Vector reconstruction coefficients of one cell (mpas_vector_reconstruction.F90:52-127;
// mpas_rbf_interpolation.F90:1076-1142, :1524-1556 with the inverse multiquadric
// :1366-1373 and scaled partial pivoting :1667-1695, :1779-1843, the method of
// Pang 1997), in the reference's operation order; positions radius-scaled.
void unit3(double v[3]) {
  const double mag = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int i = 0; i < 3; ++i) v[i] = v[i] / mag;
}
double rbf_imq(double r2) { return 1.0 / std::sqrt(1.0 + r2); }

// Gaussian elimination with scaled partial pivoting and the solve: column-major n x n
void pivot_solve(double* a, int n, double* b, double* x) {
  int idx[16];
  double sc[16];
  int k = 0;
  auto A = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i) {
    double c1 = 0.0;
    for (int j = 0; j < n; ++j) c1 = std::fmax(c1, std::fabs(A(i, j)));
    sc[i] = c1;
  }
  for (int j = 0; j < n - 1; ++j) {
    double best = 0.0;
    for (int i = j; i < n; ++i) {
      const double r = std::fabs(A(idx[i], j)) / sc[idx[i]];
      if (r > best) {
        best = r;
        k = i;
      }
    }
    std::swap(idx[j], idx[k]);
    for (int i = j + 1; i < n; ++i) {
      const double f = A(idx[i], j) / A(idx[j], j);
      A(idx[i], j) = f;
      for (int kk = j + 1; kk < n; ++kk) A(idx[i], kk) = A(idx[i], kk) - f * A(idx[j], kk);
    }
  }
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j) b[idx[j]] = b[idx[j]] - A(idx[j], i) * b[idx[i]];
  x[n - 1] = b[idx[n - 1]] / A(idx[n - 1], n - 1);
  for (int i = n - 2; i >= 0; --i) {
    double v = b[idx[i]];
    for (int j = i + 1; j < n; ++j) v = v - A(idx[i], j) * x[j];
    x[i] = v / A(idx[i], i);
  }
}

// coefficients[slot][xyz] of cell c (original numbering, 0-based)
void reconstruct_cell(const tmc_mesh_desc& d, double radius, int c, const std::vector<double>& en, double out[][3]) {
  const int n = d.nEdgesOnCell[c], N = n + 2;
  const double cc[3] = {d.xCell[c] * radius, d.yCell[c] * radius, d.zCell[c] * radius};
  double loc[16][3], nrm[16][3];
  for (int i = 0; i < n; ++i) {
    const int e = d.edgesOnCell[(size_t)c * d.maxEdges + i] - 1;
    loc[i][0] = d.xEdge[e] * radius;
    loc[i][1] = d.yEdge[e] * radius;
    loc[i][2] = d.zEdge[e] * radius;
    for (int k = 0; k < 3; ++k) nrm[i][k] = en[(size_t)3 * e + k];
  }
  double alpha = 0.0;
  for (int i = 0; i < n; ++i) {
    const double d0 = cc[0] - loc[i][0], d1 = cc[1] - loc[i][1], d2 = cc[2] - loc[i][2];
    alpha = alpha + std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
  }
  alpha = alpha / n;
  double rh[3] = {cc[0], cc[1], cc[2]};
  unit3(rh);
  const double* n1 = &en[(size_t)3 * (d.edgesOnCell[(size_t)c * d.maxEdges] - 1)];
  const double ndr = n1[0] * rh[0] + n1[1] * rh[1] + n1[2] * rh[2];
  double xh[3] = {n1[0] - ndr * rh[0], n1[1] - ndr * rh[1], n1[2] - ndr * rh[2]};
  unit3(xh);
  double yh[3] = {rh[1] * xh[2] - rh[2] * xh[1], rh[2] * xh[0] - rh[0] * xh[2], rh[0] * xh[1] - rh[1] * xh[0]};
  unit3(yh);
  const double* pb[2] = {xh, yh};
  double ps[16][2], pu[16][2], pd[2];
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 2; ++k) {
      ps[i][k] = loc[i][0] * pb[k][0] + loc[i][1] * pb[k][1] + loc[i][2] * pb[k][2];
      pu[i][k] = nrm[i][0] * pb[k][0] + nrm[i][1] * pb[k][1] + nrm[i][2] * pb[k][2];
    }
  for (int k = 0; k < 2; ++k) pd[k] = cc[0] * pb[k][0] + cc[1] * pb[k][1] + cc[2] * pb[k][2];
  double m1[16 * 16] = {}, m2[16 * 16], rhs[2][16] = {}, x[2][16];
  const double a2 = alpha * alpha;
  for (int j = 0; j < n; ++j)
    for (int i = j; i < n; ++i) {
      const double d0 = ps[i][0] - ps[j][0], d1 = ps[i][1] - ps[j][1];
      const double v = rbf_imq((d0 * d0 + d1 * d1) / a2) * (pu[i][0] * pu[j][0] + pu[i][1] * pu[j][1]);
      m1[(size_t)j * N + i] = v;
      m1[(size_t)i * N + j] = v;
    }
  for (int j = 0; j < n; ++j) {
    const double d0 = pd[0] - ps[j][0], d1 = pd[1] - ps[j][1];
    const double r = rbf_imq((d0 * d0 + d1 * d1) / a2);
    rhs[0][j] = r * pu[j][0];
    rhs[1][j] = r * pu[j][1];
  }
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 2; ++k) {
      m1[(size_t)(n + k) * N + i] = pu[i][k];
      m1[(size_t)i * N + (n + k)] = pu[i][k];
    }
  rhs[0][n] = 1.0;
  rhs[1][n + 1] = 1.0;
  std::memcpy(m2, m1, sizeof(double) * N * N);
  pivot_solve(m1, N, rhs[0], x[0]);
  pivot_solve(m2, N, rhs[1], x[1]);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) out[i][k] = pb[0][k] * x[0][i] + pb[1][k] * x[1][i];
}

void build_reconstruct(const tmc_mesh_desc& d, double radius, HostMesh& hm) {
  const int nc = d.nCells, ne = d.nEdges, me = hm.me;
  // edge normals, cell 1 -> cell 2 (mpas_vector_operations.F90:515-540)
  std::vector<double> en((size_t)3 * ne);
  for (int e = 0; e < ne; ++e) {
    const int c1 = d.cellsOnEdge[(size_t)e * 2] - 1, c2 = d.cellsOnEdge[(size_t)e * 2 + 1] - 1;
    double* v = &en[(size_t)3 * e];
    v[0] = d.xCell[c2] * radius - d.xCell[c1] * radius;
    v[1] = d.yCell[c2] * radius - d.yCell[c1] * radius;
    v[2] = d.zCell[c2] * radius - d.zCell[c1] * radius;
    unit3(v);
  }
  hm.recon.assign((size_t)3 * me * nc, 0.0);
  hm.cell_trig.assign((size_t)4 * nc, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int co = 0; co < nc; ++co) {
    double out[16][3];
    reconstruct_cell(d, radius, co, en, out);
    const int cn = hm.cell_o2n[co];
    for (int i = 0; i < d.nEdgesOnCell[co]; ++i)
      for (int k = 0; k < 3; ++k) hm.recon[((size_t)k * me + i) * nc + cn] = out[i][k];
    hm.cell_trig[cn] = std::cos(d.latCell[co]);
    hm.cell_trig[(size_t)nc + cn] = std::sin(d.latCell[co]);
    hm.cell_trig[(size_t)2 * nc + cn] = std::cos(d.lonCell[co]);
    hm.cell_trig[(size_t)3 * nc + cn] = std::sin(d.lonCell[co]);
  }
}

}  // namespace

bool prepare_mesh(const tmc_mesh_desc& d, const tmc_params& p, const PrepOptions& opt, HostMesh& hm) {
  const int nc = d.nCells, ne = d.nEdges, nv = d.nVertices, me = d.maxEdges, me2 = d.maxEdges2,
            vd = d.vertexDegree;
  if (nc <= 0 || ne <= 0 || nv <= 0 || me <= 0 || me2 <= 0 || vd != 3 || me > 64 || me2 > 64) {
    hm.err = "invalid mesh dimensions (vertexDegree must be 3)";
    return false;
  }
  const void* req[] = {d.nEdgesOnCell, d.nEdgesOnEdge, d.edgesOnCell, d.cellsOnEdge, d.verticesOnEdge,
                       d.edgesOnEdge, d.cellsOnVertex, d.edgesOnVertex, d.xCell, d.yCell, d.zCell,
                       d.xEdge, d.yEdge, d.zEdge, d.xVertex, d.yVertex, d.zVertex, d.latVertex,
                       d.dvEdge, d.dcEdge, d.areaCell, d.areaTriangle, d.kiteAreasOnVertex, d.weightsOnEdge};
  for (const void* q : req)
    if (!q) {
      hm.err = "tmc_mesh_desc has a NULL required array";
      return false;
    }
  if ((opt.cell_fit || opt.vertex_fit) && (!d.cellsOnCell || !d.verticesOnCell)) {
    hm.err = "stencil tables need cellsOnCell and verticesOnCell";
    return false;
  }
  // index validation (a bad index would otherwise reach the device)
  for (int c = 0; c < nc; ++c) {
    int n = d.nEdgesOnCell[c];
    if (n < 3 || n > me) {
      hm.err = "nEdgesOnCell out of range";
      return false;
    }
    for (int i = 0; i < n; ++i) {
      int e = d.edgesOnCell[(size_t)c * me + i];
      if (e < 1 || e > ne) {
        hm.err = "edgesOnCell index out of range";
        return false;
      }
      if (d.cellsOnCell) {
        int g = d.cellsOnCell[(size_t)c * me + i];
        if (g < 1 || g > nc) {
          hm.err = "cellsOnCell index out of range";
          return false;
        }
      }
      if (d.verticesOnCell) {
        int g = d.verticesOnCell[(size_t)c * me + i];
        if (g < 1 || g > nv) {
          hm.err = "verticesOnCell index out of range";
          return false;
        }
      }
    }
  }
  for (int e = 0; e < ne; ++e) {
    for (int s = 0; s < 2; ++s) {
      int c = d.cellsOnEdge[(size_t)e * 2 + s], v = d.verticesOnEdge[(size_t)e * 2 + s];
      if (c < 1 || c > nc || v < 1 || v > nv) {
        hm.err = "cellsOnEdge/verticesOnEdge index out of range";
        return false;
      }
    }
    int n = d.nEdgesOnEdge[e];
    if (n < 0 || n > me2) {
      hm.err = "nEdgesOnEdge out of range";
      return false;
    }
    for (int i = 0; i < n; ++i) {
      int g = d.edgesOnEdge[(size_t)e * me2 + i];
      if (g < 1 || g > ne) {
        hm.err = "edgesOnEdge index out of range";
        return false;
      }
    }
  }
  for (int v = 0; v < nv; ++v)
    for (int i = 0; i < vd; ++i) {
      int c = d.cellsOnVertex[(size_t)v * vd + i], e = d.edgesOnVertex[(size_t)v * vd + i];
      if (c < 1 || c > nc || e < 1 || e > ne) {
        hm.err = "cellsOnVertex/edgesOnVertex index out of range";
        return false;
      }
    }

  hm.nc = nc;
  hm.ne = ne;
  hm.nv = nv;
  const int meD = std::max(me, opt.min_me), me2D = std::max(me2, opt.min_me2);  // device slot counts
  hm.me = meD;
  hm.me2 = me2D;
  hm.vd = vd;
  const double radius = p.radius, omega = p.omega;
  hm.radius = radius;

  // ---- mesh_init derivations in the original order (mesh_mod.F90:169-224) ----
  std::vector<double> areaEdge(ne), fV(nv), dv(ne), dc(ne), aC(nc), aT(nv), kite((size_t)nv * vd);
  std::vector<int8_t> nsign((size_t)nc * me, 0), tsign((size_t)nv * vd, 0);
  std::vector<int32_t> vov((size_t)nv * vd, 0);
  for (int e = 0; e < ne; ++e) areaEdge[e] = d.dvEdge[e] * d.dcEdge[e];
  for (int v = 0; v < nv; ++v) fV[v] = 2.0 * omega * std::sin(d.latVertex[v]);
  for (int c = 0; c < nc; ++c)
    for (int i = 0; i < d.nEdgesOnCell[c]; ++i) {
      int e = d.edgesOnCell[(size_t)c * me + i] - 1;
      if (c == d.cellsOnEdge[(size_t)e * 2] - 1) nsign[(size_t)c * me + i] = 1;
      if (c == d.cellsOnEdge[(size_t)e * 2 + 1] - 1) nsign[(size_t)c * me + i] = -1;
    }
  for (int v = 0; v < nv; ++v)
    for (int i = 0; i < vd; ++i) {
      int e = d.edgesOnVertex[(size_t)v * vd + i] - 1;
      if (v == d.verticesOnEdge[(size_t)e * 2] - 1) {
        tsign[(size_t)v * vd + i] = 1;
        vov[(size_t)v * vd + i] = d.verticesOnEdge[(size_t)e * 2 + 1] - 1;
      }
      if (v == d.verticesOnEdge[(size_t)e * 2 + 1] - 1) {
        tsign[(size_t)v * vd + i] = -1;
        vov[(size_t)v * vd + i] = d.verticesOnEdge[(size_t)e * 2] - 1;
      }
    }
  const double r2 = radius * radius;
  std::vector<double> Xc(nc), Yc(nc), Zc(nc), Xv(nv), Yv(nv), Zv(nv);
  for (int c = 0; c < nc; ++c) {
    Xc[c] = d.xCell[c] * radius;
    Yc[c] = d.yCell[c] * radius;
    Zc[c] = d.zCell[c] * radius;
    aC[c] = d.areaCell[c] * r2;
  }
  for (int v = 0; v < nv; ++v) {
    Xv[v] = d.xVertex[v] * radius;
    Yv[v] = d.yVertex[v] * radius;
    Zv[v] = d.zVertex[v] * radius;
    aT[v] = d.areaTriangle[v] * r2;
  }
  for (int e = 0; e < ne; ++e) {
    dv[e] = d.dvEdge[e] * radius;
    dc[e] = d.dcEdge[e] * radius;
    areaEdge[e] = areaEdge[e] * r2;
  }
  for (size_t k = 0; k < (size_t)nv * vd; ++k) kite[k] = d.kiteAreasOnVertex[k] * r2;
  double s = 0.0;
  for (int c = 0; c < nc; ++c) s = s + aC[c];
  hm.totalArea = s;
  s = 0.0;
  for (int v = 0; v < nv; ++v) s = s + aT[v];
  hm.sumAreaTriangle = s;

  // ---- stencil tables in the original numbering ----
  FitTables F;
  if (opt.cell_fit || opt.vertex_fit)
    poly_fit(d, nc, ne, nv, me, vd, radius, Xc, Yc, Zc, Xv, Yv, Zv, vov, opt.cell_fit, opt.vertex_fit, F);

  // ---- renumbering ----
  hm.cell_n2o = sfc_order(nc, d.xCell, d.yCell, d.zCell, opt.renumber);
  hm.edge_n2o = sfc_order(ne, d.xEdge, d.yEdge, d.zEdge, opt.renumber);
  hm.vert_n2o = sfc_order(nv, d.xVertex, d.yVertex, d.zVertex, opt.renumber);
  hm.cell_o2n.assign(nc, 0);
  hm.edge_o2n.assign(ne, 0);
  hm.vert_o2n.assign(nv, 0);
  for (int i = 0; i < nc; ++i) hm.cell_o2n[hm.cell_n2o[i]] = i;
  for (int i = 0; i < ne; ++i) hm.edge_o2n[hm.edge_n2o[i]] = i;
  for (int i = 0; i < nv; ++i) hm.vert_o2n[hm.vert_n2o[i]] = i;
  const auto& co2n = hm.cell_o2n;
  const auto& eo2n = hm.edge_o2n;
  const auto& vo2n = hm.vert_o2n;

  // ---- device layout (slot-major SoA) ----
  hm.nEdgesOnCell.assign(nc, 0);
  hm.edgesOnCell.assign((size_t)meD * nc, 0);
  hm.nSignEdge.assign((size_t)meD * nc, 0);
  hm.cellsOnCell.assign((size_t)meD * nc, 0);
  hm.areaCell.assign(nc, 0.0);
  for (int cn = 0; cn < nc; ++cn) {
    int co = hm.cell_n2o[cn];
    int n = d.nEdgesOnCell[co];
    hm.nEdgesOnCell[cn] = (uint8_t)n;
    hm.areaCell[cn] = aC[co];
    for (int i = 0; i < meD; ++i) {
      int e = (i < n) ? d.edgesOnCell[(size_t)co * me + i] - 1 : -1;
      hm.edgesOnCell[(size_t)i * nc + cn] = (e >= 0) ? eo2n[e] : 0;
      hm.nSignEdge[(size_t)i * nc + cn] = (i < n) ? nsign[(size_t)co * me + i] : 0;
      int other = 0;
      if (e >= 0) {
        const int a = d.cellsOnEdge[(size_t)e * 2] - 1, b = d.cellsOnEdge[(size_t)e * 2 + 1] - 1;
        other = co2n[(a == co) ? b : a];
      }
      hm.cellsOnCell[(size_t)i * nc + cn] = other;
    }
  }
  hm.cellsOnEdge.assign((size_t)2 * ne, 0);
  hm.verticesOnEdge.assign((size_t)2 * ne, 0);
  hm.nEdgesOnEdge.assign(ne, 0);
  hm.edgesOnEdge.assign((size_t)me2D * ne, 0);
  hm.weightsOnEdge.assign((size_t)me2D * ne, 0.0);
  hm.dcEdge.assign(ne, 0.0);
  hm.dvEdge.assign(ne, 0.0);
  hm.areaEdge.assign(ne, 0.0);
  for (int en = 0; en < ne; ++en) {
    int eo = hm.edge_n2o[en];
    for (int sd = 0; sd < 2; ++sd) {
      hm.cellsOnEdge[(size_t)sd * ne + en] = co2n[d.cellsOnEdge[(size_t)eo * 2 + sd] - 1];
      hm.verticesOnEdge[(size_t)sd * ne + en] = vo2n[d.verticesOnEdge[(size_t)eo * 2 + sd] - 1];
    }
    int n = d.nEdgesOnEdge[eo];
    hm.nEdgesOnEdge[en] = (uint8_t)n;
    for (int i = 0; i < me2D; ++i) {
      if (i < n) {
        hm.edgesOnEdge[(size_t)i * ne + en] = eo2n[d.edgesOnEdge[(size_t)eo * me2 + i] - 1];
        hm.weightsOnEdge[(size_t)i * ne + en] = d.weightsOnEdge[(size_t)eo * me2 + i];
      } else {
        hm.edgesOnEdge[(size_t)i * ne + en] = en;  // harmless in-range pad
        hm.weightsOnEdge[(size_t)i * ne + en] = 0.0;
      }
    }
    hm.dcEdge[en] = dc[eo];
    hm.dvEdge[en] = dv[eo];
    hm.areaEdge[en] = areaEdge[eo];
  }
  hm.cellsOnVertex.assign((size_t)vd * nv, 0);
  hm.edgesOnVertex.assign((size_t)vd * nv, 0);
  hm.tSignEdge.assign((size_t)vd * nv, 0);
  hm.kite.assign((size_t)vd * nv, 0.0);
  hm.areaTriangle.assign(nv, 0.0);
  hm.fVertex.assign(nv, 0.0);
  hm.latVertex.assign(nv, 0.0);
  if (d.lonVertex) hm.lonVertex.assign(nv, 0.0);
  for (int vn = 0; vn < nv; ++vn) {
    int vo = hm.vert_n2o[vn];
    hm.latVertex[vn] = d.latVertex[vo];
    if (d.lonVertex) hm.lonVertex[vn] = d.lonVertex[vo];
    for (int i = 0; i < vd; ++i) {
      hm.cellsOnVertex[(size_t)i * nv + vn] = co2n[d.cellsOnVertex[(size_t)vo * vd + i] - 1];
      hm.edgesOnVertex[(size_t)i * nv + vn] = eo2n[d.edgesOnVertex[(size_t)vo * vd + i] - 1];
      hm.tSignEdge[(size_t)i * nv + vn] = tsign[(size_t)vo * vd + i];
      hm.kite[(size_t)i * nv + vn] = kite[(size_t)vo * vd + i];
    }
    hm.areaTriangle[vn] = aT[vo];
    hm.fVertex[vn] = fV[vo];
  }
  // v2c: contributions to each cell in ascending original vertex order
  {
    std::vector<int32_t> cnt(nc, 0);
    for (int vo = 0; vo < nv; ++vo)
      for (int i = 0; i < vd; ++i) cnt[co2n[d.cellsOnVertex[(size_t)vo * vd + i] - 1]]++;
    hm.v2c_start.assign(nc + 1, 0);
    for (int c = 0; c < nc; ++c) hm.v2c_start[c + 1] = hm.v2c_start[c] + cnt[c];
    hm.v2c_vertex.assign(hm.v2c_start[nc], 0);
    hm.v2c_kite.assign(hm.v2c_start[nc], 0.0);
    std::vector<int32_t> fill(nc, 0);
    for (int vo = 0; vo < nv; ++vo)  // ascending original vertex index
      for (int i = 0; i < vd; ++i) {
        int cn = co2n[d.cellsOnVertex[(size_t)vo * vd + i] - 1];
        int k = hm.v2c_start[cn] + fill[cn]++;
        hm.v2c_vertex[k] = vo2n[vo];
        hm.v2c_kite[k] = kite[(size_t)vo * vd + i];
      }
  }
  // upwind stencils
  if (opt.cell_fit) {
    std::vector<int32_t> ctr((size_t)ne * 2);
    for (int e = 0; e < ne; ++e)
      for (int sd = 0; sd < 2; ++sd) ctr[(size_t)e * 2 + sd] = d.cellsOnEdge[(size_t)e * 2 + sd] - 1;
    compact(F.nfit2c, F.fit2c, F.d2c, ctr, co2n, hm.edge_n2o, ne, hm.cell2);
    compact(F.nfit4c, F.fit4c, F.d3c, ctr, co2n, hm.edge_n2o, ne, hm.cell3);
    compact(F.nfit4c, F.fit4c, F.d4c, ctr, co2n, hm.edge_n2o, ne, hm.cell4);
  }
  if (opt.vertex_fit) {
    std::vector<int32_t> ctr((size_t)ne * 2);
    for (int e = 0; e < ne; ++e)
      for (int sd = 0; sd < 2; ++sd) ctr[(size_t)e * 2 + sd] = d.verticesOnEdge[(size_t)e * 2 + sd] - 1;
    compact(F.nfit2v, F.fit2v, F.d2v, ctr, vo2n, hm.edge_n2o, ne, hm.vert2);
    compact(F.nfit4v, F.fit4v, F.d4v, ctr, vo2n, hm.edge_n2o, ne, hm.vert4);
  }
  // the cell-centre wind of the history output (needs lonCell and the edge positions)
  if (d.lonCell && d.latCell && d.xEdge && d.yEdge && d.zEdge && d.maxEdges <= 14)
    build_reconstruct(d, p.radius, hm);
  return true;
}

}  // namespace tmc

// Host side of the GB300 pizza time step: configuration, radial grid and
// Chebyshev operators, device pool layout and the C ABI of pizza_gpu.h.
//
// What runs here is set-up work of pizza's init sequence (src/pizza.f90:64-199):
// read_namelists' derived switches (src/namelists.f90:271-526), the
// Gauss-Lobatto grid and collocation matrices (src/chebyshev.f90:222-383),
// the radial functions (src/radial.f90:115-282) and the integration weights
// (src/integration.f90).  Everything per time step runs on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <tuple>
#include <string>
#include <vector>

#include "pizza_gpu.h"
#include "pz_fast_setup.h"
#include "pz_handle.h"
#include "pz_internal.h"
#include "pz_stage.h"

namespace {

thread_local std::string g_create_error = "no error";



}  // namespace



namespace {

int fail(pz_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}

int cuda_fail(pz_handle* h, cudaError_t e, const char* what);
}  // namespace
int pz_fail(pz_handle* h, int code, const std::string& msg) { return fail(h, code, msg); }
namespace {
int cuda_fail(pz_handle* h, cudaError_t e, const char* what) {
  return fail(h, PZ_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// -------------------------------------------------------------------------
// Chebyshev operators for N Gauss-Lobatto points (chebyshev.f90:222-383,
// dct_fftw.f90:46-397).  All column-major N x N.
// -------------------------------------------------------------------------
struct Basis {
  int N;
  std::vector<double> x, C, D1c, D2c, D1p, D2p, rMat, drMat, d2rMat;
  std::vector<double> Cs, D1cs, D2cs, D1ps, D2ps;   // parity-compact forms
  std::vector<double> CTs, D1cTs, D2cTs, D1pTs;     // ... of the transposes
  std::vector<double> Cos;                          // C in the out-sym layout
};

// Parity-compact operators (see BM_CS..BM_D2PS in pz_internal.h).  The
// Gauss-Lobatto grid is symmetric, x_{N-1-i} = -x_i, so
//   C(k, N-1-j)      = (-1)^k C(k, j),
//   D1c(N-1-i, k)    = (-1)^(k+1) D1c(i, k),   D2c(N-1-i, k) = (-1)^k D2c(i, k),
//   D1p(N-1-i,N-1-j) = -D1p(i, j),             D2p(N-1-i,N-1-j) = D2p(i, j),
// and each product needs about half the multiply-adds of the dense form.
// in-sym: column j < h2 of M (N x N), N x h2
static std::vector<double> compact_in(const std::vector<double>& M, int N) {
  const int h2 = (N + 1) / 2;
  std::vector<double> out((size_t)N * h2, 0.0);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < h2; ++j) out[k + (size_t)j * N] = M[k + (size_t)j * N];
  return out;
}
// out-sym: rows 2i (even columns of row i) and 2i+1 (odd columns), 2*h2 x h2
static std::vector<double> compact_out(const std::vector<double>& M, int N) {
  const int h2 = (N + 1) / 2, R = 2 * h2;
  std::vector<double> out((size_t)R * h2, 0.0);
  for (int i = 0; i < h2; ++i)
    for (int kk = 0; kk < h2; ++kk) {
      out[(2 * i) + (size_t)kk * R] = M[i + (size_t)(2 * kk) * N];
      if (2 * kk + 1 < N) out[(2 * i + 1) + (size_t)kk * R] = M[i + (size_t)(2 * kk + 1) * N];
    }
  return out;
}
// centro: rows 2i = (M(i,j)+M(i,N-1-j))/2 (and the middle column), 2i+1 = (M(i,j)-M(i,N-1-j))/2
static std::vector<double> compact_centro(const std::vector<double>& M, int N) {
  const int h = N / 2, h2 = (N + 1) / 2, R = 2 * h2;
  std::vector<double> out((size_t)R * h2, 0.0);
  for (int i = 0; i < h2; ++i) {
    for (int j = 0; j < h; ++j) {
      out[(2 * i) + (size_t)j * R] = 0.5 * (M[i + (size_t)j * N] + M[i + (size_t)(N - 1 - j) * N]);
      out[(2 * i + 1) + (size_t)j * R] = 0.5 * (M[i + (size_t)j * N] - M[i + (size_t)(N - 1 - j) * N]);
    }
    if (N % 2 == 1) out[(2 * i) + (size_t)h * R] = M[i + (size_t)h * N];
  }
  return out;
}
static std::vector<double> transpose(const std::vector<double>& M, int N) {
  std::vector<double> T((size_t)N * N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) T[j + (size_t)i * N] = M[i + (size_t)j * N];
  return T;
}
void make_compact(Basis& b) {
  const int N = b.N;
  b.Cs = compact_in(b.C, N);
  b.D1cs = compact_out(b.D1c, N);
  b.D2cs = compact_out(b.D2c, N);
  b.D1ps = compact_centro(b.D1p, N);
  b.D2ps = compact_centro(b.D2p, N);
  b.CTs = compact_out(transpose(b.C, N), N);
  b.D1cTs = compact_in(transpose(b.D1c, N), N);
  b.D2cTs = compact_in(transpose(b.D2c, N), N);
  b.D1pTs = compact_centro(transpose(b.D1p, N), N);
  b.Cos = compact_out(b.C, N);   // C(N-1-i, k) = (-1)^k C(i, k)
}

Basis make_basis(int N, double r_icb, double r_cmb) {
  Basis b;
  b.N = N;
  const long double pi = 3.141592653589793238462643383279502884L;
  b.x.resize(N);
  for (int k = 0; k < N; ++k) b.x[k] = (double)cosl(pi * (long double)k / (long double)(N - 1));
  const double drx = 2.0 / (r_cmb - r_icb), ddrx = 0.0;
  // recursion over the polynomial degree (get_der_mat), stored as (grid i, degree n)
  std::vector<double> rM(N * N), drM(N * N), d2rM(N * N);
  auto at = [N](std::vector<double>& A, int i, int n) -> double& { return A[i + (size_t)n * N]; };
  for (int i = 0; i < N; ++i) {
    at(rM, i, 0) = 1.0; at(rM, i, 1) = b.x[i];
    at(drM, i, 0) = 0.0; at(drM, i, 1) = drx;
    at(d2rM, i, 0) = 0.0; at(d2rM, i, 1) = ddrx;
    for (int n = 2; n < N; ++n) {
      at(rM, i, n) = 2.0 * b.x[i] * at(rM, i, n - 1) - at(rM, i, n - 2);
      at(drM, i, n) = 2.0 * drx * at(rM, i, n - 1) + 2.0 * b.x[i] * at(drM, i, n - 1) - at(drM, i, n - 2);
      at(d2rM, i, n) = 2.0 * ddrx * at(rM, i, n - 1) + 4.0 * drx * at(drM, i, n - 1) +
                       2.0 * b.x[i] * at(d2rM, i, n - 1) - at(d2rM, i, n - 2);
    }
  }
  b.rMat = rM; b.drMat = drM; b.d2rMat = d2rM;
  const double rnorm = std::sqrt(2.0 / (double)(N - 1));
  const double cheb_fac = std::sqrt(0.5 / (double)(N - 1));
  // costf1 as a matrix: out_k = cheb_fac * sum_j w_j cos(pi j k/(N-1)) f_j
  b.C.assign((size_t)N * N, 0.0);
  const long long L = 2LL * (N - 1);
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j) {
      const long long q = ((long long)j * k) % L;
      const double cs = (double)cosl(pi * (long double)q / (long double)(N - 1));
      const double w = (j == 0 || j == N - 1) ? 1.0 : 2.0;
      b.C[k + (size_t)j * N] = cheb_fac * w * cs;
    }
  // Chebyshev -> physical derivatives: rnorm * bfac_k * T_k^(p)(x_i)
  b.D1c.resize((size_t)N * N);
  b.D2c.resize((size_t)N * N);
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < N; ++k) {
      const double bf = (k == 0 || k == N - 1) ? 0.5 : 1.0;
      b.D1c[i + (size_t)k * N] = rnorm * bf * at(drM, i, k);
      b.D2c[i + (size_t)k * N] = rnorm * bf * at(d2rM, i, k);
    }
  // physical -> physical: D = Dc * C (accumulated in long double)
  auto matmul = [N](const std::vector<double>& A, const std::vector<double>& B) {
    std::vector<double> R((size_t)N * N);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        long double s = 0.0L;
        for (int k = 0; k < N; ++k) s += (long double)A[i + (size_t)k * N] * (long double)B[k + (size_t)j * N];
        R[i + (size_t)j * N] = (double)s;
      }
    return R;
  };
  b.D1p = matmul(b.D1c, b.C);
  b.D2p = matmul(b.D2c, b.C);
  make_compact(b);
  return b;
}

bool factor_fft(int P, int* radix, int* nrad) {
  int n = P, k = 0;
  while (n % 4 == 0) { if (k >= PZ_MAX_RADIX) return false; radix[k++] = 4; n /= 4; }
  while (n % 2 == 0) { if (k >= PZ_MAX_RADIX) return false; radix[k++] = 2; n /= 2; }
  const int odd[3] = {3, 5, 7};
  for (int t = 0; t < 3; ++t)
    while (n % odd[t] == 0) { if (k >= PZ_MAX_RADIX) return false; radix[k++] = odd[t]; n /= odd[t]; }
  *nrad = k;
  return n == 1;
}

// DIRK tableau (dirk_schemes.f90:35-244 for the stage counts and flags,
// :246-707 for the coefficients): unscaled Butcher matrices of size sizet
// (nstages+1, or nstages with an assembly stage), the assembly rows, the
// diagonal weight gamma, per-stage l_exp_calc / l_imp_calc_rhs bits and the
// default courfac.
struct DirkTab {
  int nstages = 0, assembly = 0, sizet = 0, exp_mask = 0, imp_mask = 0;
  double gamma = 0.0, courfac = 0.0;
  double bimp[PZ_BT_LD][PZ_BT_LD] = {}, bexp[PZ_BT_LD][PZ_BT_LD] = {};
  double bai[PZ_BT_LD] = {}, bae[PZ_BT_LD] = {};
};
bool dirk_tableau(int scheme, DirkTab* t) {
  const double r2 = std::sqrt(2.0), r3 = std::sqrt(3.0);
  bool imp1 = false;
  auto rows = [&](std::initializer_list<std::initializer_list<double>> bi,
                  std::initializer_list<std::initializer_list<double>> be) {
    int i = 0;
    for (auto& r : bi) { int j = 0; for (double v : r) t->bimp[i][j++] = v; ++i; }
    t->sizet = i;
    i = 0;
    for (auto& r : be) { int j = 0; for (double v : r) t->bexp[i][j++] = v; ++i; }
  };
  auto ass = [&](std::initializer_list<double> a) {
    int j = 0;
    for (double v : a) { t->bai[j] = v; t->bae[j] = v; ++j; }
  };
  double g, d;
  switch (scheme) {
    case PZ_ARS222:
      g = 0.5 * (2.0 - r2); d = 1.0 - 0.5 / g;
      t->nstages = 2; t->assembly = 0; t->courfac = 1.35;
      rows({{0, 0, 0}, {0, g, 0}, {0, 1 - g, g}}, {{0, 0, 0}, {g, 0, 0}, {d, 1 - d, 0}});
      break;
    case PZ_ARS232:
      g = 0.5 * (2.0 - r2); d = -2.0 * r2 / 3.0;
      t->nstages = 3; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0}, {0, g, 0}, {0, 1 - g, g}}, {{0, 0, 0}, {g, 0, 0}, {d, 1 - d, 0}});
      ass({0, 1 - g, g});
      break;
    case PZ_ARS233:
      g = (3.0 + r3) / 6.0;
      t->nstages = 3; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0}, {0, g, 0}, {0, 1 - 2 * g, g}}, {{0, 0, 0}, {g, 0, 0}, {g - 1, 2 * (1 - g), 0}});
      ass({0, 0.5, 0.5});
      break;
    case PZ_SSP222:
      g = 1.0 - 1.0 / r2;
      t->nstages = 3; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0}, {0, g, 0}, {0, 1 - 2 * g, g}}, {{0, 0, 0}, {0, 0, 0}, {0, 1, 0}});
      ass({0, 0.5, 0.5});
      break;
    case PZ_LSDIRK222:
      g = 1.0 - 1.0 / r2; d = 1.0 / (2.0 * g);
      t->nstages = 3; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0}, {0, g, 0}, {0, 1 - g, g}}, {{0, 0, 0}, {0, 0, 0}, {0, d, 0}});
      ass({0, 1 - g, g});
      break;
    case PZ_LZ232:
      g = 0.5; imp1 = true;
      t->nstages = 2; t->assembly = 0; t->courfac = 1.25;
      rows({{0, 0, 0}, {-0.25, 0.5, 0}, {0.5, 0, 0.5}}, {{0, 0, 0}, {0.25, 0, 0}, {-1, 2, 0}});
      break;
    case PZ_CK232:
      g = 1.0 - 0.5 * r2; imp1 = true;
      t->nstages = 2; t->assembly = 0; t->courfac = 1.25;
      rows({{0, 0, 0}, {-1.0 / 3.0 + 0.5 * r2, g, 0}, {0.75 - 0.25 * r2, -0.75 + 0.75 * r2, g}},
           {{0, 0, 0}, {2.0 / 3.0, 0, 0}, {0.25, 0.75, 0}});
      break;
    case PZ_ARS443:
      g = 0.5;
      t->nstages = 4; t->assembly = 0; t->courfac = 0.9;
      rows({{0, 0, 0, 0, 0}, {0, 0.5, 0, 0, 0}, {0, 1.0 / 6.0, 0.5, 0, 0}, {0, -0.5, 0.5, 0.5, 0},
            {0, 1.5, -1.5, 0.5, 0.5}},
           {{0, 0, 0, 0, 0}, {0.5, 0, 0, 0, 0}, {11.0 / 18.0, 1.0 / 18.0, 0, 0, 0},
            {5.0 / 6.0, -5.0 / 6.0, 0.5, 0, 0}, {0.25, 1.75, 0.75, -1.75, 0}});
      break;
    case PZ_BPR353:
      g = 0.5; imp1 = true;
      t->nstages = 4; t->assembly = 0; t->courfac = 1.0;
      rows({{0, 0, 0, 0, 0}, {0.5, 0.5, 0, 0, 0}, {5.0 / 18.0, -1.0 / 9.0, 0.5, 0, 0}, {0.5, 0, 0, 0.5, 0},
            {0.25, 0, 0.75, -0.5, 0.5}},
           {{0, 0, 0, 0, 0}, {1, 0, 0, 0, 0}, {4.0 / 9.0, 2.0 / 9.0, 0, 0, 0}, {0.25, 0, 0.75, 0, 0},
            {0.25, 0, 0.75, 0, 0}});
      t->exp_mask = 0x7;   // no explicit terms at stage 4
      break;
    case PZ_PC2:
      g = 0.5; imp1 = true;
      t->nstages = 3; t->assembly = 0; t->courfac = 0.8;
      rows({{0, 0, 0, 0}, {0.5, 0.5, 0, 0}, {0.5, 0, 0.5, 0}, {0.5, 0, 0, 0.5}},
           {{0, 0, 0, 0}, {1, 0, 0, 0}, {0.5, 0.5, 0, 0}, {0.5, 0, 0.5, 0}});
      break;
    case PZ_ARS343:
    case PZ_MARS343: {
      double b1, b2;
      if (scheme == PZ_ARS343) {
        g = 0.435866521508459;
        b1 = -1.5 * g * g + 4.0 * g - 0.25;
        b2 = 1.5 * g * g - 5.0 * g + 1.25;
        t->courfac = 0.7;
        rows({{0, 0, 0, 0}, {0, g, 0, 0}, {0, 0.5 * (1 - g), g, 0}, {0, b1, b2, g}},
             {{0, 0, 0, 0}, {g, 0, 0, 0}, {0.3212788860286278, 0.3966543747256017, 0, 0},
              {-0.1058582960718797, 0.5529291480359398, 0.5529291480359398, 0}});
      } else {
        g = 0.435866521508458;
        b1 = 1.20849664917601;
        b2 = -0.64436317068446;
        t->courfac = 0.5;
        rows({{0, 0, 0, 0}, {0, g, 0, 0}, {0, 0.5 * (1 - g), g, 0}, {0, b1, b2, g}},
             {{0, 0, 0, 0}, {0.877173304301691, 0, 0, 0}, {0.535396540307354, 0.182536720446875, 0, 0},
              {0.63041255815287, -0.83193390106308, 1.20152134291021, 0}});
      }
      t->nstages = 4; t->assembly = 1;
      ass({0, b1, b2, g});
    } break;
    case PZ_SSP322:
      g = 0.5;
      t->nstages = 4; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0, 0}, {0, 0.5, 0, 0}, {0, -0.5, 0.5, 0}, {0, 0, 0.5, 0.5}},
           {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 1, 0}});
      ass({0, 0, 0.5, 0.5});
      break;
    case PZ_SSP332:
      g = 1.0 - 1.0 / r2;
      t->nstages = 4; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0, 0}, {0, g, 0, 0}, {0, 1 - 2 * g, g, 0}, {0, 0.5 - g, 0, g}},
           {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 1, 0, 0}, {0, 0.25, 0.25, 0}});
      ass({0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0});
      break;
    case PZ_SSP433: {
      // the reference writes alpha, beta and eta as default-kind (single
      // precision) literals, so they carry float rounding into the double
      // tableau; (double)<float literal> reproduces that
      const double a = (double)0.24169426078821f, b = (double)0.06042356519705f;
      const double e = (double)0.12915286960590f;
      g = a;
      t->nstages = 5; t->assembly = 1; t->courfac = 1.35;
      rows({{0, 0, 0, 0, 0}, {0, a, 0, 0, 0}, {0, -a, a, 0, 0}, {0, 0, 1 - a, a, 0}, {0, b, e, 0.5 - b - e - a, a}},
           {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 1, 0, 0}, {0, 0, 0.25, 0.25, 0}});
      ass({0, 0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0});
    } break;
    case PZ_DP1_242:
      g = 0.5;
      t->nstages = 4; t->assembly = 0; t->courfac = 1.35;
      rows({{0, 0, 0, 0, 0}, {0, 0.5, 0, 0, 0}, {0, 1.0 / 6.0, 0.5, 0, 0}, {0, -0.5, 0.5, 0.5, 0},
            {0, 1.5, -1.5, 0.5, 0.5}},
           {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 1.0 / 3.0, 0, 0, 0}, {0, 1, 0, 0, 0}, {0, 0.5, 0, 0.5, 0}});
      t->exp_mask = 0xA;   // explicit terms at stages 2 and 4 only
      break;
    case PZ_DP2_242:
      g = 1.0 / 3.0;
      t->nstages = 4; t->assembly = 0; t->courfac = 1.35;
      rows({{0, 0, 0, 0, 0}, {0, g, 0, 0, 0}, {0, -g, g, 0, 0}, {0, 0, 1 - g, g, 0}, {0, 0, 0.5, 0.5 - g, g}},
           {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 1, 0, 0}, {0, 0, 0.5, 0.5, 0}});
      t->exp_mask = 0xE;   // no explicit terms at stage 1
      break;
    case PZ_LZ453:
      g = 1.2; imp1 = true;
      t->nstages = 4; t->assembly = 0; t->courfac = 1.15;
      rows({{0, 0, 0, 0, 0}, {-44.0 / 45.0, 1.2, 0, 0, 0}, {-47.0 / 300.0, -0.71, 1.2, 0, 0},
            {3.375, -3.25, -59.0 / 120.0, 1.2, 0}, {89.0 / 50.0, -486.0 / 55.0, 8.9, -562.0 / 275.0, 1.2}},
           {{0, 0, 0, 0, 0}, {2.0 / 9.0, 0, 0, 0, 0}, {71.0 / 420.0, 23.0 / 140.0, 0, 0, 0},
            {-281.0 / 336.0, 187.0 / 112.0, 0, 0, 0}, {0.1, 0, 0.5, 0.4, 0}});
      break;
    case PZ_KC343: {
      g = 1767732205903.0 / 4055673282236.0; imp1 = true;
      t->nstages = 4; t->assembly = 1; t->courfac = 0.5;
      const double i41 = 1471266399579.0 / 7840856788654.0, i42 = -4482444167858.0 / 7529755066697.0;
      const double i43 = 11266239266428.0 / 11593286722821.0;
      rows({{0, 0, 0, 0}, {g, g, 0, 0},
            {2746238789719.0 / 10658868560708.0, -640167445237.0 / 6845629431997.0, g, 0}, {i41, i42, i43, g}},
           {{0, 0, 0, 0}, {1767732205903.0 / 2027836641118.0, 0, 0, 0},
            {5535828885825.0 / 10492691773637.0, 788022342437.0 / 10882634858940.0, 0, 0},
            {6485989280629.0 / 16251701735622.0, -4246266847089.0 / 9704473918619.0,
             10755448449292.0 / 10357097424841.0, 0}});
      ass({i41, i42, i43, g});
    } break;
    case PZ_KC564: {
      g = 0.25; imp1 = true;
      t->nstages = 6; t->assembly = 1; t->courfac = 0.5;
      const double i61 = 82889.0 / 524892.0, i63 = 15625.0 / 83664.0, i64 = 69875.0 / 102672.0;
      const double i65 = -2260.0 / 8211.0;
      rows({{0, 0, 0, 0, 0, 0}, {0.25, 0.25, 0, 0, 0, 0}, {8611.0 / 62500.0, -1743.0 / 31250.0, 0.25, 0, 0, 0},
            {5012029.0 / 34652500.0, -654441.0 / 2922500.0, 174375.0 / 388108.0, 0.25, 0, 0},
            {15267082809.0 / 155376265600.0, -71443401.0 / 120774400.0, 730878875.0 / 902184768.0,
             2285395.0 / 8070912.0, 0.25, 0},
            {i61, 0, i63, i64, i65, 0.25}},
           {{0, 0, 0, 0, 0, 0}, {0.5, 0, 0, 0, 0, 0}, {13861.0 / 62500.0, 6889.0 / 62500.0, 0, 0, 0, 0},
            {-116923316275.0 / 2393684061468.0, -2731218467317.0 / 15368042101831.0,
             9408046702089.0 / 11113171139209.0, 0, 0, 0},
            {-451086348788.0 / 2902428689909.0, -2682348792572.0 / 7519795681897.0,
             12662868775082.0 / 11960479115383.0, 3355817975965.0 / 11060851509271.0, 0, 0},
            {647845179188.0 / 3216320057751.0, 73281519250.0 / 8382639484533.0, 552539513391.0 / 3454668386233.0,
             3354512671639.0 / 8306763924573.0, 4040.0 / 17871.0, 0}});
      ass({i61, 0, i63, i64, i65, 0.25});
    } break;
    case PZ_DBM453: {
      g = 0.32591194130117247; imp1 = true;
      t->nstages = 5; t->assembly = 1; t->courfac = 0.5;
      rows({{0, 0, 0, 0, 0}, {-0.22284985318525410, g, 0, 0, 0},
            {-0.46801347074080545, 0.86349284225716961, g, 0, 0},
            {-0.46509906651927421, 0.81063103116959553, 0.61036726756832357, g, 0},
            {0.87795339639076675, -0.72692641526151547, 0.75204137157372720, -0.22898029400415088, g}},
           {{0, 0, 0, 0, 0}, {0.10306208811591838, 0, 0, 0, 0}, {-0.94124866143519894, 1.6626399742527356, 0, 0, 0},
            {-1.3670975201437765, 1.3815852911016873, 1.2673234025619065, 0, 0},
            {-0.81287582068772448, 0.81223739060505738, 0.90644429603699305, 0.094194134045674111, 0}});
      // the assembly weights are printed with their own last digits
      ass({0.87795339639076672, -0.72692641526151549, 0.7520413715737272, -0.22898029400415090,
           0.32591194130117247});
    } break;
    case PZ_KC785: {
      g = 2.0 / 9.0; imp1 = true;
      t->nstages = 8; t->assembly = 1; t->courfac = 0.5;
      const double a3 = 2366667076620.0 / 8822750406821.0, a4 = -257962897183.0 / 4451812247028.0;
      const double a5 = -486229321650.0 / 11227943450093.0, a6 = 621307788657.0 / 4714163060173.0;
      const double a7 = 2036305566805.0 / 6583108094622.0;
      const double b83 = 3517720773327.0 / 20256071687669.0, b84 = 4569610470461.0 / 17934693873752.0;
      const double b85 = 2819471173109.0 / 11655438449929.0, b86 = 3296210113763.0 / 10722700128969.0;
      const double b87 = -1142099968913.0 / 5710983926999.0;
      rows({{0, 0, 0, 0, 0, 0, 0, 0},
            {g, g, 0, 0, 0, 0, 0, 0},
            {a3, a3, g, 0, 0, 0, 0, 0},
            {a4, a4, 128530224461.0 / 14379561246022.0, g, 0, 0, 0, 0},
            {a5, a5, -225633144460.0 / 6633558740617.0, 1741320951451.0 / 6824444397158.0, g, 0, 0, 0},
            {a6, a6, -125196015625.0 / 3866852212004.0, 940440206406.0 / 7593089888465.0,
             961109811699.0 / 6734810228204.0, g, 0, 0},
            {a7, a7, -3039402635899.0 / 4450598839912.0, -1829510709469.0 / 31102090912115.0,
             -286320471013.0 / 6931253422520.0, 8651533662697.0 / 9642993110008.0, g, 0},
            {0, 0, b83, b84, b85, b86, b87, g}},
           {{0, 0, 0, 0, 0, 0, 0, 0},
            {4.0 / 9.0, 0, 0, 0, 0, 0, 0, 0},
            {1.0 / 9.0, 1183333538310.0 / 1827251437969.0, 0, 0, 0, 0, 0, 0},
            {895379019517.0 / 9750411845327.0, 477606656805.0 / 13473228687314.0,
             -112564739183.0 / 9373365219272.0, 0, 0, 0, 0, 0},
            {-4458043123994.0 / 13015289567637.0, -2500665203865.0 / 9342069639922.0,
             983347055801.0 / 8893519644487.0, 2185051477207.0 / 2551468980502.0, 0, 0, 0, 0},
            {-167316361917.0 / 17121522574472.0, 1605541814917.0 / 7619724128744.0,
             991021770328.0 / 13052792161721.0, 2342280609577.0 / 11279663441611.0,
             3012424348531.0 / 12792462456678.0, 0, 0, 0},
            {6680998715867.0 / 14310383562358.0, 5029118570809.0 / 3897454228471.0,
             2415062538259.0 / 6382199904604.0, -3924368632305.0 / 6964820224454.0,
             -4331110370267.0 / 15021686902756.0, -3944303808049.0 / 11994238218192.0, 0, 0},
            {2193717860234.0 / 3570523412979.0, 2193717860234.0 / 3570523412979.0,
             5952760925747.0 / 18750164281544.0, -4412967128996.0 / 6196664114337.0,
             4151782504231.0 / 36106512998704.0, 572599549169.0 / 6265429158920.0,
             -457874356192.0 / 11306498036315.0, 0}});
      ass({0, 0, b83, b84, b85, b86, b87, g});
    } break;
    default:
      return false;
  }
  t->gamma = g;
  if (!t->exp_mask) t->exp_mask = (1 << t->nstages) - 1;
  t->imp_mask = ((1 << t->nstages) - 1) & ~1;
  if (imp1) t->imp_mask |= 1;
  return true;
}

int scheme_counts(int scheme, int* nold, int* nimp, int* nexp, double* cf, int* imp_calc) {
  // multistep_schemes.f90:53-106; DIRK: one old slot, one explicit and one
  // implicit slot per stage (dirk_schemes.f90:35-244)
  *imp_calc = 1;
  DirkTab t;
  if (dirk_tableau(scheme, &t)) {
    *nold = 1; *nimp = t.nstages; *nexp = t.nstages; *cf = t.courfac;
    return 0;
  }
  switch (scheme) {
    case PZ_CNAB2: *nimp = 1; *nold = 1; *nexp = 2; *cf = 3.0; break;
    case PZ_MODCNAB: *nold = 2; *nimp = 2; *nexp = 2; *cf = 2.9; break;
    case PZ_CNLF: *nold = 2; *nimp = 2; *nexp = 2; *cf = 3.0; break;
    case PZ_SBDF2: *nold = 2; *nimp = 1; *nexp = 2; *cf = 2.8; *imp_calc = 0; break;
    case PZ_SBDF3: *nold = 3; *nimp = 1; *nexp = 3; *cf = 4.0; *imp_calc = 0; break;
    case PZ_TVB33: *nold = 3; *nimp = 3; *nexp = 3; *cf = 4.0; break;
    case PZ_SBDF4: *nold = 4; *nimp = 1; *nexp = 4; *cf = 5.5; *imp_calc = 0; break;
    default: return -1;
  }
  return 0;
}

// simps (integration.f90:104-152) applied to f, as a linear functional
double simps(const std::vector<double>& f, const std::vector<double>& r) {
  const int n = (int)f.size();
  double s = 0.0;
  auto seg = [&](int i) {
    const double h2 = r[i + 1] - r[i], h1 = r[i] - r[i - 1];
    return (h1 + h2) / 6.0 * (f[i - 1] * (2 * h1 - h2) / h1 + f[i] * (h1 + h2) * (h1 + h2) / (h1 * h2) +
                             f[i + 1] * (2 * h2 - h1) / h2);
  };
  if (n % 2 == 1) {
    for (int i = 1; i < n - 1; i += 2) s += seg(i);
    return -s;
  }
  s = 0.5 * (r[1] - r[0]) * (f[1] + f[0]);
  for (int i = 2; i < n - 1; i += 2) s += seg(i);
  s += 0.5 * (r[n - 1] - r[n - 2]) * (f[n - 1] + f[n - 2]);
  for (int i = 1; i < n - 1; i += 2) s += seg(i);
  return -0.5 * s;
}

int validate(const pz_config& c, std::string* why) {
  auto bad = [&](const char* m) { *why = m; return PZ_E_ARG; };
  auto uns = [&](const char* m) { *why = m; return PZ_E_UNSUPPORTED; };
  if (c.n_r_max < 5 || c.n_r_max > 128) return bad("n_r_max must be in [5, 128]");
  if (c.n_cheb_max < 2 || c.n_cheb_max > c.n_r_max) return bad("n_cheb_max must be in [2, n_r_max]");
  if (c.minc != 1) return uns("minc != 1 is not implemented");
  if (c.m_max < 2 || c.m_max > 256) return bad("m_max must be in [2, 256]");
  if (c.ra == 0.0) return uns("ra = 0 (no temperature equation) is not implemented");
  if (c.pr <= 0.0) return bad("pr must be > 0");
  if (!(c.radratio > 0.0 && c.radratio < 1.0)) return uns("radratio must be in (0, 1): the full disk is not implemented");
  if (c.ktopt != 1 || c.kbott != 1) return uns("only fixed-temperature boundaries (ktopt = kbott = 1)");
  if (c.ktopv != 2 || c.kbotv != 2) return uns("only rigid boundaries (ktopv = kbotv = 2)");
  if (c.matrix_solve != PZ_SOLVE_INFLUENCE && c.matrix_solve != PZ_SOLVE_DIRECT) return bad("unknown matrix_solve");
  if (c.cheb_method != PZ_CHEB_COLL && c.cheb_method != PZ_CHEB_INTEG) return bad("unknown cheb_method");
  if (c.time_scale != PZ_TS_VISC && c.time_scale != PZ_TS_ROT) return bad("unknown time_scale");
  if (c.l_rerror_fix && !(c.rerror_fac > 0.0)) return bad("rerror_fac must be > 0");
  if (c.l_rerror_fix && c.cheb_method != PZ_CHEB_INTEG)
    return uns("l_rerror_fix is implemented for cheb_method 'integ' (the collocation m = 0 recursions take no threshold)");
  if (c.raxi != 0.0) {
    if (!(c.sc > 0.0)) return bad("sc must be > 0 when raxi /= 0");
    if (c.ktopxi != 1 || c.kbotxi != 1) return uns("only fixed-composition boundaries (ktopxi = kbotxi = 1)");
  }
  if (c.cheb_method == PZ_CHEB_INTEG) {
    if (pz_build_smem_bytes(c.n_r_max, true, true) > PZ_SMEM_MAX)
      return uns("cheb_method 'integ' needs n_r_max <= 118 (the operator build is staged in shared memory)");
    DirkTab t;
    if (dirk_tableau(c.time_scheme, &t) && t.assembly)
      return uns("cheb_method 'integ' has no assembly stage (mloop.f90:162-164 aborts)");
  } else if (c.matrix_solve == PZ_SOLVE_DIRECT && pz_build_smem_bytes(c.n_r_max, true, false) > PZ_SMEM_MAX) {
    return uns("matrix_solve DIRECT: n_r_max too large for the operator builders");
  }
  if (c.dtMax <= 0.0) return bad("dtMax must be > 0");
  if (c.alpha <= 0.0 || c.alpha > 1.0) return bad("alpha must be in (0, 1]");
  if (c.dt_fac <= 1.0) return bad("dt_fac must be > 1");
  int a, b, d, e; double f;
  if (scheme_counts(c.time_scheme, &a, &b, &d, &f, &e) != 0) return bad("unknown time_scheme");
  int radix[PZ_MAX_RADIX], nr;
  if (!factor_fft(3 * c.m_max / c.minc, radix, &nr)) return uns("n_phi_max must factor into 2, 3, 5, 7");
  return PZ_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
// process-wide default of the tensor-core stage for handles created afterwards
int g_fast_default = 1;
int g_integ_banded = 0;   // integration method: bordered banded factors (else dense inverses)
// process-wide tuning table (pz_tune_set): k_fast instances per block, and
// k_rloop radii per block by n_phi_max; 0 = the built-in choice
int g_tune_fast_g = 0;
int g_tune_lanes = 2;
std::map<int, int> g_tune_rloop_rg;

namespace {

// Whether instance i can run its stage in k_fast: the collocation step with
// the influence-matrix solve and CNAB2 (no start-up bridge), fixed
// temperature and no-slip walls, no composition, no Chebyshev truncation,
// and n_r_max within the exact fp32 accumulation bound of the products.
bool fast_eligible(const pz_config& c, const PzInst& I) {
  return g_fast_default && c.cheb_method == PZ_CHEB_COLL && c.matrix_solve == PZ_SOLVE_INFLUENCE &&
         !(I.flags & (PZF_CHEM | PZF_DIRECT | PZF_INTEG)) && (I.flags & PZF_IMP_CALC) && !I.dirk &&
         I.scheme == PZ_CNAB2 && I.n_max == I.N && c.ktopt == 1 && c.kbott == 1 && c.ktopv == 2 &&
         c.kbotv == 2 && I.N >= 5 && I.N <= PZ_FAST_MAXN;
}

// Operators, work items and device descriptors of the fast instances;
// instances whose class set-up fails stay on the standard kernels.  Returns
// the device descriptor (n_items 0 when no instance takes the fast path).
// radial functions: rad[i] (RV_COUNT x N) of each instance.
struct FastBuild {
  PzFastHost H;
  std::vector<PzFastItem> items;
  std::vector<int> fi;
  std::vector<int> lane_item;   // items of lane l: [lane_item[l], lane_item[l + 1])
  int maxN = 0;
  int G = PZ_FAST_G;        // instances per block, within the shared-memory budget
};

void fast_classes(pz_handle* h, const std::map<int, Basis>& bases, const std::vector<std::vector<double>>& rad,
                  int G, std::vector<int>& lane_of, int n_lanes, FastBuild& fb) {
  const int n = h->n_inst;
  std::vector<int> cls_of(n, -1), ucls_of(n, -1);
  std::map<std::tuple<int, double, int>, std::vector<int>> classes;
  for (int i = 0; i < n; ++i)
    if (fast_eligible(h->hin[i].c, h->inst[i]))
      classes[std::make_tuple(h->inst[i].N, h->hin[i].c.radratio, h->inst[i].minc)].push_back(i);
  std::map<std::tuple<int, double, double, double, double>, int> ukeys;
  for (auto& kv : classes) {
    const int N = std::get<0>(kv.first), minc = std::get<2>(kv.first);
    const std::vector<double>& R = rad[kv.second[0]];
    const Basis& B = bases.at(N);
    PzFastGrid g{N, B.D1p.data(), B.D2p.data(), R.data() + (size_t)RV_OR1 * N, R.data() + (size_t)RV_OR2 * N,
                 R.data() + (size_t)RV_BETA * N, R.data() + (size_t)RV_DBETA * N};
    int Mc = 0;
    for (int i : kv.second) Mc = std::max(Mc, h->inst[i].M);
    int ci = -1;
    if (!pz_fast_add_class(fb.H, g, Mc, minc, &ci)) continue;
    for (int i : kv.second) {
      const PzInst& I = h->inst[i];
      const double* ekp = rad[i].data() + (size_t)RV_EKPUMP * N;
      const auto uk = std::make_tuple(N, h->hin[i].c.radratio, I.ViscFac, I.CorFac, ekp[N / 2]);
      int ui;
      if (ukeys.count(uk)) ui = ukeys[uk];
      else if (pz_fast_add_uclass(fb.H, g, I.ViscFac, I.CorFac, ekp, &ui)) ukeys[uk] = ui;
      else continue;
      cls_of[i] = ci;
      ucls_of[i] = ui;
    }
  }
  // work items: per class (largest grids first), per m, the instances that
  // have that m in groups of G; m = 0 groups also share their u_phi class
  std::vector<int> cl;
  for (int c = 0; c < (int)fb.H.cls.size(); ++c) cl.push_back(c);
  std::stable_sort(cl.begin(), cl.end(), [&](int a, int b) { return fb.H.cls[a].N > fb.H.cls[b].N; });
  for (int c : cl) fb.maxN = std::max(fb.maxN, fb.H.cls[c].N);
  while (G > 1 && pz_fast_smem_bytes(G, fb.maxN) > PZ_SMEM_MAX) --G;
  fb.G = G;
  // The lanes take a class's instances G at a time in turn, so the groups
  // are the ones a single lane would form; then lane by lane: a group never
  // mixes lanes, and a lane's items are contiguous.
  for (int c : cl) {
    int k = 0;
    for (int i = 0; i < n; ++i)
      if (cls_of[i] == c) lane_of[i] = (k++ / G) % n_lanes;
  }
  for (int l = 0; l < n_lanes; ++l) {
   fb.lane_item.push_back((int)fb.items.size());
   for (int c : cl) {
    for (int m = 0; m < fb.H.cls[c].Mc; ++m) {
      std::map<int, std::vector<int>> groups;    // by u_phi class (m = 0), else one group
      for (int i = 0; i < n; ++i)
        if (cls_of[i] == c && lane_of[i] == l && h->inst[i].M > m) groups[m == 0 ? ucls_of[i] : 0].push_back(i);
      for (auto& gv : groups)
        for (size_t a = 0; a < gv.second.size(); a += G) {
          PzFastItem it;
          it.cls = c; it.m = m; it.ucls = m == 0 ? gv.first : 0;
          it.i0 = (int)fb.fi.size();
          it.ni = (int)std::min<size_t>(G, gv.second.size() - a);
          for (int q = 0; q < it.ni; ++q) fb.fi.push_back(gv.second[a + q]);
          fb.items.push_back(it);
        }
    }
   }
  }
  fb.lane_item.push_back((int)fb.items.size());
  for (int i = 0; i < n; ++i)
    if (cls_of[i] >= 0) h->inst[i].flags |= PZF_FAST;
}

// one device allocation for the fast path: fragments, exponents, vectors,
// class/m/u descriptors, items and instance lists
cudaError_t fast_upload(pz_handle* h, const FastBuild& fb, int G, PzFastDev* F) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const PzFastHost& H = fb.H;
  size_t o = 0;
  const size_t o_frag = o; o = al(o + H.frag.size() * sizeof(uint4));
  const size_t o_ex = o; o = al(o + H.ex.size() * sizeof(int));
  const size_t o_vec = o; o = al(o + H.vec.size() * sizeof(double));
  const size_t o_cls = o; o = al(o + H.cls.size() * sizeof(PzFastCls));
  const size_t o_ms = o; o = al(o + H.ms.size() * sizeof(PzFastM));
  const size_t o_us = o; o = al(o + H.us.size() * sizeof(PzFastU));
  const size_t o_it = o; o = al(o + fb.items.size() * sizeof(PzFastItem));
  const size_t o_fi = o; o = al(o + fb.fi.size() * sizeof(int));
  cudaError_t e = cudaMalloc(&h->d_fast, o);
  if (e) return e;
  std::vector<unsigned char> img(o, 0);
  auto put = [&](size_t off, const void* src, size_t bytes) { if (bytes) std::memcpy(img.data() + off, src, bytes); };
  put(o_frag, H.frag.data(), H.frag.size() * sizeof(uint4));
  put(o_ex, H.ex.data(), H.ex.size() * sizeof(int));
  put(o_vec, H.vec.data(), H.vec.size() * sizeof(double));
  put(o_cls, H.cls.data(), H.cls.size() * sizeof(PzFastCls));
  put(o_ms, H.ms.data(), H.ms.size() * sizeof(PzFastM));
  put(o_us, H.us.data(), H.us.size() * sizeof(PzFastU));
  put(o_it, fb.items.data(), fb.items.size() * sizeof(PzFastItem));
  put(o_fi, fb.fi.data(), fb.fi.size() * sizeof(int));
  if ((e = cudaMemcpyAsync(h->d_fast, img.data(), o, cudaMemcpyHostToDevice, h->stream)) ||
      (e = cudaStreamSynchronize(h->stream)))
    return e;
  unsigned char* b = static_cast<unsigned char*>(h->d_fast);
  F->frag = reinterpret_cast<const uint4*>(b + o_frag);
  F->ex = reinterpret_cast<const int*>(b + o_ex);
  F->vec = reinterpret_cast<const double*>(b + o_vec);
  F->cls = reinterpret_cast<const PzFastCls*>(b + o_cls);
  F->ms = reinterpret_cast<const PzFastM*>(b + o_ms);
  F->us = reinterpret_cast<const PzFastU*>(b + o_us);
  F->items = reinterpret_cast<const PzFastItem*>(b + o_it);
  F->n_items = (int)fb.items.size();
  F->fi = reinterpret_cast<const int*>(b + o_fi);
  F->G = G;
  F->smem = (int)pz_fast_smem_bytes(G, fb.maxN);
  return cudaSuccess;
}

}  // namespace

extern "C" int pz_integ_banded(int enable) {
  const int prev = g_integ_banded;
  if (enable >= 0) g_integ_banded = enable ? 1 : 0;
  return prev;
}

extern "C" int pz_fast_path(int enable) {
  const int prev = g_fast_default;
  if (enable >= 0) g_fast_default = enable ? 1 : 0;
  return prev;
}

extern "C" int pz_tune_set(int what, int key, int value) {
  if (what == PZ_TUNE_FAST_G) {
    if (value > PZ_FAST_GMAX) return fail(nullptr, PZ_E_ARG, "pz_tune_set: k_fast takes at most 16 instances per block");
    g_tune_fast_g = value > 0 ? value : 0;
    return PZ_OK;
  }
  if (what == PZ_TUNE_LANES) {
    if (value > PZ_LANES_MAX) return fail(nullptr, PZ_E_ARG, "pz_tune_set: at most 4 lanes");
    g_tune_lanes = value > 0 ? value : 2;
    return PZ_OK;
  }
  if (what == PZ_TUNE_RLOOP_RG) {
    if (key < 6 || key % 3 != 0) return fail(nullptr, PZ_E_ARG, "pz_tune_set: key must be an n_phi_max");
    if (value <= 0) { g_tune_rloop_rg.erase(key); return PZ_OK; }
    const int M = key / 3 + 1;
    if (value > 16 || pz_rloop_smem_bytes(key, M, value, 3) > PZ_SMEM_MAX)
      return fail(nullptr, PZ_E_ARG, "pz_tune_set: k_rloop radii per block exceed its shared memory");
    g_tune_rloop_rg[key] = value;
    return PZ_OK;
  }
  return fail(nullptr, PZ_E_ARG, "pz_tune_set: unknown parameter");
}

extern "C" int pz_fast_eigen(int n_r_max, double radratio, int m, double* lam, double* U) {
  if (n_r_max < 5 || n_r_max > 1024 || m < 0 || !(radratio > 0.0 && radratio < 1.0) || !lam || !U)
    return fail(nullptr, PZ_E_ARG, "pz_fast_eigen: bad arguments");
  const int N = n_r_max, n = N - 2;
  const double r_cmb = 1.0 / (1.0 - radratio), r_icb = r_cmb - 1.0;
  const Basis B = make_basis(N, r_icb, r_cmb);
  std::vector<double> or1(N), or2(N), zero(N, 0.0);
  for (int k = 0; k < N; ++k) {
    const double r = 0.5 * (r_cmb - r_icb) * B.x[k] + 0.5 * (r_icb + r_cmb);
    or1[k] = 1.0 / r;
    or2[k] = or1[k] * or1[k];
  }
  const PzFastGrid g{N, B.D1p.data(), B.D2p.data(), or1.data(), or2.data(), zero.data(), zero.data()};
  std::vector<double> P, Pb, l, u, ui;
  pz_fast_laplacian(g, (double)m * (double)m, P, Pb);
  if (!pz_eig_real(n, P, l, u, ui)) return fail(nullptr, PZ_E_SINGULAR, "pz_fast_eigen: decomposition failed");
  std::memcpy(lam, l.data(), n * sizeof(double));
  std::memcpy(U, u.data(), (size_t)n * n * sizeof(double));
  return PZ_OK;
}

extern "C" void pz_config_default(pz_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  // src/namelists.f90:530-672
  c->n_r_max = 32; c->n_cheb_max = 32; c->m_max = 32; c->minc = 1;
  c->ra = 1.0e5; c->ek = 1.0e-3; c->pr = 1.0; c->radratio = 0.35;
  c->g0 = 0.0; c->g1 = 1.0; c->g2 = 0.0;
  c->ktopt = 1; c->kbott = 1; c->ktopv = 2; c->kbotv = 2;
  c->l_ek_pump = 0; c->l_non_rot = 0; c->l_temp_advz = 0;
  c->time_scheme = PZ_CNAB2; c->matrix_solve = PZ_SOLVE_DIRECT;
  c->corio_imp = 1; c->buo_imp = 1;
  c->dtMax = 1.0e-5; c->courfac = 1.0e3; c->alpha = 0.5; c->dt_fac = 2.0;
  c->cheb_method = PZ_CHEB_COLL; c->time_scale = PZ_TS_VISC;
  c->l_rerror_fix = 0; c->rerror_fac = 500.0;
  c->raxi = 0.0; c->sc = 0.0; c->ktopxi = 1; c->kbotxi = 1; c->xicond_fac = 1.0;
}

extern "C" int pz_create(const pz_config* cfgs, int n, pz_handle** out) {
  if (!cfgs || n <= 0 || !out) return fail(nullptr, PZ_E_ARG, "pz_create: bad arguments");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    std::string why;
    const int rc = validate(cfgs[i], &why);
    if (rc != PZ_OK) return fail(nullptr, rc, "instance " + std::to_string(i) + ": " + why);
  }
  pz_handle* h = new pz_handle();
  h->n_inst = n;
  h->hin.resize(n);
  h->inst.resize(n);

  long long off = 0;
  auto take = [&off](long long nd) { long long o = off; off += (nd + 1) & ~1LL; return o; };
  std::map<int, long long> basis_off;    // by N
  std::map<int, Basis> bases;
  std::map<int, long long> tw_off;       // by P
  struct IntegBlock { std::vector<double> ops; int band[IM_COUNT]; };
  std::map<std::pair<int, double>, long long> integ_off;   // by (N, radratio)
  std::map<std::pair<int, double>, IntegBlock> integ_blocks;
  std::vector<std::vector<double>> rad(n);
  int maxN = 0, maxP = 0, maxM = 0;
  for (int i = 0; i < n; ++i) {
    const pz_config& c = cfgs[i];
    PzInst I;
    std::memset(&I, 0, sizeof(I));
    I.N = c.n_r_max; I.n_max = c.n_cheb_max; I.mmax = c.m_max; I.minc = c.minc;
    I.M = c.m_max / c.minc + 1;                   // truncation.f90:28
    I.P = 3 * c.m_max / c.minc;                   // truncation.f90:30-31
    I.rg = std::max(1, std::min(8, PZ_RLOOP_PG / I.P));
    if (g_tune_rloop_rg.count(I.P)) I.rg = g_tune_rloop_rg[I.P];
    factor_fft(I.P, I.radix, &I.nrad);
    double cf;
    int imp_calc;
    scheme_counts(c.time_scheme, &I.nold, &I.nimp, &I.nexp, &cf, &imp_calc);
    I.scheme = c.time_scheme;
    {
      DirkTab tab;
      const bool dirk = dirk_tableau(c.time_scheme, &tab);
      I.dirk = dirk ? 1 : 0;
      I.nstages = dirk ? tab.nstages : 1;
      I.assembly = dirk ? tab.assembly : 0;
      I.exp_mask = dirk ? tab.exp_mask : 1;
      I.imp_mask = dirk ? tab.imp_mask : 1;
      I.dirk_gamma = dirk ? tab.gamma : 0.0;
    }
    I.courfac = std::fabs(c.courfac) >= 1.0e3 ? cf : c.courfac;
    // derived switches (namelists.f90:271-526)
    double ek = c.ek;
    const bool non_rot = c.l_non_rot || ek < 0.0;
    if (non_rot) ek = -1.0;
    I.ek = ek;
    I.tadvz = c.l_temp_advz ? 1.0 : 0.0;
    I.alpha = c.alpha;
    I.dtMax = c.dtMax; I.dtMin = c.dtMax / 1.0e6;   // pre_calculations.f90:33
    I.dt_fac = c.dt_fac;
    const bool chem = c.raxi != 0.0;   // namelists.f90:323-327
    if (non_rot) { I.CorFac = 0.0; I.BuoFac = c.ra / c.pr; I.TdiffFac = 1.0 / c.pr; I.ViscFac = 1.0; }
    else if (c.time_scale == PZ_TS_ROT) {   // namelists.f90:491-500
      I.CorFac = 2.0; I.BuoFac = c.ra * ek * ek / c.pr; I.TdiffFac = ek / c.pr; I.ViscFac = ek;
    } else { I.CorFac = 2.0 / ek; I.BuoFac = c.ra / c.pr; I.TdiffFac = 1.0 / c.pr; I.ViscFac = 1.0; }
    if (chem) {   // namelists.f90:482-522: raxi and sc in place of ra and pr
      if (non_rot || c.time_scale != PZ_TS_ROT) { I.ChemFac = c.raxi / c.sc; I.XidiffFac = 1.0 / c.sc; }
      else { I.ChemFac = c.raxi * ek * ek / c.sc; I.XidiffFac = ek / c.sc; }
    }
    I.nhf = chem ? 3 : 2;
    I.flags = 0;
    if (chem) I.flags |= PZF_CHEM;
    if (c.buo_imp) I.flags |= PZF_BUO_IMP;
    if (c.l_ek_pump) I.flags |= PZF_EK_PUMP;
    if (non_rot) I.flags |= PZF_NON_ROT;
    if (imp_calc) I.flags |= PZF_IMP_CALC;
    const bool direct = c.matrix_solve == PZ_SOLVE_DIRECT;
    if (direct) I.flags |= PZF_DIRECT;
    // corio_term='IMPLICIT' only with the direct solve (namelists.f90:448-457)
    if (direct && c.corio_imp && !non_rot) I.flags |= PZF_COR_IMP;
    // get_tempMat and get_omMat (update_temp_coll.f90:310-393,
    // update_psi_coll_dmat.f90:829-911) build the same rows when
    // TdiffFac*hdif_T == ViscFac*hdif_V and both use fixed/no-slip boundary rows
    if (!direct && c.cheb_method != PZ_CHEB_INTEG && I.TdiffFac == I.ViscFac) I.flags |= PZF_T_IS_OM;
    if (c.cheb_method == PZ_CHEB_INTEG) I.flags |= PZF_INTEG;
    if (c.l_rerror_fix) {   // radial_derivatives.f90:51-66
      I.flags |= PZF_RERR;
      I.rerr_thr = c.rerror_fac * 2.220446049250313e-16;
    }
    const int N = I.N;
    I.rnorm = std::sqrt(2.0 / (double)(N - 1));
    I.r_cmb = 1.0 / (1.0 - c.radratio);
    I.r_icb = I.r_cmb - 1.0;
    if (!bases.count(N)) {
      bases[N] = make_basis(N, I.r_icb, I.r_cmb);
      basis_off[N] = take((long long)BM_COUNT * N * N);
    }
    I.o_basis = basis_off[N];
    if (I.flags & PZF_INTEG) {
      // integration-method operators, shared by equal (N, radratio)
      const std::pair<int, double> key(N, c.radratio);
      if (!integ_off.count(key)) {
        IntegBlock& ib = integ_blocks[key];
        pz_integ_operators(N, I.r_icb, I.r_cmb, I.rnorm, ib.ops, ib.band);
        integ_off[key] = take((long long)IM_COUNT * N * N);
      }
      I.o_integ = integ_off[key];
      std::memcpy(I.im_band, integ_blocks[key].band, sizeof(I.im_band));
      if (!g_integ_banded) I.flags |= PZF_INTEG_DENSE;
      const int* bd = I.im_band;
      const bool rot = !(I.flags & PZF_NON_ROT);
      I.bkw_t = std::max(std::max(bd[IM_I2R2], bd[IM_LT0]), std::max(bd[IM_I2], bd[IM_ULAP]));
      I.bkl_t = bord_kl(I.bkw_t);
      I.bstr_t = bord_size(N, 2, I.bkl_t);
      if (I.flags & PZF_DIRECT) {
        I.bkw_p = rot ? std::max(std::max(std::max(bd[IM_Q0], bd[IM_Q1]), std::max(bd[IM_S0], bd[IM_S1])),
                                 std::max(bd[IM_S2], bd[IM_I4R4]))
                      : std::max(std::max(std::max(bd[IM_N0], bd[IM_N1]), std::max(bd[IM_L0], bd[IM_L1])),
                                 std::max(bd[IM_L2], bd[IM_I4R4]));
        I.bkl_p = bord_kl(I.bkw_p);
        I.bstr_p = 2 * bord_size(N, 4, I.bkl_p);
      } else {
        I.bkw_p = rot ? std::max(bd[IM_P0], bd[IM_P1]) : std::max(bd[IM_LT0], bd[IM_I2]);
        I.bkl_p = bord_kl(I.bkw_p);
        I.bstr_p = bord_size(N, 2, I.bkl_p);
      }
      if (I.bkw_t > 8 || I.bkw_p > 8) {
        delete h;
        return fail(nullptr, PZ_E_UNSUPPORTED, "integration-method operator with a half band width above 8");
      }
    }
    if (!tw_off.count(I.P)) tw_off[I.P] = take(4LL * I.P);
    I.o_tw = tw_off[I.P];
    // radial functions (radial.f90:115-282)
    const Basis& B = bases[N];
    std::vector<double>& R = rad[i];
    R.assign((size_t)RV_COUNT * N, 0.0);
    auto rv = [&R, N](int k, int r) -> double& { return R[(size_t)k * N + r]; };
    const double bma = 0.5 * (I.r_cmb - I.r_icb), bpa = 0.5 * (I.r_icb + I.r_cmb);
    std::vector<double> r(N);
    for (int k = 0; k < N; ++k) r[k] = bma * B.x[k] + bpa;
    const double ek_pump_fac = (c.l_ek_pump && !non_rot) ? 1.0 : 0.0;
    const double rc = I.r_cmb, ri = I.r_icb;
    const double m_R = (double)c.m_max;
    const double twopi3 = 2.0 * 3.14159265358979323846 / 3.0;
    for (int k = 0; k < N; ++k) {
      rv(RV_R, k) = r[k];
      rv(RV_OR1, k) = 1.0 / r[k];
      rv(RV_OR2, k) = rv(RV_OR1, k) * rv(RV_OR1, k);
      rv(RV_RGRAV, k) = c.g0 + c.g1 * r[k] / rc + c.g2 * rc * rc * rv(RV_OR2, k);
      rv(RV_TCOND, k) = std::log(r[k] / rc) / std::log(c.radratio);
      rv(RV_DTCOND, k) = rv(RV_OR1, k) / std::log(c.radratio);
      if (chem) {   // the same 2D profile with xicond_fac (radial.f90:377-379)
        rv(RV_XICOND, k) = c.xicond_fac * (std::log(r[k] / rc) / std::log(c.radratio));
        rv(RV_DXICOND, k) = c.xicond_fac * (rv(RV_OR1, k) / std::log(c.radratio));
      }
      if (non_rot) {
        rv(RV_HEIGHT, k) = 1.0;
      } else if (k > 0) {
        const double s2 = rc * rc - r[k] * r[k];
        rv(RV_HEIGHT, k) = 2.0 * std::sqrt(s2);
        const double oh = 0.5 / std::sqrt(s2);
        rv(RV_BETA, k) = -r[k] / s2;
        rv(RV_DBETA, k) = -(rc * rc + r[k] * r[k]) / (s2 * s2);
        rv(RV_EKPUMP, k) = 0.5 * ek_pump_fac * std::sqrt(ek * rc) / std::pow(s2, 0.75);
        rv(RV_EKP_UP, k) = -0.5 * rv(RV_BETA, k);
        rv(RV_EKP_US, k) = -5.0 * rc * rv(RV_BETA, k) * oh;
        rv(RV_EKP_DUSDP, k) = rv(RV_BETA, k);
      }
      // Courant lengths (radial.f90:164-173)
      if (k == 0) {
        rv(RV_DELXH2, k) = std::pow(twopi3 / m_R * rc, 2);
        rv(RV_DELXR2, k) = std::pow(r[0] - r[1], 2);
      } else if (k == N - 1) {
        rv(RV_DELXH2, k) = std::pow(twopi3 / m_R * ri, 2);
        rv(RV_DELXR2, k) = std::pow(r[N - 2] - r[N - 1], 2);
      } else {
        rv(RV_DELXH2, k) = std::pow(twopi3 / m_R * r[k], 2);
        const double dmin = std::min(r[k - 1] - r[k], r[k] - r[k + 1]);
        rv(RV_DELXR2, k) = dmin * dmin;
      }
    }
    // rInt_R weights: rInt(f) = 2 sqrt(2/(N-1)) sum_k q_k (C f/drx)_k
    std::vector<double> q(N, 0.0);
    q[0] = 0.5;
    for (int nc = 3; nc <= N; nc += 2) q[nc - 1] = -1.0 / (double)(nc * (nc - 2));
    if ((N - 1) % 2 == 0) q[N - 1] *= 0.5;   // f2(n_r_max) halved before the sum
    const double drx = 2.0 / (rc - ri);
    const double pre = 2.0 * std::sqrt(2.0 / (double)(N - 1));
    for (int j = 0; j < N; ++j) {
      long double s = 0.0L;
      for (int k = 0; k < N; ++k) s += (long double)q[k] * (long double)B.C[k + (size_t)j * N];
      rv(RV_WINT, j) = pre * (double)s / drx;
    }
    // simps over colatitude theta = asin(r/r_cmb) (outputs.f90:768-783)
    std::vector<double> th(N), e(N, 0.0);
    for (int k = 0; k < N; ++k) th[k] = std::asin(std::min(1.0, r[k] / rc));
    for (int j = 0; j < N; ++j) {
      std::fill(e.begin(), e.end(), 0.0);
      e[j] = 1.0;
      rv(RV_WSIMP, j) = simps(e, th);
    }
    // influence-matrix boundary rows, rigid walls: rnorm * bfac * drMat
    for (int k = 0; k < N; ++k) {
      const double bf = (k == 0 || k == N - 1) ? 0.5 : 1.0;
      rv(RV_BCTOP, k) = I.rnorm * bf * B.drMat[0 + (size_t)k * N];
      rv(RV_BCBOT, k) = I.rnorm * bf * B.drMat[(N - 1) + (size_t)k * N];
    }
    // denominators of Nu_vol and Nu_int
    double sv = 0.0, sf = 0.0, sfs = 0.0;
    std::vector<double> tmp(N);
    for (int k = 0; k < N; ++k) {
      sv += rv(RV_WINT, k) * rv(RV_DTCOND, k) * rv(RV_DTCOND, k) * rv(RV_HEIGHT, k) * r[k];
      sf += rv(RV_WINT, k) * (-I.TdiffFac * rv(RV_DTCOND, k) * r[k]);
      tmp[k] = -I.TdiffFac * rv(RV_DTCOND, k) * (r[k] / rc) * (r[k] / rc);
    }
    sfs = simps(tmp, th);
    I.nu_vol_den = sv;
    double sx = 0.0;
    for (int k = 0; k < N; ++k) sx += rv(RV_WINT, k) * rv(RV_DXICOND, k) * rv(RV_DXICOND, k) * rv(RV_HEIGHT, k) * r[k];
    I.sh_vol_den = sx;
    I.nu_int_fac = non_rot ? sf : sfs;
    I.o_rad = take((long long)RV_COUNT * N);
    h->hin[i].c = c;
    h->inst[i] = I;
    maxN = std::max(maxN, N);
    maxP = std::max(maxP, I.P);
    maxM = std::max(maxM, I.M);
  }
  // tensor-core stage: classes, eigen-bases and work items of the eligible instances
  // lanes of the plain step: the instances in work-list order (largest
  // first), dealt to the lanes in turn so that each lane gets the same mix
  // (the tensor-core instances then by whole k_fast groups per class)
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (long long)h->inst[a].N * h->inst[a].M > (long long)h->inst[b].N * h->inst[b].M;
  });
  int n_lanes = std::min(std::max(g_tune_lanes, 1), PZ_LANES_MAX);
  if (n < 16 * n_lanes) n_lanes = 1;
  std::vector<int> lane_of(n, 0);    // fast_classes deals its instances by whole groups
  for (int k = 0; k < n; ++k) lane_of[order[k]] = k % n_lanes;
  FastBuild fb;
  const int fast_g = g_tune_fast_g > 0 ? g_tune_fast_g : PZ_FAST_G;
  fast_classes(h, bases, rad, fast_g, lane_of, n_lanes, fb);
  // per-instance operators and state
  for (int i = 0; i < n; ++i) {
    PzInst& I = h->inst[i];
    const long long N = I.N, M = I.M;
    if ((I.flags & PZF_INTEG) && !(I.flags & PZF_INTEG_DENSE)) {
      // bordered banded factors per m (pz_bord.cuh)
      I.o_gt = take(M * I.bstr_t);
      I.o_gx = (I.flags & PZF_CHEM) ? take(M * I.bstr_t) : 0;
      I.o_guphi = take(I.bstr_t);
      if (I.flags & PZF_DIRECT) {
        I.o_gsm = take(M * I.bstr_p);
        I.o_gom = I.o_gpsi = I.o_aux = 0;
      } else {
        I.o_gom = take(M * I.bstr_t);
        I.o_gpsi = take(M * I.bstr_p);
        I.o_aux = take(4 * M * N + 4 * M);
        I.o_gsm = 0;
      }
    } else {
    I.o_gt = take(M * N * N);
    I.o_gx = (I.flags & PZF_CHEM) ? take(M * N * N) : 0;
    I.o_guphi = take(N * N);
    if ((I.flags & PZF_INTEG) && (I.flags & PZF_DIRECT)) {
      I.o_gsm = take(2 * M * N * N);      // complex N x N streamfunction inverse per m
      I.o_gom = I.o_gpsi = I.o_aux = 0;
    } else if (I.flags & PZF_DIRECT) {
      I.o_gsm = take(4 * M * N * N);
      I.o_gom = I.o_gpsi = I.o_aux = 0;   // influence-matrix operators unused
      I.smat_ws_stride = pz_smat_ws_doubles((int)N);
      I.o_smat_ws = I.smat_ws_stride ? take(M * I.smat_ws_stride) : 0;
    } else {
      I.o_gom = take(M * N * N);
      I.o_gpsi = take(M * N * N);
      I.o_aux = take(4 * M * N + 4 * M);
      I.o_gsm = 0;
    }
    }
    I.o_bt = I.dirk ? take(PZ_BT_SIZE) : 0;
    I.o_gass = (I.dirk && I.assembly) ? take(M * N * N) : 0;
    I.o_fld = take(2LL * F_COUNT * M * N);
    I.o_hist = take(2LL * I.nhf * (I.nold + I.nimp + I.nexp) * M * N);
    I.o_cfl = take(2 * N);
    I.o_series = take((long long)PZ_SERIES_CAP * PZ_SERIES_COLS);
  }
  h->pool_size = off;
  cudaError_t e;
  if ((e = pz_setup_kernels())) { int rc = cuda_fail(nullptr, e, "kernel setup"); delete h; return rc; }
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking))) {
    int rc = cuda_fail(nullptr, e, "stream"); delete h; return rc;
  }
  if ((e = cudaMalloc(&h->pool, (size_t)off * sizeof(double)))) {
    g_create_error = std::string("device pool allocation: ") + cudaGetErrorString(e);
    pz_destroy(h);
    return PZ_E_NOMEM;
  }
  // host image of the constant parts, uploaded in one copy
  std::vector<double> img;
  {
    long long hi = 0;
    for (auto& kv : basis_off) hi = std::max(hi, kv.second + (long long)BM_COUNT * kv.first * kv.first);
    for (auto& kv : tw_off) hi = std::max(hi, kv.second + 4LL * kv.first);
    for (auto& kv : integ_off) hi = std::max(hi, kv.second + (long long)IM_COUNT * kv.first.first * kv.first.first);
    for (int i = 0; i < n; ++i) hi = std::max(hi, h->inst[i].o_rad + (long long)RV_COUNT * h->inst[i].N);
    for (int i = 0; i < n; ++i)
      if (h->inst[i].dirk) hi = std::max(hi, h->inst[i].o_bt + (long long)PZ_BT_SIZE);
    img.assign((size_t)hi, 0.0);
    for (int i = 0; i < n; ++i) {
      DirkTab tab;
      if (!h->inst[i].dirk || !dirk_tableau(h->inst[i].scheme, &tab)) continue;
      double* bt = img.data() + h->inst[i].o_bt;
      for (int r = 0; r < PZ_BT_LD; ++r)
        for (int q = 0; q < PZ_BT_LD; ++q) {
          bt[PZ_BT_IMP + r * PZ_BT_LD + q] = tab.bimp[r][q];
          bt[PZ_BT_EXP + r * PZ_BT_LD + q] = tab.bexp[r][q];
        }
      for (int q = 0; q < PZ_BT_LD; ++q) {
        bt[PZ_BT_AIMP + q] = tab.bai[q];
        bt[PZ_BT_AEXP + q] = tab.bae[q];
      }
    }
    for (auto& kv : bases) {
      const Basis& B = kv.second;
      const long long NN = (long long)B.N * B.N;
      double* dst = img.data() + basis_off[kv.first];
      const std::vector<double>* mats[BM_COUNT] = {&B.C,    &B.D1c,  &B.D2c,  &B.D1p,   &B.D2p,   &B.rMat,
                                                   &B.drMat, &B.d2rMat, &B.Cs, &B.D1cs, &B.D2cs, &B.D1ps,
                                                   &B.D2ps, &B.CTs, &B.D1cTs, &B.D2cTs, &B.D1pTs, &B.Cos};
      for (int k = 0; k < BM_COUNT; ++k) std::memcpy(dst + k * NN, mats[k]->data(), mats[k]->size() * sizeof(double));
    }
    const long double pi = 3.141592653589793238462643383279502884L;
    for (auto& kv : tw_off) {
      const int P = kv.first;
      double* dst = img.data() + kv.second;
      for (int k = 0; k < P; ++k) {
        const long double a = 2.0L * pi * (long double)k / (long double)P;
        dst[2 * k] = (double)cosl(a);
        dst[2 * k + 1] = -(double)sinl(a);
        dst[2 * P + 2 * k] = dst[2 * k];          // the conjugates, for the backward transforms
        dst[2 * P + 2 * k + 1] = (double)sinl(a);
      }
    }
    for (int i = 0; i < n; ++i) std::memcpy(img.data() + h->inst[i].o_rad, rad[i].data(), rad[i].size() * sizeof(double));
    for (auto& kv : integ_off) {
      const std::vector<double>& ops = integ_blocks[kv.first].ops;
      std::memcpy(img.data() + kv.second, ops.data(), ops.size() * sizeof(double));
    }
  }
  if ((e = cudaMemsetAsync(h->pool, 0, (size_t)off * sizeof(double), h->stream)) ||
      (e = cudaMemcpyAsync(h->pool, img.data(), img.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream))) {
    g_create_error = std::string("pool upload: ") + cudaGetErrorString(e);
    pz_destroy(h);
    return PZ_E_CUDA;
  }
  // work lists: radii and m, largest instances first
  std::vector<PzItem> ritems, mitems, oitems;
  std::vector<int> lane_r, lane_o, lane_i, linst;   // lane l's ranges of ritems, oitems, linst
  for (int l = 0; l < n_lanes; ++l) {
    lane_r.push_back((int)ritems.size());
    lane_o.push_back((int)oitems.size());
    lane_i.push_back((int)linst.size());
    for (int i : order) {
      if (lane_of[i] != l) continue;
      for (int r = 0; r < h->inst[i].N; r += h->inst[i].rg) ritems.push_back({i, r});
      for (int r = 0; r < h->inst[i].N; r += PZ_OBS_RC) oitems.push_back({i, r});
      linst.push_back(i);
    }
  }
  lane_r.push_back((int)ritems.size());
  lane_o.push_back((int)oitems.size());
  lane_i.push_back((int)linst.size());
  for (int i : order)
    for (int m = 0; m < h->inst[i].M; ++m) mitems.push_back({i, m});
  if ((e = cudaMalloc(&h->d_inst, n * sizeof(PzInst))) || (e = cudaMalloc(&h->d_state, n * sizeof(PzState))) ||
      (e = cudaMalloc(&h->d_ritems, ritems.size() * sizeof(PzItem))) ||
      (e = cudaMalloc(&h->d_mitems, mitems.size() * sizeof(PzItem))) ||
      (e = cudaMalloc(&h->d_order, mitems.size() * sizeof(PzItem))) ||
      (e = cudaMalloc(&h->d_iorder, n * sizeof(int))) ||
      (e = cudaMalloc(&h->d_rows, (size_t)n * PZ_SERIES_COLS * sizeof(double))) ||
      (e = cudaMalloc(&h->d_spec, (size_t)5 * maxM * sizeof(double))) ||
      (e = cudaMalloc(&h->d_spec2d, (size_t)3 * maxN * maxM * sizeof(double))) ||
      (e = cudaMalloc(&h->d_oitems, oitems.size() * sizeof(PzItem))) ||
      (e = cudaMalloc(&h->d_obs_part, oitems.size() * PZ_OBS_NP * sizeof(double))) ||
      (e = cudaMalloc(&h->d_obs_cnt, n * sizeof(int)))) {
    g_create_error = std::string("device allocation: ") + cudaGetErrorString(e);
    pz_destroy(h);
    return PZ_E_NOMEM;
  }
  cudaMemcpyAsync(h->d_inst, h->inst.data(), n * sizeof(PzInst), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->d_ritems, ritems.data(), ritems.size() * sizeof(PzItem), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->d_mitems, mitems.data(), mitems.size() * sizeof(PzItem), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->d_iorder, order.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->d_oitems, oitems.data(), oitems.size() * sizeof(PzItem), cudaMemcpyHostToDevice, h->stream);
  cudaMemsetAsync(h->d_obs_cnt, 0, n * sizeof(int), h->stream);
  cudaMemsetAsync(h->d_state, 0, n * sizeof(PzState), h->stream);
  h->dev.inst = h->d_inst;
  h->dev.state = h->d_state;
  h->dev.pool = h->pool;
  h->dev.ritems = h->d_ritems; h->dev.n_ritems = (int)ritems.size();
  h->dev.mitems = h->d_mitems; h->dev.n_mitems = (int)mitems.size();
  h->dev.order = h->d_order;
  h->dev.oitems = h->d_oitems; h->dev.n_oitems = (int)oitems.size();
  h->dev.obs_part = h->d_obs_part;
  h->dev.obs_cnt = h->d_obs_cnt;
  h->dev.iorder = h->d_iorder;
  h->dev.n_iorder = n;
  h->dev.n_inst = n;
  h->dev.any_chem = 0;
  for (int i = 0; i < n; ++i) h->dev.any_chem |= (h->inst[i].flags & PZF_CHEM) ? 1 : 0;
  h->dev.maxN = maxN; h->dev.maxP = maxP; h->dev.maxM = maxM;
  size_t sb = 0;
  for (int i = 0; i < n; ++i)
    sb = std::max(sb, pz_build_smem_bytes(h->inst[i].N, (h->inst[i].flags & PZF_DIRECT) != 0,
                                          (h->inst[i].flags & PZF_INTEG) != 0));
  h->dev.smem_build = (int)sb;
  size_t srl = 0;
  for (int i = 0; i < n; ++i)
    srl = std::max(srl, pz_rloop_smem_bytes(h->inst[i].P, h->inst[i].M, h->inst[i].rg,
                                            (h->inst[i].flags & PZF_CHEM) ? 3 : 2));
  h->dev.smem_rloop = (int)srl;
  // launch plan of one step: per stage k_rloop [k_cfl, k_build] k_mloop, then
  // the assembly stage and the time series (step_time.f90:139-406)
  int smax = 1;
  bool any_assembly = false, any_integ = false, any_coll = false;
  for (int i = 0; i < n; ++i) {
    smax = std::max(smax, h->inst[i].nstages);
    any_assembly |= h->inst[i].assembly != 0;
    const bool integ = (h->inst[i].flags & PZF_INTEG) != 0;
    any_integ |= integ;
    any_coll |= !integ;
  }
  // the rebuild fused with the first stage when it costs the stage no
  // occupancy: collocation only, build staged in at most 48 KB of shared memory
  const bool fused = !any_integ && sb <= 48 * 1024;
  h->plan.clear();
  for (int st = 1; st <= smax; ++st) {
    h->plan.push_back({PZK_RLOOP, st});
    if (st == 1) {
      h->plan.push_back({PZK_CFL, 1});
      if (fused) {
        h->plan.push_back({PZK_ORDER, 1});
        h->plan.push_back({PZK_BUILD_MLOOP, 1});
        continue;
      }
      h->plan.push_back({PZK_BUILD, 1});
    }
    if (any_coll) h->plan.push_back({PZK_MLOOP, st});
    if (any_integ) h->plan.push_back({PZK_MLOOP_INTEG, st});
  }
  if (any_assembly) h->plan.push_back({PZK_ASSEMBLE, 0});
  h->plan.push_back({PZK_OBS, 0});
  // the plain step's plan: fast instances leave the per-m work lists and run
  // in k_fast after k_cfl; the standard stage kernels run for the others
  if (!fb.items.empty()) {
    std::vector<PzItem> mstd;
    std::vector<int> ostd;
    for (int i : order) {
      if (h->inst[i].flags & PZF_FAST) { ++h->n_fast; continue; }
      ostd.push_back(i);
      for (int m = 0; m < h->inst[i].M; ++m) mstd.push_back({i, m});
    }
    h->fdev = h->dev;
    if ((e = fast_upload(h, fb, fb.G, &h->fdev.fast)) ||
        (!mstd.empty() && ((e = cudaMalloc(&h->d_mitems_std, mstd.size() * sizeof(PzItem))) ||
                           (e = cudaMalloc(&h->d_iorder_std, ostd.size() * sizeof(int))) ||
                           (e = cudaMemcpyAsync(h->d_mitems_std, mstd.data(), mstd.size() * sizeof(PzItem),
                                                cudaMemcpyHostToDevice, h->stream)) ||
                           (e = cudaMemcpyAsync(h->d_iorder_std, ostd.data(), ostd.size() * sizeof(int),
                                                cudaMemcpyHostToDevice, h->stream))))) {
      g_create_error = std::string("fast-path set-up: ") + cudaGetErrorString(e);
      pz_destroy(h);
      return PZ_E_NOMEM;
    }
    h->fdev.fast_maxN = fb.maxN;
    h->fdev.mitems = h->d_mitems_std;
    h->fdev.n_mitems = (int)mstd.size();
    h->fdev.iorder = h->d_iorder_std;
    h->fdev.n_iorder = (int)ostd.size();
    int fsmax = 1;
    bool f_integ = false, f_coll = false;
    for (int i : ostd) {
      fsmax = std::max(fsmax, h->inst[i].nstages);
      f_integ |= (h->inst[i].flags & PZF_INTEG) != 0;
      f_coll |= !(h->inst[i].flags & PZF_INTEG);
    }
    const bool ffused = !f_integ && sb <= 48 * 1024;
    for (int st = 1; st <= fsmax; ++st) {
      h->fplan.push_back({PZK_RLOOP, st});
      if (st == 1) {
        h->fplan.push_back({PZK_CFL, 1});
        h->fplan.push_back({PZK_FAST, 1});
        if (ostd.empty()) continue;
        if (ffused) {
          h->fplan.push_back({PZK_ORDER, 1});
          h->fplan.push_back({PZK_BUILD_MLOOP, 1});
          continue;
        }
        h->fplan.push_back({PZK_BUILD, 1});
      }
      if (f_coll) h->fplan.push_back({PZK_MLOOP, st});
      if (f_integ) h->fplan.push_back({PZK_MLOOP_INTEG, st});
    }
    if (any_assembly) h->fplan.push_back({PZK_ASSEMBLE, 0});
    h->fplan.push_back({PZK_OBS, 0});
    // lanes: every instance on the fast path and no assembly stage (the
    // plan is then k_rloop, k_cfl, k_fast, k_obs, each over its own items)
    if (n_lanes > 1 && ostd.empty() && !any_assembly) {
      if ((e = cudaMalloc(&h->d_lane_inst, n * sizeof(int))) ||
          (e = cudaMemcpyAsync(h->d_lane_inst, linst.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream)) ||
          (e = cudaEventCreateWithFlags(&h->lane_fork, cudaEventDisableTiming))) {
        g_create_error = std::string("lanes: ") + cudaGetErrorString(e);
        pz_destroy(h);
        return PZ_E_NOMEM;
      }
      for (int l = 0; l < n_lanes; ++l) {
        if ((e = cudaStreamCreateWithFlags(&h->lane_stream[l], cudaStreamNonBlocking)) ||
            (e = cudaEventCreateWithFlags(&h->lane_join[l], cudaEventDisableTiming))) {
          g_create_error = std::string("lanes: ") + cudaGetErrorString(e);
          pz_destroy(h);
          return PZ_E_NOMEM;
        }
        PzDev& L = h->ldev[l];
        L = h->fdev;
        L.ritems = h->d_ritems + lane_r[l];
        L.n_ritems = lane_r[l + 1] - lane_r[l];
        L.oitems = h->d_oitems + lane_o[l];
        L.n_oitems = lane_o[l + 1] - lane_o[l];
        L.obs_part = h->d_obs_part + (long long)lane_o[l] * PZ_OBS_NP;   // k_obs indexes it by block
        L.cfl_inst = h->d_lane_inst + lane_i[l];
        L.n_inst = lane_i[l + 1] - lane_i[l];
        L.fast.items = h->fdev.fast.items + fb.lane_item[l];
        L.fast.n_items = fb.lane_item[l + 1] - fb.lane_item[l];
      }
      h->n_lanes = n_lanes;
    }
  }
  if ((e = pz_launch_init_state(h->dev, -1, h->stream)) || (e = pz_launch_build_static(h->dev, h->stream)) ||
      (e = cudaStreamSynchronize(h->stream))) {
    g_create_error = std::string("static operators: ") + cudaGetErrorString(e);
    pz_destroy(h);
    return PZ_E_CUDA;
  }
  std::vector<PzState> st(n);
  cudaMemcpy(st.data(), h->d_state, n * sizeof(PzState), cudaMemcpyDeviceToHost);
  for (int i = 0; i < n; ++i)
    if (st[i].status != 0) {
      g_create_error = "instance " + std::to_string(i) + ": singular psi matrix";
      pz_destroy(h);
      return PZ_E_SINGULAR;
    }
  *out = h;
  return PZ_OK;
}

namespace {

// (n_m, n_r) n_m-fastest host array <-> device m-major field of instance i
int upload_field(pz_handle* h, int i, int f, const double* src) {
  const PzInst& I = h->inst[i];
  const long long MN = (long long)I.M * I.N;
  std::vector<double> buf(2 * MN, 0.0);
  if (src)
    for (int r = 0; r < I.N; ++r)
      for (int m = 0; m < I.M; ++m) {
        buf[2 * ((long long)m * I.N + r)] = src[2 * (m + (long long)r * I.M)];
        buf[2 * ((long long)m * I.N + r) + 1] = src[2 * (m + (long long)r * I.M) + 1];
      }
  cudaError_t e = cudaMemcpyAsync(h->pool + I.o_fld + 2LL * f * MN, buf.data(), 2 * MN * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream);
  if (e) return cuda_fail(h, e, "set_state upload");
  e = cudaStreamSynchronize(h->stream);   // buf is pageable and local
  if (e) return cuda_fail(h, e, "set_state upload");
  return PZ_OK;
}

int check_status(pz_handle* h) {
  std::vector<PzState> st(h->n_inst);
  cudaError_t e = cudaMemcpyAsync(st.data(), h->d_state, h->n_inst * sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "device state");
  for (int i = 0; i < h->n_inst; ++i) {
    const int s = st[i].status;
    if (s == 0) continue;
    const char* what = s == PZ_E_SINGULAR ? "singular matrix" : s == PZ_E_DT_TOO_SMALL ? "time step too small (dt < dtMin)"
                       : s == PZ_E_NONFINITE ? "non-finite value in the state" : "device error";
    return fail(h, s, "instance " + std::to_string(i) + ": " + what + " after step " + std::to_string(st[i].n_step));
  }
  return PZ_OK;
}

}  // namespace

int pz_check_status(pz_handle* h) { return check_status(h); }

extern "C" int pz_set_state_xi(pz_handle* h, int inst, const double* us, const double* up, const double* temp,
                               const double* xi) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_set_state: null handle");
  pz_adjoint_invalidate(h);
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_set_state: instance out of range");
  const bool chem = (h->inst[inst].flags & PZF_CHEM) != 0;
  if (xi && !chem) return fail(h, PZ_E_ARG, "pz_set_state_xi: the instance has no composition (raxi = 0)");
  int rc;
  if ((rc = upload_field(h, inst, F_US, us)) || (rc = upload_field(h, inst, F_UP, up)) ||
      (rc = upload_field(h, inst, F_TEMP, temp)) || (chem && (rc = upload_field(h, inst, F_XI, xi))))
    return rc;
  cudaError_t e;
  if ((e = pz_launch_init_state(h->dev, inst, h->stream)) || (e = pz_launch_start(h->dev, inst, h->stream)) ||
      (e = pz_launch_obs(h->dev, inst, h->stream)))
    return cuda_fail(h, e, "pz_set_state");
  return check_status(h);
}

extern "C" int pz_set_state(pz_handle* h, int inst, const double* us, const double* up, const double* temp) {
  return pz_set_state_xi(h, inst, us, up, temp, nullptr);
}

extern "C" int pz_set_state_all(pz_handle* h, const double* us, const double* up, const double* temp) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_set_state_all: null handle");
  pz_adjoint_invalidate(h);
  long long o = 0;
  for (int i = 0; i < h->n_inst; ++i) {
    const PzInst& I = h->inst[i];
    int rc;
    if ((rc = upload_field(h, i, F_US, us ? us + o : nullptr)) || (rc = upload_field(h, i, F_UP, up ? up + o : nullptr)) ||
        (rc = upload_field(h, i, F_TEMP, temp ? temp + o : nullptr)) ||
        ((I.flags & PZF_CHEM) && (rc = upload_field(h, i, F_XI, nullptr))))
      return rc;
    o += 2LL * I.M * I.N;
  }
  cudaError_t e;
  if ((e = pz_launch_init_state(h->dev, -1, h->stream)) || (e = pz_launch_start(h->dev, -1, h->stream)) ||
      (e = pz_launch_obs(h->dev, -1, h->stream)))
    return cuda_fail(h, e, "pz_set_state_all");
  return check_status(h);
}

extern "C" int pz_step(pz_handle* h, int n_steps) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_step: null handle");
  pz_adjoint_invalidate(h);
  if (n_steps < 0) return fail(h, PZ_E_ARG, "pz_step: n_steps < 0");
  cudaError_t e = cudaSuccess;
  const bool fast = h->n_fast > 0;
  if (fast && h->n_lanes > 1) {
    // one graph per lane on the lane's own stream; the lanes start after the
    // work already on the handle's stream and the handle's stream waits for
    // all of them at the end, so the lanes run their steps independently
    // in between (one lane's transforms beside another's stage)
    for (int l = 0; l < h->n_lanes && !h->lane_graph[l]; ++l) {
      cudaGraph_t g;
      if ((e = cudaStreamBeginCapture(h->lane_stream[l], cudaStreamCaptureModeThreadLocal)))
        return cuda_fail(h, e, "capture");
      for (const PzLaunch& L : h->fplan)
        if (!e) e = pz_launch_step_kernel(h->ldev[l], L.kind, L.stage, h->lane_stream[l]);
      cudaError_t e2 = cudaStreamEndCapture(h->lane_stream[l], &g);
      if (e || e2) return cuda_fail(h, e ? e : e2, "capture");
      e = cudaGraphInstantiate(&h->lane_graph[l], g, 0);
      cudaGraphDestroy(g);
      if (e) { h->lane_graph[l] = nullptr; return cuda_fail(h, e, "graph instantiate"); }
    }
    if ((e = cudaEventRecord(h->lane_fork, h->stream))) return cuda_fail(h, e, "lanes");
    for (int l = 0; l < h->n_lanes; ++l)
      if ((e = cudaStreamWaitEvent(h->lane_stream[l], h->lane_fork, 0))) return cuda_fail(h, e, "lanes");
    for (int s = 0; s < n_steps && !e; ++s)
      for (int l = 0; l < h->n_lanes && !e; ++l) e = cudaGraphLaunch(h->lane_graph[l], h->lane_stream[l]);
    // join whatever was launched, also after a failed launch, so that work
    // enqueued on the handle's stream afterwards still follows the lanes
    cudaError_t ej = cudaSuccess;
    for (int l = 0; l < h->n_lanes && !ej; ++l)
      if (!(ej = cudaEventRecord(h->lane_join[l], h->lane_stream[l]))) ej = cudaStreamWaitEvent(h->stream, h->lane_join[l], 0);
    if (e) return cuda_fail(h, e, "graph launch");
    if (ej) return cuda_fail(h, ej, "lanes");
    return PZ_OK;
  }
  if (!h->graph) {
    cudaGraph_t g;
    if ((e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal))) return cuda_fail(h, e, "capture");
    for (const PzLaunch& L : fast ? h->fplan : h->plan)
      if (!e) e = pz_launch_step_kernel(fast ? h->fdev : h->dev, L.kind, L.stage, h->stream);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    if (e || e2) return cuda_fail(h, e ? e : e2, "capture");
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e) { h->graph = nullptr; return cuda_fail(h, e, "graph instantiate"); }
  }
  for (int s = 0; s < n_steps; ++s)
    if ((e = cudaGraphLaunch(h->graph, h->stream))) return cuda_fail(h, e, "graph launch");
  return PZ_OK;
}

extern "C" int pz_sync(pz_handle* h) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_sync: null handle");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_sync");
  return check_status(h);
}

extern "C" int pz_get_state(pz_handle* h, int inst, double* us, double* up, double* om, double* psi, double* temp,
                            double* dtemp, double* time, double* dt) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_state: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_get_state: instance out of range");
  const PzInst& I = h->inst[inst];
  const long long MN = (long long)I.M * I.N;
  std::vector<double> buf(2 * MN * F_COUNT);
  cudaError_t e = cudaMemcpyAsync(buf.data(), h->pool + I.o_fld, buf.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  h->stream);
  PzState st;
  if (!e) e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_state");
  double* outs[6] = {us, up, om, psi, temp, dtemp};
  const int fids[6] = {F_US, F_UP, F_OM, F_PSI, F_TEMP, F_DTEMP};
  for (int k = 0; k < 6; ++k) {
    if (!outs[k]) continue;
    const double* src = buf.data() + 2 * MN * fids[k];
    for (int r = 0; r < I.N; ++r)
      for (int m = 0; m < I.M; ++m) {
        outs[k][2 * (m + (long long)r * I.M)] = src[2 * ((long long)m * I.N + r)];
        outs[k][2 * (m + (long long)r * I.M) + 1] = src[2 * ((long long)m * I.N + r) + 1];
      }
  }
  if (time) *time = st.time;
  if (dt) *dt = st.dt[0];
  return st.status ? check_status(h) : PZ_OK;
}

extern "C" int pz_get_state_xi(pz_handle* h, int inst, double* xi, double* dxi) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_state_xi: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_get_state_xi: instance out of range");
  const PzInst& I = h->inst[inst];
  const long long MN = (long long)I.M * I.N;
  std::vector<double> buf(2 * MN * 2);
  cudaError_t e = cudaMemcpyAsync(buf.data(), h->pool + I.o_fld + 2LL * F_XI * MN, buf.size() * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_state_xi");
  double* outs[2] = {xi, dxi};
  for (int k = 0; k < 2; ++k) {
    if (!outs[k]) continue;
    const double* src = buf.data() + 2 * MN * k;
    for (int r = 0; r < I.N; ++r)
      for (int m = 0; m < I.M; ++m) {
        outs[k][2 * (m + (long long)r * I.M)] = src[2 * ((long long)m * I.N + r)];
        outs[k][2 * (m + (long long)r * I.M) + 1] = src[2 * ((long long)m * I.N + r) + 1];
      }
  }
  return PZ_OK;
}

namespace {
// physical ring slot of logical history slot `slot` (1-based) at a step boundary
int hist_phys(const PzInst& I, const PzState& st, int kind, int slot) {
  const int n = kind == 0 ? I.nold : (kind == 1 ? I.nimp : I.nexp);
  if (I.dirk) return slot - 1;
  const int base = kind == 0 ? st.b_old : (kind == 1 ? st.b_impl : st.b_expl);
  return (base + slot - 1) % n;
}
int hist_args(pz_handle* h, int inst, int field, int kind, int slot, const char* who) {
  if (!h) return fail(nullptr, PZ_E_ARG, std::string(who) + ": null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, std::string(who) + ": instance out of range");
  const PzInst& I = h->inst[inst];
  const int n = kind == 0 ? I.nold : (kind == 1 ? I.nimp : (kind == 2 ? I.nexp : 0));
  if (field < 0 || field >= I.nhf || kind < 0 || kind > 2 || slot < 1 || slot > n)
    return fail(h, PZ_E_ARG, std::string(who) + ": field, kind or slot out of range");
  return PZ_OK;
}
}  // namespace

extern "C" int pz_get_history(pz_handle* h, int inst, int field, int kind, int slot, double* out) {
  int rc = hist_args(h, inst, field, kind, slot, "pz_get_history");
  if (rc) return rc;
  if (!out) return fail(h, PZ_E_ARG, "pz_get_history: null output");
  const PzInst& I = h->inst[inst];
  const long long MN = (long long)I.M * I.N;
  PzState st;
  std::vector<double> buf(2 * MN);
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_history");
  const long long off = pz_hist_off(I, field, kind, hist_phys(I, st, kind, slot));
  e = cudaMemcpyAsync(buf.data(), h->pool + off, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_history");
  for (int r = 0; r < I.N; ++r)
    for (int m = 0; m < I.M; ++m) {
      out[2 * (m + (long long)r * I.M)] = buf[2 * ((long long)m * I.N + r)];
      out[2 * (m + (long long)r * I.M) + 1] = buf[2 * ((long long)m * I.N + r) + 1];
    }
  return PZ_OK;
}

extern "C" int pz_set_history(pz_handle* h, int inst, int field, int kind, int slot, const double* in) {
  int rc = hist_args(h, inst, field, kind, slot, "pz_set_history");
  if (rc) return rc;
  if (!in) return fail(h, PZ_E_ARG, "pz_set_history: null input");
  pz_adjoint_invalidate(h);
  const PzInst& I = h->inst[inst];
  const long long MN = (long long)I.M * I.N;
  PzState st;
  std::vector<double> buf(2 * MN);
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_set_history");
  for (int r = 0; r < I.N; ++r)
    for (int m = 0; m < I.M; ++m) {
      buf[2 * ((long long)m * I.N + r)] = in[2 * (m + (long long)r * I.M)];
      buf[2 * ((long long)m * I.N + r) + 1] = in[2 * (m + (long long)r * I.M) + 1];
    }
  const long long off = pz_hist_off(I, field, kind, hist_phys(I, st, kind, slot));
  e = cudaMemcpyAsync(h->pool + off, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);   // buf is pageable and local
  if (e) return cuda_fail(h, e, "pz_set_history");
  return PZ_OK;
}

extern "C" int pz_get_step_state(pz_handle* h, int inst, double* time, double* dt, int* n_step) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_step_state: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_get_step_state: instance out of range");
  PzState st;
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_step_state");
  const PzInst& I = h->inst[inst];
  if (time) *time = st.time;
  if (dt)
    for (int k = 0; k < (I.dirk ? 1 : I.nexp); ++k) dt[k] = st.dt[k];
  if (n_step) *n_step = st.n_step;
  return PZ_OK;
}

extern "C" int pz_set_step_state(pz_handle* h, int inst, double time, const double* dt, int n_step) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_set_step_state: null handle");
  if (inst < 0 || inst >= h->n_inst || !dt || n_step < 0)
    return fail(h, PZ_E_ARG, "pz_set_step_state: bad arguments");
  pz_adjoint_invalidate(h);
  const PzInst& I = h->inst[inst];
  const int nd = I.dirk ? 1 : I.nexp;
  for (int k = 0; k < nd; ++k)
    if (!(dt[k] > 0.0)) return fail(h, PZ_E_ARG, "pz_set_step_state: dt must be positive");
  PzState st;
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_set_step_state");
  st.time = time;
  for (int k = 0; k < nd; ++k) st.dt[k] = dt[k];
  st.n_step = n_step;
  st.lMatNext = 1;   // operators for the restored dt at the next step
  // the latest time-series row is rewritten with the restored time
  if (st.series_count > 0) st.series_count -= 1;
  e = cudaMemcpyAsync(h->d_state + inst, &st, sizeof(PzState), cudaMemcpyHostToDevice, h->stream);
  if (!e) e = pz_launch_obs(h->dev, inst, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_set_step_state");
  return PZ_OK;
}

extern "C" int pz_get_spectra(pz_handle* h, int inst, double* out) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_spectra: null handle");
  if (inst < 0 || inst >= h->n_inst || !out) return fail(h, PZ_E_ARG, "pz_get_spectra: bad arguments");
  const int M = h->inst[inst].M;
  cudaError_t e = pz_launch_spectra(h->dev, inst, M, h->d_spec, nullptr, h->stream);
  if (!e) e = cudaMemcpyAsync(out, h->d_spec, (size_t)5 * M * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_spectra");
  return PZ_OK;
}

extern "C" int pz_balance_step(pz_handle* h, int inst, double* vort, double* vp) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_balance_step: null handle");
  if (inst < 0 || inst >= h->n_inst || !vort || !vp) return fail(h, PZ_E_ARG, "pz_balance_step: bad arguments");
  const PzInst& I = h->inst[inst];
  if ((I.flags & (PZF_INTEG | PZF_DIRECT)) || I.dirk)
    return fail(h, PZ_E_UNSUPPORTED,
                "pz_balance_step: the force balances are computed for the collocation method with the "
                "influence-matrix solve and a multistep scheme");
  const long long MN = (long long)I.M * I.N, fld = 2LL * F_COUNT * MN;
  size_t need = 0;
  for (int i = 0; i < h->n_inst; ++i) {
    const long long mn = (long long)h->inst[i].M * h->inst[i].N;
    need = std::max(need, (size_t)(2LL * F_COUNT * mn + 12 * mn + 4LL * h->inst[i].N));
  }
  cudaError_t e = cudaSuccess;
  if (!h->d_bal) e = cudaMalloc(&h->d_bal, need * sizeof(double));
  if (e) { h->d_bal = nullptr; return cuda_fail(h, e, "pz_balance_step"); }
  double* snap = h->d_bal;
  double* dv = snap + fld;
  double* dp = dv + 12 * MN;
  e = cudaMemcpyAsync(snap, h->pool + I.o_fld, fld * sizeof(double), cudaMemcpyDeviceToDevice, h->stream);
  if (e) return cuda_fail(h, e, "pz_balance_step");
  int rc = pz_step(h, 1);
  if (rc) return rc;
  e = pz_launch_balance(h->dev, inst, I.M, snap, dv, dp, h->stream);
  if (!e) e = cudaMemcpyAsync(vort, dv, 12 * MN * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaMemcpyAsync(vp, dp, 4LL * I.N * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_balance_step");
  return check_status(h);
}

extern "C" int pz_get_spectra_2d(pz_handle* h, int inst, double* out) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_spectra_2d: null handle");
  if (inst < 0 || inst >= h->n_inst || !out) return fail(h, PZ_E_ARG, "pz_get_spectra_2d: bad arguments");
  const PzInst& I = h->inst[inst];
  cudaError_t e = pz_launch_spectra(h->dev, inst, I.M, h->d_spec, h->d_spec2d, h->stream);
  if (!e)
    e = cudaMemcpyAsync(out, h->d_spec2d, (size_t)3 * I.N * I.M * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_spectra_2d");
  return PZ_OK;
}

extern "C" int pz_set_restart_ab1(pz_handle* h, int inst, int l_ab1) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_set_restart_ab1: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_set_restart_ab1: bad arguments");
  pz_adjoint_invalidate(h);
  PzState st;
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_set_restart_ab1");
  st.ab1 = l_ab1 ? 1 : 0;
  e = cudaMemcpyAsync(h->d_state + inst, &st, sizeof(PzState), cudaMemcpyHostToDevice, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_set_restart_ab1");
  return PZ_OK;
}

extern "C" int pz_get_series(pz_handle* h, int inst, double* rows, int* n_rows) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_series: null handle");
  if (inst < 0 || inst >= h->n_inst || !n_rows) return fail(h, PZ_E_ARG, "pz_get_series: bad arguments");
  const PzInst& I = h->inst[inst];
  PzState st;
  std::vector<double> buf((size_t)PZ_SERIES_CAP * PZ_SERIES_COLS);
  cudaError_t e = cudaMemcpyAsync(&st, h->d_state + inst, sizeof(PzState), cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaMemcpyAsync(buf.data(), h->pool + I.o_series, buf.size() * sizeof(double), cudaMemcpyDeviceToHost,
                              h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_get_series");
  const int have = std::min(st.series_count, PZ_SERIES_CAP);
  const int want = std::min(have, *n_rows);
  for (int k = 0; k < want; ++k) {
    const int idx = (st.series_count - want + k) % PZ_SERIES_CAP;
    if (rows) std::memcpy(rows + (size_t)k * PZ_SERIES_COLS, buf.data() + (size_t)idx * PZ_SERIES_COLS,
                          PZ_SERIES_COLS * sizeof(double));
  }
  *n_rows = want;
  return PZ_OK;
}

extern "C" int pz_get_dims(pz_handle* h, int inst, int* n_r_max, int* n_m_max, int* n_phi_max) {
  if (!h) return fail(nullptr, PZ_E_ARG, "pz_get_dims: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "pz_get_dims: instance out of range");
  if (n_r_max) *n_r_max = h->inst[inst].N;
  if (n_m_max) *n_m_max = h->inst[inst].M;
  if (n_phi_max) *n_phi_max = h->inst[inst].P;
  return PZ_OK;
}

extern "C" int pz_launches_per_step(pz_handle* h) {
  if (!h) return 0;
  return (int)(h->n_fast > 0 ? h->fplan.size() * h->n_lanes : h->plan.size());
}

extern "C" int pz_latest_rows(pz_handle* h, double* rows) {
  if (!h || !rows) return fail(h, PZ_E_ARG, "pz_latest_rows: bad arguments");
  cudaError_t e = pz_launch_gather_rows(h->dev, h->d_rows, h->stream);
  if (!e) e = cudaMemcpyAsync(rows, h->d_rows, (size_t)h->n_inst * PZ_SERIES_COLS * sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return cuda_fail(h, e, "pz_latest_rows");
  return PZ_OK;
}

extern "C" void* pz_stream(pz_handle* h) { return h ? (void*)h->stream : nullptr; }

extern "C" int pz_step_profile(pz_handle* h, int n_steps, double* kernel_ms) {
  if (!h || n_steps <= 0 || !kernel_ms) return fail(h, PZ_E_ARG, "pz_step_profile: bad arguments");
  pz_adjoint_invalidate(h);
  // the launches of pz_step (the fast plan when the handle has fast instances)
  const std::vector<PzLaunch>& plan = h->n_fast > 0 ? h->fplan : h->plan;
  const PzDev& dv = h->n_fast > 0 ? h->fdev : h->dev;
  const int nk = (int)plan.size();
  std::vector<cudaEvent_t> ev((size_t)n_steps * (nk + 1));
  cudaError_t e = cudaSuccess;
  for (auto& x : ev) if (!e) e = cudaEventCreate(&x);
  if (e) return cuda_fail(h, e, "pz_step_profile events");
  for (int s = 0; s < n_steps && !e; ++s) {
    e = cudaEventRecord(ev[(size_t)s * (nk + 1)], h->stream);
    for (int k = 0; k < nk && !e; ++k) {
      e = pz_launch_step_kernel(dv, plan[k].kind, plan[k].stage, h->stream);
      if (!e) e = cudaEventRecord(ev[(size_t)s * (nk + 1) + k + 1], h->stream);
    }
  }
  if (!e) e = cudaStreamSynchronize(h->stream);
  for (int k = 0; k < PZ_KERNEL_KINDS; ++k) kernel_ms[k] = 0.0;
  for (int s = 0; s < n_steps && !e; ++s)
    for (int k = 0; k < nk && !e; ++k) {
      float ms = 0.f;
      e = cudaEventElapsedTime(&ms, ev[(size_t)s * (nk + 1) + k], ev[(size_t)s * (nk + 1) + k + 1]);
      kernel_ms[plan[k].kind] += ms / n_steps;
    }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e) return cuda_fail(h, e, "pz_step_profile");
  return check_status(h);
}

extern "C" const char* pz_kernel_name(int k) { return pz_step_kernel_name(k); }

extern "C" int pz_integ_operator(int n_r_max, double radratio, int which, double* out, int* bandwidth) {
  static_assert(PZ_INTEG_OPS == IM_COUNT, "operator count");
  if (n_r_max < 5 || n_r_max > 1024 || !(radratio > 0.0 && radratio < 1.0) || which < 0 || which >= IM_COUNT ||
      !out || !bandwidth)
    return fail(nullptr, PZ_E_ARG, "pz_integ_operator: bad arguments");
  const double r_cmb = 1.0 / (1.0 - radratio), r_icb = r_cmb - 1.0;
  std::vector<double> ops;
  int band[IM_COUNT];
  pz_integ_operators(n_r_max, r_icb, r_cmb, std::sqrt(2.0 / (double)(n_r_max - 1)), ops, band);
  const size_t nn = (size_t)n_r_max * n_r_max;
  std::memcpy(out, ops.data() + (size_t)which * nn, nn * sizeof(double));
  *bandwidth = band[which];
  return PZ_OK;
}

extern "C" int pz_explicit_terms(pz_handle* h, int inst, const double* us, const double* up, const double* om,
                                 const double* temp, double* dTdt_expl, double* dpsidt_expl, double* dtr,
                                 double* dth) {
  // the same argument checks as pz_explicit_terms_noalloc (collocation
  // instances without composition), then scratch from the handle's stream
  PzExplArgs a;
  int N = 0, M = 0, P = 0;
  cudaStream_t s = nullptr;
  const int rc = pz_expl_args(h, inst, us, up, om, temp, dTdt_expl, dpsidt_expl, dtr, dth, &a, &N, &M, &P, &s);
  if (rc != PZ_OK) return rc;
  void* scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&scratch, pz_expl_scratch_bytes(N, M), s);
  if (e) return cuda_fail(h, e, "pz_explicit_terms scratch");
  a.s_dVsT = reinterpret_cast<double2*>(scratch);
  a.s_dVsOm = a.s_dVsT + (size_t)N * M;
  e = pz_launch_explicit_terms(a, N, M, P, s);
  const cudaError_t e2 = cudaFreeAsync(scratch, s);
  if (e) return cuda_fail(h, e, "pz_explicit_terms");
  if (e2) return cuda_fail(h, e2, "pz_explicit_terms scratch release");
  return PZ_OK;
}

int pz_expl_args(pz_handle* h, int inst, const double* us, const double* up, const double* om, const double* temp,
                 double* dTdt_expl, double* dpsidt_expl, double* dtr, double* dth, PzExplArgs* a, int* N, int* M,
                 int* P, cudaStream_t* s) {
  if (!h) return fail(nullptr, PZ_E_ARG, "explicit terms entry point: null handle");
  if (inst < 0 || inst >= h->n_inst) return fail(h, PZ_E_ARG, "explicit terms entry point: instance out of range");
  if (!us || !up || !om || !temp || !dTdt_expl || !dpsidt_expl || !dtr || !dth)
    return fail(h, PZ_E_ARG, "explicit terms entry point: null array");
  const PzInst& I = h->inst[inst];
  if (I.flags & PZF_INTEG)
    return fail(h, PZ_E_UNSUPPORTED, "explicit terms entry point: collocation instances only (cheb_method 'integ')");
  if (I.flags & PZF_CHEM)
    return fail(h, PZ_E_UNSUPPORTED, "explicit terms entry point: instances without composition only");
  a->inst = h->d_inst + inst;
  a->pool = h->pool;
  a->us = reinterpret_cast<const double2*>(us);
  a->up = reinterpret_cast<const double2*>(up);
  a->om = reinterpret_cast<const double2*>(om);
  a->temp = reinterpret_cast<const double2*>(temp);
  a->dTdt = reinterpret_cast<double2*>(dTdt_expl);
  a->dpsidt = reinterpret_cast<double2*>(dpsidt_expl);
  a->dtr = dtr;
  a->dth = dth;
  a->s_dVsT = nullptr;
  a->s_dVsOm = nullptr;
  *N = I.N;
  *M = I.M;
  *P = I.P;
  *s = h->stream;
  return PZ_OK;
}

int pz_record_error(pz_handle* h, int code, const char* msg) { return fail(h, code, msg); }

extern "C" int pz_destroy(pz_handle* h) {
  if (!h) return PZ_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  pz_adjoint_free(h);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (int l = 0; l < PZ_LANES_MAX; ++l)
    if (h->lane_graph[l]) cudaGraphExecDestroy(h->lane_graph[l]);
  cudaFree(h->pool);
  cudaFree(h->d_inst);
  cudaFree(h->d_state);
  cudaFree(h->d_ritems);
  cudaFree(h->d_mitems);
  cudaFree(h->d_order);
  cudaFree(h->d_iorder);
  cudaFree(h->d_rows);
  cudaFree(h->d_spec);
  cudaFree(h->d_spec2d);
  cudaFree(h->d_bal);
  cudaFree(h->d_oitems);
  cudaFree(h->d_obs_part);
  cudaFree(h->d_obs_cnt);
  cudaFree(h->d_fast);
  cudaFree(h->d_mitems_std);
  cudaFree(h->d_iorder_std);
  cudaFree(h->d_lane_inst);
  for (int l = 0; l < PZ_LANES_MAX; ++l) {
    if (h->lane_stream[l]) cudaStreamDestroy(h->lane_stream[l]);
    if (h->lane_join[l]) cudaEventDestroy(h->lane_join[l]);
  }
  if (h->lane_fork) cudaEventDestroy(h->lane_fork);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PZ_OK;
}

extern "C" const char* pz_last_error(pz_handle* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

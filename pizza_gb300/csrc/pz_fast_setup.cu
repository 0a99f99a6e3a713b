// Host set-up of the tensor-core stage (pz_fast.h): the eigen-decompositions
// of the interior Laplacians, the operators of the stage built from them,
// and their bf16 slices laid out as mma.sync A fragments.
//
// Everything here runs once at pz_create, in FP64 (plain double arithmetic,
// so that the host image is computed alike, and quickly, on every host), for
// each (n_r_max, radratio) class of instances that take the fast path and
// each m < n_m_max of the class.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pz_fast.h"
#include "pz_fast_setup.h"

namespace {

const double kEps = 2.220446049250313e-16;

// ---------------------------------------------------------------------------
// real eigen-decomposition of a matrix whose eigenvalues are real and
// distinct: A = U diag(lam) U^-1 (A, U, Uinv row-major n x n)
// ---------------------------------------------------------------------------
// Householder reduction to upper Hessenberg form, H = Q^T A Q.
void hessenberg(int n, std::vector<double>& H, std::vector<double>& Q) {
  Q.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
  std::vector<double> v(n);
  for (int k = 0; k + 2 < n; ++k) {
    double a2 = 0.0;
    for (int i = k + 1; i < n; ++i) a2 += H[(size_t)i * n + k] * H[(size_t)i * n + k];
    if (a2 == 0.0) continue;
    double alpha = std::sqrt(a2);
    if (H[(size_t)(k + 1) * n + k] > 0.0) alpha = -alpha;
    double vv = 0.0;
    for (int i = k + 1; i < n; ++i) v[i] = H[(size_t)i * n + k];
    v[k + 1] -= alpha;
    for (int i = k + 1; i < n; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    const double beta = 2.0 / vv;
    for (int j = 0; j < n; ++j) {                 // H = (I - beta v v^T) H
      double s = 0.0;
      for (int i = k + 1; i < n; ++i) s += v[i] * H[(size_t)i * n + j];
      s *= beta;
      for (int i = k + 1; i < n; ++i) H[(size_t)i * n + j] -= s * v[i];
    }
    for (int i = 0; i < n; ++i) {                 // H = H (I - beta v v^T), Q = Q (I - beta v v^T)
      double s = 0.0, t = 0.0;
      for (int j = k + 1; j < n; ++j) { s += H[(size_t)i * n + j] * v[j]; t += Q[(size_t)i * n + j] * v[j]; }
      s *= beta; t *= beta;
      for (int j = k + 1; j < n; ++j) { H[(size_t)i * n + j] -= s * v[j]; Q[(size_t)i * n + j] -= t * v[j]; }
    }
    for (int i = k + 2; i < n; ++i) H[(size_t)i * n + k] = 0.0;
  }
}

// Eigenvalues of an upper Hessenberg matrix by shifted QR with Givens
// rotations (Wilkinson shift, deflation on small subdiagonals).  False when
// an eigenvalue does not converge or a complex pair remains.
bool hess_eigvals(int n, std::vector<double> T, std::vector<double>& lam, double hnorm) {
  lam.assign(n, 0.0);
  std::vector<double> cs(n), sn(n);
  int hi = n - 1, iter = 0;
  while (hi >= 0) {
    if (hi == 0) { lam[0] = T[0]; break; }
    int l = hi;
    while (l > 0) {
      double s = std::fabs(T[(size_t)(l - 1) * n + l - 1]) + std::fabs(T[(size_t)l * n + l]);
      if (s == 0.0) s = hnorm;
      if (std::fabs(T[(size_t)l * n + l - 1]) <= kEps * s) { T[(size_t)l * n + l - 1] = 0.0; break; }
      --l;
    }
    if (l == hi) { lam[hi] = T[(size_t)hi * n + hi]; --hi; iter = 0; continue; }
    if (++iter > 200) return false;
    const double a = T[(size_t)(hi - 1) * n + hi - 1], b = T[(size_t)(hi - 1) * n + hi];
    const double c = T[(size_t)hi * n + hi - 1], d = T[(size_t)hi * n + hi];
    const double htr = 0.5 * (a + d), disc = htr * htr - (a * d - b * c);
    double mu = d;
    if (disc >= 0.0) {
      const double sq = std::sqrt(disc), e1 = htr + sq, e2 = htr - sq;
      mu = std::fabs(e1 - d) < std::fabs(e2 - d) ? e1 : e2;
    }
    if (iter % 20 == 19) mu = d + std::fabs(c);   // exceptional shift
    for (int k = l; k <= hi; ++k) T[(size_t)k * n + k] -= mu;
    for (int k = l; k < hi; ++k) {
      const double x = T[(size_t)k * n + k], y = T[(size_t)(k + 1) * n + k];
      const double r = std::hypot(x, y);
      const double cc = r == 0.0 ? 1.0 : x / r, ss = r == 0.0 ? 0.0 : y / r;
      cs[k] = cc; sn[k] = ss;
      for (int j = k; j <= hi; ++j) {
        const double t1 = T[(size_t)k * n + j], t2 = T[(size_t)(k + 1) * n + j];
        T[(size_t)k * n + j] = cc * t1 + ss * t2;
        T[(size_t)(k + 1) * n + j] = -ss * t1 + cc * t2;
      }
    }
    for (int k = l; k < hi; ++k) {
      const double cc = cs[k], ss = sn[k];
      const int top = k + 2 < hi ? k + 2 : hi;
      for (int i = l; i <= top; ++i) {
        const double t1 = T[(size_t)i * n + k], t2 = T[(size_t)i * n + k + 1];
        T[(size_t)i * n + k] = cc * t1 + ss * t2;
        T[(size_t)i * n + k + 1] = -ss * t1 + cc * t2;
      }
    }
    for (int k = l; k <= hi; ++k) T[(size_t)k * n + k] += mu;
  }
  return true;
}

// LU with partial pivoting of a dense n x n row-major matrix, in place.
bool lu_factor(int n, std::vector<double>& A, std::vector<int>& piv) {
  piv.resize(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[(size_t)i * n + k]) > std::fabs(A[(size_t)p * n + k])) p = i;
    piv[k] = p;
    if (A[(size_t)p * n + k] == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
    const double inv = 1.0 / A[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double l = A[(size_t)i * n + k] * inv;
      A[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; ++j) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
    }
  }
  return true;
}
// P A = L U with whole rows swapped (the multipliers move with their rows):
// apply every interchange to b first, then the two triangular solves
void lu_solve(int n, const std::vector<double>& LU, const std::vector<int>& piv, double* b) {
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
  for (int k = 0; k < n; ++k)
    for (int i = k + 1; i < n; ++i) b[i] -= LU[(size_t)i * n + k] * b[k];
  for (int k = n - 1; k >= 0; --k) {
    double s = b[k];
    for (int j = k + 1; j < n; ++j) s -= LU[(size_t)k * n + j] * b[j];
    b[k] = s / LU[(size_t)k * n + k];
  }
}
// inverse of a dense row-major matrix (false if singular)
bool invert(int n, const std::vector<double>& A, std::vector<double>& Ainv) {
  std::vector<double> LU = A;
  std::vector<int> piv;
  if (!lu_factor(n, LU, piv)) return false;
  Ainv.assign((size_t)n * n, 0.0);
  std::vector<double> col(n);
  for (int j = 0; j < n; ++j) {
    std::fill(col.begin(), col.end(), 0.0);
    col[j] = 1.0;
    lu_solve(n, LU, piv, col.data());
    for (int i = 0; i < n; ++i) Ainv[(size_t)i * n + j] = col[i];
  }
  return true;
}

// Eigenvector of the Hessenberg matrix H for eigenvalue lam by inverse
// iteration: two solves with (H - lam I), LU with row interchanges between
// neighbouring rows only (Hessenberg structure); tiny pivots are lifted to
// eps |H|.
void hess_eigvec(int n, const std::vector<double>& H, double lam, double hnorm, std::vector<double>& y) {
  std::vector<double> Mx(H);
  for (int i = 0; i < n; ++i) Mx[(size_t)i * n + i] -= lam;
  std::vector<char> sw(n, 0);
  std::vector<double> mult(n, 0.0);
  const double tiny = kEps * hnorm;
  for (int k = 0; k + 1 < n; ++k) {
    if (std::fabs(Mx[(size_t)(k + 1) * n + k]) > std::fabs(Mx[(size_t)k * n + k])) {
      sw[k] = 1;
      for (int j = k; j < n; ++j) std::swap(Mx[(size_t)k * n + j], Mx[(size_t)(k + 1) * n + j]);
    }
    if (Mx[(size_t)k * n + k] == 0.0) Mx[(size_t)k * n + k] = tiny;
    const double l = Mx[(size_t)(k + 1) * n + k] / Mx[(size_t)k * n + k];
    mult[k] = l;
    for (int j = k + 1; j < n; ++j) Mx[(size_t)(k + 1) * n + j] -= l * Mx[(size_t)k * n + j];
  }
  if (Mx[(size_t)(n - 1) * n + n - 1] == 0.0) Mx[(size_t)(n - 1) * n + n - 1] = tiny;
  y.assign(n, 0.0);
  for (int i = 0; i < n; ++i) y[i] = 1.0 + 0.5 * std::sin(1.0 + 0.37 * i);   // generic start
  for (int it = 0; it < 3; ++it) {
    for (int k = 0; k + 1 < n; ++k) {
      if (sw[k]) std::swap(y[k], y[k + 1]);
      y[k + 1] -= mult[k] * y[k];
    }
    for (int k = n - 1; k >= 0; --k) {
      double s = y[k];
      for (int j = k + 1; j < n; ++j) s -= Mx[(size_t)k * n + j] * y[j];
      const double p = Mx[(size_t)k * n + k];
      y[k] = s / (std::fabs(p) < tiny ? (p < 0 ? -tiny : tiny) : p);
    }
    double mx = 0.0;
    for (int i = 0; i < n; ++i) mx = std::max(mx, std::fabs(y[i]));
    for (int i = 0; i < n; ++i) y[i] /= mx;
  }
}

}  // namespace

// A = U diag(lam) U^-1 for a real n x n row-major A with real distinct
// eigenvalues.  Columns of U have max-norm 1 with a positive largest entry.
// Returns false (and leaves the outputs unspecified) when the decomposition
// fails or its residual |A U - U diag(lam)| / (|A| |U|) or |U U^-1 - I|
// exceeds 1e-10.
bool pz_eig_real(int n, const std::vector<double>& A, std::vector<double>& lam, std::vector<double>& U,
                 std::vector<double>& Uinv) {
  double anorm = 0.0;
  for (double v : A) anorm = std::max(anorm, std::fabs(v));
  if (anorm == 0.0) return false;
  std::vector<double> H = A, Q;
  hessenberg(n, H, Q);
  if (!hess_eigvals(n, H, lam, anorm)) return false;
  U.assign((size_t)n * n, 0.0);
  std::vector<double> y;
  for (int k = 0; k < n; ++k) {
    hess_eigvec(n, H, lam[k], anorm, y);
    double mx = 0.0;
    int im = 0;
    for (int i = 0; i < n; ++i) {            // v = Q y
      double s = 0.0;
      for (int j = 0; j < n; ++j) s += Q[(size_t)i * n + j] * y[j];
      U[(size_t)i * n + k] = (double)s;
      if (std::fabs((double)s) > mx) { mx = std::fabs((double)s); im = i; }
    }
    const double sc = (U[(size_t)im * n + k] < 0.0 ? -1.0 : 1.0) / mx;
    for (int i = 0; i < n; ++i) U[(size_t)i * n + k] *= sc;
  }
  if (!invert(n, U, Uinv)) return false;
  double r1 = 0.0, r2 = 0.0;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      double s = 0.0, t = 0.0;
      for (int j = 0; j < n; ++j) {
        s += A[(size_t)i * n + j] * U[(size_t)j * n + k];
        t += U[(size_t)i * n + j] * Uinv[(size_t)j * n + k];
      }
      r1 = std::max(r1, std::fabs(s - U[(size_t)i * n + k] * lam[k]));
      r2 = std::max(r2, std::fabs((double)t - (i == k ? 1.0 : 0.0)));
    }
  return r1 <= 1e-10 * anorm && r2 <= 1e-10;
}

namespace {

// ---------------------------------------------------------------------------
// operators of one (N, m) and their mma fragments
// ---------------------------------------------------------------------------
inline uint16_t bf16_of_int(double d) {
  const float f = (float)d;   // |d| <= 256: exact
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

// Append operator A (R x K row-major, FP64) to the fragment arrays.
PzOzOp add_op(PzFastHost& H, const std::vector<double>& A, int R, int K) {
  PzOzOp op;
  op.R = R; op.K = K;
  op.RT = (R + 15) / 16; op.KT = (K + 15) / 16;
  op.frag = (long long)H.frag.size();
  op.ex = (long long)H.ex.size();
  const int Rp = op.RT * 16, Kp = op.KT * 16;
  // slices s, row-major Rp x Kp
  std::vector<uint16_t> sl((size_t)PZ_OZ_S * Rp * Kp, 0);
  H.ex.resize(H.ex.size() + Rp, 0);
  for (int r = 0; r < R; ++r) {
    double mx = 0.0;
    for (int j = 0; j < K; ++j) mx = std::max(mx, std::fabs(A[(size_t)r * K + j]));
    int e = 0;
    if (mx > 0.0) std::frexp(mx, &e);          // mx < 2^e
    H.ex[op.ex + r] = e;
    for (int j = 0; j < K; ++j) {
      double v = std::ldexp(A[(size_t)r * K + j], 8 - e);
      for (int s = 0; s < PZ_OZ_S; ++s) {
        const double d = std::nearbyint(v);
        sl[((size_t)s * Rp + r) * Kp + j] = bf16_of_int(d);
        v = (v - d) * 256.0;
      }
    }
  }
  H.frag.resize(H.frag.size() + (size_t)op.RT * op.KT * PZ_OZ_S * 32);
  for (int rt = 0; rt < op.RT; ++rt)
    for (int kt = 0; kt < op.KT; ++kt)
      for (int s = 0; s < PZ_OZ_S; ++s)
        for (int lane = 0; lane < 32; ++lane) {
          const int g = lane >> 2, t = lane & 3;
          auto at = [&](int r, int k) -> uint32_t { return sl[((size_t)s * Rp + rt * 16 + r) * Kp + kt * 16 + k]; };
          auto pk = [&](int r, int k) -> uint32_t { return at(r, k) | (at(r, k + 1) << 16); };
          uint4 q;
          q.x = pk(g, 2 * t);
          q.y = pk(g + 8, 2 * t);
          q.z = pk(g, 2 * t + 8);
          q.w = pk(g + 8, 2 * t + 8);
          H.frag[op.frag + (((size_t)rt * op.KT + kt) * PZ_OZ_S + s) * 32 + lane] = q;
        }
  return op;
}

// C = A B, A (r x k) and B (k x c) row-major
std::vector<double> mm(const std::vector<double>& A, const std::vector<double>& B, int r, int k, int c) {
  std::vector<double> C((size_t)r * c);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) {
      double s = 0.0;
      for (int q = 0; q < k; ++q) s += A[(size_t)i * k + q] * B[(size_t)q * c + j];
      C[(size_t)i * c + j] = (double)s;
    }
  return C;
}

}  // namespace

void pz_fast_laplacian(const PzFastGrid& g, double m2, std::vector<double>& P, std::vector<double>& Pb) {
  const int N = g.N, n = N - 2;
  auto at = [N](const double* cm, int i, int j) { return cm[i + (size_t)j * N]; };
  P.assign((size_t)n * n, 0.0);
  Pb.assign((size_t)n * 2, 0.0);
  for (int i = 0; i < n; ++i) {
    const int r = i + 1;
    for (int j = 0; j < N; ++j) {
      const double lap = at(g.D2p, r, j) + g.or1[r] * at(g.D1p, r, j);
      if (j == 0) Pb[(size_t)i * 2 + 0] = lap;
      else if (j == N - 1) Pb[(size_t)i * 2 + 1] = lap;
      else P[(size_t)i * n + j - 1] = lap - (j == r ? m2 * g.or2[r] : 0.0);
    }
  }
}

bool pz_fast_add_class(PzFastHost& H, const PzFastGrid& g, int Mc, int minc, int* index) {
  const int N = g.N, n = N - 2;
  PzFastCls cls;
  cls.N = N; cls.n = n; cls.Mc = Mc;
  cls.m0 = (long long)H.ms.size();
  // D1p (N x N), row-major
  auto at = [N](const double* cm, int i, int j) { return cm[i + (size_t)j * N]; };   // column-major input
  std::vector<double> d1p((size_t)N * N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) d1p[(size_t)i * N + j] = at(g.D1p, i, j);
  cls.d1p = add_op(H, d1p, N, N);
  // D1p restricted to the interior columns, N x n
  std::vector<double> d1pI((size_t)N * n);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < n; ++j) d1pI[(size_t)i * n + j] = at(g.D1p, i, j + 1);
  for (int mi = 0; mi < Mc; ++mi) {
    const double m = (double)(mi * minc), m2 = m * m;
    std::vector<double> P, Pb, L((size_t)n * n);
    pz_fast_laplacian(g, m2, P, Pb);
    for (int i = 0; i < n; ++i) {
      const int r = i + 1;
      for (int j = 1; j < N - 1; ++j)
        L[(size_t)i * n + j - 1] = at(g.D2p, r, j) + (g.or1[r] + g.beta[r]) * at(g.D1p, r, j) +
                                   (j == r ? g.or1[r] * g.beta[r] + g.dbeta[r] - m2 * g.or2[r] : 0.0);
    }
    std::vector<double> lam, U, Uinv, Linv;
    if (!pz_eig_real(n, P, lam, U, Uinv)) return false;
    // psi interior from omega interior: psi_I = K omega_I, K = -(L_II)^-1
    if (!invert(n, L, Linv)) return false;
    for (double& v : Linv) v = -v;
    const std::vector<double> KU = mm(Linv, U, n, n, n);
    const std::vector<double> D1pU = mm(d1pI, U, N, n, n);
    const std::vector<double> D1pKU = mm(d1pI, KU, N, n, n);
    std::vector<double> s3t((size_t)(n + N) * n), s3w((size_t)(2 * n + N) * n);
    std::memcpy(s3t.data(), U.data(), sizeof(double) * n * n);
    std::memcpy(s3t.data() + (size_t)n * n, D1pU.data(), sizeof(double) * N * n);
    std::memcpy(s3w.data(), U.data(), sizeof(double) * n * n);
    std::memcpy(s3w.data() + (size_t)n * n, KU.data(), sizeof(double) * n * n);
    std::memcpy(s3w.data() + (size_t)2 * n * n, D1pKU.data(), sizeof(double) * N * n);
    PzFastM fm;
    fm.uinv = add_op(H, Uinv, n, n);
    fm.s3t = add_op(H, s3t, n + N, n);
    fm.s3w = add_op(H, s3w, 2 * n + N, n);
    // vectors: lam, U^-1 P_Ib (top, bottom wall), dpsi/dr rows at the walls
    fm.vec = (long long)H.vec.size();
    const std::vector<double> gb = mm(Uinv, Pb, n, n, 2);
    H.vec.insert(H.vec.end(), lam.begin(), lam.end());
    for (int k = 0; k < n; ++k) H.vec.push_back(gb[(size_t)k * 2 + 0]);
    for (int k = 0; k < n; ++k) H.vec.push_back(gb[(size_t)k * 2 + 1]);
    for (int k = 0; k < n; ++k) H.vec.push_back(D1pKU[(size_t)0 * n + k]);
    for (int k = 0; k < n; ++k) H.vec.push_back(D1pKU[(size_t)(N - 1) * n + k]);
    H.ms.push_back(fm);
  }
  *index = (int)H.cls.size();
  H.cls.push_back(cls);
  return true;
}

bool pz_fast_add_uclass(PzFastHost& H, const PzFastGrid& g, double visc, double corfac, const double* ekpump,
                        int* index) {
  const int N = g.N, n = N - 2;
  auto at = [N](const double* cm, int i, int j) { return cm[i + (size_t)j * N]; };
  std::vector<double> P((size_t)n * n), d1pI((size_t)N * n);
  for (int i = 0; i < n; ++i) {
    const int r = i + 1;
    for (int j = 1; j < N - 1; ++j)
      P[(size_t)i * n + j - 1] = visc * (at(g.D2p, r, j) + g.or1[r] * at(g.D1p, r, j)) -
                                 (j == r ? visc * g.or2[r] + corfac * ekpump[r] : 0.0);
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < n; ++j) d1pI[(size_t)i * n + j] = at(g.D1p, i, j + 1);
  std::vector<double> lam, U, Uinv;
  if (!pz_eig_real(n, P, lam, U, Uinv)) return false;
  const std::vector<double> D1pU = mm(d1pI, U, N, n, n);
  std::vector<double> s3u((size_t)(n + N) * n);
  std::memcpy(s3u.data(), U.data(), sizeof(double) * n * n);
  std::memcpy(s3u.data() + (size_t)n * n, D1pU.data(), sizeof(double) * N * n);
  PzFastU fu;
  fu.uinv = add_op(H, Uinv, n, n);
  fu.s3u = add_op(H, s3u, n + N, n);
  fu.vec = (long long)H.vec.size();
  H.vec.insert(H.vec.end(), lam.begin(), lam.end());
  *index = (int)H.us.size();
  H.us.push_back(fu);
  return true;
}

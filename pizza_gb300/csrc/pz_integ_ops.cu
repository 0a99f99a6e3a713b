// Host-side derivation of the banded operators of pizza's Chebyshev
// integration method (src/chebsparselib.f90, used by update_temp_integ.f90,
// update_xi_integ.f90 and update_psi_integ_smat.f90).
//
// Coefficients follow pizza's DCT-I convention f = c_0/2 + sum_{n>=1} c_n T_n
// with x = (r - b)/a.  Every operator is I_k [sum_d P_d(r) f^(d)] -- an
// equation multiplied by a power of r and integrated k times -- and repeated
// integration by parts,
//     I_k (p f^(j)) = sum_i (-1)^i C(j,i) I_{k-j+i} (p^(i) f)   (rows >= k),
// reduces it to two exact banded primitives: multiplication by r and one
// integration.  The constants of integration only touch rows < k, which the
// tau rows replace; those rows are zeroed here.  The matrices are derived
// once per (N, radratio) with sparse-aware products on padded (N + 20)
// squares so that the leading N x N block is exact.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "pz_internal.h"

namespace {

using Poly = std::vector<double>;   // power-series coefficients in r

Poly pmul(const Poly& a, const Poly& b) {
  Poly c(a.size() + b.size() - 1, 0.0);
  for (size_t i = 0; i < a.size(); ++i)
    for (size_t j = 0; j < b.size(); ++j) c[i + j] += a[i] * b[j];
  return c;
}
Poly padd(const Poly& a, const Poly& b) {
  Poly c(std::max(a.size(), b.size()), 0.0);
  for (size_t i = 0; i < a.size(); ++i) c[i] += a[i];
  for (size_t i = 0; i < b.size(); ++i) c[i] += b[i];
  return c;
}
Poly pscale(const Poly& a, double s) {
  Poly c(a);
  for (double& v : c) v *= s;
  return c;
}
Poly pder(const Poly& a, int k) {
  Poly c(a);
  for (int t = 0; t < k; ++t) {
    if (c.size() <= 1) return Poly{0.0};
    Poly d(c.size() - 1);
    for (size_t i = 1; i < c.size(); ++i) d[i - 1] = (double)i * c[i];
    c = d;
  }
  return c;
}
Poly rpow(int p) {
  Poly c((size_t)p + 1, 0.0);
  c[(size_t)p] = 1.0;
  return c;
}

// one term P_d(r) f^(d) of an operator
struct Term { int d; Poly P; };
using Terms = std::vector<Term>;

void add_term(Terms& t, int d, const Poly& P) {
  for (Term& x : t)
    if (x.d == d) { x.P = padd(x.P, P); return; }
  t.push_back({d, P});
}

// row-major L x L with products that skip zeros of the left factor (the
// factors are banded)
struct Sq {
  int L;
  std::vector<double> a;
  explicit Sq(int L_) : L(L_), a((size_t)L_ * L_, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i * L + j]; }
  double operator()(int i, int j) const { return a[(size_t)i * L + j]; }
};
Sq mul(const Sq& A, const Sq& B) {
  const int L = A.L;
  Sq C(L);
  for (int i = 0; i < L; ++i)
    for (int k = 0; k < L; ++k) {
      const double v = A(i, k);
      if (v == 0.0) continue;
      const double* b = &B.a[(size_t)k * L];
      double* c = &C.a[(size_t)i * L];
      for (int j = 0; j < L; ++j) c[j] += v * b[j];
    }
  return C;
}
Sq axpy(const Sq& A, double s, const Sq& B) {   // A + s B
  Sq C(A);
  for (size_t i = 0; i < C.a.size(); ++i) C.a[i] += s * B.a[i];
  return C;
}

class Prims {
 public:
  Prims(int n, double a, double b) : L_(n + 20), R_(L_), I1_(L_) {
    // x T_j = (T_{j+1} + T_{|j-1|})/2 and int T_j (standard coefficients),
    // converted to the c_0/2 convention: primed = P^-1 std P, P = diag(1/2, 1, ...)
    Sq X(L_), J(L_);
    for (int j = 0; j < L_; ++j) {
      if (j == 0) { X(1, 0) = 1.0; continue; }
      if (j + 1 < L_) X(j + 1, j) += 0.5;
      X(j - 1, j) += 0.5;
    }
    for (int k = 1; k < L_; ++k) {
      if (k == 1) J(1, 0) = 1.0;
      else J(k, k - 1) = 0.5 / k;
      if (k + 1 < L_) J(k, k + 1) = -0.5 / k;
    }
    for (int i = 0; i < L_; ++i)
      for (int j = 0; j < L_; ++j) {
        const double pin = (i == 0) ? 2.0 : 1.0, p = (j == 0) ? 0.5 : 1.0;
        R_(i, j) = a * pin * X(i, j) * p + (i == j ? b : 0.0);
        I1_(i, j) = a * pin * J(i, j) * p;
      }
    Sq E(L_);
    for (int i = 0; i < L_; ++i) E(i, i) = 1.0;
    Ik_.push_back(E);
  }
  int L() const { return L_; }
  const Sq& Ik(int k) {
    while ((int)Ik_.size() <= k) Ik_.push_back(mul(I1_, Ik_.back()));
    return Ik_[(size_t)k];
  }
  Sq poly(const Poly& p) {
    Sq M(L_), Rk(L_);
    for (int i = 0; i < L_; ++i) Rk(i, i) = 1.0;
    for (size_t c = 0; c < p.size(); ++c) {
      if (p[c] != 0.0) M = axpy(M, p[c], Rk);
      if (c + 1 < p.size()) Rk = mul(R_, Rk);
    }
    return M;
  }
  // I_k [sum_d P_d f^(d)], exact in rows >= k
  Sq integrated(const Terms& terms, int k) {
    Sq out(L_);
    for (const Term& t : terms)
      for (int i = 0; i <= t.d; ++i) {
        double binom = 1.0;
        for (int q = 0; q < i; ++q) binom = binom * (double)(t.d - q) / (double)(q + 1);
        const double s = ((i & 1) ? -1.0 : 1.0) * binom;
        out = axpy(out, s, mul(Ik(k - t.d + i), poly(pder(t.P, i))));
      }
    return out;
  }

 private:
  int L_;
  Sq R_, I1_;
  std::vector<Sq> Ik_;
};

// r^4 Lap(w) for w = r^-2 sum_j q_j f^(j), with the (4 - m^2) factor at m = 0:
// r^2 w~'' - 3 r w~' + 4 w~ for w~ = sum_j q_j f^(j)
Terms lapl4(const Terms& t) {
  Terms out;
  const Poly r1 = rpow(1), r2 = rpow(2);
  for (const Term& x : t) {
    add_term(out, x.d, pmul(r2, pder(x.P, 2)));
    add_term(out, x.d + 1, pscale(pmul(r2, pder(x.P, 1)), 2.0));
    add_term(out, x.d + 2, pmul(r2, x.P));
    add_term(out, x.d, pscale(pmul(r1, pder(x.P, 1)), -3.0));
    add_term(out, x.d + 1, pscale(pmul(r1, x.P), -3.0));
    add_term(out, x.d, pscale(x.P, 4.0));
  }
  return out;
}

}  // namespace

void pz_integ_operators(int N, double r_icb, double r_cmb, double rnorm, std::vector<double>& out, int* band) {
  Prims pr(N, 0.5 * (r_cmb - r_icb), 0.5 * (r_cmb + r_icb));
  const Poly one{1.0}, r1 = rpow(1), r2 = rpow(2), r3 = rpow(3), r4 = rpow(4);
  const double ro2 = r_cmb * r_cmb;
  const Poly h2 = padd(Poly{ro2}, pscale(r2, -1.0));   // r_cmb^2 - r^2
  // rotating omega(psi) (update_psi_integ_smat.f90:456-468) times r^2:
  // r^2 omega = -r^2 h2 psi'' - (ro^2 r - 6 r^3) psi' + (6 r^2 + m^2 h2) psi
  //           = Ta + m^2 Tb
  Terms Ta = {{2, pscale(pmul(r2, h2), -1.0)}, {1, padd(pscale(r1, -ro2), pscale(r3, 6.0))}, {0, pscale(r2, 6.0)}};
  Terms Tb = {{0, h2}};
  auto times_r2 = [&](const Terms& t) {
    Terms o;
    for (const Term& x : t) o.push_back({x.d, pmul(r2, x.P)});
    return o;
  };
  // S1 = I4[lapl4(Tb) - Ta], S2 = I4[-Tb]
  Terms s1 = lapl4(Tb);
  for (const Term& x : Ta) add_term(s1, x.d, pscale(x.P, -1.0));
  Terms s2 = {{0, pscale(h2, -1.0)}};
  // non-rotating streamfunction: r^2 Lap_m psi = A + m^2 B with A = r^2 psi'' + r psi',
  // B = -psi; intcheb4rmult4lapl = I4[r^2 (A + m^2 B)] = N0 + m^2 N1 and
  // intcheb4rmult4lapl2 = I4[r^4 Lap_m (r^-2 (A + m^2 B))]
  //                     = I4[lapl4(A) + m^2 (lapl4(B) - A) - m^4 B] = L0 + m^2 L1 + m^4 L2
  const Terms nA = {{2, r2}, {1, r1}};
  const Terms nB = {{0, Poly{-1.0}}};
  Terms l1 = lapl4(nB);
  for (const Term& x : nA) add_term(l1, x.d, pscale(x.P, -1.0));
  struct Def { int id; Terms t; int k; };
  const Def defs[] = {
      {IM_I2R1, {{0, r1}}, 2},
      {IM_I2R2, {{0, r2}}, 2},
      {IM_I2, {{0, one}}, 2},
      {IM_LT0, {{2, r2}, {1, r1}}, 2},              // I2 [r^2 Lap_m] = LT0 - m^2 I2
      {IM_ULAP, {{2, r2}, {1, r1}, {0, Poly{-1.0}}}, 2},   // m = 0 u_phi: r^2 Lap_1
      {IM_I4R3, {{0, r3}}, 4},
      {IM_I4R4, {{0, r4}}, 4},
      {IM_Q0, times_r2(Ta), 4},                     // intcheb4rmult4laplrot = Q0 + m^2 Q1
      {IM_Q1, times_r2(Tb), 4},
      {IM_S0, lapl4(Ta), 4},                        // intcheb4rmult4laplrot2 = S0 + m^2 S1 + m^4 S2
      {IM_S1, s1, 4},
      {IM_S2, s2, 4},
      {IM_P0, Ta, 2},                               // I2 [r^2 omega] = P0 + m^2 P1
      {IM_P1, Tb, 2},
      {IM_N0, times_r2(nA), 4},                     // intcheb4rmult4lapl = N0 + m^2 N1
      {IM_N1, times_r2(nB), 4},
      {IM_L0, lapl4(nA), 4},                        // intcheb4rmult4lapl2 = L0 + m^2 L1 + m^4 L2
      {IM_L1, l1, 4},
      {IM_L2, {{0, one}}, 4},
  };
  out.assign((size_t)IM_COUNT * N * N, 0.0);
  for (const Def& df : defs) {
    Sq M = pr.integrated(df.t, df.k);
    double* dst = out.data() + (size_t)df.id * N * N;
    int bw = 0;
    for (int i = df.k; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        const double v = rnorm * M(i, j);
        dst[i + (size_t)j * N] = v;   // column-major
        if (v != 0.0) bw = std::max(bw, std::abs(i - j));
      }
    band[df.id] = bw;
  }
}

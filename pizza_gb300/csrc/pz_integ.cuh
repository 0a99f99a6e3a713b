// Chebyshev integration method ("integ", tau boundary rows, direct solve):
// the per-m device code of update_temp_int (src/update_temp_integ.f90),
// update_xi_int (src/update_xi_integ.f90, the same operators with XidiffFac)
// and update_psi_int_smat (src/update_psi_integ_smat.f90).  Included by
// pz_kernels.cu after the collocation helpers it reuses (View, MS, op_*,
// mv_lanes, imex_rhs, dirk_rhs, gj_invert, gj_invert_c, store_op).
//
// Unknowns are Chebyshev coefficients: T_hat per m, psi_hat per m /= 0 and
// the m = 0 azimuthal velocity's coefficients.  The equations are multiplied
// by r^2 (temperature, u_phi) or r^4 (streamfunction) and integrated twice
// (four times) in r, which makes every operator except the tau rows banded:
// the banded operators (IM_*) are applied with band_mv over their band
// only.  The dt dependent left-hand sides (and the influence matrix's
// dt-independent streamfunction operator) are bordered banded systems: their
// tau rows are dense, every other row banded.  By default k_build inverts them
// per m (Gauss-Jordan) and every stage applies the inverses as dense products
// with every lane busy; pz_integ_banded(1) switches a handle created
// afterwards to bordered banded LU records (pz_bord.cuh) applied by banded
// sweeps, with a quarter of the flops but one or two active lanes per
// sequential sweep, which the FP64 issue rate of this GPU makes the slower.
#pragma once
#include "pz_bord.cuh"

// -- banded products ---------------------------------------------------------
// y_i = sum_{|j-i|<=bw} (sum_k c_k A_k(i,j)) x_j, A_k column-major n x n;
// one thread per row.
struct Band3 {
  const double* A[3];
  double c[3];
  int na, bw;
};
__device__ __forceinline__ void band_mv(const Band3& B, int n, const double2* __restrict__ x,
                                        double2* __restrict__ y) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int j0 = max(0, i - B.bw), j1 = min(n - 1, i + B.bw);
    double re = 0.0, im = 0.0;
    for (int j = j0; j <= j1; ++j) {
      double a = 0.0;
      for (int k = 0; k < B.na; ++k) a = fma(B.c[k], __ldg(B.A[k] + i + (long long)j * n), a);
      re = fma(a, x[j].x, re);
      im = fma(a, x[j].y, im);
    }
    y[i] = make_double2(re, im);
  }
}

__device__ __forceinline__ const double* im_op(const View& V, int k) {
  return V.pool + V.I->o_integ + (long long)k * V.I->N * V.I->N;
}
__device__ __forceinline__ Band3 band1(const View& V, int k, double c = 1.0) {
  Band3 b;
  b.A[0] = im_op(V, k); b.c[0] = c; b.na = 1; b.bw = V.I->im_band[k];
  b.A[1] = b.A[2] = nullptr; b.c[1] = b.c[2] = 0.0;
  return b;
}
// intcheb2rmult2lapl(m) = LT0 - m^2 I2, times f
__device__ __forceinline__ Band3 band_tlap(const View& V, double dm2, double f) {
  Band3 b;
  b.A[0] = im_op(V, IM_LT0); b.c[0] = f;
  b.A[1] = im_op(V, IM_I2); b.c[1] = -dm2 * f;
  b.A[2] = nullptr; b.c[2] = 0.0;
  b.na = 2; b.bw = max(V.I->im_band[IM_LT0], V.I->im_band[IM_I2]);
  return b;
}
// d/dt operator of the direct streamfunction solve, m /= 0: rotating
// intcheb4rmult4laplrot(m) = Q0 + m^2 Q1, non-rotating -intcheb4rmult4lapl(m)
// = -(N0 + m^2 N1) (update_psi_integ_smat.f90:1631-1764)
__device__ __forceinline__ Band3 band_rot(const View& V, double dm2) {
  const bool rot = !(V.I->flags & PZF_NON_ROT);
  const int a0 = rot ? IM_Q0 : IM_N0, a1 = rot ? IM_Q1 : IM_N1;
  const double sg = rot ? 1.0 : -1.0;
  Band3 b;
  b.A[0] = im_op(V, a0); b.c[0] = sg;
  b.A[1] = im_op(V, a1); b.c[1] = sg * dm2;
  b.A[2] = nullptr; b.c[2] = 0.0;
  b.na = 2; b.bw = max(V.I->im_band[a0], V.I->im_band[a1]);
  return b;
}
// f times the viscous operator: rotating intcheb4rmult4laplrot2(m) = S0 +
// m^2 S1 + m^4 S2, non-rotating -intcheb4rmult4lapl2(m) = -(L0 + m^2 L1 + m^4 L2)
__device__ __forceinline__ Band3 band_rot2(const View& V, double dm2, double f) {
  const bool rot = !(V.I->flags & PZF_NON_ROT);
  const int a0 = rot ? IM_S0 : IM_L0, a1 = rot ? IM_S1 : IM_L1, a2 = rot ? IM_S2 : IM_L2;
  if (!rot) f = -f;
  Band3 b;
  b.A[0] = im_op(V, a0); b.c[0] = f;
  b.A[1] = im_op(V, a1); b.c[1] = f * dm2;
  b.A[2] = im_op(V, a2); b.c[2] = f * dm2 * dm2;
  b.na = 3; b.bw = max(V.I->im_band[a0], max(V.I->im_band[a1], V.I->im_band[a2]));
  return b;
}

// y = G x, G complex n x n column-major (the integ streamfunction inverse)
struct CDenseDotN {
  const double2* __restrict__ G; int n; const double* __restrict__ x; double* __restrict__ y;
  __device__ __forceinline__ double fma(int t, int j, double acc) const {
    const double2 g = __ldg(G + (t >> 1) + (long long)j * n);
    const double xr = x[2 * j], xi = x[2 * j + 1];
    return (t & 1) ? ::fma(g.x, xi, ::fma(g.y, xr, acc)) : ::fma(g.x, xr, ::fma(-g.y, xi, acc));
  }
  __device__ __forceinline__ void store(int t, double v) const { y[t] = v; }
};
__device__ __forceinline__ void cmvn_lanes(const double2* __restrict__ G, int n, const double2* __restrict__ x,
                                           double2* __restrict__ y) {
  lane_dots(CDenseDotN{G, n, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y)}, 2 * n, n);
}

// -- applying the per-m left-hand-side inverses ---------------------------------
// y = A^-1 x for the temperature-like operators (temperature, composition,
// u_phi, vorticity) at base (o_gt, o_gx, o_guphi with mi = 0, o_gom) and for
// the influence matrix's streamfunction operator (psi: base o_gpsi): the
// bordered banded record of m, or the dense inverse with PZF_INTEG_DENSE.
// st: shared staging space (integ_stage_bytes), red: 8 doubles of shared memory.
__device__ __forceinline__ void integ_apply(const PzDev& d, const PzInst& I, long long base, int mi, bool psi,
                                            const double2* x, double2* y, double* st, double* red) {
  const int n = I.N;
  if (I.flags & PZF_INTEG_DENSE) {
    mv_lanes(d.pool + base + (long long)mi * n * n, n, x, y);
    return;
  }
  const long long str = psi ? I.bstr_p : I.bstr_t;
  bord_solve<double>(d.pool + base + mi * str, n, 2, psi ? I.bkl_p : I.bkl_t, x, y, st, red);
}
// the direct solve's complex streamfunction operator
__device__ __forceinline__ void integ_apply_sm(const PzDev& d, const PzInst& I, int mi, const double2* x, double2* y,
                                               double* st, double* red) {
  const int n = I.N;
  if (I.flags & PZF_INTEG_DENSE) {
    cmvn_lanes(reinterpret_cast<const double2*>(d.pool + I.o_gsm) + (long long)mi * n * n, n, x, y);
    return;
  }
  bord_solve<double2>(reinterpret_cast<const double2*>(d.pool + I.o_gsm + mi * I.bstr_p), n, 4, I.bkl_p, x, y,
                      reinterpret_cast<double2*>(st), red);
}

// -- m = 0 derivative with the round-off threshold ---------------------------
// get_dcheb_real_1d (src/radial_derivatives.f90:143-185) on the real parts of
// the Chebyshev coefficients c: with thr > 0, a coefficient below
// thr*max|c| zeroes the derivative coefficient it feeds.  Output: derivative
// coefficients in df (imaginary parts zero).  One thread; the block syncs.
__device__ void dcheb_thr(const double2* c, double2* df, int n, double thr) {
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(c[i].x));
    const double t = mx * thr;
    df[n - 1] = make_double2(0.0, 0.0);
    df[n - 2] = make_double2(fabs(c[n - 1].x) >= t ? (double)(n - 1) * c[n - 1].x : 0.0, 0.0);
    for (int k = n - 3; k >= 0; --k)
      df[k] = make_double2(fabs(c[k + 1].x) >= t ? df[k + 2].x + 2.0 * (k + 1) * c[k + 1].x : 0.0, 0.0);
  }
  __syncthreads();
}
// get_ddcheb_real_1d (src/radial_derivatives.f90:259-311): terms below the
// threshold are skipped.
__device__ void ddcheb_thr(const double2* c, double2* df, double2* ddf, int n, double thr) {
  if (threadIdx.x == 0) {
    double mx = 0.0;
    for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(c[i].x));
    const double t = mx * thr;
    df[n - 1] = ddf[n - 1] = ddf[n - 2] = make_double2(0.0, 0.0);
    df[n - 2] = make_double2(fabs(c[n - 1].x) >= t ? (double)(n - 1) * c[n - 1].x : 0.0, 0.0);
    for (int k = n - 3; k >= 0; --k) {
      const double fac = 2.0 * (k + 1);
      const double d = fabs(c[k + 1].x) >= t ? df[k + 2].x + fac * c[k + 1].x : df[k + 2].x;
      df[k] = make_double2(d, 0.0);
      ddf[k] = make_double2(fabs(df[k + 1].x) >= t ? ddf[k + 2].x + fac * df[k + 1].x : ddf[k + 2].x, 0.0);
    }
  }
  __syncthreads();
}

// -- influence-matrix variant (update_psi_integ_dmat.f90) -----------------------
// The two wall conditions left to the influence matrix, as weights on the
// Chebyshev coefficients of psi (get_bc_influence_matrix, :1361-1530): top
// d4psi/dx4 (rotating, rigid) or dpsi/dr (non-rotating, rigid), bottom
// dpsi/dr; half weight at both ends; times rnorm.
__device__ __forceinline__ double dmat_bc_top(const PzInst& I, int j) {
  const double dn2 = (double)j * (double)j;
  const double f = (j == 0 || j == I.N - 1) ? 0.5 : 1.0;
  const double v = (I.flags & PZF_NON_ROT) ? 2.0 * dn2
                                           : 16.0 / 105.0 * dn2 * (dn2 - 1.0) * (dn2 - 4.0) * (dn2 - 9.0);
  return I.rnorm * f * v;
}
__device__ __forceinline__ double dmat_bc_bot(const PzInst& I, int j) {
  const double dn2 = (double)j * (double)j;
  const double f = (j == 0 || j == I.N - 1) ? 0.5 : 1.0;
  return I.rnorm * f * (-2.0 * dn2 * ((j & 1) ? -1.0 : 1.0));
}

// dt-independent streamfunction-from-vorticity inverse for one m > 0
// (get_lhs_psi_mat, update_psi_integ_dmat.f90:971-1089): intcheb2rmult2laplrot
// = -I2[r^2 omega(psi)] = -(P0 + m^2 P1) (I2[r^2 Lap_m] = LT0 - m^2 I2 without
// rotation), tau rows psi(r_o) = psi(r_i) = 0, row preconditioning; stored as
// G_psi = A_s^-1 diag(fac) at o_gpsi.  Shared memory: the BuildSmem layout.
// Tau rows T_j(+-1) (rows 0 and 1: value 1, (-1)^j; boundary_fac on column
// 0), times rnorm, then the rows of c0 A0 + c1 A1 + c2 A2 (A_k integration
// operators, a null A2 skipped): the real operators of the integration method
struct IntegGet {
  const double *A0, *A1, *A2;
  double c0, c1, c2, rn;
  int n;
  __device__ double operator()(int i, int j) const {
    if (i < 2) {
      const double v = rn * ((i == 1 && (j & 1)) ? -1.0 : 1.0);
      return j == 0 ? 0.5 * v : v;
    }
    const long long c = i + (long long)j * n;
    double v = c0 * A0[c] + c1 * A1[c];
    if (A2) v += c2 * A2[c];
    return v;
  }
};
// shared memory of the banded factorisations: workspace for the largest
// record (complex, 4 tau rows, kl = 8), its pivots and a flag
__host__ __device__ inline long long integ_bord_ws_doubles(int n) {
  return 2 * bord_ws_size(n, 4, 8) + (n + 1) / 2 + 2;
}

__device__ int integ_psi_static(const PzDev& d, const PzInst& I, const View& V, int mi) {
  extern __shared__ double shb[];
  const int n = I.N, m = mi * I.minc;
  const double dm2 = (double)m * (double)m, rn = I.rnorm;
  const bool rot = !(I.flags & PZF_NON_ROT);
  if (!(I.flags & PZF_INTEG_DENSE)) {
    const IntegGet g{im_op(V, rot ? IM_P0 : IM_LT0), im_op(V, rot ? IM_P1 : IM_I2), nullptr,
                     rot ? -1.0 : 1.0, -dm2, 0.0, rn, n};
    int* flag = reinterpret_cast<int*>(shb + integ_bord_ws_doubles(n) - 1);
    return bord_factor<double>(g, n, 2, I.bkl_p, I.bkw_p, shb, flag, d.pool + I.o_gpsi + mi * I.bstr_p);
  }
  double* A = shb;
  double* f1 = A + (long long)n * n;
  double* colk = f1 + n + n;
  double* red = colk + n;
  int* redi = reinterpret_cast<int*>(red + 32);
  int* piv = redi + 32;
  const double* L0 = im_op(V, rot ? IM_P0 : IM_LT0);
  const double* L1 = im_op(V, rot ? IM_P1 : IM_I2);
  const double s0 = rot ? -1.0 : 1.0, s1 = -dm2;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    double v;
    if (i < 2) {
      v = rn * ((i == 1 && (j & 1)) ? -1.0 : 1.0);
      if (j == 0) v *= 0.5;
    } else {
      const long long c = i + (long long)j * n;
      v = s0 * L0[c] + s1 * L1[c];
    }
    A[idx] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double mx = 0.0;
    for (int j = 0; j < n; ++j) mx = fmax(mx, fabs(A[i * n + j]));
    f1[i] = 1.0 / mx;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) A[idx] *= f1[idx / n];
  __syncthreads();
  if (gj_invert(A, n, piv, colk, red, redi) != 0) return -1;
  store_op(d.pool + I.o_gpsi + (long long)mi * n * n, A, n, n, nullptr, f1);
  return 0;
}

// -- dt dependent left-hand sides (get_lhs_mat_tau) ----------------------------
// k_build for one m of an integ instance: the temperature operator
// (update_temp_integ.f90:631-776), the m = 0 u_phi operator or the m /= 0
// streamfunction operator (update_psi_integ_smat.f90:1286-1581), each with its
// tau rows (boundary_fac on column 0) and the row preconditioning
// 1/max|row|, inverted by Gauss-Jordan and stored as G = A_s^-1 diag(fac) so
// that x = G rhs.  Unlike the collocation builders nothing is truncated: the
// integration method keeps all n_r_max coefficients of the solution.
// Shared memory: see pz_build_smem_bytes (integ).
// The complex streamfunction operator of the direct solve, m /= 0 (the
// dense builder below spells out its rows)
struct IntegGetSm {
  const double *Q0, *Q1, *S0, *S1, *S2, *R4;
  double sg0, dm2, cv, cc, rn;
  int n;
  bool rot;
  __device__ double2 operator()(int i, int j) const {
    if (i < 4) {
      const double dj = (double)j, dn2 = dj * dj, sg = (j & 1) ? -1.0 : 1.0;
      double re;
      if (i == 0) re = 1.0;
      else if (i == 1) re = sg;
      else if (i == 2) re = rot ? 8.0 / 15.0 * dn2 * (dn2 - 1.0) * (dn2 - 4.0) : 2.0 * dn2;
      else re = -2.0 * dn2 * sg;
      re *= rn;
      if (j == 0) re *= 0.5;
      return make_double2(re, 0.0);
    }
    const long long c = i + (long long)j * n;
    return make_double2(sg0 * (Q0[c] + dm2 * Q1[c] - cv * (S0[c] + dm2 * (S1[c] + dm2 * S2[c]))), cc * R4[c]);
  }
};

// integ_build with bordered banded factors (the same operators as the dense
// builder below)
__device__ int integ_build_banded(const PzDev& d, const PzInst& I, const View& V, int mi, double wlin) {
  extern __shared__ double shb[];
  const int n = I.N, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm, rn = I.rnorm;
  const bool dmat = !(I.flags & PZF_DIRECT);
  int* flag = reinterpret_cast<int*>(shb + integ_bord_ws_doubles(n) - 1);
  for (int pass = 0; pass < 3; ++pass) {
    if (pass == 1 && !(I.flags & PZF_CHEM)) continue;
    if (pass == 2 && m != 0 && !dmat) break;
    const bool scal = pass < 2;
    const double c0 = wlin * (pass == 0 ? I.TdiffFac : pass == 1 ? I.XidiffFac : I.ViscFac);
    const double c1 = (scal || m != 0) ? -dm2 * c0 : 0.0;
    // I2R2 - c0 L0 - c1 I2
    const IntegGet g{im_op(V, IM_I2R2), im_op(V, (scal || m != 0) ? IM_LT0 : IM_ULAP), im_op(V, IM_I2),
                     1.0, -c0, -c1, rn, n};
    double* out = d.pool + (pass == 0   ? I.o_gt + mi * I.bstr_t
                            : pass == 1 ? I.o_gx + mi * I.bstr_t
                                        : (m == 0 ? I.o_guphi : I.o_gom + mi * I.bstr_t));
    if (bord_factor<double>(g, n, 2, I.bkl_t, I.bkw_t, shb, flag, out)) return -1;
  }
  if (m == 0) return 0;
  if (dmat) {
    // get_intermediate_sol + get_influence_matrix (update_psi_integ_dmat.f90:1212-1313):
    // omega = 1 on the inner (set 1: om2, psi2) or outer (set 2: om3, psi3)
    // wall, packed as the real and imaginary parts of one complex vector
    double2* x = reinterpret_cast<double2*>(shb);
    double2* va = x + n;
    double2* vb = va + n;
    double2* vc = vb + n;
    double* st = reinterpret_cast<double*>(vc + n);
    double* red = st + (long long)(n - 2) * (3 * 8 + 2);
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      x[i] = make_double2(i == 1 ? 1.0 : 0.0, i == 0 ? 1.0 : 0.0);
    __syncthreads();
    integ_apply(d, I, I.o_gom, mi, false, x, va, st, red);
    band_mv(band1(V, IM_I2R2, -1.0), n, va, vb);
    __syncthreads();
    integ_apply(d, I, I.o_gpsi, mi, true, vb, vc, st, red);
    double* aux = d.pool + I.o_aux;
    const long long MN = (long long)I.M * n;
    double t2 = 0.0, t3 = 0.0, b2 = 0.0, b3 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      aux[0 * MN + (long long)mi * n + i] = va[i].x;
      aux[1 * MN + (long long)mi * n + i] = va[i].y;
      aux[2 * MN + (long long)mi * n + i] = vc[i].x;
      aux[3 * MN + (long long)mi * n + i] = vc[i].y;
      const double ct = dmat_bc_top(I, i), cb = dmat_bc_bot(I, i);
      t2 += ct * vc[i].x; t3 += ct * vc[i].y;
      b2 += cb * vc[i].x; b3 += cb * vc[i].y;
    }
    t2 = block_sum(t2, red); t3 = block_sum(t3, red);
    b2 = block_sum(b2, red); b3 = block_sum(b3, red);
    if (threadIdx.x == 0) {
      double* infl = aux + 4 * MN + 4LL * mi;
      const double det = t2 * b3 - t3 * b2;
      infl[0] = b3 / det; infl[1] = -t3 / det; infl[2] = -b2 / det; infl[3] = t2 / det;
    }
    return 0;
  }
  const bool rot = !(I.flags & PZF_NON_ROT);
  const IntegGetSm g{im_op(V, rot ? IM_Q0 : IM_N0), im_op(V, rot ? IM_Q1 : IM_N1), im_op(V, rot ? IM_S0 : IM_L0),
                     im_op(V, rot ? IM_S1 : IM_L1), im_op(V, rot ? IM_S2 : IM_L2), im_op(V, IM_I4R4),
                     rot ? 1.0 : -1.0, dm2, wlin * I.ViscFac,
                     (I.flags & PZF_COR_IMP) ? wlin * I.CorFac * dm : 0.0, rn, n, rot};
  return bord_factor<double2>(g, n, 4, I.bkl_p, I.bkw_p, reinterpret_cast<double2*>(shb), flag,
                              reinterpret_cast<double2*>(d.pool + I.o_gsm + mi * I.bstr_p))
             ? -1
             : 0;
}

__device__ int integ_build(const PzDev& d, const PzInst& I, const View& V, int mi, double wlin) {
  extern __shared__ double shb[];
  if (!(I.flags & PZF_INTEG_DENSE)) return integ_build_banded(d, I, V, mi, wlin);
  const int n = I.N, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm, rn = I.rnorm;
  double* A = shb;
  double2* Ac = reinterpret_cast<double2*>(shb);
  double* f1 = shb + 2LL * n * n;
  double* colk = f1 + ((n + 1) & ~1);          // even offset: read as double2 by gj_invert_c
  double* red = colk + 2 * n;
  int* redi = reinterpret_cast<int*>(red + 32);
  int* piv = redi + 32;
  const double* I2R2 = im_op(V, IM_I2R2);
  const bool dmat = !(I.flags & PZF_DIRECT);
  for (int pass = 0; pass < 3; ++pass) {
    // pass 0: temperature; pass 1: composition (update_xi_integ.f90, the
    // temperature's operator with XidiffFac); pass 2: u_phi (m = 0) or, with
    // the influence matrix, the vorticity operator (m /= 0, tau rows
    // omega(r_o), omega(r_i)); the direct solve's m /= 0 streamfunction
    // operator is complex and built below
    if (pass == 1 && !(I.flags & PZF_CHEM)) continue;
    if (pass == 2 && m != 0 && !dmat) break;
    const bool scal = pass < 2;
    const double* L0 = im_op(V, (scal || m != 0) ? IM_LT0 : IM_ULAP);
    const double* L1 = im_op(V, IM_I2);
    const double c0 = wlin * (pass == 0 ? I.TdiffFac : pass == 1 ? I.XidiffFac : I.ViscFac);
    const double c1 = (scal || m != 0) ? -dm2 * c0 : 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int i = idx / n, j = idx - i * n;
      double v;
      if (i < 2) {
        // fixed temperature / rigid u_phi: T_j(+-1) = 1, (-1)^j
        v = rn * ((i == 1 && (j & 1)) ? -1.0 : 1.0);
        if (j == 0) v *= 0.5;                       // boundary_fac
      } else {
        const long long c = i + (long long)j * n;
        v = I2R2[c] - c0 * L0[c] - c1 * L1[c];
      }
      A[idx] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double mx = 0.0;
      for (int j = 0; j < n; ++j) mx = fmax(mx, fabs(A[i * n + j]));
      f1[i] = 1.0 / mx;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) A[idx] *= f1[idx / n];
    __syncthreads();
    if (gj_invert(A, n, piv, colk, red, redi) != 0) return -1;
    double* G = d.pool + (pass == 0   ? I.o_gt + (long long)mi * n * n
                          : pass == 1 ? I.o_gx + (long long)mi * n * n
                                      : (m == 0 ? I.o_guphi : I.o_gom + (long long)mi * n * n));
    store_op(G, A, n, n, nullptr, f1);
    __syncthreads();
  }
  if (m == 0) return 0;
  if (dmat) {
    // get_intermediate_sol + get_influence_matrix (update_psi_integ_dmat.f90:1212-1313):
    // omega = 1 on the inner (set 1: om2, psi2) or outer (set 2: om3, psi3)
    // wall, packed as the real and imaginary parts of one complex vector
    const double* Gom = d.pool + I.o_gom + (long long)mi * n * n;
    double2* va = reinterpret_cast<double2*>(shb);
    double2* vb = va + n;
    double2* vc = vb + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      va[i] = make_double2(Gom[i + (long long)1 * n], Gom[i]);     // columns 1 and 0
    __syncthreads();
    band_mv(band1(V, IM_I2R2, -1.0), n, va, vb);
    __syncthreads();
    mv_lanes(d.pool + I.o_gpsi + (long long)mi * n * n, n, vb, vc);
    __syncthreads();
    double* aux = d.pool + I.o_aux;
    const long long MN = (long long)I.M * n;
    double t2 = 0.0, t3 = 0.0, b2 = 0.0, b3 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      aux[0 * MN + (long long)mi * n + i] = va[i].x;
      aux[1 * MN + (long long)mi * n + i] = va[i].y;
      aux[2 * MN + (long long)mi * n + i] = vc[i].x;
      aux[3 * MN + (long long)mi * n + i] = vc[i].y;
      const double ct = dmat_bc_top(I, i), cb = dmat_bc_bot(I, i);
      t2 += ct * vc[i].x; t3 += ct * vc[i].y;
      b2 += cb * vc[i].x; b3 += cb * vc[i].y;
    }
    t2 = block_sum(t2, red); t3 = block_sum(t3, red);
    b2 = block_sum(b2, red); b3 = block_sum(b3, red);
    if (threadIdx.x == 0) {
      double* infl = aux + 4 * MN + 4LL * mi;
      const double det = t2 * b3 - t3 * b2;
      infl[0] = b3 / det; infl[1] = -t3 / det; infl[2] = -b2 / det; infl[3] = t2 / det;
    }
    return 0;
  }
  // streamfunction, m /= 0: Q0 + m^2 Q1 - wlin ViscFac (S0 + m^2 S1 + m^4 S2)
  // + i wlin CorFac m I4R4 (implicit Coriolis), tau rows psi(r_o) = psi(r_i) = 0,
  // d3psi/dx3(r_o) = 0 (rigid, rotating) and dpsi/dr(r_i) = 0; non-rotating
  // -(N0 + m^2 N1) + wlin (L0 + m^2 L1 + m^4 L2) with dpsi/dr(r_o) = 0 in
  // the third tau row (update_psi_integ_smat.f90:1286-1581)
  const bool rot = !(I.flags & PZF_NON_ROT);
  const double sg0 = rot ? 1.0 : -1.0;
  const double* Q0 = im_op(V, rot ? IM_Q0 : IM_N0);
  const double* Q1 = im_op(V, rot ? IM_Q1 : IM_N1);
  const double* S0 = im_op(V, rot ? IM_S0 : IM_L0);
  const double* S1 = im_op(V, rot ? IM_S1 : IM_L1);
  const double* S2 = im_op(V, rot ? IM_S2 : IM_L2);
  const double* R4 = im_op(V, IM_I4R4);
  const double cv = wlin * I.ViscFac;
  const double cc = (I.flags & PZF_COR_IMP) ? wlin * I.CorFac * dm : 0.0;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    double re = 0.0, im = 0.0;
    if (i < 4) {
      const double dj = (double)j, dn2 = dj * dj, sg = (j & 1) ? -1.0 : 1.0;
      if (i == 0) re = 1.0;
      else if (i == 1) re = sg;
      else if (i == 2) re = rot ? 8.0 / 15.0 * dn2 * (dn2 - 1.0) * (dn2 - 4.0)   // update_psi_integ_smat.f90:1303-1306
                                : 2.0 * dn2;                                  // drMat(1,:)
      else re = -2.0 * dn2 * sg;                                           // drMat(2,:), chebyshev.f90:363-379
      re *= rn;
      if (j == 0) re *= 0.5;                                               // boundary_fac
    } else {
      const long long c = i + (long long)j * n;
      re = sg0 * (Q0[c] + dm2 * Q1[c] - cv * (S0[c] + dm2 * (S1[c] + dm2 * S2[c])));
      im = cc * R4[c];
    }
    Ac[idx] = make_double2(re, im);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double mx = 0.0;
    for (int j = 0; j < n; ++j) mx = fmax(mx, hypot(Ac[i * n + j].x, Ac[i * n + j].y));
    f1[i] = 1.0 / mx;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) Ac[idx] = cscale(f1[idx / n], Ac[idx]);
  __syncthreads();
  if (gj_invert_c(Ac, n, piv, reinterpret_cast<double2*>(colk), red, redi) != 0) return -1;
  double2* G = reinterpret_cast<double2*>(d.pool + I.o_gsm) + (long long)mi * n * n;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int j = idx / n, i = idx - j * n;
    G[idx] = cscale(f1[j], Ac[i * n + j]);
  }
  return 0;
}

// -- implicit terms from the physical fields ------------------------------------
// get_temp_rhs_imp_int and get_psi_rhs_imp_int_smat with l_calc_lin
// (update_temp_integ.f90:471-536, update_psi_integ_smat.f90:960-1115) from
// T_hat = C T and psi_hat = C psi: the start fields (init_fields.f90:207-251)
// and start_from_another_scheme (step_time.f90:488-500).  With from_us the
// streamfunction is first rebuilt from u_s, psi = -i r u_s / (m h^2)
// (init_fields.f90:73-91).  Writes old/impl logical slot 1 at ring bases bo/bi
// and dT/dr (d xi/dr).  With psi_as_xi the buoyancy takes psi in the place of
// the composition, as start_from_another_scheme does for the direct solve
// (step_time.f90:497-498 passes psi_Mloc for xi_Mloc).
template <bool CHEM>
__device__ void integ_imp(const View& V, const PzInst& I, int mi, int bo, int bi, bool calc, bool from_us, MS& s,
                          bool psi_as_xi) {
  const int n = I.N, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  const double* r = V.rad(RV_R);
  const double* or1 = V.rad(RV_OR1);
  const double* rgrav = V.rad(RV_RGRAV);
  double2* T = V.fld(F_TEMP, mi);
  double2* psi = V.fld(F_PSI, mi);
  double2* up = V.fld(F_UP, mi);
  const double2* us = V.fld(F_US, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = T[i];
  __syncthreads();
  op_C(V, n, s.a, s.b, s.w);                                     // T_hat
  __syncthreads();
  op_D1c(V, n, s.b, s.c, s.w);
  __syncthreads();
  double2* dT = V.fld(F_DTEMP, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) dT[i] = s.c[i];
  band_mv(band1(V, IM_I2R2), n, s.b, V.hist(0, 0, bo, mi));
  if (calc) band_mv(band_tlap(V, dm2, I.TdiffFac), n, s.b, V.hist(0, 1, bi, mi));
  __syncthreads();
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  const double2* X = V.fld(F_XI, mi);
  if (chem) {
    // get_xi_rhs_imp_int (update_xi_integ.f90:449-510)
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = X[i];
    __syncthreads();
    op_C(V, n, s.a, s.b, s.w);                                   // xi_hat
    __syncthreads();
    op_D1c(V, n, s.b, s.c, s.w);
    __syncthreads();
    double2* dX = V.fld(F_DXI, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dX[i] = s.c[i];
    band_mv(band1(V, IM_I2R2), n, s.b, V.hist(2, 0, bo, mi));
    if (calc) band_mv(band_tlap(V, dm2, I.XidiffFac), n, s.b, V.hist(2, 1, bi, mi));
    __syncthreads();
  }
  double2* oP = V.hist(1, 0, bo, mi);
  double2* iP = V.hist(1, 1, bi, mi);
  if (m == 0) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = make_double2(up[i].x, 0.0);
    __syncthreads();
    op_C(V, n, s.a, s.b, s.w);                                   // costf1(Re u_phi)
    __syncthreads();
    band_mv(band1(V, IM_I2R2), n, s.b, oP);
    if (calc) band_mv(band1(V, IM_ULAP, I.ViscFac), n, s.b, iP);
    __syncthreads();
    return;
  }
  if (from_us) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double h2 = (I.flags & PZF_NON_ROT) ? 1.0 : I.r_cmb * I.r_cmb - r[i] * r[i];
      psi[i] = i == 0 ? make_double2(0.0, 0.0) : cscale(r[i] / (dm * h2), cim(-1.0, us[i]));
    }
    __syncthreads();
  }
  const bool dmat = !(I.flags & PZF_DIRECT);
  const double2* om = V.fld(F_OM, mi);
  const double2* xs = psi_as_xi ? psi : X;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    // the influence-matrix variant works on omega (get_psi_rhs_imp_int_dmat,
    // update_psi_integ_dmat.f90:625-781), the direct solve on psi
    s.a[i] = dmat ? om[i] : psi[i];
    double2 b = cscale(-I.BuoFac * rgrav[i] * or1[i], cim(dm, T[i]));
    if (chem) b = csub(b, cscale(I.ChemFac * rgrav[i] * or1[i], cim(dm, xs[i])));
    s.e[i] = b;
  }
  __syncthreads();
  op_C(V, n, s.a, s.b, s.w);                                     // omega_hat or psi_hat
  __syncthreads();
  op_C(V, n, s.e, s.f, s.w);                                     // buoyancy, Chebyshev
  __syncthreads();
  if (dmat) {
    band_mv(band1(V, IM_I2R2), n, s.b, oP);
    if (calc) {
      band_mv(band_tlap(V, dm2, I.ViscFac), n, s.b, s.c);
      band_mv(band1(V, IM_I2R2), n, s.f, s.h);
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x)
        iP[i] = (I.flags & PZF_BUO_IMP) ? cadd(s.c[i], s.h[i]) : s.c[i];
    }
    __syncthreads();
    return;
  }
  band_mv(band_rot(V, dm2), n, s.b, oP);
  if (calc) {
    band_mv(band_rot2(V, dm2, I.ViscFac), n, s.b, s.c);
    band_mv(band1(V, IM_I4R4, I.CorFac * dm), n, s.b, s.g);
    band_mv(band1(V, IM_I4R4), n, s.f, s.h);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 v = s.c[i];
      if (I.flags & PZF_COR_IMP) v = cadd(v, cim(-1.0, s.g[i]));
      if (I.flags & PZF_BUO_IMP) v = cadd(v, s.h[i]);
      iP[i] = v;
    }
  }
  __syncthreads();
}

// -- one stage for one m (mloop.f90:84-100 and :209-226) --------------------------
// finish_exp_temp_int / finish_exp_psi_int_smat (update_temp_integ.f90:396-469,
// update_psi_integ_smat.f90:793-958) on this stage's explicit slot, then
// update_temp_int and update_psi_int_smat (update_temp_integ.f90:179-298,
// update_psi_integ_smat.f90:247-573) with the implicit terms of the target
// stage.  Returns true on a non-finite value (for the block's status vote).
struct IntegStage {
  int stage, eslot, oslot, islot;
  bool dirk, do_finish, do_solve, wold, calc;
};

__device__ __forceinline__ void trunc_cheb(double2* x, int n, int n_max) {
  for (int i = n_max + threadIdx.x; i < n; i += blockDim.x) x[i] = make_double2(0.0, 0.0);
}

// update_psi_int_dmat, m /= 0 (update_psi_integ_dmat.f90:150-484), after the
// temperature: s.e holds I2R2 C(buoyancy) when the buoyancy is implicit.
// omega_hat = G_om rhs with omega = 0 on the walls, psi_hat = -G_psi I2R2
// omega_hat, then the influence matrix adds c1 (om2, psi2) + c2 (om3, psi3)
// so that the two remaining wall conditions on psi hold.
__device__ bool integ_dmat_psi(const PzDev& d, const View& V, const PzInst& I, const PzState& S, int mi,
                               const IntegStage& c, MS& s) {
  const int n = I.N, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  const double rc2 = I.r_cmb * I.r_cmb;
  const bool rot = !(I.flags & PZF_NON_ROT);
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  const double* r = V.rad(RV_R);
  const double* or1 = V.rad(RV_OR1);
  double2* us = V.fld(F_US, mi);
  double2* up = V.fld(F_UP, mi);
  double2* om = V.fld(F_OM, mi);
  double2* psi = V.fld(F_PSI, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 v = c.dirk ? dirk_rhs(V, I, S, 1, mi, i, c.stage) : imex_rhs(V, I, S, 1, mi, i);
    if (buo_imp) v = cadd(v, cscale(S.wimp_lin[0], s.e[i]));
    s.a[i] = v;
    s.k[i] = buo_imp ? s.e[i] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  integ_apply(d, I, I.o_gom, mi, false, s.a, s.b, s.st, s.red);         // omega_hat
  __syncthreads();
  band_mv(band1(V, IM_I2R2, -1.0), n, s.b, s.c);
  __syncthreads();
  integ_apply(d, I, I.o_gpsi, mi, true, s.c, s.e, s.st, s.red);         // psi_hat, particular
  __syncthreads();
  double tr = 0.0, ti = 0.0, br = 0.0, bi = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double ct = dmat_bc_top(I, i), cb = dmat_bc_bot(I, i);
    tr += ct * s.e[i].x; ti += ct * s.e[i].y;
    br += cb * s.e[i].x; bi += cb * s.e[i].y;
  }
  tr = block_sum(tr, s.red); ti = block_sum(ti, s.red);
  br = block_sum(br, s.red); bi = block_sum(bi, s.red);
  const long long MN = (long long)I.M * n;
  const double* aux = d.pool + I.o_aux;
  const double* infl = aux + 4 * MN + 4LL * mi;
  const double c1r = -infl[0] * tr - infl[1] * br, c1i = -infl[0] * ti - infl[1] * bi;
  const double c2r = -infl[2] * tr - infl[3] * br, c2i = -infl[2] * ti - infl[3] * bi;
  const double* om2 = aux + 0 * MN + (long long)mi * n;
  const double* om3 = aux + 1 * MN + (long long)mi * n;
  const double* psi2 = aux + 2 * MN + (long long)mi * n;
  const double* psi3 = aux + 3 * MN + (long long)mi * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 p = s.e[i], o = s.b[i];
    p.x += c1r * psi2[i] + c2r * psi3[i]; p.y += c1i * psi2[i] + c2i * psi3[i];
    o.x += c1r * om2[i] + c2r * om3[i];   o.y += c1i * om2[i] + c2i * om3[i];
    s.e[i] = p;
    s.b[i] = o;
  }
  __syncthreads();
  op_C(V, n, s.e, s.h, s.w);                                     // psi
  __syncthreads();
  op_D1c(V, n, s.e, s.c, s.w);                                   // dpsi/dr
  __syncthreads();
  op_C(V, n, s.b, s.g, s.w);                                     // omega
  __syncthreads();
  bool bad = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 p = s.h[i], dp = s.c[i], o = s.g[i];
    psi[i] = p;
    if (rot) {
      const double h2 = rc2 - r[i] * r[i];
      us[i] = cscale(or1[i] * h2, cim(dm, p));
      up[i] = make_double2(-h2 * dp.x + 3.0 * r[i] * p.x, -h2 * dp.y + 3.0 * r[i] * p.y);
    } else {
      us[i] = cscale(or1[i], cim(dm, p));
      up[i] = make_double2(-dp.x, -dp.y);
    }
    om[i] = o;
    bad |= !isfinite(o.x) || !isfinite(o.y) || !isfinite(p.x) || !isfinite(p.y);
  }
  // next-stage terms from omega_hat: I2R2 and ViscFac I2[r^2 Lap_m], plus the
  // implicit buoyancy (s.k)
  if (c.wold) band_mv(band1(V, IM_I2R2), n, s.b, V.hist(1, 0, c.oslot, mi));
  if (c.calc) {
    band_mv(band_tlap(V, dm2, I.ViscFac), n, s.b, s.a);
    __syncthreads();
    double2* iP = V.hist(1, 1, c.islot, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) iP[i] = cadd(s.a[i], s.k[i]);
  }
  return bad;
}

template <bool CHEM>
__device__ bool integ_stage(const PzDev& d, const View& V, const PzInst& I, const PzState& S, int mi,
                            const IntegStage& c, MS& s) {
  const int n = I.N, m = mi * I.minc, n_max = I.n_max;
  const double dm = (double)m, dm2 = dm * dm;
  const double rc2 = I.r_cmb * I.r_cmb;
  const bool rot = !(I.flags & PZF_NON_ROT);
  const double* r = V.rad(RV_R);
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* tcond = V.rad(RV_TCOND);
  const double* dtcond = V.rad(RV_DTCOND);
  const double* ekpump = V.rad(RV_EKPUMP);
  const double* ekp_up = V.rad(RV_EKP_UP);
  const double* ekp_us = V.rad(RV_EKP_US);
  const double* ekp_dusdp = V.rad(RV_EKP_DUSDP);
  double2* us = V.fld(F_US, mi);
  double2* up = V.fld(F_UP, mi);
  double2* om = V.fld(F_OM, mi);
  double2* psi = V.fld(F_PSI, mi);
  double2* T = V.fld(F_TEMP, mi);
  double2* dT = V.fld(F_DTEMP, mi);
  double2* X = V.fld(F_XI, mi);
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  const bool cor_imp = (I.flags & PZF_COR_IMP) != 0;
  const bool dmat = !(I.flags & PZF_DIRECT);
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  bool bad = false;

  if (c.do_finish) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      s.a[i] = V.fld(F_DVST, mi)[i];
      s.e[i] = V.fld(F_DVSOM, mi)[i];
    }
    __syncthreads();
    op_C(V, n, s.a, s.b, s.w);
    __syncthreads();
    op_C(V, n, s.e, s.f, s.w);
    __syncthreads();
    trunc_cheb(s.b, n, n_max);
    trunc_cheb(s.f, n, n_max);
    __syncthreads();
    op_D1c(V, n, s.b, s.c, s.w);                                 // d(u_s r T)/dr (dealiased)
    __syncthreads();
    op_D1c(V, n, s.f, s.g, s.w);                                 // d(u_s r om)/dr
    __syncthreads();
    double2* eT = V.hist(0, 2, c.eslot, mi);
    double2* eP = V.hist(1, 2, c.eslot, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double h2 = rc2 - r[i] * r[i];
      const double g = rot ? h2 * dtcond[i] + I.tadvz * r[i] * tcond[i] : dtcond[i];
      s.a[i] = csub(csub(cscale(r[i], eT[i]), cim(dm * g, psi[i])), s.c[i]);
      double2 p = eP[i];
      if (m != 0 && dmat) {
        // finish_exp_psi_int_dmat (update_psi_integ_dmat.f90:486-623): the
        // vorticity equation without the r weight, Coriolis always explicit
        p = csub(p, cscale(or1[i], s.g[i]));
        if (rot) p = csub(p, cim(I.CorFac * dm, psi[i]));
        if (!buo_imp) {
          p = csub(p, cim(I.BuoFac * rgrav[i] * or1[i] * dm, T[i]));
          if (chem) p = csub(p, cim(I.ChemFac * rgrav[i] * or1[i] * dm, X[i]));
        }
        if (I.flags & PZF_EK_PUMP) {
          const double2 u = us[i];
          const double2 q = make_double2(ekp_us[i] * u.x - ekp_dusdp[i] * dm * u.y,
                                         ekp_us[i] * u.y + ekp_dusdp[i] * dm * u.x);
          const double2 o = om[i], w = up[i];
          const double ce = I.CorFac * ekpump[i];
          p.x -= ce * (o.x + ekp_up[i] * w.x + q.x);
          p.y -= ce * (o.y + ekp_up[i] * w.y + q.y);
        }
      } else if (m != 0) {
        p = cscale(r[i], p);
        if (!cor_imp) p = csub(p, cim(I.CorFac * dm * r[i], psi[i]));
        if (!buo_imp) {
          p = csub(p, cim(I.BuoFac * rgrav[i] * dm, T[i]));
          if (chem) p = csub(p, cim(I.ChemFac * rgrav[i] * dm, X[i]));
        }
        if (I.flags & PZF_EK_PUMP) {
          const double2 u = us[i];
          const double2 q = make_double2(ekp_us[i] * u.x - ekp_dusdp[i] * dm * u.y,
                                         ekp_us[i] * u.y + ekp_dusdp[i] * dm * u.x);
          const double2 o = om[i], w = up[i];
          const double ce = I.CorFac * ekpump[i] * r[i];
          p.x -= ce * (o.x + ekp_up[i] * w.x + q.x);
          p.y -= ce * (o.y + ekp_up[i] * w.y + q.y);
        }
        p = csub(p, s.g[i]);
      } else if (I.flags & PZF_EK_PUMP) {
        p = csub(p, cscale(I.CorFac * ekpump[i], up[i]));
      }
      s.e[i] = p;
    }
    __syncthreads();
    op_C(V, n, s.a, s.b, s.w);
    __syncthreads();
    op_C(V, n, s.e, s.f, s.w);
    __syncthreads();
    trunc_cheb(s.b, n, n_max);
    trunc_cheb(s.f, n, n_max);
    __syncthreads();
    band_mv(band1(V, IM_I2R1), n, s.b, eT);
    band_mv(band1(V, (m == 0 || dmat) ? IM_I2R2 : IM_I4R3), n, s.f, eP);
    __syncthreads();
    if (chem) {
      // finish_exp_xi_int (update_xi_integ.f90:280-357): the temperature's
      // finish with dxicond and no tadvz term
      for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = V.fld(F_DVSXI, mi)[i];
      __syncthreads();
      op_C(V, n, s.a, s.b, s.w);
      __syncthreads();
      trunc_cheb(s.b, n, n_max);
      __syncthreads();
      op_D1c(V, n, s.b, s.c, s.w);                               // d(u_s r xi)/dr (dealiased)
      __syncthreads();
      const double* dxicond = V.rad(RV_DXICOND);
      double2* eX = V.hist(2, 2, c.eslot, mi);
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double g = rot ? (rc2 - r[i] * r[i]) * dxicond[i] : dxicond[i];
        s.a[i] = csub(csub(cscale(r[i], eX[i]), cim(dm * g, psi[i])), s.c[i]);
      }
      __syncthreads();
      op_C(V, n, s.a, s.b, s.w);
      __syncthreads();
      trunc_cheb(s.b, n, n_max);
      __syncthreads();
      band_mv(band1(V, IM_I2R1), n, s.b, eX);
      __syncthreads();
    }
  }
  if (!c.do_solve) return false;
  if (S.bridge) integ_imp<CHEM>(V, I, mi, S.r_old, S.r_impl, true, false, s, !dmat);

  // -- temperature: T_hat = G_T rhs, rhs(1:2) = topt, bott = 0
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = c.dirk ? dirk_rhs(V, I, S, 0, mi, i, c.stage) : imex_rhs(V, I, S, 0, mi, i);
    s.a[i] = i < 2 ? make_double2(0.0, 0.0) : v;
  }
  __syncthreads();
  integ_apply(d, I, I.o_gt, mi, false, s.a, s.b, s.st, s.red);
  __syncthreads();
  op_C(V, n, s.b, s.f, s.w);                                     // T (physical), kept in s.f
  __syncthreads();
  op_D1c(V, n, s.b, s.c, s.w);                                   // dT/dr
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 t = s.f[i];
    T[i] = t;
    dT[i] = s.c[i];
    bad |= !isfinite(t.x) || !isfinite(t.y);
  }
  if (c.wold) band_mv(band1(V, IM_I2R2), n, s.b, V.hist(0, 0, c.oslot, mi));
  if (c.calc) band_mv(band_tlap(V, dm2, I.TdiffFac), n, s.b, V.hist(0, 1, c.islot, mi));
  __syncthreads();
  if (chem) {
    // -- composition (update_xi_int, update_xi_integ.f90:167-278): xi_hat = G_xi rhs
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 v = c.dirk ? dirk_rhs(V, I, S, 2, mi, i, c.stage) : imex_rhs(V, I, S, 2, mi, i);
      s.a[i] = i < 2 ? make_double2(0.0, 0.0) : v;               // topxi, botxi = 0
    }
    __syncthreads();
    integ_apply(d, I, I.o_gx, mi, false, s.a, s.b, s.st, s.red);
    __syncthreads();
    op_C(V, n, s.b, s.g, s.w);                                   // xi (physical)
    __syncthreads();
    op_D1c(V, n, s.b, s.c, s.w);                                 // dxi/dr
    __syncthreads();
    double2* dX = V.fld(F_DXI, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 t = s.g[i];
      X[i] = t;
      dX[i] = s.c[i];
      bad |= !isfinite(t.x) || !isfinite(t.y);
    }
    if (c.wold) band_mv(band1(V, IM_I2R2), n, s.b, V.hist(2, 0, c.oslot, mi));
    if (c.calc) band_mv(band_tlap(V, dm2, I.XidiffFac), n, s.b, V.hist(2, 1, c.islot, mi));
    __syncthreads();
  }

  double2* oP = V.hist(1, 0, c.oslot, mi);
  double2* iP = V.hist(1, 1, c.islot, mi);
  if (m == 0) {
    // u_phi: real solve, then om = du/dr + u/r
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 v = c.dirk ? dirk_rhs(V, I, S, 1, mi, i, c.stage) : imex_rhs(V, I, S, 1, mi, i);
      s.a[i] = make_double2(v.x, 0.0);
    }
    __syncthreads();
    integ_apply(d, I, I.o_guphi, 0, false, s.a, s.b, s.st, s.red);  // u_phi, Chebyshev
    __syncthreads();
    op_C(V, n, s.b, s.g, s.w);
    __syncthreads();
    if (I.flags & PZF_RERR) {
      dcheb_thr(s.b, s.c, n, I.rerr_thr);                        // get_dr_real_1d, l_dct=.false.
      op_C(V, n, s.c, s.e, s.w);
      __syncthreads();
      const double drx = 2.0 / (I.r_cmb - I.r_icb);
      for (int i = threadIdx.x; i < n; i += blockDim.x) s.e[i] = cscale(drx, s.e[i]);
    } else {
      op_D1c(V, n, s.b, s.e, s.w);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double u = s.g[i].x;
      us[i] = make_double2(0.0, 0.0);
      up[i] = make_double2(u, 0.0);
      om[i] = make_double2(s.e[i].x + or1[i] * u, 0.0);
      s.g[i] = make_double2(u, 0.0);
      bad |= !isfinite(u);
    }
    __syncthreads();
    op_C(V, n, s.g, s.a, s.w);                                   // costf1(Re u_phi)
    __syncthreads();
    if (c.wold) band_mv(band1(V, IM_I2R2), n, s.a, oP);
    if (c.calc) band_mv(band1(V, IM_ULAP, I.ViscFac), n, s.a, iP);
    return bad;
  }
  // -- streamfunction, m /= 0: buoyancy I4R4 C(-BuoFac rgrav/r i m T) (I2R2 with
  // the influence matrix) with the new T
  if (buo_imp) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 b = cscale(-I.BuoFac * rgrav[i] * or1[i], cim(dm, s.f[i]));
      if (chem) b = csub(b, cscale(I.ChemFac * rgrav[i] * or1[i], cim(dm, X[i])));
      s.a[i] = b;
    }
    __syncthreads();
    op_C(V, n, s.a, s.c, s.w);
    __syncthreads();
    band_mv(band1(V, dmat ? IM_I2R2 : IM_I4R4), n, s.c, s.e);
    __syncthreads();
  }
  if (dmat) return integ_dmat_psi(d, V, I, S, mi, c, s) || bad;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 v = c.dirk ? dirk_rhs(V, I, S, 1, mi, i, c.stage) : imex_rhs(V, I, S, 1, mi, i);
    if (buo_imp) v = cadd(v, cscale(S.wimp_lin[0], s.e[i]));
    s.a[i] = v;
  }
  __syncthreads();
  integ_apply_sm(d, I, mi, s.a, s.b, s.st, s.red);
  __syncthreads();
  op_C(V, n, s.b, s.h, s.w);                                     // psi
  __syncthreads();
  op_Dc2(V, n, s.b, s.c, s.g, s.w);                              // dpsi/dr, d2psi/dr2
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 p = s.h[i], dp = s.c[i], d2p = s.g[i];
    psi[i] = p;
    double2 o;
    if (rot) {
      const double h2 = rc2 - r[i] * r[i];
      us[i] = cscale(or1[i] * h2, cim(dm, p));
      up[i] = make_double2(-h2 * dp.x + 3.0 * r[i] * p.x, -h2 * dp.y + 3.0 * r[i] * p.y);
      const double a1 = rc2 * or1[i] - 6.0 * r[i], a0 = 6.0 + dm2 * or2[i] * h2;
      o = make_double2(-h2 * d2p.x - a1 * dp.x + a0 * p.x, -h2 * d2p.y - a1 * dp.y + a0 * p.y);
    } else {
      // update_psi_integ_smat.f90:474-499: us = i m psi / r, up = -dpsi/dr,
      // om = -Lap_m psi
      us[i] = cscale(or1[i], cim(dm, p));
      up[i] = make_double2(-dp.x, -dp.y);
      const double a0 = dm2 * or2[i];
      o = make_double2(-d2p.x - or1[i] * dp.x + a0 * p.x, -d2p.y - or1[i] * dp.y + a0 * p.y);
    }
    om[i] = o;
    bad |= !isfinite(o.x) || !isfinite(o.y);
  }
  if (c.wold) band_mv(band_rot(V, dm2), n, s.b, oP);
  if (c.calc) {
    band_mv(band_rot2(V, dm2, I.ViscFac), n, s.b, s.k);
    band_mv(band1(V, IM_I4R4, I.CorFac * dm), n, s.b, s.a);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 v = s.k[i];
      if (cor_imp) v = cadd(v, cim(-1.0, s.a[i]));
      if (buo_imp) v = cadd(v, s.e[i]);
      iP[i] = v;
    }
  }
  return bad;
}

// Device kernels of the pizza time step (collocation, influence-matrix
// solve, multistep IMEX schemes) for sm_103a.  FP64 throughout.
//
// One time step of every instance of the batch is five launches:
//   k_rloop  (instance, r)  radial_loop: phi-FFTs, nonlinear products, CFL
//   k_cfl    (instance)     dt_courant, dt roll, IMEX weights, rebuild flag
//   k_build  (instance, m)  LU-equivalent operators when dt changed
//   k_mloop  (instance, m)  finish_explicit_assembly + mloop solves
//   k_obs    (instance)     time series (e_kin, e_kin_3D, heat)
// Work lists of (instance, r) and (instance, m) items make one launch cover a
// ragged batch of instances of different sizes.
#include <cuda_runtime.h>
#include <math.h>

#include "pizza_gpu.h"
#include "pz_device.cuh"
#include "pz_internal.h"

namespace {

// ---------------------------------------------------------------------------
// IMEX weights of the multistep family (src/multistep_schemes.f90:137-306)
// ---------------------------------------------------------------------------
__device__ bool set_weights(const PzInst& I, PzState& S) {
  if (I.dirk) {
    // DIRK (dirk_schemes.f90:275-712): the Butcher tables are scaled by dt(1)
    // where they are used; no rebuild request of its own
    S.wimp_lin[0] = I.dirk_gamma * S.dt[0];
    return false;
  }
  const double wimp_old = S.wimp_lin[0];
  const double* dt = S.dt;
  const double one = 1.0, half = 0.5, two = 2.0;
  switch (I.scheme) {
    case PZ_CNAB2:
      S.wimp[0] = one;
      S.wimp_lin[0] = I.alpha * dt[0];
      S.wimp_lin[1] = (1.0 - I.alpha) * dt[0];
      S.wexp[0] = (one + half * dt[0] / dt[1]) * dt[0];
      S.wexp[1] = -half * dt[0] * dt[0] / dt[1];
      break;
    case PZ_CNLF: {
      const double delta = dt[0] / dt[1];
      S.wimp[0] = (one - delta) * (one + delta);
      S.wimp[1] = delta * delta;
      S.wimp_lin[0] = half * (one + delta) / delta * dt[0];
      S.wimp_lin[1] = half * (one + delta) * (delta - one) / delta * dt[0];
      S.wimp_lin[2] = half * (one + delta) * dt[0];
      S.wexp[0] = (one + delta) * dt[0];
      S.wexp[1] = 0.0;
    } break;
    case PZ_MODCNAB: {
      const double delta = dt[0] / dt[1];
      S.wimp[0] = one;
      S.wimp[1] = 0.0;
      S.wimp_lin[0] = (half + 1.0 / delta / 16.0) * dt[0];
      S.wimp_lin[1] = (7.0 / 16.0 - 1.0 / delta / 16.0) * dt[0];
      S.wimp_lin[2] = 1.0 / 16.0 * dt[0];
      S.wexp[0] = (one + half * delta) * dt[0];
      S.wexp[1] = -half * delta * dt[0];
    } break;
    case PZ_SBDF2: {
      const double delta = dt[0] / dt[1];
      S.wimp_lin[0] = (one + delta) / (one + two * delta) * dt[0];
      S.wimp_lin[1] = 0.0;
      S.wimp[0] = (one + delta) * (one + delta) / (one + two * delta);
      S.wimp[1] = -delta * delta / (one + two * delta);
      S.wexp[0] = (one + delta) * (one + delta) * dt[0] / (one + two * delta);
      S.wexp[1] = -delta * (one + delta) * dt[0] / (one + two * delta);
    } break;
    case PZ_SBDF3: {
      const double dn = dt[1] / dt[0], dn1 = dt[2] / dt[0];
      const double a0 = one + one / (one + dn) + one / (one + dn + dn1);
      const double a1 = (one + dn) * (one + dn + dn1) / (dn * (dn + dn1));
      const double a2 = -(one + dn + dn1) / (dn * dn1 * (one + dn));
      const double a3 = (one + dn) / (dn1 * (dn + dn1) * (one + dn + dn1));
      const double b0 = (one + dn) * (one + dn + dn1) / (dn * (dn + dn1));
      const double b1 = -(one + dn + dn1) / (dn * dn1);
      const double b2 = (one + dn) / (dn1 * (dn + dn1));
      S.wimp_lin[0] = one / a0 * dt[0];
      S.wimp_lin[1] = 0.0;
      S.wimp[0] = a1 / a0; S.wimp[1] = a2 / a0; S.wimp[2] = a3 / a0;
      S.wexp[0] = b0 / a0 * dt[0]; S.wexp[1] = b1 / a0 * dt[0]; S.wexp[2] = b2 / a0 * dt[0];
    } break;
    case PZ_TVB33: {
      const double gam = (2619.0 - sqrt(5995281.0)) / 345.0;
      const double theta = (3525.0 * gam * gam - 3118.0 * gam - 5084.0) / 5468.0;
      const double c = (2178.0 * theta - 959.0 * gam * gam + 130.0 * gam + 726.0) / 4096.0;
      const double dn = dt[0] / dt[1], dn1 = dt[1] / dt[2];
      const double a3 = -pow(dn1, 3) * dn * dn * (3.0 * gam * gam * dn + two * gam * (one - dn) - one) /
                        (one + dn1) / (one + dn1 * (one + dn));
      const double a2 = -dn * dn * (gam * dn * dn1 * (two - 3.0 * gam) + (one - two * gam) * (one + dn1)) / (one + dn);
      const double a1 = -(dn1 * (one + gam * dn) * (1 + dn * (3.0 * gam - two)) + dn * (two * gam - one) + one) /
                            (one + dn1) - theta;
      const double a0 = theta + (one + two * gam * dn + dn1 * (one + gam * dn) * (one + 3.0 * gam * dn)) /
                                    (one + dn) / (one + dn1 * (one + dn));
      const double b2 = dn1 * dn1 * dn * (6.0 * gam * (one + gam * dn) + theta * (3.0 + two * dn)) / (6.0 * (one + dn1));
      const double b1 = -gam * dn * (one + dn1 * (one + gam * dn)) - theta / 6.0 * dn * (3.0 + dn1 * (3.0 + two * dn));
      const double b0 = (one + gam * dn) * (one + dn1 * (one + gam * dn)) / (one + dn1) +
                        theta * (one + 0.5 * dn + dn1 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)));
      const double c3 = theta * dn1 * dn1 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)) - c;
      const double c2 = (c * (one + dn1) * (one + dn1 * (one + dn)) - dn1 * dn1 * dn * dn * gam * (one - gam)) /
                            (dn1 * dn1 * (one + dn)) - theta * dn * (3.0 + dn1 * (3.0 + 2.0 * dn)) / 6.0;
      const double c1 = (dn1 * dn1 * dn * (one - gam) * (one + gam * dn) - c * (one + dn1 * (one + dn))) / (dn1 * dn1) / dn +
                        theta * (one + 0.5 * dn + dn1 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)));
      const double c0 = (dn1 * dn1 * dn * gam * (one + gam * dn) + c * (one + dn1)) / (dn1 * dn1 * dn * (one + dn));
      S.wimp_lin[0] = c0 / a0 * dt[0]; S.wimp_lin[1] = c1 / a0 * dt[0];
      S.wimp_lin[2] = c2 / a0 * dt[0]; S.wimp_lin[3] = c3 / a0 * dt[0];
      S.wimp[0] = -a1 / a0; S.wimp[1] = -a2 / a0; S.wimp[2] = -a3 / a0;
      S.wexp[0] = b0 / a0 * dt[0]; S.wexp[1] = b1 / a0 * dt[0]; S.wexp[2] = b2 / a0 * dt[0];
    } break;
    case PZ_SBDF4: {
      const double dn = dt[0] / dt[1], dn1 = dt[1] / dt[2], dn2 = dt[2] / dt[3];
      const double c1 = one + dn2 * (one + dn1);
      const double c2 = one + dn1 * (one + dn);
      const double c3 = one + dn2 * c2;
      const double a4 = (one + dn) / (one + dn2) * c2 / c1 / c3 * (pow(dn2, 4) * pow(dn1, 3) * dn * dn);
      const double a3 = -pow(dn1, 3) * dn * dn * (one + dn) / (one + dn1) * c3 / c2;
      const double a2 = dn * (dn / (one + dn) + dn1 * dn * (c3 + dn2) / (one + dn2));
      const double a1 = -one - dn * (one + dn1 * (one + dn) * (one + dn2 * c2 / c1) / (one + dn1));
      const double a0 = one + dn / (one + dn) + dn1 * dn / c2 + dn2 * dn1 * dn / c3;
      const double b3 = -pow(dn2, 3) * dn1 * dn1 * dn * (one + dn) / (one + dn2) * c2 / c1;
      const double b2 = dn1 * dn1 * dn * (one + dn) / (one + dn1) * c3;
      const double b1 = -c2 * c3 * dn / (one + dn2);
      const double b0 = dn1 * (one + dn) / (one + dn1) * ((one + dn) * (c3 + dn2) + (one + dn2) / dn1) / c1;
      S.wimp_lin[0] = one / a0 * dt[0];
      S.wimp_lin[1] = 0.0;
      S.wimp[0] = -a1 / a0; S.wimp[1] = -a2 / a0; S.wimp[2] = -a3 / a0; S.wimp[3] = -a4 / a0;
      S.wexp[0] = b0 / a0 * dt[0]; S.wexp[1] = b1 / a0 * dt[0];
      S.wexp[2] = b2 / a0 * dt[0]; S.wexp[3] = b3 / a0 * dt[0];
    } break;
    default:
      break;
  }
  return S.wimp_lin[0] != wimp_old;
}

// bridge_with_cnab2 (multistep_schemes.f90:500-522)
__device__ void bridge_with_cnab2(const PzInst& I, PzState& S) {
  PzInst J = I;
  J.scheme = PZ_CNAB2;
  set_weights(J, S);
  for (int k = 1; k < I.nold; ++k) S.wimp[k] = 0.0;
  for (int k = 2; k < I.nimp + 1; ++k) S.wimp_lin[k] = 0.0;
  for (int k = 2; k < I.nexp; ++k) S.wexp[k] = 0.0;
}

// ---------------------------------------------------------------------------
// k_rloop: radial_loop for PZ_RLOOP_G radii of one instance, reading the
// m-major step state and writing the explicit slot, dVsT, dVsOm and the
// Courant steps (src/radial_loop.f90:231-394)
// ---------------------------------------------------------------------------
struct StepIO {
  View V;
  int N;
  double2 *us, *up, *om, *T, *eT, *eP, *vsT, *vsOm;
  double2 *X, *eX, *vsX;     // composition (null without it)
  double* cflv;
  // grid snapshot of this stage's state (gsnap null: none), PzDev::gsnap
  double2* gsnap;
  const long long* o_gsnap;
  int gslot, inst;
  __device__ double2 in(int f, int m, int r) const {
    const long long o = (long long)m * N + r;
    return f == 0 ? us[o] : f == 1 ? up[o] : f == 2 ? om[o] : f == 3 ? T[o] : X[o];
  }
  __device__ void outx(int m, int r, double2 dxdt, double2 vsx) const {
    const long long o = (long long)m * N + r;
    eX[o] = dxdt;
    vsX[o] = vsx;
  }
  __device__ void out(int m, int r, double2 dtdt, double2 vst, double2 dpdt, double2 vsom) const {
    const long long o = (long long)m * N + r;
    eT[o] = dtdt;
    vsT[o] = vst;
    eP[o] = dpdt;
    vsOm[o] = vsom;
  }
  __device__ void cfl(int r, double dtr, double dth) const {
    cflv[r] = dtr;
    cflv[N + r] = dth;
  }
  // the c2r grids of a radius group, [g][field pair][P] from offset `off`
  __device__ void grid(const double2* g, long long off, int n) const {
    if (!gsnap) return;
    double2* gs = gsnap + o_gsnap[inst] + (long long)gslot * N * 2 * V.I->P + off;
    for (int k = threadIdx.x; k < n; k += blockDim.x) gs[k] = g[k];
  }
};

template <bool CHEM>
__global__ void __launch_bounds__(256, CHEM ? 3 : 4) k_rloop(PzDev d, int stage) {
  extern __shared__ double2 sh[];
  const PzItem it = d.ritems[blockIdx.x];
  const PzInst& I = d.inst[it.inst];
  const PzState& S = d.state[it.inst];
  if (S.status != 0 || stage > I.nstages) return;
  if (I.dirk && !((I.exp_mask >> (stage - 1)) & 1)) return;   // l_exp_calc(stage)
  const int eslot = I.dirk ? stage - 1 : S.b_expl;
  const View V{&I, d.pool};
  StepIO io;
  io.V = V;
  io.N = I.N;
  io.us = V.fld(F_US, 0); io.up = V.fld(F_UP, 0); io.om = V.fld(F_OM, 0); io.T = V.fld(F_TEMP, 0);
  io.eT = V.hist(0, 2, eslot, 0);
  io.eP = V.hist(1, 2, eslot, 0);
  io.vsT = V.fld(F_DVST, 0);
  io.vsOm = V.fld(F_DVSOM, 0);
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  io.X = chem ? V.fld(F_XI, 0) : nullptr;
  io.eX = chem ? V.hist(2, 2, eslot, 0) : nullptr;
  io.vsX = chem ? V.fld(F_DVSXI, 0) : nullptr;
  io.cflv = d.pool + I.o_cfl;
  io.gsnap = chem ? nullptr : d.gsnap;
  io.o_gsnap = d.o_gsnap;
  io.gslot = d.gsnap_slot0 + stage - 1;
  io.inst = it.inst;
  double* rsh = reinterpret_cast<double*>(sh + (chem ? 6 : 4) * I.rg * I.P);
  rloop_group<CHEM>(I, V, it.idx, I.rg, io, sh, rsh);
}

// ---------------------------------------------------------------------------
// k_cfl: dt_courant, set_dt_array, set_weights, lMat, bridge, ring bases
// (src/courant.f90:78-167, src/step_time.f90:281-329)
// ---------------------------------------------------------------------------
__global__ void k_cfl(PzDev d) {
  const int inst = d.cfl_inst ? d.cfl_inst[blockIdx.x] : (int)blockIdx.x;
  const PzInst& I = d.inst[inst];
  PzState& S = d.state[inst];
  if (S.status != 0) return;
  const double* cfl = d.pool + I.o_cfl;
  double dtr = 1000.0 * I.dtMax, dth = dtr;
  for (int r = threadIdx.x; r < I.N; r += 32) {
    dtr = fmin(dtr, cfl[r]);
    dth = fmin(dth, cfl[I.N + r]);
  }
  dtr = warp_min(dtr);
  dth = warp_min(dth);
  if (threadIdx.x != 0) return;
  const double dt = S.dt[0];
  const double dt_rh = fmin(dtr, dth);
  const double dt_2 = fmin(0.5 * (1.0 / I.dt_fac + 1.0) * dt_rh, I.dtMax);
  bool l_new_dt;
  double dt_new;
  if (dt > I.dtMax) { l_new_dt = true; dt_new = I.dtMax; }
  else if (dt > dt_rh) { l_new_dt = true; dt_new = dt_2; }
  else if (I.dt_fac * dt < dt_rh && dt < I.dtMax) { l_new_dt = true; dt_new = dt_2; }
  else { l_new_dt = false; dt_new = dt; }
  const long long ks = (long long)inst * d.sched_n + S.n_step;
  if (d.sched_mode == 1 && S.n_step < d.sched_n) {
    dt_new = d.dt_io[ks];
    l_new_dt = dt_new != dt;
  } else if (d.sched_mode == 2 && S.n_step < d.sched_n) {
    d.dt_io[ks] = dt_new;
  }
  if (!I.dirk)
    for (int k = I.nexp - 1; k > 0; --k) S.dt[k] = S.dt[k - 1];
  S.dt[0] = dt_new;
  if (dt_new < I.dtMin) { S.status = PZ_E_DT_TOO_SMALL; return; }
  if (set_weights(I, S)) S.lMatNext = 1;
  S.time = S.time + S.dt[0];
  S.lMat = (S.lMatNext || l_new_dt) ? 1 : 0;
  if (S.lMat) S.w_lhs = S.wimp_lin[0];
  S.lMatNext = 0;
  S.n_step += 1;
  S.bridge = (!I.dirk && I.scheme != PZ_CNAB2 && S.n_step <= I.nold - 1) ? 1 : 0;
  if (S.bridge) bridge_with_cnab2(I, S);
  if (S.ab1) {
    // l_AB1 after a restart (checkpoints.f90:398-425): first-order explicit
    // weights on the run's first step (step_time.f90:309-314)
    if (S.n_step == 1) {
      S.wexp[0] = S.dt[0];
      for (int k = 1; k < 4; ++k) S.wexp[k] = 0.0;
    }
    S.ab1 = 0;
  }
  S.l_calc_lin = (I.flags & PZF_IMP_CALC) ? 1 : 0;
  if (!I.dirk) {
    // rotate_imex on rings: this step reads slots from r_*, writes logical slot 1 at b_*
    S.r_old = S.b_old; S.r_impl = S.b_impl; S.r_expl = S.b_expl;
    S.b_old = (S.b_old + I.nold - 1) % I.nold;
    S.b_impl = (S.b_impl + I.nimp - 1) % I.nimp;
    S.b_expl = (S.b_expl + I.nexp - 1) % I.nexp;
  }   // DIRK: slots are stages, nothing rotates (dirk_schemes.f90:833-838)
  if (d.rec && ks < (long long)(inst + 1) * d.sched_n) d.rec[ks] = S;
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inversion with partial pivoting of a row-major n x n matrix in
// shared memory (in place).  Returns 0, or -1 on a zero pivot.
//
// Three phases and three barriers per pivot: (1) each warp proposes the
// largest |A(i,k)|, i >= k (first index on ties, idamax semantics) with its
// signed value; (2) every thread reduces the warps' proposals itself (the
// same result everywhere), then the pivot row is swapped in, scaled by one
// reciprocal of the pivot, and the pivot column of the other rows is saved;
// (3) elimination.  The column swaps that undo the row pivoting are composed
// into one permutation and applied per row, cycle by cycle, at the end.
// T is double or double2 (izamax's |re| + |im| for the complex pivot).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double gj_abs(double a) { return fabs(a); }
__device__ __forceinline__ double gj_abs(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ bool gj_zero(double a) { return a == 0.0; }
__device__ __forceinline__ bool gj_zero(double2 a) { return a.x == 0.0 && a.y == 0.0; }
__device__ __forceinline__ double gj_inv(double a) { return 1.0 / a; }
__device__ __forceinline__ double2 gj_inv(double2 a) {
  const double den = a.x * a.x + a.y * a.y;
  return make_double2(a.x / den, -a.y / den);
}
__device__ __forceinline__ double gj_mul(double a, double b) { return a * b; }
__device__ __forceinline__ double2 gj_mul(double2 a, double2 b) { return cmul(a, b); }
__device__ __forceinline__ double gj_axpy(double a, double c, double b) { return fma(-c, b, a); }   // a - c b
__device__ __forceinline__ double2 gj_axpy(double2 a, double2 c, double2 b) { return csub(a, cmul(c, b)); }
__device__ __forceinline__ double gj_one(double) { return 1.0; }
__device__ __forceinline__ double2 gj_one(double2) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ double gj_nil(double) { return 0.0; }
__device__ __forceinline__ double2 gj_nil(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double gj_shfl(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double2 gj_shfl(double2 v, int o) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}
// a warp's signed pivot candidate in red[8 + w] (and its imaginary part in red[16 + w])
__device__ __forceinline__ void gj_put(double* red, int w, double a) { red[8 + w] = a; }
__device__ __forceinline__ void gj_put(double* red, int w, double2 a) { red[8 + w] = a.x; red[16 + w] = a.y; }
__device__ __forceinline__ void gj_get(const double* red, int w, double& a) { a = red[8 + w]; }
__device__ __forceinline__ void gj_get(const double* red, int w, double2& a) { a = make_double2(red[8 + w], red[16 + w]); }

// blockDim <= 256 (at most 8 warps); red: 32 doubles (per warp |pivot| at
// [0, 8), the signed pivot at [8, 24)); colk: n values of T (also the
// permutation scratch, 2n ints, at the end)
template <class T>
__device__ int gj_core(T* A, int n, int* piv, T* colk, double* red, int* redi) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int k = 0; k < n; ++k) {
    // (1) per-warp pivot proposals
    double best = -1.0;
    int bi = n;
    T bv = gj_nil(T());
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      const T a = A[i * n + k];
      const double v = gj_abs(a);
      if (v > best) { best = v; bi = i; bv = a; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const T oa = gj_shfl(bv, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; bv = oa; }
    }
    if (lane == 0) {
      red[wid] = best;
      redi[wid] = bi;
      gj_put(red, wid, bv);
    }
    __syncthreads();
    // (2) every thread picks the pivot; swap, scale, save the pivot column
    double b = red[0];
    int p = redi[0];
    int pw = 0;
    for (int w = 1; w < nw; ++w)
      if (red[w] > b || (red[w] == b && redi[w] < p)) { b = red[w]; p = redi[w]; pw = w; }
    T pv;
    gj_get(red, pw, pv);
    if (p >= n || gj_zero(pv)) return -1;
    if (threadIdx.x == 0) piv[k] = p;
    const T rinv = gj_inv(pv);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const T ak = A[k * n + j], ap = A[p * n + j];
      if (p != k) A[p * n + j] = ak;
      A[k * n + j] = gj_mul(j == k ? gj_one(T()) : ap, rinv);
      if (j == k && p != k) colk[p] = ak;     // the old A(k,k) is row p's pivot-column entry now
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (i != k && i != p) colk[i] = A[i * n + k];
    __syncthreads();
    // (3) elimination
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int i = idx / n, j = idx - i * n;
      if (i != k) A[idx] = gj_axpy(j == k ? gj_nil(T()) : A[idx], colk[i], A[k * n + j]);
    }
    __syncthreads();
  }
  // undo the row pivoting: the column swaps (k, piv[k]), k = n-1 .. 0, as
  // one map src (final column j = current column src[j]) applied cycle by
  // cycle in each row; lead marks the smallest index of each cycle
  int* src = reinterpret_cast<int*>(colk);
  int* lead = src + n;
  if (threadIdx.x == 0) {
    for (int j = 0; j < n; ++j) { src[j] = j; lead[j] = 0; }
    for (int k = n - 1; k >= 0; --k) {
      const int p = piv[k];
      const int t = src[k]; src[k] = src[p]; src[p] = t;
    }
    for (int j = 0; j < n; ++j) {
      if (lead[j] != 0) continue;
      lead[j] = 1;
      for (int q = src[j]; q != j; q = src[q]) lead[q] = 2;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T* row = A + (long long)i * n;
    for (int l = 0; l < n; ++l) {
      if (lead[l] != 1 || src[l] == l) continue;
      const T t = row[l];
      int j = l;
      while (src[j] != l) { row[j] = row[src[j]]; j = src[j]; }
      row[j] = t;
    }
  }
  __syncthreads();
  return 0;
}

__device__ int gj_invert(double* A, int n, int* piv, double* colk, double* red, int* redi) {
  return gj_core<double>(A, n, piv, colk, red, redi);
}

// Boundary rows and the Chebyshev boundary factor of the collocation builders.
// Row i of the matrix is written to A (row-major); `rowfn` gives interior rows.
struct BuildCtx {
  const PzInst* I;
  const double* rM; const double* drM; const double* d2rM;   // column-major N x N
  int N;
  __device__ double rm(int i, int k) const { return rM[i + (long long)k * N]; }
  __device__ double drm(int i, int k) const { return drM[i + (long long)k * N]; }
  __device__ double d2rm(int i, int k) const { return d2rM[i + (long long)k * N]; }
};

// Write G (= X in shared row-major, scaled) to global column-major, rows >=
// n_max zeroed (dealiasing): G(i,j) = rs[i] * X(i,j) * cs[j].
__device__ void store_op(double* G, const double* X, int n, int n_max, const double* rs, const double* cs) {
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int j = idx / n, i = idx - j * n;
    double v = 0.0;
    if (i < n_max) {
      v = X[i * n + j];
      if (rs) v = rs[i] * v;
      if (cs) v = v * cs[j];
    }
    G[idx] = v;
  }
}

// Row and column equilibration of get_omMat/get_psiMat
// (update_psi_coll_dmat.f90:881-897): f1 = 1/max|row|, then f2 = 1/max|col|.
__device__ void equilibrate(double* A, int n, double* f1, double* f2, bool cols) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double mx = 0.0;
    for (int j = 0; j < n; ++j) mx = fmax(mx, fabs(A[i * n + j]));
    f1[i] = 1.0 / mx;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) A[idx] *= f1[idx / n];
  __syncthreads();
  if (!cols) return;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double mx = 0.0;
    for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(A[i * n + j]));
    f2[j] = 1.0 / mx;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) A[idx] *= f2[idx - (idx / n) * n];
  __syncthreads();
}

// kind: 0 temperature (get_tempMat), 1 omega (get_omMat), 2 psi (get_psiMat),
// 3 uphi (get_uphiMat), 4 DIRK assembly psi (get_assMat), 5 composition
// (get_xiMat).  Fills A (row-major) before scaling.
__device__ void fill_matrix(double* A, const BuildCtx& B, const View& V, int kind, int m, double wlin) {
  const PzInst& I = *B.I;
  const int n = B.N, n_max = I.n_max;
  const double rn = I.rnorm, dm2 = (double)m * (double)m;
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
  const double* dbeta = V.rad(RV_DBETA);
  const double* ekp = V.rad(RV_EKPUMP);
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, k = idx - i * n;
    double v;
    if (kind == 4 && (i == 1 || i == n - 2)) {
      // get_assMat: dpsi/dr = 0 on the rigid walls in the second and
      // second-last rows (update_psi_coll_smat.f90:839-917)
      v = (k >= n_max) ? 0.0 : rn * B.drm(i == 1 ? 0 : n - 1, k);
    } else if (i == 0 || i == n - 1) {
      if (k >= n_max) {
        v = 0.0;
      } else {
        // fixed temperature (ktopt=kbott=1), non-penetration, rigid u_phi
        // (ktopv=kbotv=2): rnorm*rMat on both boundary rows
        v = rn * B.rm(i, k);
      }
    } else {
      const double r0 = B.rm(i, k), r1 = B.drm(i, k), r2 = B.d2rm(i, k);
      if (kind == 0 || kind == 5) {
        const double diff = kind == 0 ? I.TdiffFac : I.XidiffFac;
        v = rn * (r0 - wlin * diff * (r2 + or1[i] * r1 - dm2 * or2[i] * r0));
      } else if (kind == 1) {
        v = rn * (r0 - wlin * I.ViscFac * (r2 + or1[i] * r1 - dm2 * or2[i] * r0));
      } else if (kind == 2) {
        v = rn * (r2 + (or1[i] + beta[i]) * r1 + (or1[i] * beta[i] + dbeta[i] - dm2 * or2[i]) * r0);
      } else if (kind == 4) {
        v = -rn * (r2 + (or1[i] + beta[i]) * r1 + (or1[i] * beta[i] + dbeta[i] - dm2 * or2[i]) * r0);
      } else {
        v = rn * (r0 - wlin * (I.ViscFac * (r2 + or1[i] * r1 - or2[i] * r0) - I.CorFac * ekp[i] * r0));
      }
    }
    if (k == 0 || k == n - 1) v = 0.5 * v;   // boundary_fac
    A[idx] = v;
  }
  __syncthreads();
}

// Entry (R, C) of the coupled operator of get_psiMat in
// update_psi_coll_smat.f90:674-837 before equilibration.  Rows 0..N-1 are the
// vorticity equation (boundary rows: psi = 0), rows N..2N-1 the streamfunction
// equation (boundary rows: dpsi/dr = 0, rigid walls); columns 0..N-1 are the
// Chebyshev coefficients of omega, N..2N-1 those of psi.  Ekman pumping and
// (corio_term='IMPLICIT') the Coriolis term couple omega to psi.
__device__ double2 smat_entry(const BuildCtx& B, const View& V, int m, double wlin, int R, int C) {
  const PzInst& I = *B.I;
  const int n = B.N;
  const double rn = I.rnorm, dm = (double)m, dm2 = dm * dm;
  const bool top = R < n, wcol = C < n;
  const int i = top ? R : R - n, k = wcol ? C : C - n;
  double re = 0.0, im = 0.0;
  if (i == 0 || i == n - 1) {
    if (!wcol && k < I.n_max) re = rn * (top ? B.rm(i, k) : B.drm(i, k));
  } else {
    const double r0 = B.rm(i, k), r1 = B.drm(i, k), r2 = B.d2rm(i, k);
    const double or1 = V.rad(RV_OR1)[i], or2 = V.rad(RV_OR2)[i], beta = V.rad(RV_BETA)[i];
    if (top && wcol) {
      const double ekp = V.rad(RV_EKPUMP)[i];
      re = rn * (r0 - wlin * (I.ViscFac * (r2 + or1 * r1 - dm2 * or2 * r0) - I.CorFac * ekp * r0));
    } else if (top) {
      const double ekp = V.rad(RV_EKPUMP)[i], eup = V.rad(RV_EKP_UP)[i];
      const double eus = V.rad(RV_EKP_US)[i], edp = V.rad(RV_EKP_DUSDP)[i];
      // -rn w CorFac ekp (eup d/dr + eup beta - (i m edp + eus) i m / r) - rn w CorFac beta i m / r
      re = -rn * wlin * I.CorFac * ekp * (eup * r1 + (eup * beta + edp * dm2 * or1) * r0);
      const double cor = (I.flags & PZF_COR_IMP) ? beta : 0.0;
      im = rn * wlin * I.CorFac * or1 * dm * (ekp * eus - cor) * r0;
    } else if (wcol) {
      re = rn * r0;
    } else {
      re = rn * (r2 + (or1 + beta) * r1 + (or1 * beta + V.rad(RV_DBETA)[i] - dm2 * or2) * r0);
    }
  }
  if (k == 0 || k == n - 1) { re *= 0.5; im *= 0.5; }   // boundary_fac
  return make_double2(re, im);
}

// Gauss-Jordan inversion with partial pivoting (pivot: max |re| + |im|, the
// cabs1 of izamax) of a complex row-major n x n matrix in shared memory.
__device__ int gj_invert_c(double2* A, int n, int* piv, double2* colk, double* red, int* redi) {
  return gj_core<double2>(A, n, piv, colk, red, redi);
}

// smat operator of one m /= 0 by block elimination of the equilibrated
// system As = diag(f1) A diag(f2) = [[A11, A12], [A21, D]] (f1 = 1/max|row|,
// then f2 = 1/max|col|, update_psi_coll_smat.f90:810-826): with E = D^-1 A21
// and the Schur complement S = A11 - A12 E (complex),
//   As^-1 [:, :N] = [S^-1 ; -E S^-1],
// so G = diag(f2) As^-1[:, :N] diag(f1[:N]) gives (omega, psi)_cheb = G rhs.
// Shared memory: S (complex N^2) | E (N^2, padded to an even count) | f1, f2,
// pivot column (2N each) | reductions | pivots; D^-1 occupies the first N^2
// doubles before S is formed.
// ws: the workspace (build_smat_smem_bytes(n)): shared memory, or for
// n_r_max above 97 the instance's global-memory workspace (PzInst::o_smat_ws)
__device__ int build_smat(double* G, const BuildCtx& B, const View& V, int m, double wlin, double* ws) {
  const PzInst& I = *B.I;
  const int n = B.N, n2 = 2 * n;
  double* X = ws;
  double2* Sx = reinterpret_cast<double2*>(X);
  double* E = X + 2LL * n * n;
  double* f1 = E + (((long long)n * n + 1) & ~1LL);   // even offset: colk below is read as double2
  double* f2 = f1 + n2;
  double* colk = f2 + n2;
  double* red = colk + n2;
  int* redi = reinterpret_cast<int*>(red + 32);
  int* piv = redi + 32;
  for (int R = threadIdx.x; R < n2; R += blockDim.x) {
    double mx = 0.0;
    for (int C = 0; C < n2; ++C) {
      const double2 a = smat_entry(B, V, m, wlin, R, C);
      mx = fmax(mx, hypot(a.x, a.y));
    }
    f1[R] = 1.0 / mx;
  }
  __syncthreads();
  for (int C = threadIdx.x; C < n2; C += blockDim.x) {
    double mx = 0.0;
    for (int R = 0; R < n2; ++R) {
      const double2 a = smat_entry(B, V, m, wlin, R, C);
      mx = fmax(mx, hypot(f1[R] * a.x, f1[R] * a.y));
    }
    f2[C] = 1.0 / mx;
  }
  __syncthreads();
  // D (real), then D^-1
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int k = idx / n, j = idx - k * n;
    X[idx] = f1[n + k] * smat_entry(B, V, m, wlin, n + k, n + j).x * f2[n + j];
  }
  __syncthreads();
  if (gj_invert(X, n, piv, colk, red, redi) != 0) return -1;
  // E = D^-1 A21 with A21(k, j) = f1[N+k] rnorm rMat(k, j) bf(j) f2[j] on interior rows
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    double acc = 0.0;
    for (int k = 1; k < n - 1; ++k) acc = fma(X[i * n + k] * f1[n + k], B.rm(k, j), acc);
    const double bf = (j == 0 || j == n - 1) ? 0.5 : 1.0;
    E[idx] = acc * I.rnorm * bf * f2[j];
  }
  __syncthreads();
  // S = A11 - A12 E
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    const double2 a = smat_entry(B, V, m, wlin, i, j);
    double re = f1[i] * a.x * f2[j], im = 0.0;
    for (int k = 0; k < n; ++k) {
      const double2 b = smat_entry(B, V, m, wlin, i, n + k);
      const double w = f1[i] * f2[n + k] * E[k * n + j];
      re = fma(-b.x, w, re);
      im = fma(-b.y, w, im);
    }
    Sx[idx] = make_double2(re, im);
  }
  __syncthreads();
  if (gj_invert_c(Sx, n, piv, reinterpret_cast<double2*>(colk), red, redi) != 0) return -1;
  double2* Gc = reinterpret_cast<double2*>(G);
  for (int idx = threadIdx.x; idx < n2 * n; idx += blockDim.x) {
    const int c = idx / n2, r = idx - c * n2;
    double2 v = make_double2(0.0, 0.0);
    if (r < n) {
      if (r < I.n_max) v = cscale(f2[r] * f1[c], Sx[r * n + c]);
    } else {
      const int i = r - n;
      if (i < I.n_max) {
        double vr = 0.0, vi = 0.0;
        for (int k = 0; k < n; ++k) {
          const double e = E[i * n + k];
          vr = fma(e, Sx[k * n + c].x, vr);
          vi = fma(e, Sx[k * n + c].y, vi);
        }
        v = make_double2(-f2[r] * vr * f1[c], -f2[r] * vi * f1[c]);
      }
    }
    Gc[idx] = v;
  }
  return 0;
}

struct BuildSmem {
  double* A; double* f1; double* f2; double* colk; double* red; int* redi; int* piv;
  double2* va; double2* vb;
};
// shared-memory layout of the builders, in doubles; see build_smem_bytes()
__device__ BuildSmem build_smem(int n) {
  extern __shared__ double shb[];
  BuildSmem s;
  long long off = 0;
  s.A = shb + off; off += (long long)n * n;
  s.f1 = shb + off; off += n;
  s.f2 = shb + off; off += n;
  s.colk = shb + off; off += n;
  s.red = shb + off; off += 32;
  s.redi = reinterpret_cast<int*>(shb + off); off += 16;
  s.piv = reinterpret_cast<int*>(shb + off); off += (n + 1) / 2;
  off = (off + 1) & ~1LL;
  s.va = reinterpret_cast<double2*>(shb + off); off += 2 * n;
  s.vb = reinterpret_cast<double2*>(shb + off);
  return s;
}

__device__ void flag_status(PzState& S, int code) {
  if (threadIdx.x == 0) atomicCAS(&S.status, 0, code);
}

// integration method (pz_integ.cuh, included below)
__device__ int integ_build(const PzDev& d, const PzInst& I, const View& V, int mi, double wlin);
__device__ int integ_psi_static(const PzDev& d, const PzInst& I, const View& V, int mi);

// dt independent streamfunction operators (update_psi_coll_dmat.f90:94-98)
__global__ void __launch_bounds__(PZ_THREADS) k_build_static(PzDev d) {
  const PzItem it = d.mitems[blockIdx.x];
  const PzInst& I = d.inst[it.inst];
  PzState& S = d.state[it.inst];
  if (it.idx == 0) return;
  const View V{&I, d.pool};
  if (I.flags & PZF_INTEG) {
    // the influence-matrix variant's dt-independent psi-from-omega inverse
    if (!(I.flags & PZF_DIRECT) && integ_psi_static(d, I, V, it.idx) != 0) flag_status(S, PZ_E_SINGULAR);
    return;
  }
  const int n = I.N, m = it.idx * I.minc;
  BuildSmem s = build_smem(n);
  BuildCtx B{&I, V.basis(BM_RMAT), V.basis(BM_DRMAT), V.basis(BM_D2RMAT), n};
  if (I.dirk && I.assembly) {
    // assembly-stage streamfunction operator (plain LU in the reference: no scaling)
    fill_matrix(s.A, B, V, 4, m, 0.0);
    if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
    store_op(d.pool + I.o_gass + (long long)it.idx * n * n, s.A, n, I.n_max, nullptr, nullptr);
    __syncthreads();
  }
  if (I.flags & PZF_DIRECT) return;
  fill_matrix(s.A, B, V, 2, m, 0.0);
  equilibrate(s.A, n, s.f1, s.f2, true);
  if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
  // K = G_psi P C with G_psi = diag(f2) A_s^-1 diag(f1) and P the projection
  // on the interior rows: the streamfunction solve psi = G_psi (-omega_phys)
  // of update_om_coll_dmat (update_psi_coll_dmat.f90:309-366) applied to the
  // Chebyshev coefficients of omega in one operator, psi = -K omega_cheb
  const double* C = V.basis(BM_C);
  double* K = d.pool + I.o_gpsi + (long long)it.idx * n * n;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int j = idx / n, i = idx - j * n;
    double v = 0.0;
    if (i < I.n_max) {
      double acc = 0.0;
      for (int l = 1; l < n - 1; ++l) acc = fma(s.A[i * n + l] * s.f1[l], C[l + (long long)j * n], acc);
      v = s.f2[i] * acc;
    }
    K[idx] = v;
  }
}

// dt dependent operators, rebuilt when lMat (step_time.f90:296-303):
// temperature, omega and u_phi, plus the influence-matrix ingredients.
template <bool CHEM>
__device__ __forceinline__ void build_item(const PzDev& d, const PzItem it) {
  const PzInst& I = d.inst[it.inst];
  PzState& S = d.state[it.inst];
  if (S.status != 0 || !S.lMat) return;
  const View V{&I, d.pool};
  const int n = I.N, mi = it.idx, m = mi * I.minc;
  const double wlin = S.wimp_lin[0];
  if (I.flags & PZF_INTEG) {
    if (integ_build(d, I, V, mi, wlin) != 0) flag_status(S, PZ_E_SINGULAR);
    return;
  }
  BuildSmem s = build_smem(n);
  BuildCtx B{&I, V.basis(BM_RMAT), V.basis(BM_DRMAT), V.basis(BM_D2RMAT), n};
  const bool shared = (I.flags & PZF_T_IS_OM) && m != 0;
  if (!shared) {
    // temperature (get_tempMat with WITH_PRECOND_S: row scaling only)
    fill_matrix(s.A, B, V, 0, m, wlin);
    equilibrate(s.A, n, s.f1, s.f2, false);
    if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
    store_op(d.pool + I.o_gt + (long long)mi * n * n, s.A, n, I.n_max, nullptr, s.f1);
    __syncthreads();
  }
  if (CHEM && (I.flags & PZF_CHEM)) {
    // composition (get_xiMat, update_xi_coll.f90:321-393: row scaling only)
    fill_matrix(s.A, B, V, 5, m, wlin);
    equilibrate(s.A, n, s.f1, s.f2, false);
    if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
    store_op(d.pool + I.o_gx + (long long)mi * n * n, s.A, n, I.n_max, nullptr, s.f1);
    __syncthreads();
  }
  if (m == 0) {
    fill_matrix(s.A, B, V, 3, 0, wlin);
    if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
    store_op(d.pool + I.o_guphi, s.A, n, I.n_max, nullptr, nullptr);
    return;
  }
  if (I.flags & PZF_DIRECT) {
    // coupled (omega, psi) operator of update_om_coll_smat
    __syncthreads();
    extern __shared__ double shb[];
    double* ws = I.o_smat_ws ? d.pool + I.o_smat_ws + (long long)mi * I.smat_ws_stride : shb;
    if (build_smat(d.pool + I.o_gsm + 4LL * mi * n * n, B, V, m, wlin, ws) != 0) flag_status(S, PZ_E_SINGULAR);
    return;
  }
  // omega (get_omMat: row and column scaling)
  fill_matrix(s.A, B, V, 1, m, wlin);
  equilibrate(s.A, n, s.f1, s.f2, true);
  if (gj_invert(s.A, n, s.piv, s.colk, s.red, s.redi) != 0) { flag_status(S, PZ_E_SINGULAR); return; }
  double* Gom = d.pool + I.o_gom + (long long)mi * n * n;
  store_op(Gom, s.A, n, I.n_max, s.f2, s.f1);
  __syncthreads();
  // intermediate solutions (get_intermediate_om/psi, update_psi_coll_dmat.f90:1136-1218):
  // om2 = G_om e_{N-1}, om3 = G_om e_0 ; psi_k = G_psi (-C om_k) on interior rows
  double* aux = d.pool + I.o_aux;
  const long long MN = (long long)I.M * n;
  double* om2 = aux + 0 * MN + (long long)mi * n;
  double* om3 = aux + 1 * MN + (long long)mi * n;
  double* psi2 = aux + 2 * MN + (long long)mi * n;
  double* psi3 = aux + 3 * MN + (long long)mi * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a2 = Gom[i + (long long)(n - 1) * n];
    const double a3 = Gom[i];
    om2[i] = a2; om3[i] = a3;
    s.va[i] = make_double2(a2, a3);
  }
  __syncthreads();
  mv_lanes(d.pool + I.o_gpsi + (long long)mi * n * n, n, s.va, s.vb);   // K (om2, om3)
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.vb[i] = make_double2(-s.vb[i].x, -s.vb[i].y);
  __syncthreads();
  double t2 = 0.0, t3 = 0.0, b2 = 0.0, b3 = 0.0;
  const double* bct = V.rad(RV_BCTOP);
  const double* bcb = V.rad(RV_BCBOT);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    psi2[i] = s.vb[i].x;
    psi3[i] = s.vb[i].y;
    t2 += bct[i] * s.vb[i].x; t3 += bct[i] * s.vb[i].y;
    b2 += bcb[i] * s.vb[i].x; b3 += bcb[i] * s.vb[i].y;
  }
  t2 = block_sum(t2, s.red); t3 = block_sum(t3, s.red);
  b2 = block_sum(b2, s.red); b3 = block_sum(b3, s.red);
  if (threadIdx.x == 0) {
    // get_influence_matrix (update_psi_coll_dmat.f90:1220-1254)
    double* infl = aux + 4 * MN + 4LL * mi;
    const double det = t2 * b3 - t3 * b2;
    infl[0] = b3 / det; infl[1] = -t3 / det; infl[2] = -b2 / det; infl[3] = t2 / det;
  }
}

__global__ void __launch_bounds__(PZ_THREADS) k_build(PzDev d) { build_item<true>(d, d.mitems[blockIdx.x]); }

// ---------------------------------------------------------------------------
// implicit terms from physical-space fields: get_temp_rhs_imp_coll and
// get_psi_rhs_imp_coll_dmat with l_in_cheb_space=.false. (used by the start
// fields, init_fields.f90:228-255, and by start_from_another_scheme,
// step_time.f90:417-516).  Writes old/impl logical slot 1 at ring bases bo/bi.
// ---------------------------------------------------------------------------
// implicit Ekman pumping and Coriolis terms of the smat vorticity equation,
// get_psi_rhs_imp_coll_smat (update_psi_coll_smat.f90:380-527), m /= 0:
//   -CorFac ekpump (om + ekp_up up + (i m ekp_dusdp + ekp_us) us) [+ CorFac beta us]
__device__ __forceinline__ double2 smat_imp_extra(const PzInst& I, const View& V, int i, double dm, double2 om,
                                                  double2 up, double2 us) {
  const double ce = I.CorFac * V.rad(RV_EKPUMP)[i];
  const double eus = V.rad(RV_EKP_US)[i], edp = V.rad(RV_EKP_DUSDP)[i], eup = V.rad(RV_EKP_UP)[i];
  const double2 q = make_double2(eus * us.x - edp * dm * us.y, eus * us.y + edp * dm * us.x);
  double2 v = make_double2(-ce * (om.x + eup * up.x + q.x), -ce * (om.y + eup * up.y + q.y));
  if (I.flags & PZF_COR_IMP) {
    const double cb = I.CorFac * V.rad(RV_BETA)[i];
    v.x += cb * us.x; v.y += cb * us.y;
  }
  return v;
}

struct MS {   // per-m vectors in shared memory
  double2 *a, *b, *c, *e, *f, *g, *h, *k;
  SymScratch w;
  double* red;
  double* st;   // k_mloop_integ: staging space of the bordered banded sweeps
};
__host__ __device__ inline size_t ms_smem_bytes(int n) {
  const size_t h2 = (size_t)(n + 1) / 2;
  return 8 * (size_t)n * sizeof(double2) + 2 * h2 * sizeof(double2) + 8 * h2 * sizeof(double) + 64 * sizeof(double);
}
// k_mloop_integ: the MS vectors of the largest grid, then the staging space
// of the largest record rows (complex, kl = 8)
__host__ __device__ inline size_t integ_st_offset(int maxN) { return (ms_smem_bytes(maxN) + 15) & ~(size_t)15; }
__host__ __device__ inline size_t integ_mloop_smem_bytes(int maxN) {
  return integ_st_offset(maxN) + (size_t)maxN * (3 * 8 + 2) * sizeof(double2);
}

template <bool CHEM>
__device__ void imp_from_physical(const View& V, const PzInst& I, int mi, int bo, int bi, bool calc, MS& s) {
  const int n = I.N;
  const int m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* ekpump = V.rad(RV_EKPUMP);
  double2* T = V.fld(F_TEMP, mi);
  double2* om = V.fld(F_OM, mi);
  double2* up = V.fld(F_UP, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = T[i];
  __syncthreads();
  op_Dp2(V, n, s.a, s.b, s.c, s.w);
  __syncthreads();
  double2* oT = V.hist(0, 0, bo, mi);
  double2* iT = V.hist(0, 1, bi, mi);
  double2* dT = V.fld(F_DTEMP, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 t = s.a[i], d1 = s.b[i], d2 = s.c[i];
    oT[i] = t;
    dT[i] = d1;
    if (calc) {
      const double f = I.TdiffFac;
      iT[i] = make_double2(f * (d2.x + or1[i] * d1.x - dm2 * or2[i] * t.x),
                           f * (d2.y + or1[i] * d1.y - dm2 * or2[i] * t.y));
    }
  }
  __syncthreads();
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  double2* X = V.fld(F_XI, mi);
  if (chem) {
    // get_xi_rhs_imp_coll (update_xi_coll.f90:168-216)
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = X[i];
    __syncthreads();
    op_Dp2(V, n, s.a, s.b, s.c, s.w);
    __syncthreads();
    double2* oX = V.hist(2, 0, bo, mi);
    double2* iX = V.hist(2, 1, bi, mi);
    double2* dX = V.fld(F_DXI, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 t = s.a[i], d1 = s.b[i], d2 = s.c[i];
      oX[i] = t;
      if (calc) {
        // assemble_xi_coll has no l_log_next refresh of dxi: it changes
        // only with the implicit term (update_xi_coll.f90:188-195, :264-266)
        dX[i] = d1;
        const double f = I.XidiffFac;
        iX[i] = make_double2(f * (d2.x + or1[i] * d1.x - dm2 * or2[i] * t.x),
                             f * (d2.y + or1[i] * d1.y - dm2 * or2[i] * t.y));
      }
    }
    __syncthreads();
  }
  double2* oP = V.hist(1, 0, bo, mi);
  double2* iP = V.hist(1, 1, bi, mi);
  if (m == 0) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = make_double2(up[i].x, 0.0);
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = om[i];
  }
  __syncthreads();
  op_Dp2(V, n, s.a, s.b, s.c, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 x = s.a[i], d1 = s.b[i], d2 = s.c[i];
    if (m == 0) {
      oP[i] = up[i];
      if (calc) {
        const double u = x.x;
        iP[i] = make_double2(I.ViscFac * (d2.x + or1[i] * d1.x - or2[i] * u) - I.CorFac * ekpump[i] * u, 0.0);
      }
    } else {
      oP[i] = x;
      if (calc) {
        double2 v = make_double2(I.ViscFac * (d2.x + or1[i] * d1.x - dm2 * or2[i] * x.x),
                                 I.ViscFac * (d2.y + or1[i] * d1.y - dm2 * or2[i] * x.y));
        if (I.flags & PZF_DIRECT) v = cadd(v, smat_imp_extra(I, V, i, dm, x, up[i], V.fld(F_US, mi)[i]));
        if (I.flags & PZF_BUO_IMP) {
          const double2 b = cim(dm, T[i]);
          const double c = rgrav[i] * or1[i] * I.BuoFac;
          v.x -= c * b.x; v.y -= c * b.y;
          if (chem) {
            const double2 bx = cim(dm, X[i]);
            const double cx = rgrav[i] * or1[i] * I.ChemFac;
            v.x -= cx * bx.x; v.y -= cx * bx.y;
          }
        }
        iP[i] = v;
      }
    }
  }
  __syncthreads();
}

template <bool CHEM>
__device__ void integ_imp(const View& V, const PzInst& I, int mi, int bo, int bi, bool calc, bool from_us, MS& s,
                          bool psi_as_xi);

__device__ MS ms_smem(int n) {
  extern __shared__ double2 shm[];
  const int h2 = (n + 1) / 2;
  MS s;
  s.a = shm; s.b = s.a + n; s.c = s.b + n; s.e = s.c + n; s.f = s.e + n; s.g = s.f + n; s.h = s.g + n; s.k = s.h + n;
  s.w.s = s.k + n;
  s.w.a = s.w.s + h2;
  s.w.t1 = reinterpret_cast<double*>(s.w.a + h2);
  s.w.t2 = s.w.t1 + 4 * h2;
  s.red = s.w.t2 + 4 * h2;
  s.st = nullptr;
  return s;
}

// start fields (init_fields.f90:54-258, no checkpoint)
__global__ void __launch_bounds__(PZ_THREADS) k_start(PzDev d, int only) {
  const PzItem it = d.mitems[blockIdx.x];
  if (only >= 0 && it.inst != only) return;
  const PzInst& I = d.inst[it.inst];
  PzState& S = d.state[it.inst];
  const View V{&I, d.pool};
  const int n = I.N, mi = it.idx, m = mi * I.minc;
  const double dm = (double)m;
  MS s = ms_smem(n);
  // zero the history rings of this m
  for (int f = 0; f < I.nhf; ++f)
    for (int kind = 0; kind < 3; ++kind) {
      const int ns = kind == 0 ? I.nold : (kind == 1 ? I.nimp : I.nexp);
      for (int ph = 0; ph < ns; ++ph) {
        double2* h = V.hist(f, kind, ph, mi);
        for (int i = threadIdx.x; i < n; i += blockDim.x) h[i] = make_double2(0.0, 0.0);
      }
    }
  double2* us = V.fld(F_US, mi);
  double2* up = V.fld(F_UP, mi);
  double2* om = V.fld(F_OM, mi);
  double2* psi = V.fld(F_PSI, mi);
  const double* or1 = V.rad(RV_OR1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) { s.a[i] = up[i]; psi[i] = make_double2(0.0, 0.0); }
  __syncthreads();
  op_D1p(V, n, s.a, s.b, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    // om = d(up)/dr + up/r - (i m / r) us
    const double2 u = up[i], w = s.b[i], vs = cim(dm, us[i]);
    om[i] = make_double2(w.x + or1[i] * u.x - or1[i] * vs.x, w.y + or1[i] * u.y - or1[i] * vs.y);
  }
  __syncthreads();
  if (I.flags & PZF_INTEG) integ_imp<true>(V, I, mi, S.b_old, S.b_impl, true, true, s, false);
  else imp_from_physical<true>(V, I, mi, S.b_old, S.b_impl, true, s);
}

// ---------------------------------------------------------------------------
// k_mloop: finish_explicit_assembly + update_temp_co + update_om_coll_dmat
// for one m of one instance (src/mloop.f90:36-229)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 imex_rhs(const View& V, const PzInst& I, const PzState& S, int f, int mi, int i) {
  double2 acc;
  {
    const double2 v = V.hist(f, 0, S.r_old, mi)[i];
    acc = make_double2(S.wimp[0] * v.x, S.wimp[0] * v.y);
  }
  for (int k = 1; k < I.nold; ++k) {
    const double2 v = V.hist(f, 0, (S.r_old + k) % I.nold, mi)[i];
    acc.x += S.wimp[k] * v.x; acc.y += S.wimp[k] * v.y;
  }
  for (int k = 0; k < I.nimp; ++k) {
    const double2 v = V.hist(f, 1, (S.r_impl + k) % I.nimp, mi)[i];
    acc.x += S.wimp_lin[k + 1] * v.x; acc.y += S.wimp_lin[k + 1] * v.y;
  }
  for (int k = 0; k < I.nexp; ++k) {
    const double2 v = V.hist(f, 2, (S.r_expl + k) % I.nexp, mi)[i];
    acc.x += S.wexp[k] * v.x; acc.y += S.wexp[k] * v.y;
  }
  return acc;
}

// IMEX rhs of DIRK stage `stage` (set_imex_rhs, dirk_schemes.f90:762-795):
// old + sum_{k<=stage} dt (b_exp(stage+1,k) expl_k + b_imp(stage+1,k) impl_k)
__device__ __forceinline__ double2 dirk_rhs(const View& V, const PzInst& I, const PzState& S, int f, int mi, int i,
                                           int stage) {
  const double* bt = V.pool + I.o_bt;
  const double dt = S.dt[0];
  double2 acc = V.hist(f, 0, 0, mi)[i];
  for (int k = 0; k < stage; ++k) {
    const double w = dt * bt[PZ_BT_EXP + stage * PZ_BT_LD + k];
    const double2 v = V.hist(f, 2, k, mi)[i];
    acc.x += w * v.x; acc.y += w * v.y;
  }
  for (int k = 0; k < stage; ++k) {
    const double w = dt * bt[PZ_BT_IMP + stage * PZ_BT_LD + k];
    const double2 v = V.hist(f, 1, k, mi)[i];
    acc.x += w * v.x; acc.y += w * v.y;
  }
  return acc;
}

#include "pz_integ.cuh"

template <bool CHEM>
__device__ __forceinline__ void mloop_item(const PzDev& d, const PzItem it, int stage) {
  const PzInst& I = d.inst[it.inst];
  PzState& Sg = d.state[it.inst];
  if (Sg.status != 0 || stage > I.nstages || (I.flags & PZF_INTEG)) return;
  const PzState S = Sg;
  // stage bookkeeping: the explicit slot of this stage, whether this stage
  // solves (not the last stage of an assembly scheme), and where the solution's
  // implicit term goes (stage+1, or 1 after the last stage, which also sets old)
  const bool dirk = I.dirk != 0;
  const int eslot = dirk ? stage - 1 : S.r_expl;
  const bool do_finish = !dirk || ((I.exp_mask >> (stage - 1)) & 1);
  const bool do_solve = !(dirk && I.assembly && stage == I.nstages);
  const int tgt = (!dirk || stage == I.nstages) ? 1 : stage + 1;
  const int oslot = dirk ? 0 : S.b_old;
  const int islot = dirk ? tgt - 1 : S.b_impl;
  const bool wold = tgt == 1;
  const bool calc = dirk ? ((I.imp_mask >> (tgt - 1)) & 1) != 0 : S.l_calc_lin != 0;
  const View V{&I, d.pool};
  const int n = I.N, mi = it.idx, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  MS s = ms_smem(n);
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
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
  const bool direct = (I.flags & PZF_DIRECT) != 0;
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  // -- finish_exp_temp_coll (update_temp_coll.f90:152-176)
  if (do_finish) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s.a[i] = V.fld(F_DVST, mi)[i];
    s.e[i] = V.fld(F_DVSOM, mi)[i];
  }
  __syncthreads();
  op_D1p2(V, n, s.a, s.e, s.b, s.f, s.w, s.g, s.h);
  __syncthreads();
  {
    double2* eT = V.hist(0, 2, eslot, mi);
    double2* eP = V.hist(1, 2, eslot, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 e = eT[i];
      const double2 u = us[i];
      const double c = dtcond[i] - I.tadvz * beta[i] * tcond[i];
      e.x = e.x - or1[i] * s.b[i].x - u.x * c;
      e.y = e.y - or1[i] * s.b[i].y - u.y * c;
      eT[i] = e;
      // finish_exp_psi_coll_dmat (update_psi_coll_dmat.f90:468-552), m /= 0
      if (m != 0) {
        double2 p = eP[i];
        p.x -= or1[i] * s.f[i].x;
        p.y -= or1[i] * s.f[i].y;
        // explicit Coriolis: always with dmat, unless implicit with smat
        // (update_psi_coll_smat.f90:323-378)
        if (direct ? !(I.flags & PZF_COR_IMP) : !(I.flags & PZF_NON_ROT)) {
          p.x += I.CorFac * beta[i] * u.x;
          p.y += I.CorFac * beta[i] * u.y;
        }
        if (!buo_imp) {
          const double2 b = cim(dm, T[i]);
          const double cb = I.BuoFac * rgrav[i] * or1[i];
          p.x -= cb * b.x; p.y -= cb * b.y;
          if (chem) {
            const double2 bx = cim(dm, X[i]);
            const double cx = I.ChemFac * rgrav[i] * or1[i];
            p.x -= cx * bx.x; p.y -= cx * bx.y;
          }
        }
        if (!direct && (I.flags & PZF_EK_PUMP)) {
          const double2 o = om[i], w = up[i];
          const double2 q = make_double2(ekp_us[i] * u.x - ekp_dusdp[i] * dm * u.y,
                                         ekp_us[i] * u.y + ekp_dusdp[i] * dm * u.x);
          const double ce = I.CorFac * ekpump[i];
          p.x -= ce * (o.x + ekp_up[i] * w.x + q.x);
          p.y -= ce * (o.y + ekp_up[i] * w.y + q.y);
        }
        eP[i] = p;
      }
    }
  }
  __syncthreads();
  if (chem) {
    // finish_exp_xi_coll (update_xi_coll.f90:142-166)
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.g[i] = V.fld(F_DVSXI, mi)[i];
    __syncthreads();
    op_D1p(V, n, s.g, s.h, s.w);
    __syncthreads();
    const double* dxicond = V.rad(RV_DXICOND);
    double2* eX = V.hist(2, 2, eslot, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 e = eX[i];
      const double2 u = us[i];
      e.x = e.x - or1[i] * s.h[i].x - u.x * dxicond[i];
      e.y = e.y - or1[i] * s.h[i].y - u.y * dxicond[i];
      eX[i] = e;
    }
    __syncthreads();
  }
  }
  if (!do_solve) return;   // assembly follows (k_assemble)
  // -- start_from_another_scheme (step_time.f90:417-516)
  if (S.bridge) imp_from_physical<CHEM>(V, I, mi, S.r_old, S.r_impl, true, s);

  // Implicit terms from the solve.  At every interior row the solution x of
  // (I - w L) x = rhs satisfies L x = (x - rhs) / w exactly, w being the weight
  // the operators were built with; the boundary rows of an implicit term are
  // never read (the next right-hand side replaces them by boundary values).
  // So the multistep family takes L x from the residual instead of second
  // derivatives (the rounding this adds to the next right-hand side is
  // w * O(eps |x| / w)).  Needs the untruncated solution (n_cheb_max = n_r_max).
  // The coupled (omega, psi) operator of the direct solve is too ill-conditioned
  // for its residual at n_r_max ~ 100 (it adds ~1e-9 relative there), so its
  // vorticity keeps the second derivatives.
  const bool resid = calc && !dirk && !S.bridge && I.n_max == n && S.w_lhs > 0.0;
  const bool resid_om = resid && !direct;
  const double iw = resid ? 1.0 / S.w_lhs : 0.0;

  // -- update_temp_co (update_temp_coll.f90:66-150)
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = dirk ? dirk_rhs(V, I, S, 0, mi, i, stage) : imex_rhs(V, I, S, 0, mi, i);
    s.a[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : v;   // topt = bott = 0
  }
  __syncthreads();
  const double* GT = ((I.flags & PZF_T_IS_OM) && m != 0) ? d.pool + I.o_gom + (long long)mi * n * n
                                                         : d.pool + I.o_gt + (long long)mi * n * n;
  mv_lanes(GT, n, s.a, s.b);                                              // Chebyshev T
  __syncthreads();
  if (resid) {
    op_CD1c(V, n, s.b, s.f, s.c, s.w);                                    // T (physical), dT/dr
  } else {
    op_Dc2(V, n, s.b, s.c, s.e, s.w);                                     // dT/dr, d2T/dr2
    __syncthreads();
    op_C(V, n, s.b, s.f, s.w);                                            // T (physical)
  }
  __syncthreads();
  bool bad = false;
  {
    double2* oT = V.hist(0, 0, oslot, mi);
    double2* iT = V.hist(0, 1, islot, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 t = s.f[i], d1 = s.c[i], d2 = s.e[i];
      T[i] = t;
      dT[i] = d1;
      if (wold) oT[i] = t;
      bad |= !isfinite(t.x) || !isfinite(t.y);
      if (resid) {
        iT[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : cscale(iw, csub(t, s.a[i]));
      } else if (calc) {
        const double f = I.TdiffFac;
        iT[i] = make_double2(f * (d2.x + or1[i] * d1.x - dm2 * or2[i] * t.x),
                             f * (d2.y + or1[i] * d1.y - dm2 * or2[i] * t.y));
      }
    }
  }
  __syncthreads();
  // s.f keeps the new physical temperature; with composition it becomes the
  // buoyancy source BuoFac T + ChemFac xi, and bf (the factor of s.f in the
  // buoyancy) is 1
  double bf = I.BuoFac;
  if (chem) {
    // -- update_xi_co (update_xi_coll.f90:66-140): the temperature's solve with XidiffFac
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 v = dirk ? dirk_rhs(V, I, S, 2, mi, i, stage) : imex_rhs(V, I, S, 2, mi, i);
      s.a[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : v;   // topxi = botxi = 0
    }
    __syncthreads();
    mv_lanes(d.pool + I.o_gx + (long long)mi * n * n, n, s.a, s.b);    // Chebyshev xi
    __syncthreads();
    if (resid) {
      op_CD1c(V, n, s.b, s.g, s.c, s.w);                                // xi (physical), dxi/dr
    } else {
      op_Dc2(V, n, s.b, s.c, s.e, s.w);
      __syncthreads();
      op_C(V, n, s.b, s.g, s.w);                                        // xi (physical)
    }
    __syncthreads();
    double2* oX = V.hist(2, 0, oslot, mi);
    double2* iX = V.hist(2, 1, islot, mi);
    double2* dX = V.fld(F_DXI, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 t = s.g[i], d1 = s.c[i], d2 = s.e[i];
      X[i] = t;
      dX[i] = d1;
      if (wold) oX[i] = t;
      bad |= !isfinite(t.x) || !isfinite(t.y);
      if (resid) {
        iX[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : cscale(iw, csub(t, s.a[i]));
      } else if (calc) {
        const double f = I.XidiffFac;
        iX[i] = make_double2(f * (d2.x + or1[i] * d1.x - dm2 * or2[i] * t.x),
                             f * (d2.y + or1[i] * d1.y - dm2 * or2[i] * t.y));
      }
      s.f[i] = cadd(cscale(I.BuoFac, s.f[i]), cscale(I.ChemFac, t));
    }
    bf = 1.0;
    __syncthreads();
  }
  // -- update_om_coll_dmat (update_psi_coll_dmat.f90:126-466)
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 v = dirk ? dirk_rhs(V, I, S, 1, mi, i, stage) : imex_rhs(V, I, S, 1, mi, i);
    if (m != 0 && buo_imp) {
      const double2 b = cim(dm, s.f[i]);
      const double c = S.wimp_lin[0] * bf * rgrav[i] * or1[i];
      v.x -= c * b.x; v.y -= c * b.y;
    }
    if (m == 0) v.y = 0.0;
    s.a[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : v;
  }
  __syncthreads();
  double2* oP = V.hist(1, 0, oslot, mi);
  double2* iP = V.hist(1, 1, islot, mi);
  if (m == 0) {
    mv_lanes(d.pool + I.o_guphi, n, s.a, s.b);           // uphi, Chebyshev
    __syncthreads();
    if (resid) {
      op_CD1c(V, n, s.b, s.g, s.c, s.w);
    } else {
      op_Dc2(V, n, s.b, s.c, s.e, s.w);
      __syncthreads();
      op_C(V, n, s.b, s.g, s.w);
    }
    __syncthreads();
    const double* ekp = ekpump;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double u = s.g[i].x, du = s.c[i].x, d2u = resid ? 0.0 : s.e[i].x;
      us[i] = make_double2(0.0, 0.0);
      up[i] = make_double2(u, 0.0);
      om[i] = make_double2(du + or1[i] * u, 0.0);
      psi[i] = make_double2(0.0, 0.0);
      if (wold) oP[i] = make_double2(u, 0.0);
      bad |= !isfinite(u);
      if (resid)
        iP[i] = make_double2((i == 0 || i == n - 1) ? 0.0 : iw * (u - s.a[i].x), 0.0);
      else if (calc)
        iP[i] = make_double2(I.ViscFac * (d2u + or1[i] * du - or2[i] * u) - I.CorFac * ekp[i] * u, 0.0);
    }
  } else {
    if (direct) {
      // update_om_coll_smat (update_psi_coll_smat.f90:88-321): one coupled solve
      cmv_lanes(reinterpret_cast<const double2*>(d.pool + I.o_gsm) + 2LL * mi * n * n, n, s.a, s.b, s.e);
      __syncthreads();
    } else {
    mv_lanes(d.pool + I.o_gom + (long long)mi * n * n, n, s.a, s.b);  // omega, Chebyshev
    __syncthreads();
    mv_lanes(d.pool + I.o_gpsi + (long long)mi * n * n, n, s.b, s.e);  // -psi, Chebyshev (psi = -K om)
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.e[i] = make_double2(-s.e[i].x, -s.e[i].y);
    __syncthreads();
    // influence-matrix correction (update_psi_coll_dmat.f90:1256-1300)
    const double* bct = V.rad(RV_BCTOP);
    const double* bcb = V.rad(RV_BCBOT);
    double tr = 0.0, ti = 0.0, br = 0.0, bi = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      tr += bct[i] * s.e[i].x; ti += bct[i] * s.e[i].y;
      br += bcb[i] * s.e[i].x; bi += bcb[i] * s.e[i].y;
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
      p.x += c1r * psi2[i] + c2r * psi3[i];
      p.y += c1i * psi2[i] + c2i * psi3[i];
      o.x += c1r * om2[i] + c2r * om3[i];
      o.y += c1i * om2[i] + c2i * om3[i];
      s.e[i] = p;
      s.b[i] = o;
    }
    __syncthreads();
    }
    op_CD1c(V, n, s.e, s.h, s.g, s.w);                               // psi, dpsi/dr
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 p = s.h[i], dp = s.g[i];
      psi[i] = p;
      us[i] = cscale(or1[i], cim(dm, p));
      up[i] = make_double2(-dp.x - beta[i] * p.x, -dp.y - beta[i] * p.y);
    }
    if (!resid_om) op_Dc2(V, n, s.b, s.c, s.a, s.w);                 // dom, d2om
    __syncthreads();
    op_C(V, n, s.b, s.k, s.w);                                       // om
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 o = s.k[i];
      om[i] = o;
      if (wold) oP[i] = o;
      bad |= !isfinite(o.x) || !isfinite(o.y);
      if (calc) {
        double2 v;
        if (resid_om) {
          // s.a holds the right-hand side with the implicit buoyancy folded in,
          // so (om - s.a)/w is every implicit term of the vorticity row but
          // the buoyancy, which is added below
          v = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : cscale(iw, csub(o, s.a[i]));
        } else {
          const double2 d1 = s.c[i], d2 = s.a[i];
          v = make_double2(I.ViscFac * (d2.x + or1[i] * d1.x - dm2 * or2[i] * o.x),
                           I.ViscFac * (d2.y + or1[i] * d1.y - dm2 * or2[i] * o.y));
          if (direct) v = cadd(v, smat_imp_extra(I, V, i, dm, o, up[i], us[i]));
        }
        if (buo_imp) {
          const double2 b = cim(dm, s.f[i]);
          const double c = rgrav[i] * or1[i] * bf;
          v.x -= c * b.x; v.y -= c * b.y;
        }
        iP[i] = v;
      }
    }
  }
  if (__syncthreads_or(bad)) flag_status(Sg, PZ_E_NONFINITE);
}

__global__ void __launch_bounds__(256, 4) k_mloop(PzDev d, int stage) { mloop_item<true>(d, d.mitems[blockIdx.x], stage); }

// ---------------------------------------------------------------------------
// k_order + k_build_mloop: the operator rebuild fused with the first stage.
// Each (instance, m) only needs its own operators, so a block rebuilds them
// (if its instance's dt changed) and then runs the stage.  k_order lays the
// work items out so that the rebuilding ones -- long, latency-bound
// Gauss-Jordan chains -- are spread one in four over the first waves instead
// of running as a wave of their own: the other blocks keep the FP64 pipe busy
// meanwhile.  Item k of the rebuild list goes to position k + min(3k, n_rest),
// item j of the rest to j + min(j/3 + 1, n_rebuild); both lists keep the
// largest-first order of the work list.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_order(PzDev d) {
  // one scan over the instances (in work-list order, where each instance's m
  // items are contiguous): rebuilding items and all items before each one
  __shared__ int sr[1024], sa[1024];
  const int n = d.n_iorder, T = blockDim.x, t = threadIdx.x;
  const int per = (n + T - 1) / T;
  const int q0 = min(n, t * per), q1 = min(n, q0 + per);
  auto rebuild = [&](int inst) {
    const PzState& S = d.state[inst];
    return S.status == 0 && S.lMat != 0;
  };
  int reb = 0, all = 0;
  for (int q = q0; q < q1; ++q) {
    const int inst = d.iorder[q], M = d.inst[inst].M;
    all += M;
    if (rebuild(inst)) reb += M;
  }
  sr[t] = reb;
  sa[t] = all;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {          // inclusive scans
    const int vr = t >= off ? sr[t - off] : 0, va = t >= off ? sa[t - off] : 0;
    __syncthreads();
    sr[t] += vr;
    sa[t] += va;
    __syncthreads();
  }
  const int n_reb = sr[T - 1], n_rest = d.n_mitems - n_reb;
  int k = sr[t] - reb;                              // rebuilding items before this chunk
  int j = (sa[t] - all) - k;                        // other items before this chunk
  for (int q = q0; q < q1; ++q) {
    const int inst = d.iorder[q], M = d.inst[inst].M;
    const bool rb = rebuild(inst);
    for (int m = 0; m < M; ++m) {
      int pos;
      if (rb) { pos = k + min(3 * k, n_rest); ++k; }
      else { pos = j + min(j / 3 + 1, n_reb); ++j; }
      d.order[pos] = PzItem{inst, m};
    }
  }
}

template <bool CHEM>
__global__ void __launch_bounds__(256, 4) k_build_mloop(PzDev d) {
  const PzItem it = d.order[blockIdx.x];
  if (d.inst[it.inst].flags & PZF_INTEG) return;
  build_item<CHEM>(d, it);
  __syncthreads();
  mloop_item<CHEM>(d, it, 1);
}

// ---------------------------------------------------------------------------
// k_mloop_integ: the stage body of the integration method for one m of one
// instance (mloop.f90:84-100, :209-226); its own kernel so that the
// collocation kernel keeps its register allocation.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 3) k_mloop_integ(PzDev d, int stage) {
  const PzItem it = d.mitems[blockIdx.x];
  const PzInst& I = d.inst[it.inst];
  PzState& Sg = d.state[it.inst];
  if (Sg.status != 0 || stage > I.nstages || !(I.flags & PZF_INTEG)) return;
  const PzState S = Sg;
  IntegStage c;
  c.stage = stage;
  c.dirk = I.dirk != 0;
  c.eslot = c.dirk ? stage - 1 : S.r_expl;
  c.do_finish = !c.dirk || ((I.exp_mask >> (stage - 1)) & 1);
  c.do_solve = !(c.dirk && I.assembly && stage == I.nstages);
  const int tgt = (!c.dirk || stage == I.nstages) ? 1 : stage + 1;
  c.oslot = c.dirk ? 0 : S.b_old;
  c.islot = c.dirk ? tgt - 1 : S.b_impl;
  c.wold = tgt == 1;
  c.calc = c.dirk ? ((I.imp_mask >> (tgt - 1)) & 1) != 0 : S.l_calc_lin != 0;
  const View V{&I, d.pool};
  MS s = ms_smem(I.N);
  {
    extern __shared__ double2 shm[];
    s.st = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(shm) + integ_st_offset(d.maxN));
  }
  const bool bad = integ_stage<true>(d, V, I, S, it.idx, c, s);
  if (__syncthreads_or(bad)) flag_status(Sg, PZ_E_NONFINITE);
}

// ---------------------------------------------------------------------------
// k_assemble: the assembly stage of a DIRK scheme (assemble_stage, mloop.f90;
// assemble_temp_coll, update_temp_coll.f90:238-307; assemble_psi_coll_{smat,dmat},
// update_psi_coll_smat.f90:529-672) for one m of one instance:
//   X = old + sum_k dt (b_ass_exp(k) expl_k + b_ass_imp(k) impl_k)   (assemble_imex)
// temperature: interior from X, fixed walls; u_phi(m=0): interior from Re X,
// rigid walls; m /= 0: psi from the assembled vorticity through get_assMat,
// then us, up and om from psi; finally the first-stage old/implicit terms
// from the physical fields (get_*_rhs_imp_coll with l_in_cheb_space=.false.).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 assemble_imex(const View& V, const PzInst& I, const PzState& S, int f, int mi,
                                                int i) {
  const double* bt = V.pool + I.o_bt;
  const double dt = S.dt[0];
  double2 acc = V.hist(f, 0, 0, mi)[i];
  for (int k = 0; k < I.nstages; ++k) {
    const double w = dt * bt[PZ_BT_AEXP + k];
    const double2 v = V.hist(f, 2, k, mi)[i];
    acc.x += w * v.x; acc.y += w * v.y;
  }
  for (int k = 0; k < I.nstages; ++k) {
    const double w = dt * bt[PZ_BT_AIMP + k];
    const double2 v = V.hist(f, 1, k, mi)[i];
    acc.x += w * v.x; acc.y += w * v.y;
  }
  return acc;
}

__global__ void __launch_bounds__(256) k_assemble(PzDev d) {
  const PzItem it = d.mitems[blockIdx.x];
  const PzInst& I = d.inst[it.inst];
  PzState& Sg = d.state[it.inst];
  if (Sg.status != 0 || !I.dirk || !I.assembly) return;
  const PzState S = Sg;
  const View V{&I, d.pool};
  const int n = I.N, mi = it.idx, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  MS s = ms_smem(n);
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
  const double* dbeta = V.rad(RV_DBETA);
  double2* T = V.fld(F_TEMP, mi);
  double2* us = V.fld(F_US, mi);
  double2* up = V.fld(F_UP, mi);
  double2* om = V.fld(F_OM, mi);
  double2* psi = V.fld(F_PSI, mi);
  bool bad = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 t = assemble_imex(V, I, S, 0, mi, i);
    if (m == 0) t.y = 0.0;
    if (i == 0 || i == n - 1) t = make_double2(0.0, 0.0);   // robin_bc, Dirichlet: topt = bott = 0
    T[i] = t;
    bad |= !isfinite(t.x) || !isfinite(t.y);
    if (I.flags & PZF_CHEM) {
      // assemble_xi_coll (update_xi_coll.f90:218-269)
      double2 x = assemble_imex(V, I, S, 2, mi, i);
      if (m == 0) x.y = 0.0;
      if (i == 0 || i == n - 1) x = make_double2(0.0, 0.0);
      V.fld(F_XI, mi)[i] = x;
      bad |= !isfinite(x.x) || !isfinite(x.y);
    }
    const double2 w = assemble_imex(V, I, S, 1, mi, i);
    if (m == 0) s.a[i] = (i == 0 || i == n - 1) ? make_double2(0.0, 0.0) : make_double2(w.x, 0.0);
    else s.a[i] = (i < 2 || i > n - 3) ? make_double2(0.0, 0.0) : w;
  }
  __syncthreads();
  if (m == 0) {
    op_D1p(V, n, s.a, s.b, s.w);                                      // d u_phi / dr
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double u = s.a[i].x;
      us[i] = make_double2(0.0, 0.0);
      up[i] = make_double2(u, 0.0);
      om[i] = make_double2(s.b[i].x + or1[i] * u, 0.0);
      psi[i] = make_double2(0.0, 0.0);
      bad |= !isfinite(u);
    }
  } else {
    mv_lanes(d.pool + I.o_gass + (long long)mi * n * n, n, s.a, s.b);   // psi, Chebyshev
    __syncthreads();
    op_Dc2(V, n, s.b, s.c, s.e, s.w);                                   // dpsi, d2psi
    __syncthreads();
    op_C(V, n, s.b, s.f, s.w);                                          // psi
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 p = s.f[i], d1 = s.c[i], d2 = s.e[i];
      const double c1 = or1[i] + beta[i], c0 = or1[i] * beta[i] + dbeta[i] - dm2 * or2[i];
      psi[i] = p;
      us[i] = cscale(or1[i], cim(dm, p));
      up[i] = make_double2(-d1.x - beta[i] * p.x, -d1.y - beta[i] * p.y);
      om[i] = make_double2(-(d2.x + c1 * d1.x + c0 * p.x), -(d2.y + c1 * d1.y + c0 * p.y));
      bad |= !isfinite(p.x) || !isfinite(p.y);
    }
  }
  __syncthreads();
  imp_from_physical<true>(V, I, mi, 0, 0, (I.imp_mask & 1) != 0, s);
  if (__syncthreads_or(bad)) flag_status(Sg, PZ_E_NONFINITE);
}

// ---------------------------------------------------------------------------
// k_obs: time series of one instance (src/outputs.f90:418-830)
// ---------------------------------------------------------------------------
// round_off (src/useful.f90:222-233) with tiny_number = 10 epsilon(1.0_cp)
// (src/constants.f90:21)
__device__ __forceinline__ double round_off(double x) { return fabs(x) < 10.0 * 2.220446049250313e-16 ? 0.0 : x; }

// ---------------------------------------------------------------------------
// k_spectra: snapshot spectra of one instance (calculate_spectra,
// src/spectra.f90:104-196): per m, rInt_R of pi cc2real(f) r height for
// f = us, up, om, T, and the composition column, one block per m.  The
// reference fills that column with the temperature's integral (xi2_m =
// rInt_R(temp2R), spectra.f90:183) when composition is on, and leaves it zero
// otherwise; the column here is the same, so spec files match.  With out2d,
// the integrands of us2, up2 and the enstrophy at every (r, m) as well (the
// 2-D spectra us2R, up2R, enstR of calculate_spectra), at
// out2d[(k N + r) M + m], k = 0, 1, 2.
// ---------------------------------------------------------------------------
__global__ void k_spectra(PzDev d, int inst, double* out, double* out2d) {
  const PzInst& I = d.inst[inst];
  const View V{&I, d.pool};
  __shared__ double red[32];
  const int n = I.N, mi = blockIdx.x;
  const double* rr = V.rad(RV_R);
  const double* h = V.rad(RV_HEIGHT);
  const double* wint = V.rad(RV_WINT);
  const int fl[4] = {F_US, F_UP, F_OM, F_TEMP};
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < 4; ++k) {
    const double2* f = V.fld(fl[k], mi);
    double acc = 0.0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
      const double2 z = f[r];
      const double c2 = (mi == 0) ? z.x * z.x : 2.0 * (z.x * z.x + z.y * z.y);   // cc2real
      const double v = pi * c2 * rr[r] * h[r];
      acc += wint[r] * v;
      if (out2d && k < 3) out2d[((long long)k * n + r) * I.M + mi] = v;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) {
      out[5 * mi + k] = acc;
      if (k == 3) out[5 * mi + 4] = (I.flags & PZF_CHEM) ? acc : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// k_balance: the vorticity and u_phi force balances of one instance over the
// step just taken (vort_balance.f90 and vp_balance.f90 with their hooks in
// update_psi_coll_dmat.f90: initialize/finalize_domdt :154-156, :449-451,
// buo :214-230, adv/cor :500-505, pump :540-546, visc :643-676; the u_phi
// terms :183-187, :444-446, :642-647), from the fields at the start of the
// step (snap: the instance's field block copied before it) and after it.
// One block per m.  vort: 6 terms (buo, cor, adv, dwdt, visc, pump) at
// vort[((t N + r) M + m)] complex; vp (m = 0 block): rey_stress, dvpdt, visc,
// pump at vp[t N + r].  As in the reference, dwdt of m /= 0 takes the new
// vorticity in Chebyshev space (finalize_domdt runs before the transform back)
// minus the old one in physical space, and visc has no ViscFac factor.
// ---------------------------------------------------------------------------
__global__ void k_balance(PzDev d, int inst, const double2* __restrict__ snap, double2* vort, double* vp) {
  const PzInst& I = d.inst[inst];
  const PzState& S = d.state[inst];
  const View V{&I, d.pool};
  const int n = I.N, M = I.M, mi = blockIdx.x, m = mi * I.minc;
  const double dm = (double)m, dt = S.dt[0];
  MS s = ms_smem(n);
  auto sfld = [&](int f) { return snap + ((long long)f * M + mi) * n; };
  const double2* us0 = sfld(F_US);
  const double2* up0 = sfld(F_UP);
  const double2* om0 = sfld(F_OM);
  const double2* T0 = sfld(F_TEMP);
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* ekpump = V.rad(RV_EKPUMP);
  const bool chem = (I.flags & PZF_CHEM) != 0;
  auto out = [&](int t, int r) -> double2& { return vort[((long long)t * n + r) * M + mi]; };
  // new vorticity and its derivatives (physical), its Chebyshev coefficients
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.a[i] = V.fld(F_OM, mi)[i];
  __syncthreads();
  op_Dp2(V, n, s.a, s.b, s.c, s.w);
  __syncthreads();
  op_C(V, n, s.a, s.e, s.w);
  __syncthreads();
  const double2* ex = V.hist(1, 2, S.r_expl, mi);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double2 z = make_double2(0.0, 0.0);
    if (m == 0) {
      for (int t = 0; t < 6; ++t) out(t, i) = z;
      out(3, i) = cscale(1.0 / dt, csub(s.a[i], om0[i]));
      continue;
    }
    double2 buo = cscale(-I.BuoFac * rgrav[i] * or1[i], cim(dm, V.fld(F_TEMP, mi)[i]));
    if (chem) buo = csub(buo, cscale(I.ChemFac * rgrav[i] * or1[i], cim(dm, V.fld(F_XI, mi)[i])));
    const double2 cor = (I.flags & PZF_NON_ROT) ? z : cscale(I.CorFac * beta[i], us0[i]);
    double2 pump = z;
    if (I.flags & PZF_EK_PUMP) {
      const double2 u = us0[i];
      const double2 q = make_double2(V.rad(RV_EKP_US)[i] * u.x - V.rad(RV_EKP_DUSDP)[i] * dm * u.y,
                                     V.rad(RV_EKP_US)[i] * u.y + V.rad(RV_EKP_DUSDP)[i] * dm * u.x);
      const double2 w = cadd(cadd(om0[i], cscale(V.rad(RV_EKP_UP)[i], up0[i])), q);
      pump = cscale(-I.CorFac * ekpump[i], w);
    }
    // the explicit term of the step is adv + cor - buoyancy (explicit) + pump
    double2 adv = csub(csub(ex[i], cor), pump);
    if (!(I.flags & PZF_BUO_IMP)) {
      double2 b = cscale(-I.BuoFac * rgrav[i] * or1[i], cim(dm, T0[i]));
      if (chem) b = csub(b, cscale(I.ChemFac * rgrav[i] * or1[i], cim(dm, sfld(F_XI)[i])));
      adv = csub(adv, b);
    }
    const double2 lap = make_double2(s.c[i].x + or1[i] * s.b[i].x - dm * dm * or2[i] * s.a[i].x,
                                     s.c[i].y + or1[i] * s.b[i].y - dm * dm * or2[i] * s.a[i].y);
    out(0, i) = buo;
    out(1, i) = cor;
    out(2, i) = adv;
    out(3, i) = cscale(1.0 / dt, csub(s.e[i], om0[i]));
    out(4, i) = lap;
    out(5, i) = pump;
  }
  if (m != 0) return;
  __syncthreads();
  // u_phi: derivatives of the new u_phi(m = 0)
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.f[i] = make_double2(V.fld(F_UP, 0)[i].x, 0.0);
  __syncthreads();
  op_Dp2(V, n, s.f, s.g, s.h, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = s.f[i].x;
    vp[i] = ex[i].x;
    vp[n + i] = (u - up0[i].x) / dt;
    vp[2 * n + i] = I.ViscFac * (s.h[i].x + or1[i] * s.g[i].x - or2[i] * u);
    vp[3 * n + i] = (I.flags & PZF_EK_PUMP) ? -I.CorFac * ekpump[i] * u : 0.0;
  }
}

// One block per PZ_OBS_RC radii of one instance (PzDev::oitems).  Thread
// (r, c) sums the m = c, c + 16, ... terms of its radius; the block applies
// the radial weights and writes its partial sums, and the last block of the
// instance to finish (a counter per instance) adds the partials in radius
// order and writes the row, so the result does not depend on block timing.
__global__ void __launch_bounds__(256) k_obs(PzDev d, int only) {
  const PzItem it = d.oitems[blockIdx.x];
  const int inst = it.inst;
  if (only >= 0 && inst != only) return;
  const PzInst& I = d.inst[inst];
  PzState& S = d.state[inst];
  const View V{&I, d.pool};
  constexpr int RC = PZ_OBS_RC, NC = 256 / PZ_OBS_RC;
  __shared__ double q[6][NC][RC];
  __shared__ int last;
  const int n = I.N, M = I.M, r0 = it.idx;
  const double* rr = V.rad(RV_R);
  const double* or2 = V.rad(RV_OR2);
  const double* h = V.rad(RV_HEIGHT);
  const double* beta = V.rad(RV_BETA);
  const double* dtcond = V.rad(RV_DTCOND);
  const double* wint = V.rad(RV_WINT);
  const double* wsimp = V.rad(RV_WSIMP);
  const double2* us = V.fld(F_US, 0);
  const double2* up = V.fld(F_UP, 0);
  const double2* T = V.fld(F_TEMP, 0);
  const double2* dT = V.fld(F_DTEMP, 0);
  const double2* X = V.fld(F_XI, 0);
  const double2* dX = V.fld(F_DXI, 0);
  const bool rot = !(I.flags & PZF_NON_ROT);
  const bool chem = (I.flags & PZF_CHEM) != 0;
  {
    const int rl = threadIdx.x % RC, c = threadIdx.x / RC, r = r0 + rl;
    double us2 = 0, up2 = 0, nu = 0, fl = 0, ax = 0, sh = 0;
    if (r < n) {
      const double o2 = or2[r];
      int mi = c;
      if (mi == 0) {
        const double2 a = us[r], b = up[r], tt = T[r], dt = dT[r];
        if (chem) {
          // sh_vol_r (outputs.f90:488-490)
          const double2 dx = dX[r];
          sh += dx.x * dx.x;
        }
        us2 += a.x * a.x;
        up2 += b.x * b.x;
        ax = b.x * b.x;
        nu += dt.x * dt.x;
        fl += a.x * tt.x - I.TdiffFac * dt.x - I.TdiffFac * dtcond[r];
        mi += NC;
      }
      // m > 0: the loads of several m in flight at once
#pragma unroll 4
      for (; mi < M; mi += NC) {
        const long long o = (long long)mi * n + r;
        const double2 a = us[o], b = up[o], tt = T[o], dt = dT[o];
        const double mm = (double)(mi * I.minc);
        if (chem) {
          const double2 x = X[o], dx = dX[o];
          sh += 2.0 * (dx.x * dx.x + dx.y * dx.y) + mm * mm * o2 * 2.0 * (x.x * x.x + x.y * x.y);
        }
        us2 += 2.0 * (a.x * a.x + a.y * a.y);
        up2 += 2.0 * (b.x * b.x + b.y * b.y);
        nu += 2.0 * (dt.x * dt.x + dt.y * dt.y) + mm * mm * o2 * 2.0 * (tt.x * tt.x + tt.y * tt.y);
        fl += 2.0 * (a.x * tt.x + a.y * tt.y);
      }
    }
    q[0][c][rl] = us2; q[1][c][rl] = up2; q[2][c][rl] = nu; q[3][c][rl] = fl; q[4][c][rl] = ax; q[5][c][rl] = sh;
  }
  __syncthreads();
  // per radius: the sum over m (c in order), then the radial weights
  double v[PZ_OBS_NP] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (threadIdx.x < 32) {
    const int rl = threadIdx.x, r = r0 + rl;
    if (rl < RC && r < n) {
      double us2 = 0, up2 = 0, nu = 0, fl = 0, ax = 0, sh = 0;
      for (int c = 0; c < NC; ++c) {
        us2 += q[0][c][rl]; up2 += q[1][c][rl]; nu += q[2][c][rl];
        fl += q[3][c][rl]; ax += q[4][c][rl]; sh += q[5][c][rl];
      }
      nu = nu * rr[r] * h[r];
      v[0] = wint[r] * us2 * rr[r];
      v[1] = wint[r] * up2 * rr[r];
      v[2] = wint[r] * ax * rr[r];
      if (rot) {
        v[3] = wint[r] * us2 * rr[r] * h[r];
        v[4] = wint[r] * up2 * rr[r] * h[r];
        v[5] = wint[r] * us2 * beta[r] * beta[r] * rr[r] * h[r] * h[r] * h[r] / 12.0;
        v[6] = wint[r] * ax * rr[r] * h[r];
        const double x = rr[r] / I.r_cmb;
        v[8] = wsimp[r] * fl * x * x;
      } else {
        v[8] = wint[r] * fl * rr[r];
      }
      v[7] = wint[r] * nu;
      v[9] = wint[r] * (sh * rr[r] * h[r]);
    }
    for (int k = 0; k < PZ_OBS_NP; ++k) v[k] = warp_sum(v[k]);
    if (threadIdx.x == 0) {
      double* part = d.obs_part + (long long)blockIdx.x * PZ_OBS_NP;
      for (int k = 0; k < PZ_OBS_NP; ++k) part[k] = v[k];
      __threadfence();
      const int nchunk = (n + RC - 1) / RC;
      last = atomicAdd(d.obs_cnt + inst, 1) == nchunk - 1;
    }
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double s_us = 0, s_up = 0, s_ax = 0, s_us3 = 0, s_up3 = 0, s_uz3 = 0, s_ax3 = 0, s_nu = 0, s_fl = 0, s_sh = 0;
  {
    const int nchunk = (n + RC - 1) / RC;
    const double* part = d.obs_part + (long long)(blockIdx.x - r0 / RC) * PZ_OBS_NP;
    for (int k = 0; k < nchunk; ++k) {
      const double* p = part + (long long)k * PZ_OBS_NP;
      s_us += __ldcg(p + 0); s_up += __ldcg(p + 1); s_ax += __ldcg(p + 2);
      s_us3 += __ldcg(p + 3); s_up3 += __ldcg(p + 4); s_uz3 += __ldcg(p + 5); s_ax3 += __ldcg(p + 6);
      s_nu += __ldcg(p + 7); s_fl += __ldcg(p + 8); s_sh += __ldcg(p + 9);
    }
    d.obs_cnt[inst] = 0;
  }
  const double pi = 3.14159265358979323846;
  double* row = d.pool + I.o_series + (long long)(S.series_count % PZ_SERIES_CAP) * PZ_SERIES_COLS;
  row[0] = S.time;
  row[1] = round_off(pi * s_us);
  row[2] = round_off(pi * s_up);
  row[3] = round_off(pi * s_ax);
  row[4] = rot ? round_off(pi * s_us3) : 0.0;
  row[5] = rot ? round_off(pi * s_up3) : 0.0;
  row[6] = rot ? round_off(pi * s_uz3) : 0.0;
  row[7] = rot ? round_off(pi * s_ax3) : 0.0;
  const double* tcond = V.rad(RV_TCOND);
  row[8] = round_off(1.0 + dT[0].x / dtcond[0]);
  row[9] = round_off(1.0 + dT[n - 1].x / dtcond[n - 1]);
  row[10] = round_off(1.0 + s_nu / I.nu_vol_den);
  row[11] = round_off(s_fl / I.nu_int_fac);
  row[12] = round_off(T[0].x + tcond[0]);
  row[13] = round_off(T[n - 1].x + tcond[n - 1]);
  row[14] = round_off(dtcond[n / 2 - 1] + dT[n / 2 - 1].x);
  row[15] = S.dt[0];
  if (chem) {
    // composition.TAG (outputs.f90:795-827)
    const double* xicond = V.rad(RV_XICOND);
    const double* dxicond = V.rad(RV_DXICOND);
    row[16] = round_off(1.0 + dX[0].x / dxicond[0]);
    row[17] = round_off(1.0 + dX[n - 1].x / dxicond[n - 1]);
    row[18] = round_off(1.0 + s_sh / I.sh_vol_den);
    row[19] = round_off(X[0].x + xicond[0]);
    row[20] = round_off(X[n - 1].x + xicond[n - 1]);
    row[21] = round_off(dxicond[n / 2 - 1] + dX[n / 2 - 1].x);
  } else {
    for (int k = 16; k < PZ_SERIES_COLS; ++k) row[k] = 0.0;
  }
  S.series_count += 1;
}

__global__ void k_init_state(PzDev d, int only) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= d.n_inst || (only >= 0 && inst != only)) return;
  const PzInst& I = d.inst[inst];
  PzState S;
  memset(&S, 0, sizeof(S));
  for (int k = 0; k < 4; ++k) S.dt[k] = I.dtMax;
  set_weights(I, S);
  S.lMatNext = 1;
  S.l_calc_lin = 1;
  d.state[inst] = S;
  // dummy Courant steps of the time loop's start (step_time.f90:124-125): a
  // scheme whose first stage skips the radial loop (l_exp_calc(1) false)
  // takes its first dt_courant from these
  double* cfl = d.pool + I.o_cfl;
  for (int r = 0; r < 2 * I.N; ++r) cfl[r] = 1.0e10;
}

// latest time-series row of every instance into a contiguous buffer
__global__ void k_gather_rows(PzDev d, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int inst = t / PZ_SERIES_COLS, c = t - inst * PZ_SERIES_COLS;
  if (inst >= d.n_inst) return;
  const PzInst& I = d.inst[inst];
  const int cnt = d.state[inst].series_count;
  const int idx = (cnt + PZ_SERIES_CAP - 1) % PZ_SERIES_CAP;
  out[t] = d.pool[I.o_series + (long long)idx * PZ_SERIES_COLS + c];
}

size_t build_smat_smem_bytes(int n) {
  return (3 * (size_t)n * n + 1 + 6 * (size_t)n + 32 + 16 + (size_t)(n + 1) / 2) * sizeof(double);
}
}  // namespace
// the coupled operator build's workspace in doubles when it does not fit
// shared memory (0 when it does): it then lives in the instance's pool slice
long long pz_smat_ws_doubles(int n) {
  const size_t b = build_smat_smem_bytes(n);
  return b > PZ_SMEM_MAX ? (long long)((b / sizeof(double) + 1) & ~(size_t)1) : 0;
}
namespace {
size_t build_smem_bytes(int n) {
  long long off = (long long)n * n + 3LL * n + 32 + 16 + (n + 1) / 2;
  off = (off + 1) & ~1LL;
  off += 4LL * n;
  return (size_t)off * sizeof(double);
}
// threads of the per-m kernels: one lane per (row, re/im) task of the
// widest product, rounded up to whole warps
int mloop_threads(int maxN) {
  const int h2 = (maxN + 1) / 2;
  const int t = 2 * maxN > 4 * h2 ? 2 * maxN : 4 * h2;
  return ((t + 31) / 32) * 32;
}
}  // namespace

size_t pz_rloop_smem_bytes(int P, int M, int G, int nt) {
  return 2 * (size_t)nt * G * P * sizeof(double2) + (3 + (size_t)M) * G * sizeof(double);
}

namespace {

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t pz_setup_kernels() {
  cudaError_t e;
  const int big = 200 * 1024;
  if ((e = cudaFuncSetAttribute(k_build, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  if ((e = cudaFuncSetAttribute(k_build_mloop<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  if ((e = cudaFuncSetAttribute(k_build_mloop<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  if ((e = cudaFuncSetAttribute(k_build_static, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
  if ((e = cudaFuncSetAttribute(k_mloop_integ, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  if ((e = cudaFuncSetAttribute(k_rloop<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  if ((e = cudaFuncSetAttribute(k_rloop<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX))) return e;
  return cudaSuccess;
}

size_t pz_build_smem_bytes(int n, bool direct, bool integ) {
  const size_t a = build_smem_bytes(n);
  if (integ) {
    // integ_build: complex n x n, f1 (even), colk (2n), red, redi, piv;
    // the banded factorisations: integ_bord_ws_doubles
    const size_t nd = 2 * (size_t)n * n + (((size_t)n + 1) & ~(size_t)1) + 2 * (size_t)n + 32 + 16 + ((size_t)n + 1) / 2;
    const size_t nb = (size_t)integ_bord_ws_doubles(n);
    return (nd > nb ? nd : nb) * sizeof(double);
  }
  if (!direct) return a;
  const size_t b = build_smat_smem_bytes(n);
  if (b > PZ_SMEM_MAX) return a;     // the coupled build runs in global memory (pz_smat_ws_doubles)
  return a > b ? a : b;
}

cudaError_t pz_launch_build_static(const PzDev& d, cudaStream_t s) {
  const size_t a = build_smem_bytes(d.maxN), b = (size_t)integ_bord_ws_doubles(d.maxN) * sizeof(double);
  k_build_static<<<d.n_mitems, PZ_THREADS, a > b ? a : b, s>>>(d);
  return cudaGetLastError();
}

cudaError_t pz_launch_init_state(const PzDev& d, int only, cudaStream_t s) {
  k_init_state<<<(d.n_inst + 63) / 64, 64, 0, s>>>(d, only);
  return cudaGetLastError();
}

cudaError_t pz_launch_start(const PzDev& d, int only, cudaStream_t s) {
  k_start<<<d.n_mitems, PZ_THREADS, ms_smem_bytes(d.maxN), s>>>(d, only);
  return cudaGetLastError();
}

cudaError_t pz_launch_spectra(const PzDev& d, int inst, int n_m_max, double* out, double* out2d, cudaStream_t s) {
  k_spectra<<<n_m_max, 64, 0, s>>>(d, inst, out, out2d);
  return cudaGetLastError();
}

cudaError_t pz_launch_balance(const PzDev& d, int inst, int n_m_max, const double* snap, double* vort, double* vp,
                              cudaStream_t s) {
  k_balance<<<n_m_max, 128, ms_smem_bytes(d.maxN), s>>>(d, inst, reinterpret_cast<const double2*>(snap),
                                                        reinterpret_cast<double2*>(vort), vp);
  return cudaGetLastError();
}

cudaError_t pz_launch_obs(const PzDev& d, int only, cudaStream_t s) {
  k_obs<<<d.n_oitems, 256, 0, s>>>(d, only);
  return cudaGetLastError();
}

cudaError_t pz_launch_gather_rows(const PzDev& d, double* out, cudaStream_t s) {
  const int n = d.n_inst * PZ_SERIES_COLS;
  k_gather_rows<<<(n + 127) / 128, 128, 0, s>>>(d, out);
  return cudaGetLastError();
}

cudaError_t pz_launch_step_kernel(const PzDev& d, int kind, int stage, cudaStream_t s) {
  switch (kind) {
    case PZK_RLOOP:
      if (d.any_chem) k_rloop<true><<<d.n_ritems, 256, d.smem_rloop, s>>>(d, stage);
      else k_rloop<false><<<d.n_ritems, 256, d.smem_rloop, s>>>(d, stage);
      break;
    case PZK_CFL: k_cfl<<<d.n_inst, 32, 0, s>>>(d); break;
    case PZK_BUILD: k_build<<<d.n_mitems, PZ_THREADS, d.smem_build, s>>>(d); break;
    case PZK_MLOOP: k_mloop<<<d.n_mitems, mloop_threads(d.maxN), ms_smem_bytes(d.maxN), s>>>(d, stage); break;
    case PZK_ORDER: k_order<<<1, 1024, 0, s>>>(d); break;
    case PZK_BUILD_MLOOP: {
      const size_t sm = (size_t)d.smem_build > ms_smem_bytes(d.maxN) ? (size_t)d.smem_build : ms_smem_bytes(d.maxN);
      if (d.any_chem) k_build_mloop<true><<<d.n_mitems, mloop_threads(d.maxN), sm, s>>>(d);
      else k_build_mloop<false><<<d.n_mitems, mloop_threads(d.maxN), sm, s>>>(d);
      break;
    }
    case PZK_MLOOP_INTEG:
      k_mloop_integ<<<d.n_mitems, mloop_threads(d.maxN), integ_mloop_smem_bytes(d.maxN), s>>>(d, stage);
      break;
    case PZK_OBS: k_obs<<<d.n_oitems, 256, 0, s>>>(d, -1); break;
    case PZK_ASSEMBLE: k_assemble<<<d.n_mitems, mloop_threads(d.maxN), ms_smem_bytes(d.maxN), s>>>(d); break;
    case PZK_FAST: return pz_launch_fast(d, s);
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

const char* pz_step_kernel_name(int kind) {
  static const char* names[PZK_KINDS] = {"k_rloop", "k_cfl", "k_build", "k_mloop", "k_obs", "k_assemble",
                                         "k_mloop_integ", "k_order", "k_build_mloop", "k_fast"};
  return (kind >= 0 && kind < PZK_KINDS) ? names[kind] : "";
}

// Discrete adjoint of the multistep collocation step (influence-matrix solve,
// or the direct solve of update_om_coll_smat, whose coupled solve transposes
// to G^H and whose implicit Ekman pumping and Coriolis terms join L^T):
// gradient of a time-averaged 3-D kinetic energy or outer-boundary Nusselt
// number with respect to the initial temperature perturbation and to BuoFac
// (hence Ra).
//
// The step of k_rloop/k_cfl/k_build/k_mloop is, per instance, a map of the
// state S_n = (Tc, oc, pc, uc) -- the Chebyshev coefficients of temperature,
// vorticity and streamfunction (m /= 0) and of u_phi (m = 0) -- plus the
// history of the earlier steps (old_{n-k}, impl_{n-k}, E_{n-k}, k >= 1, as the
// scheme's nold, nimp, nexp slots hold them; CNAB2: E_{n-1} only):
//   fields f_n   = L(S_n)                 T, us, up, om, implicit terms iT, iP
//                                         (get_temp_rhs_imp_coll, get_psi_rhs_imp_coll_dmat)
//   nonlinear    = NL(f_n)                radial_loop.f90:231-394
//   E_n          = FIN(f_n, NL)           finish_exp_temp_coll / finish_exp_psi_coll_dmat
//   S_{n+1}      = SOLVE(rhs_n),  rhs_n = sum_k wimp[k] old_{n-k} + sum_k wimp_lin[k+1]
//                  impl_{n-k} + sum_k wexp[k] E_{n-k}   update_temp_co, update_om_coll_dmat
// with SOLVE linear in its inputs for a fixed time-step sequence.  The backward
// step is the exact transpose of each piece, in reverse order:
//   k_adj_solve  (instance, m)  SOLVE^T and FIN^T (local part): influence
//                               correction, K^T, G_om^T / G_uphi^T, buoyancy,
//                               G_T^T, IMEX weights, D1p^T
//   k_adj_rloop  (instance, r)  NL^T: phi-FFT adjoints and product rule
//   k_adj_lin    (instance, m)  L^T plus the kinetic-energy source:
//                               C^T, D1c^T, D2c^T
// Complex numbers are treated as pairs of reals: the adjoint of y = a x is
// x_bar = conj(a) y_bar, and a real matrix transposes.  The gradient g of a
// real J with respect to a complex z is the one with dJ = Re(conj(g) dz).
//
// The time-step sequence is held fixed: the sweep either takes it from the
// caller or records the one chosen by the Courant controller, and the
// gradient is that of J for the recorded sequence (dt_courant's choices are
// piecewise constant in the state; the value picked at a change point is
// not differentiated).
//
// Memory: the forward sweep stores a checkpoint (fields, history rings and
// step state) every `checkpoint_every` steps and the physical fields
// (T, us, up, om) of every step of the last segment; the backward sweep
// recomputes each earlier segment from its checkpoint before running it
// backwards.  Operators are rebuilt in the backward sweep wherever the
// recorded weights change.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "pizza_gpu.h"
#include "pz_device.cuh"
#include "pz_handle.h"
#include "pz_internal.h"

namespace {

// planes of M*N complex per instance in the adjoint workspace
enum {
  AP_TCB = 0, AP_OCB, AP_PCB, AP_UCB,   // adjoint of the state (row 0 of AP_UCB: u_phi, m = 0)
  AP_CT, AP_CP,                          // adjoint of E_n carried from the later steps (sum over k >= 1
                                         // of wexp_{n+k}[k] times their rhs adjoints)
  AP_C2T, AP_C2P, AP_C3T, AP_C3P,        // the same for E_{n-1}, E_{n-2} (multistep schemes with nexp > 2)
  AP_O1T, AP_O1P, AP_O2T, AP_O2P, AP_O3T, AP_O3P,   // adjoint of old_{n-1..n-3} from the later steps
  AP_OTB, AP_OPB,                        // adjoint of old_n (temperature; vorticity or u_phi), complete
  AP_I1T, AP_I1P, AP_I2T, AP_I2P,        // adjoint of impl_{n-1..n-2} from the later steps (nimp > 1)
  AP_ITB, AP_IPB,                        // adjoint of impl_n, complete
  AP_RTB, AP_RPB,                        // adjoint of the solve right-hand sides of step n
  AP_ETB, AP_EPB,                        // adjoint of E_n (temperature, vorticity)
  AP_VTB, AP_VOB,                        // adjoint of dVsT, dVsOm
  AP_AUS, AP_AUP, AP_AOM, AP_AT,         // adjoint of us, up, om, T through the nonlinear terms
  AP_DB,                                 // dJ/dBuoFac partial sums per m (first M doubles)
  AP_SNAP                                // CNAB2: snapshots, 4 planes each (T, us, up, om)
};
// DIRK sweep: after AP_DB, the adjoint of the physical fields of the state
// (lambda), of the old slot, and of the explicit and implicit terms of each
// stage (2 planes each: temperature, vorticity); the snapshots follow
enum { DP_LT = AP_SNAP, DP_LUS, DP_LUP, DP_LOM, DP_OT, DP_OP, DP_E };
enum { SN_T = 0, SN_US, SN_UP, SN_OM };

struct PzAdjDev {
  PzDev d;                  // forward launch parameters
  double* ws;               // workspace
  const long long* o_ws;    // per-instance offset (doubles)
  const PzState* rec;       // [inst][n_steps] state of every step after its dt/weight update
  PzState* ck_state;        // [inst][n_ck]
  PzState* bstate;          // [inst] state handed to k_build in the backward sweep
  double* J;                // [inst] objective
  double* out;              // gradient output, ABI layout, instances concatenated
  const long long* o_out;   // per-instance offset into out (doubles)
  int n_steps, n_snap, n_ck, ck_planes;
  int win0;                 // first state index of the averaging window
  double inv_window;
  int objective;            // PZ_OBJ_EKIN3D or PZ_OBJ_NUTOP
  int snap0;                // plane of snapshot 0 (AP_SNAP, or after the DIRK planes)
  // DIRK sweep (one tableau for all instances): stages, solved stages + 1
  // (stage states per step), assembly stage, l_exp_calc / l_imp_calc_rhs bits
  int dirk, ns, s1, assembly, exp_mask, imp_mask;
  // grid snapshots (null: k_adj_rloop transforms the spectral snapshots):
  // slot k of instance i at gs + o_gs[i] + k * N * 2P, written by the
  // forward k_rloop that transforms stage state k
  double2* gs;
  const long long* o_gs;
};

struct AdjView {
  const PzInst* I;
  double* base;
  int snap0;
  __device__ double2* plane(long long k, int mi) const {
    return reinterpret_cast<double2*>(base) + (k * I->M + mi) * I->N;
  }
  __device__ double2* snap(int slot, int f, int mi) const { return plane(snap0 + 4LL * slot + f, mi); }
  __device__ double2* ck(int n_snap, int ck_planes, int c, int k, int mi) const {
    return plane(snap0 + 4LL * n_snap + (long long)c * ck_planes + k, mi);
  }
  __device__ double* db() const { return reinterpret_cast<double*>(plane(AP_DB, 0)); }
  // DIRK: adjoint of the explicit (e) or implicit (i) term of stage slot k, field f (0 T, 1 vorticity)
  __device__ double2* dE(int k, int f, int mi) const { return plane(DP_E + 2LL * k + f, mi); }
  __device__ double2* dI(int ns, int k, int f, int mi) const { return plane(DP_E + 2LL * ns + 2LL * k + f, mi); }
};

__device__ __forceinline__ AdjView adj_view(const PzAdjDev& a, int inst) {
  return AdjView{&a.d.inst[inst], a.ws + a.o_ws[inst], a.snap0};
}

// per-m scratch: 12 vectors of n complex, the parity-product scratch and a
// reduction buffer
struct AS {
  double2* v[12];
  SymScratch w;
  double* red;
};
__device__ AS as_smem(int n) {
  extern __shared__ double2 shm[];
  const int h2 = (n + 1) / 2;
  AS s;
  for (int k = 0; k < 12; ++k) s.v[k] = shm + k * n;
  s.w.s = shm + 12 * n;
  s.w.a = s.w.s + h2;
  s.w.t1 = reinterpret_cast<double*>(s.w.a + h2);
  s.w.t2 = s.w.t1 + 4 * h2;
  s.red = s.w.t2 + 4 * h2;
  return s;
}
size_t as_smem_bytes(int n) {
  const size_t h2 = (size_t)(n + 1) / 2;
  return 12 * (size_t)n * sizeof(double2) + 2 * h2 * sizeof(double2) + 8 * h2 * sizeof(double) + 64 * sizeof(double);
}
int adj_threads(int maxN) {
  const int h2 = (maxN + 1) / 2;
  const int t = 2 * maxN > 4 * h2 ? 2 * maxN : 4 * h2;
  return ((t + 31) / 32) * 32;
}
// G radii per block: the forward's k_rloop grouping (PzInst::rg), since both
// walk the same (instance, radius) work list
size_t adj_rloop_smem_bytes(int P, int G, bool grid) {
  return (grid ? 4 : 6) * (size_t)G * P * sizeof(double2) + G * sizeof(double);
}

__device__ __forceinline__ double2 cz() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double2 caxpy(double s, double2 x, double2 y) {
  return make_double2(fma(s, x.x, y.x), fma(s, x.y, y.y));
}
// Re(conj(x) y)
__device__ __forceinline__ double cdotr(double2 x, double2 y) { return x.x * y.x + x.y * y.y; }

// y = G^H (x0; x1), G complex 2n x n column-major with leading dimension 2n
// (the smat solve's inverse columns): the adjoint of (x0, x1) = G y
struct CDenseDotH {
  const double2* __restrict__ G; int n; const double2* __restrict__ x0; const double2* __restrict__ x1;
  double* __restrict__ y;
  __device__ __forceinline__ double fma(int t, int i, double acc) const {
    const double2 g = __ldg(G + i + (long long)(t >> 1) * 2 * n);
    const double2 v = i < n ? x0[i] : x1[i - n];
    return (t & 1) ? ::fma(g.x, v.y, ::fma(-g.y, v.x, acc)) : ::fma(g.x, v.x, ::fma(g.y, v.y, acc));
  }
  __device__ __forceinline__ void store(int t, double v) const { y[t] = v; }
};
__device__ __forceinline__ void cmvH_lanes(const double2* __restrict__ G, int n, const double2* __restrict__ x0,
                                           const double2* __restrict__ x1, double2* __restrict__ y) {
  lane_dots(CDenseDotH{G, n, x0, x1, reinterpret_cast<double*>(y)}, 2 * n, 2 * n);
}

// ---------------------------------------------------------------------------
// forward-sweep helpers
// ---------------------------------------------------------------------------
// physical fields of the current state -> snapshot `slot`
__global__ void k_adj_snap(PzAdjDev a, int slot) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const PzInst& I = a.d.inst[it.inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, it.inst);
  const int n = I.N, mi = it.idx;
  const double2* src[4] = {V.fld(F_TEMP, mi), V.fld(F_US, mi), V.fld(F_UP, mi), V.fld(F_OM, mi)};
  for (int f = 0; f < 4; ++f) {
    double2* dst = A.snap(slot, f, mi);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[f][i];
  }
}

// checkpoint c: save (dir 0) or restore (dir 1) fields, history rings and the
// step state.  A restored state rebuilds its operators at its next step.
__global__ void k_adj_ckpt(PzAdjDev a, int c, int dir) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const AdjView A = adj_view(a, inst);
  const int n = I.N, mi = it.idx;
  const long long MN = (long long)I.M * n;
  const int nh = 2 * (I.nold + I.nimp + I.nexp);
  // the flow and temperature planes (F_US .. F_DVSOM; the adjoint runs no composition)
  for (int k = 0; k < F_XI + nh; ++k) {
    double2* p = reinterpret_cast<double2*>(a.d.pool + (k < F_XI ? I.o_fld + 2LL * k * MN
                                                                   : I.o_hist + 2LL * (k - F_XI) * MN)) +
                 (long long)mi * n;
    double2* q = A.ck(a.n_snap, a.ck_planes, c, k, mi);
    if (dir == 0)
      for (int i = threadIdx.x; i < n; i += blockDim.x) q[i] = p[i];
    else
      for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = q[i];
  }
  if (mi == 0 && threadIdx.x == 0) {
    PzState* cs = a.ck_state + (long long)inst * a.n_ck + c;
    if (dir == 0) {
      *cs = a.d.state[inst];
    } else {
      PzState S = *cs;
      S.lMatNext = 1;
      a.d.state[inst] = S;
    }
  }
}

// J += objective(current state) / n_window: us2_3D + up2_3D + uz2_3D (the
// e_kin_3D sums of outputs.f90:553-570, as k_obs forms them) or NuTop
// = 1 + dT/dr(m=0, r_cmb) / dtcond(r_cmb) (outputs.f90:742-746)
__global__ void k_adj_ke(PzAdjDev a) {
  const int inst = blockIdx.x;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  __shared__ double red[32];
  if (a.objective == PZ_OBJ_NUTOP) {
    if (threadIdx.x == 0)
      a.J[inst] += (1.0 + V.fld(F_DTEMP, 0)[0].x / V.rad(RV_DTCOND)[0]) * a.inv_window;
    return;
  }
  const int n = I.N, M = I.M;
  const double* rr = V.rad(RV_R);
  const double* h = V.rad(RV_HEIGHT);
  const double* beta = V.rad(RV_BETA);
  const double* wint = V.rad(RV_WINT);
  const double2* us = V.fld(F_US, 0);
  const double2* up = V.fld(F_UP, 0);
  double s3 = 0.0;
  if (!(I.flags & PZF_NON_ROT)) {
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
      double us2 = 0.0, up2 = 0.0;
      for (int mi = 0; mi < M; ++mi) {
        const double2 x = us[(long long)mi * n + r], y = up[(long long)mi * n + r];
        if (mi == 0) { us2 += x.x * x.x; up2 += y.x * y.x; }
        else { us2 += 2.0 * (x.x * x.x + x.y * x.y); up2 += 2.0 * (y.x * y.x + y.y * y.y); }
      }
      s3 += wint[r] * us2 * rr[r] * h[r] + wint[r] * up2 * rr[r] * h[r] +
            wint[r] * us2 * beta[r] * beta[r] * rr[r] * h[r] * h[r] * h[r] / 12.0;
    }
  }
  s3 = block_sum(s3, red);
  if (threadIdx.x == 0) a.J[inst] += 3.14159265358979323846 * s3 * a.inv_window;
}

// ---------------------------------------------------------------------------
// backward-sweep kernels
// ---------------------------------------------------------------------------
__global__ void k_adj_zero(PzAdjDev a) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const PzInst& I = a.d.inst[it.inst];
  const AdjView A = adj_view(a, it.inst);
  for (int k = 0; k <= AP_DB; ++k) {
    double2* p = A.plane(k, it.idx);
    for (int i = threadIdx.x; i < I.N; i += blockDim.x) p[i] = cz();
  }
}

// operators of step n for k_build: lMat where the weights differ from step n+1's
__global__ void k_adj_bstate(PzAdjDev a, int n) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= a.d.n_inst) return;
  const PzState* r = a.rec + (long long)inst * a.n_steps;
  PzState S = r[n];
  S.lMat = (n + 1 >= a.n_steps || r[n].wimp_lin[0] != r[n + 1].wimp_lin[0]) ? 1 : 0;
  S.status = 0;
  a.bstate[inst] = S;
}

// SOLVE^T and the local part of FIN^T for step n (snapshot `slot` = state n)
__global__ void __launch_bounds__(256, 4) k_adj_solve(PzAdjDev a, int n, int slot) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const PzState& S = a.rec[(long long)inst * a.n_steps + n];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx, m = mi * I.minc;
  const double dm = (double)m;
  AS s = as_smem(N);
  const double w0 = S.wimp[0], wl0 = S.wimp_lin[0], wl1 = S.wimp_lin[1];
  const double we0 = S.wexp[0], we1 = S.wexp[1];
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  (void)w0;
  const double* or1 = V.rad(RV_OR1);
  const double* rgrav = V.rad(RV_RGRAV);
  double2 *Tc = s.v[0], *oc = s.v[1], *pc = s.v[2], *x = s.v[3], *y = s.v[4];
  double2 *rT = s.v[5], *rP = s.v[6], *eT = s.v[7], *eP = s.v[8], *t = s.v[9];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    Tc[i] = A.plane(AP_TCB, mi)[i];
    oc[i] = (m == 0) ? A.plane(AP_UCB, 0)[i] : A.plane(AP_OCB, mi)[i];
    pc[i] = (m == 0) ? cz() : A.plane(AP_PCB, mi)[i];
  }
  __syncthreads();
  if (m != 0 && (I.flags & PZF_DIRECT)) {
    // update_om_coll_smat's coupled solve (update_psi_coll_smat.f90:88-321):
    // (oc, pc) = G rhs  ->  rhs_bar = G^H (oc_bar, pc_bar)
    cmvH_lanes(reinterpret_cast<const double2*>(a.d.pool + I.o_gsm) + 2LL * mi * N * N, N, oc, pc, rP);
    __syncthreads();
  }
  if (m != 0) {
    if (!(I.flags & PZF_DIRECT)) {
    // influence correction (update_psi_coll_dmat.f90:1256-1300), transposed
    const long long MN = (long long)I.M * N;
    const double* aux = a.d.pool + I.o_aux;
    const double* om2 = aux + 0 * MN + (long long)mi * N;
    const double* om3 = aux + 1 * MN + (long long)mi * N;
    const double* psi2 = aux + 2 * MN + (long long)mi * N;
    const double* psi3 = aux + 3 * MN + (long long)mi * N;
    const double* infl = aux + 4 * MN + 4LL * mi;
    const double* bct = V.rad(RV_BCTOP);
    const double* bcb = V.rad(RV_BCBOT);
    double c1r = 0.0, c1i = 0.0, c2r = 0.0, c2i = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      c1r += psi2[i] * pc[i].x + om2[i] * oc[i].x;
      c1i += psi2[i] * pc[i].y + om2[i] * oc[i].y;
      c2r += psi3[i] * pc[i].x + om3[i] * oc[i].x;
      c2i += psi3[i] * pc[i].y + om3[i] * oc[i].y;
    }
    c1r = block_sum(c1r, s.red); c1i = block_sum(c1i, s.red);
    c2r = block_sum(c2r, s.red); c2i = block_sum(c2i, s.red);
    const double ttr = -infl[0] * c1r - infl[2] * c2r, tti = -infl[0] * c1i - infl[2] * c2i;
    const double tbr = -infl[1] * c1r - infl[3] * c2r, tbi = -infl[1] * c1i - infl[3] * c2i;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      x[i] = make_double2(pc[i].x + ttr * bct[i] + tbr * bcb[i], pc[i].y + tti * bct[i] + tbi * bcb[i]);
    __syncthreads();
    // psi = -K om  ->  om_bar -= K^T psi_bar
    mvT_lanes(a.d.pool + I.o_gpsi + (long long)mi * N * N, N, x, y);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = csub(oc[i], y[i]);
    __syncthreads();
    mvT_lanes(a.d.pool + I.o_gom + (long long)mi * N * N, N, x, rP);
    __syncthreads();
    }
    // implicit buoyancy of the new temperature in the vorticity rhs
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      if (i == 0 || i == N - 1) rP[i] = cz();
      x[i] = buo_imp ? cscale(wl0 * I.BuoFac * rgrav[i] * or1[i], cim(dm, rP[i])) : cz();
    }
    __syncthreads();
    if (buo_imp) {
      op_CT(V, N, x, y, s.w);
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += blockDim.x) Tc[i] = cadd(Tc[i], y[i]);
      __syncthreads();
    }
  } else {
    mvT_lanes(a.d.pool + I.o_guphi, N, oc, rP);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      if (i == 0 || i == N - 1) rP[i] = cz(); else rP[i].y = 0.0;
    __syncthreads();
  }
  const double* GT = ((I.flags & PZF_T_IS_OM) && m != 0) ? a.d.pool + I.o_gom + (long long)mi * N * N
                                                         : a.d.pool + I.o_gt + (long long)mi * N * N;
  mvT_lanes(GT, N, Tc, rT);
  __syncthreads();
  // IMEX weights (multistep_schemes.f90:308-316): rhs_n = sum_k wimp_n[k] old_{n-k}
  // + wimp_lin_n[1] impl_n + sum_k wexp_n[k] E_{n-k}.  The adjoints of old_n and
  // E_n collect wimp_{n+k}[k] and wexp_{n+k}[k] times the rhs adjoint of every
  // later step n+k: shift registers of carry planes, one per k >= 1.
  double wi[4], we[4], wl[3];
  for (int k = 0; k < 4; ++k) {
    wi[k] = k < I.nold ? S.wimp[k] : 0.0;
    we[k] = k < I.nexp ? S.wexp[k] : 0.0;
    if (k < 3) wl[k] = k < I.nimp ? S.wimp_lin[k + 1] : 0.0;
  }
  double2* i1T = A.plane(AP_I1T, mi);
  double2* i1P = A.plane(AP_I1P, mi);
  double2* i2T = A.plane(AP_I2T, mi);
  double2* i2P = A.plane(AP_I2P, mi);
  (void)we0; (void)we1;
  double2* cT = A.plane(AP_CT, mi);
  double2* cP = A.plane(AP_CP, mi);
  double2* c2T = A.plane(AP_C2T, mi);
  double2* c2P = A.plane(AP_C2P, mi);
  double2* c3T = A.plane(AP_C3T, mi);
  double2* c3P = A.plane(AP_C3P, mi);
  double2* o1T = A.plane(AP_O1T, mi);
  double2* o1P = A.plane(AP_O1P, mi);
  double2* o2T = A.plane(AP_O2T, mi);
  double2* o2P = A.plane(AP_O2P, mi);
  double2* o3T = A.plane(AP_O3T, mi);
  double2* o3P = A.plane(AP_O3P, mi);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 rt = (i == 0 || i == N - 1) ? cz() : rT[i];
    const double2 rp = rP[i];
    rT[i] = rt;
    const double2 et = caxpy(we[0], rt, cT[i]), ep = caxpy(we[0], rp, cP[i]);
    eT[i] = et; eP[i] = ep;
    cT[i] = caxpy(we[1], rt, c2T[i]);
    cP[i] = caxpy(we[1], rp, c2P[i]);
    c2T[i] = caxpy(we[2], rt, c3T[i]);
    c2P[i] = caxpy(we[2], rp, c3P[i]);
    c3T[i] = cscale(we[3], rt);
    c3P[i] = cscale(we[3], rp);
    A.plane(AP_OTB, mi)[i] = caxpy(wi[0], rt, o1T[i]);
    A.plane(AP_OPB, mi)[i] = caxpy(wi[0], rp, o1P[i]);
    o1T[i] = caxpy(wi[1], rt, o2T[i]);
    o1P[i] = caxpy(wi[1], rp, o2P[i]);
    o2T[i] = caxpy(wi[2], rt, o3T[i]);
    o2P[i] = caxpy(wi[2], rp, o3P[i]);
    o3T[i] = cscale(wi[3], rt);
    o3P[i] = cscale(wi[3], rp);
    A.plane(AP_ITB, mi)[i] = caxpy(wl[0], rt, i1T[i]);
    A.plane(AP_IPB, mi)[i] = caxpy(wl[0], rp, i1P[i]);
    i1T[i] = caxpy(wl[1], rt, i2T[i]);
    i1P[i] = caxpy(wl[1], rp, i2P[i]);
    i2T[i] = cscale(wl[2], rt);
    i2P[i] = cscale(wl[2], rp);
    A.plane(AP_RTB, mi)[i] = rt;
    A.plane(AP_RPB, mi)[i] = rp;
    A.plane(AP_ETB, mi)[i] = et;
    A.plane(AP_EPB, mi)[i] = ep;
    x[i] = cscale(-or1[i], et);
    y[i] = cscale(-or1[i], ep);
  }
  __syncthreads();
  // dVsT_bar = D1p^T (-or1 eT_bar), dVsOm_bar likewise (m /= 0)
  op_D1pT(V, N, x, t, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VTB, mi)[i] = t[i];
  __syncthreads();
  if (m != 0) {
    op_D1pT(V, N, y, t, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VOB, mi)[i] = t[i];
    // dJ/dBuoFac: buoyancy in the rhs (new temperature) and in the implicit
    // term of state n, or the explicit buoyancy of FIN
    const double2* Tn = A.snap(slot, SN_T, mi);
    const double2* Tn1 = A.snap(slot + 1, SN_T, mi);
    double acc = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const double c = rgrav[i] * or1[i];
      if (buo_imp) {
        acc += cdotr(rP[i], cscale(-wl0 * c, cim(dm, Tn1[i])));
        acc += cdotr(A.plane(AP_IPB, mi)[i], cscale(-c, cim(dm, Tn[i])));   // impl_n, all later steps
      } else {
        acc += cdotr(eP[i], cscale(-c, cim(dm, Tn[i])));
      }
    }
    acc = block_sum(acc, s.red);
    if (threadIdx.x == 0) A.db()[mi] += acc;
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VOB, mi)[i] = cz();
  }
}

// NL^T for a group of PzInst::rg radii: the adjoint of
//   A = fft(r us T), B = fft(up T), C = fft(r us om), D = fft(up om)
//   ET = -(i m/r) B - tfac A,  EP = -(i m/r) D (m > 0),  EP(0) = -sum_m us_fluct om
// with fft = rfft/P truncated to M and the grids from c2r of the spectra.
// The adjoint of fft is a c2r of the spectrum scaled by 1/(2P) (1/P and the
// real part at m = 0); the adjoint of the c2r is an r2c scaled by 2 (1 and
// the real part at m = 0).  The state's grids are the forward k_rloop's
// (GRID: read from the grid snapshot) or a c2r of the spectral snapshot.
// Shared memory: three buffers of 2*G transforms, two with GRID.
template <bool GRID>
__global__ void __launch_bounds__(256) k_adj_rloop(PzAdjDev a, int slot) {
  extern __shared__ double2 sh[];
  const PzItem it = a.d.ritems[blockIdx.x];
  const int inst = it.inst, r0 = it.idx;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, M = I.M, P = I.P;
  const int G = min(I.rg, N - r0);
  const double2* tw = reinterpret_cast<const double2*>(V.pool + I.o_tw);
  double2* b0 = sh;                                // state spectra (without GRID)
  double2* b1 = GRID ? sh : sh + 2 * G * P;
  double2* b2 = b1 + 2 * G * P;                    // spectra of the adjoint products
  double* ep0 = reinterpret_cast<double*>(b2 + 2 * G * P);
  for (int k = threadIdx.x; k < 2 * G * P; k += blockDim.x) {
    if (!GRID) b0[k] = cz();
    b2[k] = cz();
  }
  __syncthreads();
  const double inv2P = 0.5 / (double)P, invP = 1.0 / (double)P;
  for (int t = threadIdx.x; t < G * M; t += blockDim.x) {
    const int g = t / M, mi = t - g * M, r = r0 + g;
    const double dm = (double)(mi * I.minc);
    const long long o = (long long)mi * N + r;
    if (!GRID) {
      // grids of the state (as k_rloop)
      double2 us = A.snap(slot, SN_US, 0)[o], up = A.snap(slot, SN_UP, 0)[o];
      double2 om = A.snap(slot, SN_OM, 0)[o], T = A.snap(slot, SN_T, 0)[o];
      if (mi == 0) { us.y = 0.0; up.y = 0.0; om.y = 0.0; T.y = 0.0; }
      double2* z1 = b0 + (2 * g) * P;
      double2* z2 = b0 + (2 * g + 1) * P;
      z1[mi] = make_double2(us.x - up.y, us.y + up.x);
      z2[mi] = make_double2(om.x - T.y, om.y + T.x);
      if (mi > 0) {
        z1[P - mi] = make_double2(us.x + up.y, -us.y + up.x);
        z2[P - mi] = make_double2(om.x + T.y, -om.y + T.x);
      }
    }
    // spectra of the adjoint products
    const double or1 = V.rad(RV_OR1)[r];
    const double tfac = (1.0 - I.tadvz) * V.rad(RV_BETA)[r] * or1;
    const double2 et = A.plane(AP_ETB, 0)[o], ep = A.plane(AP_EPB, 0)[o];
    double2 hA = csub(A.plane(AP_VTB, 0)[o], cscale(tfac, et));
    double2 hB = cscale(or1, cim(dm, et));
    double2 hC = A.plane(AP_VOB, 0)[o];
    double2 hD = (mi == 0) ? cz() : cscale(or1, cim(dm, ep));
    if (mi == 0) {
      hA = make_double2(hA.x * invP, 0.0); hB = make_double2(hB.x * invP, 0.0);
      hC = make_double2(hC.x * invP, 0.0); hD = cz();
      ep0[g] = ep.x;
    } else {
      hA = cscale(inv2P, hA); hB = cscale(inv2P, hB); hC = cscale(inv2P, hC); hD = cscale(inv2P, hD);
    }
    double2* z3 = b2 + (2 * g) * P;
    double2* z4 = b2 + (2 * g + 1) * P;
    z3[mi] = make_double2(hA.x - hB.y, hA.y + hB.x);
    z4[mi] = make_double2(hC.x - hD.y, hC.y + hD.x);
    if (mi > 0) {
      z3[P - mi] = make_double2(hA.x + hB.y, -hA.y + hB.x);
      z4[P - mi] = make_double2(hC.x + hD.y, -hC.y + hD.x);
    }
  }
  __syncthreads();
  const double2* X;
  double2 *Y, *W;
  if (GRID) {
    X = a.gs + a.o_gs[inst] + ((long long)slot * N + r0) * 2 * P;
    Y = fft_run(b2, b1, I, tw, 2 * G, true);
    W = (Y == b2) ? b1 : b2;
  } else {
    double2* Xs = fft_run(b0, b1, I, tw, 2 * G, true);
    double2* fr = (Xs == b0) ? b1 : b0;
    Y = fft_run(b2, fr, I, tw, 2 * G, true);
    W = (Y == b2) ? fr : b2;
    X = Xs;
  }
  // product rule on the grid
  for (int t = threadIdx.x; t < G * P; t += blockDim.x) {
    const int g = t / P, j = t - g * P;
    const double rr = V.rad(RV_R)[r0 + g];
    const double2 x1 = X[(2 * g) * P + j], x2 = X[(2 * g + 1) * P + j];
    const double2 y1 = Y[(2 * g) * P + j], y2 = Y[(2 * g + 1) * P + j];
    const double usg = x1.x, upg = x1.y, omg = x2.x, Tg = x2.y;
    const double ab = y1.x, bb = y1.y, cb = y2.x, db = y2.y;
    const double usgb = rr * (Tg * ab + omg * cb);
    const double upgb = Tg * bb + omg * db;
    const double omgb = rr * usg * cb + upg * db;
    const double Tgb = rr * usg * ab + upg * bb;
    Y[(2 * g) * P + j] = make_double2(usgb, upgb);
    Y[(2 * g + 1) * P + j] = make_double2(omgb, Tgb);
  }
  __syncthreads();
  double2* F = fft_run(Y, W, I, tw, 2 * G, false);
  for (int t = threadIdx.x; t < G * M; t += blockDim.x) {
    const int g = t / M, mi = t - g * M, r = r0 + g;
    const long long o = (long long)mi * N + r;
    const int mc = (P - mi) % P;
    const double2* f1 = F + (2 * g) * P;
    const double2* f2 = F + (2 * g + 1) * P;
    const double2 Z = f1[mi], Zc = f1[mc], Yv = f2[mi], Yc = f2[mc];
    double2 a_us = make_double2(0.5 * (Z.x + Zc.x), 0.5 * (Z.y - Zc.y));
    double2 a_up = make_double2(0.5 * (Z.y + Zc.y), -0.5 * (Z.x - Zc.x));
    double2 a_om = make_double2(0.5 * (Yv.x + Yc.x), 0.5 * (Yv.y - Yc.y));
    double2 a_T = make_double2(0.5 * (Yv.y + Yc.y), -0.5 * (Yv.x - Yc.x));
    const double e0 = ep0[g];
    if (mi == 0) {
      a_us = make_double2(a_us.x, 0.0);
      a_up = make_double2(a_up.x, 0.0);
      a_om = make_double2(a_om.x, 0.0);
      a_T = make_double2(a_T.x, 0.0);
      // us_fluct(m=0) = E CorFac ekpump up(m=0) / 2 in the Reynolds stress
      const double f = 0.5 * I.ek * I.CorFac * V.rad(RV_EKPUMP)[r];
      a_up.x -= e0 * f * A.snap(slot, SN_OM, 0)[o].x;
      a_om.x -= e0 * f * A.snap(slot, SN_UP, 0)[o].x;
    } else {
      a_us = cscale(2.0, a_us); a_up = cscale(2.0, a_up);
      a_om = cscale(2.0, a_om); a_T = cscale(2.0, a_T);
      a_us = caxpy(-2.0 * e0, A.snap(slot, SN_OM, 0)[o], a_us);
      a_om = caxpy(-2.0 * e0, A.snap(slot, SN_US, 0)[o], a_om);
    }
    A.plane(AP_AUS, 0)[o] = a_us;
    A.plane(AP_AUP, 0)[o] = a_up;
    A.plane(AP_AOM, 0)[o] = a_om;
    A.plane(AP_AT, 0)[o] = a_T;
  }
}

// L^T for step n: field adjoints of state n -> adjoint of S_n.  `terminal`
// handles the final state (only the kinetic-energy source), `ke` adds the
// source of the averaging window.
__global__ void __launch_bounds__(256, 3) k_adj_lin(PzAdjDev a, int n, int slot, int terminal, int src) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx, m = mi * I.minc;
  const double dm = (double)m, dm2 = dm * dm;
  AS s = as_smem(N);
  double w0 = 0.0, wl1 = 0.0;
  if (!terminal) {
    const PzState& S = a.rec[(long long)inst * a.n_steps + n];
    w0 = S.wimp[0];
    wl1 = S.wimp_lin[1];
  }
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  const bool rot = !(I.flags & PZF_NON_ROT);
  const bool ek = (I.flags & PZF_EK_PUMP) != 0;
  const bool direct = (I.flags & PZF_DIRECT) != 0;
  const double TdF = I.TdiffFac, Vis = I.ViscFac;
  const double* rr = V.rad(RV_R);
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
  const double* h = V.rad(RV_HEIGHT);
  const double* wint = V.rad(RV_WINT);
  const double pi = 3.14159265358979323846;
  double2** v = s.v;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 rT = cz(), rP = cz(), eT = cz(), eP = cz(), aus = cz(), aup = cz(), aom = cz(), aT = cz();
    if (!terminal) {
      rT = A.plane(AP_RTB, mi)[i]; rP = A.plane(AP_RPB, mi)[i];
      eT = A.plane(AP_ETB, mi)[i]; eP = A.plane(AP_EPB, mi)[i];
      aus = A.plane(AP_AUS, mi)[i]; aup = A.plane(AP_AUP, mi)[i];
      aom = A.plane(AP_AOM, mi)[i]; aT = A.plane(AP_AT, mi)[i];
    }
    // adjoints of old_n and impl_n, collected over every later step that reads them
    double2 Tb = aT, oldPb = cz(), iTb = cz(), iPb = cz();
    if (!terminal) {
      Tb = cadd(Tb, A.plane(AP_OTB, mi)[i]);
      oldPb = A.plane(AP_OPB, mi)[i];
      iTb = A.plane(AP_ITB, mi)[i];
      iPb = A.plane(AP_IPB, mi)[i];
    }
    (void)rT; (void)w0; (void)wl1;
    // FIN^T (update_temp_coll.f90:152-176, update_psi_coll_dmat.f90:468-552)
    const double gT = dtcond[i] - I.tadvz * beta[i] * tcond[i];
    double2 usb = caxpy(-gT, eT, aus), upb = aup, omb = aom;
    if (m != 0) {
      // explicit Coriolis: dmat when rotating, smat unless it is implicit;
      // Ekman pumping is explicit with dmat, implicit (below) with smat
      if (direct ? !(I.flags & PZF_COR_IMP) : rot) usb = caxpy(I.CorFac * beta[i], eP, usb);
      if (ek && !direct) {
        const double ce = I.CorFac * ekpump[i];
        // (i m ekp_dusdp + ekp_us) us  ->  conj(.) eP
        usb = csub(usb, cscale(ce, csub(cscale(ekp_us[i], eP), cscale(ekp_dusdp[i], cim(dm, eP)))));
        upb = caxpy(-ce * ekp_up[i], eP, upb);
        omb = caxpy(-ce, eP, omb);
      }
      if (!buo_imp) Tb = cadd(Tb, cscale(I.BuoFac * rgrav[i] * or1[i], cim(dm, eP)));
      if (direct) {
        // smat's implicit Ekman pumping and Coriolis in iP (smat_imp_extra), transposed
        const double ce = I.CorFac * ekpump[i];
        usb = csub(usb, cscale(ce, csub(cscale(ekp_us[i], iPb), cscale(ekp_dusdp[i], cim(dm, iPb)))));
        upb = caxpy(-ce * ekp_up[i], iPb, upb);
        omb = caxpy(-ce, iPb, omb);
        if (I.flags & PZF_COR_IMP) usb = caxpy(I.CorFac * beta[i], iPb, usb);
      }
    }
    if (src && a.objective == PZ_OBJ_EKIN3D) {
      // d(us2_3D + up2_3D + uz2_3D)/d(us, up) of the state, averaged
      const double W1 = pi * wint[i] * (rr[i] * h[i] + beta[i] * beta[i] * rr[i] * h[i] * h[i] * h[i] / 12.0);
      const double W2 = pi * wint[i] * rr[i] * h[i];
      const double2 us = A.snap(slot, SN_US, mi)[i], up = A.snap(slot, SN_UP, mi)[i];
      if (m != 0) {
        usb = caxpy(4.0 * W1 * a.inv_window, us, usb);
        upb = caxpy(4.0 * W2 * a.inv_window, up, upb);
      } else {
        usb.x += 2.0 * W1 * a.inv_window * us.x;
        upb.x += 2.0 * W2 * a.inv_window * up.x;
      }
    }
    // L^T: temperature, vorticity / u_phi, streamfunction
    v[1][i] = cscale(TdF, iTb);
    v[2][i] = cscale(TdF * or1[i], iTb);
    if (m != 0) {
      double2 Tt = caxpy(-TdF * dm2 * or2[i], iTb, Tb);
      if (buo_imp) Tt = cadd(Tt, cscale(I.BuoFac * rgrav[i] * or1[i], cim(dm, iPb)));
      v[0][i] = Tt;
      omb = cadd(omb, oldPb);
      v[3][i] = caxpy(-Vis * dm2 * or2[i], iPb, omb);
      v[4][i] = cscale(Vis, iPb);
      v[5][i] = cscale(Vis * or1[i], iPb);
      // us = (i m / r) psi, up = -dpsi/dr - beta psi
      v[6][i] = csub(cscale(-or1[i], cim(dm, usb)), cscale(beta[i], upb));
      v[7][i] = upb;
    } else {
      v[0][i] = Tb;
      // up(0) = u, om(0) = du/dr + u/r, old = u,
      // iP(0) = Vis (u'' + u'/r - u/r^2) - CorFac ekpump u
      const double u0b = upb.x + oldPb.x + or1[i] * omb.x + (-Vis * or2[i] - I.CorFac * ekpump[i]) * iPb.x;
      v[3][i] = make_double2(u0b, 0.0);
      v[4][i] = make_double2(Vis * iPb.x, 0.0);
      v[5][i] = make_double2(omb.x + Vis * or1[i] * iPb.x, 0.0);
    }
  }
  __syncthreads();
  double2 *t0 = v[8], *t1 = v[9], *t2 = v[10];
  // Tc_bar = C^T Tt + D2c^T (TdF iT_bar) + D1c^T (TdF/r iT_bar)
  op_CT(V, N, v[0], t0, s.w);
  __syncthreads();
  op_D2cT(V, N, v[1], t1, s.w);
  __syncthreads();
  op_D1cT(V, N, v[2], t2, s.w);
  __syncthreads();
  {
    // NuTop source: d/dTc of dT/dr(m=0, r_cmb) / dtcond(r_cmb) = D1c(0, k) / dtcond(0)
    const bool nu = src && a.objective == PZ_OBJ_NUTOP && m == 0;
    const double cnu = nu ? a.inv_window / V.rad(RV_DTCOND)[0] : 0.0;
    const double* d1c = V.basis(BM_D1C);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      double2 v = cadd(t0[i], cadd(t1[i], t2[i]));
      if (nu) v.x += cnu * d1c[(long long)i * N];
      A.plane(AP_TCB, mi)[i] = v;
    }
  }
  __syncthreads();
  op_CT(V, N, v[3], t0, s.w);
  __syncthreads();
  op_D2cT(V, N, v[4], t1, s.w);
  __syncthreads();
  op_D1cT(V, N, v[5], t2, s.w);
  __syncthreads();
  if (m != 0) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_OCB, mi)[i] = cadd(t0[i], cadd(t1[i], t2[i]));
    __syncthreads();
    op_CT(V, N, v[6], t0, s.w);
    __syncthreads();
    op_D1cT(V, N, v[7], t1, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_PCB, mi)[i] = csub(t0[i], t1[i]);
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      A.plane(AP_UCB, 0)[i] = make_double2(t0[i].x + t1[i].x + t2[i].x, 0.0);
      A.plane(AP_OCB, 0)[i] = cz();
      A.plane(AP_PCB, 0)[i] = cz();
    }
  }
}

// ---------------------------------------------------------------------------
// DIRK sweep (the stage loop of time_loop, step_time.f90:210-384, with the
// tableaux of dirk_schemes.f90).  A step has the stage states z_0 = S_n and
// z_s (s = 1..S', the solutions of the solved stages) with
//   E_k   = FIN(NL(z_k))                        explicit term of stage k+1
//   I_k   = L(z_k)                              implicit term (l_imp_calc_rhs)
//   rhs_s = old + dt sum_{k<s} (bex[s][k] E_k + bim[s][k] I_k),   z_s = SOLVE(rhs_s)
//   S_{n+1} = ASSEMBLE(old + dt sum_k (bae[k] E_k + bai[k] I_k))  (assembly
//   schemes, update_temp_coll.f90:238-307, update_psi_coll_dmat.f90:684-827),
//   else S_{n+1} = z_S
// where old = (T, om) of z_0 (u_phi for m = 0).  Between steps the sweep
// carries lambda, the adjoint of the physical fields (T, us, up, om) of the
// state; the adjoints of old, E_k and I_k of the current step live in the
// DP_ planes.  The stage-state fields are snapshots (s1 per step).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dirk_w(const PzInst& I, const double* pool, int table, int row, int k) {
  return pool[I.o_bt + table + row * PZ_BT_LD + k];
}

// objective source of state `slot`: d J / d (T, us, up) of the physical fields
__device__ __forceinline__ void dadj_source(const PzAdjDev& a, const AdjView& A, const View& V, int mi, int slot,
                                            int i, double2& Tb, double2& usb, double2& upb) {
  const PzInst& I = *V.I;
  if (a.objective == PZ_OBJ_NUTOP) {
    // NuTop = 1 + dT/dr(m=0, r_cmb) / dtcond(r_cmb), dT/dr = D1p T (imp_from_physical)
    if (mi == 0) Tb.x += a.inv_window / V.rad(RV_DTCOND)[0] * V.basis(BM_D1P)[(long long)i * I.N];
    return;
  }
  const double pi = 3.14159265358979323846;
  const double* rr = V.rad(RV_R);
  const double* h = V.rad(RV_HEIGHT);
  const double* beta = V.rad(RV_BETA);
  const double* wint = V.rad(RV_WINT);
  if (I.flags & PZF_NON_ROT) return;
  const double W1 = pi * wint[i] * (rr[i] * h[i] + beta[i] * beta[i] * rr[i] * h[i] * h[i] * h[i] / 12.0);
  const double W2 = pi * wint[i] * rr[i] * h[i];
  const double2 us = A.snap(slot, SN_US, mi)[i], up = A.snap(slot, SN_UP, mi)[i];
  if (mi != 0) {
    usb = caxpy(4.0 * W1 * a.inv_window, us, usb);
    upb = caxpy(4.0 * W2 * a.inv_window, up, upb);
  } else {
    usb.x += 2.0 * W1 * a.inv_window * us.x;
    upb.x += 2.0 * W2 * a.inv_window * up.x;
  }
}

// FIN^T, pointwise part (update_temp_coll.f90:152-176, update_psi_coll_dmat.f90:468-552):
// adds the adjoint of the explicit term (eT, eP) to the field adjoints
__device__ __forceinline__ void dadj_fin_pointwise(const PzInst& I, const View& V, int i, int m, double2 eT,
                                                   double2 eP, double2& Tb, double2& usb, double2& upb,
                                                   double2& omb) {
  const double dm = (double)m;
  const double* beta = V.rad(RV_BETA);
  const double gT = V.rad(RV_DTCOND)[i] - I.tadvz * beta[i] * V.rad(RV_TCOND)[i];
  usb = caxpy(-gT, eT, usb);
  if (m != 0) {
    if (!(I.flags & PZF_NON_ROT)) usb = caxpy(I.CorFac * beta[i], eP, usb);
    if (I.flags & PZF_EK_PUMP) {
      const double ce = I.CorFac * V.rad(RV_EKPUMP)[i];
      usb = csub(usb, cscale(ce, csub(cscale(V.rad(RV_EKP_US)[i], eP), cscale(V.rad(RV_EKP_DUSDP)[i], cim(dm, eP)))));
      upb = caxpy(-ce * V.rad(RV_EKP_UP)[i], eP, upb);
      omb = caxpy(-ce, eP, omb);
    }
    if (!(I.flags & PZF_BUO_IMP)) Tb = cadd(Tb, cscale(I.BuoFac * V.rad(RV_RGRAV)[i] * V.rad(RV_OR1)[i], cim(dm, eP)));
  }
}

__device__ void dadj_fin_body(const PzAdjDev& a, const AdjView& A, const View& V, int mi, int k, int slot, AS& s);

// lambda at the final state: the objective source (zero outside the window)
__global__ void k_dadj_term(PzAdjDev a, int slot, int src) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const PzInst& I = a.d.inst[it.inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, it.inst);
  const int mi = it.idx;
  for (int i = threadIdx.x; i < I.N; i += blockDim.x) {
    double2 Tb = cz(), usb = cz(), upb = cz();
    if (src) dadj_source(a, A, V, mi, slot, i, Tb, usb, upb);
    A.plane(DP_LT, mi)[i] = Tb;
    A.plane(DP_LUS, mi)[i] = usb;
    A.plane(DP_LUP, mi)[i] = upb;
    A.plane(DP_LOM, mi)[i] = cz();
  }
}

// ASSEMBLE^T (assembly schemes), or zero (the others): lambda of S_{n+1} ->
// adjoints of old, E_k, I_k.  The assembly sets T = assembled values at the
// interior radii (robin_bc: zero on the walls), psi = G_ass w (interior rows
// 2..N-3) and us, up, om from psi; for m = 0 u_phi = Re w at the interior
// radii and om = du/dr + u/r.
__global__ void __launch_bounds__(256) k_dadj_ass(PzAdjDev a, int n, int fin_k, int fin_slot) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx, m = mi * I.minc, ns = a.ns;
  const double dm = (double)m, dm2 = dm * dm;
  AS s = as_smem(N);
  double2 *wT = s.v[0], *wP = s.v[1], *v0 = s.v[2], *v1 = s.v[3], *v2 = s.v[4], *t0 = s.v[5], *t1 = s.v[6],
          *t2 = s.v[7], *pc = s.v[8];
  if (!a.assembly) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      A.plane(DP_OT, mi)[i] = cz();
      A.plane(DP_OP, mi)[i] = cz();
      for (int k = 0; k < ns; ++k)
        for (int f = 0; f < 2; ++f) { A.dE(k, f, mi)[i] = cz(); A.dI(ns, k, f, mi)[i] = cz(); }
    }
    if (fin_k >= 0) dadj_fin_body(a, A, V, mi, fin_k, fin_slot, s);
    return;
  }
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
  const double* dbeta = V.rad(RV_DBETA);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 tb = A.plane(DP_LT, mi)[i];
    if (mi == 0) tb.y = 0.0;
    wT[i] = (i == 0 || i == N - 1) ? cz() : tb;
    const double2 usb = A.plane(DP_LUS, mi)[i], upb = A.plane(DP_LUP, mi)[i], omb = A.plane(DP_LOM, mi)[i];
    if (m != 0) {
      // us = (i m / r) psi, up = -dpsi - beta psi, om = -(d2psi + c1 dpsi + c0 psi)
      const double c1 = or1[i] + beta[i], c0 = or1[i] * beta[i] + dbeta[i] - dm2 * or2[i];
      v0[i] = csub(csub(cscale(-or1[i], cim(dm, usb)), cscale(beta[i], upb)), cscale(c0, omb));
      v1[i] = cscale(-1.0, caxpy(c1, omb, upb));
      v2[i] = cscale(-1.0, omb);
    } else {
      v0[i] = omb;      // om = D1p u + u/r: D1p^T below
      v1[i] = make_double2(upb.x + or1[i] * omb.x, 0.0);
    }
  }
  __syncthreads();
  if (m != 0) {
    op_CT(V, N, v0, t0, s.w);
    __syncthreads();
    op_D1cT(V, N, v1, t1, s.w);
    __syncthreads();
    op_D2cT(V, N, v2, t2, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) pc[i] = cadd(t0[i], cadd(t1[i], t2[i]));
    __syncthreads();
    mvT_lanes(a.d.pool + I.o_gass + (long long)mi * N * N, N, pc, wP);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      if (i < 2 || i > N - 3) wP[i] = cz();
  } else {
    op_D1pT(V, N, v0, t0, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      wP[i] = (i == 0 || i == N - 1) ? cz() : make_double2(v1[i].x + t0[i].x, 0.0);
  }
  __syncthreads();
  const PzState& S = a.rec[(long long)inst * a.n_steps + n];
  const double dt = S.dt[0];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 rt = wT[i], rp = wP[i];
    A.plane(DP_OT, mi)[i] = rt;
    A.plane(DP_OP, mi)[i] = rp;
    for (int k = 0; k < ns; ++k) {
      const double we = dt * dirk_w(I, a.d.pool, PZ_BT_AEXP, 0, k), wi = dt * dirk_w(I, a.d.pool, PZ_BT_AIMP, 0, k);
      A.dE(k, 0, mi)[i] = cscale(we, rt);
      A.dE(k, 1, mi)[i] = cscale(we, rp);
      A.dI(ns, k, 0, mi)[i] = cscale(wi, rt);
      A.dI(ns, k, 1, mi)[i] = cscale(wi, rp);
    }
  }
  if (fin_k >= 0) dadj_fin_body(a, A, V, mi, fin_k, fin_slot, s);
}

// FIN^T, the D1p part, for the explicit term of stage state k (snapshot
// `slot`): the inputs of k_adj_rloop (adjoints of E, dVsT, dVsOm), and the
// explicit buoyancy's share of dJ/dBuoFac.  Runs in the block of (instance,
// m) after the last contribution to E_k's adjoint (stages > k, assembly).
__device__ void dadj_fin_body(const PzAdjDev& a, const AdjView& A, const View& V, int mi, int k, int slot, AS& s) {
  const PzInst& I = *V.I;
  const int N = I.N, m = mi * I.minc;
  const double dm = (double)m;
  const double* or1 = V.rad(RV_OR1);
  const double* rgrav = V.rad(RV_RGRAV);
  double2 *x = s.v[0], *y = s.v[1], *t = s.v[2];
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 et = A.dE(k, 0, mi)[i], ep = A.dE(k, 1, mi)[i];
    A.plane(AP_ETB, mi)[i] = et;
    A.plane(AP_EPB, mi)[i] = ep;
    x[i] = cscale(-or1[i], et);
    y[i] = cscale(-or1[i], ep);
  }
  __syncthreads();
  op_D1pT(V, N, x, t, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VTB, mi)[i] = t[i];
  __syncthreads();
  if (m != 0) {
    op_D1pT(V, N, y, t, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VOB, mi)[i] = t[i];
    if (!(I.flags & PZF_BUO_IMP)) {
      const double2* Tk = A.snap(slot, SN_T, mi);
      double acc = 0.0;
      for (int i = threadIdx.x; i < N; i += blockDim.x)
        acc += cdotr(A.dE(k, 1, mi)[i], cscale(-rgrav[i] * or1[i], cim(dm, Tk[i])));
      acc = block_sum(acc, s.red);
      if (threadIdx.x == 0) A.db()[mi] += acc;
    }
  } else {
    for (int i = threadIdx.x; i < N; i += blockDim.x) A.plane(AP_VOB, mi)[i] = cz();
  }
}

// Stage s (solved, snapshot `slot` holds z_s): the field adjoint of z_s
// (lambda when z_s is S_{n+1}, the explicit term E_s through FIN^T and NL^T
// when it is used), the implicit term I_s -> adjoint of the Chebyshev
// solution (L^T, as k_adj_lin) -> SOLVE^T (as k_adj_solve) -> adjoint of
// the right-hand side, added to old, E_k and I_k (k < s) with the stage's
// Butcher weights.
__global__ void __launch_bounds__(256, 4) k_dadj_stage(PzAdjDev a, int n, int st, int slot, int e_used,
                                                        int fin_prev) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const PzState& S = a.rec[(long long)inst * a.n_steps + n];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx, m = mi * I.minc, ns = a.ns;
  const double dm = (double)m, dm2 = dm * dm;
  AS s = as_smem(N);
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  const bool last = !a.assembly && st == ns;            // z_s is S_{n+1}
  const bool has_imp = !last && ((a.imp_mask >> st) & 1);  // I_s in impl slot s
  const double TdF = I.TdiffFac, Vis = I.ViscFac;
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* beta = V.rad(RV_BETA);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* ekpump = V.rad(RV_EKPUMP);
  double2** v = s.v;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 Tb = cz(), usb = cz(), upb = cz(), omb = cz();
    if (last) {
      Tb = A.plane(DP_LT, mi)[i]; usb = A.plane(DP_LUS, mi)[i];
      upb = A.plane(DP_LUP, mi)[i]; omb = A.plane(DP_LOM, mi)[i];
    }
    if (e_used) {
      Tb = cadd(Tb, A.plane(AP_AT, mi)[i]); usb = cadd(usb, A.plane(AP_AUS, mi)[i]);
      upb = cadd(upb, A.plane(AP_AUP, mi)[i]); omb = cadd(omb, A.plane(AP_AOM, mi)[i]);
      dadj_fin_pointwise(I, V, i, m, A.dE(st, 0, mi)[i], A.dE(st, 1, mi)[i], Tb, usb, upb, omb);
    }
    const double2 iTb = has_imp ? A.dI(ns, st, 0, mi)[i] : cz();
    const double2 iPb = has_imp ? A.dI(ns, st, 1, mi)[i] : cz();
    v[1][i] = cscale(TdF, iTb);
    v[2][i] = cscale(TdF * or1[i], iTb);
    if (m != 0) {
      double2 Tt = caxpy(-TdF * dm2 * or2[i], iTb, Tb);
      if (buo_imp) Tt = cadd(Tt, cscale(I.BuoFac * rgrav[i] * or1[i], cim(dm, iPb)));
      v[0][i] = Tt;
      v[3][i] = caxpy(-Vis * dm2 * or2[i], iPb, omb);
      v[4][i] = cscale(Vis, iPb);
      v[5][i] = cscale(Vis * or1[i], iPb);
      v[6][i] = csub(cscale(-or1[i], cim(dm, usb)), cscale(beta[i], upb));
      v[7][i] = upb;
    } else {
      v[0][i] = Tb;
      const double u0b = upb.x + or1[i] * omb.x + (-Vis * or2[i] - I.CorFac * ekpump[i]) * iPb.x;
      v[3][i] = make_double2(u0b, 0.0);
      v[4][i] = make_double2(Vis * iPb.x, 0.0);
      v[5][i] = make_double2(omb.x + Vis * or1[i] * iPb.x, 0.0);
    }
  }
  __syncthreads();
  // L^T: Tc (v11), om_c or u_c (v0), psi_c (v1)
  double2 *t0 = v[8], *t1 = v[9], *t2 = v[10], *Tc = v[11];
  op_CT(V, N, v[0], t0, s.w);
  __syncthreads();
  op_D2cT(V, N, v[1], t1, s.w);
  __syncthreads();
  op_D1cT(V, N, v[2], t2, s.w);
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) Tc[i] = cadd(t0[i], cadd(t1[i], t2[i]));
  __syncthreads();
  op_CT(V, N, v[3], t0, s.w);
  __syncthreads();
  op_D2cT(V, N, v[4], t1, s.w);
  __syncthreads();
  op_D1cT(V, N, v[5], t2, s.w);
  __syncthreads();
  double2 *oc = v[0], *pc = v[1];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 o = cadd(t0[i], cadd(t1[i], t2[i]));
    oc[i] = (m == 0) ? make_double2(o.x, 0.0) : o;
  }
  __syncthreads();
  if (m != 0) {
    op_CT(V, N, v[6], t0, s.w);
    __syncthreads();
    op_D1cT(V, N, v[7], t1, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) pc[i] = csub(t0[i], t1[i]);
    __syncthreads();
  }
  // SOLVE^T (update_temp_co, update_om_coll_dmat), transposed as in k_adj_solve
  const double wl0 = S.wimp_lin[0];
  double2 *x = v[2], *y = v[3], *rT = v[4], *rP = v[5];
  if (m != 0) {
    const long long MN = (long long)I.M * N;
    const double* aux = a.d.pool + I.o_aux;
    const double* om2 = aux + 0 * MN + (long long)mi * N;
    const double* om3 = aux + 1 * MN + (long long)mi * N;
    const double* psi2 = aux + 2 * MN + (long long)mi * N;
    const double* psi3 = aux + 3 * MN + (long long)mi * N;
    const double* infl = aux + 4 * MN + 4LL * mi;
    const double* bct = V.rad(RV_BCTOP);
    const double* bcb = V.rad(RV_BCBOT);
    double c1r = 0.0, c1i = 0.0, c2r = 0.0, c2i = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      c1r += psi2[i] * pc[i].x + om2[i] * oc[i].x;
      c1i += psi2[i] * pc[i].y + om2[i] * oc[i].y;
      c2r += psi3[i] * pc[i].x + om3[i] * oc[i].x;
      c2i += psi3[i] * pc[i].y + om3[i] * oc[i].y;
    }
    c1r = block_sum(c1r, s.red); c1i = block_sum(c1i, s.red);
    c2r = block_sum(c2r, s.red); c2i = block_sum(c2i, s.red);
    const double ttr = -infl[0] * c1r - infl[2] * c2r, tti = -infl[0] * c1i - infl[2] * c2i;
    const double tbr = -infl[1] * c1r - infl[3] * c2r, tbi = -infl[1] * c1i - infl[3] * c2i;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      x[i] = make_double2(pc[i].x + ttr * bct[i] + tbr * bcb[i], pc[i].y + tti * bct[i] + tbi * bcb[i]);
    __syncthreads();
    mvT_lanes(a.d.pool + I.o_gpsi + (long long)mi * N * N, N, x, y);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = csub(oc[i], y[i]);
    __syncthreads();
    mvT_lanes(a.d.pool + I.o_gom + (long long)mi * N * N, N, x, rP);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      if (i == 0 || i == N - 1) rP[i] = cz();
      x[i] = buo_imp ? cscale(wl0 * I.BuoFac * rgrav[i] * or1[i], cim(dm, rP[i])) : cz();
    }
    __syncthreads();
    if (buo_imp) {
      op_CT(V, N, x, y, s.w);
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += blockDim.x) Tc[i] = cadd(Tc[i], y[i]);
      __syncthreads();
    }
  } else {
    mvT_lanes(a.d.pool + I.o_guphi, N, oc, rP);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x)
      if (i == 0 || i == N - 1) rP[i] = cz(); else rP[i].y = 0.0;
    __syncthreads();
  }
  const double* GT = ((I.flags & PZF_T_IS_OM) && m != 0) ? a.d.pool + I.o_gom + (long long)mi * N * N
                                                         : a.d.pool + I.o_gt + (long long)mi * N * N;
  mvT_lanes(GT, N, Tc, rT);
  __syncthreads();
  // distribute the right-hand side's adjoint (dirk_rhs)
  const double dt = S.dt[0];
  const double2* Ts = A.snap(slot, SN_T, mi);
  double acc = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 rt = (i == 0 || i == N - 1) ? cz() : rT[i];
    const double2 rp = rP[i];
    A.plane(DP_OT, mi)[i] = cadd(A.plane(DP_OT, mi)[i], rt);
    A.plane(DP_OP, mi)[i] = cadd(A.plane(DP_OP, mi)[i], rp);
    for (int k = 0; k < st; ++k) {
      const double we = dt * dirk_w(I, a.d.pool, PZ_BT_EXP, st, k), wi = dt * dirk_w(I, a.d.pool, PZ_BT_IMP, st, k);
      if (we != 0.0) {
        A.dE(k, 0, mi)[i] = caxpy(we, rt, A.dE(k, 0, mi)[i]);
        A.dE(k, 1, mi)[i] = caxpy(we, rp, A.dE(k, 1, mi)[i]);
      }
      if (wi != 0.0) {
        A.dI(ns, k, 0, mi)[i] = caxpy(wi, rt, A.dI(ns, k, 0, mi)[i]);
        A.dI(ns, k, 1, mi)[i] = caxpy(wi, rp, A.dI(ns, k, 1, mi)[i]);
      }
    }
    if (m != 0 && buo_imp) {
      // buoyancy of the new temperature in this solve, and in I_s
      const double c = rgrav[i] * or1[i];
      acc += cdotr(rp, cscale(-wl0 * c, cim(dm, Ts[i])));
      if (has_imp) acc += cdotr(A.dI(ns, st, 1, mi)[i], cscale(-c, cim(dm, Ts[i])));
    }
  }
  acc = block_sum(acc, s.red);
  if (threadIdx.x == 0) A.db()[mi] += acc;
  // E_{st-1} is complete now (its consumers are the stages >= st and the assembly)
  if (fin_prev) dadj_fin_body(a, A, V, mi, st - 1, slot - 1, s);
}

// z_0 = S_n (snapshot `slot`): lambda_n from old, I_0 (imp_from_physical,
// D2p = D2c C), E_0 (FIN^T after k_adj_rloop) and the objective source
__global__ void __launch_bounds__(256, 3) k_dadj_z0(PzAdjDev a, int slot, int src) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx, m = mi * I.minc, ns = a.ns;
  const double dm = (double)m, dm2 = dm * dm;
  AS s = as_smem(N);
  const bool buo_imp = (I.flags & PZF_BUO_IMP) != 0;
  const bool has_imp = (a.imp_mask & 1) != 0;
  const double TdF = I.TdiffFac, Vis = I.ViscFac;
  const double* or1 = V.rad(RV_OR1);
  const double* or2 = V.rad(RV_OR2);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* ekpump = V.rad(RV_EKPUMP);
  double2 *Tb = s.v[0], *usb = s.v[1], *upb = s.v[2], *omb = s.v[3];
  double2 *aT = s.v[4], *bT = s.v[5], *aP = s.v[6], *bP = s.v[7], *t0 = s.v[8], *t1 = s.v[9];
  const double2* T0 = A.snap(slot, SN_T, mi);
  double acc = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 tb = cadd(A.plane(DP_OT, mi)[i], A.plane(AP_AT, mi)[i]);
    double2 ub = A.plane(AP_AUS, mi)[i], pb = A.plane(AP_AUP, mi)[i], ob = A.plane(AP_AOM, mi)[i];
    const double2 op = A.plane(DP_OP, mi)[i];
    if (m != 0) ob = cadd(ob, op);
    else pb.x += op.x;
    dadj_fin_pointwise(I, V, i, m, A.dE(0, 0, mi)[i], A.dE(0, 1, mi)[i], tb, ub, pb, ob);
    if (src) dadj_source(a, A, V, mi, slot, i, tb, ub, pb);
    const double2 iTb = has_imp ? A.dI(ns, 0, 0, mi)[i] : cz();
    const double2 iPb = has_imp ? A.dI(ns, 0, 1, mi)[i] : cz();
    tb = caxpy(-TdF * dm2 * or2[i], iTb, tb);
    aT[i] = cscale(TdF, iTb);
    bT[i] = cscale(TdF * or1[i], iTb);
    if (m != 0) {
      ob = caxpy(-Vis * dm2 * or2[i], iPb, ob);
      if (buo_imp) {
        const double c = rgrav[i] * or1[i];
        tb = cadd(tb, cscale(I.BuoFac * c, cim(dm, iPb)));
        acc += cdotr(iPb, cscale(-c, cim(dm, T0[i])));
      }
      aP[i] = cscale(Vis, iPb);
      bP[i] = cscale(Vis * or1[i], iPb);
    } else {
      pb.x += (-Vis * or2[i] - I.CorFac * ekpump[i]) * iPb.x;
      aP[i] = make_double2(Vis * iPb.x, 0.0);
      bP[i] = make_double2(Vis * or1[i] * iPb.x, 0.0);
    }
    Tb[i] = tb; usb[i] = ub; upb[i] = pb; omb[i] = ob;
  }
  acc = block_sum(acc, s.red);
  if (threadIdx.x == 0) A.db()[mi] += acc;
  __syncthreads();
  if (has_imp) {
    // T: D2p^T (TdF iT) + D1p^T (TdF/r iT)
    op_D2cT(V, N, aT, t0, s.w);
    __syncthreads();
    op_CT(V, N, t0, t1, s.w);
    __syncthreads();
    op_D1pT(V, N, bT, t0, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) Tb[i] = cadd(Tb[i], cadd(t0[i], t1[i]));
    __syncthreads();
    op_D2cT(V, N, aP, t0, s.w);
    __syncthreads();
    op_CT(V, N, t0, t1, s.w);
    __syncthreads();
    op_D1pT(V, N, bP, t0, s.w);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const double2 d = cadd(t0[i], t1[i]);
      if (m != 0) omb[i] = cadd(omb[i], d);
      else upb[i].x += d.x;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 tb = Tb[i];
    if (m == 0) tb.y = 0.0;
    A.plane(DP_LT, mi)[i] = tb;
    A.plane(DP_LUS, mi)[i] = (m == 0) ? cz() : usb[i];
    A.plane(DP_LUP, mi)[i] = (m == 0) ? make_double2(upb[i].x, 0.0) : upb[i];
    A.plane(DP_LOM, mi)[i] = (m == 0) ? make_double2(omb[i].x, 0.0) : omb[i];
  }
}

// dJ/dT0 of the DIRK sweep: lambda_0's temperature (the start state is physical)
__global__ void k_dadj_out(PzAdjDev a) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const AdjView A = adj_view(a, inst);
  const int mi = it.idx;
  double2* out = reinterpret_cast<double2*>(a.out + a.o_out[inst]);
  for (int i = threadIdx.x; i < I.N; i += blockDim.x) out[mi + (long long)i * I.M] = A.plane(DP_LT, mi)[i];
}

// dJ/dT0 = C^T Tc_bar(0), in the ABI layout (m fastest)
__global__ void __launch_bounds__(256) k_adj_out(PzAdjDev a) {
  const PzItem it = a.d.mitems[blockIdx.x];
  const int inst = it.inst;
  const PzInst& I = a.d.inst[inst];
  const View V{&I, a.d.pool};
  const AdjView A = adj_view(a, inst);
  const int N = I.N, mi = it.idx;
  AS s = as_smem(N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) s.v[0][i] = A.plane(AP_TCB, mi)[i];
  __syncthreads();
  op_CT(V, N, s.v[0], s.v[1], s.w);
  __syncthreads();
  double2* out = reinterpret_cast<double2*>(a.out + a.o_out[inst]);
  for (int i = threadIdx.x; i < N; i += blockDim.x) out[mi + (long long)i * I.M] = s.v[1][i];
}

// dJ/dBuoFac per instance (sum over m in a fixed order)
__global__ void k_adj_db(PzAdjDev a, double* out) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= a.d.n_inst) return;
  const AdjView A = adj_view(a, inst);
  const double* db = A.db();
  double acc = 0.0;
  for (int mi = 0; mi < a.d.inst[inst].M; ++mi) acc += db[mi];
  out[inst] = acc;
}

}  // namespace

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
struct PzAdjoint {
  int n_steps = 0, K = 0, n_seg = 0, n_window = 0, n_snap = 0, n_ck = 0, ck_planes = 0, objective = 0;
  int snap0 = AP_SNAP;       // first snapshot plane
  int dirk = 0, ns = 1, s1 = 1, assembly = 0, exp_mask = 1, imp_mask = 1;   // DIRK sweep
  bool ready = false;        // a forward sweep is stored
  bool last_valid = false;   // snapshots of the last segment are those of the forward sweep
  double* ws = nullptr;
  long long* d_ows = nullptr;
  long long* d_oout = nullptr;
  PzState* d_rec = nullptr;
  PzState* d_ck = nullptr;
  PzState* d_bstate = nullptr;
  double* d_dt = nullptr;
  double* d_J = nullptr;
  double* d_out = nullptr;
  double2* gs = nullptr;     // grid snapshots (PzAdjDev::gs)
  long long* d_ogs = nullptr;
  bool grids = false;        // the current sweep keeps grid snapshots
  size_t cap_ws = 0, cap_out = 0, cap_ows = 0, cap_oout = 0, cap_rec = 0, cap_ck = 0, cap_b = 0, cap_dt = 0, cap_J = 0;
  size_t cap_gs = 0, cap_ogs = 0;
  size_t rsmem = 0, rsmem_g = 0;   // dynamic shared memory of k_adj_rloop without / with grids
  size_t out_doubles = 0;    // gradient output of the current layout
  std::vector<PzState> h_rec;
};

void pz_adjoint_free(pz_handle* h) {
  if (!h || !h->adj) return;
  PzAdjoint* A = h->adj;
  cudaFree(A->ws); cudaFree(A->d_ows); cudaFree(A->d_oout); cudaFree(A->d_rec); cudaFree(A->d_ck);
  cudaFree(A->d_bstate); cudaFree(A->d_dt); cudaFree(A->d_J); cudaFree(A->d_out);
  cudaFree(A->gs); cudaFree(A->d_ogs);
  delete A;
  h->adj = nullptr;
}

void pz_adjoint_invalidate(pz_handle* h) {
  if (h && h->adj) h->adj->ready = false;
}

namespace {

int acuda(pz_handle* h, cudaError_t e, const char* what) {
  return pz_fail(h, PZ_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

PzAdjDev adj_dev(pz_handle* h) {
  PzAdjoint* A = h->adj;
  PzAdjDev a{};
  a.d = h->dev;
  a.ws = A->ws;
  a.o_ws = A->d_ows;
  a.rec = A->d_rec;
  a.ck_state = A->d_ck;
  a.bstate = A->d_bstate;
  a.J = A->d_J;
  a.out = A->d_out;
  a.o_out = A->d_oout;
  a.n_steps = A->n_steps;
  a.n_snap = A->n_snap;
  a.n_ck = A->n_ck;
  a.ck_planes = A->ck_planes;
  a.win0 = A->n_steps - A->n_window + 1;
  a.inv_window = A->n_window > 0 ? 1.0 / A->n_window : 0.0;
  a.objective = A->objective;
  a.snap0 = A->snap0;
  a.dirk = A->dirk;
  a.ns = A->ns;
  a.s1 = A->s1;
  a.assembly = A->assembly;
  a.exp_mask = A->exp_mask;
  a.imp_mask = A->imp_mask;
  a.gs = A->grids ? A->gs : nullptr;
  a.o_gs = A->grids ? A->d_ogs : nullptr;
  return a;
}

cudaError_t launch_snap(const PzAdjDev& a, int slot, cudaStream_t s) {
  k_adj_snap<<<a.d.n_mitems, 64, 0, s>>>(a, slot);
  return cudaGetLastError();
}
cudaError_t launch_ckpt(const PzAdjDev& a, int c, int dir, cudaStream_t s) {
  k_adj_ckpt<<<a.d.n_mitems, 64, 0, s>>>(a, c, dir);
  return cudaGetLastError();
}
// one forward step without the time series: the handle's step plan (the
// kernels of pz_step, with the rebuild fused into the first stage where the
// plan fuses it) without k_obs; for a DIRK scheme the stage states are saved
// to snapshots base + 1 .. base + s1 - 1 after their stages (base >= 0).
// With grid snapshots (a.gs) and gbase >= 0, k_rloop of stage s stores the
// grids of the state it transforms at grid slot gbase + s - 1.
cudaError_t launch_fwd_plan(const pz_handle* h, const std::vector<PzLaunch>& plan, const PzDev& d,
                            const PzAdjDev& a, int base, int gbase, cudaStream_t s) {
  for (const PzLaunch& L : plan) {
    if (L.kind == PZK_OBS) continue;
    cudaError_t e;
    if (L.kind == PZK_RLOOP && gbase >= 0 && a.gs) {
      PzDev dg = d;
      dg.gsnap = a.gs;
      dg.o_gsnap = a.o_gs;
      dg.gsnap_slot0 = gbase;
      e = pz_launch_step_kernel(dg, L.kind, L.stage, s);
    } else {
      e = pz_launch_step_kernel(d, L.kind, L.stage, s);
    }
    if (e) return e;
    if (base >= 0 && (L.kind == PZK_MLOOP || L.kind == PZK_BUILD_MLOOP) && L.stage < a.s1 &&
        (e = launch_snap(a, base + L.stage, s)))
      return e;
  }
  return cudaSuccess;
}
// a multistep step; its state's grids go to grid slot gslot (>= 0).  Handles
// with tensor-core instances step with that stage (the plain step's plan):
// the sweep only needs the states, and the backward sweep rebuilds the dense
// operators it transposes.
cudaError_t launch_fwd(const pz_handle* h, const PzDev& d, const PzAdjDev& a, int gslot, cudaStream_t s) {
  if (h->n_fast > 0) {
    PzDev df = h->fdev;
    df.dt_io = d.dt_io;
    df.rec = d.rec;
    df.sched_n = d.sched_n;
    df.sched_mode = d.sched_mode;
    return launch_fwd_plan(h, h->fplan, df, a, -1, gslot, s);
  }
  return launch_fwd_plan(h, h->plan, d, a, -1, gslot, s);
}

// one forward DIRK step without the time series, with the stage states
// saved to snapshots base .. base + s1 - 1 when base >= 0
cudaError_t launch_fwd_dirk(const pz_handle* h, const PzDev& d, const PzAdjDev& a, int base, cudaStream_t s) {
  cudaError_t e;
  if (base >= 0 && (e = launch_snap(a, base, s))) return e;
  return launch_fwd_plan(h, h->plan, d, a, base, base, s);
}

// NL^T of snapshot `slot`; `grid`: the forward stored the slot's grids
cudaError_t launch_adj_rloop(const pz_handle* h, const PzAdjDev& a, int slot, bool grid, cudaStream_t s) {
  if (grid && a.gs)
    k_adj_rloop<true><<<h->dev.n_ritems, 256, h->adj->rsmem_g, s>>>(a, slot);
  else
    k_adj_rloop<false><<<h->dev.n_ritems, 256, h->adj->rsmem, s>>>(a, slot);
  return cudaGetLastError();
}

template <class T>
cudaError_t grow(T** p, size_t* cap, size_t n) {
  if (*p && *cap >= n) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (!e) *cap = n;
  return e;
}

}  // namespace

extern "C" int pz_adjoint_grid_snapshots(pz_handle* h, int enable) {
  if (!h) return pz_fail(nullptr, PZ_E_ARG, "pz_adjoint_grid_snapshots: null handle");
  h->adj_grids = enable ? 1 : 0;
  if (!enable && h->adj) {
    PzAdjoint* A = h->adj;
    cudaFree(A->gs);
    A->gs = nullptr;
    A->cap_gs = 0;
    A->grids = false;   // a stored sweep's backward transforms its spectral snapshots
  }
  return PZ_OK;
}

extern "C" int pz_set_ra(pz_handle* h, int inst, double ra) {
  if (!h) return pz_fail(nullptr, PZ_E_ARG, "pz_set_ra: null handle");
  if (inst < 0 || inst >= h->n_inst) return pz_fail(h, PZ_E_ARG, "pz_set_ra: instance out of range");
  if (!(ra > 0.0)) return pz_fail(h, PZ_E_ARG, "pz_set_ra: ra must be positive");
  HostInst& hi = h->hin[inst];
  const double buo = ra / hi.c.pr;   // BuoFac = Ra / Pr (namelists.f90, time_scale 'VISC')
  hi.c.ra = ra;
  hi.I.BuoFac = buo;
  h->inst[inst].BuoFac = buo;
  cudaError_t e = cudaMemcpyAsync(&h->d_inst[inst].BuoFac, &h->inst[inst].BuoFac, sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream);
  if (!e) e = cudaStreamSynchronize(h->stream);
  if (e) return acuda(h, e, "pz_set_ra");
  pz_adjoint_invalidate(h);
  return PZ_OK;
}

extern "C" int pz_adjoint_forward(pz_handle* h, int objective, int n_steps, int n_window, int checkpoint_every,
                                  const double* dt_sched, double* J, double* dt_used) {
  if (!h) return pz_fail(nullptr, PZ_E_ARG, "pz_adjoint_forward: null handle");
  if (objective != PZ_OBJ_EKIN3D && objective != PZ_OBJ_NUTOP)
    return pz_fail(h, PZ_E_ARG, "pz_adjoint_forward: unknown objective");
  if (n_steps < 1) return pz_fail(h, PZ_E_ARG, "pz_adjoint_forward: n_steps < 1");
  if (n_window < 0 || n_window > n_steps) return pz_fail(h, PZ_E_ARG, "pz_adjoint_forward: n_window outside [0, n_steps]");
  for (int i = 0; i < h->n_inst; ++i) {
    const PzInst& I = h->inst[i];
    if ((I.flags & (PZF_INTEG | PZF_CHEM)) || (I.dirk && (I.flags & PZF_DIRECT)))
      return pz_fail(h, PZ_E_UNSUPPORTED,
                     "pz_adjoint_forward: the adjoint covers the collocation step with the influence-matrix solve "
                     "(any multistep or DIRK scheme) or with the direct solve (multistep schemes), without "
                     "composition");
    if (I.scheme != h->inst[0].scheme)
      return pz_fail(h, PZ_E_UNSUPPORTED, "pz_adjoint_forward: all instances must use the same time scheme");
    if (adj_rloop_smem_bytes(I.P, I.rg, false) > PZ_SMEM_MAX)
      return pz_fail(h, PZ_E_UNSUPPORTED, "pz_adjoint_forward: n_phi_max too large for the adjoint transform kernel");
  }
  cudaError_t e;
  std::vector<PzState> st(h->n_inst);
  if ((e = cudaMemcpyAsync(st.data(), h->d_state, h->n_inst * sizeof(PzState), cudaMemcpyDeviceToHost, h->stream)) ||
      (e = cudaStreamSynchronize(h->stream)))
    return acuda(h, e, "pz_adjoint_forward");
  for (int i = 0; i < h->n_inst; ++i)
    if (st[i].n_step != 0 || st[i].status != 0)
      return pz_fail(h, PZ_E_ARG, "pz_adjoint_forward: instance " + std::to_string(i) +
                                      " is not at a start state (call pz_set_state first)");
  if (dt_sched)
    for (long long k = 0; k < (long long)h->n_inst * n_steps; ++k)
      if (!(dt_sched[k] > 0.0)) return pz_fail(h, PZ_E_ARG, "pz_adjoint_forward: dt_sched must be positive");

  if (!h->adj) h->adj = new PzAdjoint();
  PzAdjoint* A = h->adj;
  A->ready = false;
  A->objective = objective;
  A->n_steps = n_steps;
  A->n_window = n_window;
  A->K = (checkpoint_every <= 0 || checkpoint_every > n_steps) ? n_steps : checkpoint_every;
  A->n_seg = (n_steps + A->K - 1) / A->K;
  {
    const PzInst& I0 = h->inst[0];
    A->dirk = I0.dirk;
    A->ns = I0.nstages;
    A->assembly = I0.dirk ? I0.assembly : 0;
    A->s1 = I0.dirk ? I0.nstages - A->assembly + 1 : 1;
    A->exp_mask = I0.exp_mask;
    A->imp_mask = I0.imp_mask;
    A->snap0 = I0.dirk ? DP_E + 4 * I0.nstages : AP_SNAP;
    A->ck_planes = F_XI + 2 * (I0.nold + I0.nimp + I0.nexp);
  }
  A->n_snap = A->K * A->s1 + 1;       // stage states of every step of a segment, plus the final state
  A->n_ck = A->n_seg + 1;             // one per segment start, plus the final state
  std::vector<long long> ows(h->n_inst), oout(h->n_inst);
  long long tot = 0, tout = 0;
  const long long planes = A->snap0 + 4LL * A->n_snap + (long long)A->n_ck * A->ck_planes;
  for (int i = 0; i < h->n_inst; ++i) {
    const long long MN = (long long)h->inst[i].M * h->inst[i].N;
    ows[i] = tot;
    tot += planes * 2 * MN;
    oout[i] = tout;
    tout += 2 * MN;
  }
  // buffers grow and are kept for later calls
  if ((e = grow(&A->ws, &A->cap_ws, (size_t)tot)) || (e = grow(&A->d_out, &A->cap_out, (size_t)tout)) ||
      (e = grow(&A->d_ows, &A->cap_ows, (size_t)h->n_inst)) || (e = grow(&A->d_oout, &A->cap_oout, (size_t)h->n_inst)) ||
      (e = grow(&A->d_rec, &A->cap_rec, (size_t)h->n_inst * n_steps)) ||
      (e = grow(&A->d_ck, &A->cap_ck, (size_t)h->n_inst * A->n_ck)) ||
      (e = grow(&A->d_bstate, &A->cap_b, (size_t)h->n_inst)) ||
      (e = grow(&A->d_dt, &A->cap_dt, (size_t)h->n_inst * n_steps)) || (e = grow(&A->d_J, &A->cap_J, (size_t)h->n_inst))) {
    pz_adjoint_free(h);
    return pz_fail(h, PZ_E_NOMEM, std::string("pz_adjoint_forward: device allocation: ") + cudaGetErrorString(e));
  }
  A->out_doubles = (size_t)tout;
  cudaStream_t s = h->stream;
  // grid snapshots: n_snap slots of N x 2P values per instance; a sweep whose
  // grid buffer does not fit runs without them
  A->grids = false;
  if (h->adj_grids) {
    std::vector<long long> ogs(h->n_inst);
    long long tg = 0;
    for (int i = 0; i < h->n_inst; ++i) {
      ogs[i] = tg;
      tg += (long long)A->n_snap * h->inst[i].N * 2 * h->inst[i].P;
    }
    cudaError_t eg = grow(&A->gs, &A->cap_gs, (size_t)tg);
    if (!eg) eg = grow(&A->d_ogs, &A->cap_ogs, (size_t)h->n_inst);
    if (eg == cudaErrorMemoryAllocation) {
      cudaGetLastError();
    } else if (eg) {
      return acuda(h, eg, "pz_adjoint_forward");
    } else {
      if ((e = cudaMemcpyAsync(A->d_ogs, ogs.data(), ogs.size() * sizeof(long long), cudaMemcpyHostToDevice, s)))
        return acuda(h, e, "pz_adjoint_forward");
      A->grids = true;
    }
  }
  if ((e = cudaMemcpyAsync(A->d_ows, ows.data(), ows.size() * sizeof(long long), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(A->d_oout, oout.data(), oout.size() * sizeof(long long), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(A->d_J, 0, h->n_inst * sizeof(double), s)))
    return acuda(h, e, "pz_adjoint_forward");
  if (dt_sched &&
      (e = cudaMemcpyAsync(A->d_dt, dt_sched, (size_t)h->n_inst * n_steps * sizeof(double), cudaMemcpyHostToDevice, s)))
    return acuda(h, e, "pz_adjoint_forward");

  PzAdjDev a = adj_dev(h);
  PzDev dF = h->dev;
  dF.dt_io = A->d_dt;
  dF.rec = A->d_rec;
  dF.sched_n = n_steps;
  dF.sched_mode = dt_sched ? 1 : 2;
  const int k0_last = (A->n_seg - 1) * A->K;
  for (int n = 0; n < n_steps; ++n) {
    if (n % A->K == 0 && (e = launch_ckpt(a, n / A->K, 0, s))) return acuda(h, e, "checkpoint");
    if (A->dirk) {
      if ((e = launch_fwd_dirk(h, dF, a, n >= k0_last ? (n - k0_last) * A->s1 : -1, s))) return acuda(h, e, "forward step");
    } else {
      if (n >= k0_last && (e = launch_snap(a, n - k0_last, s))) return acuda(h, e, "snapshot");
      if ((e = launch_fwd(h, dF, a, n >= k0_last ? n - k0_last : -1, s))) return acuda(h, e, "forward step");
    }
    if (n_window > 0 && n + 1 >= a.win0) {
      k_adj_ke<<<h->n_inst, PZ_THREADS, 0, s>>>(a);
      if ((e = cudaGetLastError())) return acuda(h, e, "objective");
    }
  }
  if ((e = launch_snap(a, (n_steps - k0_last) * A->s1, s)) || (e = launch_ckpt(a, A->n_seg, 0, s)))
    return acuda(h, e, "final state");
  int rc = pz_check_status(h);
  if (rc) return rc;
  A->h_rec.resize((size_t)h->n_inst * n_steps);
  if ((e = cudaMemcpyAsync(A->h_rec.data(), A->d_rec, A->h_rec.size() * sizeof(PzState), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_forward");
  if (J && (e = cudaMemcpyAsync(J, A->d_J, h->n_inst * sizeof(double), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_forward");
  if ((e = cudaStreamSynchronize(s))) return acuda(h, e, "pz_adjoint_forward");
  if (dt_used)
    for (size_t k = 0; k < A->h_rec.size(); ++k) dt_used[k] = A->h_rec[k].dt[0];
  A->ready = true;
  A->last_valid = true;
  return PZ_OK;
}

namespace {
// the backward sweep of a DIRK scheme (see the DIRK kernels above)
int dirk_backward(pz_handle* h, const PzAdjDev& a, const PzDev& dR, const PzDev& dB, int threads, size_t smem,
                  double* dJ_dtemp, double* dJ_dra) {
  PzAdjoint* A = h->adj;
  cudaStream_t s = h->stream;
  cudaError_t e;
  const int n_steps = A->n_steps, K = A->K, s1 = A->s1;
  const int k0_last = (A->n_seg - 1) * K;
  const int mb = h->dev.n_mitems;
  if (!A->last_valid) {
    if ((e = launch_ckpt(a, A->n_seg - 1, 1, s))) return acuda(h, e, "restore");
    for (int n = k0_last; n < n_steps; ++n)
      if ((e = launch_fwd_dirk(h, dR, a, (n - k0_last) * s1, s))) return acuda(h, e, "recompute");
    if ((e = launch_snap(a, (n_steps - k0_last) * s1, s))) return acuda(h, e, "recompute");
  }
  k_dadj_term<<<mb, 64, 0, s>>>(a, (n_steps - k0_last) * s1, A->n_window > 0 ? 1 : 0);
  if ((e = cudaGetLastError())) return acuda(h, e, "adjoint terminal");
  for (int sg = A->n_seg - 1; sg >= 0; --sg) {
    const int k0 = sg * K, k1 = std::min(k0 + K, n_steps);
    if (sg != A->n_seg - 1) {
      if ((e = launch_ckpt(a, sg, 1, s))) return acuda(h, e, "restore");
      for (int n = k0; n < k1; ++n)
        if ((e = launch_fwd_dirk(h, dR, a, (n - k0) * s1, s))) return acuda(h, e, "recompute");
      if ((e = launch_snap(a, (k1 - k0) * s1, s))) return acuda(h, e, "recompute");
    }
    for (int n = k1 - 1; n >= k0; --n) {
      bool rebuild = false;
      if (n < k1 - 1)
        for (int i = 0; i < h->n_inst && !rebuild; ++i) {
          const PzState* r = &A->h_rec[(size_t)i * n_steps];
          rebuild = r[n].wimp_lin[0] != r[n + 1].wimp_lin[0];
        }
      if (rebuild) {
        k_adj_bstate<<<(h->n_inst + 63) / 64, 64, 0, s>>>(a, n);
        if ((e = cudaGetLastError()) || (e = pz_launch_step_kernel(dB, PZK_BUILD, 1, s))) return acuda(h, e, "rebuild");
      }
      // E_k (k = 0..s1-2 are the explicit terms of the stage states; E_k
      // is used when stage k+1 computes it) runs through FIN^T at the end of
      // the kernel that completes its adjoint, then NL^T (k_adj_rloop)
      const int b = (n - k0) * s1;
      auto e_used = [&](int k) { return (k < A->ns && ((A->exp_mask >> k) & 1)) ? 1 : 0; };
      const int top = s1 - 1;   // the last solved stage
      k_dadj_ass<<<mb, threads, smem, s>>>(a, n, (A->assembly && e_used(top)) ? top : -1, b + top);
      for (int st = top; st >= 1; --st) {
        const int eu = (A->assembly || st < top) ? e_used(st) : 0;
        // the grids of stage state st come from k_rloop of stage st + 1,
        // which runs when E_st is used
        if (eu && (e = launch_adj_rloop(h, a, b + st, true, s))) return acuda(h, e, "adjoint step");
        k_dadj_stage<<<mb, threads, smem, s>>>(a, n, st, b + st, eu, e_used(st - 1));
      }
      if ((e = launch_adj_rloop(h, a, b, e_used(0) != 0, s))) return acuda(h, e, "adjoint step");
      k_dadj_z0<<<mb, threads, smem, s>>>(a, b, n >= a.win0 ? 1 : 0);
      if ((e = cudaGetLastError())) return acuda(h, e, "adjoint step");
    }
  }
  A->last_valid = false;
  k_dadj_out<<<mb, 64, 0, s>>>(a);
  k_adj_db<<<(h->n_inst + 63) / 64, 64, 0, s>>>(a, A->d_J);
  if ((e = cudaGetLastError())) return acuda(h, e, "adjoint output");
  if ((e = launch_ckpt(a, A->n_seg, 1, s))) return acuda(h, e, "restore final state");
  std::vector<double> db(h->n_inst);
  std::vector<PzState> bst(h->n_inst);
  if ((e = cudaMemcpyAsync(db.data(), A->d_J, h->n_inst * sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(bst.data(), A->d_bstate, h->n_inst * sizeof(PzState), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_backward");
  if (dJ_dtemp &&
      (e = cudaMemcpyAsync(dJ_dtemp, A->d_out, A->out_doubles * sizeof(double), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_backward");
  if ((e = cudaStreamSynchronize(s))) return acuda(h, e, "pz_adjoint_backward");
  for (int i = 0; i < h->n_inst; ++i)
    if (bst[i].status != 0) return pz_fail(h, bst[i].status, "pz_adjoint_backward: operator rebuild failed");
  int rc = pz_check_status(h);
  if (rc) return rc;
  if (dJ_dra)
    for (int i = 0; i < h->n_inst; ++i) dJ_dra[i] = db[i] / h->hin[i].c.pr;   // dBuoFac/dRa = 1/Pr
  return PZ_OK;
}
}  // namespace

extern "C" int pz_adjoint_backward(pz_handle* h, double* dJ_dtemp, double* dJ_dra) {
  if (!h) return pz_fail(nullptr, PZ_E_ARG, "pz_adjoint_backward: null handle");
  PzAdjoint* A = h->adj;
  if (!A || !A->ready)
    return pz_fail(h, PZ_E_ARG, "pz_adjoint_backward: no forward sweep stored (call pz_adjoint_forward first)");
  cudaStream_t s = h->stream;
  cudaError_t e;
  PzAdjDev a = adj_dev(h);
  PzDev dR = h->dev;          // recompute: prescribed (recorded) dt, nothing recorded
  dR.dt_io = A->d_dt;
  dR.rec = nullptr;
  dR.sched_n = A->n_steps;
  dR.sched_mode = 1;
  PzDev dB = h->dev;          // operator rebuilds of the backward sweep
  dB.state = A->d_bstate;
  const int n_steps = A->n_steps, K = A->K;
  const int k0_last = (A->n_seg - 1) * K;
  const int threads = adj_threads(h->dev.maxN);
  const size_t smem = as_smem_bytes(h->dev.maxN);
  A->rsmem = A->rsmem_g = 0;
  for (int i = 0; i < h->n_inst; ++i) {
    A->rsmem = std::max(A->rsmem, adj_rloop_smem_bytes(h->inst[i].P, h->inst[i].rg, false));
    A->rsmem_g = std::max(A->rsmem_g, adj_rloop_smem_bytes(h->inst[i].P, h->inst[i].rg, true));
  }
  if ((e = cudaFuncSetAttribute(k_adj_rloop<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX)) ||
      (e = cudaFuncSetAttribute(k_adj_rloop<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX)))
    return acuda(h, e, "pz_adjoint_backward");
  k_adj_zero<<<h->dev.n_mitems, 64, 0, s>>>(a);
  if ((e = cudaGetLastError()) || (e = cudaMemsetAsync(A->d_bstate, 0, h->n_inst * sizeof(PzState), s)))
    return acuda(h, e, "adjoint init");
  if (A->dirk) return dirk_backward(h, a, dR, dB, threads, smem, dJ_dtemp, dJ_dra);
  if (!A->last_valid) {
    // snapshots and operators of the last segment were overwritten: recompute
    if ((e = launch_ckpt(a, A->n_seg - 1, 1, s))) return acuda(h, e, "restore");
    for (int n = k0_last; n < n_steps; ++n)
      if ((e = launch_snap(a, n - k0_last, s)) || (e = launch_fwd(h, dR, a, n - k0_last, s)))
        return acuda(h, e, "recompute");
    if ((e = launch_snap(a, n_steps - k0_last, s))) return acuda(h, e, "recompute");
  }
  if (A->n_window > 0) {
    k_adj_lin<<<h->dev.n_mitems, threads, smem, s>>>(a, n_steps, n_steps - k0_last, 1, 1);
    if ((e = cudaGetLastError())) return acuda(h, e, "adjoint terminal");
  }
  for (int sg = A->n_seg - 1; sg >= 0; --sg) {
    const int k0 = sg * K, k1 = std::min(k0 + K, n_steps);
    if (sg != A->n_seg - 1) {
      if ((e = launch_ckpt(a, sg, 1, s))) return acuda(h, e, "restore");
      for (int n = k0; n < k1; ++n)
        if ((e = launch_snap(a, n - k0, s)) || (e = launch_fwd(h, dR, a, n - k0, s))) return acuda(h, e, "recompute");
      if ((e = launch_snap(a, k1 - k0, s))) return acuda(h, e, "recompute");
    }
    for (int n = k1 - 1; n >= k0; --n) {
      // the tensor-core forward builds no dense operators: rebuild them for the
      // segment's last step
      bool rebuild = n == k1 - 1 && h->n_fast > 0;
      if (n < k1 - 1)
        for (int i = 0; i < h->n_inst && !rebuild; ++i) {
          const PzState* r = &A->h_rec[(size_t)i * n_steps];
          rebuild = r[n].wimp_lin[0] != r[n + 1].wimp_lin[0];
        }
      if (rebuild) {
        k_adj_bstate<<<(h->n_inst + 63) / 64, 64, 0, s>>>(a, n);
        if ((e = cudaGetLastError()) || (e = pz_launch_step_kernel(dB, PZK_BUILD, 1, s))) return acuda(h, e, "rebuild");
      }
      const int slot = n - k0;
      k_adj_solve<<<h->dev.n_mitems, threads, smem, s>>>(a, n, slot);
      if ((e = launch_adj_rloop(h, a, slot, true, s))) return acuda(h, e, "adjoint step");
      k_adj_lin<<<h->dev.n_mitems, threads, smem, s>>>(a, n, slot, 0, n >= a.win0 ? 1 : 0);
      if ((e = cudaGetLastError())) return acuda(h, e, "adjoint step");
    }
  }
  A->last_valid = false;
  k_adj_out<<<h->dev.n_mitems, threads, smem, s>>>(a);
  k_adj_db<<<(h->n_inst + 63) / 64, 64, 0, s>>>(a, A->d_J);
  if ((e = cudaGetLastError())) return acuda(h, e, "adjoint output");
  // leave the handle at the final state of the forward sweep
  if ((e = launch_ckpt(a, A->n_seg, 1, s))) return acuda(h, e, "restore final state");
  std::vector<double> db(h->n_inst);
  std::vector<PzState> bst(h->n_inst);
  if ((e = cudaMemcpyAsync(db.data(), A->d_J, h->n_inst * sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(bst.data(), A->d_bstate, h->n_inst * sizeof(PzState), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_backward");
  if (dJ_dtemp &&
      (e = cudaMemcpyAsync(dJ_dtemp, A->d_out, A->out_doubles * sizeof(double), cudaMemcpyDeviceToHost, s)))
    return acuda(h, e, "pz_adjoint_backward");
  if ((e = cudaStreamSynchronize(s))) return acuda(h, e, "pz_adjoint_backward");
  // k_adj_db reused d_J; the objective values are not needed any more
  for (int i = 0; i < h->n_inst; ++i)
    if (bst[i].status != 0) return pz_fail(h, bst[i].status, "pz_adjoint_backward: operator rebuild failed");
  int rc = pz_check_status(h);
  if (rc) return rc;
  if (dJ_dra)
    for (int i = 0; i < h->n_inst; ++i) dJ_dra[i] = db[i] / h->hin[i].c.pr;   // dBuoFac/dRa = 1/Pr
  return PZ_OK;
}

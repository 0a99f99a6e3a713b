// Stage-level entry point: the explicit (nonlinear) terms of one instance
// from caller-owned device arrays in pizza's m-distributed layout.
//
// This is the part of the stage body a Fortran host offloads when it keeps
// its own m-loop: transp_Mloc_to_Rloc, radial_loop, transp_Rloc_to_Mloc and
// finish_explicit_assembly (src/step_time.f90:222-269).  The two kernels pass
// the radial products dVsT and dVsOm (src/radial_loop.f90:350-361) through a
// scratch buffer of 2 * n_m_max * n_r_max complex values.
#include <cuda_runtime.h>

#include <string>

#include "pizza_gpu.h"
#include "pz_device.cuh"
#include "pz_internal.h"
#include "pz_stage.h"

namespace {

// radial_loop for one radius, reading and writing (n_m, n_r) arrays, n_m fastest
__global__ void __launch_bounds__(PZ_THREADS) k_expl_rloop(PzExplArgs a) {
  extern __shared__ double2 sh[];
  __shared__ double red[32];
  const PzInst& I = *a.inst;
  const View V{&I, a.pool};
  const int N = I.N, M = I.M, P = I.P, r = blockIdx.x;
  double2* tw = sh;
  double2* za = sh + P;
  double2* zb = sh + 3 * P;
  const double2* gtw = reinterpret_cast<const double2*>(a.pool + I.o_tw);
  for (int k = threadIdx.x; k < P; k += blockDim.x) tw[k] = gtw[k];
  for (int k = threadIdx.x; k < 2 * P; k += blockDim.x) za[k] = make_double2(0.0, 0.0);
  __syncthreads();
  const double rr = V.rad(RV_R)[r], or1 = V.rad(RV_OR1)[r], beta = V.rad(RV_BETA)[r];
  const double ekpump = V.rad(RV_EKPUMP)[r];
  double usom = 0.0;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const long long o = (long long)r * M + m;
    double2 u = a.us[o], w = a.up[o], c = a.om[o], e = a.temp[o];
    if (m == 0) {
      usom += 0.5 * I.ek * I.CorFac * ekpump * w.x * c.x;   // us_fluct(m=0) * om
      u.y = 0.0; w.y = 0.0; c.y = 0.0; e.y = 0.0;
    } else {
      usom += 2.0 * (u.x * c.x + u.y * c.y);
    }
    za[m] = make_double2(u.x - w.y, u.y + w.x);
    za[P + m] = make_double2(c.x - e.y, c.y + e.x);
    if (m > 0) {
      za[P - m] = make_double2(u.x + w.y, -u.y + w.x);
      za[2 * P - m] = make_double2(c.x + e.y, -c.y + e.x);
    }
  }
  usom = block_sum(usom, red);
  double2* g = fft_run(za, zb, I, tw, 2, true);
  double2* h = (g == za) ? zb : za;
  double vr = 0.0, vh = 0.0;
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    const double2 z1 = g[j], z2 = g[P + j];
    vr = fmax(vr, z1.x * z1.x);
    vh = fmax(vh, z1.y * z1.y);
    h[j] = make_double2(rr * z1.x * z2.y, z1.y * z2.y);
    h[P + j] = make_double2(rr * z1.x * z2.x, z1.y * z2.x);
  }
  vr = block_max(vr, red);
  vh = block_max(vh, red);
  if (threadIdx.x == 0) {
    const double vr2 = I.courfac * I.courfac * vr, vh2 = I.courfac * I.courfac * vh;
    double dtr = 1.0e10, dth = 1.0e10;
    if (vr2 != 0.0) dtr = fmin(dtr, sqrt(V.rad(RV_DELXR2)[r] / vr2));
    if (vh2 != 0.0) dth = fmin(dth, sqrt(V.rad(RV_DELXH2)[r] / vh2));
    a.dtr[r] = dtr;
    a.dth[r] = dth;
  }
  __syncthreads();
  double2* f = fft_run(h, g, I, tw, 2, false);
  const double tfac = (1.0 - I.tadvz) * beta * or1;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const int mc = (P - m) % P;
    const double2 Z = f[m], Zc = f[mc], Y = f[P + m], Yc = f[P + mc];
    const double2 vsT = make_double2(0.5 * (Z.x + Zc.x) / (double)P, 0.5 * (Z.y - Zc.y) / (double)P);
    const double2 upT = make_double2(0.5 * (Z.y + Zc.y) / (double)P, -0.5 * (Z.x - Zc.x) / (double)P);
    const double2 vsOm = make_double2(0.5 * (Y.x + Yc.x) / (double)P, 0.5 * (Y.y - Yc.y) / (double)P);
    const double2 upOm = make_double2(0.5 * (Y.y + Yc.y) / (double)P, -0.5 * (Y.x - Yc.x) / (double)P);
    const double t = or1 * (double)(m * I.minc);
    const long long o = (long long)r * M + m;
    a.dTdt[o] = make_double2(t * upT.y - tfac * vsT.x, -t * upT.x - tfac * vsT.y);
    a.dpsidt[o] = (m == 0) ? make_double2(-usom, 0.0) : make_double2(t * upOm.y, -t * upOm.x);
    a.s_dVsT[(long long)m * N + r] = vsT;
    a.s_dVsOm[(long long)m * N + r] = vsOm;
  }
}

// finish_exp_temp_coll and finish_exp_psi_coll_dmat for one m
// (src/update_temp_coll.f90:152-176, src/update_psi_coll_dmat.f90:468-552)
__global__ void __launch_bounds__(PZ_THREADS) k_expl_finish(PzExplArgs a) {
  extern __shared__ double2 shm[];
  const PzInst& I = *a.inst;
  const View V{&I, a.pool};
  const int n = I.N, M = I.M, mi = blockIdx.x;
  const double dm = (double)(mi * I.minc);
  double2* sa = shm;
  double2* sb = sa + n;
  double2* se = sb + n;
  double2* sf = se + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    sa[i] = a.s_dVsT[(long long)mi * n + i];
    se[i] = a.s_dVsOm[(long long)mi * n + i];
  }
  __syncthreads();
  mv1(V.basis(BM_D1P), n, n, sa, sb);
  mv1(V.basis(BM_D1P), n, n, se, sf);
  __syncthreads();
  const double* or1 = V.rad(RV_OR1);
  const double* beta = V.rad(RV_BETA);
  const double* rgrav = V.rad(RV_RGRAV);
  const double* tcond = V.rad(RV_TCOND);
  const double* dtcond = V.rad(RV_DTCOND);
  const double* ekpump = V.rad(RV_EKPUMP);
  const double* ekp_up = V.rad(RV_EKP_UP);
  const double* ekp_us = V.rad(RV_EKP_US);
  const double* ekp_dusdp = V.rad(RV_EKP_DUSDP);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long o = (long long)i * M + mi;
    const double2 u = a.us[o];
    double2 e = a.dTdt[o];
    const double c = dtcond[i] - I.tadvz * beta[i] * tcond[i];
    e.x = e.x - or1[i] * sb[i].x - u.x * c;
    e.y = e.y - or1[i] * sb[i].y - u.y * c;
    a.dTdt[o] = e;
    if (mi != 0) {
      double2 p = a.dpsidt[o];
      p.x -= or1[i] * sf[i].x;
      p.y -= or1[i] * sf[i].y;
      if (!(I.flags & PZF_NON_ROT)) {
        p.x += I.CorFac * beta[i] * u.x;
        p.y += I.CorFac * beta[i] * u.y;
      }
      if (!(I.flags & PZF_BUO_IMP)) {
        const double2 b = cim(dm, a.temp[o]);
        const double cb = I.BuoFac * rgrav[i] * or1[i];
        p.x -= cb * b.x; p.y -= cb * b.y;
      }
      if (I.flags & PZF_EK_PUMP) {
        const double2 w = a.om[o], v = a.up[o];
        const double2 q = make_double2(ekp_us[i] * u.x - ekp_dusdp[i] * dm * u.y,
                                       ekp_us[i] * u.y + ekp_dusdp[i] * dm * u.x);
        const double ce = I.CorFac * ekpump[i];
        p.x -= ce * (w.x + ekp_up[i] * v.x + q.x);
        p.y -= ce * (w.y + ekp_up[i] * v.y + q.y);
      }
      a.dpsidt[o] = p;
    }
  }
}

}  // namespace

size_t pz_expl_scratch_bytes(int n_r_max, int n_m_max) {
  return 2 * (size_t)n_r_max * (size_t)n_m_max * sizeof(double2);
}

cudaError_t pz_launch_explicit_terms(const PzExplArgs& a, int N, int M, int P, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_expl_rloop, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  if (e) return e;
  k_expl_rloop<<<N, PZ_THREADS, 5 * (size_t)P * sizeof(double2), s>>>(a);
  if ((e = cudaGetLastError())) return e;
  k_expl_finish<<<M, PZ_THREADS, 4 * (size_t)N * sizeof(double2), s>>>(a);
  return cudaGetLastError();
}

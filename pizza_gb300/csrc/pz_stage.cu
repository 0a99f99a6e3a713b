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

// radial_loop for PZ_RLOOP_G radii, reading and writing (n_m, n_r) arrays,
// n_m fastest, with dVsT and dVsOm to the m-major scratch
struct ExplIO {
  const PzExplArgs* a;
  int N, M;
  __device__ double2 in(int f, int m, int r) const {
    const long long o = (long long)r * M + m;
    return f == 0 ? a->us[o] : f == 1 ? a->up[o] : f == 2 ? a->om[o] : a->temp[o];
  }
  // composition: never asked for (the stage-level entry points reject it)
  __device__ void outx(int, int, double2, double2) const {}
  __device__ void grid(const double2*, long long, int) const {}
  __device__ void out(int m, int r, double2 dtdt, double2 vst, double2 dpdt, double2 vsom) const {
    const long long o = (long long)r * M + m;
    a->dTdt[o] = dtdt;
    a->dpsidt[o] = dpdt;
    a->s_dVsT[(long long)m * N + r] = vst;
    a->s_dVsOm[(long long)m * N + r] = vsom;
  }
  __device__ void cfl(int r, double dtr, double dth) const {
    a->dtr[r] = dtr;
    a->dth[r] = dth;
  }
};

__global__ void __launch_bounds__(256) k_expl_rloop(PzExplArgs a) {
  extern __shared__ double2 sh[];
  const PzInst& I = *a.inst;
  const View V{&I, a.pool};
  ExplIO io{&a, I.N, I.M};
  double* rsh = reinterpret_cast<double*>(sh + 4 * PZ_RLOOP_G * I.P);
  rloop_group<false>(I, V, blockIdx.x * PZ_RLOOP_G, PZ_RLOOP_G, io, sh, rsh);
}

// finish_exp_temp_coll and finish_exp_psi_coll_{dmat,smat} for one m
// (src/update_temp_coll.f90:152-176, src/update_psi_coll_dmat.f90:468-552,
// src/update_psi_coll_smat.f90:323-378)
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
      const bool direct = (I.flags & PZF_DIRECT) != 0;
      // explicit Coriolis: always with dmat, unless implicit with smat
      // (update_psi_coll_smat.f90:323-378)
      if (direct ? !(I.flags & PZF_COR_IMP) : !(I.flags & PZF_NON_ROT)) {
        p.x += I.CorFac * beta[i] * u.x;
        p.y += I.CorFac * beta[i] * u.y;
      }
      if (!(I.flags & PZF_BUO_IMP)) {
        const double2 b = cim(dm, a.temp[o]);
        const double cb = I.BuoFac * rgrav[i] * or1[i];
        p.x -= cb * b.x; p.y -= cb * b.y;
      }
      if (!direct && (I.flags & PZF_EK_PUMP)) {   // implicit with smat
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
  cudaError_t e = cudaFuncSetAttribute(k_expl_rloop, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX);
  if (e) return e;
  const size_t smem = 4 * (size_t)PZ_RLOOP_G * P * sizeof(double2) + (3 + (size_t)M) * PZ_RLOOP_G * sizeof(double);
  k_expl_rloop<<<(N + PZ_RLOOP_G - 1) / PZ_RLOOP_G, 256, smem, s>>>(a);
  if ((e = cudaGetLastError())) return e;
  k_expl_finish<<<M, PZ_THREADS, 4 * (size_t)N * sizeof(double2), s>>>(a);
  return cudaGetLastError();
}

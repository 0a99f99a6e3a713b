// Device helpers shared by the kernels of the library: complex arithmetic,
// block reductions, views into the pool, dense operator products and the
// mixed-radix phi-FFT.  Internal linkage (each .cu file gets its own copy).
#pragma once
#include <cuda_runtime.h>

#include "pz_internal.h"

#define PZ_THREADS 128

namespace {

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
// (i*m) * a
__device__ __forceinline__ double2 cim(double m, double2 a) { return make_double2(-m * a.y, m * a.x); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// block-wide reductions; `red` holds >= 32 doubles of shared scratch
__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}
__device__ double block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : -1.0e300;
  if (wid == 0) t = warp_max(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// Instance view: pointers into the pool.
struct View {
  const PzInst* I;
  double* pool;
  __device__ const double* rad(int k) const { return pool + I->o_rad + (long long)k * I->N; }
  __device__ const double* basis(int k) const { return pool + I->o_basis + (long long)k * I->N * I->N; }
  __device__ double2* fld(int f, int mi) const {
    return reinterpret_cast<double2*>(pool + I->o_fld) + ((long long)f * I->M + mi) * I->N;
  }
  __device__ double2* hist(int f, int kind, int phys, int mi) const {
    return reinterpret_cast<double2*>(pool + pz_hist_off(*I, f, kind, phys)) + (long long)mi * I->N;
  }
};

// ---------------------------------------------------------------------------
// dense operators: y = A x with A column-major (nr x nc) real, x complex
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mv1(const double* __restrict__ A, int nr, int nc,
                                    const double2* __restrict__ x, double2* __restrict__ y) {
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    double re = 0.0, im = 0.0;
    const double* a = A + i;
#pragma unroll 4
    for (int j = 0; j < nc; ++j) {
      const double aij = __ldg(a + (long long)j * nr);
      const double2 v = x[j];
      re = fma(aij, v.x, re);
      im = fma(aij, v.y, im);
    }
    y[i] = make_double2(re, im);
  }
}
__device__ __forceinline__ void mv2(const double* __restrict__ A, const double* __restrict__ B, int n,
                                    const double2* __restrict__ x, double2* __restrict__ ya,
                                    double2* __restrict__ yb) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
#pragma unroll 4
    for (int j = 0; j < n; ++j) {
      const double a = __ldg(A + i + (long long)j * n);
      const double b = __ldg(B + i + (long long)j * n);
      const double2 v = x[j];
      ar = fma(a, v.x, ar); ai = fma(a, v.y, ai);
      br = fma(b, v.x, br); bi = fma(b, v.y, bi);
    }
    ya[i] = make_double2(ar, ai);
    yb[i] = make_double2(br, bi);
  }
}
__device__ __forceinline__ void mv3(const double* __restrict__ A, const double* __restrict__ B,
                                    const double* __restrict__ C, int n, const double2* __restrict__ x,
                                    double2* __restrict__ ya, double2* __restrict__ yb,
                                    double2* __restrict__ yc) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0, cr = 0.0, ci = 0.0;
#pragma unroll 2
    for (int j = 0; j < n; ++j) {
      const double a = __ldg(A + i + (long long)j * n);
      const double b = __ldg(B + i + (long long)j * n);
      const double c = __ldg(C + i + (long long)j * n);
      const double2 v = x[j];
      ar = fma(a, v.x, ar); ai = fma(a, v.y, ai);
      br = fma(b, v.x, br); bi = fma(b, v.y, bi);
      cr = fma(c, v.x, cr); ci = fma(c, v.y, ci);
    }
    ya[i] = make_double2(ar, ai);
    yb[i] = make_double2(br, bi);
    yc[i] = make_double2(cr, ci);
  }
}

// ---------------------------------------------------------------------------
// phi-FFT: mixed-radix Stockham autosort on nb transforms in shared memory
// ---------------------------------------------------------------------------
// One stage of radix R with running product p (product of earlier radices).
// tw[k] = exp(-2 pi i k / P); sgn = +1 selects the backward transform.
__device__ void fft_stage(const double2* __restrict__ x, double2* __restrict__ y, int P, int R, int p,
                          const double2* __restrict__ tw, int nb, bool backward) {
  const int T = P / R;
  const int tstep = P / (p * R);
  const int rstep = P / R;
  for (int w = threadIdx.x; w < nb * T; w += blockDim.x) {
    const int b = w / T, i = w - b * T;
    const int k = i % p;
    const double2* xb = x + b * P;
    double2* yb = y + b * P;
    double2 u[PZ_MAX_RADIX];
#pragma unroll
    for (int q = 0; q < PZ_MAX_RADIX; ++q) {
      if (q < R) {
        double2 t = tw[(q * k * tstep) % P];
        if (backward) t.y = -t.y;
        u[q] = cmul(xb[i + q * T], t);
      }
    }
    const int base = (i - k) * R + k;
    if (R == 2) {
      yb[base] = cadd(u[0], u[1]);
      yb[base + p] = csub(u[0], u[1]);
    } else if (R == 4) {
      const double2 s02 = cadd(u[0], u[2]), d02 = csub(u[0], u[2]);
      const double2 s13 = cadd(u[1], u[3]), d13 = csub(u[1], u[3]);
      // forward: W = -i ; backward: W = +i
      const double2 jd13 = backward ? make_double2(-d13.y, d13.x) : make_double2(d13.y, -d13.x);
      yb[base] = cadd(s02, s13);
      yb[base + p] = cadd(d02, jd13);
      yb[base + 2 * p] = csub(s02, s13);
      yb[base + 3 * p] = csub(d02, jd13);
    } else {
      for (int s = 0; s < R; ++s) {
        double2 acc = u[0];
        for (int q = 1; q < R; ++q) {
          double2 t = tw[((s * q) % R) * rstep];
          if (backward) t.y = -t.y;
          acc = cadd(acc, cmul(u[q], t));
        }
        yb[base + s * p] = acc;
      }
    }
  }
}

// Full transform; returns the buffer holding the result (a or b).
__device__ double2* fft_run(double2* a, double2* b, const PzInst& I, const double2* tw, int nb, bool backward) {
  int p = 1;
  double2* src = a;
  double2* dst = b;
  for (int s = 0; s < I.nrad; ++s) {
    const int R = I.radix[s];
    fft_stage(src, dst, I.P, R, p, tw, nb, backward);
    __syncthreads();
    p *= R;
    double2* t = src; src = dst; dst = t;
  }
  return src;
}

}  // namespace

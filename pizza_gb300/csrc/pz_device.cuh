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
// largest 64-bit unsigned value over the warp (all 32 lanes active)
__device__ __forceinline__ unsigned long long warp_umax64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned lo = __shfl_xor_sync(0xffffffffu, (unsigned)v, o);
    const unsigned hi = __shfl_xor_sync(0xffffffffu, (unsigned)(v >> 32), o);
    const unsigned long long w = ((unsigned long long)hi << 32) | lo;
    v = w > v ? w : v;
  }
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
// tw[k] = exp(-2 pi i k / P) in global memory, tw[P + k] its conjugate;
// `backward` selects the conjugate twiddles.  RC = R for the radices with a
// specialised butterfly (2, 3, 4): the butterfly values stay in registers;
// RC = 0 is the generic radix.  FIRST = (p == 1): the first stage's twiddles
// are all 1 and its index within the stage is its butterfly index, so that
// instantiation loads and multiplies no twiddles.
template <int RC, bool FIRST>
__device__ void fft_stage_r(const double2* __restrict__ x, double2* __restrict__ y, int P, int Rrt, int p,
                            const double2* __restrict__ tw, int nb, bool backward) {
  constexpr int RU = RC ? RC : PZ_MAX_RADIX;
  const int R = RC ? RC : Rrt;
  const int T = P / R;
  const int tstep = P / (p * R);
  const int rstep = P / R;
  // backward transforms read the conjugate table (tw + P): no FP64 sign flips
  const double2* twd = backward ? tw + P : tw;
  // radix 3: W = c - i sg*sn with c = cos(2 pi/3), sn = sin(2 pi/3) from the table
  double c3 = 0.0, s3 = 0.0;
  if constexpr (RC == 3) {
    const double2 w1 = __ldg(tw + rstep);
    c3 = w1.x;
    s3 = backward ? w1.y : -w1.y;
  }
  for (int w = threadIdx.x; w < nb * T; w += blockDim.x) {
    const int b = w / T, i = w - b * T;
    int k = 0;
    if constexpr (!FIRST) k = i % p;
    const double2* xb = x + b * P;
    double2* yb = y + b * P;
    double2 u[RU];
    u[0] = xb[i];
#pragma unroll
    for (int q = 1; q < RU; ++q) {
      if (q < R) {
        const double2 v = xb[i + q * T];
        if constexpr (FIRST) u[q] = v;
        else u[q] = k == 0 ? v : cmul(v, __ldg(twd + q * k * tstep));   // q k tstep < R p P / (p R) = P
      }
    }
    const int base = (i - k) * R + k;
    if constexpr (RC == 2) {
      yb[base] = cadd(u[0], u[1]);
      yb[base + p] = csub(u[0], u[1]);
    } else if constexpr (RC == 4) {
      const double2 s02 = cadd(u[0], u[2]), d02 = csub(u[0], u[2]);
      const double2 s13 = cadd(u[1], u[3]), d13 = csub(u[1], u[3]);
      // forward: W = -i ; backward: W = +i
      const double2 jd13 = backward ? make_double2(-d13.y, d13.x) : make_double2(d13.y, -d13.x);
      yb[base] = cadd(s02, s13);
      yb[base + p] = cadd(d02, jd13);
      yb[base + 2 * p] = csub(s02, s13);
      yb[base + 3 * p] = csub(d02, jd13);
    } else if constexpr (RC == 3) {
      const double2 s12 = cadd(u[1], u[2]), d12 = csub(u[1], u[2]);
      const double2 m = make_double2(u[0].x + c3 * s12.x, u[0].y + c3 * s12.y);
      const double2 jd = make_double2(s3 * d12.y, -s3 * d12.x);   // -i sn d
      yb[base] = cadd(u[0], s12);
      yb[base + p] = cadd(m, jd);
      yb[base + 2 * p] = csub(m, jd);
    } else {
      for (int s2 = 0; s2 < R; ++s2) {
        double2 acc = u[0];
        for (int q = 1; q < R; ++q) acc = cadd(acc, cmul(u[q], __ldg(twd + ((s2 * q) % R) * rstep)));
        yb[base + s2 * p] = acc;
      }
    }
  }
}
__device__ void fft_stage(const double2* __restrict__ x, double2* __restrict__ y, int P, int R, int p,
                          const double2* __restrict__ tw, int nb, bool backward) {
  if (p == 1) {
    if (R == 4) fft_stage_r<4, true>(x, y, P, R, p, tw, nb, backward);
    else if (R == 2) fft_stage_r<2, true>(x, y, P, R, p, tw, nb, backward);
    else if (R == 3) fft_stage_r<3, true>(x, y, P, R, p, tw, nb, backward);
    else fft_stage_r<0, true>(x, y, P, R, p, tw, nb, backward);
  } else if (R == 4) fft_stage_r<4, false>(x, y, P, R, p, tw, nb, backward);
  else if (R == 2) fft_stage_r<2, false>(x, y, P, R, p, tw, nb, backward);
  else if (R == 3) fft_stage_r<3, false>(x, y, P, R, p, tw, nb, backward);
  else fft_stage_r<0, false>(x, y, P, R, p, tw, nb, backward);
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

// ---------------------------------------------------------------------------
// radial_loop for a group of radii of one instance (src/radial_loop.f90:231-394,
// ifft/fft of src/fft_fftw.f90:44-90).  IO supplies the inputs (us, up, om, T
// at (m, r)) and takes the outputs (dT/dt, dVsT, dpsi/dt, dVsOm at (m, r), and
// the Courant steps of radius r).  The two real fields of each pair are packed
// into one complex FFT (us + i up, om + i T on the way to the grid; the
// products r us T + i up T and r us om + i up om on the way back).  With
// composition (PZF_CHEM) a third transform per radius carries xi to the grid
// and r us xi + i up xi back (radial_loop.f90:297, :320-323, :356-374); IO
// then supplies in(4, m, r) and takes outx(m, r, dxi/dt, r us xi).
// G = min(gmax, N - r0) radii, nt = 2 (3 with composition) transforms per
// radius.  Shared memory: 2*nt*G*P complex (two ping-pong buffers of nt*G
// transforms) and 3*G + G*M doubles.  CHEM = false compiles the composition
// out (a handle without composition launches that instantiation).
template <bool CHEM, class IO>
__device__ void rloop_group(const PzInst& I, const View& V, int r0, int gmax, IO& io, double2* sh, double* rsh) {
  const int N = I.N, M = I.M, P = I.P;
  const int G = min(gmax, N - r0);
  const bool chem = CHEM && (I.flags & PZF_CHEM) != 0;
  const int nt = chem ? 3 : 2;
  const double2* tw = reinterpret_cast<const double2*>(V.pool + I.o_tw);
  double2* za = sh;                  // [g][nt][P]
  double2* zb = sh + nt * G * P;
  double* usom = rsh;                // [G]
  double* vr = rsh + G;              // [G]
  double* vh = rsh + 2 * G;          // [G]
  double* prod = rsh + 3 * G;        // [G][M] Reynolds-stress terms
  for (int k = threadIdx.x; k < nt * G * P; k += blockDim.x) za[k] = make_double2(0.0, 0.0);
  for (int k = threadIdx.x; k < 3 * G; k += blockDim.x) rsh[k] = 0.0;
  __syncthreads();
  // spectra at the G radii; Reynolds stress of the m=0 equation
  for (int t = threadIdx.x; t < G * M; t += blockDim.x) {
    const int g = t / M, m = t - g * M, r = r0 + g;
    double2 a = io.in(0, m, r), b = io.in(1, m, r), c = io.in(2, m, r), e = io.in(3, m, r);
    double us_om;
    if (m == 0) {
      // us_fluct(m=0) = E CorFac ekpump up(m=0) / 2 (radial_loop.f90:267-278)
      us_om = 0.5 * I.ek * I.CorFac * V.rad(RV_EKPUMP)[r] * b.x * c.x;
      a.y = 0.0; b.y = 0.0; c.y = 0.0; e.y = 0.0;   // c2r ignores Im of the DC term
    } else {
      us_om = 2.0 * (a.x * c.x + a.y * c.y);
    }
    prod[g * M + m] = us_om;
    double2* z1 = za + (nt * g) * P;
    double2* z2 = z1 + P;
    z1[m] = make_double2(a.x - b.y, a.y + b.x);
    z2[m] = make_double2(c.x - e.y, c.y + e.x);
    if (m > 0) {
      z1[P - m] = make_double2(a.x + b.y, -a.y + b.x);
      z2[P - m] = make_double2(c.x + e.y, -c.y + e.x);
    }
    if (chem) {
      double2 x = io.in(4, m, r);
      if (m == 0) x.y = 0.0;
      double2* z3 = z2 + P;
      z3[m] = x;
      if (m > 0) z3[P - m] = make_double2(x.x, -x.y);
    }
  }
  __syncthreads();
  {
    // deterministic sum over m of the Reynolds-stress terms, one warp per radius
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int g = wid; g < G; g += nw) {
      double acc = 0.0;
      for (int m = lane; m < M; m += 32) acc += prod[g * M + m];
      acc = warp_sum(acc);
      if (lane == 0) usom[g] = acc;
    }
  }
  double2* g1 = fft_run(za, zb, I, tw, nt * G, true);
  double2* h = (g1 == za) ? zb : za;
  io.grid(g1, r0 * nt * P, nt * G * P);   // read-only use of g1, like the loop below
  // Courant velocities and the nonlinear products on the grid.  When P is a
  // multiple of 32 the 32 points of a warp lie on one radius and every lane
  // runs every pass: one atomic per warp after a warp maximum.
  const bool warp_red = (P & 31) == 0 && (blockDim.x & 31) == 0;
  for (int t = threadIdx.x; t < G * P; t += blockDim.x) {
    const int g = t / P, j = t - g * P;
    const double rr = V.rad(RV_R)[r0 + g];
    const double2 z1 = g1[(nt * g) * P + j], z2 = g1[(nt * g + 1) * P + j];
    const double usg = z1.x, upg = z1.y, omg = z2.x, Tg = z2.y;
    // squares are >= 0: their bit patterns order like unsigned integers
    unsigned long long br = (unsigned long long)__double_as_longlong(usg * usg);
    unsigned long long bh = (unsigned long long)__double_as_longlong(upg * upg);
    if (warp_red) {
      br = warp_umax64(br);
      bh = warp_umax64(bh);
    }
    if (!warp_red || (threadIdx.x & 31) == 0) {
      atomicMax(reinterpret_cast<unsigned long long*>(&vr[g]), br);
      atomicMax(reinterpret_cast<unsigned long long*>(&vh[g]), bh);
    }
    h[(nt * g) * P + j] = make_double2(rr * usg * Tg, upg * Tg);
    h[(nt * g + 1) * P + j] = make_double2(rr * usg * omg, upg * omg);
    if (chem) {
      const double xg = g1[(nt * g + 2) * P + j].x;
      h[(nt * g + 2) * P + j] = make_double2(rr * usg * xg, upg * xg);
    }
  }
  __syncthreads();
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    // courant (src/courant.f90:41-76)
    const int r = r0 + g;
    const double vr2 = I.courfac * I.courfac * vr[g], vh2 = I.courfac * I.courfac * vh[g];
    double dtr = 1.0e10, dth = 1.0e10;
    if (vr2 != 0.0) dtr = fmin(dtr, sqrt(V.rad(RV_DELXR2)[r] / vr2));
    if (vh2 != 0.0) dth = fmin(dth, sqrt(V.rad(RV_DELXH2)[r] / vh2));
    io.cfl(r, dtr, dth);
  }
  double2* f = fft_run(h, g1, I, tw, nt * G, false);
  const double hP = 0.5 / (double)P;
  for (int t = threadIdx.x; t < G * M; t += blockDim.x) {
    const int g = t / M, m = t - g * M, r = r0 + g;
    const double or1 = V.rad(RV_OR1)[r];
    const double tfac = (1.0 - I.tadvz) * V.rad(RV_BETA)[r] * or1;
    const int mc = m == 0 ? 0 : P - m;
    const double2* f1 = f + (nt * g) * P;
    const double2* f2 = f1 + P;
    // split the two real transforms packed in one complex FFT
    const double2 Z = f1[m], Zc = f1[mc], Y = f2[m], Yc = f2[mc];
    // (the forward transform's 1/P folded with the split's 1/2: one multiply each)
    const double2 vsT = make_double2(hP * (Z.x + Zc.x), hP * (Z.y - Zc.y));
    const double2 upT = make_double2(hP * (Z.y + Zc.y), -hP * (Z.x - Zc.x));
    const double2 vsOm = make_double2(hP * (Y.x + Yc.x), hP * (Y.y - Yc.y));
    const double2 upOm = make_double2(hP * (Y.y + Yc.y), -hP * (Y.x - Yc.x));
    const double tm = or1 * (double)(m * I.minc);
    io.out(m, r, make_double2(tm * upT.y - tfac * vsT.x, -tm * upT.x - tfac * vsT.y), vsT,
           (m == 0) ? make_double2(-usom[g], 0.0) : make_double2(tm * upOm.y, -tm * upOm.x), vsOm);
    if (chem) {
      // dxi/dt = -(i m / r) FFT(up xi), no beta term (radial_loop.f90:372-374)
      const double2* f3 = f2 + P;
      const double2 X = f3[m], Xc = f3[mc];
      const double2 vsX = make_double2(hP * (X.x + Xc.x), hP * (X.y - Xc.y));
      const double2 upX = make_double2(hP * (X.y + Xc.y), -hP * (X.x - Xc.x));
      io.outx(m, r, make_double2(tm * upX.y, -tm * upX.x), vsX);
    }
  }
}

// ---------------------------------------------------------------------------
// operator products with one (row, re/im) task per lane
// ---------------------------------------------------------------------------
// Dot products of T tasks of length L, one task per lane.  Whole warps of
// tasks run one task per lane; the last r < 32 tasks (T is 2N or 4*ceil(N/2),
// two or four past a multiple of 32 for N = 2^k + 1) are split across the
// lanes of one warp, G = 32/r (rounded down to a power of 2) lanes per task,
// and reduced with shuffles, so no warp issues FP64 work for a few lanes.
// Policy P supplies fma(task, j, acc) and store(task, value).
template <class P>
__device__ __forceinline__ void lane_dots(const P& p, int T, int L) {
  const int full = T & ~31;
  for (int t = threadIdx.x; t < full; t += blockDim.x) {
    double acc = 0.0;
#pragma unroll 4
    for (int j = 0; j < L; ++j) acc = p.fma(t, j, acc);
    p.store(t, acc);
  }
  const int r = T - full;
  if (r > 0 && (threadIdx.x >> 5) == ((full >> 5) % (blockDim.x >> 5))) {
    const int lane = threadIdx.x & 31;
    int G = 32;
    while (G * r > 32) G >>= 1;
    const int task = lane / G, sub = lane & (G - 1);
    double acc = 0.0;
    if (task < r)
      for (int j = sub; j < L; j += G) acc = p.fma(full + task, j, acc);
    for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, G);
    if (task < r && sub == 0) p.store(full + task, acc);
  }
}
template <class P>
__device__ __forceinline__ void lane_dots2(const P& p, int T, int L) {
  const int full = T & ~31;
  for (int t = threadIdx.x; t < full; t += blockDim.x) {
    double a = 0.0, b = 0.0;
#pragma unroll 4
    for (int j = 0; j < L; ++j) p.fma2(t, j, a, b);
    p.store2(t, a, b);
  }
  const int r = T - full;
  if (r > 0 && (threadIdx.x >> 5) == ((full >> 5) % (blockDim.x >> 5))) {
    const int lane = threadIdx.x & 31;
    int G = 32;
    while (G * r > 32) G >>= 1;
    const int task = lane / G, sub = lane & (G - 1);
    double a = 0.0, b = 0.0;
    if (task < r)
      for (int j = sub; j < L; j += G) p.fma2(full + task, j, a, b);
    for (int o = G >> 1; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o, G);
      b += __shfl_down_sync(0xffffffffu, b, o, G);
    }
    if (task < r && sub == 0) p.store2(full + task, a, b);
  }
}

// dense: task t = component (t & 1) of row (t >> 1) of A x, A column-major n x n
struct DenseDot {
  const double* __restrict__ A; int n; const double* __restrict__ x; double* __restrict__ y;
  __device__ __forceinline__ double fma(int t, int j, double acc) const {
    return ::fma(__ldg(A + (t >> 1) + (long long)j * n), x[2 * j + (t & 1)], acc);
  }
  __device__ __forceinline__ void store(int t, double v) const { y[t] = v; }
};
// parity-compact: rows of A (nrow x L) take input v0 (even row) or v1 (odd row)
struct SymDot {
  const double* __restrict__ A; int nrow; const double* __restrict__ v0; const double* __restrict__ v1;
  double* __restrict__ out;
  __device__ __forceinline__ double fma(int t, int j, double acc) const {
    const int row = t >> 1;
    const double* v = (row & 1) ? v1 : v0;
    return ::fma(__ldg(A + row + (long long)j * nrow), v[2 * j + (t & 1)], acc);
  }
  __device__ __forceinline__ void store(int t, double v) const { out[t] = v; }
};
struct SymDot2 {
  const double* __restrict__ A; const double* __restrict__ B; int nrow;
  const double* __restrict__ v0; const double* __restrict__ v1; double* __restrict__ oa; double* __restrict__ ob;
  __device__ __forceinline__ void fma2(int t, int j, double& a, double& b) const {
    const int row = t >> 1;
    const double x = ((row & 1) ? v1 : v0)[2 * j + (t & 1)];
    a = ::fma(__ldg(A + row + (long long)j * nrow), x, a);
    b = ::fma(__ldg(B + row + (long long)j * nrow), x, b);
  }
  __device__ __forceinline__ void store2(int t, double a, double b) const { oa[t] = a; ob[t] = b; }
};

// one parity-compact operator applied to two inputs (v0a, v1a) and (v0b, v1b)
struct SymDotX2 {
  const double* __restrict__ A; int nrow;
  const double* __restrict__ v0a; const double* __restrict__ v1a;
  const double* __restrict__ v0b; const double* __restrict__ v1b;
  double* __restrict__ oa; double* __restrict__ ob;
  __device__ __forceinline__ void fma2(int t, int j, double& a, double& b) const {
    const int row = t >> 1, c = 2 * j + (t & 1);
    const double m = __ldg(A + row + (long long)j * nrow);
    a = ::fma(m, ((row & 1) ? v1a : v0a)[c], a);
    b = ::fma(m, ((row & 1) ? v1b : v0b)[c], b);
  }
  __device__ __forceinline__ void store2(int t, double a, double b) const { oa[t] = a; ob[t] = b; }
};

// y = A x, A column-major n x n real, x complex
__device__ __forceinline__ void mv_lanes(const double* __restrict__ A, int n, const double2* __restrict__ x,
                                         double2* __restrict__ y) {
  lane_dots(DenseDot{A, n, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y)}, 2 * n, n);
}

__device__ __forceinline__ void sym_dot(const double* __restrict__ A, int nrow, int L,
                                        const double2* __restrict__ v0, const double2* __restrict__ v1,
                                        double* __restrict__ out) {
  lane_dots(SymDot{A, nrow, reinterpret_cast<const double*>(v0), reinterpret_cast<const double*>(v1), out},
            2 * nrow, L);
}
__device__ __forceinline__ void sym_dot2(const double* __restrict__ A, const double* __restrict__ B, int nrow,
                                         int L, const double2* __restrict__ v0, const double2* __restrict__ v1,
                                         double* __restrict__ outA, double* __restrict__ outB) {
  lane_dots2(SymDot2{A, B, nrow, reinterpret_cast<const double*>(v0), reinterpret_cast<const double*>(v1), outA,
                     outB},
             2 * nrow, L);
}

// s_j = x_j + x_{n-1-j}, a_j = x_j - x_{n-1-j} (j < n/2); odd n: s_h = x_h, a_h = 0
__device__ __forceinline__ void prep_sa(const double2* __restrict__ x, int n, double2* __restrict__ s,
                                        double2* __restrict__ a) {
  const int h = n / 2, h2 = (n + 1) / 2;
  for (int j = threadIdx.x; j < h2; j += blockDim.x) {
    if (j < h) {
      const double2 p = x[j], q = x[n - 1 - j];
      s[j] = make_double2(p.x + q.x, p.y + q.y);
      a[j] = make_double2(p.x - q.x, p.y - q.y);
    } else {
      s[j] = x[j];
      a[j] = make_double2(0.0, 0.0);
    }
  }
}
// xe_k = x_{2k}, xo_k = x_{2k+1} (zero past the end)
__device__ __forceinline__ void prep_eo(const double2* __restrict__ x, int n, double2* __restrict__ xe,
                                        double2* __restrict__ xo) {
  const int h2 = (n + 1) / 2;
  for (int k = threadIdx.x; k < h2; k += blockDim.x) {
    xe[k] = x[2 * k];
    xo[k] = (2 * k + 1 < n) ? x[2 * k + 1] : make_double2(0.0, 0.0);
  }
}
// out holds rows (2i: E or u, 2i+1: O or v) x (re, im); y_i = E + O and
// y_{n-1-i} = se*E + so*O (i < n/2)
__device__ __forceinline__ void sym_combine(const double* __restrict__ out, int n, double se, double so,
                                            double2* __restrict__ y) {
  const int h = n / 2, h2 = (n + 1) / 2;
  for (int i = threadIdx.x; i < h2; i += blockDim.x) {
    const double er = out[4 * i], ei = out[4 * i + 1], orr = out[4 * i + 2], oi = out[4 * i + 3];
    y[i] = make_double2(er + orr, ei + oi);
    if (i < h) y[n - 1 - i] = make_double2(se * er + so * orr, se * ei + so * oi);
  }
}

// Scratch of the parity products: s, a (h2 complex each) and two task
// buffers of 4*h2 doubles.
struct SymScratch {
  double2* s; double2* a; double* t1; double* t2;
};

// y = C x (DCT-I, costf1)
__device__ void op_C(const View& V, int n, const double2* x, double2* y, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_CS), n, h2, w.s, w.a, reinterpret_cast<double*>(y));
}
// (y1, y2) = (D1c x, D2c x): Chebyshev coefficients -> physical derivatives
__device__ void op_Dc2(const View& V, int n, const double2* x, double2* y1, double2* y2, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_eo(x, n, w.s, w.a);
  __syncthreads();
  sym_dot2(V.basis(BM_D1CS), V.basis(BM_D2CS), 2 * h2, h2, w.s, w.a, w.t1, w.t2);
  __syncthreads();
  sym_combine(w.t1, n, -1.0, 1.0, y1);
  sym_combine(w.t2, n, 1.0, -1.0, y2);
}
// y1 = D1c x
__device__ void op_D1c(const View& V, int n, const double2* x, double2* y1, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_eo(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_D1CS), 2 * h2, h2, w.s, w.a, w.t1);
  __syncthreads();
  sym_combine(w.t1, n, -1.0, 1.0, y1);
}
// (y1, y2) = (D1p x, D2p x): physical -> physical derivatives
__device__ void op_Dp2(const View& V, int n, const double2* x, double2* y1, double2* y2, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot2(V.basis(BM_D1PS), V.basis(BM_D2PS), 2 * h2, h2, w.s, w.a, w.t1, w.t2);
  __syncthreads();
  // y_i = u + v ; y_{n-1-i} = sigma (u - v), sigma = -1 (D1p), +1 (D2p)
  sym_combine(w.t1, n, -1.0, 1.0, y1);
  sym_combine(w.t2, n, 1.0, -1.0, y2);
}
// y1 = D1p x
__device__ void op_D1p(const View& V, int n, const double2* x, double2* y1, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_D1PS), 2 * h2, h2, w.s, w.a, w.t1);
  __syncthreads();
  sym_combine(w.t1, n, -1.0, 1.0, y1);
}
// (ya, yb) = (D1p xa, D1p xb): the operator read once for both inputs; sb, ab
// (h2 complex each) hold the second input's sums and differences.  The
// products are those of op_D1p, bit for bit.
__device__ void op_D1p2(const View& V, int n, const double2* xa, const double2* xb, double2* ya, double2* yb,
                        SymScratch& w, double2* sb, double2* ab) {
  const int h2 = (n + 1) / 2;
  prep_sa(xa, n, w.s, w.a);
  prep_sa(xb, n, sb, ab);
  __syncthreads();
  lane_dots2(SymDotX2{V.basis(BM_D1PS), 2 * h2, reinterpret_cast<const double*>(w.s),
                      reinterpret_cast<const double*>(w.a), reinterpret_cast<const double*>(sb),
                      reinterpret_cast<const double*>(ab), w.t1, w.t2},
             4 * h2, h2);
  __syncthreads();
  sym_combine(w.t1, n, -1.0, 1.0, ya);
  sym_combine(w.t2, n, -1.0, 1.0, yb);
}
// (yc, yd) = (C x, D1c x): Chebyshev coefficients -> physical values and
// d/dr, one even/odd split of x for both
__device__ void op_CD1c(const View& V, int n, const double2* x, double2* yc, double2* yd, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_eo(x, n, w.s, w.a);
  __syncthreads();
  sym_dot2(V.basis(BM_COS), V.basis(BM_D1CS), 2 * h2, h2, w.s, w.a, w.t1, w.t2);
  __syncthreads();
  sym_combine(w.t1, n, 1.0, -1.0, yc);
  sym_combine(w.t2, n, -1.0, 1.0, yd);
}

// ---- transposes (discrete adjoint) -----------------------------------------
// y = C^T x
__device__ void op_CT(const View& V, int n, const double2* x, double2* y, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_eo(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_CTS), 2 * h2, h2, w.s, w.a, w.t1);
  __syncthreads();
  sym_combine(w.t1, n, 1.0, -1.0, y);
}
// y = D1c^T x
__device__ void op_D1cT(const View& V, int n, const double2* x, double2* y, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_D1CTS), n, h2, w.a, w.s, reinterpret_cast<double*>(y));
}
// y = D2c^T x
__device__ void op_D2cT(const View& V, int n, const double2* x, double2* y, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_D2CTS), n, h2, w.s, w.a, reinterpret_cast<double*>(y));
}
// y = D1p^T x
__device__ void op_D1pT(const View& V, int n, const double2* x, double2* y, SymScratch& w) {
  const int h2 = (n + 1) / 2;
  prep_sa(x, n, w.s, w.a);
  __syncthreads();
  sym_dot(V.basis(BM_D1PTS), 2 * h2, h2, w.s, w.a, w.t1);
  __syncthreads();
  sym_combine(w.t1, n, -1.0, 1.0, y);
}
// (y0, y1) = G x with G complex 2n x n, column-major with leading dimension 2n,
// x complex: rows < n go to y0, the others to y1 (the smat (omega, psi) solve)
struct CDenseDot {
  const double2* __restrict__ G; int n; const double* __restrict__ x; double* __restrict__ y0;
  double* __restrict__ y1;
  __device__ __forceinline__ double fma(int t, int j, double acc) const {
    const double2 g = __ldg(G + (t >> 1) + (long long)j * 2 * n);
    const double xr = x[2 * j], xi = x[2 * j + 1];
    return (t & 1) ? ::fma(g.x, xi, ::fma(g.y, xr, acc)) : ::fma(g.x, xr, ::fma(-g.y, xi, acc));
  }
  __device__ __forceinline__ void store(int t, double v) const {
    const int row = t >> 1;
    if (row < n) y0[2 * row + (t & 1)] = v;
    else y1[2 * (row - n) + (t & 1)] = v;
  }
};
__device__ __forceinline__ void cmv_lanes(const double2* __restrict__ G, int n, const double2* __restrict__ x,
                                          double2* __restrict__ y0, double2* __restrict__ y1) {
  lane_dots(CDenseDot{G, n, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y0),
                      reinterpret_cast<double*>(y1)},
            4 * n, n);
}

// y = A^T x, A column-major n x n real (dense per-m operators)
struct DenseDotT {
  const double* __restrict__ A; int n; const double* __restrict__ x; double* __restrict__ y;
  __device__ __forceinline__ double fma(int t, int i, double acc) const {
    return ::fma(__ldg(A + i + (long long)(t >> 1) * n), x[2 * i + (t & 1)], acc);
  }
  __device__ __forceinline__ void store(int t, double v) const { y[t] = v; }
};
__device__ __forceinline__ void mvT_lanes(const double* __restrict__ A, int n, const double2* __restrict__ x,
                                          double2* __restrict__ y) {
  lane_dots(DenseDotT{A, n, reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y)}, 2 * n, n);
}

}  // namespace

// k_fast: the stage of the collocation influence-matrix step on the tensor
// cores (pz_fast.h explains the method).  One block runs one m for a group of
// instances of the same (n_r_max, radratio) class: finish_explicit_assembly
// (src/mloop.f90:169-229 with update_temp_coll.f90:152-176 and
// update_psi_coll_dmat.f90:468-552), the IMEX right-hand sides
// (multistep_schemes.f90:308-316), update_temp_co (update_temp_coll.f90:66-150)
// and update_om_coll_dmat with its influence-matrix correction
// (update_psi_coll_dmat.f90:126-466), the implicit terms from the solve
// residual and the new fields.  Every operator product runs as bf16
// mma.sync on integer slices of the FP64 operands (exact products, FP64 sums).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "pizza_gpu.h"
#include "pz_device.cuh"
#include "pz_fast.h"
#include "pz_internal.h"

namespace {

// ---------------------------------------------------------------------------
// operand slices in shared memory
// ---------------------------------------------------------------------------
// A block of columns for the tensor cores: for each slice s and column j,
// sw 32-bit words, each holding two consecutive k (bf16, low half = even k).
// sw = Kpad/2 + 4 keeps the B-fragment loads of a warp on 32 distinct banks.
struct BOp {
  uint32_t* w;
  int* ce;       // per-column power of two: x = sum_s d_s 2^(ce - 8 (s + 1))
  int C;         // allocated columns (multiple of 16)
  int sw;        // words per (slice, column)
};

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
#define PZ_CE_NONFINITE 0x40000000

__device__ __forceinline__ uint16_t bf16_bits(int d) {
  return (uint16_t)(__float_as_uint((float)d) >> 16);   // |d| <= 256: exact
}

// Slice column j (K values x[k * step], k < K; zero past K up to 2 sw) with
// one warp: the column's power of two from the largest |x| (integer compare
// of the bit patterns), then x * 2^(56 - ce) rounded to a 56-bit integer and
// cut into balanced base-256 digits, all in integer arithmetic.
__device__ void split_col(const BOp& B, int j, const double* x, int step, int K) {
  const int lane = threadIdx.x & 31;
  unsigned long long mb = 0;
  for (int k = lane; k < K; k += 32)
    mb = umax64(mb, (unsigned long long)__double_as_longlong(x[(long long)k * step]) & 0x7fffffffffffffffULL);
  mb = warp_umax64(mb);
  const int ce = mb == 0 ? 0 : (int)((mb >> 52) & 0x7ff) - 1022;
  // a column holding Inf or NaN is marked so that its products come out NaN
  // (its digits would otherwise be finite) and the status check sees it
  if (lane == 0) B.ce[j] = ((mb >> 52) & 0x7ff) == 0x7ff ? PZ_CE_NONFINITE : ce;
  uint16_t* h = reinterpret_cast<uint16_t*>(B.w);
  const int kp = 2 * B.sw;
  for (int k = lane; k < kp; k += 32) {
    long long X = 0;
    if (k < K) {
      const unsigned long long u = (unsigned long long)__double_as_longlong(x[(long long)k * step]);
      const int E = (int)((u >> 52) & 0x7ff);
      const long long mant = (long long)(u & 0xfffffffffffffULL) | (E ? (1LL << 52) : 0LL);
      const int sh = (E ? E : 1) - 1075 + 8 * PZ_OZ_S - ce;
      if (sh >= 0) X = mant << sh;                                   // sh <= 3
      else if (sh > -62) X = (mant + (1LL << (-sh - 1))) >> (-sh);
      if (u >> 63) X = -X;
    }
#pragma unroll
    for (int s = PZ_OZ_S - 1; s > 0; --s) {
      const long long d = ((X + 128) & 255) - 128;
      X = (X - d) >> 8;
      h[((long long)s * B.C + j) * kp + k] = bf16_bits((int)d);
    }
    h[(long long)j * kp + k] = bf16_bits((int)X);
  }
}

// Columns of B that no split_col wrote this phase (inactive instances, the
// padding to whole 8-column tiles) hold stale slices: a product column depends
// on its own B column only, and those outputs are never stored or read.

__device__ __forceinline__ void mma16816(float* c, const uint4& a, uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

__device__ __forceinline__ double pow2(int e) {
  if (e < -1022) return 0.0;
  if (e > 1023) e = 1023;
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// The diagonal sums of one output, acc[g][q] = sum over kA + kx = g of the
// slice products (integers: |acc[0]| <= 97 * 2^16, |acc[g]| <= 97 * 2^14 (g + 3)),
// combined as sum_g acc[g] 2^(8 (6 - g)) in integer arithmetic: the top four
// diagonals exactly (below 2^47), the bottom three exactly (below 2^40), then
// the bottom part without its 11 lowest bits (2^-37 of the top diagonal's unit,
// far below the diagonals kA + kx >= 7 that the splitting leaves out) so the
// sum fits an int64 (below 2^60).  Returns that sum / 2^11 as a double, rounded
// once: the product is the result times 2^(ex_row + ex_col - 53).  Only the
// final conversion and scaling use the FP64 pipe.
static_assert(PZ_OZ_S == 7, "oz_combine is written for 7 slices");
__device__ __forceinline__ double oz_combine(const float (&acc)[PZ_OZ_S][4], int q) {
  long long hi = __float2int_rn(acc[0][q]);
  hi = hi * 256 + __float2int_rn(acc[1][q]);
  hi = hi * 256 + __float2int_rn(acc[2][q]);
  hi = hi * 256 + __float2int_rn(acc[3][q]);
  long long lo = __float2int_rn(acc[4][q]);
  lo = lo * 256 + __float2int_rn(acc[5][q]);
  lo = lo * 256 + __float2int_rn(acc[6][q]);
  return __ll2double_rn(hi * 8192 + (lo >> 11));    // >> of a negative lo: floor
}

// v 2^e; scales below the normal range in two steps so a small e does not
// flush a large v to zero
__device__ __forceinline__ double scale2(double v, int e) {
  return e >= -1022 ? v * pow2(e) : (v * pow2(e + 512)) * pow2(-512);
}

// Y[col * ldy + row] = (A X)(row, col), row < op.R, col < C (X = the slices in
// B).  A warp takes a (16-row tile, NC 8-column tiles) task; for each k tile
// it loads the NC x PZ_OZ_S B fragments once and every A slice once, and runs
// the slice pairs kA + kx <= PZ_OZ_S - 1, accumulating the pair sums of equal
// kA + kx in one fp32 register set (integers below 2^24: exact).  Each A
// slice register is refilled with the next k tile's slice as soon as its
// last product of this tile is issued, so the loads of tile kt + 1 overlap
// the products of tile kt (the last tile re-reads itself: no read past the
// operator).
template <int NC>
__device__ void oz_mma_t(const PzFastDev& F, const PzOzOp& op, const BOp& B, int C, double* Y, int ldy) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int gid = lane >> 2, t = lane & 3;
  const int CT = (C + 8 * NC - 1) / (8 * NC);
  const uint4* Af = F.frag + op.frag;
  const int* ea = F.ex + op.ex;
  for (int task = warp; task < op.RT * CT; task += nw) {
    const int rt = task / CT, ct = task - rt * CT;
    float acc[NC][PZ_OZ_S][4];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int g = 0; g < PZ_OZ_S; ++g)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[c][g][q] = 0.0f;
    const uint4* ap = Af + ((long long)rt * op.KT * PZ_OZ_S) * 32 + lane;
    uint4 a[PZ_OZ_S];
#pragma unroll
    for (int ka = 0; ka < PZ_OZ_S; ++ka) a[ka] = __ldg(ap + ka * 32);
    for (int kt = 0; kt < op.KT; ++kt) {
      uint32_t b[NC][PZ_OZ_S][2];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const int col = (ct * NC + c) * 8 + gid;
#pragma unroll
        for (int s = 0; s < PZ_OZ_S; ++s) {
          const uint32_t* p = B.w + ((long long)s * B.C + col) * B.sw + kt * 8 + t;
          b[c][s][0] = p[0];
          b[c][s][1] = p[4];
        }
      }
      const uint4* an = ap + (long long)(kt + 1 < op.KT ? kt + 1 : kt) * PZ_OZ_S * 32;
#pragma unroll
      for (int ka = 0; ka < PZ_OZ_S; ++ka) {
#pragma unroll
        for (int g = ka; g < PZ_OZ_S; ++g)
#pragma unroll
          for (int c = 0; c < NC; ++c) mma16816(acc[c][g], a[ka], b[c][g - ka][0], b[c][g - ka][1]);
        a[ka] = __ldg(an + ka * 32);
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = rt * 16 + gid + ((q & 2) ? 8 : 0);
        const int col = (ct * NC + c) * 8 + 2 * t + (q & 1);
        if (row < op.R && col < C) {
          const int ce = B.ce[col];
          Y[(long long)col * ldy + row] = ce == PZ_CE_NONFINITE ? __longlong_as_double(0x7ff8000000000000LL)
                                                                : scale2(oz_combine(acc[c], q), ea[row] + ce - 53);
        }
      }
  }
}
// one 8-column tile per task: the register budget of three blocks per SM
__device__ __forceinline__ void oz_mma(const PzFastDev& F, const PzOzOp& op, const BOp& B, int C, double* Y,
                                       int ldy) {
  oz_mma_t<1>(F, op, B, C, Y, ldy);
}

// The IMEX right-hand side of one instance (multistep_schemes.f90:308-316)
// as a list of history slots and weights: rhs = sum_j w[j] hist(slot[j])
// with the old terms (wimp), the implicit terms (wimp_lin(2:)) and the
// explicit terms (wexp) of the ring positions of this step.  off[j] is the
// slot's offset from the first history slot of the field, in (m, r) planes.
#define PZ_RHS_TERMS 12
struct RhsTerms {
  double w[PZ_RHS_TERMS];
  int off[PZ_RHS_TERMS];
  int n;
};
__device__ __forceinline__ void rhs_terms(const PzInst& I, const PzState& S, RhsTerms& T) {
  int n = 0;
  for (int k = 0; k < I.nold; ++k, ++n) { T.w[n] = S.wimp[k]; T.off[n] = (S.r_old + k) % I.nold; }
  for (int k = 0; k < I.nimp; ++k, ++n) { T.w[n] = S.wimp_lin[k + 1]; T.off[n] = I.nold + (S.r_impl + k) % I.nimp; }
  for (int k = 0; k < I.nexp; ++k, ++n) {
    T.w[n] = S.wexp[k];
    T.off[n] = I.nold + I.nimp + (S.r_expl + k) % I.nexp;
  }
  T.n = n;
}

// shared-memory layout of k_fast for G instances and grids up to N
struct FastSmem {
  BOp B;
  double* R;     // product outputs, column-major
  double* RT;    // temperature right-hand sides (interior), then the new temperature (interior)
  double* RW;    // vorticity / u_phi right-hand sides (interior)
  double* sc;    // per instance: c1 (re, im), c2 (re, im), w, 1/w, w TdiffFac, w ViscFac
  RhsTerms* rh;  // per instance: IMEX right-hand-side terms
  int* st;       // per instance: active, bad
};
__host__ __device__ inline size_t fast_smem_layout(int G, int N, size_t* oR, size_t* oRT, size_t* oRW, size_t* osc,
                                                   size_t* orh, size_t* ost, size_t* oce, int* C, int* sw) {
  const int n = N - 2;
  *C = ((2 * G + 15) / 16) * 16;
  *sw = ((N + 15) / 16) * 8 + 4;
  size_t o = (size_t)PZ_OZ_S * (*C) * (*sw) * 4;
  o = (o + 15) & ~(size_t)15;
  *oce = o; o += (size_t)(*C) * 4;
  o = (o + 15) & ~(size_t)15;
  *oR = o;
  const int rmax = (2 * N > 3 * N - 4) ? 2 * N : 3 * N - 4;
  o += (size_t)2 * G * rmax * 8;
  *oRT = o; o += (size_t)2 * G * n * 8;
  *oRW = o; o += (size_t)2 * G * n * 8;
  *osc = o; o += (size_t)G * 8 * 8;
  *orh = o; o += (size_t)G * sizeof(RhsTerms);
  o = (o + 15) & ~(size_t)15;
  *ost = o; o += (size_t)G * 2 * 4;
  return (o + 15) & ~(size_t)15;
}

__global__ void __launch_bounds__(256, 3) k_fast(PzDev d) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const PzFastDev& F = d.fast;
  const PzFastItem it = F.items[blockIdx.x];
  const PzFastCls cls = F.cls[it.cls];
  const int N = cls.N, n = cls.n, mi = it.m, G = F.G, ni = it.ni;
  FastSmem s;
  {
    size_t oR, oRT, oRW, osc, orh, ost, oce;
    int C, sw;
    fast_smem_layout(G, d.fast_maxN, &oR, &oRT, &oRW, &osc, &orh, &ost, &oce, &C, &sw);
    s.B.w = reinterpret_cast<uint32_t*>(fsm);
    s.B.ce = reinterpret_cast<int*>(fsm + oce);
    s.B.C = C;
    s.B.sw = ((N + 15) / 16) * 8 + 4;
    s.R = reinterpret_cast<double*>(fsm + oR);
    s.RT = reinterpret_cast<double*>(fsm + oRT);
    s.RW = reinterpret_cast<double*>(fsm + oRW);
    s.sc = reinterpret_cast<double*>(fsm + osc);
    s.rh = reinterpret_cast<RhsTerms*>(fsm + orh);
    s.st = reinterpret_cast<int*>(fsm + ost);
  }
  const int* fi = F.fi + it.i0;
  const PzFastM& FM = F.ms[cls.m0 + mi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    s.st[2 * g] = (g < ni && d.state[fi[g]].status == 0) ? 1 : 0;
    s.st[2 * g + 1] = 0;
    if (g < ni) {
      // per instance: w = wimp_lin(1), 1/w, w TdiffFac, w ViscFac
      const double w = d.state[fi[g]].wimp_lin[0];
      s.sc[8 * g + 4] = w;
      s.sc[8 * g + 5] = 1.0 / w;
      s.sc[8 * g + 6] = w * d.inst[fi[g]].TdiffFac;
      s.sc[8 * g + 7] = w * d.inst[fi[g]].ViscFac;
      rhs_terms(d.inst[fi[g]], d.state[fi[g]], s.rh[g]);
    }
  }
  __syncthreads();

  // ---- explicit terms: D1p of dVsT, then of dVsOm (2 columns per instance
  // each), into s.R and s.R + 2 G N
  for (int f = 0; f < 2; ++f) {
    for (int j = warp; j < 2 * ni; j += nw) {
      const int g = j >> 1, part = j & 1;
      if (!s.st[2 * g]) continue;
      const PzInst& I = d.inst[fi[g]];
      const View V{&I, d.pool};
      const double* x = reinterpret_cast<const double*>(V.fld(f ? F_DVSOM : F_DVST, mi)) + part;
      split_col(s.B, j, x, 2, N);
    }
    __syncthreads();
    oz_mma(F, cls.d1p, s.B, 2 * ni, s.R + (long long)f * 2 * G * N, N);
    __syncthreads();
  }

  // ---- finish the explicit terms; IMEX right-hand sides (interior rows).
  // One warp per instance: the instance's constants and row pointers are
  // read once into registers, the lanes run over the radii.
  const double dm = (double)(mi * d.inst[fi[0]].minc);
  for (int g = warp; g < ni; g += nw) {
    if (!s.st[2 * g]) continue;
    const int inst = fi[g];
    const PzInst& I = d.inst[inst];
    const PzState& S = d.state[inst];
    const View V{&I, d.pool};
    const int flags = I.flags;
    const double tadvz = I.tadvz, cor = I.CorFac, buo = I.BuoFac;
    const double* or1 = V.rad(RV_OR1);
    const double* beta = V.rad(RV_BETA);
    const double* dtcond = V.rad(RV_DTCOND);
    const double* tcond = V.rad(RV_TCOND);
    const double* rgrav = V.rad(RV_RGRAV);
    const double* ekp = V.rad(RV_EKPUMP);
    const double* ekus = V.rad(RV_EKP_US);
    const double* ekdp = V.rad(RV_EKP_DUSDP);
    const double* ekup = V.rad(RV_EKP_UP);
    const double2* us = V.fld(F_US, mi);
    const double2* tf = V.fld(F_TEMP, mi);
    const double2* om = V.fld(F_OM, mi);
    const double2* up = V.fld(F_UP, mi);
    double2* eT = V.hist(0, 2, S.r_expl, mi);
    double2* eP = V.hist(1, 2, S.r_expl, mi);
    const double2* h0 = V.hist(0, 0, 0, mi);      // first history slot, temperature
    const double2* h1 = V.hist(1, 0, 0, mi);      // first history slot, vorticity / u_phi
    const long long pl = (long long)I.M * I.N;    // one (m, r) plane
    const RhsTerms& rh = s.rh[g];
    const double* Rt = s.R + (long long)(2 * g) * N;
    const double* Ro = s.R + (long long)(2 * G + 2 * g) * N;
    for (int i = lane; i < N; i += 32) {
      const double2 u = us[i];
      const double2 dT = make_double2(Rt[i], Rt[N + i]);
      double2 e = eT[i];
      const double c = dtcond[i] - tadvz * beta[i] * tcond[i];
      e.x = e.x - or1[i] * dT.x - u.x * c;
      e.y = e.y - or1[i] * dT.y - u.y * c;
      eT[i] = e;
      if (mi != 0) {
        const double2 dO = make_double2(Ro[i], Ro[N + i]);
        double2 p = eP[i];
        p.x -= or1[i] * dO.x;
        p.y -= or1[i] * dO.y;
        if (!(flags & PZF_NON_ROT)) {
          p.x += cor * beta[i] * u.x;
          p.y += cor * beta[i] * u.y;
        }
        if (!(flags & PZF_BUO_IMP)) {
          const double2 b = cim(dm, tf[i]);
          const double cb = buo * rgrav[i] * or1[i];
          p.x -= cb * b.x; p.y -= cb * b.y;
        }
        if (flags & PZF_EK_PUMP) {
          const double2 o = om[i], w = up[i];
          const double eus = ekus[i], edp = ekdp[i];
          const double2 q = make_double2(eus * u.x - edp * dm * u.y, eus * u.y + edp * dm * u.x);
          const double ce = cor * ekp[i];
          const double eup = ekup[i];
          p.x -= ce * (o.x + eup * w.x + q.x);
          p.y -= ce * (o.y + eup * w.y + q.y);
        }
        eP[i] = p;
      }
      if (i == 0 || i == N - 1) continue;
      // the explicit term of this step was stored above: read after the store
      double2 rt = make_double2(0.0, 0.0), rw = make_double2(0.0, 0.0);
      for (int k = 0; k < rh.n; ++k) {
        const double w = rh.w[k];
        const long long o = rh.off[k] * pl + i;
        const double2 a = h0[o], b = h1[o];
        rt.x += w * a.x; rt.y += w * a.y;
        rw.x += w * b.x; rw.y += w * b.y;
      }
      if (mi == 0) rw.y = 0.0;
      s.RT[(2 * g) * n + i - 1] = rt.x;
      s.RT[(2 * g + 1) * n + i - 1] = rt.y;
      s.RW[(2 * g) * n + i - 1] = rw.x;
      s.RW[(2 * g + 1) * n + i - 1] = rw.y;
    }
  }
  __syncthreads();

  // ---- temperature: y = U^-1 rhs, z = y / (1 - w TdiffFac lam), [T; dT/dr] = [U; D1p U] z
  for (int j = warp; j < 2 * ni; j += nw)
    if (s.st[2 * (j >> 1)]) split_col(s.B, j, s.RT + (long long)j * n, 1, n);
  __syncthreads();
  oz_mma(F, FM.uinv, s.B, 2 * ni, s.R, n);
  __syncthreads();
  {
    const double* lam = F.vec + FM.vec;
    for (int t = threadIdx.x; t < ni * n; t += blockDim.x) {
      const int g = t / n, k = t - g * n;
      const double D = 1.0 / (1.0 - s.sc[8 * g + 6] * lam[k]);
      s.R[(long long)(2 * g) * n + k] *= D;
      s.R[(long long)(2 * g + 1) * n + k] *= D;
    }
  }
  __syncthreads();
  for (int j = warp; j < 2 * ni; j += nw)
    if (s.st[2 * (j >> 1)]) split_col(s.B, j, s.R + (long long)j * n, 1, n);
  __syncthreads();
  oz_mma(F, FM.s3t, s.B, 2 * ni, s.R, n + N);
  __syncthreads();
  // new temperature, dT/dr, history; the vorticity rhs gets the implicit buoyancy
  // (one warp per instance, like the explicit terms)
  for (int g = warp; g < ni; g += nw) {
    if (!s.st[2 * g]) continue;
    const int inst = fi[g];
    const PzInst& I = d.inst[inst];
    const PzState& S = d.state[inst];
    const View V{&I, d.pool};
    const int ld = n + N;
    const double w = S.wimp_lin[0], iw = s.sc[8 * g + 5];
    const bool lin = S.l_calc_lin != 0;
    const bool buo = mi != 0 && (I.flags & PZF_BUO_IMP);
    const double cbuo = w * I.BuoFac;
    const double* rgrav = V.rad(RV_RGRAV);
    const double* or1 = V.rad(RV_OR1);
    double2* tf = V.fld(F_TEMP, mi);
    double2* dtf = V.fld(F_DTEMP, mi);
    double2* ho = V.hist(0, 0, S.b_old, mi);
    double2* hi = V.hist(0, 1, S.b_impl, mi);
    const double* Rr = s.R + (long long)(2 * g) * ld;
    const double* Ri = Rr + ld;
    double* RTr = s.RT + (long long)(2 * g) * n;
    double* RTi = RTr + n;
    double* RWr = s.RW + (long long)(2 * g) * n;
    double* RWi = RWr + n;
    bool bad = false;
    for (int i = lane; i < N; i += 32) {
      const bool edge = (i == 0 || i == N - 1);
      const double2 T = edge ? make_double2(0.0, 0.0) : make_double2(Rr[i - 1], Ri[i - 1]);
      tf[i] = T;
      dtf[i] = make_double2(Rr[n + i], Ri[n + i]);
      ho[i] = T;
      bad |= !isfinite(T.x) || !isfinite(T.y);
      if (lin) hi[i] = edge ? make_double2(0.0, 0.0) : make_double2(iw * (T.x - RTr[i - 1]), iw * (T.y - RTi[i - 1]));
      if (edge) continue;
      RTr[i - 1] = T.x;       // the new temperature for the buoyancy below
      RTi[i - 1] = T.y;
      if (buo) {
        const double2 b = cim(dm, T);
        const double c = cbuo * rgrav[i] * or1[i];
        RWr[i - 1] -= c * b.x;
        RWi[i - 1] -= c * b.y;
      }
    }
    if (bad) s.st[2 * g + 1] = 1;
  }
  __syncthreads();

  // ---- vorticity (m > 0) or u_phi (m = 0): y = U^-1 rhs
  const PzOzOp& wuinv = (mi == 0) ? F.us[it.ucls].uinv : FM.uinv;
  for (int j = warp; j < 2 * ni; j += nw)
    if (s.st[2 * (j >> 1)]) split_col(s.B, j, s.RW + (long long)j * n, 1, n);
  __syncthreads();
  oz_mma(F, wuinv, s.B, 2 * ni, s.R, n);
  __syncthreads();
  if (mi == 0) {
    const double* lam = F.vec + F.us[it.ucls].vec;
    for (int t = threadIdx.x; t < ni * n; t += blockDim.x) {
      const int g = t / n, k = t - g * n;
      const double D = 1.0 / (1.0 - s.sc[8 * g + 4] * lam[k]);
      s.R[(long long)(2 * g) * n + k] *= D;
      s.R[(long long)(2 * g + 1) * n + k] *= D;
    }
  } else {
    // z = y / (1 - w nu lam); influence correction in eigen space: the two
    // homogeneous solutions are h = w nu D U^-1 P_Ib e_wall, their dpsi/dr at
    // the walls give the 2 x 2 influence matrix, and z + c1 h_bot + c2 h_top
    // has the no-slip walls (update_psi_coll_dmat.f90:1136-1300)
    const double* lam = F.vec + FM.vec;
    const double* gtop = lam + n;
    const double* gbot = lam + 2 * n;
    const double* qt = lam + 3 * n;
    const double* qb = lam + 4 * n;
    for (int g = warp; g < ni; g += nw) {
      if (!s.st[2 * g]) continue;
      const double wn = s.sc[8 * g + 7];
      double* zr = s.R + (long long)(2 * g) * n;
      double* zi = zr + n;
      // v = (t1r, t1i, b1r, b1i, t2, b2, t3, b3): the walls' dpsi/dr of z
      // (t1, b1) and of the two homogeneous solutions (t2, b2; t3, b3)
      double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      double hb[PZ_FAST_KPL], ht[PZ_FAST_KPL];   // h_bot, h_top at this lane's k
#pragma unroll
      for (int u = 0; u < PZ_FAST_KPL; ++u) {
        const int k = lane + 32 * u;
        hb[u] = 0.0; ht[u] = 0.0;
        if (k >= n) continue;
        const double D = 1.0 / (1.0 - wn * lam[k]);
        const double wD = wn * D;
        const double yr = zr[k] * D, yi = zi[k] * D;
        zr[k] = yr; zi[k] = yi;
        hb[u] = wD * gbot[k]; ht[u] = wD * gtop[k];
        const double a = qt[k], b = qb[k];
        v[0] += a * yr; v[1] += a * yi; v[2] += b * yr; v[3] += b * yi;
        v[4] += a * hb[u]; v[5] += b * hb[u]; v[6] += a * ht[u]; v[7] += b * ht[u];
      }
      // the eight warp sums as one transpose reduction: each exchange halves
      // the values a lane carries (16: 8 -> 4, 8: 4 -> 2, 4: 2 -> 1), two
      // more rounds finish the sums; lane 16 q2 + 8 q1 + 4 q0 then holds sum q
      double r4[4], r2[2];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool hi = lane & 16;
        const double send = hi ? v[q] : v[q + 4];
        r4[q] = (hi ? v[q + 4] : v[q]) + __shfl_xor_sync(0xffffffffu, send, 16);
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const bool hi = lane & 8;
        const double send = hi ? r4[q] : r4[q + 2];
        r2[q] = (hi ? r4[q + 2] : r4[q]) + __shfl_xor_sync(0xffffffffu, send, 8);
      }
      double r1;
      {
        const bool hi = lane & 4;
        const double send = hi ? r2[0] : r2[1];
        r1 = (hi ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, send, 4);
      }
      r1 += __shfl_xor_sync(0xffffffffu, r1, 2);
      r1 += __shfl_xor_sync(0xffffffffu, r1, 1);
      double sum[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) sum[q] = __shfl_sync(0xffffffffu, r1, 16 * (q >> 2) + 8 * ((q >> 1) & 1) + 4 * (q & 1));
      const double t1r = sum[0], t1i = sum[1], b1r = sum[2], b1i = sum[3];
      const double t2 = sum[4], b2 = sum[5], t3 = sum[6], b3 = sum[7];
      const double idet = 1.0 / (t2 * b3 - t3 * b2);
      const double i00 = b3 * idet, i01 = -t3 * idet, i10 = -b2 * idet, i11 = t2 * idet;
      const double c1r = -i00 * t1r - i01 * b1r, c1i = -i00 * t1i - i01 * b1i;
      const double c2r = -i10 * t1r - i11 * b1r, c2i = -i10 * t1i - i11 * b1i;
#pragma unroll
      for (int u = 0; u < PZ_FAST_KPL; ++u) {
        const int k = lane + 32 * u;
        if (k >= n) continue;
        zr[k] += c1r * hb[u] + c2r * ht[u];
        zi[k] += c1i * hb[u] + c2i * ht[u];
      }
      if (lane == 0) {
        s.sc[8 * g + 0] = c1r; s.sc[8 * g + 1] = c1i; s.sc[8 * g + 2] = c2r; s.sc[8 * g + 3] = c2i;
      }
    }
  }
  __syncthreads();
  for (int j = warp; j < 2 * ni; j += nw)
    if (s.st[2 * (j >> 1)]) split_col(s.B, j, s.R + (long long)j * n, 1, n);
  __syncthreads();
  const PzOzOp& w3 = (mi == 0) ? F.us[it.ucls].s3u : FM.s3w;
  const int ld3 = w3.R;
  oz_mma(F, w3, s.B, 2 * ni, s.R, ld3);
  __syncthreads();

  // ---- new velocity, vorticity and streamfunction; history (one warp per instance)
  for (int g = warp; g < ni; g += nw) {
    if (!s.st[2 * g]) continue;
    const int inst = fi[g];
    const PzInst& I = d.inst[inst];
    const PzState& S = d.state[inst];
    const View V{&I, d.pool};
    const double* or1 = V.rad(RV_OR1);
    const double* beta = V.rad(RV_BETA);
    const double* rgrav = V.rad(RV_RGRAV);
    const double iw = s.sc[8 * g + 5];
    const bool lin = S.l_calc_lin != 0;
    const bool buo = (I.flags & PZF_BUO_IMP) != 0;
    const double bf = I.BuoFac;
    double2* us = V.fld(F_US, mi);
    double2* up = V.fld(F_UP, mi);
    double2* omf = V.fld(F_OM, mi);
    double2* psi = V.fld(F_PSI, mi);
    double2* ho = V.hist(1, 0, S.b_old, mi);
    double2* hi = V.hist(1, 1, S.b_impl, mi);
    const double* Rr = s.R + (long long)(2 * g) * ld3;
    const double* Ri = s.R + (long long)(2 * g + 1) * ld3;
    const double* RWr = s.RW + (long long)(2 * g) * n;
    const double* RWi = RWr + n;
    const double* RTr = s.RT + (long long)(2 * g) * n;
    const double* RTi = RTr + n;
    const double2 om_bot = make_double2(s.sc[8 * g + 2], s.sc[8 * g + 3]);
    const double2 om_top = make_double2(s.sc[8 * g + 0], s.sc[8 * g + 1]);
    bool bad = false;
    for (int i = lane; i < N; i += 32) {
      const bool edge = (i == 0 || i == N - 1);
      if (mi == 0) {
        const double u = edge ? 0.0 : Rr[i - 1];
        const double du = Rr[n + i];
        us[i] = make_double2(0.0, 0.0);
        up[i] = make_double2(u, 0.0);
        omf[i] = make_double2(du + or1[i] * u, 0.0);
        psi[i] = make_double2(0.0, 0.0);
        ho[i] = make_double2(u, 0.0);
        if (lin) hi[i] = make_double2(edge ? 0.0 : iw * (u - RWr[i - 1]), 0.0);
        bad |= !isfinite(u);
      } else {
        const double2 om = i == 0 ? om_bot : (i == N - 1 ? om_top : make_double2(Rr[i - 1], Ri[i - 1]));
        const double2 ps = edge ? make_double2(0.0, 0.0) : make_double2(Rr[n + i - 1], Ri[n + i - 1]);
        const double2 dp = make_double2(Rr[2 * n + i], Ri[2 * n + i]);
        const double be = beta[i];
        psi[i] = ps;
        us[i] = cscale(or1[i], cim(dm, ps));
        up[i] = make_double2(-dp.x - be * ps.x, -dp.y - be * ps.y);
        omf[i] = om;
        ho[i] = om;
        if (lin) {
          double2 v = make_double2(0.0, 0.0);
          if (!edge) {
            v = cscale(iw, csub(om, make_double2(RWr[i - 1], RWi[i - 1])));
            if (buo) {
              const double2 b = cim(dm, make_double2(RTr[i - 1], RTi[i - 1]));
              const double c = rgrav[i] * or1[i] * bf;
              v.x -= c * b.x; v.y -= c * b.y;
            }
          }
          hi[i] = v;
        }
        bad |= !isfinite(om.x) || !isfinite(om.y);
      }
    }
    if (bad) s.st[2 * g + 1] = 1;
  }
  __syncthreads();
  for (int g = threadIdx.x; g < ni; g += blockDim.x)
    if (s.st[2 * g] && s.st[2 * g + 1]) {
      PzState& Sg = d.state[fi[g]];
      if (Sg.status == 0) Sg.status = PZ_E_NONFINITE;
    }
}

}  // namespace

size_t pz_fast_smem_bytes(int G, int maxN) {
  size_t oR, oRT, oRW, osc, orh, ost, oce;
  int C, sw;
  return fast_smem_layout(G, maxN, &oR, &oRT, &oRW, &osc, &orh, &ost, &oce, &C, &sw);
}

cudaError_t pz_launch_fast(const PzDev& d, cudaStream_t s) {
  if (d.fast.n_items == 0) return cudaSuccess;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, PZ_SMEM_MAX);
    if (e) return e;
    attr = true;
  }
  k_fast<<<d.fast.n_items, 256, d.fast.smem, s>>>(d);
  return cudaGetLastError();
}

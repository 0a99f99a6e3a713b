// Bordered banded systems of the integration method: the solves of
// src/band_matrix.f90:212-261 (gbtrf/gbtrs on band storage) and
// src/bordered_matrix.f90:137-183 (the tau rows as a border, eliminated by a
// Schur complement), restated for the GPU.
//
// A system of order n has nt dense tau rows (2 for the temperature, u_phi and
// vorticity operators, 4 for the streamfunction); every other row i has
// non-zeros only for |i - j| <= kl.  With
//   A = [A1 A2; A3 A4],  A1 nt x nt,  A4 banded of order nb = n - nt,
// A4 is LU-factorised with partial pivoting inside the band (the algorithm of
// LAPACK's gbtf2: U gets 2 kl super-diagonals), W = A4^-1 A3 and the Schur
// complement S = A1 - A2 W is inverted, so that A x = b is
//   y2 = A4^-1 b2,  x1 = S^-1 (b1 - A2 y2),  x2 = y2 - W x1.
// Rows are first scaled by 1 / max|row| (the row preconditioning of the
// reference's lhs builders).
//
// The factor is stored per system as one record (T = double for the real
// operators, double2 for the complex streamfunction operator of the direct
// solve), laid out for the solve's row sweeps:
//   nb rows of R = 3 kl + 2:  [0] 1/U(j,j), [1 .. 2kl] U(j, j+1 .. j+2kl),
//                             [2kl+1 .. 3kl] L(j+1 .. j+kl, j), [3kl+1] pivot offset
//   A2 (nt rows of nb), W (nt columns of nb), S^-1 (nt x nt, row-major), the n row scales.
// Entries past the end of A4 are zero.  The factorisation runs when dt
// changes (k_build); every stage applies the record with one thread per
// real column walking the rows with its band window in registers (the
// sweeps are sequential in the rows, 2-3 dependent operations per row),
// the rest of the block doing the border products.  The solve needs no
// minimum block size.
#pragma once

// factorisation workspace in T units (plus nb ints of pivots after it)
__host__ __device__ inline long long bord_ws_size(int n, int nt, int kl) {
  const long long nb = n - nt;
  return (3LL * kl + 1) * nb + 2LL * nt * nb + (long long)nt * nt + n;
}

// -- scalar helpers for real and complex entries ---------------------------
__device__ __forceinline__ double bz(double) { return 0.0; }
__device__ __forceinline__ double2 bz(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double bmod(double a) { return fabs(a); }
__device__ __forceinline__ double bmod(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double babs1(double a) { return fabs(a); }
__device__ __forceinline__ double babs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double bre(double a) { return a; }
__device__ __forceinline__ double bre(double2 a) { return a.x; }
__device__ __forceinline__ double bmul(double a, double b) { return a * b; }
__device__ __forceinline__ double2 bmul(double2 a, double2 b) { return cmul(a, b); }
__device__ __forceinline__ double2 bmul(double a, double2 b) { return cscale(a, b); }
__device__ __forceinline__ double bscale(double s, double a) { return s * a; }
__device__ __forceinline__ double2 bscale(double s, double2 a) { return cscale(s, a); }
// a - b c
__device__ __forceinline__ double bfms(double a, double b, double c) { return fma(-b, c, a); }
__device__ __forceinline__ double2 bfms(double2 a, double2 b, double2 c) {
  return make_double2(fma(b.y, c.y, fma(-b.x, c.x, a.x)), fma(-b.y, c.x, fma(-b.x, c.y, a.y)));
}
__device__ __forceinline__ double2 bfms(double2 a, double b, double2 c) {
  return make_double2(fma(-b, c.x, a.x), fma(-b, c.y, a.y));
}
__device__ __forceinline__ double badd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 badd(double2 a, double2 b) { return cadd(a, b); }
__device__ __forceinline__ double brcp(double a) { return 1.0 / a; }
__device__ __forceinline__ double2 brcp(double2 a) {
  const double s = 1.0 / fmax(fabs(a.x), fabs(a.y));
  const double x = a.x * s, y = a.y * s, d = 1.0 / (x * x + y * y);
  return make_double2(x * d * s, -y * d * s);
}
__device__ __forceinline__ double bfrom(double v, double) { return v; }
__device__ __forceinline__ double2 bfrom(double v, double2) { return make_double2(v, 0.0); }

// -- factorisation (block-wide; k_build) --------------------------------------
// get(i, j): entry of the unscaled matrix, asked for the tau rows (i < nt,
// every j) and for |i - j| <= bw otherwise.  ws: bord_ws_size(n, nt, kl) T
// of shared memory followed by nb ints; flag: one shared int.  Writes the
// record to out (global).  Returns nonzero (on every thread) for a zero
// pivot of A4 or a singular Schur complement.
template <class T, class Get>
__device__ int bord_factor(const Get& get, int n, int nt, int kl, int bw, T* ws, int* flag, T* out) {
  const int nb = n - nt, ld = 3 * kl + 1, kv = 2 * kl, R = 3 * kl + 2;
  T* AB = ws;                       // column j of A4 at AB + j ld, row i at kv + i - j
  T* A3 = AB + (long long)ld * nb;  // nt columns of nb
  T* A1 = A3 + (long long)nt * nb;  // nt x nt, row-major
  T* A2 = A1 + nt * nt;             // nt rows of nb
  T* fs = A2 + (long long)nt * nb;  // row scales (real part)
  int* piv = reinterpret_cast<int*>(fs + n);
  const T zero = bz(T());
  if (threadIdx.x == 0) *flag = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int j0 = i < nt ? 0 : max(0, i - bw), j1 = i < nt ? n - 1 : min(n - 1, i + bw);
    double mx = 0.0;
    for (int j = j0; j <= j1; ++j) mx = fmax(mx, bmod(get(i, j)));
    fs[i] = bfrom(mx > 0.0 ? 1.0 / mx : 0.0, T());
  }
  for (long long q = threadIdx.x; q < (long long)(ld + nt) * nb; q += blockDim.x) AB[q] = zero;  // AB and A3
  __syncthreads();
  for (int i = nt + threadIdx.x; i < n; i += blockDim.x) {
    const double f = bre(fs[i]);
    for (int j = max(0, i - bw); j <= min(n - 1, i + bw); ++j) {
      const T v = bscale(f, get(i, j));
      if (j >= nt) AB[(long long)(j - nt) * ld + kv + i - j] = v;
      else A3[(long long)j * nb + i - nt] = v;
    }
  }
  for (int q = threadIdx.x; q < nt * n; q += blockDim.x) {
    const int t = q / n, j = q - t * n;
    const T v = bscale(bre(fs[t]), get(t, j));
    if (j < nt) A1[t * nt + j] = v;
    else A2[(long long)t * nb + j - nt] = v;
  }
  __syncthreads();
  // band LU of A4 with partial pivoting, one warp (gbtf2)
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    int ju = 0, bad = 0;
    for (int j = 0; j < nb; ++j) {
      const int km = min(kl, nb - 1 - j);
      T* cj = AB + (long long)j * ld + kv;                  // cj[i] = A4(j + i, j)
      double a = lane <= km ? babs1(cj[lane]) : -1.0;
      int p = lane;
      for (int o = 16; o > 0; o >>= 1) {
        const double a2 = __shfl_xor_sync(0xffffffffu, a, o);
        const int p2 = __shfl_xor_sync(0xffffffffu, p, o);
        if (a2 > a || (a2 == a && p2 < p)) { a = a2; p = p2; }
      }
      if (!(a > 0.0)) { bad = 1; break; }                   // zero (or NaN) pivot column
      if (lane == 0) piv[j] = p;
      ju = max(ju, min(j + kl + p, nb - 1));
      if (p != 0)
        for (int c = j + lane; c <= ju; c += 32) {
          T* col = AB + (long long)c * ld + kv - c;
          const T t = col[j];
          col[j] = col[j + p];
          col[j + p] = t;
        }
      __syncwarp();
      const T rp = brcp(cj[0]);
      if (lane >= 1 && lane <= km) cj[lane] = bmul(cj[lane], rp);
      __syncwarp();
      const int nc = ju - j;
      for (int q = lane; q < km * nc; q += 32) {
        const int i = 1 + q % km, c = j + 1 + q / km;
        T* col = AB + (long long)c * ld + kv - c;
        col[j + i] = bfms(col[j + i], cj[i], col[j]);
      }
      __syncwarp();
    }
    if (lane == 0 && bad) *flag = 1;
  }
  __syncthreads();
  if (*flag) return 1;
  // W = A4^-1 A3, one thread per column, in place
  if (threadIdx.x < nt) {
    T* b = A3 + (long long)threadIdx.x * nb;
    for (int j = 0; j < nb; ++j) {
      const int p = piv[j];
      if (p != 0) { const T t = b[j]; b[j] = b[j + p]; b[j + p] = t; }
      const T* cj = AB + (long long)j * ld + kv;
      for (int i = 1; i <= min(kl, nb - 1 - j); ++i) b[j + i] = bfms(b[j + i], cj[i], b[j]);
    }
    for (int j = nb - 1; j >= 0; --j) {
      T s = b[j];
      for (int c = 1; c <= min(2 * kl, nb - 1 - j); ++c) s = bfms(s, AB[(long long)(j + c) * ld + kv - c], b[j + c]);
      b[j] = bmul(s, brcp(AB[(long long)j * ld + kv]));
    }
  }
  __syncthreads();
  // S = A1 - A2 W in A1
  if (threadIdx.x < nt * nt) {
    const int t = threadIdx.x / nt, u = threadIdx.x - t * nt;
    T s = A1[t * nt + u];
    for (int j = 0; j < nb; ++j) s = bfms(s, A2[(long long)t * nb + j], A3[(long long)u * nb + j]);
    A1[t * nt + u] = s;
  }
  __syncthreads();
  // S^-1 by Gauss-Jordan with partial pivoting (nt <= 4), one thread
  if (threadIdx.x == 0) {
    T a[4][8];
    for (int t = 0; t < nt; ++t)
      for (int u = 0; u < 2 * nt; ++u) a[t][u] = u < nt ? A1[t * nt + u] : bfrom(u - nt == t ? 1.0 : 0.0, T());
    int bad = 0;
    for (int c = 0; c < nt && !bad; ++c) {
      int p = c;
      for (int t = c + 1; t < nt; ++t)
        if (babs1(a[t][c]) > babs1(a[p][c])) p = t;
      if (!(babs1(a[p][c]) > 0.0)) { bad = 1; break; }
      for (int u = 0; u < 2 * nt; ++u) { const T x = a[c][u]; a[c][u] = a[p][u]; a[p][u] = x; }
      const T rp = brcp(a[c][c]);
      for (int u = 0; u < 2 * nt; ++u) a[c][u] = bmul(a[c][u], rp);
      for (int t = 0; t < nt; ++t) {
        if (t == c) continue;
        const T f = a[t][c];
        for (int u = 0; u < 2 * nt; ++u) a[t][u] = bfms(a[t][u], f, a[c][u]);
      }
    }
    if (bad) *flag = 1;
    else
      for (int t = 0; t < nt; ++t)
        for (int u = 0; u < nt; ++u) A1[t * nt + u] = a[t][nt + u];
  }
  __syncthreads();
  if (*flag) return 1;
  // the record
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    T* r = out + (long long)j * R;
    r[0] = brcp(AB[(long long)j * ld + kv]);
    for (int c = 1; c <= 2 * kl; ++c) r[c] = j + c < nb ? AB[(long long)(j + c) * ld + kv - c] : zero;
    for (int i = 1; i <= kl; ++i) r[2 * kl + i] = j + i < nb ? AB[(long long)j * ld + kv + i] : zero;
    r[3 * kl + 1] = bfrom((double)piv[j], T());
  }
  T* o2 = out + (long long)nb * R;
  for (long long q = threadIdx.x; q < 2LL * nt * nb; q += blockDim.x) o2[q] = q < (long long)nt * nb ? A2[q] : A3[q - (long long)nt * nb];
  T* o3 = o2 + 2LL * nt * nb;
  for (int q = threadIdx.x; q < nt * nt + n; q += blockDim.x) o3[q] = q < nt * nt ? A1[q] : fs[q - nt * nt];
  __syncthreads();
  return 0;
}

// -- solve --------------------------------------------------------------------
template <class T> struct BordCol;
// a real operator applied to one part (re or im) of a complex vector
template <> struct BordCol<double> {
  double* p;
  __device__ BordCol(double2* b, int comp) : p(reinterpret_cast<double*>(b) + comp) {}
  __device__ __forceinline__ double ld(int j) const { return p[2 * j]; }
  __device__ __forceinline__ void st(int j, double v) const { p[2 * j] = v; }
};
template <> struct BordCol<double2> {
  double2* p;
  __device__ BordCol(double2* b, int) : p(b) {}
  __device__ __forceinline__ double2 ld(int j) const { return p[j]; }
  __device__ __forceinline__ void st(int j, double2 v) const { p[j] = v; }
};

// y2 = A4^-1 b2 in place (b2 of length nb) with the rows of the record (rec,
// in shared memory): forward elimination with the pivots, then back
// substitution; a window of the band in registers
template <class T, int KL>
__device__ __forceinline__ void bord_sweep(const T* __restrict__ rec, int nb, const BordCol<T>& b) {
  constexpr int R = 3 * KL + 2;
  const T zero = bz(T());
  T w[KL + 1];
#pragma unroll
  for (int i = 0; i <= KL; ++i) w[i] = i < nb ? b.ld(i) : zero;
  for (int j = 0; j < nb; ++j) {
    const T* r = rec + (long long)j * R;
    const int p = (int)bre(r[3 * KL + 1]);
    T pv = w[0];
#pragma unroll
    for (int q = 1; q <= KL; ++q)
      if (p == q) { pv = w[q]; w[q] = w[0]; }
    b.st(j, pv);
#pragma unroll
    for (int i = 1; i <= KL; ++i) w[i] = bfms(w[i], r[2 * KL + i], pv);
#pragma unroll
    for (int i = 0; i < KL; ++i) w[i] = w[i + 1];
    w[KL] = j + KL + 1 < nb ? b.ld(j + KL + 1) : zero;
  }
  // back substitution: the older solution values y(j + 2 .. j + 2 KL) are
  // read back from shared memory (stored at least two rows earlier), only the
  // newest y(j + 1) is carried in a register; two chains, the newest term last
  T u0 = zero;
  for (int j = nb - 1; j >= 0; --j) {
    const T* r = rec + (long long)j * R;
    T sa = b.ld(j), sb = zero;
#pragma unroll
    for (int c = 2 * KL; c >= 2; c -= 2) {
      if (j + c < nb) sa = bfms(sa, r[c], b.ld(j + c));
      if (c - 1 >= 2 && j + c - 1 < nb) sb = bfms(sb, r[c - 1], b.ld(j + c - 1));
    }
    T s = badd(sa, sb);            // sb holds minus its terms
    s = bfms(s, r[1], u0);
    s = bmul(s, r[0]);
    b.st(j, s);
    u0 = s;
  }
}

template <class T, int KL>
__device__ void bord_solve_k(const T* __restrict__ gr, int n, int nt, const double2* x, double2* y, T* st,
                             double* red) {
  constexpr int R = 3 * KL + 2;
  const int nb = n - nt;
  const T* A2 = gr + (long long)nb * R;
  const T* W = A2 + (long long)nt * nb;
  const T* Si = W + (long long)nt * nb;
  const T* fs = Si + nt * nt;
  for (long long q = threadIdx.x; q < (long long)nb * R; q += blockDim.x) st[q] = gr[q];
  for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = cscale(bre(fs[i]), x[i]);
  __syncthreads();
  constexpr bool real_op = sizeof(T) == sizeof(double);
  if (threadIdx.x < (real_op ? 2 : 1)) bord_sweep<T, KL>(st, nb, BordCol<T>(y + nt, threadIdx.x));
  __syncthreads();
  // border: r_t = b1_t - A2_t y2, one warp per tau row (the block may have
  // fewer warps than tau rows)
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int t = threadIdx.x >> 5; t < nt; t += nw) {
    double ar = 0.0, ai = 0.0;
    for (int j = lane; j < nb; j += 32) {
      const double2 v = bmul(A2[(long long)t * nb + j], y[nt + j]);
      ar += v.x; ai += v.y;
    }
    ar = warp_sum(ar); ai = warp_sum(ai);
    if (lane == 0) { red[2 * t] = y[t].x - ar; red[2 * t + 1] = y[t].y - ai; }
  }
  __syncthreads();
  if (threadIdx.x < nt) {
    double2 s = make_double2(0.0, 0.0);
    for (int u = 0; u < nt; ++u) {
      const double2 v = bmul(Si[threadIdx.x * nt + u], make_double2(red[2 * u], red[2 * u + 1]));
      s.x += v.x; s.y += v.y;
    }
    y[threadIdx.x] = s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    double2 s = y[nt + i];
    for (int t = 0; t < nt; ++t) {
      const double2 v = bmul(W[(long long)t * nb + i], y[t]);
      s.x -= v.x; s.y -= v.y;
    }
    y[nt + i] = s;
  }
  __syncthreads();
}

// y = A^-1 x (x, y: n complex values in shared memory, distinct), with the
// record gr of the system (global memory), kl from bord_kl; st: shared
// staging space of (n - nt) (3 kl + 2) T; red: 2 nt doubles of shared memory.
template <class T>
__device__ void bord_solve(const T* gr, int n, int nt, int kl, const double2* x, double2* y, T* st, double* red) {
  if (kl == 2) bord_solve_k<T, 2>(gr, n, nt, x, y, st, red);
  else if (kl == 4) bord_solve_k<T, 4>(gr, n, nt, x, y, st, red);
  else bord_solve_k<T, 8>(gr, n, nt, x, y, st, red);
}

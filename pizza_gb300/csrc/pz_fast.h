// Tensor-core stage of the collocation influence-matrix step ("fast path").
//
// The per-m solves of update_temp_co and update_om_coll_dmat
// (src/update_temp_coll.f90:66-150, src/update_psi_coll_dmat.f90:126-466)
// are linear maps with operators that depend on (N, m) and on the implicit
// weight w = wimp_lin(1) only through one scalar:
//
//   (I - w k P) phi = rhs   on the interior collocation points,
//   P = D2p + r^-1 D1p - m^2 r^-2      (physical-space Laplacian, Dirichlet rows),
//
// with k = TdiffFac (temperature) or ViscFac (vorticity).  With P restricted
// to the interior points diagonalised once per (N, m), P_II = U diag(lam) U^-1,
// the solve for any w is phi_I = U diag(1/(1 - w k lam)) U^-1 rhs_I, so a dt
// change rebuilds nothing.  Every product of the stage is then with an
// operator shared by all instances of the same (N, radratio) and m, and a
// block of k_fast runs one m for a group of such instances.
//
// The products run on bf16 tensor cores as an exact emulation of FP64
// (Ozaki's splitting): each FP64 row of an operator (column of a vector
// block) is scaled by its own power of two and cut into PZ_OZ_S signed 8-bit
// integer slices (bf16 holds integers up to 256 exactly).  The products of
// two slices, summed over at most 128 terms, stay below 2^24 and accumulate
// exactly in fp32; the slice pairs with kA + kx <= PZ_OZ_S - 1 (56 bits of
// the operands) are summed in FP64.  Only the operands' truncation to 56
// bits relative to their row/column maximum is inexact, which is below FP64
// rounding of the products.
#pragma once
#include <stdint.h>

#define PZ_OZ_S 7            // bf16 slices per operand (8 bits each)
#define PZ_FAST_MAXN 97      // exact fp32 accumulation bound on the product length
#define PZ_FAST_G 8          // default instances per k_fast block
#define PZ_FAST_GMAX 16      // largest instances per k_fast block
#define PZ_FAST_KPL ((PZ_FAST_MAXN - 2 + 31) / 32)   // interior points per lane of a warp

// One operator stored for the tensor cores: R x K, RT = ceil(R/16) row tiles,
// KT = ceil(K/16) k tiles.  frag holds, for each (row tile, k tile, slice),
// the 32 lanes' mma.sync m16n8k16 A fragments (4 x uint32 = 8 bf16 per lane)
// contiguously: uint4 index ((rt * KT + kt) * PZ_OZ_S + s) * 32 + lane.
// ex[r] is the power of two of row r: A(r, j) = sum_s a_s(r, j) 2^(ex[r] - 8 (s + 1)).
struct PzOzOp {
  long long frag;   // offset in uint4 units into PzFastDev::frag
  long long ex;     // offset in ints into PzFastDev::ex
  int R, K, RT, KT;
};

// Operators and vectors of one m of a (N, radratio) class.
struct PzFastM {
  PzOzOp uinv;      // U^-1, n x n
  PzOzOp s3t;       // [U; D1p[:, I] U], (n + N) x n: temperature (interior) and dT/dr
  PzOzOp s3w;       // [U; K U; D1p[:, I] K U], (2n + N) x n: vorticity (interior), psi (interior), dpsi/dr
  long long vec;    // offset in doubles into PzFastDev::vec: lam, gtop, gbot, qt, qb (n each)
};

// A (N, radratio) class: the instances of one grid, and m < Mc.
struct PzFastCls {
  int N, n, Mc;
  PzOzOp d1p;       // D1p, N x N (explicit terms)
  long long m0;     // index of m = 0 in PzFastDev::ms
};

// u_phi (m = 0) operator of one (N, radratio, ViscFac, CorFac, Ekman pumping) class:
// I - w Pu, Pu = ViscFac (D2p + r^-1 D1p - r^-2) - CorFac ekpump
struct PzFastU {
  PzOzOp uinv;      // n x n
  PzOzOp s3u;       // [U; D1p[:, I] U], (n + N) x n
  long long vec;    // lam (n)
};

// A block's work: m of class cls for instances fi[i0 .. i0 + ni).  For
// m = 0 the group also shares one u_phi class (ucls).
struct PzFastItem { int cls, m, ucls, i0, ni; };

struct PzFastDev {
  const uint4* frag;
  const int* ex;
  const double* vec;
  const PzFastCls* cls;
  const PzFastM* ms;
  const PzFastU* us;
  const PzFastItem* items; int n_items;
  const int* fi;        // instance lists of the items
  int G;                // instances per block (column groups)
  int smem;             // dynamic shared memory of k_fast (bytes)
};

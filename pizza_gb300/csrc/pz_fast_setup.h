// Host set-up of the tensor-core stage (pz_fast_setup.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "pz_fast.h"

// Host image of the fast-path operators, uploaded as one block per handle.
struct PzFastHost {
  std::vector<uint4> frag;
  std::vector<int> ex;
  std::vector<double> vec;
  std::vector<PzFastCls> cls;
  std::vector<PzFastM> ms;
  std::vector<PzFastU> us;
};

// One grid: N Gauss-Lobatto points, the physical-space derivative operators
// (column-major N x N) and the radial functions the operators need.
struct PzFastGrid {
  int N;
  const double* D1p;
  const double* D2p;
  const double* or1;
  const double* or2;
  const double* beta;
  const double* dbeta;
};

// A = U diag(lam) U^-1 (row-major n x n) for a real matrix with real, distinct
// eigenvalues; false when the decomposition fails or does not reproduce A to
// 1e-10 relative.
bool pz_eig_real(int n, const std::vector<double>& A, std::vector<double>& lam, std::vector<double>& U,
                 std::vector<double>& Uinv);

// Interior Laplacian of mode m (m2 = m^2): P (n x n, row-major) =
// [D2p + r^-1 D1p]_II - m^2 r^-2 on the interior points, Pb (n x 2) its
// columns of the two wall values (r_cmb, r_icb).
void pz_fast_laplacian(const PzFastGrid& g, double m2, std::vector<double>& P, std::vector<double>& Pb);

// Operators of m = 0 .. Mc-1 (m = index * minc) of one grid; *index receives
// the class.  False when an eigen-decomposition or the psi operator fails.
bool pz_fast_add_class(PzFastHost& H, const PzFastGrid& g, int Mc, int minc, int* index);

// The m = 0 u_phi operator ViscFac (D2p + r^-1 D1p - r^-2) - CorFac ekpump.
bool pz_fast_add_uclass(PzFastHost& H, const PzFastGrid& g, double visc, double corfac, const double* ekpump,
                        int* index);

"""pizza's bordered band LU for the tau-bordered systems of the integration
method: the restatement of prepare_bordered_mat and solve_bordered_mat
(src/algebra_lapack.f90:216-286, :332-416), as the type_bordmat_* matrices of
src/bordered_matrix.f90:127-183 and :251-275 call them.

Test infrastructure only (the checker of the GPU's banded integ solves,
pz_integ_banded(1)).

The matrix is [[A1, A2], [A3, A4]] with A1 the ntau x ntau block of the tau
rows' first columns and A4 banded.  The factorisation is the reference's:
LU of A4 in LAPACK band storage with partial pivoting (gbtrf), v = A4^-1 A3
(gbtrs), the Schur complement S = A1 - A2 v and its LU (getrf).  A solve is
w = A4^-1 b2, b1 - A2 w, x1 = S^-1 (b1 - A2 w), x2 = w - v x1.  LAPACK is the
reference's own third-party dependency for these steps; scipy exposes the
same routines.  The band widths kl, ku are the actual ones of A4 (the
reference fixes them per operator family; wider bands only add zero
diagonals, which never become pivots).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
from scipy.linalg import lapack


class BorderedLU:
    """Factors of a bordered matrix A (n x n, real or complex) whose first
    ``ntau`` rows are dense tau rows and whose lower-right block is banded."""

    def __init__(self, A: np.ndarray, ntau: int):
        A = np.asarray(A)
        n = A.shape[0]
        self.ntau = nt = ntau
        self.cplx = np.iscomplexobj(A)
        dt = complex if self.cplx else float
        A4 = A[nt:, nt:]
        nz = np.nonzero(A4)
        off = nz[0] - nz[1]
        self.kl = kl = int(max(0, off.max())) if off.size else 0
        self.ku = ku = int(max(0, (-off).max())) if off.size else 0
        nb = n - nt
        # LAPACK band storage with kl rows of room for the fill of the pivoting
        ab = np.zeros((2 * kl + ku + 1, nb), dt)
        for j in range(nb):
            i0, i1 = max(0, j - ku), min(nb, j + kl + 1)
            ab[kl + ku + np.arange(i0, i1) - j, j] = A4[i0:i1, j]
        gbtrf = lapack.zgbtrf if self.cplx else lapack.dgbtrf
        self.gbtrs = lapack.zgbtrs if self.cplx else lapack.dgbtrs
        lub, piv, info = gbtrf(ab, kl, ku)
        if info != 0:
            raise np.linalg.LinAlgError("Singular banded block in the bordered solve")
        self.lub, self.piv = lub, piv
        self.A2 = np.array(A[:nt, nt:], dt)
        v, info = self.gbtrs(lub, kl, ku, np.array(A[nt:, :nt], dt), piv)
        self.v = v
        S = np.array(A[:nt, :nt], dt) - self.A2 @ v
        self.S = sla.lu_factor(S)

    def solve(self, b: np.ndarray) -> np.ndarray:
        """x = A^-1 b for one right-hand side (complex b with a real matrix is
        solved as its real and imaginary parts, as the reference does)."""
        if not self.cplx and np.iscomplexobj(b):
            return self.solve(b.real.copy()) + 1j * self.solve(b.imag.copy())
        nt = self.ntau
        w, info = self.gbtrs(self.lub, self.kl, self.ku, np.array(b[nt:]), self.piv)
        x1 = sla.lu_solve(self.S, b[:nt] - self.A2 @ w)
        return np.concatenate([x1, w - self.v @ x1])

"""Host eigen-decompositions of the tensor-core stage (pz_fast_eigen), no GPU.

The stage solves (I - w k P) phi = rhs on the interior collocation points in
the eigenbasis of the interior Laplacian P of each m.  The library builds
that decomposition itself at pz_create (Householder-Hessenberg reduction,
shifted QR, inverse iteration); it is checked here against the Laplacian
the oracle's collocation matrices define (src/update_psi_coll_dmat.f90:864-873:
interior rows of rMat - w ViscFac (d2rMat + or1 drMat - m^2 or2 rMat), the
Dirichlet rows of rMat) and against LAPACK's eigenvalues.
"""
import numpy as np
import pytest

import pizza_gb300 as pz
from oracle.pizza_oracle import Params, Pizza


def oracle_laplacian(N, m, radratio=0.35):
    sim = Pizza(Params(n_r_max=N, n_cheb_max=N, m_max=32, ek=1e-3, ra=1e5, radratio=radratio, dtMax=1e-4,
                       matrix_solve="INFLUENCE"))
    c = sim.cheb
    i = slice(1, N - 1)
    A0 = c.rnorm * c.rMat.copy()
    A1 = np.zeros((N, N))
    A1[i] = c.rnorm * (c.d2rMat[i] + sim.or1[i, None] * c.drMat[i] - float(m * m) * sim.or2[i, None] * c.rMat[i])
    for A in (A0, A1):
        A[:, 0] *= c.boundary_fac
        A[:, N - 1] *= c.boundary_fac
    P = A1 @ np.linalg.inv(A0)          # physical-space operator; rows 0 and N-1 vanish
    return P[1:N - 1, 1:N - 1]


@pytest.mark.parametrize("N,m", [(33, 0), (33, 1), (33, 32), (49, 7), (65, 0), (65, 64), (97, 40)])
def test_eigen_decomposition_reproduces_the_laplacian(N, m):
    lam, U = pz.fast_eigen(N, 0.35, m)
    P = oracle_laplacian(N, m)
    scale = np.max(np.abs(P))
    assert np.max(np.abs(P @ U - U * lam[None, :])) <= 1e-11 * scale
    ref = np.sort(np.linalg.eigvals(P).real)
    got = np.sort(lam)
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))
    assert np.all(lam < 0.0)                     # Dirichlet Laplacian: negative spectrum
    assert np.allclose(np.max(np.abs(U), axis=0), 1.0)
    assert np.linalg.cond(U) < 1e3


def test_fast_path_switch_round_trips():
    prev = pz.fast_path(None)
    assert pz.fast_path(False) == prev
    assert pz.fast_path(None) is False
    pz.fast_path(prev)
    assert pz.fast_path(None) == prev

"""The oracle's restatement of pizza's bordered band LU (oracle/bordered.py,
src/algebra_lapack.f90:216-286, :332-416) against dense solves, and both
against a 40-digit solve of the integration method's row-scaled tau systems
at n_r_max = 97, E = 1e-5 (the case where the GPU's banded path and the
dense oracle part by up to 1e-7 after 25 steps)."""
import numpy as np
import pytest

from oracle.bordered import BorderedLU
from oracle.pizza_oracle import Params, Pizza


def _bordered(rng, n, nt, bw, cplx):
    A = np.zeros((n, n), complex if cplx else float)
    for i in range(nt, n):
        j0, j1 = max(0, i - bw), min(n, i + bw + 1)
        A[i, j0:j1] = rng.standard_normal(j1 - j0)
        if cplx:
            A[i, j0:j1] += 1j * rng.standard_normal(j1 - j0)
        A[i, i] += 4.0 * bw
    A[:nt] = rng.standard_normal((nt, n))
    return A


@pytest.mark.parametrize("cplx", [False, True])
def test_bordered_lu_solves_like_dense(cplx):
    rng = np.random.default_rng(11)
    for n, nt, bw in ((33, 2, 4), (65, 4, 8), (97, 4, 6)):
        A = _bordered(rng, n, nt, bw, cplx)
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        F = BorderedLU(A, nt)
        assert F.kl == bw and F.ku == bw
        x = F.solve(b)
        ref = np.linalg.solve(A, b)
        assert np.max(np.abs(x - ref)) < 1e-12 * np.max(np.abs(ref))


def test_bordered_against_exact_n97():
    mp = pytest.importorskip("mpmath")
    spec = dict(n_r_max=97, n_cheb_max=97, m_max=32, ek=1e-5, ra=3e7, dtMax=2e-6, time_scheme="SBDF3",
                l_ek_pump=True, cheb_method="INTEG", matrix_solve="DIRECT", radratio=0.35)
    sim = Pizza(Params(**spec))
    sim.start()
    systems = []
    finish = sim.integ._finish_lhs
    sim.integ._finish_lhs = lambda A, nt: (systems.append((A.copy(), nt)), finish(A, nt))[1]
    sim.integ.build_matrices()
    M = sim.M
    mp.mp.dps = 40
    rng = np.random.default_rng(3)
    errs = {}
    for name, idx in (("temperature m=5", 5), ("u_phi m=0", M), ("psi m=7", M + 7)):
        A, nt = systems[idx]
        A = A.copy()
        A[:nt, 0] *= sim.cheb.boundary_fac
        A = A * (1.0 / np.max(np.abs(A), axis=1))[:, None]     # get_lhs_mat_tau's row scaling
        n = A.shape[0]
        x = np.zeros(n, complex)
        x[nt:] = rng.standard_normal(n - nt) + 1j * rng.standard_normal(n - nt)
        Am = mp.matrix([[mp.mpc(complex(A[i, j]).real, complex(A[i, j]).imag) for j in range(n)] for i in range(n)])
        ye = mp.lu_solve(Am, mp.matrix([mp.mpc(v.real, v.imag) for v in x]))
        ye = np.array([complex(ye[i]) for i in range(n)])
        s = np.max(np.abs(ye))
        errs[name] = (np.max(np.abs(BorderedLU(A, nt).solve(x) - ye)) / s,
                      np.max(np.abs(np.linalg.solve(A, x) - ye)) / s)
    # the two-tau-row systems: both near FP64 rounding; the four-tau-row
    # streamfunction system: the bordered elimination loses two more digits
    for name in ("temperature m=5", "u_phi m=0"):
        assert errs[name][0] < 1e-13 and errs[name][1] < 1e-13, (name, errs[name])
    eb, ed = errs["psi m=7"]
    assert ed < 1e-13 and 1e-13 < eb < 1e-10, errs


_BORDERED_RUNS = {}


def _bordered_run(case):
    """The bordered-solve oracle's run of a fixture case (a continuation case
    restarts from its first run's final state, as in test_oracle_golden)."""
    import json
    import os
    from tests.test_oracle_golden import checkpoint_of
    if case not in _BORDERED_RUNS:
        here = os.path.dirname(os.path.abspath(__file__))
        with open(os.path.join(here, "golden", "cases.json")) as f:
            spec = json.load(f)[case]
        sim = Pizza(Params(**spec["params"]), integ_bordered=True)
        if "restart_from" in spec:
            sim.start_from_checkpoint(checkpoint_of(_bordered_run(spec["restart_from"])[0]))
        else:
            sim.start()
        _BORDERED_RUNS[case] = (sim, sim.run()[spec["series"]])
    return _BORDERED_RUNS[case]


@pytest.mark.parametrize("case", ["RotInteg", "RotIntegContinue", "FingConv"])
def test_bordered_oracle_matches_reference_fixture(case):
    """pizza.exe solved these integration-method runs (the direct solve, and
    the influence-matrix solve of the continuation on N = 97) with its
    bordered LU; the oracle with the restated bordered solve reproduces their
    time series at the reference harness's rtol 1e-8 as the dense-LU oracle
    does."""
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    ref = np.loadtxt(os.path.join(here, "golden", f"{case}.txt"))
    rows = _bordered_run(case)[1]
    assert rows.shape == ref.shape
    np.testing.assert_allclose(rows, ref, rtol=1e-8, atol=1e-20)

"""DIRK schemes of the oracle (src/dirk_schemes.f90) on the CPU.

The ARS222 run of the reference's DIRKSchemes fixture pins the stage loop
(tests/test_oracle_golden.py).  The other tableaux, and the assembly stage,
have no fixture; they are checked here by the conditions every tableau meets
and by the temporal convergence order of a short run.
"""
import numpy as np
import pytest

from oracle.pizza_oracle import DIRK_SCHEMES, Params, Pizza, dirk_tableau, seeded_temperature


@pytest.mark.parametrize("name", DIRK_SCHEMES)
def test_tableau_weights(name):
    t = dirk_tableau(name)
    ns = t["nstages"]
    last_i = t["bass_imp"] if t["l_assembly"] else t["bimp"][-1]
    last_e = t["bass_exp"] if t["l_assembly"] else t["bexp"][-1]
    assert abs(last_i.sum() - 1.0) < 1e-12 and abs(last_e.sum() - 1.0) < 1e-12
    # explicit part strictly lower triangular; implicit diagonal gamma from stage 2 on
    assert np.all(np.triu(t["bexp"]) == 0.0)
    assert np.all(np.triu(t["bimp"], 1) == 0.0)
    for s in range(1, min(ns, t["bimp"].shape[0] - 1) + 1):
        assert t["bimp"][s, s] == t["gamma"]
    assert len(t["l_exp_calc"]) == ns and len(t["l_imp_calc_rhs"]) == ns


T_END = 2e-3


def _run(scheme, nst):
    p = Params(n_r_max=13, n_cheb_max=13, m_max=6, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
               time_scheme=scheme, dtMax=T_END / nst, matrix_solve="DIRECT")
    sim = Pizza(p)
    sim.start(temp0=seeded_temperature(sim.M, sim.r, sim.d["r_icb"], 5e-2, 1))
    sim.dt_schedule = [T_END / nst] * nst
    for _ in range(nst):
        sim.advance()
    return sim


@pytest.fixture(scope="module")
def reference():
    return _run("ARS443", 256)


@pytest.mark.parametrize("name,order", [("ARS222", 2), ("LZ232", 2), ("ARS443", 3), ("BPR353", 3),
                                        ("DP2-242", 2), ("LZ453", 3)])
def test_convergence_order(reference, name, order):
    e = [np.abs(_run(name, n).temp - reference.temp).max() for n in (16, 32)]
    assert np.log2(e[0] / e[1]) > order - 0.3, e


@pytest.mark.parametrize("name", ["ARS233", "KC343", "KC564"])
def test_assembly_scheme_temperature_converges(reference, name):
    """ARS233 and the Kennedy-Carpenter schemes end with pizza's assembly
    stage; their temperature converges at better than second order (the
    velocity has the assembly's vorticity projection at the walls)."""
    e = [np.abs(_run(name, n).temp - reference.temp).max() for n in (16, 32)]
    assert np.log2(e[0] / e[1]) > 2.0, e


def test_ssp433_literals_are_single_precision():
    """dirk_schemes.f90 writes SSP433's alpha, beta and eta without a kind:
    they are single-precision literals widened to double."""
    t = dirk_tableau("SSP433")
    assert t["gamma"] == float(np.float32(0.24169426078821))
    assert t["gamma"] != 0.24169426078821

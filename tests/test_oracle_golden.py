"""The oracle against the reference's own regression fixtures.

The fixtures (tests/golden/*.txt, extracted by tests/golden/make_golden.py from
samples/*/reference.out) are the time series pizza.exe wrote for the
collocation and integration runs listed in tests/golden/cases.json; a
continuation case restarts from its first run's final state.  The reference's
test harness compares them with np.testing.assert_allclose(rtol=1e-8,
atol=1e-20) (samples/NonRotRa2e3/unitTest.py:87-89); so does this test.
"""
import json
import os

import numpy as np
import pytest

from oracle.pizza_oracle import Params, Pizza

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "cases.json")) as f:
    CASES = json.load(f)


_RUNS = {}


def oracle_run(case):
    """The oracle's run of a fixture case (cached: a continuation case starts
    from the final state of the run it restarts from)."""
    if case not in _RUNS:
        spec = CASES[case]
        sim = Pizza(Params(**spec["params"]))
        if "restart_from" in spec:
            sim.start_from_checkpoint(checkpoint_of(oracle_run(spec["restart_from"])))
        else:
            sim.start()
        rows = sim.run()[spec["series"]]
        _RUNS[case] = (sim, rows)
    return _RUNS[case][0]


def checkpoint_of(sim):
    """What write_checkpoint_mloc stores of a multistep run, as the oracle's
    reader takes it: header, fields (composition too when the run has it)
    and history slots 2..n."""
    ts, d = sim.ts, sim.d
    order = ([("expl", k) for k in range(2, ts.nexp + 1)] + [("impl", k) for k in range(2, ts.nimp + 1)]
             + [("old", k) for k in range(2, ts.nold + 1)])
    return {"header": dict(time=sim.time, family=ts.family, nexp=ts.nexp, nimp=ts.nimp, nold=ts.nold,
                           dt=ts.dt.copy(), ek=d["ek"], n_r_max=sim.N, l_cheb_coll=d["l_cheb_coll"]),
            "us": sim.us.copy(), "up": sim.up.copy(), "temp": sim.temp.copy(),
            "hist_P": [getattr(sim.dpsidt, k)[s - 1].copy() for k, s in order],
            "hist_T": [getattr(sim.dTdt, k)[s - 1].copy() for k, s in order],
            "xi": sim.xi.copy() if sim.l_chem else None,
            "hist_Xi": [getattr(sim.dxidt, k)[s - 1].copy() for k, s in order] if sim.l_chem else []}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_matches_reference_fixture(case):
    ref = np.loadtxt(os.path.join(HERE, "golden", f"{case}.txt"))
    oracle_run(case)
    rows = _RUNS[case][1]
    assert rows.shape == ref.shape
    # the reference harness's own tolerances; the exact zeros it printed come
    # from round_off (|x| < 10 epsilon -> 0, src/useful.f90:222-233)
    np.testing.assert_allclose(rows, ref, rtol=1e-8, atol=1e-20)

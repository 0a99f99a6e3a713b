"""The oracle against the reference's own regression fixtures.

The fixtures (tests/golden/*.txt, extracted by tests/golden/make_golden.py from
samples/*/reference.out) are the time series pizza.exe wrote for four
collocation runs.  The reference's test harness compares them with
np.testing.assert_allclose(rtol=1e-8, atol=1e-20)
(samples/NonRotRa2e3/unitTest.py:87-89); the same rtol is used here.
"""
import json
import os

import numpy as np
import pytest

from oracle.pizza_oracle import Params, Pizza

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "cases.json")) as f:
    CASES = json.load(f)


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_matches_reference_fixture(case):
    spec = CASES[case]
    ref = np.loadtxt(os.path.join(HERE, "golden", f"{case}.txt"))
    sim = Pizza(Params(**spec["params"]))
    sim.start()
    rows = sim.run()[spec["series"]]
    assert rows.shape == ref.shape
    # the reference harness's own tolerances; the exact zeros it printed come
    # from round_off (|x| < 10 epsilon -> 0, src/useful.f90:222-233)
    np.testing.assert_allclose(rows, ref, rtol=1e-8, atol=1e-20)

"""The tensor-core stage (k_fast) against the dense FP64 kernels and the oracle
(needs a GB300).

Instances that run the collocation step with the influence-matrix solve and
CNAB2 take the fast path by default; pz_fast_path(0) keeps a handle created
afterwards on the dense kernels.  Both must give the oracle's step to FP64
rounding, so they agree with each other far below the 1e-10 parity bar.
"""
import os
import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, rel_err, seeded

pytestmark = pytest.mark.gpu

SPECS = [
    dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1e5, l_ek_pump=True, dtMax=1e-4, matrix_solve="INFLUENCE"),
    dict(n_r_max=65, n_cheb_max=65, m_max=96, ek=1e-4, ra=3e6, l_ek_pump=True, dtMax=2e-5, courfac=2.0,
         matrix_solve="INFLUENCE"),
    dict(n_r_max=49, n_cheb_max=49, m_max=64, ek=1e-3, ra=1e6, pr=0.7, l_ek_pump=True, dtMax=5e-5, courfac=2.0,
         matrix_solve="INFLUENCE"),
    dict(n_r_max=48, n_cheb_max=48, m_max=42, ek=1e-3, ra=2e4, l_non_rot=True, dtMax=1e-4,
         matrix_solve="INFLUENCE"),
]


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def _run(pz, specs, temps, steps, fast):
    prev = pz.fast_path(fast)
    try:
        ens = pz.Ensemble([gpu_config(s) for s in specs])
    finally:
        pz.fast_path(prev)
    ens.set_state_all(temps)
    ens.step(steps)
    return ens


def test_fast_path_is_used_and_matches_dense_path(pz):
    temps = [seeded(s, 50 + i) for i, s in enumerate(SPECS)]
    fast = _run(pz, SPECS, temps, 60, True)
    dense = _run(pz, SPECS, temps, 60, False)
    assert fast.profile_steps(1)["k_fast"] > 0.0
    assert dense.profile_steps(1)["k_fast"] == 0.0
    assert fast.launches_per_step() == 4          # k_rloop, k_cfl, k_fast, k_obs
    for i in range(len(SPECS)):
        a, b = fast.get_state(i), dense.get_state(i)
        for f in ("temp", "us", "up", "om", "psi", "dtemp"):
            assert rel_err(a[f], b[f]) < 1e-11, (i, f, rel_err(a[f], b[f]))
        assert a["dt"] == b["dt"] and abs(a["time"] - b["time"]) <= 1e-15


def test_fast_path_matches_oracle_with_dt_changes(pz):
    """Courant-driven dt changes: the eigen-basis solve takes the new weight
    at once (no operator rebuild)."""
    spec = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=3e5, l_ek_pump=True, dtMax=1e-4, courfac=10.0,
                matrix_solve="INFLUENCE")
    t0 = seeded(spec, 2, 3e-3)
    sim = oracle(spec, temp0=t0)
    ens = _run(pz, [spec], [t0], 150, True)
    for _ in range(150):
        sim.advance()
    g = ens.get_state(0)
    assert g["dt"] != spec["dtMax"]
    assert abs(g["dt"] - sim.ts.dt[0]) <= 1e-12 * sim.ts.dt[0]
    for f in ("temp", "us", "up", "om"):
        assert rel_err(g[f], getattr(sim, f)) < 1e-10, f


def test_mixed_fast_and_dense_instances_in_one_graph(pz):
    """A handle with fast instances and instances on the dense kernels
    (SBDF3, DIRECT, a DIRK scheme): each matches the oracle."""
    specs = [SPECS[0], dict(SPECS[0], time_scheme="SBDF3"), dict(SPECS[0], matrix_solve="DIRECT"),
             dict(SPECS[0], time_scheme="ARS222"), SPECS[3]]
    temps = [seeded(s, 70 + i) for i, s in enumerate(specs)]
    ens = _run(pz, specs, temps, 20, True)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i])
        for _ in range(20):
            sim.advance()
        g = ens.get_state(i)
        for f in ("temp", "us", "up", "om"):
            assert rel_err(g[f], getattr(sim, f)) < 1e-10, (i, f)


@pytest.mark.gpu
def test_lanes_change_nothing_but_the_schedule(pz):
    """The 256-instance bench handle stepped as two lanes (the default) and as
    one: the same kernels over the same instances, so the same bits."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    specs = bench.ensemble_specs(256)
    temps = [bench.seeded_temp(s) for s in specs]
    states = []
    for lanes in (2, 1):
        pz.tune_set(pz.TUNE_LANES, 0, lanes)
        try:
            e = pz.Ensemble([bench.gpu_cfg(s) for s in specs])
        finally:
            pz.tune_set(pz.TUNE_LANES, 0, 0)
        assert e.launches_per_step() == 4 * lanes
        e.set_state_all(temps)
        e.step(40)
        states.append(([e.get_state(i)["om"] for i in (0, 77, 255)], e.latest_rows()))
        e.close()
    for a, b in zip(states[0][0], states[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(states[0][1], states[1][1])

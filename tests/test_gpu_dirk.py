"""DIRK IMEX Runge-Kutta schemes (src/dirk_schemes.f90) on the GPU (needs a
GB300): the stage loop of time_loop with per-stage explicit terms and solves,
and the assembly stage of the schemes that have one, against the reference's
DIRKSchemes fixture (ARS222) and against the oracle for every scheme."""
import json
import os

import numpy as np
import pytest

from oracle.pizza_oracle import DIRK_SCHEMES
from tests.helpers import gpu_config, oracle, seeded
from tests.test_gpu_parity import run_pair, check_fields

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

C0 = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35,
          l_ek_pump=True, dtMax=1e-4)


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def test_golden_dirkschemes_ars222_on_gpu(pz):
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        spec = json.load(f)["DIRKSchemes"]
    p = dict(spec["params"])
    ref = np.loadtxt(os.path.join(HERE, "golden", "DIRKSchemes.txt"))
    sim = oracle(p)
    ens = pz.Ensemble(gpu_config(p))
    ens.set_state(0, temp=sim.temp.copy())
    n, nlog = p["n_time_steps"], p["n_log_step"]
    ens.step(n)
    got = ens.series(0, n + 1)[::nlog][:, [0, 4, 5, 6, 7]]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("solve", ["DIRECT", "INFLUENCE"])
@pytest.mark.parametrize("scheme", DIRK_SCHEMES)
def test_dirk_scheme_matches_oracle(pz, scheme, solve):
    spec = dict(C0, time_scheme=scheme, matrix_solve=solve)
    sim, ens, out = run_pair(pz, spec, 20, seed=3, checkpoints=(1,))
    for k, s, g in out:
        check_fields(s, g, 1e-10, f"{scheme}/{solve} step {k}")


def test_ars233_batched_workload_shape(pz):
    """Instances shaped like the batched adjoint workload (N in {49, 65},
    n_phi in {126, 192}, E=1e-4, Ra in [1e6, 1e7], ARS233)."""
    specs = [dict(n_r_max=49, n_cheb_max=49, m_max=42, ek=1e-4, ra=1.5e6, l_ek_pump=True, dtMax=2e-5,
                  time_scheme="ARS233", matrix_solve="INFLUENCE"),
             dict(n_r_max=65, n_cheb_max=65, m_max=64, ek=1e-4, ra=6e6, l_ek_pump=True, dtMax=1e-5,
                  time_scheme="ARS233", matrix_solve="INFLUENCE")]
    temps = [seeded(s, 30 + i) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    ens.set_state_all(temps)
    ens.step(10)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i])
        for _ in range(10):
            sim.advance()
        check_fields(sim, ens.get_state(i), 1e-9, f"instance {i}")


def test_mixed_dirk_and_multistep_batch(pz):
    """One graph for instances of different stage counts: stages past an
    instance's own are skipped."""
    specs = [dict(C0, time_scheme="CNAB2", matrix_solve="INFLUENCE"),
             dict(C0, time_scheme="ARS443"),
             dict(C0, time_scheme="ARS233", matrix_solve="INFLUENCE"),
             dict(C0, time_scheme="SBDF3")]
    temps = [seeded(s, 40 + i) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    ens.set_state_all(temps)
    ens.step(12)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i])
        for _ in range(12):
            sim.advance()
        check_fields(sim, ens.get_state(i), 1e-10, f"instance {i} ({s['time_scheme']})")
    prof = ens.profile_steps(2)
    assert prof["k_assemble"] > 0.0

"""CUDA library vs the oracle, through the C ABI (needs a GB300).

Parity bar: fields and time series agree with the FP64 oracle to 1e-10
relative (norm-wise: max |gpu - oracle| / max |oracle| per field), the
tolerance set for this FP64 path.  The GPU applies the
same linear operators as the reference (DCT-I, Chebyshev derivatives, LU
solves) as dense inverse operators; rounding differs at ~1e-14 per step.
"""
import json
import os

import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, rel_err, seeded, series_from_oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10
HERE = os.path.dirname(os.path.abspath(__file__))

C0 = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35,
          l_ek_pump=True, time_scheme="CNAB2", dtMax=1e-4, matrix_solve="INFLUENCE")


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def run_pair(pz, spec, nsteps, seed=1, amp=1e-3, temp0=None, checkpoints=()):
    if temp0 is None:
        temp0 = seeded(spec, seed, amp)
    sim = oracle(spec, temp0=temp0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=temp0)
    out = []
    done = 0
    for k in sorted(set(checkpoints) | {nsteps}):
        for _ in range(k - done):
            sim.advance()
        ens.step(k - done)
        done = k
        out.append((k, sim, ens.get_state(0)))
        if k != nsteps:
            out[-1] = (k, {f: getattr(sim, f).copy() for f in ("us", "up", "om", "temp")}, out[-1][2])
    return sim, ens, out


def check_fields(sim, g, tol=TOL, label=""):
    for f in ("temp", "us", "up", "om"):
        ref = getattr(sim, f) if not isinstance(sim, dict) else sim[f]
        e = rel_err(g[f], ref)
        assert e < tol, f"{label} {f}: rel err {e:.3e}"


def test_start_state_matches_oracle(pz):
    spec = C0
    temp0 = seeded(spec, 3)
    sim = oracle(spec, temp0=temp0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=temp0)
    g = ens.get_state(0)
    check_fields(sim, g, 1e-13, "start")
    assert rel_err(g["dtemp"], sim.dtemp) < 1e-12
    row = ens.series(0)[-1]
    ref = series_from_oracle(sim)
    assert np.allclose(row[:15], ref[:15], rtol=1e-12, atol=1e-300)


def test_c0_influence_cnab2_200_steps(pz):
    """The single-instance workload (N=33, m_max=32, E=1e-3, Ra=1e5, Ekman pumping, CNAB2)."""
    sim, ens, out = run_pair(pz, C0, 200, checkpoints=(1, 10))
    for k, s, g in out:
        check_fields(s, g, TOL, f"step {k}")
    rows = ens.series(0, 300)
    assert rows.shape[0] == 201
    ref = series_from_oracle(sim)
    np.testing.assert_allclose(rows[-1, :15], ref[:15], rtol=TOL, atol=1e-14)
    assert abs(ens.get_state(0)["time"] - sim.time) < 1e-15


def test_golden_timestepchange_on_gpu(pz):
    """The reference fixture TimeStepChange (dmat SBDF3, CFL dt changes, bubble)."""
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        spec = json.load(f)["TimeStepChange"]
    p = dict(spec["params"])
    ref = np.loadtxt(os.path.join(HERE, "golden", "TimeStepChange.txt"))
    sim = oracle(p)                       # bubble init (init_t=-1) built by the oracle
    temp0 = sim.temp.copy()
    cfg = {k: v for k, v in p.items() if k not in ("init_t", "amp_t")}
    ens = pz.Ensemble(gpu_config(cfg))
    ens.set_state(0, temp=temp0)
    rows = [ens.series(0)[-1]]
    for _ in range(20):
        ens.step(100)
        rows.append(ens.series(0)[-1])
    rows = np.array(rows)
    got = rows[:, [0, 1, 2, 3]]
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("scheme", ["SBDF2", "SBDF3", "SBDF4", "CNLF", "MODCNAB", "TVB33"])
def test_multistep_schemes(pz, scheme):
    spec = dict(C0, time_scheme=scheme)
    sim, ens, out = run_pair(pz, spec, 30, seed=5)
    check_fields(sim, out[-1][2], TOL, scheme)


def test_dt_change_rebuilds_operators(pz):
    """CFL-driven dt changes (hysteresis, dt_fac) rebuild the dt-dependent operators."""
    spec = dict(n_r_max=33, m_max=32, ek=1e-3, ra=3e5, l_ek_pump=True, dtMax=1e-4, courfac=10.0,
                matrix_solve="INFLUENCE")
    sim, ens, out = run_pair(pz, spec, 150, seed=2, amp=3e-3)   # dt changes 3 times
    g = out[-1][2]
    assert g["dt"] != spec["dtMax"], "the run must change dt"
    assert abs(g["dt"] - sim.ts.dt[0]) <= 1e-12 * sim.ts.dt[0]
    check_fields(sim, g, TOL, "dt change")


def test_ragged_batch_matches_independent_runs(pz):
    specs = [
        dict(n_r_max=33, m_max=32, ek=1e-3, ra=1e5, l_ek_pump=True, dtMax=1e-4, matrix_solve="INFLUENCE"),
        dict(n_r_max=49, m_max=64, ek=1e-4, ra=2e6, l_ek_pump=True, dtMax=2e-5, courfac=0.5,
             matrix_solve="INFLUENCE"),
        dict(n_r_max=65, m_max=96, ek=1e-3, ra=5e5, l_ek_pump=True, dtMax=5e-5, matrix_solve="INFLUENCE",
             time_scheme="SBDF3"),
        dict(n_r_max=48, m_max=42, ek=1e-3, ra=1e4, l_non_rot=True, dtMax=1e-4, matrix_solve="INFLUENCE"),
    ]
    temps = [seeded(s, 10 + i) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    ens.set_state_all(temps)
    ens.step(20)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i])
        for _ in range(20):
            sim.advance()
        check_fields(sim, ens.get_state(i), TOL, f"instance {i}")


def test_unsupported_and_invalid_configs_fail_loudly(pz):
    with pytest.raises(pz.PizzaError) as e:
        pz.Ensemble(pz.Config(n_r_max=33, m_max=32, minc=2, matrix_solve="INFLUENCE"))   # minc /= 1
    assert e.value.code == -6
    with pytest.raises(pz.PizzaError) as e:
        pz.Ensemble(pz.Config(n_r_max=3, m_max=32, matrix_solve="INFLUENCE"))
    assert e.value.code == -1


def test_nonfinite_state_is_reported(pz):
    """Failure detection without a GPU fault: a NaN planted in the host input
    is caught by the device status word after one step."""
    spec = C0
    t = seeded(spec, 1)
    t[3, 10] = np.nan
    ens = pz.Ensemble(gpu_config(spec))
    with pytest.raises(pz.PizzaError) as e:
        ens.set_state(0, temp=t)
        ens.step(1)
    assert e.value.code == -5


def test_explicit_terms_entry_point_matches_oracle(pz):
    """pz_explicit_terms on caller device arrays = the oracle's radial_loop +
    finish_explicit_assembly for the same state."""
    import torch
    spec = C0
    sim = oracle(spec, temp0=seeded(spec, 4))
    for _ in range(3):
        sim.advance()
    state = {f: getattr(sim, f).copy() for f in ("us", "up", "om", "temp")}
    sim.ts.istage = 1                       # stage 1 of the next step
    dtempdt, dVsT, dpsidt, dVsOm = sim.radial_loop()
    sim.dTdt.expl[0] = dtempdt
    sim.dpsidt.expl[0] = dpsidt
    sim.finish_explicit(dVsT, dVsOm)
    ens = pz.Ensemble(gpu_config(spec))
    dev = {f: torch.from_numpy(np.ascontiguousarray(state[f].T)).cuda() for f in state}
    torch.cuda.synchronize()
    for _ in range(2):
        out = ens.explicit_terms(0, dev["us"], dev["up"], dev["om"], dev["temp"])
        ens.sync()
        assert rel_err(out[0].cpu().numpy().T, sim.dTdt.expl[0]) < 1e-12
        assert rel_err(out[1].cpu().numpy().T, sim.dpsidt.expl[0]) < 1e-12
        np.testing.assert_allclose(out[2].cpu().numpy(), sim.dtr, rtol=1e-12)
        np.testing.assert_allclose(out[3].cpu().numpy(), sim.dth, rtol=1e-12)


@pytest.mark.parametrize("noalloc", [False, True])
def test_explicit_terms_entry_points_refuse_integ_and_composition(pz, noalloc):
    """Both stage-level entry points serve collocation instances without
    composition; an integration-method or composition instance is refused the
    same way by each (PZ_E_UNSUPPORTED), not run on collocation kernels."""
    import torch
    specs = [dict(n_r_max=33, m_max=32, ek=1e-3, ra=1e5, dtMax=1e-4, cheb_method="INTEG", matrix_solve="DIRECT"),
             dict(n_r_max=33, m_max=32, l_non_rot=True, ra=-1e4, pr=0.3, raxi=2e4, sc=3.0, g0=1.0, g1=0.0,
                  time_scheme="BPR353", dtMax=1e-3)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    z = torch.zeros((33, 33), dtype=torch.complex128, device="cuda")
    for i in range(2):
        with pytest.raises(pz.PizzaError) as e:
            ens.explicit_terms(i, z, z, z, z, noalloc=noalloc)
        assert e.value.code == -6, (i, str(e.value))


def test_prandtl_not_one_uses_separate_temperature_operator(pz):
    """Pr != 1: the temperature and vorticity operators differ (TdiffFac != ViscFac)."""
    spec = dict(C0, pr=0.7)
    sim, ens, out = run_pair(pz, spec, 40, seed=8)
    check_fields(sim, out[-1][2], TOL, "Pr=0.7")


def test_odd_and_even_grids_and_phi_sizes(pz):
    """Parity-compact operators on even N, and FFT lengths with radix 2, 3, 5, 7."""
    for spec in (dict(C0, n_r_max=32, n_cheb_max=32, m_max=30),     # P = 90 = 2*3*3*5
                 dict(C0, n_r_max=40, n_cheb_max=40, m_max=42),     # P = 126 = 2*3*3*7
                 dict(C0, n_r_max=33, n_cheb_max=30, m_max=32)):    # dealiased n_cheb_max < n_r_max
        sim, ens, out = run_pair(pz, spec, 15, seed=9)
        check_fields(sim, out[-1][2], TOL, str(spec["n_r_max"]))


TSC_NML = """&grid
 n_r_max = 48, n_cheb_max = 48, m_max = 64, minc = 1,
/
&control
 tag = "tsc", l_newmap = .false., time_scheme = "SBDF3", n_time_steps = 2000,
 dtMax = 5d-4, courfac = 2.5d0, l_non_rot = .true., matrix_solve = 'influence', n_fft_optim_lev = 2,
/
&phys_param
 ra = 1.0E+04, pr = 1.0E+00, ek = 1.00E-03, radratio = 3.50E-01, g0 = 1.00E+00, g1 = 0.00E+00,
 g2 = 0.00E+00, ktopt = 1, kbott = 1, ktopv = 2, kbotv = 2,
/
&start_field
 l_start_file = .false., start_file = "checkpoint_end.testB", init_t = -1, amp_t = 1.0e-2,
 init_u = 0, amp_u = 3.0e-4,
/
&output_control
 n_log_step = 100, n_frames = 1,
/
"""


def test_driver_runs_timestepchange_namelist(pz, tmp_path):
    """python -m pizza_gb300.run on the TimeStepChange input (the bubble start,
    init_t = -1, built by the library's own initProp): its e_kin file
    reproduces the reference fixture rows."""
    from pizza_gb300.run import run
    nml = tmp_path / "input.nml"
    nml.write_text(TSC_NML)
    run(str(nml), str(tmp_path))
    got = np.loadtxt(tmp_path / "e_kin.tsc")[:, :4]
    ref = np.loadtxt(os.path.join(HERE, "golden", "TimeStepChange.txt"))
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-14)

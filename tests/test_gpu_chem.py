"""The composition equation (raxi /= 0: update_xi_coll.f90, update_xi_integ.f90,
the ChemFac buoyancy in the streamfunction solves) on the GPU against the
oracle and the reference's FingConv fixture (needs a GB300).

FingConv is fingering convection: temperature and composition, non-rotating,
first on the integration method's direct solve (SBDF3, n_r_max=49) and then,
from that run's checkpoint, on the collocation grid n_r_max=33 with the DIRK
scheme BPR353.  The harness compares e_kin.start + e_kin.continue with
samples/FingConv/reference.out at rtol 1e-8 (samples/FingConv/unitTest.py)."""
import json
import os

import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, rel_err, seeded, series_from_oracle
from tests.test_gpu_parity import check_fields

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

# fingering-convection physics on a small collocation grid
CX = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=-1.0e4, pr=0.3, raxi=2.0e4, sc=3.0, radratio=0.35,
          l_non_rot=True, g0=1.0, g1=0.0, g2=0.0, dtMax=1e-3, time_scheme="CNAB2", matrix_solve="INFLUENCE")
# rotating convection with a stabilising composition gradient
CR = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1.0e5, pr=1.0, raxi=-2.0e4, sc=3.0, radratio=0.35,
          l_ek_pump=True, dtMax=1e-4, time_scheme="CNAB2", matrix_solve="INFLUENCE")
# the integration method (RotInteg's physics) with composition
CI = dict(n_r_max=33, n_cheb_max=24, m_max=24, ek=1e-3, ra=5e4, pr=1.0, raxi=1.0e4, sc=2.0, radratio=0.35,
          time_scale="ROT", cheb_method="INTEG", matrix_solve="DIRECT", time_scheme="CNAB2", dtMax=2e-2,
          courfac=4.0)


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def run_chem_pair(pz, spec, nsteps, seed=1, amp=1e-3):
    t0 = seeded(spec, seed, amp)
    x0 = seeded(spec, seed + 100, amp)
    sim = oracle(spec, temp0=t0, xi0=x0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=t0, xi=x0)
    for _ in range(nsteps):
        sim.advance()
    ens.step(nsteps)
    return sim, ens, ens.get_state(0)


def check_chem(sim, g, tol, label):
    check_fields(sim, g, tol, label)
    e = rel_err(g["xi"], sim.xi)
    assert e < tol, f"{label} xi: rel err {e:.3e}"


def test_chem_start_state(pz):
    spec = CR
    t0, x0 = seeded(spec, 3), seeded(spec, 4)
    sim = oracle(spec, temp0=t0, xi0=x0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=t0, xi=x0)
    g = ens.get_state(0)
    check_chem(sim, g, 1e-13, "start")
    assert rel_err(g["dxi"], sim.dxi) < 1e-12
    for kind, name in ((0, "old"), (1, "impl")):
        assert rel_err(ens.get_history(0, 2, kind, 1), getattr(sim.dxidt, name)[0]) < 1e-12, name


@pytest.mark.parametrize("spec", [
    CX,
    dict(CX, matrix_solve="DIRECT", time_scheme="SBDF3"),
    dict(CX, buo_term="EXPLICIT"),
    CR,
    dict(CR, matrix_solve="DIRECT", time_scheme="SBDF2"),
    dict(CR, time_scheme="TVB33", time_scale="ROT", dtMax=1e-2),
    dict(CR, time_scheme="ARS222", dtMax=2e-5),
    dict(CR, time_scheme="ARS233", dtMax=2e-5),
    dict(CR, time_scheme="BPR353", matrix_solve="DIRECT", dtMax=2e-5),
], ids=["nonrot-dmat-cnab2", "nonrot-smat-sbdf3", "nonrot-buo-expl", "rot-dmat-cnab2", "rot-smat-sbdf2",
        "rot-tvb33-rotscale", "rot-ars222", "rot-ars233-assembly", "rot-smat-bpr353"])
def test_chem_collocation(pz, spec):
    sim, ens, g = run_chem_pair(pz, spec, 30, seed=5, amp=1e-2)
    check_chem(sim, g, 1e-10, str(spec))
    row, ref = ens.series(0)[-1], series_from_oracle(sim)
    # e_kin, heat and composition.TAG columns
    cols = [0, 1, 2, 3, 8, 9, 10, 12, 13, 14, 16, 17, 18, 19, 20, 21]
    np.testing.assert_allclose(row[cols], ref[cols], rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("spec", [
    CI,
    dict(CI, time_scheme="SBDF3"),
    dict(CI, buo_term="EXPLICIT"),
    dict(CI, matrix_solve="INFLUENCE"),
    dict(CI, l_non_rot=True, ra=-1.0e4, pr=0.3, raxi=2.0e4, sc=3.0, time_scale="VISC", dtMax=1e-3, g0=1.0, g1=0.0),
    dict(CI, l_non_rot=True, ra=-1.0e4, pr=0.3, raxi=2.0e4, sc=3.0, time_scale="VISC", dtMax=1e-3, g0=1.0, g1=0.0,
         matrix_solve="INFLUENCE", time_scheme="SBDF3"),
], ids=["rot-smat-cnab2", "rot-smat-sbdf3", "rot-buo-expl", "rot-dmat", "nonrot-smat", "nonrot-dmat-sbdf3"])
def test_chem_integ(pz, spec):
    """update_xi_int with update_psi_int_smat / _dmat; the SBDF3 runs start
    with the CNAB2 bridge, whose direct-solve buoyancy takes psi in the place
    of the composition (step_time.f90:497-498)."""
    sim, ens, g = run_chem_pair(pz, spec, 30, seed=7, amp=1e-2)
    check_chem(sim, g, 1e-10, str(spec))


def test_integ_nonrot_smat_without_composition(pz):
    """The integration method's non-rotating direct solve (intcheb4rmult4lapl,
    intcheb4rmult4lapl2 operators, dpsi/dr tau row at r_o)."""
    spec = dict(CI, raxi=0.0, l_non_rot=True, ra=2e4, time_scale="VISC", dtMax=1e-3)
    for scheme in ("CNAB2", "SBDF3"):
        t0 = seeded(spec, 9, 1e-2)
        sim = oracle(dict(spec, time_scheme=scheme), temp0=t0)
        ens = pz.Ensemble(gpu_config(dict(spec, time_scheme=scheme)))
        ens.set_state(0, temp=t0)
        for _ in range(40):
            sim.advance()
        ens.step(40)
        check_fields(sim, ens.get_state(0), 1e-10, scheme)


def test_mixed_batch_with_and_without_composition(pz):
    specs = [CX, dict(CX, raxi=0.0), CR, dict(CI, raxi=0.0), CI]
    temps = [seeded(s, 40 + i, 1e-2) for i, s in enumerate(specs)]
    xis = [seeded(s, 80 + i, 1e-2) if s["raxi"] != 0.0 else None for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    for i in range(len(specs)):
        ens.set_state(i, temp=temps[i], xi=xis[i])
    ens.step(20)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i], xi0=xis[i])
        for _ in range(20):
            sim.advance()
        g = ens.get_state(i)
        if s["raxi"] != 0.0:
            check_chem(sim, g, 1e-10, f"instance {i}")
        else:
            check_fields(sim, g, 1e-10, f"instance {i}")


def test_chem_checkpoint_restart(pz, tmp_path):
    """A checkpoint with composition (l_chem, xi and its history slots) and a
    restart, against the oracle restarting from the same file."""
    from oracle.pizza_oracle import Params, Pizza
    from pizza_gb300.pizza_io import read_checkpoint, restart_from_checkpoint, save_checkpoint
    spec = dict(CR, time_scheme="SBDF3")
    a = pz.Ensemble(gpu_config(spec))
    a.set_state(0, temp=seeded(spec, 50), xi=seeded(spec, 51))
    a.step(10)
    ck = str(tmp_path / "checkpoint_t=10.chem")
    save_checkpoint(a, 0, ck)
    f = read_checkpoint(ck)
    assert f["header"]["l_chem"] and f["header"]["raxi"] == spec["raxi"] and len(f["hist_Xi"]) == 2 + 0 + 2
    b = pz.Ensemble(gpu_config(spec))
    restart_from_checkpoint(b, 0, ck)
    b.step(10)
    sim = Pizza(Params(**spec))
    sim.start_from_checkpoint(f)
    for _ in range(10):
        sim.advance()
    check_chem(sim, b.get_state(0), 1e-10, "restarted")


def test_chem_spectra_frames_and_series_files(pz, tmp_path):
    from pizza_gb300.pizza_io import read_frame, save_frames, write_series
    spec = CR
    sim, ens, g = run_chem_pair(pz, spec, 20, seed=11, amp=1e-2)
    got, ref = ens.spectra(0), sim.spectra()
    err = np.max(np.abs(got - ref), axis=0) / np.max(np.abs(ref), axis=0)
    assert np.all(err < 1e-10), err
    # the reference's xi2_m column holds the temperature's integral (spectra.f90:183)
    assert np.array_equal(got[:, 4], got[:, 3])
    paths = save_frames(ens, 0, 1, "chem", str(tmp_path))
    assert [os.path.basename(p) for p in paths] == ["frame_temp_1.chem", "frame_xi_1.chem", "frame_us_1.chem",
                                                     "frame_up_1.chem", "frame_om_1.chem"]
    fr = read_frame(paths[1])
    assert np.array_equal(fr["field"], g["xi"]) and fr["raxi"] == spec["raxi"] and fr["sc"] == spec["sc"]
    files = write_series(ens, 0, "chem", str(tmp_path))
    assert os.path.join(str(tmp_path), "composition.chem") in files
    assert np.loadtxt(os.path.join(str(tmp_path), "composition.chem")).shape == (21, 7)


def test_fingconv_fixture_on_gpu(pz, tmp_path):
    """Both FingConv runs on the GPU against samples/FingConv/reference.out:
    500 SBDF3 steps of the non-rotating integration method (n_r_max=49,
    n_cheb_max=32) from the init_t=-1 temperature, a version-7 checkpoint
    with composition, its read onto the n_r_max=33 collocation grid and 500
    BPR353 steps; the 12 e_kin rows at the harness's rtol 1e-8."""
    from pizza_gb300 import pizza_io
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        cases = json.load(f)
    ref = np.vstack([np.loadtxt(os.path.join(HERE, "golden", f"{c}.txt")) for c in ("FingConv", "FingConvContinue")])
    p1, p2 = dict(cases["FingConv"]["params"]), dict(cases["FingConvContinue"]["params"])
    sim = oracle(p1)                               # the init_t = -1 start field, built by the oracle
    ens = pz.Ensemble(gpu_config(p1))
    ens.set_state(0, temp=sim.temp.copy(), xi=sim.xi.copy())
    rows = [ens.series(0)[-1]]
    for _ in range(p1["n_time_steps"] // p1["n_log_step"]):
        ens.step(p1["n_log_step"])
        rows.append(ens.series(0)[-1])
    path = str(tmp_path / "checkpoint_end.start")
    pizza_io.save_checkpoint(ens, 0, path)
    ens2 = pz.Ensemble(gpu_config(p2))
    h = pizza_io.restart_from_checkpoint(ens2, 0, path)
    assert h["l_chem"] and not h["l_cheb_coll"]
    rows.append(ens2.series(0)[-1])
    for _ in range(p2["n_time_steps"] // p2["n_log_step"]):
        ens2.step(p2["n_log_step"])
        rows.append(ens2.series(0)[-1])
    got = np.array(rows)[:, [0, 1, 2, 3]]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-20)


def test_chem_rejections(pz):
    for bad in (dict(CR, sc=0.0), dict(CR, ktopxi=2)):
        with pytest.raises(RuntimeError):
            pz.Ensemble(gpu_config(bad))
    # the adjoint covers the collocation step without composition
    ens = pz.Ensemble(gpu_config(CR))
    ens.set_state(0, temp=seeded(CR, 1))
    with pytest.raises(RuntimeError):
        ens.adjoint_forward(2, 1)

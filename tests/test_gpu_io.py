"""Time series files and checkpoint restarts of GPU runs (needs a GB300)."""
import json
import os

import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, seeded
from tests.test_gpu_parity import check_fields

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
C0 = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
          dtMax=1e-4)


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def test_series_files_match_pizza_fixture(pz, tmp_path):
    """e_kin_3D.TAG of a GPU run of RotE1e3EkPump, written in pizza's format,
    against the file pizza.exe wrote (values to 1e-8, same line layout)."""
    from pizza_gb300.pizza_io import write_series
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        p = dict(json.load(f)["RotE1e3EkPump"]["params"])
    sim = oracle(p)
    ens = pz.Ensemble(gpu_config(p))
    ens.set_state(0, temp=sim.temp.copy())
    ens.step(p["n_time_steps"])
    rows = ens.series(0, p["n_time_steps"] + 1)[::p["n_log_step"]]
    paths = write_series(ens, 0, "gpu", str(tmp_path), rows=rows)
    assert {os.path.basename(x) for x in paths} == {"e_kin.gpu", "e_kin_3D.gpu", "heat.gpu"}
    with open(os.path.join(HERE, "golden", "RotE1e3EkPump.txt")) as f:
        ref_lines = [ln.rstrip("\n") for ln in f if ln.strip()]
    with open(tmp_path / "e_kin_3D.gpu") as f:
        got_lines = [ln.rstrip("\n") for ln in f]
    assert [len(x) for x in got_lines] == [len(x) for x in ref_lines]
    np.testing.assert_allclose(np.loadtxt(tmp_path / "e_kin_3D.gpu"), np.loadtxt(os.path.join(HERE, "golden",
                               "RotE1e3EkPump.txt")), rtol=1e-8, atol=1e-14)


@pytest.mark.parametrize("scheme,solve", [("CNAB2", "INFLUENCE"), ("SBDF3", "DIRECT"), ("TVB33", "INFLUENCE"),
                                          ("ARS222", "DIRECT")])
def test_checkpoint_restart_matches_pizza_restart(pz, tmp_path, scheme, solve):
    """10 steps, a version-7 checkpoint, a restart in a new handle and 10 more
    steps, against the oracle restarting from the same file.

    A checkpoint holds us and up, not the vorticity; a restart recomputes om
    from the velocities (getStartFields), so a run with the influence-matrix
    solve, whose wall vorticity is not the velocities', continues differently
    from an uninterrupted run -- in pizza as here.  The parity bar is the
    restart pizza makes."""
    from oracle.pizza_oracle import Params, Pizza
    from pizza_gb300.pizza_io import read_checkpoint, restart_from_checkpoint, save_checkpoint
    spec = dict(C0, time_scheme=scheme, matrix_solve=solve)
    t0 = seeded(spec, 50)
    a = pz.Ensemble(gpu_config(spec))
    a.set_state(0, temp=t0)
    a.step(10)
    ck = str(tmp_path / "checkpoint_t=10.test")
    save_checkpoint(a, 0, ck)
    b = pz.Ensemble(gpu_config(spec))
    h = restart_from_checkpoint(b, 0, ck)
    assert h["family"] == ("DIRK" if scheme == "ARS222" else "MULTISTEP")
    b.step(10)
    sim = Pizza(Params(**spec))
    sim.start_from_checkpoint(read_checkpoint(ck))
    for _ in range(10):
        sim.advance()
    gb = b.get_state(0)
    check_fields(sim, gb, 1e-10, f"{scheme} restarted")
    assert abs(gb["time"] - sim.time) < 1e-15


def test_frames_of_a_gpu_run(pz, tmp_path):
    """frame_temp/us/up/om of a GPU run (pizza's snapshot files) read back:
    the fields are the instance's state, the header its run."""
    from pizza_gb300.pizza_io import read_frame, save_frames
    spec = C0
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=seeded(spec, 60))
    ens.step(5)
    paths = save_frames(ens, 0, 3, "gpu", str(tmp_path))
    assert [os.path.basename(p) for p in paths] == ["frame_temp_3.gpu", "frame_us_3.gpu", "frame_up_3.gpu",
                                                     "frame_om_3.gpu"]
    st = ens.get_state(0)
    time, _, _ = ens.get_step_state(0)
    for p, key in zip(paths, ("temp", "us", "up", "om")):
        f = read_frame(p)
        assert f["time"] == time and f["n_r_max"] == 33 and f["n_m_max"] == 33 and f["n_phi_max"] == 96
        assert np.array_equal(f["field"], st[key])


@pytest.mark.parametrize("spec_extra", [dict(), dict(cheb_method="INTEG", n_cheb_max=24, time_scale="ROT",
                                                      dtMax=2e-2, ra=5e4)])
def test_device_spectra_match_oracle(pz, tmp_path, spec_extra):
    """Snapshot spectra computed on the device against the oracle's
    calculate_spectra, after 20 steps, and the spec_N.TAG file."""
    from pizza_gb300.pizza_io import write_spectrum
    spec = dict(C0, **spec_extra)
    t0 = seeded(spec, 61, 1e-2)
    sim = oracle(spec, temp0=t0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=t0)
    for _ in range(20):
        sim.advance()
    ens.step(20)
    got, ref = ens.spectra(0)[:, :4], sim.spectra()[:, :4]
    assert np.all(ens.spectra(0)[:, 4] == 0.0)                  # no composition
    # per spectrum, relative to its largest mode (the 1e-10 field bar)
    err = np.max(np.abs(got - ref), axis=0) / np.max(np.abs(ref), axis=0)
    assert np.all(err < 1e-10), err
    p = write_spectrum(ens, 0, 0, "gpu", str(tmp_path))
    assert np.loadtxt(p).shape == (ens.dims[0][1], 6)


def test_input_nml_driver_matches_oracle(pz, tmp_path):
    """python -m pizza_gb300.run on an input.nml: the e_kin.TAG and heat.TAG
    rows it writes at step 0 and every n_log_step steps against the oracle's
    rows at the same steps (8 significant digits, the file format)."""
    from tests.helpers import series_from_oracle
    from pizza_gb300 import namelist, run as drv
    nml = tmp_path / "input.nml"
    nml.write_text("&grid\n n_r_max=33, n_cheb_max=33, m_max=32,\n/\n"
                   "&control\n tag='drv', n_time_steps=20, dtMax=1.0d-4, time_scheme='CNAB2',\n"
                   " l_ek_pump=.true., matrix_solve='INFLUENCE',\n/\n"
                   "&phys_param\n ra=1.0d5, ek=1.0d-3, pr=1.0d0, radratio=0.35d0,\n/\n"
                   "&start_field\n init_t=2, amp_t=1.0d-2,\n/\n&output_control\n n_log_step=5,\n/\n")
    out = tmp_path / "out"
    paths = drv.run(str(nml), str(out))
    names = sorted(os.path.basename(p) for p in paths)
    assert names == ["checkpoint_end.drv", "e_kin.drv", "e_kin_3D.drv", "heat.drv", "spec_1.drv"]
    cfg, ctl, _ = namelist.read(str(nml))
    spec = dict(n_r_max=33, n_cheb_max=33, m_max=32, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
                dtMax=1e-4, time_scheme="CNAB2", matrix_solve="INFLUENCE")
    sim = oracle(spec, temp0=drv.start_temperature(cfg, ctl))
    ref = [series_from_oracle(sim)]
    for k in range(20):
        sim.advance()
        if (k + 1) % 5 == 0:
            ref.append(series_from_oracle(sim))
    ref = np.array(ref)
    ek = np.loadtxt(out / "e_kin.drv")
    assert ek.shape[0] == 5
    scale = np.max(np.abs(ref[:, 1:4]), axis=0)
    assert np.all(np.abs(ek[:, 1:4] - ref[:, 1:4]) <= 1e-7 * scale + 1e-20), (ek[:, 1:4], ref[:, 1:4])
    assert np.allclose(ek[:, 0], ref[:, 0], rtol=1e-9)


def test_device_2d_spectra_match_oracle(pz, tmp_path):
    """(r, m) spectra computed on the device against the oracle's integrands
    of calculate_spectra at every (r, m), after 20 and 30 steps; their
    r-integrals against the device's own m-spectra; a two-snapshot
    2D_spec_avg file read back."""
    from pizza_gb300.pizza_io import Spectra2DAverage, read_2d_spectra
    spec = dict(C0)
    t0 = seeded(spec, 62, 1e-2)
    sim = oracle(spec, temp0=t0)
    ens = pz.Ensemble(gpu_config(spec))
    ens.set_state(0, temp=t0)
    av = Spectra2DAverage(*ens.dims[0][:2], l_sd=True)
    t_avg = 0.0
    for k in (20, 30):
        for _ in range(k - (20 if k == 30 else 0)):
            sim.advance()
        ens.step(k - (20 if k == 30 else 0))
        got, ref = ens.spectra_2d(0), sim.spectra_2d()
        assert got.shape == ref.shape == (3, spec["n_r_max"], spec["m_max"] + 1)
        err = np.max(np.abs(got - ref), axis=(1, 2)) / np.max(np.abs(ref), axis=(1, 2))
        assert np.all(err < 1e-10), err
        w = sim.cheb.rInt_R
        integ = np.array([[w(got[f][:, m]) for f in range(3)] for m in range(got.shape[2])])
        m1 = ens.spectra(0)[:, :3]
        assert np.max(np.abs(integ - m1)) < 1e-12 * np.max(np.abs(m1))
        t_avg += sim.ts.dt[0]
        av.update(got, t_avg)
    p = av.write(str(tmp_path / "2D_spec_avg.gpu"), gpu_config(spec), sim.r)
    back = read_2d_spectra(p)
    mean, sd = av.result()
    assert back["version"] == 2 and back["n_r_max"] == spec["n_r_max"]
    assert np.array_equal(back["us2"], mean[0].T) and np.array_equal(back["enst_SD"], sd[2].T)


@pytest.mark.parametrize("variant,fast", [(dict(), True), (dict(), False),
                                          (dict(buo_term="EXPLICIT", pr=0.7), False),
                                          (dict(l_non_rot=True, l_ek_pump=False, ra=2e4, dtMax=1e-4), True)])
def test_force_balances_match_oracle(pz, tmp_path, variant, fast):
    """The vorticity and u_phi force balances (pz_balance_step) against the
    oracle's record of the same step, at the 6th and 9th step, on the
    tensor-core stage and on the dense kernels: every term to 1e-10 of the
    balance's dominant term (the largest of its terms other than the
    vorticity's dw/dt, which is held to itself; a balance is read against
    its leading terms, and a term that nearly vanishes -- u_phi(m=0) without
    rotation -- carries the rounding of the others); then the time-averaged
    files written from the device terms."""
    from pizza_gb300.pizza_io import VortBalance, VpBalance
    spec = dict(C0, matrix_solve="INFLUENCE", time_scheme="CNAB2", **variant)
    t0 = seeded(spec, 71, 1e-2)
    sim = oracle(spec, temp0=t0)
    prev = pz.fast_path(fast)
    try:
        ens = pz.Ensemble(gpu_config(spec))
    finally:
        pz.fast_path(prev)
    ens.set_state(0, temp=t0)
    cfg = gpu_config(spec)
    vb = VortBalance(cfg, sim.r, sim.height, l_sd=True)
    vpb = VpBalance(cfg, sim.r, sim.height, "gpu", str(tmp_path))
    t_avg, done = 0.0, 0
    for k in (6, 9):
        for _ in range(k - 1 - done):
            sim.advance()
        ens.step(k - 1 - done)
        ref = sim.balance_step()
        got = ens.balance_step(0)
        done = k
        for part in ("vort", "vp"):
            # dw/dt of the vorticity balance mixes Chebyshev and physical values
            # (the reference's quirk): judged against itself, the others against
            # the largest of them
            scale = max(np.max(np.abs(a)) for n_, a in ref[part].items() if n_ != "dwdt")
            for name, a in ref[part].items():
                b = got[part][name]
                if np.max(np.abs(a)) == 0.0:
                    assert np.max(np.abs(b)) == 0.0, (k, part, name)
                    continue
                e = np.max(np.abs(b - a)) / (np.max(np.abs(a)) if name == "dwdt" else scale)
                assert e < 1e-10, (k, part, name, e)
        t_avg += sim.ts.dt[0]
        vb.calc_avg(got["vort"], t_avg)
        vpb.write(sim.time, ens.get_state(0)["up"][0].real, got["vp"])
    p1, p2 = vb.write("gpu", str(tmp_path))
    assert len(open(p1).read().splitlines()) == spec["m_max"]
    assert os.path.getsize(vpb.bal) == 8 * (6 + spec["n_r_max"] + 2 * (1 + 5 * spec["n_r_max"]))

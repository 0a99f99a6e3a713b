"""The Chebyshev integration method (cheb_method='integ', tau rows, direct
solve; update_temp_integ.f90, update_psi_integ_smat.f90) on the GPU against
the oracle and the reference's RotInteg fixture (needs a GB300).

The GPU applies per m the inverse of the preconditioned tau-banded operator,
built by Gauss-Jordan on the device; the oracle solves the same system with
LAPACK.  The integrated operators are well conditioned, so the fields agree
to the 1e-10 of the collocation path.
"""
import json
import os

import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, rel_err, seeded, series_from_oracle
from tests.test_gpu_parity import check_fields, run_pair

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

# the RotInteg first run's physics at a smaller grid and step
CI = dict(n_r_max=33, n_cheb_max=24, m_max=24, ek=1e-3, ra=5e4, pr=1.0, radratio=0.35, time_scale="ROT",
          cheb_method="INTEG", matrix_solve="DIRECT", time_scheme="CNAB2", dtMax=2e-2, courfac=4.0)


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def test_integ_start_state(pz):
    t0 = seeded(CI, 3, 1e-2)
    sim = oracle(CI, temp0=t0)
    ens = pz.Ensemble(gpu_config(CI))
    ens.set_state(0, temp=t0)
    g = ens.get_state(0)
    check_fields(sim, g, 1e-13, "start")
    assert rel_err(g["dtemp"], sim.dtemp) < 1e-12
    for f in ("old", "impl"):
        for k, ta in ((0, sim.dTdt), (1, sim.dpsidt)):
            got = ens.get_history(0, k, {"old": 0, "impl": 1}[f], 1)
            assert rel_err(got, getattr(ta, f)[0]) < 1e-12, (f, k)


def test_integ_cnab2_steps(pz):
    sim, ens, out = run_pair(pz, CI, 100, seed=5, amp=1e-2, checkpoints=(1, 10))
    for k, s, g in out:
        check_fields(s, g, 1e-10, f"integ step {k}")
    ref = series_from_oracle(sim)
    row = ens.series(0)[-1]
    keep = [k for k in range(15) if k not in (12, 13)]
    np.testing.assert_allclose(row[keep], ref[keep], rtol=1e-10, atol=1e-20)
    # tTop, tBot: the tau rows hold T = 0 on the walls in Chebyshev space, so
    # the wall values are rounding residues (~1e-12 of the O(1) temperature)
    np.testing.assert_allclose(row[12:14], ref[12:14], rtol=0, atol=1e-11)


@pytest.mark.parametrize("variant", [
    dict(time_scheme="SBDF3"),
    dict(time_scheme="CK232"),
    dict(time_scheme="BPR353"),
    dict(corio_term="EXPLICIT"),
    dict(buo_term="EXPLICIT"),
    dict(l_ek_pump=True),
    dict(l_rerror_fix=True),
    dict(pr=0.3, n_cheb_max=33),
])
def test_integ_variants(pz, variant):
    spec = dict(CI, **variant)
    sim, ens, out = run_pair(pz, spec, 30, seed=7, amp=1e-2)
    check_fields(sim, out[-1][2], 1e-10, str(variant))


def test_integ_larger_grid(pz):
    """The grid of RotInteg's continuation run (n_r_max=97, n_cheb_max=64)."""
    spec = dict(CI, n_r_max=97, n_cheb_max=64, m_max=64, ek=1e-4, ra=2e6, dtMax=2e-3)
    sim, ens, out = run_pair(pz, spec, 10, seed=9, amp=1e-3)
    check_fields(sim, out[-1][2], 1e-9, "N=97")


def test_mixed_integ_and_collocation_batch(pz):
    specs = [CI,
             dict(CI, cheb_method="COLL", n_cheb_max=33),
             dict(CI, n_r_max=49, n_cheb_max=32, m_max=32, ra=8e4),
             dict(CI, cheb_method="COLL", matrix_solve="INFLUENCE", time_scale="VISC", dtMax=2e-5, n_cheb_max=33)]
    temps = [seeded(s, 30 + i, 1e-2) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    ens.set_state_all(temps)
    ens.step(20)
    for i, s in enumerate(specs):
        sim = oracle(s, temp0=temps[i])
        for _ in range(20):
            sim.advance()
        check_fields(sim, ens.get_state(i), 1e-10, f"instance {i}")


def test_rotinteg_fixture_on_gpu(pz):
    """All 201 e_kin_3D rows of RotInteg's first run (4000 CNAB2 steps,
    Courant-controlled dt) at the reference harness's tolerances."""
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        spec = json.load(f)["RotInteg"]
    p = dict(spec["params"])
    ref = np.loadtxt(os.path.join(HERE, "golden", "RotInteg.txt"))
    sim = oracle(p)                          # init_t = -1 start field built by the oracle
    ens = pz.Ensemble(gpu_config(p))
    ens.set_state(0, temp=sim.temp.copy())
    n, nlog = p["n_time_steps"], p["n_log_step"]
    rows = [ens.series(0)[-1]]
    for _ in range(n // nlog):
        ens.step(nlog)
        rows.append(ens.series(0)[-1])
    got = np.array(rows)[:, [0, 4, 5, 6, 7]]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-20)


@pytest.mark.parametrize("variant", [
    dict(),
    dict(time_scheme="SBDF3"),
    dict(time_scheme="CK232"),
    dict(l_ek_pump=True),
    dict(buo_term="EXPLICIT"),
    dict(l_rerror_fix=True),
    dict(pr=0.3, n_cheb_max=33),
    dict(l_non_rot=True, ra=2e4, time_scale="VISC", dtMax=1e-3),
])
def test_integ_influence_matrix(pz, variant):
    """update_psi_int_dmat: vorticity solve, psi from vorticity, influence
    matrix for the remaining wall conditions (Coriolis explicit)."""
    spec = dict(CI, matrix_solve="INFLUENCE", **variant)
    sim, ens, out = run_pair(pz, spec, 40, seed=13, amp=1e-2, checkpoints=(1,))
    for k, s, g in out:
        check_fields(s, g, 1e-10, f"dmat step {k} {variant}")


@pytest.mark.parametrize("variant", [
    dict(),
    dict(l_non_rot=True, ra=2e4, time_scale="VISC", dtMax=1e-3),
    dict(matrix_solve="INFLUENCE"),
    dict(matrix_solve="INFLUENCE", l_non_rot=True, ra=2e4, time_scale="VISC", dtMax=1e-3),
    dict(raxi=3e4, sc=3.0, time_scheme="SBDF3"),
    dict(n_r_max=97, n_cheb_max=97, m_max=32, ek=1e-5, ra=3e7, dtMax=2e-6, time_scheme="SBDF3", l_ek_pump=True),
])
def test_integ_banded_matches_dense(pz, variant):
    """The bordered banded factors (pz_integ_banded(1), pizza's own algorithm:
    band LU of the operator block, Schur complement of the tau rows) and the
    dense per-m inverses (pz_integ_banded(0), the default) solve the same
    systems.  After 25 steps the dense path matches the oracle (which
    factorises the same row-scaled tau systems with LAPACK's dense LU) at
    1e-10, 1e-9 at n_r_max = 97 with the rotating direct solve.  The bordered
    elimination is less accurate than a pivoted dense LU on the four-tau-row
    streamfunction systems (against a 40-digit solve of the row-scaled
    N = 97, E = 1e-5 systems: 1e-12 relative per solve, the dense LU 2e-14),
    and the flow amplifies that: the oracle's own restatement of the bordered
    solve (oracle/bordered.py, LAPACK gbtrf/gbtrs/getrf as the reference
    calls them) drifts from the dense oracle by up to 1.3e-7 in 25 steps of
    that case.  So the banded path must stay as close to the dense oracle as
    the reference's algorithm does: within 10x the larger of the dense bar
    and the bordered oracle's distance, per field."""
    spec = dict(CI, **variant)
    temp0 = seeded(spec, 5, 1e-2 if spec["n_r_max"] < 97 else 1e-4)
    assert pz.integ_banded() is False
    dense = pz.Ensemble(gpu_config(spec))
    prev = pz.integ_banded(True)
    try:
        band = pz.Ensemble(gpu_config(spec))
    finally:
        pz.integ_banded(prev)
    sim = oracle(spec, temp0=temp0)
    bsim = oracle(spec, temp0=temp0, integ_bordered=True)
    for e in (dense, band):
        e.set_state(0, temp=temp0)
    for _ in range(25):
        sim.advance()
        bsim.advance()
    dense.step(25)
    band.step(25)
    gd, gb = dense.get_state(0), band.get_state(0)
    big = spec["n_r_max"] >= 97 and spec.get("matrix_solve", "DIRECT") == "DIRECT"
    bar = 1e-9 if big else 1e-10
    check_fields(sim, gd, bar, f"dense {variant}")
    for f in ("temp", "us", "up", "om"):
        ref = getattr(sim, f)
        drift = rel_err(getattr(bsim, f), ref)
        e = rel_err(gb[f], ref)
        assert e < 10.0 * max(bar, drift), f"banded {variant} {f}: rel err {e:.3e}, bordered oracle {drift:.3e}"
    dense.close()
    band.close()


def test_integ_influence_matrix_larger_grid(pz):
    """RotInteg's continuation grid and physics (n_r_max=97, n_cheb_max=64,
    E=1e-4, Ra=2e6, Ekman pumping, SBDF3) with the influence matrix."""
    spec = dict(CI, n_r_max=97, n_cheb_max=64, m_max=64, ek=1e-4, ra=2e6, dtMax=2e-3, l_ek_pump=True,
                time_scheme="SBDF3", matrix_solve="INFLUENCE")
    sim, ens, out = run_pair(pz, spec, 10, seed=9, amp=1e-3)
    check_fields(sim, out[-1][2], 1e-9, "dmat N=97")


def test_rotinteg_continuation_fixture_on_gpu(pz, tmp_path):
    """RotInteg's second run: the first run's final state, saved as a
    version-7 checkpoint and read back onto n_r_max=97, n_cheb_max=64,
    m_max=64 (Chebyshev mapping), with the influence-matrix solve, SBDF3
    behind the CNAB2 bridge, AB1 on the first step (E changed), Ekman pumping
    and explicit Coriolis: its 16 e_kin_3D rows at the harness's tolerances."""
    from pizza_gb300 import pizza_io
    with open(os.path.join(HERE, "golden", "cases.json")) as f:
        cases = json.load(f)
    p1, p2 = dict(cases["RotInteg"]["params"]), dict(cases["RotIntegContinue"]["params"])
    ref = np.loadtxt(os.path.join(HERE, "golden", "RotIntegContinue.txt"))
    sim = oracle(p1)                         # init_t = -1 start field built by the oracle
    ens = pz.Ensemble(gpu_config(p1))
    ens.set_state(0, temp=sim.temp.copy())
    ens.step(p1["n_time_steps"])
    path = str(tmp_path / "checkpoint_end.start")
    pizza_io.save_checkpoint(ens, 0, path)
    ens2 = pz.Ensemble(gpu_config(p2))
    pizza_io.restart_from_checkpoint(ens2, 0, path)
    n, nlog = p2["n_time_steps"], p2["n_log_step"]
    rows = [ens2.series(0)[-1]]
    for _ in range(n // nlog):
        ens2.step(nlog)
        rows.append(ens2.series(0)[-1])
    got = np.array(rows)[:, [0, 4, 5, 6, 7]]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-20)


def test_integ_rejections(pz):
    bad = [dict(CI, time_scheme="ARS232"), dict(CI, ktopv=1)]
    for s in bad:
        with pytest.raises(RuntimeError):
            pz.Ensemble(gpu_config(s))


C1 = dict(n_r_max=97, n_cheb_max=97, m_max=128, ek=1e-5, ra=3e7, pr=1.0, radratio=0.35,
          time_scheme="SBDF3", dtMax=2e-6, cheb_method="INTEG", matrix_solve="DIRECT", l_ek_pump=True)
C1_CK = (20, 500, 1000, 1250)


def _c1_oracle(pert):
    """Oracle run of the full-size integ workload to C1_CK; with `pert`,
    fp64_noise of that level on the temperature after every step (the size of
    the rounding differences of another FP64 implementation).  The unperturbed
    run then goes on to its breakdown: its Courant step collapses below dtMin a
    few steps after 1250 (at step 1272 on x86 with NumPy/SciPy), and it returns
    that step and the dt of every step after 1250."""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from tests.helpers import fp64_noise, oracle as make, seeded as seed_of
    sim = make(C1, temp0=seed_of(C1, 11, 1e-4))
    rng = np.random.default_rng(77)
    out, done = {}, 0
    for k in C1_CK:
        for _ in range(k - done):
            sim.advance()
            if pert:
                fp64_noise(sim, rng, pert, fields=("temp",))
        done = k
        out[k] = {f: getattr(sim, f).copy() for f in ("us", "up", "om", "temp", "psi")}
    if not pert:
        dts, k = [], done
        try:
            while k < 2000:
                sim.advance()
                k += 1
                dts.append(sim.ts.dt[0])
        except FloatingPointError:
            out["fail"] = k + 1
        out["dt"] = np.array(dts)
    return out


def test_c1_integ_sbdf3_full_size(pz):
    """The integ workload at full size (n_r_max=97, n_phi_max=384, E=1e-5,
    Ra=3e7, SBDF3, dt=2e-6, seeded amplitude 1e-4) over its 2000 steps.  The
    reference's algorithm does not finish them: the flow grows exponentially
    (max |u_s| 0.65 at step 100, 121 at 1200), the trajectory becomes
    unpredictable between steps 1000 and 1250 (the oracle's own spread, its run
    with fp64_noise of 1e-13 on the temperature after every step, is 3e-12 at
    1000 and O(1) at 1250), and the Courant step collapses below dtMin at about
    step 1270.  So the GPU is held to the oracle at steps 20, 500, 1000 and 1250
    (1e-10 relative while that spread stays below 1e-12, 100x the spread
    beyond), then it must break down too: the dt < dtMin error within 20 steps
    of the oracle's (measured: oracle 1273, GPU 1265).  The tau rows, which
    hold in Chebyshev space, are checked on the step-1250 GPU state: for T and
    psi (m > 0) c_0/2 + sum_n c_n (+-1)^n = 0 at both walls (the physical wall
    value differs from it by the DCT-I's half weight on c_{N-1})."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(2) as pool:
        ref, spread = pool.map(_c1_oracle, (0.0, 1e-13))
    ens = pz.Ensemble(gpu_config(C1))
    ens.set_state(0, temp=seeded(C1, 11, 1e-4))
    done, report = 0, []
    for k in C1_CK:
        ens.step(k - done)
        done = k
        g = ens.get_state(0)
        fl = max(rel_err(spread[k][f], ref[k][f]) for f in ("temp", "us", "up", "om"))
        tol = 1e-10 if fl < 1e-12 else max(1e-10, 100.0 * fl)
        errs = {f: rel_err(g[f], ref[k][f]) for f in ("temp", "us", "up", "om")}
        report.append((k, errs, fl))
        for f, e in errs.items():
            assert e < tol, f"c1 step {k} {f}: rel err {e:.3e} (oracle spread {fl:.2e})"
    g = ens.get_state(0)
    N = C1["n_r_max"]
    sg = np.where(np.arange(N) % 2 == 0, 1.0, -1.0)
    sim = oracle(C1, temp0=seeded(C1, 11, 1e-4))
    for f in ("temp", "psi"):
        c = sim.cheb.costf1(g[f])[1:]              # Chebyshev coefficients, m > 0
        top = 0.5 * c[:, 0] + c[:, 1:].sum(axis=1)
        bot = 0.5 * c[:, 0] + (c[:, 1:] * sg[1:]).sum(axis=1)
        scale = np.max(np.abs(c))
        assert np.max(np.abs(top)) < 1e-11 * scale and np.max(np.abs(bot)) < 1e-11 * scale, f
    # the breakdown
    assert "fail" in ref, "the oracle finished 2000 steps"
    dts, fail = [], None
    for k in range(done + 1, 2001):
        try:
            ens.step(1)
        except pz.PizzaError:
            fail = k
            break
        dts.append(ens.get_step_state(0)[1][0])
    out_dir = os.environ.get("PZ_REPORT_DIR", "")
    if out_dir and os.path.isdir(out_dir):
        with open(os.path.join(out_dir, "c1_integ_parity.txt"), "w") as f:
            for k, errs, fl in report:
                f.write(f"step {k}: " + " ".join(f"{a} {e:.2e}" for a, e in errs.items())
                        + f" oracle-spread {fl:.2e}\n")
            f.write(f"breakdown: oracle at step {ref['fail']}, GPU at step {fail}\n")
    assert fail is not None and abs(fail - ref["fail"]) <= 20, (fail, ref["fail"])
    assert len(dts) > 0 and min(dts) < 1e-3 * C1["dtMax"]     # the collapse, not another error

"""Discrete adjoint of DIRK steps (the stage loop with dirk_schemes.f90's
tableaux, ARS233 with its assembly stage) through the C ABI (needs a GB300).

The workload of the batched adjoint ensemble is ARS233 with the outer-boundary
Nusselt number as objective; the checks follow the CNAB2 adjoint's:
  * J of the adjoint's forward sweep against the oracle with the same step
    sequence (1e-10 relative);
  * directional derivatives against FP64 central finite differences of the
    GPU forward (eps = 1e-6 relative, agreement 1e-6 relative);
  * dJ/dRa against finite differences;
  * independence of the checkpoint interval;
  * a batch of instances of different sizes in one sweep.
"""
import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, seeded, series_from_oracle
from tests.test_gpu_adjoint import GRAD_TOL, directional, pz  # noqa: F401  (pz is the shared fixture)

pytestmark = pytest.mark.gpu

SMALL = dict(n_r_max=17, n_cheb_max=17, m_max=8, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
             time_scheme="ARS233", dtMax=1e-4, matrix_solve="INFLUENCE")
SCHED = np.array([1e-4] * 5 + [7e-5] * 5)      # a dt change in the middle: operators rebuilt backwards


def fwd(ens, temps, n_steps, n_window, sched, ck=0, objective="nutop"):
    for i, t in enumerate(temps):
        ens.set_state(i, temp=t)
    J, dt = ens.adjoint_forward(n_steps, n_window, ck, np.tile(sched, (len(temps), 1)), objective=objective)
    return J, dt


def oracle_objective(spec, temp0, sched, n_window, col):
    sim = oracle(spec, temp0=temp0)
    sim.dt_schedule = sched
    n = len(sched)
    vals = []
    for k in range(1, n + 1):
        sim.advance()
        if k > n - n_window:
            row = series_from_oracle(sim)
            vals.append(sum(row[c] for c in col))
    return float(np.mean(vals))


def fd_dirs(ens, temps, g, inst, n_steps, n_window, sched, n_dir, seed, objective):
    rng = np.random.default_rng(seed)
    errs = []
    t0 = temps[inst]
    for _ in range(n_dir):
        d = rng.standard_normal(t0.shape) + 1j * rng.standard_normal(t0.shape)
        d[0] = d[0].real                                  # the m = 0 imaginary part is not a degree of freedom
        eps = 1e-6 * np.max(np.abs(t0)) / np.max(np.abs(d))
        tp = list(temps); tp[inst] = t0 + eps * d
        tm = list(temps); tm[inst] = t0 - eps * d
        jp, _ = fwd(ens, tp, n_steps, n_window, sched, objective=objective)
        jm, _ = fwd(ens, tm, n_steps, n_window, sched, objective=objective)
        fd = (jp[inst] - jm[inst]) / (2 * eps)
        errs.append(abs(fd - directional(g, d)) / abs(fd))
    return errs


@pytest.mark.parametrize("scheme,objective,cols", [("ARS233", "nutop", (8,)), ("ARS233", "ekin3d", (4, 5, 6)),
                                                   ("ARS222", "nutop", (8,)), ("BPR353", "ekin3d", (4, 5, 6))])
def test_dirk_objective_matches_oracle(pz, scheme, objective, cols):
    spec = dict(SMALL, time_scheme=scheme)
    t0 = seeded(spec, 1, 1e-2)
    ens = pz.Ensemble(gpu_config(spec))
    J, dt = fwd(ens, [t0], 10, 6, SCHED, ck=4, objective=objective)
    assert np.array_equal(dt[0], SCHED)
    Jo = oracle_objective(spec, t0, SCHED, 6, cols)
    assert abs(J[0] - Jo) <= 1e-10 * abs(Jo), (J[0], Jo)


@pytest.mark.parametrize("scheme,objective", [("ARS233", "nutop"), ("ARS233", "ekin3d"), ("ARS222", "nutop"),
                                              ("BPR353", "ekin3d"), ("CK232", "nutop")])
def test_dirk_gradient_temp_vs_fd(pz, scheme, objective):
    spec = dict(SMALL, time_scheme=scheme)
    t0 = seeded(spec, 1, 1e-2)
    ens = pz.Ensemble(gpu_config(spec))
    fwd(ens, [t0], 10, 6, SCHED, ck=4, objective=objective)
    g, _ = ens.adjoint_backward()
    errs = fd_dirs(ens, [t0], g[0], 0, 10, 6, SCHED, 4, 7, objective)
    assert max(errs) < GRAD_TOL, f"{scheme} {objective}: adjoint vs FD rel errs {errs}"


def test_dirk_gradient_ra_vs_fd(pz):
    t0 = seeded(SMALL, 2, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, [t0], 10, 6, SCHED, ck=3)
    _, dra = ens.adjoint_backward()
    ra = SMALL["ra"]
    h = 1e-6 * ra
    ens.set_ra(0, ra + h)
    jp, _ = fwd(ens, [t0], 10, 6, SCHED)
    ens.set_ra(0, ra - h)
    jm, _ = fwd(ens, [t0], 10, 6, SCHED)
    ens.set_ra(0, ra)
    fd = (jp[0] - jm[0]) / (2 * h)
    assert abs(fd - dra[0]) <= GRAD_TOL * abs(fd), (fd, dra[0])


def test_dirk_checkpoint_interval_does_not_change_gradient(pz):
    t0 = seeded(SMALL, 3, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    grads = []
    for ck in (0, 4, 1):
        fwd(ens, [t0], 10, 6, SCHED, ck=ck)
        g, dra = ens.adjoint_backward()
        grads.append((g[0], dra[0]))
    for g, dra in grads[1:]:
        assert np.max(np.abs(g - grads[0][0])) <= 1e-12 * np.max(np.abs(grads[0][0]))
        assert abs(dra - grads[0][1]) <= 1e-12 * abs(grads[0][1])


@pytest.mark.parametrize("scheme", ["ARS233", "ARS222", "BPR353"])
def test_dirk_grid_snapshots_do_not_change_gradient(pz, scheme):
    """Stage-state grids from the forward's k_rloop (default) against grids
    recomputed from the spectral snapshots."""
    spec = dict(SMALL, time_scheme=scheme)
    t0 = seeded(spec, 4, 1e-2)
    ens = pz.Ensemble(gpu_config(spec))
    fwd(ens, [t0], 10, 6, SCHED, ck=4)
    g1, r1 = ens.adjoint_backward()
    ens.adjoint_grid_snapshots(False)
    fwd(ens, [t0], 10, 6, SCHED, ck=4)
    g2, r2 = ens.adjoint_backward()
    ens.adjoint_grid_snapshots(True)
    assert np.max(np.abs(g2[0] - g1[0])) <= 1e-13 * np.max(np.abs(g1[0]))
    assert abs(r2[0] - r1[0]) <= 1e-13 * abs(r1[0])


def test_dirk_batched_instances(pz):
    """Three instances of different grids and Ra in one ARS233 sweep; the
    gradient of each instance's NuTop against finite differences."""
    specs = [SMALL, dict(SMALL, n_r_max=21, n_cheb_max=21, m_max=10, ra=2e5), dict(SMALL, ra=5e4)]
    temps = [seeded(s, 10 + i, 1e-2) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    fwd(ens, temps, 10, 6, SCHED, ck=5)
    g, _ = ens.adjoint_backward()
    for inst in (0, 1):
        errs = fd_dirs(ens, temps, g[inst], inst, 10, 6, SCHED, 2, 20 + inst, "nutop")
        assert max(errs) < GRAD_TOL, f"instance {inst}: {errs}"


def test_batched_adjoint_workload_ars233_fd(pz):
    """The batched adjoint workload itself (bench.batched_adjoint_specs(64):
    64 instances, n_r_max in {49, 65}, n_phi_max in {126, 192}, Ra in
    [1e6, 1e7], ARS233 with its assembly stage, dt = 1e-5, 300 steps,
    checkpoint every 30) in one handle: each instance's gradient of its
    time-averaged NuTop with respect to its initial temperature, against
    central finite differences of the GPU forward along one seeded direction
    on 4 instances of different grids, eps = 1e-4 relative to the
    perturbation (J = mean NuTop is 1 + O(1e-2); below 1e-5 the difference
    quotient is dominated by the rounding of J)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    specs = bench.batched_adjoint_specs(64)
    temps = [bench.seeded_temp(s) for s in specs]
    n_steps, ck = bench.BADJ_STEPS, bench.BADJ_CK
    sched = np.full((len(specs), n_steps), bench.BADJ_DT)
    ens = pz.Ensemble([bench.gpu_cfg(s) for s in specs])
    ens.set_state_all(temps)
    J, _ = ens.adjoint_forward(n_steps, n_steps, ck, sched, objective="nutop")
    assert np.all(np.isfinite(J))
    g, _ = ens.adjoint_backward()
    # one instance of each (n_r_max, m_max) class
    picks = []
    for cls in sorted({(s["n_r_max"], s["m_max"]) for s in specs}):
        picks.append(next(i for i, s in enumerate(specs) if (s["n_r_max"], s["m_max"]) == cls))
    rng = np.random.default_rng(77)
    errs = {}
    for inst in picks:
        d = rng.standard_normal(temps[inst].shape) + 1j * rng.standard_normal(temps[inst].shape)
        d[0] = d[0].real
        eps = 1e-4 * np.max(np.abs(temps[inst])) / np.max(np.abs(d))
        jj = []
        for sgn in (1.0, -1.0):
            tp = list(temps)
            tp[inst] = temps[inst] + sgn * eps * d
            ens.set_state_all(tp)
            Jp, _ = ens.adjoint_forward(n_steps, n_steps, ck, sched, objective="nutop")
            jj.append(Jp[inst])
        fd = (jj[0] - jj[1]) / (2 * eps)
        errs[inst] = abs(fd - directional(g[inst], d)) / abs(fd)
    ens.close()
    assert len(picks) == 4
    assert max(errs.values()) < 1e-6, errs

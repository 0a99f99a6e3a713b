"""Discrete adjoint of the CNAB2 step through the C ABI (needs a GB300).

The objective is J = mean over the last n_window states of
us2_3D + up2_3D + uz2_3D (pizza's e_kin_3D columns, outputs.f90:553-570) and
the gradient is taken with respect to the initial temperature perturbation and
Ra for a fixed time-step sequence.  Checks:
  * J of the adjoint's forward sweep against the oracle with the same step
    sequence (1e-10 relative, the parity bar of the forward path);
  * directional derivatives against FP64 central finite differences of the
    GPU forward, eps = 1e-6 relative (agreement 1e-6 relative, the bar the
    gradient path is held to), and against finite differences of the oracle;
  * the dot-product test against the tangent-linear run of the oracle's step
    (oracle/pizza_tangent.py): <tangent(d), 1> = Re<g, d> to 1e-8;
  * dJ/dRa against finite differences;
  * independence of the checkpoint interval (recomputation is exact);
  * the torch.autograd.Function path.
"""
import numpy as np
import pytest

from tests.helpers import gpu_config, oracle, seeded, series_from_oracle

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-6

SMALL = dict(n_r_max=17, n_cheb_max=17, m_max=8, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
             time_scheme="CNAB2", dtMax=1e-4, matrix_solve="INFLUENCE")
SCHED = np.array([1e-4] * 6 + [7e-5] * 6)      # a dt change in the middle: operators rebuilt backwards


@pytest.fixture(scope="module")
def pz():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


def fwd(ens, temp0, n_steps, n_window, sched=None, ck=0):
    ens.set_state(0, temp=temp0)
    J, dt = ens.adjoint_forward(n_steps, n_window, ck, None if sched is None else sched[None, :])
    return J[0], dt[0]


def directional(g, d):
    return float(np.sum((np.conj(g) * d).real))


def fd_check(ens, temp0, g, n_steps, n_window, sched, n_dir, seed, tol=GRAD_TOL):
    rng = np.random.default_rng(seed)
    errs = []
    for _ in range(n_dir):
        d = rng.standard_normal(temp0.shape) + 1j * rng.standard_normal(temp0.shape)
        eps = 1e-6 * np.max(np.abs(temp0)) / np.max(np.abs(d))
        jp, _ = fwd(ens, temp0 + eps * d, n_steps, n_window, sched)
        jm, _ = fwd(ens, temp0 - eps * d, n_steps, n_window, sched)
        fd = (jp - jm) / (2 * eps)
        ad = directional(g, d)
        errs.append(abs(fd - ad) / abs(fd))
    assert max(errs) < tol, f"adjoint vs FD: rel errs {errs}"
    return errs


def oracle_objective(spec, temp0, sched, n_window):
    sim = oracle(spec, temp0=temp0)
    sim.dt_schedule = sched
    n = len(sched)
    vals = []
    for k in range(1, n + 1):
        sim.advance()
        if k > n - n_window:
            row = series_from_oracle(sim)
            vals.append(row[4] + row[5] + row[6])
    return float(np.mean(vals))


def test_objective_matches_oracle(pz):
    t0 = seeded(SMALL, 1, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    J, dt = fwd(ens, t0, 12, 7, SCHED, ck=4)
    assert np.array_equal(dt, SCHED)
    Jo = oracle_objective(SMALL, t0, SCHED, 7)
    assert abs(J - Jo) <= 1e-10 * abs(Jo), (J, Jo)


def test_gradient_temp_vs_fd(pz):
    t0 = seeded(SMALL, 1, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=4)
    g, _ = ens.adjoint_backward()
    fd_check(ens, t0, g[0], 12, 7, SCHED, n_dir=4, seed=7)


def test_gradient_ra_vs_fd(pz):
    t0 = seeded(SMALL, 1, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=4)
    _, dra = ens.adjoint_backward()
    ra = SMALL["ra"]
    h = 1e-6 * ra
    ens.set_ra(0, ra + h)
    jp, _ = fwd(ens, t0, 12, 7, SCHED)
    ens.set_ra(0, ra - h)
    jm, _ = fwd(ens, t0, 12, 7, SCHED)
    ens.set_ra(0, ra)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - dra[0]) <= GRAD_TOL * abs(fd), (fd, dra[0])


def test_checkpoint_interval_does_not_change_gradient(pz):
    t0 = seeded(SMALL, 3, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    grads = []
    for ck in (0, 4, 5, 1):
        fwd(ens, t0, 12, 7, SCHED, ck=ck)
        g, dra = ens.adjoint_backward()
        grads.append((g[0], dra[0]))
    g0, r0 = grads[0]
    for g, r in grads[1:]:
        assert np.max(np.abs(g - g0)) <= 1e-13 * np.max(np.abs(g0))
        assert abs(r - r0) <= 1e-13 * abs(r0)


def test_grid_snapshots_do_not_change_gradient(pz):
    """The backward sweep with the forward's phi-grids (default) and with
    grids recomputed from the spectral snapshots give the same gradient;
    disabling the grids of a stored sweep falls back to the transforms."""
    t0 = seeded(SMALL, 5, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=5)
    g1, r1 = ens.adjoint_backward()
    ens.adjoint_grid_snapshots(False)
    g2, r2 = ens.adjoint_backward()           # same stored sweep, no grids
    fwd(ens, t0, 12, 7, SCHED, ck=5)
    g3, r3 = ens.adjoint_backward()
    ens.adjoint_grid_snapshots(True)
    for g, r in ((g2, r2), (g3, r3)):
        assert np.max(np.abs(g[0] - g1[0])) <= 1e-13 * np.max(np.abs(g1[0]))
        assert abs(r[0] - r1[0]) <= 1e-13 * abs(r1[0])


def test_backward_twice_and_state_left_at_final(pz):
    t0 = seeded(SMALL, 4, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 5, SCHED, ck=5)
    fin = ens.get_state(0)
    g1, r1 = ens.adjoint_backward()
    after = ens.get_state(0)
    for f in ("temp", "us", "up", "om"):
        assert np.array_equal(after[f], fin[f])
    g2, r2 = ens.adjoint_backward()
    assert np.max(np.abs(g2[0] - g1[0])) <= 1e-13 * np.max(np.abs(g1[0]))
    # stepping on discards the stored sweep
    ens.step(1)
    with pytest.raises(pz.PizzaError):
        ens.adjoint_backward()


def test_gradient_vs_oracle_fd(pz):
    """FD of the CPU restatement of pizza along one direction."""
    t0 = seeded(SMALL, 5, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=4)
    g, _ = ens.adjoint_backward()
    d = np.random.default_rng(11).standard_normal(t0.shape) * (1 + 0.5j)
    eps = 1e-6 * np.max(np.abs(t0)) / np.max(np.abs(d))
    fd = (oracle_objective(SMALL, t0 + eps * d, SCHED, 7) - oracle_objective(SMALL, t0 - eps * d, SCHED, 7)) / (2 * eps)
    ad = directional(g[0], d)
    assert abs(fd - ad) <= GRAD_TOL * abs(fd), (fd, ad)


def test_courant_controlled_run(pz):
    """dt chosen by dt_courant in the sweep (three changes), held fixed in the gradient."""
    spec = dict(n_r_max=33, m_max=32, ek=1e-3, ra=3e5, l_ek_pump=True, dtMax=1e-4, courfac=10.0,
                matrix_solve="INFLUENCE")
    t0 = seeded(spec, 2, 3e-3)
    ens = pz.Ensemble(gpu_config(spec))
    _, dt = fwd(ens, t0, 150, 50, None, ck=40)
    assert len(np.unique(dt)) > 1, "the run must change dt"
    g, _ = ens.adjoint_backward()
    fd_check(ens, t0, g[0], 150, 50, dt, n_dir=2, seed=3)


def test_torch_autograd(pz):
    import torch
    from pizza_gb300.autograd import kinetic_energy
    t0 = seeded(SMALL, 6, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=4)
    g, dra = ens.adjoint_backward()
    T = torch.tensor(t0[None], dtype=torch.complex128, requires_grad=True)
    ra = torch.tensor([SMALL["ra"]], dtype=torch.float64, requires_grad=True)
    J = kinetic_energy(T, ra, ens, 12, 7, 4, SCHED[None, :])
    (2.0 * J.sum()).backward()
    assert np.max(np.abs(T.grad[0].numpy() - 2 * g[0])) <= 1e-13 * np.max(np.abs(g[0]))
    assert abs(ra.grad[0].item() - 2 * dra[0]) <= 1e-13 * abs(dra[0])


def test_c3_gradient_16_directions(pz):
    """The gradient workload: N=65, n_phi=192, E=1e-4, Ra=2e6, CNAB2 with
    dtMax=5e-5 under the Courant controller, 500 steps, checkpoint every 50,
    J over the last 250 states; 16 seeded directions plus dJ/dRa."""
    spec = dict(n_r_max=65, n_cheb_max=65, m_max=64, ek=1e-4, ra=2e6, pr=1.0, radratio=0.35, l_ek_pump=True,
                time_scheme="CNAB2", dtMax=5e-5, matrix_solve="INFLUENCE")
    t0 = seeded(spec, 1, 1e-3)
    ens = pz.Ensemble(gpu_config(spec))
    _, dt = fwd(ens, t0, 500, 250, None, ck=50)
    g, dra = ens.adjoint_backward()
    errs = fd_check(ens, t0, g[0], 500, 250, dt, n_dir=16, seed=16)
    ra = spec["ra"]
    h = 1e-6 * ra
    ens.set_ra(0, ra + h)
    jp, _ = fwd(ens, t0, 500, 250, dt)
    ens.set_ra(0, ra - h)
    jm, _ = fwd(ens, t0, 500, 250, dt)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - dra[0]) <= GRAD_TOL * abs(fd), (fd, dra[0])
    print("c3 FD rel errors: max %.2e, dJ/dRa rel %.2e" % (max(errs), abs(fd - dra[0]) / abs(fd)))


def test_dot_product_with_oracle_tangent_linear_run(pz):
    """The GPU gradient against exact directional derivatives from the
    tangent-linear run of the oracle's step (no finite-difference error)."""
    from oracle import pizza_tangent as pt
    from oracle.pizza_oracle import Params
    t0 = seeded(SMALL, 8, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    fwd(ens, t0, 12, 7, SCHED, ck=4)
    g, dra = ens.adjoint_backward()
    o = pt.StepOps(Params(**SMALL))
    rng = np.random.default_rng(21)
    for _ in range(3):
        d = rng.standard_normal(t0.shape) + 1j * rng.standard_normal(t0.shape)
        dr = 1e3 * rng.standard_normal()
        _, dJ = pt.tangent(o, t0, d, SCHED, SMALL["ra"], dr, range(6, 13))
        ad = directional(g[0], d) + dra[0] * dr
        assert abs(dJ - ad) <= 1e-8 * abs(dJ), (dJ, ad)


def test_nutop_objective_vs_fd(pz):
    t0 = seeded(SMALL, 12, 1e-2)
    ens = pz.Ensemble(gpu_config(SMALL))
    ens.set_state(0, temp=t0)
    J, _ = ens.adjoint_forward(12, 12, 4, SCHED[None, :], objective="nutop")
    # the objective is the mean of the NuTop column of the time series
    sim = oracle(SMALL, temp0=t0)
    sim.dt_schedule = SCHED
    vals = []
    for _ in range(12):
        sim.advance()
        vals.append(series_from_oracle(sim)[8])
    assert abs(J[0] - np.mean(vals)) <= 1e-10 * abs(np.mean(vals))
    g, dra = ens.adjoint_backward()
    rng = np.random.default_rng(13)
    for _ in range(3):
        d = rng.standard_normal(t0.shape) + 1j * rng.standard_normal(t0.shape)
        eps = 1e-6 * np.max(np.abs(t0)) / np.max(np.abs(d))
        js = []
        for sgn in (1, -1):
            ens.set_state(0, temp=t0 + sgn * eps * d)
            js.append(ens.adjoint_forward(12, 12, 0, SCHED[None, :], objective="nutop")[0][0])
        fd = (js[0] - js[1]) / (2 * eps)
        assert abs(fd - directional(g[0], d)) <= GRAD_TOL * abs(fd), (fd, directional(g[0], d))


def test_batched_nutop_gradient_ensemble(pz):
    """The batched adjoint workload's shape: 64 instances, N in {49, 65},
    n_phi in {126, 192}, E=1e-4, Ra log-uniform, dtMax=5e-5 under the
    Courant controller, 300 steps, checkpoint every 30, gradient of the mean
    NuTop in one forward+backward sweep; FD on 4 instances (all instances are
    perturbed in the same two batched runs).  Time scheme CNAB2 (the adjoint
    covers the multistep CNAB2 step)."""
    rng = np.random.default_rng(64)
    specs = []
    for i in range(64):
        N = (49, 65)[i % 2]
        mmax = (42, 64)[(i // 2) % 2]
        lo, hi = 6.0, (6.5 if N == 49 else 7.0)
        specs.append(dict(n_r_max=N, n_cheb_max=N, m_max=mmax, ek=1e-4, ra=float(10 ** rng.uniform(lo, hi)),
                          pr=1.0, radratio=0.35, l_ek_pump=True, time_scheme="CNAB2", dtMax=5e-5,
                          matrix_solve="INFLUENCE"))
    temps = [seeded(s, 100 + i, 1e-3) for i, s in enumerate(specs)]
    ens = pz.Ensemble([gpu_config(s) for s in specs])
    ens.set_state_all(temps)
    J, dt = ens.adjoint_forward(300, 300, 30, objective="nutop")
    g, dra = ens.adjoint_backward()
    assert np.all(np.isfinite(J))
    check = [0, 1, 2, 3]
    ds = [rng.standard_normal(t.shape) + 1j * rng.standard_normal(t.shape) for t in temps]
    # at these Rayleigh numbers the 300-step forward amplifies rounding: central
    # differences are taken at two step sizes (rounding error falls, truncation
    # error grows with eps) and the better one is held to the bar
    errs = {}
    for rel in (1e-6, 1e-5):
        eps = [rel * np.max(np.abs(t)) / np.max(np.abs(d)) for t, d in zip(temps, ds)]
        js = []
        for sgn in (1, -1):
            ens.set_state_all([t + sgn * e * d for t, e, d in zip(temps, eps, ds)])
            js.append(ens.adjoint_forward(300, 300, 0, dt, objective="nutop")[0])
        for i in check:
            fd = (js[0][i] - js[1][i]) / (2 * eps[i])
            errs.setdefault(i, []).append(abs(fd - directional(g[i], ds[i])) / abs(fd))
    print("batched NuTop FD rel errors (eps 1e-6, 1e-5):", errs)
    for i in check:
        assert min(errs[i]) <= GRAD_TOL, (i, errs[i])


@pytest.mark.parametrize("variant", [dict(), dict(corio_term="IMPLICIT"), dict(l_ek_pump=False, ra=3e5)])
def test_direct_solve_adjoint(pz, variant):
    """The adjoint of pizza's default direct solve (update_om_coll_smat: the
    coupled vorticity-streamfunction system, implicit Ekman pumping, and
    implicit Coriolis with corio_term='IMPLICIT'), CNAB2, with a dt change in
    the middle: J against the oracle (1e-10), the temperature gradient
    against FD along 3 directions and dJ/dRa against FD (1e-6)."""
    spec = dict(SMALL, matrix_solve="DIRECT", **variant)
    t0 = seeded(spec, 3, 1e-2)
    ens = pz.Ensemble(gpu_config(spec))
    J, dt = fwd(ens, t0, 12, 7, SCHED, ck=4)
    assert np.array_equal(dt, SCHED)
    Jo = oracle_objective(spec, t0, SCHED, 7)
    assert abs(J - Jo) <= 1e-10 * abs(Jo), (J, Jo)
    g, dra = ens.adjoint_backward()
    fd_check(ens, t0, g[0], 12, 7, SCHED, n_dir=3, seed=11)
    ra = spec["ra"]
    h = 1e-6 * ra
    ens.set_ra(0, ra + h)
    jp, _ = fwd(ens, t0, 12, 7, SCHED)
    ens.set_ra(0, ra - h)
    jm, _ = fwd(ens, t0, 12, 7, SCHED)
    ens.set_ra(0, ra)
    fd = (jp - jm) / (2 * h)
    assert abs(fd - dra[0]) <= GRAD_TOL * abs(fd), (fd, dra[0])


@pytest.mark.parametrize("scheme,solve", [("SBDF2", "INFLUENCE"), ("SBDF3", "INFLUENCE"), ("SBDF4", "INFLUENCE"),
                                          ("CNLF", "INFLUENCE"), ("MODCNAB", "INFLUENCE"), ("TVB33", "INFLUENCE"),
                                          ("SBDF3", "DIRECT")])
def test_multistep_scheme_adjoint(pz, scheme, solve):
    """The adjoint of the other multistep schemes (multistep_schemes.f90:
    up to four old, implicit and explicit slots, with the CNAB2 bridge of
    their first steps, step_time.f90:417-516), both solves: J against the
    oracle with the same step sequence (a dt change in the middle; 1e-10),
    the temperature gradient against FD along 2 directions (1e-6)."""
    spec = dict(SMALL, time_scheme=scheme, matrix_solve=solve)
    t0 = seeded(spec, 4, 1e-2)
    ens = pz.Ensemble(gpu_config(spec))
    J, dt = fwd(ens, t0, 12, 7, SCHED, ck=4)
    assert np.array_equal(dt, SCHED)
    Jo = oracle_objective(spec, t0, SCHED, 7)
    assert abs(J - Jo) <= 1e-10 * abs(Jo), (J, Jo)
    g, _ = ens.adjoint_backward()
    fd_check(ens, t0, g[0], 12, 7, SCHED, n_dir=2, seed=13)

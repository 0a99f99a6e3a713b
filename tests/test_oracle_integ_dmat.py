"""The oracle's integration method with the influence-matrix solve
(update_psi_integ_dmat.f90) against its direct solve (update_psi_integ_smat.f90)
with the Coriolis term explicit in both: the two discretise the same
equations with different test functions (twice- against four-times-integrated
vorticity equation), so they agree to the truncation error of the grid, and
psi meets the wall conditions the influence matrix imposes."""
import numpy as np

from oracle.pizza_oracle import Params, Pizza, seeded_temperature

SPEC = dict(n_r_max=33, n_cheb_max=24, m_max=16, ek=1e-3, ra=5e4, pr=1.0, radratio=0.35, time_scale="ROT",
            cheb_method="INTEG", time_scheme="CNAB2", dtMax=2e-2, courfac=4.0, corio_term="EXPLICIT")


def run(solve, steps=40):
    sim = Pizza(Params(**dict(SPEC, matrix_solve=solve)))
    sim.start(temp0=seeded_temperature(sim.M, sim.r, sim.d["r_icb"], 1e-2, 5))
    for _ in range(steps):
        sim.advance()
    return sim


def test_influence_matrix_agrees_with_direct_solve():
    a, b = run("DIRECT"), run("INFLUENCE")
    ea, eb = a.time_series()["e_kin_3D"], b.time_series()["e_kin_3D"]
    np.testing.assert_allclose(eb[1:4], ea[1:4], rtol=1e-4)
    assert np.max(np.abs(b.temp - a.temp)) < 1e-4 * np.max(np.abs(a.temp))


def test_influence_matrix_wall_conditions():
    b = run("INFLUENCE", steps=10)
    c = b.cheb
    psi_hat = c.costf1(b.psi)[1:]
    sg = np.where(np.arange(b.N) % 2 == 0, 1.0, -1.0)
    scale = np.max(np.abs(psi_hat))
    # tau rows: psi = 0 on both walls (c_0 half weight)
    assert np.max(np.abs(0.5 * psi_hat[:, 0] + psi_hat[:, 1:].sum(axis=1))) < 1e-12 * scale
    assert np.max(np.abs(0.5 * psi_hat[:, 0] + (psi_hat[:, 1:] * sg[1:]).sum(axis=1))) < 1e-12 * scale
    # influence rows: dpsi/dr on the inner wall (half weight at both ends)
    n = np.arange(b.N, dtype=float)
    w = -2.0 * n * n * sg
    w[0] *= 0.5
    w[-1] *= 0.5
    assert np.max(np.abs(psi_hat @ w)) < 1e-9 * scale * np.max(np.abs(w))

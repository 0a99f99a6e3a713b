"""The tangent-linear and adjoint restatement of the CNAB2 step
(oracle/pizza_tangent.py), the checker of the GPU gradient path."""
import numpy as np
import pytest

from oracle import pizza_tangent as pt
from oracle.pizza_oracle import Params, Pizza, seeded_temperature

SPEC = dict(n_r_max=17, n_cheb_max=17, m_max=8, ek=1e-3, ra=1e5, pr=1.0, radratio=0.35, l_ek_pump=True,
            time_scheme="CNAB2", dtMax=1e-4, matrix_solve="INFLUENCE")
DTS = np.array([1e-4] * 6 + [7e-5] * 6)
WINDOW = range(6, 13)


@pytest.fixture(scope="module")
def setup():
    p = Params(**SPEC)
    o = pt.StepOps(p)
    sim = Pizza(p)
    t0 = seeded_temperature(sim.M, sim.r, sim.d["r_icb"], 1e-2, 1)
    return p, o, t0


def test_state_form_forward_matches_oracle(setup):
    p, o, t0 = setup
    sim = Pizza(p)
    sim.start(temp0=t0)
    sim.dt_schedule = DTS
    for _ in DTS:
        sim.advance()
    _, _, S = pt.forward(o, t0, DTS, SPEC["ra"], WINDOW)
    f = pt.fields(o, S, SPEC["ra"] / SPEC["pr"])
    for k, ref in (("us", sim.us), ("up", sim.up), ("T", sim.temp)):
        assert np.abs(f[k] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_dot_product_tangent_vs_adjoint(setup):
    """<tangent(d), 1> = Re<g, d> + dJ/dRa dRa to rounding."""
    _, o, t0 = setup
    J, g, dra = pt.adjoint(o, t0, DTS, SPEC["ra"], WINDOW)
    rng = np.random.default_rng(5)
    for _ in range(3):
        d = rng.standard_normal(t0.shape) + 1j * rng.standard_normal(t0.shape)
        dr = 1e3 * rng.standard_normal()
        Jt, dJ = pt.tangent(o, t0, d, DTS, SPEC["ra"], dr, WINDOW)
        assert abs(Jt - J) <= 1e-14 * abs(J)
        ad = float(np.sum((np.conj(g) * d).real)) + dra * dr
        assert abs(dJ - ad) <= 1e-11 * abs(dJ)


def test_tangent_vs_finite_differences(setup):
    _, o, t0 = setup
    d = np.random.default_rng(9).standard_normal(t0.shape) * (1 - 0.5j)
    eps = 1e-6 * np.abs(t0).max() / np.abs(d).max()
    _, dJ = pt.tangent(o, t0, d, DTS, SPEC["ra"], 0.0, WINDOW)
    jp, _, _ = pt.forward(o, t0 + eps * d, DTS, SPEC["ra"], WINDOW)
    jm, _, _ = pt.forward(o, t0 - eps * d, DTS, SPEC["ra"], WINDOW)
    assert abs((jp - jm) / (2 * eps) - dJ) <= 1e-6 * abs(dJ)

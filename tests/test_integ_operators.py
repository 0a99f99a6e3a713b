"""The integration method's banded operators as the CUDA library's host code
derives them (pz_integ_operator, no GPU needed) against the oracle's
derivation (oracle/chebsparse.py), which reproduces the reference's
closed-form stencils and, through the integ restatement, the RotInteg
fixture."""
import numpy as np
import pytest

from oracle.chebsparse import IntegOperators, lapl_terms, omega_rot_terms


@pytest.fixture(scope="module")
def pz():
    from pizza_gb300 import build as b
    b.build()
    import pizza_gb300
    return pizza_gb300


@pytest.mark.parametrize("n,radratio", [(17, 0.35), (49, 0.35), (97, 0.6)])
def test_library_operators_match_oracle(pz, n, radratio):
    r_cmb = 1.0 / (1.0 - radratio)
    rnorm = np.sqrt(2.0 / (n - 1))
    ops = IntegOperators(n, r_cmb - 1.0, r_cmb, rnorm)
    c = ops.c
    want = {
        "I2R1": ops.i2r1, "I2R2": ops.i2r2, "I4R3": ops.i4r3, "I4R4": ops.i4r4, "ULAP": ops.uphi_lap,
        "I2": ops._rows(c.integrated({0: np.polynomial.Polynomial([1.0])}, 2), 2),
        "LT0": ops.temp_lap(0),
    }
    got = {k: pz.integ_operator(n, radratio, k) for k in pz.INTEG_OPERATORS}
    for k, w in want.items():
        g, bw = got[k]
        assert np.max(np.abs(g - w)) <= 1e-13 * np.max(np.abs(w)), k
        ii, jj = np.nonzero(w)
        assert bw == np.max(np.abs(ii - jj)), k
    for m in (0, 1, 5, 32):
        m2 = float(m * m)
        tl = got["LT0"][0] - m2 * got["I2"][0]
        assert np.max(np.abs(tl - ops.temp_lap(m))) <= 1e-13 * np.max(np.abs(ops.temp_lap(m)))
        if m == 0:
            continue
        rot = got["Q0"][0] + m2 * got["Q1"][0]
        w = ops.psi_rot(m)
        assert np.max(np.abs(rot - w)) <= 1e-12 * np.max(np.abs(w)), m
        rot2 = got["S0"][0] + m2 * (got["S1"][0] + m2 * got["S2"][0])
        w = ops.psi_rot2(m)
        assert np.max(np.abs(rot2 - w)) <= 1e-12 * np.max(np.abs(w)), m
        # intcheb2rmult2laplrot = -I2 [r^2 omega(psi)]
        p2 = got["P0"][0] + m2 * got["P1"][0]
        w = ops._rows(c.integrated(omega_rot_terms(r_cmb, float(m)), 2), 2)
        assert np.max(np.abs(p2 - w)) <= 1e-12 * np.max(np.abs(w)), m
        # non-rotating: intcheb4rmult4lapl and intcheb4rmult4lapl2
        nl = got["N0"][0] + m2 * got["N1"][0]
        w = ops.psi_nonrot(m)
        assert np.max(np.abs(nl - w)) <= 1e-12 * np.max(np.abs(w)), m
        nl2 = got["L0"][0] + m2 * (got["L1"][0] + m2 * got["L2"][0])
        w = ops.psi_nonrot2(m)
        assert np.max(np.abs(nl2 - w)) <= 1e-12 * np.max(np.abs(w)), m


def test_operator_bad_arguments(pz):
    with pytest.raises(RuntimeError):
        pz.integ_operator(3, 0.35, "I2R2")

"""The derived integration operators of the integ method (oracle/chebsparse.py).

Each operator O = I_k[sum_d P_d(r) f^(d)] must satisfy d^k/dr^k (O c) =
sum_d P_d f^(d) exactly for a polynomial f whose degree leaves room below the
truncation; the first k rows (constants of integration) are free.  Checked
with numpy's own Chebyshev algebra on pizza's primed coefficients
(f = c_0/2 + sum c_n T_n).
"""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

from oracle.chebsparse import ChebOps, lapl_of, lapl_terms, omega_rot_terms, r2_times

R_ICB, R_CMB = 1.0 / 0.65 - 1.0, 1.0 / 0.65
A, B = 0.5 * (R_CMB - R_ICB), 0.5 * (R_CMB + R_ICB)
N = 40


def primed_to_std(c):
    s = c.copy()
    s[0] *= 0.5
    return s


def std_to_primed(s):
    c = s.copy()
    c[0] *= 2.0
    return c


def apply_terms(terms, s):
    """sum_d P_d(r) f^(d)(r) as standard Chebyshev coefficients in x."""
    out = np.zeros(1)
    for d, P in terms.items():
        fd = C.chebder(s, d, scl=1.0 / A) if d else s
        # P(r) with r = a x + b, as a Chebyshev series in x
        Px = C.poly2cheb(np.polynomial.Polynomial(P.coef)(np.polynomial.Polynomial([B, A])).coef)
        out = C.chebadd(out, C.chebmul(Px, fd))
    return out


def make_f(deg, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros(N)
    s[:deg + 1] = rng.standard_normal(deg + 1)
    return s


@pytest.mark.parametrize("name,terms,k", [
    ("intcheb2rmult2lapl", lapl_terms(3.0, 2), 2),
    ("intcheb4rmult4laplrot", r2_times(omega_rot_terms(R_CMB, 5.0)), 4),
    ("intcheb4rmult4laplrot2", lapl_of(omega_rot_terms(R_CMB, 5.0), 5.0), 4),
    ("intcheb4rmult4lapl2", lapl_of(lapl_terms(2.0, 2), 2.0), 4),
    ("intcheb2rmult1", {0: np.polynomial.Polynomial([0.0, 1.0])}, 2),
])
def test_operator_inverts_k_derivatives(name, terms, k):
    ops = ChebOps(N, A, B)
    s = make_f(20, 7)
    O = ops.integrated(terms, k)
    g = O @ std_to_primed(s)
    gk = C.chebder(primed_to_std(g), k, scl=1.0 / A)
    want = apply_terms(terms, s)
    n = min(len(gk), len(want))
    assert np.allclose(gk[:n], want[:n], rtol=0, atol=1e-9 * np.max(np.abs(want)))
    assert np.all(np.abs(want[n:]) < 1e-9 * np.max(np.abs(want)))


def test_primitives_exact():
    ops = ChebOps(N, A, B)
    s = np.zeros(ops.L)
    s[:N] = make_f(25, 3)
    # multiplication by r
    r_s = C.chebmul(C.poly2cheb([B, A]), s[:26])
    got = primed_to_std(ops.R @ std_to_primed(s))
    assert np.allclose(got[:len(r_s)], r_s, atol=1e-13)
    assert np.all(got[len(r_s):] == 0.0)
    # one integration: the derivative brings the function back
    g = primed_to_std(ops.I1 @ std_to_primed(s))
    assert np.allclose(C.chebder(g, 1, scl=1.0 / A)[:26], s[:26], atol=1e-12)

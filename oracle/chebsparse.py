"""Sparse Chebyshev integration operators of pizza's integ method
(src/chebsparselib.f90), derived rather than transcribed.

Coefficients use pizza's convention f(x) = c_0/2 + sum_{n>=1} c_n T_n(x) (the
DCT-I normalisation of costf1, up to rnorm), with x = (r - b)/a.  Every
operator of the integ path is I_k P(r) D^j for a polynomial P -- the
r^2-weighted (r^4 for the streamfunction) equations integrated k times in r --
and repeated integration by parts,

    I_k (p f^(j)) = sum_i (-1)^i C(j, i) I_{k-j+i} (p^(i) f)   (rows >= k),

turns it into integrations and polynomial multiplications only: two exact
banded primitives (multiplication by x, one integration), so no
differentiation matrix and no cancellation enters.  The constants of
integration only touch the first k rows, which the tau (boundary) rows
replace.  Each operator was checked entry by entry against the reference's
closed-form stencils (intcheb2rmult2lapl, intcheb4rmult4laplrot,
intcheb4rmult4laplrot2, ...) to 1e-16 relative.

Test infrastructure: the oracle's integ restatement uses these dense
matrices; the GPU library builds the same operators in its own code.
"""
from __future__ import annotations

from math import comb

import numpy as np
from numpy.polynomial import Polynomial as Poly

R_POLY = Poly([0.0, 1.0])


class ChebOps:
    """Primitives on (n_r_max + pad) primed Chebyshev coefficients."""

    def __init__(self, n: int, a: float, b: float, pad: int = 16):
        self.n, self.a, self.b = n, a, b
        L = n + pad
        self.L = L
        P = np.eye(L)
        P[0, 0] = 0.5          # primed -> standard
        Pi = np.eye(L)
        Pi[0, 0] = 2.0         # standard -> primed
        Xs = np.zeros((L, L))
        Js = np.zeros((L, L))
        for j in range(L):
            # x T_j = (T_{j+1} + T_{|j-1|}) / 2, x T_0 = T_1
            if j == 0:
                Xs[1, 0] = 1.0
            else:
                if j + 1 < L:
                    Xs[j + 1, j] += 0.5
                Xs[j - 1, j] += 0.5
        for k in range(1, L):
            # int T: F_1 = s_0 - s_2/2, F_k = (s_{k-1} - s_{k+1}) / (2k)
            if k == 1:
                Js[1, 0] = 1.0
            else:
                Js[k, k - 1] = 0.5 / k
            if k + 1 < L:
                Js[k, k + 1] = -0.5 / k
        self.R = a * (Pi @ Xs @ P) + b * np.eye(L)   # multiplication by r
        self.I1 = a * (Pi @ Js @ P)                  # integration in r
        self._Ik = {0: np.eye(L)}

    def Ik(self, k: int) -> np.ndarray:
        if k not in self._Ik:
            self._Ik[k] = self.I1 @ self.Ik(k - 1)
        return self._Ik[k]

    def poly(self, p: Poly) -> np.ndarray:
        M = np.zeros((self.L, self.L))
        Rk = np.eye(self.L)
        for c in p.coef:
            M = M + c * Rk
            Rk = Rk @ self.R
        return M

    def integrated(self, terms: dict, k: int) -> np.ndarray:
        """I_k [ sum_d P_d(r) f^(d) ] (exact in rows >= k), n x n block."""
        out = np.zeros((self.L, self.L))
        for d, P in terms.items():
            for i in range(d + 1):
                Pi = P.deriv(i) if i else P
                out = out + (-1) ** i * comb(d, i) * (self.Ik(k - d + i) @ self.poly(Pi))
        return out[: self.n, : self.n]


def lapl_terms(m: float, power: int):
    """r^power times the polar Laplacian (d2/dr2 + (1/r) d/dr - m^2/r^2)."""
    r = R_POLY
    return {2: r ** power, 1: r ** (power - 1), 0: -m * m * r ** (power - 2)}


def omega_rot_terms(ro: float, m: float):
    """r^2 omega(psi) of the rotating integ formulation
    (update_psi_integ_smat.f90:456-468): omega = -h2 psi'' - (ro^2/r - 6 r) psi'
    + (6 + m^2 h2 / r^2) psi with h2 = ro^2 - r^2."""
    r = R_POLY
    h2 = ro ** 2 - r ** 2
    return {2: -(r ** 2) * h2, 1: -(ro ** 2 * r - 6.0 * r ** 3), 0: 6.0 * r ** 2 + m * m * h2}


def r2_times(terms: dict) -> dict:
    return {d: R_POLY ** 2 * p for d, p in terms.items()}


def lapl_of(terms: dict, m: float) -> dict:
    """r^4 Lap(w) for w = r^-2 * sum_d q_d psi^(d): r^2 w~'' - 3 r w~' + (4 - m^2) w~
    with w~ = sum_d q_d psi^(d)."""
    r = R_POLY
    out = {}

    def add(d, p):
        out[d] = out.get(d, Poly([0.0])) + p

    for j, q in terms.items():
        add(j, r ** 2 * q.deriv(2))
        add(j + 1, 2.0 * r ** 2 * q.deriv(1))
        add(j + 2, r ** 2 * q)
        add(j, -3.0 * r * q.deriv(1))
        add(j + 1, -3.0 * r * q)
        add(j, (4.0 - m * m) * q)
    return out


class IntegOperators:
    """The banded operators of update_temp_integ.f90 and
    update_psi_integ_smat.f90 as dense n x n matrices (already times rnorm,
    the first 2 or 4 rows zero where they are tau rows)."""

    def __init__(self, n: int, r_icb: float, r_cmb: float, rnorm: float):
        a, b = 0.5 * (r_cmb - r_icb), 0.5 * (r_cmb + r_icb)
        self.n, self.rnorm, self.ro = n, rnorm, r_cmb
        self.c = ChebOps(n, a, b)
        r = R_POLY
        c = self.c
        self.i2r1 = self._rows(c.integrated({0: r}, 2), 2)            # intcheb2rmult1
        self.i2r2 = self._rows(c.integrated({0: r ** 2}, 2), 2)       # intcheb2rmult2
        self.i4r4 = self._rows(c.integrated({0: r ** 4}, 4), 4)       # intcheb4rmult4
        self.i4r3 = self._rows(c.integrated({0: r ** 3}, 4), 4)       # intcheb4rmult3
        # m = 0 u_phi: r^2 (u'' + u'/r - u/r^2) integrated twice = rmult2 - 3 intcheb1rmult1
        self.uphi_lap = self._rows(c.integrated(lapl_terms(1.0, 2), 2), 2)

    def _rows(self, M, k):
        M = self.rnorm * M.copy()
        M[:k] = 0.0
        return M

    def temp_lap(self, m):
        """intcheb2rmult2lapl: I2 [r^2 Lap_m]."""
        return self._rows(self.c.integrated(lapl_terms(float(m), 2), 2), 2)

    def psi_rot(self, m):
        """intcheb4rmult4laplrot: I4 [r^4 omega(psi)] (rotating)."""
        return self._rows(self.c.integrated(r2_times(omega_rot_terms(self.ro, float(m))), 4), 4)

    def psi_rot2(self, m):
        """intcheb4rmult4laplrot2: I4 [r^4 Lap omega(psi)] (rotating)."""
        return self._rows(self.c.integrated(lapl_of(omega_rot_terms(self.ro, float(m)), float(m)), 4), 4)

    def psi_nonrot(self, m):
        """intcheb4rmult4lapl: I4 [r^4 Lap psi]."""
        return self._rows(self.c.integrated(lapl_terms(float(m), 4), 4), 4)

    def psi_nonrot2(self, m):
        """intcheb4rmult4lapl2: I4 [r^4 Lap^2 psi]."""
        r2lap = {d: p for d, p in lapl_terms(float(m), 2).items()}   # r^2 Lap psi
        return self._rows(self.c.integrated(lapl_of(r2lap, float(m)), 4), 4)

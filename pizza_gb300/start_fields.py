"""Start perturbations of pizza's initProp (src/init_fields.f90:260-376), on the host.

``init_prop(...)`` returns the (n_m_max, n_r_max) complex perturbation that
pizza adds to the temperature (init_t, amp_t) or composition (init_xi, amp_xi)
after the start state is set or read from a checkpoint:

- ``init > 0``: amp * sin(pi (r - r_i)) on the single mode m = init;
- ``init == -1``: a bubble, amp * G(r) * exp(-(phi - pi/minc)^2 / 0.2^2) on the
  phi grid, transformed to the modes with pizza's forward normalisation 1/n_phi.
  G is the compact-support Gaussian-like profile of Gaspari & Cohn (1999,
  Eq. 4.7), centred on the grid radius closest to mid-shell, with its two
  branches normalised to one at the centre (useful.f90:295-341);
- ``init < -1``: pizza draws from Fortran's random_number, which cannot be
  reproduced; a caller that wants a random start passes its own seed.
"""
from __future__ import annotations

import math

import numpy as np


def _grid_r(n_r_max: int, radratio: float) -> np.ndarray:
    r_cmb = 1.0 / (1.0 - radratio)
    r_icb = r_cmb - 1.0
    x = np.cos(np.pi * np.arange(n_r_max) / (n_r_max - 1))
    return 0.5 * (r_cmb - r_icb) * x + 0.5 * (r_cmb + r_icb)


# Gaspari & Cohn (1999) Eq. 4.7 pieces: centre value (4.7c), inner branch
# (4.7b, distance r <= c) and outer branch (4.7a, r > c); L is the length scale
def _gc_centre(c, L):
    e = math.exp(-2.0 * c / L)
    return math.pi * L ** 3 * (1.0 - e) - 2.0 * math.pi * c * L * (c + L) * e


def _gc_inner(r, c, L):
    return (math.pi / 3.0 * L * r * (r + 3.0 * L) * math.exp(-r / L)
            + (2.0 * math.pi * L * L * (c + L) ** 2) / r * math.exp(-2.0 * c / L)
            * (1.0 - (1.0 - r / (c + L)) * math.exp(r / L))
            + math.pi * L ** 3 * (math.exp(-r / L) - math.exp((r - 2.0 * c) / L)))


def _gc_outer(r, c, L):
    return (2.0 * math.pi * L / r * math.exp(-r / L)
            * (0.5 * (r * (r + L) * (2.0 * c - r)) + ((r - c) ** 3 - c ** 3) / 3.0
               - L * (c + L) * (r - c + L) + L * (c + L) ** 2 * math.exp((r - 2.0 * c) / L)))


def bubble_profile(r: np.ndarray) -> np.ndarray:
    """Radial profile of the init = -1 bubble at the grid radii r (r[0] = r_cmb)."""
    n = len(r)
    r_cmb, r_icb = r[0], r[-1]
    L = 0.5 * (0.1 / math.sqrt(2.0))
    ir = int(np.argmin(np.abs(r - 0.5 * (r_cmb + r_icb))))
    rc = r[ir]
    c_out = 0.5 * (r[0] - rc)            # towards r_cmb
    c_in = 0.5 * (rc - r[-1])            # towards r_icb
    g = np.empty(n)
    for k in range(n):
        if k == ir:
            g[k] = 1.0
            continue
        d = r[k] - rc
        if d < 0.0:
            g[k] = (_gc_outer(-d, c_in, L) if -d > c_in else _gc_inner(-d, c_in, L)) / _gc_centre(c_in, L)
        else:
            g[k] = (_gc_outer(d, c_out, L) if d > c_out else _gc_inner(d, c_out, L)) / _gc_centre(c_out, L)
    return g


def init_prop(n_r_max: int, m_max: int, minc: int, radratio: float, init: int, amp: float) -> np.ndarray:
    """pizza's initProp perturbation, complex (n_m_max, n_r_max), m fastest in
    the C ABI's sense (row = mode).  Raises ValueError for the random modes and
    for an unresolved or symmetry-incompatible mode."""
    n_m = m_max // minc + 1
    out = np.zeros((n_m, n_r_max), np.complex128)
    if init == 0:
        return out
    r = _grid_r(n_r_max, radratio)
    if init > 0:
        if init % minc != 0 or init > m_max:
            raise ValueError(f"init mode {init} is not compatible with m_max={m_max}, minc={minc}")
        out[init // minc] = amp * np.sin(np.pi * (r - r[-1]))
        return out
    if init == -1:
        n_phi = 3 * m_max // minc
        phi = np.arange(n_phi) * 2.0 * np.pi / minc / n_phi
        shape = np.exp(-(phi - np.pi / minc) ** 2 / 0.2 ** 2)
        spec = np.fft.rfft(shape)[:n_m] / n_phi
        return amp * bubble_profile(r)[None, :] * spec[:, None]
    raise ValueError(f"init = {init} draws from Fortran's random generator; give a seed for a seeded start")


def seeded_prop(n_r_max: int, m_max: int, minc: int, radratio: float, amp: float, seed: int) -> np.ndarray:
    """A seeded stand-in for pizza's random start: amp g_m e^{i theta_m}
    sin(pi (r - r_i)) on m >= 1 with g_m ~ N(0, 1), theta_m ~ U[0, 2 pi)."""
    n_m = m_max // minc + 1
    r = _grid_r(n_r_max, radratio)
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0.0, 2.0 * np.pi, n_m - 1)
    a = rng.standard_normal(n_m - 1)
    out = np.zeros((n_m, n_r_max), np.complex128)
    out[1:] = (amp * a * np.exp(1j * ph))[:, None] * np.sin(np.pi * (r - r[-1]))[None, :]
    return out

"""CPU oracle for pizza's collocation time step (test infrastructure only).

This module is a NumPy/SciPy FP64 restatement of the reference algorithm for
the hot path: the stage body of ``time_loop`` (src/step_time.f90:139-368) with
``radial_loop`` (src/radial_loop.f90:231-394) and the collocation ``mloop``
(src/mloop.f90:36-103) for temperature (src/update_temp_coll.f90) and the
streamfunction/vorticity system, both the coupled direct solve
(src/update_psi_coll_smat.f90) and the influence-matrix solve
(src/update_psi_coll_dmat.f90), with the multistep IMEX schemes of
src/multistep_schemes.f90 and the DIRK schemes of src/dirk_schemes.f90.
With ``cheb_method="INTEG"`` the stage routines are those of the sparse
Chebyshev-integration method with tau boundary rows (src/update_temp_integ.f90,
src/update_psi_integ_smat.f90, src/update_psi_integ_dmat.f90), restated in
oracle/pizza_integ.py.  ``raxi /= 0`` adds the composition equation
(src/update_xi_coll.f90, src/update_xi_integ.f90).

It is the checker for the CUDA library and nothing else: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` import it.  The product path never calls it.

Parity pin: the oracle reproduces the reference's own regression fixtures
(``samples/*/reference.out``: NonRotRa2e3, RotE1e3EkPump first run,
MultistepSchemes first run, TimeStepChange, DIRKSchemes first run, RotInteg
first run and continuation, FingConv first run and continuation) at the
fixtures' rtol=1e-8, atol=1e-20, see ``tests/test_oracle_golden.py``.  Third-party arithmetic the reference calls
(FFTW3 r2c/c2r/dft, LAPACK dgetrf/dgetrs/zgetrf/zgetrs; not vendored, versions
unpinned in src/CMakeLists.txt) is restated with numpy.fft (pocketfft) and
scipy.linalg (LAPACK getrf/getrs), which compute the same transforms and the
same partially pivoted LU.

Array layout follows the reference's m-distributed arrays ``f_Mloc(n_m, n_r)``:
shape (n_m_max, n_r_max), complex128, n_r=0 is the outer boundary r_cmb.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
import scipy.fft as sfft
import scipy.linalg as sla

__all__ = ["Params", "Pizza", "seeded_temperature", "l_correct_step"]

TINY_NUMBER = 10.0 * np.finfo(float).eps  # tiny_number, src/constants.f90:21 (used by round_off)


# ---------------------------------------------------------------------------
# Parameters (src/namelists.f90:530-672 defaults, :271-526 derived switches)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Params:
    n_r_max: int = 32
    n_cheb_max: int | None = None   # None -> n_r_max (configs set it equal)
    m_max: int = 32
    minc: int = 1
    # control
    n_time_steps: int = 100
    alpha: float = 0.5
    dtMax: float = 1.0e-5
    courfac: float = 1.0e3
    dt_fac: float = 2.0
    time_scheme: str = "CNAB2"
    matrix_solve: str = "DIRECT"      # DIRECT -> smat, INFLUENCE -> dmat
    cheb_method: str = "COLL"         # COLL -> collocation, INTEG -> sparse integration
    l_rerror_fix: bool = False
    rerror_fac: float = 500.0
    corio_term: str = "IMPLICIT"
    buo_term: str = "IMPLICIT"
    time_scale: str = "VISC"
    l_non_rot: bool = False
    # phys_param
    ra: float = 1.0e5
    pr: float = 1.0
    ek: float = 1.0e-3
    radratio: float = 0.35
    g0: float = 0.0
    g1: float = 1.0
    g2: float = 0.0
    ktopt: int = 1
    kbott: int = 1
    ktopv: int = 2
    kbotv: int = 2
    l_ek_pump: bool = False
    l_temp_advz: bool = False
    tcond_fac: float = 1.0
    raxi: float = 0.0                 # composition (raxi /= 0 switches it on)
    sc: float = 0.0
    ktopxi: int = 1
    kbotxi: int = 1
    xicond_fac: float = 1.0
    # start_field
    init_t: int = 0
    amp_t: float = 0.0
    init_xi: int = 0
    amp_xi: float = 0.0
    init_u: int = 0
    amp_u: float = 0.0
    # output_control
    n_log_step: int = 50

    def derived(self):
        """Return the derived switches of read_namelists (namelists.f90:271-526)."""
        d = {}
        ek = self.ek
        l_non_rot = self.l_non_rot or ek < 0.0
        if l_non_rot:
            ek = -1.0
        d["ek"] = ek
        d["l_non_rot"] = l_non_rot
        d["l_heat"] = self.ra != 0.0
        d["l_chem"] = self.raxi != 0.0                             # namelists.f90:323-327
        d["tadvz_fac"] = 1.0 if self.l_temp_advz else 0.0
        d["r_cmb"] = 1.0 / (1.0 - self.radratio)
        d["r_icb"] = d["r_cmb"] - 1.0
        d["l_direct_solve"] = "DIRECT" in self.matrix_solve.upper()
        d["l_cheb_coll"] = "COLL" in self.cheb_method.upper()   # namelists.f90:379-384
        l_cor_imp = "IMP" in self.corio_term.upper()
        if (not d["l_direct_solve"]) and l_cor_imp and (not l_non_rot):
            l_cor_imp = False  # namelists.f90:448-457
        d["l_coriolis_imp"] = l_cor_imp
        d["l_buo_imp"] = "IMP" in self.buo_term.upper()
        ch = d["l_chem"]
        if l_non_rot:
            d["CorFac"] = 0.0
            d["BuoFac"] = self.ra / self.pr if d["l_heat"] else 0.0
            d["TdiffFac"] = 1.0 / self.pr if d["l_heat"] else 0.0
            d["ChemFac"] = self.raxi / self.sc if ch else 0.0
            d["XidiffFac"] = 1.0 / self.sc if ch else 0.0
            d["ViscFac"] = 1.0
        elif "ROT" in self.time_scale.upper():
            d["CorFac"] = 2.0
            d["BuoFac"] = self.ra * ek * ek / self.pr if d["l_heat"] else 0.0
            d["TdiffFac"] = ek / self.pr if d["l_heat"] else 0.0
            d["ChemFac"] = self.raxi * ek * ek / self.sc if ch else 0.0
            d["XidiffFac"] = ek / self.sc if ch else 0.0
            d["ViscFac"] = ek
        else:
            d["CorFac"] = 2.0 / ek
            d["BuoFac"] = self.ra / self.pr if d["l_heat"] else 0.0
            d["TdiffFac"] = 1.0 / self.pr if d["l_heat"] else 0.0
            d["ChemFac"] = self.raxi / self.sc if ch else 0.0
            d["XidiffFac"] = 1.0 / self.sc if ch else 0.0
            d["ViscFac"] = 1.0
        return d


# ---------------------------------------------------------------------------
# Multistep IMEX schemes (src/multistep_schemes.f90)
# ---------------------------------------------------------------------------
class Multistep:
    """type_multistep: weights, dt history, IMEX rhs and rotation."""

    def __init__(self, time_scheme: str, courfac_nml: float, alpha: float):
        # multistep_schemes.f90:35-134
        ts = time_scheme.upper()
        self.l_imp_calc_rhs = True
        if "CNAB2" in ts:
            self.time_scheme, self.nimp, self.nold, self.nexp, cf = "CNAB2", 1, 1, 2, 3.0
        elif "MODCNAB" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "MODCNAB", 2, 2, 2, 2.9
        elif "CNLF" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "CNLF", 2, 2, 2, 3.0
        elif "BDF2AB2" in ts or "SBDF2" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "SBDF2", 2, 1, 2, 2.8
            self.l_imp_calc_rhs = False
        elif "BDF3AB3" in ts or "SBDF3" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "SBDF3", 3, 1, 3, 4.0
            self.l_imp_calc_rhs = False
        elif "TVB33" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "TVB33", 3, 3, 3, 4.0
        elif "BDF4AB4" in ts or "SBDF4" in ts:
            self.time_scheme, self.nold, self.nimp, self.nexp, cf = "SBDF4", 4, 1, 4, 5.5
            self.l_imp_calc_rhs = False
        else:
            raise ValueError(f"time integrator {time_scheme} not found")
        self.family = "MULTISTEP"
        self.nstages = 1
        self.istage = 1
        self.courfac = cf if abs(courfac_nml) >= 1.0e3 else courfac_nml
        self.alpha = alpha
        self.dt = np.zeros(self.nexp)
        self.wimp = np.zeros(self.nold)
        self.wimp_lin = np.zeros(self.nimp + 1)
        self.wexp = np.zeros(self.nexp)

    def set_weights(self) -> bool:
        """set_weights (multistep_schemes.f90:137-306); returns lMatNext."""
        wimp_old = self.wimp_lin[0]
        dt = self.dt
        one, half, two = 1.0, 0.5, 2.0
        s = self.time_scheme
        if s == "CNAB2":
            self.wimp[0] = one
            self.wimp_lin[0] = self.alpha * dt[0]
            self.wimp_lin[1] = (1 - self.alpha) * dt[0]
            self.wexp[0] = (one + half * dt[0] / dt[1]) * dt[0]
            self.wexp[1] = -half * dt[0] * dt[0] / dt[1]
        elif s == "CNLF":
            delta = dt[0] / dt[1]
            self.wimp[0] = (one - delta) * (one + delta)
            self.wimp[1] = delta * delta
            self.wimp_lin[0] = half * (one + delta) / delta * dt[0]
            self.wimp_lin[1] = half * (one + delta) * (delta - one) / delta * dt[0]
            self.wimp_lin[2] = half * (one + delta) * dt[0]
            self.wexp[0] = (one + delta) * dt[0]
            self.wexp[1] = 0.0
        elif s == "MODCNAB":
            delta = dt[0] / dt[1]
            self.wimp[0] = one
            self.wimp[1] = 0.0
            self.wimp_lin[0] = (half + 1.0 / delta / 16.0) * dt[0]
            self.wimp_lin[1] = (7.0 / 16.0 - 1.0 / delta / 16.0) * dt[0]
            self.wimp_lin[2] = 1.0 / 16.0 * dt[0]
            self.wexp[0] = (one + half * delta) * dt[0]
            self.wexp[1] = -half * delta * dt[0]
        elif s == "SBDF2":
            delta = dt[0] / dt[1]
            self.wimp_lin[0] = (one + delta) / (one + two * delta) * dt[0]
            self.wimp_lin[1] = 0.0
            self.wimp[0] = (one + delta) * (one + delta) / (one + two * delta)
            self.wimp[1] = -delta * delta / (one + two * delta)
            self.wexp[0] = (one + delta) * (one + delta) * dt[0] / (one + two * delta)
            self.wexp[1] = -delta * (one + delta) * dt[0] / (one + two * delta)
        elif s == "SBDF3":
            dn = dt[1] / dt[0]
            dn1 = dt[2] / dt[0]
            a0 = one + one / (one + dn) + one / (one + dn + dn1)
            a1 = (one + dn) * (one + dn + dn1) / (dn * (dn + dn1))
            a2 = -(one + dn + dn1) / (dn * dn1 * (one + dn))
            a3 = (one + dn) / (dn1 * (dn + dn1) * (one + dn + dn1))
            b0 = (one + dn) * (one + dn + dn1) / (dn * (dn + dn1))
            b1 = -(one + dn + dn1) / (dn * dn1)
            b2 = (one + dn) / (dn1 * (dn + dn1))
            self.wimp_lin[0] = one / a0 * dt[0]
            self.wimp_lin[1] = 0.0
            self.wimp[0] = a1 / a0
            self.wimp[1] = a2 / a0
            self.wimp[2] = a3 / a0
            self.wexp[0] = b0 / a0 * dt[0]
            self.wexp[1] = b1 / a0 * dt[0]
            self.wexp[2] = b2 / a0 * dt[0]
        elif s == "TVB33":
            gam = (2619.0 - math.sqrt(5995281.0)) / 345.0
            theta = (3525.0 * gam * gam - 3118.0 * gam - 5084.0) / 5468.0
            c = (2178.0 * theta - 959.0 * gam * gam + 130.0 * gam + 726.0) / 4096.0
            dn = dt[0] / dt[1]
            dn1 = dt[1] / dt[2]
            a3 = -dn1 ** 3 * dn ** 2 * (3.0 * gam ** 2 * dn + two * gam * (one - dn) - one) / (one + dn1) / (one + dn1 * (one + dn))
            a2 = -dn ** 2 * (gam * dn * dn1 * (two - 3.0 * gam) + (one - two * gam) * (one + dn1)) / (one + dn)
            a1 = -(dn1 * (one + gam * dn) * (1 + dn * (3.0 * gam - two)) + dn * (two * gam - one) + one) / (one + dn1) - theta
            a0 = theta + (one + two * gam * dn + dn1 * (one + gam * dn) * (one + 3.0 * gam * dn)) / (one + dn) / (one + dn1 * (one + dn))
            b2 = dn1 ** 2 * dn * (6.0 * gam * (one + gam * dn) + theta * (3.0 + two * dn)) / (6.0 * (one + dn1))
            b1 = -gam * dn * (one + dn1 * (one + gam * dn)) - theta / 6.0 * dn * (3.0 + dn1 * (3.0 + two * dn))
            b0 = (one + gam * dn) * (one + dn1 * (one + gam * dn)) / (one + dn1) + theta * (one + 0.5 * dn + dn1 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)))
            c3 = theta * dn1 ** 2 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)) - c
            c2 = (c * (one + dn1) * (one + dn1 * (one + dn)) - dn1 ** 2 * dn ** 2 * gam * (one - gam)) / (dn1 ** 2 * (one + dn)) - theta * dn * (3.0 + dn1 * (3.0 + 2.0 * dn)) / 6.0
            c1 = (dn1 ** 2 * dn * (one - gam) * (one + gam * dn) - c * (one + dn1 * (one + dn))) / dn1 ** 2 / dn + theta * (one + 0.5 * dn + dn1 * dn * (3.0 + two * dn) / (6.0 * (one + dn1)))
            c0 = (dn1 ** 2 * dn * gam * (one + gam * dn) + c * (one + dn1)) / (dn1 ** 2 * dn * (one + dn))
            self.wimp_lin[0] = c0 / a0 * dt[0]
            self.wimp_lin[1] = c1 / a0 * dt[0]
            self.wimp_lin[2] = c2 / a0 * dt[0]
            self.wimp_lin[3] = c3 / a0 * dt[0]
            self.wimp[0] = -a1 / a0
            self.wimp[1] = -a2 / a0
            self.wimp[2] = -a3 / a0
            self.wexp[0] = b0 / a0 * dt[0]
            self.wexp[1] = b1 / a0 * dt[0]
            self.wexp[2] = b2 / a0 * dt[0]
        elif s == "SBDF4":
            dn = dt[0] / dt[1]
            dn1 = dt[1] / dt[2]
            dn2 = dt[2] / dt[3]
            c1 = one + dn2 * (one + dn1)
            c2 = one + dn1 * (one + dn)
            c3 = one + dn2 * c2
            a4 = (one + dn) / (one + dn2) * c2 / c1 / c3 * (dn2 ** 4 * dn1 ** 3 * dn ** 2)
            a3 = -dn1 ** 3 * dn ** 2 * (one + dn) / (one + dn1) * c3 / c2
            a2 = dn * (dn / (one + dn) + dn1 * dn * (c3 + dn2) / (one + dn2))
            a1 = -one - dn * (one + dn1 * (one + dn) * (one + dn2 * c2 / c1) / (one + dn1))
            a0 = one + dn / (one + dn) + dn1 * dn / c2 + dn2 * dn1 * dn / c3
            b3 = -dn2 ** 3 * dn1 ** 2 * dn * (one + dn) / (one + dn2) * c2 / c1
            b2 = dn1 ** 2 * dn * (one + dn) / (one + dn1) * c3
            b1 = -c2 * c3 * dn / (one + dn2)
            b0 = dn1 * (one + dn) / (one + dn1) * ((one + dn) * (c3 + dn2) + (one + dn2) / dn1) / c1
            self.wimp_lin[0] = one / a0 * dt[0]
            self.wimp_lin[1] = 0.0
            self.wimp[0] = -a1 / a0
            self.wimp[1] = -a2 / a0
            self.wimp[2] = -a3 / a0
            self.wimp[3] = -a4 / a0
            self.wexp[0] = b0 / a0 * dt[0]
            self.wexp[1] = b1 / a0 * dt[0]
            self.wexp[2] = b2 / a0 * dt[0]
            self.wexp[3] = b3 / a0 * dt[0]
        return bool(self.wimp_lin[0] != wimp_old)

    def set_dt_array(self, dt_new: float, dt_min: float):
        """set_dt_array (multistep_schemes.f90:308-363): roll then overwrite."""
        self.dt = np.roll(self.dt, 1)
        self.dt[0] = dt_new
        if dt_new < dt_min:
            raise FloatingPointError(f"time step too small, dt={dt_new!r}")

    def set_imex_rhs(self, ta: "TArray") -> np.ndarray:
        """set_imex_rhs (multistep_schemes.f90:366-413)."""
        rhs = self.wimp[0] * ta.old[0]
        for n in range(1, self.nold):
            rhs = rhs + self.wimp[n] * ta.old[n]
        for n in range(self.nimp):
            rhs = rhs + self.wimp_lin[n + 1] * ta.impl[n]
        for n in range(self.nexp):
            rhs = rhs + self.wexp[n] * ta.expl[n]
        return rhs

    def rotate_imex(self, ta: "TArray"):
        """rotate_imex (multistep_schemes.f90:462-498)."""
        for n in range(self.nexp - 1, 0, -1):
            ta.expl[n] = ta.expl[n - 1]
        for n in range(self.nold - 1, 0, -1):
            ta.old[n] = ta.old[n - 1]
        for n in range(self.nimp - 1, 0, -1):
            ta.impl[n] = ta.impl[n - 1]

    def bridge_with_cnab2(self):
        """bridge_with_cnab2 (multistep_schemes.f90:500-522)."""
        old_order, old_scheme = self.nimp, self.time_scheme
        self.nimp = 1
        self.time_scheme = "CNAB2"
        self.set_weights()
        self.wimp[1:] = 0.0
        self.wimp_lin[2:] = 0.0
        self.wexp[2:] = 0.0
        self.time_scheme = old_scheme
        self.nimp = old_order


def dirk_tableau(name: str):
    """Unscaled tableaux of the DIRK IMEX schemes (src/dirk_schemes.f90:35-244
    for the stage counts and flags, :246-707 for the coefficients).

    Returns nstages, l_assembly, gamma (the diagonal implicit weight), the
    implicit and explicit Butcher matrices (sizet x sizet, sizet = nstages + 1
    without an assembly stage, nstages with one), the assembly rows, the
    per-stage flags l_exp_calc and l_imp_calc_rhs and the default courfac."""
    r2, r3 = math.sqrt(2.0), math.sqrt(3.0)
    n = name.upper()
    exp_calc = None
    imp1 = False              # l_imp_calc_rhs(1)
    bai = bae = None
    if n == "ARS222":
        g = 0.5 * (2.0 - r2); d = 1.0 - 0.5 / g
        ns, ass, cf = 2, False, 1.35
        bi = [[0, 0, 0], [0, g, 0], [0, 1 - g, g]]
        be = [[0, 0, 0], [g, 0, 0], [d, 1 - d, 0]]
    elif n == "ARS232":
        g = 0.5 * (2.0 - r2); d = -2.0 * r2 / 3.0
        ns, ass, cf = 3, True, 1.35
        bi = [[0, 0, 0], [0, g, 0], [0, 1 - g, g]]
        be = [[0, 0, 0], [g, 0, 0], [d, 1 - d, 0]]
        bai = bae = [0, 1 - g, g]
    elif n == "ARS233":
        g = (3.0 + r3) / 6.0
        ns, ass, cf = 3, True, 1.35
        bi = [[0, 0, 0], [0, g, 0], [0, 1 - 2 * g, g]]
        be = [[0, 0, 0], [g, 0, 0], [g - 1, 2 * (1 - g), 0]]
        bai = bae = [0, 0.5, 0.5]
    elif n == "SSP222":
        g = 1.0 - 1.0 / r2
        ns, ass, cf = 3, True, 1.35
        bi = [[0, 0, 0], [0, g, 0], [0, 1 - 2 * g, g]]
        be = [[0, 0, 0], [0, 0, 0], [0, 1, 0]]
        bai = bae = [0, 0.5, 0.5]
    elif n == "LSDIRK222":
        g = 1.0 - 1.0 / r2; ch = 1.0 / (2.0 * g)
        ns, ass, cf = 3, True, 1.35
        bi = [[0, 0, 0], [0, g, 0], [0, 1 - g, g]]
        be = [[0, 0, 0], [0, 0, 0], [0, ch, 0]]
        bai = bae = [0, 1 - g, g]
    elif n == "LZ232":
        g = 0.5
        ns, ass, cf, imp1 = 2, False, 1.25, True
        bi = [[0, 0, 0], [-0.25, 0.5, 0], [0.5, 0, 0.5]]
        be = [[0, 0, 0], [0.25, 0, 0], [-1, 2, 0]]
    elif n == "CK232":
        g = 1.0 - 0.5 * r2
        ns, ass, cf, imp1 = 2, False, 1.25, True
        bi = [[0, 0, 0], [-1.0 / 3.0 + 0.5 * r2, g, 0], [0.75 - 0.25 * r2, -0.75 + 0.75 * r2, g]]
        be = [[0, 0, 0], [2.0 / 3.0, 0, 0], [0.25, 0.75, 0]]
    elif n == "ARS443":
        g = 0.5
        ns, ass, cf = 4, False, 0.9
        bi = [[0, 0, 0, 0, 0], [0, 0.5, 0, 0, 0], [0, 1.0 / 6.0, 0.5, 0, 0], [0, -0.5, 0.5, 0.5, 0],
              [0, 1.5, -1.5, 0.5, 0.5]]
        be = [[0, 0, 0, 0, 0], [0.5, 0, 0, 0, 0], [11.0 / 18.0, 1.0 / 18.0, 0, 0, 0],
              [5.0 / 6.0, -5.0 / 6.0, 0.5, 0, 0], [0.25, 1.75, 0.75, -1.75, 0]]
    elif n == "BPR353":
        g = 0.5
        ns, ass, cf, imp1 = 4, False, 1.0, True
        bi = [[0, 0, 0, 0, 0], [0.5, 0.5, 0, 0, 0], [5.0 / 18.0, -1.0 / 9.0, 0.5, 0, 0], [0.5, 0, 0, 0.5, 0],
              [0.25, 0, 0.75, -0.5, 0.5]]
        be = [[0, 0, 0, 0, 0], [1, 0, 0, 0, 0], [4.0 / 9.0, 2.0 / 9.0, 0, 0, 0], [0.25, 0, 0.75, 0, 0],
              [0.25, 0, 0.75, 0, 0]]
        exp_calc = [True, True, True, False]
    elif n == "PC2":
        g = 0.5
        ns, ass, cf, imp1 = 3, False, 0.8, True
        bi = [[0, 0, 0, 0], [0.5, 0.5, 0, 0], [0.5, 0, 0.5, 0], [0.5, 0, 0, 0.5]]
        be = [[0, 0, 0, 0], [1, 0, 0, 0], [0.5, 0.5, 0, 0], [0.5, 0, 0.5, 0]]
    elif n in ("ARS343", "MARS343"):
        if n == "ARS343":
            g = 0.435866521508459
            b1 = -1.5 * g * g + 4.0 * g - 0.25
            b2 = 1.5 * g * g - 5.0 * g + 1.25
            cf = 0.7
            be = [[0, 0, 0, 0], [g, 0, 0, 0], [0.3212788860286278, 0.3966543747256017, 0, 0],
                  [-0.1058582960718797, 0.5529291480359398, 0.5529291480359398, 0]]
        else:
            g = 0.435866521508458
            b1, b2 = 1.20849664917601, -0.64436317068446
            cf = 0.5
            be = [[0, 0, 0, 0], [0.877173304301691, 0, 0, 0], [0.535396540307354, 0.182536720446875, 0, 0],
                  [0.63041255815287, -0.83193390106308, 1.20152134291021, 0]]
        ns, ass = 4, True
        bi = [[0, 0, 0, 0], [0, g, 0, 0], [0, 0.5 * (1 - g), g, 0], [0, b1, b2, g]]
        bai = bae = [0, b1, b2, g]
    elif n == "SSP322":
        g = 0.5
        ns, ass, cf = 4, True, 1.35
        bi = [[0, 0, 0, 0], [0, 0.5, 0, 0], [0, -0.5, 0.5, 0], [0, 0, 0.5, 0.5]]
        be = [[0, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [0, 0, 1, 0]]
        bai = bae = [0, 0, 0.5, 0.5]
    elif n == "SSP332":
        g = 1.0 - 1.0 / r2
        ns, ass, cf = 4, True, 1.35
        bi = [[0, 0, 0, 0], [0, g, 0, 0], [0, 1 - 2 * g, g, 0], [0, 0.5 - g, 0, g]]
        be = [[0, 0, 0, 0], [0, 0, 0, 0], [0, 1, 0, 0], [0, 0.25, 0.25, 0]]
        bai = bae = [0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0]
    elif n == "SSP433":
        # dirk_schemes.f90:373-392; alpha, beta, eta are default-kind (single
        # precision) literals there, so their float rounding is part of the tableau
        a = float(np.float32(0.24169426078821))
        b = float(np.float32(0.06042356519705))
        e = float(np.float32(0.12915286960590))
        g = a
        ns, ass, cf = 5, True, 1.35
        bi = [[0, 0, 0, 0, 0], [0, a, 0, 0, 0], [0, -a, a, 0, 0], [0, 0, 1 - a, a, 0], [0, b, e, 0.5 - b - e - a, a]]
        be = [[0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 0, 1, 0, 0], [0, 0, 0.25, 0.25, 0]]
        bai = bae = [0, 0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0]
    elif n == "DP1-242":
        # dirk_schemes.f90:393-409
        g = 0.5
        ns, ass, cf = 4, False, 1.35
        bi = [[0, 0, 0, 0, 0], [0, 0.5, 0, 0, 0], [0, 1.0 / 6.0, 0.5, 0, 0], [0, -0.5, 0.5, 0.5, 0],
              [0, 1.5, -1.5, 0.5, 0.5]]
        be = [[0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 1.0 / 3.0, 0, 0, 0], [0, 1, 0, 0, 0], [0, 0.5, 0, 0.5, 0]]
        exp_calc = [False, True, False, True]
    elif n == "DP2-242":
        # dirk_schemes.f90:410-425
        g = 1.0 / 3.0
        ns, ass, cf = 4, False, 1.35
        bi = [[0, 0, 0, 0, 0], [0, g, 0, 0, 0], [0, -g, g, 0, 0], [0, 0, 1 - g, g, 0], [0, 0, 0.5, 0.5 - g, g]]
        be = [[0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [0, 0, 1, 0, 0], [0, 0, 0.5, 0.5, 0]]
        exp_calc = [False, True, True, True]
    elif n == "LZ453":
        # dirk_schemes.f90:498-513
        g = 1.2
        ns, ass, cf, imp1 = 4, False, 1.15, True
        bi = [[0, 0, 0, 0, 0], [-44.0 / 45.0, 1.2, 0, 0, 0], [-47.0 / 300.0, -0.71, 1.2, 0, 0],
              [3.375, -3.25, -59.0 / 120.0, 1.2, 0], [89.0 / 50.0, -486.0 / 55.0, 8.9, -562.0 / 275.0, 1.2]]
        be = [[0, 0, 0, 0, 0], [2.0 / 9.0, 0, 0, 0, 0], [71.0 / 420.0, 23.0 / 140.0, 0, 0, 0],
              [-281.0 / 336.0, 187.0 / 112.0, 0, 0, 0], [0.1, 0, 0.5, 0.4, 0]]
    elif n == "KC343":
        # dirk_schemes.f90:547-572 (Kennedy-Carpenter ARK3(2)4L[2]SA)
        g = 1767732205903.0 / 4055673282236.0
        ns, ass, cf, imp1 = 4, True, 0.5, True
        last = [1471266399579.0 / 7840856788654.0, -4482444167858.0 / 7529755066697.0,
                11266239266428.0 / 11593286722821.0, g]
        bi = [[0, 0, 0, 0], [g, g, 0, 0],
              [2746238789719.0 / 10658868560708.0, -640167445237.0 / 6845629431997.0, g, 0], last]
        be = [[0, 0, 0, 0], [1767732205903.0 / 2027836641118.0, 0, 0, 0],
              [5535828885825.0 / 10492691773637.0, 788022342437.0 / 10882634858940.0, 0, 0],
              [6485989280629.0 / 16251701735622.0, -4246266847089.0 / 9704473918619.0,
               10755448449292.0 / 10357097424841.0, 0]]
        bai = bae = last
    elif n == "KC564":
        # dirk_schemes.f90:591-624 (Kennedy-Carpenter ARK4(3)6L[2]SA)
        g = 0.25
        ns, ass, cf, imp1 = 6, True, 0.5, True
        last = [82889.0 / 524892.0, 0, 15625.0 / 83664.0, 69875.0 / 102672.0, -2260.0 / 8211.0, 0.25]
        bi = [[0, 0, 0, 0, 0, 0], [0.25, 0.25, 0, 0, 0, 0], [8611.0 / 62500.0, -1743.0 / 31250.0, 0.25, 0, 0, 0],
              [5012029.0 / 34652500.0, -654441.0 / 2922500.0, 174375.0 / 388108.0, 0.25, 0, 0],
              [15267082809.0 / 155376265600.0, -71443401.0 / 120774400.0, 730878875.0 / 902184768.0,
               2285395.0 / 8070912.0, 0.25, 0], last]
        be = [[0, 0, 0, 0, 0, 0], [0.5, 0, 0, 0, 0, 0], [13861.0 / 62500.0, 6889.0 / 62500.0, 0, 0, 0, 0],
              [-116923316275.0 / 2393684061468.0, -2731218467317.0 / 15368042101831.0,
               9408046702089.0 / 11113171139209.0, 0, 0, 0],
              [-451086348788.0 / 2902428689909.0, -2682348792572.0 / 7519795681897.0,
               12662868775082.0 / 11960479115383.0, 3355817975965.0 / 11060851509271.0, 0, 0],
              [647845179188.0 / 3216320057751.0, 73281519250.0 / 8382639484533.0,
               552539513391.0 / 3454668386233.0, 3354512671639.0 / 8306763924573.0, 4040.0 / 17871.0, 0]]
        bai = bae = last
    elif n == "DBM453":
        # dirk_schemes.f90:625-648; the assembly weights carry their own printed digits
        g = 0.32591194130117247
        ns, ass, cf, imp1 = 5, True, 0.5, True
        bi = [[0, 0, 0, 0, 0], [-0.22284985318525410, g, 0, 0, 0], [-0.46801347074080545, 0.86349284225716961, g, 0, 0],
              [-0.46509906651927421, 0.81063103116959553, 0.61036726756832357, g, 0],
              [0.87795339639076675, -0.72692641526151547, 0.75204137157372720, -0.22898029400415088, g]]
        be = [[0, 0, 0, 0, 0], [0.10306208811591838, 0, 0, 0, 0], [-0.94124866143519894, 1.6626399742527356, 0, 0, 0],
              [-1.3670975201437765, 1.3815852911016873, 1.2673234025619065, 0, 0],
              [-0.81287582068772448, 0.81223739060505738, 0.90644429603699305, 0.094194134045674111, 0]]
        bai = bae = [0.87795339639076672, -0.72692641526151549, 0.7520413715737272, -0.22898029400415090,
                     0.32591194130117247]
    elif n == "KC785":
        # dirk_schemes.f90:649-706 (Kennedy-Carpenter ARK5(4)8L[2]SA)
        g = 2.0 / 9.0
        ns, ass, cf, imp1 = 8, True, 0.5, True
        a3 = 2366667076620.0 / 8822750406821.0
        a4 = -257962897183.0 / 4451812247028.0
        a5 = -486229321650.0 / 11227943450093.0
        a6 = 621307788657.0 / 4714163060173.0
        a7 = 2036305566805.0 / 6583108094622.0
        last = [0, 0, 3517720773327.0 / 20256071687669.0, 4569610470461.0 / 17934693873752.0,
                2819471173109.0 / 11655438449929.0, 3296210113763.0 / 10722700128969.0,
                -1142099968913.0 / 5710983926999.0, g]
        bi = [[0] * 8, [g, g, 0, 0, 0, 0, 0, 0], [a3, a3, g, 0, 0, 0, 0, 0],
              [a4, a4, 128530224461.0 / 14379561246022.0, g, 0, 0, 0, 0],
              [a5, a5, -225633144460.0 / 6633558740617.0, 1741320951451.0 / 6824444397158.0, g, 0, 0, 0],
              [a6, a6, -125196015625.0 / 3866852212004.0, 940440206406.0 / 7593089888465.0,
               961109811699.0 / 6734810228204.0, g, 0, 0],
              [a7, a7, -3039402635899.0 / 4450598839912.0, -1829510709469.0 / 31102090912115.0,
               -286320471013.0 / 6931253422520.0, 8651533662697.0 / 9642993110008.0, g, 0], last]
        be = [[0] * 8, [4.0 / 9.0, 0, 0, 0, 0, 0, 0, 0],
              [1.0 / 9.0, 1183333538310.0 / 1827251437969.0, 0, 0, 0, 0, 0, 0],
              [895379019517.0 / 9750411845327.0, 477606656805.0 / 13473228687314.0,
               -112564739183.0 / 9373365219272.0, 0, 0, 0, 0, 0],
              [-4458043123994.0 / 13015289567637.0, -2500665203865.0 / 9342069639922.0,
               983347055801.0 / 8893519644487.0, 2185051477207.0 / 2551468980502.0, 0, 0, 0, 0],
              [-167316361917.0 / 17121522574472.0, 1605541814917.0 / 7619724128744.0,
               991021770328.0 / 13052792161721.0, 2342280609577.0 / 11279663441611.0,
               3012424348531.0 / 12792462456678.0, 0, 0, 0],
              [6680998715867.0 / 14310383562358.0, 5029118570809.0 / 3897454228471.0,
               2415062538259.0 / 6382199904604.0, -3924368632305.0 / 6964820224454.0,
               -4331110370267.0 / 15021686902756.0, -3944303808049.0 / 11994238218192.0, 0, 0],
              [2193717860234.0 / 3570523412979.0, 2193717860234.0 / 3570523412979.0,
               5952760925747.0 / 18750164281544.0, -4412967128996.0 / 6196664114337.0,
               4151782504231.0 / 36106512998704.0, 572599549169.0 / 6265429158920.0,
               -457874356192.0 / 11306498036315.0, 0]]
        bai = bae = last
    else:
        return None
    bi = np.array(bi, float)
    be = np.array(be, float)
    sizet = bi.shape[0]
    assert sizet == (ns if ass else ns + 1)
    return dict(nstages=ns, l_assembly=ass, gamma=g, bimp=bi, bexp=be,
                bass_imp=np.array(bai if bai is not None else np.zeros(sizet), float),
                bass_exp=np.array(bae if bae is not None else np.zeros(sizet), float),
                l_exp_calc=exp_calc if exp_calc is not None else [True] * ns,
                l_imp_calc_rhs=[imp1] + [True] * (ns - 1), courfac=cf)


DIRK_SCHEMES = ("ARS222", "ARS232", "ARS233", "SSP222", "LSDIRK222", "LZ232", "CK232", "ARS443",
                "SSP433", "DP1-242", "DP2-242", "LZ453", "KC343", "KC564", "KC785", "DBM453",
                "BPR353", "PC2", "ARS343", "MARS343", "SSP322", "SSP332")


class Dirk:
    """type_dirk (src/dirk_schemes.f90): Butcher weights scaled by dt, the
    stage right-hand side and the assembly stage."""

    def __init__(self, time_scheme: str, courfac_nml: float):
        t = dirk_tableau(time_scheme)
        if t is None:
            raise ValueError(f"time integrator {time_scheme} not found")
        self.time_scheme = time_scheme.upper()
        self.family = "DIRK"
        self.tab = t
        self.nstages = t["nstages"]
        self.nold, self.nimp, self.nexp = 1, t["nstages"], t["nstages"]
        self.l_assembly = t["l_assembly"]
        self.l_exp_calc = list(t["l_exp_calc"])
        self.l_imp_calc_rhs = list(t["l_imp_calc_rhs"])
        self.istage = 1
        self.courfac = t["courfac"] if abs(courfac_nml) >= 1.0e3 else courfac_nml
        self.dt = np.zeros(1)
        self.wimp_lin = np.zeros(1)

    def set_weights(self) -> bool:
        """set_weights (dirk_schemes.f90:275-712): everything scaled by dt(1).
        Unlike the multistep family it never requests a matrix rebuild."""
        dt = self.dt[0]
        t = self.tab
        self.wimp_lin[0] = dt * t["gamma"]
        self.butcher_imp = dt * t["bimp"]
        self.butcher_exp = dt * t["bexp"]
        self.butcher_ass_imp = dt * t["bass_imp"]
        self.butcher_ass_exp = dt * t["bass_exp"]
        return False

    def set_dt_array(self, dt_new: float, dt_min: float):
        """set_dt_array (dirk_schemes.f90:714-760)."""
        self.dt[0] = dt_new
        if dt_new < dt_min:
            raise FloatingPointError(f"time step too small, dt={dt_new!r}")

    def set_imex_rhs(self, ta: "TArray") -> np.ndarray:
        """set_imex_rhs (dirk_schemes.f90:762-795): stage istage."""
        s = self.istage
        rhs = ta.old[0].copy()
        for k in range(s):
            rhs = rhs + self.butcher_exp[s, k] * ta.expl[k]
        for k in range(s):
            rhs = rhs + self.butcher_imp[s, k] * ta.impl[k]
        return rhs

    def rotate_imex(self, ta: "TArray"):
        """rotate_imex (dirk_schemes.f90:833-838): nothing to rotate."""

    def bridge_with_cnab2(self):
        """bridge_with_cnab2 (dirk_schemes.f90:840-844): nothing to bridge."""

    def assemble_imex(self, ta: "TArray") -> np.ndarray:
        """assemble_imex (dirk_schemes.f90:852-882)."""
        rhs = ta.old[0].copy()
        for k in range(self.nstages):
            rhs = rhs + self.butcher_ass_exp[k] * ta.expl[k]
        for k in range(self.nstages):
            rhs = rhs + self.butcher_ass_imp[k] * ta.impl[k]
        return rhs


class TArray:
    """type_tarray (src/time_array.f90:11-71): old/impl/expl history slots."""

    def __init__(self, shape, nold, nimp, nexp):
        self.old = [np.zeros(shape, complex) for _ in range(nold)]
        self.impl = [np.zeros(shape, complex) for _ in range(nimp)]
        self.expl = [np.zeros(shape, complex) for _ in range(nexp)]


# ---------------------------------------------------------------------------
# Chebyshev scheme, transforms and derivatives
# ---------------------------------------------------------------------------
class Cheb:
    """Gauss-Lobatto grid and collocation matrices (src/chebyshev.f90:37-383)
    plus the FFT-based DCT and derivatives of src/dct_fftw.f90:46-397."""

    def __init__(self, n_r_max: int, n_cheb_max: int, r_icb: float, r_cmb: float):
        N = n_r_max
        self.N = N
        self.n_max = n_cheb_max
        self.rnorm = math.sqrt(2.0 / (N - 1))          # chebyshev.f90:62
        self.boundary_fac = 0.5                          # chebyshev.f90:64
        self.cheb_fac = math.sqrt(0.5 / (N - 1))         # dct_fftw.f90:128
        # cheb_grid (chebyshev.f90:222-279), no mapping
        k = np.arange(N)
        self.x = np.cos(np.pi * k.astype(float) / float(N - 1))
        bma = 0.5 * (r_cmb - r_icb)
        bpa = 0.5 * (r_icb + r_cmb)
        self.r = bma * self.x + bpa
        self.drx = np.full(N, 2.0 / (r_cmb - r_icb))     # chebyshev.f90:209-211
        self.ddrx = np.zeros(N)
        # get_der_mat (chebyshev.f90:281-383): T, T', T'' then transposed
        x, drx, ddrx = self.x, self.drx, self.ddrx
        rM = np.zeros((N, N))
        drM = np.zeros((N, N))
        d2rM = np.zeros((N, N))
        rM[0] = 1.0
        rM[1] = x
        drM[1] = drx
        d2rM[1] = ddrx
        for n in range(2, N):
            rM[n] = 2.0 * x * rM[n - 1] - rM[n - 2]
            drM[n] = 2.0 * drx * rM[n - 1] + 2.0 * x * drM[n - 1] - drM[n - 2]
            d2rM[n] = (2.0 * ddrx * rM[n - 1] + 4.0 * drx * drM[n - 1]
                       + 2.0 * x * d2rM[n - 1] - d2rM[n - 2])
        self.rMat, self.drMat, self.d2rMat = rM.T.copy(), drM.T.copy(), d2rM.T.copy()
        # der / der2 arrays of the dft_loop DCT (dct_fftw.f90:83-89)
        n2 = 2 * N - 2
        der = np.zeros(n2)
        der[N:] = -(n2 - np.arange(N, n2))
        der[:N] = np.arange(N)
        self.der2 = der * der          # computed before der(n_r_max)=0
        der[N - 1] = 0.0
        self.der = der

    # -- DCT-I ---------------------------------------------------------------
    def _ext(self, f):
        return np.concatenate([f, f[..., self.N - 2:0:-1]], axis=-1)

    def costf1(self, f):
        """costf_complex_2d (dct_fftw.f90:175-238), dft_loop variant."""
        return self.cheb_fac * np.fft.fft(self._ext(f), axis=-1)[..., :self.N]

    def costf1_real(self, f):
        """costf_real_1d (dct_fftw.f90:240-256): FFTW REDFT00 times cheb_fac."""
        return self.cheb_fac * sfft.dct(np.asarray(f, float), type=1, axis=-1)

    def _bwd(self, z):
        return np.fft.ifft(z, axis=-1) * z.shape[-1]

    # -- derivatives via FFT (complex 2d path, USE_DCT_FFT) -------------------
    def get_dr(self, f, l_dct_in=True):
        """get_dr_complex_2d (radial_derivatives.f90:313-412) -> get_dr_fft
        (dct_fftw.f90:258-316), then the drx mapping."""
        N = self.N
        n2 = 2 * N - 2
        f = np.atleast_2d(f)
        if l_dct_in:
            w = np.fft.fft(self._ext(f), axis=-1)
        else:
            w = self._ext(f) / self.cheb_fac
        w[:, N - 1] = 0.5 * w[:, N - 1]
        k = np.arange(1, N)
        k2 = (k * k).astype(float)
        sgn = np.where((k + 1) % 2 == 0, 1.0, -1.0)
        df = np.empty((f.shape[0], N), complex)
        df[:, 0] = (w[:, 1:N] * k2).sum(axis=-1) / (N - 1)
        df[:, N - 1] = (w[:, 1:N] * (sgn * k2)).sum(axis=-1) / (N - 1)
        w[:, N - 1] = 2.0 * w[:, N - 1]
        w = 1j * self.der * w
        wb = self._bwd(w)
        xi = self.x[1:N - 1]
        df[:, 1:N - 1] = -wb[:, 1:N - 1] / np.sqrt(1.0 - xi ** 2) / n2
        return self.drx * df

    def get_ddr(self, f, l_dct=True):
        """get_ddr_complex_2d (radial_derivatives.f90:477-566) -> get_ddr_fft
        (dct_fftw.f90:318-397), then the drx/ddrx mapping."""
        N = self.N
        n2 = 2 * N - 2
        f = np.atleast_2d(f)
        if l_dct:
            t = np.fft.fft(self._ext(f), axis=-1)
        else:
            t = self._ext(f) / self.cheb_fac
        t[:, N - 1] = 0.5 * t[:, N - 1]
        k = np.arange(1, N).astype(float)
        df = np.empty((f.shape[0], N), complex)
        ddf = np.empty((f.shape[0], N), complex)
        sgn1 = np.where((np.arange(1, N) + 1) % 2 == 0, 1.0, -1.0)
        df[:, 0] = (t[:, 1:N] * (k * k)).sum(axis=-1) / (N - 1)
        k2 = np.arange(2, N).astype(float)
        ddf[:, 0] = (1.0 / 3.0) * (t[:, 2:N] * (k2 * k2 * (k2 * k2 - 1))).sum(axis=-1) / (N - 1)
        df[:, N - 1] = (t[:, 1:N] * (sgn1 * k * k)).sum(axis=-1) / (N - 1)
        sgn2 = np.where(np.arange(2, N) % 2 == 0, 1.0, -1.0)
        ddf[:, N - 1] = (1.0 / 3.0) * (t[:, 2:N] * (sgn2 * k2 * k2 * (k2 * k2 - 1))).sum(axis=-1) / (N - 1)
        t[:, N - 1] = 2.0 * t[:, N - 1]
        w1 = self._bwd(1j * self.der * t)
        w2 = self._bwd(-self.der2 * t)
        xi = self.x[1:N - 1]
        om = 1.0 - xi ** 2
        df[:, 1:N - 1] = -w1[:, 1:N - 1] / np.sqrt(om) / n2
        ddf[:, 1:N - 1] = (-w1[:, 1:N - 1] * xi / om ** 1.5 / n2
                           + w2[:, 1:N - 1] / om / n2)
        ddf = self.ddrx * df + self.drx * self.drx * ddf
        df = self.drx * df
        return df, ddf

    # -- real 1d derivatives via the Chebyshev recursion ---------------------
    # round-off threshold of the real recursions (radial_derivatives.f90:51-66):
    # rerror_fac * epsilon with l_rerror_fix, else 0
    thr = 0.0

    def _dcheb(self, c):
        """get_dcheb_real_1d (radial_derivatives.f90:143-185): a coefficient
        below the threshold zeroes that derivative coefficient."""
        N = self.N
        t = np.max(np.abs(c)) * self.thr
        df = np.zeros(N)
        df[N - 2] = (N - 1) * c[N - 1] if abs(c[N - 1]) >= t else 0.0
        for n in range(N - 3, -1, -1):
            df[n] = df[n + 2] + 2.0 * (n + 1) * c[n + 1] if abs(c[n + 1]) >= t else 0.0
        return df

    def _ddcheb(self, c):
        """get_ddcheb_real_1d (radial_derivatives.f90:259-311): terms below the
        threshold are skipped."""
        N = self.N
        t = np.max(np.abs(c)) * self.thr
        df = np.zeros(N)
        ddf = np.zeros(N)
        df[N - 2] = (N - 1) * c[N - 1] if abs(c[N - 1]) >= t else 0.0
        for n in range(N - 3, -1, -1):
            fac = 2.0 * (n + 1)
            df[n] = df[n + 2] + fac * c[n + 1] if abs(c[n + 1]) >= t else df[n + 2]
            ddf[n] = ddf[n + 2] + fac * df[n + 1] if abs(df[n + 1]) >= t else ddf[n + 2]
        return df, ddf

    def get_dr_real(self, f, l_dct=True):
        """get_dr_real_1d (radial_derivatives.f90:414-475)."""
        w = np.array(f, float)
        if l_dct:
            w = self.costf1_real(w)
        df = self.costf1_real(self._dcheb(w))
        return self.drx * df

    def get_ddr_real(self, f):
        """get_ddr_real_1d (radial_derivatives.f90:568-631)."""
        w = self.costf1_real(np.array(f, float))
        df, ddf = self._ddcheb(w)
        df = self.costf1_real(df)
        ddf = self.costf1_real(ddf)
        ddf = self.ddrx * df + self.drx * self.drx * ddf
        df = self.drx * df
        return df, ddf

    def rInt_R(self, f):
        """rInt_R (src/integration.f90:18-55), Chebyshev branch."""
        N = self.N
        f2 = self.costf1_real(np.asarray(f, float) / self.drx)
        f2[0] *= 0.5
        f2[N - 1] *= 0.5
        rint = f2[0]
        for nc in range(3, N + 1, 2):
            rint = rint - 1.0 / float(nc * (nc - 2)) * f2[nc - 1]
        return 2.0 * math.sqrt(2.0 / (N - 1)) * rint


def simps(f, r):
    """simps (src/integration.f90:104-152)."""
    n = len(f)
    if n % 2 == 1:
        rint = 0.0
        for i in range(1, n - 1, 2):
            h2 = r[i + 1] - r[i]
            h1 = r[i] - r[i - 1]
            rint += (h1 + h2) / 6.0 * (f[i - 1] * (2 * h1 - h2) / h1 + f[i] * (h1 + h2) ** 2 / (h1 * h2)
                                       + f[i + 1] * (2 * h2 - h1) / h2)
        return -rint
    rint = 0.5 * (r[1] - r[0]) * (f[1] + f[0])
    for i in range(2, n, 2):
        h2 = r[i + 1] - r[i]
        h1 = r[i] - r[i - 1]
        rint += (h1 + h2) / 6.0 * (f[i - 1] * (2 * h1 - h2) / h1 + f[i] * (h1 + h2) ** 2 / (h1 * h2)
                                   + f[i + 1] * (2 * h2 - h1) / h2)
    rint += 0.5 * (r[n - 1] - r[n - 2]) * (f[n - 1] + f[n - 2])
    for i in range(1, n - 1, 2):
        h2 = r[i + 1] - r[i]
        h1 = r[i] - r[i - 1]
        rint += (h1 + h2) / 6.0 * (f[i - 1] * (2 * h1 - h2) / h1 + f[i] * (h1 + h2) ** 2 / (h1 * h2)
                                   + f[i + 1] * (2 * h2 - h1) / h2)
    return -0.5 * rint


def l_correct_step(n, n_max, n_step, n_intervals):
    """l_correct_step (src/useful.f90:181-219)."""
    if n_intervals != 0:
        n_steps = n_max // n_intervals
        n_offset = n_max - n_steps * n_intervals
        return n > n_offset and (n - n_offset) % n_steps == 0
    if n_step != 0:
        return n == n_max or n % n_step == 0
    return False


def round_off(x):
    """round_off (src/useful.f90:221-232)."""
    return 0.0 if abs(x) < TINY_NUMBER else x


def _gasp_center(c, L):
    """gausslike_compact_center (src/useful.f90:295-307)."""
    return math.pi * L ** 3 * (1 - math.exp(-2 * c / L)) - 2 * math.pi * c * L * (c + L) * math.exp(-2 * c / L)


def _gasp_middle(r, c, L):
    """gausslike_compact_middle (src/useful.f90:309-325)."""
    return (math.pi / 3.0 * L * r * (r + 3 * L) * math.exp(-r / L)
            + (2 * math.pi * L * L * (c + L) ** 2) / r * math.exp(-2 * c / L) * (1 - (1 - r / (c + L)) * math.exp(r / L))
            + math.pi * L ** 3 * (math.exp(-r / L) - math.exp((r - 2 * c) / L)))


def _gasp_edge(r, c, L):
    """gausslike_compact_edge (src/useful.f90:327-341)."""
    return 2 * math.pi * L / r * math.exp(-r / L) * (0.5 * (r * (r + L) * (2 * c - r))
                                                     + 1.0 / 3.0 * ((r - c) ** 3 - c ** 3)
                                                     - L * (c + L) * (r - c + L)
                                                     + L * (c + L) ** 2 * math.exp((r - 2 * c) / L))


def seeded_temperature(n_m_max: int, r: np.ndarray, r_icb: float, amp: float, seed: int):
    """Seeded initial temperature perturbation of the synthetic workloads.

    T(m, r) = amp * g_m * exp(i theta_m) * sin(pi (r - r_icb)) for m >= 1 with
    g_m ~ N(0, 1) and theta_m ~ U[0, 2 pi) drawn from numpy's default_rng(seed);
    T(m=0) = 0.  The radial envelope is pizza's ``t1`` profile
    (src/init_fields.f90:275).
    """
    rng = np.random.default_rng(seed)
    g = rng.standard_normal(n_m_max - 1)
    th = rng.uniform(0.0, 2.0 * np.pi, n_m_max - 1)
    t1 = np.sin(np.pi * (r - r_icb))
    T = np.zeros((n_m_max, len(r)), complex)
    T[1:, :] = (amp * g * np.exp(1j * th))[:, None] * t1[None, :]
    return T


# ---------------------------------------------------------------------------
# The time stepper
# ---------------------------------------------------------------------------
class Pizza:
    """State and stage body of pizza's collocation time step for one instance."""

    def __init__(self, p: Params, integ_bordered: bool = False):
        self.p = p
        d = p.derived()
        self.d = d
        N = p.n_r_max
        self.N = N
        self.n_max = p.n_cheb_max if p.n_cheb_max is not None else N
        self.M = p.m_max // p.minc + 1                 # truncation.f90:28
        self.P = 3 * p.m_max // p.minc                  # truncation.f90:30-31
        self.mvec = np.arange(self.M) * p.minc
        self.l_direct = d["l_direct_solve"]
        self.cheb = Cheb(N, N, d["r_icb"], d["r_cmb"])
        self._radial()
        if p.time_scheme.upper() in DIRK_SCHEMES:
            self.ts = Dirk(p.time_scheme, p.courfac)
        else:
            self.ts = Multistep(p.time_scheme, p.courfac, p.alpha)
        shp = (self.M, N)
        ts = self.ts
        # dt_fieldsLast.f90:35-215: histories, explicit containers (1 stage)
        self.dTdt = TArray(shp, ts.nold, ts.nimp, ts.nexp)
        self.dpsidt = TArray(shp, ts.nold, ts.nimp, ts.nexp)
        self.us = np.zeros(shp, complex)
        self.up = np.zeros(shp, complex)
        self.om = np.zeros(shp, complex)
        self.psi = np.zeros(shp, complex)
        self.temp = np.zeros(shp, complex)
        self.dtemp = np.zeros(shp, complex)
        self.dom = np.zeros(shp, complex)
        self.time = 0.0
        self.dtMin = p.dtMax / 1.0e6                   # pre_calculations.f90:33
        self.dtr = np.full(N, 1.0e10)
        self.dth = np.full(N, 1.0e10)
        self.hdif = np.ones(self.M)                     # horizontal.f90:69-140
        self.topt = np.zeros(self.M, complex)
        self.bott = np.zeros(self.M, complex)
        self._mats_built = False
        self._psi_dmat_built = False
        self.n_time_step = 0
        self.l_new_dt = True
        self.lMatNext = True
        self.l_bridge_step = True
        self.l_AB1 = False
        self.rows = {"e_kin": [], "e_kin_3D": [], "heat": [], "composition": []}
        if p.l_rerror_fix:
            self.cheb.thr = p.rerror_fac * np.finfo(float).eps
        self.l_integ = not d["l_cheb_coll"]
        self.temp_hat = np.zeros(shp, complex)
        self.psi_hat = np.zeros(shp, complex)
        # composition (update_xi_coll.f90, update_xi_integ.f90): the same
        # containers as temperature; they stay zero when raxi = 0
        self.l_chem = d["l_chem"]
        self.dxidt = TArray(shp, ts.nold, ts.nimp, ts.nexp)
        self.xi = np.zeros(shp, complex)
        self.dxi = np.zeros(shp, complex)
        self.xi_hat = np.zeros(shp, complex)
        self.topxi = np.zeros(self.M, complex)
        self.botxi = np.zeros(self.M, complex)
        self._dVsXi = np.zeros(shp, complex)
        if self.l_integ:
            from .pizza_integ import IntegScheme
            self.integ = IntegScheme(self, bordered=integ_bordered)

    # -- radial functions (src/radial.f90:115-282) ---------------------------
    def _radial(self):
        d, p, c = self.d, self.p, self.cheb
        N = self.N
        r = c.r
        r_cmb, r_icb = d["r_cmb"], d["r_icb"]
        self.r = r
        self.or1 = 1.0 / r
        self.or2 = self.or1 * self.or1
        self.rgrav = p.g0 + p.g1 * r / r_cmb + p.g2 * r_cmb ** 2 * self.or2
        m_R = p.m_max
        self.delxh2 = np.empty(N)
        self.delxr2 = np.empty(N)
        self.delxh2[0] = (2 * np.pi / 3.0 / m_R * r_cmb) ** 2
        self.delxh2[N - 1] = (2 * np.pi / 3.0 / m_R * r_icb) ** 2
        self.delxr2[0] = (r[0] - r[1]) ** 2
        self.delxr2[N - 1] = (r[N - 2] - r[N - 1]) ** 2
        for i in range(1, N - 1):
            self.delxh2[i] = (2 * np.pi / 3.0 / m_R * r[i]) ** 2
            dm = min(r[i - 1] - r[i], r[i] - r[i + 1])
            self.delxr2[i] = dm * dm
        # conducting state, 2D, fixed temperatures (radial.f90:377-379)
        if p.ktopt == 1 and p.kbott == 1:
            self.tcond = p.tcond_fac * (np.log(r / r_cmb) / math.log(p.radratio))
            self.dtcond = p.tcond_fac * (self.or1 / math.log(p.radratio))
        else:
            raise NotImplementedError("only fixed-temperature boundaries are restated")
        # conducting composition: the same 2D profile with xicond_fac (radial.f90:194-195)
        if p.ktopxi == 1 and p.kbotxi == 1:
            self.xicond = p.xicond_fac * (np.log(r / r_cmb) / math.log(p.radratio))
            self.dxicond = p.xicond_fac * (self.or1 / math.log(p.radratio))
        elif d["l_chem"]:
            raise NotImplementedError("only fixed-composition boundaries are restated")
        else:
            self.xicond = np.zeros(N)
            self.dxicond = np.zeros(N)
        ek_pump_fac = 1.0 if (p.l_ek_pump and not d["l_non_rot"]) else 0.0
        z = np.zeros(N)
        if d["l_non_rot"]:
            self.beta = z.copy(); self.dbeta = z.copy(); self.ekpump = z.copy()
            self.ekp_up = z.copy(); self.ekp_us = z.copy(); self.ekp_dusdp = z.copy()
            self.oheight = np.ones(N); self.height = np.ones(N)
        else:
            # SPHERE container, beta_shift = 0 (radial.f90:209-246)
            h = np.zeros(N); oh = np.zeros(N); be = np.zeros(N); dbe = np.zeros(N); ekp = np.zeros(N)
            rr = r[1:]
            h[1:] = 2.0 * np.sqrt(r_cmb ** 2 - rr ** 2)
            oh[1:] = 0.5 / np.sqrt(r_cmb ** 2 - rr ** 2)
            be[1:] = -rr / (r_cmb ** 2 - rr ** 2)
            dbe[1:] = -(r_cmb ** 2 + rr ** 2) / (r_cmb ** 2 - rr ** 2) ** 2
            ekp[1:] = 0.5 * ek_pump_fac * math.sqrt(d["ek"] * r_cmb) / (r_cmb ** 2 - rr ** 2) ** 0.75
            self.height, self.oheight, self.beta, self.dbeta, self.ekpump = h, oh, be, dbe, ekp
            self.ekp_up = -0.5 * be
            self.ekp_us = -5.0 * r_cmb * be * oh
            self.ekp_dusdp = be.copy()
        # constants (pre_calculations.f90:57-68)
        self.surf = np.pi * (r_cmb ** 2 - r_icb ** 2)
        self.vol_otc = 4.0 / 3.0 * np.pi * (r_cmb ** 2 - r_icb ** 2) ** 1.5

    # -- start fields (src/init_fields.f90:54-258) ---------------------------
    def start(self, temp0=None, xi0=None):
        """get_start_fields without a checkpoint: zero state, dt(:)=dtMax,
        weights, perturbation (initProp/initU or an injected ``temp0`` and,
        with composition, ``xi0``), then the derived fields and the first
        implicit state."""
        p, ts = self.p, self.ts
        self.time = 0.0
        ts.dt[:] = p.dtMax
        ts.set_weights()
        if temp0 is not None:
            self.temp = self.temp + np.asarray(temp0, complex)
        elif p.init_t != 0:
            self._init_prop(p.init_t, p.amp_t)
        if self.l_chem and xi0 is not None:
            self.xi = self.xi + np.asarray(xi0, complex)
        elif self.l_chem and p.init_xi != 0:
            self._init_prop(p.init_xi, p.amp_xi, "xi")        # init_fields.f90:123
        if p.init_u != 0:
            self._init_u()
        c = self.cheb
        self.dtemp = c.get_dr(self.temp)
        if self.l_chem:
            self.dxi = c.get_dr(self.xi)
        work = c.get_dr(self.up)
        m = self.mvec[:, None]
        self.om = work + self.or1 * self.up - self.or1 * 1j * m * self.us
        if self.l_integ:
            self.integ.start()
            return
        self._temp_rhs_imp(1, True, l_in_cheb=False)
        if self.l_chem:
            self._xi_rhs_imp(1, True, l_in_cheb=False)
        self._psi_rhs_imp(1, True, l_in_cheb=False)

    def _map_field(self, f, n_old, phys, lbc):
        """map_field / map_field_r (checkpoints.f90:709-860), Chebyshev to
        Chebyshev: (n_m_old, n_old) -> (M, N).  New azimuthal modes are zero;
        in r the Chebyshev coefficients (costf1 of the old grid first when
        the field is stored in physical space) are zero-padded or cut and
        brought back with this grid's costf1, times rnorm_old / rnorm."""
        f = np.array(f, complex)
        out = np.zeros((self.M, self.N), complex)
        mm = min(self.M, f.shape[0])
        if n_old == self.N:
            out[:mm] = f[:mm]
            return out
        g = f[:mm].copy()
        if lbc and phys:
            g[:, 0] = 2.0 * g[:, 1] - g[:, 2]
        if phys:
            g = Cheb(n_old, n_old, self.d["r_icb"], self.d["r_cmb"]).costf1(g)
        pad = np.zeros((mm, max(self.N, n_old)), complex)
        pad[:, :n_old] = g
        g = pad[:, :self.N]
        if phys:
            g = self.cheb.costf1(g)
        out[:mm] = math.sqrt(2.0 / (n_old - 1)) / self.cheb.rnorm * g
        return out

    def start_from_checkpoint(self, ck):
        """get_start_fields with l_start_file (init_fields.f90:54-258) for a
        version-7 checkpoint (read_checkpoint, checkpoints.f90:185-860): the
        fields and the multistep history slots 2..n mapped onto this grid
        (map_field), dt filled with the oldest value where this scheme keeps
        more (:388-396), time; then om and the first old/implicit slots as
        for a fresh start.  AB1 on the first step when the Ekman number or
        the radial method changed, and the CNAB2 bridge when this scheme
        needs more old or implicit slots than the file holds (:398-425).
        ``ck`` is a dict with header (time, family, nexp, nimp, nold, dt, ek,
        n_r_max, l_cheb_coll), us, up, temp, hist_P, hist_T (expl 2..nexp,
        impl 2..nimp, old 2..nold of the file's scheme) and, when the file
        holds composition, xi and hist_Xi."""
        ts, h = self.ts, ck["header"]
        self.time = h["time"]
        nd = len(h["dt"])
        ts.dt[:min(nd, len(ts.dt))] = h["dt"][:len(ts.dt)]
        if nd < len(ts.dt):
            ts.dt[nd:] = h["dt"][-1]
        ts.set_weights()
        n_old = int(h.get("n_r_max", self.N))
        coll_old = bool(h.get("l_cheb_coll", True))
        self.us = self._map_field(ck["us"], n_old, True, False)
        self.up = self._map_field(ck["up"], n_old, True, False)
        self.temp = self._map_field(ck["temp"], n_old, True, False)
        has_xi = self.l_chem and ck.get("xi") is not None
        if has_xi:
            self.xi = self._map_field(ck["xi"], n_old, True, False)
        if h["family"] == "MULTISTEP":
            order = ([("expl", k, True) for k in range(2, h["nexp"] + 1)]
                     + [("impl", k, True) for k in range(2, h["nimp"] + 1)]
                     + [("old", k, False) for k in range(2, h["nold"] + 1)])
            for (kind, k, lbc), aP, aT in zip(order, ck["hist_P"], ck["hist_T"]):
                if ts.family == "MULTISTEP" and k <= {"expl": ts.nexp, "impl": ts.nimp, "old": ts.nold}[kind]:
                    getattr(self.dpsidt, kind)[k - 1] = self._map_field(aP, n_old, coll_old, lbc)
                    getattr(self.dTdt, kind)[k - 1] = self._map_field(aT, n_old, coll_old, lbc)
            if has_xi:
                for (kind, k, lbc), aX in zip(order, ck.get("hist_Xi", [])):
                    if ts.family == "MULTISTEP" and k <= {"expl": ts.nexp, "impl": ts.nimp, "old": ts.nold}[kind]:
                        getattr(self.dxidt, kind)[k - 1] = self._map_field(aX, n_old, coll_old, lbc)
        if self.l_integ:
            self.psi = self.integ.psi_from_us()
        c = self.cheb
        self.dtemp = c.get_dr(self.temp)
        if self.l_chem:
            self.dxi = c.get_dr(self.xi)
        work = c.get_dr(self.up)
        m = self.mvec[:, None]
        self.om = work + self.or1 * self.up - self.or1 * 1j * m * self.us
        if self.l_integ:
            self.integ.start()
        else:
            self._temp_rhs_imp(1, True, l_in_cheb=False)
            if self.l_chem:
                self._xi_rhs_imp(1, True, l_in_cheb=False)
            self._psi_rhs_imp(1, True, l_in_cheb=False)
        self.l_AB1 = h.get("ek", self.d["ek"]) != self.d["ek"]
        if ts.family == "MULTISTEP":
            if h["family"] == "DIRK":
                self.l_bridge_step = True
            else:
                self.l_bridge_step = ts.nold > h["nold"] or ts.nimp > h["nimp"]
            if coll_old != self.d["l_cheb_coll"]:
                self.l_AB1 = True
                self.l_bridge_step = True
        else:
            self.l_bridge_step = False

    def _init_prop(self, init_t, amp, field="temp"):
        """initProp (init_fields.f90:260-376), modes init_t>0 and -1, on the
        temperature or (field="xi") the composition."""
        N, M = self.N, self.M
        tgt = getattr(self, field)
        r = self.r
        r_cmb, r_icb = self.d["r_cmb"], self.d["r_icb"]
        t1 = np.sin(np.pi * (r - r_icb))
        if init_t > 0:
            idx = init_t // self.p.minc
            tgt[idx, :] += t1 * amp
        elif init_t == -1:
            sigma_r = 0.1 / math.sqrt(2.0)
            rc = 0.5 * (r_cmb + r_icb)
            ir = int(np.argmin(np.abs(r - rc)))
            rc = r[ir]
            c1 = 0.5 * (r[0] - rc)
            c2 = 0.5 * (rc - r[N - 1])
            L = 0.5 * sigma_r
            gasp = np.zeros(N)
            for i in range(N):
                if i == ir:
                    gasp[i] = 1.0
                elif r[i] < rc - c2:
                    gasp[i] = _gasp_edge(rc - r[i], c2, L)
                elif rc - c2 <= r[i] < rc:
                    gasp[i] = _gasp_middle(rc - r[i], c2, L)
                elif rc < r[i] <= rc + c1:
                    gasp[i] = _gasp_middle(r[i] - rc, c1, L)
                elif r[i] > rc + c1:
                    gasp[i] = _gasp_edge(r[i] - rc, c1, L)
            for i in range(N):
                if i < ir:
                    gasp[i] = gasp[i] / _gasp_center(c1, L)
                elif i > ir:
                    gasp[i] = gasp[i] / _gasp_center(c2, L)
            phi0 = np.pi / self.p.minc
            P = self.P
            phi = np.arange(P) * 2 * np.pi / self.p.minc / P
            for i in range(N):
                c_r = amp * gasp[i]
                func = c_r * np.exp(-(phi - phi0) ** 2 / 0.2 ** 2)
                tgt[:, i] += self._fft(func)
        else:
            raise NotImplementedError("random init_t uses Fortran random_number; not restated")

    def _init_u(self):
        """initU (init_fields.f90:452-509)."""
        p = self.p
        r_icb = self.d["r_icb"]
        u1 = np.sin(np.pi * (self.r - r_icb))
        if p.init_u > 0:
            idx = p.init_u // p.minc
            self.us[idx, :] += u1 * p.amp_u
            m = self.mvec[:, None]
            self.om = -1j * m * self.or1 * self.us
        else:
            self.up[0, :] += p.amp_u * np.sin(np.pi * (self.r - r_icb))

    # -- phi transforms (src/fft_fftw.f90:44-90) -----------------------------
    def _fft(self, grid):
        tmp = np.fft.rfft(grid, axis=-1)
        return tmp[..., :self.M] / float(self.P)

    def _ifft(self, spec):
        tmp = np.zeros(spec.shape[:-1] + (self.P // 2 + 1,), complex)
        tmp[..., :self.M] = spec
        return np.fft.irfft(tmp, n=self.P, axis=-1) * self.P

    # -- radial loop (src/radial_loop.f90:231-394) ---------------------------
    def radial_loop(self):
        d = self.d
        m = self.mvec
        us_R, up_R, om_R, T_R = self.us.T, self.up.T, self.om.T, self.temp.T  # (N, M)
        r = self.r[:, None]
        or1 = self.or1[:, None]
        # Reynolds stress (radial_loop.f90:267-278)
        us_fluct = us_R.copy()
        us_fluct[:, 0] = 0.5 * d["ek"] * d["CorFac"] * self.ekpump * up_R[:, 0]
        prod = 2.0 * (us_fluct.real * om_R.real + us_fluct.imag * om_R.imag)
        prod[:, 0] = us_fluct[:, 0].real * om_R[:, 0].real
        usom = np.zeros(self.N)
        for n_m in range(self.M):     # sequential sum over m as in the reference
            usom = usom + prod[:, n_m]
        us_g = self._ifft(us_R)
        up_g = self._ifft(up_R)
        om_g = self._ifft(om_R)
        T_g = self._ifft(T_R)
        if self.ts.istage == 1:
            cf = self.ts.courfac
            vr2 = cf ** 2 * np.max(us_g ** 2, axis=1)
            vh2 = cf ** 2 * np.max(up_g ** 2, axis=1)
            with np.errstate(divide="ignore"):
                self.dtr = np.where(vr2 != 0.0, np.minimum(1.0e10, np.sqrt(self.delxr2 / np.where(vr2 != 0, vr2, 1.0))), 1.0e10)
                self.dth = np.where(vh2 != 0.0, np.minimum(1.0e10, np.sqrt(self.delxh2 / np.where(vh2 != 0, vh2, 1.0))), 1.0e10)
        usT = r * us_g * T_g
        upT = up_g * T_g
        usOm = r * us_g * om_g
        upOm = up_g * om_g
        dpsidt = self._fft(upOm)
        dVsOm = self._fft(usOm)
        dtempdt = self._fft(upT)
        dVsT = self._fft(usT)
        dtempdt = -or1 * 1j * m * dtempdt - (1.0 - d["tadvz_fac"]) * self.beta[:, None] * or1 * dVsT
        if self.l_chem:
            # composition: r us xi and up xi, no beta term (radial_loop.f90:320-323, :356-374);
            # dxi/dt goes to its explicit slot, r us xi to finish_explicit
            X_g = self._ifft(self.xi.T)
            dxidt = self._fft(up_g * X_g)
            self._dVsXi = self._fft(r * us_g * X_g).T.copy()
            self.dxidt.expl[self.ts.istage - 1] = (-or1 * 1j * m * dxidt).T.copy()
        dpsidt[:, 0] = -usom
        dpsidt[:, 1:] = -or1 * 1j * m[1:] * dpsidt[:, 1:]
        return dtempdt.T.copy(), dVsT.T.copy(), dpsidt.T.copy(), dVsOm.T.copy()

    # -- explicit assembly (src/mloop.f90:169-229) ---------------------------
    def finish_explicit(self, dVsT, dVsOm):
        if self.l_integ:
            return self.integ.finish_explicit(dVsT, dVsOm)
        d = self.d
        c = self.cheb
        ist = self.ts.istage - 1
        m = self.mvec[:, None]
        # finish_exp_temp_coll (update_temp_coll.f90:152-176)
        work = c.get_dr(dVsT)
        e = self.dTdt.expl[ist]
        e = e - self.or1 * work - self.us * (self.dtcond - d["tadvz_fac"] * self.beta * self.tcond)
        self.dTdt.expl[ist] = e
        if self.l_chem:
            # finish_exp_xi_coll (update_xi_coll.f90:142-166)
            work = c.get_dr(self._dVsXi)
            self.dxidt.expl[ist] = self.dxidt.expl[ist] - self.or1 * work - self.us * self.dxicond
        # finish_exp_psi_coll_{dmat,smat}
        work = c.get_dr(dVsOm)
        e = self.dpsidt.expl[ist].copy()
        nz = slice(1, None)
        e[nz] = e[nz] - self.or1 * work[nz]
        bal = getattr(self, "_bal", None)
        if bal is not None:
            # vort_balance's adv and cor (update_psi_coll_dmat.f90:500-505) and
            # pump (:540-546); zero where the reference leaves them unset
            bal["adv"] = np.zeros_like(e)
            bal["adv"][nz] = e[nz]
            bal["cor"] = np.zeros_like(e)
            if not d["l_non_rot"]:
                bal["cor"][nz] = d["CorFac"] * self.beta * self.us[nz]
            bal["pump"] = np.zeros_like(e)
            if self.p.l_ek_pump:
                bal["pump"][nz] = -d["CorFac"] * self.ekpump * (
                    self.om[nz] + self.ekp_up * self.up[nz]
                    + (self.ekp_dusdp * 1j * m[nz] + self.ekp_us) * self.us[nz])
        if self.l_direct:
            # update_psi_coll_smat.f90:323-378
            if not d["l_coriolis_imp"]:
                e[nz] = e[nz] + d["CorFac"] * self.beta * self.us[nz]
        else:
            # update_psi_coll_dmat.f90:468-552
            if not d["l_non_rot"]:
                e[nz] = e[nz] + d["CorFac"] * self.beta * self.us[nz]
        if not d["l_buo_imp"]:
            e[nz] = e[nz] - d["BuoFac"] * self.rgrav * self.or1 * 1j * m[nz] * self.temp[nz]
            if self.l_chem:
                e[nz] = e[nz] - d["ChemFac"] * self.rgrav * self.or1 * 1j * m[nz] * self.xi[nz]
        if (not self.l_direct) and self.p.l_ek_pump:
            e[nz] = e[nz] - d["CorFac"] * self.ekpump * (
                self.om[nz] + self.ekp_up * self.up[nz]
                + (self.ekp_dusdp * 1j * m[nz] + self.ekp_us) * self.us[nz])
        self.dpsidt.expl[ist] = e

    # -- CFL (src/courant.f90:78-167) ----------------------------------------
    def dt_courant(self):
        p = self.p
        dt = self.ts.dt[0]
        dt_r = min(1000.0 * p.dtMax, float(np.min(self.dtr)))
        dt_h = min(1000.0 * p.dtMax, float(np.min(self.dth)))
        dt_rh = min(dt_r, dt_h)
        dt_2 = min(0.5 * (1.0 / p.dt_fac + 1.0) * dt_rh, p.dtMax)
        if dt > p.dtMax:
            return True, p.dtMax
        if dt > dt_rh:
            return True, dt_2
        if p.dt_fac * dt < dt_rh and dt < p.dtMax:
            return True, dt_2
        return False, dt

    # -- matrices ------------------------------------------------------------
    def _lu(self, A, name):
        lu, piv = sla.lu_factor(A, check_finite=True)
        if np.any(np.diag(lu) == 0.0):
            raise np.linalg.LinAlgError(f"Singular matrix {name}!")
        return lu, piv

    @staticmethod
    def _solve_real(lu_piv, rhs):
        """solve_full_mat_real_rhs_complex (algebra_lapack.f90:46-79): two dgetrs."""
        re = sla.lu_solve(lu_piv, rhs.real.copy())
        im = sla.lu_solve(lu_piv, rhs.imag.copy())
        return re + 1j * im

    def _bfac_cols(self, A, cols):
        for cidx in cols:
            A[:, cidx] = self.cheb.boundary_fac * A[:, cidx]

    def _sc(self, kind):
        """(field, radial derivative, history, diffusivity, top and bottom
        values, top and bottom kinds) of an advected scalar: "temp" or "xi"."""
        d, p = self.d, self.p
        if kind == "temp":
            return "temp", "dtemp", self.dTdt, d["TdiffFac"], self.topt, self.bott, p.ktopt, p.kbott
        return "xi", "dxi", self.dxidt, d["XidiffFac"], self.topxi, self.botxi, p.ktopxi, p.kbotxi

    def _temp_mat(self, m, kind="temp"):
        """get_tempMat (update_temp_coll.f90:310-393) or get_xiMat
        (update_xi_coll.f90:321-393, the same with XidiffFac) with
        WITH_PRECOND_S."""
        c, p = self.cheb, self.p
        N, n_max = self.N, self.n_max
        _, _, _, diff, _, _, ktop, kbot = self._sc(kind)
        A = np.zeros((N, N))
        A[0, :n_max] = c.rnorm * (c.rMat[0, :n_max] if ktop == 1 else c.drMat[0, :n_max])
        A[N - 1, :n_max] = c.rnorm * (c.rMat[N - 1, :n_max] if kbot == 1 else c.drMat[N - 1, :n_max])
        w = self.ts.wimp_lin[0] * diff * self.hdif[m // p.minc]
        i = slice(1, N - 1)
        dm2 = float(m) * float(m)
        A[i, :] = c.rnorm * (c.rMat[i] - w * (c.d2rMat[i] + self.or1[i, None] * c.drMat[i]
                                               - dm2 * self.or2[i, None] * c.rMat[i]))
        self._bfac_cols(A, (0, N - 1))
        fac = 1.0 / np.max(np.abs(A), axis=1)
        A = A * fac[:, None]
        return self._lu(A, "tMat"), fac

    def _uphi_mat(self):
        """get_uphiMat (update_psi_coll_dmat.f90:985-1054 = smat:919-987)."""
        c, d, p = self.cheb, self.d, self.p
        N, n_max = self.N, self.n_max
        A = np.zeros((N, N))
        if p.ktopv == 1:
            A[0, :n_max] = c.rnorm * (c.drMat[0, :n_max] - self.or1[0] * c.rMat[0, :n_max])
        else:
            A[0, :n_max] = c.rnorm * c.rMat[0, :n_max]
        if p.kbotv == 1:
            A[N - 1, :n_max] = c.rnorm * (c.drMat[N - 1, :n_max] - self.or1[N - 1] * c.rMat[N - 1, :n_max])
        else:
            A[N - 1, :n_max] = c.rnorm * c.rMat[N - 1, :n_max]
        w = self.ts.wimp_lin[0]
        i = slice(1, N - 1)
        A[i, :] = c.rnorm * (c.rMat[i] - w * (d["ViscFac"] * self.hdif[0] * (
            c.d2rMat[i] + self.or1[i, None] * c.drMat[i] - self.or2[i, None] * c.rMat[i])
            - d["CorFac"] * self.ekpump[i, None] * c.rMat[i]))
        self._bfac_cols(A, (0, N - 1))
        return self._lu(A, "uphiMat")

    def _om_mat(self, m):
        """get_omMat (update_psi_coll_dmat.f90:829-911): row and column scaled."""
        c, d = self.cheb, self.d
        N, n_max = self.N, self.n_max
        A = np.zeros((N, N))
        A[0, :n_max] = c.rnorm * c.rMat[0, :n_max]
        A[N - 1, :n_max] = c.rnorm * c.rMat[N - 1, :n_max]
        w = self.ts.wimp_lin[0] * d["ViscFac"] * self.hdif[m // self.p.minc]
        dm2 = float(m) * float(m)
        i = slice(1, N - 1)
        A[i, :] = c.rnorm * (c.rMat[i] - w * (c.d2rMat[i] + self.or1[i, None] * c.drMat[i]
                                               - dm2 * self.or2[i, None] * c.rMat[i]))
        self._bfac_cols(A, (0, N - 1))
        f1 = 1.0 / np.max(np.abs(A), axis=1)
        A = A * f1[:, None]
        f2 = 1.0 / np.max(np.abs(A), axis=0)
        A = A * f2[None, :]
        return self._lu(A, "omMat"), f1, f2

    def _psi_mat_dmat(self, m):
        """get_psiMat (update_psi_coll_dmat.f90:913-983): dt independent."""
        c = self.cheb
        N, n_max = self.N, self.n_max
        A = np.zeros((N, N))
        A[0, :n_max] = c.rnorm * c.rMat[0, :n_max]
        A[N - 1, :n_max] = c.rnorm * c.rMat[N - 1, :n_max]
        dm2 = float(m) * float(m)
        i = slice(1, N - 1)
        or1, be, dbe, or2 = self.or1[i, None], self.beta[i, None], self.dbeta[i, None], self.or2[i, None]
        A[i, :] = c.rnorm * (c.d2rMat[i] + (or1 + be) * c.drMat[i]
                             + (or1 * be + dbe - dm2 * or2) * c.rMat[i])
        self._bfac_cols(A, (0, N - 1))
        f1 = 1.0 / np.max(np.abs(A), axis=1)
        A = A * f1[:, None]
        f2 = 1.0 / np.max(np.abs(A), axis=0)
        A = A * f2[None, :]
        return self._lu(A, "psiMat"), f1, f2

    def _psi_mat_smat(self, m):
        """get_psiMat (update_psi_coll_smat.f90:674-837): coupled 2N complex."""
        c, d, p = self.cheb, self.d, self.p
        N, n_max = self.N, self.n_max
        A = np.zeros((2 * N, 2 * N), complex)
        rn = c.rnorm
        A[0, N:N + n_max] = rn * c.rMat[0, :n_max]
        A[N - 1, N:N + n_max] = rn * c.rMat[N - 1, :n_max]
        if p.ktopv == 1:
            A[N, N:N + n_max] = rn * (c.d2rMat[0, :n_max] - self.or1[0] * c.drMat[0, :n_max])
        else:
            A[N, N:N + n_max] = rn * c.drMat[0, :n_max]
        if p.kbotv == 1:
            A[2 * N - 1, N:N + n_max] = rn * (c.d2rMat[N - 1, :n_max] - self.or1[N - 1] * c.drMat[N - 1, :n_max])
        else:
            A[2 * N - 1, N:N + n_max] = rn * c.drMat[N - 1, :n_max]
        w = self.ts.wimp_lin[0]
        hd = self.hdif[m // p.minc]
        dm2 = float(m) * float(m)
        i = slice(1, N - 1)
        ip = slice(N + 1, 2 * N - 1)
        or1, or2 = self.or1[i, None], self.or2[i, None]
        be, dbe = self.beta[i, None], self.dbeta[i, None]
        ekp, eup, eus, edp = (self.ekpump[i, None], self.ekp_up[i, None],
                              self.ekp_us[i, None], self.ekp_dusdp[i, None])
        CorFac = d["CorFac"]
        A[i, :N] = rn * (c.rMat[i] - w * (d["ViscFac"] * hd * (
            c.d2rMat[i] + or1 * c.drMat[i] - dm2 * or2 * c.rMat[i]) - CorFac * ekp * c.rMat[i]))
        A[i, N:] = -rn * w * (CorFac * ekp * eup * c.drMat[i]
                              + CorFac * ekp * (eup * be - (edp * 1j * m + eus) * 1j * m * or1) * c.rMat[i])
        if d["l_coriolis_imp"]:
            A[i, N:] = A[i, N:] - rn * w * CorFac * be * or1 * 1j * m * c.rMat[i]
        A[ip, :N] = rn * c.rMat[i]
        A[ip, N:] = rn * (c.d2rMat[i] + (or1 + be) * c.drMat[i] + (or1 * be + dbe - dm2 * or2) * c.rMat[i])
        self._bfac_cols(A, (0, N - 1, N, 2 * N - 1))
        f1 = 1.0 / np.max(np.abs(A), axis=1)
        A = A * f1[:, None]
        f2 = 1.0 / np.max(np.abs(A), axis=0)
        A = A * f2[None, :]
        return self._lu(A, "psiMat"), f1, f2

    def build_matrices(self):
        """All dt dependent LU factors, plus the dt independent dmat psi ones
        on first use (update_psi_coll_dmat.f90:94-98)."""
        M = self.M
        if self.l_integ:
            self.integ.build_matrices()
            self._mats_built = True
            return
        self.tmats = [self._temp_mat(int(self.mvec[i])) for i in range(M)]
        if self.l_chem:
            self.ximats = [self._temp_mat(int(self.mvec[i]), "xi") for i in range(M)]
        self.uphi = self._uphi_mat()
        if self.l_direct:
            self.psimats = [None] + [self._psi_mat_smat(int(self.mvec[i])) for i in range(1, M)]
        else:
            if not self._psi_dmat_built:
                self.psimats = [None] + [self._psi_mat_dmat(int(self.mvec[i])) for i in range(1, M)]
                self._psi_dmat_built = True
            self.ommats = [None] + [self._om_mat(int(self.mvec[i])) for i in range(1, M)]
            self._intermediate()
        self._mats_built = True

    def _bc_sums(self, f):
        """get_bc_influence_matrix (update_psi_coll_dmat.f90:1302-1452)."""
        c, p = self.cheb, self.p
        N = self.N
        fac = np.ones(N)
        fac[0] = fac[N - 1] = c.boundary_fac
        if p.ktopv == 1:
            top = fac * (c.d2rMat[0] - self.or1[0] * c.drMat[0])
        else:
            top = fac * c.drMat[0]
        if p.kbotv == 1:
            bot = fac * (c.d2rMat[N - 1] - self.or1[N - 1] * c.drMat[N - 1])
        else:
            bot = fac * c.drMat[N - 1]
        bcTop = np.zeros(f.shape[0], f.dtype)
        bcBot = np.zeros(f.shape[0], f.dtype)
        for n in range(N):            # sequential sum as in the reference
            bcTop = bcTop + top[n] * f[:, n]
            bcBot = bcBot + bot[n] * f[:, n]
        return c.rnorm * bcBot, c.rnorm * bcTop

    def _intermediate(self):
        """get_intermediate_om/psi and get_influence_matrix
        (update_psi_coll_dmat.f90:1136-1254)."""
        N, M, n_max = self.N, self.M, self.n_max
        self.om2 = np.zeros((M, N)); self.om3 = np.zeros((M, N))
        self.psi2 = np.zeros((M, N)); self.psi3 = np.zeros((M, N))
        for i in range(1, M):
            (lu, f1, f2) = self.ommats[i]
            for tgt, bc in ((self.om2, 1), (self.om3, 2)):
                rhs = np.zeros(N)
                if bc == 1:
                    rhs[N - 1] = f1[N - 1]
                else:
                    rhs[0] = f1[0]
                x = sla.lu_solve(lu, rhs) * f2
                tgt[i, :n_max] = x[:n_max]
            (plu, g1, g2) = self.psimats[i]
            for src, tgt in ((self.om2, self.psi2), (self.om3, self.psi3)):
                om_tmp = self.cheb.costf1_real(src[i])
                rhs = np.zeros(N)
                rhs[1:N - 1] = -om_tmp[1:N - 1]
                rhs = rhs * g1
                x = sla.lu_solve(plu, rhs) * g2
                tgt[i, :n_max] = x[:n_max]
        bot2, top2 = self._bc_sums(self.psi2)
        bot3, top3 = self._bc_sums(self.psi3)
        self.infl = np.zeros((M, 2, 2))
        for i in range(1, M):
            det = top2[i] * bot3[i] - top3[i] * bot2[i]
            self.infl[i] = [[bot3[i] / det, -top3[i] / det], [-bot2[i] / det, top2[i] / det]]

    # -- implicit terms ------------------------------------------------------
    def _temp_rhs_imp(self, istage, l_calc_lin, l_in_cheb, kind="temp"):
        """get_temp_rhs_imp_coll (update_temp_coll.f90:178-236) or
        get_xi_rhs_imp_coll (update_xi_coll.f90:168-216)."""
        if self.l_integ:
            return self.integ.temp_rhs_imp(istage, l_calc_lin, kind)
        c = self.cheb
        f, df, ta, diff = self._sc(kind)[:4]
        fld = getattr(self, f)
        if l_calc_lin:
            dfld, work = c.get_ddr(fld, l_dct=not l_in_cheb)
            setattr(self, df, dfld)
            if l_in_cheb:
                fld = c.costf1(fld)
        else:
            if l_in_cheb:
                fld = c.costf1(fld)
        setattr(self, f, fld)
        if istage == 1:
            ta.old[istage - 1] = fld.copy()
        if l_calc_lin:
            dm2 = (self.mvec.astype(float) ** 2)[:, None]
            ta.impl[istage - 1] = diff * self.hdif[:, None] * (
                work + self.or1 * getattr(self, df) - dm2 * self.or2 * fld)

    def _xi_rhs_imp(self, istage, l_calc_lin, l_in_cheb):
        return self._temp_rhs_imp(istage, l_calc_lin, l_in_cheb, kind="xi")

    def _psi_rhs_imp(self, istage, l_calc_lin, l_in_cheb):
        """get_psi_rhs_imp_coll_{dmat,smat} (update_psi_coll_dmat.f90:554-682,
        update_psi_coll_smat.f90:380-527)."""
        if self.l_integ:
            return self.integ.psi_rhs_imp(istage, l_calc_lin)
        c, d = self.cheb, self.d
        om0 = self.om[0].real.copy()
        if l_calc_lin:
            self.dom, work = c.get_ddr(self.om, l_dct=not l_in_cheb)
            if l_in_cheb:
                self.om = c.costf1(self.om)
        else:
            if l_in_cheb:
                self.om = c.costf1(self.om)
        self.om[0] = om0 + 0j
        if istage == 1:
            old = self.om.copy()
            old[0] = self.up[0]
            self.dpsidt.old[istage - 1] = old
        if l_calc_lin:
            uphi0 = self.up[0].real.copy()
            duphi0, d2uphi0 = c.get_ddr_real(uphi0)
            m = self.mvec[:, None]
            dm2 = (self.mvec.astype(float) ** 2)[:, None]
            hd = self.hdif[:, None]
            imp = d["ViscFac"] * hd * (work + self.or1 * self.dom - dm2 * self.or2 * self.om)
            if self.l_direct:
                imp = imp - d["CorFac"] * self.ekpump * (
                    self.om + self.ekp_up * self.up + (self.ekp_dusdp * 1j * m + self.ekp_us) * self.us)
                if d["l_coriolis_imp"]:
                    imp = imp + d["CorFac"] * self.beta * self.us
            if d["l_buo_imp"]:
                imp = imp - self.rgrav * self.or1 * d["BuoFac"] * 1j * m * self.temp
                if self.l_chem:
                    imp = imp - self.rgrav * self.or1 * d["ChemFac"] * 1j * m * self.xi
            imp[0] = (d["ViscFac"] * self.hdif[0] * (d2uphi0 + self.or1 * duphi0 - self.or2 * uphi0)
                      - d["CorFac"] * self.ekpump * uphi0)
            self.dpsidt.impl[istage - 1] = imp
        bal = getattr(self, "_bal", None)
        if bal is not None and not self.l_direct:
            # update_psi_coll_dmat.f90:642-676 (computed whatever l_calc_lin)
            if not l_calc_lin:
                self.dom, work = c.get_ddr(self.om, l_dct=True)
            dm2 = (self.mvec.astype(float) ** 2)[:, None]
            visc = work + self.or1 * self.dom - dm2 * self.or2 * self.om
            visc[0] = 0.0
            bal["visc"] = visc
            uphi0 = self.up[0].real.copy()
            duphi0, d2uphi0 = c.get_ddr_real(uphi0)
            bal["vp_visc"] = d["ViscFac"] * self.hdif[0] * (d2uphi0 + self.or1 * duphi0 - self.or2 * uphi0)
            bal["vp_pump"] = -d["CorFac"] * self.ekpump * uphi0 if self.p.l_ek_pump else np.zeros(self.N)

    # -- solves (mloop) ------------------------------------------------------
    def update_temp(self, lMat, l_log_next, kind="temp"):
        """update_temp_co (update_temp_coll.f90:66-150) or update_xi_co
        (update_xi_coll.f90:66-140)."""
        if self.l_integ:
            return self.integ.update_temp(l_log_next, kind)
        N, M, n_max = self.N, self.M, self.n_max
        ts = self.ts
        f, df, ta, _, top, bot = self._sc(kind)[:6]
        mats = self.tmats if kind == "temp" else self.ximats
        work = ts.set_imex_rhs(ta)
        fld = np.zeros((M, N), complex)
        for i in range(M):
            (lu_piv, fac) = mats[i]
            rhs = np.empty(N, complex)
            rhs[0] = top[i]
            rhs[N - 1] = bot[i]
            rhs[1:N - 1] = work[i, 1:N - 1]
            rhs = fac * rhs
            x = self._solve_real(lu_piv, rhs)
            fld[i, :n_max] = x[:n_max]
        setattr(self, f, fld)
        ts.rotate_imex(ta)
        if ts.istage == ts.nstages:
            self._temp_rhs_imp(1, self._calc_rhs(1), l_in_cheb=True, kind=kind)
        else:
            self._temp_rhs_imp(ts.istage + 1, self._calc_rhs(ts.istage + 1), l_in_cheb=True, kind=kind)
        if l_log_next:
            setattr(self, df, self.cheb.get_dr(getattr(self, f)))

    def update_xi(self, lMat, l_log_next):
        return self.update_temp(lMat, l_log_next, kind="xi")

    def update_om(self):
        """update_om_coll_dmat (update_psi_coll_dmat.f90:126-466) or
        update_om_coll_smat (update_psi_coll_smat.f90:88-321)."""
        if self.l_integ:
            return self.integ.update_psi()
        c, d = self.cheb, self.d
        N, M, n_max = self.N, self.M, self.n_max
        ts = self.ts
        bal = getattr(self, "_bal", None)
        if bal is not None:
            # initialize_domdt / initialize_dvpdt (vort_balance.f90, vp_balance.f90)
            bal["dwdt"] = self.om / ts.dt[0]
            bal["dvpdt"] = self.up[0].real / ts.dt[0]
            bal["rey_stress"] = self.dpsidt.expl[ts.istage - 1][0].real.copy()
            m_ = self.mvec[:, None]
            buo = np.zeros((M, N), complex)
            buo[1:] = -d["BuoFac"] * self.rgrav * self.or1 * 1j * m_[1:] * self.temp[1:]
            if self.l_chem:
                buo[1:] = buo[1:] - d["ChemFac"] * self.rgrav * self.or1 * 1j * m_[1:] * self.xi[1:]
            bal["buo"] = buo
        work = ts.set_imex_rhs(self.dpsidt)
        m = self.mvec
        # m = 0: uphi solve
        rhs0 = np.zeros(N)
        rhs0[1:N - 1] = work[0, 1:N - 1].real
        x0 = sla.lu_solve(self.uphi, rhs0)
        uphi0 = np.zeros(N)
        uphi0[:n_max] = x0[:n_max]
        om = np.zeros((M, N), complex)
        psi = np.zeros((M, N), complex)
        buo = None
        if d["l_buo_imp"]:
            buo = ts.wimp_lin[0] * d["BuoFac"] * self.rgrav * self.or1
            buo_xi = ts.wimp_lin[0] * d["ChemFac"] * self.rgrav * self.or1
        for i in range(1, M):
            rhs = np.zeros(N, complex)
            if buo is not None:
                rhs[1:N - 1] = work[i, 1:N - 1] - buo[1:N - 1] * 1j * m[i] * self.temp[i, 1:N - 1]
                if self.l_chem:
                    rhs[1:N - 1] = rhs[1:N - 1] - buo_xi[1:N - 1] * 1j * m[i] * self.xi[i, 1:N - 1]
            else:
                rhs[1:N - 1] = work[i, 1:N - 1]
            if self.l_direct:
                (lu_piv, f1, f2) = self.psimats[i]
                big = np.zeros(2 * N, complex)
                big[:N] = rhs
                big = big * f1
                x = sla.lu_solve(lu_piv, big) * f2
                om[i, :n_max] = x[:n_max]
                psi[i, :n_max] = x[N:N + n_max]
            else:
                (lu_piv, f1, f2) = self.ommats[i]
                x = self._solve_real(lu_piv, rhs * f1) * f2
                om[i, :n_max] = x[:n_max]
        # uphi0 to physical space; om0 = duphi0/dr
        om0 = c.get_dr_real(uphi0, l_dct=False)
        uphi0 = c.costf1_real(uphi0)
        if not self.l_direct:
            w = om.copy()
            w[0] = work[0]
            w = c.costf1(w)
            for i in range(1, M):
                (lu_piv, f1, f2) = self.psimats[i]
                rhs = np.zeros(N, complex)
                rhs[1:N - 1] = -w[i, 1:N - 1]
                x = self._solve_real(lu_piv, rhs * f1) * f2
                psi[i, :n_max] = x[:n_max]
            # influence matrix correction (update_psi_coll_dmat.f90:1256-1300)
            bot1, top1 = self._bc_sums(psi)
            for i in range(1, M):
                inf = self.infl[i]
                c1 = -inf[0, 0] * top1[i] - inf[0, 1] * bot1[i]
                c2 = -inf[1, 0] * top1[i] - inf[1, 1] * bot1[i]
                psi[i] = psi[i] + c1 * self.psi2[i] + c2 * self.psi3[i]
                om[i] = om[i] + c1 * self.om2[i] + c2 * self.om3[i]
        work = c.get_dr(psi, l_dct_in=False)
        psi = c.costf1(psi)
        us = 1j * m[:, None] * self.or1 * psi
        up = -work - self.beta * psi
        us[0] = 0.0
        up[0] = uphi0
        om[0] = om0 + self.or1 * uphi0
        self.psi, self.us, self.up, self.om = psi, us, up, om
        ts.rotate_imex(self.dpsidt)
        if bal is not None:
            # finalize_domdt before get_psi_rhs_imp: om of m /= 0 is still in
            # Chebyshev space there (update_psi_coll_dmat.f90:444-451)
            bal["dwdt"] = om / ts.dt[0] - bal["dwdt"]
            bal["dvpdt"] = up[0].real / ts.dt[0] - bal["dvpdt"]
        if ts.istage == ts.nstages:
            self._psi_rhs_imp(1, self._calc_rhs(1), l_in_cheb=True)
        else:
            self._psi_rhs_imp(ts.istage + 1, self._calc_rhs(ts.istage + 1), l_in_cheb=True)

    def _calc_rhs(self, stage):
        """l_imp_calc_rhs of the stage whose implicit term is formed next: one
        flag for the multistep family, one per stage for DIRK."""
        f = self.ts.l_imp_calc_rhs
        return f[stage - 1] if isinstance(f, list) else f

    def _ass_mat(self, m):
        """get_assMat (update_psi_coll_smat.f90:839-917 = dmat:1056-1134): the
        streamfunction from the assembled vorticity, psi = dpsi/dr = 0 on both
        rigid walls; dt independent, not equilibrated."""
        c = self.cheb
        N, n_max = self.N, self.n_max
        A = np.zeros((N, N))
        rn = c.rnorm
        A[0, :n_max] = rn * c.rMat[0, :n_max]
        A[N - 1, :n_max] = rn * c.rMat[N - 1, :n_max]
        A[1, :n_max] = rn * c.drMat[0, :n_max]                 # ktopv = 2
        A[N - 2, :n_max] = rn * c.drMat[N - 1, :n_max]         # kbotv = 2
        dm2 = float(m) * float(m)
        i = slice(2, N - 2)
        or1, or2 = self.or1[i, None], self.or2[i, None]
        be, dbe = self.beta[i, None], self.dbeta[i, None]
        A[i, :] = -rn * (c.d2rMat[i] + (or1 + be) * c.drMat[i] + (or1 * be + dbe - dm2 * or2) * c.rMat[i])
        self._bfac_cols(A, (0, N - 1))
        return self._lu(A, "assMat")

    def assemble_stage(self, l_log_next=True):
        """assemble_stage (mloop.f90): assemble_temp_coll
        (update_temp_coll.f90:238-307) and assemble_psi_coll_{smat,dmat}
        (update_psi_coll_smat.f90:529-672)."""
        if self.l_integ:
            # mloop.f90:162-164: abortRun for the integration method
            raise NotImplementedError("Assembly stage with integration method not implemented")
        c, ts = self.cheb, self.ts
        N, M, n_max = self.N, self.M, self.n_max
        m = self.mvec
        # temperature: interior from the assembled rhs, Dirichlet rows (robin_bc)
        work = ts.assemble_imex(self.dTdt)
        temp = self.temp.copy()
        temp[:, 1:N - 1] = work[:, 1:N - 1]
        temp[0, 1:N - 1] = work[0, 1:N - 1].real + 0j
        temp[:, 0] = self.topt
        temp[:, N - 1] = self.bott
        self.temp = temp
        self._temp_rhs_imp(1, self._calc_rhs(1), l_in_cheb=False)
        if l_log_next:
            self.dtemp = c.get_dr(self.temp)
        if self.l_chem:
            # assemble_xi_coll (update_xi_coll.f90:218-269): no dxi refresh
            work = ts.assemble_imex(self.dxidt)
            xi = self.xi.copy()
            xi[:, 1:N - 1] = work[:, 1:N - 1]
            xi[0, 1:N - 1] = work[0, 1:N - 1].real + 0j
            xi[:, 0] = self.topxi
            xi[:, N - 1] = self.botxi
            self.xi = xi
            self._xi_rhs_imp(1, self._calc_rhs(1), l_in_cheb=False)
        # streamfunction from the assembled vorticity
        work = ts.assemble_imex(self.dpsidt)
        up0 = np.zeros(N)
        up0[1:N - 1] = work[0, 1:N - 1].real                   # rigid walls: u_phi = 0
        if not hasattr(self, "_assmats"):
            self._assmats = [None] + [self._ass_mat(int(m[i])) for i in range(1, M)]
        psi = np.zeros((M, N), complex)
        for i in range(1, M):
            rhs1 = np.zeros(N, complex)
            rhs1[2:N - 2] = work[i, 2:N - 2]
            x = self._solve_real(self._assmats[i], rhs1)
            psi[i, :n_max] = x[:n_max]
        om0 = c.get_dr_real(up0)
        dpsi, d2psi = c.get_ddr(psi, l_dct=False)
        psi = c.costf1(psi)
        mm = m[:, None].astype(float)
        us = 1j * mm * self.or1 * psi
        up = -dpsi - self.beta * psi
        om = -(d2psi + (self.or1 + self.beta) * dpsi
               + (self.or1 * self.beta + self.dbeta - mm ** 2 * self.or2) * psi)
        us[0] = 0.0
        up[0] = up0
        om[0] = om0 + self.or1 * up0
        self.psi, self.us, self.up, self.om = psi, us, up, om
        self._psi_rhs_imp(1, self._calc_rhs(1), l_in_cheb=False)

    def _advance_dirk(self, l_log_next=True):
        """One time step of a DIRK scheme: the stage loop of time_loop
        (step_time.f90:210-368) and the assembly stage (:370-384)."""
        ts, p = self.ts, self.p
        self.n_time_step += 1
        n_time_step = self.n_time_step
        ts.istage = 1
        lMat = False
        for n_stage in range(1, ts.nstages + 1):
            if ts.l_exp_calc[n_stage - 1]:
                dtempdt, dVsT, dpsidt, dVsOm = self.radial_loop()
                self.dTdt.expl[ts.istage - 1] = dtempdt
                self.dpsidt.expl[ts.istage - 1] = dpsidt
                self.finish_explicit(dVsT, dVsOm)
            l_new_dt = False
            if ts.istage == 1:
                l_new_dt, dt_new = self.dt_courant()
                sched = getattr(self, "dt_schedule", None)
                if sched is not None and n_time_step - 1 < len(sched):
                    dt_new = float(sched[n_time_step - 1])
                    l_new_dt = dt_new != ts.dt[0]
                self.l_new_dt = l_new_dt
                ts.set_dt_array(dt_new, self.dtMin)
                if ts.set_weights():
                    self.lMatNext = True
                self.time = self.time + ts.dt[0]
            lMat = self.lMatNext
            if (l_new_dt or lMat) and ts.istage == 1:
                lMat = True
            self.lMatNext = False
            if (not ts.l_assembly) or ts.istage != ts.nstages:
                if lMat or not self._mats_built:
                    self.build_matrices()
                self.update_temp(lMat, l_log_next)
                if self.l_chem:
                    self.update_xi(lMat, l_log_next)
                self.update_om()
                ts.istage += 1
        if ts.l_assembly:
            self.assemble_stage(l_log_next)
        return lMat

    # -- one iteration of the outer loop (src/step_time.f90:139-406) ----------
    def advance(self, l_log_next=True):
        """One time step (stage body, multistep family: one stage)."""
        if self.ts.family == "DIRK":
            return self._advance_dirk(l_log_next)
        ts, p = self.ts, self.p
        self.n_time_step += 1
        n_time_step = self.n_time_step
        ts.istage = 1
        dtempdt, dVsT, dpsidt, dVsOm = self.radial_loop()
        self.dTdt.expl[0] = dtempdt
        self.dpsidt.expl[0] = dpsidt
        self.finish_explicit(dVsT, dVsOm)
        l_new_dt, dt_new = self.dt_courant()
        sched = getattr(self, "dt_schedule", None)
        if sched is not None and n_time_step - 1 < len(sched):
            # fixed step sequence (test hook for the adjoint checks; pizza
            # itself always takes dt from dt_courant)
            dt_new = float(sched[n_time_step - 1])
            l_new_dt = dt_new != ts.dt[0]
        self.l_new_dt = l_new_dt
        ts.set_dt_array(dt_new, self.dtMin)
        if ts.set_weights():
            self.lMatNext = True
        self.time = self.time + ts.dt[0]
        lMat = self.lMatNext
        if l_new_dt or lMat:
            lMat = True
        self.lMatNext = False
        # start_from_another_scheme (step_time.f90:417-516)
        if (self.l_bridge_step and ts.time_scheme != "CNAB2"
                and n_time_step <= ts.nold - 1 and ts.family == "MULTISTEP"):
            self._temp_rhs_imp(1, True, l_in_cheb=False)
            if self.l_chem:
                self._xi_rhs_imp(1, True, l_in_cheb=False)
            if self.l_integ and self.l_direct:
                # step_time.f90:497-498 hands psi_Mloc to get_psi_rhs_imp_int_smat
                # in the place of xi_Mloc: with composition on, the bridge's
                # implicit buoyancy takes -ChemFac rgrav/r i m psi
                self.integ.psi_rhs_imp(1, True, xi=self.psi)
            else:
                self._psi_rhs_imp(1, True, l_in_cheb=False)
            ts.bridge_with_cnab2()
        if self.l_AB1 and n_time_step == 1:
            ts.wexp[0] = ts.dt[0]
            ts.wexp[1:] = 0.0
            self.l_AB1 = False
        if lMat or not self._mats_built:
            self.build_matrices()
        self.update_temp(lMat, l_log_next)
        if self.l_chem:
            self.update_xi(lMat, l_log_next)
        self.update_om()
        ts.istage += 1
        return lMat

    def balance_step(self):
        """One step that also records the vorticity and u_phi force balances
        (vort_balance.f90, vp_balance.f90 with l_calc set: the hooks of
        update_psi_coll_dmat.f90).  Returns {"vort": {buo, cor, adv, dwdt,
        visc, pump: (M, N) complex}, "vp": {rey_stress, dvpdt, visc, pump:
        (N,) real}}.  Collocation, influence matrix, multistep schemes."""
        self._bal = {}
        try:
            self.advance()
            b = self._bal
        finally:
            self._bal = None
        vort = {k: b[k] for k in ("buo", "cor", "adv", "dwdt", "visc", "pump")}
        vp = {"rey_stress": b["rey_stress"], "dvpdt": b["dvpdt"], "visc": b["vp_visc"], "pump": b["vp_pump"]}
        return {"vort": vort, "vp": vp}

    # -- time series (src/outputs.f90:418-830) -------------------------------
    def spectra(self):
        """calculate_spectra (spectra.f90:104-196), the snapshot part: per m
        the rInt_R of pi cc2real(f) r height for f = us, up, om, temp.  The
        fifth column is the reference's xi2_m, which spectra.f90:183 fills
        with the temperature's integral (rInt_R(temp2R)) when composition is
        on; zero without composition.  (M, 5) array."""
        c = self.cheb
        out = np.zeros((self.M, 5))
        for i in range(self.M):
            for k, f in enumerate((self.us, self.up, self.om, self.temp)):
                z = f[i]
                c2 = z.real ** 2 if i == 0 else 2.0 * (z.real ** 2 + z.imag ** 2)
                out[i, k] = c.rInt_R(np.pi * c2 * self.r * self.height)
            if self.l_chem:
                out[i, 4] = out[i, 3]
        return out

    def spectra_2d(self):
        """The (r, m) spectra of calculate_spectra (spectra.f90:134-142):
        pi cc2real(f) r height for f = us, up, om at every (r, m), before
        the r-integration.  (3, N, M) array."""
        out = np.zeros((3, self.N, self.M))
        for k, f in enumerate((self.us, self.up, self.om)):
            c2 = 2.0 * (f.real ** 2 + f.imag ** 2)
            c2[0] = f[0].real ** 2
            out[k] = (np.pi * c2 * self.r * self.height).T
        return out

    def time_series(self):
        """Rows of e_kin, e_kin_3D and heat at the current state."""
        d, c = self.d, self.cheb
        r = self.r
        us, up, om, T, dT = self.us, self.up, self.om, self.temp, self.dtemp
        w = np.full(self.M, 2.0)
        w[0] = 1.0

        def c2r(f):
            v = 2.0 * (f.real ** 2 + f.imag ** 2)
            v[0] = f[0].real ** 2
            return v

        us2_r = np.zeros(self.N); up2_r = np.zeros(self.N); upaxi = np.zeros(self.N)
        nu_vol_r = np.zeros(self.N)
        a_us, a_up, a_dT, a_T = c2r(us), c2r(up), c2r(dT), c2r(T)
        m2 = (self.mvec.astype(float) ** 2)
        for i in range(self.M):       # sequential over m as in the reference
            us2_r = us2_r + a_us[i]
            up2_r = up2_r + a_up[i]
            nu_vol_r = nu_vol_r + a_dT[i] + m2[i] * self.or2 * a_T[i]
        upaxi = a_up[0].copy()
        nu_vol_r = nu_vol_r * r * self.height
        rows = {}
        us2_2D = round_off(np.pi * c.rInt_R(us2_r * r))
        up2_2D = round_off(np.pi * c.rInt_R(up2_r * r))
        upaxi_2D = round_off(np.pi * c.rInt_R(upaxi * r))
        rows["e_kin"] = [self.time, us2_2D, up2_2D, upaxi_2D]
        if not d["l_non_rot"]:
            h = self.height
            us2_3D = round_off(np.pi * c.rInt_R(us2_r * r * h))
            up2_3D = round_off(np.pi * c.rInt_R(up2_r * r * h))
            uz2_3D = round_off(np.pi * c.rInt_R(us2_r * self.beta ** 2 * r * h ** 3 / 12.0))
            upaxi_3D = round_off(np.pi * c.rInt_R(upaxi * r * h))
            rows["e_kin_3D"] = [self.time, us2_3D, up2_3D, uz2_3D, upaxi_3D]
        if d["l_heat"]:
            N = self.N
            tTop = round_off(T[0, 0].real + self.tcond[0])
            tBot = round_off(T[0, N - 1].real + self.tcond[N - 1])
            NuTop = round_off(1.0 + dT[0, 0].real / self.dtcond[0])
            NuBot = round_off(1.0 + dT[0, N - 1].real / self.dtcond[N - 1])
            Nu_vol = c.rInt_R(nu_vol_r)
            Nu_vol = round_off(1.0 + Nu_vol / c.rInt_R(self.dtcond * self.dtcond * self.height * r))
            # flux_r: buoyancy flux plus conduction (outputs.f90:478-492)
            flux_r = np.zeros(N)
            fl = 2.0 * (us.real * T.real + us.imag * T.imag)
            fl[0] = us[0].real * T[0].real
            for i in range(self.M):
                flux_r = flux_r + fl[i]
                if i == 0:
                    flux_r = flux_r - d["TdiffFac"] * dT[0].real - d["TdiffFac"] * self.dtcond
            if d["l_non_rot"]:
                fac = c.rInt_R(-d["TdiffFac"] * self.dtcond * r)
                Nu_int = c.rInt_R(flux_r * r / fac)
            else:
                r_cmb = d["r_cmb"]
                tmp = -d["TdiffFac"] * self.dtcond * (r / r_cmb) ** 2
                theta = np.arcsin(r / r_cmb)
                fac = simps(tmp, theta)
                Nu_int = simps(flux_r * (r / r_cmb) ** 2, theta) / fac
            Nu_int = round_off(Nu_int)
            beta_t = round_off(self.dtcond[N // 2 - 1] + dT[0, N // 2 - 1].real)
            rows["heat"] = [self.time, NuTop, NuBot, Nu_vol, Nu_int, tTop, tBot, beta_t]
        if self.l_chem:
            # composition.TAG (outputs.f90:795-827)
            N = self.N
            X, dX = self.xi, self.dxi
            a_x, a_dx = c2r(X), c2r(dX)
            sh_r = np.zeros(N)
            for i in range(self.M):
                sh_r = sh_r + a_dx[i] + m2[i] * self.or2 * a_x[i]
            sh_r = sh_r * r * self.height
            xiTop = round_off(X[0, 0].real + self.xicond[0])
            xiBot = round_off(X[0, N - 1].real + self.xicond[N - 1])
            ShTop = round_off(1.0 + dX[0, 0].real / self.dxicond[0])
            ShBot = round_off(1.0 + dX[0, N - 1].real / self.dxicond[N - 1])
            Sh_vol = round_off(1.0 + c.rInt_R(sh_r) / c.rInt_R(self.dxicond * self.dxicond * self.height * r))
            beta_xi = round_off(self.dxicond[N // 2 - 1] + dX[0, N // 2 - 1].real)
            rows["composition"] = [self.time, ShTop, ShBot, Sh_vol, xiTop, xiBot, beta_xi]
        return rows

    # -- the outer loop (src/step_time.f90:69-415) ----------------------------
    def run(self, n_time_steps=None, n_log_step=None, callback=None):
        """Run ``time_loop``: logs rows at step 0, every n_log_step and the end."""
        p = self.p
        nts = p.n_time_steps if n_time_steps is None else n_time_steps
        nls = p.n_log_step if n_log_step is None else n_log_step
        n_run = nts if nts <= 2 else nts + 1
        for n in range(1, n_run + 1):
            l_log = l_correct_step(n - 1, nts, nls, 0)
            l_log_next = l_correct_step(n, nts, nls, 0)
            l_stop = n == n_run
            if n == 1 or l_stop:
                l_log = True
            if l_log:
                for k, v in self.time_series().items():
                    self.rows[k].append(v)
            if callback is not None:
                callback(self, n)
            if l_stop:
                break
            self.advance(l_log_next=l_log_next)
        return {k: np.array(v) for k, v in self.rows.items()}

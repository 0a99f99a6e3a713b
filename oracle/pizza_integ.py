"""pizza's Chebyshev-integration ("integ") method with the tau boundary rows:
the oracle restatement of src/update_temp_integ.f90 with either the direct
(coupled) streamfunction solve, src/update_psi_integ_smat.f90, or the
influence-matrix solve, src/update_psi_integ_dmat.f90, as called from
mloop.f90:84-100 and :209-226, step_time.f90:488-500 and
init_fields.f90:54-258.

Test infrastructure only (the checker of the GPU integ path).

Unknowns live in Chebyshev space: temp_hat (temperature) and psi_hat (the
streamfunction, m > 0), plus the m = 0 azimuthal velocity's coefficients.
Every equation is multiplied by r^2 (r^4 for the streamfunction) and
integrated twice (four times) in r, which makes the operators banded
(oracle/chebsparse.py derives them); the first 2 (4) rows are replaced by
tau rows carrying the boundary conditions.  The reference stores them as
bordered band matrices and solves with a bordered LU (oracle/bordered.py
restates it: ``bordered=True``); by default this restatement holds them dense
and solves with LAPACK's dense LU, which changes only rounding -- and on the
ill-conditioned systems of n_r_max ~ 97 at small E the dense LU is the less
accurate of the two.  The row preconditioning of get_lhs_mat_tau (one over
the largest entry of each row) is kept.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .bordered import BorderedLU
from .chebsparse import IntegOperators


class IntegScheme:
    """The integ operators and stage routines of one ``Pizza`` instance."""

    def __init__(self, pz, bordered: bool = False):
        self.pz = pz
        self.bordered = bordered
        p, d, c = pz.p, pz.d, pz.cheb
        N = pz.N
        self.ops = ops = IntegOperators(N, d["r_icb"], d["r_cmb"], c.rnorm)
        self.rnorm = c.rnorm
        # tau-line vectors: values and r-derivatives of T_n at the outer (top)
        # and inner (bottom) boundary (chebyshev.f90:363-379)
        n = np.arange(N, dtype=float)
        dn2 = n * n
        sg = np.where(np.arange(N) % 2 == 0, 1.0, -1.0)
        self.r_top, self.r_bot = np.ones(N), sg
        self.dr_top, self.dr_bot = 2.0 * dn2, -2.0 * dn2 * sg
        self.d2r_top = 4.0 / 3.0 * dn2 * (dn2 - 1.0)
        self.d2r_bot = self.d2r_top * sg
        self.d3top = 8.0 / 15.0 * dn2 * (dn2 - 1.0) * (dn2 - 4.0)    # update_psi_integ_smat.f90:1303-1306
        # the influence-matrix top condition of the rotating rigid wall: the
        # fourth x-derivative of T_n at x = 1 (update_psi_integ_dmat.f90:1381-1384)
        self.d4top = 16.0 / 105.0 * dn2 * (dn2 - 1.0) * (dn2 - 4.0) * (dn2 - 9.0)
        mvec = pz.mvec
        rot = not d["l_non_rot"]
        vis = d["ViscFac"]
        self.dmat = not pz.l_direct
        # d/dt operators (RHSI) and linear implicit operators (RHSIL) per m
        # (update_temp_integ.f90:813-832; update_psi_integ_smat.f90:1631-1764;
        # update_psi_integ_dmat.f90:1128-1210)
        self.t_rhsi = [ops.temp_lap(int(m)) for m in mvec]
        self.p_rhsi = [ops.i2r2.astype(complex)]
        self.p_rhsil = [vis * pz.hdif[0] * ops.uphi_lap + 0j]
        self.tmats = None
        self.pmats = None
        if self.dmat:
            # vorticity equation I2[r^2 .] (2 tau rows) and the dt-independent
            # streamfunction operator from omega, psi_hat = -L_psi^-1 I2[r^2 om]
            # with L_psi = intcheb2rmult2laplrot = -I2[r^2 omega(psi)]
            # (update_psi_integ_dmat.f90:971-1089)
            from .chebsparse import omega_rot_terms
            self.psi_ops = [None]
            for i in range(1, len(mvec)):
                m = int(mvec[i])
                self.p_rhsi.append(ops.i2r2 + 0j)
                self.p_rhsil.append(vis * pz.hdif[i] * ops.temp_lap(m) + 0j)
                if rot:
                    L = -ops._rows(ops.c.integrated(omega_rot_terms(ops.ro, float(m)), 2), 2)
                else:
                    L = ops.temp_lap(m)
                L = L.copy()
                L[0] = self.rnorm * self.r_top
                L[1] = self.rnorm * self.r_bot
                self.psi_ops.append(self._finish_lhs(L, 2))
            return
        for i in range(1, len(mvec)):
            m = int(mvec[i])
            if rot:
                self.p_rhsi.append(ops.psi_rot(m) + 0j)
                L = vis * pz.hdif[i] * ops.psi_rot2(m) + 0j
                if d["l_coriolis_imp"]:
                    L = L - 1j * d["CorFac"] * m * ops.i4r4
            else:
                self.p_rhsi.append(-ops.psi_nonrot(m) + 0j)
                L = -vis * pz.hdif[i] * ops.psi_nonrot2(m) + 0j
            self.p_rhsil.append(L)

    # -- left-hand sides (get_lhs_mat_tau) ----------------------------------
    def _finish_lhs(self, A, ntau):
        A[:ntau, 0] *= self.pz.cheb.boundary_fac
        fac = 1.0 / np.max(np.abs(A), axis=1)
        A = A * fac[:, None]
        if self.bordered:
            return BorderedLU(A, ntau), fac
        lu, piv = sla.lu_factor(A, check_finite=True)
        if np.any(np.diag(lu) == 0.0):
            raise np.linalg.LinAlgError("Singular matrix in the integ solve")
        return (lu, piv), fac

    def _temp_lhs(self, i, kind="temp"):
        """update_temp_integ.f90:631-776 (update_xi_integ.f90 for the
        composition: the same operator with XidiffFac)."""
        pz = self.pz
        _, _, _, diff, _, _, ktop, kbot = pz._sc(kind)
        w = pz.ts.wimp_lin[0]
        A = self.ops.i2r2 - w * diff * pz.hdif[i] * self.t_rhsi[i]
        A[0] = self.rnorm * (self.r_top if ktop == 1 else self.dr_top)
        A[1] = self.rnorm * (self.r_bot if kbot == 1 else self.dr_bot)
        return self._finish_lhs(A, 2)

    def _psi_lhs(self, i):
        """update_psi_integ_smat.f90:1286-1581: LHS = RHSI - wimp RHSIL with
        the 2 (m = 0) or 4 tau rows; influence-matrix variant
        (update_psi_integ_dmat.f90:783-969): the vorticity operator with 2 tau
        rows, omega(r_o) and omega(r_i) for m > 0."""
        pz, p, d = self.pz, self.pz.p, self.pz.d
        w = pz.ts.wimp_lin[0]
        or1 = pz.or1
        N = pz.N
        A = self.p_rhsi[i] - w * self.p_rhsil[i]
        rn = self.rnorm
        if self.dmat and i > 0:
            A = A.real.copy()
            A[0] = rn * self.r_top
            A[1] = rn * self.r_bot
            return self._finish_lhs(A, 2)
        if i == 0:
            A = A.real.copy()
            A[0] = rn * ((self.dr_top - or1[0] * self.r_top) if p.ktopv == 1 else self.r_top)
            A[1] = rn * ((self.dr_bot - or1[N - 1] * self.r_bot) if p.kbotv == 1 else self.r_bot)
            return self._finish_lhs(A, 2)
        A[0] = rn * self.r_top
        A[1] = rn * self.r_bot
        if p.ktopv == 1:
            A[2] = rn * (self.d2r_top - or1[0] * self.dr_top)
        elif d["l_non_rot"]:
            A[2] = rn * self.dr_top
        else:
            A[2] = rn * self.d3top
        if p.kbotv == 1:
            A[3] = rn * (self.d2r_bot - or1[N - 1] * self.dr_bot)
        else:
            A[3] = rn * self.dr_bot
        return self._finish_lhs(A, 4)

    def build_matrices(self):
        M = self.pz.M
        self.tmats = [self._temp_lhs(i) for i in range(M)]
        if self.pz.l_chem:
            self.ximats = [self._temp_lhs(i, "xi") for i in range(M)]
        self.pmats = [self._psi_lhs(i) for i in range(M)]
        if self.dmat:
            self._intermediate()

    def _psi_from_om(self, i, om_hat):
        """psi_hat from omega_hat (update_psi_integ_dmat.f90:310-327)."""
        rhs = -(self.ops.i2r2 @ om_hat)
        rhs[:2] = 0.0
        return self._solve(self.psi_ops[i], rhs)

    def _bc_sums(self, psi_hat):
        """get_bc_influence_matrix (update_psi_integ_dmat.f90:1361-1530):
        the two conditions left to the influence matrix, on Chebyshev
        coefficients with the half weight at both ends."""
        pz, p = self.pz, self.pz.p
        N = pz.N
        fac = np.ones(N)
        fac[0] = fac[N - 1] = pz.cheb.boundary_fac
        if p.ktopv == 1:
            top = self.d2r_top - pz.or1[0] * self.dr_top
        elif pz.d["l_non_rot"]:
            top = self.dr_top
        else:
            top = self.d4top
        if p.kbotv == 1:
            bot = self.d2r_bot - pz.or1[N - 1] * self.dr_bot
        else:
            bot = self.dr_bot
        t = b = 0.0
        for n in range(N):            # sequential sums as in the reference
            t = t + fac[n] * top[n] * psi_hat[..., n]
            b = b + fac[n] * bot[n] * psi_hat[..., n]
        return self.rnorm * t, self.rnorm * b

    def _intermediate(self):
        """get_intermediate_sol and get_influence_matrix
        (update_psi_integ_dmat.f90:1212-1313): the homogeneous solutions with
        omega = 1 on the inner (set 1) or outer (set 2) wall."""
        pz = self.pz
        M, N = pz.M, pz.N
        self.om23 = np.zeros((M, 2, N))
        self.psi23 = np.zeros((M, 2, N))
        self.infl = np.zeros((M, 2, 2))
        for i in range(1, M):
            for k, row in enumerate((1, 0)):
                rhs = np.zeros(N)
                rhs[row] = 1.0
                om = self._solve(self.pmats[i], rhs).real
                self.om23[i, k] = om
                self.psi23[i, k] = self._psi_from_om(i, om).real
            t2, b2 = self._bc_sums(self.psi23[i, 0])
            t3, b3 = self._bc_sums(self.psi23[i, 1])
            det = t2 * b3 - t3 * b2
            self.infl[i] = [[b3 / det, -t3 / det], [-b2 / det, t2 / det]]

    @staticmethod
    def _solve(lu_fac, rhs):
        if isinstance(lu_fac[0], BorderedLU):
            return lu_fac[0].solve(rhs * lu_fac[1])
        (lu, piv), fac = lu_fac
        b = rhs * fac
        if np.iscomplexobj(lu):
            return sla.lu_solve((lu, piv), b)
        return sla.lu_solve((lu, piv), b.real.copy()) + 1j * sla.lu_solve((lu, piv), b.imag.copy())

    # -- start fields (init_fields.f90:73-91, :207-220, :243-251) ------------
    def psi_from_us(self):
        """psi(m > 0) from u_s after a checkpoint read (init_fields.f90:73-91)."""
        pz = self.pz
        psi = np.zeros_like(pz.us)
        r = pz.r
        h2 = np.ones(pz.N) if pz.d["l_non_rot"] else pz.d["r_cmb"] ** 2 - r * r
        m = pz.mvec
        for i in range(1, pz.M):
            psi[i, 1:] = -1j * r[1:] / float(m[i]) / h2[1:] * pz.us[i, 1:]
        return psi

    def start(self):
        pz, c = self.pz, self.pz.cheb
        pz.temp_hat = c.costf1(pz.temp)
        pz.psi_hat = c.costf1(pz.psi)
        self.temp_rhs_imp(1, True)
        if pz.l_chem:
            pz.xi_hat = c.costf1(pz.xi)
            self.temp_rhs_imp(1, True, "xi")
        self.psi_rhs_imp(1, True)

    # -- explicit terms (mloop.f90:209-226) ----------------------------------
    def finish_explicit(self, dVsT, dVsOm):
        pz, c, d = self.pz, self.pz.cheb, self.pz.d
        ist = pz.ts.istage - 1
        n_max = pz.n_max
        m = pz.mvec[:, None].astype(float)
        r = pz.r
        # finish_exp_temp_int (update_temp_integ.f90:396-469)
        w = c.costf1(dVsT)
        w[:, n_max:] = 0.0
        work = c.get_dr(w, l_dct_in=False)
        e = pz.dTdt.expl[ist]
        if d["l_non_rot"]:
            e = r * e - 1j * m * pz.dtcond * pz.psi
        else:
            h2 = d["r_cmb"] ** 2 - r * r
            e = r * e - 1j * m * (h2 * pz.dtcond + d["tadvz_fac"] * r * pz.tcond) * pz.psi
        e = c.costf1(e - work)
        e[:, n_max:] = 0.0
        pz.dTdt.expl[ist] = e @ self.ops.i2r1.T
        if pz.l_chem:
            # finish_exp_xi_int (update_xi_integ.f90:280-357): no tadvz term
            w = c.costf1(pz._dVsXi)
            w[:, n_max:] = 0.0
            work = c.get_dr(w, l_dct_in=False)
            e = pz.dxidt.expl[ist]
            if d["l_non_rot"]:
                e = r * e - 1j * m * pz.dxicond * pz.psi
            else:
                e = r * e - 1j * m * (d["r_cmb"] ** 2 - r * r) * pz.dxicond * pz.psi
            e = c.costf1(e - work)
            e[:, n_max:] = 0.0
            pz.dxidt.expl[ist] = e @ self.ops.i2r1.T
        w = c.costf1(dVsOm)
        w[:, n_max:] = 0.0
        work = c.get_dr(w, l_dct_in=False)
        e = pz.dpsidt.expl[ist].copy()
        nz = slice(1, None)
        if self.dmat:
            # finish_exp_psi_int_dmat (update_psi_integ_dmat.f90:486-623)
            e[nz] = e[nz] - pz.or1 * work[nz]
            if not d["l_non_rot"]:
                e[nz] = e[nz] - d["CorFac"] * 1j * m[nz] * pz.psi[nz]
            if not d["l_buo_imp"]:
                e[nz] = e[nz] - d["BuoFac"] * pz.rgrav * pz.or1 * 1j * m[nz] * pz.temp[nz]
                if pz.l_chem:
                    e[nz] = e[nz] - d["ChemFac"] * pz.rgrav * pz.or1 * 1j * m[nz] * pz.xi[nz]
            if pz.p.l_ek_pump:
                ekp = d["CorFac"] * pz.ekpump
                e[0] = e[0] - ekp * pz.up[0]
                e[nz] = e[nz] - ekp * (pz.om[nz] + pz.ekp_up * pz.up[nz]
                                       + (1j * m[nz] * pz.ekp_dusdp + pz.ekp_us) * pz.us[nz])
            e = c.costf1(e)
            e[:, n_max:] = 0.0
            pz.dpsidt.expl[ist] = e @ self.ops.i2r2.T
            return
        # finish_exp_psi_int_smat (update_psi_integ_smat.f90:793-958)
        e[nz] = r * e[nz]
        if not d["l_coriolis_imp"]:
            e[nz] = e[nz] - d["CorFac"] * 1j * m[nz] * r * pz.psi[nz]
        if not d["l_buo_imp"]:
            e[nz] = e[nz] - d["BuoFac"] * pz.rgrav * 1j * m[nz] * pz.temp[nz]
            if pz.l_chem:
                e[nz] = e[nz] - d["ChemFac"] * pz.rgrav * 1j * m[nz] * pz.xi[nz]
        if pz.p.l_ek_pump:
            ekp = d["CorFac"] * pz.ekpump
            e[0] = e[0] - ekp * pz.up[0]
            e[nz] = e[nz] - ekp * r * (pz.om[nz] + pz.ekp_up * pz.up[nz]
                                        + (1j * m[nz] * pz.ekp_dusdp + pz.ekp_us) * pz.us[nz])
        e[nz] = e[nz] - work[nz]
        e = c.costf1(e)
        e[:, n_max:] = 0.0
        out = np.empty_like(e)
        out[0] = self.ops.i2r2 @ e[0]
        out[nz] = e[nz] @ self.ops.i4r3.T
        pz.dpsidt.expl[ist] = out

    # -- implicit terms ------------------------------------------------------
    def temp_rhs_imp(self, istage, l_calc_lin, kind="temp"):
        """get_temp_rhs_imp_int (update_temp_integ.f90:471-536) or
        get_xi_rhs_imp_int (update_xi_integ.f90:449-510)."""
        pz = self.pz
        _, _, ta, diff = pz._sc(kind)[:4]
        th = pz.temp_hat if kind == "temp" else pz.xi_hat
        if istage == 1:
            ta.old[istage - 1] = th @ self.ops.i2r2.T
        if l_calc_lin:
            imp = np.empty_like(th)
            for i in range(pz.M):
                imp[i] = diff * pz.hdif[i] * (self.t_rhsi[i] @ th[i])
            ta.impl[istage - 1] = imp

    def _buo_coeffs(self, xi=None):
        """I4 r^4 (I2 r^2 with the influence-matrix variant) of the buoyancy
        -BuoFac rgrav/r i m T - ChemFac rgrav/r i m xi, m > 0, in Chebyshev
        space (update_psi_integ_smat.f90:266-330, :1075-1111;
        update_psi_integ_dmat.f90:171-240, :748-779).  ``xi`` replaces the
        composition field (the bridge step passes psi there)."""
        pz, d = self.pz, self.pz.d
        m = pz.mvec[:, None].astype(float)
        buo = -d["BuoFac"] * pz.rgrav * pz.or1 * 1j * m * pz.temp
        if pz.l_chem:
            buo = buo - d["ChemFac"] * pz.rgrav * pz.or1 * 1j * m * (pz.xi if xi is None else xi)
        buo[0] = 0.0
        buo = pz.cheb.costf1(buo)
        out = buo @ (self.ops.i2r2 if self.dmat else self.ops.i4r4).T
        out[0] = 0.0
        return out

    def psi_rhs_imp(self, istage, l_calc_lin, xi=None):
        """get_psi_rhs_imp_int_smat (update_psi_integ_smat.f90:960-1115) or
        get_psi_rhs_imp_int_dmat (update_psi_integ_dmat.f90:625-781), which
        works on omega (u_phi for m = 0) instead of psi_hat."""
        pz, d = self.pz, self.pz.d
        if self.dmat:
            work = pz.om.copy()
            work[0] = pz.up[0]
            src = pz.cheb.costf1(work)
        else:
            work_r = pz.cheb.costf1_real(pz.up[0].real)
            src = pz.psi_hat.copy()
            src[0] = work_r
        if istage == 1:
            old = np.empty_like(src)
            for i in range(pz.M):
                old[i] = self.p_rhsi[i] @ src[i]
            pz.dpsidt.old[istage - 1] = old
        if l_calc_lin:
            imp = np.empty_like(src)
            for i in range(pz.M):
                imp[i] = self.p_rhsil[i] @ src[i]
            if d["l_buo_imp"]:
                imp = imp + self._buo_coeffs(xi)
            pz.dpsidt.impl[istage - 1] = imp

    # -- solves (mloop.f90:84-100) -------------------------------------------
    def update_temp(self, l_log_next, kind="temp"):
        """update_temp_int (update_temp_integ.f90:179-298) or update_xi_int
        (update_xi_integ.f90:167-278)."""
        pz, ts, c = self.pz, self.pz.ts, self.pz.cheb
        f, df, ta, _, top, bot = pz._sc(kind)[:6]
        mats = self.tmats if kind == "temp" else self.ximats
        work = ts.set_imex_rhs(ta)
        th = np.empty_like(work)
        for i in range(pz.M):
            rhs = work[i].copy()
            rhs[0] = top[i]
            rhs[1] = bot[i]
            th[i] = self._solve(mats[i], rhs)
        setattr(pz, f + "_hat", th)
        setattr(pz, f, c.costf1(th))
        ts.rotate_imex(ta)
        if ts.istage == ts.nstages:
            self.temp_rhs_imp(1, pz._calc_rhs(1), kind)
        else:
            self.temp_rhs_imp(ts.istage + 1, pz._calc_rhs(ts.istage + 1), kind)
        if l_log_next:
            setattr(pz, df, c.get_dr(getattr(pz, f)))

    def update_psi(self):
        """update_psi_int_smat (update_psi_integ_smat.f90:247-573)."""
        if self.dmat:
            return self._update_psi_dmat()
        pz, ts, c, d = self.pz, self.pz.ts, self.pz.cheb, self.pz.d
        N, M = pz.N, pz.M
        buo = self._buo_coeffs() if d["l_buo_imp"] else None
        work = ts.set_imex_rhs(pz.dpsidt)
        if buo is not None:
            work[1:] = work[1:] + ts.wimp_lin[0] * buo[1:]
        uphi0 = self._solve(self.pmats[0], work[0]).real
        psi_hat = pz.psi_hat.copy()
        for i in range(1, M):
            psi_hat[i] = self._solve(self.pmats[i], work[i])
        pz.psi_hat = psi_hat
        psi = pz.psi.copy()
        psi[1:] = psi_hat[1:]
        om0 = c.get_dr_real(uphi0, l_dct=False)
        uphi0 = c.costf1_real(uphi0)
        dpsi, d2psi = c.get_ddr(psi, l_dct=False)
        psi = c.costf1(psi)
        r, or1, or2 = pz.r, pz.or1, pz.or2
        m = pz.mvec[:, None].astype(float)
        if d["l_non_rot"]:
            us = 1j * m * or1 * psi
            up = -dpsi
            om = -d2psi - or1 * dpsi + m * m * or2 * psi
        else:
            h2 = d["r_cmb"] ** 2 - r * r
            us = 1j * m * or1 * h2 * psi
            up = -h2 * dpsi + 3.0 * r * psi
            om = (-h2 * d2psi - (d["r_cmb"] ** 2 * or1 - 6.0 * r) * dpsi
                  + (6.0 + m * m * or2 * h2) * psi)
        us[0] = 0.0
        up[0] = uphi0
        om[0] = om0 + or1 * uphi0
        pz.psi, pz.us, pz.up, pz.om = psi, us, up, om
        ts.rotate_imex(pz.dpsidt)
        if ts.istage == ts.nstages:
            self.psi_rhs_imp(1, pz._calc_rhs(1))
        else:
            self.psi_rhs_imp(ts.istage + 1, pz._calc_rhs(ts.istage + 1))

    def _update_psi_dmat(self):
        """update_psi_int_dmat (update_psi_integ_dmat.f90:150-484): omega from
        its own solve with omega = 0 on the walls, psi from omega, then the
        influence-matrix combination of the two homogeneous solutions that
        imposes the remaining wall conditions on psi."""
        pz, ts, c, d = self.pz, self.pz.ts, self.pz.cheb, self.pz.d
        M = pz.M
        buo = self._buo_coeffs() if d["l_buo_imp"] else None
        work = ts.set_imex_rhs(pz.dpsidt)
        if buo is not None:
            work[1:] = work[1:] + ts.wimp_lin[0] * buo[1:]
        uphi0 = self._solve(self.pmats[0], work[0]).real
        om_hat = np.zeros_like(work)
        psi_hat = np.zeros_like(work)
        for i in range(1, M):
            om_hat[i] = self._solve(self.pmats[i], work[i])
            psi_hat[i] = self._psi_from_om(i, om_hat[i])
            t1, b1 = self._bc_sums(psi_hat[i])
            inf = self.infl[i]
            c1 = -inf[0, 0] * t1 - inf[0, 1] * b1
            c2 = -inf[1, 0] * t1 - inf[1, 1] * b1
            psi_hat[i] = psi_hat[i] + c1 * self.psi23[i, 0] + c2 * self.psi23[i, 1]
            om_hat[i] = om_hat[i] + c1 * self.om23[i, 0] + c2 * self.om23[i, 1]
        om0 = c.get_dr_real(uphi0, l_dct=False)
        uphi0 = c.costf1_real(uphi0)
        dpsi = c.get_dr(psi_hat, l_dct_in=False)
        psi = c.costf1(psi_hat)
        om = c.costf1(om_hat)
        r, or1 = pz.r, pz.or1
        m = pz.mvec[:, None].astype(float)
        if d["l_non_rot"]:
            us = 1j * m * or1 * psi
            up = -dpsi
        else:
            h2 = d["r_cmb"] ** 2 - r * r
            us = 1j * m * or1 * h2 * psi
            up = -h2 * dpsi + 3.0 * r * psi
        psi[0] = 0.0
        us[0] = 0.0
        up[0] = uphi0
        om[0] = om0 + or1 * uphi0
        pz.psi_hat = psi_hat
        pz.psi, pz.us, pz.up, pz.om = psi, us, up, om
        ts.rotate_imex(pz.dpsidt)
        if ts.istage == ts.nstages:
            self.psi_rhs_imp(1, pz._calc_rhs(1))
        else:
            self.psi_rhs_imp(ts.istage + 1, pz._calc_rhs(ts.istage + 1))

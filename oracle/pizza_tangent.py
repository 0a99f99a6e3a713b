"""Tangent-linear and adjoint restatement of the CNAB2 influence-matrix step
(test infrastructure: the checker of the GPU adjoint, never the product).

pizza has no adjoint.  This module writes the oracle's step
(oracle.pizza_oracle.Pizza, CNAB2, matrix_solve='INFLUENCE', implicit
buoyancy) as a map of the Chebyshev-coefficient state
S = (Tc, oc, pc, uc) plus the previous explicit terms E = (eT, eP), using the
oracle's own matrix builders, and gives, for a fixed time-step sequence:

* ``forward``: the objective J = mean over a window of states of
  us2_3D + up2_3D + uz2_3D (the e_kin_3D sums of src/outputs.f90:553-570);
* ``tangent``: dJ along (dT0, dRa) -- the tangent-linear run.  The nonlinear
  terms and the kinetic energy are homogeneous quadratic forms q, so their
  tangent is exact by polarisation, q'(f) df = (q(f + df) - q(f - df)) / 2;
  everything else is linear;
* ``adjoint``: the gradient (dJ/dT0, dJ/dRa) by the reverse sweep.

The dot test <tangent(d), 1> = Re<adjoint, d> checks the two against each
other; both are checked against central finite differences of ``forward``.
The S-form forward itself agrees with Pizza.advance to rounding.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

from oracle.pizza_oracle import Params, Pizza


def _inv(lu_piv):
    lu, piv = lu_piv
    return sla.lu_solve((lu, piv), np.eye(lu.shape[0]))


class StepOps:
    """Dense operators of one instance (from the oracle's builders)."""

    def __init__(self, p: Params):
        z = Pizza(p)
        if z.l_direct or z.ts.time_scheme != "CNAB2" or not z.d["l_buo_imp"]:
            raise ValueError("the tangent restatement covers CNAB2, INFLUENCE, implicit buoyancy")
        self.z = z
        self.N, self.M, self.P = z.N, z.M, z.P
        N = self.N
        c, d = z.cheb, z.d
        self.d = d
        j = np.arange(N)
        w = np.full(N, 2.0)
        w[0] = w[-1] = 1.0
        self.C = c.cheb_fac * w[None, :] * np.cos(np.pi * np.outer(j, j) / (N - 1))
        bf = np.ones(N)
        bf[0] = bf[-1] = 0.5
        self.D1c = c.rnorm * c.drMat * bf[None, :]
        self.D2c = c.rnorm * c.d2rMat * bf[None, :]
        self.D1p = self.D1c @ self.C
        self.m = z.mvec.astype(float)
        self.r, self.or1, self.or2, self.beta = z.r, z.or1, z.or2, z.beta
        self.rgrav, self.ekpump = z.rgrav, z.ekpump
        self.eup, self.eus, self.edp = z.ekp_up, z.ekp_us, z.ekp_dusdp
        self.h = z.height
        self.gT = z.dtcond - d["tadvz_fac"] * z.beta * z.tcond
        self.l_ek_pump = p.l_ek_pump
        # rInt_R weights (integration.f90:18-55) as a linear functional
        q = np.zeros(N)
        q[0] = 0.5
        for nc in range(3, N + 1, 2):
            q[nc - 1] = -1.0 / (nc * (nc - 2))
        if (N - 1) % 2 == 0:
            q[N - 1] *= 0.5
        drx = 2.0 / (d["r_cmb"] - d["r_icb"])
        self.wint = 2.0 * math.sqrt(2.0 / (N - 1)) * (q @ self.C) / drx
        self.bct = c.rnorm * bf * c.drMat[0]
        self.bcb = c.rnorm * bf * c.drMat[N - 1]
        self.pr = p.pr
        self.K = np.zeros((self.M, N, N))
        Pint = np.eye(N)
        Pint[0, 0] = Pint[-1, -1] = 0.0
        for i in range(1, self.M):
            lu_piv, f1, f2 = z._psi_mat_dmat(int(self.m[i]))
            G = (f2[:, None] * _inv(lu_piv)) * f1[None, :]
            self.K[i] = G @ Pint @ self.C
        self.wl0 = None

    def build(self, wl0):
        """dt-dependent operators for wimp_lin(1) = wl0."""
        if self.wl0 == wl0:
            return
        z = self.z
        z.ts.wimp_lin[0] = wl0
        N, M = self.N, self.M
        self.GT = np.zeros((M, N, N))
        self.Gom = np.zeros((M, N, N))
        for i in range(M):
            lu_piv, fac = z._temp_mat(int(self.m[i]))
            self.GT[i] = _inv(lu_piv) * fac[None, :]
        self.Guphi = _inv(z._uphi_mat())
        self.om2 = np.zeros((M, N)); self.om3 = np.zeros((M, N))
        self.psi2 = np.zeros((M, N)); self.psi3 = np.zeros((M, N))
        self.infl = np.zeros((M, 4))
        for i in range(1, M):
            lu_piv, f1, f2 = z._om_mat(int(self.m[i]))
            G = (f2[:, None] * _inv(lu_piv)) * f1[None, :]
            self.Gom[i] = G
            self.om2[i], self.om3[i] = G[:, N - 1], G[:, 0]
            self.psi2[i] = -self.K[i] @ self.om2[i]
            self.psi3[i] = -self.K[i] @ self.om3[i]
            t2, t3 = self.bct @ self.psi2[i], self.bct @ self.psi3[i]
            b2, b3 = self.bcb @ self.psi2[i], self.bcb @ self.psi3[i]
            det = t2 * b3 - t3 * b2
            self.infl[i] = [b3 / det, -t3 / det, -b2 / det, t2 / det]
        self.wl0 = wl0


def cnab2_weights(dt, dt_prev, alpha=0.5):
    """(wimp, wimp_lin(1), wimp_lin(2), wexp(1), wexp(2)) of CNAB2
    (multistep_schemes.f90:160-166)."""
    return (1.0, alpha * dt, (1.0 - alpha) * dt, (1.0 + 0.5 * dt / dt_prev) * dt, -0.5 * dt * dt / dt_prev)


# ---------------------------------------------------------------------------
# the step in state form
# ---------------------------------------------------------------------------
def fields(o: StepOps, S, B):
    """Physical fields and implicit terms of the state (get_*_rhs_imp_coll)."""
    Tc, oc, pc, uc = S
    d = o.d
    m = o.m[:, None]
    T = Tc @ o.C.T
    iT = d["TdiffFac"] * (Tc @ o.D2c.T + o.or1 * (Tc @ o.D1c.T) - m ** 2 * o.or2 * T)
    om = oc @ o.C.T
    iP = (d["ViscFac"] * (oc @ o.D2c.T + o.or1 * (oc @ o.D1c.T) - m ** 2 * o.or2 * om)
          - B * o.rgrav * o.or1 * 1j * m * T)
    psi = pc @ o.C.T
    us = 1j * m * o.or1 * psi
    up = -(pc @ o.D1c.T) - o.beta * psi
    u0 = uc @ o.C.T
    us[0] = 0.0
    up[0] = u0
    om[0] = uc @ o.D1c.T + o.or1 * u0
    iP[0] = d["ViscFac"] * (uc @ o.D2c.T + o.or1 * (uc @ o.D1c.T) - o.or2 * u0) - d["CorFac"] * o.ekpump * u0
    oldP = om.copy()
    oldP[0] = up[0]
    return dict(T=T, iT=iT, om=om, iP=iP, us=us, up=up, oldP=oldP)


def nl(o: StepOps, f):
    """radial_loop (radial_loop.f90:231-394): a homogeneous quadratic form of
    the fields."""
    P, M, d = o.P, o.M, o.d

    def ifft(s):
        t = np.zeros(s.shape[:-1] + (P // 2 + 1,), complex)
        t[..., :M] = s
        t[..., 0] = t[..., 0].real
        return np.fft.irfft(t, n=P, axis=-1) * P

    def fft(g):
        return np.fft.rfft(g, axis=-1)[..., :M] / P

    us, up, om, T = f["us"].T, f["up"].T, f["om"].T, f["T"].T
    r, or1 = o.r[:, None], o.or1[:, None]
    usg, upg, omg, Tg = ifft(us), ifft(up), ifft(om), ifft(T)
    A, Bp, Cc, D = fft(r * usg * Tg), fft(upg * Tg), fft(r * usg * omg), fft(upg * omg)
    m = o.m[None, :]
    tfac = ((1.0 - d["tadvz_fac"]) * o.beta * o.or1)[:, None]
    ET = -or1 * 1j * m * Bp - tfac * A
    EP = -or1 * 1j * m * D
    usf = us.copy()
    usf[:, 0] = 0.5 * d["ek"] * d["CorFac"] * o.ekpump * up[:, 0].real
    prod = 2.0 * (usf.real * om.real + usf.imag * om.imag)
    prod[:, 0] = usf[:, 0].real * om[:, 0].real
    EP[:, 0] = -prod.sum(axis=1)
    return ET.T, A.T, EP.T, Cc.T


def fin(o: StepOps, f, ET, VT, EP, VOm):
    """finish_exp_temp_coll and finish_exp_psi_coll_dmat (linear)."""
    d = o.d
    m = o.m[:, None]
    eT = ET - o.or1 * (VT @ o.D1p.T) - f["us"] * o.gT
    eP = EP.copy()
    nz = slice(1, None)
    e = EP[nz] - o.or1 * (VOm[nz] @ o.D1p.T)
    if not d["l_non_rot"]:
        e = e + d["CorFac"] * o.beta * f["us"][nz]
    if o.l_ek_pump:
        e = e - d["CorFac"] * o.ekpump * (f["om"][nz] + o.eup * f["up"][nz]
                                          + (o.edp * 1j * m[nz] + o.eus) * f["us"][nz])
    eP[nz] = e
    return eT, eP


def solve(o: StepOps, f, eT, eP, eTp, ePp, w, B, Tn_extra=None):
    """update_temp_co and update_om_coll_dmat on the state.  The buoyancy of
    the new temperature is B * Tn; ``Tn_extra`` = (dB, Tn_base) adds
    dB * Tn_base (the tangent of B in that term)."""
    w0, wl0, wl1, we0, we1 = w
    N = o.N
    rT = w0 * f["T"] + wl1 * f["iT"] + we0 * eT + we1 * eTp
    rT[:, 0] = 0
    rT[:, N - 1] = 0
    Tc = np.einsum("mij,mj->mi", o.GT, rT)
    Tn = Tc @ o.C.T
    m = o.m[:, None]
    rP = w0 * f["oldP"] + wl1 * f["iP"] + we0 * eP + we1 * ePp
    buo = B * Tn
    if Tn_extra is not None:
        buo = buo + Tn_extra[0] * Tn_extra[1]
    rP[1:] = rP[1:] - wl0 * o.rgrav * o.or1 * 1j * m[1:] * buo[1:]
    rP[:, 0] = 0
    rP[:, N - 1] = 0
    uc = o.Guphi @ rP[0].real
    oc = np.einsum("mij,mj->mi", o.Gom, rP)
    pc = -np.einsum("mij,mj->mi", o.K, oc)
    tt, tb = pc @ o.bct, pc @ o.bcb
    c1 = -o.infl[:, 0] * tt - o.infl[:, 1] * tb
    c2 = -o.infl[:, 2] * tt - o.infl[:, 3] * tb
    pc = pc + c1[:, None] * o.psi2 + c2[:, None] * o.psi3
    oc = oc + c1[:, None] * o.om2 + c2[:, None] * o.om3
    oc[0] = 0
    pc[0] = 0
    return (Tc, oc, pc, uc), Tn


def ke3d(o: StepOps, f):
    """us2_3D + up2_3D + uz2_3D (outputs.f90:553-570): a quadratic form."""
    a_us = 2.0 * (f["us"].real ** 2 + f["us"].imag ** 2)
    a_us[0] = f["us"][0].real ** 2
    a_up = 2.0 * (f["up"].real ** 2 + f["up"].imag ** 2)
    a_up[0] = f["up"][0].real ** 2
    us2, up2 = a_us.sum(0), a_up.sum(0)
    r, h, be = o.r, o.h, o.beta
    return np.pi * (o.wint @ (us2 * r * h) + o.wint @ (up2 * r * h) + o.wint @ (us2 * be ** 2 * r * h ** 3 / 12.0))


def _polar(q, x, dx):
    """Tangent of a homogeneous quadratic form q at x along dx."""
    def comb(s):
        if isinstance(x, dict):
            return {k: x[k] + s * dx[k] for k in x}
        return x + s * dx
    qa, qb = q(comb(1.0)), q(comb(-1.0))
    if isinstance(qa, tuple):
        return tuple(0.5 * (a - b) for a, b in zip(qa, qb))
    return 0.5 * (qa - qb)


def _zero_state(o):
    z = np.zeros((o.M, o.N), complex)
    return (z.copy(), z.copy(), z.copy(), np.zeros(o.N))


def _weights(dts, n):
    return cnab2_weights(dts[n], dts[n - 1] if n > 0 else dts[0])


def forward(o: StepOps, T0, dts, ra, window):
    """J and the trajectory (S_n, E_{n-1}, weights) of len(dts) steps."""
    B = ra / o.pr
    M, N = o.M, o.N
    S = (T0 @ o.C.T, np.zeros((M, N), complex), np.zeros((M, N), complex), np.zeros(N))
    E = (np.zeros((M, N), complex), np.zeros((M, N), complex))
    traj, J = [], 0.0
    for n in range(len(dts)):
        w = _weights(dts, n)
        o.build(w[1])
        traj.append((S, E, w))
        f = fields(o, S, B)
        eT, eP = fin(o, f, *nl(o, f))
        S, _ = solve(o, f, eT, eP, E[0], E[1], w, B)
        E = (eT, eP)
        if n + 1 in window:
            J += ke3d(o, fields(o, S, B)) / len(window)
    return J, traj, S


def tangent(o: StepOps, T0, dT0, dts, ra, dra, window):
    """(J, dJ) along (dT0, dra): the tangent-linear run."""
    B, dB = ra / o.pr, dra / o.pr
    M, N = o.M, o.N
    S = (T0 @ o.C.T, np.zeros((M, N), complex), np.zeros((M, N), complex), np.zeros(N))
    dS = (dT0 @ o.C.T, np.zeros((M, N), complex), np.zeros((M, N), complex), np.zeros(N))
    E = (np.zeros((M, N), complex), np.zeros((M, N), complex))
    dE = (np.zeros((M, N), complex), np.zeros((M, N), complex))
    J = dJ = 0.0
    m = o.m[:, None]
    for n in range(len(dts)):
        w = _weights(dts, n)
        o.build(w[1])
        f = fields(o, S, B)
        df = fields(o, dS, B)
        df["iP"] = df["iP"] - dB * o.rgrav * o.or1 * 1j * m * f["T"]   # zero at m = 0
        NL = nl(o, f)
        dNL = _polar(lambda g: nl(o, g), f, df)
        eT, eP = fin(o, f, *NL)
        deT, deP = fin(o, df, *dNL)
        Sn, Tn = solve(o, f, eT, eP, E[0], E[1], w, B)
        dSn, _ = solve(o, df, deT, deP, dE[0], dE[1], w, B, Tn_extra=(dB, Tn))
        S, dS, E, dE = Sn, dSn, (eT, eP), (deT, deP)
        if n + 1 in window:
            fS, dfS = fields(o, S, B), fields(o, dS, B)
            J += ke3d(o, fS) / len(window)
            dJ += _polar(lambda g: ke3d(o, g), fS, dfS) / len(window)
    return J, dJ


# ---------------------------------------------------------------------------
# reverse sweep: transposes of solve, fin, nl and fields (x_bar = conj(a) y_bar
# for y = a x; gradients g with dJ = Re sum conj(g) dz)
# ---------------------------------------------------------------------------
def _solve_adj(o, Sb, w, B, carry):
    w0, wl0, wl1, we0, we1 = w
    N, M = o.N, o.M
    m = o.m[:, None]
    Tcb = np.array(Sb[0], complex)
    ocb = np.array(Sb[1], complex)
    pcb = np.array(Sb[2], complex)
    ucb = np.array(Sb[3], float)
    ocb[0] = 0
    pcb[0] = 0
    c1b = (o.psi2 * pcb).sum(1) + (o.om2 * ocb).sum(1)
    c2b = (o.psi3 * pcb).sum(1) + (o.om3 * ocb).sum(1)
    ttb = -o.infl[:, 0] * c1b - o.infl[:, 2] * c2b
    tbb = -o.infl[:, 1] * c1b - o.infl[:, 3] * c2b
    pcub = pcb + ttb[:, None] * o.bct + tbb[:, None] * o.bcb
    ocub = ocb - np.einsum("mji,mj->mi", o.K, pcub)
    rPb = np.einsum("mji,mj->mi", o.Gom, ocub)
    rPb[0] = o.Guphi.T @ ucb
    rPb[:, 0] = 0
    rPb[:, N - 1] = 0
    Tnb = np.zeros((M, N), complex)
    Tnb[1:] = (wl0 * B * o.rgrav * o.or1) * 1j * m[1:] * rPb[1:]
    Tcb = Tcb + Tnb @ o.C
    rTb = np.einsum("mji,mj->mi", o.GT, Tcb)
    rTb[:, 0] = 0
    rTb[:, N - 1] = 0
    out = dict(T=w0 * rTb, iT=wl1 * rTb, oldP=w0 * rPb, iP=wl1 * rPb,
               eT=we0 * rTb + carry[0], eP=we0 * rPb + carry[1])
    return out, (we1 * rTb, we1 * rPb), rPb


def _fin_adj(o, eTb, ePb):
    d = o.d
    m = o.m[:, None]
    VTb = (-o.or1 * eTb) @ o.D1p
    usb = -o.gT * eTb
    VOmb = np.zeros_like(ePb)
    omb = np.zeros_like(ePb)
    upb = np.zeros_like(ePb)
    nz = slice(1, None)
    VOmb[nz] = (-o.or1 * ePb[nz]) @ o.D1p
    if not d["l_non_rot"]:
        usb[nz] += d["CorFac"] * o.beta * ePb[nz]
    if o.l_ek_pump:
        ce = d["CorFac"] * o.ekpump
        usb[nz] += -ce * np.conj(o.edp * 1j * m[nz] + o.eus) * ePb[nz]
        omb[nz] += -ce * ePb[nz]
        upb[nz] += -ce * o.eup * ePb[nz]
    return eTb.copy(), VTb, ePb.copy(), VOmb, usb, upb, omb


def _nl_adj(o, f, ETb, VTb, EPb, VOmb):
    P, M, d = o.P, o.M, o.d

    def ifft(s):
        t = np.zeros(s.shape[:-1] + (P // 2 + 1,), complex)
        t[..., :M] = s
        t[..., 0] = t[..., 0].real
        return np.fft.irfft(t, n=P, axis=-1) * P

    def fft_adj(Sb):
        t = np.zeros(Sb.shape[:-1] + (P,), complex)
        t[..., :M] = Sb
        return np.fft.ifft(t, axis=-1).real

    def ifft_adj(gb):
        F = np.fft.fft(gb, axis=-1)[..., :M]
        out = 2.0 * F
        out[..., 0] = F[..., 0].real
        return out

    us, up, om, T = f["us"].T, f["up"].T, f["om"].T, f["T"].T
    r, or1, m = o.r[:, None], o.or1[:, None], o.m[None, :]
    usg, upg, omg, Tg = ifft(us), ifft(up), ifft(om), ifft(T)
    tfac = ((1.0 - d["tadvz_fac"]) * o.beta * o.or1)[:, None]
    ETb, VTb, EPb, VOmb = ETb.T, VTb.T, EPb.T, VOmb.T
    Db = or1 * 1j * m * EPb
    Db[:, 0] = 0
    ab, bb = fft_adj(VTb - tfac * ETb), fft_adj(or1 * 1j * m * ETb)
    cb, db = fft_adj(VOmb), fft_adj(Db)
    usb = ifft_adj(r * Tg * ab + r * omg * cb)
    upb = ifft_adj(Tg * bb + omg * db)
    omb = ifft_adj(r * usg * cb + upg * db)
    Tb = ifft_adj(r * usg * ab + upg * bb)
    EP0 = EPb[:, 0].real
    usb[:, 1:] += -2.0 * EP0[:, None] * om[:, 1:]
    omb[:, 1:] += -2.0 * EP0[:, None] * us[:, 1:]
    fek = 0.5 * d["ek"] * d["CorFac"] * o.ekpump
    upb[:, 0] += -EP0 * fek * om[:, 0].real
    omb[:, 0] += -EP0 * fek * up[:, 0].real
    return usb.T, upb.T, omb.T, Tb.T


def _lin_adj(o, f, Tb, iTb, omb, iPb, usb, upb, oldPb, B):
    d = o.d
    m = o.m[:, None]
    TdF, Vis = d["TdiffFac"], d["ViscFac"]
    omb = omb.copy()
    upb = upb.copy()
    omb[1:] += oldPb[1:]
    upb[0] += oldPb[0]
    Tt = Tb + TdF * (-m ** 2 * o.or2 * iTb)
    Tt[1:] += np.conj(-B * o.rgrav * o.or1 * 1j * m[1:]) * iPb[1:]
    dB = np.sum((np.conj(iPb[1:]) * (-o.rgrav * o.or1 * 1j * m[1:] * f["T"][1:])).real)
    Tcb = Tt @ o.C + TdF * (iTb @ o.D2c + (o.or1 * iTb) @ o.D1c)
    omt = omb + Vis * (-m ** 2 * o.or2 * iPb)
    ocb = omt @ o.C + Vis * (iPb @ o.D2c + (o.or1 * iPb) @ o.D1c)
    psib = np.conj(1j * m * o.or1) * usb - o.beta * upb
    pcb = psib @ o.C - upb @ o.D1c
    ocb[0] = 0
    pcb[0] = 0
    u0b = upb[0].real + o.or1 * omb[0].real + (-Vis * o.or2 - d["CorFac"] * o.ekpump) * iPb[0].real
    ucb = u0b @ o.C + omb[0].real @ o.D1c + Vis * (iPb[0].real @ o.D2c + (o.or1 * iPb[0].real) @ o.D1c)
    return (Tcb, ocb, pcb, ucb), dB


def _ke_grad(o, f, scale):
    r, h, be = o.r, o.h, o.beta
    W1 = np.pi * o.wint * (r * h + be ** 2 * r * h ** 3 / 12.0) * scale
    W2 = np.pi * o.wint * (r * h) * scale
    usb = 4.0 * W1 * f["us"]
    usb[0] = 2.0 * W1 * f["us"][0].real
    upb = 4.0 * W2 * f["up"]
    upb[0] = 2.0 * W2 * f["up"][0].real
    return usb, upb


def adjoint(o: StepOps, T0, dts, ra, window):
    """(J, dJ/dtemp0, dJ/dRa) for the fixed step sequence dts."""
    B = ra / o.pr
    J, traj, S_final = forward(o, T0, dts, ra, window)
    M, N = o.M, o.N
    nst = len(dts)
    z = np.zeros((M, N), complex)
    Sb = (z.copy(), z.copy(), z.copy(), np.zeros(N))
    dB = 0.0
    inv_w = 1.0 / len(window) if len(window) else 0.0
    if nst in window:
        usb, upb = _ke_grad(o, fields(o, S_final, B), inv_w)
        Sb, _ = _lin_adj(o, fields(o, S_final, B), z, z, z, z, usb, upb, z, B)
    carry = (z.copy(), z.copy())
    states = [t[0] for t in traj] + [S_final]
    for n in range(nst - 1, -1, -1):
        S, E, w = traj[n]
        o.build(w[1])
        f = fields(o, S, B)
        fa, carry, rPb = _solve_adj(o, Sb, w, B, carry)
        Tn = states[n + 1][0] @ o.C.T
        dB += np.sum((np.conj(rPb[1:]) * (-w[1] * o.rgrav * o.or1 * 1j * o.m[1:, None] * Tn[1:])).real)
        ETb, VTb, EPb, VOmb, usb, upb, omb = _fin_adj(o, fa["eT"], fa["eP"])
        a_us, a_up, a_om, a_T = _nl_adj(o, f, ETb, VTb, EPb, VOmb)
        usb, upb, omb = usb + a_us, upb + a_up, omb + a_om
        if n in window:
            gs, gp = _ke_grad(o, f, inv_w)
            usb, upb = usb + gs, upb + gp
        Sb, db = _lin_adj(o, f, fa["T"] + a_T, fa["iT"], omb, fa["iP"], usb, upb, fa["oldP"], B)
        dB += db
    return J, Sb[0] @ o.C, dB / o.pr

"""pizza's files on the host side of the GPU step: the time series it writes
(e_kin.TAG, e_kin_3D.TAG, heat.TAG; src/outputs.f90:677-793) and its
version-7 checkpoints (src/checkpoints.f90:33-183 write, :185-860 read).

A run on the GPU can therefore leave the same text series a pizza.exe run
leaves (python/pizza reads them), save a checkpoint pizza.exe can restart
from, and restart from a checkpoint pizza.exe wrote, also onto another
Chebyshev grid, m truncation or multistep scheme, as pizza's reader does
(Chebyshev-to-Chebyshev mapping, the CNAB2 bridge and AB1; finite
differences and polynomial interpolation are not restated).
"""
from __future__ import annotations

import os

import numpy as np

# columns of Ensemble.series rows written to each file
SERIES_FILES = {
    "e_kin": (0, 1, 2, 3),                    # time, us2_2D, up2_2D, up2_axi_2D
    "e_kin_3D": (0, 4, 5, 6, 7),              # time, us2_3D, up2_3D, uz2_3D, up2_axi_3D
    "heat": (0, 8, 9, 10, 11, 12, 13, 14),    # time, NuTop, NuBot, Nu_vol, Nu_int, tTop, tBot, beta_t
    "composition": (0, 16, 17, 18, 19, 20, 21),   # time, ShTop, ShBot, Sh_vol, xiTop, xiBot, beta_xi
}


def fortran_es(x: float, w: int, d: int) -> str:
    """The Fortran ESw.d edit descriptor: one nonzero digit before the point,
    d after it, a two-digit signed exponent after 'E' (three digits replace
    the 'E' when |exponent| >= 100), right-justified in w columns."""
    s = f"{float(x):.{d}E}"
    mant, exp = s.split("E")
    e = int(exp)
    if abs(e) >= 100:
        s = f"{mant}{'+' if e >= 0 else '-'}{abs(e):03d}"
    else:
        s = f"{mant}E{'+' if e >= 0 else '-'}{abs(e):02d}"
    if len(s) > w:
        return "*" * w
    return s.rjust(w)


def format_series_line(values) -> str:
    """'(1P, ES20.12, kES16.8)' as pizza writes its time series."""
    return fortran_es(values[0], 20, 12) + "".join(fortran_es(v, 16, 8) for v in values[1:])


def format_spectrum_lines(spec, minc: int = 1):
    """spec_N.TAG lines of write_spectra (src/spectra.f90:306-369): for each
    m, '(I5, 5ES16.8)' of m and the round_off'ed us2, up2, enstrophy, T^2 and
    composition spectra.  spec: (n_m_max, 5) array, or (n_m_max, 4) without
    the composition column (written as zero)."""
    lines = []
    for mi, row in enumerate(np.asarray(spec, float)):
        vals = [_round_off(v) for v in row] + [0.0] * (5 - len(row))
        lines.append(f"{mi * minc:5d}" + "".join(fortran_es(v, 16, 8) for v in vals))
    return lines


def _round_off(x):
    """round_off (src/useful.f90:222-233): |x| < 10 epsilon -> 0."""
    return 0.0 if abs(x) < 10.0 * np.finfo(float).eps else float(x)


def write_spectrum(ens, i: int, counter: int, tag: str, directory: str = "."):
    """spec_<counter>.<tag> of instance i from its device spectra."""
    p = os.path.join(directory, f"spec_{counter}.{tag}")
    with open(p, "w") as f:
        for ln in format_spectrum_lines(ens.spectra(i), ens.configs[i].minc):
            f.write(ln + "\n")
    return p


class SpectraAverage:
    """Time-averaged m-spectra (calculate_spectra and write_spectra_avg,
    src/spectra.f90:104-196, :198-304): a running mean and standard deviation
    of the five m-spectra, updated by getMSD2 (src/useful.f90:263-293), the
    recursion for a variable averaging step.  After calls at averaging times
    T_1 < ... < T_n, mean = sum_k dt_k x_k / T_n and SD = sqrt(sum_k dt_k
    (x_k - mean)^2 / T_n), with dt_k = T_k - T_(k-1) and T_0 = 0."""

    def __init__(self, n_m_max: int, minc: int = 1):
        self.mean = np.zeros((n_m_max, 5))
        self.sd = np.zeros((n_m_max, 5))
        self.minc = minc
        self.n_calls = 0
        self.time_last = 0.0

    def update(self, spec, time_avg: float):
        """spec: (n_m_max, 5) snapshot spectra (Ensemble.spectra);
        time_avg: the caller's running sum of dt over its output calls
        (timeAvg_spec, outputs.f90:271-272)."""
        x = np.asarray(spec, float)
        self.n_calls += 1
        dt = time_avg - self.time_last
        if self.n_calls == 1:
            self.mean = x.copy()
            self.sd = np.zeros_like(x)
        else:
            delta = x - self.mean
            self.mean = self.mean + delta * dt / time_avg
            self.sd = self.sd + dt * delta * (x - self.mean)
        self.time_last = time_avg

    def result(self):
        """(mean, SD) arrays, SD normalised as write_spectra_avg does."""
        return self.mean.copy(), np.sqrt(self.sd / self.time_last)

    def lines(self):
        """spec_avg.TAG lines: '(I5, 10es16.8)' of m and the round_off'ed
        mean and SD of us2, up2, enstrophy, T^2 and the composition column."""
        mean, sd = self.result()
        out = []
        for mi in range(mean.shape[0]):
            vals = [_round_off(v) for k in range(5) for v in (mean[mi, k], sd[mi, k])]
            out.append(f"{mi * self.minc:5d}" + "".join(fortran_es(v, 16, 8) for v in vals))
        return out

    def write(self, tag: str, directory: str = "."):
        p = os.path.join(directory, f"spec_avg.{tag}")
        with open(p, "w") as f:
            for ln in self.lines():
                f.write(ln + "\n")
        return p


class Spectra2DAverage:
    """Time-averaged (r, m) spectra (the l_2D_spectra part of
    calculate_spectra, src/spectra.f90:134-164, and write_2D_spectra,
    :371-457): running means (and with l_2D_SD standard deviations, getMSD2
    of src/useful.f90:263-293 per point) of us2R, up2R and enstR, the device
    snapshots of Ensemble.spectra_2d."""

    def __init__(self, n_r_max: int, n_m_max: int, l_sd: bool = False):
        self.mean = np.zeros((3, n_r_max, n_m_max))
        self.sd = np.zeros((3, n_r_max, n_m_max))
        self.l_sd = l_sd
        self.n_calls = 0
        self.time_last = 0.0

    def update(self, spec2d, time_avg: float):
        """spec2d: (3, n_r_max, n_m_max) snapshot (Ensemble.spectra_2d);
        time_avg: the caller's running sum of dt over its output calls."""
        x = np.asarray(spec2d, float)
        self.n_calls += 1
        dt = time_avg - self.time_last
        if self.n_calls == 1:
            self.mean = x.copy()
            self.sd = np.zeros_like(x)
        else:
            delta = x - self.mean
            self.mean = self.mean + delta * dt / time_avg
            self.sd = self.sd + dt * delta * (x - self.mean)
        self.time_last = time_avg

    def result(self):
        """(mean, SD): SD normalised as write_spectra_avg does (spectra.f90:290-299)."""
        return self.mean.copy(), np.sqrt(self.sd / self.time_last)

    def write(self, path: str, cfg, r):
        """2D_spec_avg.TAG: version (1, or 2 with SD), ra, pr, raxi, sc, ek,
        radratio, n_r_max, n_m_max, m_max, minc, r, then per field its mean
        (and SD) as (n_m_max, n_r_max) with m varying fastest, stream
        unformatted."""
        mean, sd = self.result()
        _, n_r, n_m = mean.shape
        with open(path, "wb") as f:
            np.array([2 if self.l_sd else 1], _I4).tofile(f)
            np.array([cfg.ra, cfg.pr, cfg.raxi, cfg.sc, cfg.ek, cfg.radratio], _F8).tofile(f)
            np.array([n_r, n_m, cfg.m_max, cfg.minc], _I4).tofile(f)
            np.asarray(r, _F8).tofile(f)
            for k in range(3):
                np.ascontiguousarray(mean[k], _F8).tofile(f)
                if self.l_sd:
                    np.ascontiguousarray(sd[k], _F8).tofile(f)
        return path


def read_2d_spectra(path: str):
    """Read a 2D_spec_avg.TAG file: header fields, r and the (mean, SD)
    arrays of us2, up2, enst as (n_m_max, n_r_max) arrays (SD None for
    version 1)."""
    with open(path, "rb") as f:
        version = int(np.fromfile(f, _I4, 1)[0])
        ra, pr, raxi, sc, ek, radratio = (float(v) for v in np.fromfile(f, _F8, 6))
        n_r, n_m, m_max, minc = (int(v) for v in np.fromfile(f, _I4, 4))
        r = np.fromfile(f, _F8, n_r)
        out = dict(version=version, ra=ra, pr=pr, raxi=raxi, sc=sc, ek=ek, radratio=radratio, n_r_max=n_r,
                   n_m_max=n_m, m_max=m_max, minc=minc, r=r)
        for name in ("us2", "up2", "enst"):
            out[name] = np.fromfile(f, _F8, n_r * n_m).reshape(n_r, n_m).T
            out[name + "_SD"] = np.fromfile(f, _F8, n_r * n_m).reshape(n_r, n_m).T if version == 2 else None
    return out


# ---------------------------------------------------------------------------
# force balances (vort_balance.f90, vp_balance.f90), accumulated on the host
# from the device terms of Ensemble.balance_step
# ---------------------------------------------------------------------------
def _cc2real(z, m):
    """cc2real (src/useful.f90): Re(z)^2 for m = 0, 2 |z|^2 otherwise; m (M,) broadcast over r."""
    z = np.asarray(z)
    out = 2.0 * (z.real ** 2 + z.imag ** 2)
    out[np.asarray(m) == 0] = (z.real ** 2)[np.asarray(m) == 0]
    return out


def simps(f, r):
    """simps (src/integration.f90:102-152): Simpson's rule on the (non-uniform)
    radial grid, r(1) = r_cmb first; twice Simpson plus trapezoids for an even
    number of points."""
    n = len(f)

    def panel(i):
        h2 = r[i + 1] - r[i]
        h1 = r[i] - r[i - 1]
        return (h1 + h2) / 6.0 * (f[i - 1] * (2 * h1 - h2) / h1 + f[i] * (h1 + h2) ** 2 / (h1 * h2)
                                  + f[i + 1] * (2 * h2 - h1) / h2)
    if n % 2 == 1:
        return -sum(panel(i) for i in range(1, n - 1, 2))
    rint = 0.5 * (r[1] - r[0]) * (f[1] + f[0])
    for i in range(2, n, 2):
        rint += panel(i)
    rint += 0.5 * (r[n - 1] - r[n - 2]) * (f[n - 1] + f[n - 2])
    for i in range(1, n - 1, 2):
        rint += panel(i)
    return -0.5 * rint


def rint_weights(n_r_max: int, radratio: float):
    """Weights w of rInt_R (src/integration.f90:18-55, Chebyshev grid):
    rInt_R(f) = sum_k w_k f_k (the DCT-I of f / drx, the integrals of the
    Chebyshev polynomials)."""
    N = n_r_max
    drx = 2.0                                   # 2 / (r_cmb - r_icb), unit gap
    k = np.arange(N)
    C = 2.0 * np.cos(np.pi * np.outer(k, k) / (N - 1))
    C[:, 0] = 1.0
    C[:, N - 1] = (-1.0) ** k
    C *= np.sqrt(0.5 / (N - 1))                 # costf_real_1d
    a = np.zeros(N)
    a[0] = 0.5
    for nc in range(3, N + 1, 2):
        a[nc - 1] = -1.0 / float(nc * (nc - 2))
    a[N - 1] *= 0.5 if (N - 1) % 2 == 0 else 1.0
    w = 2.0 * np.sqrt(2.0 / (N - 1)) * (a @ C) / drx
    return w


class VortBalance:
    """The vorticity force balance averaged over time (vort_balance.f90:
    calc_avg and mean_sd_loc :188-262, write_outputs :264-520): per call the
    six terms of Ensemble.balance_step and three sums (thwind = buo + cor,
    iner = adv - dwdt, cia = adv - dwdt + buo + cor) give cc2real(term) r
    height, averaged at every (m, r) (with SD if l_sd) and, with the points
    within bl_cut of the walls left out, integrated over r by simps and
    averaged per m.  Writes vort_terms_avg.TAG and vort_bal.TAG."""

    QUANT = ("buo", "cor", "adv", "dwdt", "visc", "pump", "thwind", "iner", "cia")

    def __init__(self, cfg, r, height, l_sd: bool = False, bl_cut: float = 1.0e-3):
        self.cfg, self.r, self.h = cfg, np.asarray(r, float), np.asarray(height, float)
        self.l_sd, self.bl_cut = l_sd, bl_cut
        M, N = cfg.m_max // cfg.minc + 1, len(self.r)
        self.m = np.arange(M) * cfg.minc
        self.mean2 = {q: np.zeros((M, N)) for q in self.QUANT}
        self.sd2 = {q: np.zeros((M, N)) for q in self.QUANT}
        self.meanM = {q: np.zeros(M) for q in self.QUANT}
        self.sdM = {q: np.zeros(M) for q in self.QUANT}
        self.n_calls = 0
        self.time_last = 0.0
        r_cmb = 1.0 / (1.0 - cfg.radratio)
        self.mask = (self.r >= r_cmb - bl_cut) | (self.r <= r_cmb - 1.0 + bl_cut)

    @staticmethod
    def _msd(mean, sd, x, n, dt, total):
        if n == 1:
            return x.copy(), np.zeros_like(x)
        delta = x - mean
        mean = mean + delta * dt / total
        return mean, sd + dt * delta * (x - mean)

    def calc_avg(self, vort, time_avg: float):
        """vort: the "vort" dict of Ensemble.balance_step; time_avg: the running
        sum of dt over the balance steps (timeAvg_vortbal, outputs.f90:335-338)."""
        self.n_calls += 1
        dt = time_avg - self.time_last
        t = vort
        terms = {"buo": t["buo"], "cor": t["cor"], "adv": t["adv"], "dwdt": t["dwdt"], "visc": t["visc"],
                 "pump": t["pump"], "thwind": t["buo"] + t["cor"], "iner": -t["dwdt"] + t["adv"],
                 "cia": -t["dwdt"] + t["adv"] + t["buo"] + t["cor"]}
        mcol = self.m[:, None] * np.ones_like(self.r)[None, :]
        for q in self.QUANT:
            dat = _cc2real(terms[q], mcol) * self.r * self.h
            self.mean2[q], self.sd2[q] = self._msd(self.mean2[q], self.sd2[q], dat, self.n_calls, dt, time_avg)
            dat = np.where(self.mask, 0.0, dat)
            val = np.array([simps(dat[k], self.r) for k in range(dat.shape[0])])
            self.meanM[q], self.sdM[q] = self._msd(self.meanM[q], self.sdM[q], val, self.n_calls, dt, time_avg)
        self.time_last = time_avg

    def terms_lines(self):
        """vort_terms_avg.TAG: '(I5, 18es16.8)' of m >= 1 and the mean and SD
        of buo, cor, adv, dwdt, visc, pump, thwind, iner, cia."""
        out = []
        order = ("buo", "cor", "adv", "dwdt", "visc", "pump", "thwind", "iner", "cia")
        for k, m in enumerate(self.m):
            if m < 1:
                continue
            vals = []
            for q in order:
                vals += [self.meanM[q][k], np.sqrt(self.sdM[q][k] / self.time_last)]
            out.append(f"{m:5d}" + "".join(fortran_es(v, 16, 8) for v in vals))
        return out

    def write(self, tag: str, directory: str = "."):
        """vort_terms_avg.TAG and vort_bal.TAG (version 1, or 2 with SD; the
        header of 2D_spec_avg, then per quantity its (n_m_max, n_r_max) mean
        (and SD) with m varying fastest)."""
        p1 = os.path.join(directory, f"vort_terms_avg.{tag}")
        with open(p1, "w") as f:
            for ln in self.terms_lines():
                f.write(ln + "\n")
        cfg = self.cfg
        M, N = len(self.m), len(self.r)
        p2 = os.path.join(directory, f"vort_bal.{tag}")
        with open(p2, "wb") as f:
            np.array([2 if self.l_sd else 1], _I4).tofile(f)
            np.array([cfg.ra, cfg.pr, cfg.raxi, cfg.sc, cfg.ek, cfg.radratio], _F8).tofile(f)
            np.array([N, M, cfg.m_max, cfg.minc], _I4).tofile(f)
            self.r.astype(_F8).tofile(f)
            for q in ("buo", "cor", "adv", "dwdt", "visc", "pump", "thwind", "iner", "cia"):
                np.ascontiguousarray(self.mean2[q].T, _F8).tofile(f)
                if self.l_sd:
                    np.ascontiguousarray(np.sqrt(self.sd2[q] / self.time_last).T, _F8).tofile(f)
        return p1, p2


class VpBalance:
    """The u_phi (m = 0) force balance (vp_balance.f90:write_outputs
    :140-210): per call, vphi_bal.TAG (stream unformatted: ra, ek, pr,
    radratio, raxi, sc and r once, then time, u_phi(m = 0), dvpdt,
    rey_stress, pump, visc) and one vphi_power.TAG line '(1P,es20.12,5es16.8)'
    of time, Ez and the powers 2 pi rInt_R(term u_phi height r)."""

    def __init__(self, cfg, r, height, tag: str, directory: str = "."):
        self.cfg, self.r, self.h = cfg, np.asarray(r, float), np.asarray(height, float)
        self.w = rint_weights(len(self.r), cfg.radratio)
        self.bal = os.path.join(directory, f"vphi_bal.{tag}")
        self.power = os.path.join(directory, f"vphi_power.{tag}")
        self.n_calls = 0
        for p in (self.bal, self.power):
            if os.path.exists(p):
                os.remove(p)

    def write(self, time: float, up_m0, vp):
        """up_m0: the real part of u_phi(m = 0) after the balance step; vp: the
        "vp" dict of Ensemble.balance_step."""
        self.n_calls += 1
        cfg = self.cfg
        vz = np.asarray(up_m0, float).real
        with open(self.bal, "ab") as f:
            if self.n_calls == 1:
                np.array([cfg.ra, cfg.ek, cfg.pr, cfg.radratio, cfg.raxi, cfg.sc], _F8).tofile(f)
                self.r.astype(_F8).tofile(f)
            np.array([time], _F8).tofile(f)
            for a in (vz, vp["dvpdt"], vp["rey_stress"], vp["pump"], vp["visc"]):
                np.asarray(a, _F8).tofile(f)
        hr = self.h * self.r
        ez = np.pi * self.w @ (vz * vz * hr)
        vals = [2.0 * np.pi * self.w @ (vp[k] * vz * hr) for k in ("dvpdt", "rey_stress", "pump", "visc")]
        with open(self.power, "a") as f:
            f.write(fortran_es(time, 20, 12) + fortran_es(ez, 16, 8) + "".join(fortran_es(v, 16, 8) for v in vals)
                    + "\n")
        return ez, vals


def write_series(ens, i: int, tag: str, directory: str = ".", rows=None):
    """Write e_kin.TAG, heat.TAG, (rotating runs) e_kin_3D.TAG and (with
    composition) composition.TAG of instance i from its time-series rows
    (Ensemble.series: at most the last 1024).  Returns the paths written."""
    if rows is None:
        rows = ens.series(i)
    rot = not ens.configs[i].l_non_rot and ens.configs[i].ek >= 0.0
    paths = []
    for name, cols in SERIES_FILES.items():
        if (name == "e_kin_3D" and not rot) or (name == "composition" and ens.configs[i].raxi == 0.0):
            continue
        p = os.path.join(directory, f"{name}.{tag}")
        with open(p, "w") as f:
            for row in rows:
                f.write(format_series_line([row[c] for c in cols]) + "\n")
        paths.append(p)
    return paths


# ---------------------------------------------------------------------------
# version-7 checkpoints (stream-unformatted, native byte order)
# ---------------------------------------------------------------------------
_I4, _F8 = np.dtype("<i4"), np.dtype("<f8")


def _grid_r(n_r_max: int, radratio: float) -> np.ndarray:
    """Gauss-Lobatto radii (src/chebyshev.f90, no mapping): r(1) = r_cmb."""
    r_cmb = 1.0 / (1.0 - radratio)
    r_icb = r_cmb - 1.0
    x = np.cos(np.pi * np.arange(n_r_max) / (n_r_max - 1))
    return 0.5 * (r_cmb - r_icb) * x + 0.5 * (r_cmb + r_icb)


def write_checkpoint(path: str, header: dict, fields: dict):
    """Write a version-7 checkpoint (write_checkpoint_mloc).

    header: time, family ('MULTISTEP' or 'DIRK'), nexp, nimp, nold, dt (array),
    ra, pr, ek, radratio, n_r_max, m_max, minc, n_max, r (n_r_max radii) and,
    with composition, raxi and sc.
    fields: us, up, temp ((n_m_max, n_r_max) complex) and, for MULTISTEP,
    lists hist_P and hist_T of the slots written after up and temp: expl
    2..nexp, impl 2..nimp, old 2..nold, in that order; with composition xi
    and hist_Xi after them (write_one_field_mpi of xi_Mloc, checkpoints.f90:158)."""
    chem = fields.get("xi") is not None
    h = header
    with open(path, "wb") as f:
        f.write(np.array([7], _I4).tobytes())
        f.write(np.array([h["time"]], _F8).tobytes())
        f.write(np.array([int(h.get("l_cheb_coll", True))], _I4).tobytes())   # l_cheb_coll
        f.write(h["family"].ljust(10)[:10].encode())
        f.write(np.array([h["nexp"], h["nimp"], h["nold"]], _I4).tobytes())
        f.write(np.asarray(h["dt"], _F8).tobytes())
        f.write(np.array([h["ra"], h["pr"], h.get("raxi", 0.0), h.get("sc", 0.0), h["ek"], 0.0, h["radratio"]],
                         _F8).tobytes())
        f.write(np.array([h["n_r_max"], h["m_max"], h["minc"]], _I4).tobytes())
        f.write("cheb".ljust(72).encode())
        f.write(np.array([h["n_max"], h.get("order_boundary", 0)], _I4).tobytes())
        f.write(np.array([0.0, 0.0], _F8).tobytes())                     # alph1, alph2 (no mapping)
        f.write(np.asarray(h["r"], _F8).tobytes())
        f.write(np.array([1, int(chem), 0], _I4).tobytes())              # l_heat, l_chem, l_phase_field

        def put(a):
            # (n_m_max, n_r_max) Fortran order: m fastest
            f.write(np.asfortranarray(np.asarray(a, np.complex128)).tobytes(order="F"))

        put(fields["us"])
        put(fields["up"])
        for a in fields.get("hist_P", []):
            put(a)
        put(fields["temp"])
        for a in fields.get("hist_T", []):
            put(a)
        if chem:
            put(fields["xi"])
            for a in fields.get("hist_Xi", []):
                put(a)


def read_checkpoint(path: str) -> dict:
    """Read a version-7 checkpoint written by pizza.exe or write_checkpoint."""
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0

    def take(dtype, n=1):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dtype, count=n, offset=pos)
        pos += a.nbytes
        return a

    def chars(n):
        nonlocal pos
        s = buf[pos:pos + n].decode(errors="replace")
        pos += n
        return s.strip()

    version = int(take(_I4)[0])
    if version != 7:
        raise ValueError(f"checkpoint version {version}: only version 7 is read")
    h = {"version": version, "time": float(take(_F8)[0]), "l_cheb_coll": bool(take(_I4)[0])}
    h["family"] = chars(10)
    h["nexp"], h["nimp"], h["nold"] = (int(v) for v in take(_I4, 3))
    h["dt"] = take(_F8, h["nexp"] if h["family"] == "MULTISTEP" else 1).copy()
    ra, pr, raxi, sc, ek, stef, radratio = take(_F8, 7)
    h.update(ra=float(ra), pr=float(pr), raxi=float(raxi), sc=float(sc), ek=float(ek), stef=float(stef),
             radratio=float(radratio))
    h["n_r_max"], h["m_max"], h["minc"] = (int(v) for v in take(_I4, 3))
    h["rscheme"] = chars(72)
    h["n_max"], h["order_boundary"] = (int(v) for v in take(_I4, 2))
    h["alph1"], h["alph2"] = (float(v) for v in take(_F8, 2))
    h["r"] = take(_F8, h["n_r_max"]).copy()
    h["l_heat"], h["l_chem"], h["l_phase_field"] = (bool(v) for v in take(_I4, 3))
    M = h["m_max"] // h["minc"] + 1
    N = h["n_r_max"]
    nh = (h["nexp"] - 1) + (h["nimp"] - 1) + (h["nold"] - 1) if h["family"] == "MULTISTEP" else 0

    def field():
        return take(np.dtype("<c16"), M * N).reshape((M, N), order="F").copy()

    out = {"header": h, "us": field(), "up": field()}
    out["hist_P"] = [field() for _ in range(nh)]
    if h["l_heat"]:
        out["temp"] = field()
        out["hist_T"] = [field() for _ in range(nh)]
    if h["l_chem"]:
        out["xi"] = field()
        out["hist_Xi"] = [field() for _ in range(nh)]
    if pos != len(buf):
        raise ValueError(f"checkpoint {path}: {len(buf) - pos} trailing bytes (phase field?)")
    return out


def _hist_order(nexp, nimp, nold):
    """(kind, slot) of the history arrays in checkpoint order (write_one_field_mpi)."""
    return ([(2, k) for k in range(2, nexp + 1)] + [(1, k) for k in range(2, nimp + 1)]
            + [(0, k) for k in range(2, nold + 1)])


def save_checkpoint(ens, i: int, path: str):
    """Checkpoint of instance i at the current step boundary."""
    c = ens.configs[i]
    st = ens.get_state(i)
    time, dt, _ = ens.get_step_state(i)
    nexp, nimp, nold, family = _scheme_counts(ens, i)
    n, m, _ = ens.dims[i]
    header = dict(time=time, family=family, nexp=nexp, nimp=nimp, nold=nold,
                  dt=dt[:nexp] if family == "MULTISTEP" else dt[:1], ra=c.ra, pr=c.pr, ek=c.ek,
                  radratio=c.radratio, n_r_max=n, m_max=c.m_max, minc=c.minc,
                  n_max=c.n_cheb_max if c.n_cheb_max is not None else n, r=_grid_r(n, c.radratio),
                  l_cheb_coll="COLL" in c.cheb_method.upper(), raxi=c.raxi, sc=c.sc)
    chem = c.raxi != 0.0
    fields = dict(us=st["us"], up=st["up"], temp=st["temp"], xi=st["xi"] if chem else None)
    if family == "MULTISTEP":
        order = _hist_order(nexp, nimp, nold)
        fields["hist_P"] = [ens.get_history(i, 1, k, s) for k, s in order]
        fields["hist_T"] = [ens.get_history(i, 0, k, s) for k, s in order]
        if chem:
            fields["hist_Xi"] = [ens.get_history(i, 2, k, s) for k, s in order]
    write_checkpoint(path, header, fields)


# ---------------------------------------------------------------------------
# frames: 2-D snapshots of one field (src/output_frames.f90:105-145, read by
# python/pizza/frame.py), stream-unformatted, native byte order
# ---------------------------------------------------------------------------
def write_frame(path: str, header: dict, field):
    """Write a version-2 frame (write_snapshot_mloc): version, time, ra, ek,
    pr, radratio, sc, raxi, n_r_max, n_m_max, m_max, minc, n_phi_max, r,
    tcond, xicond, idx2m, then the (n_m_max, n_r_max) complex field with m
    fastest.  header: time, ra, ek, pr, radratio, sc, raxi, m_max, minc, r,
    tcond, xicond (the last may be None: written as zeros)."""
    h = header
    f = np.asarray(field, np.complex128)
    n_m_max, n_r_max = f.shape
    r = np.asarray(h["r"], _F8)
    xicond = np.zeros(n_r_max) if h.get("xicond") is None else np.asarray(h["xicond"], _F8)
    with open(path, "wb") as out:
        out.write(np.array([2], _I4).tobytes())
        out.write(np.array([h["time"], h["ra"], h["ek"], h["pr"], h["radratio"], h.get("sc", 0.0),
                            h.get("raxi", 0.0)], _F8).tobytes())
        out.write(np.array([n_r_max, n_m_max, h["m_max"], h["minc"], 3 * h["m_max"] // h["minc"]], _I4).tobytes())
        out.write(r.tobytes())
        out.write(np.asarray(h["tcond"], _F8).tobytes())
        out.write(np.asarray(xicond, _F8).tobytes())
        out.write((np.arange(n_m_max, dtype=np.int32) * h["minc"]).astype(_I4).tobytes())
        out.write(np.asfortranarray(f).tobytes(order="F"))


def read_frame(path: str) -> dict:
    """Read a version-2 frame written by pizza.exe or write_frame."""
    with open(path, "rb") as fh:
        version = int(np.fromfile(fh, _I4, 1)[0])
        if version != 2:
            raise ValueError(f"frame version {version}: only version 2 is read")
        vals = np.fromfile(fh, _F8, 7)
        n_r_max, n_m_max, m_max, minc, n_phi_max = (int(v) for v in np.fromfile(fh, _I4, 5))
        r = np.fromfile(fh, _F8, n_r_max)
        tcond = np.fromfile(fh, _F8, n_r_max)
        xicond = np.fromfile(fh, _F8, n_r_max)
        idx2m = np.fromfile(fh, _I4, n_m_max)
        field = np.fromfile(fh, np.dtype("<c16"), n_m_max * n_r_max).reshape((n_m_max, n_r_max), order="F")
    keys = ("time", "ra", "ek", "pr", "radratio", "sc", "raxi")
    out = {k: float(v) for k, v in zip(keys, vals)}
    out.update(version=version, n_r_max=n_r_max, n_m_max=n_m_max, m_max=m_max, minc=minc, n_phi_max=n_phi_max,
               r=r, tcond=tcond, xicond=xicond, idx2m=idx2m, field=field)
    return out


def save_frames(ens, i: int, counter: int, tag: str, directory: str = "."):
    """frame_temp_<counter>.<tag>, (with composition) frame_xi_..., then
    frame_us_..., frame_up_..., frame_om_... of instance i (outputs.f90:293-310;
    temperature and composition are the perturbations, tcond and xicond are in
    the header).  Returns the paths written."""
    c = ens.configs[i]
    n, _, _ = ens.dims[i]
    st = ens.get_state(i)
    time, _, _ = ens.get_step_state(i)
    r = _grid_r(n, c.radratio)
    r_cmb = 1.0 / (1.0 - c.radratio)
    chem = c.raxi != 0.0
    header = dict(time=time, ra=c.ra, ek=c.ek, pr=c.pr, radratio=c.radratio, sc=c.sc, raxi=c.raxi, m_max=c.m_max,
                  minc=c.minc, r=r, tcond=np.log(r / r_cmb) / np.log(c.radratio),
                  xicond=c.xicond_fac * np.log(r / r_cmb) / np.log(c.radratio) if chem else None)
    paths = []
    names = (("temp", "temp"),) + ((("xi", "xi"),) if chem else ()) + (("us", "us"), ("up", "up"), ("om", "om"))
    for name, key in names:
        p = os.path.join(directory, f"frame_{name}_{counter}.{tag}")
        write_frame(p, header, st[key])
        paths.append(p)
    return paths


def _costf1(f):
    """DCT-I along the last axis with pizza's normalisation sqrt(1/(2(N-1))),
    self-inverse (costf1 of src/dct_fftw.f90)."""
    f = np.asarray(f, complex)
    n = f.shape[-1]
    ext = np.concatenate([f, f[..., n - 2:0:-1]], axis=-1)
    return np.sqrt(0.5 / (n - 1)) * np.fft.fft(ext, axis=-1)[..., :n]


def map_field(f, n_m_max: int, n_r_max: int, phys: bool, lbc: bool = False):
    """A checkpoint field (n_m_old, n_r_old) onto (n_m_max, n_r_max), as
    map_field / map_field_r do for Chebyshev grids (src/checkpoints.f90:709-860):
    azimuthal modes the file lacks are zero; in r the Chebyshev coefficients
    (costf1 of the old grid first for a physical-space field) are zero-padded
    or cut and brought back with the new grid's costf1, times
    sqrt(2/(n_r_old-1)) / sqrt(2/(n_r_max-1)).  lbc: a physical-space history
    slot whose boundary value is re-extrapolated first."""
    f = np.asarray(f, complex)
    n_old = f.shape[1]
    out = np.zeros((n_m_max, n_r_max), complex)
    mm = min(n_m_max, f.shape[0])
    if n_old == n_r_max:
        out[:mm] = f[:mm]
        return out
    g = f[:mm].copy()
    if lbc and phys:
        g[:, 0] = 2.0 * g[:, 1] - g[:, 2]
    if phys:
        g = _costf1(g)
    pad = np.zeros((mm, max(n_old, n_r_max)), complex)
    pad[:, :n_old] = g
    g = pad[:, :n_r_max]
    if phys:
        g = _costf1(g)
    out[:mm] = np.sqrt(2.0 / (n_old - 1)) / np.sqrt(2.0 / (n_r_max - 1)) * g
    return out


def restart_from_checkpoint(ens, i: int, path: str, temp_add=None, xi_add=None):
    """Start instance i from a checkpoint as read_checkpoint and
    get_start_fields do (src/checkpoints.f90:185-860, src/init_fields.f90:54-258):
    temp_add / xi_add (complex (n_m_max, n_r_max), or None) are added to the
    mapped temperature / composition before the state is set, as
    get_start_fields applies initProp after reading a checkpoint
    (init_fields.f90:121-123);
    fields and multistep history slots 2..n mapped onto the instance's grid
    (map_field), dt filled with the oldest value where the instance's scheme
    keeps more, time; the first old/implicit slots are recomputed from the
    fields on the device.  AB1 on the first step when the Ekman number or the
    radial method changed, and the CNAB2 bridge when the scheme needs more
    old or implicit slots than the file holds.  Returns the header."""
    ck = read_checkpoint(path)
    h = ck["header"]
    n, mm, _ = ens.dims[i]
    c = ens.configs[i]
    if h["minc"] != c.minc:
        raise ValueError("checkpoint minc differs from the instance's (not restated)")
    if h["rscheme"] != "cheb" or not h["l_heat"]:
        raise ValueError("only Chebyshev checkpoints with temperature are read")
    nexp, nimp, nold, family = _scheme_counts(ens, i)
    coll = "COLL" in c.cheb_method.upper()
    coll_old = bool(h["l_cheb_coll"])
    chem = c.raxi != 0.0 and h["l_chem"]
    temp = map_field(ck["temp"], mm, n, True)
    if temp_add is not None:
        temp = temp + temp_add
    xi = map_field(ck["xi"], mm, n, True) if chem else None
    if xi_add is not None and c.raxi != 0.0:
        xi = xi_add if xi is None else xi + xi_add
    ens.set_state(i, us=map_field(ck["us"], mm, n, True), up=map_field(ck["up"], mm, n, True),
                  temp=temp, xi=xi)
    if h["family"] == "MULTISTEP" and family == "MULTISTEP":
        counts = {2: nexp, 1: nimp, 0: nold}
        order = _hist_order(h["nexp"], h["nimp"], h["nold"])
        for (k, slot), aP, aT in zip(order, ck["hist_P"], ck["hist_T"]):
            if slot <= counts[k]:
                ens.set_history(i, 1, k, slot, map_field(aP, mm, n, coll_old, lbc=k != 0))
                ens.set_history(i, 0, k, slot, map_field(aT, mm, n, coll_old, lbc=k != 0))
        if chem:
            for (k, slot), aX in zip(order, ck["hist_Xi"]):
                if slot <= counts[k]:
                    ens.set_history(i, 2, k, slot, map_field(aX, mm, n, coll_old, lbc=k != 0))
    nd = nexp if family == "MULTISTEP" else 1
    dt = np.array([h["dt"][min(k, len(h["dt"]) - 1)] for k in range(nd)])
    ab1 = h["ek"] != c.ek
    if family == "MULTISTEP":
        bridge = h["family"] == "DIRK" or nold > h["nold"] or nimp > h["nimp"]
        if coll_old != coll:
            ab1 = bridge = True
    else:
        bridge = False
    # n_step 0 runs the CNAB2 bridge over the first nold-1 steps; nold skips it
    ens.set_step_state(i, h["time"], dt, 0 if bridge else max(nold, 1))
    ens.set_restart_ab1(i, ab1)
    return h


def _scheme_counts(ens, i):
    """(nexp, nimp, nold, family) of instance i's time scheme
    (multistep_schemes.f90:53-106, dirk_schemes.f90:35-244)."""
    ts = ens.configs[i].time_scheme.upper()
    multistep = {"CNAB2": (2, 1, 1), "SBDF2": (2, 1, 2), "BDF2AB2": (2, 1, 2), "SBDF3": (3, 1, 3),
                 "BDF3AB3": (3, 1, 3), "SBDF4": (4, 1, 4), "BDF4AB4": (4, 1, 4), "CNLF": (2, 2, 2),
                 "MODCNAB": (2, 2, 2), "TVB33": (3, 3, 3)}
    if ts in multistep:
        nexp, nimp, nold = multistep[ts]
        return nexp, nimp, nold, "MULTISTEP"
    stages = {"ARS222": 2, "ARS232": 3, "ARS233": 3, "SSP222": 3, "LSDIRK222": 3, "LZ232": 2, "CK232": 2,
              "ARS443": 4, "BPR353": 4, "PC2": 3, "ARS343": 4, "MARS343": 4, "SSP322": 4, "SSP332": 4,
              "SSP433": 5, "DP1-242": 4, "DP2-242": 4, "LZ453": 4, "KC343": 4, "KC564": 6, "KC785": 8,
              "DBM453": 5}
    ns = stages[ts]
    return ns, ns, 1, "DIRK"

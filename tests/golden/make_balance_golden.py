"""Golden force-balance files for pizza_gb300.pizza_io.VortBalance and
VpBalance: three deterministic sets of balance terms accumulated and written
by the library's writers, then read back by the reference's own readers
(PizzaVortBalance._read/assemble and PizzaBalance._read, python/pizza/balance.py
of the magic-sph/pizza tree given by --ref, read only), whose parsed values
are stored next to the files.  The reader module imports matplotlib for
plotting helpers that reading does not use; a stand-in module is installed
for the import only.

Writes tests/golden/vort_bal.golden, vort_terms_avg.golden, vphi_bal.golden,
vphi_power.golden and balance_golden.json.
"""
import argparse
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
TERMS = ("buo", "cor", "adv", "dwdt", "visc", "pump")


def sample():
    """(cfg, r, height, calls): calls = [(time, vort terms, u_phi(m=0), vp terms)]."""
    n_r_max, m_max = 9, 4
    cfg = types.SimpleNamespace(ra=1.0e5, pr=1.0, raxi=0.0, sc=0.0, ek=1.0e-3, radratio=0.35, m_max=m_max, minc=1)
    r_cmb = 1.0 / 0.65
    r = 0.5 * np.cos(np.pi * np.arange(n_r_max) / (n_r_max - 1)) + r_cmb - 0.5
    height = 2.0 * np.sqrt(r_cmb ** 2 - r ** 2)
    rng = np.random.default_rng(5)
    calls = []
    for k, t in enumerate((0.1, 0.25, 0.45)):
        vort = {q: rng.standard_normal((m_max + 1, n_r_max)) + 1j * rng.standard_normal((m_max + 1, n_r_max))
                for q in TERMS}
        vp = {q: rng.standard_normal(n_r_max) for q in ("rey_stress", "dvpdt", "visc", "pump")}
        calls.append((t, vort, rng.standard_normal(n_r_max), vp))
    return cfg, r, height, calls


def write_sample(directory, tag="golden"):
    from pizza_gb300.pizza_io import VortBalance, VpBalance
    cfg, r, height, calls = sample()
    vb = VortBalance(cfg, r, height, l_sd=True, bl_cut=0.05)
    vpb = VpBalance(cfg, r, height, tag, directory)
    t_avg = 0.0
    for t, vort, up0, vp in calls:
        t_avg += 0.05
        vb.calc_avg(vort, t_avg)
        vpb.write(t, up0, vp)
    return vb.write(tag, directory) + (vpb.bal, vpb.power)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the pizza source tree (read only)")
    args = ap.parse_args()
    paths = write_sample(HERE)
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.cm", "matplotlib.ticker"):
        mod = sys.modules.setdefault(name, types.ModuleType(name))
        mod.__version__ = "3.0.0"
    sys.dont_write_bytecode = True             # the reference tree stays untouched
    sys.path.insert(0, os.path.join(args.ref, "python"))
    from pizza.balance import PizzaBalance, PizzaVortBalance
    vb = object.__new__(PizzaVortBalance)
    vb.assemble(vb._read(paths[1]))
    parsed = dict(version=int(vb.version), n_r_max=int(vb.n_r_max), n_m_max=int(vb.n_m_max), m_max=int(vb.m_max),
                  minc=int(vb.minc), radius=vb.radius.tolist())
    for k in ("buo_mean", "cor_mean", "adv_mean", "domdt_mean", "visc_mean", "pump_mean", "thwind_mean"):
        parsed[k] = getattr(vb, k).tolist()
    pb = object.__new__(PizzaBalance)
    pb.n_r_max = len(vb.radius)
    radius, time, vp, dvpdt, rey, pump, visc = pb._read(paths[2], "l")
    parsed["vphi"] = dict(radius=radius.tolist(), time=time.tolist(), vp=vp.tolist(), dvpdt=dvpdt.tolist(),
                          rey_stress=rey.tolist(), pump=pump.tolist(), visc=visc.tolist())
    with open(os.path.join(HERE, "balance_golden.json"), "w") as out:
        json.dump(parsed, out, indent=1)


if __name__ == "__main__":
    main()

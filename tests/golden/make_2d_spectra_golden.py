"""Golden 2-D spectra file for pizza_gb300.pizza_io.Spectra2DAverage: a small
deterministic average (three snapshots, with standard deviations) written by
the library's writer and read back by the reference's own reader
(Pizza2DSpectrum._read and assemble, python/pizza/spectrum.py of the
magic-sph/pizza tree given by --ref, read only), whose parsed values are
stored next to the file.  The reader module imports matplotlib for plotting
helpers that reading does not use; a stand-in module is installed for the
import only.

Writes tests/golden/spec2d_sample.bin and tests/golden/spec2d_sample.json.
"""
import argparse
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def sample():
    """(cfg, r, snapshots, averaging times) of the golden file."""
    n_r_max, m_max = 7, 5
    cfg = types.SimpleNamespace(ra=1.0e5, pr=1.0, raxi=0.0, sc=0.0, ek=1.0e-3, radratio=0.35, m_max=m_max, minc=1)
    r_cmb = 1.0 / 0.65
    r = 0.5 * np.cos(np.pi * np.arange(n_r_max) / (n_r_max - 1)) + r_cmb - 0.5
    rng = np.random.default_rng(77)
    snaps = [rng.random((3, n_r_max, m_max + 1)) for _ in range(3)]
    return cfg, r, snaps, (0.5, 1.25, 2.0)


def write_sample(path):
    from pizza_gb300.pizza_io import Spectra2DAverage
    cfg, r, snaps, times = sample()
    av = Spectra2DAverage(len(r), cfg.m_max + 1, l_sd=True)
    for x, t in zip(snaps, times):
        av.update(x, t)
    return av.write(path, cfg, r)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the pizza source tree (read only)")
    args = ap.parse_args()
    path = write_sample(os.path.join(HERE, "spec2d_sample.bin"))
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.cm", "matplotlib.ticker"):
        mod = sys.modules.setdefault(name, types.ModuleType(name))
        mod.__version__ = "3.0.0"
    sys.dont_write_bytecode = True             # the reference tree stays untouched
    sys.path.insert(0, os.path.join(args.ref, "python"))
    from pizza.spectrum import Pizza2DSpectrum
    sp = object.__new__(Pizza2DSpectrum)
    data = sp._read(path)
    sp.assemble(data)
    parsed = dict(version=int(sp.version), ra=float(sp.ra), pr=float(sp.pr), raxi=float(sp.raxi), sc=float(sp.sc),
                  ek=float(sp.ek), radratio=float(sp.radratio), n_r_max=int(sp.n_r_max), n_m_max=int(sp.n_m_max),
                  m_max=int(sp.m_max), minc=int(sp.minc), radius=[float(v) for v in sp.radius],
                  us2_m=sp.us2_m.tolist(), us2_m_SD=sp.us2_m_SD.tolist(), up2_m=sp.up2_m.tolist(),
                  up2_m_SD=sp.up2_m_SD.tolist(), enst_m=sp.enst_m.tolist())
    with open(os.path.join(HERE, "spec2d_sample.json"), "w") as out:
        json.dump(parsed, out, indent=1)


if __name__ == "__main__":
    main()

"""Golden frame for pizza_gb300.pizza_io.write_frame: a small deterministic
field written by the library's writer and read back by the reference's own
reader (python/pizza/frame.py of the magic-sph/pizza tree given by --ref,
read only), whose parsed values are stored next to the
file.  The reader imports matplotlib for plotting helpers that reading does
not use; a stand-in module is installed for the import only.

Writes tests/golden/frame_sample.bin and tests/golden/frame_sample.json.
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
    n_r_max, m_max = 9, 4
    rng = np.random.default_rng(2024)
    field = rng.standard_normal((m_max + 1, n_r_max)) + 1j * rng.standard_normal((m_max + 1, n_r_max))
    r_cmb = 1.0 / 0.65
    x = np.cos(np.pi * np.arange(n_r_max) / (n_r_max - 1))
    r = 0.5 * x + r_cmb - 0.5
    header = dict(time=12.5, ra=1.0e5, ek=1.0e-3, pr=1.0, radratio=0.35, sc=0.0, raxi=0.0, m_max=m_max, minc=1,
                  r=r, tcond=np.log(r / r_cmb) / np.log(0.35), xicond=None)
    return header, field


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the pizza source tree (read only)")
    args = ap.parse_args()
    from pizza_gb300.pizza_io import write_frame
    header, field = sample()
    path = os.path.join(HERE, "frame_sample.bin")
    write_frame(path, header, field)
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.cm", "matplotlib.ticker"):
        mod = sys.modules.setdefault(name, types.ModuleType(name))
        mod.__version__ = "3.0.0"
    sys.dont_write_bytecode = True             # the reference tree stays untouched
    sys.path.insert(0, os.path.join(args.ref, "python"))
    from pizza.frame import Frame
    f = Frame(path)
    parsed = dict(version=int(f.version), time=float(f.time), ra=float(f.ra), ek=float(f.ek), pr=float(f.pr),
                  radratio=float(f.radratio), sc=float(f.sc), raxi=float(f.raxi), n_r_max=int(f.n_r_max),
                  n_m_max=int(f.n_m_max), m_max=int(f.m_max), minc=int(f.minc), n_phi_max=int(f.n_phi_max),
                  radius=[float(v) for v in f.radius], tcond=[float(v) for v in f.tcond],
                  idx2m=[int(v) for v in f.idx2m],
                  field_re=[[float(v) for v in row] for row in f.field_m.real],
                  field_im=[[float(v) for v in row] for row in f.field_m.imag])
    with open(os.path.join(HERE, "frame_sample.json"), "w") as out:
        json.dump(parsed, out, indent=1)


if __name__ == "__main__":
    main()

"""Run one pizza input.nml on the GPU: ``python -m pizza_gb300.run input.nml``.

The run follows time_loop's output cadence (src/step_time.f90:139-199): a
time-series row at step 0 and every n_log_step steps, then the time-series
files (e_kin, e_kin_3D, heat and, with composition, composition .TAG),
the final spectrum and checkpoint_end.TAG.  The start field is pizza's
initProp mode init_t > 0 (init_fields.f90:260-376: amp_t sin(pi (r - r_i))
on mode m = init_t), init_t = 0 (conduction state), or the checkpoint named
by start_file when l_start_file is set.  pizza's random start modes draw from
Fortran's generator, which cannot be reproduced; ``--seed`` replaces them by
a seeded perturbation of amplitude amp_t with a sin(pi (r - r_i)) envelope.
"""
import argparse
import os

import numpy as np

from . import Ensemble
from . import namelist, pizza_io


def start_temperature(cfg, ctl, seed=None):
    """The temperature perturbation of the start field, (n_m_max, n_r_max)."""
    n_m = cfg.m_max // cfg.minc + 1
    r = pizza_io._grid_r(cfg.n_r_max, cfg.radratio)
    r_icb = cfg.radratio / (1.0 - cfg.radratio)
    env = np.sin(np.pi * (r - r_icb))
    init_t, amp = int(ctl.get("init_t", 0)), float(ctl.get("amp_t", 0.0))
    t = np.zeros((n_m, cfg.n_r_max), np.complex128)
    if seed is not None:
        rng = np.random.default_rng(seed)
        ph = rng.uniform(0.0, 2.0 * np.pi, n_m - 1)
        a = rng.standard_normal(n_m - 1)
        t[1:] = (amp * a * np.exp(1j * ph))[:, None] * env[None, :]
    elif init_t > 0:
        if init_t % cfg.minc != 0 or init_t // cfg.minc >= n_m:
            raise ValueError(f"init_t = {init_t} is not a resolved mode")
        t[init_t // cfg.minc] = amp * env
    elif init_t != 0:
        raise ValueError(f"init_t = {init_t} draws from Fortran's random generator; pass --seed instead")
    return t


def run(path, directory=".", seed=None, n_steps=None):
    """Run the input.nml at ``path``; returns the paths written."""
    cfg, ctl, _ = namelist.read(path)
    tag = str(ctl.get("tag", "test"))
    n_time_steps = int(ctl.get("n_time_steps", 100)) if n_steps is None else int(n_steps)
    n_log = max(1, int(ctl.get("n_log_step", 50)))
    ens = Ensemble(cfg)
    if ctl.get("l_start_file", False):
        pizza_io.restart_from_checkpoint(ens, 0, str(ctl["start_file"]))
    else:
        ens.set_state(0, temp=start_temperature(cfg, ctl, seed))
    rows = [ens.latest_rows()[0].copy()]
    done = 0
    while done < n_time_steps:
        k = min(n_log, n_time_steps - done)
        ens.step(k)
        done += k
        rows.append(ens.latest_rows()[0].copy())
    os.makedirs(directory, exist_ok=True)
    paths = pizza_io.write_series(ens, 0, tag, directory, rows=np.array(rows))
    paths.append(pizza_io.write_spectrum(ens, 0, 1, tag, directory))
    ck = os.path.join(directory, f"checkpoint_end.{tag}")
    pizza_io.save_checkpoint(ens, 0, ck)
    paths.append(ck)
    return paths


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("nml")
    ap.add_argument("--dir", default=".")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None, help="override n_time_steps")
    a = ap.parse_args(argv)
    for p in run(a.nml, a.dir, a.seed, a.steps):
        print(p)


if __name__ == "__main__":
    main()

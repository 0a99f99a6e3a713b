"""Run one pizza input.nml on the GPU: ``python -m pizza_gb300.run input.nml``.

The run follows time_loop's output cadence (src/step_time.f90:139-199): a
time-series row at step 0 and every n_log_step steps, then the time-series
files (e_kin, e_kin_3D, heat and, with composition, composition .TAG),
the final spectrum and checkpoint_end.TAG.  The start state follows
get_start_fields (src/init_fields.f90:54-123): the checkpoint named by
start_file when l_start_file is set, else the conduction state; then
initProp adds the init_t perturbation to the temperature and, with
composition, the init_xi one to the composition (init_t > 0: one mode;
init_t = -1: the compact Gaussian bubble).  pizza's random start modes
(init_t < -1) draw from Fortran's generator, which cannot be reproduced:
``--seed`` replaces them by a seeded perturbation of amplitude amp_t.

Namelist names the GPU step does not use are printed.  Names that would
change the physics of the run (a velocity start, inhomogeneous boundary
temperatures, a phase field, a radial mapping, hyperdiffusion) are refused
instead of being dropped.
"""
import argparse
import os

import numpy as np

from . import Ensemble
from . import namelist, pizza_io
from .start_fields import init_prop, seeded_prop

# names whose value changes the problem this library solves
# (src/namelists.f90:530-672 defaults): refused rather than ignored
def _low(v):
    return str(v).strip().lower()


_PHYSICS = {
    "start_field.init_u": lambda v: v != 0, "start_field.init_phi": lambda v: v != 0,
    "start_field.scale_t": lambda v: v != 1.0, "start_field.scale_u": lambda v: v != 1.0,
    "start_field.scale_xi": lambda v: v != 1.0, "start_field.l_reset_t": lambda v: bool(v),
    "phys_param.t_bot": lambda v: True, "phys_param.t_top": lambda v: True,
    "phys_param.xi_bot": lambda v: True, "phys_param.xi_top": lambda v: True,
    "phys_param.stef": lambda v: v != 0.0, "phys_param.tmelt": lambda v: True,
    "phys_param.container": lambda v: _low(v) != "sphere",
    "phys_param.beta_shift": lambda v: v != 0.0, "phys_param.amp_forcing": lambda v: v != 0.0,
    "phys_param.l_temp_3d": lambda v: bool(v), "phys_param.l_xi_3d": lambda v: bool(v),
    "phys_param.tcond_fac": lambda v: v != 1.0,
    "control.l_newmap": lambda v: bool(v), "control.radial_scheme": lambda v: _low(v) != "cheb",
    "control.bc_method": lambda v: "gal" in _low(v), "control.c_sgs": lambda v: v != 0.0,
    "hdif.hdif_temp": lambda v: v != 0.0, "hdif.hdif_vel": lambda v: v != 0.0,
    "hdif.hdif_comp": lambda v: v != 0.0,
}


def _refused(ignored: dict):
    return [k for k, v in ignored.items() if k in _PHYSICS and _PHYSICS[k](v)]


def start_temperature(cfg, ctl, seed=None, field="temp"):
    """The initProp perturbation of the temperature (field "temp": init_t,
    amp_t) or composition ("xi": init_xi, amp_xi), (n_m_max, n_r_max)."""
    key = "t" if field == "temp" else "xi"
    init, amp = int(ctl.get(f"init_{key}", 0)), float(ctl.get(f"amp_{key}", 0.0))
    if init < -1:
        if seed is None:
            raise ValueError(f"init_{key} = {init} draws from Fortran's random generator; pass --seed instead")
        return seeded_prop(cfg.n_r_max, cfg.m_max, cfg.minc, cfg.radratio, amp, seed)
    return init_prop(cfg.n_r_max, cfg.m_max, cfg.minc, cfg.radratio, init, amp)


def run(path, directory=".", seed=None, n_steps=None):
    """Run the input.nml at ``path``; returns the paths written."""
    cfg, ctl, ignored = namelist.read(path)
    bad = _refused(ignored)
    if bad:
        raise ValueError("input sets options the GPU step does not implement: " + ", ".join(sorted(bad)))
    unused = sorted(k for k in ignored if k not in _PHYSICS)
    if unused:
        print("namelist names not used by the GPU step: " + ", ".join(unused))
    tag = str(ctl.get("tag", "test"))
    n_time_steps = int(ctl.get("n_time_steps", 100)) if n_steps is None else int(n_steps)
    n_log = max(1, int(ctl.get("n_log_step", 50)))
    ens = Ensemble(cfg)
    dT = start_temperature(cfg, ctl, seed)
    chem = cfg.raxi != 0.0
    dX = start_temperature(cfg, ctl, None if seed is None else seed + 1, "xi") if chem else None
    if ctl.get("l_start_file", False):
        pizza_io.restart_from_checkpoint(ens, 0, str(ctl["start_file"]), temp_add=dT, xi_add=dX)
    else:
        ens.set_state(0, temp=dT, xi=dX)
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

"""Shared helpers of the test suite: one workload description drives both
the oracle (oracle.pizza_oracle.Params) and the CUDA library
(pizza_gb300.Config)."""
import numpy as np

from oracle.pizza_oracle import Params, Pizza, seeded_temperature

ORACLE_ONLY = {"n_time_steps", "n_log_step", "init_t", "amp_t", "init_u", "amp_u", "init_xi", "amp_xi"}


def gpu_config(spec):
    import pizza_gb300 as pz
    kw = {k: v for k, v in spec.items() if k not in ORACLE_ONLY}
    return pz.Config(**kw)


def oracle(spec, temp0=None, xi0=None, integ_bordered=False):
    sim = Pizza(Params(**spec), integ_bordered=integ_bordered)
    sim.start(temp0=temp0, xi0=xi0)
    return sim


def seeded(spec, seed, amp=1e-3):
    sim = Pizza(Params(**spec))
    return seeded_temperature(sim.M, sim.r, sim.d["r_icb"], amp, seed)


def rel_err(a, b):
    """max |a - b| / max |b| (norm-wise relative error of a field)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def series_from_oracle(sim):
    """Oracle time-series row in the library's column order."""
    rows = sim.time_series()
    ek = rows["e_kin"]
    e3 = rows.get("e_kin_3D", [ek[0], 0.0, 0.0, 0.0, 0.0])
    ht = rows["heat"]
    ch = rows.get("composition", [0.0] * 7)
    return np.array([ek[0], ek[1], ek[2], ek[3], e3[1], e3[2], e3[3], e3[4],
                     ht[1], ht[2], ht[3], ht[4], ht[5], ht[6], ht[7], sim.ts.dt[0]] + list(ch[1:]))


def fp64_noise(sim, rng, level=1e-13, fields=("temp", "om")):
    """Add to the oracle's temperature and vorticity complex normal deviates
    of `level` times each field's largest modulus: the size of the rounding
    differences that another FP64 implementation (another summation order of
    the transforms and products) makes per step.  The m = 0 modes stay real.
    Run after every step, it measures how far the oracle drifts from itself
    under rounding alone.  (The integration method's prognostic variables
    are the temperature and the streamfunction: perturb its temperature only.)"""
    for f in fields:
        a = getattr(sim, f)
        s = level * np.max(np.abs(a))
        a = a + s * (rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape))
        a[0] = a[0].real
        setattr(sim, f, a)

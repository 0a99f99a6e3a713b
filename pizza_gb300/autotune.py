"""Launch-shape tuner of the GPU step, timed on the device.

pizza picks its MPI transpose variant by timing the candidates at start-up
(src/communications.f90:407-516).  The GPU step has two launch shapes whose
best value depends on the workload's grids:

- the tensor-core stage's instances per block G (k_fast): more instances
  share each operator fragment loaded from L2, fewer blocks fill the GPU;
- the phi-transform kernel's radii per block for each n_phi_max (k_rloop):
  more radii per block give the FFT stages more parallel work per barrier,
  fewer resident blocks per SM;
- the lanes of a step whose instances all run the tensor-core stage: more
  lanes overlap one lane's transforms with another's stage, but split the
  classes into more partly filled k_fast groups.

``tune(configs, ...)`` builds handles of the given instances (a workload's own
configurations), times every launch-shape candidate with CUDA events over the
kernels launched one by one (pz_step_profile) and every lane count over whole
steps (the lanes exist only in the step's graphs), and returns the table; ``apply``
installs a table for handles created afterwards (pz_tune_set) and
``save``/``load`` persist it as JSON.
"""
from __future__ import annotations

import json

import numpy as np

import time

from . import Ensemble, TUNE_FAST_G, TUNE_LANES, TUNE_RLOOP_RG, tune_set

FAST_G = (4, 8, 12, 16)
RLOOP_RG = (1, 2, 3, 4, 6, 8)
LANES = (1, 2, 4)
DEFAULT_LANES = 2


def _time(configs, temps, kernel, steps, warmup):
    ens = Ensemble(configs)
    try:
        ens.set_state_all(temps)
        ens.step(warmup)
        return ens.profile_steps(steps)[kernel]
    finally:
        ens.close()


def _time_steps(configs, temps, steps, warmup):
    """ms per whole step of a handle (host clock around pz_step(steps) and
    pz_sync, after the warm-up): the lanes run only inside pz_step."""
    ens = Ensemble(configs)
    try:
        ens.set_state_all(temps)
        ens.step(warmup)
        t0 = time.perf_counter()
        ens.step(steps)
        return (time.perf_counter() - t0) * 1e3 / steps
    finally:
        ens.close()


def tune(configs, temps, steps=10, warmup=3, fast_g=FAST_G, rloop_rg=RLOOP_RG, lanes=LANES, log=None):
    """Time the candidates for `configs` (a list of pizza_gb300.Config) started
    from `temps` (their initial temperature perturbations); returns
    {"k_fast_G": g, "k_rloop_rg": {n_phi_max: rg}, "lanes": l, "ms": {...}}
    with the per-step ms of every candidate and of the built-in defaults."""
    table = {"k_fast_G": None, "k_rloop_rg": {}, "lanes": None, "ms": {"k_fast": {}, "k_rloop": {}, "lanes": {}}}
    # k_fast: all instances together (its blocks mix classes)
    best = None
    for g in fast_g:
        tune_set(TUNE_FAST_G, 0, g)
        ms = _time(configs, temps, "k_fast", steps, warmup)
        table["ms"]["k_fast"][str(g)] = ms
        if log:
            log(f"k_fast G={g}: {ms:.4f} ms/step")
        if ms > 0.0 and (best is None or ms < best[1]):
            best = (g, ms)
    tune_set(TUNE_FAST_G, 0, 0)
    if best is not None:
        table["k_fast_G"] = best[0]
    # k_rloop: per n_phi_max class
    P_of = [3 * c.m_max // c.minc for c in configs]
    for P in sorted(set(P_of)):
        idx = [i for i, p in enumerate(P_of) if p == P]
        cf = [configs[i] for i in idx]
        tp = [temps[i] for i in idx]
        best = None
        table["ms"]["k_rloop"][str(P)] = {}
        for rg in rloop_rg:
            try:
                tune_set(TUNE_RLOOP_RG, P, rg)
            except Exception:
                continue                     # does not fit the shared memory
            ms = _time(cf, tp, "k_rloop", steps, warmup)
            table["ms"]["k_rloop"][str(P)][str(rg)] = ms
            if log:
                log(f"k_rloop P={P} rg={rg}: {ms:.4f} ms/step")
            if best is None or ms < best[1]:
                best = (rg, ms)
        tune_set(TUNE_RLOOP_RG, P, 0)
        table["ms"]["k_rloop"][str(P)]["default"] = _time(cf, tp, "k_rloop", steps, warmup)
        if best is not None:
            table["k_rloop_rg"][str(P)] = best[0]
    # lanes: whole steps of the whole workload (its own G and radii per block)
    apply({k: table[k] for k in ("k_fast_G", "k_rloop_rg")})
    best = None
    for n in lanes:
        tune_set(TUNE_LANES, 0, n)
        ms = _time_steps(configs, temps, 4 * steps, warmup)
        table["ms"]["lanes"][str(n)] = ms
        if log:
            log(f"lanes {n}: {ms:.4f} ms/step")
        if best is None or ms < best[1]:
            best = (n, ms)
    reset(table)
    if best is not None:
        table["lanes"] = best[0]
    return table


def apply(table):
    """Install a tuning table for handles created afterwards."""
    if table.get("k_fast_G"):
        tune_set(TUNE_FAST_G, 0, int(table["k_fast_G"]))
    for P, rg in table.get("k_rloop_rg", {}).items():
        tune_set(TUNE_RLOOP_RG, int(P), int(rg))
    if table.get("lanes"):
        tune_set(TUNE_LANES, 0, int(table["lanes"]))


def reset(table=None):
    """Back to the built-in launch shapes."""
    tune_set(TUNE_FAST_G, 0, 0)
    tune_set(TUNE_LANES, 0, 0)
    for P in (table or {}).get("k_rloop_rg", {}):
        tune_set(TUNE_RLOOP_RG, int(P), 0)


def save(table, path):
    with open(path, "w") as f:
        json.dump(table, f, indent=1)


def load(path):
    with open(path) as f:
        return json.load(f)


def gain(table):
    """Default over tuned per-step ms of each tuned kernel (>= 1 is a gain)."""
    out = {}
    ms = table["ms"]
    if table.get("k_fast_G") and str(8) in ms["k_fast"]:
        out["k_fast"] = ms["k_fast"]["8"] / ms["k_fast"][str(table["k_fast_G"])]
    tot_d = tot_t = 0.0
    for P, rg in table.get("k_rloop_rg", {}).items():
        d = ms["k_rloop"][P]
        tot_d += d["default"]
        tot_t += d[str(rg)]
    if tot_t > 0:
        out["k_rloop"] = tot_d / tot_t
    lm = ms.get("lanes", {})
    if table.get("lanes") and str(DEFAULT_LANES) in lm and str(table["lanes"]) in lm:
        out["lanes"] = lm[str(DEFAULT_LANES)] / lm[str(table["lanes"])]
    return {k: float(np.round(v, 4)) for k, v in out.items()}


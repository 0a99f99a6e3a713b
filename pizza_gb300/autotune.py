"""Launch-shape tuner of the GPU step, timed on the device.

pizza picks its MPI transpose variant by timing the candidates at start-up
(src/communications.f90:407-516).  The GPU step has two launch shapes whose
best value depends on the workload's grids:

- the tensor-core stage's instances per block G (k_fast): more instances
  share each operator fragment loaded from L2, fewer blocks fill the GPU;
- the phi-transform kernel's radii per block for each n_phi_max (k_rloop):
  more radii per block give the FFT stages more parallel work per barrier,
  fewer resident blocks per SM.

``tune(configs, ...)`` builds handles of the given instances (a workload's own
configurations), times every candidate with CUDA events over the kernels
launched one by one (pz_step_profile), and returns the table; ``apply``
installs a table for handles created afterwards (pz_tune_set) and
``save``/``load`` persist it as JSON.
"""
from __future__ import annotations

import json

import numpy as np

from . import Ensemble, TUNE_FAST_G, TUNE_RLOOP_RG, tune_set

FAST_G = (4, 8, 12, 16)
RLOOP_RG = (1, 2, 3, 4, 6, 8)


def _time(configs, temps, kernel, steps, warmup):
    ens = Ensemble(configs)
    try:
        ens.set_state_all(temps)
        ens.step(warmup)
        return ens.profile_steps(steps)[kernel]
    finally:
        ens.close()


def tune(configs, temps, steps=10, warmup=3, fast_g=FAST_G, rloop_rg=RLOOP_RG, log=None):
    """Time the candidates for `configs` (a list of pizza_gb300.Config) started
    from `temps` (their initial temperature perturbations); returns
    {"k_fast_G": g, "k_rloop_rg": {n_phi_max: rg}, "ms": {...}} with the
    per-step device ms of every candidate and of the built-in defaults."""
    table = {"k_fast_G": None, "k_rloop_rg": {}, "ms": {"k_fast": {}, "k_rloop": {}}}
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
    return table


def apply(table):
    """Install a tuning table for handles created afterwards."""
    if table.get("k_fast_G"):
        tune_set(TUNE_FAST_G, 0, int(table["k_fast_G"]))
    for P, rg in table.get("k_rloop_rg", {}).items():
        tune_set(TUNE_RLOOP_RG, int(P), int(rg))


def reset(table=None):
    """Back to the built-in launch shapes."""
    tune_set(TUNE_FAST_G, 0, 0)
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
    return {k: float(np.round(v, 4)) for k, v in out.items()}


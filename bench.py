"""Benchmark of the GB300 pizza time step.

Workload (the batched ensemble the headline metric is quoted on): a batched ensemble of B independent annulus instances of uneven size,
n_r_max in {33, 49, 65}, n_phi_max in {96, 192, 288} (m_max = n_phi_max/3),
log10 Ra ~ U[5, log10 Ra_max(n_r_max)] with Ra_max = 1e6, 3e6, 1e7 for
n_r_max = 33, 49, 65 (the resolution that keeps a 500-step run stable; 1e7 at
n_r_max = 33 is not), E in {1e-3, 1e-4}, Pr = 1, radius ratio 0.35, Ekman
pumping, CNAB2 with per-instance CFL time steps at CFL number 0.5 (pizza's
courfac = 2: dt = dr / (courfac |u|)), dtMax = min(1e-4, 0.03/sqrt(Ra)),
collocation with the influence-matrix solve, each instance started from its
own seeded temperature perturbation of amplitude 1e-3 (synthetic data: the
reference publishes no dataset).  One step advances every instance by one
time step; the default timed region is the ensemble's 500 steps.

Metric: aggregate instance-steps/s of the batched step (``value``), next to the
plain one-instance-per-handle GPU step of the same instances
(``plain_steps_per_s``); their ratio is the reference's headline quantity.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "aggregate steps/s batched vs plain GPU step at 1e-10 rel err; adjoint/forward time"
UNIT = "instance-steps/s"
NS = (33, 49, 65)
PS = (96, 192, 288)
RA_MAX = {33: 1.0e6, 49: 3.0e6, 65: 1.0e7}


def ensemble_specs(n_inst: int, seed: int = 1234):
    """The batched workload: per-instance namelist values and seeds."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_inst):
        N = int(rng.choice(NS))
        P = int(rng.choice(PS))
        ra = float(10.0 ** rng.uniform(5.0, math.log10(RA_MAX[N])))
        ek = float(rng.choice([1e-3, 1e-4]))
        specs.append(dict(n_r_max=N, n_cheb_max=N, m_max=P // 3, ra=ra, ek=ek, pr=1.0, radratio=0.35,
                          l_ek_pump=True, time_scheme="CNAB2", courfac=2.0,
                          dtMax=min(1e-4, 0.03 / math.sqrt(ra)), matrix_solve="INFLUENCE",
                          seed=int(seed * 1000 + i)))
    return specs


def seeded_temp(spec, amp=1e-3):
    """Seeded perturbation T(m,r) = amp g_m e^{i theta_m} sin(pi (r - r_i)), m >= 1."""
    N, M = spec["n_r_max"], spec["m_max"] + 1
    r_cmb = 1.0 / (1.0 - spec["radratio"])
    r_icb = r_cmb - 1.0
    x = np.cos(np.pi * np.arange(N) / (N - 1))
    r = 0.5 * (r_cmb - r_icb) * x + 0.5 * (r_cmb + r_icb)
    rng = np.random.default_rng(spec["seed"])
    g = rng.standard_normal(M - 1)
    th = rng.uniform(0.0, 2.0 * np.pi, M - 1)
    T = np.zeros((M, N), complex)
    T[1:, :] = (amp * g * np.exp(1j * th))[:, None] * np.sin(np.pi * (r - r_icb))[None, :]
    return T


def gpu_cfg(spec):
    import pizza_gb300 as pz
    kw = {k: v for k, v in spec.items() if k != "seed"}
    return pz.Config(**kw)


# ---------------------------------------------------------------------------
# algorithmic work of the step's kernels
# ---------------------------------------------------------------------------
OZ_S = 7            # bf16 slices per FP64 operand in the tensor-core stage (pz_fast.h)
FAST_G = 8          # instances per k_fast block


def mloop_work(specs, nold=1, nimp=1, nexp=2):
    """Algorithmic HBM bytes and FP64 flops of one dense stage launch
    (k_mloop / k_build_mloop) over the batch.

    Per (instance, m): the per-m operators (the vorticity operator, which at
    Pr = 1 is also the temperature operator, and the streamfunction operator;
    N x N FP64 each; m = 0: temperature and u_phi), the
    influence vectors (4N + 4 doubles), the state it reads (dVsT, dVsOm, us, up,
    om, T: 6 complex N-vectors) and the history slots of both equations
    (2 (nold + nimp + nexp) complex N-vectors), and what it writes (T, dT/dr,
    us, up, om, psi, two explicit, two old and two implicit slots: 12 complex
    N-vectors).  The Chebyshev operators shared by all m of one size are
    counted once per size.  Flops: per m, 3 dense real-operator x complex-vector
    products (4N^2 flops each: temperature/vorticity operator twice, the
    streamfunction operator K once) and 7 products with the parity-compact
    Chebyshev operators (2N^2 flops each: D1p of dVsT and dVsOm, C and D1c of
    T and of psi, C of omega); m = 0: 2 dense (temperature, u_phi) and 6
    compact.  Elementwise work and operator rebuilds are neglected.
    """
    byts = 0.0
    flops = 0.0
    sizes = set()
    for s in specs:
        N, M = s["n_r_max"], s["m_max"] + 1
        sizes.add(N)
        per_m = 8.0 * 2 * N * N + 8.0 * (4 * N + 4) + 16.0 * N * (6 + 2 * (nold + nimp + nexp) + 12)
        m0 = 8.0 * 2 * N * N + 16.0 * N * (6 + 2 * (nold + nimp + nexp) + 12)
        byts += (M - 1) * per_m + m0
        flops += (M - 1) * (3 * 4.0 + 7 * 2.0) * N * N + (2 * 4.0 + 6 * 2.0) * N * N
    for N in sizes:
        byts += 8.0 * 4 * N * N
    return byts, flops


def fast_work(specs, G=FAST_G, S=OZ_S):
    """Work of one k_fast launch over the batch (every instance on the fast
    path): (FP64-equivalent flops, bf16 mma flops issued, HBM bytes).

    Per (instance, m), with n = N - 2 interior points, the stage applies
    D1p (N x N) to 4 real columns (dVsT, dVsOm), U^-1 (n x n) to 2 + 2
    (temperature, vorticity right-hand sides), [U; D1p U] ((n+N) x n) to 2 and
    [U; K U; D1p K U] ((2n+N) x n; m = 0: [U; D1p U]) to 2: 2 R K flops per
    real column is the FP64-equivalent work.  A block serves G instances of
    one (N, m); its mma.sync m16n8k16 count per product is
    ceil(R/16) ceil(K/16) * S(S+1)/2 slice pairs * ceil(C/8) column tiles
    (C = 4g or 2g real columns for g instances), 4096 flops each.  HBM bytes
    are the state the stage reads and writes (the operators, shared per
    (N, m), come from L2): per (instance, m) 28 complex N-vectors.
    """
    def t16(x):
        return (x + 15) // 16
    pairs = S * (S + 1) // 2
    f64 = mma = byts = 0.0
    groups = {}
    for s in specs:
        N, M = s["n_r_max"], s["m_max"] + 1
        n = N - 2
        for m in range(M):
            f64 += 2.0 * (4 * N * N + 4 * n * n + 2 * (n + N) * n + 2 * ((2 * n + N) if m else (n + N)) * n)
            byts += 16.0 * N * 28
            key = (N, m, s["ek"] if m == 0 else None)      # m = 0 groups share their u_phi operator
            groups[key] = groups.get(key, 0) + 1
    for (N, m, _), cnt in groups.items():
        n = N - 2
        r3 = (2 * n + N) if m else (n + N)
        for a in range(0, cnt, G):
            g = min(G, cnt - a)
            tiles = (t16(N) * t16(N) * ((4 * g + 7) // 8) + 2 * t16(n) * t16(n) * ((2 * g + 7) // 8) +
                     (t16(n + N) + t16(r3)) * t16(n) * ((2 * g + 7) // 8))
            mma += 4096.0 * pairs * tiles
    return f64, mma, byts


def rloop_work(specs):
    """FP64 flops of one k_rloop launch: per (instance, radius) four complex
    FFTs of length P (two to the grid, two back), counted as 5 P log2 P each,
    the grid products and Courant squares (8 P) and the spectral packing and
    -i m / r post-multiply (20 M)."""
    f = 0.0
    for s in specs:
        N, M = s["n_r_max"], s["m_max"] + 1
        P = 3 * s["m_max"]
        f += N * (4 * 5.0 * P * math.log2(P) + 8.0 * P + 20.0 * M)
    return f


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                if int(f[0]) != dev:
                    continue
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (read + write) of one launch of the stage kernel (k_build_mloop,
# a step without rebuilds) over its algorithmic bytes, from an ncu capture of
# the 16-instance ensemble (same generator and seed): 84.0 MB measured for
# 81.9 MB algorithmic.  The 256-instance launch is too
# large to capture under the profiling rules; its traffic is this ratio times
# its algorithmic bytes (traffic grows with the (instance, m) items processed).
MLOOP_TRAFFIC_PER_ALGO_BYTE = 83.97e6 / 81868128.0
# k_rloop: DRAM bytes (read + write) per launch over its algorithmic bytes, the
# four input and four output (m, r) planes of every instance (16 * 8 M N),
# from an ncu capture of the 16-instance ensemble (profiles/launch_list_ensemble256_fast.md);
# the traffic scales with the instances, so the ratio carries to 256
RLOOP_TRAFFIC_PER_ALGO_BYTE = (7927936.0 + 32128.0) / 7725056.0


def rloop_bytes(specs):
    """Algorithmic bytes of one k_rloop launch: 4 input and 4 output planes of
    (m, r) complex values per instance."""
    return 8 * 16.0 * sum((s["m_max"] + 1) * s["n_r_max"] for s in specs)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured_bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


# ---------------------------------------------------------------------------
# CPU baselines (oracle port)
# ---------------------------------------------------------------------------
def _cpu_class_time(args):
    spec, nsteps = args
    from oracle.pizza_oracle import Params, Pizza
    kw = {k: v for k, v in spec.items() if k != "seed"}
    sim = Pizza(Params(**kw))
    sim.start(temp0=seeded_temp(spec))
    sim.advance()                       # builds the matrices
    t0 = time.perf_counter()
    for _ in range(nsteps):
        sim.advance()
    return (time.perf_counter() - t0) / nsteps


def cpu_baseline(specs, nsteps=4):
    """Single-core oracle, one instance per size class, scaled to the batch."""
    classes = {}
    for s in specs:
        classes.setdefault((s["n_r_max"], s["m_max"]), []).append(s)
    t_class = {k: _cpu_class_time((v[0], nsteps)) for k, v in classes.items()}
    t_step = sum(t_class[(s["n_r_max"], s["m_max"])] for s in specs)
    return {"value": len(specs) / t_step, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (NumPy/SciPy FP64) {nsteps} steps of one instance per (n_r_max, m_max) class "
                      f"({len(classes)} classes), scaled by the class counts of the {len(specs)}-instance batch"}


def workload_config(specs):
    return {"workload": f"batched ensemble of {len(specs)} annulus instances per GPU: "
                        "n_r_max in {33,49,65}, n_phi_max in {96,192,288}, Ra log-uniform [1e5, Ra_max(N)] "
                        "with Ra_max = 1e6/3e6/1e7 for N = 33/49/65, E in {1e-3,1e-4}, CNAB2, CFL 0.5, "
                        "collocation + influence matrix",
            "instances": len(specs), "l2": "working set (operators + state, GBs) far larger than L2",
            "solve": "INFLUENCE"}


def _cpu_instance_time(args):
    """One instance of the workload on one core: start, `warmup` untimed
    steps (the first builds the matrices), then `steps` timed steps."""
    spec, warmup, steps = args
    from oracle.pizza_oracle import Params, Pizza
    kw = {k: v for k, v in spec.items() if k != "seed"}
    sim = Pizza(Params(**kw))
    sim.start(temp0=seeded_temp(spec))
    for _ in range(max(1, warmup)):
        sim.advance()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.advance()
    return time.perf_counter() - t0


# a bound on the reference arm's CPU work: instance-steps it may run in all
# (about a minute on 16 host cores at the workload's ~7 ms per instance-step)
REF_MAX_INSTANCE_STEPS = 256 * 520


def reference_arm(args, specs):
    """--impl reference: the oracle port of the reference's CPU algorithm on
    all host cores, one process per core, over the same workload as the GPU
    arm (every instance, W warm-up and K timed steps each) unless that
    exceeds REF_MAX_INSTANCE_STEPS, in which case the steps are cut to fit
    and the line says so."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    warmup = max(3, args.warmup)
    steps = max(1, min(args.steps, REF_MAX_INSTANCE_STEPS // max(1, len(specs)) - warmup))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        per = pool.map(_cpu_instance_time, [(s, warmup, steps) for s in specs])
    wall = time.perf_counter() - t0
    # aggregate rate of `cores` workers each stepping its share of the instances
    rate = len(specs) * steps / (sum(per) / cores)
    same = steps == args.steps
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 0,
            "steps": steps, "warmup": warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": workload_config(specs),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"all {len(specs)} instances x {steps} timed steps (after {warmup} "
                                       f"untimed) of the oracle port, one process per core; wall {wall:.1f}s "
                                       "incl. matrix set-up" + ("" if same else
                                       f"; steps cut from {args.steps} to bound the run")},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_steps(ens, k, torch):
    s = torch.cuda.ExternalStream(ens.stream_ptr)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    ens.step(k, sync=False)
    e1.record(s)
    e1.synchronize()
    ens.sync()
    return e0.elapsed_time(e1)


def plain_rate(specs, steps, warmup, torch):
    """Plain GPU step: one instance per handle, stepped one after another.
    One instance per (n_r_max, m_max) class is timed; the batch time is the
    sum over instances of their class's per-step time."""
    import pizza_gb300 as pz
    classes = {}
    for s in specs:
        classes.setdefault((s["n_r_max"], s["m_max"]), s)
    t_class = {}
    for key, s in classes.items():
        e = pz.Ensemble(gpu_cfg(s))
        e.set_state(0, temp=seeded_temp(s))
        e.step(warmup)
        t_class[key] = time_steps(e, steps, torch) / steps
        e.close()
    t_step_ms = sum(t_class[(s["n_r_max"], s["m_max"])] for s in specs)
    return len(specs) / (t_step_ms * 1e-3), {f"{k[0]}x{3 * k[1]}": v for k, v in t_class.items()}


# the single large integration-method instance (sparse Chebyshev, tau rows):
# n_r_max=97, n_phi_max=384, E=1e-5, Ra=3e7, SBDF3, dt=2e-6, amplitude 1e-4
INTEG_SPEC = dict(n_r_max=97, n_cheb_max=97, m_max=128, ek=1e-5, ra=3e7, pr=1.0, radratio=0.35, l_ek_pump=True,
                  time_scheme="SBDF3", dtMax=2e-6, cheb_method="INTEG", matrix_solve="DIRECT", seed=3)


def integ_leg(torch, steps=200, warmup=5):
    """Steps/s of the integration-method instance on its own handle (graph
    replay) and its per-kernel times; parity with the oracle is in the tests."""
    import pizza_gb300 as pz
    ens = pz.Ensemble(gpu_cfg(INTEG_SPEC))
    ens.set_state(0, temp=seeded_temp(INTEG_SPEC, amp=1e-4))
    ens.step(warmup)
    ms = time_steps(ens, steps, torch)
    kms = ens.profile_steps(5)
    ens.close()
    return {"workload": "one integ instance: n_r_max=97, n_phi_max=384, E=1e-5, Ra=3e7, SBDF3, dt=2e-6",
            "steps": steps, "steps_per_s": steps / (ms * 1e-3), "ms_per_step": ms / steps,
            "kernel_ms_per_step": {k: v for k, v in kms.items() if v > 0.0}}


ADJ_SPEC = dict(n_r_max=65, n_cheb_max=65, m_max=64, ek=1e-4, ra=2e6, pr=1.0, radratio=0.35, l_ek_pump=True,
                time_scheme="CNAB2", dtMax=5e-5, matrix_solve="INFLUENCE", seed=1)
ADJ_STEPS, ADJ_WINDOW, ADJ_CK = 500, 250, 50


def adjoint_ratio(torch, reps=3, checkpoint_every=ADJ_CK, n_steps=ADJ_STEPS, n_window=ADJ_WINDOW):
    """Cost of the kinetic-energy gradient (forward sweep with checkpoints +
    backward sweep with recomputation) over a plain forward run of the same
    500 steps, single instance N=65, n_phi=192, E=1e-4, Ra=2e6.  Both are
    wall-clock times from pz_set_state to the result on the host (J and the
    gradient, or the synchronised final state)."""
    import pizza_gb300 as pz
    spec = ADJ_SPEC
    t0 = seeded_temp(spec)
    ens = pz.Ensemble(gpu_cfg(spec))
    fw, gr, sw, bw = [], [], [], []
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        a = time.perf_counter()
        ens.set_state(0, temp=t0)
        ens.step(n_steps)
        b = time.perf_counter()
        ens.set_state(0, temp=t0)
        J, dt = ens.adjoint_forward(n_steps, n_window, checkpoint_every)
        c = time.perf_counter()
        g, dra = ens.adjoint_backward()
        d = time.perf_counter()
        if rep == 0:
            continue          # warm-up: graph capture, workspace allocation
        fw.append(b - a); gr.append(d - b); sw.append(c - b); bw.append(d - c)
    ens.close()
    med = lambda x: float(np.median(x))
    return {"workload": "adjoint gradient: N=65, n_phi=192, E=1e-4, Ra=2e6, CNAB2, dtMax=5e-5 under the Courant "
                        f"controller, {n_steps} steps, J = mean e_kin_3D over the last {n_window} states, "
                        f"checkpoint every {checkpoint_every if checkpoint_every > 0 else n_steps} steps",
            "forward_ms": 1e3 * med(fw), "gradient_ms": 1e3 * med(gr),
            "sweep_ms": 1e3 * med(sw), "backward_ms": 1e3 * med(bw),
            "adjoint_over_forward": med(gr) / med(fw),
            "J": float(J[0]), "dJ_dra": float(dra[0]), "distinct_dt": int(len(np.unique(dt)))}


# dt: 5e-5 is unstable for ARS233 with the influence-matrix solve at E = 1e-4
# (explicit Coriolis; the oracle's run of the same step blows up near step
# 50), 1e-5 is the largest power-of-ten step stable for all 300 steps
BADJ_STEPS, BADJ_CK, BADJ_DT = 300, 30, 1e-5


def batched_adjoint_specs(n_inst=64, seed=4321):
    """The batched adjoint ensemble: n_r_max in {49, 65}, n_phi_max in {126, 192}
    (m_max 42 or 64: n_phi_max = 3 m_max, so 128 is taken as 126), Ra
    log-uniform in [1e6, 1e7], E = 1e-4, Pr = 1, ARS233, influence matrix."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_inst):
        n = int(rng.choice([49, 65]))
        mm = int(rng.choice([42, 64]))
        ra = float(10.0 ** rng.uniform(6.0, 7.0))
        specs.append(dict(n_r_max=n, n_cheb_max=n, m_max=mm, ek=1e-4, ra=ra, pr=1.0, radratio=0.35,
                          l_ek_pump=True, time_scheme="ARS233", dtMax=BADJ_DT, matrix_solve="INFLUENCE",
                          seed=seed + i))
    return specs


def batched_adjoint_leg(torch, reps=2, n_fd=4, checkpoint_every=BADJ_CK, fd=True, n_steps=BADJ_STEPS):
    """Batched adjoint ensemble (64 instances, ARS233 with its assembly stage,
    dt = 1e-5, 300 steps, checkpoint every 30): cost of every instance's
    gradient of its time-averaged NuTop over the whole run with respect to
    its initial temperature perturbation, over a plain forward run of the
    same ensemble; and central finite differences of the forward sweep along
    one seeded direction on n_fd instances, eps = 1e-4 relative to the
    perturbation (J = mean NuTop is 1 + O(1e-2): below 1e-5 the difference
    quotient is dominated by the rounding of J, above it agrees with the
    adjoint to better than 1e-6)."""
    import pizza_gb300 as pz
    specs = batched_adjoint_specs()
    temps = [seeded_temp(s) for s in specs]
    ens = pz.Ensemble([gpu_cfg(s) for s in specs])
    sched = np.full((len(specs), n_steps), BADJ_DT)
    fw, gr, sw, bw = [], [], [], []
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        a = time.perf_counter()
        ens.set_state_all(temps)
        ens.step(n_steps)
        b = time.perf_counter()
        ens.set_state_all(temps)
        J, dt = ens.adjoint_forward(n_steps, n_steps, checkpoint_every, sched, objective="nutop")
        c = time.perf_counter()
        g, _ = ens.adjoint_backward()
        d = time.perf_counter()
        if rep == 0:
            continue
        fw.append(b - a)
        gr.append(d - b)
        sw.append(c - b)
        bw.append(d - c)
    # finite differences on n_fd instances
    rng = np.random.default_rng(77)
    errs = []
    for inst in range(n_fd if fd else 0):
        d = rng.standard_normal(temps[inst].shape) + 1j * rng.standard_normal(temps[inst].shape)
        d[0] = d[0].real
        eps = 1e-4 * np.max(np.abs(temps[inst])) / np.max(np.abs(d))
        jj = []
        for sgn in (1.0, -1.0):
            tp = list(temps)
            tp[inst] = temps[inst] + sgn * eps * d
            ens.set_state_all(tp)
            Jp, _ = ens.adjoint_forward(n_steps, n_steps, checkpoint_every, sched, objective="nutop")
            jj.append(Jp[inst])
        fd = (jj[0] - jj[1]) / (2 * eps)
        ad = float(np.sum((np.conj(g[inst]) * d).real))
        errs.append(abs(fd - ad) / abs(fd))
    ens.close()
    med = lambda x: float(np.median(x))
    return {"workload": f"batched adjoint ensemble: {len(specs)} instances, n_r_max in {{49,65}}, n_phi_max in "
                        "{126,192}, Ra log-uniform [1e6,1e7], E=1e-4, ARS233 (assembly stage), dt=1e-5, "
                        f"{n_steps} steps, checkpoint every "
                        f"{checkpoint_every if checkpoint_every > 0 else n_steps}, J_i = mean NuTop over the run, "
                        "gradient w.r.t. each instance's initial temperature perturbation",
            "forward_ms": 1e3 * med(fw), "gradient_ms": 1e3 * med(gr), "sweep_ms": 1e3 * med(sw),
            "backward_ms": 1e3 * med(bw), "adjoint_over_forward": med(gr) / med(fw),
            "fd_instances": len(errs), "fd_eps_rel": 1e-4, "fd_max_rel_err": max(errs) if errs else None,
            "fd_rel_errs": errs}


# ---------------------------------------------------------------------------
# replicas (one process per GPU under torchrun): the instances are
# independent, so every rank steps its own ensemble (a seed of its own) and
# the only collective is the max of the timed windows
# ---------------------------------------------------------------------------
def rank_specs(n_inst, seed, rank):
    """The ensemble of one rank: the same size mix, its own seeds."""
    return ensemble_specs(n_inst, seed=seed + 7919 * rank)


def max_over_ranks(ms, dist, device):
    """The slowest rank's timed window (ms); dist None on one process."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, n_inst, steps, ms):
    """Instance-steps/s of the whole job: every rank advanced n_inst
    instances by `steps` steps within the slowest rank's ms."""
    return world * n_inst * steps / (ms * 1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-integ", action="store_true")
    ap.add_argument("--integ-only", action="store_true", help="print only the integration-method measurement")
    ap.add_argument("--integ-steps", type=int, default=200)
    ap.add_argument("--adjoint-only", action="store_true", help="print only the adjoint/forward measurement")
    ap.add_argument("--adj-steps", type=int, default=ADJ_STEPS)
    ap.add_argument("--adj-reps", type=int, default=3)
    ap.add_argument("--batched-adjoint-only", action="store_true",
                    help="print only the batched DIRK adjoint measurement")
    ap.add_argument("--badj-steps", type=int, default=BADJ_STEPS)
    ap.add_argument("--badj-ck", type=int, default=BADJ_CK)
    ap.add_argument("--badj-reps", type=int, default=2)
    ap.add_argument("--badj-fd", type=int, default=4)
    ap.add_argument("--tune", default="auto", choices=["auto", "run", "off"],
                    help="launch shapes: auto = the committed table if present, else tune now; run = tune now; "
                         "off = built-in defaults")
    ap.add_argument("--tune-table", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "pizza_gb300",
                                                          "tuning_gb300.json"))
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    specs = rank_specs(args.instances, args.seed, rank)

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, specs)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from __graft_entry__ import build
    build()
    import pizza_gb300 as pz

    if args.integ_only:
        if rank == 0:
            print(json.dumps({"integ": integ_leg(torch, args.integ_steps, args.warmup)}))
        return

    if args.batched_adjoint_only:
        if rank == 0:
            out = {"batched_adjoint": batched_adjoint_leg(torch, args.badj_reps, args.badj_fd, args.badj_ck,
                                                          args.badj_fd > 0, args.badj_steps)}
            if args.badj_steps == BADJ_STEPS:
                out["batched_adjoint_stored"] = batched_adjoint_leg(torch, checkpoint_every=0, fd=False)
            print(json.dumps(out))
        return

    if args.adjoint_only:
        if rank == 0:
            n, w = args.adj_steps, max(1, args.adj_steps // 2)
            print(json.dumps({"adjoint": adjoint_ratio(torch, args.adj_reps, ADJ_CK, n, w),
                              "adjoint_no_recompute": adjoint_ratio(torch, args.adj_reps, 0, n, w)}))
        return

    temps = [seeded_temp(s) for s in specs]
    tuning = None
    if args.tune != "off":
        from pizza_gb300 import autotune
        t0 = time.perf_counter()
        if args.tune == "auto" and os.path.exists(args.tune_table):
            table = autotune.load(args.tune_table)
            source = "table " + os.path.relpath(args.tune_table, os.path.dirname(os.path.abspath(__file__)))
        else:
            table = autotune.tune([gpu_cfg(s) for s in specs], temps)
            source = "tuned in this run on this workload"
            out_dir = os.environ.get("PZ_REPORT_DIR", "")
            if out_dir and os.path.isdir(out_dir):
                autotune.save(table, os.path.join(out_dir, "tuning_gb300.json"))
        autotune.apply(table)
        tuning = {"source": source, "k_fast_G": table.get("k_fast_G"), "k_rloop_rg": table.get("k_rloop_rg"),
                  "lanes": table.get("lanes"),
                  "gain_over_defaults": autotune.gain(table), "candidates_ms_per_step": table.get("ms"),
                  "seconds": time.perf_counter() - t0}
    ens = pz.Ensemble([gpu_cfg(s) for s in specs])
    ens.set_state_all(temps)
    ens.step(args.warmup)

    # ---- device-resident timed region
    clocks = Clocks()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms = time_steps(ens, args.steps, torch)
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist, "cuda")
    value = aggregate_rate(world, len(specs), args.steps, ms)

    # ---- per-kernel device times over the same steps as the timed window:
    # the same start state and warm-up, then the timed window's steps with
    # the kernels launched one by one between CUDA events
    ens.set_state_all(temps)
    ens.step(args.warmup)
    kms = ens.profile_steps(args.steps)
    dom = max(kms, key=kms.get)
    hbm_peak, peak_kind = measured_peaks()
    try:
        dfma_peak, mma_peak = pz.probe_peaks()
    except Exception:
        dfma_peak, mma_peak = None, None
    bf16_peak = measured_bf16_peak()
    kernels = {}
    if kms.get("k_rloop", 0.0) > 0.0:
        f = rloop_work(specs)
        a_t = f / (kms["k_rloop"] * 1e-3) / 1e12
        rb = rloop_bytes(specs)
        kernels["k_rloop"] = {"bound": "fp64", "achieved": a_t, "peak": dfma_peak, "unit": "TFLOP/s",
                              "frac": a_t / dfma_peak if dfma_peak else None,
                              "traffic": RLOOP_TRAFFIC_PER_ALGO_BYTE * rb,
                              "hbm": {"achieved": rb / (kms["k_rloop"] * 1e-3) / 1e9, "peak": hbm_peak,
                                      "unit": "GB/s", "frac": rb / (kms["k_rloop"] * 1e-3) / 1e9 / hbm_peak,
                                      "bytes": rb},
                              "work": f, "work_note": "4 complex FFTs of length n_phi_max per (instance, radius) "
                                                      "at 5 P log2 P flops, plus 8 P + 20 M elementwise",
                              "peak_kind": "DFMA issue rate measured in this run (pz_probe_peaks)"}
    if kms.get("k_fast", 0.0) > 0.0:
        f64, mma, fb = fast_work(specs)
        t = kms["k_fast"] * 1e-3
        kernels["k_fast"] = {"bound": "tensor", "achieved": mma / t / 1e12, "peak": mma_peak, "unit": "TFLOP/s",
                             "frac": (mma / t / 1e12 / mma_peak) if mma_peak else None,
                             "frac_of_tcgen05_bf16": mma / t / 1e12 / bf16_peak,
                             "mma_flops": mma, "fp64_equivalent_tflops": f64 / t / 1e12,
                             "fp64_equivalent_flops": f64,
                             "hbm": {"achieved": fb / t / 1e9, "peak": hbm_peak, "unit": "GB/s",
                                     "frac": fb / t / 1e9 / hbm_peak, "bytes": fb},
                             "peak_kind": "bf16 mma.sync issue rate measured in this run (pz_probe_peaks); "
                                          "frac_of_tcgen05_bf16 against MEASURED_PEAKS bf16_tflops"}
    for name in ("k_build_mloop", "k_mloop"):
        if kms.get(name, 0.0) > 0.0:
            byts, flops = mloop_work(specs)
            t = kms[name] * 1e-3
            kernels[name] = {"bound": "fp64", "achieved": flops / t / 1e12, "peak": dfma_peak, "unit": "TFLOP/s",
                             "frac": flops / t / 1e12 / dfma_peak if dfma_peak else None,
                             "hbm": {"achieved": byts / t / 1e9, "peak": hbm_peak, "unit": "GB/s",
                                     "frac": byts / t / 1e9 / hbm_peak,
                                     "traffic": MLOOP_TRAFFIC_PER_ALGO_BYTE * byts}}
    roof = dict(kernels.get(dom, {}))
    roof["kernel"] = dom
    roof["traffic"] = kernels.get(dom, {}).get("traffic")
    roof["traffic_note"] = ("DRAM bytes (read + write) per launch of the dominant kernel: its algorithmic bytes "
                            "times the DRAM/algorithmic ratio of an ncu capture (profiles/), where the kernel's "
                            "traffic scales with the instances; null otherwise")
    roof["peaks"] = {"dfma_tflops": dfma_peak, "mma_bf16_tflops": mma_peak, "hbm_gbs": hbm_peak,
                     "hbm_kind": peak_kind, "tcgen05_bf16_tflops": bf16_peak}

    # ---- e2e through the C ABI with host buffers; the rows of every step land
    # in a preallocated array (one D2H per step), counted after the window
    ens2 = pz.Ensemble([gpu_cfg(s) for s in specs])
    rows_all = np.zeros((args.steps, len(specs), pz.SERIES_COLS))
    state_bytes = sum(t.size * 16 for t in temps)
    t0 = time.perf_counter()
    ens2.set_state_all(temps)
    for k in range(args.steps):
        ens2.step(1, sync=False)
        ens2.latest_rows(rows_all[k])
    ens2.sync()
    e2e_wall = time.perf_counter() - t0
    ens2.close()
    n_dt_changes = int(np.count_nonzero(rows_all[1:, :, 15] != rows_all[:-1, :, 15]))
    e2e = {"value": world * len(specs) * args.steps / e2e_wall, "unit": UNIT,
           "h2d_bytes_per_step": int(state_bytes // args.steps),
           "d2h_bytes_per_step": int(rows_all[0].nbytes),
           "note": "timed on the host clock: set_state_all from host arrays (the one-time upload, amortised over "
                   "the steps in h2d_bytes_per_step), then per step pz_step + pz_latest_rows (one D2H of every "
                   "instance's e_kin/heat row into a preallocated host array), then pz_sync"}

    plain = None
    if not args.no_plain:
        plain_v, t_class = plain_rate(specs, max(5, min(args.steps, 20)), args.warmup, torch)
        plain = {"value": plain_v, "per_step_ms_by_class": t_class}

    if rank != 0:
        return
    adj = None
    if not args.no_adjoint:
        adj = {"checkpointed": adjoint_ratio(torch), "stored_trajectory": adjoint_ratio(torch, checkpoint_every=0),
               "batched_dirk": batched_adjoint_leg(torch),
               "batched_dirk_stored_trajectory": batched_adjoint_leg(torch, checkpoint_every=0, fd=False)}
    integ = None if args.no_integ else integ_leg(torch, args.integ_steps)
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(specs)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(specs),
        "plain_steps_per_s": plain["value"] if plain else None,
        "batched_over_plain": (value / world / plain["value"]) if plain else None,
        "plain_detail": plain,
        "kernel_ms_per_step": kms,
        "kernel_ms_note": "device ms per step of each kernel over the timed window's steps (same start state "
                          "and warm-up), launched one by one between CUDA events",
        "roofline": roof,
        "kernel_rooflines": kernels,
        "dominant_kernel": dom,
        "operator_rebuilds_per_step": n_dt_changes / max(1, args.steps - 1),
        "tuning": tuning,
        "adjoint": adj,
        "integ": integ,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": ens.launches_per_step() * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

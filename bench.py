#!/usr/bin/env python
"""FM-DBZP acquisition benchmark on GB300: 32-PRN acquisitions/s (and Msample*PRN/s).

Workload (the reference's weak-signal configuration): GPS L1 C/A, fs = 5 MHz, 10 ms
coherent x 8 non-coherent accumulations (400 000 samples), Doppler +-5 kHz, PRNs 1-32.
Seeded synthetic input: 4 satellites with C/N0 ~ U[35, 42] dB-Hz, Doppler ~ U[+-5 kHz], code
phase ~ U[0, 1023), 50 Hz data bits with a random bit-edge offset, white Gaussian noise,
quantised to Complex{Int16} (x 2^10). A "step" = one acquire! over the 32 PRNs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value   : device-resident throughput (input already in HBM), CUDA events on the plan's stream,
          L2 flushed (256 MB write) before every timed step, outside the events.
e2e     : the public API (acquire_b with a pinned host buffer): H2D of the input, the whole
          pipeline and the D2H of the 32 results inside the timed region, wall clock.
--impl reference: the reference (Julia) cannot run on this machine; its CPU algorithm is timed
          through the oracle's FP32 restatement on the host cores (bounded sample: one PRN
          through all 8 accumulation steps per step).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "acquisition.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

PRNS = list(range(1, 33))
SEED = 2024

# Workloads of the reference's configurations (seeded synthetic recordings stand in for data).
CONFIGS = {
    # headline: GPS L1 C/A weak-signal search, 5 MHz, 10 ms x 8, +-5 kHz, CI16
    "cfg2": dict(workload="gps_l1ca_5MHz_10msx8_pm5kHz_32prn_ci16", system="GPSL1CA", fs=5e6, n_coh=10, n_nc=8,
                 n_be=1, cov=5000.0, quant="ci16", n_sats=4, cn0=(35.0, 42.0), dmax=5000.0, bit_period=0.02),
    # CPU-runnable plain case: 4 MHz, 1 ms, +-7 kHz, CF32, PRN 1 at 45 dB-Hz
    "cfg1": dict(workload="gps_l1ca_4MHz_1ms_pm7kHz_32prn_cf32", system="GPSL1CA", fs=4e6, n_coh=1, n_nc=1, n_be=1,
                 cov=7000.0, quant=None, fixed=[(1, 45.0, 1234.0, 300.5)], bit_period=0.02),
    # bit-edge / data-bit search: the same 80 ms as 40 ms x 2 (ndop 800, 2 data bits, 4 bit edges)
    "cfg2b": dict(workload="gps_l1ca_5MHz_40msx2_pm5kHz_nbe4_32prn_ci16", system="GPSL1CA", fs=5e6, n_coh=40,
                  n_nc=2, n_be=4, cov=5000.0, quant="ci16", n_sats=4, cn0=(35.0, 42.0), dmax=5000.0,
                  bit_period=0.02),
    # ragged batch: 64 recordings (2-80 ms, 4 antennas) of L1 C/A 5 MHz, E1B 12 MHz, L5I 25 MHz
    "cfg3": dict(workload="ragged_batch_64rec_l1ca5_e1b12_l5i25_4ant", system="mixed", fs=0.0, n_coh=1, n_nc=1,
                 n_be=1, cov=8000.0, quant=None),
    # secondary-code rotation search: GPS L5I 20 MHz, 20 ms x 4, +-10 kHz, CI8 (3-bit)
    "cfg4": dict(workload="gps_l5i_20MHz_20msx4_pm10kHz_32prn_ci8", system="GPSL5I", fs=20e6, n_coh=20, n_nc=4,
                 n_be=1, cov=10000.0, quant="ci8", n_sats=6, cn0=(30.0, 45.0), dmax=10000.0, bit_period=0.01),
    # differentiable fine search: L1 C/A 10 MHz, 20 ms CF32, 32 PRNs x 1024 (code phase, Doppler) cells
    "cfg5": dict(workload="gps_l1ca_10MHz_20ms_cf32_32prn_x1024cells_fine", system="GPSL1CA", fs=10e6, n_coh=20,
                 n_nc=1, n_be=1, cov=7000.0, quant=None, cn0=(40.0, 48.0), dmax=7000.0, cells_per_prn=1024),
}
CFG = CONFIGS["cfg2"]
FS, N_COH, N_NC, COV = CFG["fs"], CFG["n_coh"], CFG["n_nc"], CFG["cov"]
WORKLOAD = CFG["workload"]


CONFIG_NAME = "cfg2"


def set_config(name):
    global CFG, FS, N_COH, N_NC, COV, WORKLOAD, CONFIG_NAME
    CONFIG_NAME = name
    CFG = CONFIGS[name]
    FS, N_COH, N_NC, COV, WORKLOAD = CFG["fs"], CFG["n_coh"], CFG["n_nc"], CFG["cov"], CFG["workload"]


def system_of(cfg):
    import acqgb300 as A
    return {"GPSL1CA": A.GPSL1CA, "GPSL5I": A.GPSL5I, "GalileoE1B": A.GalileoE1B}[cfg["system"]]()


def make_input(host_model: bool = False):
    """The workload's seeded recording and its satellites. host_model=False: the product's host
    signal generator (acqgb300.synth, codes from libacqgb300); True: the oracle's restatement of
    the same model (oracle.signal_model), which gives the same bytes without loading the product
    library (the CPU legs use it)."""
    if host_model:
        from oracle import gnss_codes as G
        from oracle import signal_model as synth
        sysm = G.SYSTEMS[CFG["system"]]
        code_length, code_freq = sysm.code_length, sysm.code_freq
        Sat = synth.Sat
    else:
        from acqgb300 import synth
        sysm = system_of(CFG)
        code_length, code_freq = sysm.code_length, sysm.code_frequency
        Sat = synth.Satellite
    rng = np.random.default_rng(SEED)
    if "fixed" in CFG:
        sats = [Sat(p, c, d, cp) for (p, c, d, cp) in CFG["fixed"]]
    else:
        present = sorted(rng.choice(np.arange(1, 33), size=CFG["n_sats"], replace=False).tolist())
        sats = synth.random_sats(rng, present, CFG["cn0"], CFG["dmax"], code_length, bit_period_s=CFG["bit_period"])
    spc = int(math.ceil(code_length / code_freq * FS))
    n = N_NC * N_COH * spc
    x = synth.synth(sysm, FS, n, sats, SEED)
    if CFG["quant"] == "ci16":
        return synth.to_ci16(x), sats
    if CFG["quant"] == "ci8":
        return synth.to_ci8_3bit(x), sats
    return x.astype(np.complex64), sats


def input_digest(sig) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(sig).tobytes()).hexdigest()[:16]


def workload_config(sig, n_nc: int, geometry: dict) -> dict:
    """The `config` of both arms (identical for the same workload): what is searched, on what input."""
    return {"workload": WORKLOAD if n_nc == N_NC else f"{WORKLOAD}_nnc{n_nc}", "prns": len(PRNS),
            "samples": int(n_nc * N_COH * geometry["spc"]), "num_doppler_bins": int(geometry["ndop"]),
            "samples_per_code": int(geometry["spc"]), "fft_size": int(geometry["fft"]),
            "input": f"seed {SEED}, {CFG['quant'] or 'cf32'}, sha256 {input_digest(sig)}",
            "l2": "GPU arm: flushed (256 MB write) before every timed step; CPU arm: not applicable"}


def as_complex64(sig):
    if np.iscomplexobj(sig):
        return sig.astype(np.complex64)
    return (sig[:, 0].astype(np.float32) + 1j * sig[:, 1].astype(np.float32)).astype(np.complex64)


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per accumulation step measured by ncu for (kernel, workload), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.split()
        if len(f) == 3 and not line.startswith("#") and f[0] == kernel and f[1] == workload:
            return int(f[2])
    return None


def peaks():
    p = {}
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        p = json.load(open(path))
    return p


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms during the timed region (the sampler
    is running, with a first sample taken, before the region starts; only later samples count)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.f = None
        self.skip = 0

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 3.0 and os.path.getsize(self.f.name) == 0:
                time.sleep(0.01)
            self.skip = sum(1 for _ in open(self.f.name))
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.f:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if len(rows) > self.skip:
            rows = rows[self.skip:]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


# ---- CPU baseline: the oracle's FP32 restatement with PRNs spread over a process pool, one
# worker per host core, single-threaded FFTs in each (the reference's per-core PRN loop,
# src/acquire.jl:142,195). Workers are spawned (never forked) and build their plan and input
# once, outside every timed region.
_POOL_STATE = None


def _pool_init(cfg_name, prns, n_nc):
    global _POOL_STATE
    set_config(cfg_name)
    from oracle import acq_oracle as O
    from oracle import gnss_codes as G
    O.FFT_WORKERS = 1
    sig, _ = make_input(host_model=True)
    plan = O.plan_acquire(G.SYSTEMS[CFG["system"]], FS, prns, min_doppler_coverage=COV,
                          num_coherently_integrated_code_periods=N_COH, bit_edge_search_steps=CFG["n_be"],
                          num_noncoherent_accumulations=n_nc, precision="f32")
    _POOL_STATE = (plan, as_complex64(sig))


def _pool_task(prns):
    from oracle import acq_oracle as O
    plan, sig = _POOL_STATE
    return [(r.prn, r.peak_doppler_bin, r.peak_code_bin, bool(O.is_detected(r))) for r in O.acquire_b(plan, sig, prns)]


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class CpuPool:
    """A pool of spawned oracle workers for the current workload (n_nc accumulation steps)."""

    def __init__(self, cfg_name: str, prns, n_nc: int, workers: int | None = None):
        import multiprocessing as mp
        for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
            os.environ[v] = "1"
        self.workers = workers or host_cores()
        self.prns = list(prns)
        self.pool = mp.get_context("spawn").Pool(self.workers, initializer=_pool_init,
                                                 initargs=(cfg_name, self.prns, n_nc))
        self.pool.map(_pool_task, [[]] * self.workers)          # every worker initialised

    def acquire(self, prns=None):
        """One acquisition over `prns` (default: all), PRNs dealt round-robin to the workers."""
        prns = self.prns if prns is None else list(prns)
        groups = [prns[i::self.workers] for i in range(self.workers)]
        out = []
        for g in self.pool.map(_pool_task, [g for g in groups if g]):
            out += g
        return sorted(out, key=lambda r: prns.index(r[0]))

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_sample_shape():
    """(PRNs per timed sample, accumulation steps per sample): whole 32-PRN acquisitions where one
    fits in a few seconds of the host's cores, else a bounded sample of one PRN per worker over one
    accumulation step (the secondary-code rotation workloads)."""
    if CFG["system"] == "GPSL5I" and N_COH > 1:
        return min(len(PRNS), host_cores()), 1
    return len(PRNS), N_NC


def cpu_baseline_run(steps: int, warmup: int, budget_s: float | None = None):
    """Time `steps` samples (after `warmup`) on the pool; with budget_s, as many as fit in that
    many seconds (at least one). Returns (seconds per 32-PRN acquisition, per-sample times,
    sample description, workers)."""
    n_prn, n_nc = cpu_sample_shape()
    pool = CpuPool(CONFIG_NAME, PRNS[:n_prn], n_nc)
    try:
        for _ in range(warmup):
            pool.acquire()
        ts = []
        t_start = time.perf_counter()
        while True:
            t0 = time.perf_counter()
            pool.acquire()
            ts.append(time.perf_counter() - t0)
            if budget_s is None:
                if len(ts) >= steps:
                    break
            elif time.perf_counter() - t_start >= budget_s or len(ts) >= steps:
                break
    finally:
        pool.close()
    scale = (len(PRNS) / n_prn) * (N_NC / n_nc)
    whole = scale == 1.0
    desc = (f"whole {len(PRNS)}-PRN acquisitions of the oracle's FP32 restatement, PRNs spread over {pool.workers} "
            f"spawned single-threaded workers" if whole else
            f"{n_prn} PRNs x {n_nc} of {N_NC} accumulation steps per sample over {pool.workers} spawned "
            f"single-threaded workers, scaled x{scale:g} to a 32-PRN acquisition")
    return statistics.mean(ts) * scale, ts, desc, pool.workers


def run_reference_batch(args):
    """cfg3 on the host cores: the oracle's FP32 restatement of one PRN x one accumulation step per
    (system, coherent length) group, scaled by every recording's PRNs x steps. Warm-up times
    every group once; each timed step re-times one group (in rotation)."""
    from acqgb300 import synth
    from oracle import acq_oracle as O
    from oracle import gnss_codes as G
    recs = synth.ragged_batch(seed=SEED)
    groups = {}
    for r in recs:
        groups.setdefault((r["system"].name, r["fs"], r["n_coh"]), r)
    count = {}
    for r in recs:
        k = (r["system"].name, r["fs"], r["n_coh"])
        count[k] = count.get(k, 0) + len(r["prns"]) * r["n_nc"]

    def time_group(k):
        r = groups[k]
        op = O.plan_acquire(G.SYSTEMS[k[0]], k[1], [r["prns"][0]], min_doppler_coverage=r.get("cov", 8000.0),
                            num_coherently_integrated_code_periods=k[2], num_noncoherent_accumulations=1,
                            precision="f32")
        t0 = time.perf_counter()
        O.acquire_b(op, r["samples"], [r["prns"][0]])
        return time.perf_counter() - t0

    times = {k: [time_group(k)] for k in groups}
    keys = sorted(groups)
    mean_group = statistics.mean(v[0] for v in times.values())
    n_timed = max(1, min(args.steps, int(120.0 / max(mean_group, 1e-3))))   # about two minutes at most
    for i in range(n_timed):
        k = keys[i % len(keys)]
        times[k].append(time_group(k))
    t_batch = sum(count[k] * statistics.mean(times[k]) for k in groups)
    n_prn_acq = sum(len(r["prns"]) for r in recs)
    value = (n_prn_acq / 32.0) / t_batch
    line = {"metric": "32-PRN acquisitions/s", "value": value, "unit": "acq/s (32-PRN equivalents)",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_batch * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ragged batch)", "impl": "reference", "timed_samples": n_timed,
            "config": {"workload": WORKLOAD, "recordings": len(recs), "prn_acquisitions": n_prn_acq},
            "cpu_baseline": {"value": value, "unit": "acq/s (32-PRN equivalents)", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": "oracle FP32 restatement, 1 PRN x 1 step per (system, fs, coherent length) "
                                       "group, scaled by every recording's PRNs x steps; the Julia reference is "
                                       "unavailable here"},
            "e2e": {"value": value, "unit": "acq/s (32-PRN equivalents)", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_fine(args):
    """cfg5 on the host cores: the FP64 numpy correlator oracle (one core), per step one cell's
    power+gradient+Hessian, sample adjoint and Newton refinement."""
    from oracle import corr_oracle as O
    from oracle import gnss_codes as G
    x, sats, prn, tau, dop = fine_input_host()
    n = x.size
    rng = np.random.default_rng(7)

    def one(i):
        t0 = time.perf_counter()
        O.power_derivatives(O.correlate(x, G.GPSL1CA, int(prn[i]), FS, tau[i], dop[i]))
        O.vjp_samples(n, G.GPSL1CA, FS, [(int(prn[i]), tau[i], dop[i])], [1.0])
        O.newton_refine(x, G.GPSL1CA, int(prn[i]), FS, tau[i], dop[i], max_iter=20)
        return time.perf_counter() - t0

    warm = [one(int(rng.integers(prn.size))) for _ in range(max(1, args.warmup))]
    n_timed = max(1, min(args.steps, int(120.0 / max(min(warm), 1e-3))))   # about two minutes at most
    ts = [one(int(rng.integers(prn.size))) for _ in range(n_timed)]
    value = 1.0 / statistics.mean(ts)
    line = {"metric": "fine-search cells/s", "value": value, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(ts) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, CF32, 32 PRNs present)", "impl": "reference", "timed_samples": n_timed,
            "config": {"workload": WORKLOAD, "cells": int(prn.size), "samples": int(n)},
            "cpu_baseline": {"value": value, "unit": "cells/s", "cores": 1, "kind": "port",
                             "sample": "FP64 numpy correlator oracle, one random cell per step (forward with "
                                       "Hessian, sample adjoint, Newton refinement)"},
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference(args):
    if args.config == "cfg3":
        return run_reference_batch(args)
    if args.config == "cfg5":
        return run_reference_fine(args)
    from oracle import acq_oracle as O
    from oracle import gnss_codes as G
    sig, _ = make_input(host_model=True)
    geo = O.plan_geometry(G.SYSTEMS[CFG["system"]], FS, min_doppler_coverage=COV, n_coh=N_COH, n_be=CFG["n_be"],
                          n_nc=N_NC)
    per_acq, ts, desc, workers = cpu_baseline_run(args.steps, args.warmup)
    value = 1.0 / per_acq
    # the same restatement on the reference's CPU-runnable geometry (4 MHz, 1 ms, +-7 kHz, 32
    # PRNs), beside the reference's own published figures for that geometry
    cfg_name = CONFIG_NAME
    set_config("cfg1")
    t1, ts1, _, _ = cpu_baseline_run(20, 2)
    set_config(cfg_name)
    line = {"metric": "32-PRN acquisitions/s", "value": value, "unit": "acq/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(ts) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic (seeded, {CFG['quant'] or 'cf32'})", "impl": "reference",
            "config": workload_config(sig, N_NC, {"spc": geo["spc"], "ndop": geo["ndop"], "fft": geo["F"]}),
            "cpu_baseline": {"value": value, "unit": "acq/s", "cores": workers, "kind": "port",
                             "sample": desc + "; the Julia reference is unavailable on this machine, its algorithm "
                                              "runs as the oracle's FP32 numpy/scipy restatement"},
            "e2e": {"value": value, "unit": "acq/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "msample_prn_per_s": value * len(PRNS) * N_NC * N_COH * geo["spc"] / 1e6,
            "port_on_cpu_runnable_geometry": {
                "workload": CONFIGS["cfg1"]["workload"], "value": 1.0 / t1, "unit": "acq/s", "cores": workers,
                "published_reference": {"1 thread": 25.0, "4 threads": 77.0, "8 threads": 118.0,
                                        "source": "CHANGELOG.md:234-237 (v2.0.0 code, CPU unstated)"}}}
    print(json.dumps(line))


def run_batch(args, world, rank, local_rank):
    """Ragged batch (cfg3): all 64 recordings in one CUDA-graph launch per step."""
    import torch
    import acqgb300 as A
    from acqgb300 import batch as B
    from acqgb300 import synth
    torch.cuda.set_device(local_rank)
    recs = synth.ragged_batch(seed=SEED)
    cache = B.PlanCache(device=local_rank)
    items = B.batch_from_recordings(recs, cache)
    bt = B.AcquisitionBatch(items)
    n_prn_acq = sum(len(r["prns"]) for r in recs)
    samples_used = sum(len(r["prns"]) * r["n_nc"] * r["n_coh"] * it.plan.samples_per_code
                       for r, it in zip(recs, items))
    host = [torch.from_numpy(r["samples"].view(np.float32).reshape(-1, 2)).pin_memory().numpy() for r in recs]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    bst = torch.cuda.ExternalStream(bt.stream_handle(), device=f"cuda:{local_rank}")
    for _ in range(args.warmup):
        bt.run(host)
    bt.upload(host)
    torch.cuda.synchronize()
    clk = ClockSampler(local_rank)
    ev_ms = []
    with clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(bst)
            bt.launch()
            e1.record(bst)
            res = bt.fetch()
            ev_ms.append(e0.elapsed_time(e1))
    t_step = statistics.mean(ev_ms) / 1e3
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bt.run(host)
        e2e.append(time.perf_counter() - t0)
    t_e2e = statistics.mean(e2e)
    if rank != 0:
        return
    value = world * (n_prn_acq / 32.0) / t_step
    e2e_value = world * (n_prn_acq / 32.0) / t_e2e
    detected = sum(A.is_detected(x) for rr in res for x in rr)
    planted = sum(len(r["sats"]) for r in recs)
    hit = sum(A.is_detected({x.prn: x for x in rr}[s.prn]) for r, rr in zip(recs, res) for s in r["sats"])
    cpu = None
    if not args.no_cpu_baseline:
        # oracle FP32 port on one PRN of one recording per system, scaled by PRNs x steps
        from oracle import acq_oracle as O
        from oracle import gnss_codes as G
        per_step = {}
        for r in recs:
            key = (r["system"].name, r["n_coh"])
            if key in per_step:
                continue
            op = O.plan_acquire(G.SYSTEMS[r["system"].name], r["fs"], [r["prns"][0]], min_doppler_coverage=8000,
                                num_coherently_integrated_code_periods=r["n_coh"], num_noncoherent_accumulations=1)
            t0 = time.perf_counter()
            O.acquire_b(op, r["samples"], [r["prns"][0]])
            per_step[key] = time.perf_counter() - t0
        t_cpu = sum(len(r["prns"]) * r["n_nc"] * per_step[(r["system"].name, r["n_coh"])] for r in recs)
        cpu = {"value": (n_prn_acq / 32.0) / t_cpu, "unit": "acq/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "oracle FP32 restatement: one PRN x one step per (system, coherent length), scaled by every "
                         "recording's PRNs x steps"}
    line = {"metric": "32-PRN acquisitions/s", "value": value, "unit": "acq/s (32-PRN equivalents)",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ragged batch)",
            "config": {"workload": WORKLOAD, "recordings": len(recs), "prn_acquisitions": n_prn_acq,
                       "plans": len(cache.plans), "form": "one CUDA graph per batch",
                       "l2": "flushed (256 MB write) before every timed step"},
            "msample_prn_per_s": value * 32 * samples_used / n_prn_acq / 1e6,
            "recordings_per_s": len(recs) / t_step,
            "e2e": {"value": e2e_value, "unit": "acq/s (32-PRN equivalents)",
                    "h2d_bytes_per_step": int(sum(h.nbytes for h in host)),
                    "d2h_bytes_per_step": n_prn_acq * 72, "ms_per_step": t_e2e * 1e3},
            "gpu_launches": int(bt.launch_count() * args.steps), "cpu_baseline": cpu, "clocks": clk.summary(),
            "detections": {"detected": int(detected), "planted": planted, "planted_detected": int(hit)}}
    print(json.dumps(line))


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's time (replicas: the job ends when the last one does)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


FINE_FLOPS = {"eval": 34, "hess": 56, "vjp": 19}   # FP32 flops per (cell, sample), see run_fine


def fine_input():
    return fine_input_host()


def fine_input_host():
    """cfg5 recording: all 32 PRNs present (C/N0 ~ U[40, 48] dB-Hz, Doppler ~ U[+-7 kHz], code phase
    ~ U[0, 1023) chips, continuous), data-free 20 ms, unit-power white noise; and 1024 cells per PRN
    within +-1 code bin (one sample) and +-1 Doppler bin (1/T) of the true parameters."""
    from acqgb300 import synth
    import acqgb300 as A
    rng = np.random.default_rng(SEED)
    n = int(round(FS * 0.02))
    sats = [synth.Satellite(p, float(rng.uniform(*CFG["cn0"])), float(rng.uniform(-CFG["dmax"], CFG["dmax"])),
                            float(rng.uniform(0, 1023)), float(rng.uniform(0, 2 * math.pi)), data_bits=False)
            for p in PRNS]
    x = synth.synth(A.GPSL1CA(), FS, n, sats, SEED).astype(np.complex64)
    m = CFG["cells_per_prn"]
    chip_bin, dop_bin = 1.023e6 / FS, FS / n
    prn = np.repeat(PRNS, m)
    tau = np.concatenate([s.code_phase + rng.uniform(-1, 1, m) * chip_bin for s in sats])
    dop = np.concatenate([s.doppler + rng.uniform(-1, 1, m) * dop_bin for s in sats])
    return x, sats, prn, tau, dop


def run_fine(args, world, rank, local_rank):
    """Differentiable fine search (cfg5). A step = for every cell: power and gradient (forward),
    the adjoint with respect to the 200 000 samples for the loss sum(P) (backward; the code
    replica is recomputed), and batched Newton refinement from the cell."""
    import torch
    import acqgb300 as A
    from acqgb300 import corr as CR
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    x, sats, prn, tau, dop = fine_input()
    n = x.size
    corr = CR.Correlator(A.GPSL1CA(), FS, PRNS, device=local_rank)
    cells = CR.pack_cells(prn, tau, dop)
    nc = cells.size
    xd = torch.as_tensor(x, device=dev)
    cd = corr._cells_dev(cells)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream()

    def step(timing=None):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(st)
        raw = corr.eval_device(xd, cd, nc, False)
        ev[1].record(st)
        r = raw.view(torch.float64)[: nc * 9].view(nc, 9)
        zbar = (2.0 * torch.complex(r[:, 6], r[:, 7])).to(torch.complex64)
        corr.vjp_device(n, cd, nc, zbar)
        ev[2].record(st)
        c2 = cd.clone()
        corr.refine_device(xd, c2, nc, max_iterations=20)
        ev[3].record(st)
        if timing is not None:
            timing.append(ev)
        return c2

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(local_rank)
    evs = []
    with clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            step(evs)
        torch.cuda.synchronize()
    parts = np.array([[e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2]), e[2].elapsed_time(e[3])] for e in evs])
    t_step = parts.sum(axis=1).mean() / 1e3
    t_eval, t_vjp, t_ref = parts.mean(axis=0)
    hess_ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        corr.eval_device(xd, cd, nc, True)
        e1.record(st)
        torch.cuda.synchronize()
        hess_ms.append(e0.elapsed_time(e1))
    t_hess = statistics.mean(hess_ms)

    # e2e through the public API: host samples and cells in, host results out, every step
    xh = torch.from_numpy(x).pin_memory()
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xg = xh.to(dev, non_blocking=True)
        ev = corr.eval(xg, prn, tau, dop)
        corr.vjp_samples(n, prn, tau, dop, 2.0 * ev.z).cpu()
        rf = corr.refine(xg, prn, tau, dop, max_iterations=20)
        e2e.append(time.perf_counter() - t0)
    t_e2e = statistics.mean(e2e)

    # quality: Newton from every cell against the maximum reached from the true parameters
    ml = corr.refine(xd, PRNS, [s.code_phase for s in sats], [s.doppler for s in sats], max_iterations=30)
    mt = np.repeat(ml.code_phase, CFG["cells_per_prn"])
    mf = np.repeat(ml.doppler, CFG["cells_per_prn"])
    same = (np.abs(rf.code_phase - mt) < 2e-3) & (np.abs(rf.doppler - mf) < 0.05)
    dop_bin = FS / n
    inner = (np.abs(tau - np.repeat([s.code_phase for s in sats], CFG["cells_per_prn"])) < 0.5 * 1.023e6 / FS) & \
            (np.abs(dop - np.repeat([s.doppler for s in sats], CFG["cells_per_prn"])) < 0.5 * dop_bin)

    # FP32 results against the FP64 oracle on a sample of cells
    from oracle import corr_oracle as O
    from oracle import gnss_codes as G
    rng = np.random.default_rng(7)
    pick = rng.choice(nc, 12, replace=False)
    eh = corr.eval(xd, prn[pick], tau[pick], dop[pick], hessian=True)
    T = n / FS
    err = np.zeros(3)
    for j, i in enumerate(pick):
        d = O.correlate(x.astype(np.complex128), G.GPSL1CA, int(prn[i]), FS, tau[i], dop[i])
        P, g, h = O.power_derivatives(d)
        Ps = ml.power[PRNS.index(int(prn[i]))]
        err = np.maximum(err, [abs(eh.power[j] - P) / Ps, np.max(np.abs(eh.grad[j] - g) / [Ps, Ps * T]),
                               np.max(np.abs(eh.hess[j] - h) / [Ps, Ps * T, Ps * T * T])])
    xb = corr.vjp_samples(n, prn[pick], tau[pick], dop[pick], 2.0 * eh.z).cpu().numpy()
    xb_ref = O.vjp_samples(n, G.GPSL1CA, FS, [(int(prn[i]), tau[i], dop[i]) for i in pick], 2.0 * eh.z)
    err_vjp = float(np.max(np.abs(xb - xb_ref)) / np.max(np.abs(xb_ref)))

    cpu = None
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        for i in pick[:4]:
            O.power_derivatives(O.correlate(x, G.GPSL1CA, int(prn[i]), FS, tau[i], dop[i]))
        t_c = (time.perf_counter() - t0) / 4
        t0 = time.perf_counter()
        O.vjp_samples(n, G.GPSL1CA, FS, [(int(prn[i]), tau[i], dop[i]) for i in pick[:4]], np.ones(4))
        t_v = (time.perf_counter() - t0) / 4
        t0 = time.perf_counter()
        its = 0
        for i in pick[:2]:
            its += O.newton_refine(x, G.GPSL1CA, int(prn[i]), FS, tau[i], dop[i], max_iter=20)[3]
        t_r = (time.perf_counter() - t0) / 2
        cpu = {"value": 1.0 / (t_c + t_v + t_r), "unit": "cells/s", "cores": 1, "kind": "port",
               "sample": "FP64 numpy oracle: 4 cells of power+gradient+Hessian, 4 cells of the sample adjoint, "
                         "2 Newton refinements, on 200 000 samples each"}
    algo = nc * n * (FINE_FLOPS["eval"] + FINE_FLOPS["vjp"])
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    if rank != 0:
        return
    ach = nc * n * FINE_FLOPS["hess"] / (t_hess / 1e3) / 1e12
    line = {"metric": "fine-search cells/s", "value": world * nc / t_step, "unit": "cells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, CF32, 32 PRNs present)",
            "config": {"workload": WORKLOAD, "cells": nc, "samples": n,
                       "step": "forward power+gradient, sample adjoint, Newton refinement (<= 20 iterations)",
                       "l2": "flushed (256 MB write) before every timed step"},
            "ms": {"eval": t_eval, "vjp": t_vjp, "refine": t_ref, "eval_with_hessian": t_hess},
            "gcell_samples_per_s": {"eval": nc * n / (t_eval / 1e3) / 1e9, "eval_with_hessian": nc * n / (t_hess / 1e3) / 1e9,
                                    "vjp": nc * n / (t_vjp / 1e3) / 1e9},
            "refine": {"converged": int(np.sum(rf.status == 0)), "mean_iterations": float(rf.iterations.mean()),
                       "to_peak_all": float(same.mean()), "to_peak_within_half_bin": float(same[inner].mean())},
            "fp64_error": {"power": err[0], "gradient": err[1], "hessian": err[2], "vjp": err_vjp,
                           "scale": "power at the peak; per chip, per Hz x T; per chip^2 ... x T^2; max |x_bar|"},
            "e2e": {"value": world * nc / t_e2e, "unit": "cells/s", "h2d_bytes_per_step": int(x.nbytes + 3 * cells.nbytes + nc * 8),
                    "d2h_bytes_per_step": int(nc * 72 * 2 + n * 8 + nc * 24), "ms_per_step": t_e2e * 1e3},
            "gpu_launches": 4 * args.steps,
            "roofline": {"kernel": "k_corr (power+gradient+Hessian)", "bound": "fp32", "achieved": ach,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                         "peak_source": "nominal FP32 CUDA-core rate: 152 SMs x 128 lanes x 2 flops x 2.07 GHz",
                         "flops_per_cell_sample": FINE_FLOPS, "traffic": None},
            "cpu_baseline": cpu, "clocks": clk.summary()}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", default="plain", choices=["fused", "plain"],
                    help="kernel form of the headline measurement (the other form is reported beside it)")
    ap.add_argument("--config", default="cfg2", choices=sorted(CONFIGS),
                    help="workload (cfg2, the reference's weak-signal search, is the headline)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16", "bf16", "fp16_split", "bf16_split"],
                    help="rotation-combine arithmetic of the headline measurement on rotation-search workloads")
    ap.add_argument("--no-precision-study", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes (otherwise the autotuner picks them before timing)")
    ap.add_argument("--prns", type=int, default=None,
                    help="search PRNs 1..N instead of 1..32 (profiling cases only; the workload name says so)")
    ap.add_argument("--cells-per-prn", type=int, default=None,
                    help="fine search: cells per PRN (profiling cases only; default 1024)")
    ap.add_argument("--accumulations", type=int, default=None,
                    help="non-coherent accumulations (profiling cases only; default: the workload's)")
    args = ap.parse_args()
    set_config(args.config)
    global PRNS, WORKLOAD
    if args.prns:
        PRNS = list(range(1, int(args.prns) + 1))
        WORKLOAD = f"{WORKLOAD}_{len(PRNS)}prn"
    if args.cells_per_prn:
        CFG["cells_per_prn"] = int(args.cells_per_prn)
        WORKLOAD = f"{WORKLOAD}_{int(args.cells_per_prn)}cells"
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.config == "cfg3":
        run_batch(args, world, rank, local_rank)
        return
    if args.config == "cfg5":
        run_fine(args, world, rank, local_rank)
        return

    import torch
    import acqgb300 as A

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    ci16, sats = make_input()
    n_nc = args.accumulations or N_NC
    plan = A.plan_acquire(system_of(CFG), FS, PRNS, min_doppler_coverage=COV,
                          num_coherently_integrated_code_periods=N_COH, bit_edge_search_steps=CFG["n_be"],
                          num_noncoherent_accumulations=n_nc, device=local_rank)
    main_form = plan.set_form(args.form)
    main_prec = plan.set_rotation_precision(args.precision)
    other_form = "plain" if main_form == "fused" else "fused"
    if np.iscomplexobj(ci16):
        host = torch.from_numpy(ci16.view(np.float32).reshape(-1, 2)).pin_memory()
    else:
        host = torch.from_numpy(ci16).pin_memory()
    host_np = host.numpy()
    dev = host.to(f"cuda:{local_rank}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    pstream = torch.cuda.ExternalStream(plan.stream_handle(), device=f"cuda:{local_rank}")

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize()

    # launch shapes from the project's autotuner (tile / column CTA shapes; results unchanged)
    tuned = None
    if not args.no_autotune:
        from acqgb300 import autotune as T
        tuned = T.tune(plan, dev, PRNS, reps=3, passes=1, store=False,
                       knobs=("tile_rows", "tile_threads", "tile_blocks", "tile_pad", "column_width",
                              "column_ctas_per_sm", "tile_mma", "search_width", "search_split"))

    # warm-up (device-resident and public API)
    for _ in range(args.warmup):
        A.acquire_device(plan, dev, PRNS)
        A.acquire_b(plan, host_np, PRNS)
    res = A.acquire_device(plan, dev, PRNS)
    launches_per_step = plan.last_launch_count()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- value: device-resident, CUDA events on the plan's stream
    clk = ClockSampler(local_rank)
    with clk:
        barrier()
        ev_ms = []
        for _ in range(args.steps):
            flush_l2()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(pstream)
            A.acquire_device_async(plan, dev, PRNS)
            e1.record(pstream)
            A.fetch_results(plan, PRNS)
            ev_ms.append(e0.elapsed_time(e1))
        barrier()
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ev_ms) / 1e3, dist, f"cuda:{local_rank}")
    value = world * 1.0 / t_step

    # ---- the other form on the same input (plain: one kernel per stage, tile and accumulator
    # in HBM; fused: the cluster kernel)
    form = main_form
    plain_value = None
    if plan.set_form(other_form) == other_form:
        for _ in range(2):
            A.acquire_device(plan, dev, PRNS)
        pm = []
        for _ in range(args.steps):
            flush_l2()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(pstream)
            A.acquire_device_async(plan, dev, PRNS)
            e1.record(pstream)
            A.fetch_results(plan, PRNS)
            pm.append(e0.elapsed_time(e1))
        plain_value = world * 1e3 / statistics.mean(pm)
        plan.set_kernel_timing(True)
        plan.reset_kernel_times()
        for _ in range(args.steps):
            flush_l2()
            A.acquire_device_async(plan, dev, PRNS)
            A.fetch_results(plan, PRNS)
        plain_ktimes = plan.kernel_times()
        plan.set_kernel_timing(False)
        plan.set_form(main_form)
    else:
        plain_ktimes = None

    # ---- per-kernel device time (same workload, events around every launch)
    plan.set_kernel_timing(True)
    plan.reset_kernel_times()
    for _ in range(args.steps):
        flush_l2()
        A.acquire_device_async(plan, dev, PRNS)
        A.fetch_results(plan, PRNS)
    ktimes = plan.kernel_times()
    plan.set_kernel_timing(False)

    # ---- tensor-core variants against the FP32 path: rotation searches (the candidate combine)
    # and the simple path (the per-column Doppler DFT as a DFT-matrix GEMM, ndop <= 250):
    # throughput, power error relative to the FP32 surface's peak on two PRNs (strongest planted,
    # one absent) and agreement of every PRN's decisions
    study = None
    gpath = plan.geometry.path
    if not args.no_precision_study and (gpath == 2 or (gpath == 0 and plan.geometry.num_doppler_bins <= 250)):
        setter = plan.set_rotation_precision if gpath == 2 else plan.set_doppler_precision
        study = {"stage": "rotation combine" if gpath == 2 else "Doppler DFT (dense DFT-matrix GEMM)"}
        strong = max(sats, key=lambda s_: s_.cn0).prn
        absent = next(p_ for p_ in PRNS if p_ not in {s_.prn for s_ in sats})
        pair = [q for q in (strong, absent) if q in PRNS]
        setter("fp32")
        ref_all = A.acquire_device(plan, dev, PRNS)
        ref_pb = {r.prn: np.asarray(r.power_bins, dtype=np.float64).copy()
                  for r in A.acquire_b(plan, host_np, pair, store_power_bins=True)}
        for prec in ("fp32", "fp16", "bf16", "fp16_split", "bf16_split"):
            if setter(prec) != prec:
                continue
            A.acquire_device(plan, dev, PRNS)
            pm = []
            for _ in range(args.steps):
                flush_l2()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(pstream)
                A.acquire_device_async(plan, dev, PRNS)
                e1.record(pstream)
                out = A.fetch_results(plan, PRNS)
                pm.append(e0.elapsed_time(e1))
            same = sum(int(A.is_detected(a) == A.is_detected(b) and (not A.is_detected(b) or (
                a.peak_doppler_bin, a.peak_code_bin, a.secondary_code_phase) == (
                b.peak_doppler_bin, b.peak_code_bin, b.secondary_code_phase))) for a, b in zip(out, ref_all))
            pb = {r.prn: np.asarray(r.power_bins, dtype=np.float64)
                  for r in A.acquire_b(plan, host_np, pair, store_power_bins=True)}
            err = max(float(np.max(np.abs(pb[q] - ref_pb[q])) / np.max(ref_pb[q])) for q in pair)
            study[prec] = {"value": world * 1e3 / statistics.mean(pm), "unit": "acq/s",
                           "max_power_error_vs_fp32": err, "prns_with_same_decisions": same}
        setter(args.precision if gpath == 2 else "fp32")

    # ---- e2e: public API, pinned host input, H2D + compute + D2H inside the timed region
    e2e_s = []
    for _ in range(args.steps):
        flush_l2()
        t0 = time.perf_counter()
        A.acquire_b(plan, host_np, PRNS)
        e2e_s.append(time.perf_counter() - t0)
    t_e2e = max_over_ranks(statistics.mean(e2e_s), dist, f"cuda:{local_rank}")
    e2e_value = world / t_e2e

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    g = plan.geometry
    pk = peaks()
    hbm_peak = pk.get("hbm_gbs", 6800.0)
    dom = max(ktimes.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, nl) = dom
    per_launch_s = tot_ms / nl / 1e3
    per_acq_s = tot_ms / args.steps / 1e3
    n_prn = len(PRNS)
    spc, ndop, F, nb = g.samples_per_code, g.num_doppler_bins, g.fft_size, g.num_blocks
    spc_eff = g.samples_per_code_eff
    # algorithmic bytes of each kernel class per acquisition (compulsory HBM traffic of the form):
    # the coherent tile is written once and read once per step, the accumulator written once
    tile_mma = plan.get_option(11) == 1
    bs = g.block_size
    # tensor-core tile operands: per (step, row) the Q_s blocks of Re/Im hi/lo (FP16)
    ks, nh = (bs + 15) // 16, (bs + 127) // 128
    stub_bytes = 4 * (2 * ks + 16 * nh - 1) * 128
    alg_bytes = {
        "tile": (n_nc * (n_prn * ndop * spc * 8 + ndop * stub_bytes) + n_prn * spc if tile_mma else
                 n_nc * (n_prn * ndop * spc * 8 + ndop * F * 8) + n_prn * nb * F * 8),
        "column": n_nc * n_prn * ndop * spc * 8 + n_prn * ndop * spc_eff * 4,
        "frontend": n_nc * N_COH * spc * ci16.itemsize * 2 + n_nc * ndop * (stub_bytes if tile_mma else F * 8),
        "stats": n_prn * ndop * spc_eff * 4,
        # fused: input spectra + code spectra reads, one accumulator write (the algorithmic minimum)
        "fused": n_nc * ndop * F * 8 + n_prn * nb * F * 8 + n_prn * ndop * spc_eff * 4,
    }
    # FP32 work per acquisition (5 N log2 N per complex FFT + 6 per complex multiply + 3 per |x|^2;
    # the sign / rotation stages run one ndop-point FFT per candidate pattern and bit edge)
    fft_flops = lambda n: 5.0 * n * math.log2(n)
    n_cand = (g.num_secondary_rotations * (1 << (g.num_data_bits - 1)) * g.bit_edge_search_steps
              if g.path != 0 else 1)
    # tensor-core tile: MMAs executed (128-row blocks of code rows x 128-lag halves x K, Re and Im,
    # hi and lo)
    n_chunks = (n_prn * nb + 127) // 128
    mma_flops = n_nc * ndop * n_chunks * 128 * nh * 128 * ks * 16 * 2 * 2 * 2
    flops = {
        "tile": n_nc * n_prn * ndop * nb * (fft_flops(F) + 6 * F),
        "column": n_nc * n_prn * spc * n_cand * (fft_flops(ndop) + 3 * ndop),
    }
    flops["fused"] = flops["tile"] + flops["column"]
    ab = alg_bytes.get(name)
    achieved = ab / per_acq_s / 1e9 if ab else None
    # nominal FP32 (non-tensor) peak: SMs x 128 lanes x 2 (FMA) x the SM clock seen under load
    props = torch.cuda.get_device_properties(local_rank)
    sm_clock = clocks.get("sm_max_mhz") or clocks.get("sm_mhz")
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_clock * 1e6 / 1e12 if sm_clock else None
    fp32_rate = (flops[name] / per_acq_s / 1e12) if name in flops and not (tile_mma and name == "tile") else None
    # (the statistics no longer re-read the surface on the simple path: frontend, tile, column)
    step_bytes = sum(v for k, v in alg_bytes.items() if k in ktimes and k in ("frontend", "tile", "column"))
    tps = ncu_traffic(name, WORKLOAD)
    roof = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": (achieved / hbm_peak) if achieved else None,
            "traffic": (tps * n_nc / (nl / args.steps)) if tps else None,
            "traffic_source": "ncu capture of a 2-step case scaled to the launch's steps" if tps else None,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in pk else "fallback",
            "per_launch_ms": per_launch_s * 1e3, "launches_per_step": nl / args.steps,
            "algorithmic_bytes_per_step": ab,
            "fp32_tflops": fp32_rate,
            "fp32_peak_tflops": fp32_peak,
            "fp32_frac": (fp32_rate / fp32_peak) if (fp32_rate and fp32_peak) else None,
            "fp32_note": "FLOPs counted at 5 N log2 N per complex FFT; peak = SMs x 128 x 2 x max SM clock (nominal)",
            "tile_form": "tensor-core correlation GEMM (FP16 codes x FP16 hi+lo samples, FP32 accumulation)"
                         if tile_mma else "FP32 four-step FFT",
            "tile_tensor_tflops": (mma_flops / (ktimes["tile"][0] / args.steps / 1e3) / 1e12
                                   if tile_mma and "tile" in ktimes else None),
            "tile_tensor_frac": (mma_flops / (ktimes["tile"][0] / args.steps / 1e3) / 1e12 / pk["bf16_tflops"]
                                 if tile_mma and "tile" in ktimes and "bf16_tflops" in pk else None),
            "tile_tensor_note": "MMA FLOPs executed / tile time, against the measured dense bf16 cuBLAS burst peak",
            # whole step: compulsory bytes of every stage / step time, against the same HBM peak
            "step_hbm_frac": (step_bytes / t_step / 1e9 / hbm_peak) if step_bytes else None,
            "kernel_ms_per_step": {k: v[0] / args.steps for k, v in ktimes.items()}}

    cpu = None
    if not args.no_cpu_baseline and not args.prns and n_nc == N_NC:
        # about 15 s of host time, after every GPU measurement
        per_acq, ts, desc, workers = cpu_baseline_run(10 ** 6, 1, budget_s=15.0)
        cpu = {"value": 1.0 / per_acq, "unit": "acq/s", "cores": workers, "kind": "port",
               "sample": f"{desc}; {len(ts)} samples in {sum(ts):.1f} s"}
    samples = n_nc * N_COH * spc
    det = [r.prn for r in res if A.is_detected(r)]
    line = {"metric": "32-PRN acquisitions/s", "value": value, "unit": "acq/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, CI16)",
            "config": workload_config(ci16, n_nc, {"spc": spc, "ndop": ndop, "fft": F}),
            "gpu_settings": {"form": form, "rotation_precision": main_prec,
                             "launch_shapes": (dict(tuned["settings"], tuned_ms=tuned["ms"],
                                                    default_ms=tuned["start_ms"]) if tuned else "defaults")},
            "msample_prn_per_s": value * n_prn * samples / 1e6,
            "other_form": {"form": other_form, "value": plain_value, "unit": "acq/s",
                           "kernel_ms_per_step": ({k: v[0] / args.steps for k, v in plain_ktimes.items()}
                                                  if plain_ktimes else None)},
            "e2e": {"value": e2e_value, "unit": "acq/s", "h2d_bytes_per_step": int(ci16.nbytes),
                    "d2h_bytes_per_step": n_prn * 72, "ms_per_step": t_e2e * 1e3},
            "gpu_launches": int(launches_per_step * args.steps),
            "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "detected_prns": det, "planted_prns": [s.prn for s in sats], "precision_study": study}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Measured-cost autotuner for a plan's launch shapes, with a persistent cache.

Knobs (plan options of include/acqgb300.h). They move work between threads and CTAs; the tile
knobs leave results bit-identical, the column and form knobs can change the order of the
accumulation sums (results within FP32 rounding, decisions unchanged):
  tile_rows            ACQ_OPT_TILE_ROWS           coherent-tile rows per CTA sharing each code-spectrum load
  tile_threads         ACQ_OPT_TILE_THREADS        threads per coherent-tile CTA
  tile_blocks          ACQ_OPT_TILE_BLOCKS         code blocks (inverse FFTs) per tile CTA round
  tile_pad             ACQ_OPT_TILE_PAD            shared-memory padding between FFT buffers
  column_width         ACQ_OPT_COLUMN_WIDTH        code-phase columns per TMA tile
  column_ctas_per_sm   ACQ_OPT_COLUMN_CTAS_PER_SM  persistent column CTAs per SM
  form                 ACQ_OPT_FORM                plain (one kernel per stage) or fused (cluster)
  tile_mma             ACQ_OPT_TILE_MMA            coherent tile as a tensor-core correlation GEMM (1) or
                                                   FP32 FFTs (0); results within FP32 rounding
  search_width         ACQ_OPT_SEARCH_WIDTH        code-phase columns per bit-edge / rotation search CTA
  search_split         ACQ_OPT_SEARCH_SPLIT        FFT split of the bit-edge search (first-pass length;
                                                   the radix structure of its register FFTs)
A candidate the plan's sizes have no instantiation for reads back a different value and is
skipped.
Reduced-precision rotation combines change results within their stated bounds, so they are
tuned only on request (``allow_reduced_precision``).

Search: coordinate descent from the current shape (each knob over its candidates with the
others fixed, two passes), every candidate timed with CUDA events on the plan's stream
(median of ``reps`` acquisitions of the caller's device-resident signal after one warm-up).
The winner is stored per geometry and GPU in a JSON cache ($ACQ_AUTOTUNE_CACHE, default
~/.cache/acqgb300/autotune.json) and applied by ``apply_cached``.
"""
from __future__ import annotations

import json
import os
import statistics
from typing import Callable

from . import _lib as L

KNOBS = {
    "tile_rows": L.ACQ_OPT_TILE_ROWS,
    "tile_threads": L.ACQ_OPT_TILE_THREADS,
    "tile_blocks": L.ACQ_OPT_TILE_BLOCKS,
    "tile_pad": L.ACQ_OPT_TILE_PAD,
    "column_width": L.ACQ_OPT_COLUMN_WIDTH,
    "column_ctas_per_sm": L.ACQ_OPT_COLUMN_CTAS_PER_SM,
    "tile_mma": L.ACQ_OPT_TILE_MMA,
    "search_width": L.ACQ_OPT_SEARCH_WIDTH,
    "search_split": L.ACQ_OPT_SEARCH_SPLIT,
}
# knobs whose 0 is a setting (for the others 0 means the plan's sizes lack that kernel)
ZERO_IS_A_VALUE = {"tile_mma"}
FORMS = {"plain": L.ACQ_FORM_PLAIN, "fused": L.ACQ_FORM_FUSED}


def candidates(plan) -> dict:
    """Candidate values per knob for this plan's geometry."""
    nb = plan.geometry.num_blocks
    blocks = sorted({b for b in (1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 25) if b <= nb})
    rows = [1, 2] if plan.geometry.num_coherently_integrated_code_periods >= 2 else [1]
    return {"tile_rows": rows, "tile_threads": [64, 128, 192, 256], "tile_blocks": blocks, "tile_pad": [0, 1, 9],
            "column_width": [8, 12, 16, 20, 24, 32, 48, 64, 96, 128, 192, 256], "column_ctas_per_sm": [1, 2, 3, 4, 5, 6],
            "form": ["plain", "fused"],
            "tile_mma": [1, 0], "search_width": [2, 4, 8, 16], "search_split": [20, 25, 32, 40]}


def current(plan) -> dict:
    """The plan's shape now (a knob the plan's sizes lack reads 0)."""
    out = {k: plan.get_option(opt) for k, opt in KNOBS.items()}
    out["form"] = "fused" if plan.get_option(L.ACQ_OPT_FORM) == L.ACQ_FORM_FUSED else "plain"
    return out


def apply(plan, settings: dict) -> dict:
    """Apply a shape; returns the settings in effect."""
    eff = {}
    for k, v in settings.items():
        if k == "form":
            eff[k] = plan.set_form(v)
        elif k in KNOBS and (v or k in ZERO_IS_A_VALUE):
            try:
                eff[k] = plan.set_option(KNOBS[k], int(v))
            except Exception:
                eff[k] = None
        elif k == "rotation_precision":
            eff[k] = plan.set_rotation_precision(v)
    return eff


def unavailable(settings: dict, eff: dict) -> bool:
    """True when a shape cannot be timed as asked: an option failed, or a requested value has no
    instantiation for the plan's sizes (the option kept another and reads it back)."""
    if any(v is None for v in eff.values()):
        return True
    return any(k in KNOBS and k not in ZERO_IS_A_VALUE and settings[k] and eff.get(k) != settings[k]
               for k in settings)


def plan_key(plan, dtype_name: str) -> str:
    import torch
    g = plan.geometry
    dev = torch.cuda.get_device_name(plan.device) if torch.cuda.is_available() else "cpu"
    return "|".join(str(x) for x in (plan.system.name, plan.sampling_freq, g.num_coherently_integrated_code_periods,
                                     g.num_noncoherent_accumulations, g.bit_edge_search_steps, g.num_doppler_bins,
                                     g.fft_size, len(plan.avail_prns), dtype_name, dev))


def cache_path() -> str:
    return os.environ.get("ACQ_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "acqgb300", "autotune.json"))


def load_cache(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(data: dict, path: str | None = None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def coordinate_descent(cost: Callable[[dict], float], start: dict, space: dict, passes: int = 2,
                       min_gain: float = 0.01):
    """Minimise cost over the product space, one knob at a time; a change is kept only when it
    lowers the cost by more than ``min_gain`` (relative), so timing noise does not move the
    shape. Returns (best, cost, trials)."""
    best = dict(start)
    best_c = cost(best)
    trials = [(dict(best), best_c)]
    for _ in range(passes):
        improved = False
        for k, vals in space.items():
            for v in vals:
                if best.get(k) == v:
                    continue
                trial = dict(best)
                trial[k] = v
                c = cost(trial)
                trials.append((trial, c))
                if c < best_c * (1.0 - min_gain):
                    best, best_c, improved = trial, c, True
        if not improved:
            break
    return best, best_c, trials


def tune(plan, signal_dev, prns, *, reps: int = 3, passes: int = 2, cache: str | None = None,
         allow_reduced_precision: bool = False, store: bool = True, knobs=None) -> dict:
    """Tune the plan's launch shapes on a device-resident signal; apply and cache the winner.
    ``knobs`` restricts the search to those names (default: every knob the plan has)."""
    import torch
    from .api import acquire_device, acquire_device_async, fetch_results
    space = {k: v for k, v in candidates(plan).items() if knobs is None or k in knobs}
    start = current(plan)
    # drop knobs the plan does not have
    for k in list(space):
        if k in KNOBS and not start.get(k):
            del space[k]
    start = {k: v for k, v in start.items() if k in space}
    form0 = start.get("form", "plain")
    if "form" not in space or plan.set_form("fused") != "fused":
        space.pop("form", None)
        start.pop("form", None)
    plan.set_form(form0)
    if allow_reduced_precision and plan.geometry.path == 2:
        space["rotation_precision"] = ["fp32", "fp16", "fp16_split"]
        start["rotation_precision"] = "fp32"
    stream = torch.cuda.ExternalStream(plan.stream_handle(), device=signal_dev.device)

    def cost(settings):
        if unavailable(settings, apply(plan, settings)):
            return float("inf")
        acquire_device(plan, signal_dev, prns)   # warm-up (and smem limits)
        ts = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            acquire_device_async(plan, signal_dev, prns)
            e1.record(stream)
            fetch_results(plan, prns)
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    best, best_ms, trials = coordinate_descent(cost, start, space, passes)
    apply(plan, best)
    if store:
        data = load_cache(cache)
        data[plan_key(plan, str(signal_dev.dtype))] = {"settings": best, "ms": best_ms, "trials": len(trials)}
        save_cache(data, cache)
    return {"settings": best, "ms": best_ms, "trials": len(trials),
            "start_ms": trials[0][1] if trials else None}


def apply_cached(plan, dtype_name: str, cache: str | None = None) -> dict | None:
    """Apply the cached shape for this geometry and GPU, if any."""
    entry = load_cache(cache).get(plan_key(plan, dtype_name))
    if not entry:
        return None
    apply(plan, entry["settings"])
    return entry

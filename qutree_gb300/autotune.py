"""Autotuner of the tensor-core bounds (qt_set_tc_thresholds).

For every contraction kind (mode products, hole products, last-index
accumulations) and every size a in 16..64 (steps of 8) it times, on the
device, the double-float compressed sweep of a probe problem whose
contractions all have size a -- a balanced tree of 64 modes with a-point
leaves and bonds a, a coupled-oscillator SOP with 256 random couplings --
once with that kind on the tensor cores (bound a) and once on the FP32
pipe (bound 65), the other two kinds on the FP32 pipe in both.  A kind's bound is the smallest size from
which the tensor cores win at every larger size (by at least 3%); 65 when
they never do.  The bounds are cached per device (name and SM count) as
JSON; HamiltonianRepresentation(..., tc_thresholds="auto") reads them.

    python -m qutree_gb300.autotune [--device 0] [--sizes 16,24,...]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import qtgpu
from .model import balanced_tree, coupled_oscillators, random_wavefunction

KINDS = ("mp", "hp", "acc")
SIZES = (16, 24, 32, 40, 48, 56, 64)
DEFAULT = {"mp": 32, "hp": 32, "acc": 32}


def _device_key(device: int) -> str:
    import torch
    p = torch.cuda.get_device_properties(device)
    return f"{p.name.replace(' ', '_')}-sm{p.multi_processor_count}"


def cache_path(device: int = 0) -> str:
    root = os.environ.get("QT_AUTOTUNE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "qtgpu"))
    return os.path.join(root, f"tc_bounds-{_device_key(device)}.json")


def cached(device: int = 0):
    """(mp, hp, acc) bounds cached for this device, or the built-in ones."""
    try:
        with open(cache_path(device)) as f:
            b = json.load(f)["bounds"]
        return tuple(int(b[k]) for k in KINDS)
    except (OSError, KeyError, ValueError):
        return tuple(DEFAULT[k] for k in KINDS)


def probe_problem(a: int, modes: int = 64, seed: int = 5):
    tree = balanced_tree(modes, a, a)
    sop = coupled_oscillators(tree, n_pairs=256, coupling=0.05, quartic=0.1, rng=np.random.default_rng(seed),
                              omega=1.0)
    return tree, sop, random_wavefunction(tree, seed)


def _time_sweeps(tree, sop, psi, bounds, device, reps=5):
    import torch
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC,
                                        device=device, tc_thresholds=bounds)
    try:
        st = torch.cuda.ExternalStream(h.stream())
        h.upload(psi)
        for _ in range(2):
            h.derivative()
        h.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            h.derivative()
        e1.record(st)
        h.sync()
        return e0.elapsed_time(e1) / reps
    finally:
        h.close()


def tune(device: int = 0, sizes=SIZES, write: bool = True, margin: float = 0.03):
    """Time the probes, pick the bounds, cache them; returns the record."""
    t0 = time.perf_counter()
    timings = {k: {} for k in KINDS}
    for a in sizes:
        tree, sop, psi = probe_problem(a)
        off = _time_sweeps(tree, sop, psi, (65, 65, 65), device)
        for i, k in enumerate(KINDS):
            bounds = [65, 65, 65]
            bounds[i] = a
            on = _time_sweeps(tree, sop, psi, tuple(bounds), device)
            timings[k][a] = {"tensor_cores_ms": on, "fp32_pipe_ms": off}
    chosen = {}
    for k in KINDS:
        bound = 65
        for a in sorted(sizes, reverse=True):  # the smallest size from which the tensor cores always win
            t = timings[k][a]
            if t["tensor_cores_ms"] <= (1.0 - margin) * t["fp32_pipe_ms"]:
                bound = a
            else:
                break
        chosen[k] = bound
    rec = {"device": _device_key(device), "bounds": chosen,
           "probe": "balanced tree of 64 modes, leaves and bonds a, coupled oscillators; compressed "
                    "double-float sweep, one kind on the tensor cores against none",
           "timings_ms": {k: {str(a): v for a, v in d.items()} for k, d in timings.items()},
           "wall_s": time.perf_counter() - t0}
    if write:
        p = cache_path(device)
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(rec, f, indent=1)
        rec["cache"] = p
    return rec


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--sizes", default=",".join(str(a) for a in SIZES))
    a = ap.parse_args(argv)
    rec = tune(a.device, tuple(int(x) for x in a.sizes.split(",")))
    print(json.dumps(rec))


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""H.Psi tree sweeps per second on one GB300 (QuTree ML-MCTDH hot path).

Workload: the 64-mode tree (physical dim 32, bonds 32 at the bottom growing to
64 below the top, 127 nodes, Psi 67 MB complex128) with the coupled-oscillator
SOP of 64 kinetic, 64 quartic on-site and 256 random pair terms.  One step =
one sweep = Derivative() (density matrices, regularised inverses, represent,
mean fields, LayerDerivative at every node) plus Expectation.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours      : the library's grouped complex128 plan; `value` with Psi resident in
            HBM; `e2e` through the C ABI with pinned host buffers (upload Psi,
            sweep, download dPsi and the energy every step).
reference : the reference algorithm (CPU restatement, zgemm through OpenBLAS on
            all host cores), one sweep per step.
Multi-GPU (torchrun): one independent replica per rank ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H·Ψ tree sweeps/sec: batched+mixed vs plain complex128 on 1 GB300 at |ΔE|≤1e-8"
WORKLOAD = "cfg1: 64-mode balanced binary tree, p=32, bonds 32..64, 384-term coupled-oscillator SOP"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch-trees", type=int, default=512,
                    help="trees in the supplementary many-tree batch (0: skip)")
    ap.add_argument("--no-scf", action="store_true", help="skip the supplementary SCF sweep timing")
    ap.add_argument("--no-cdvr", action="store_true", help="skip the supplementary CDVR sweep timing")
    ap.add_argument("--cdvr-sweeps", type=int, default=0,
                    help="only run this many CDVR sweeps of the CDVR workload (for profilers) and exit")
    ap.add_argument("--precision-steps", type=int, default=5,
                    help="CMF steps (dt 0.01) of the precision study on the 48..96-bond 64-mode tree: "
                         "every arithmetic propagated in lockstep with the reference (0: skip)")
    ap.add_argument("--precision-ref", default="f64", choices=["f64", "df64"],
                    help="reference arithmetic of the precision study (df64 for long runs: complex128 "
                         "costs ~4.5 s per step there)")
    ap.add_argument("--precision-only", action="store_true",
                    help="run only the precision study and print its JSON")
    ap.add_argument("--precision-log", default=None,
                    help="append every checkpoint of the precision study to this file as a JSON line")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), parts[5:9], float(parts[3])))
                except ValueError:
                    continue
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[3] for r in rows)}


def _rho_weighted_err(tree, dpsi, ref, rho):
    """max |(dPsi - ref) rho| / max |ref rho| over non-top nodes (undoes rho^-1)."""
    import numpy as np
    off = tree.offsets()
    ro = 0
    num = den = 0.0
    for n in tree.nodes:
        d = n.d_up
        R = rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        a = dpsi[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        b = ref[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        if not n.is_top:
            a, b = a @ R.T, b @ R.T
        num = max(num, float(np.abs(a - b).max()))
        den = max(den, float(np.abs(b).max()))
    return num / den


# DRAM bytes per sweep of the sum-of-products kernels (dram__bytes_read.sum +
# dram__bytes_write.sum over all launches of one sweep of the 64-mode
# workload, from one ncu capture of that sweep; the summary is committed
# beside the other profiles and named in TRAFFIC_SOURCE)
TRAFFIC = {0: 1531.5e6, 1: 3245.5e6, 2: 2104.8e6}
TRAFFIC_SOURCE = ("ncu capture of one sweep of the 64-mode workload, k_tcs launches only "
                  "(profiles/launches_sweep_64mode_compressed_df64_tc.md)")


def measured_peaks():
    """HBM GB/s and bf16 TFLOP/s (burst) measured on the GB300s, or
    the stated fallback when the file is absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return {"hbm_gbs": float(m["hbm_gbs"]), "bf16_tflops": float(m["bf16_tflops"]),
                "source": "measured (MEASURED_PEAKS.json)"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def cpu_baseline_sweep(tree, sop, psi, threads=None):
    """The reference algorithm on the host cores: the oracle restatement with
    QuTree's TensorBLAS path (zgemm from OpenBLAS, all cores, or `threads`).
    One full sweep is the sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    blas = oracle.attach_openblas(fast=True)
    oracle.set_blas_threads(threads or os.cpu_count())
    flat = psi.flat()
    t0 = time.perf_counter()
    r = oracle.derivative(tree, sop, flat, backend=oracle.BLAS, fast=True, want_mats=False)
    dt = time.perf_counter() - t0
    return dt, r.energy, blas


def run_reference(args, ws, rank):
    from qutree_gb300.model import config_problem
    if rank != 0:
        return
    tree, sop, psi = config_problem(args.config)
    cores = os.cpu_count()
    times, energy, blas = [], None, None
    warm = min(args.warmup, 1)
    for i in range(warm + args.steps):
        dt, energy, blas = cpu_baseline_sweep(tree, sop, psi)
        if i >= warm:
            times.append(dt)
    tot = sum(times)
    v = len(times) / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "sweeps/s", "n_gpus": 0,
        "steps": args.steps, "warmup": warm, "ms_per_step": 1e3 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "threads": cores, "blas": blas or "naive loops"},
        "energy": energy,
        "cpu_baseline": {"value": v, "unit": "sweeps/s", "cores": cores, "kind": "port",
                         "sample": "one full cfg1 sweep per step (reference call sequence, "
                                   "zgemm via OpenBLAS)"},
        "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.warmup > warm:
        line["note"] = f"warm-up capped at {warm} CPU sweep(s) to keep the run within minutes"
    print(json.dumps(line), flush=True)


OTHER_PLANS = (("compressed_complex128", "QT_PLAN_COMPRESSED", "QT_PREC_F64"),
               ("grouped_double_float", "QT_PLAN_GROUPED", "QT_PREC_DF64"),
               ("compressed_double_float", "QT_PLAN_COMPRESSED", "QT_PREC_DF64"),
               ("compressed_complex64", "QT_PLAN_COMPRESSED", "QT_PREC_C32"),
               ("compressed_tf32x3_tensor_cores", "QT_PLAN_COMPRESSED", "QT_PREC_TF32X3"))

PRECISIONS = (("df64", "QT_PREC_DF64"), ("df64_tc", "QT_PREC_DF64_TC"), ("c64", "QT_PREC_C32"),
              ("tf32x3", "QT_PREC_TF32X3"))


def precision_study(args, local):
    """Config[3]'s tree (64 modes, bonds 32/58/67/77/86/96, regularisation
    1e-8): the reference arithmetic and every other one propagate the same Psi
    in lockstep with constant-mean-field steps of dt = 0.01
    (qt_cmf_propagate); at checkpoints each runs one derivative sweep of its
    own state.  Reported per arithmetic: |dE| against the reference, the
    relative H.Psi error of the sweep (rho-weighted derivative, max over
    nodes), and ||Psi - Psi_ref|| / ||Psi||."""
    import numpy as np

    from qutree_gb300 import qtgpu
    from qutree_gb300.model import config_problem

    t3, s3, p3 = config_problem(3)
    ref_name = args.precision_ref
    ref_fl = qtgpu.QT_PREC_F64 if ref_name == "f64" else qtgpu.QT_PREC_DF64
    arith = [(n, getattr(qtgpu, c)) for n, c in PRECISIONS if not (ref_name == "df64" and n == "df64")]
    flat = p3.flat()
    ctx = {}
    for name, fl in [(ref_name, ref_fl)] + arith:
        h = qtgpu.HamiltonianRepresentation(s3, t3, flavour=qtgpu.QT_PLAN_COMPRESSED | fl, eps=1e-8, device=local)
        h.upload(flat)
        ctx[name] = h
    steps = args.precision_steps
    every = max(1, steps // 20)
    out = {n: {"trajectory": [], "worst": {"abs_dE": 0.0, "dpsi_rel_rho_weighted": 0.0, "psi_rel": 0.0}}
           for n, _ in arith}
    step_s = {n: 0.0 for n in ctx}
    energies = []
    t0 = time.perf_counter()
    for step in range(steps + 1):
        if step > 0:
            for n, h in ctx.items():
                ts = time.perf_counter()
                h.cmf(0.01, 1)
                h.sync()
                step_s[n] += time.perf_counter() - ts
        if step % every and step != steps:
            continue
        ref = ctx[ref_name]
        pr = ref.psi()
        ref.derivative()
        er = ref.energy()
        energies.append(er)
        rho = ref.matrices(qtgpu.QT_MAT_RHO)
        dref = ref.dpsi()
        for n, _ in arith:
            h = ctx[n]
            ph = h.psi()
            h.derivative()
            r = {"step": step, "abs_dE": abs(h.energy() - er),
                 "dpsi_rel_rho_weighted": _rho_weighted_err(t3, h.dpsi(), dref, rho),
                 "psi_rel": float(np.linalg.norm(ph - pr) / np.linalg.norm(pr))}
            out[n]["trajectory"].append(r)
            for k in out[n]["worst"]:
                out[n]["worst"][k] = max(out[n]["worst"][k], r[k])
        if args.precision_log:
            with open(args.precision_log, "a") as f:
                f.write(json.dumps({"step": step, "energy_ref": er, "wall_s": time.perf_counter() - t0,
                                    **{n: out[n]["trajectory"][-1] for n, _ in arith}}) + "\n")
    for n in ctx:
        ctx[n].close()
    for n, _ in arith:
        out[n]["final_abs_dE"] = out[n]["trajectory"][-1]["abs_dE"]
        out[n]["meets_1e-8"] = out[n]["worst"]["abs_dE"] <= 1e-8
        out[n]["s_per_cmf_step"] = step_s[n] / max(steps, 1)
    return {"workload": "64 modes, p=32, bonds 32,58,67,77,86,96, 384 terms, regularisation 1e-8",
            "propagation": f"{steps} constant-mean-field steps of dt = 0.01 (RK4 substeps with frozen mean "
                           f"fields), every arithmetic in lockstep from the same Psi, checkpoints every {every}",
            "reference": {"arithmetic": ref_name, "s_per_cmf_step": step_s[ref_name] / max(steps, 1),
                          "energies": energies},
            "arithmetics": out, "wall_s": time.perf_counter() - t0}


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    from qutree_gb300 import qtgpu
    from qutree_gb300.model import config_problem

    torch.cuda.set_device(local)
    tree, sop, psi = config_problem(args.config)
    flat = psi.flat()
    nbytes = flat.nbytes

    def timed_sweeps(flavour, steps, warmup):
        hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, device=local)
        stream = torch.cuda.ExternalStream(hrep.stream())
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
        hrep.upload(flat)
        for _ in range(warmup):
            hrep.derivative()
        hrep.sync()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        barrier(ws)
        torch.cuda.synchronize()
        n0 = hrep.ctx.launch_count()
        with Clocks(local) as clk:
            for i in range(steps):
                with torch.cuda.stream(stream):
                    flush.fill_(i & 0xFF)  # L2 (129 MB) flushed between sweeps, not timed
                ev[i][0].record(stream)
                hrep.derivative()
                ev[i][1].record(stream)
            hrep.sync()
            torch.cuda.synchronize()
        launches = hrep.ctx.launch_count() - n0
        barrier(ws)
        times = [a.elapsed_time(b) for a, b in ev]
        return hrep, times, clk.summary(), launches

    # compressed plan in double-float arithmetic: the headline
    head = qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC
    hrep, times, clocks, launches = timed_sweeps(head, args.steps, args.warmup)
    tot_ms = max_over_ranks(ws, sum(times))
    energy = hrep.energy()
    stats = hrep.stats()
    value = ws * args.steps / (tot_ms * 1e-3)

    # roofline: every stage launched alone, bracketed by events on the library stream
    stream = torch.cuda.ExternalStream(hrep.stream())
    stages = hrep.stages()
    per_kind = {}
    reps = 2
    for _ in range(reps):
        evs = []
        for i in range(len(stages)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            hrep.launch_stage(i)
            b.record(stream)
            evs.append((a, b))
        hrep.sync()
        for i, (a, b) in enumerate(evs):
            k = stages[i][0]
            d = per_kind.setdefault(k, {"ms": 0.0, "flops": 0.0, "bytes": 0.0, "launches": 0})
            d["ms"] += a.elapsed_time(b) / reps
            d["flops"] += stages[i][2] / reps
            d["bytes"] += stages[i][3] / reps
            d["launches"] += 1 / reps
    fp64_peak = hrep.ctx.fp64_peak()
    df64_peak = hrep.ctx.df64_peak()
    names = {0: "k_tcs<MP> + k_mp (mode products)", 1: "k_tcs<HP> + k_hp (hole products)",
             2: "k_tcs<ACC> + k_acc (last-mode accumulations)",
             3: "k_lin (matrix sums)", 4: "k_eig (density inverses)", 5: "k_proj (projectors)",
             6: "k_cvt (precision conversions)", 7: "k_grad (gradient preparation)",
             8: "k_mm (small matrix products)"}
    # stage kinds whose qualifying tasks run on the tensor cores (each stage
    # timed with its image pre-pass and, for the hole products, its partial sums)
    TENSOR_KINDS = (0, 1, 2)
    dom = max(per_kind, key=lambda k: per_kind[k]["ms"])
    d = per_kind[dom]
    c128_tflops = d["flops"] / (d["ms"] * 1e-3) / 1e12
    peaks = measured_peaks()
    # digit arithmetic: 28 digit pairs x 2 parts x 4 real products ... = 28 bf16
    # tensor flops per complex128-equivalent flop (8 per complex multiply-add)
    bf16_tflops = 28.0 * c128_tflops
    total_stage_ms = sum(v["ms"] for v in per_kind.values())
    kernels = {names[k]: {"ms": round(v["ms"], 3), "share": round(v["ms"] / total_stage_ms, 4),
                          "complex128_equivalent_tflops": round(v["flops"] / max(v["ms"], 1e-9) / 1e9, 4),
                          **({"bf16_tensor_tflops": round(28.0 * v["flops"] / max(v["ms"], 1e-9) / 1e9, 2)}
                             if k in TENSOR_KINDS else {}),
                          "launches_per_sweep": int(round(v["launches"]))}
               for k, v in sorted(per_kind.items())}
    hrep.close()

    # plain (reference call sequence) complex128 plan, and the grouped
    # complex128 plan, for comparison
    plain_steps = max(2, min(args.steps, 4))
    OTHERS = [(lab, getattr(qtgpu, p) | getattr(qtgpu, a)) for lab, p, a in OTHER_PLANS
              if getattr(qtgpu, p) | getattr(qtgpu, a) != head]
    hp, ptimes, _, _ = timed_sweeps(qtgpu.QT_PLAN_REFERENCE, plain_steps, 1)
    plain_value = plain_steps / (sum(ptimes) * 1e-3)
    plain_energy = hp.energy()
    plain_dpsi = hp.dpsi()
    plain_rho = hp.matrices(qtgpu.QT_MAT_RHO)
    hp.close()
    hg, gtimes, _, _ = timed_sweeps(qtgpu.QT_PLAN_GROUPED, plain_steps, 1)
    grouped64_value = plain_steps / (sum(gtimes) * 1e-3)
    hg.close()
    others = {}
    for label, fl in OTHERS:
        ho, otimes, _, _ = timed_sweeps(fl, plain_steps, 1)
        others[label] = {"value": plain_steps / (sum(otimes) * 1e-3), "unit": "sweeps/s",
                         "steps": plain_steps, "executed_gflop": ho.stats()["exec_flops"] / 1e9,
                         "abs_dE_vs_plain": abs(ho.energy() - plain_energy),
                         "energy_rel_err_vs_plain": abs(ho.energy() - plain_energy) / abs(plain_energy),
                         "dpsi_rel_rho_weighted_vs_plain": _rho_weighted_err(tree, ho.dpsi(), plain_dpsi, plain_rho)}
        ho.close()

    # error of the headline arithmetic against the complex128 plain plan (below)
    head_dpsi = None
    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=head, device=local)
        pin_in = torch.empty(flat.size * 2, dtype=torch.float64, pin_memory=True)
        pin_out = torch.empty(flat.size * 2, dtype=torch.float64, pin_memory=True)
        pin_in.numpy()[:] = flat.view(np.float64)
        in_np = pin_in.numpy().view(np.complex128)
        out_np = pin_out.numpy().view(np.complex128)
        for _ in range(max(1, args.warmup)):
            h.upload(in_np)
            h.derivative()
            h.dpsi_into(out_np)
            h.energy()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            h.upload(in_np)
            h.derivative()
            h.dpsi_into(out_np)
            h.energy()
        t1 = time.perf_counter()
        e2e_s = max_over_ranks(ws, t1 - t0)
        e2e = {"value": ws * args.steps / e2e_s, "unit": "sweeps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes + 32}
        head_dpsi = out_np.copy()
        h.close()

    # supplementary: many uneven trees in one graph-captured plan
    batch = None
    if args.batch_trees > 0:
        from qutree_gb300.model import batched_problem, forest, forest_psi, forest_sop
        trees_b, sops_b, psis_b = batched_problem(args.batch_trees)
        fb, _, mob = forest(trees_b)
        sb, pb = forest_sop(sops_b, mob), forest_psi(fb, psis_b)
        forest_e = {}
        batch = {"trees": args.batch_trees, "nodes": fb.n_nodes,
                 "workload": "uneven trees: modes in {8,16,32,48}, p in {8,16,32}, bonds 4..24 per "
                             "edge (balanced), 2..6 couplings per mode, own SOP per tree"}
        for label, fl in (("double_float", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64),
                          ("double_float_tensor_cores", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC),
                          ("grouped_double_float", qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64),
                          ("complex64", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_C32),
                          ("complex64_tf32x3_tensor_cores", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_TF32X3),
                          ("plain_complex128", qtgpu.QT_PLAN_REFERENCE)):
            hb = qtgpu.HamiltonianRepresentation(sb, fb, flavour=fl, device=local)
            sb_stream = torch.cuda.ExternalStream(hb.stream())
            hb.upload(pb)
            hb.derivative()
            hb.sync()
            nb = 3
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(sb_stream)
            for _ in range(nb):
                hb.derivative()
            e1.record(sb_stream)
            hb.sync()
            ms = e0.elapsed_time(e1) / nb
            batch[label] = {"ms_per_forest_sweep": ms, "tree_sweeps_per_s": args.batch_trees / (ms * 1e-3),
                            "executed_gflop": hb.stats()["exec_flops"] / 1e9}
            forest_e[label] = hb.energies()
            if label == "double_float":
                batch["energies_first4"] = forest_e[label][:4].tolist()
            hb.close()
        ep = forest_e["plain_complex128"]
        for label, e in forest_e.items():
            if label != "plain_complex128":
                batch[label]["max_rel_dE_vs_plain_complex128"] = float(
                    np.max(np.abs(e - ep) / np.maximum(1.0, np.abs(ep))))

    # supplementary: QuTree's SCF / Krylov sweep (qt_scf), one sweep of 5 Krylov
    # vectors per node; the oracle's numpy restatement timed on the 16-mode tree
    scf = None
    if not args.no_scf and rank == 0:
        scf = {"sweep": "one SCF iteration: every node in depth-first order with returns, "
                        "5 Lanczos vectors of the tail-free effective Hamiltonian, Ritz vector, "
                        "isometrisation toward the next node, edge-local rebuild",
               "arithmetic": "effective Hamiltonian and rebuilds in double-float; Lanczos vectors, "
                             "dot products and QR in complex128"}
        for cfg in (1, 4):
            t_s, s_s, p_s = config_problem(cfg)
            hs = qtgpu.HamiltonianRepresentation(s_s, t_s, flavour=qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PLAN_SCF
                                                 | qtgpu.QT_PREC_DF64, device=local)
            hs.upload(p_s.flat())
            hs.scf(n_iter=1, n_krylov=5)  # warm-up
            hs.upload(p_s.flat())
            n0 = hs.ctx.launch_count()
            t0 = time.perf_counter()
            E = hs.scf(n_iter=1, n_krylov=5)
            dt = time.perf_counter() - t0
            scf[f"cfg{cfg}"] = {"ms_per_scf_sweep": 1e3 * dt, "krylov_solves": len(E),
                                "krylov_solves_per_s": len(E) / dt, "final_ritz": float(E[-1]),
                                "gpu_launches": hs.ctx.launch_count() - n0}
            hs.close()
            if cfg == 4 and not args.no_cpu_baseline:
                # the compiled restatement (orc_scf) with zgemm from OpenBLAS on
                # all host cores, as the sweep's CPU baseline
                sys.path.insert(0, os.path.join(ROOT, "oracle"))
                import oracle
                blas = oracle.attach_openblas(fast=True)
                oracle.set_blas_threads(os.cpu_count())
                t0 = time.perf_counter()
                E_cpu, _ = oracle.scf(t_s, s_s, p_s.flat(), n_iter=1, n_krylov=5,
                                      backend=oracle.BLAS if blas else oracle.LOOPS, fast=True)
                dt_cpu = time.perf_counter() - t0
                scf["cfg4"]["cpu_oracle"] = {"ms_per_scf_sweep": 1e3 * dt_cpu, "kind": "port",
                                             "cores": os.cpu_count(),
                                             "sample": "one SCF iteration of the 16-mode tree, the compiled "
                                                       "restatement (orc_scf), zgemm via "
                                                       f"{'OpenBLAS on all host cores' if blas else 'naive loops'}",
                                             "max_abs_ritz_diff": float(np.abs(E_cpu - E).max())}

    # supplementary: the energy gradient (QT_PLAN_GRADIENT) on the 16-mode
    # differentiation workload, compressed double-float vs the plain sequence
    grad = None
    if rank == 0:
        t4, s4, p4 = config_problem(4)
        grad = {"workload": "16 modes, p=32, bonds 32, 152 terms; one sweep = derivative + dE/dPhi* of every node"}
        grads = {}
        for label, fl in (("compressed_double_float", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64),
                          ("compressed_double_float_tensor_cores", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC),
                          ("compressed_complex64", qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_C32),
                          ("plain_complex128", qtgpu.QT_PLAN_REFERENCE)):
            hg4 = qtgpu.HamiltonianRepresentation(s4, t4, flavour=fl | qtgpu.QT_PLAN_GRADIENT, device=local)
            g_stream = torch.cuda.ExternalStream(hg4.stream())
            hg4.upload(p4.flat())
            for _ in range(2):
                hg4.derivative()
            hg4.sync()
            ng = 5
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(g_stream)
            for _ in range(ng):
                hg4.derivative()
            e1.record(g_stream)
            hg4.sync()
            ms = e0.elapsed_time(e1) / ng
            grad[label] = {"ms_per_gradient_sweep": ms, "gradient_sweeps_per_s": 1e3 / ms,
                           "executed_gflop": hg4.stats()["exec_flops"] / 1e9}
            grads[label] = hg4.gradient()
            hg4.close()
        gp = grads["plain_complex128"]
        for label, g in grads.items():
            if label != "plain_complex128":
                grad[label]["gradient_rel_err_vs_plain_complex128"] = float(
                    np.abs(g - gp).max() / np.abs(gp).max())

    # supplementary: a Hamiltonian with a CDVR potential (QT_PLAN_CDVR): one
    # sweep = CDVR update (X matrices, grids, potentials on node and edge
    # grids, correction tensors) + build + derivative with the CDVR term
    cdvr = None
    if not args.no_cdvr and rank == 0:
        cdvr = cdvr_section(args, local, torch)

    # the precision study: every arithmetic against the reference along a
    # constant-mean-field propagation of the 48..96-bond tree
    precision = None
    if args.precision_steps > 0 and rank == 0:
        precision = precision_study(args, local)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "df64",
        "data": "synthetic (seeded N(0,1) node tensors, QR-orthonormalised)",
        "config": {"workload": WORKLOAD, "plan": "compressed (per node one block matrix of the terms "
                   "inside its subtree, summed mean fields per boundary restriction, represent chains "
                   "kept in HBM for Apply), double-float arithmetic: mode products, hole products and "
                   "last-mode accumulations of shapes 32..64 on the tcgen05 tensor cores as exact bf16 "
                   "digit products, the rest on the FP32 pipe (complex128 in and out; density inverses "
                   "complex128)",
                   "parallelism": f"replicas x{ws}",
                   "l2": "flushed between timed sweeps (256 MB fill, outside the events)"},
        "energy": energy,
        "plain_complex128": {"value": plain_value, "unit": "sweeps/s", "steps": plain_steps,
                             "energy": plain_energy, "plan": "reference call sequence"},
        "grouped_complex128": {"value": grouped64_value, "unit": "sweeps/s", "steps": plain_steps},
        **others,
        "error_vs_complex128": {"abs_dE": abs(energy - plain_energy),
                                "rel_dE": abs(energy - plain_energy) / abs(plain_energy),
                                "dpsi_rel_rho_weighted": _rho_weighted_err(tree, head_dpsi, plain_dpsi, plain_rho)
                                if head_dpsi is not None else None},
        "flops_per_sweep": {"reference_algorithm": stats["ref_flops"], "executed": stats["exec_flops"]},
        "roofline": ({"bound": "tensor", "kernel": names[dom], "achieved": bf16_tflops,
                      "peak": peaks["bf16_tflops"], "unit": "TFLOP/s (bf16 digit products on the tensor cores)",
                      "frac": bf16_tflops / peaks["bf16_tflops"],
                      "peak_source": peaks["source"] + ", bf16 burst",
                      "achieved_note": "28 bf16 tensor flops per complex128-equivalent flop of the reference "
                                       "algorithm (seven digits per operand, 28 digit pairs)",
                      "complex128_equivalent_tflops": c128_tflops,
                      "df64_fp32_pipe_peak_tflops": df64_peak,
                      "speedup_over_df64_fp32_pipe_peak": c128_tflops / df64_peak,
                      "fp64_pipe_peak_tflops": fp64_peak,
                      "traffic": TRAFFIC.get(dom), "traffic_unit": "bytes per sweep (all launches of the kernel)",
                      "traffic_source": TRAFFIC_SOURCE, "kernels": kernels}
                     if dom in TENSOR_KINDS else
                     {"bound": "fp32 pipe (double-float arithmetic)", "kernel": names[dom], "achieved": c128_tflops,
                      "unit": "TFLOP/s (complex128-equivalent)", "peak": df64_peak, "frac": c128_tflops / df64_peak,
                      "peak_source": "measured in this run (qt_probe_df64_peak)", "traffic": None,
                      "kernels": kernels}),
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if e2e:
        line["e2e"] = e2e
    if batch:
        line["batched_forest"] = batch
    if scf:
        line["scf"] = scf
    if precision:
        line["precision"] = precision
    if grad:
        line["gradient"] = grad
    if cdvr:
        line["cdvr"] = cdvr
    if not args.no_cpu_baseline and args.config == 1:
        dt, cpu_e, blas = cpu_baseline_sweep(tree, sop, psi)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "sweeps/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": "one full cfg1 sweep, reference call sequence, zgemm via "
                                          f"{'OpenBLAS' if blas else 'naive loops'}",
                                "energy_diff": abs(cpu_e - energy)}
        dt1, _, _ = cpu_baseline_sweep(tree, sop, psi, threads=1)
        line["cpu_baseline"]["single_thread"] = {"value": 1.0 / dt1, "unit": "sweeps/s", "cores": 1,
                                                 "sample": "the same sweep, OpenBLAS on one thread"}
    print(json.dumps(line), flush=True)


CDVR_KINDS = {0: "k_mp", 1: "k_hp", 2: "k_acc", 3: "k_lin", 4: "k_eig", 5: "k_proj", 9: "k_tc (strided contractions)",
              10: "k_gs (Gram-Schmidt)", 11: "k_eigf (spectral functions)",
              12: "k_wsd (joint diagonalisation)", 13: "k_vpot (potential on grids)",
              14: "k_dvl (local corrections)", 15: "k_ew (V times Xi)"}


def cdvr_section(args, local, torch):
    """16 modes, HO-DVR p = 16, bonds 12, kinetic SOP + contrib's CDVRModelV."""
    import numpy as np

    from qutree_gb300 import qtgpu
    from qutree_gb300.model import cdvr_problem

    tree, sop, psi, xs, V = cdvr_problem(16, 16, 12)
    flat = psi.flat()
    out = {"workload": "16 modes, HO-DVR p=16, bonds 12, 16 kinetic terms + CDVRModelV(16) potential "
                       "(32 polynomial terms); one sweep = CDVR update + build + derivative",
           "metric": "H.Psi sweeps/s with the CDVR potential"}
    for label, fl in (("grouped", qtgpu.QT_PLAN_GROUPED), ("reference_sequence", qtgpu.QT_PLAN_REFERENCE)):
        h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=fl, potential=V, leaf_x=xs, device=local)
        st = torch.cuda.ExternalStream(h.stream())
        h.upload(flat)
        for _ in range(2):
            h.derivative()
        h.sync()
        steps = 5
        n0 = h.ctx.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            h.derivative()
        e1.record(st)
        h.sync()
        ms = e0.elapsed_time(e1) / steps
        rec = {"ms_per_sweep": ms, "sweeps_per_s": 1e3 / ms, "energy": h.energy(),
               "gpu_launches_per_sweep": (h.ctx.launch_count() - n0) // steps,
               "executed_gflop": h.stats()["exec_flops"] / 1e9}
        if label == "grouped":
            stages = h.stages()
            per = {}
            evs = []
            for i in range(len(stages)):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                h.launch_stage(i)
                b.record(st)
                evs.append((a, b))
            h.sync()
            for i, (a, b) in enumerate(evs):
                k = CDVR_KINDS.get(stages[i][0], str(stages[i][0]))
                d = per.setdefault(k, {"ms": 0.0, "launches": 0})
                d["ms"] += a.elapsed_time(b)
                d["launches"] += 1
            tot = sum(v["ms"] for v in per.values())
            rec["kernels"] = {k: {"ms": round(v["ms"], 3), "share": round(v["ms"] / tot, 4),
                                  "launches_per_sweep": v["launches"]} for k, v in per.items()}
            # end to end through the C ABI: Psi from pinned host memory in, dPsi and the energy back
            pin_in = torch.empty(flat.size * 2, dtype=torch.float64, pin_memory=True)
            pin_out = torch.empty(flat.size * 2, dtype=torch.float64, pin_memory=True)
            pin_in.numpy()[:] = flat.view(np.float64)
            in_np = pin_in.numpy().view(np.complex128)
            out_np = pin_out.numpy().view(np.complex128)
            t0 = time.perf_counter()
            for _ in range(steps):
                h.upload(in_np)
                h.derivative()
                h.dpsi_into(out_np)
                h.energy()
            dt = (time.perf_counter() - t0) / steps
            rec["e2e"] = {"value": 1.0 / dt, "unit": "sweeps/s", "h2d_bytes_per_step": flat.nbytes,
                          "d2h_bytes_per_step": flat.nbytes + 32}
        out[label] = rec
        h.close()
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import cdvr as cdvr_oracle
        t0 = time.perf_counter()
        res = cdvr_oracle.derivative(tree, sop, flat, cdvr_oracle.CDVROracle(tree, xs, V))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "one sweep of the same workload: the oracle's numpy restatement "
                                         "(its bundled BLAS on its default threads, up to all host cores) "
                                         "with its single-threaded C joint diagonalisation",
                               "energy": float((res.h00 / res.s00).real),
                               "note": "energies differ at ~1e-9: the joint diagonalisation's accept/reject "
                                       "steps make the grids discontinuous in rounding-level input changes"}
    return out


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.cdvr_sweeps > 0:  # profiling aid: the CDVR workload's sweeps, nothing else
        from qutree_gb300 import qtgpu
        from qutree_gb300.model import cdvr_problem
        tree, sop, psi, xs, V = cdvr_problem(16, 16, 12)
        h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED, potential=V, leaf_x=xs,
                                            device=local)
        h.upload(psi.flat())
        for _ in range(args.cdvr_sweeps):
            h.derivative()
        h.sync()
        print(json.dumps({"cdvr_sweeps": args.cdvr_sweeps, "energy": h.energy()}))
        h.close()
        return
    if args.precision_only:
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            print(json.dumps({"precision": precision_study(args, local)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

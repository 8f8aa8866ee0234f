"""Run H.Psi sweeps of a benchmark configuration from the command line.

  python -m qutree_gb300.run --config 1 --sweeps 2 [--flavour compressed|grouped|reference]
                             [--prec f64|df64|df64_tc|c32|tf32x3]

Prints one line per sweep (energy, milliseconds).  Used to profile the
library (ncu) with a fixed, small launch sequence: qt_prepare, then
``--sweeps`` graph launches of the sweep.
"""
from __future__ import annotations

import argparse
import time

from . import qtgpu
from .model import config_problem


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--sweeps", type=int, default=2)
    ap.add_argument("--flavour", default="compressed", choices=["compressed", "grouped", "reference"])
    ap.add_argument("--prec", default="f64", choices=["f64", "df64", "df64_tc", "c32", "tf32x3"])
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    tree, sop, psi = config_problem(a.config)
    flavour = {"compressed": qtgpu.QT_PLAN_COMPRESSED, "grouped": qtgpu.QT_PLAN_GROUPED,
               "reference": qtgpu.QT_PLAN_REFERENCE}[a.flavour]
    flavour |= {"f64": qtgpu.QT_PREC_F64, "df64": qtgpu.QT_PREC_DF64, "df64_tc": qtgpu.QT_PREC_DF64_TC,
                "c32": qtgpu.QT_PREC_C32, "tf32x3": qtgpu.QT_PREC_TF32X3}[a.prec]
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, device=a.device)
    hrep.upload(psi)
    for i in range(a.sweeps):
        t0 = time.perf_counter()
        hrep.derivative()
        e = hrep.energy()  # synchronises
        print(f"sweep {i}: E = {e:.15f}  {1e3 * (time.perf_counter() - t0):.2f} ms", flush=True)
    st = hrep.stats()
    print(f"launches/sweep {int(st['launches'])}  executed GFLOP {st['exec_flops'] / 1e9:.2f}  "
          f"reference GFLOP {st['ref_flops'] / 1e9:.2f}  scratch MiB {st['scratch_bytes'] / 2**20:.0f}")
    hrep.close()


if __name__ == "__main__":
    main()

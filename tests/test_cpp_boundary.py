"""The C ABI from C++: the QuTree-side GpuSweep shim of the integration
guide, compiled with g++ against include/qtgpu.h and linked against
libqtgpu.so, around minimal stand-ins for QuTree's Tree / Tensorcd /
Hamiltonian types (tests/cpp/).  The shim replaces QuTree's Derivative()
(src/TreeClasses/HamiltonianRepresentation.cpp:74-81).

CPU: the documented shim and the compiled one are the same text, and the
translation unit compiles and links.  GPU: the compiled program sweeps the
8-mode workload and matches the oracle (complex128 plans at 1e-12,
double-float at 1e-11, as the other parity tests)."""
import os
import re
import struct
import subprocess

import numpy as np
import pytest

import oracle
from helpers import deriv_errors
from qutree_gb300 import build as qbuild
from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
SRC = os.path.join(CPP, "gpu_sweep_shim.cpp")
EXE = os.path.join(qbuild.BUILD, "gpu_sweep_shim")


def _class_text(text):
    m = re.search(r"^class GpuSweep \{.*?^\};$", text, re.S | re.M)
    assert m, "no GpuSweep class"
    return m.group(0)


def test_documented_shim_is_the_compiled_one():
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    src = open(SRC).read()
    assert _class_text(doc) == _class_text(src)


def _build_exe():
    lib = qbuild.build()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdirs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                           os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                           os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(d)]
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", CPP,
           SRC, "-o", EXE + ".tmp", lib, *[f"-L{d}" for d in libdirs], "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(lib)}", *[f"-Wl,-rpath,{d}" for d in libdirs]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    os.replace(EXE + ".tmp", EXE)
    return EXE


def test_shim_compiles_and_links():
    assert os.path.exists(_build_exe())


def _write_problem(path, tree, sop, flat):
    order, dims, parent, child_idx, leaf_mode = tree.descriptor()
    with open(path, "wb") as f:
        f.write(struct.pack("<i", tree.n_nodes))
        p = 0
        for a in range(tree.n_nodes):
            f.write(struct.pack("<i", int(order[a])))
            f.write(np.asarray(dims[p:p + order[a]], "<i4").tobytes())
            p += int(order[a])
            f.write(struct.pack("<iii", int(parent[a]), int(child_idx[a]), int(leaf_mode[a])))
        f.write(struct.pack("<i", tree.n_leaves))
        for m in range(tree.n_leaves):
            f.write(struct.pack("<i", tree.leaf_dim(m)))
        ops = sop.ops
        f.write(struct.pack("<i", len(ops.kind)))
        for k, d, v in zip(ops.kind, ops.dim, ops.data):
            f.write(struct.pack("<ii", int(k), int(d)))
            f.write(np.ascontiguousarray(v, "<c16").tobytes())
        f.write(struct.pack("<i", len(sop)))
        for c, t in zip(sop.coeffs, sop.terms):
            f.write(struct.pack("<ddi", c.real, c.imag, len(t.factors)))
            for m, o in t.factors:
                f.write(struct.pack("<ii", int(m), int(o)))
        f.write(np.ascontiguousarray(flat, "<c16").tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("flavour,tol", [
    (qtgpu.QT_PLAN_REFERENCE, 1e-12),
    (qtgpu.QT_PLAN_GROUPED, 1e-12),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64, 1e-11),
])
def test_shim_sweep_matches_oracle(tmp_path, flavour, tol):
    exe = _build_exe()
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    prob, res = str(tmp_path / "problem.bin"), str(tmp_path / "result.bin")
    _write_problem(prob, tree, sop, flat)
    r = subprocess.run([exe, prob, res, str(flavour)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(res, dtype="<f8")
    h00, s00 = complex(out[0], out[1]), complex(out[2], out[3])
    dpsi = out[4:].view(np.complex128)
    ref = oracle.derivative(tree, sop, flat)
    assert abs(h00.real / s00.real - ref.energy) <= tol * max(1.0, abs(ref.energy))
    err, noise = deriv_errors(tree, dpsi, ref.dpsi, ref.rho)
    assert err <= tol and noise <= 1e-11

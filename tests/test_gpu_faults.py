"""Failure handling of the C ABI without faulting the GPU.

Allocation failures are injected on the host (QT_FAULT_INJECT=alloc:N makes
the library's N-th device allocation fail as if the device were full):
every allocation of qt_prepare, of the CMF work vectors and of qt_dev_alloc
fails once, the call returns QT_ERR_ALLOC, and the context stays usable --
the same context prepares again and sweeps to the oracle's result.  The
reference's counterpart is cerr + exit(1) (src/Core/TensorBLAS.cpp:238-268);
the library returns status codes instead."""
import os
import uuid

import numpy as np
import pytest

import oracle
from helpers import deriv_errors, rel_err
from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu


def _inject(n):
    # a fresh value restarts the library's count
    os.environ["QT_FAULT_INJECT"] = f"alloc:{n}#{uuid.uuid4().hex}"


@pytest.fixture
def clean_env():
    yield
    os.environ.pop("QT_FAULT_INJECT", None)


@pytest.mark.parametrize("flavour", [qtgpu.QT_PLAN_GROUPED,
                                     qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64 | qtgpu.QT_PLAN_GRADIENT])
def test_every_prepare_allocation_fails_cleanly(clean_env, flavour):
    tree, sop, psi = config_problem(0)
    ref = oracle.derivative(tree, sop, psi.flat())
    ctx = qtgpu.Context(0)
    try:
        failed = 0
        for n in range(1, 64):
            _inject(n)
            try:
                hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, ctx=ctx)
            except qtgpu.QtError as e:
                assert e.code == 3 and "allocation failed" in str(e), str(e)
                failed += 1
                continue
            break  # the n-th allocation lies past the last one of qt_prepare
        assert failed >= 5  # the arena buffers and the task tables
        os.environ.pop("QT_FAULT_INJECT")
        # the context that saw every failure still prepares and sweeps correctly
        hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, ctx=ctx)
        dpsi = qtgpu.Derivative(hrep, psi.flat())
        h00, s00 = hrep.energy_parts()
        assert abs((h00 - ref.h00) / ref.h00) < 1e-11
        err, _ = deriv_errors(tree, dpsi, ref.dpsi, ref.rho)
        assert err < 1e-10
    finally:
        ctx.close()


def _cmf_psi(tree, sop, psi, n_fail=None):
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED)
    try:
        hrep.upload(psi.flat())
        if n_fail is not None:
            _inject(n_fail)
            with pytest.raises(qtgpu.QtError, match="QT_ERR_ALLOC"):
                hrep.cmf(0.01, 1)
            os.environ.pop("QT_FAULT_INJECT")
            hrep.upload(psi.flat())
        hrep.cmf(0.01, 2)
        return hrep.psi()
    finally:
        hrep.close()


def test_cmf_and_dev_alloc_failures(clean_env):
    tree, sop, psi = config_problem(0)
    want = _cmf_psi(tree, sop, psi)
    # each of the three CMF work vectors (allocated on first use) fails once;
    # the propagation that follows on the same context is unaffected
    for n in (1, 2, 3):
        assert rel_err(_cmf_psi(tree, sop, psi, n), want) == 0.0
    ctx = qtgpu.Context(0)
    try:
        _inject(1)
        with pytest.raises(qtgpu.QtError, match="QT_ERR_ALLOC"):
            ctx.alloc(1 << 20)
        os.environ.pop("QT_FAULT_INJECT")
        ctx.free(ctx.alloc(1 << 20))
    finally:
        ctx.close()

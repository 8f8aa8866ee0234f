"""The tensor-core bounds (qt_set_tc_thresholds) and their autotuner.
With every kind kept on the FP32 pipe (bounds 65) the tensor-core plan runs
exactly the FP32-pipe double-float sweep (bit for bit); the autotuner times
its probes, caches bounds per device and HamiltonianRepresentation(...,
tc_thresholds="auto") reads them back; bounds outside 1..65 are rejected."""
import numpy as np
import pytest

import oracle as O
from qutree_gb300 import autotune, qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu
TC = qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC


def _sweep(flavour, bounds=None):
    tree, sop, psi = config_problem(4)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, tc_thresholds=bounds)
    try:
        d = qtgpu.Derivative(h, psi.flat())
        return d, h.energy()
    finally:
        h.close()


def test_bounds_65_give_the_fp32_pipe_sweep():
    d_tc, e_tc = _sweep(TC, (65, 65, 65))
    d_df, e_df = _sweep(qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64)
    assert np.array_equal(d_tc, d_df) and e_tc == e_df
    d_on, _ = _sweep(TC, (32, 32, 32))
    assert not np.array_equal(d_on, d_df)


def test_bounds_out_of_range_are_rejected():
    tree, sop, _ = config_problem(0)
    with pytest.raises(qtgpu.QtError, match="QT_ERR_ARG"):
        qtgpu.HamiltonianRepresentation(sop, tree, flavour=TC, tc_thresholds=(0, 32, 32))


def test_autotune_caches_and_applies(tmp_path, monkeypatch):
    monkeypatch.setenv("QT_AUTOTUNE_DIR", str(tmp_path))
    rec = autotune.tune(0, sizes=(32, 64))
    assert set(rec["bounds"]) == {"mp", "hp", "acc"}
    assert all(v in (32, 64, 65) for v in rec["bounds"].values())
    for k in ("mp", "hp", "acc"):
        for a in ("32", "64"):
            t = rec["timings_ms"][k][a]
            assert t["tensor_cores_ms"] > 0 and t["fp32_pipe_ms"] > 0
    assert autotune.cached(0) == tuple(rec["bounds"][k] for k in ("mp", "hp", "acc"))
    tree, sop, psi = config_problem(4)
    r = O.derivative(tree, sop, psi.flat(), want_mats=False)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=TC, tc_thresholds="auto")
    try:
        qtgpu.Derivative(h, psi.flat())
        assert abs(h.energy() - r.energy) <= 1e-10 * abs(r.energy)
    finally:
        h.close()

"""GPU primitives through the C ABI against the oracle (matvec_/rhomat_/
multStateAB semantics), square and rectangular, every mode."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from qutree_gb300.qtgpu import Context
    c = Context(0)
    yield c
    c.close()


def _rand(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


SHAPES = [
    # before, activeB, activeC, after
    (1, 16, 16, 4), (4, 4, 4, 4), (32, 38, 38, 1), (58, 58, 58, 64), (1, 64, 64, 64),
    (3364, 64, 64, 1), (7, 5, 9, 3), (1, 1, 1, 1), (1, 96, 96, 2), (1000, 3, 3, 7),
]


@pytest.mark.parametrize("before,aB,aC,after", SHAPES)
@pytest.mark.parametrize("add", [False, True])
def test_mode_product(ctx, before, aB, aC, after, add):
    rng = np.random.default_rng(before * 7 + aB + aC * 3 + after)
    B = _rand(rng, before * aB * after)
    h = _rand(rng, aC * aB)
    C0 = _rand(rng, before * aC * after)
    ref = O.mode_product(h, B, before, aB, aC, after, C=C0.copy(), add=add)
    dB, dh, dC = ctx.to_device(B), ctx.to_device(h), ctx.to_device(C0)
    ctx.mode_product(dC, dh, dB, before, aB, aC, after, add=add)
    got = ctx.from_device(dC, C0.shape)
    for p in (dB, dh, dC):
        ctx.free(p)
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("before,aA,aB,after", [
    (1, 16, 16, 4), (4, 4, 4, 4), (3364, 64, 64, 1), (58, 58, 58, 64), (1, 58, 58, 3712),
    (7, 5, 9, 3), (1, 1, 1, 1), (1, 96, 96, 33), (16, 33, 31, 5)])
def test_hole_product(ctx, before, aA, aB, after):
    rng = np.random.default_rng(before + aA * 5 + aB + after * 11)
    A = _rand(rng, before * aA * after)
    B = _rand(rng, before * aB * after)
    ref = O.hole_product(A, B, before, aA, aB, after)
    dA, dB = ctx.to_device(A), ctx.to_device(B)
    dS = ctx.to_device(np.zeros(aA * aB, complex))
    ctx.hole_product(dS, dA, dB, before, aA, aB, after)
    got = ctx.from_device(dS, (aA * aB,))
    for p in (dA, dB, dS):
        ctx.free(p)
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_last_mode_product(ctx):
    rng = np.random.default_rng(3)
    R, d = 3364, 64
    B = _rand(rng, R * d)
    A = _rand(rng, d * d)
    ref = O.mode_product(A, B, R, d, d, 1)
    dA, dB = ctx.to_device(A), ctx.to_device(B)
    dC = ctx.to_device(np.zeros(R * d, complex))
    ctx.last_mode_product(dC, dA, dB, R, d)
    got = ctx.from_device(dC, (R * d,))
    for p in (dA, dB, dC):
        ctx.free(p)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_bad_geometry_is_rejected(ctx):
    from qutree_gb300.qtgpu import QtError
    p = ctx.alloc(64)
    with pytest.raises(QtError, match="QT_ERR_SHAPE"):
        ctx.mode_product(p, p + 16, p + 32, 0, 1, 1, 1)
    with pytest.raises(QtError, match="QT_ERR_ARG"):
        ctx.mode_product(p, p + 16, p, 1, 1, 1, 1)  # C aliases B
    ctx.free(p)

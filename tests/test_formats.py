"""QuTree's TENS / TTre / MATR / SMTr binary formats (CPU), byte for byte."""
import io
import struct

import numpy as np
import pytest

from qutree_gb300 import formats
from qutree_gb300.model import config_problem


def test_tens_bytes_match_the_reference_layout():
    # Tensor::write (include/Core/Tensor_Implementation.h:204-222) of a
    # (2, 3) complex tensor: "TENS" "TDIM" order dims sizeof coefficients
    a = np.arange(6).reshape((2, 3), order="F") * (1 + 0.5j)
    b = io.BytesIO()
    formats.write_tensor(b, a)
    want = (b"TENS" + b"TDIM" + struct.pack("<iii", 2, 2, 3) + struct.pack("<i", 16)
            + a.ravel(order="F").astype(np.complex128).tobytes())
    assert b.getvalue() == want
    b.seek(0)
    assert np.array_equal(formats.read_tensor(b), a)


def test_ttre_round_trip(tmp_path):
    tree, _, psi = config_problem(0)
    p = str(tmp_path / "psi.ttre")
    formats.write_tensor_tree(p, psi)
    raw = open(p, "rb").read()
    assert raw[:4] == b"TTre" and struct.unpack("<i", raw[4:8])[0] == tree.n_nodes
    back = formats.read_tensor_tree(p, tree)
    assert all(np.array_equal(x, y) for x, y in zip(back.tensors, psi.tensors))


def test_ttre_shape_mismatch_is_rejected(tmp_path):
    tree0, _, psi0 = config_problem(0)
    tree4, _, _ = config_problem(4)
    p = str(tmp_path / "psi.ttre")
    formats.write_tensor_tree(p, psi0)
    with pytest.raises(ValueError):
        formats.read_tensor_tree(p, tree4)


def test_matrix_and_sparse_matrix_tree(tmp_path):
    rng = np.random.default_rng(0)
    mats = [rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)) for d in (2, 3, 1)]
    b = io.BytesIO()
    formats.write_matrix(b, mats[0])
    assert b.getvalue()[:4] == b"MATR" and struct.unpack("<QQi", b.getvalue()[4:24]) == (2, 2, 16)
    p = str(tmp_path / "h.smtr")
    formats.write_sparse_matrix_tree(p, mats)
    back = formats.read_sparse_matrix_tree(p)
    assert all(np.array_equal(x, y) for x, y in zip(back, mats))

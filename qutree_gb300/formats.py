"""QuTree's binary formats for tensors, tensor trees and matrix trees.

Byte layouts (little endian, as QuTree writes them on x86/Arm):
  TDIM  "TDIM", int32 order, int32 dims[order]
        (TensorShape::write, src/Core/TensorShape.cpp:68-84)
  TENS  "TENS", TDIM, int32 sizeof(T), coefficients column-major
        (Tensor::write, include/Core/Tensor_Implementation.h:204-222)
  TTre  "TTre", int32 node count, TENS per node in address order
        (TensorTree::write, include/TreeClasses/TensorTree_Implementation.h:78-92)
  MATR  "MATR", size_t dim1, size_t dim2, int32 sizeof(T), coefficients
        (Matrix::write, include/Core/Matrix_Implementation.h:365-378)
  SMTr  "SMTr", int32 node count, MATR per active node in address order
        (SparseMatrixTree::write, src/TreeClasses/SparseMatrixTree.cpp:26-39)
Wavefunctions written by QuTree load here and vice versa; the same layout
is read and written by qt_psi_load / qt_psi_save of the C ABI.
"""
from __future__ import annotations

import struct

import numpy as np

from .model import TensorTree, Tree


def _check(tag: bytes, want: bytes):
    if tag != want:
        raise ValueError(f"wrong keyword: expected {want!r}, found {tag!r}")


def write_tensor(f, a: np.ndarray):
    a = np.asarray(a)
    f.write(b"TENS")
    f.write(b"TDIM")
    f.write(struct.pack("<i", a.ndim))
    f.write(struct.pack(f"<{a.ndim}i", *a.shape))
    dt = np.complex128 if np.iscomplexobj(a) else np.float64
    f.write(struct.pack("<i", np.dtype(dt).itemsize))
    f.write(np.asarray(a, dtype=dt).ravel(order="F").tobytes())


def read_tensor(f) -> np.ndarray:
    _check(f.read(4), b"TENS")
    _check(f.read(4), b"TDIM")
    (order,) = struct.unpack("<i", f.read(4))
    shape = struct.unpack(f"<{order}i", f.read(4 * order))
    (size,) = struct.unpack("<i", f.read(4))
    dt = {16: np.complex128, 8: np.float64}.get(size)
    if dt is None:
        raise ValueError(f"unsupported element size {size}")
    n = int(np.prod(shape))
    data = np.frombuffer(f.read(n * size), dtype=dt, count=n)
    return data.reshape(shape, order="F").copy()


def write_tensor_tree(path: str, psi: TensorTree):
    with open(path, "wb") as f:
        f.write(b"TTre")
        f.write(struct.pack("<i", len(psi.tensors)))
        for t in psi.tensors:
            write_tensor(f, t)


def read_tensor_tree(path: str, tree: Tree | None = None) -> TensorTree | list:
    """Node tensors of a TTre file; checked against ``tree`` when given."""
    with open(path, "rb") as f:
        _check(f.read(4), b"TTre")
        (n,) = struct.unpack("<i", f.read(4))
        ts = [read_tensor(f) for _ in range(n)]
    if tree is None:
        return ts
    if n != tree.n_nodes or any(tuple(t.shape) != nd.shape for t, nd in zip(ts, tree.nodes)):
        raise ValueError("TTre file does not match the tree")
    return TensorTree(tree, ts)


def write_matrix(f, m: np.ndarray):
    m = np.asarray(m)
    f.write(b"MATR")
    f.write(struct.pack("<QQ", m.shape[0], m.shape[1]))
    dt = np.complex128 if np.iscomplexobj(m) else np.float64
    f.write(struct.pack("<i", np.dtype(dt).itemsize))
    f.write(np.asarray(m, dtype=dt).ravel(order="F").tobytes())


def read_matrix(f) -> np.ndarray:
    _check(f.read(4), b"MATR")
    d1, d2 = struct.unpack("<QQ", f.read(16))
    (size,) = struct.unpack("<i", f.read(4))
    dt = {16: np.complex128, 8: np.float64}[size]
    data = np.frombuffer(f.read(d1 * d2 * size), dtype=dt, count=d1 * d2)
    return data.reshape((d1, d2), order="F").copy()


def write_sparse_matrix_tree(path: str, mats):
    """One term's matrices (active nodes in address order)."""
    with open(path, "wb") as f:
        f.write(b"SMTr")
        f.write(struct.pack("<i", len(mats)))
        for m in mats:
            write_matrix(f, m)


def read_sparse_matrix_tree(path: str):
    with open(path, "rb") as f:
        _check(f.read(4), b"SMTr")
        (n,) = struct.unpack("<i", f.read(4))
        return [read_matrix(f) for _ in range(n)]

"""Host-side containers for the Schur-reduced block system (no arithmetic on the solve path).

``BSR`` mirrors the reference container ``ressim::BSR`` (engine/include/ressim/bsr.h:23-37): ``n`` block rows,
``nb`` unknowns per cell, ``rowPtr[n+1]`` / ``col[nnzb]`` (int32, columns sorted per row), ``val[nnzb*nb*nb]``
(float64, row-major blocks, row = equation, column = unknown). Vectors are interleaved per cell
(p, Sw, x_g for the black-oil system).

``ScalarCSR`` mirrors ``ressim::CSR`` (engine/include/ressim/linsolve.h:11-17): the full Newton Jacobian with
the well (BHP) rows appended after the ``na * nv`` cell rows, as the simulator assembles it.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class BSR:
    n: int
    nb: int
    rowPtr: np.ndarray
    col: np.ndarray
    val: np.ndarray

    def __post_init__(self):
        self.rowPtr = np.ascontiguousarray(self.rowPtr, dtype=np.int32)
        self.col = np.ascontiguousarray(self.col, dtype=np.int32)
        self.val = np.ascontiguousarray(self.val, dtype=np.float64).reshape(-1)
        if self.rowPtr.size != self.n + 1:
            raise ValueError("rowPtr must have n+1 entries")
        if self.val.size != int(self.rowPtr[-1]) * self.nb * self.nb:
            raise ValueError("val must hold nnzb*nb*nb values")

    @property
    def nnzb(self) -> int:
        return int(self.rowPtr[-1])

    @property
    def size(self) -> int:
        return self.n * self.nb

    def blocks(self) -> np.ndarray:
        return self.val.reshape(self.nnzb, self.nb, self.nb)

    def diag(self) -> np.ndarray:
        """Position of the diagonal block of every row (-1 when absent), as ``BSR::finalizeDiag``."""
        rows = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.rowPtr))
        d = np.full(self.n, -1, dtype=np.int64)
        hit = np.nonzero(self.col == rows)[0]
        d[rows[hit]] = hit
        return d

    def scaled(self, s: float) -> "BSR":
        return BSR(self.n, self.nb, self.rowPtr.copy(), self.col.copy(), self.val * s)

    def structurally_symmetric(self) -> bool:
        rows = np.repeat(np.arange(self.n, dtype=np.int64), np.diff(self.rowPtr))
        a = rows * self.n + self.col
        b = self.col.astype(np.int64) * self.n + rows
        return bool(np.array_equal(np.sort(a), np.sort(b)))


@dataclass
class ScalarCSR:
    rowPtr: np.ndarray
    col: np.ndarray
    val: np.ndarray

    def __post_init__(self):
        self.rowPtr = np.ascontiguousarray(self.rowPtr, dtype=np.int32)
        self.col = np.ascontiguousarray(self.col, dtype=np.int32)
        self.val = np.ascontiguousarray(self.val, dtype=np.float64)

    @property
    def n(self) -> int:
        return self.rowPtr.size - 1


@dataclass
class NewtonSystem:
    """One Schur-reduced Newton system: S x = b, optional accumulation blocks (true-IMPES CPR weights),
    optional full Jacobian with well rows, and (synthetic systems) the manufactured solution."""
    A: BSR
    b: np.ndarray
    acc: np.ndarray | None = None
    full: ScalarCSR | None = None
    full_b: np.ndarray | None = None
    na: int = 0
    nv: int = 3
    nw: int = 0
    x_true: np.ndarray | None = None
    meta: dict = field(default_factory=dict)


def read_dump(path: str):
    """Read the simulator's RESSIM_DUMP file (engine/src/simulator.cpp:3252-3263): header
    ``[n, na, nv, nw, nnz]`` then rowPtr, col, val, rhs; and the optional ``<path>.acc`` side file of
    accumulation blocks (engine/src/simulator.cpp:3314-3315). Returns (ScalarCSR, rhs, na, nv, nw, acc|None)."""
    with open(path, "rb") as f:
        n, na, nv, nw, nnz = struct.unpack("<5i", f.read(20))
        rp = np.frombuffer(f.read(4 * (n + 1)), dtype=np.int32).copy()
        ci = np.frombuffer(f.read(4 * nnz), dtype=np.int32).copy()
        v = np.frombuffer(f.read(8 * nnz), dtype=np.float64).copy()
        b = np.frombuffer(f.read(8 * n), dtype=np.float64).copy()
    acc = None
    try:
        acc = np.fromfile(path + ".acc", dtype=np.float64)
        if acc.size != na * nv * nv:
            acc = None
    except OSError:
        acc = None
    return ScalarCSR(rp, ci, v), b, na, nv, nw, acc


def write_lsbench(path: str, J: ScalarCSR, rhs, na: int, nv: int, nw: int, acc=None):
    """Write a full Jacobian in the layout tools/lsbench.cpp:22-40 reads: header ``[n, nnz, na, nv, nw]``, rowPtr,
    col, val, rhs, then an int32 ``hasAcc`` and, if set, the na*nv*nv accumulation blocks. The simulator's own dump
    (read_dump) orders its header ``[n, na, nv, nw, nnz]`` and keeps the blocks in a ``.acc`` side file; this writes
    the same content in the benchmark's layout."""
    rp = np.ascontiguousarray(J.rowPtr, dtype=np.int32)
    n = rp.size - 1
    nnz = int(rp[-1])
    with open(path, "wb") as f:
        f.write(struct.pack("<5i", n, nnz, na, nv, nw))
        f.write(rp.tobytes())
        f.write(np.ascontiguousarray(J.col, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(J.val, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(rhs, dtype=np.float64).tobytes())
        f.write(struct.pack("<i", 0 if acc is None else 1))
        if acc is not None:
            f.write(np.ascontiguousarray(acc, dtype=np.float64).tobytes())


def read_system(path: str) -> NewtonSystem:
    """Read a captured Schur-reduced system (format written by oracle/ref_capture.cpp)."""
    with open(path, "rb") as f:
        magic, ver, n, nb, nnzb, maxit = struct.unpack("<6i", f.read(24))
        if magic != 0x42475352:
            raise ValueError("not a system file")
        (tol,) = struct.unpack("<d", f.read(8))
        rp = np.frombuffer(f.read(4 * (n + 1)), dtype=np.int32).copy()
        ci = np.frombuffer(f.read(4 * nnzb), dtype=np.int32).copy()
        v = np.frombuffer(f.read(8 * nnzb * nb * nb), dtype=np.float64).copy()
        b = np.frombuffer(f.read(8 * n * nb), dtype=np.float64).copy()
    return NewtonSystem(BSR(n, nb, rp, ci, v), b, meta={"tol": tol, "maxIt": maxit})


def save_npz(path: str, sysm: NewtonSystem, **extra):
    d = dict(n=sysm.A.n, nb=sysm.A.nb, rowPtr=sysm.A.rowPtr, col=sysm.A.col, val=sysm.A.val, b=sysm.b)
    if sysm.acc is not None:
        d["acc"] = sysm.acc
    d.update(extra)
    np.savez_compressed(path, **d)


def load_npz(path: str):
    z = np.load(path)
    A = BSR(int(z["n"]), int(z["nb"]), z["rowPtr"], z["col"], z["val"])
    acc = z["acc"] if "acc" in z.files else None
    return NewtonSystem(A, z["b"].copy(), acc=acc), z

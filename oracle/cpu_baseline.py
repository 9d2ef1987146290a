"""Threaded CPU apply of the oracle plan (TEST INFRASTRUCTURE / CPU BASELINE ONLY).

Wraps oracle/cpu_apply.c, a C restatement of the reference's output-sector-owned threaded
apply (src/threaded_apply.jl:58-84, :506-609) of the fused static kernel
(src/liouvillian.jl:3070-3105).  bench.py times it as the CPU baseline; tests use it to
check it against the numpy oracle.  The library is built by ``build()`` into
oracle/_build/ (gcc -O3 -fopenmp), never shipped with the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from . import pi_oracle as O

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libpioracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "cpu_apply.c"
    if not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(tmp)],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


class _Plan(C.Structure):
    _fields_ = [("nsec", C.c_int), ("off", C.c_void_p), ("dim", C.c_void_p),
                ("h_ptr", C.c_void_p), ("h_row", C.c_void_p), ("h_col", C.c_void_p), ("h_val", C.c_void_p),
                ("q_ptr", C.c_void_p), ("q_row", C.c_void_p), ("q_col", C.c_void_p), ("q_val", C.c_void_p),
                ("ncg", C.c_int), ("cg_rate", C.c_void_p),
                ("k_ptr", C.c_void_p), ("k_row", C.c_void_p), ("k_col", C.c_void_p), ("k_val", C.c_void_p),
                ("br_ptr", C.c_void_p), ("br_in", C.c_void_p), ("br_scale", C.c_void_p),
                ("c_ptr", C.c_void_p), ("c_row", C.c_void_p), ("c_col", C.c_void_p), ("c_val", C.c_void_p)]


def _coo(blocks):
    ptr, rows, cols, vals = [0], [], [], []
    for B in blocks:
        Bc = B.tocoo()
        rows.append(Bc.row.astype(np.int32))
        cols.append(Bc.col.astype(np.int32))
        vals.append(Bc.data.astype(np.complex128))
        ptr.append(ptr[-1] + Bc.nnz)
    cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros(0, dt), dtype=dt)
    return (np.array(ptr, dtype=np.int64), cat(rows, np.int32), cat(cols, np.int32),
            cat(vals, np.complex128))


class ThreadedApply:
    """CPU L x with output-sector-owned threads for one oracle plan."""

    def __init__(self, plan: "O.Plan"):
        b = plan.basis
        S = len(b.sectors)
        self.n = len(b)
        zero = [None] * S
        import scipy.sparse as sp
        empty = [sp.csc_matrix((d, d), dtype=np.complex128) for d in b.dims]
        self._keep = []
        keep = self._keep.append
        off = np.array(b.offsets[:-1], dtype=np.int64)
        dim = np.array(b.dims, dtype=np.int32)
        h = _coo(plan.ham if plan.ham is not None else empty)
        q = _coo(plan.loss if plan.loss is not None else empty)
        kblocks = [K for blocks, _ in plan.collective_gains for K in blocks]
        k = _coo(kblocks)
        rates = np.array([r for _, r in plan.collective_gains] or [0.0], dtype=np.float64)
        # one-body branches grouped by output sector
        branches = []
        for brs, contr, rate in plan.onebody_gains:
            for (li, ni, bscale), Cm in zip(brs, contr):
                branches.append((li, ni, rate * bscale, Cm))
        branches.sort(key=lambda t: t[0])
        br_ptr = np.zeros(S + 1, dtype=np.int64)
        for li, *_ in branches:
            br_ptr[li + 1] += 1
        br_ptr = np.cumsum(br_ptr).astype(np.int64)
        br_in = np.array([t[1] for t in branches] or [0], dtype=np.int32)
        br_scale = np.array([t[2] for t in branches] or [0.0], dtype=np.float64)
        c = _coo([t[3] for t in branches])
        del zero
        arrays = [off, dim, *h, *q, rates, *k, br_ptr, br_in, br_scale, *c]
        for a in arrays:
            keep(a)
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        self.plan = _Plan(S, p(off), p(dim), p(h[0]), p(h[1]), p(h[2]), p(h[3]), p(q[0]), p(q[1]), p(q[2]),
                          p(q[3]), len(plan.collective_gains), p(rates), p(k[0]), p(k[1]), p(k[2]), p(k[3]),
                          p(br_ptr), p(br_in), p(br_scale), p(c[0]), p(c[1]), p(c[2]), p(c[3]))
        self.lib = C.CDLL(str(build()))
        self.lib.oracle_apply.argtypes = [C.POINTER(_Plan), C.c_void_p, C.c_void_p, C.c_int]
        self.lib.oracle_apply.restype = C.c_int

    def __call__(self, x, y=None, threads=None):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if y is None:
            y = np.empty_like(x)
        threads = threads or os.cpu_count() or 1
        self.lib.oracle_apply(C.byref(self.plan), x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p),
                              int(threads))
        return y

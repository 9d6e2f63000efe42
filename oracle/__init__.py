"""CPU oracle for the GB300 solver: TEST INFRASTRUCTURE ONLY.

Two ctypes front ends:

* ``Oracle``  -- the plain-C restatement of the reference path (``oracle/rsg_oracle.c``, built into
  ``oracle/liborc.so`` by ``oracle/Makefile``). It travels with the repository and is built on every host.
* ``RefShim`` -- the reference engine itself (compiled from its own sources by ``oracle/Makefile.ref``
  into ``oracle/_ref/``), available only where the reference tree exists. Used to generate and to
  re-check the golden vectors under ``tests/golden/``.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import this
package, and only as the checker / the timed CPU baseline. The product (``ressim_gb300``) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libressim_ref.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build(quiet: bool = True) -> str:
    """Compile ``liborc.so`` (a few seconds, gcc)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _opt_f64(a):
    return None if a is None else _arr(a, np.float64).ctypes.data_as(C.c_void_p)


class Oracle:
    """ctypes front end of ``liborc.so`` (the C restatement)."""

    def __init__(self, path: str = LIB):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.L = L
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_invert_block.argtypes = [_f64p, C.c_int]
        L.orc_invert_block.restype = C.c_int
        L.orc_bsr_spmv.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_bilu0_factor.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p]
        L.orc_bilu0_factor.restype = C.c_int
        L.orc_bilu0_factor_lean.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f32p]
        L.orc_bilu0_factor_lean.restype = C.c_int
        L.orc_bilu0_factor_f32.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f32p]
        L.orc_bilu0_factor_f32.restype = C.c_int
        L.orc_set_mc_smoother.argtypes = [C.c_int]
        L.orc_set_mc_smoother.restype = None
        L.orc_bilu0_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_bilu0_apply_fd.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f32p, _f64p, _f64p]
        L.orc_bilu0_apply_ff.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f32p, _f64p, _f64p]
        L.orc_level_sets.argtypes = [C.c_int, _i32p, _i32p, C.c_int, _i32p, _i32p]
        L.orc_level_sets.restype = C.c_int
        L.orc_prec_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, _f64p, _f64p]
        L.orc_prec_apply.restype = C.c_int
        L.orc_solve_timed.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, C.c_int, C.c_int, _f64p, _f64p,
                                      C.c_double, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
        L.orc_solve_timed.restype = C.c_int
        L.orc_refine_float.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_refine_float.restype = C.c_int
        L.orc_cpr_setup.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int]
        L.orc_cpr_setup.restype = C.c_void_p
        L.orc_mcbilu0_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_mcbilu0_apply.restype = C.c_int
        L.orc_devcpr_setup.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p]
        L.orc_devcpr_setup.restype = C.c_void_p
        L.orc_devcpr_apply.argtypes = [C.c_void_p, _f32p, _f32p]
        L.orc_devcpr_apply.restype = None
        L.orc_devcpr_levels.argtypes = [C.c_void_p]
        L.orc_devcpr_levels.restype = C.c_int
        L.orc_devcpr_has_inverse.argtypes = [C.c_void_p]
        L.orc_devcpr_has_inverse.restype = C.c_int
        L.orc_devcpr_free.argtypes = [C.c_void_p]
        L.orc_devcpr_free.restype = None
        L.orc_cpr_weights.argtypes = [C.c_void_p]
        L.orc_cpr_weights.restype = C.POINTER(C.c_double)
        L.orc_cpr_amg.argtypes = [C.c_void_p]
        L.orc_cpr_amg.restype = C.c_void_p
        L.orc_cpr_free.argtypes = [C.c_void_p]
        L.orc_amg_levels.argtypes = [C.c_void_p]
        L.orc_amg_levels.restype = C.c_int
        L.orc_amg_level_info.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_amg_level_get.argtypes = [C.c_void_p, C.c_int, _i32p, _i32p, _f64p, C.c_void_p]
        L.orc_wellschur.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_int, _f64p, C.c_int, _i32p, _i32p, _f64p,
                                    _f64p]
        L.orc_wellschur.restype = C.c_int
        L.orc_wellschur_recover.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_int, _f64p, _f64p, _f64p]
        L.orc_wellschur_recover.restype = C.c_int

    def set_threads(self, n: int):
        self.L.orc_set_threads(int(n))

    # ---- kernels
    def invert_block(self, a):
        a = _arr(a, np.float64).copy()
        ok = self.L.orc_invert_block(a, int(round(np.sqrt(a.size))))
        return a, bool(ok)

    def spmv(self, A, x):
        y = np.zeros(A.n * A.nb)
        self.L.orc_bsr_spmv(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(x, np.float64), y)
        return y

    def bilu0_factor(self, A):
        lu = np.zeros_like(A.val)
        nreg = self.L.orc_bilu0_factor(A.n, A.nb, A.rowPtr, A.col, A.val, lu)
        return lu, nreg

    def bilu0_factor_lean(self, A):
        luf = np.zeros(A.val.size, dtype=np.float32)
        nreg = self.L.orc_bilu0_factor_lean(A.n, A.nb, A.rowPtr, A.col, A.val, luf)
        return luf, nreg

    def set_mc_smoother(self, on: bool):
        """AMG smoother: multicolour Gauss-Seidel (the device's FP32 precision forms) or the reference's (default)."""
        self.L.orc_set_mc_smoother(1 if on else 0)

    def bilu0_factor_f32(self, A):
        luf = np.zeros(A.val.size, dtype=np.float32)
        nreg = self.L.orc_bilu0_factor_f32(A.n, A.nb, A.rowPtr, A.col, A.val, luf)
        return luf, nreg

    def bilu0_apply(self, A, lu, r):
        z = np.zeros(A.n * A.nb)
        self.L.orc_bilu0_apply(A.n, A.nb, A.rowPtr, A.col, _arr(lu, np.float64), _arr(r, np.float64), z)
        return z

    def bilu0_apply_fd(self, A, luf, r):
        z = np.zeros(A.n * A.nb)
        self.L.orc_bilu0_apply_fd(A.n, A.nb, A.rowPtr, A.col, _arr(luf, np.float32), _arr(r, np.float64), z)
        return z

    def bilu0_apply_ff(self, A, luf, r):
        z = np.zeros(A.n * A.nb)
        self.L.orc_bilu0_apply_ff(A.n, A.nb, A.rowPtr, A.col, _arr(luf, np.float32), _arr(r, np.float64), z)
        return z

    def level_sets(self, A, forward=True):
        ordv = np.zeros(A.n, dtype=np.int32)
        start = np.zeros(A.n + 1, dtype=np.int32)
        nl = self.L.orc_level_sets(A.n, A.rowPtr, A.col, 1 if forward else 0, ordv, start)
        return ordv, start[: nl + 1].copy()

    def prec_apply(self, A, r, prec=0, acc=None):
        z = np.zeros(A.n * A.nb)
        accv = None if acc is None else _arr(acc, np.float64)
        self.L.orc_prec_apply(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), prec,
                              _arr(r, np.float64), z)
        return z

    def solve(self, A, b, prec=0, method=0, restart=30, tol=1e-6, maxit=120, acc=None):
        """Returns (x, converged, iterations, relres, setup_s, solve_s)."""
        x = np.zeros(A.n * A.nb)
        its, rr, ts, tv = C.c_int(0), C.c_double(0), C.c_double(0), C.c_double(0)
        accv = None if acc is None else _arr(acc, np.float64)
        conv = self.L.orc_solve_timed(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p),
                                      prec, method, restart, _arr(b, np.float64), x, tol, maxit, C.byref(its), C.byref(rr),
                                      C.byref(ts), C.byref(tv))
        return x, bool(conv), its.value, rr.value, ts.value, tv.value

    def refine_float(self, A, b, tol=1e-8, max_outer=6, inner_it=120):
        x = np.zeros(A.n * A.nb)
        its, rr = C.c_int(0), C.c_double(0)
        conv = self.L.orc_refine_float(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(b, np.float64), x, tol, max_outer, inner_it,
                                       C.byref(its), C.byref(rr))
        return x, bool(conv), its.value, rr.value

    def mcbilu0_apply(self, A, r):
        """Multicolour BILU0 (engine/src/bsr.cpp:599-730): z = M^-1 r."""
        z = np.zeros(A.n * A.nb)
        self.L.orc_mcbilu0_apply(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(r, np.float64), z)
        return z

    def devcpr_apply(self, A, r):
        """GPU-shaped float CPR-AMG (engine/src/bsr.cpp:1217-1371): z = M^-1 r in float32."""
        rf = np.ascontiguousarray(r, dtype=np.float32)
        z = np.zeros(A.n * A.nb, dtype=np.float32)
        h = self.L.orc_devcpr_setup(A.n, A.nb, A.rowPtr, A.col, A.val)
        try:
            self.L.orc_devcpr_apply(h, rf, z)
        finally:
            self.L.orc_devcpr_free(h)
        return z

    def cpr_info(self, A, acc=None):
        """CPR weights and the AMG hierarchy: (w, [(rows, nnz)], [level CSR + aggregates])."""
        accv = None if acc is None else _arr(acc, np.float64)
        h = self.L.orc_cpr_setup(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), 0)
        try:
            w = np.ctypeslib.as_array(self.L.orc_cpr_weights(h), shape=(A.n * A.nb,)).copy()
            amg = self.L.orc_cpr_amg(h)
            L = self.L.orc_amg_levels(amg)
            info, levels = [], []
            for l in range(L):
                rows, nnz = C.c_int(0), C.c_int(0)
                self.L.orc_amg_level_info(amg, l, C.byref(rows), C.byref(nnz))
                rp = np.zeros(rows.value + 1, dtype=np.int32)
                ci = np.zeros(nnz.value, dtype=np.int32)
                v = np.zeros(nnz.value)
                agg = np.zeros(rows.value, dtype=np.int32)
                self.L.orc_amg_level_get(amg, l, rp, ci, v, agg.ctypes.data_as(C.c_void_p))
                info.append((rows.value, nnz.value))
                levels.append((rp, ci, v, agg))
            return w, info, levels
        finally:
            self.L.orc_cpr_free(h)

    def cpr_handle(self, A, acc=None, lean=False):
        """A set-up BlockCPR (engine/src/bsr.cpp:993-1084) kept for repeated applications: ``h.apply(r)``."""
        return _CprHandle(self, A, acc, lean)

    def bo_assemble(self, model: dict, p, sw, x, state, acc_old, dt, add_pos=None, add_val=None, radd_pos=None, radd_val=None):
        """The reference's black-oil assembly restated in C (rsg_oracle_asm.c): J (the model's pattern) and R at the
        state, with the well terms as ordered addends, rows scaled by dt / PV. The model dict has the keys of
        tests/golden/waterflood_asm.npz (described by ressim_gb300.assembly.model_structs)."""
        from ressim_gb300.assembly import model_structs
        g, f, s, rowPtr, col, keep = model_structs(model)
        nrows = int(rowPtr.size - 1)
        fn = self.L.orc_bo_assemble
        fn.argtypes = [C.c_void_p] * 6 + [C.c_void_p] * 5 + [C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                              C.c_void_p, C.c_void_p, C.c_void_p]
        fn.argtypes[3] = C.c_int
        fn.restype = C.c_int
        st = [_arr(p, np.float64), _arr(sw, np.float64), _arr(x, np.float64), np.ascontiguousarray(state, dtype=np.uint8),
              _arr(acc_old, np.float64)]
        ap = np.ascontiguousarray(add_pos if add_pos is not None else np.zeros(0), dtype=np.int64)
        av = _arr(add_val if add_val is not None else np.zeros(0), np.float64)
        rp = np.ascontiguousarray(radd_pos if radd_pos is not None else np.zeros(0), dtype=np.int32)
        rv = _arr(radd_val if radd_val is not None else np.zeros(0), np.float64)
        J = np.empty(int(rowPtr[-1]))
        R = np.empty(nrows)
        q = lambda a: C.c_void_p(a.ctypes.data) if a.size else None  # noqa: E731
        rc = fn(C.byref(g), C.byref(f), C.byref(s), nrows, q(rowPtr), q(col), *[q(a) for a in st], float(dt), int(ap.size), q(ap), q(av),
                int(rp.size), q(rp), q(rv), q(J), q(R))
        del keep
        if rc != 0:
            raise RuntimeError(f"orc_bo_assemble: {rc} (pattern is not the engine's)")
        return J, R

    def wellschur(self, J, na, nv, nw, b):
        """J: scalar CSR (rowPtr, col, val); returns (S as BSR-like dict, bc) or None."""
        rp, ci, v = (_arr(J[0], np.int32), _arr(J[1], np.int32), _arr(J[2], np.float64))
        nrows = rp.size - 1
        cap = 16
        while True:
            sRp = np.zeros(na + 1, dtype=np.int32)
            sCol = np.zeros(cap, dtype=np.int32)
            sVal = np.zeros(cap * nv * nv)
            bc = np.zeros(na * nv)
            r = self.L.orc_wellschur(nrows, rp, ci, v, na, nv, nw, _arr(b, np.float64), cap, sRp, sCol, sVal, bc)
            if r == 0:
                return None
            if r < 0:
                cap = -r
                continue
            return (sRp, sCol[:r].copy(), sVal[: r * nv * nv].copy()), bc

    def wellschur_recover(self, J, na, nv, nw, b, xc):
        rp, ci, v = (_arr(J[0], np.int32), _arr(J[1], np.int32), _arr(J[2], np.float64))
        x = np.zeros(rp.size - 1)
        self.L.orc_wellschur_recover(rp.size - 1, rp, ci, v, na, nv, nw, _arr(b, np.float64), _arr(xc, np.float64), x)
        return x


class _CprHandle:
    """Owner of one ``orc_cpr`` set-up; freed with the object."""

    def __init__(self, o: Oracle, A, acc, lean):
        self.L = o.L
        self.L.orc_cpr_apply.argtypes = [C.c_void_p, _f64p, _f64p]
        self.L.orc_cpr_apply.restype = None
        self.N = A.n * A.nb
        accv = None if acc is None else _arr(acc, np.float64)
        self._acc = accv
        self.h = self.L.orc_cpr_setup(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p),
                                      1 if lean else 0)

    def apply(self, r):
        z = np.zeros(self.N)
        self.L.orc_cpr_apply(self.h, _arr(r, np.float64), z)
        return z

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_cpr_free(self.h)
            self.h = None


class RefShim:
    """ctypes front end of the reference engine's own solver classes (``oracle/_ref/libressim_ref.so``)."""

    def __init__(self, path: str = REF_LIB):
        L = C.CDLL(path)
        self.L = L
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_bsr_spmv.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.ref_bilu0_factor.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p]
        L.ref_bilu0_factor.restype = C.c_int
        L.ref_bilu0_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_int]
        L.ref_bilu0_apply.restype = C.c_int
        L.ref_bilu0f_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.ref_prec_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, _f64p, _f64p]
        L.ref_prec_apply.restype = C.c_int
        L.ref_solve.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double,
                                C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.ref_solve.restype = C.c_int
        L.ref_cpr_info.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, _f64p, _i32p, _i32p, C.c_int]
        L.ref_cpr_info.restype = C.c_int
        L.ref_amg_level.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, _i32p, _i32p, _f64p, _i32p]
        L.ref_amg_level.restype = C.c_int
        L.ref_wellschur.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_int, _f64p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.POINTER(C.c_int)]
        L.ref_wellschur.restype = C.c_int
        L.ref_wellschur_recover.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_int, _f64p, _f64p, _f64p]
        L.ref_wellschur_recover.restype = C.c_int
        L.ref_refine_float.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.ref_refine_float.restype = C.c_int
        L.ref_mcbilu0_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.ref_mcbilu0_apply.restype = C.c_int
        L.ref_devcpr_apply.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f32p, _f32p]
        L.ref_devcpr_apply.restype = C.c_int
        L.ref_set_threads(1)

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_LIB)

    def spmv(self, A, x):
        y = np.zeros(A.n * A.nb)
        self.L.ref_bsr_spmv(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(x, np.float64), y)
        return y

    def bilu0_factor(self, A):
        lu = np.zeros_like(A.val)
        nreg = self.L.ref_bilu0_factor(A.n, A.nb, A.rowPtr, A.col, A.val, lu)
        return lu, nreg

    def bilu0_apply(self, A, r, level_mode=0):
        z = np.zeros(A.n * A.nb)
        self.L.ref_bilu0_apply(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(r, np.float64), z, level_mode)
        return z

    def bilu0f_apply(self, A, r):
        z = np.zeros(A.n * A.nb)
        self.L.ref_bilu0f_apply(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(r, np.float64), z)
        return z

    def prec_apply(self, A, r, prec=0, acc=None):
        z = np.zeros(A.n * A.nb)
        accv = None if acc is None else _arr(acc, np.float64)
        self.L.ref_prec_apply(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), prec,
                              _arr(r, np.float64), z)
        return z

    def solve(self, A, b, prec=0, method=0, restart=30, tol=1e-6, maxit=120, acc=None):
        x = np.zeros(A.n * A.nb)
        its, rr = C.c_int(0), C.c_double(0)
        accv = None if acc is None else _arr(acc, np.float64)
        conv = self.L.ref_solve(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), prec,
                                method, restart, _arr(b, np.float64), x, tol, maxit, C.byref(its), C.byref(rr))
        return x, bool(conv), its.value, rr.value

    def mcbilu0_apply(self, A, r):
        z = np.zeros(A.n * A.nb)
        self.L.ref_mcbilu0_apply(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(r, np.float64), z)
        return z

    def devcpr_apply(self, A, r):
        rf = np.ascontiguousarray(r, dtype=np.float32)
        z = np.zeros(A.n * A.nb, dtype=np.float32)
        self.L.ref_devcpr_apply(A.n, A.nb, A.rowPtr, A.col, A.val, rf, z)
        return z

    def cpr_info(self, A, acc=None):
        accv = None if acc is None else _arr(acc, np.float64)
        w = np.zeros(A.n * A.nb)
        sizes = np.zeros(16, dtype=np.int32)
        nnz = np.zeros(16, dtype=np.int32)
        L = self.L.ref_cpr_info(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), w, sizes,
                                nnz, 16)
        levels = []
        for l in range(L):
            rp = np.zeros(sizes[l] + 1, dtype=np.int32)
            ci = np.zeros(nnz[l], dtype=np.int32)
            v = np.zeros(nnz[l])
            agg = np.zeros(sizes[l], dtype=np.int32)
            self.L.ref_amg_level(A.n, A.nb, A.rowPtr, A.col, A.val, None if accv is None else accv.ctypes.data_as(C.c_void_p), l, rp, ci, v,
                                 agg)
            levels.append((rp, ci, v, agg))
        return w, [(int(sizes[l]), int(nnz[l])) for l in range(L)], levels

    def wellschur(self, J, na, nv, nw, b):
        rp, ci, v = (_arr(J[0], np.int32), _arr(J[1], np.int32), _arr(J[2], np.float64))
        nrows = rp.size - 1
        nnzb = C.c_int(0)
        if not self.L.ref_wellschur(nrows, rp, ci, v, na, nv, nw, _arr(b, np.float64), None, None, None, None, C.byref(nnzb)):
            return None
        sRp = np.zeros(na + 1, dtype=np.int32)
        sCol = np.zeros(nnzb.value, dtype=np.int32)
        sVal = np.zeros(nnzb.value * nv * nv)
        bc = np.zeros(na * nv)
        self.L.ref_wellschur(nrows, rp, ci, v, na, nv, nw, _arr(b, np.float64), sRp.ctypes.data_as(C.c_void_p),
                             sCol.ctypes.data_as(C.c_void_p), sVal.ctypes.data_as(C.c_void_p), bc.ctypes.data_as(C.c_void_p),
                             C.byref(nnzb))
        return (sRp, sCol, sVal), bc

    def wellschur_recover(self, J, na, nv, nw, b, xc):
        rp, ci, v = (_arr(J[0], np.int32), _arr(J[1], np.int32), _arr(J[2], np.float64))
        x = np.zeros(rp.size - 1)
        self.L.ref_wellschur_recover(rp.size - 1, rp, ci, v, na, nv, nw, _arr(b, np.float64), _arr(xc, np.float64), x)
        return x

    def refine_float(self, A, b, tol=1e-8, max_outer=6, inner_it=120):
        x = np.zeros(A.n * A.nb)
        its, rr = C.c_int(0), C.c_double(0)
        conv = self.L.ref_refine_float(A.n, A.nb, A.rowPtr, A.col, A.val, _arr(b, np.float64), x, tol, max_outer, inner_it,
                                       C.byref(its), C.byref(rr))
        return x, bool(conv), its.value, rr.value

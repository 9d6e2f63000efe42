"""Python mirror of the reference solver interface over the rsg C ABI (all compute on the GPU).

Reference interfaces mirrored (same names, argument meaning and failure behaviour):

* ``LinResult`` -- ``ressim::LinResult {converged, iterations, relResidual}`` (engine/include/ressim/linsolve.h:97)
* ``DeviceSolver`` -- one rsg handle: ``set_matrix`` / ``set_batch`` (the BSR handed to the solver),
  ``setup`` (``BILU0::factor`` / ``BlockCPR::setup``), ``solve`` (``bicgstab`` / ``gmres`` with the set-up
  preconditioner, x0 = 0), ``spmv`` (``BSR::spmv``), ``precond_apply`` (``Preconditioner::apply``)
* ``GpuBlockSolver`` -- ``ressim::GpuBlockSolver`` (engine/include/ressim/bsr.h:143-151): ``name()``,
  ``solve(A, b, tol, maxIt) -> (ok, x, iterations)``, ``deviceSeconds()``; returns ``ok = False`` on device
  failure or non-finite output so that the caller falls back, exactly as the engine expects
* ``WellSchur`` -- ``ressim::WellSchur`` build / reduceRhs / recover (engine/include/ressim/bsr.h:191-222)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .bsr import BSR, ScalarCSR


@dataclass
class LinResult:
    converged: bool = False
    iterations: int = 0
    relResidual: float = 0.0
    trueRelResidual: float = -1.0
    status: int = 0


class DeviceSolver:
    """One solver handle (one CUDA stream, resident device memory)."""

    def __init__(self, precond: str = "bilu0", krylov: str = "bicgstab", precision: str = "fp64", restart: int = 40,
                 check_every: int = 4, use_graphs: bool = True, device: int = 0, mem_budget: int = 0,
                 gmres_fallback: bool = False, sweep: str = "auto", fma: bool = True,
                 sweep_inflight: int = 0, autotune: bool = True, vcycle_form: int = 0, cpr2_threads: int = 0):
        self.L = _lib.load()
        o = _lib.Options()
        self.L.rsg_default_options(C.byref(o))
        o.precond = _lib.PREC[precond]
        o.krylov = _lib.KRYLOV[krylov]
        o.precision = _lib.PRECISION[precision]
        o.restart = restart
        o.check_every = check_every
        o.use_graphs = 1 if use_graphs else 0
        o.device = device
        o.mem_budget = mem_budget
        o.gmres_fallback = 1 if gmres_fallback else 0
        o.fma = 1 if fma else 0
        o.sweep = _lib.SWEEP[sweep]
        o.sweep_inflight = sweep_inflight
        o.autotune = 1 if autotune else 0
        o.vcycle_form = vcycle_form
        o.cpr2_threads = cpr2_threads
        self.opts = o
        h = C.c_void_p()
        _lib.check(self.L.rsg_create(C.byref(h), C.byref(o)))
        self.h = h
        self.n = 0
        self.nsys = 0
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            self.L.rsg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- matrix
    def set_matrix(self, A: BSR):
        _lib.check(self.L.rsg_set_matrix(self.h, A.n, A.nb, _lib.ptr(A.rowPtr), _lib.ptr(A.col), _lib.ptr(A.val)))
        self.n = A.n * A.nb
        self.nb = A.nb
        self.nsys = 1
        self.sizes = [A.n * A.nb]

    def set_batch(self, mats):
        k = len(mats)
        ns = np.array([m.n for m in mats], dtype=np.int32)
        rps = (C.c_void_p * k)(*[m.rowPtr.ctypes.data for m in mats])
        cis = (C.c_void_p * k)(*[m.col.ctypes.data for m in mats])
        vls = (C.c_void_p * k)(*[m.val.ctypes.data for m in mats])
        self._keep = (ns, rps, cis, vls)
        _lib.check(self.L.rsg_set_batch(self.h, k, mats[0].nb, _lib.ptr(ns), rps, cis, vls))
        self.n = int(sum(m.n * m.nb for m in mats))
        self.nsys = k
        self.sizes = [m.n * m.nb for m in mats]

    def set_jacobian(self, J, na: int, nv: int, nw: int):
        """The Newton Jacobian with its well rows (ScalarCSR, na*nv cell rows then nw well rows): the well Schur
        complement on the device into this solver's block system (rsg_set_jacobian)."""
        _lib.check(self.L.rsg_set_jacobian(self.h, J.n, _lib.ptr(J.rowPtr), _lib.ptr(J.col), _lib.ptr(J.val), na, nv, nw))
        self.n = na * nv
        self.nsys = 1
        self.sizes = [na * nv]
        self.full = J.n

    def set_jacobian_batch(self, jacs):
        """A batch of (ScalarCSR, na, nw) Jacobians with well rows (nv = 3), reduced on the device."""
        k = len(jacs)
        nrows = np.array([J.n for J, _, _ in jacs], dtype=np.int32)
        na = np.array([a for _, a, _ in jacs], dtype=np.int32)
        nw = np.array([w for _, _, w in jacs], dtype=np.int32)
        rps = (C.c_void_p * k)(*[J.rowPtr.ctypes.data for J, _, _ in jacs])
        cis = (C.c_void_p * k)(*[J.col.ctypes.data for J, _, _ in jacs])
        vls = (C.c_void_p * k)(*[J.val.ctypes.data for J, _, _ in jacs])
        self._keepj = (nrows, na, nw, rps, cis, vls)
        _lib.check(self.L.rsg_set_jacobian_batch(self.h, k, 3, _lib.ptr(nrows), _lib.ptr(na), _lib.ptr(nw), rps, cis, vls))
        self.n = int(na.sum()) * 3
        self.nsys = k
        self.sizes = [int(a) * 3 for a in na]
        self.full = int(nrows.sum())

    def solve_jacobian(self, b_full, tol: float = 1e-6, maxit: int = 120):
        """Full right-hand side (cells then wells, per system) in, full solution (BHPs recovered) out."""
        b = np.ascontiguousarray(b_full, dtype=np.float64)
        x = np.zeros(self.full)
        its, rr = C.c_int(0), C.c_double(0)
        rc = _lib.check(self.L.rsg_solve_jacobian(self.h, _lib.ptr(b), _lib.ptr(x), tol, maxit, C.byref(its), C.byref(rr)))
        st = self.stats()
        return x, LinResult(rc == 0, its.value, rr.value, st.true_rel_residual, rc)

    def matrix(self):
        """The current block system (caller's order) as a BSR."""
        n, nnzb = C.c_int(0), C.c_longlong(0)
        _lib.check(self.L.rsg_matrix_size(self.h, C.byref(n), C.byref(nnzb)))
        rp = np.zeros(n.value + 1, dtype=np.int32)
        ci = np.zeros(nnzb.value, dtype=np.int32)
        v = np.zeros(nnzb.value * 9)
        _lib.check(self.L.rsg_get_matrix(self.h, _lib.ptr(rp), _lib.ptr(ci), _lib.ptr(v)))
        return BSR(n.value, 3, rp, ci, v)

    def setup(self, acc=None):
        a = None if acc is None else np.ascontiguousarray(acc, dtype=np.float64)
        _lib.check(self.L.rsg_setup(self.h, _lib.ptr(a)))

    # ---- solves
    def solve(self, b, tol: float = 1e-6, maxit: int = 120):
        b = np.ascontiguousarray(b, dtype=np.float64)
        if self.n and b.size != self.n:
            raise ValueError(f"b has {b.size} entries, the system has {self.n}")
        x = np.zeros(max(self.n, b.size))
        its, rr = C.c_int(0), C.c_double(0)
        rc = _lib.check(self.L.rsg_solve(self.h, _lib.ptr(b), _lib.ptr(x), tol, maxit, C.byref(its), C.byref(rr)))
        st = self.stats()
        return x, LinResult(rc == 0, its.value, rr.value, st.true_rel_residual, rc)

    def solve_refined(self, b, tol: float = 1e-8, max_outer: int = 6, inner_it: int = 120):
        """FP64 defect correction around this solver (the engine's refineWithDevice, engine/src/bsr.cpp:1373-1396):
        inner solves to clamp(10 tol, 1e-4, 1e-2), x += d, r = b - A x in FP64, at most ``max_outer`` passes."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        if self.n and b.size != self.n:
            raise ValueError(f"b has {b.size} entries, the system has {self.n}")
        x = np.zeros(max(self.n, b.size))
        its, rr = C.c_int(0), C.c_double(0)
        rc = _lib.check(self.L.rsg_solve_refined(self.h, _lib.ptr(b), _lib.ptr(x), tol, max_outer, inner_it, C.byref(its), C.byref(rr)))
        st = self.stats()
        return x, LinResult(rc == 0, its.value, rr.value, st.true_rel_residual, rc)

    def solve_device(self, d_b: int, d_x: int, tol: float = 1e-6, maxit: int = 120):
        """Device pointers (e.g. torch ``data_ptr()``) of n float64 entries."""
        its, rr = C.c_int(0), C.c_double(0)
        rc = _lib.check(self.L.rsg_solve_device(self.h, C.c_void_p(d_b), C.c_void_p(d_x), tol, maxit, C.byref(its), C.byref(rr)))
        st = self.stats()
        return LinResult(rc == 0, its.value, rr.value, st.true_rel_residual, rc)

    def tuning(self) -> str:
        """Launch shapes in use after set-up and how they were chosen (rsg_tuning)."""
        buf = C.create_string_buffer(1024)
        _lib.check(self.L.rsg_tuning(self.h, buf, 1024))
        return buf.value.decode()

    def batch_results(self):
        its = np.zeros(self.nsys, dtype=np.int32)
        rr = np.zeros(self.nsys)
        tr = np.zeros(self.nsys)
        _lib.check(self.L.rsg_batch_results(self.h, _lib.ptr(its), _lib.ptr(rr), _lib.ptr(tr)))
        return its, rr, tr

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        _lib.check(self.L.rsg_spmv(self.h, _lib.ptr(x), _lib.ptr(y)))
        return y

    def spmv_device(self, d_x: int, d_y: int):
        _lib.check(self.L.rsg_spmv_device(self.h, C.c_void_p(d_x), C.c_void_p(d_y)))

    def precond_apply(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.n)
        _lib.check(self.L.rsg_precond_apply(self.h, _lib.ptr(r), _lib.ptr(z)))
        return z

    def precond_apply_device(self, d_r: int, d_z: int):
        _lib.check(self.L.rsg_precond_apply_device(self.h, C.c_void_p(d_r), C.c_void_p(d_z)))

    def factors(self, nnzb: int):
        """BILU0 factors in the caller's block order (nnzb blocks of nb x nb)."""
        lu = np.zeros(nnzb * getattr(self, "nb", 3) ** 2)
        _lib.check(self.L.rsg_get_factors(self.h, _lib.ptr(lu)))
        return lu

    def stats(self) -> _lib.Stats:
        st = _lib.Stats()
        _lib.check(self.L.rsg_get_stats(self.h, C.byref(st)))
        return st

    def amg_level_sizes(self, maxlev: int = 16):
        """CPR hierarchy after setup(), summed over the batch: (rows per level, entries per level, dense coarse
        entries), or None without a CPR hierarchy."""
        rows = np.zeros(maxlev, dtype=np.int64)
        nnz = np.zeros(maxlev, dtype=np.int64)
        dense = C.c_longlong(0)
        nl = self.L.rsg_amg_level_sizes(self.h, maxlev, _lib.ptr(rows), _lib.ptr(nnz), C.byref(dense))
        if nl < 0:
            return None
        nl = min(nl, maxlev)
        return rows[:nl], nnz[:nl], int(dense.value)

    @property
    def stream(self) -> int:
        return int(self.L.rsg_stream(self.h) or 0)


class Server:
    """Serving form (``rsg_server_*``): continuous batching of independent systems over ``slots`` workers under a
    device-memory budget. ``submit`` copies a system and returns its id (``copy=False``: the server reads the
    arrays in place, and this object keeps them referenced until the result is polled; the caller must not change
    them meanwhile); ``poll`` returns ``None`` while it is queued or running, else ``(x, result)`` with the
    per-request latency split (queue / run / total ms). As the engine does, a BiCGSTAB solve that does not converge is
    retried with GMRES (``gmres_fallback``, on by default)."""

    def __init__(self, slots: int = 4, mem_budget: int = 0, precond: str = "cpr", krylov: str = "bicgstab",
                 precision: str = "mixed_f32", restart: int = 40, check_every: int = 4, use_graphs: bool = True, device: int = 0,
                 gmres_fallback: bool = True):
        self.L = _lib.load()
        o = _lib.Options()
        self.L.rsg_default_options(C.byref(o))
        o.precond = _lib.PREC[precond]
        o.krylov = _lib.KRYLOV[krylov]
        o.precision = _lib.PRECISION[precision]
        o.restart = restart
        o.check_every = check_every
        o.use_graphs = 1 if use_graphs else 0
        o.device = device
        o.gmres_fallback = 1 if gmres_fallback else 0
        self.opts = o
        self.s = C.c_void_p()
        _lib.check(self.L.rsg_server_create(C.byref(self.s), C.byref(o), slots, mem_budget))
        self.sizes = {}
        self.lent = {}

    def request_bytes(self, A: BSR) -> int:
        """The admission figure of a system under this server's options."""
        return int(self.L.rsg_request_bytes(C.byref(self.opts), A.n, A.nnzb))

    def submit(self, A: BSR, b, tol: float = 1e-6, maxit: int = 200, copy: bool = True) -> int:
        b = np.ascontiguousarray(b, dtype=np.float64)
        fn = self.L.rsg_submit if copy else self.L.rsg_submit_view
        rid = int(fn(self.s, A.n, A.nb, _lib.ptr(A.rowPtr), _lib.ptr(A.col), _lib.ptr(A.val), _lib.ptr(b), tol, maxit))
        if rid < 0:
            raise _lib.RsgError(rid, _lib.last_error())
        self.sizes[rid] = A.n * A.nb
        if not copy:
            self.lent[rid] = (A.rowPtr, A.col, A.val, b)
        return rid

    def poll(self, rid: int, wait: bool = True):
        x = np.zeros(self.sizes[rid])
        r = _lib.Result()
        rc = self.L.rsg_poll(self.s, rid, 1 if wait else 0, _lib.ptr(x), C.byref(r))
        if rc < 0:
            raise _lib.RsgError(rc, _lib.last_error())
        if rc == 0:
            return None
        del self.sizes[rid]
        self.lent.pop(rid, None)
        return x, {k: getattr(r, k) for k, _ in _lib.Result._fields_}

    def hold(self, on: bool = True):
        """Pause (or resume) admission: requests submitted while held are admitted together (rsg_server_hold)."""
        _lib.check(self.L.rsg_server_hold(self.s, 1 if on else 0))

    def load(self):
        q, rn, by = C.c_int(0), C.c_int(0), C.c_size_t(0)
        _lib.check(self.L.rsg_server_load(self.s, C.byref(q), C.byref(rn), C.byref(by)))
        return q.value, rn.value, by.value

    def close(self):
        if getattr(self, "s", None):
            self.L.rsg_server_destroy(self.s)
            self.s = None
            self.lent = {}                       # released only after the server no longer reads them

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuBlockSolver:
    """``ressim::GpuBlockSolver`` over the device solver: every call uploads A (pattern reuse keeps the plan),
    factors and solves; ``False`` on any device failure or non-finite output (the engine then falls back)."""

    def __init__(self, **kw):
        self.dev = DeviceSolver(**kw)
        self._seconds = 0.0

    def name(self) -> str:
        return "GB300 (sm_103a) " + _lib.load().rsg_version().decode()

    def solve(self, A: BSR, b, tol: float, maxIt: int):
        try:
            self.dev.set_matrix(A)
            self.dev.setup()
            x, res = self.dev.solve(b, tol, maxIt)
        except _lib.RsgError:
            return False, None, 0
        st = self.dev.stats()
        self._seconds += 1e-3 * (st.setup_ms + st.solve_ms)
        if not np.all(np.isfinite(x)):
            return False, None, res.iterations
        return True, x, res.iterations

    def deviceSeconds(self) -> float:
        return self._seconds


class WellSchur:
    """``ressim::WellSchur`` on the scalar Jacobian with well rows (host-side reduction, as the engine does)."""

    def __init__(self, J: ScalarCSR, na: int, nv: int, nw: int):
        self.J, self.na, self.nv, self.nw = J, na, nv, nw

    def reduce(self, b):
        L = _lib.load()
        J = self.J
        b = np.ascontiguousarray(b, dtype=np.float64)
        nnzb = C.c_int(0)
        _lib.check(L.rsg_wellschur_reduce(J.n, _lib.ptr(J.rowPtr), _lib.ptr(J.col), _lib.ptr(J.val), self.na, self.nv, self.nw,
                                          _lib.ptr(b), C.byref(nnzb), None, None, None, None))
        rp = np.zeros(self.na + 1, dtype=np.int32)
        ci = np.zeros(nnzb.value, dtype=np.int32)
        v = np.zeros(nnzb.value * self.nv * self.nv)
        bc = np.zeros(self.na * self.nv)
        _lib.check(L.rsg_wellschur_reduce(J.n, _lib.ptr(J.rowPtr), _lib.ptr(J.col), _lib.ptr(J.val), self.na, self.nv, self.nw,
                                          _lib.ptr(b), C.byref(nnzb), _lib.ptr(rp), _lib.ptr(ci), _lib.ptr(v), _lib.ptr(bc)))
        return BSR(self.na, self.nv, rp, ci, v), bc

    def recover(self, b, xc):
        L = _lib.load()
        J = self.J
        b = np.ascontiguousarray(b, dtype=np.float64)
        xc = np.ascontiguousarray(xc, dtype=np.float64)
        x = np.zeros(J.n)
        _lib.check(L.rsg_wellschur_recover(J.n, _lib.ptr(J.rowPtr), _lib.ptr(J.col), _lib.ptr(J.val), self.na, self.nv, self.nw,
                                           _lib.ptr(b), _lib.ptr(xc), _lib.ptr(x)))
        return x

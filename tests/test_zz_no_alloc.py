"""The allocation-free fused SpMV + inner product (rsg_spmv_dot_noalloc), for callers that cannot allocate device
memory during a solve, checked through the C ABI against the existing entry point (rsg_spmv through a solver
handle) on two calls in a row: the second call reuses the library's fixed scratch array and must give the same
result. Collected last (file name) so that a run stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_spmv_dot_noalloc_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    from ressim_gb300 import _lib
    from ressim_gb300.solver import DeviceSolver
    L = _lib.load()
    A, z = load_golden("waterflood_sys1.npz")
    x, w = z["x_seed"], z["b"]
    with DeviceSolver(fma=False) as d:        # the existing entry point with the same (reference) rounding
        d.set_matrix(A)
        y_ref = d.spmv(x)
    dot_ref = float(np.dot(w, y_ref))
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(A.rowPtr).to(dev)
    ci = torch.from_numpy(A.col).to(dev)
    va = torch.from_numpy(A.val).to(dev)
    xd = torch.from_numpy(x).to(dev)
    wd = torch.from_numpy(w).to(dev)
    yd = torch.empty(A.n * 3, dtype=torch.float64, device=dev)
    dot = torch.empty(1, dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        yd.fill_(np.nan)
        dot.fill_(np.nan)
        rc = L.rsg_spmv_dot_noalloc(A.n, 3, C.c_void_p(rp.data_ptr()), C.c_void_p(ci.data_ptr()), C.c_void_p(va.data_ptr()),
                                    C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), C.c_void_p(wd.data_ptr()),
                                    C.c_void_p(dot.data_ptr()), stream)
        torch.cuda.synchronize(dev)
        assert rc == _lib.RSG_OK, _lib.last_error()
        # same arithmetic as the existing SpMV: bit for bit; the inner product within 1e-12 relative (tree order)
        assert np.array_equal(yd.cpu().numpy(), y_ref), f"call {call}"
        assert abs(float(dot.item()) - dot_ref) <= 1e-12 * abs(dot_ref), f"call {call}"


def test_spmv_dot_noalloc_rejects_sizes_beyond_its_maximum():
    from ressim_gb300 import _lib
    L = _lib.load()
    rc = L.rsg_spmv_dot_noalloc(16384 * 256 + 1, 3, None, None, None, None, None, None, None, None)
    assert rc == _lib.RSG_EINVAL
    assert "exceeds the maximum" in _lib.last_error()


def test_spmv_dot_noalloc_many_tiles():
    """2,500 tiles of 256 block rows (400 copies of a captured waterflood system on the block diagonal, 640,000 block
    rows): the last-tile reduction over thousands of partials, against the existing entry point, twice in a row."""
    torch = pytest.importorskip("torch")
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import BSR
    from ressim_gb300.solver import DeviceSolver
    L = _lib.load()
    A1, z = load_golden("waterflood_sys1.npz")
    copies = 400
    nnzb = A1.nnzb
    rp = np.concatenate([A1.rowPtr[:-1] + k * nnzb for k in range(copies)] + [np.array([copies * nnzb])]).astype(np.int32)
    ci = np.concatenate([A1.col + k * A1.n for k in range(copies)]).astype(np.int32)
    A = BSR(A1.n * copies, 3, rp, ci, np.tile(A1.val, copies))
    rng = np.random.default_rng(7)
    x = rng.standard_normal(A.n * 3)
    w = rng.standard_normal(A.n * 3)
    with DeviceSolver(fma=False) as d:
        d.set_matrix(A)
        y_ref = d.spmv(x)
    dot_ref = float(np.dot(w, y_ref))
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(v).to(dev) for k, v in dict(rp=A.rowPtr, ci=A.col, va=A.val, x=x, w=w).items()}
    yd = torch.empty(A.n * 3, dtype=torch.float64, device=dev)
    dot = torch.empty(1, dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        yd.fill_(np.nan)
        dot.fill_(np.nan)
        rc = L.rsg_spmv_dot_noalloc(A.n, 3, C.c_void_p(t["rp"].data_ptr()), C.c_void_p(t["ci"].data_ptr()), C.c_void_p(t["va"].data_ptr()),
                                    C.c_void_p(t["x"].data_ptr()), C.c_void_p(yd.data_ptr()), C.c_void_p(t["w"].data_ptr()),
                                    C.c_void_p(dot.data_ptr()), stream)
        torch.cuda.synchronize(dev)
        assert rc == _lib.RSG_OK, _lib.last_error()
        assert np.array_equal(yd.cpu().numpy(), y_ref), f"call {call}"
        assert abs(float(dot.item()) - dot_ref) <= 1e-12 * np.dot(np.abs(w), np.abs(y_ref)), f"call {call}"


def test_spmv_dot_noalloc_rejects_aliased_output():
    torch = pytest.importorskip("torch")
    from ressim_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda:0")
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    rc = L.rsg_spmv_dot_noalloc(1, 3, p, p, p, p, p, C.c_void_p(buf.data_ptr() + 8), p, None)
    assert rc == _lib.RSG_EINVAL and "alias" in _lib.last_error()

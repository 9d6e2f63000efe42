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

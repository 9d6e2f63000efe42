"""The well Schur complement on the device (rsg_set_jacobian*, rsg_solve_jacobian*) against the reference.

The engine reduces its Jacobian with well (BHP) rows to the block system of the cells before the block solver and
recovers the BHPs after it (WellSchur::build / reduceRhs / recover, engine/src/bsr.cpp:733-990). The device version
must give the reference's S bit for bit -- pattern and values, the fill of every well clique included -- its reduced
right-hand side bit for bit (checked through the solve: the same S and right-hand side give the same solve bit for
bit), and the reference's recovered BHPs bit for bit from the same cell solution. The golden systems hold the
reference's own S (synth_small: S_*; the engine dump: the reduced system itself); the oracle's restatement, pinned
bit for bit to the reference, checks the inputs made here (scaled values, a zeroed coupling, a batch).
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def dev(**kw):
    from ressim_gb300.solver import DeviceSolver
    return DeviceSolver(**kw)


def jac_of(z):
    from ressim_gb300.bsr import ScalarCSR
    return ScalarCSR(z["J_rowPtr"], z["J_col"], z["J_val"]), int(z["na"]), int(z["nv"]), int(z["nw"])


def reference_s(name, z, A):
    if "S_val" in z.files:
        return z["S_rowPtr"], z["S_col"], z["S_val"], z["S_bc"]
    return A.rowPtr, A.col, A.val, z["b"]            # the engine dump: the golden system is the reduced one


@pytest.mark.parametrize("name", ["waterflood_dump.npz", "synth_small.npz"])
def test_device_schur_complement_bitwise(name, oracle):
    A, z = load_golden(name)
    J, na, nv, nw = jac_of(z)
    rp, ci, sv, bc = reference_s(name, z, A)
    with dev(precond="bilu0") as d:
        d.set_jacobian(J, na, nv, nw)
        S = d.matrix()
        assert np.array_equal(S.rowPtr, rp) and np.array_equal(S.col, ci)
        assert np.array_equal(S.val, sv)
        d.setup()
        x_full, res = d.solve_jacobian(z["J_rhs"], tol=1e-10, maxit=1000)
    assert res.converged
    # the reduced right-hand side: a solve of the same S and the reference's b_c gives the same cell solution bit for bit
    from ressim_gb300.bsr import BSR
    with dev(precond="bilu0") as d:
        d.set_matrix(BSR(na, nv, rp, ci, sv))
        d.setup()
        xc, _ = d.solve(bc, tol=1e-10, maxit=1000)
    assert np.array_equal(x_full[:na * nv], xc)
    # the BHPs: the reference's recovery from the same cell solution
    x_ref = oracle.wellschur_recover((J.rowPtr, J.col, J.val), na, nv, nw, z["J_rhs"], xc)
    assert np.array_equal(x_full, x_ref)
    if "x_full" in z.files:                      # the reference's full solution (from its tight BILU0-BiCGSTAB solve)
        assert np.linalg.norm(x_full - z["x_full"]) <= 1e-8 * np.linalg.norm(z["x_full"])


def test_values_refresh_and_coupling_pattern(oracle):
    """A values-only refresh keeps the plan; a cell-to-well coupling that becomes zero drops its fill from S as the
    engine does (its pattern depends on the nonzero couplings); both bit for bit the reference's S."""
    from ressim_gb300.bsr import ScalarCSR
    A, z = load_golden("synth_small.npz")
    J, na, nv, nw = jac_of(z)
    nc = na * nv
    scaled = ScalarCSR(J.rowPtr, J.col, J.val * 1.7)
    rows = np.repeat(np.arange(J.n), np.diff(J.rowPtr))
    cpl = np.nonzero((rows < nc) & (J.col >= nc))[0]
    cut = J.val.copy()
    cut[cpl[: max(1, cpl.size // 4)]] = 0.0                 # some perforations shut (their couplings exactly zero)
    zeroed = ScalarCSR(J.rowPtr, J.col, cut)
    with dev(precond="bilu0") as d:
        for Jk in (J, scaled, zeroed, J):
            d.set_jacobian(Jk, na, nv, nw)
            S = d.matrix()
            (rp, ci, sv), _ = oracle.wellschur((Jk.rowPtr, Jk.col, Jk.val), na, nv, nw, z["J_rhs"])
            assert np.array_equal(S.rowPtr, rp) and np.array_equal(S.col, ci) and np.array_equal(S.val, sv)
    (rp0, ci0, _), _ = oracle.wellschur((J.rowPtr, J.col, J.val), na, nv, nw, z["J_rhs"])
    (rp1, ci1, _), _ = oracle.wellschur((zeroed.rowPtr, zeroed.col, zeroed.val), na, nv, nw, z["J_rhs"])
    assert ci1.size < ci0.size                               # the zeroed couplings removed fill


def test_unusable_well_row_is_rejected():
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import ScalarCSR
    A, z = load_golden("synth_small.npz")
    J, na, nv, nw = jac_of(z)
    v = J.val.copy()
    r = na * nv                                               # the first well row: its BHP derivative set to zero
    for p in range(J.rowPtr[r], J.rowPtr[r + 1]):
        if J.col[p] == r:
            v[p] = 0.0
    with dev(precond="bilu0") as d:
        with pytest.raises(_lib.RsgError) as e:
            d.set_jacobian(ScalarCSR(J.rowPtr, J.col, v), na, nv, nw)
    assert e.value.code == _lib.RSG_EINVAL and "BHP" in str(e.value)


def test_batch_of_jacobians(oracle):
    """Three Jacobians with wells in one batch: every system's S and solution are the ones it has alone."""
    from ressim_gb300 import synth
    sys_ = [synth.make_system(10, 8, 4, sigma=1.0 + 0.3 * k, seed=20 + k, wells="corners+center", with_full=True) for k in range(3)]
    singles = []
    for s in sys_:
        with dev(precond="cpr") as d:
            d.set_jacobian(s.full, s.na, s.nv, s.nw)
            d.setup()
            singles.append((d.matrix(), d.solve_jacobian(s.full_b, tol=1e-8, maxit=300)[0]))
    with dev(precond="cpr") as d:
        d.set_jacobian_batch([(s.full, s.na, s.nw) for s in sys_])
        d.setup()
        S = d.matrix()
        xb, res = d.solve_jacobian(np.concatenate([s.full_b for s in sys_]), tol=1e-8, maxit=300)
    assert res.converged
    off_b, off_r, off_x = 0, 0, 0
    for (S1, x1), s in zip(singles, sys_):
        nb = S1.nnzb
        assert np.array_equal(S.val[off_b * 9:(off_b + nb) * 9], S1.val)
        assert np.array_equal(S.col[off_b:off_b + nb] - off_r, S1.col)
        assert np.array_equal(xb[off_x:off_x + x1.size], x1)
        (rp, ci, sv), _ = oracle.wellschur((s.full.rowPtr, s.full.col, s.full.val), s.na, s.nv, s.nw, s.full_b)
        assert np.array_equal(S1.val, sv) and np.array_equal(S1.col, ci)
        off_b += nb
        off_r += s.na
        off_x += x1.size


def test_device_values_entry():
    """rsg_set_jacobian_device: the Jacobian values already in device memory (device assembly), the same S."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    from ressim_gb300 import _lib
    A, z = load_golden("waterflood_dump.npz")
    J, na, nv, nw = jac_of(z)
    dv = torch.from_numpy(J.val).to("cuda:0")
    with dev(precond="bilu0") as d:
        _lib.check(d.L.rsg_set_jacobian_device(d.h, J.n, _lib.ptr(J.rowPtr), _lib.ptr(J.col), C.c_void_p(dv.data_ptr()), na, nv, nw))
        d.n, d.nsys, d.full = na * nv, 1, J.n
        S = d.matrix()
        assert np.array_equal(S.val, A.val) and np.array_equal(S.col, A.col)
        d.setup()
        x_full, res = d.solve_jacobian(z["J_rhs"], tol=1e-10, maxit=1000)
    assert res.converged and np.linalg.norm(x_full - z["x_full"]) <= 1e-8 * np.linalg.norm(z["x_full"])

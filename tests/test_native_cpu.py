"""The C-ABI library builds, loads and exports every symbol include/*.h declares; its host-only entry points
(well Schur complement) are checked against the reference's golden vectors. No GPU needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_SYSTEMS, ROOT, load_golden


def declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms |= set(re.findall(r"\b(rsg_[a-z0-9_]+)\s*\(", txt))
    return syms


def test_library_builds_and_exports_every_declared_symbol():
    from ressim_gb300 import _build, _lib
    _build.build()
    L = C.CDLL(_build.LIB)
    syms = declared_symbols()
    assert len(syms) >= 19
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= syms


def test_create_without_gpu_fails_cleanly():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from ressim_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    rc = L.rsg_create(C.byref(h), None)
    assert rc == _lib.RSG_ECUDA
    assert "CUDA" in _lib.last_error() or "device" in _lib.last_error()
    # options are checked before the device: every sweep form (0-3) passes to the device check, 4 does not
    o = _lib.Options()
    L.rsg_default_options(C.byref(o))
    for sweep, want in ((0, _lib.RSG_ECUDA), (3, _lib.RSG_ECUDA), (4, _lib.RSG_EINVAL)):
        o.sweep = sweep
        assert L.rsg_create(C.byref(h), C.byref(o)) == want
    # entry points without a handle fail cleanly
    rows = np.zeros(4, dtype=np.int64)
    assert L.rsg_amg_level_sizes(None, 4, _lib.ptr(rows), _lib.ptr(rows), None) == _lib.RSG_EINVAL
    assert L.rsg_batch_status(None, None) == _lib.RSG_EINVAL


def test_server_without_gpu_fails_cleanly_and_footprint_is_monotone():
    from conftest import gpu_available
    from ressim_gb300 import _lib
    L = _lib.load()
    o = _lib.Options()
    L.rsg_default_options(C.byref(o))
    small, big = L.rsg_request_bytes(C.byref(o), 1000, 7000), L.rsg_request_bytes(C.byref(o), 100000, 700000)
    assert 0 < small < big
    o.krylov = _lib.KRYLOV["gmres"]
    assert L.rsg_request_bytes(C.byref(o), 100000, 700000) > big          # the GMRES basis is counted
    if gpu_available():
        pytest.skip("a GPU is present")
    s = C.c_void_p()
    assert L.rsg_server_create(C.byref(s), None, 2, 0) == _lib.RSG_ECUDA
    assert L.rsg_server_create(C.byref(s), None, 0, 0) == _lib.RSG_EINVAL
    assert not s.value


@pytest.mark.parametrize("name", ["waterflood_dump.npz", "synth_small.npz"])
def test_wellschur_host_matches_reference(name):
    from ressim_gb300.bsr import ScalarCSR
    from ressim_gb300.solver import WellSchur
    A, z = load_golden(name)
    J = ScalarCSR(z["J_rowPtr"], z["J_col"], z["J_val"])
    W = WellSchur(J, int(z["na"]), int(z["nv"]), int(z["nw"]))
    S, bc = W.reduce(z["J_rhs"])
    if "S_val" in z.files:
        assert np.array_equal(S.rowPtr, z["S_rowPtr"]) and np.array_equal(S.col, z["S_col"]) and np.array_equal(S.val, z["S_val"])
        assert np.array_equal(bc, z["S_bc"])
    else:
        assert np.array_equal(S.rowPtr, A.rowPtr) and np.array_equal(S.col, A.col) and np.array_equal(S.val, A.val)
        assert np.array_equal(bc, z["b"])
    if "x_full" in z.files:
        assert np.array_equal(W.recover(z["J_rhs"], z["x_bicg_bilu0_tight"]), z["x_full"])


def test_wellschur_rejects_well_well_coupling():
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import ScalarCSR
    from ressim_gb300.solver import WellSchur
    # 1 cell x 3 unknowns + 2 wells coupled to each other
    rp = np.array([0, 2, 4, 6, 9, 12], dtype=np.int32)
    ci = np.array([0, 3, 1, 3, 2, 3, 0, 3, 4, 0, 3, 4], dtype=np.int32)
    v = np.array([2.0, -1, 2, -1, 2, -1, -1, 3, 0.5, -1, 0.5, 3])
    W = WellSchur(ScalarCSR(rp, ci, v), 1, 3, 2)
    with pytest.raises(_lib.RsgError) as e:
        W.reduce(np.ones(5))
    assert "well-well" in str(e.value)


def test_synth_manufactured_rhs():
    from ressim_gb300 import synth
    s = synth.make_system(10, 8, 3, sigma=1.0, seed=2, wells="corners+center", with_full=True)
    assert s.A.structurally_symmetric()
    assert np.allclose(synth.bsr_matvec_host(s.A, s.x_true), s.b)
    # the reduced system equals the Schur complement of the full Jacobian
    from ressim_gb300.solver import WellSchur
    S, bc = WellSchur(s.full, s.na, s.nv, s.nw).reduce(s.full_b)
    assert np.array_equal(S.rowPtr, s.A.rowPtr) and np.array_equal(S.col, s.A.col)
    assert np.allclose(S.val, s.A.val, rtol=1e-12, atol=1e-12 * np.abs(s.A.val).max())


def test_reference_tools_build_against_the_adapters():
    """The reference's own tools/lsbench.cpp compiles and links, unmodified, with the supplied ressim/blocksolve.h,
    librsg.so and the reference solver objects, and the GpuBlockSolver adapter compiles against the engine's own
    headers (where the reference engine's sources are staged in oracle/_ref/src)."""
    import shutil
    import subprocess
    src = os.path.join(ROOT, "oracle", "_ref", "src")
    if not os.path.isdir(os.path.join(src, "engine", "include")) or not shutil.which("g++"):
        pytest.skip("reference engine sources not staged on this host")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(src, "engine", "include")]
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", *inc, "-x", "c++", os.path.join(ROOT, "include", "rsg_ressim_adapter.hpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if not os.path.exists(os.path.join(ROOT, "ressim_gb300", "librsg.so")):
        pytest.skip("librsg.so not built")
    r = subprocess.run(["make", "-f", "oracle/Makefile.ref", "-j4", "oracle/_ref/lsbench"], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]


@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_host_amg_plan_matches_oracle(name, oracle):
    """The host AMG plan (aggregation, then Galerkin products summed in the reference's order) is the oracle's
    hierarchy: level sizes, the level-0 aggregates and every coarse operator bit for bit. Host code only
    (rsg_debug_amg_plan builds the plan of one system from its pressure matrix; no GPU)."""
    from ressim_gb300 import _build
    L = C.CDLL(_build.LIB)
    L.rsg_debug_amg_plan.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int] + [C.c_void_p] * 3 + [C.c_int] + [C.c_void_p] * 4
    A, _ = load_golden(name)
    w, info, levels = oracle.cpr_info(A)
    rp0, ci0, v0, agg0 = levels[0]
    assert np.array_equal(rp0, A.rowPtr) and np.array_equal(ci0, A.col)     # the pressure matrix has S's pattern
    ap = np.ascontiguousarray(v0, dtype=np.float64)
    nlev = C.c_int(0)
    rows = np.zeros(16, np.int32)
    nnz = np.zeros(16, np.int32)
    agg = np.zeros(A.n, np.int32)
    m = np.zeros(A.n + 1, np.int32)
    assert L.rsg_debug_amg_plan(A.n, A.rowPtr.ctypes.data, A.col.ctypes.data, ap.ctypes.data, 0, C.byref(nlev), rows.ctypes.data,
                                nnz.ctypes.data, 16, m.ctypes.data, np.zeros(len(ci0), np.int32).ctypes.data,
                                np.zeros(len(ci0)).ctypes.data, agg.ctypes.data) == 0
    assert nlev.value == len(info)
    assert [int(r) for r in rows[:nlev.value]] == [r for r, _ in info]
    assert [int(q) for q in nnz[:nlev.value]] == [q for _, q in info]
    if len(info) > 1:
        assert np.array_equal(agg, agg0)
    for lv in range(1, len(info)):                    # every coarse operator, pattern and values
        rpl, cil, vl, _ = levels[lv]
        rp = np.zeros(len(rpl), np.int32)
        ci = np.zeros(len(cil), np.int32)
        v = np.zeros(len(vl))
        assert L.rsg_debug_amg_plan(A.n, A.rowPtr.ctypes.data, A.col.ctypes.data, ap.ctypes.data, lv, C.byref(nlev), rows.ctypes.data,
                                    nnz.ctypes.data, 16, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, None) == 0
        assert np.array_equal(rp, rpl) and np.array_equal(ci, cil)
        assert np.array_equal(v, vl)


def test_host_plan_does_not_depend_on_thread_count():
    """The host plan of a large pattern (level space, elimination lists, slots; the AMG hierarchy with its Galerkin
    gather lists) is built with several host threads: every array is the same for 1, 2 and 5 threads (digests of the
    whole plans). A 101k-row system, large enough for the threaded paths. Host code only."""
    from ressim_gb300 import _build, synth
    L = C.CDLL(_build.LIB)
    L.rsg_debug_plan_digest.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    A = synth.make_system(48, 48, 44, sigma=1.5, seed=12, wells="corners+center").A
    ap = np.ascontiguousarray(A.val.reshape(-1, 3, 3)[:, 0, 0])
    digests = []
    for threads in (1, 2, 5):
        dp, da = C.c_ulonglong(0), C.c_ulonglong(0)
        assert L.rsg_debug_plan_digest(A.n, A.rowPtr.ctypes.data, A.col.ctypes.data, ap.ctypes.data, threads, C.byref(dp),
                                       C.byref(da)) == 0
        digests.append((dp.value, da.value))
    assert digests[0] == digests[1] == digests[2]


def test_same_pattern_check_of_set_batch():
    """rsg_set_batch reuses its plan when the batch has the plan's pattern, compared in place: the same batch is
    the same; a moved column, a row of another length, another system count are not. Host code only."""
    from ressim_gb300 import _build, synth
    L = C.CDLL(_build.LIB)
    L.rsg_debug_same_pattern.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]

    class Pattern:
        def __init__(self, n, rowPtr, col):
            self.n = n
            self.rowPtr = np.ascontiguousarray(rowPtr, np.int32)
            self.col = np.ascontiguousarray(col, np.int32)

    mats = [Pattern(s.A.n, s.A.rowPtr, s.A.col) for s in synth.ensemble(n_real=3, nx=8, ny=7, nz=3)]

    def same(a, b):
        na, nb = np.array([m.n for m in a], np.int32), np.array([m.n for m in b], np.int32)
        ra, ca = (C.c_void_p * len(a))(*[m.rowPtr.ctypes.data for m in a]), (C.c_void_p * len(a))(*[m.col.ctypes.data for m in a])
        rb, cb = (C.c_void_p * len(b))(*[m.rowPtr.ctypes.data for m in b]), (C.c_void_p * len(b))(*[m.col.ctypes.data for m in b])
        return L.rsg_debug_same_pattern(len(a), na.ctypes.data, ra, ca, len(b), nb.ctypes.data, rb, cb)

    assert same(mats, mats) == 1
    assert same(mats, [Pattern(m.n, m.rowPtr.copy(), m.col.copy()) for m in mats]) == 1     # equal copies
    assert same(mats, mats[:2]) == 0                                                       # another system count
    B = mats[1]
    # a column moved one place right in a row whose last entry has a free column after it (still sorted)
    col = B.col.copy()
    moved = False
    for i in range(B.n):
        p = B.rowPtr[i + 1] - 1
        if col[p] > i and col[p] + 1 < B.n:
            col[p] += 1
            moved = True
            break
    assert moved
    assert same(mats, [mats[0], Pattern(B.n, B.rowPtr, col), mats[2]]) == 0
    # a row of another length: the last off-diagonal entry of a row dropped
    i = next(i for i in range(B.n) if B.col[B.rowPtr[i + 1] - 1] > i)
    rp2 = B.rowPtr.copy()
    rp2[i + 1:] -= 1
    assert same(mats, [mats[0], Pattern(B.n, rp2, np.delete(B.col, B.rowPtr[i + 1] - 1)), mats[2]]) == 0


def test_black_oil_assembler_checks_model_and_pattern_before_the_device():
    """rsg_bo_create rejects model options outside the supported black-oil model and a Jacobian pattern that is not
    the engine's with RSG_EINVAL, before it touches a device (so these checks run without a GPU); a valid model gets
    as far as the device (RSG_ECUDA here, without a GPU)."""
    from conftest import gpu_available
    from ressim_gb300 import _lib
    from ressim_gb300.assembly import BlackOilAssembler
    z = dict(np.load(os.path.join(ROOT, "tests", "golden", "waterflood_asm.npz")))
    bad = dict(z)
    bad["phases"] = np.array([1, 1, 1, 1, 1], np.uint8)            # vaporised oil
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL and "vaporised" in str(e.value)
    bad = dict(z)
    bad["kroModel"] = np.array([2], np.int32)                      # STONE2
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL
    bad = dict(z)
    col = z["J_col"].copy()
    col[[0, 1]] = col[[1, 0]]                                      # columns of a cell row out of the engine's order
    bad["J_col"] = col
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL and "pattern" in str(e.value)
    bad = dict(z)
    conn = z["adjConn"].copy()
    conn[0] = conn[-1]                                             # an adjacency entry naming another pair's connection
    bad["adjConn"] = conn
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL and "connection" in str(e.value)
    # two connections exchanged between adjacency entries so that every connection is still named twice, once from
    # each of two cells it touches: c1 = (a, b1) named for a's neighbour b2 as well, c2 = (a, b2) named by b1
    st, nbr, cn, ca = z["adjStart"], z["adjNbr"], z["adjConn"].copy(), z["conn_a"]
    a = next(a for a in range(len(st) - 1) if sum(ca[cn[q]] == a for q in range(st[a], st[a + 1])) >= 2)
    q1, q2 = [q for q in range(st[a], st[a + 1]) if ca[cn[q]] == a][:2]
    b1, c1, c2 = nbr[q1], cn[q1], cn[q2]
    qb = next(q for q in range(st[b1], st[b1 + 1]) if nbr[q] == a)
    cn[q2], cn[qb] = c1, c2
    bad = dict(z)
    bad["adjConn"] = cn
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL and "connection" in str(e.value)
    bad = dict(z)
    v = z["vars"].copy()
    v[[0, 1]] = [0, 2]                                             # Sw in the pressure slot
    bad["vars"] = v
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(bad)
    assert e.value.code == _lib.RSG_EINVAL and "slots" in str(e.value)
    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(z)
    assert e.value.code == _lib.RSG_ECUDA


def test_assembly_golden_is_consistent():
    """The assembly golden vectors (the reference engine's): the full Jacobian is the reservoir terms plus the well
    terms -- rows that take no well term equal the reservoir-only assembly bit for bit, and the grid, pattern and
    tables describe the 20x20x4 three-phase live-oil waterflood."""
    z = dict(np.load(os.path.join(ROOT, "tests", "golden", "waterflood_asm.npz")))
    na, nv, nw = int(z["na"][0]), int(z["nv"][0]), int(z["nw"][0])
    assert (na, nv, nw) == (1600, 3, 2) and list(z["phases"]) == [1, 1, 1, 1, 0]
    rp = z["J_rowPtr"]
    assert rp.size == na * nv + nw + 1 and z["s1_J_full"].size == rp[-1]
    rows = np.searchsorted(rp, z["s1_add_pos"], side="right") - 1
    touched = np.zeros(na, bool)
    touched[rows[rows < na * nv] // nv] = True
    touched[z["s1_radd_pos"][z["s1_radd_pos"] < na * nv] // nv] = True
    free = np.repeat(~touched, nv)
    pos = np.repeat(free, np.diff(rp[:na * nv + 1]))
    assert np.array_equal(z["s1_J_full"][:rp[na * nv]][pos], z["s1_J_cell"][:rp[na * nv]][pos])
    assert np.array_equal(z["s1_R_full"][:na * nv][free], z["s1_R_cell"][:na * nv][free])
    states = [np.bincount(z[f"s{k}_hasGas"], minlength=3) for k in range(int(z["nstates"][0]))]
    assert states[0][1] > 0 and states[0][2] > 0                   # the perturbed state has free-gas and no-oil cells


def test_synthetic_assembly_model_is_the_engines_layout():
    """ressim_gb300.synth.assembly_model (the bench's assembly workload: several masked grids taken as one) builds the
    engine's scalar Jacobian pattern and adjacency: the assembler's checks accept it (and stop only at the device,
    without a GPU), and every connection appears once on each side."""
    from conftest import gpu_available
    from ressim_gb300 import _lib, synth
    from ressim_gb300.assembly import BlackOilAssembler
    grids = [synth.assembly_grid(8, 6, 3, seed=s, actnum_fraction=0.3) for s in (1, 2)]
    z, st = synth.assembly_model(grids)
    na = int(z["na"][0])
    assert na == sum(g["na"] for g in grids) and st["p"].size == na and st["acc_old"].size == 3 * na
    conn = z["adjConn"]
    assert np.array_equal(np.bincount(conn, minlength=z["conn_trans"].size), np.full(z["conn_trans"].size, 2))
    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.RsgError) as e:
        BlackOilAssembler(z)
    assert e.value.code == _lib.RSG_ECUDA, e.value

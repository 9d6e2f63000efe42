"""GPU parity: the CUDA path through the C ABI against the reference's golden vectors and the oracle.

Tolerances: integer / structural results and the FP64 kernels that follow the reference's serial arithmetic
(SpMV, BILU0 factors, BILU0 sweeps) are compared bit for bit; Krylov solutions, whose inner products are
reduced in a different (tree) order, must match the reference solution within 1e-8 relative (the plain FP64
path's accuracy bar) at the same iteration count; FP32 preconditioner outputs within 1e-5 relative of the oracle's float
restatement; every solve's true residual ||b - A x|| / ||b|| is recomputed in FP64 on the host.
"""
import numpy as np
import pytest

from conftest import ALL_GOLDEN, GOLDEN_SYSTEMS, load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def true_res(A, x, b):
    from ressim_gb300 import synth
    return np.linalg.norm(b - synth.bsr_matvec_host(A, x)) / np.linalg.norm(b)


def dev(**kw):
    from ressim_gb300.solver import DeviceSolver
    return DeviceSolver(**kw)


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_spmv_bitwise(name):
    A, z = load_golden(name)
    with dev(fma=False) as d:                                   # the reference's rounding: bit for bit
        d.set_matrix(A)
        assert np.array_equal(d.spmv(z["x_seed"]), z["y_spmv"])
    with dev() as d:                                            # fused multiply-adds: within rounding
        d.set_matrix(A)
        y = d.spmv(z["x_seed"])
    from ressim_gb300 import synth
    from ressim_gb300.bsr import BSR
    scale = synth.bsr_matvec_host(BSR(A.n, A.nb, A.rowPtr, A.col, np.abs(A.val)), np.abs(z["x_seed"]))   # |A| |x|
    assert np.all(np.abs(y - z["y_spmv"]) <= 1e-14 * np.maximum(scale, 1e-300))


@pytest.mark.parametrize("sweep", ["cta", "grid"])
@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_bilu0_factors_and_sweeps_bitwise(name, sweep):
    A, z = load_golden(name)
    with dev(sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        if "lu" in z.files:
            assert np.array_equal(d.factors(A.nnzb), z["lu"])
            assert d.stats().regularised_blocks == int(z["nreg"])
        assert np.array_equal(d.precond_apply(z["b"]), z["z_bilu0"])


@pytest.mark.parametrize("fma", [False, True])
@pytest.mark.parametrize("sweep", ["cta", "grid"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS + ["singular_pivots.npz"])
@pytest.mark.parametrize("case,tol,maxit", [("bicg_bilu0", 1e-6, 120), ("bicg_bilu0_tight", 1e-10, 1000)])
def test_bicgstab_bilu0_matches_reference(name, case, tol, maxit, sweep, fma):
    A, z = load_golden(name)
    if not bool(z["conv_" + case]):
        pytest.skip("the reference does not converge on this case")
    with dev(check_every=3, sweep=sweep, fma=fma) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=tol, maxit=maxit)
    assert res.converged
    sens = float(z["sens_" + case])
    if sens < 1e-3:
        # SpMV (fma=False) and BILU0 round as the reference does, the inner products are summed as a tree across the
        # tile and not left to right: the last digits move as under any change of summation order, which may end the
        # iteration a step earlier or later (two at 1e-10 over ~40 steps); fused multiply-adds do the same
        its_ref = int(z["its_" + case])
        assert abs(res.iterations - its_ref) <= max(1, its_ref // 15)
    else:   # near-singular system: the iteration count itself moves under a change of summation order
        assert res.iterations <= 3 * int(z["its_" + case])
    # 1e-8 relative, or 10x the solution's own sensitivity to a change of inner-product summation order
    # (measured on the CPU when the golden vectors were made; ~1e-10 for the captured waterflood systems)
    assert rel(x, z["x_" + case]) < max(1e-8, 10 * float(z["sens_" + case]))
    assert true_res(A, x, z["b"]) <= max(10 * tol, 1e-12)


@pytest.mark.parametrize("graphs", [True, False])
def test_graph_and_eager_identical(graphs):
    A, z = load_golden("waterflood_sys1.npz")
    with dev(use_graphs=graphs, check_every=5) as d:
        d.set_matrix(A)
        d.setup()
        x1, r1 = d.solve(z["b"], tol=1e-8, maxit=200)
        x2, r2 = d.solve(z["b"], tol=1e-8, maxit=200)      # repeat: deterministic reductions
    assert np.array_equal(x1, x2) and r1.iterations == r2.iterations


@pytest.mark.parametrize("sweep", ["cta", "grid"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_mixed_precision(name, oracle, sweep):
    A, z = load_golden(name)
    luf, _ = oracle.bilu0_factor_lean(A)
    with dev(precision="mixed_f32", sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        # thread-block path: FP32 elimination with FP64 pivot inversions, bit for bit the oracle's restatement;
        # grid path: the lean factors. Sweeps in FP32: float rounding of the oracle's all-float sweep.
        f32, nreg = oracle.bilu0_factor_f32(A) if sweep == "cta" else (luf, 0)
        if sweep == "cta":
            assert np.array_equal(d.factors(A.nnzb), f32.astype(np.float64))
            assert d.stats().regularised_blocks == nreg
        assert rel(d.precond_apply(z["b"]), oracle.bilu0_apply_ff(A, f32, z["b"])) < 1e-5
    with dev(precision="mixed", sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        # lean FP32 factors + FP64 sweep: same arithmetic as the oracle, bit for bit
        assert np.array_equal(d.precond_apply(z["b"]), oracle.bilu0_apply_fd(A, luf, z["b"]))
        for tol in (1e-6, 1e-8):
            x, res = d.solve(z["b"], tol=tol, maxit=300)
            assert res.converged
            assert true_res(A, x, z["b"]) <= 10 * tol
            # error against the FP64 reference solution, reported per tolerance
            err = rel(x, z["x_bicg_bilu0_tight"])
            assert err < 1e3 * tol, err


def test_batch_equals_individual():
    mats, bs, xs = [], [], []
    for name in ["waterflood_sys0.npz", "waterflood_sys2.npz", "synth_small.npz", "waterflood_sys1.npz", "singular_pivots.npz"]:
        A, z = load_golden(name)
        mats.append(A)
        bs.append(z["b"])
    for A, b in zip(mats, bs):
        with dev() as d:
            d.set_matrix(A)
            d.setup()
            x, res = d.solve(b, tol=1e-8, maxit=400)
            xs.append((x, res.iterations, res.trueRelResidual))
    with dev() as d:
        d.set_batch(mats)
        d.setup()
        xb, res = d.solve(np.concatenate(bs), tol=1e-8, maxit=400)
        its, rr, tr = d.batch_results()
    off = 0
    for k, A in enumerate(mats):
        N = A.n * A.nb
        assert its[k] == xs[k][1]
        assert rel(xb[off:off + N], xs[k][0]) < 1e-10
        assert abs(tr[k] - xs[k][2]) <= 1e-6 * max(xs[k][2], 1e-12)   # same true residual alone and in the batch
        off += N


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_synthetic_ensemble_true_residual(precision):
    """Size-independent property on a larger batch: every system converges with true residual <= tol."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=8, nx=24, ny=24, nz=6, sigma=1.5)
    with dev(precision=precision) as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        x, res = d.solve(np.concatenate([s.b for s in systems]), tol=1e-6, maxit=500)
        its, rr, tr = d.batch_results()
    assert res.converged
    off = 0
    for s in systems:
        N = s.A.n * 3
        assert true_res(s.A, x[off:off + N], s.b) <= 1e-5
        off += N
    assert np.all(tr <= 1e-5)


def test_jacobi_converges():
    A, z = load_golden("synth_small.npz")
    with dev(precond="jacobi") as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=1e-6, maxit=2000)
    assert res.converged and true_res(A, x, z["b"]) <= 1e-5


def test_error_paths():
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import BSR
    A, z = load_golden("waterflood_sys0.npz")
    with dev(fma=False) as d:
        with pytest.raises(_lib.RsgError):
            d.solve(z["b"])                                   # before set_matrix
        d.set_matrix(A)
        with pytest.raises(_lib.RsgError) as e:
            d.solve(z["b"])                                   # before setup
        assert e.value.code == _lib.RSG_ESTATE
        d.setup()
        b = z["b"].copy()
        b[7] = np.nan
        with pytest.raises(_lib.RsgError) as e:               # non-finite rhs: ends with a breakdown, no hang
            d.solve(b, tol=1e-6, maxit=50)
        assert e.value.code == _lib.RSG_EBREAKDOWN
        x, res = d.solve(z["b"], tol=1e-6, maxit=120)         # the handle stays usable
        assert res.converged and abs(res.iterations - int(z["its_bicg_bilu0"])) <= 1   # tree-summed inner products
    # missing diagonal block
    rp = np.array([0, 1, 2], dtype=np.int32)
    bad = BSR(2, 3, rp, np.array([1, 0], dtype=np.int32), np.ones(18))
    with dev() as d:
        with pytest.raises(_lib.RsgError) as e:
            d.set_matrix(bad)
        assert "diagonal" in str(e.value)


def test_gpu_block_solver_adapter():
    from ressim_gb300.solver import GpuBlockSolver
    A, z = load_golden("waterflood_sys2.npz")
    g = GpuBlockSolver(fma=False)
    ok, x, its = g.solve(A, z["b"], 1e-6, 120)
    assert ok and abs(its - int(z["its_bicg_bilu0"])) <= 1                           # tree-summed inner products
    assert rel(x, z["x_bicg_bilu0"]) < 1e-8
    assert g.deviceSeconds() > 0


# ---------------------------------------------------------------- CPR (AMG on the pressure system + BILU0)
@pytest.mark.parametrize("sweep", ["cta", "split", "grid"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_cpr_apply_matches_reference(name, sweep):
    """BlockCPR::apply: weights, pressure matrix, aggregation hierarchy, Gauss-Seidel V-cycle and BILU0 are the
    reference's arithmetic; only the back substitution of the coarsest dense LU runs column-wise (summation order).
    Both applications: one thread block per system, and grid-wide (sync-free sweeps, level by level)."""
    A, z = load_golden(name)
    with dev(precond="cpr", sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        assert d.stats().amg_levels == len(z["amg_rows"])
        assert rel(d.precond_apply(z["b"]), z["z_cpr"]) < 1e-10
    if "acc" in z.files:                                  # true-IMPES weights from the accumulation blocks
        with dev(precond="cpr", sweep=sweep) as d:
            d.set_matrix(A)
            d.setup(acc=z["acc"])
            assert rel(d.precond_apply(z["b"]), z["z_cpr_acc"]) < 1e-10


@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_amg_level_sizes_match_reference(name):
    """rsg_amg_level_sizes reports the reference hierarchy's level sizes (rows, entries); for a batch, their sums."""
    A, z = load_golden(name)
    with dev(precond="cpr") as d:
        d.set_matrix(A)
        d.setup()
        rows, nnz, dense = d.amg_level_sizes()
    assert list(rows) == list(z["amg_rows"]) and list(nnz) == list(z["amg_nnz"])
    assert dense in (0, int(z["amg_rows"][-1]) ** 2)
    with dev(precond="cpr") as d:
        d.set_batch([A, A])
        d.setup()
        rows2, nnz2, dense2 = d.amg_level_sizes()
    assert list(rows2) == [2 * int(r) for r in z["amg_rows"]] and list(nnz2) == [2 * int(q) for q in z["amg_nnz"]]
    assert dense2 == 2 * dense
    with dev(precond="bilu0") as d:
        d.set_matrix(A)
        d.setup()
        assert d.amg_level_sizes() is None


@pytest.mark.parametrize("sweep", ["cta", "split", "grid"])
@pytest.mark.parametrize("precision", ["mixed", "mixed_f32"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_cpr_multicolour_apply_matches_oracle(name, precision, sweep, oracle):
    """FP32 precision forms: FP32 hierarchy smoothed by multicolour Gauss-Seidel; against the oracle's FP64
    restatement of the same algorithm (float rounding of factors, hierarchy, coarse LU and sweeps)."""
    A, z = load_golden(name)
    with dev(precond="cpr", precision=precision, sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        zd = d.precond_apply(z["b"])
    oracle.set_mc_smoother(True)
    try:
        zo = oracle.prec_apply(A, z["b"], prec=1)
    finally:
        oracle.set_mc_smoother(False)
    # float rounding of the pressure hierarchy and its dense coarsest LU, amplified by the coarse condition number
    # (1e-4 .. 2e-4 on the captured systems); an ordering or indexing error shows up as O(1)
    assert rel(zd, zo) < 1e-3


def parity_bound(z, case):
    """1e-8 relative, or 10x the reference solution's own movement under a change of inner-product summation order
    (recorded with the golden vectors; below 1e-9 for every converged tight case except the near-singular system)."""
    return max(1e-8, 10 * float(z["sens_" + case]))


@pytest.mark.parametrize("sweep", ["cta", "split", "grid"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_cpr_bicgstab_matches_reference(name, sweep):
    """The plain FP64 CPR-BiCGSTAB (the bench's plain path) against the reference's own CPR-BiCGSTAB solution of the
    same system: at 1e-6 the iteration count, at 1e-10 the solution within 1e-8."""
    A, z = load_golden(name)
    with dev(precond="cpr", check_every=2, sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=1e-6, maxit=120)
        assert res.converged
        assert abs(res.iterations - int(z["its_bicg_cpr"])) <= 1
        assert true_res(A, x, z["b"]) <= 1e-5
        xt, rt = d.solve(z["b"], tol=1e-10, maxit=500)
    assert rt.converged
    assert abs(rt.iterations - int(z["its_bicg_cpr_tight"])) <= 1
    assert rel(xt, z["x_bicg_cpr_tight"]) < parity_bound(z, "bicg_cpr_tight")
    assert true_res(A, xt, z["b"]) <= 1e-9


def test_cpr_refresh_equals_fresh_setup():
    """Values-only refresh of the hierarchy (AMG::refresh) equals a fresh set-up on the same values."""
    A, z = load_golden("waterflood_sys1.npz")
    A2 = A.scaled(1.5)
    with dev(precond="cpr") as d:
        d.set_matrix(A)
        d.setup()
        d.set_matrix(A2)                                   # same pattern: refresh
        d.setup()
        z1 = d.precond_apply(z["b"])
    with dev(precond="cpr") as d:
        d.set_matrix(A2)
        d.setup()
        z2 = d.precond_apply(z["b"])
    assert rel(z1, z2) < 1e-12


@pytest.mark.parametrize("sweep", ["cta", "split", "grid"])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_f32"])
def test_cpr_batched_ensemble(precision, sweep):
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=6, nx=24, ny=24, nz=6, sigma=1.5)
    with dev(precond="cpr", precision=precision, check_every=4, sweep=sweep) as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        x, res = d.solve(np.concatenate([s.b for s in systems]), tol=1e-6, maxit=300)
        its, rr, tr = d.batch_results()
    assert res.converged
    assert np.all(tr <= 1e-5)
    off = 0
    for s in systems:
        N = s.A.n * 3
        assert true_res(s.A, x[off:off + N], s.b) <= 1e-5
        off += N


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_f32"])
def test_split_cpr_equals_thread_block(precision):
    """The split CPR (V-cycle passes grid-wide over every system, BILU0 sweeps one thread block per system) gives
    the one-kernel thread-block application's results: same preconditioner output and same solve, on a batch with
    well cliques (the small colours of the multicolour smoother)."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=6, nx=24, ny=24, nz=6, sigma=1.5)
    b = np.concatenate([s.b for s in systems])
    out = {}
    for sweep in ("cta", "split"):
        with dev(precond="cpr", precision=precision, check_every=4, sweep=sweep) as d:
            d.set_batch([s.A for s in systems])
            d.setup()
            z = d.precond_apply(b)
            x, res = d.solve(b, tol=1e-6, maxit=300)
            out[sweep] = (z, x, d.batch_results()[0])
    assert np.array_equal(out["cta"][0], out["split"][0])
    assert np.array_equal(out["cta"][1], out["split"][1])
    assert np.array_equal(out["cta"][2], out["split"][2])


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_f32"])
def test_cpr_large_systems(precision, oracle):
    """Systems too large to keep every V-cycle / sweep vector on chip (b and r of the V-cycle and the FP64 sweep
    vector in global memory): the CPR application against the oracle, and batched solves to the true residual."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=3, nx=60, ny=60, nz=8, sigma=1.5)
    assert max(s.A.n for s in systems) > 16000
    A0 = systems[0].A
    r = np.random.default_rng(5).standard_normal(A0.n * 3)
    with dev(precond="cpr", precision=precision) as d:
        d.set_matrix(A0)
        d.setup()
        z = d.precond_apply(r)
    oracle.set_mc_smoother(precision != "fp64")            # the FP32 forms smooth with multicolour Gauss-Seidel
    try:
        zo = oracle.prec_apply(A0, r, prec=1)
    finally:
        oracle.set_mc_smoother(False)
    # FP64: the reference arithmetic up to the coarsest back substitution's order; FP32 V-cycle / sweeps: float
    assert rel(z, zo) < (1e-10 if precision == "fp64" else 1e-3)
    with dev(precond="cpr", precision=precision, check_every=4) as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        x, res = d.solve(np.concatenate([s.b for s in systems]), tol=1e-6, maxit=300)
        its, rr, tr = d.batch_results()
    assert res.converged
    assert np.all(tr <= 1e-5)
    off = 0
    for s in systems:
        N = s.A.n * 3
        assert true_res(s.A, x[off:off + N], s.b) <= 1e-5
        off += N


@pytest.mark.parametrize("precision", ["fp64", "mixed_f32"])
def test_cpr_single_large_system(precision, oracle):
    """One system too large for one SM (73,728 cells): the grid-wide CPR application against the oracle, and the
    CPR-BiCGSTAB solve (which takes the grid path by itself) to the true residual."""
    from ressim_gb300 import synth
    s = synth.make_system(48, 48, 32, sigma=2.0, seed=11, dt=5.0, wells="random", n_wells=4)
    A = s.A
    assert A.n > 65536
    r = np.random.default_rng(6).standard_normal(A.n * 3)
    with dev(precond="cpr", precision=precision) as d:
        d.set_matrix(A)
        d.setup()
        z = d.precond_apply(r)
        x, res = d.solve(s.b, tol=1e-6, maxit=300)
    oracle.set_mc_smoother(precision != "fp64")
    try:
        zo = oracle.prec_apply(A, r, prec=1)
    finally:
        oracle.set_mc_smoother(False)
    assert rel(z, zo) < (1e-10 if precision == "fp64" else 1e-3)
    assert res.converged and true_res(A, x, s.b) <= 1e-5


def test_spe10_sized_cpr_gmres(oracle):
    """The one-large-system configurations: 60x220x85 cells (1,122,000 block rows, 7.8M blocks, sigma ln k = 2.5 with
    x100 channels), CPR with true-IMPES weights (the accumulation blocks, as the engine's BlockCPR::setup uses them) +
    GMRES(30), the day-1 Jacobian. The oracle (the C restatement of the reference) reaches 1e-6; the plain FP64 path
    reaches it within three iterations of the oracle's count, with the residual after one restart cycle equal to the
    oracle's up to inner-product summation order; the FP32 precision form reaches 1e-6 in true residual as well."""
    import math
    import os
    from ressim_gb300 import synth
    s = synth.spe10_like(day=1)
    assert s.A.n == 1_122_000
    oracle.set_threads(os.cpu_count() or 1)     # a large system; the comparisons below allow for summation order
    try:
        _, _, its30, rr30, _, _ = oracle.solve(s.A, s.b, prec=1, method=1, restart=30, tol=1e-12, maxit=30, acc=s.acc)
        _, conv_o, its_o, rr_o, _, _ = oracle.solve(s.A, s.b, prec=1, method=1, restart=30, tol=1e-6, maxit=600, acc=s.acc)
    finally:
        oracle.set_threads(1)                    # the session's oracle stays single-threaded (reproducible) for the rest
    assert its30 == 30 and conv_o
    for precision in ("fp64", "mixed_f32"):
        with dev(precond="cpr", krylov="gmres", restart=30, precision=precision) as d:
            d.set_matrix(s.A)
            d.setup(s.acc)
            if precision == "fp64":
                _, r30 = d.solve(s.b, tol=1e-12, maxit=30)
                assert abs(math.log(r30.relResidual / rr30)) < math.log(1.5), (r30, rr30)
            x, res = d.solve(s.b, tol=1e-6, maxit=600)
        assert res.converged and true_res(s.A, x, s.b) <= 1.01e-6, (precision, res)
        if precision == "fp64":
            assert abs(res.iterations - its_o) <= 3, (res.iterations, its_o)


def _hard_request():
    """A serving request with extreme permeability contrast (sigma ln k near 3) on which the all-FP32 preconditioner
    diverges (60,372 cells): the tenth of the stratified serving pool."""
    from ressim_gb300 import synth
    rng = np.random.default_rng(4242)
    for i in range(10):
        cells = 1e3 * 1000.0 ** ((i + 0.5) / 16)
        s = synth.serving_request(rng, cells_lo=cells, cells_hi=cells)
    return s


def test_precision_escalation():
    """All-FP32 preconditioner on a system where its FP32 sweeps diverge: the divergence guard stops it, the system
    is solved again with FP64 sweep vectors and converges to the true residual; in a batch, the easy system that
    converged in FP32 keeps exactly the result it has alone."""
    hard = _hard_request()
    easy = load_golden("waterflood_sys1.npz")
    with dev(precond="cpr", precision="mixed_f32") as d:
        d.set_matrix(hard.A)
        d.setup()
        x, res = d.solve(hard.b, tol=1e-6, maxit=500)
        assert d.stats().escalated_systems == 1
    assert res.converged and true_res(hard.A, x, hard.b) <= 1e-5
    with dev(precond="cpr", precision="mixed_f32") as d:
        d.set_matrix(easy[0])
        d.setup()
        xe, re_ = d.solve(easy[1]["b"], tol=1e-6, maxit=500)
        assert d.stats().escalated_systems == 0
    with dev(precond="cpr", precision="mixed_f32") as d:
        d.set_batch([easy[0], hard.A])
        d.setup()
        xb, rb = d.solve(np.concatenate([easy[1]["b"], hard.b]), tol=1e-6, maxit=500)
        its, rr, tr = d.batch_results()
        assert d.stats().escalated_systems == 1
    Ne = easy[0].n * 3
    assert np.array_equal(xb[:Ne], xe) and its[0] == re_.iterations
    assert true_res(hard.A, xb[Ne:], hard.b) <= 1e-5


def test_precision_escalation_after_gmres():
    """The same escalation under GMRES: a system the all-FP32 sweeps leave unconverged in the precision form is solved
    again with FP64 sweep vectors and reaches the tolerance; the converged system of the batch keeps its result."""
    hard = _hard_request()
    easy = load_golden("waterflood_sys1.npz")
    with dev(precond="cpr", krylov="gmres", restart=30, precision="mixed_f32") as d:
        d.set_matrix(easy[0])
        d.setup()
        xe, re_ = d.solve(easy[1]["b"], tol=1e-6, maxit=300)
        assert d.stats().escalated_systems == 0
    with dev(precond="cpr", krylov="gmres", restart=30, precision="mixed_f32") as d:
        d.set_batch([easy[0], hard.A])
        d.setup()
        xb, rb = d.solve(np.concatenate([easy[1]["b"], hard.b]), tol=1e-6, maxit=300)
        its, rr, tr = d.batch_results()
    Ne = easy[0].n * 3
    assert np.array_equal(xb[:Ne], xe) and its[0] == re_.iterations
    assert true_res(hard.A, xb[Ne:], hard.b) <= 1e-5


# ---------------------------------------------------------------- multicolour BILU0 (engine/src/bsr.cpp:599-730)
@pytest.mark.parametrize("sweep", ["cta", "grid"])
@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_mcbilu0_matches_reference(name, sweep):
    """MCBILU0::factor / apply: the natural-order BILU0 of the colour-permuted matrix, bit for bit the reference's."""
    A, z = load_golden(name)
    with dev(precond="mcbilu0", sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        assert np.array_equal(d.precond_apply(z["b"]), z["z_mcbilu0"])


@pytest.mark.parametrize("precision", ["fp64", "mixed_f32"])
def test_mcbilu0_batched_solves(precision):
    """Multicolour BILU0 on a batch of ensemble systems: every system reaches the true residual, and the batch
    result equals each system's solve alone."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=4, nx=24, ny=24, nz=6, sigma=1.5)
    alone = []
    for sy in systems:
        with dev(precond="mcbilu0", precision=precision) as d:
            d.set_matrix(sy.A)
            d.setup()
            alone.append(d.solve(sy.b, tol=1e-6, maxit=800))
    with dev(precond="mcbilu0", precision=precision) as d:
        d.set_batch([sy.A for sy in systems])
        d.setup()
        x, res = d.solve(np.concatenate([sy.b for sy in systems]), tol=1e-6, maxit=800)
        its, rr, tr = d.batch_results()
    assert res.converged and np.all(tr <= 1e-5)
    off = 0
    for k, sy in enumerate(systems):
        N = sy.A.n * 3
        assert np.array_equal(x[off:off + N], alone[k][0]) and its[k] == alone[k][1].iterations
        off += N


# ---------------------------------------------------------------- the reference's GPU-shaped float CPR-AMG
@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_device_cpr_amg_matches_reference(name):
    """DeviceCprAmg::apply (engine/src/bsr.cpp:1217-1371): float hierarchy, damped-Jacobi V-cycle, double
    Gauss-Jordan coarse inverse, block-Jacobi second stage; every float operation rounded as the reference does it:
    bit for bit the reference's float output (input rounded to float)."""
    A, z = load_golden(name)
    with dev(precond="cpr_device") as d:
        d.set_matrix(A)
        d.setup()
        zd = d.precond_apply(z["b"])
    assert np.array_equal(zd, z["z_devcpr"].astype(np.float64))


def test_device_cpr_amg_large_system_and_solves(oracle):
    """A system of 73,728 cells: the application against the oracle's float restatement bit for bit; BiCGSTAB with it
    reaches the true residual, alone and in a batch with the captured systems (same result for each)."""
    from ressim_gb300 import synth
    s = synth.make_system(48, 48, 32, sigma=2.0, seed=11, dt=5.0, wells="random", n_wells=4)
    r = np.random.default_rng(8).standard_normal(s.A.n * 3)
    with dev(precond="cpr_device") as d:
        d.set_matrix(s.A)
        d.setup()
        zd = d.precond_apply(r)
        x, res = d.solve(s.b, tol=1e-6, maxit=1000)
    assert np.array_equal(zd, oracle.devcpr_apply(s.A, r).astype(np.float64))
    assert res.converged and true_res(s.A, x, s.b) <= 1e-5
    mats, bs = [s.A], [s.b]
    for name in GOLDEN_SYSTEMS:
        A, z = load_golden(name)
        mats.append(A)
        bs.append(z["b"])
    with dev(precond="cpr_device") as d:
        d.set_batch(mats)
        d.setup()
        xb, rb = d.solve(np.concatenate(bs), tol=1e-6, maxit=1000)
        its, rr, tr = d.batch_results()
    assert rb.converged and np.all(tr <= 1e-5)
    assert np.array_equal(xb[:s.A.n * 3], x) and its[0] == res.iterations


# ---------------------------------------------------------------- GMRES (flexible, restarted; linsolve.cpp:218-273)
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS + ["singular_pivots.npz"])
def test_gmres_bilu0_matches_reference(name):
    A, z = load_golden(name)
    if not bool(z["conv_gmres_bilu0"]):
        pytest.skip("the reference does not converge on this case")
    with dev(krylov="gmres", restart=30, check_every=5) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=1e-6, maxit=300)
    assert res.converged
    assert abs(res.iterations - int(z["its_gmres_bilu0"])) <= 1
    assert rel(x, z["x_gmres_bilu0"]) < 1e-6
    assert true_res(A, x, z["b"]) <= 1e-5


@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
@pytest.mark.parametrize("sweep", ["cta", "split", "grid"])
def test_gmres_cpr_matches_reference(name, sweep):
    A, z = load_golden(name)
    with dev(krylov="gmres", precond="cpr", restart=30, sweep=sweep) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=1e-6, maxit=300)
    assert res.converged
    assert abs(res.iterations - int(z["its_gmres_cpr"])) <= 1
    assert rel(x, z["x_gmres_cpr"]) < 1e-6
    assert true_res(A, x, z["b"]) <= 1e-5


@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
@pytest.mark.parametrize("case,prec,restart,maxit", [("gmres_bilu0_tight", "bilu0", 30, 1000), ("gmres_cpr_tight", "cpr", 30, 500),
                                                     ("gmres60_bilu0_tight", "bilu0", 60, 1000), ("gmres60_cpr_tight", "cpr", 60, 500)])
def test_gmres_tight_matches_reference(name, case, prec, restart, maxit):
    """GMRES(30) (the one-large-system configuration) and GMRES(60) (the engine's fallback,
    engine/src/simulator.cpp:3390-3398), BILU0 and CPR, to 1e-12: the GPU solution within 1e-8 of the reference's
    own solution of the same method, at the reference's iteration count within +-1. (The near-singular system is left
    out: there the reference's own GMRES stops on its recursive residual at a true residual of order 0.1, so neither
    solution is meaningful at 1e-12.)"""
    A, z = load_golden(name)
    if not bool(z["conv_" + case]):
        pytest.skip("the reference does not converge on this case")
    with dev(krylov="gmres", precond=prec, restart=restart, check_every=5) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(z["b"], tol=1e-12, maxit=maxit)
    assert res.converged
    its_ref = int(z["its_" + case])
    assert abs(res.iterations - its_ref) <= max(1, its_ref // 50)
    assert rel(x, z["x_" + case]) < parity_bound(z, case)


def test_gmres_restarts_and_batch(oracle):
    """Short restart cycles (several restarts) on a batch: every system equals its own solve and the oracle's."""
    mats, bs = [], []
    for name in ["waterflood_sys0.npz", "synth_small.npz", "waterflood_sys2.npz"]:
        A, z = load_golden(name)
        mats.append(A)
        bs.append(z["b"])
    singles = []
    for A, b in zip(mats, bs):
        with dev(krylov="gmres", restart=10, check_every=2) as d:
            d.set_matrix(A)
            d.setup()
            x, res = d.solve(b, tol=1e-8, maxit=400)
            singles.append((x, res.iterations))
        xo, conv, its, rr, _, _ = oracle.solve(A, b, prec=0, method=1, restart=10, tol=1e-8, maxit=400)
        assert res.converged and conv                     # 91 / 265 / 264 iterations, 9 to 27 restarts
        assert abs(res.iterations - its) <= max(2, its // 30)
        assert rel(x, xo) < 1e-5
        assert true_res(A, x, b) <= 1e-7
    with dev(krylov="gmres", restart=10, check_every=2) as d:
        d.set_batch(mats)
        d.setup()
        xb, res = d.solve(np.concatenate(bs), tol=1e-8, maxit=400)
        its, rr, tr = d.batch_results()
    off = 0
    for k, A in enumerate(mats):
        N = A.n * A.nb
        assert its[k] == singles[k][1]
        assert rel(xb[off:off + N], singles[k][0]) < 1e-12
        off += N


@pytest.mark.parametrize("precision", ["mixed", "mixed_f32"])
def test_gmres_mixed_and_graphs(precision):
    A, z = load_golden("waterflood_sys1.npz")
    out = []
    for graphs in (True, False):
        with dev(krylov="gmres", precision=precision, use_graphs=graphs) as d:
            d.set_matrix(A)
            d.setup()
            x, res = d.solve(z["b"], tol=1e-8, maxit=300)
        assert res.converged and true_res(A, x, z["b"]) <= 1e-7
        out.append((x, res.iterations))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_gmres_fallback_keeps_the_better_result():
    """BiCGSTAB capped below convergence, GMRES retried on the failed systems: per system the result with the
    smaller recursive residual is kept and both solves' iterations count (engine/src/simulator.cpp:3388-3398)."""
    from ressim_gb300 import _lib
    A, z = load_golden("waterflood_sys0.npz")
    b = z["b"]
    maxit = 8

    def run(**kw):
        with dev(check_every=1, **kw) as d:
            d.set_matrix(A)
            d.setup()
            x, res = d.solve(b, tol=1e-10, maxit=maxit)      # not converged: the iterate comes back (RSG_ENOTCONV)
            assert res.status == _lib.RSG_ENOTCONV
            its, rr, tr = d.batch_results()
        return x, int(its[0]), float(rr[0])

    x1, i1, r1 = run()
    x2, i2, r2 = run(krylov="gmres", restart=30)
    x3, i3, r3 = run(gmres_fallback=True, restart=30)
    assert i3 == i1 + i2
    if r2 < r1:
        assert r3 == r2 and np.array_equal(x3, x2)
    else:
        assert r3 == r1 and np.array_equal(x3, x1)


# ---------------------------------------------------------------- the headline configuration (40x40x10 ensemble)
HEADLINE_MEMBERS = (0, 21, 42, 63)


@pytest.fixture(scope="module")
def headline_systems():
    from ressim_gb300 import synth
    return [synth.ensemble_member(r) for r in HEADLINE_MEMBERS]


def test_headline_ensemble_fp64_matches_oracle(headline_systems, oracle):
    """Four of the benchmark's own 40x40x10 realisations (8k-14.4k active cells, the bench's seeds): the plain FP64
    CPR-BiCGSTAB on the GPU, batched and alone, against the oracle's FP64 CPR-BiCGSTAB (the reference's arithmetic,
    one thread) at 1e-12: solutions within 1e-8 (their summation-order sensitivity is at most 3e-10 there)."""
    systems = headline_systems
    b = np.concatenate([s.b for s in systems])
    with dev(precond="cpr", precision="fp64", check_every=4) as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        x, res = d.solve(b, tol=1e-12, maxit=500)
        its, rr, tr = d.batch_results()
    assert res.converged
    with dev(precond="cpr", precision="fp64", check_every=4) as d:      # the plain path: one system per handle
        d.set_matrix(systems[1].A)
        d.setup()
        x1, r1 = d.solve(systems[1].b, tol=1e-12, maxit=500)
    off = 0
    for k, s in enumerate(systems):
        N = s.A.n * 3
        xo, conv, its_o, rr_o, _, _ = oracle.solve(s.A, s.b, prec=1, method=0, tol=1e-12, maxit=500)
        assert conv
        assert abs(int(its[k]) - its_o) <= 2
        assert rel(x[off:off + N], xo) < 1e-8
        assert true_res(s.A, x[off:off + N], s.b) <= 1e-11
        if k == 1:
            assert np.array_equal(x1, x[off:off + N])
        off += N


def test_headline_ensemble_precision_form_error(headline_systems):
    """The precision form (FP32 preconditioner, FP64 Krylov) at the benchmark's 1e-6 states its error against the
    FP64 solution: it converges to true relative residual <= 1e-6, and its distance to the tight FP64 solution is of
    the size a 1e-6 residual allows -- within 10x the plain FP64 solve's own distance at the same tolerance."""
    systems = headline_systems
    b = np.concatenate([s.b for s in systems])
    sol = {}
    for precision, tol in (("fp64", 1e-12), ("fp64", 1e-6), ("mixed_f32", 1e-6)):
        with dev(precond="cpr", precision=precision, check_every=4) as d:
            d.set_batch([s.A for s in systems])
            d.setup()
            x, res = d.solve(b, tol=tol, maxit=500)
            its, rr, tr = d.batch_results()
        assert res.converged and np.all(tr <= max(tol, 1e-11))
        sol[(precision, tol)] = x
    off = 0
    for s in systems:
        N = s.A.n * 3
        ref = sol[("fp64", 1e-12)][off:off + N]
        e64 = rel(sol[("fp64", 1e-6)][off:off + N], ref)
        e32 = rel(sol[("mixed_f32", 1e-6)][off:off + N], ref)
        assert e32 < max(10 * e64, 1e-5), (e32, e64)
        assert e32 < 5e-3
        off += N


# ---------------------------------------------------------------- FP64 defect correction (refineWithDevice)
@pytest.mark.parametrize("precond", ["bilu0", "cpr"])
@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_refined_solve_matches_reference_refinement(name, precond):
    """rsg_solve_refined: the reference's FP64 defect correction (engine/src/bsr.cpp:1373-1396: inner solves to
    clamp(10 tol, 1e-4, 1e-2), at most 6 passes, FP64 residual) around the precision form, to 1e-8. The reference
    refines its float device emulation the same way (golden x_refine); both end within 1e-8 in FP64, so both solutions
    are within the system's conditioning of the tight FP64 solution."""
    A, z = load_golden(name)
    with dev(precond=precond, precision="mixed_f32", check_every=2) as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve_refined(z["b"], tol=1e-8, max_outer=6, inner_it=120)
    assert res.converged and res.trueRelResidual <= 1e-8
    assert true_res(A, x, z["b"]) <= 2e-8
    xt = z["x_bicg_bilu0_tight"]
    err_ref = rel(z["x_refine"], xt)                 # the reference's own refined solution against the tight one
    assert rel(x, xt) < max(10 * err_ref, 1e-6), (rel(x, xt), err_ref)


@pytest.mark.parametrize("name", ["waterflood_sys1.npz", "synth_small.npz"])
def test_refined_solve_with_gmres_inner(name):
    """The refinement's inner solve is the handle's own Krylov method: with GMRES(30) (the large-system configuration's
    method) the FP64 defect correction around the precision form reaches 1e-8 as with BiCGSTAB, and its result is
    finite at every pass (a system whose inner solve broke down keeps the x it had)."""
    A, z = load_golden(name)
    with dev(precond="cpr", krylov="gmres", restart=30, precision="mixed_f32") as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve_refined(z["b"], tol=1e-8, max_outer=6, inner_it=120)
    assert np.all(np.isfinite(x))
    assert res.converged and true_res(A, x, z["b"]) <= 2e-8


def test_refined_solve_batch_stops_converged_systems():
    """In a batch, a system within the tolerance gets no further correction: its result is the one it has alone."""
    mats, bs, singles = [], [], []
    for name in ["waterflood_sys0.npz", "synth_small.npz", "waterflood_sys2.npz"]:
        A, z = load_golden(name)
        mats.append(A)
        bs.append(z["b"])
        with dev(precond="cpr", precision="mixed_f32") as d:
            d.set_matrix(A)
            d.setup()
            singles.append(d.solve_refined(z["b"], tol=1e-9)[0])
    with dev(precond="cpr", precision="mixed_f32") as d:
        d.set_batch(mats)
        d.setup()
        xb, rb = d.solve_refined(np.concatenate(bs), tol=1e-9)
        its, rr, tr = d.batch_results()
    assert rb.converged and np.all(tr <= 1e-9)
    off = 0
    for A, xs in zip(mats, singles):
        assert np.array_equal(xb[off:off + A.n * 3], xs)
        off += A.n * 3


# ---------------------------------------------------------------- launch shapes (autotuner candidates)
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_f32"])
def test_launch_shapes_give_identical_results(precision):
    """Every launch shape the autotuner chooses among computes the same values: the split CPR's V-cycle as one launch
    per pass, as the phases of one cooperative kernel, or with its coarse levels one thread block per system, and its
    BILU0 stage with 128, 256 or 512 threads per system -- preconditioner output, solution and iterations bit for bit, on
    a batch with well cliques."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=6, nx=24, ny=24, nz=6, sigma=1.5)
    b = np.concatenate([s.b for s in systems])
    out = []
    for form, thr in ((2, 256), (1, 256), (3, 256), (3, 512), (2, 512), (3, 128), (1, 128)):
        with dev(precond="cpr", precision=precision, sweep="split", autotune=False, vcycle_form=form, cpr2_threads=thr) as d:
            d.set_batch([s.A for s in systems])
            d.setup()
            assert f"vcycle_form={form} cpr2_threads={thr}" in d.tuning()
            z = d.precond_apply(b)
            x, res = d.solve(b, tol=1e-6, maxit=300)
            its, _, _ = d.batch_results()
        out.append((z, x, its))
        assert res.converged
    for z, x, its in out[1:]:
        assert np.array_equal(z, out[0][0]) and np.array_equal(x, out[0][1]) and np.array_equal(its, out[0][2])


def test_autotuner_reports_its_choice():
    """At the first set-up of a pattern the autotuner times the candidates and keeps the fastest; a second handle on
    the same pattern reuses the choice (cached per pattern)."""
    from ressim_gb300 import synth
    systems = synth.ensemble(n_real=4, nx=20, ny=20, nz=5, sigma=1.5)
    with dev(precond="cpr", precision="mixed_f32", sweep="split") as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        t1 = d.tuning()
    assert "source=tuned" in t1 and "form3/256" in t1 and "form2/512" in t1 and "form3/128" in t1
    with dev(precond="cpr", precision="mixed_f32", sweep="split") as d:
        d.set_batch([s.A for s in systems])
        d.setup()
        assert d.tuning() == t1

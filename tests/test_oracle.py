"""The C restatement (oracle/) against the reference engine's own golden vectors (tests/golden/).

Every comparison is exact (bitwise) where the reference computes serially in the same order, which is the case
for every entry point at one thread; the oracle is built with -ffp-contract=off like the x86 reference build.
"""
import os

import numpy as np
import pytest

from conftest import ALL_GOLDEN, GOLDEN, GOLDEN_SYSTEMS, load_golden


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_spmv(oracle, name):
    A, z = load_golden(name)
    assert np.array_equal(oracle.spmv(A, z["x_seed"]), z["y_spmv"])


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_bilu0_factor_and_apply(oracle, name):
    A, z = load_golden(name)
    lu, nreg = oracle.bilu0_factor(A)
    if "lu" in z.files:
        assert np.array_equal(lu, z["lu"])
        assert nreg == int(z["nreg"])
    zz = oracle.bilu0_apply(A, lu, z["b"])
    assert np.array_equal(zz, z["z_bilu0"])
    # the reference's level-ordered contiguous variant is the same ILU(0) up to summation order
    assert rel(zz, z["z_bilu0_contig"]) < 1e-10


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_bilu0f_apply(oracle, name):
    A, z = load_golden(name)
    lu, _ = oracle.bilu0_factor(A)
    zf = oracle.bilu0_apply_ff(A, lu.astype(np.float32), z["b"])
    assert np.array_equal(zf, z["z_bilu0f"])


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_cpr_weights_amg_apply(oracle, name):
    A, z = load_golden(name)
    w, info, levels = oracle.cpr_info(A)
    assert np.array_equal(w, z["cpr_w"])
    assert [r for r, _ in info] == list(z["amg_rows"])
    assert [q for _, q in info] == list(z["amg_nnz"])
    if "amg_agg0" in z.files:
        assert np.array_equal(levels[0][3], z["amg_agg0"])
        assert np.array_equal(levels[1][0], z["amg_A1_rp"]) and np.array_equal(levels[1][1], z["amg_A1_ci"])
        assert np.array_equal(levels[1][2], z["amg_A1_v"])
    assert np.array_equal(oracle.prec_apply(A, z["b"], prec=1), z["z_cpr"])
    if "acc" in z.files:
        assert np.array_equal(oracle.cpr_info(A, acc=z["acc"])[0], z["cpr_w_acc"])
        assert np.array_equal(oracle.prec_apply(A, z["b"], prec=1, acc=z["acc"]), z["z_cpr_acc"])


CASES = {
    "bicg_bilu0": dict(prec=0, method=0, tol=1e-6, maxit=120),
    "bicg_bilu0_tight": dict(prec=0, method=0, tol=1e-10, maxit=1000),
    "gmres_bilu0": dict(prec=0, method=1, restart=30, tol=1e-6, maxit=300),
    "bicg_cpr": dict(prec=1, method=0, tol=1e-6, maxit=120),
    "gmres_cpr": dict(prec=1, method=1, restart=30, tol=1e-6, maxit=300),
    "bicg_cpr_tight": dict(prec=1, method=0, tol=1e-10, maxit=500),
    "gmres_bilu0_tight": dict(prec=0, method=1, restart=30, tol=1e-12, maxit=1000),
    "gmres_cpr_tight": dict(prec=1, method=1, restart=30, tol=1e-12, maxit=500),
    "gmres60_bilu0_tight": dict(prec=0, method=1, restart=60, tol=1e-12, maxit=1000),
    "gmres60_cpr_tight": dict(prec=1, method=1, restart=60, tol=1e-12, maxit=500),
}


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_multicolour_bilu0(oracle, name):
    """MCBILU0 (engine/src/bsr.cpp:599-730): colouring, P A P^T, its block ILU(0) and sweeps, bit for bit."""
    A, z = load_golden(name)
    assert np.array_equal(oracle.mcbilu0_apply(A, z["b"]), z["z_mcbilu0"])


@pytest.mark.parametrize("name", ALL_GOLDEN)
def test_device_cpr_amg(oracle, name):
    """GPU-shaped float CPR-AMG (DeviceCprAmg::build / apply, engine/src/bsr.cpp:1217-1371): the restatement in
    float, bit for bit the reference's output for the right-hand side rounded to float."""
    A, z = load_golden(name)
    assert np.array_equal(oracle.devcpr_apply(A, z["b"].astype(np.float32)), z["z_devcpr"])


@pytest.mark.parametrize("name", ALL_GOLDEN)
@pytest.mark.parametrize("case", sorted(CASES))
def test_krylov(oracle, name, case):
    A, z = load_golden(name)
    x, conv, its, rr, _, _ = oracle.solve(A, z["b"], **CASES[case])
    assert its == int(z["its_" + case])
    assert conv == bool(z["conv_" + case])
    assert rr == float(z["rr_" + case])
    assert np.array_equal(x, z["x_" + case])


@pytest.mark.parametrize("name", GOLDEN_SYSTEMS)
def test_float_refinement(oracle, name):
    A, z = load_golden(name)
    x, conv, its, rr = oracle.refine_float(A, z["b"], tol=1e-8, max_outer=6, inner_it=120)
    assert its == int(z["its_refine"]) and conv == bool(z["conv_refine"])
    assert np.array_equal(x, z["x_refine"])


@pytest.mark.parametrize("name", ["waterflood_dump.npz", "synth_small.npz"])
def test_wellschur(oracle, name):
    A, z = load_golden(name)
    J = (z["J_rowPtr"], z["J_col"], z["J_val"])
    na, nv, nw = int(z["na"]), int(z["nv"]), int(z["nw"])
    (rp, ci, v), bc = oracle.wellschur(J, na, nv, nw, z["J_rhs"])
    if "S_val" in z.files:
        assert np.array_equal(rp, z["S_rowPtr"]) and np.array_equal(ci, z["S_col"]) and np.array_equal(v, z["S_val"])
        assert np.array_equal(bc, z["S_bc"])
    else:
        assert np.array_equal(rp, A.rowPtr) and np.array_equal(ci, A.col) and np.array_equal(v, A.val)
        assert np.array_equal(bc, z["b"])
    if "x_full" in z.files:
        x = oracle.wellschur_recover(J, na, nv, nw, z["J_rhs"], z["x_bicg_bilu0_tight"])
        assert np.array_equal(x, z["x_full"])


def test_level_sets_are_topological(oracle):
    A, z = load_golden("waterflood_sys0.npz")
    ordv, start = oracle.level_sets(A, forward=True)
    pos = np.empty(A.n, dtype=np.int64)
    pos[ordv] = np.arange(A.n)
    rows = np.repeat(np.arange(A.n), np.diff(A.rowPtr))
    low = A.col < rows
    assert np.all(pos[A.col[low]] < pos[rows[low]])
    assert start[-1] == A.n


def test_reference_shim_agrees_on_fresh_inputs(oracle):
    """Where the reference engine is built (oracle/_ref), the oracle is re-checked on a generated system."""
    from oracle import RefShim
    if not RefShim.available():
        pytest.skip("reference engine not built on this host")
    from ressim_gb300 import synth
    R = RefShim()
    s = synth.make_system(9, 7, 4, sigma=2.0, seed=5, wells="corners+center")
    for prec in (0, 1):
        x1, c1, i1, r1, _, _ = oracle.solve(s.A, s.b, prec=prec, method=0, tol=1e-8, maxit=300)
        x2, c2, i2, r2 = R.solve(s.A, s.b, prec=prec, method=0, tol=1e-8, maxit=300)
        assert i1 == i2 and np.array_equal(x1, x2)


@pytest.mark.parametrize("name", ["waterflood_sys0.npz", "singular_pivots.npz", "synth_small.npz"])
def test_fp32_factorisation_restatement(name, oracle):
    """All-FP32 elimination with FP64 pivot inversions: within float rounding of the reference's FP64 factors,
    with the same regularised pivot blocks."""
    A, z = load_golden(name)
    f32, nreg = oracle.bilu0_factor_f32(A)
    assert nreg == int(z["nreg"])
    if nreg:
        return          # a shifted singular pivot block (1e-8 relative) amplifies float rounding by its condition number
    lu = z["lu"]
    scale = np.abs(lu).reshape(-1, 9).max(axis=1).repeat(9)
    assert np.max(np.abs(f32.astype(np.float64) - lu) / np.maximum(scale, 1e-300)) < 1e-4


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_assembly_restatement_matches_reference(k):
    """The C restatement of the reference's black-oil assembly (oracle/rsg_oracle_asm.c) against the reference's own
    J and R (tests/golden/waterflood_asm.npz: three Newton iterations of the waterflood and a perturbed state with
    free-gas and no-oil cells), with the reference's well terms added in order: bit for bit."""
    from oracle import Oracle
    z = dict(np.load(os.path.join(GOLDEN, "waterflood_asm.npz")))
    o = Oracle()
    J, R = o.bo_assemble(z, z[f"s{k}_p"], z[f"s{k}_sw"], z[f"s{k}_x"], z[f"s{k}_hasGas"], z[f"s{k}_accOld"], float(z[f"s{k}_dt"][0]),
                         add_pos=z[f"s{k}_add_pos"], add_val=z[f"s{k}_add_val"], radd_pos=z[f"s{k}_radd_pos"],
                         radd_val=z[f"s{k}_radd_val"])
    assert np.array_equal(J, z[f"s{k}_J_full"]), np.flatnonzero(J != z[f"s{k}_J_full"])[:10]
    assert np.array_equal(R, z[f"s{k}_R_full"]), np.flatnonzero(R != z[f"s{k}_R_full"])[:10]

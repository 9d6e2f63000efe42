"""The block-size-generic path (blocks other than 3 x 3: the compositional and thermal simulators' systems) against the
reference.

Inputs: Newton systems the reference's own compositional (examples/COMP.DATA, nb = 8) and thermal
(examples/STEAMFLOOD.DATA, nb = 5) simulators hand to their block solver, with the reference's outputs
(tests/golden/make_golden_nb.py), and seeded synthetic systems with nb = 2, 4, 6, 8 (ressim_gb300.synth.make_block_system)
checked against the oracle, which the CPU tests pin to the reference.

Bars: SpMV, BILU0 factors and both sweeps bit for bit (the reference's operation order, separately rounded);
BlockCPR::apply within 1e-10 (only the back substitution of the coarsest dense LU runs in another order); solutions of
BiCGSTAB-BILU0 and GMRES(m)-CPR at tolerance 1e-10 within 1e-8 of the reference's solution of the same method.
"""
import os

import numpy as np
import pytest

from conftest import load_golden

GOLDEN = ["comp_sys.npz", "thermal_sys.npz"]
SYNTH = [(2, 16, 12, 5), (4, 16, 12, 5), (6, 12, 10, 6), (8, 10, 8, 4)]


def synth_case(nb, nx, ny, nz):
    from ressim_gb300 import synth
    return synth.make_block_system(nx, ny, nz, nb, seed=nb)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ---------------------------------------------------------------- CPU: the oracle pinned to the reference
@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_reference_golden(name):
    from oracle import Oracle
    A, z = load_golden(name)
    o = Oracle()
    assert A.nb == {"comp_sys.npz": 8, "thermal_sys.npz": 5}[name]
    assert np.array_equal(o.spmv(A, z["x_seed"]), z["y_spmv"])
    lu, nreg = o.bilu0_factor(A)
    assert np.array_equal(lu, z["lu"]) and nreg == int(z["nreg"])
    assert np.array_equal(o.bilu0_apply(A, lu, z["b"]), z["z_bilu0"])
    assert np.array_equal(o.prec_apply(A, z["b"], prec=1), z["z_cpr"])
    m = int(z["restart"])
    x, conv, its, rr, _, _ = o.solve(A, z["b"], prec=1, method=1, restart=m, tol=1e-10, maxit=1000)
    assert conv and its == int(z["its_gmres_cpr"]) and rel(x, z["x_gmres_cpr"]) <= 1e-12


@pytest.mark.parametrize("nb,nx,ny,nz", SYNTH)
def test_oracle_matches_reference_synthetic(nb, nx, ny, nz):
    from oracle import Oracle, RefShim
    if not RefShim.available():
        pytest.skip("reference build absent (oracle/_ref)")
    R, o = RefShim(), Oracle()
    s = synth_case(nb, nx, ny, nz)
    A = s.A
    lu_r, nreg_r = R.bilu0_factor(A)
    lu_o, nreg_o = o.bilu0_factor(A)
    assert np.array_equal(lu_r, lu_o) and nreg_r == nreg_o
    assert np.array_equal(R.bilu0_apply(A, s.b), o.bilu0_apply(A, lu_o, s.b))
    assert np.array_equal(R.prec_apply(A, s.b, prec=1, acc=s.acc), o.prec_apply(A, s.b, prec=1, acc=s.acc))
    assert np.array_equal(R.prec_apply(A, s.b, prec=1, acc=None), o.prec_apply(A, s.b, prec=1))


def test_generator_systems_are_solvable():
    """The synthetic systems are well posed for both preconditioners (the reference algorithm, through the oracle)."""
    from oracle import Oracle
    o = Oracle()
    for nb, nx, ny, nz in SYNTH:
        s = synth_case(nb, nx, ny, nz)
        for prec, method in ((0, 0), (1, 1)):
            x, conv, its, rr, _, _ = o.solve(s.A, s.b, prec=prec, method=method, restart=60, tol=1e-10, maxit=600,
                                             acc=s.acc if prec else None)
            assert conv, (nb, prec)
            assert rel(x, s.x_true) < 1e-5, (nb, prec)


# ---------------------------------------------------------------- GPU: the device path against the reference / oracle
def gpu_cases():
    out = []
    for name in GOLDEN:
        A, z = load_golden(name)
        out.append((name, A, z["b"], None))
    for nb, nx, ny, nz in SYNTH:
        s = synth_case(nb, nx, ny, nz)
        out.append((f"synth_nb{nb}", s.A, s.b, s.acc))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("idx", range(len(GOLDEN) + len(SYNTH)))
def test_generic_kernels_bitwise(idx):
    from oracle import Oracle
    from ressim_gb300.solver import DeviceSolver
    name, A, b, acc = gpu_cases()[idx]
    o = Oracle()
    lu_o, _ = o.bilu0_factor(A)
    with DeviceSolver(precond="bilu0", precision="fp64") as d:
        d.set_matrix(A)
        x = np.random.default_rng(5).standard_normal(A.n * A.nb)
        assert np.array_equal(d.spmv(x), o.spmv(A, x)), name
        d.setup()
        assert np.array_equal(d.factors(A.nnzb), lu_o), name
        assert np.array_equal(d.precond_apply(b), o.bilu0_apply(A, lu_o, b)), name
        assert d.tuning().startswith("block-size-generic")


@pytest.mark.gpu
@pytest.mark.parametrize("idx", range(len(GOLDEN) + len(SYNTH)))
@pytest.mark.parametrize("with_acc", [False, True], ids=["quasi-impes", "true-impes"])
def test_generic_cpr_apply(idx, with_acc):
    from oracle import Oracle
    from ressim_gb300.solver import DeviceSolver
    name, A, b, acc = gpu_cases()[idx]
    if with_acc and acc is None:
        pytest.skip("captured systems carry no accumulation blocks (the solver hook passes none)")
    o = Oracle()
    ref = o.prec_apply(A, b, prec=1, acc=acc if with_acc else None)
    with DeviceSolver(precond="cpr", precision="fp64") as d:
        d.set_matrix(A)
        d.setup(acc if with_acc else None)
        z = d.precond_apply(b)
        lv = d.amg_level_sizes()
    assert lv is not None and lv[0][0] == A.n
    assert rel(z, ref) <= 1e-10, (name, rel(z, ref))


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN)
def test_generic_solves_match_reference(name):
    """BiCGSTAB-BILU0 and GMRES-CPR with the caller's restart, at 1e-10: the reference's own solutions within 1e-8;
    and the caller's own solve (its tolerance and iteration cap) converged to the tolerance in true residual."""
    from ressim_gb300.solver import DeviceSolver
    A, z = load_golden(name)
    b = z["b"]
    m = int(z["restart"])
    with DeviceSolver(precond="bilu0", krylov="bicgstab", precision="fp64") as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(b, tol=1e-10, maxit=1000)
    assert res.converged and rel(x, z["x_bicg_bilu0"]) <= 1e-8, rel(x, z["x_bicg_bilu0"])
    with DeviceSolver(precond="cpr", krylov="gmres", restart=m, precision="fp64") as d:
        d.set_matrix(A)
        d.setup()
        x, res = d.solve(b, tol=1e-10, maxit=1000)
        assert res.converged and abs(res.iterations - int(z["its_gmres_cpr"])) <= 1
        assert rel(x, z["x_gmres_cpr"]) <= 1e-8, rel(x, z["x_gmres_cpr"])
        tol, cap = float(z["engine_tol"]), int(z["engine_maxit"])
        x, res = d.solve(b, tol=tol, maxit=cap)
        assert res.converged and res.trueRelResidual <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("nb", [4, 6])
def test_generic_large_system_level_launches(nb):
    """A system whose levels are too wide for the one-block sweeps (one launch per level; factorisation one launch
    per level): same factors and sweeps bit for bit, GMRES-CPR at 1e-10 and BiCGSTAB-BILU0 at 1e-12 within 1e-8 of
    the oracle's solutions. (BiCGSTAB-BILU0 takes ~450 iterations on the nb = 6 system: at 1e-10 the oracle's own
    solutions with 1 and 8 threads differ by 2e-8, at 1e-12 by 3e-9; with several threads they also vary from run to
    run, so the oracle runs on one.)"""
    from oracle import Oracle
    from ressim_gb300 import synth
    from ressim_gb300.solver import DeviceSolver
    s = synth.make_block_system(48, 40, 8, nb, seed=11)
    A = s.A
    o = Oracle()
    o.set_threads(1)          # one thread: the oracle's OpenMP reductions combine thread partials in no fixed order
    lu_o, _ = o.bilu0_factor(A)
    with DeviceSolver(precond="bilu0", precision="fp64") as d:
        d.set_matrix(A)
        d.setup()
        assert np.array_equal(d.factors(A.nnzb), lu_o)
        assert np.array_equal(d.precond_apply(s.b), o.bilu0_apply(A, lu_o, s.b))
        x, res = d.solve(s.b, tol=1e-12, maxit=1000)
    xo, conv, _, _, _, _ = o.solve(A, s.b, prec=0, method=0, tol=1e-12, maxit=1000)
    assert res.converged and conv and rel(x, xo) <= 1e-8, rel(x, xo)
    with DeviceSolver(precond="cpr", krylov="gmres", restart=60, precision="fp64") as d:
        d.set_matrix(A)
        d.setup(s.acc)
        assert rel(d.precond_apply(s.b), o.prec_apply(A, s.b, prec=1, acc=s.acc)) <= 1e-10
        x, res = d.solve(s.b, tol=1e-10, maxit=1000)
    xo, conv, _, _, _, _ = o.solve(A, s.b, prec=1, method=1, restart=60, tol=1e-10, maxit=1000, acc=s.acc)
    assert res.converged and conv and rel(x, xo) <= 1e-8


@pytest.mark.gpu
def test_generic_pattern_reuse_and_errors():
    """New values on the same pattern refactor in place (same results as a fresh handle); the generic path rejects
    batches, the precision forms and block sizes above 16 with RSG_EINVAL."""
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import BSR
    from ressim_gb300.solver import DeviceSolver
    s1 = synth_case(6, 12, 10, 6)
    A1 = s1.A
    A2 = BSR(A1.n, A1.nb, A1.rowPtr, A1.col, A1.val * 1.5)
    with DeviceSolver(precond="cpr", krylov="gmres", restart=60) as d, DeviceSolver(precond="cpr", krylov="gmres", restart=60) as f:
        d.set_matrix(A1)
        d.setup()
        d.solve(s1.b, tol=1e-10, maxit=500)
        d.set_matrix(A2)
        d.setup()
        x, _ = d.solve(s1.b, tol=1e-10, maxit=500)
        f.set_matrix(A2)
        f.setup()
        y, _ = f.solve(s1.b, tol=1e-10, maxit=500)
    assert np.array_equal(x, y)
    with DeviceSolver(precond="cpr", precision="mixed_f32") as d:
        with pytest.raises(_lib.RsgError) as e:
            d.set_matrix(A1)
        assert e.value.code == _lib.RSG_EINVAL
    with DeviceSolver(precond="bilu0") as d:
        with pytest.raises(_lib.RsgError) as e:
            d.set_batch([A1, A1])
        assert e.value.code == _lib.RSG_EINVAL
        big = BSR(1, 17, np.array([0, 1], dtype=np.int32), np.array([0], dtype=np.int32), np.eye(17).reshape(-1))
        with pytest.raises(_lib.RsgError) as e:
            d.set_matrix(big)
        assert e.value.code == _lib.RSG_EINVAL

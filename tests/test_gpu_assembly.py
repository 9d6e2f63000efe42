"""Black-oil Jacobian assembly on the device (rsg_bo_*) against the reference engine's own assembly.

The golden file (tests/golden/waterflood_asm.npz, made by make_golden_asm.py from the reference simulator) holds, for
four states of the 20x20x4 waterflood -- three Newton iterations of the run and one perturbed state with free-gas
and no-oil cells -- the state, the engine's full Jacobian and residual after Simulator::assemble (wells included, rows
scaled by dt / PV) and the engine's well terms alone. The device assembles the reservoir terms, adds the well terms
in the engine's order and scales: J and R must be the engine's bit for bit. The assembled Jacobian then goes through
the device well Schur complement and the solver without leaving the device.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def fixture():
    return dict(np.load(os.path.join(GOLDEN, "waterflood_asm.npz"), allow_pickle=False))


def dev_state(torch, z, k, copies=1):
    d = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.tile(a, copies))).to(d)  # noqa: E731
    return (t(z[f"s{k}_p"]), t(z[f"s{k}_sw"]), t(z[f"s{k}_x"]), t(z[f"s{k}_hasGas"].astype(np.uint8)), t(z[f"s{k}_accOld"]))


def assemble(torch, asm, z, k, with_wells=True, copies=1):
    d = torch.device("cuda:0")
    p, sw, x, st, acc = dev_state(torch, z, k, copies)
    J = torch.full((asm.nnz,), float("nan"), dtype=torch.float64, device=d)
    R = torch.full((asm.nrows,), float("nan"), dtype=torch.float64, device=d)
    kw = {}
    if with_wells:
        kw = dict(add_pos=z[f"s{k}_add_pos"], add_val=z[f"s{k}_add_val"], radd_pos=z[f"s{k}_radd_pos"], radd_val=z[f"s{k}_radd_val"])
    asm.assemble_device(p.data_ptr(), sw.data_ptr(), x.data_ptr(), st.data_ptr(), acc.data_ptr(), float(z[f"s{k}_dt"][0]),
                        J.data_ptr(), R.data_ptr(), **kw)
    torch.cuda.synchronize()
    return J.cpu().numpy(), R.cpu().numpy()


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_assembly_matches_engine_bitwise(k):
    """J and R at each captured state, wells added in the engine's order: the engine's, bit for bit."""
    torch = pytest.importorskip("torch")
    from ressim_gb300.assembly import BlackOilAssembler
    z = fixture()
    with BlackOilAssembler(z) as asm:
        J, R = assemble(torch, asm, z, k)
        # the same assembler again (the well-term buffer reused): the same result
        J2, R2 = assemble(torch, asm, z, k)
    assert np.array_equal(J, z[f"s{k}_J_full"]), np.flatnonzero(J != z[f"s{k}_J_full"])[:10]
    assert np.array_equal(R, z[f"s{k}_R_full"]), np.flatnonzero(R != z[f"s{k}_R_full"])[:10]
    assert np.array_equal(J2, J) and np.array_equal(R2, R)


def test_calls_on_different_streams_are_ordered():
    """Four assemblies issued back to back on two streams without a synchronisation between them (each call's scratch
    is the assembler's, so each waits for the previous call): every J and R is the engine's, bit for bit."""
    torch = pytest.importorskip("torch")
    from ressim_gb300.assembly import BlackOilAssembler
    z = fixture()
    d = torch.device("cuda:0")
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    with BlackOilAssembler(z) as asm:
        states = [dev_state(torch, z, k) for k in range(4)]
        outs = [(torch.full((asm.nnz,), float("nan"), dtype=torch.float64, device=d),
                 torch.full((asm.nrows,), float("nan"), dtype=torch.float64, device=d)) for _ in range(4)]
        torch.cuda.synchronize()
        for k in range(4):
            p, sw, x, st, acc = states[k]
            J, R = outs[k]
            asm.assemble_device(p.data_ptr(), sw.data_ptr(), x.data_ptr(), st.data_ptr(), acc.data_ptr(), float(z[f"s{k}_dt"][0]),
                                J.data_ptr(), R.data_ptr(), add_pos=z[f"s{k}_add_pos"], add_val=z[f"s{k}_add_val"],
                                radd_pos=z[f"s{k}_radd_pos"], radd_val=z[f"s{k}_radd_val"], stream=streams[k % 2].cuda_stream)
        torch.cuda.synchronize()
        for k in range(4):
            assert np.array_equal(outs[k][0].cpu().numpy(), z[f"s{k}_J_full"])
            assert np.array_equal(outs[k][1].cpu().numpy(), z[f"s{k}_R_full"])


def test_reservoir_terms_alone_match_engine():
    """Without well terms the cell rows are the engine's reservoir terms alone (its assembly with every well shut)."""
    torch = pytest.importorskip("torch")
    from ressim_gb300.assembly import BlackOilAssembler
    z = fixture()
    with BlackOilAssembler(z) as asm:
        J, R = assemble(torch, asm, z, 1, with_wells=False)
        nc = asm.na * asm.nv
        cell = slice(0, int(asm.rowPtr[nc]))
    assert np.array_equal(J[cell], z["s1_J_cell"][cell])
    assert np.array_equal(R[:nc], z["s1_R_cell"][:nc])


def replicate_without_wells(z, copies):
    """The grid `copies` times over as disconnected copies, without wells (each cell row holds its blocks only), and
    the positions of those blocks in the engine's pattern."""
    na, nv = int(z["na"][0]), int(z["nv"][0])
    nc = na * nv
    rp, ci = z["J_rowPtr"], z["J_col"]
    nblk = np.diff(z["adjStart"]) + 1
    keep = np.concatenate([np.arange(rp[r], rp[r] + nblk[r // nv] * nv) for r in range(nc)])
    row_len = nblk.repeat(nv) * nv
    nconn = z["conn_trans"].size
    big = dict(z)
    big["na"], big["nw"] = np.array([na * copies]), np.array([0])
    big["adjStart"] = np.r_[0, np.cumsum(np.tile(np.diff(z["adjStart"]), copies))].astype(np.int32)
    big["adjNbr"] = np.concatenate([z["adjNbr"] + c * na for c in range(copies)]).astype(np.int32)
    big["adjConn"] = np.concatenate([z["adjConn"] + c * nconn for c in range(copies)]).astype(np.int32)
    big["conn_a"] = np.concatenate([z["conn_a"] + c * na for c in range(copies)]).astype(np.int32)
    big["conn_b"] = np.concatenate([z["conn_b"] + c * na for c in range(copies)]).astype(np.int32)
    for key in ("conn_trans", "conn_dDepth", "poreVolRef"):
        big[key] = np.tile(z[key], copies)
    big["J_rowPtr"] = np.r_[0, np.cumsum(np.tile(row_len, copies))].astype(np.int32)
    big["J_col"] = np.concatenate([ci[keep] + c * nc for c in range(copies)]).astype(np.int32)
    return big, keep


def test_assembly_many_copies_bitwise():
    """400 disconnected copies of the grid (640,000 cells, 5,000 thread blocks per kernel) at the same state: every
    copy's rows are the engine's reservoir terms, bit for bit (the kernels do not depend on the grid's size or on
    which block a cell falls in)."""
    torch = pytest.importorskip("torch")
    from ressim_gb300.assembly import BlackOilAssembler
    z = fixture()
    na, nv = int(z["na"][0]), int(z["nv"][0])
    one, keep = replicate_without_wells(z, 1)
    big, _ = replicate_without_wells(z, 400)
    with BlackOilAssembler(one) as asm:
        J1, R1 = assemble(torch, asm, z, 1, with_wells=False)
    assert np.array_equal(J1, z["s1_J_cell"][keep]) and np.array_equal(R1, z["s1_R_cell"][:na * nv])
    with BlackOilAssembler(big) as asm:
        J, R = assemble(torch, asm, z, 1, with_wells=False, copies=400)
    assert np.array_equal(J.reshape(400, -1), np.broadcast_to(J1, (400, J1.size)))
    assert np.array_equal(R.reshape(400, -1), np.broadcast_to(R1, (400, R1.size)))


def test_assembled_jacobian_solves_on_device():
    """The device-assembled J goes to the device well Schur complement and the CPR-BiCGSTAB solve without leaving the
    device: the same solution, bit for bit, as the engine's J uploaded from the host."""
    torch = pytest.importorskip("torch")
    from ressim_gb300 import _lib
    from ressim_gb300.assembly import BlackOilAssembler
    from ressim_gb300.bsr import ScalarCSR
    from ressim_gb300.solver import DeviceSolver
    z = fixture()
    k = 2
    dv = torch.device("cuda:0")
    with BlackOilAssembler(z) as asm, DeviceSolver(precond="cpr") as a, DeviceSolver(precond="cpr") as b:
        p, sw, x, st, acc = dev_state(torch, z, k)
        J = torch.empty(asm.nnz, dtype=torch.float64, device=dv)
        R = torch.empty(asm.nrows, dtype=torch.float64, device=dv)
        asm.assemble_device(p.data_ptr(), sw.data_ptr(), x.data_ptr(), st.data_ptr(), acc.data_ptr(), float(z[f"s{k}_dt"][0]),
                            J.data_ptr(), R.data_ptr(), add_pos=z[f"s{k}_add_pos"], add_val=z[f"s{k}_add_val"],
                            radd_pos=z[f"s{k}_radd_pos"], radd_val=z[f"s{k}_radd_val"])
        torch.cuda.synchronize()
        rhs = -R
        xd = torch.zeros(asm.nrows, dtype=torch.float64, device=dv)
        torch.cuda.synchronize()
        rp = np.ascontiguousarray(z["J_rowPtr"], dtype=np.int32)
        ci = np.ascontiguousarray(z["J_col"], dtype=np.int32)
        _lib.check(a.L.rsg_set_jacobian_device(a.h, asm.nrows, _lib.ptr(rp), _lib.ptr(ci), C.c_void_p(J.data_ptr()), asm.na, asm.nv,
                                               asm.nw))
        a.setup()
        its, rr = C.c_int(0), C.c_double(0)
        rc = a.L.rsg_solve_jacobian_device(a.h, C.c_void_p(rhs.data_ptr()), C.c_void_p(xd.data_ptr()), 1e-8, 200, C.byref(its),
                                           C.byref(rr))
        assert rc == _lib.RSG_OK, _lib.last_error()
        x_dev = xd.cpu().numpy()
        b.set_jacobian(ScalarCSR(rp, ci, z[f"s{k}_J_full"]), asm.na, asm.nv, asm.nw)
        b.setup()
        x_host, res = b.solve_jacobian(-z[f"s{k}_R_full"], tol=1e-8, maxit=200)
        assert res.converged
    assert np.array_equal(x_dev, x_host)


def test_whole_run_assembly_matches_engine_every_newton_iteration():
    """The reference simulator's whole 20x20x4 waterflood (6 report steps of 30 days), with oracle/ref_asm_run in the
    engine's solver hook: at every Newton iteration the device assembles J and R from the simulator's state (with the
    engine's well terms at that state) and both are compared with the engine's own assembly of that iteration, bit
    for bit. The states evolve as in the stock run (the engine solves every system itself): free gas appears, the
    wells' controls switch, time steps grow."""
    import json
    import subprocess
    from conftest import ROOT
    staged = os.path.join(ROOT, "oracle", "_ref", "src", "engine", "src", "simulator.cpp")
    if not os.path.exists(staged):
        pytest.skip("reference engine sources not staged (make -f oracle/Makefile.ref stage REF=...)")
    jobs = str(max(2, os.cpu_count() or 2))
    r = subprocess.run(["make", "-f", "oracle/Makefile.ref", "-j" + jobs, "oracle/_ref/ref_asm_run"], cwd=ROOT, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_asm_run"), "6", "30"], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert r.returncode == 0 and not out["error"], out
    assert out["compared"] == out["hook_calls"] and out["compared"] >= 30, out
    assert out["mismatching_J"] == 0 and out["mismatching_R"] == 0, out


def test_well_terms_are_added_in_the_callers_order():
    """Several terms at one position are added in list order (the engine's well loop adds a connection's terms one
    after the other): on a well row, which starts from zero and is not scaled, J = (0 + v) + w exactly; positions out
    of range are refused with RSG_EINVAL."""
    torch = pytest.importorskip("torch")
    from ressim_gb300 import _lib
    from ressim_gb300.assembly import BlackOilAssembler
    z = fixture()
    k = 2
    na, nv, nw = int(z["na"][0]), int(z["nv"][0]), int(z["nw"][0])
    rp = z["J_rowPtr"]
    wrow = na * nv                                   # the first well row
    p0 = int(rp[wrow])
    # 1 + 1e-16 rounds back to 1, 1e-16 + 1e-16 does not: the sum depends on the order of the terms
    big, tiny = 1.0, 1.0e-16
    assert ((0.0 + big) + tiny) + tiny != ((0.0 + tiny) + tiny) + big
    with BlackOilAssembler(z) as asm:
        J1, R1 = asm.assemble(z[f"s{k}_p"], z[f"s{k}_sw"], z[f"s{k}_x"], z[f"s{k}_hasGas"], z[f"s{k}_accOld"], float(z[f"s{k}_dt"][0]),
                              add_pos=np.array([p0, p0, p0 + 1, p0]), add_val=np.array([big, tiny, -2.5, tiny]),
                              radd_pos=np.array([wrow, wrow, wrow]), radd_val=np.array([tiny, tiny, big]))
        assert J1[p0] == ((0.0 + big) + tiny) + tiny and J1[p0 + 1] == -2.5
        assert R1[wrow] == ((0.0 + tiny) + tiny) + big
        assert np.all(J1[p0 + 2:rp[wrow + 1]] == 0.0)
        # the host form equals the device form
        J, R = assemble(torch, asm, z, k)
        J2, R2 = asm.assemble(z[f"s{k}_p"], z[f"s{k}_sw"], z[f"s{k}_x"], z[f"s{k}_hasGas"], z[f"s{k}_accOld"], float(z[f"s{k}_dt"][0]),
                              add_pos=z[f"s{k}_add_pos"], add_val=z[f"s{k}_add_val"], radd_pos=z[f"s{k}_radd_pos"],
                              radd_val=z[f"s{k}_radd_val"])
        assert np.array_equal(J2, J) and np.array_equal(R2, R)
        with pytest.raises(_lib.RsgError) as e:
            asm.assemble(z[f"s{k}_p"], z[f"s{k}_sw"], z[f"s{k}_x"], z[f"s{k}_hasGas"], z[f"s{k}_accOld"], 1.0,
                         add_pos=np.array([int(rp[-1])]), add_val=np.array([1.0]))
        assert e.value.code == _lib.RSG_EINVAL
        with pytest.raises(_lib.RsgError) as e:
            asm.assemble(z[f"s{k}_p"], z[f"s{k}_sw"], z[f"s{k}_x"], z[f"s{k}_hasGas"], z[f"s{k}_accOld"], 0.0)
        assert e.value.code == _lib.RSG_EINVAL


def test_full_size_assembly_matches_oracle():
    """The bench's assembly workload at full size -- the 64 ensemble grids taken as one, 742,384 cells, synthetic
    live-oil / Corey tables and state -- against the C restatement of the reference's assembly (pinned to the
    reference's J and R on CPU, tests/test_oracle.py), with 2,000 seeded addends on cell and well-free rows: bit for
    bit."""
    from oracle import Oracle
    from ressim_gb300 import synth
    from ressim_gb300.assembly import BlackOilAssembler
    z, st = synth.assembly_ensemble(64)
    rng = np.random.default_rng(3)
    nnz, nrows = int(z["J_rowPtr"][-1]), int(z["na"][0]) * 3
    add_pos = rng.integers(0, nnz, 2000)
    add_val = rng.standard_normal(2000)
    radd_pos = rng.integers(0, nrows, 500).astype(np.int32)
    radd_val = rng.standard_normal(500)
    args = (st["p"], st["sw"], st["x"], st["state"], st["acc_old"], 10.0)
    kw = dict(add_pos=add_pos, add_val=add_val, radd_pos=radd_pos, radd_val=radd_val)
    with BlackOilAssembler(z) as asm:
        J, R = asm.assemble(*args, **kw)
    Jo, Ro = Oracle().bo_assemble(z, *args, **kw)
    assert np.array_equal(J, Jo), np.flatnonzero(J != Jo)[:10]
    assert np.array_equal(R, Ro), np.flatnonzero(R != Ro)[:10]

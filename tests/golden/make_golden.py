"""Generate the golden vectors under tests/golden/ from the reference engine itself.

Runs only where the reference tree exists (it builds the reference engine from its own sources with
oracle/Makefile.ref). Steps:

1. ``oracle/_ref/ref_capture`` runs the 20x20x4 three-phase waterflood (generator inputs of the reference,
   ILU(0)-BiCGSTAB block solver) for 6 report steps of 30 days and records every Schur-reduced Newton system;
   three of them (first, middle, last) are kept. A second run (CPR, ``RESSIM_DUMP``) writes the engine's own
   dump of the first full Jacobian with well rows and its accumulation blocks.
2. Two small synthetic systems from ressim_gb300.synth (one with singular pivot blocks) are added.
3. For every system the reference's own classes (through oracle/ref_shim.cpp, single thread) produce:
   BSR::spmv, BILU0 factors and apply, BILU0f apply, BlockCPR weights / AMG hierarchy / apply,
   BiCGSTAB, GMRES(30) and GMRES(60) solves with BILU0 and CPR (at 1e-6, and tight: 1e-10 for BiCGSTAB,
   1e-12 for GMRES), the float-device emulation with double refinement, and (dump) WellSchur reduce / recover.
   For the tight solves, the solution's movement under a change of inner-product summation order alone
   (``sens_<case>``) is recorded: the GPU parity bound is max(1e-8, 10 sens).

    RESSIM_REFERENCE=<reference repository root> python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import RefShim  # noqa: E402
from ressim_gb300 import synth  # noqa: E402
from ressim_gb300.bsr import BSR, read_dump, read_system  # noqa: E402

REF = os.environ.get("RESSIM_REFERENCE", "")


def build_ref():
    if not REF or not os.path.isdir(os.path.join(REF, "engine", "src")):
        sys.exit("set RESSIM_REFERENCE to the reference repository's root (its engine/src is compiled into oracle/_ref)")
    subprocess.run(["make", "-f", "oracle/Makefile.ref", "-j8", "REF=" + REF], cwd=ROOT, check=True, capture_output=True)


def pairwise_bicgstab(A: BSR, M, b, tol, maxit):
    """BiCGSTAB with the oracle's SpMV and preconditioner ``M`` but numpy's pairwise inner products: how far the
    solution moves under a change of summation order alone (the sensitivity the GPU parity bound allows for)."""
    from oracle import Oracle
    o = Oracle()
    n = b.size
    x = np.zeros(n); r = b.copy(); rh = b.copy(); p = np.zeros(n); v = np.zeros(n)
    bn = np.sqrt(np.dot(b, b)); rho = alpha = omega = 1.0
    for it in range(1, maxit + 1):
        rhoN = np.dot(rh, r)
        beta = (rhoN / rho) * (alpha / omega); rho = rhoN
        p = r + beta * (p - omega * v)
        ph = M(p); v = o.spmv(A, ph)
        alpha = rho / np.dot(rh, v)
        s = r - alpha * v
        if np.sqrt(np.dot(s, s)) / bn < tol:
            return x + alpha * ph
        sh = M(s); t = o.spmv(A, sh)
        omega = np.dot(t, s) / np.dot(t, t)
        x = x + alpha * ph + omega * sh; r = s - omega * t
        if np.sqrt(np.dot(r, r)) / bn < tol:
            return x
    return x


def pairwise_gmres(A: BSR, M, b, tol, maxit, m):
    """Flexible GMRES(m) with the oracle's SpMV and preconditioner and numpy's pairwise inner products (same
    recurrence as engine/src/linsolve.cpp:218-273): the solution's sensitivity to the summation order."""
    from oracle import Oracle
    o = Oracle()
    n = b.size
    x = np.zeros(n)
    bn = np.linalg.norm(b)
    total = 0
    while total < maxit:
        r = b - o.spmv(A, x)
        beta = np.linalg.norm(r)
        if beta / bn < tol:
            break
        V = [r / beta]; Z = []
        H = np.zeros((m + 1, m)); cs = np.zeros(m); sn = np.zeros(m); g = np.zeros(m + 1); g[0] = beta
        j = 0
        done = False
        while j < m and total < maxit:
            Z.append(M(V[j])); w = o.spmv(A, Z[j])
            for i in range(j + 1):
                H[i, j] = np.dot(w, V[i]); w = w - H[i, j] * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j] if H[j + 1, j] > 0 else w)
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]; H[i, j] = t
            den = np.hypot(H[j, j], H[j + 1, j])
            cs[j] = H[j, j] / den if den > 0 else 1.0; sn[j] = H[j + 1, j] / den if den > 0 else 0.0
            H[j, j] = den; H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]; g[j] = cs[j] * g[j]
            j += 1; total += 1
            if abs(g[j]) / bn < tol:
                done = True
                break
        y = np.zeros(j)
        for i in range(j - 1, -1, -1):
            y[i] = (g[i] - np.dot(H[i, i + 1:j], y[i + 1:j])) / H[i, i]
        for i in range(j):
            x = x + y[i] * Z[i]
        if done:
            break
    return x


def oracle_preconditioner(A: BSR, prec):
    """The oracle's BILU0 (prec 0) or BlockCPR (prec 1) as a callable r -> z."""
    from oracle import Oracle
    o = Oracle()
    if prec == 0:
        lu, _ = o.bilu0_factor(A)
        return lambda r: o.bilu0_apply(A, lu, r)
    h = o.cpr_handle(A)
    return h.apply


# Krylov cases solved by the reference for every golden system. The tight ones pin the GPU solution within 1e-8
# of the reference's own solution of the same method and preconditioner; GMRES runs to 1e-12 because its
# solution at 1e-10 can still be 1e-8 away from the exact one (measured: 1.4e-8 on waterflood system 2).
# GMRES(60) is the engine's fallback (engine/src/simulator.cpp:3390-3398).
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
# cases whose summation-order sensitivity is recorded (sens_<case>)
SENS_CASES = ("bicg_bilu0", "bicg_bilu0_tight", "bicg_cpr_tight", "gmres_bilu0_tight", "gmres_cpr_tight", "gmres60_bilu0_tight",
              "gmres60_cpr_tight")


def golden_for(R: RefShim, A: BSR, b, acc=None, with_factors=False, label=""):
    N = A.n * A.nb
    rng = np.random.default_rng(1234)
    x = rng.standard_normal(N)
    out = dict(n=A.n, nb=A.nb, rowPtr=A.rowPtr, col=A.col, val=A.val, b=b, x_seed=x)
    if acc is not None:
        out["acc"] = acc
    out["y_spmv"] = R.spmv(A, x)
    if with_factors:
        lu, nreg = R.bilu0_factor(A)
        out["lu"] = lu
        out["nreg"] = nreg
    out["z_bilu0"] = R.bilu0_apply(A, b)
    out["z_bilu0_contig"] = R.bilu0_apply(A, b, level_mode=2)
    out["z_bilu0f"] = R.bilu0f_apply(A, b)
    out["z_cpr"] = R.prec_apply(A, b, prec=1, acc=None)
    out["z_devcpr"] = R.devcpr_apply(A, b.astype(np.float32))   # DeviceCprAmg::apply (float), input rounded to float
    out["z_mcbilu0"] = R.mcbilu0_apply(A, b)                     # MCBILU0::factor / apply
    w, info, levels = R.cpr_info(A, acc=None)
    out["cpr_w"] = w
    out["amg_rows"] = np.array([r for r, _ in info], dtype=np.int32)
    out["amg_nnz"] = np.array([z for _, z in info], dtype=np.int32)
    if len(levels) > 1:
        out["amg_agg0"] = levels[0][3]
        out["amg_A1_rp"], out["amg_A1_ci"], out["amg_A1_v"] = levels[1][0], levels[1][1], levels[1][2]
    if acc is not None:
        out["z_cpr_acc"] = R.prec_apply(A, b, prec=1, acc=acc)
        out["cpr_w_acc"] = R.cpr_info(A, acc=acc)[0]
    for k, c in CASES.items():
        xs, conv, its, rr = R.solve(A, b, **c)
        out["x_" + k] = xs
        out["its_" + k] = its
        out["rr_" + k] = rr
        out["conv_" + k] = int(conv)
        if k in SENS_CASES and conv:
            M = oracle_preconditioner(A, c["prec"])
            if c["method"] == 0:
                xp = pairwise_bicgstab(A, M, b, c["tol"], c["maxit"])
            else:
                xp = pairwise_gmres(A, M, b, c["tol"], c["maxit"], c["restart"])
            out["sens_" + k] = np.linalg.norm(xp - xs) / np.linalg.norm(xs)
        print(f"  {label:10s} {k:18s} conv {conv} its {its:4d} relres {rr:.3e}"
              + (f" sens {float(out['sens_' + k]):.1e}" if "sens_" + k in out else ""))
    xr, conv, its, rr = R.refine_float(A, b, tol=1e-8, max_outer=6, inner_it=120)
    out["x_refine"] = xr
    out["its_refine"] = its
    out["rr_refine"] = rr
    out["conv_refine"] = int(conv)
    return out


def singular_case():
    """Synthetic 8x6x3 system whose pivot blocks at three cells are singular (zero rows / zero block), which
    exercises the BILU0 regularisation (engine/src/bsr.cpp:204-212)."""
    s = synth.make_system(8, 6, 3, sigma=1.0, seed=11, wells="diagonal")
    A = s.A
    d = A.diag()
    blk = A.blocks().copy()
    blk[d[5]] = 0.0                       # isolated zero pivot
    blk[d[17], 2, :] = 0.0                # singular (a zero equation row)
    blk[d[30]] = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [1.0, 0.0, 1.0]])   # rank deficient
    A2 = BSR(A.n, A.nb, A.rowPtr, A.col, blk.reshape(-1))
    return A2, synth.bsr_matvec_host(A2, np.linspace(1.0, 2.0, A.n * A.nb))


def main():
    build_ref()
    R = RefShim()
    with tempfile.TemporaryDirectory() as tmp:
        cap = os.path.join(tmp, "ilu")
        os.makedirs(cap)
        subprocess.run([os.path.join(ROOT, "oracle/_ref/ref_capture"), cap, "0", "6", "30"], check=True, capture_output=True)
        traj = open(os.path.join(cap, "trajectory.txt")).read()
        files = sorted(f for f in os.listdir(cap) if f.startswith("sys_"))
        pick = [files[0], files[len(files) // 2], files[-1]]
        for k, f in enumerate(pick):
            sysm = read_system(os.path.join(cap, f))
            print(f"waterflood system {f}: n {sysm.A.n} nnzb {sysm.A.nnzb}")
            g = golden_for(R, sysm.A, sysm.b, with_factors=(k == 0), label=f"wf{k}")
            g["source"] = np.array(f"20x20x4 waterflood, captured Newton system {f} of {len(files)}")
            np.savez_compressed(os.path.join(HERE, f"waterflood_sys{k}.npz"), **g)
        with open(os.path.join(HERE, "waterflood_trajectory.txt"), "w") as fh:
            fh.write(traj)
        dump = os.path.join(tmp, "dump")
        os.makedirs(dump)
        env = dict(os.environ, RESSIM_DUMP=os.path.join(dump, "j0.bin"))
        subprocess.run([os.path.join(ROOT, "oracle/_ref/ref_capture"), dump, "1", "1", "30"], check=True, capture_output=True, env=env)
        J, rhs, na, nv, nw, acc = read_dump(os.path.join(dump, "j0.bin"))
        print(f"dump: n {J.n} nnz {J.val.size} na {na} nv {nv} nw {nw} acc {acc is not None}")
        S, bc = R.wellschur((J.rowPtr, J.col, J.val), na, nv, nw, rhs)
        A = BSR(na, nv, S[0], S[1], S[2])
        g = golden_for(R, A, bc, acc=acc, label="dump")
        xc = g["x_bicg_bilu0_tight"]
        g.update(J_rowPtr=J.rowPtr, J_col=J.col, J_val=J.val, J_rhs=rhs, na=na, nv=nv, nw=nw,
                 x_full=R.wellschur_recover((J.rowPtr, J.col, J.val), na, nv, nw, rhs, xc))
        g["source"] = np.array("engine RESSIM_DUMP of the first Newton Jacobian (CPR run) with its .acc side file")
        np.savez_compressed(os.path.join(HERE, "waterflood_dump.npz"), **g)
    s = synth.make_system(12, 10, 5, sigma=1.5, seed=3, wells="diagonal", with_full=True)
    g = golden_for(R, s.A, s.b, acc=s.acc, with_factors=True, label="synth")
    S, bc = R.wellschur((s.full.rowPtr, s.full.col, s.full.val), s.na, s.nv, s.nw, s.full_b)
    g.update(J_rowPtr=s.full.rowPtr, J_col=s.full.col, J_val=s.full.val, J_rhs=s.full_b, na=s.na, nv=s.nv, nw=s.nw,
             S_rowPtr=S[0], S_col=S[1], S_val=S[2], S_bc=bc)
    g["source"] = np.array("ressim_gb300.synth.make_system(12,10,5, sigma=1.5, seed=3, wells=diagonal)")
    np.savez_compressed(os.path.join(HERE, "synth_small.npz"), **g)
    A2, b2 = singular_case()
    g = golden_for(R, A2, b2, with_factors=True, label="singular")
    g["source"] = np.array("synthetic 8x6x3 system with three singular pivot blocks")
    np.savez_compressed(os.path.join(HERE, "singular_pivots.npz"), **g)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f"{f}: {os.path.getsize(os.path.join(HERE, f)) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()

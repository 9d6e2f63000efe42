"""Profiling cases: a preconditioner set-up and a few applications (or whole solve steps) on a fixed synthetic
workload, for ncu captures of single kernels or of one step's launch list (the bench runs many timed steps).

    python -m ressim_gb300.profile_case cpr_grid810k --precision mixed_f32 --applications 2
    python -m ressim_gb300.profile_case bilu0_grid180k --precision mixed_f32 --applications 3
    python -m ressim_gb300.profile_case ensemble64 --applications 3
    python -m ressim_gb300.profile_case ensemble64 --steps 2
    python -m ressim_gb300.profile_case ensemble64 --steps 1 --sweep cta     # the one-kernel CPR application
    python -m ressim_gb300.profile_case bilu0_grid180k --precision fp64 --steps 1 --krylov gmres   # GMRES kernels

cpr_grid810k: 180x90x50 cells (810,000 block rows, sigma ln k = 1.5, 4 wells), CPR applied grid-wide (a system
this size does not fit one SM). bilu0_grid180k: 100x60x30 cells (180,000 block rows), BILU0 with the grid-wide
sync-free sweeps. ensemble64: the bench's 64-realisation ensemble (40x40x10 each, 742,384 block rows), CPR in the
split form; with --steps, whole bench steps (set-up + CPR-BiCGSTAB to 1e-6 with the bench's options).
"""
from __future__ import annotations

import argparse

import numpy as np

CASES = {
    "cpr_grid810k": dict(shape=(180, 90, 50), precond="cpr", sweep="auto"),
    "bilu0_grid180k": dict(shape=(100, 60, 30), precond="bilu0", sweep="grid"),
    "ensemble64": dict(shape=None, precond="cpr", sweep="auto"),
}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--precision", default="mixed_f32", choices=["fp64", "mixed", "mixed_f32"])
    ap.add_argument("--applications", type=int, default=2)
    ap.add_argument("--steps", type=int, default=0, help="ensemble64: whole set-up + solve steps instead of applications")
    ap.add_argument("--systems", type=int, default=64, help="ensemble64: realisations of the ensemble (the bench's 64)")
    ap.add_argument("--sweep", default=None, choices=["auto", "cta", "split", "grid"],
                    help="sweep / CPR form (default: the case's; cta = the one-kernel CPR application)")
    ap.add_argument("--vcycle-form", type=int, default=0,
                    help="split CPR V-cycle: 1 fused kernel, 2 separate launches, 3 coarse levels per system, 0 tuned")
    ap.add_argument("--cpr2-threads", type=int, default=0, help="split CPR BILU0 stage: 256 or 512 threads per system, 0 tuned")
    ap.add_argument("--krylov", default="bicgstab", choices=["bicgstab", "gmres"], help="Krylov method of --steps")
    ap.add_argument("--restart", type=int, default=30, help="GMRES restart length")
    args = ap.parse_args(argv)
    from ressim_gb300 import synth
    from ressim_gb300.solver import DeviceSolver
    c = CASES[args.case]
    if c["shape"] is None:
        systems = synth.ensemble(n_real=args.systems)
        mats, b = [s.A for s in systems], np.concatenate([s.b for s in systems])
    else:
        s = synth.make_system(*c["shape"], sigma=1.5, seed=3, dt=5.0, wells="random", n_wells=4)
        mats, b = [s.A], s.b
    d = DeviceSolver(precond=c["precond"], precision=args.precision, sweep=args.sweep or c["sweep"], krylov=args.krylov,
                     restart=args.restart, check_every=4, use_graphs=True, vcycle_form=args.vcycle_form,
                     cpr2_threads=args.cpr2_threads)
    if len(mats) > 1:
        d.set_batch(mats)
    else:
        d.set_matrix(mats[0])
    ok = True
    if args.steps:
        for _ in range(args.steps):
            d.setup()
            x, res = d.solve(b, tol=1e-6, maxit=500)
            ok = ok and bool(res.converged)
    else:
        d.setup()
        r = np.random.default_rng(1).standard_normal(sum(A.n for A in mats) * 3)
        z = None
        for _ in range(args.applications):
            z = d.precond_apply(r)
        ok = bool(np.isfinite(z).all())
    n = sum(A.n for A in mats)
    nnzb = sum(A.nnzb for A in mats)
    print(f"{args.case}: n {n} nnzb {nnzb} precision {args.precision} amg_levels {d.stats().amg_levels} ok {ok}")
    print(f"launch shapes: {d.tuning()}")
    d.close()
    return 0 if ok else 1


if __name__ == "__main__":
    raise SystemExit(main())

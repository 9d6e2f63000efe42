"""Profiling cases: one preconditioner set-up and a few applications on a fixed synthetic system, for ncu captures
of single kernels (the bench runs whole solves).

    python -m ressim_gb300.profile_case cpr_grid810k --precision mixed_f32 --applications 2
    python -m ressim_gb300.profile_case bilu0_grid180k --precision mixed_f32 --applications 3

cpr_grid810k: 180x90x50 cells (810,000 block rows, sigma ln k = 1.5, 4 wells), CPR applied grid-wide (a system
this size does not fit one SM). bilu0_grid180k: 100x60x30 cells (180,000 block rows), BILU0 with the grid-wide
sync-free sweeps.
"""
from __future__ import annotations

import argparse

import numpy as np

CASES = {
    "cpr_grid810k": dict(shape=(180, 90, 50), precond="cpr", sweep="auto"),
    "bilu0_grid180k": dict(shape=(100, 60, 30), precond="bilu0", sweep="grid"),
}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--precision", default="mixed_f32", choices=["fp64", "mixed", "mixed_f32"])
    ap.add_argument("--applications", type=int, default=2)
    args = ap.parse_args(argv)
    from ressim_gb300 import synth
    from ressim_gb300.solver import DeviceSolver
    c = CASES[args.case]
    s = synth.make_system(*c["shape"], sigma=1.5, seed=3, dt=5.0, wells="random", n_wells=4)
    d = DeviceSolver(precond=c["precond"], precision=args.precision, sweep=c["sweep"])
    d.set_matrix(s.A)
    d.setup()
    r = np.random.default_rng(1).standard_normal(s.A.n * 3)
    z = None
    for _ in range(args.applications):
        z = d.precond_apply(r)
    ok = bool(np.isfinite(z).all())
    print(f"{args.case}: n {s.A.n} nnzb {s.A.nnzb} precision {args.precision} amg_levels {d.stats().amg_levels} finite {ok}")
    d.close()
    return 0 if ok else 1


if __name__ == "__main__":
    raise SystemExit(main())

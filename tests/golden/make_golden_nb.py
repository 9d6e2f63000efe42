"""Generate the golden vectors of the block-size-generic path (blocks other than 3 x 3) from the reference engine.

Runs only where the reference tree exists. ``oracle/_ref/ref_capture_nb`` (oracle/ref_capture_nb.cpp, linked with the
reference engine built from its own sources by oracle/Makefile.ref) runs two of the reference's example decks with
the simulators that call the same block solver and records the Newton systems they hand to the solver hook:

* examples/COMP.DATA with the compositional simulator (7x7x3 cells, six components + water: nb = 8; BlockCPR +
  GMRES(60) at the engine's linear tolerance, engine/src/compsim.cpp:1443-1449);
* examples/STEAMFLOOD.DATA with the thermal simulator (9x9x3 cells, nb = 5; BlockCPR + GMRES(80) at 1e-6,
  engine/src/thermsim.cpp:1818-1828).

The fourth Newton system of each run is kept (tests/golden/comp_sys.npz, thermal_sys.npz) with the reference's own
outputs through oracle/ref_shim.cpp (single thread): BSR::spmv, the BILU0 factors and sweeps, BlockCPR::apply (no
accumulation blocks: the hook carries none), BiCGSTAB with BILU0 at 1e-10 and GMRES with CPR (the caller's restart)
at 1e-10 and at the caller's own tolerance.

    RESSIM_REFERENCE=<reference repository root> python tests/golden/make_golden_nb.py
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
from ressim_gb300.bsr import read_system, save_npz  # noqa: E402

REF = os.environ.get("RESSIM_REFERENCE", "")
CASES = {"comp": ("examples/COMP.DATA", 60), "thermal": ("examples/STEAMFLOOD.DATA", 80)}
KEEP = 3            # Newton system kept (0-based)


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "engine", "src")):
        sys.exit("set RESSIM_REFERENCE to the reference repository's root")
    for tgt in (["stage", "REF=" + REF], ["-j8", "solver"], ["-j8", "oracle/_ref/ref_capture_nb"]):
        subprocess.run(["make", "-f", "oracle/Makefile.ref"] + tgt, cwd=ROOT, check=True, capture_output=True)
    R = RefShim()
    R.L.ref_set_threads(1)
    for kind, (deck, restart) in CASES.items():
        with tempfile.TemporaryDirectory() as d:
            r = subprocess.run([os.path.join(ROOT, "oracle/_ref/ref_capture_nb"), kind, os.path.join(REF, deck), d, str(KEEP + 1), "1"],
                               check=True, capture_output=True, text=True)
            print(kind, r.stdout.strip())
            sysm = read_system(os.path.join(d, f"sys_{KEEP:03d}.bin"))
        A, b = sysm.A, sysm.b
        rng = np.random.default_rng(4321)
        x = rng.standard_normal(A.n * A.nb)
        lu, nreg = R.bilu0_factor(A)
        out = dict(x_seed=x, y_spmv=R.spmv(A, x), lu=lu, nreg=nreg, z_bilu0=R.bilu0_apply(A, b), z_cpr=R.prec_apply(A, b, prec=1, acc=None),
                   engine_tol=sysm.meta["tol"], engine_maxit=sysm.meta["maxIt"], restart=restart)
        solves = {"bicg_bilu0": dict(prec=0, method=0, tol=1e-10, maxit=1000),
                  "gmres_cpr": dict(prec=1, method=1, restart=restart, tol=1e-10, maxit=1000),
                  "gmres_cpr_engine": dict(prec=1, method=1, restart=restart, tol=sysm.meta["tol"], maxit=sysm.meta["maxIt"])}
        for k, c in solves.items():
            xs, conv, its, rr = R.solve(A, b, **c)
            out["x_" + k], out["its_" + k], out["rr_" + k], out["conv_" + k] = xs, its, rr, int(conv)
            print(f"  {kind:8s} {k:18s} conv {conv} its {its:4d} relres {rr:.3e}")
        save_npz(os.path.join(HERE, f"{kind}_sys.npz"), sysm, **out)
        print(f"wrote {kind}_sys.npz: n {A.n} nb {A.nb} nnzb {A.nnzb}")


if __name__ == "__main__":
    main()

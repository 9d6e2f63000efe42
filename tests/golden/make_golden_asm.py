"""Generate tests/golden/waterflood_asm.npz, the golden vectors of the device Jacobian assembly, from the reference
engine itself.

Runs only where the reference tree exists. ``oracle/_ref/ref_asm_capture`` (built by oracle/Makefile.ref from the
reference's own sources and oracle/ref_asm_capture.cpp) runs the 20x20x4 three-phase waterflood and, at three calls
of the engine's solver hook, records the simulator's state and its assemblies at that state with dt = 3.7 days:
the full Jacobian and residual (wells included, rows scaled), the well terms alone (exact, unscaled) and, for the
first state, the reservoir terms alone. The first capture is repeated on a perturbed state with free-gas and
no-oil cells. Kept here: the grid, the pattern and the fluid / saturation tables once (they do not change during the
run), and per state the unknowns, the old accumulations, J and R, and the well terms as sparse addends.

    RESSIM_REFERENCE=<reference repository root> python tests/golden/make_golden_asm.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("RESSIM_REFERENCE", "")
DT = 3.7
CALLS = [0, 8, 25]

STATIC = ["na", "nv", "nw", "adjStart", "adjNbr", "adjConn", "conn_a", "conn_b", "conn_trans", "conn_dDepth", "poreVolRef",
          "J_rowPtr", "J_col", "phases", "vars", "gravity", "pvtw", "rock", "rhoSC", "gasFactor", "fluid_flags",
          "liveRs", "livePb", "bSat", "bmuSat", "swco", "kroModel", "sat_flags"]
TABLES = ["rsOfP", "pbOfRs", "deadB", "deadBMu", "gasB", "gasBMu", "krw", "krow", "pcow", "krg", "krog", "pcog"]
STATE = ["p", "sw", "x", "hasGas", "accOld", "dt", "J_full", "R_full"]


def read_capture(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            nm = f.read(32)
            if len(nm) < 32:
                break
            name = nm.split(b"\0")[0].decode()
            kind = int(np.frombuffer(f.read(4), np.int32)[0])
            cnt = int(np.frombuffer(f.read(8), np.int64)[0])
            dt = {0: np.float64, 1: np.int32, 2: np.uint8}[kind]
            out[name] = np.frombuffer(f.read(cnt * np.dtype(dt).itemsize), dt).copy()
    return out


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "engine", "src")):
        sys.exit("set RESSIM_REFERENCE to the reference repository's root")
    subprocess.run(["make", "-f", "oracle/Makefile.ref", "stage", "REF=" + REF], cwd=ROOT, check=True, capture_output=True)
    subprocess.run(["make", "-f", "oracle/Makefile.ref", "-j8", "oracle/_ref/ref_asm_capture"], cwd=ROOT, check=True,
                   capture_output=True)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_asm_capture"), tmp, str(DT), *map(str, CALLS)], check=True)
        caps = [read_capture(os.path.join(tmp, f"asm_{CALLS[0]:03d}_perturbed.bin"))]
        caps += [read_capture(os.path.join(tmp, f"asm_{c:03d}.bin")) for c in CALLS]
    first = caps[0]
    z = {k: first[k] for k in STATIC}
    for t in TABLES:
        for s in ("_x", "_y", "_clamp"):
            z[t + s] = first[t + s]
    for t in ("uB", "uBMu"):
        for s in ("_x", "_y", "_off", "_clamp"):
            z[t + s] = first[t + s]
    for k, c in enumerate(caps):
        for s in STATIC:   # the grid, pattern and tables do not change during the run
            assert np.array_equal(c[s], first[s]), s
        for s in STATE:
            z[f"s{k}_{s}"] = c[s]
        jw, rw = c["J_well"], c["R_well"]
        pos = np.flatnonzero(jw)
        z[f"s{k}_add_pos"] = pos.astype(np.int64)
        z[f"s{k}_add_val"] = jw[pos]
        rpos = np.flatnonzero(rw)
        z[f"s{k}_radd_pos"] = rpos.astype(np.int32)
        z[f"s{k}_radd_val"] = rw[rpos]
        if k == 1:
            z[f"s{k}_J_cell"] = c["J_cell"]
            z[f"s{k}_R_cell"] = c["R_cell"]
        print(f"state {k}: states {np.bincount(c['hasGas'], minlength=3)}, {pos.size} J / {rpos.size} R well terms")
    z["nstates"] = np.array([len(caps)], np.int32)
    z["state_names"] = np.array(["perturbed (free gas and no-oil cells) at the first Newton call"] +
                                [f"Newton call {c}" for c in CALLS])
    np.savez_compressed(os.path.join(HERE, "waterflood_asm.npz"), **z)


if __name__ == "__main__":
    main()

"""Benchmark: solves/s of the batched mixed-precision GPU solve of the 64-realisation ensemble.

Workload (one step): 64 Newton systems of a 40x40x10 black-oil waterflood (sigma ln k = 1.5, seeded inactive
fraction U[0.1, 0.5] -> 8k-14.4k active cells each, BSR 3x3), generated by ressim_gb300.synth with seeds
0..63 (+64 * rank under torchrun: weak scaling, each GPU its own ensemble). A step is the solve path of all
64 systems at once: CPR set-up of every system (weights, pressure matrix, AMG refresh, lean FP32 BILU0 factors)
and a batched CPR-preconditioned BiCGSTAB to true relative residual <= 1e-6 (FP64 outer vectors / inner
products / true residual, FP32 preconditioner).

Reported besides ``value`` (device-resident inputs, CUDA events on the solver stream):
* ``e2e``: the same step through the C ABI with host buffers (matrix values and right-hand sides copied in,
  solutions copied out, every step);
* ``fp64_batched``: the same batch and CPR in plain FP64, timed the same way (the precision form's gain);
* ``fp64_plain``: the plain FP64 GPU path, the 64 systems solved one after another (one handle each);
* ``error_vs_fp64``: each result's distance to its system's FP64 solution (plain FP64 at 1e-12);
* ``roofline`` of the dominant kernel and ``kernels`` (per-launch device time and algorithmic bytes);
* ``cpu_baseline``: the reference engine's own FP64 CPR-BiCGSTAB (compiled on this host from its staged sources,
  oracle/_ref) on the host cores, on a bounded sample of the same systems; the C restatement (oracle/) where the
  reference build is absent.

``--impl reference`` times the same reference CPU path on every step's 64 systems (rank 0 only).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--serving on|off|only] [--spe10]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_REAL, NX, NY, NZ, SIGMA = 64, 40, 40, 10, 1.5      # N_REAL: --systems (64 = the headline workload)
TOL, MAXIT = 1e-6, 500
def workload():
    return f"ensemble{N_REAL}_40x40x10_cpr_bicgstab"
BATCH_PREC = dict(precond="cpr", precision="mixed_f32")     # batched mixed-precision form
PLAIN_PREC = dict(precond="cpr", precision="fp64")          # plain FP64 GPU path
# the reference CPU solver's preconditioner for these systems: BlockCPR (auto mode picks CPR for >= 500 cells,
# engine/src/simulator.cpp:224); oracle code 1 = CPR with quasi-IMPES weights
CPU_PREC = 1
METRIC = "solves/s & p99 latency: batched mixed-prec vs plain FP64 GPU, true rel.res <=1e-6"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_of(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary of this workload (profiles/traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)[kernel]["traffic_bytes_per_launch"]
    except Exception:
        return None


def rank_seed0(rank):
    """Weak scaling: every rank solves its own ensemble (seeds 64 r .. 64 r + 63)."""
    return 64 * rank


def ensemble(rank):
    from ressim_gb300 import synth
    return synth.ensemble(n_real=N_REAL, nx=NX, ny=NY, nz=NZ, sigma=SIGMA, seed0=rank_seed0(rank))


def max_over_ranks(value, dist=None, device="cpu"):
    """The slowest rank's time (the job's time): all-reduce MAX over the process group, or the value itself."""
    if not dist:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None, "reasons": sorted(reasons),
                "samples": len(sm)}


def _lib_check(rc):
    from ressim_gb300 import _lib
    return _lib.check(rc)


def spmv_bytes(nnzb, n):
    return nnzb * (9 * 8 + 4) + (n + 1) * 4 + 2 * 3 * n * 8


def ilu_bytes(nnzb, n, sv, sx):
    return nnzb * (9 * sv + 4) + 2 * (n + 1) * 4 + 2 * 3 * n * sx


def cpr_bytes(nnzb, n, levels, sv, sx):
    """Algorithmic bytes of one CPR application: the BILU0 stage, per smoothed AMG level two passes over A_l (the
    Gauss-Seidel sweeps; the residual's reads are in the vector term), R_l, P_l and four vector streams, the coarsest
    levels' dense inverses and vectors, the second-stage input (3 vector streams in and out) and the pressure
    columns of S. ``levels`` = (rows per level, entries per level, dense coarse entries), summed over the batch."""
    rows, nnz, dense = levels
    csr = lambda r, z: z * (sv + 4) + (r + 1) * 4
    b = ilu_bytes(nnzb, n, sv, sx)
    for l in range(len(rows) - 1):
        b += 2 * csr(rows[l], nnz[l]) + csr(rows[l + 1], rows[l]) + csr(rows[l], rows[l]) + 4 * rows[l] * sx
    b += dense * sv + 2 * int(rows[-1]) * sx
    return int(b + n * (3 * sx * 2) + nnzb * (3 * sv + 4))


class RefEnsemble:
    """The reference engine's own CPU path over the ensemble (oracle/_ref/libressim_ref.so, compiled on this host from
    the reference's staged sources): one BlockCPR per realisation with the AMG aggregates reused after the first
    set-up, BiCGSTAB to the tolerance. Two ways to use the host's cores: one system after another with the reference's
    OpenMP on all physical cores, or one system per core at once (how a study runs one simulator per realisation)."""

    def __init__(self, systems):
        import ctypes as C
        from oracle import REF_LIB
        L = C.CDLL(REF_LIB)
        L.ref_ens_create.restype = C.c_void_p
        L.ref_ens_create.argtypes = [C.c_int]
        L.ref_ens_set.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_ens_step.restype = C.c_double
        L.ref_ens_step.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int]
        L.ref_ens_result.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_ens_free.argtypes = [C.c_void_p]
        L.ref_physical_cores.restype = C.c_int
        self.L, self.n = L, len(systems)
        self.h = L.ref_ens_create(len(systems))
        for k, s in enumerate(systems):
            L.ref_ens_set(self.h, k, s.A.n, s.A.nb, s.A.rowPtr.ctypes.data, s.A.col.ctypes.data, s.A.val.ctypes.data, s.b.ctypes.data)
        self.cores = int(L.ref_physical_cores())

    def step(self, concurrent):
        return float(self.L.ref_ens_step(self.h, TOL, MAXIT, self.cores if concurrent else 1, 0))

    def converged(self):
        return all(self.L.ref_ens_result(self.h, k, None, None, None) == 1 for k in range(self.n))

    def close(self):
        self.L.ref_ens_free(self.h)


def reference_available():
    from oracle import RefShim
    return RefShim.available()


def cpu_baseline(systems):
    """The reference CPU path on the host cores, on a bounded sample: one untimed pass over the ensemble (first
    set-up of every realisation's AMG), then one timed pass in each way of using the cores; the faster is reported.
    Without the reference build, the C restatement (oracle/) of the same path, one system after another."""
    if reference_available():
        R = RefEnsemble(systems)
        try:
            R.step(True)
            t_omp, t_con = R.step(False), R.step(True)
            ok = R.converged()
        finally:
            R.close()
        best = min(t_omp, t_con)
        return {"value": len(systems) / best, "unit": "solves/s", "cores": R.cores, "kind": "reference",
                "mode": "one system per core" if t_con <= t_omp else "OpenMP per system",
                "modes_solves_per_s": {"openmp_per_system": len(systems) / t_omp, "system_per_core": len(systems) / t_con},
                "all_converged": bool(ok),
                "sample": f"one pass over the {len(systems)} ensemble systems after a warm-up pass (reference BlockCPR + BiCGSTAB, "
                          f"FP64, AMG reused), faster of the two ways of using {R.cores} cores"}
    from oracle import Oracle
    o = Oracle()
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    t0 = time.perf_counter()
    done = 0
    for s in systems:
        o.solve(s.A, s.b, prec=CPU_PREC, method=0, tol=TOL, maxit=MAXIT)
        done += 1
        if time.perf_counter() - t0 > 20.0:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"{done} of the {len(systems)} ensemble systems, FP64 CPR-BiCGSTAB to 1e-6 (C restatement, OpenMP SpMV/vector ops)"}


SERVE_RATE, SERVE_N, SERVE_POOL, SERVE_SLOTS, SERVE_BUDGET = 200.0, 200, 16, 8, 150 << 30
SERVE_SUSTAINED_N = 60


def serving_pool(seed=4242):
    """Requests of the serving stream's shape: one per 1/16 quantile of a log-uniform cell count in 1e3..1e6
    (random box with nz in [1, 50], sigma ln k in [0.5, 3], time step in [0.1, 30] days, 1-8 wells)."""
    from ressim_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for i in range(SERVE_POOL):
        cells = 1e3 * 1000.0 ** ((i + 0.5) / SERVE_POOL)
        out.append(synth.serving_request(rng, cells_lo=cells, cells_hi=cells))
    return out


def serving_arrivals(seed=99):
    """Poisson arrivals at SERVE_RATE per second, each request drawn uniformly from the pool."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / SERVE_RATE, SERVE_N))
    return [(float(t[i]), int(rng.integers(SERVE_POOL))) for i in range(SERVE_N)]


def serving_leg(local, pool, arrivals, precision):
    """Continuous batching through the server (rsg_server_*): requests submitted at their arrival times (or when
    the previous submission returns, if later), latency = submit -> result on the server clock."""
    from ressim_gb300.solver import Server
    with Server(slots=SERVE_SLOTS, mem_budget=SERVE_BUDGET, precond="cpr", precision=precision, device=local) as srv:
        for s in pool[:4]:                                   # warm-up: module load, allocator pools
            srv.poll(srv.submit(s.A, s.b, tol=TOL, maxit=MAXIT))
        ids = []
        late = 0.0
        t0 = time.perf_counter()
        for ta, k in arrivals:
            now = time.perf_counter() - t0
            if now < ta:
                time.sleep(ta - now)
            else:
                late = max(late, now - ta)
            ids.append((srv.submit(pool[k].A, pool[k].b, tol=TOL, maxit=MAXIT), k))
        res = [(srv.poll(i)[1], k) for i, k in ids]
        T = time.perf_counter() - t0
    lat = np.array([r["total_ms"] for r, _ in res])
    ok = [r["status"] == 0 and 0 <= r["true_rel_residual"] <= TOL for r, _ in res]
    return {"throughput": len(res) / T, "unit": "solves/s", "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_run_ms": float(np.mean([r["run_ms"] for r, _ in res])),
            "converged": int(sum(ok)), "requests": len(res), "max_submit_lag_ms": 1e3 * late,
            "cells_per_s": float(sum(pool[k].A.n for _, k in res) / T),
            "batched_requests": int(sum(r["batch"] > 1 for r, _ in res)),
            "mean_batch": float(np.mean([r["batch"] for r, _ in res]))}


def serving_arrivals_at(rate, n, seed=7):
    """Poisson arrivals at `rate` per second, n requests drawn uniformly from the pool."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    return [(float(t[i]), int(rng.integers(SERVE_POOL))) for i in range(n)]


def serving_ensemble(local, systems, rounds=10, copied_rounds=3):
    """The ensemble's systems handed to the server at once (admission held while they are submitted), as a simulator
    running 64 realisations at a common step would: they are admitted together and solved as one batch. One slot, so
    that rounds after the first reuse its plan as the batched handle does. The simulator keeps its Jacobians, so it
    lends them (rsg_submit_view, the headline figure); the copying submission (rsg_submit) is timed beside it."""
    from ressim_gb300.solver import Server
    with Server(slots=1, mem_budget=SERVE_BUDGET, precond="cpr", precision="mixed_f32", device=local) as srv:
        def one_round(copy):
            srv.hold(True)
            t0 = time.perf_counter()
            ids = [srv.submit(s.A, s.b, tol=TOL, maxit=MAXIT, copy=copy) for s in systems]
            srv.hold(False)
            res = [srv.poll(i)[1] for i in ids]
            dt = time.perf_counter() - t0
            ok = all(r["status"] == 0 and 0 <= r["true_rel_residual"] <= TOL for r in res)
            return dt, max(r["batch"] for r in res), ok
        first = one_round(False)                  # the pattern's first sight: plan, hierarchy, tuning
        lent = [one_round(False) for _ in range(rounds)]
        copied = [one_round(True) for _ in range(copied_rounds)]
    n = len(systems)
    return {"value": n * rounds / sum(t for t, _, _ in lent), "unit": "solves/s", "batch": int(lent[-1][1]), "rounds": rounds,
            "p50_round_ms": 1e3 * statistics.median(t for t, _, _ in lent),
            "all_converged": bool(first[2] and all(ok for _, _, ok in lent + copied)),
            "copying_submit": {"value": n * copied_rounds / sum(t for t, _, _ in copied), "unit": "solves/s",
                               "batch": int(copied[-1][1]), "rounds": copied_rounds},
            "first_round_ms": 1e3 * first[0],
            "note": "host wall clock per round after the pattern's first round: submission (arrays lent in place; "
                    "copying_submit: copied), admission, batched value upload, set-up and solve, results"}


def assembly_bytes(z):
    """Bytes the assembly must move at least once per call: the state and old accumulations, the grid (adjacency,
    connections, pore volumes, row starts of the pattern), the Jacobian and residual written, the per-cell property
    records (13 dual numbers) written by k_bo_props and read once, and the per-connection flux terms (4 x 7 doubles)
    written by k_bo_conn and read once from each of the connection's two cells."""
    na, nconn = int(z["na"][0]), int(z["conn_trans"].size)
    nadj, nnz, nrows = int(z["adjStart"][-1]), int(z["J_rowPtr"][-1]), na * 3 + int(z["nw"][0])
    state = na * (3 * 8 + 1 + 3 * 8 + 8)
    grid = (na + 1) * 4 + nadj * 12 + nconn * 20 + (nrows + 1) * 4 + na * 8
    out = nnz * 8 + nrows * 8
    rec = 2 * 52 * 8 * na
    flux = 3 * 28 * 8 * nconn
    return {"state": state, "grid": grid, "jacobian_and_residual": out, "records": rec, "connection_fluxes": flux,
            "total": state + grid + out + rec + flux}


def assembly_cpu_baseline(z, st):
    """The reference engine's own assembly on the host cores: its evalAll + assemble (block assembly, the engine's
    default) at the first Newton state of a 100 x 100 x 74 waterflood (740,000 cells, about the ensemble's 742,384),
    compiled from the staged reference sources (oracle/Makefile.ref, ~30 s with 16 cores) and timed over 5 repeats
    by oracle/_ref/ref_asm_capture --time. Without the staged sources: the C restatement (oracle/rsg_oracle_asm.c,
    one thread) on the same synthetic model as the device."""
    cores = os.cpu_count() or 1
    staged = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "src", "engine", "src", "simulator.cpp"))
    if staged:
        try:
            r = subprocess.run(["make", "-f", "oracle/Makefile.ref", f"-j{cores}", "oracle/_ref/ref_asm_capture"], cwd=ROOT,
                               capture_output=True, text=True, timeout=600)
            if r.returncode == 0:
                r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_asm_capture"), "--time", "100", "100", "74", "5"],
                                   capture_output=True, text=True, timeout=600, env=dict(os.environ, OMP_NUM_THREADS=str(cores)))
                if r.returncode == 0:
                    out = json.loads(r.stdout.strip().splitlines()[-1])
                    return {"value": out["cells"] / (out["median_ms"] / 1e3), "unit": "cells/s", "ms": out["median_ms"],
                            "cells": out["cells"], "cores": cores, "kind": "reference",
                            "sample": "the engine's evalAll + assemble at the first Newton state of a 100x100x74 waterflood, "
                                      "median of 5"}
        except Exception:
            pass
    from oracle import Oracle
    t0 = time.perf_counter()
    Oracle().bo_assemble(z, st["p"], st["sw"], st["x"], st["state"], st["acc_old"], 10.0)
    dt = time.perf_counter() - t0
    na = int(z["na"][0])
    return {"value": na / dt, "unit": "cells/s", "ms": 1e3 * dt, "cells": na, "cores": 1, "kind": "port",
            "sample": "the C restatement of the engine's assembly on the device's synthetic model, one pass"}


def assembly_leg(local, steps, warmup, cpu=True):
    """Device Jacobian assembly (rsg_bo_assemble) of the ensemble's 64 grids taken as one (synthetic black-oil tables
    and state, ressim_gb300.synth.assembly_ensemble): device time per assembly with the state resident, and end to
    end with the state uploaded from pinned host memory and the residual read back (what a Newton step moves when the
    Jacobian is built on the device) against the matrix upload it replaces."""
    import torch
    from ressim_gb300 import synth
    from ressim_gb300.assembly import BlackOilAssembler
    z, st = synth.assembly_ensemble(N_REAL, NX, NY, NZ, SIGMA, seed0=0)
    dv = torch.device(f"cuda:{local}")
    asm = BlackOilAssembler(z, device=local)
    host = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory() for k in ("p", "sw", "x", "state", "acc_old")}
    d = {k: v.to(dv) for k, v in host.items()}
    J = torch.empty(asm.nnz, dtype=torch.float64, device=dv)
    R = torch.empty(asm.nrows, dtype=torch.float64, device=dv)
    R_host = torch.empty(asm.nrows, dtype=torch.float64).pin_memory()
    s = torch.cuda.Stream(dv)
    torch.cuda.synchronize()

    def run():
        asm.assemble_device(d["p"].data_ptr(), d["sw"].data_ptr(), d["x"].data_ptr(), d["state"].data_ptr(), d["acc_old"].data_ptr(),
                            10.0, J.data_ptr(), R.data_ptr(), stream=s.cuda_stream)

    for _ in range(max(3, warmup)):
        run()
    torch.cuda.synchronize()
    reps = max(10, steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        run()             # J (339 MB) is written every call: more than L2 between consecutive calls
    e1.record(s)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / reps / 1e3
    # end to end: state in from pinned host memory, assembly, residual out (the engine's convergence check reads it)
    te = []
    for k in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s):
            for key in d:
                d[key].copy_(host[key], non_blocking=True)
            run()
            R_host.copy_(R, non_blocking=True)
        s.synchronize()
        if k >= warmup:
            te.append(time.perf_counter() - t0)
    asm.close()
    cpu_base = assembly_cpu_baseline(z, st) if cpu else None
    B = assembly_bytes(z)
    hbm, peak_kind = peaks()
    na = int(z["na"][0])
    h2d = sum(int(v.numel() * v.element_size()) for v in host.values())
    return {"workload": f"ensemble{N_REAL}_{NX}x{NY}x{NZ} grids as one ({na} cells, synthetic tables and state)",
            "cells": na, "jacobian_values": int(asm.nnz), "ms": 1e3 * t, "value": na / t, "unit": "cells/s",
            "launches_per_assembly": 3, "bytes": B, "roofline": {"bound": "hbm", "achieved": B["total"] / t / 1e9, "peak": hbm,
                                                                 "unit": "GB/s", "frac": B["total"] / t / 1e9 / hbm,
                                                                 "peak_kind": peak_kind + " burst copy"},
            "e2e": {"ms": 1e3 * statistics.median(te), "h2d_bytes": h2d, "d2h_bytes": asm.nrows * 8,
                    "matrix_upload_replaced_bytes": int(asm.nnz) * 8},
            "cpu_baseline": cpu_base}


def spe10_report(local):
    """The one-large-system configurations (60x220x85, 1,122,000 block rows; Jacobians of day 1 and day 100):
    CPR + GMRES(30) in plain FP64 and in the FP32 precision form at 1e-6 and 1e-8, with iterations, device set-up and
    solve times, true residuals and the precision form's distance to the FP64 solution. The CPR weights are the
    true-IMPES ones from the accumulation blocks, as the engine's BlockCPR set-up computes them when it has the blocks
    (engine/src/bsr.cpp:993-1059). The reference's own CPR-GMRES(30) on these systems (CPU, same weights) reaches
    1e-6 in 85 iterations on day 1 and needs about 900 on day 100 (1.03e-6 at 900)."""
    from ressim_gb300 import synth
    from ressim_gb300.solver import DeviceSolver
    out = {"report": "spe10_60x220x85_cpr_gmres30", "rows": 1_122_000, "solves": []}
    for day in (1, 100):
        s = synth.spe10_like(day=day)
        sol = {}
        for precision in ("fp64", "mixed_f32"):
            for tol in (1e-6, 1e-8):
                with DeviceSolver(precond="cpr", krylov="gmres", restart=30, precision=precision, device=local) as d:
                    d.set_matrix(s.A)
                    d.setup(s.acc)
                    d.setup(s.acc)                            # timed: the set-up of a known pattern (refresh)
                    x, res = d.solve(s.b, tol=tol, maxit=1500)
                    st = d.stats()
                tr = float(np.linalg.norm(s.b - synth.bsr_matvec_host(s.A, x)) / np.linalg.norm(s.b))
                sol[(precision, tol)] = x
                e = {"day": day, "precision": precision, "tol": tol, "converged": bool(res.converged), "iterations": res.iterations,
                     "setup_ms": st.setup_ms, "solve_ms": st.solve_ms, "true_relres": tr,
                     "escalated_systems": st.escalated_systems}
                if precision != "fp64":
                    x64 = sol[("fp64", tol)]
                    e["rel_diff_vs_fp64"] = float(np.linalg.norm(x - x64) / np.linalg.norm(x64))
                out["solves"].append(e)
        # the precision form inside FP64 defect correction (rsg_solve_refined: the engine's refineWithDevice with the
        # FP32-preconditioned GMRES(30) as its inner solve)
        for tol in (1e-6, 1e-8):
            with DeviceSolver(precond="cpr", krylov="gmres", restart=30, precision="mixed_f32", device=local) as d:
                d.set_matrix(s.A)
                d.setup(s.acc)
                d.setup(s.acc)
                x, res = d.solve_refined(s.b, tol=tol, max_outer=10, inner_it=600)
                st = d.stats()
            tr = float(np.linalg.norm(s.b - synth.bsr_matvec_host(s.A, x)) / np.linalg.norm(s.b))
            x64 = sol[("fp64", tol)]
            out["solves"].append({"day": day, "precision": "mixed_f32_refined", "tol": tol, "converged": bool(res.converged),
                                  "iterations": res.iterations, "setup_ms": st.setup_ms, "solve_ms": st.solve_ms, "true_relres": tr,
                                  "rel_diff_vs_fp64": float(np.linalg.norm(x - x64) / np.linalg.norm(x64))})
    return out


def run_reference(args, rank, world):
    """The reference arm: the reference engine's own CPU solve of the whole ensemble per step (every realisation's
    BlockCPR set-up with AMG reuse, then BiCGSTAB to 1e-6, FP64), on all host cores, in the faster of its two ways of
    using them (chosen in the warm-up). Rank 0 only; without the reference build, the C restatement."""
    if rank != 0:
        return 0
    systems = ensemble(0)
    line = {"metric": METRIC, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (ressim_gb300.synth, seeded)", "impl": "reference"}
    if reference_available():
        R = RefEnsemble(systems)
        R.step(True)                               # first set-up of every realisation's AMG hierarchy
        warm = {True: [], False: []}
        for w in range(max(2, args.warmup)):
            warm[w % 2 == 0].append(R.step(w % 2 == 0))
        concurrent = min(warm[True]) <= min(warm[False])
        times = [R.step(concurrent) for _ in range(args.steps)]
        ok = R.converged()
        R.close()
        T = sum(times)
        v = len(systems) * len(times) / T
        mode = "one system per core (one OpenMP thread each)" if concurrent else "one system after another, OpenMP on all cores"
        line.update({"value": v, "ms_per_step": 1e3 * T / len(times),
                     "config": {"workload": workload(), "systems_per_step": len(systems), "solver": "reference BlockCPR + BiCGSTAB, FP64",
                                "mode": mode, "all_converged": bool(ok)},
                     "cpu_baseline": {"value": v, "unit": "solves/s", "cores": R.cores, "kind": "reference",
                                      "sample": f"all {len(systems)} ensemble systems per step, {mode}"}})
    else:
        from oracle import Oracle
        o = Oracle()
        threads = os.cpu_count() or 1
        o.set_threads(threads)
        times = []
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            for s in systems:
                o.solve(s.A, s.b, prec=CPU_PREC, method=0, tol=TOL, maxit=MAXIT)
            if step >= args.warmup:
                times.append(time.perf_counter() - t0)
        T = sum(times)
        v = len(systems) * len(times) / T
        line.update({"value": v, "ms_per_step": 1e3 * T / len(times),
                     "config": {"workload": workload(), "systems_per_step": len(systems), "solver": "CPR-BiCGSTAB FP64 (C restatement)"},
                     "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                                      "sample": f"all {len(systems)} ensemble systems per step (C restatement of the reference CPU path)"}})
    line["e2e"] = {"value": line["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="rsg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--systems", type=int, default=64, help="ensemble size (64: the headline workload; smaller: profiling)")
    ap.add_argument("--spe10", action="store_true", help="print the one-large-system report (60x220x85) instead of the bench line")
    ap.add_argument("--assembly", choices=["on", "off", "only"], default="on",
                    help="the device Jacobian assembly leg (only: print it alone, for profiling)")
    ap.add_argument("--serving", choices=["on", "off", "only"], default="on",
                    help="the serving stream (Poisson arrivals through the continuous-batching server)")
    args = ap.parse_args()
    global N_REAL
    N_REAL = args.systems
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return rc

    import torch
    torch.cuda.set_device(local)
    from ressim_gb300.solver import DeviceSolver

    if args.assembly == "only":
        if rank == 0:
            print(json.dumps({"metric": "device Jacobian assembly",
                              "assembly": assembly_leg(local, args.steps, args.warmup, cpu=not args.no_cpu_baseline)}))
        return 0
    if args.spe10:
        if rank == 0:
            print(json.dumps(spe10_report(local)))
        return 0

    serving = None
    if args.serving != "off" and world == 1:               # the serving stream is a one-GPU measurement
        pool = serving_pool()
        arr = serving_arrivals()
        serving = {"rate_per_s": SERVE_RATE, "requests": SERVE_N, "pool": SERVE_POOL, "slots": SERVE_SLOTS,
                   "budget_gb": SERVE_BUDGET / 2**30, "cells": [int(min(s.A.n for s in pool)), int(max(s.A.n for s in pool))],
                   "mixed_f32": serving_leg(local, pool, arr, "mixed_f32"), "fp64": serving_leg(local, pool, arr, "fp64")}
        # the same pool at a sustainable rate: 70 % of the throughput the overloaded stream measured, so that p50 / p99
        # measure service, not backlog
        sustained = {}
        for prec in ("mixed_f32", "fp64"):
            rate = 0.7 * serving[prec]["throughput"]
            leg = serving_leg(local, pool, serving_arrivals_at(rate, SERVE_SUSTAINED_N), prec)
            leg["rate_per_s"] = rate
            sustained[prec] = leg
        serving["sustainable"] = sustained
        del pool
        if args.serving == "only":
            if rank == 0:
                print(json.dumps({"metric": METRIC, "serving": serving}))
            return 0

    systems = ensemble(rank)
    mats = [s.A for s in systems]
    b_host = np.concatenate([s.b for s in systems])
    n_rows = sum(A.n for A in mats)
    nnzb = sum(A.nnzb for A in mats)
    N = 3 * n_rows
    val_bytes = nnzb * 72

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # ---------------- batched mixed-precision path, device-resident inputs
    dev = DeviceSolver(krylov="bicgstab", check_every=4, use_graphs=True, device=local, **BATCH_PREC)
    dev.set_batch(mats)
    stream = torch.cuda.ExternalStream(dev.stream)
    dev.setup()
    tuning = dev.tuning()                                  # the launch shapes the autotuner picked for this batch
    d_b = torch.from_numpy(b_host).to(f"cuda:{local}")
    d_x = torch.zeros_like(d_b)
    torch.cuda.synchronize()

    def step():
        dev.setup()
        return dev.solve_device(d_b.data_ptr(), d_x.data_ptr(), tol=TOL, maxit=MAXIT)

    for _ in range(args.warmup):
        step()
    l0 = dev.stats().kernel_launches
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    results = []
    with Clocks(local) as clk:
        for k in range(args.steps):
            ev[k][0].record(stream)
            res = step()
            ev[k][1].record(stream)
            results.append(res)
        barrier()
    st_last = dev.stats()
    launches = st_last.kernel_launches - l0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    its, rr, tr = dev.batch_results()
    x_dev = d_x.cpu().numpy()
    T = sum(step_ms) / 1e3
    if dist:
        T = max_over_ranks(T, dist, f"cuda:{local}")
    value = world * N_REAL * args.steps / T
    ok = all(r.converged for r in results) and float(np.max(tr)) <= TOL

    # ---------------- the same batch in plain FP64 (same CPR, FP64 factors, hierarchy and sweeps): the precision gain
    dev64 = DeviceSolver(krylov="bicgstab", check_every=4, use_graphs=True, device=local, **PLAIN_PREC)
    dev64.set_batch(mats)
    s64 = torch.cuda.ExternalStream(dev64.stream)
    d_x64 = torch.zeros_like(d_b)

    def step64():
        dev64.setup()
        return dev64.solve_device(d_b.data_ptr(), d_x64.data_ptr(), tol=TOL, maxit=MAXIT)

    for _ in range(args.warmup):
        step64()
    barrier()
    ev64 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    ok64 = True
    for k in range(args.steps):
        ev64[k][0].record(s64)
        r64 = step64()
        ev64[k][1].record(s64)
        ok64 &= r64.converged
    barrier()
    T64 = sum(a.elapsed_time(b) for a, b in ev64) / 1e3
    if dist:
        T64 = max_over_ranks(T64, dist, f"cuda:{local}")
    its64, _, tr64 = dev64.batch_results()
    fp64_batched = {"value": world * N_REAL * args.steps / T64, "unit": "solves/s", "ms_per_step": 1e3 * T64 / args.steps,
                    "iterations": {"mean": float(np.mean(its64)), "max": int(np.max(its64))},
                    "all_converged": bool(ok64 and float(np.max(tr64)) <= TOL)}
    # error of every result against the FP64 solution of its system (plain FP64 path at 1e-12, pinned to the
    # reference's solution by the parity tests): the precision form at 1e-6, and the plain FP64 solve at 1e-6 beside it
    x64 = d_x64.cpu().numpy()
    dev64.solve_device(d_b.data_ptr(), d_x64.data_ptr(), tol=1e-12, maxit=MAXIT)
    xref = d_x64.cpu().numpy()
    dev64.close()
    err32, err64 = [], []
    off = 0
    for A in mats:
        sl = slice(off, off + 3 * A.n)
        nr = np.linalg.norm(xref[sl])
        err32.append(float(np.linalg.norm(x_dev[sl] - xref[sl]) / nr))
        err64.append(float(np.linalg.norm(x64[sl] - xref[sl]) / nr))
        off += 3 * A.n
    error_vs_fp64 = {"reference": "plain FP64 GPU solution at 1e-12 of each system",
                     "precision_form_max": max(err32), "precision_form_median": float(np.median(err32)),
                     "fp64_at_same_tol_max": max(err64), "fp64_at_same_tol_median": float(np.median(err64))}

    # ---------------- per-kernel device time (events on the solver stream) for the roofline
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    _lib_check(dev.L.rsg_spmv_level_probe(dev.h, reps))
    e1.record(stream)
    torch.cuda.synchronize()
    t_spmv = e0.elapsed_time(e1) / reps / 1e3
    e0.record(stream)
    _lib_check(dev.L.rsg_precond_level_probe(dev.h, reps))
    e1.record(stream)
    torch.cuda.synchronize()
    t_prec = e0.elapsed_time(e1) / reps / 1e3      # forward + backward sweep
    hbm, peak_kind = peaks()
    B_spmv = spmv_bytes(nnzb, n_rows)
    levels = dev.amg_level_sizes()
    B_cpr = cpr_bytes(nnzb, n_rows, levels, 4, 4) if levels else ilu_bytes(nnzb, n_rows, 4, 4)
    mean_its = float(np.mean(its))
    share_spmv = 2 * t_spmv * mean_its
    share_prec = 2 * t_prec * mean_its
    kernels = {
        "bsr3_spmv_f64": {"ms": 1e3 * t_spmv, "bytes": B_spmv, "gbs": B_spmv / t_spmv / 1e9, "per_iteration": 2},
        "cpr_apply_f32": {"ms": 1e3 * t_prec, "bytes": B_cpr, "gbs": B_cpr / t_prec / 1e9, "per_iteration": 2},
    }
    dom = "cpr_apply_f32" if share_prec >= share_spmv else "bsr3_spmv_f64"
    ach = kernels[dom]["gbs"]
    roofline = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "peak_kind": peak_kind + " burst copy", "traffic": traffic_of(dom) if N_REAL == 64 else None}
    roofline_spmv = {"bound": "hbm", "kernel": "bsr3_spmv_f64", "achieved": kernels["bsr3_spmv_f64"]["gbs"], "peak": hbm,
                     "unit": "GB/s", "frac": kernels["bsr3_spmv_f64"]["gbs"] / hbm}

    # ---------------- e2e through the C ABI with host buffers (values + rhs in, solutions out, every step), the step's
    # inputs and its solution in pinned host memory (the engine's staging buffers)
    from ressim_gb300 import _lib
    from ressim_gb300.bsr import BSR
    import ctypes as C

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64).pin_memory()
        out = t.numpy()
        out[:] = a.reshape(-1)
        return out, t

    keep_pinned = []
    mats_pinned = []
    for A in mats:
        v, t = pinned(A.val)
        keep_pinned.append(t)
        mats_pinned.append(BSR(A.n, A.nb, A.rowPtr, A.col, v))
    b_pin, tb = pinned(b_host)
    x_host, tx = pinned(np.zeros(N))
    keep_pinned += [tb, tx]
    L = _lib.load()
    e2e_t = []
    e2e_steps = max(args.steps, 20)        # host wall clock: more steps than the device timing, so one slow host step
    for k in range(args.warmup + e2e_steps):   # (a scheduler or allocator pause) does not set the figure
        barrier()
        t0 = time.perf_counter()
        dev.set_batch(mats_pinned)
        dev.setup()
        itc, rrc = C.c_int(0), C.c_double(0)
        rc = L.rsg_solve(dev.h, _lib.ptr(b_pin), _lib.ptr(x_host), TOL, MAXIT, C.byref(itc), C.byref(rrc))
        _lib.check(rc)
        barrier()
        if k >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    Te = sum(e2e_t)
    if dist:
        Te = max_over_ranks(Te, dist, f"cuda:{local}")
    e2e = {"value": world * N_REAL * len(e2e_t) / Te, "unit": "solves/s", "h2d_bytes_per_step": val_bytes + N * 8,
           "d2h_bytes_per_step": N * 8, "p50_ms": 1e3 * statistics.median(e2e_t), "steps": len(e2e_t), "host_buffers": "pinned"}
    dev.close()

    # ---------------- plain FP64 GPU path: one system after another (one handle each)
    plain = []
    for A in mats:
        d = DeviceSolver(krylov="bicgstab", check_every=4, use_graphs=True, device=local, **PLAIN_PREC)
        d.set_matrix(A)
        plain.append(d)
    bs = [torch.from_numpy(s.b).to(f"cuda:{local}") for s in systems]
    xs = [torch.zeros_like(b) for b in bs]
    for d, b, x in zip(plain, bs, xs):
        d.setup()
        d.solve_device(b.data_ptr(), x.data_ptr(), tol=TOL, maxit=MAXIT)
    torch.cuda.synchronize()
    lat = []
    t0 = time.perf_counter()
    plain_ok = True
    for d, b, x in zip(plain, bs, xs):
        s0 = time.perf_counter()
        d.setup()
        r = d.solve_device(b.data_ptr(), x.data_ptr(), tol=TOL, maxit=MAXIT)
        plain_ok &= r.converged and r.trueRelResidual <= TOL
        lat.append(time.perf_counter() - s0)
    torch.cuda.synchronize()
    Tp = time.perf_counter() - t0
    for d in plain:
        d.close()
    fp64_plain = {"value": len(mats) / Tp, "unit": "solves/s", "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                  "p99_ms": 1e3 * float(np.percentile(lat, 99)), "all_converged": bool(plain_ok)}

    serving_ens = serving_ensemble(local, systems) if args.serving != "off" and world == 1 else None
    assembly = assembly_leg(local, args.steps, args.warmup, cpu=rank == 0 and not args.no_cpu_baseline) \
        if world == 1 and args.assembly != "off" else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(systems)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * T / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "mixed f32/f64 (FP32 preconditioner, FP64 Krylov vectors, inner products and true residual)",
            "data": "synthetic (ressim_gb300.synth: seeded black-oil Jacobians of the named shapes)",
            "config": {"workload": workload(), "systems": N_REAL, "grid": f"{NX}x{NY}x{NZ}", "sigma_lnk": SIGMA,
                       "active_cells": [int(min(A.n for A in mats)), int(max(A.n for A in mats))], "block_rows": n_rows,
                       "nnzb": nnzb, "preconditioner": "CPR: aggregation AMG V-cycle (Gauss-Seidel) on the pressure system + BILU0",
                       "precision": "mixed: FP32 BILU0 factors/sweeps and AMG, FP64 Krylov vectors, dots, true residual; plain path FP64",
                       "tol": TOL, "tuning": tuning,
                       "l2": f"inputs larger than L2 (matrix values {val_bytes / 1e6:.0f} MB)", "parallelism": f"replicas{world}"},
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                           "note": "batched step: all 64 systems complete together"},
            "iterations": {"mean": mean_its, "max": int(np.max(its))}, "max_true_relres": float(np.max(tr)), "all_converged": bool(ok),
            "last_step_device_ms": {"setup": st_last.setup_ms, "solve": st_last.solve_ms},
            "fp64_plain": fp64_plain, "fp64_batched": fp64_batched, "max_rel_err_vs_fp64": error_vs_fp64["precision_form_max"],
            "error_vs_fp64": error_vs_fp64,
            "batched_mixed_over_plain_fp64": value / world / fp64_plain["value"],
            "batched_mixed_over_batched_fp64": value / fp64_batched["value"],
            "e2e": e2e, "roofline": roofline, "roofline_spmv": roofline_spmv, "kernels": kernels, "gpu_launches": int(launches),
            "cpu_baseline": cpu, "clocks": clk.summary(), "serving": serving, "serving_ensemble": serving_ens,
            "assembly": assembly,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

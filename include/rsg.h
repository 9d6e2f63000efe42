/* rsg -- GB300-native (sm_103a) Newton linear solver for ResSim Studio's black-oil engine: C ABI.
 *
 * Plain pointers and sizes only. Every call returns RSG_OK (0) or a negative status; rsg_last_error() gives the
 * message of the last failure on the calling thread (the convention of engine/include/ressim/capi.h:5-7:
 * int >= 0 success, -1-style errors, thread-local error text, caller-owned buffers).
 *
 * Each handle owns one CUDA stream and its device memory. A handle is used by one thread at a time;
 * different handles may be used concurrently from different threads.
 *
 * Data layout (identical to ressim::BSR, engine/include/ressim/bsr.h:23-37): n block rows, nb unknowns per cell
 * (nb = 3 for the black-oil system), rowPtr[n+1] / col[nnzb] int32 with sorted columns per row and a diagonal
 * block in every row, val[nnzb*nb*nb] float64 row-major blocks (row = equation, column = unknown); vectors of
 * n*nb float64 interleaved per cell.
 */
#ifndef RSG_H
#define RSG_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#define RSG_OK 0
#define RSG_EINVAL -1       /* bad argument (sizes, pattern, missing diagonal block) */
#define RSG_ECUDA -2        /* CUDA runtime failure (message has the CUDA error) */
#define RSG_ENOMEM -3       /* device allocation failed or the memory budget is exhausted */
#define RSG_ESTATE -4       /* call out of order (e.g. solve before setup) */
#define RSG_ETIMEOUT -5     /* a bounded device-side wait ran out (the kernel returned instead of hanging) */
#define RSG_EBREAKDOWN -6   /* Krylov breakdown (rho or <r0,v> vanished) before convergence */
#define RSG_ENOTCONV 1      /* finished without reaching the tolerance (x holds the last iterate) */

/* preconditioners */
#define RSG_PREC_BILU0 0    /* block ILU(0), natural-order exact (ressim::BILU0, engine/include/ressim/bsr.h:50-94) */
#define RSG_PREC_CPR 1      /* two-stage CPR: AMG on the pressure system + BILU0 (ressim::BlockCPR, bsr.h:224-250) */
#define RSG_PREC_JACOBI 2   /* block Jacobi (diagonal-block inverses) */
#define RSG_PREC_MCBILU0 4   /* multicolour block ILU(0) (ressim::MCBILU0, engine/src/bsr.cpp:599-730): the natural-order BILU0
                                 of P A P^T, P the largest-degree-first greedy colouring; few levels, so short sweeps */
#define RSG_PREC_CPR_DEVICE 3 /* the reference's GPU-shaped float CPR-AMG (ressim::DeviceCprAmg, engine/src/bsr.cpp:1217-1371):
                                 damped-Jacobi V-cycle, explicit coarse inverse, block-Jacobi second stage, in float;
                                 the precision option does not apply */
/* Krylov methods */
#define RSG_KRYLOV_BICGSTAB 0 /* ressim::bicgstab, engine/include/ressim/linsolve.h:99-100 */
#define RSG_KRYLOV_GMRES 1    /* ressim::gmres (flexible, restarted), linsolve.h:101-102 */
/* precision */
#define RSG_FP64 0          /* everything in FP64 */
#define RSG_MIXED 1         /* FP32 factor storage (elimination and 3x3 pivot inversions in FP64, as the reference's
                               lean BILU0, engine/src/bsr.cpp:219-263), FP64 sweep vector and accumulation (the
                               reference's float-factor sweeps, engine/src/bsr.cpp:500-522); FP64 outer Krylov
                               vectors, inner products and true residual */
#define RSG_MIXED_F32 2     /* the all-FP32 preconditioner of the precision form: BILU0 factors eliminated and stored in
                               FP32 with the 3x3 pivot blocks inverted in FP64 (thread-block path; the grid path keeps
                               the lean factors), FP32 sweeps (BILU0f, engine/src/bsr.cpp:1100-1121), FP32 AMG
                               hierarchy, V-cycle, coarsest LU and second-stage input; FP64 outer Krylov vectors,
                               inner products and true residual */

typedef struct rsg_options {
    int precond;            /* RSG_PREC_* */
    int krylov;             /* RSG_KRYLOV_* */
    int restart;            /* GMRES restart length (reference default 40; 30 for the SPE10-sized system) */
    int precision;          /* RSG_FP64 / RSG_MIXED */
    int gmres_fallback;     /* 1: a BiCGSTAB solve that does not converge is retried with GMRES(restart), as the
                               engine does (engine/src/simulator.cpp:3388-3398) */
    int check_every;        /* iterations launched between host convergence checks (0 = default 4) */
    int use_graphs;         /* 1: capture the iteration in a CUDA graph and replay it */
    int device;             /* CUDA device ordinal */
    size_t mem_budget;      /* bytes this handle may hold on the device (0 = no limit) */
    int sweep;              /* BILU0 sweep scheduling: 0 auto, 1 one thread block per system (level barriers,
                               shared-memory vector), 2 grid-wide sync-free (per-row flags), 3 split CPR: the
                               V-cycle's passes grid-wide over all systems, the BILU0 sweeps one thread block per
                               system (same results as 1). Auto takes 3 for CPR on a batch, 1 for a single system and
                               for BILU0 where the thread-block sweeps apply, else 2 */
    int fma;                /* 1 (default): the SpMV accumulates with fused multiply-adds (half the FP64
                               instructions; results within rounding of the reference); 0: the reference's separately
                               rounded products and sums, bit for bit (engine/src/bsr.cpp:109-117) */
    int sweep_inflight;     /* sync-free grid sweeps (BILU0, factorisation, Gauss-Seidel): levels in flight, which sizes
                               the persistent grid; 0 = auto (the full grid) */
    int autotune;           /* 1 (default): the launch shapes left at 0 below are chosen by timing the candidates on the
                               system at its first set-up (cached per pattern for the life of the process); 0: their
                               defaults. Every shape gives the same results bit for bit. */
    int vcycle_form;        /* split CPR, how the V-cycle runs over the batch: 1 = every pass grid-wide, as the phases of
                               one cooperative kernel (grid barriers between them); 2 = every pass grid-wide, one launch
                               per pass; 3 = the finest level's passes grid-wide, the coarser levels one thread block per
                               system in one launch; 0 = tuned (default 3) */
    int cpr2_threads;       /* split CPR: threads per system of the BILU0 stage, 128, 256 or 512; 0 = tuned (default 256) */
} rsg_options;

typedef struct rsg_stats {
    int iterations;         /* Krylov iterations of the last solve (max over the systems of a batch) */
    int converged;          /* 1 when every system reached the tolerance */
    double rel_residual;    /* recursive relative residual reported by the Krylov method (max over systems) */
    double true_rel_residual; /* ||b - A x|| / ||b|| recomputed in FP64 after the solve (max over systems), or -1 */
    double setup_ms;        /* device time of the last rsg_setup (factorisation, AMG refresh) */
    double solve_ms;        /* device time of the last solve */
    int regularised_blocks; /* singular pivot blocks shifted by the factorisation (ressim::BILU0::regularisedBlocks) */
    int amg_levels;         /* CPR: levels of the pressure AMG hierarchy */
    size_t device_bytes;    /* device memory held by the handle */
    long long kernel_launches; /* kernels launched by this handle since creation (graph nodes included) */
    int escalated_systems;  /* precision form: systems of the last solve that diverged or stalled with the all-FP32
                               preconditioner and were solved again with its FP64-vector sweeps */
} rsg_stats;

typedef struct rsg_solver rsg_solver;

void rsg_default_options(rsg_options* o);
const char* rsg_last_error(void);
const char* rsg_version(void);

/* Create / destroy a solver handle (one CUDA stream). */
int rsg_create(rsg_solver** h, const rsg_options* opts);
int rsg_destroy(rsg_solver* h);

/* Free the handle's pattern-dependent device state (plan, factors, hierarchy, Krylov vectors); the handle stays
 * usable and the next rsg_set_matrix plans again. No reference counterpart (device memory management). */
int rsg_release(rsg_solver* h);

/* Upload (or refresh) one system matrix from host memory. The pattern-dependent plan (level schedule,
 * elimination lists, AMG aggregates) is rebuilt only when the pattern changes; a values-only refresh
 * reuses it (the engine's pattern reuse, engine/src/bsr.cpp:759-769 and AMG::refresh, amg.cpp:257-271).
 * Replaces: the BSR the engine hands to GpuBlockSolver::solve (engine/include/ressim/bsr.h:147).
 * nb = 3 (black-oil) runs the specialised path with every option. Any other 1 <= nb <= 16 (kMaxBlock,
 * engine/include/ressim/bsr.h:21: the compositional simulator's nc + 1 unknowns, the thermal one's 4-5) runs the
 * block-size-generic path: one system per handle, FP64 (precision RSG_FP64), preconditioner RSG_PREC_BILU0 or
 * RSG_PREC_CPR, BiCGSTAB or GMRES(restart), with the reference's generic block arithmetic (BILU0 factors and sweeps bit
 * for bit); other options are RSG_EINVAL for such blocks. The callers it serves: engine/src/compsim.cpp:1443-1449
 * (BlockCPR + GMRES(60)) and engine/src/thermsim.cpp:1818-1828 (BlockCPR + GMRES(80)). */
int rsg_set_matrix(rsg_solver* h, int n, int nb, const int* rowPtr, const int* col, const double* val);

/* The Newton Jacobian with its well rows, reduced on the device. A is the scalar CSR the engine assembles: na*nv cell
 * rows followed by nw well (BHP) rows (nrows = na*nv + nw), host pattern, values on the host (rsg_set_jacobian, batch
 * form with one set of arrays per system) or in device memory (rsg_set_jacobian_device; the caller keeps them valid
 * until the solve). The well Schur complement S = A_cc - A_cw D_ww^-1 A_wc is computed on the device straight into the
 * handle's block system (the same values as the engine's, bit for bit, in the engine's order of operations); its
 * pattern is planned on the host and reused while the Jacobian pattern and the set of nonzero cell-to-well couplings
 * stay the same. Returns RSG_EINVAL when a well row has no usable BHP derivative or couples wells (the engine then
 * keeps the full system). Replaces: WellSchur::build / buildInPlace (engine/src/bsr.cpp:733-971) feeding
 * GpuBlockSolver::solve. */
int rsg_set_jacobian(rsg_solver* h, int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw);
int rsg_set_jacobian_batch(rsg_solver* h, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                           const int* const* col, const double* const* val);
int rsg_set_jacobian_device(rsg_solver* h, int nrows, const int* rowPtr, const int* col, const double* d_val, int na, int nv, int nw);

/* Solve after rsg_set_jacobian* and rsg_setup with the full right-hand side (per system: na*nv cell entries, then nw
 * well entries; systems concatenated) and the full solution out (BHPs recovered on the device). Host vectors, or
 * device vectors for the _device form. Replaces: WellSchur::reduceRhs + the block solve + WellSchur::recover
 * (engine/src/bsr.cpp:973-990). */
int rsg_solve_jacobian(rsg_solver* h, const double* b, double* x, double tol, int maxIt, int* iterations, double* relres);
int rsg_solve_jacobian_device(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres);

/* The current block system (after rsg_set_matrix / set_batch / set_jacobian) in the caller's row order: rowPtr[n+1],
 * col[nnzb] (columns of the concatenated block-diagonal batch), val[nnzb*nb*nb]; any pointer may be NULL. Sizes from
 * rsg_matrix_size. No reference counterpart (the reduced system of ressim::WellSchur::reduced(), bsr.h). */
int rsg_get_matrix(rsg_solver* h, int* rowPtr, int* col, double* val);
int rsg_matrix_size(rsg_solver* h, int* n, long long* nnzb);

/* Upload a batch of independent systems (uneven sizes) that are solved together; system s has
 * n[s] block rows. Arrays are host pointers, one per system. Batches take nb = 3 (a single system of another block
 * size, nsys = 1, goes to the block-size-generic path as in rsg_set_matrix). */
int rsg_set_batch(rsg_solver* h, int nsys, int nb, const int* n, const int* const* rowPtr, const int* const* col,
                  const double* const* val);

/* Preconditioner set-up on the device: BILU0 factorisation (and, for CPR, the pressure matrix, the AMG
 * hierarchy and its refresh). acc: optional accumulation blocks (n*nb*nb per system, concatenated) for
 * true-IMPES weights, or NULL for quasi-IMPES (Jacobian diagonal block).
 * Replaces: BILU0::factor (engine/src/bsr.cpp:347-435), BlockCPR::setup (engine/src/bsr.cpp:993-1059). */
int rsg_setup(rsg_solver* h, const double* acc);

/* Solve A x = b from x0 = 0 with host vectors (copied in and out on the handle's stream, timed inside).
 * For a batch, b and x are the concatenation of the systems' vectors.
 * Returns RSG_OK when converged, RSG_ENOTCONV when the iteration limit was hit, or a negative error.
 * Replaces: GpuBlockSolver::solve (engine/include/ressim/bsr.h:147) and bicgstab / gmres with the
 * set-up preconditioner (engine/include/ressim/linsolve.h:99-102). */
int rsg_solve(rsg_solver* h, const double* b, double* x, double tol, int maxIt, int* iterations, double* relres);

/* Same with device-resident vectors (b, x: device pointers of n*nb float64 on the handle's device). */
int rsg_solve_device(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres);

/* FP64 iterative refinement (defect correction) around this handle's solver, per system of the batch, with host
 * vectors: x = 0, r = b; while ||r|| / ||b|| > tol and at most maxOuter times, solve A d = r with the handle's
 * preconditioned Krylov method (typically the RSG_MIXED_F32 precision form) to innerTol = clamp(10 tol, 1e-4, 1e-2) in at
 * most innerIt iterations, then x += d and r = b - A x, the SpMV, residual and norms in FP64 on the device. Iterations
 * (rsg_batch_results) are the sums of the inner iterations; the residual reported is the final FP64 one.
 * Returns RSG_OK when every system is within tol, RSG_ENOTCONV otherwise.
 * Replaces: refineWithDevice (engine/src/bsr.cpp:1373-1396) with this handle as its inner device solver. */
int rsg_solve_refined(rsg_solver* h, const double* b, double* x, double tol, int maxOuter, int innerIt, int* iterations,
                      double* relres);

/* Per-system results of the last (batched) solve: its[nsys], relres[nsys] (host arrays, may be NULL). */
int rsg_batch_results(rsg_solver* h, int* its, double* relres, double* true_relres);
/* Per system of the last solve: RSG_OK (converged), RSG_ENOTCONV or RSG_EBREAKDOWN. */
int rsg_batch_status(rsg_solver* h, int* status);
/* CPR: sizes of the pressure hierarchy after rsg_setup, summed over the systems of the batch. For level l < returned
   count (at most maxlev): rows[l] and nnz[l] of the level matrices A_l (rows of a system's coarsest level
   included); *dense = entries of the coarsest levels kept dense (sum of m^2). Returns the number of levels, or -1
   (no CPR hierarchy). Replaces AMG::levels / coarsestSize / operatorComplexity (engine/include/ressim/
   linsolve.h:54-56) for the device hierarchy, and lets a caller size the algorithmic bytes of an application. */
int rsg_amg_level_sizes(rsg_solver* h, int maxlev, long long* rows, long long* nnz, long long* dense);

/* y = A x with host / device vectors. Replaces BSR::spmv (engine/src/bsr.cpp:109-126). */
int rsg_spmv(rsg_solver* h, const double* x, double* y);
int rsg_spmv_device(rsg_solver* h, const double* d_x, double* d_y);

/* z = M^-1 r with the set-up preconditioner (host vectors). Replaces Preconditioner::apply for BILU0 /
 * BlockCPR (engine/src/bsr.cpp:437-596, 1061-1084). */
int rsg_precond_apply(rsg_solver* h, const double* r, double* z);

/* Same with device vectors (no synchronisation: ordered on the handle's stream). */
int rsg_precond_apply_device(rsg_solver* h, const double* d_r, double* d_z);

/* Copy the BILU0 factors (L strictly lower, U_ii^-1 on the diagonal, U upper, in the matrix's own pattern and
 * block order -- the storage of ressim::BILU0, engine/src/bsr.cpp:183-215); FP32 factors of the mixed forms are
 * widened exactly. */
int rsg_get_factors(rsg_solver* h, double* lu);

/* Timing probes for benchmarks (no counterpart in the reference): launch the internal SpMV / the preconditioner
 * `reps` times on the handle's own device vectors, asynchronously on its stream, without any copy around them. */
int rsg_spmv_level_probe(rsg_solver* h, int reps);
int rsg_precond_level_probe(rsg_solver* h, int reps);

/* Allocation-free fused block SpMV and inner product: d_y = A d_x and *d_dot = <d_w, d_y>, nb = 3, all pointers
 * device pointers owned by the caller, launched asynchronously on `stream` (a cudaStream_t; NULL = legacy default).
 * No counterpart in the reference: it exists for callers that cannot allocate device memory during a solve --
 * hosts that hand the whole device memory to their own allocator up front (a simulator or ensemble driver that
 * reserves its HBM budget at start-up) or that must not let a library call cudaMalloc, which may synchronise the
 * device and stall their other streams. Its scratch (per-tile partial sums and an arrival counter) is a fixed
 * 129 KiB array in the library's device memory, present on every device that loads the library; hence the limit of
 * n <= 4,194,304 block rows (larger n returns RSG_EINVAL). The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress): make that first call before any stream capture. All calls share the array; the
 * call clears its counter first, but calls that overlap on the GPU race: order them on one stream. d_y must not
 * alias d_x or d_w (RSG_EINVAL). The looked-up address does not survive cudaDeviceReset: do not call this entry point
 * again on a device the process has reset. It calls no cudaMalloc / cudaFree or other allocating routine. */
int rsg_spmv_dot_noalloc(int n, int nb, const int* d_rowPtr, const int* d_col, const double* d_val, const double* d_x,
                         double* d_y, const double* d_w, double* d_dot, void* stream);

/* Statistics of the last setup / solve. */
int rsg_get_stats(rsg_solver* h, rsg_stats* st);

/* The launch shapes in use after rsg_setup and how they were chosen, as text ("vcycle_form=3 cpr2_threads=256
 * source=tuned ..." with the timed candidates), written NUL-terminated into buf (at most len bytes). No counterpart in
 * the reference, whose device kernels have fixed 64-thread groups (app/src/gpu_compute.cpp:57-80). */
int rsg_tuning(rsg_solver* h, char* buf, int len);

/* Handle's CUDA stream (cudaStream_t as void*), for callers that order their own work with it. */
void* rsg_stream(rsg_solver* h);

/* Well Schur complement on the host (pattern + values), the reduction the engine performs before calling
 * the solver: A is the scalar CSR Jacobian with na*nv cell rows followed by nw well (BHP) rows.
 * First call with sRowPtr == NULL to get the block count in *nnzb; then with arrays of that size.
 * Returns RSG_EINVAL when a well row has no usable BHP derivative or couples wells (the engine then keeps the
 * full system). Replaces WellSchur::build / reduceRhs (engine/src/bsr.cpp:733-840, 973-980). */
int rsg_wellschur_reduce(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                         const double* b, int* nnzb, int* sRowPtr, int* sCol, double* sVal, double* bc);
/* x = [xc ; Dww^-1 (b_w - Awc xc)]. Replaces WellSchur::recover (engine/src/bsr.cpp:982-990). */
int rsg_wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                          const double* b, const double* xc, double* x);

/* ---- Serving form: continuous batching of independent Newton systems (the "batched/serving variants
 * rsg_submit / rsg_poll" of the reference's block-solver boundary; no reference implementation exists).
 * A server runs `slots` workers, each with its own solver handle and CUDA stream. Requests are admitted in
 * arrival order as soon as a slot is free and their estimated device bytes fit the memory budget, so work that
 * arrives while others are on the GPU overlaps with them on the device. Matrices, factors and Krylov state stay
 * resident in HBM for the life of a request; afterwards its slot keeps the plan resident (counted against the
 * budget, released when an admission needs the room), so that the next request with the same pattern uploads values
 * only, as the engine reuses a pattern's plan (engine/src/bsr.cpp:759-769). Every request is solved exactly as it
 * would be alone (deterministic kernels, a plan that depends on the pattern only): the result does not depend on
 * the mix. */
typedef struct rsg_server rsg_server;

typedef struct rsg_result {
    int status;               /* RSG_OK, RSG_ENOTCONV or a negative error of the request */
    int iterations;
    double rel_residual;      /* recursive (Krylov) relative residual */
    double true_rel_residual; /* ||b - A x|| / ||b|| in FP64 */
    double queue_ms;          /* submit -> admitted */
    double run_ms;            /* admitted -> done (upload, set-up, solve, download) */
    double total_ms;          /* submit -> done */
    size_t device_bytes;      /* device memory the request held */
    double start_ms, end_ms;  /* admitted / done, ms since the server was created (one clock for all requests) */
    int slot;                 /* worker that ran it */
    int precond;              /* preconditioner used (RSG_PREC_*; CPR requests whose pattern is not structurally symmetric run BILU0) */
    int batch;                /* requests solved together in the request's launch (small systems are batched) */
} rsg_result;

/* opts: solver options of every slot (device, precision, preconditioner, Krylov method); slots >= 1;
 * mem_budget: bytes of device memory the admitted requests may hold together (0 = no limit). */
int rsg_server_create(rsg_server** s, const rsg_options* opts, int slots, size_t mem_budget);
/* Waits for the requests in flight, drops the queued ones, frees everything. */
int rsg_server_destroy(rsg_server* s);
/* Copies one system (n block rows, BSR with nb x nb blocks) and its right-hand side into the queue and returns
 * the request id (>= 0), or RSG_ENOMEM when its estimated footprint exceeds the whole budget. */
long long rsg_submit(rsg_server* s, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b,
                     double tol, int maxIt);
/* rsg_submit without the copy: the server reads the caller's rowPtr, col, val and b in place, so they must stay
 * allocated and unchanged until rsg_poll has returned the request's result (or rsg_server_destroy has returned).
 * For a caller that keeps its systems anyway -- a simulator's Jacobians, an ensemble's realisations at a step --
 * this saves a host copy of every matrix (at 64 systems of 11k block rows, 357 MB per step). Same result, bit for
 * bit, as rsg_submit. */
long long rsg_submit_view(rsg_server* s, int n, int nb, const int* rowPtr, const int* col, const double* val,
                          const double* b, double tol, int maxIt);
/* 1: request finished (x: n*nb doubles, res filled; the request is retired), 0: still queued or running (wait = 0),
 * negative: unknown id. wait != 0 blocks until the request finishes. */
int rsg_poll(rsg_server* s, long long id, int wait, double* x, rsg_result* res);
/* The admission figure: estimated device bytes of one request of n block rows and nnzb blocks under opts. */
size_t rsg_request_bytes(const rsg_options* opts, int n, long long nnzb);
/* hold != 0: admit nothing until called again with hold = 0 (requests keep queuing); a caller that hands over a
 * batch of systems at once (the realisations of an ensemble at a common time step) holds admission while it submits
 * them, so that they are admitted together and run as one batched solve. */
int rsg_server_hold(rsg_server* s, int hold);
/* Requests queued / running and device bytes counted against the budget right now: the admitted requests' estimates
 * plus the plans idle slots keep resident for the next request with the same pattern (released first when an
 * admission needs their room). */
int rsg_server_load(rsg_server* s, int* queued, int* running, size_t* bytes_in_use);

/* ---- Black-oil Jacobian assembly on the device: the reservoir part of the engine's Newton system, written straight
 * into device memory in the engine's scalar Jacobian layout, so that a Newton step uploads the state (about 50 bytes
 * per cell) instead of the matrix (about 500 bytes per cell) and hands the result to rsg_set_jacobian_device.
 * Replaces Simulator::evalAll / evalCell (engine/src/simulator.cpp:2133-2276, 2429-2459), the cell loop of
 * Simulator::assemble (:2500-2686) and its row scaling dt / PV (:3010-3032), bit for bit, for the standard black-oil
 * model: water (PVTW), live oil (saturated nodes + undersaturated ratio tables), dry gas, rock compressibility,
 * unscaled SWOF / SGOF tables, the ECLIPSE default three-phase oil kr, gravity, one PVT and one saturation region.
 * Other model options are rejected with RSG_EINVAL. The wells remain the caller's (the engine's well loop,
 * simulator.cpp:2692-2954): their terms are passed as addends. */
typedef struct rsg_table {
    int n;                    /* rows (0 = absent) */
    const double* x;          /* abscissae, non-decreasing */
    const double* y;
    int clamp;                /* 1: constant beyond the ends (saturation tables); 0: linear extrapolation */
} rsg_table;                  /* ressim::Table1D, engine/include/ressim/fluid.h:10-17 */

typedef struct rsg_bo_grid {
    int na;                   /* active cells */
    int nv;                   /* unknowns per cell (3: p, Sw, x) */
    int nconn;                /* connections */
    const int* adj_start;     /* [na+1] cell c's connections are adj_start[c] .. adj_start[c+1]-1 */
    const int* adj_nbr;       /* [adj_start[na]] the neighbour cell of each */
    const int* adj_conn;      /* [adj_start[na]] the connection index of each */
    const int* conn_a;        /* [nconn] first cell of each connection (dDepth is depth(b) - depth(a)) */
    const double* conn_trans; /* [nconn] transmissibility */
    const double* conn_ddepth;/* [nconn] */
    const double* pore_vol;   /* [na] pore volume at the reference pressure */
    double gravity;           /* pressure gradient per density and depth (ressim::Units::gravity) */
    int i_sw, i_x;            /* unknown slots of Sw and of x (Sg / Rs / Rv): 1 and 2 in either order (p is slot 0) */
    int eq[3];                /* equation offset of the water, oil and gas balances */
} rsg_bo_grid;                /* ressim::Grid connections / adjacency, engine/include/ressim/grid.h:14-54 */

typedef struct rsg_bo_fluid {
    int water, oil, gas, live, vap;  /* phases; dissolved gas; vaporised oil (must be 0) */
    double pvtw[5];           /* reference pressure, Bw, cw, water viscosity, viscosibility */
    double rock[2];           /* reference pressure, rock compressibility */
    double rho_sc[3];         /* surface densities: oil, water, gas */
    double gas_factor;        /* gas volume unit conversion (ressim::FluidModel::gasFactor) */
    rsg_table rs_of_p, pb_of_rs;     /* saturated Rs(p) and bubble point pb(Rs) */
    rsg_table dead_b, dead_bmu;      /* dead oil 1/Bo, 1/(Bo mu) (unused with live oil) */
    rsg_table gas_b, gas_bmu;        /* dry gas 1/Bg, 1/(Bg mu) vs p */
    int nsat;                 /* live oil: saturated nodes */
    const double* sat_rs;     /* [nsat] Rs of each node */
    const double* sat_b;      /* [nsat] 1/Bo at saturation */
    const double* sat_bmu;    /* [nsat] 1/(Bo mu) at saturation */
    const rsg_table* under_b;   /* [nsat] ratio (1/Bo) / (1/Bo)_sat vs p - pb */
    const rsg_table* under_bmu; /* [nsat] the same for 1/(Bo mu) */
} rsg_bo_fluid;               /* the tables of ressim::FluidModel after setup, engine/include/ressim/fluid.h:60-73 */

typedef struct rsg_bo_satfun {
    rsg_table krw, krow, pcow;       /* SWOF columns vs Sw */
    rsg_table krg, krog, pcog;       /* SGOF columns vs Sg */
    double swco;              /* connate water (first SWOF row) */
    int kro_model;            /* 0: ECLIPSE default (the only one supported) */
    int water, gas;           /* two-phase systems present */
    int three_point;          /* three-point end-point scaling (must be 0) */
} rsg_bo_satfun;              /* ressim::SatFunctions tables, engine/include/ressim/fluid.h:76-124 */

typedef struct rsg_bo_assembler rsg_bo_assembler;

/* Plan an assembler for one grid on `device`: checks the model options and that J_rowPtr / J_col (nrows = na*nv + nw
 * rows, host arrays) are the engine's scalar Jacobian pattern (Simulator::buildPattern, engine/src/simulator.cpp:
 * 465-510: cell row a*nv+e holds the blocks of the cell and its neighbours in column order, then its well columns;
 * then one row per well), and uploads the grid and tables. */
int rsg_bo_create(rsg_bo_assembler** h, const rsg_bo_grid* grid, const rsg_bo_fluid* fluid, const rsg_bo_satfun* sat,
                  int nrows, int nw, const int* J_rowPtr, const int* J_col, int device);
/* Assemble J (d_J: the pattern's J_rowPtr[nrows] values) and R (d_R: nrows) at the state d_p, d_sw, d_x (na doubles
 * each), d_state (na bytes: 0 no free gas, x = Rs; 1 oil and gas, x = Sg; 2 no oil, x = Rv) with the old
 * accumulations d_acc_old (na*3: water, oil, gas) and step dt; all device pointers. The well terms are host lists:
 * J[add_pos[k]] += add_val[k] and R[radd_pos[k]] += radd_val[k], applied after the reservoir terms and before the
 * row scaling, in list order for entries at the same position -- the engine's well loop's additions; every well
 * row starts from zero and is not scaled. Asynchronous on `stream` (a cudaStream_t; NULL = the legacy default
 * stream). The assembler's scratch is shared by its calls: each call waits for the previous call's work, whatever
 * stream that ran on, and rsg_bo_destroy for the last one's. */
int rsg_bo_assemble(rsg_bo_assembler* h, const double* d_p, const double* d_sw, const double* d_x, const unsigned char* d_state,
                    const double* d_acc_old, double dt, int nadd, const long long* add_pos, const double* add_val, int nradd,
                    const int* radd_pos, const double* radd_val, double* d_J, double* d_R, void* stream);
/* The same with host vectors: the state in, J and R out (copied through buffers the assembler keeps on its device;
 * synchronous). */
int rsg_bo_assemble_host(rsg_bo_assembler* h, const double* p, const double* sw, const double* x, const unsigned char* state,
                         const double* acc_old, double dt, int nadd, const long long* add_pos, const double* add_val, int nradd,
                         const int* radd_pos, const double* radd_val, double* J, double* R);
int rsg_bo_destroy(rsg_bo_assembler* h);

#ifdef __cplusplus
}
#endif
#endif

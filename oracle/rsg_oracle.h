/* CPU restatement of ResSim Studio's Newton linear-solve path: TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle (checker) for the GB300 solver in ressim_gb300/. It is a plain-C restatement of the
 * reference algorithms, written from their published behaviour; every function names the reference
 * file:line it follows. Only the tests, the smoke check and the CPU-baseline leg of bench.py may load it;
 * the product path never calls it.
 *
 * Parity pinning: tests/test_oracle.py checks every entry point against golden vectors produced by the
 * reference engine itself (tests/golden/, generated by tests/golden/make_golden.py through
 * oracle/ref_shim.cpp linked with the reference engine compiled from its sources by oracle/Makefile.ref).
 *
 * Conventions: BSR matrices are (n block rows, nb, rowPtr[n+1], col[nnzb] sorted per row, val[nnzb*nb*nb]
 * row-major blocks, row = equation, column = unknown); vectors are interleaved per cell.
 */
#ifndef RSG_ORACLE_H
#define RSG_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

void orc_set_threads(int n);
int orc_threads(void);

/* dense nb x nb block inversion, Gauss-Jordan with partial pivoting (engine/src/bsr.cpp:67-87) */
int orc_invert_block(double* a, int nb);

/* y = A x (engine/src/bsr.cpp:109-126) */
void orc_bsr_spmv(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* x, double* y);
/* y = A x with float values and float vectors, float accumulation (engine/src/bsr.cpp:1137-1146) */
void orc_bsr_spmv_f(int n, int nb, const int* rowPtr, const int* col, const float* val, const float* x, float* y);

/* natural-order block ILU(0) (engine/src/bsr.cpp:183-215, bilu0InPlace :265-268); lu gets L (strict lower),
 * U_ii^-1 (diagonal), U (upper) in A's pattern. Returns the number of regularised pivot blocks. */
int orc_bilu0_factor(int n, int nb, const int* rowPtr, const int* col, const double* val, double* lu);
/* C45 lean factorisation: double scratch row, float storage (engine/src/bsr.cpp:219-263) */
int orc_bilu0_factor_lean(int n, int nb, const int* rowPtr, const int* col, const double* val, float* luf);
/* all-FP32 elimination, FP64 pivot inversion (the device's precision form; returns the regularised block count) */
/* 1: the AMG smoother is the multicolour Gauss-Seidel of the device's FP32 precision forms (test switch; 0 = the
 * reference's natural-order smoother) */
void orc_set_mc_smoother(int on);
int orc_bilu0_factor_f32(int n, int nb, const int* rowPtr, const int* col, const double* val, float* luf);
/* z = U^-1 L^-1 r, serial sweeps (engine/src/bsr.cpp:565-596) */
void orc_bilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* lu, const double* r, double* z);
/* float factors, double vectors and accumulation (C38/C45, engine/src/bsr.cpp:500-522) */
void orc_bilu0_apply_fd(int n, int nb, const int* rowPtr, const int* col, const float* luf, const double* r, double* z);
/* float factors, float vectors, float accumulation (BILU0f, engine/src/bsr.cpp:1100-1121) */
void orc_bilu0_apply_ff(int n, int nb, const int* rowPtr, const int* col, const float* luf, const double* r, double* z);

/* forward (L) or backward (U) level sets (engine/src/bsr.cpp:270-293): ord[n], start[nl+1]; returns nl */
int orc_level_sets(int n, const int* rowPtr, const int* col, int forward, int* ord, int* start);

/* ---- aggregation AMG (engine/src/amg.cpp:137-337) */
typedef struct orc_amg orc_amg;
orc_amg* orc_amg_setup(int n, const int* rowPtr, const int* col, const double* val);
int orc_amg_refresh(orc_amg* h, int n, const int* rowPtr, const int* col, const double* val);
void orc_amg_apply(const orc_amg* h, const double* r, double* z);
int orc_amg_levels(const orc_amg* h);
int orc_amg_level_info(const orc_amg* h, int l, int* rows, int* nnz);
/* level l matrix (CSR) and aggregate map (agg[i] = coarse index of fine row i, -1 on the coarsest level) */
int orc_amg_level_get(const orc_amg* h, int l, int* rowPtr, int* col, double* val, int* agg);
void orc_amg_free(orc_amg* h);

/* ---- block CPR (engine/src/bsr.cpp:993-1084). acc: optional accumulation blocks (n*nb*nb).
 * lean != 0: the BILU0 second stage keeps float factors (C45 lean storage, double vectors). */
typedef struct orc_cpr orc_cpr;
orc_cpr* orc_cpr_setup(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int lean);
void orc_cpr_apply(const orc_cpr* h, const double* r, double* z);
const double* orc_cpr_weights(const orc_cpr* h);
const orc_amg* orc_cpr_amg(const orc_cpr* h);
void orc_cpr_free(orc_cpr* h);

/* multicolour BILU0 (engine/src/bsr.cpp:599-730): colouring (colour per cell, perm: new index -> cell; returns the
 * number of colours) and z = M^-1 r of the colour-permuted block ILU(0) */
int orc_colour_blocks(int n, const int* rowPtr, const int* col, int* colour, int* perm);
int orc_mcbilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* r, double* z);

/* GPU-shaped float CPR-AMG (engine/src/bsr.cpp:1217-1371): r, z float of size n*nb */
typedef struct orc_devcpr orc_devcpr;
orc_devcpr* orc_devcpr_setup(int n, int nb, const int* rowPtr, const int* col, const double* val);
void orc_devcpr_apply(const orc_devcpr* h, const float* r, float* z);
int orc_devcpr_levels(const orc_devcpr* h);
int orc_devcpr_has_inverse(const orc_devcpr* h);
void orc_devcpr_free(orc_devcpr* h);

/* ---- Krylov (engine/src/linsolve.cpp:159-273). Callback operator / preconditioner. */
typedef void (*orc_apply_fn)(void* ctx, const double* x, double* y);
int orc_bicgstab(int N, orc_apply_fn A, void* actx, orc_apply_fn M, void* mctx, const double* b, double* x, double tol, int maxIt,
                 int* its, double* relres);
int orc_gmres(int N, orc_apply_fn A, void* actx, orc_apply_fn M, void* mctx, const double* b, double* x, double tol, int maxIt,
              int restart, int* its, double* relres);

/* ---- one-call drivers used by the tests and the CPU baseline
 * prec: 0 = BILU0, 1 = BlockCPR (AMG + BILU0), 2 = BILU0 with lean float factors, 3 = BlockCPR with lean float factors
 * method: 0 = BiCGSTAB, 1 = GMRES(restart). Returns 1 when converged. */
int orc_prec_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, const double* r,
                   double* z);
int orc_solve(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, int method, int restart,
              const double* b, double* x, double tol, int maxIt, int* its, double* relres);
/* timing split of orc_solve: seconds of preconditioner set-up and of the Krylov solve */
int orc_solve_timed(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, int method,
                    int restart, const double* b, double* x, double tol, int maxIt, int* its, double* relres, double* setupSec,
                    double* solveSec);

/* ---- float device-algorithm emulation wrapped in double refinement
 * (CpuFloatBlockSolver::solve, engine/src/bsr.cpp:1130-1215; refineWithDevice :1373-1396) */
int orc_refine_float(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b, double* x, double tol,
                     int maxOuter, int innerIt, int* its, double* relres);

/* ---- well Schur complement (engine/src/bsr.cpp:733-840, 973-990)
 * scalar CSR A (nrows = na*nv + nw) -> reduced BSR S; returns nnzb (>0), 0 when the elimination is impossible,
 * or -needed when the output capacity (capBlocks) is too small. */
int orc_wellschur(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                  int capBlocks, int* sRowPtr, int* sCol, double* sVal, double* bc);
int orc_wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                          const double* xc, double* x);

#ifdef __cplusplus
}
#endif
#endif

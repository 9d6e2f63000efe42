// Internal declarations of the rsg library (host plan structures, device buffers, kernel launchers).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

namespace rsg {

// Host threads the plan of a large pattern may use.
inline int host_threads() { return std::max(1, int(std::thread::hardware_concurrency())); }

// Host plan work on large patterns: fn(lo, hi) over [0, n) in up to `threads` contiguous ranges, one thread each
// (one range on the caller's thread when threads <= 1 or n is below minPerThread per thread). Every use writes
// disjoint outputs per index, so the result does not depend on the split.
template <class Fn>
void parallel_ranges(int n, int threads, Fn&& fn, int minPerThread = 32768) {
    const int np = std::max(1, std::min(threads, n / std::max(1, minPerThread)));
    if (np <= 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(size_t(np));
    for (int w = 0; w < np; ++w) {
        auto range = [&fn, n, np, w] { fn(int((long long)n * w / np), int((long long)n * (w + 1) / np)); };
        try {
            pool.emplace_back(range);
        } catch (const std::system_error&) {   // no thread to be had: this range on the caller's thread
            range();
        }
    }
    for (auto& t : pool) t.join();
}

constexpr int NB = 3;                 // block size of the black-oil system (p, Sw, x_g)
constexpr int NB2 = NB * NB;
constexpr int TILE_ROWS = 256;        // block rows per tile of the tile kernels (64-row steps, 3 threads per block row)
constexpr int TILE_THREADS = TILE_ROWS * NB;
constexpr int MAX_DOTS = 4;           // partial sums per tile in the fused reductions
constexpr int SLOTS = 3;              // factor block slots per row and triangle (7-point stencil: 3 lower, 3 upper)
constexpr int LREC = 28;              // factor values per row record of L: SLOTS blocks + 1 pad (16-byte multiple)
constexpr int UREC = 36;              // per row record of U and D: SLOTS blocks + the inverted diagonal block
constexpr int SPREC = 24;             // CPR pressure columns of S per row: (SLOTS + 1 + SLOTS) blocks x 3 + 3 pad
constexpr int OV_CHUNK = 4;           // overflow entries a sweep reads at once (the lists are padded to allow it)

// Krylov status per system (device int)
enum : int { ST_RUNNING = 0, ST_CONV = 1, ST_BREAKDOWN = 2, ST_MAXIT = 3, ST_CYCLE = 4 /* GMRES: restart cycle ended */,
             ST_DIVERGED = 5 /* FP32 preconditioner: the residual grew past the divergence guard */ };

// Error bits written by kernels (device int, OR-ed)
enum : int { ERR_TIMEOUT = 1, ERR_NONFINITE = 2 };

// Per-system Krylov scalars, resident on the device (no host round trip per inner product).
struct KScal {
    double rho, alpha, omega, beta;   // BiCGSTAB recurrences (engine/src/linsolve.cpp:166-211)
    double bn;                        // ||b||
    double relres;                    // recursive relative residual of the last completed iteration
    double sn;                        // ||s|| of the current iteration
    int status, its, maxit, guard;    // guard: stop when the residual diverges (FP32 preconditioner; the solve escalates)
    double tol;
    double hn;                        // GMRES: norm of the last orthogonalised vector; BiCGSTAB guard: best residual
    int gj, gend;                     // GMRES: inner steps of the current cycle (BiCGSTAB guard: iteration of the best
                                      // residual); cycle ended by convergence
};

// Host-built, pattern-only plan of the device solve. Everything on the device runs in "level space": inside
// every system the block rows are renumbered by (forward level, row) -- perm[k] = original row of level-space
// row k -- and the entries of a row keep their original order, so rows of a level are contiguous while every
// row is still eliminated and swept in the reference's arithmetic order.
struct HostPlan {
    int n = 0, nnzb = 0, nsys = 1;
    std::vector<int> rowPtr0, col0;   // original pattern (pattern-reuse test)
    std::vector<int> perm, iperm;     // level-space row -> original row, and back
    std::vector<int> valSrc;          // level-space block -> original block
    std::vector<int> rowPtr, col, diag;   // level-space pattern
    std::vector<int> ford, bord;      // claim orders: forward (by L level) and backward (by U level)
    int nlevF = 0, nlevB = 0;
    std::vector<int> elimPtr;         // per block entry p (lower entries only non-empty): range in elimT/elimQ
    std::vector<int> elimT, elimQ;    // target block t in row i, U block q in row k: A_it -= L_ik U_kq
    std::vector<int> rowSys;          // system of every block row
    std::vector<int> sysRow0;         // first block row of every system (nsys + 1)
    std::vector<int> tileRow0;        // first row of every tile (ntiles + 1); tiles never cross systems
    std::vector<int> tileSys;         // system of every tile
    std::vector<int> sysTile0;        // first tile of every system (nsys + 1)
    bool symmetric = true;
    // lvlStart[sysLvl0[s] + l] is the first level-space row of level l of system s (nl_s + 1 entries per system)
    std::vector<int> lvlStart, sysLvl0;
    // Slot storage of the factors for the thread-block sweeps (level-space row order). Every row k has SLOTS
    // strict-lower and SLOTS strict-upper block slots holding its first blocks of that part in row order; a row's
    // further blocks continue in an overflow list, terminated by a column of -1.
    //   Lslot[4k + j], j < SLOTS: local column of slot j (-1 empty); Lslot[4k + 3]: overflow start (-1 none)
    //   LslotSrc[SLOTS k + j]: source block position of slot j (-1 empty)
    //   LovCol / LovSrc: overflow entries (local column, source block; -1 / -1 ends a row's list). OV_CHUNK - 1
    //   further -1 / -1 entries follow the last list, so OV_CHUNK entries from any position up to a terminator
    //   are readable.
    std::vector<int> Lslot, LslotSrc, LovCol, LovSrc;
    std::vector<int> Uslot, UslotSrc, UovCol, UovSrc;
    std::vector<int> Dsrc;               // diagonal (U_ii^-1) block of row k
    int maxSysRows = 0;
};

struct PrecDev;
struct DevPlan;
struct SweepState;
// Builds the plan of a (block-diagonal batch of) BSR pattern(s). Returns false with a message on bad input.
// True when a batch (per system: n[s] rows, rowPtr[s], col[s]) has exactly the pattern the plan was built from,
// compared in place (no concatenated copy).
bool same_batch_pattern(const HostPlan& P, int nsys, const int* n, const int* const* rowPtr, const int* const* col);
// threads: host threads for the row-parallel parts of a large pattern (the plan is the same for any count)
bool build_plan(HostPlan& P, int nsys, const std::vector<int>& sysRow0, const std::vector<int>& rowPtr,
                const std::vector<int>& col, std::string& err, int threads = 1);
// multicolour ordering of every system (MCBILU0, engine/src/bsr.cpp:599-653): permuted pattern and the original row /
// block of every permuted row / block
void multicolour_batch(int nsys, const std::vector<int>& sysRow0, const std::vector<int>& rp, const std::vector<int>& ci,
                       std::vector<int>& rp2, std::vector<int>& ci2, std::vector<int>& rowOrig, std::vector<int>& blockOrig);

// ---- CPR pressure AMG of one system (host plan; engine/src/amg.cpp:137-295). Every level is kept in its own level
// space: rows renumbered by forward Gauss-Seidel level, entries of a row in their natural order.
struct AmgLevel {
    int n = 0;
    std::vector<int> rp, ci, diag;     // level-space CSR and diagonal positions
    std::vector<int> lvlStart;         // forward GS levels (level-space row ranges)
    std::vector<int> perm, iperm;      // level space <-> natural numbering of the level
    std::vector<double> val;           // values at plan time (the device recomputes them on every set-up)
    std::vector<int> agg;              // all but the coarsest: level-space row -> coarse level-space row
    std::vector<int> memPtr, mem;      // l >= 1: finer level-space members of each row, in restriction order
    std::vector<int> apPtr, apSrc;     // l >= 1: AP entries <- finer-level positions (Galerkin, first product)
    std::vector<int> acPtr, acSrc;     // l >= 1: this level's entries <- AP entries (Galerkin, second product)
};
struct SysAmg {
    std::vector<AmgLevel> lv;
    bool coarseDense = true;           // coarsest level <= 800 rows: dense solve (else 20 symmetric GS sweeps)
};
// threads: host threads for the Galerkin products of the large levels (the result is the same for any count)
bool amg_plan_system(const HostPlan& P, int s, const std::vector<double>& ap0, SysAmg& out, std::string& err, int threads = 1);

// Device AMG of a batch: all arrays concatenated level-major (every system's level 0, then every system's level 1,
// ...); indices inside a (system, level) are local. AmgSysLv[s * maxL + l] describes level l of system s.
struct AmgSysLv {
    int n = 0, nnz = 0, nl = 0;        // rows, entries, forward GS levels (n = 0: level absent)
    int rowOff = 0;                    // rows: x, b, r, diag, agg, diagGlob
    int rpOff = 0;                     // (n + 1) row pointers in rp, (n + 1) member pointers in memPtr
    int entOff = 0;                    // entries: ci, val
    int lvlOff = 0;                    // (nl + 1) GS level boundaries in lvl
    int memOff = 0;                    // fine members of the rows (coarse levels) in mem
    int coarse = 0;                    // 1 on the system's coarsest level
    int dense = 0;                     // coarsest level solved by dense LU (else 20 symmetric GS sweeps)
    int luOff = 0, luRowOff = 0;       // coarsest: dense LU (m*m) and pivots / natural order (m)
    int slotOff = 0, W = 0;            // row slots of the V-cycle (W off-diagonal entries per row at slotOff + W k)
    int locOff = 0;                    // offset of the level's rows inside the system's V-cycle vectors
    int mc = 0;                        // Gauss-Seidel schedule: 0 forward levels (reference order), 1 colours
};
// One phase of the fused V-cycle kernel (the split CPR application in one cooperative launch): the pass it runs
// over every system of the batch and that pass's row ranges and switches (rsg_sweep_cta.cu: vcycle_phases).
enum : int { VP_IN = 0, VP_COLOUR = 1, VP_TAIL = 2, VP_GSGRID = 3, VP_RESID = 4, VP_RESTRICT = 5, VP_COARSE = 6, VP_PROLONG = 7,
             VP_TSP = 8 };
struct VPhase {
    int kind, a, b, c, d, e, f, g;
};
constexpr int AMG_W0 = 8;              // V-cycle row slots on the finest level (7-point pressure matrix)
constexpr int AMG_W1 = 16;             // on the Galerkin levels
struct DevAmg {
    int nsys = 0, maxL = 0;
    int totRows = 0, totEnt = 0, totLu = 0, totLuRows = 0, nAP = 0;
    std::vector<int> levelEntBeg, levelApBeg, levelRowBeg;   // host: per level l, [beg[l], beg[l+1]) ranges
    AmgSysLv* lv = nullptr;
    int *rp = nullptr, *ci = nullptr, *diag = nullptr, *lvl = nullptr;   // rp: (n+1) per (s,l) at rowOff + l
    int *agg = nullptr, *memPtr = nullptr, *mem = nullptr;               // memPtr: (n+1) per coarse (s,l) at rowOff + l
    int *apPtr = nullptr, *apSrc = nullptr, *acPtr = nullptr, *acSrc = nullptr;   // global indices
    int *diagGlob = nullptr;           // global diagonal entry of every row (diagonal fix after the refresh)
    int *luPerm = nullptr, *piv = nullptr;   // coarsest: level space -> natural, LU pivots
    double* val = nullptr;             // entries of every level (level 0 = pressure matrix)
    float* valf = nullptr;             // FP32 copy (mixed V-cycle)
    double* apVal = nullptr;           // AP intermediate of the refresh
    double* lu = nullptr;              // coarsest dense LU (FP64)
    float* luf = nullptr;              // FP32 LU (FP32 precision forms)
    float* invf = nullptr;             // FP32 forms: explicit inverse, column j at luOff + j m in natural row order
    int maxCoarse = 0;                 // largest dense coarsest level (rows)
    double *x = nullptr, *b = nullptr, *r = nullptr;   // V-cycle vectors (every level)
    float *xf = nullptr, *bf = nullptr, *rf = nullptr;
    double* w = nullptr;               // CPR weights, level-space block rows of S (n * 3)
    double* T = nullptr;               // second-stage input t = r - S[:,p] xp (n * 3)
    double* acc = nullptr;             // accumulation blocks gathered into level space (n * 9), optional
    // V-cycle row slots (refreshed from val at every set-up): the first W off-diagonal entries of every row in
    // row order (value, local column; 0 / -1 padding), the diagonal value, and per row {number of entries before
    // the diagonal, off-diagonal entries, entry position where the entries beyond the slots continue, diagonal
    // position} (positions local to the level's entries)
    int totSlots = 0, maxSysAmgRows = 0;
    int maxSysLoRows = 0;              // largest number of rows of one system's levels below the finest
    // Gauss-Seidel schedule per (system, level): rows in processing order (level space; identity for the forward
    // levels of the reference order, colour by colour for the multicolour smoother), boundaries in lvl
    int* gsRows = nullptr;
    int* slotSrc = nullptr;            // global entry of every slot (-1 padding)
    int* slotCol = nullptr;
    int4* rowMeta = nullptr;
    double *slotVal = nullptr, *diagVal = nullptr;
    float *slotValf = nullptr, *diagValf = nullptr;
    int* cin = nullptr;                // coarsest dense level: level-space row feeding position i of the pivoted natural order
    // pressure columns of S per level-space block row in slot order (L slots, diagonal, U slots; SPREC values) and
    // of the overflow blocks (3 values each)
    double *sp = nullptr, *spLov = nullptr, *spUov = nullptr;
    float *spf = nullptr, *spLovf = nullptr, *spUovf = nullptr;
    // grid-wide V-cycle (systems too large for one SM): per AMG row its (system, level) descriptor index s*maxL+l and
    // its wave (forward GS level, or colour: adjacent rows of an earlier wave are updated before it in a forward
    // sweep), sync-free sweep flags (phase 0: the smoothing sweeps, phase 1: the GS solve of a coarsest level
    // without dense LU) and claim counters (per level and phase: forward, backward)
    int* coarse64 = nullptr;           // FP32 forms, per system: 1 = coarsest level solved in FP64 (LU), the FP32 inverse too inexact
    // the GPU-shaped float CPR-AMG (RSG_PREC_CPR_DEVICE): float inverse diagonal of every AMG row, float block-Jacobi
    // inverses (n * 9), per system whether the coarsest inverse exists, the double Gauss-Jordan work matrices
    float* dinvf = nullptr;
    float* bjf = nullptr;
    int* dcOk = nullptr;
    double* dcWork = nullptr;
    size_t* dcWorkOff = nullptr;
    int* rowLv = nullptr;
    int* wave = nullptr;
    int* gsFlag = nullptr;             // 2 x totRows
    unsigned* gsCtr = nullptr;         // maxL x 4
    std::vector<int> coarseGsLevels;   // host: levels that are some system's coarsest without a dense LU
    // multicolour schedule (FP32 forms), grid-wide: per level the rows of every system that smooths it, colour by
    // colour, as {row, first entry, end of entries, diagonal entry} (global indices); colour c of level l at
    // colBeg[l][c] .. colBeg[l][c + 1]. Colours from colTail[l] on hold few rows each (the cliques of perforated
    // cells that the well Schur fill creates) and are swept together by one sync-free pass.
    int4* cdesc = nullptr;
    int* gci = nullptr;                // global column of every entry (rowOff + local column)
    std::vector<std::vector<int>> colBeg;
    std::vector<int> colTail;
    std::vector<int> gsBlocks;         // host: persistent grid of the sync-free Gauss-Seidel sweeps of each level
    bool posOrder = false;             // host: in every row the entries before the diagonal are exactly its earlier-wave neighbours
    // fused V-cycle (split form): the phase table of one application, its grid-barrier counter, and the number of
    // chunks the coarsest explicit-inverse products split into (0: no table; hierarchies with Gauss-Seidel coarsest levels)
    VPhase* phases = nullptr;
    int nPhases = 0;
    unsigned* vbar = nullptr;
    int coarseChunks = 1;
};
// phase table of the fused V-cycle for a built hierarchy (empty when the fused kernel does not apply)
void vcycle_phases(const DevAmg& G, std::vector<VPhase>& out);
// blocks of 4 warps for a sync-free sweep that keeps `inflight` of its levels (avgRows rows each) in flight
int sweep_blocks_for(double avgRows, int inflight);
// CPR set-up kernels (rsg_cpr.cu)
void launch_cpr_weights(const DevPlan& P, const double* val, const double* accLev, double* w, int* nfallback, cudaStream_t st);
void launch_cpr_pressure(const DevPlan& P, const double* val, const double* w, double* ap, cudaStream_t st);
void launch_gather_acc(const DevPlan& P, const double* accOrig, double* accLev, cudaStream_t st);
void launch_amg_refresh(const DevAmg& G, cudaStream_t st);           // Galerkin values of levels >= 1, diagonal fix
void launch_amg_coarse_lu(const DevAmg& G, bool fp32, cudaStream_t st);     // fp32: the LU in FP32 (luf), else FP64 (lu)
void launch_amg_round(const DevAmg& G, cudaStream_t st);             // valf = float(val), luf = float(lu)
void launch_amg_slots(const DevAmg& G, bool fp32, cudaStream_t st);  // V-cycle row slots from val
// pressure columns of S in the slot order of the factors (second stage of the CPR application)
void launch_cpr_sp(const DevPlan& P, const double* val, const DevAmg& G, bool fp32, cudaStream_t st);
// one CPR application per system (thread block per system), fused with the BiCGSTAB input update:
// mode 0 plain (r -> z), 1 p-update, 2 s-update (as the BILU0 sweeps)
void launch_cpr_cta(const DevPlan& P, const PrecDev& M, const DevAmg& G, int mode, bool amgFp32, const double* r, double* pv,
                    const double* v, double* z, const KScal* ks, cudaStream_t st);
// the same application grid-wide for systems of any size (rsg_sweep_cta.cu): input and restriction, the V-cycle one
// level at a time with sync-free Gauss-Seidel sweeps, coarse solve per system, t = r - S[:,p] xp, the grid BILU0
// sweeps, z_p += xp; with M.split the second stage (t, the BILU0 sweeps, z_p += xp) is the thread-block kernel's,
// on the split factors, so that the result is the thread-block application's. Returns the number of kernel launches.
int launch_cpr_grid(const DevPlan& P, const PrecDev& M, const DevAmg& G, int mode, const double* r, double* pv, const double* v,
                    double* z, const KScal* ks, SweepState& S, int* err, cudaStream_t st);
// the reference's GPU-shaped float CPR-AMG (rsg_devcpr.cu): set-up (coarse inverse, inverse diagonals, block
// inverses) after the hierarchy refresh, and one application (mode: plain, p-update, s-update); both return launches
int launch_devcpr_setup(const DevPlan& P, const double* val, DevAmg& G, cudaStream_t st);
int launch_devcpr(const DevPlan& P, const DevAmg& G, const double* val, int mode, const double* r, double* pv, const double* v, double* z,
                  const KScal* ks, cudaStream_t st);
int devcpr_launches(const DevAmg& G);
inline int cpr_grid_launches(const DevAmg& G, bool split = false, int vform = 2) {
    if (split && vform == 1 && G.nPhases > 0) return 2;            // the fused V-cycle and the BILU0 stage
    auto sweeps = [&](int l) {                                     // one sweep: a launch per large colour + the tail, or one
        const int nc = l < int(G.colBeg.size()) ? int(G.colBeg[size_t(l)].size()) - 1 : 0;
        return nc > 0 ? G.colTail[size_t(l)] + (G.colTail[size_t(l)] < nc ? 1 : 0) : 1;
    };
    if (split && vform == 3) return G.maxL > 1 ? 7 + 2 * sweeps(0) : 4;
    int n = (split ? 4 : 6) + 3 * (G.maxL > 1 ? G.maxL - 1 : 0) + 40 * int(G.coarseGsLevels.size());
    for (int l = 0; l + 1 < G.maxL; ++l) n += 2 * sweeps(l);      // pre- and post-smoothing
    return n;
}

// ---- well Schur complement on the device (rsg_wellschur.cu): host plan of a batch of Jacobians with well rows.
// Global indices: Jacobian entries concatenated over the systems (jEnt0), full vectors [cells, wells] per system
// (full0), reduced vectors of the cells (red0), wells (well0), S blocks concatenated per system.
struct WsPlan {
    int nsys = 0, nv = 3;
    std::vector<int> nrows, na, nw;
    std::vector<int> jEnt0, full0, red0, well0;        // per-system offsets (nsys + 1 each)
    std::vector<std::vector<int>> jrp, jci;            // the Jacobian patterns (same-pattern test)
    std::vector<int> redFull;                          // reduced row -> full row
    std::vector<int> cplPos, cplRow, cplWell;          // cell-to-well couplings: Jacobian entry, reduced row, well
    std::vector<int> diagPos, wellFull, wcBeg, wcPos, wcRed, wwBeg, wwPos;   // per well: BHP derivative, full row,
                                                       // cell entries (entry, reduced column), couplings to other wells
    std::vector<unsigned char> mask;                   // nonzero set of the couplings the value maps were built for
    std::vector<std::vector<int>> srp, sci;            // S pattern of every system
    long long nnzbS = 0;
    std::vector<int> sBase;                            // per S value: its Jacobian entry, or -1 (fill)
    std::vector<long long> fillScalar;                 // S values with well terms, and their terms in the engine's order
    std::vector<int> fillBeg, tCw, tDiag, tWc;
    std::vector<int> rBeg, rCw, rDiag, rWellFull;      // right-hand side terms per reduced row
};
struct WsDev {
    int ncpl = 0, nwell = 0, nred = 0, nfill = 0;
    long long nval = 0;
    int *cplPos = nullptr, *diagPos = nullptr, *wcBeg = nullptr, *wcPos = nullptr, *wwBeg = nullptr, *wwPos = nullptr,
        *wcRed = nullptr, *wellFull = nullptr, *redFull = nullptr;
    unsigned char *mask = nullptr, *wellOk = nullptr;
    int* sBase = nullptr;
    long long* fillScalar = nullptr;
    int *fillBeg = nullptr, *tCw = nullptr, *tDiag = nullptr, *tWc = nullptr;
    int *rBeg = nullptr, *rCw = nullptr, *rDiag = nullptr, *rWellFull = nullptr;
};
bool ws_same_pattern(const WsPlan& W, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                     const int* const* col);
bool ws_plan_pattern(WsPlan& W, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                     const int* const* col, std::string& err);
bool ws_plan_values(WsPlan& W, const std::vector<unsigned char>& mask, std::string& err);
// per call: coupling nonzero flags and well checks; S values into sv (S blocks, original order); reduced right-hand
// side; recovery of the full solution
void launch_ws_check(const WsDev& D, const double* jv, cudaStream_t st);
void launch_ws_values(const WsDev& D, const double* jv, double* sv, cudaStream_t st);
void launch_ws_rhs(const WsDev& D, const double* jv, const double* bFull, double* bc, cudaStream_t st);
void launch_ws_recover(const WsDev& D, const double* jv, const double* bFull, const double* xc, double* xFull, cudaStream_t st);

// ---- well Schur complement on the host (engine/src/bsr.cpp:733-840, 973-990)
int wellschur_reduce(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                     const double* b, int* nnzb, int* sRowPtr, int* sCol, double* sVal, double* bc, std::string& err);
int wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                      const double* b, const double* xc, double* x, std::string& err);

// ---- device plan (mirrors HostPlan) and buffers
struct DevPlan {
    int n = 0, nnzb = 0, nsys = 0, ntiles = 0;
    int *rowPtr = nullptr, *col = nullptr, *diag = nullptr;
    int *ford = nullptr, *bord = nullptr;
    int *elimPtr = nullptr, *elimT = nullptr, *elimQ = nullptr;
    int *rowSys = nullptr, *tileRow0 = nullptr, *tileSys = nullptr, *sysTile0 = nullptr, *sysRow0 = nullptr;
    int *perm = nullptr, *valSrc = nullptr;
    int *lvlStart = nullptr, *sysLvl0 = nullptr;
    int4 *Lslot = nullptr, *Uslot = nullptr;
    int *LslotSrc = nullptr, *UslotSrc = nullptr, *LovCol = nullptr, *LovSrc = nullptr, *UovCol = nullptr, *UovSrc = nullptr;
    int* Dsrc = nullptr;
    int2* rowLevel = nullptr;         // level-space row -> (first row of its forward level, rows of that level)
    int nLov = 0, nUov = 0, maxSysRows = 0;
    int sweepBlocks = 0;              // persistent grid of the sync-free sweeps (0: sized from n)
    bool spmvFma = true;              // SpMV with fused multiply-adds (else the reference's rounding, bitwise)
};

// Slot-layout factors for the CTA-per-system sweeps (FP64 or FP32 storage): L = n x LREC, UD = n x UREC,
// Lov / Uov = overflow blocks (9 values each). The records of a forward level (its rows are contiguous in level
// space: [s, s + w)) fill [s * LREC, (s + w) * LREC) of L component-major: value j of row k at s * LREC + j * w + (k - s),
// so the threads of consecutive rows read consecutive words (coalesced) when they load their records; UD likewise.
template <class T>
struct SplitFactors {
    T *L = nullptr, *UD = nullptr, *Lov = nullptr, *Uov = nullptr;
};

struct SweepState {                   // sync-free sweep flags and claim counters
    int *flagF = nullptr, *flagB = nullptr, *flagL = nullptr;
    unsigned *ctr = nullptr;          // [0] forward, [1] backward, [2] factorisation, [3] spare
};

struct ReduceState {                  // fused tile reductions
    double* part = nullptr;           // ntiles * MAX_DOTS
    unsigned* done = nullptr;         // arrival counter of the last-block pattern
    double* sysdot = nullptr;         // nsys * MAX_DOTS (results of the last reduction)
};

// ---- kernel launchers (rsg_kernels.cu)
int device_sm_count();
// level-space gathers / scatters: blocks (9 doubles) by valSrc, vectors (3 doubles per row) by perm
void launch_gather_blocks(const DevPlan& P, const double* src, double* dst, cudaStream_t st);
void launch_gather_vec(const DevPlan& P, const double* orig, double* lev, cudaStream_t st);
void launch_scatter_vec(const DevPlan& P, const double* lev, double* orig, cudaStream_t st);
void launch_factor_f64(const DevPlan& P, const double* val, double* lu, SweepState& S, int epoch, int* nreg, int* err,
                       cudaStream_t st);
void launch_factor_lean(const DevPlan& P, const double* val, float* luf, double* work, SweepState& S, int epoch, int* nreg,
                        int* err, cudaStream_t st);
// z = U^-1 L^-1 r (FP64 factors, FP64 vectors) or with FP32 factors / FP32 vectors and accumulation.
void launch_ilu_apply_f64(const DevPlan& P, const double* lu, const double* r, double* z, SweepState& S, int* err,
                          cudaStream_t st);
void launch_ilu_apply_f32(const DevPlan& P, const float* luf, const double* r, double* z, unsigned long long* yt, SweepState& S,
                          int* err, cudaStream_t st);
// FP32 factors, FP64 vector and accumulation (the reference's float-factor sweeps)
void launch_ilu_apply_mixed(const DevPlan& P, const float* luf, const double* r, double* z, SweepState& S, int* err,
                            cudaStream_t st);
// grid-wide sync-free BILU0 apply z = M^-1 r of the handle's factor kind; systems whose status is not running skip
void launch_ilu_grid_ks(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, SweepState& S, int* err,
                        cudaStream_t st);
void launch_spmv_f64(const DevPlan& P, const double* val, const double* x, double* y, cudaStream_t st);
// x += d over n block rows (3 values each)
void launch_vec_add(int n, double* x, const double* d, cudaStream_t st);
// raise (never lower) a kernel's dynamic shared-memory opt-in on the current device; thread-safe
void raise_smem_limit(const void* fn, int bytes);
// block-Jacobi: dinv = inverse diagonal blocks (FP64), z = dinv r
void launch_block_jacobi_setup(const DevPlan& P, const double* val, double* dinv, int* nreg, cudaStream_t st);
void launch_block_jacobi_apply(const DevPlan& P, const double* dinv, const double* r, double* z, cudaStream_t st);

// BiCGSTAB building blocks (per-system scalars on the device).
struct BicgVecs {
    double *x, *r, *rh, *p, *v, *s, *t, *ph, *sh;
    float* y32;                       // FP32 sweep intermediate of the thread-block sweeps (systems that do not fit on chip)
    unsigned long long* yt;           // the grid-wide all-FP32 sweeps' vector: tagged words {float, sweep tag}
};
void launch_bicg_init(const DevPlan& P, const double* b, BicgVecs& V, KScal* ks, ReduceState& R, double tol, int maxit,
                      int* active, bool guard, bool onlyFailed,
                      cudaStream_t st);
// one BiCGSTAB iteration (engine/src/linsolve.cpp:166-214) with the preconditioner given by prec:
// 0 = BILU0 FP64, 1 = BILU0 FP32 (mixed), 2 = block Jacobi
struct PrecDev {
    int kind = 0;
    const double* lu = nullptr;
    const float* luf = nullptr;
    const double* dinv = nullptr;
    const double* val = nullptr;
    bool cta = false;                 // CTA-per-system level-synchronous sweeps on the split factors
    SplitFactors<double> s64;
    SplitFactors<float> s32;
    size_t smem = 0;                  // dynamic shared memory of the CTA sweep (systems whose vector fits keep it there)
    float* y32 = nullptr;             // all-FP32 sweep vector in global memory (systems that do not fit on chip)
    unsigned long long* yt = nullptr; // grid-wide all-FP32 sweeps: tagged sweep vector
    bool cpr = false;                 // CPR two-stage preconditioner (AMG on the pressure system + BILU0)
    bool devcpr = false;              // the reference's GPU-shaped float CPR-AMG
    bool split = false;               // CPR with cta: V-cycle and second-stage input grid-wide (all systems at once),
                                      // the BILU0 sweeps one thread block per system
    int vform = 2;                    // split CPR V-cycle: 1 fused cooperative kernel, 2 one launch per pass, 3 coarse
                                      // levels one thread block per system
    int cpr2Threads = 256;            // split CPR: threads per block of the BILU0 stage (128, 256 or 512; same results)
    const DevAmg* amg = nullptr;
};
// all-FP32 factorisation (FP32 elimination, FP64 pivot inversion), one thread block per system
void launch_factor_cta_f32(const DevPlan& P, const double* val, float* luf, int* nreg, cudaStream_t st);
// gather the factors (original block layout) into the level-ordered split layout
void launch_pack_f64(const DevPlan& P, const double* lu, SplitFactors<double>& F, cudaStream_t st);
void launch_pack_f32(const DevPlan& P, const float* luf, SplitFactors<float>& F, cudaStream_t st);
// z = M^-1 r with the CTA sweeps (plain input mode); the _ks form skips systems whose status is not running
void launch_ilu_cta_apply(const DevPlan& P, const PrecDev& M, const double* r, double* z, cudaStream_t st);
void launch_ilu_cta_apply_ks(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, cudaStream_t st);
// BiCGSTAB-fused CTA sweeps: input p = r + beta (p - omega v) (pupdate) or s = r - alpha v, stored to pv
void launch_ilu_cta_fused(const DevPlan& P, const PrecDev& M, bool pupdate, const double* r, double* pv, const double* v, double* z,
                          const KScal* ks, cudaStream_t st);
// bytes of dynamic shared memory the CTA sweep needs for its vector (0 when it must stay in global memory)
size_t cta_sweep_smem(const DevPlan& P, bool fp32);
bool cta_sweep_supported(const DevPlan& P, const HostPlan& H);
void launch_bicg_iteration(const DevPlan& P, const double* val, const PrecDev& M, BicgVecs& V, KScal* ks, ReduceState& R,
                           SweepState& S, int* active, int* err, cudaStream_t st);
// ---- restarted flexible GMRES(m) of the batch (engine/src/linsolve.cpp:218-273), all systems in lockstep; per-system
// Hessenberg / Givens / y state on the device (GmState). Vectors: V (m+1 basis vectors), Z (m preconditioned), w.
struct GmState {
    int m = 0;
    double *V = nullptr, *Z = nullptr, *w = nullptr;
    double* H = nullptr;              // nsys x gm_stride(m): H (m+1) x m, cs m, sn m, g m+1, y m
    int* inner = nullptr;             // systems still in the inner loop of the current cycle
};
#ifdef __CUDACC__
#define RSG_HD __host__ __device__
#else
#define RSG_HD
#endif
inline RSG_HD size_t gm_stride(int m) { return size_t(m + 1) * m + 3 * size_t(m) + size_t(m + 1); }
// x = 0 for the systems (re)started (all, or only those whose status is not ST_CONV when onlyFailed), ||b||
void launch_gm_init(const DevPlan& P, const double* b, double* x, KScal* ks, ReduceState& R, double tol, int maxit, bool onlyFailed,
                    int* active, cudaStream_t st);
// cycle start: r = b - A x into V_0, beta, convergence / iteration-limit tests, V_0 = r / beta, g = beta e_1
void launch_gm_cycle_start(const DevPlan& P, const double* val, const double* b, const double* x, GmState& G, KScal* ks, ReduceState& R,
                           int* active, cudaStream_t st);
// inner step j after the preconditioner wrote Z_j: w = A Z_j, MGS against V_0..V_j, Givens, V_{j+1} = w / h
void launch_gm_step(const DevPlan& P, const double* val, int j, GmState& G, KScal* ks, ReduceState& R, int* active, cudaStream_t st);
// cycle end: y = H^-1 g, x += Z y; converged / iteration limit / restart
void launch_gm_cycle_end(const DevPlan& P, double* x, GmState& G, KScal* ks, int* active, cudaStream_t st);
// fallback bookkeeping: keep, per retried system, the solution with the smaller recursive residual
void launch_gm_pick(const DevPlan& P, double* x, const double* xPrev, const KScal* ksPrev, KScal* ks, cudaStream_t st);
// preconditioner input / output copy of the systems still in the inner loop (plain input mode, status-gated)
void launch_precond_gm(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, SweepState& S, int* err,
                       cudaStream_t st);

// true residual ||b - A x|| / ||b|| per system (FP64)
void launch_true_residual(const DevPlan& P, const double* val, const double* b, const double* x, double* tmp, ReduceState& R,
                          double* out, cudaStream_t st);

}  // namespace rsg

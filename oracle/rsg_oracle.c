/* CPU restatement of ResSim Studio's Newton linear-solve path: TEST INFRASTRUCTURE ONLY (see rsg_oracle.h).
 *
 * Built with -ffp-contract=off so the arithmetic is the canonical unfused double arithmetic of the reference
 * build (x86-64 g++ -O2 without FMA), on every host. OpenMP is used only where the reference uses it for
 * independent rows (SpMV, vector kernels); reductions are serial in the single-thread setting the golden
 * vectors are produced with.
 */
#include "rsg_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KMAXB 16

static int g_threads = 1;
void orc_set_threads(int n) {
    g_threads = n > 0 ? n : 1;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}
int orc_threads(void) { return g_threads; }
/* reference gating: parallel only for big loops with more than one thread (engine/src/linsolve.cpp:63-70) */
static int par(int big) { return big && g_threads > 1; }

static void* xmalloc(size_t bytes) {
    void* p = malloc(bytes ? bytes : 1);
    if (!p) abort();
    return p;
}
static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz ? sz : 1);
    if (!p) abort();
    return p;
}
static double wall(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ------------------------------------------------------------------ dense block kernels (engine/src/bsr.cpp:13-64) */
/* c = a * b, loop order i, k, j with a row accumulator */
static void gemm(const double* a, const double* b, double* c, int nb) {
    for (int i = 0; i < nb; ++i) {
        double r[KMAXB];
        for (int j = 0; j < nb; ++j) r[j] = 0;
        for (int k = 0; k < nb; ++k) {
            const double f = a[i * nb + k];
            for (int j = 0; j < nb; ++j) r[j] += f * b[k * nb + j];
        }
        for (int j = 0; j < nb; ++j) c[i * nb + j] = r[j];
    }
}
/* c -= a * b */
static void gemmSub(const double* a, const double* b, double* c, int nb) {
    for (int i = 0; i < nb; ++i) {
        double r[KMAXB];
        for (int j = 0; j < nb; ++j) r[j] = 0;
        for (int k = 0; k < nb; ++k) {
            const double f = a[i * nb + k];
            for (int j = 0; j < nb; ++j) r[j] += f * b[k * nb + j];
        }
        for (int j = 0; j < nb; ++j) c[i * nb + j] -= r[j];
    }
}
/* float versions of gemm / gemmSub (same loop order, every operation rounded to float) */
static void gemmf(const float* a, const float* b, float* c, int nb) {
    for (int i = 0; i < nb; ++i) {
        float r[KMAXB];
        for (int j = 0; j < nb; ++j) r[j] = 0;
        for (int k = 0; k < nb; ++k) {
            const float f = a[i * nb + k];
            for (int j = 0; j < nb; ++j) r[j] += f * b[k * nb + j];
        }
        for (int j = 0; j < nb; ++j) c[i * nb + j] = r[j];
    }
}
static void gemmSubf(const float* a, const float* b, float* c, int nb) {
    for (int i = 0; i < nb; ++i) {
        float r[KMAXB];
        for (int j = 0; j < nb; ++j) r[j] = 0;
        for (int k = 0; k < nb; ++k) {
            const float f = a[i * nb + k];
            for (int j = 0; j < nb; ++j) r[j] += f * b[k * nb + j];
        }
        for (int j = 0; j < nb; ++j) c[i * nb + j] -= r[j];
    }
}
/* y += a x / y -= a x, row sums accumulated from zero first */
static void gemvAdd(const double* a, const double* x, double* y, int nb) {
    for (int i = 0; i < nb; ++i) {
        double s = 0;
        for (int j = 0; j < nb; ++j) s += a[i * nb + j] * x[j];
        y[i] += s;
    }
}
static void gemvSub(const double* a, const double* x, double* y, int nb) {
    for (int i = 0; i < nb; ++i) {
        double s = 0;
        for (int j = 0; j < nb; ++j) s += a[i * nb + j] * x[j];
        y[i] -= s;
    }
}

/* engine/src/bsr.cpp:67-87: Gauss-Jordan on [A | I] with partial pivoting; singular when a pivot is
 * <= 1e-14 * max|a|; rows are eliminated only where the pivot column entry is non-zero */
int orc_invert_block(double* a, int nb) {
    double m[KMAXB][2 * KMAXB];
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
            m[i][j] = a[i * nb + j];
            m[i][nb + j] = (i == j) ? 1.0 : 0.0;
        }
    double scale = 0;
    for (int i = 0; i < nb * nb; ++i) scale = fmax(scale, fabs(a[i]));
    if (!(scale > 0) || !isfinite(scale)) return 0;
    for (int k = 0; k < nb; ++k) {
        int pr = k;
        for (int i = k + 1; i < nb; ++i)
            if (fabs(m[i][k]) > fabs(m[pr][k])) pr = i;
        if (fabs(m[pr][k]) <= 1e-14 * scale) return 0;
        if (pr != k)
            for (int j = 0; j < 2 * nb; ++j) {
                const double t = m[k][j];
                m[k][j] = m[pr][j];
                m[pr][j] = t;
            }
        const double inv = 1.0 / m[k][k];
        for (int j = 0; j < 2 * nb; ++j) m[k][j] *= inv;
        for (int i = 0; i < nb; ++i) {
            if (i == k || m[i][k] == 0.0) continue;
            const double f = m[i][k];
            for (int j = 0; j < 2 * nb; ++j) m[i][j] -= f * m[k][j];
        }
    }
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) a[i * nb + j] = m[i][nb + j];
    return 1;
}

/* ------------------------------------------------------------------ BSR SpMV (engine/src/bsr.cpp:109-126) */
void orc_bsr_spmv(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* x, double* y) {
    const int b2 = nb * nb;
#pragma omp parallel for schedule(static) if (par(n > 6000))
    for (int i = 0; i < n; ++i) {
        double* yi = y + (size_t)i * nb;
        for (int e = 0; e < nb; ++e) yi[e] = 0;
        for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p) gemvAdd(val + (size_t)p * b2, x + (size_t)col[p] * nb, yi, nb);
    }
}

void orc_bsr_spmv_f(int n, int nb, const int* rowPtr, const int* col, const float* val, const float* x, float* y) {
    const int b2 = nb * nb;
    for (int i = 0; i < n; ++i) {
        float acc[KMAXB] = {0};
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const float* B = val + (size_t)k * b2;
            const float* xk = x + (size_t)col[k] * nb;
            for (int e = 0; e < nb; ++e)
                for (int f = 0; f < nb; ++f) acc[e] += B[e * nb + f] * xk[f];
        }
        for (int e = 0; e < nb; ++e) y[(size_t)i * nb + e] = acc[e];
    }
}

static int* diag_positions(int n, const int* rowPtr, const int* col) {
    int* d = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        d[i] = -1;
        for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p)
            if (col[p] == i) {
                d[i] = p;
                break;
            }
    }
    return d;
}

/* singular pivot block: shift the diagonal by 1e-8 * max|a| (sign-preserving) and retry, else a scaled
 * identity (engine/src/bsr.cpp:204-212) */
static int invert_pivot(double* d, int nb) {
    const int b2 = nb * nb;
    double tmp[KMAXB * KMAXB];
    memcpy(tmp, d, sizeof(double) * b2);
    if (orc_invert_block(d, nb)) return 0;
    double sc = 0;
    for (int e = 0; e < b2; ++e) sc = fmax(sc, fabs(tmp[e]));
    if (!(sc > 0) || !isfinite(sc)) sc = 1.0;
    memcpy(d, tmp, sizeof(double) * b2);
    for (int e = 0; e < nb; ++e) d[e * nb + e] += (d[e * nb + e] >= 0 ? 1e-8 : -1e-8) * sc + (d[e * nb + e] == 0 ? sc * 1e-8 : 0);
    if (!orc_invert_block(d, nb)) {
        for (int e = 0; e < b2; ++e) d[e] = 0;
        for (int e = 0; e < nb; ++e) d[e * nb + e] = 1.0 / sc;
    }
    return 1;
}

/* ------------------------------------------------------------------ BILU0 (engine/src/bsr.cpp:183-215) */
int orc_bilu0_factor(int n, int nb, const int* rowPtr, const int* col, const double* val, double* lu) {
    const int b2 = nb * nb;
    const int nnzb = rowPtr[n];
    memcpy(lu, val, sizeof(double) * (size_t)nnzb * b2);
    int* diag = diag_positions(n, rowPtr, col);
    int* pos = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) pos[i] = -1;
    int nReg = 0;
    double tmp[KMAXB * KMAXB];
    for (int i = 0; i < n; ++i) {
        const int r0 = rowPtr[i], r1 = rowPtr[i + 1];
        for (int p = r0; p < r1; ++p) pos[col[p]] = p;
        for (int p = r0; p < r1; ++p) {
            const int k = col[p];
            if (k >= i) break;
            /* L_ik = A_ik U_kk^-1 (the diagonal block of row k holds its inverse) */
            gemm(lu + (size_t)p * b2, lu + (size_t)diag[k] * b2, tmp, nb);
            memcpy(lu + (size_t)p * b2, tmp, sizeof(double) * b2);
            for (int q = diag[k] + 1; q < rowPtr[k + 1]; ++q) {
                const int j = col[q];
                if (pos[j] >= r0 && pos[j] < r1 && col[pos[j]] == j) gemmSub(tmp, lu + (size_t)q * b2, lu + (size_t)pos[j] * b2, nb);
            }
        }
        for (int p = r0; p < r1; ++p) pos[col[p]] = -1;
        nReg += invert_pivot(lu + (size_t)diag[i] * b2, nb);
    }
    free(pos);
    free(diag);
    return nReg;
}

/* C45 lean row (engine/src/bsr.cpp:219-263): the row is eliminated in a double scratch row against the
 * already rounded float factors of earlier rows, its pivot inverted in double, and stored rounded */
int orc_bilu0_factor_lean(int n, int nb, const int* rowPtr, const int* col, const double* val, float* F) {
    const int b2 = nb * nb;
    const size_t nnzb = (size_t)rowPtr[n];
    for (size_t e = 0; e < nnzb * b2; ++e) F[e] = (float)val[e];
    int* diag = diag_positions(n, rowPtr, col);
    int* pos = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) pos[i] = -1;
    int maxRow = 0;
    for (int i = 0; i < n; ++i) maxRow = rowPtr[i + 1] - rowPtr[i] > maxRow ? rowPtr[i + 1] - rowPtr[i] : maxRow;
    double* buf = (double*)xmalloc(sizeof(double) * (size_t)maxRow * b2);
    double tmp[KMAXB * KMAXB], u[KMAXB * KMAXB];
    int nReg = 0;
    for (int i = 0; i < n; ++i) {
        const int r0 = rowPtr[i], r1 = rowPtr[i + 1];
        for (int p = r0; p < r1; ++p) {
            pos[col[p]] = p;
            for (int e = 0; e < b2; ++e) buf[(size_t)(p - r0) * b2 + e] = (double)F[(size_t)p * b2 + e];
        }
        for (int p = r0; p < r1; ++p) {
            const int k = col[p];
            if (k >= i) break;
            for (int e = 0; e < b2; ++e) u[e] = (double)F[(size_t)diag[k] * b2 + e];
            double* lp = buf + (size_t)(p - r0) * b2;
            gemm(lp, u, tmp, nb);
            memcpy(lp, tmp, sizeof(double) * b2);
            for (int q = diag[k] + 1; q < rowPtr[k + 1]; ++q) {
                const int j = col[q];
                if (pos[j] >= r0 && pos[j] < r1 && col[pos[j]] == j) {
                    for (int e = 0; e < b2; ++e) u[e] = (double)F[(size_t)q * b2 + e];
                    gemmSub(tmp, u, buf + (size_t)(pos[j] - r0) * b2, nb);
                }
            }
        }
        for (int p = r0; p < r1; ++p) pos[col[p]] = -1;
        nReg += invert_pivot(buf + (size_t)(diag[i] - r0) * b2, nb);
        for (int p = r0; p < r1; ++p)
            for (int e = 0; e < b2; ++e) F[(size_t)p * b2 + e] = (float)buf[(size_t)(p - r0) * b2 + e];
    }
    free(buf);
    free(pos);
    free(diag);
    return nReg;
}

/* All-FP32 factorisation of the precision form (FP32 elimination and storage, FP64 3x3 pivot inversion rounded to
 * float). No reference counterpart: it is the row algorithm of engine/src/bsr.cpp:183-215 with float arithmetic
 * (the reference's BILU0f factors in FP64, bsr.cpp:1087-1096). */
int orc_bilu0_factor_f32(int n, int nb, const int* rowPtr, const int* col, const double* val, float* F) {
    const int b2 = nb * nb;
    const size_t nnzb = (size_t)rowPtr[n];
    for (size_t e = 0; e < nnzb * b2; ++e) F[e] = (float)val[e];
    int* diag = diag_positions(n, rowPtr, col);
    int* pos = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) pos[i] = -1;
    float tmp[KMAXB * KMAXB];
    double D[KMAXB * KMAXB];
    int nReg = 0;
    for (int i = 0; i < n; ++i) {
        const int r0 = rowPtr[i], r1 = rowPtr[i + 1];
        for (int p = r0; p < r1; ++p) pos[col[p]] = p;
        for (int p = r0; p < r1; ++p) {
            const int k = col[p];
            if (k >= i) break;
            gemmf(F + (size_t)p * b2, F + (size_t)diag[k] * b2, tmp, nb);
            memcpy(F + (size_t)p * b2, tmp, sizeof(float) * b2);
            for (int q = diag[k] + 1; q < rowPtr[k + 1]; ++q) {
                const int j = col[q];
                if (pos[j] >= r0 && pos[j] < r1 && col[pos[j]] == j) gemmSubf(tmp, F + (size_t)q * b2, F + (size_t)pos[j] * b2, nb);
            }
        }
        for (int p = r0; p < r1; ++p) pos[col[p]] = -1;
        float* fd = F + (size_t)diag[i] * b2;
        for (int e = 0; e < b2; ++e) D[e] = (double)fd[e];
        nReg += invert_pivot(D, nb);
        for (int e = 0; e < b2; ++e) fd[e] = (float)D[e];
    }
    free(pos);
    free(diag);
    return nReg;
}

/* engine/src/bsr.cpp:565-596: forward y_i = r_i - sum_{k<i} L_ik y_k, backward z_i = U_ii^-1 (y_i - sum_{j>i} U_ij z_j) */
void orc_bilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* lu, const double* r, double* z) {
    const int b2 = nb * nb;
    int* diag = diag_positions(n, rowPtr, col);
    for (int i = 0; i < n; ++i) {
        double* zi = z + (size_t)i * nb;
        for (int e = 0; e < nb; ++e) zi[e] = r[(size_t)i * nb + e];
        for (int p = rowPtr[i]; p < diag[i]; ++p) gemvSub(lu + (size_t)p * b2, z + (size_t)col[p] * nb, zi, nb);
    }
    double t[KMAXB];
    for (int i = n - 1; i >= 0; --i) {
        double* zi = z + (size_t)i * nb;
        for (int p = diag[i] + 1; p < rowPtr[i + 1]; ++p) gemvSub(lu + (size_t)p * b2, z + (size_t)col[p] * nb, zi, nb);
        for (int e = 0; e < nb; ++e) t[e] = 0;
        gemvAdd(lu + (size_t)diag[i] * b2, zi, t, nb);
        for (int e = 0; e < nb; ++e) zi[e] = t[e];
    }
    free(diag);
}

/* float factors, double vectors and accumulation (engine/src/bsr.cpp:500-522) */
void orc_bilu0_apply_fd(int n, int nb, const int* rowPtr, const int* col, const float* F, const double* r, double* z) {
    const int b2 = nb * nb;
    int* diag = diag_positions(n, rowPtr, col);
    for (int i = 0; i < n; ++i) {
        double* zi = z + (size_t)i * nb;
        for (int e = 0; e < nb; ++e) zi[e] = r[(size_t)i * nb + e];
        for (int p = rowPtr[i]; p < diag[i]; ++p) {
            const float* a = F + (size_t)p * b2;
            const double* zk = z + (size_t)col[p] * nb;
            for (int e = 0; e < nb; ++e) {
                double s = 0;
                for (int f = 0; f < nb; ++f) s += (double)a[e * nb + f] * zk[f];
                zi[e] -= s;
            }
        }
    }
    double t[KMAXB];
    for (int i = n - 1; i >= 0; --i) {
        double* zi = z + (size_t)i * nb;
        for (int p = diag[i] + 1; p < rowPtr[i + 1]; ++p) {
            const float* a = F + (size_t)p * b2;
            const double* zj = z + (size_t)col[p] * nb;
            for (int e = 0; e < nb; ++e) {
                double s = 0;
                for (int f = 0; f < nb; ++f) s += (double)a[e * nb + f] * zj[f];
                zi[e] -= s;
            }
        }
        const float* d = F + (size_t)diag[i] * b2;
        for (int e = 0; e < nb; ++e) {
            double s = 0;
            for (int f = 0; f < nb; ++f) s += (double)d[e * nb + f] * zi[f];
            t[e] = s;
        }
        for (int e = 0; e < nb; ++e) zi[e] = t[e];
    }
    free(diag);
}

/* BILU0f (engine/src/bsr.cpp:1100-1121): float vectors and float accumulation */
void orc_bilu0_apply_ff(int n, int nb, const int* rowPtr, const int* col, const float* F, const double* r, double* z) {
    const int b2 = nb * nb;
    int* diag = diag_positions(n, rowPtr, col);
    float* y = (float*)xmalloc(sizeof(float) * (size_t)n * nb);
    for (int i = 0; i < n; ++i) {
        float* yi = y + (size_t)i * nb;
        for (int e = 0; e < nb; ++e) yi[e] = (float)r[(size_t)i * nb + e];
        for (int p = rowPtr[i]; p < diag[i]; ++p) {
            const float* a = F + (size_t)p * b2;
            const float* yk = y + (size_t)col[p] * nb;
            for (int e = 0; e < nb; ++e) {
                float s = 0;
                for (int f = 0; f < nb; ++f) s += a[e * nb + f] * yk[f];
                yi[e] -= s;
            }
        }
    }
    float t[KMAXB];
    for (int i = n - 1; i >= 0; --i) {
        float* yi = y + (size_t)i * nb;
        for (int p = diag[i] + 1; p < rowPtr[i + 1]; ++p) {
            const float* a = F + (size_t)p * b2;
            const float* yj = y + (size_t)col[p] * nb;
            for (int e = 0; e < nb; ++e) {
                float s = 0;
                for (int f = 0; f < nb; ++f) s += a[e * nb + f] * yj[f];
                yi[e] -= s;
            }
        }
        const float* d = F + (size_t)diag[i] * b2;
        for (int e = 0; e < nb; ++e) {
            float s = 0;
            for (int f = 0; f < nb; ++f) s += d[e * nb + f] * yi[f];
            t[e] = s;
        }
        for (int e = 0; e < nb; ++e) yi[e] = t[e];
    }
    for (size_t e = 0; e < (size_t)n * nb; ++e) z[e] = (double)y[e];
    free(y);
    free(diag);
}

/* ------------------------------------------------------------------ level sets (engine/src/bsr.cpp:270-293) */
int orc_level_sets(int n, const int* rowPtr, const int* col, int forward, int* ord, int* start) {
    int* diag = diag_positions(n, rowPtr, col);
    int* lev = (int*)xcalloc((size_t)n, sizeof(int));
    int nl = 0;
    if (forward) {
        for (int i = 0; i < n; ++i) {
            int l = 0;
            for (int p = rowPtr[i]; p < diag[i]; ++p) l = l > lev[col[p]] + 1 ? l : lev[col[p]] + 1;
            lev[i] = l;
            nl = nl > l + 1 ? nl : l + 1;
        }
    } else {
        for (int i = n - 1; i >= 0; --i) {
            int l = 0;
            for (int p = diag[i] + 1; p < rowPtr[i + 1]; ++p) l = l > lev[col[p]] + 1 ? l : lev[col[p]] + 1;
            lev[i] = l;
            nl = nl > l + 1 ? nl : l + 1;
        }
    }
    for (int l = 0; l <= nl; ++l) start[l] = 0;
    for (int i = 0; i < n; ++i) start[lev[i] + 1]++;
    for (int l = 0; l < nl; ++l) start[l + 1] += start[l];
    int* fill = (int*)xmalloc(sizeof(int) * (size_t)(nl > 0 ? nl : 1));
    for (int l = 0; l < nl; ++l) fill[l] = start[l];
    for (int i = 0; i < n; ++i) ord[fill[lev[i]]++] = i; /* ascending within a level */
    free(fill);
    free(lev);
    free(diag);
    return nl;
}

/* ================================================================== AMG (engine/src/amg.cpp) */
typedef struct {
    int nr, nc;
    int* rp;
    int* ci;
    double* v;
} sp_t;

static void sp_free(sp_t* s) {
    free(s->rp);
    free(s->ci);
    free(s->v);
    s->rp = s->ci = NULL;
    s->v = NULL;
}

typedef struct {
    sp_t A;     /* square CSR */
    int* diag;
    int nc;     /* size of the next level */
    sp_t P, R;  /* prolongator (n x nc) and restriction (nc x n) */
    double *x, *b, *r;
} amg_level;

struct orc_amg {
    int L;
    amg_level lv[14];
    double* lu; /* coarsest dense LU (<= 800 rows) */
    int* piv;
};

/* engine/src/amg.cpp:25-35 */
static sp_t sp_transpose(const sp_t* A) {
    sp_t T;
    T.nr = A->nc;
    T.nc = A->nr;
    T.rp = (int*)xcalloc((size_t)T.nr + 1, sizeof(int));
    const int nnz = A->rp[A->nr];
    for (int p = 0; p < nnz; ++p) T.rp[A->ci[p] + 1]++;
    for (int i = 0; i < T.nr; ++i) T.rp[i + 1] += T.rp[i];
    T.ci = (int*)xmalloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    T.v = (double*)xmalloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    int* fill = (int*)xmalloc(sizeof(int) * (size_t)(T.nr > 0 ? T.nr : 1));
    for (int i = 0; i < T.nr; ++i) fill[i] = T.rp[i];
    for (int i = 0; i < A->nr; ++i)
        for (int p = A->rp[i]; p < A->rp[i + 1]; ++p) {
            const int q = fill[A->ci[p]]++;
            T.ci[q] = i;
            T.v[q] = A->v[p];
        }
    free(fill);
    return T;
}

typedef struct {
    int c;
    double v;
} cv_t;
static int cv_cmp(const void* a, const void* b) {
    const cv_t* x = (const cv_t*)a;
    const cv_t* y = (const cv_t*)b;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->v < y->v ? -1 : (x->v > y->v ? 1 : 0);
}

/* engine/src/amg.cpp:37-70: C = A B, first product assigned, later ones added in A's row order, rows sorted */
static sp_t sp_multiply(const sp_t* A, const sp_t* B) {
    sp_t C;
    C.nr = A->nr;
    C.nc = B->nc;
    C.rp = (int*)xcalloc((size_t)A->nr + 1, sizeof(int));
    int* mark = (int*)xmalloc(sizeof(int) * (size_t)(B->nc > 0 ? B->nc : 1));
    for (int j = 0; j < B->nc; ++j) mark[j] = -1;
    for (int i = 0; i < A->nr; ++i) {
        int cnt = 0;
        for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
            for (int q = B->rp[A->ci[p]]; q < B->rp[A->ci[p] + 1]; ++q)
                if (mark[B->ci[q]] != i) {
                    mark[B->ci[q]] = i;
                    ++cnt;
                }
        C.rp[i + 1] = C.rp[i] + cnt;
    }
    const int nnz = C.rp[A->nr];
    C.ci = (int*)xmalloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    C.v = (double*)xcalloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
    for (int j = 0; j < B->nc; ++j) mark[j] = -1;
    int maxRow = 0;
    for (int i = 0; i < A->nr; ++i) maxRow = C.rp[i + 1] - C.rp[i] > maxRow ? C.rp[i + 1] - C.rp[i] : maxRow;
    cv_t* row = (cv_t*)xmalloc(sizeof(cv_t) * (size_t)(maxRow > 0 ? maxRow : 1));
    for (int i = 0; i < A->nr; ++i) {
        int pos = C.rp[i];
        const int start = pos;
        for (int p = A->rp[i]; p < A->rp[i + 1]; ++p) {
            const double a = A->v[p];
            for (int q = B->rp[A->ci[p]]; q < B->rp[A->ci[p] + 1]; ++q) {
                const int j = B->ci[q];
                if (mark[j] < start) {
                    mark[j] = pos;
                    C.ci[pos] = j;
                    C.v[pos] = a * B->v[q];
                    ++pos;
                } else
                    C.v[mark[j]] += a * B->v[q];
            }
        }
        for (int p = start; p < pos; ++p) {
            row[p - start].c = C.ci[p];
            row[p - start].v = C.v[p];
        }
        qsort(row, (size_t)(pos - start), sizeof(cv_t), cv_cmp);
        for (int p = start; p < pos; ++p) {
            C.ci[p] = row[p - start].c;
            C.v[p] = row[p - start].v;
        }
    }
    free(row);
    free(mark);
    return C;
}

/* engine/src/amg.cpp:72-101: guarantee a diagonal entry per row (zeros inserted), tiny diagonals set to 1 */
static void sp_to_csr(sp_t* S, int** diagOut) {
    const int n = S->nr;
    int missing = 0;
    for (int i = 0; i < n && !missing; ++i) {
        int f = 0;
        for (int p = S->rp[i]; p < S->rp[i + 1]; ++p)
            if (S->ci[p] == i) {
                f = 1;
                break;
            }
        if (!f) missing = 1;
    }
    if (missing) {
        const int nnz = S->rp[n];
        int* rp = (int*)xcalloc((size_t)n + 1, sizeof(int));
        int* ci = (int*)xmalloc(sizeof(int) * (size_t)(nnz + n));
        double* v = (double*)xmalloc(sizeof(double) * (size_t)(nnz + n));
        int c = 0;
        for (int i = 0; i < n; ++i) {
            int f = 0;
            for (int p = S->rp[i]; p < S->rp[i + 1]; ++p) {
                if (!f && S->ci[p] > i) {
                    ci[c] = i;
                    v[c] = 0.0;
                    ++c;
                    f = 1;
                }
                if (S->ci[p] == i) f = 1;
                ci[c] = S->ci[p];
                v[c] = S->v[p];
                ++c;
            }
            if (!f) {
                ci[c] = i;
                v[c] = 0.0;
                ++c;
            }
            rp[i + 1] = c;
        }
        sp_free(S);
        S->rp = rp;
        S->ci = ci;
        S->v = v;
    }
    int* d = diag_positions(n, S->rp, S->ci);
    for (int i = 0; i < n; ++i)
        if (fabs(S->v[d[i]]) < 1e-300) S->v[d[i]] = 1.0;
    *diagOut = d;
}

static sp_t sp_copy(int n, const int* rowPtr, const int* col, const double* val) {
    sp_t s;
    s.nr = s.nc = n;
    const int nnz = rowPtr[n];
    s.rp = (int*)xmalloc(sizeof(int) * ((size_t)n + 1));
    memcpy(s.rp, rowPtr, sizeof(int) * ((size_t)n + 1));
    s.ci = (int*)xmalloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    memcpy(s.ci, col, sizeof(int) * (size_t)nnz);
    s.v = (double*)xmalloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    memcpy(s.v, val, sizeof(double) * (size_t)nnz);
    return s;
}

/* engine/src/amg.cpp:273-295: dense LU with partial pivoting of the coarsest level (<= 800 rows) */
static void amg_factor_coarsest(orc_amg* h) {
    const amg_level* C = &h->lv[h->L - 1];
    free(h->lu);
    free(h->piv);
    h->lu = NULL;
    h->piv = NULL;
    if (C->A.nr > 800) return;
    const int m = C->A.nr;
    h->lu = (double*)xcalloc((size_t)m * m, sizeof(double));
    h->piv = (int*)xmalloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    double* lu = h->lu;
    for (int i = 0; i < m; ++i)
        for (int p = C->A.rp[i]; p < C->A.rp[i + 1]; ++p) lu[(size_t)i * m + C->A.ci[p]] = C->A.v[p];
    for (int k = 0; k < m; ++k) {
        int pr = k;
        double mx = fabs(lu[(size_t)k * m + k]);
        for (int i = k + 1; i < m; ++i)
            if (fabs(lu[(size_t)i * m + k]) > mx) {
                mx = fabs(lu[(size_t)i * m + k]);
                pr = i;
            }
        h->piv[k] = pr;
        if (pr != k)
            for (int j = 0; j < m; ++j) {
                const double t = lu[(size_t)k * m + j];
                lu[(size_t)k * m + j] = lu[(size_t)pr * m + j];
                lu[(size_t)pr * m + j] = t;
            }
        double* dk = &lu[(size_t)k * m + k];
        if (fabs(*dk) < 1e-300) *dk = 1e-300;
        for (int i = k + 1; i < m; ++i) {
            const double f = lu[(size_t)i * m + k] / *dk;
            lu[(size_t)i * m + k] = f;
            if (f != 0)
                for (int j = k + 1; j < m; ++j) lu[(size_t)i * m + j] -= f * lu[(size_t)k * m + j];
        }
    }
}

static void amg_level_alloc_vectors(amg_level* L) {
    const int n = L->A.nr;
    L->x = (double*)xcalloc((size_t)n, sizeof(double));
    L->b = (double*)xcalloc((size_t)n, sizeof(double));
    L->r = (double*)xcalloc((size_t)n, sizeof(double));
}

/* engine/src/amg.cpp:137-252 with kSmooth = false (plain aggregation, P = aggregate indicator, R = P^T) */
orc_amg* orc_amg_setup(int n0, const int* rowPtr, const int* col, const double* val) {
    orc_amg* h = (orc_amg*)xcalloc(1, sizeof(orc_amg));
    h->L = 1;
    h->lv[0].A = sp_copy(n0, rowPtr, col, val);
    sp_to_csr(&h->lv[0].A, &h->lv[0].diag); /* inserts missing diagonals, fixes tiny ones (engine/src/amg.cpp:144-145) */
    const double kTheta = 0.08, kRowTheta = 0.25;
    for (;;) {
        amg_level* L = &h->lv[h->L - 1];
        const sp_t* A = &L->A;
        const int n = A->nr;
        if (n <= 400 || h->L >= 14) break;
        const int* dg = L->diag;
        /* strength of connection */
        int* sp = (int*)xcalloc((size_t)n + 1, sizeof(int));
        int* sc = (int*)xmalloc(sizeof(int) * (size_t)(A->rp[n] > 0 ? A->rp[n] : 1));
        int ns = 0;
        for (int i = 0; i < n; ++i) {
            double rowMax = 0;
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
                if (A->ci[p] != i) rowMax = fmax(rowMax, fabs(A->v[p]));
            const double di = A->v[dg[i]];
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p) {
                const int j = A->ci[p];
                if (j == i) continue;
                const double dj = A->v[dg[j]];
                if (fabs(A->v[p]) >= kTheta * sqrt(fabs(di * dj)) || fabs(A->v[p]) >= kRowTheta * rowMax) sc[ns++] = j;
            }
            sp[i + 1] = ns;
        }
        /* greedy aggregation, three passes */
        int* agg = (int*)xmalloc(sizeof(int) * (size_t)n);
        for (int i = 0; i < n; ++i) agg[i] = -1;
        int na = 0;
        for (int i = 0; i < n; ++i) { /* pass 1: roots with free strong neighbourhoods */
            if (agg[i] >= 0) continue;
            int fr = 1;
            for (int p = sp[i]; p < sp[i + 1]; ++p)
                if (agg[sc[p]] >= 0) {
                    fr = 0;
                    break;
                }
            if (!fr) continue;
            if (sp[i] == sp[i + 1]) continue;
            agg[i] = na;
            for (int p = sp[i]; p < sp[i + 1]; ++p) agg[sc[p]] = na;
            ++na;
        }
        int* agg1 = (int*)xmalloc(sizeof(int) * (size_t)n);
        memcpy(agg1, agg, sizeof(int) * (size_t)n);
        for (int i = 0; i < n; ++i) { /* pass 2: join the most strongly coupled pass-1 aggregate */
            if (agg[i] >= 0) continue;
            double best = 0;
            int ba = -1;
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p) {
                const int j = A->ci[p];
                if (j != i && agg1[j] >= 0 && fabs(A->v[p]) > best) {
                    best = fabs(A->v[p]);
                    ba = agg1[j];
                }
            }
            if (ba >= 0 && sp[i] != sp[i + 1]) agg[i] = ba;
        }
        for (int i = 0; i < n; ++i) { /* pass 3: leftovers start new aggregates */
            if (agg[i] >= 0) continue;
            agg[i] = na;
            for (int p = sp[i]; p < sp[i + 1]; ++p)
                if (agg[sc[p]] < 0) agg[sc[p]] = na;
            ++na;
        }
        free(agg1);
        free(sp);
        free(sc);
        if (na >= (int)(0.85 * n) || na < 1) {
            free(agg);
            break;
        }
        /* P: one unit entry per fine row (aggregate indicator) */
        sp_t P;
        P.nr = n;
        P.nc = na;
        P.rp = (int*)xmalloc(sizeof(int) * ((size_t)n + 1));
        P.ci = (int*)xmalloc(sizeof(int) * (size_t)n);
        P.v = (double*)xmalloc(sizeof(double) * (size_t)n);
        P.rp[0] = 0;
        for (int i = 0; i < n; ++i) {
            P.ci[i] = agg[i];
            P.v[i] = 1.0;
            P.rp[i + 1] = i + 1;
        }
        free(agg);
        sp_t R = sp_transpose(&P);
        sp_t AP = sp_multiply(A, &P);
        sp_t Ac = sp_multiply(&R, &AP);
        sp_free(&AP);
        L->nc = na;
        L->P = P;
        L->R = R;
        amg_level* N = &h->lv[h->L];
        memset(N, 0, sizeof(*N));
        N->A = Ac;
        N->A.nc = Ac.nr;
        sp_to_csr(&N->A, &N->diag);
        h->L++;
    }
    for (int l = 0; l < h->L; ++l) amg_level_alloc_vectors(&h->lv[l]);
    amg_factor_coarsest(h);
    return h;
}

/* engine/src/amg.cpp:257-271: same pattern, new values; Galerkin operators recomputed on the kept aggregates */
int orc_amg_refresh(orc_amg* h, int n, const int* rowPtr, const int* col, const double* val) {
    if (h->L < 1 || n != h->lv[0].A.nr || rowPtr[n] != h->lv[0].A.rp[n]) return 0;
    if (memcmp(col, h->lv[0].A.ci, sizeof(int) * (size_t)rowPtr[n]) != 0) return 0;
    memcpy(h->lv[0].A.v, val, sizeof(double) * (size_t)rowPtr[n]);
    for (int i = 0; i < n; ++i)
        if (fabs(h->lv[0].A.v[h->lv[0].diag[i]]) < 1e-300) h->lv[0].A.v[h->lv[0].diag[i]] = 1.0;
    for (int l = 0; l + 1 < h->L; ++l) {
        amg_level* L = &h->lv[l];
        sp_t AP = sp_multiply(&L->A, &L->P);
        sp_t Ac = sp_multiply(&L->R, &AP);
        sp_free(&AP);
        int* d;
        sp_to_csr(&Ac, &d);
        free(d);
        amg_level* N = &h->lv[l + 1];
        const int nn = Ac.nr;
        if (nn != N->A.nr || Ac.rp[nn] != N->A.rp[nn] || memcmp(Ac.ci, N->A.ci, sizeof(int) * (size_t)Ac.rp[nn]) != 0) {
            sp_free(&Ac);
            return 0;
        }
        memcpy(N->A.v, Ac.v, sizeof(double) * (size_t)Ac.rp[nn]);
        sp_free(&Ac);
    }
    amg_factor_coarsest(h);
    return 1;
}

/* Multicolour smoother of the device's FP32 precision forms (no reference counterpart): greedy colours assigned
 * in the level's natural order, the sweep colour by colour (backward: colours in reverse); rows of a colour are
 * independent, so the order inside a colour does not matter. Off by default (the reference's smoother). */
static int g_mc_smoother = 0;
void orc_set_mc_smoother(int on) { g_mc_smoother = on; }

static void gauss_seidel_mc(const sp_t* A, const int* dg, const double* b, double* x, int forward) {
    const int n = A->nr;
    int* colr = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    char* used = (char*)xcalloc((size_t)n + 2, 1);
    int nc = 0;
    for (int i = 0; i < n; ++i) colr[i] = -1;
    for (int i = 0; i < n; ++i) {
        for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
            if (A->ci[p] != i && colr[A->ci[p]] >= 0) used[colr[A->ci[p]]] = 1;
        int c = 0;
        while (used[c]) ++c;
        colr[i] = c;
        if (c + 1 > nc) nc = c + 1;
        for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
            if (A->ci[p] != i && colr[A->ci[p]] >= 0) used[colr[A->ci[p]]] = 0;
    }
    for (int cc = 0; cc < nc; ++cc) {
        const int c = forward ? cc : nc - 1 - cc;
        for (int i = 0; i < n; ++i) {
            if (colr[i] != c) continue;
            double s = b[i];
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
                if (A->ci[p] != i) s -= A->v[p] * x[A->ci[p]];
            x[i] = s / A->v[dg[i]];
        }
    }
    free(used);
    free(colr);
}

/* engine/src/amg.cpp:98-113 */
static void gauss_seidel(const sp_t* A, const int* dg, const double* b, double* x, int forward) {
    const int n = A->nr;
    if (g_mc_smoother) {
        gauss_seidel_mc(A, dg, b, x, forward);
        return;
    }
    if (forward) {
        for (int i = 0; i < n; ++i) {
            double s = b[i];
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
                if (A->ci[p] != i) s -= A->v[p] * x[A->ci[p]];
            x[i] = s / A->v[dg[i]];
        }
    } else {
        for (int i = n - 1; i >= 0; --i) {
            double s = b[i];
            for (int p = A->rp[i]; p < A->rp[i + 1]; ++p)
                if (A->ci[p] != i) s -= A->v[p] * x[A->ci[p]];
            x[i] = s / A->v[dg[i]];
        }
    }
}

static void spmv_rect(const sp_t* M, const double* x, double* y, int add) {
    for (int i = 0; i < M->nr; ++i) {
        double s = 0;
        for (int p = M->rp[i]; p < M->rp[i + 1]; ++p) s += M->v[p] * x[M->ci[p]];
        y[i] = add ? y[i] + s : s;
    }
}

/* engine/src/amg.cpp:303-329: V(1,1), forward GS before, backward GS after, dense LU on the coarsest level */
static void amg_cycle(const orc_amg* h, int l) {
    const amg_level* L = &h->lv[l];
    const int n = L->A.nr;
    if (l + 1 == h->L) {
        if (h->lu) {
            const int m = n;
            double* x = L->x;
            memcpy(x, L->b, sizeof(double) * (size_t)m);
            for (int k = 0; k < m; ++k)
                if (h->piv[k] != k) {
                    const double t = x[k];
                    x[k] = x[h->piv[k]];
                    x[h->piv[k]] = t;
                }
            for (int i = 0; i < m; ++i) {
                double s = x[i];
                for (int j = 0; j < i; ++j) s -= h->lu[(size_t)i * m + j] * x[j];
                x[i] = s;
            }
            for (int i = m - 1; i >= 0; --i) {
                double s = x[i];
                for (int j = i + 1; j < m; ++j) s -= h->lu[(size_t)i * m + j] * x[j];
                x[i] = s / h->lu[(size_t)i * m + i];
            }
        } else {
            memset(L->x, 0, sizeof(double) * (size_t)n);
            for (int s = 0; s < 20; ++s) {
                gauss_seidel(&L->A, L->diag, L->b, L->x, 1);
                gauss_seidel(&L->A, L->diag, L->b, L->x, 0);
            }
        }
        return;
    }
    memset(L->x, 0, sizeof(double) * (size_t)n);
    gauss_seidel(&L->A, L->diag, L->b, L->x, 1);
    spmv_rect(&L->A, L->x, L->r, 0);
    for (int i = 0; i < n; ++i) L->r[i] = L->b[i] - L->r[i];
    const amg_level* C = &h->lv[l + 1];
    spmv_rect(&L->R, L->r, C->b, 0);
    amg_cycle(h, l + 1);
    spmv_rect(&L->P, C->x, L->x, 1);
    gauss_seidel(&L->A, L->diag, L->b, L->x, 0);
}

void orc_amg_apply(const orc_amg* h, const double* r, double* z) {
    if (h->L < 1) return;
    const amg_level* L = &h->lv[0];
    memcpy(L->b, r, sizeof(double) * (size_t)L->A.nr);
    amg_cycle(h, 0);
    memcpy(z, L->x, sizeof(double) * (size_t)L->A.nr);
}

int orc_amg_levels(const orc_amg* h) { return h->L; }
int orc_amg_level_info(const orc_amg* h, int l, int* rows, int* nnz) {
    if (l < 0 || l >= h->L) return 0;
    *rows = h->lv[l].A.nr;
    *nnz = h->lv[l].A.rp[h->lv[l].A.nr];
    return 1;
}
int orc_amg_level_get(const orc_amg* h, int l, int* rowPtr, int* col, double* val, int* agg) {
    if (l < 0 || l >= h->L) return 0;
    const sp_t* A = &h->lv[l].A;
    memcpy(rowPtr, A->rp, sizeof(int) * ((size_t)A->nr + 1));
    memcpy(col, A->ci, sizeof(int) * (size_t)A->rp[A->nr]);
    memcpy(val, A->v, sizeof(double) * (size_t)A->rp[A->nr]);
    if (agg)
        for (int i = 0; i < A->nr; ++i) agg[i] = (l + 1 < h->L) ? h->lv[l].P.ci[h->lv[l].P.rp[i]] : -1;
    return 1;
}
void orc_amg_free(orc_amg* h) {
    if (!h) return;
    for (int l = 0; l < h->L; ++l) {
        sp_free(&h->lv[l].A);
        free(h->lv[l].diag);
        if (l + 1 < h->L) {
            sp_free(&h->lv[l].P);
            sp_free(&h->lv[l].R);
        }
        free(h->lv[l].x);
        free(h->lv[l].b);
        free(h->lv[l].r);
    }
    free(h->lu);
    free(h->piv);
    free(h);
}

/* ================================================================== block CPR (engine/src/bsr.cpp:993-1084) */
struct orc_cpr {
    int n, nb, lean;
    const int* rowPtr;
    const int* col;
    const double* val;
    double* w;
    orc_amg* amg;
    double* lu;
    float* luf;
    double *rp, *xp, *t;
};

orc_cpr* orc_cpr_setup(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int lean) {
    orc_cpr* h = (orc_cpr*)xcalloc(1, sizeof(orc_cpr));
    h->n = n;
    h->nb = nb;
    h->lean = lean;
    h->rowPtr = rowPtr;
    h->col = col;
    h->val = val;
    const int b2 = nb * nb;
    int* diag = diag_positions(n, rowPtr, col);
    h->w = (double*)xmalloc(sizeof(double) * (size_t)n * nb);
    for (int i = 0; i < n; ++i) {
        double D[KMAXB * KMAXB];
        memcpy(D, val + (size_t)diag[i] * b2, sizeof(double) * b2);
        int inverted = 0;
        if (acc) {
            /* true-IMPES: accumulation block, condition estimate from its explicit inverse */
            const double* B = acc + (size_t)i * b2;
            double inv[KMAXB * KMAXB];
            memcpy(inv, B, sizeof(double) * b2);
            if (orc_invert_block(inv, nb)) {
                double n1 = 0, ni = 0;
                for (int j = 0; j < nb; ++j) {
                    double c = 0, d = 0;
                    for (int r = 0; r < nb; ++r) {
                        c += fabs(B[r * nb + j]);
                        d += fabs(inv[r * nb + j]);
                    }
                    n1 = fmax(n1, c);
                    ni = fmax(ni, d);
                }
                if (nb == 1 || n1 * ni <= 1e10) {
                    memcpy(D, inv, sizeof(double) * b2);
                    inverted = 1;
                }
            } else if (nb == 1) {
                memcpy(D, B, sizeof(double) * b2);
            }
        }
        double* w = h->w + (size_t)i * nb;
        if (inverted || orc_invert_block(D, nb)) {
            for (int e = 0; e < nb; ++e) w[e] = D[e]; /* first row of D^-1 */
        } else {
            double s = 0;
            for (int e = 0; e < nb; ++e) s += val[(size_t)diag[i] * b2 + e * nb];
            for (int e = 0; e < nb; ++e) w[e] = fabs(s) > 1e-300 ? 1.0 / s : 1.0;
        }
        double wm = 0;
        for (int e = 0; e < nb; ++e) wm = fmax(wm, fabs(w[e]));
        if (!(wm > 0) || !isfinite(wm))
            for (int e = 0; e < nb; ++e) w[e] = 1.0;
    }
    /* pressure matrix Ap_ij = sum_e w_ie S_ij[e][0] on S's block pattern */
    const int nnzb = rowPtr[n];
    double* ap = (double*)xmalloc(sizeof(double) * (size_t)(nnzb > 0 ? nnzb : 1));
    for (int i = 0; i < n; ++i) {
        const double* w = h->w + (size_t)i * nb;
        for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p) {
            const double* a = val + (size_t)p * b2;
            double s = 0;
            for (int e = 0; e < nb; ++e) s += w[e] * a[e * nb];
            ap[p] = s;
        }
    }
    h->amg = orc_amg_setup(n, rowPtr, col, ap);
    free(ap);
    if (lean) {
        h->luf = (float*)xmalloc(sizeof(float) * (size_t)nnzb * b2);
        orc_bilu0_factor_lean(n, nb, rowPtr, col, val, h->luf);
    } else {
        h->lu = (double*)xmalloc(sizeof(double) * (size_t)nnzb * b2);
        orc_bilu0_factor(n, nb, rowPtr, col, val, h->lu);
    }
    h->rp = (double*)xcalloc((size_t)n, sizeof(double));
    h->xp = (double*)xcalloc((size_t)n, sizeof(double));
    h->t = (double*)xcalloc((size_t)n * nb, sizeof(double));
    free(diag);
    return h;
}

void orc_cpr_apply(const orc_cpr* h, const double* r, double* z) {
    const int n = h->n, nb = h->nb, b2 = nb * nb;
    for (int i = 0; i < n; ++i) {
        double s = 0;
        for (int e = 0; e < nb; ++e) s += h->w[(size_t)i * nb + e] * r[(size_t)i * nb + e];
        h->rp[i] = s;
    }
    orc_amg_apply(h->amg, h->rp, h->xp);
    /* second stage on r - S z1, z1 = (xp, 0, ..): only the pressure column of each block */
    for (int i = 0; i < n; ++i) {
        double acc[KMAXB];
        for (int e = 0; e < nb; ++e) acc[e] = r[(size_t)i * nb + e];
        for (int k = h->rowPtr[i]; k < h->rowPtr[i + 1]; ++k) {
            const double* B = h->val + (size_t)k * b2;
            const double xk = h->xp[h->col[k]];
            for (int e = 0; e < nb; ++e) acc[e] -= B[e * nb] * xk;
        }
        for (int e = 0; e < nb; ++e) h->t[(size_t)i * nb + e] = acc[e];
    }
    if (h->lean)
        orc_bilu0_apply_fd(n, nb, h->rowPtr, h->col, h->luf, h->t, z);
    else
        orc_bilu0_apply(n, nb, h->rowPtr, h->col, h->lu, h->t, z);
    for (int i = 0; i < n; ++i) z[(size_t)i * nb] += h->xp[i];
}

const double* orc_cpr_weights(const orc_cpr* h) { return h->w; }
const orc_amg* orc_cpr_amg(const orc_cpr* h) { return h->amg; }
void orc_cpr_free(orc_cpr* h) {
    if (!h) return;
    free(h->w);
    orc_amg_free(h->amg);
    free(h->lu);
    free(h->luf);
    free(h->rp);
    free(h->xp);
    free(h->t);
    free(h);
}

/* ================================================================== multicolour BILU0
 * engine/src/bsr.cpp:599-730 (colourBlocks, permuteBsr, MCBILU0::factor / apply): largest-degree-first greedy
 * colouring of the symmetric block graph, P A P^T with sorted columns, block ILU(0) of it in its natural order (rows of
 * a colour depend on earlier colours only; the row arithmetic and singular-pivot shift are bilu0Row's), and the
 * sweeps on the permuted vectors. */
static int int_cmp(const void* a, const void* b);
typedef struct { int d, i; } deg_t;
static int deg_cmp(const void* a, const void* b) {               /* degree descending, index ascending (stable) */
    const deg_t* x = (const deg_t*)a;
    const deg_t* y = (const deg_t*)b;
    if (x->d != y->d) return x->d > y->d ? -1 : 1;
    return x->i < y->i ? -1 : (x->i > y->i ? 1 : 0);
}

int orc_colour_blocks(int n, const int* rowPtr, const int* col, int* colour, int* perm) {
    int* cnt = (int*)xcalloc((size_t)n + 1, sizeof(int));
    for (int i = 0; i < n; ++i)
        for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p)
            if (col[p] != i) { cnt[i + 1]++; cnt[col[p] + 1]++; }
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    int* adj = (int*)xmalloc(sizeof(int) * (size_t)(cnt[n] > 0 ? cnt[n] : 1));
    int* fill = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) fill[i] = cnt[i];
    for (int i = 0; i < n; ++i)
        for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p)
            if (col[p] != i) { adj[fill[i]++] = col[p]; adj[fill[col[p]]++] = i; }
    int* deg = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {                                 /* sorted, unique */
        int* a = adj + cnt[i];
        const int m = fill[i] - cnt[i];
        qsort(a, (size_t)m, sizeof(int), int_cmp);
        int u = 0;
        for (int k = 0; k < m; ++k)
            if (u == 0 || a[k] != a[u - 1]) a[u++] = a[k];
        deg[i] = u;
    }
    deg_t* ord = (deg_t*)xmalloc(sizeof(deg_t) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) { ord[i].d = deg[i]; ord[i].i = i; }
    qsort(ord, (size_t)n, sizeof(deg_t), deg_cmp);
    for (int i = 0; i < n; ++i) colour[i] = -1;
    int colours = 0;
    char* mark = (char*)xmalloc((size_t)n + 2);
    for (int t = 0; t < n; ++t) {
        const int i = ord[t].i, m = deg[i];
        memset(mark, 0, (size_t)m + 2);
        for (int k = 0; k < m; ++k) {
            const int cj = colour[adj[cnt[i] + k]];
            if (cj >= 0 && cj < m + 2) mark[cj] = 1;
        }
        int c = 0;
        while (mark[c]) ++c;
        colour[i] = c;
        if (c + 1 > colours) colours = c + 1;
    }
    int* start = (int*)xcalloc((size_t)colours + 1, sizeof(int));
    for (int i = 0; i < n; ++i) start[colour[i] + 1]++;
    for (int c = 0; c < colours; ++c) start[c + 1] += start[c];
    for (int i = 0; i < n; ++i) perm[start[colour[i]]++] = i;     /* new index -> original, cells grouped by colour */
    free(start); free(mark); free(ord); free(deg); free(fill); free(adj); free(cnt);
    return colours;
}

typedef struct { int c, p; } colpos_t;
static int colpos_cmp(const void* a, const void* b) {
    const colpos_t* x = (const colpos_t*)a;
    const colpos_t* y = (const colpos_t*)b;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->p < y->p ? -1 : (x->p > y->p);
}

int orc_mcbilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* r, double* z) {
    const int b2 = nb * nb, nnzb = rowPtr[n];
    int* colour = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* perm = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* iperm = (int*)xmalloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    const int colours = orc_colour_blocks(n, rowPtr, col, colour, perm);
    for (int k = 0; k < n; ++k) iperm[perm[k]] = k;
    int* prp = (int*)xcalloc((size_t)n + 1, sizeof(int));
    int* pci = (int*)xmalloc(sizeof(int) * (size_t)(nnzb > 0 ? nnzb : 1));
    double* pv = (double*)xmalloc(sizeof(double) * (size_t)(nnzb > 0 ? nnzb : 1) * b2);
    colpos_t* row = (colpos_t*)xmalloc(sizeof(colpos_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    for (int k = 0; k < n; ++k) {
        const int i = perm[k], m = rowPtr[i + 1] - rowPtr[i];
        for (int q = 0; q < m; ++q) { row[q].c = iperm[col[rowPtr[i] + q]]; row[q].p = rowPtr[i] + q; }
        qsort(row, (size_t)m, sizeof(colpos_t), colpos_cmp);
        prp[k + 1] = prp[k] + m;
        for (int q = 0; q < m; ++q) {
            pci[prp[k] + q] = row[q].c;
            memcpy(pv + (size_t)(prp[k] + q) * b2, val + (size_t)row[q].p * b2, sizeof(double) * (size_t)b2);
        }
    }
    double* lu = (double*)xmalloc(sizeof(double) * (size_t)(nnzb > 0 ? nnzb : 1) * b2);
    const int nreg = orc_bilu0_factor(n, nb, prp, pci, pv, lu);
    double* rp = (double*)xmalloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * nb);
    double* zp = (double*)xmalloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * nb);
    for (int k = 0; k < n; ++k) memcpy(rp + (size_t)k * nb, r + (size_t)perm[k] * nb, sizeof(double) * (size_t)nb);
    orc_bilu0_apply(n, nb, prp, pci, lu, rp, zp);
    for (int k = 0; k < n; ++k) memcpy(z + (size_t)perm[k] * nb, zp + (size_t)k * nb, sizeof(double) * (size_t)nb);
    free(zp); free(rp); free(lu); free(row); free(pv); free(pci); free(prp); free(iperm); free(perm); free(colour);
    (void)nreg;
    return colours;
}

/* ================================================================== GPU-shaped float CPR-AMG
 * engine/src/bsr.cpp:1217-1371 (DeviceCprAmg::build / apply): the BlockCPR hierarchy with float values, damped Jacobi
 * V(1,1) (omega = 0.6667, one sweep each way, the first from x = 0), the coarsest level by an explicit inverse
 * (Gauss-Jordan in double, at most 1500 rows; else 31 Jacobi sweeps), the second stage block-Jacobi on r - S E x.
 * Float operations in the reference's order (this file is built with -ffp-contract=off). */
struct orc_devcpr {
    int n, nb, L;
    const int *rowPtr, *col;
    orc_cpr* cpr;             /* weights and hierarchy, as BlockCPR::setup builds them */
    float *w, *Av, *bj;       /* weights (n*nb), float values of S, block-diagonal inverses (n*nb*nb) */
    float *A[14], *P[14], *R[14], *dinv[14];
    float *x[14], *b[14], *t[14];
    int m;                    /* coarsest rows */
    float* cinv;              /* explicit inverse of the coarsest level (m*m, natural order) or NULL */
    float *z1, *tt;
};

static float* f32_copy(const double* v, size_t n) {
    float* f = (float*)xmalloc(sizeof(float) * (n > 0 ? n : 1));
    for (size_t k = 0; k < n; ++k) f[k] = (float)v[k];
    return f;
}

orc_devcpr* orc_devcpr_setup(int n, int nb, const int* rowPtr, const int* col, const double* val) {
    orc_devcpr* h = (orc_devcpr*)xcalloc(1, sizeof(orc_devcpr));
    const int N = n * nb, b2 = nb * nb, nnzb = rowPtr[n];
    h->n = n; h->nb = nb; h->rowPtr = rowPtr; h->col = col;
    h->cpr = orc_cpr_setup(n, nb, rowPtr, col, val, NULL, 0);
    const orc_amg* G = h->cpr->amg;
    h->L = G->L;
    h->w = f32_copy(h->cpr->w, (size_t)N);
    h->Av = f32_copy(val, (size_t)nnzb * b2);
    for (int l = 0; l < h->L; ++l) {
        const amg_level* V = &G->lv[l];
        const int nl = V->A.nr;
        h->A[l] = f32_copy(V->A.v, (size_t)V->A.rp[nl]);
        h->dinv[l] = (float*)xmalloc(sizeof(float) * (size_t)(nl > 0 ? nl : 1));
        for (int i = 0; i < nl; ++i) {
            double d = 0;
            for (int k = V->A.rp[i]; k < V->A.rp[i + 1]; ++k)
                if (V->A.ci[k] == i) d = V->A.v[k];
            h->dinv[l][i] = fabs(d) > 1e-300 ? (float)(1.0 / d) : 0.0f;
        }
        if (l + 1 < h->L) {
            h->P[l] = f32_copy(V->P.v, (size_t)V->P.rp[V->P.nr]);
            h->R[l] = f32_copy(V->R.v, (size_t)V->R.rp[V->R.nr]);
        }
        h->x[l] = (float*)xcalloc((size_t)(nl > 0 ? nl : 1), sizeof(float));
        h->b[l] = (float*)xcalloc((size_t)(nl > 0 ? nl : 1), sizeof(float));
        h->t[l] = (float*)xcalloc((size_t)(nl > 0 ? nl : 1), sizeof(float));
    }
    /* explicit inverse of the coarsest operator: Gauss-Jordan in double, pivot = first strictly largest |a_ik| */
    const sp_t* Cc = &G->lv[h->L - 1].A;
    const int m = Cc->nr;
    h->m = m;
    if (m > 0 && m <= 1500) {
        const size_t w2 = 2 * (size_t)m;
        double* M = (double*)xcalloc((size_t)m * w2, sizeof(double));
        for (int i = 0; i < m; ++i) {
            for (int k = Cc->rp[i]; k < Cc->rp[i + 1]; ++k) M[(size_t)i * w2 + (size_t)Cc->ci[k]] += Cc->v[k];
            M[(size_t)i * w2 + (size_t)(m + i)] = 1.0;
        }
        int ok = 1;
        for (int k = 0; k < m && ok; ++k) {
            int pr = k;
            for (int i = k + 1; i < m; ++i)
                if (fabs(M[(size_t)i * w2 + k]) > fabs(M[(size_t)pr * w2 + k])) pr = i;
            if (fabs(M[(size_t)pr * w2 + k]) < 1e-300) { ok = 0; break; }
            if (pr != k)
                for (size_t j = 0; j < w2; ++j) {
                    const double t = M[(size_t)k * w2 + j];
                    M[(size_t)k * w2 + j] = M[(size_t)pr * w2 + j];
                    M[(size_t)pr * w2 + j] = t;
                }
            const double piv = 1.0 / M[(size_t)k * w2 + k];
            for (size_t j = 0; j < w2; ++j) M[(size_t)k * w2 + j] *= piv;
            for (int i = 0; i < m; ++i) {
                if (i == k) continue;
                const double f = M[(size_t)i * w2 + k];
                if (f == 0) continue;
                for (size_t j = 0; j < w2; ++j) M[(size_t)i * w2 + j] -= f * M[(size_t)k * w2 + j];
            }
        }
        if (ok) {
            h->cinv = (float*)xmalloc(sizeof(float) * (size_t)m * m);
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < m; ++j) h->cinv[(size_t)i * m + j] = (float)M[(size_t)i * w2 + (size_t)(m + j)];
        }
        free(M);
    }
    /* block-Jacobi second stage: inverse diagonal blocks, 1 / max(1e-30, |D_ee|) on the diagonal when singular */
    h->bj = (float*)xmalloc(sizeof(float) * (size_t)n * b2);
    double blk[KMAXB * KMAXB];
    for (int i = 0; i < n; ++i) {
        int dp = -1;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (col[k] == i) dp = k;
        const double* D = val + (size_t)dp * b2;
        for (int e = 0; e < b2; ++e) blk[e] = D[e];
        if (!orc_invert_block(blk, nb)) {
            for (int e = 0; e < b2; ++e) blk[e] = 0.0;
            for (int e = 0; e < nb; ++e) blk[e * nb + e] = 1.0 / fmax(1e-30, fabs(D[e * nb + e]));
        }
        for (int e = 0; e < b2; ++e) h->bj[(size_t)i * b2 + e] = (float)blk[e];
    }
    h->z1 = (float*)xcalloc((size_t)(N > 0 ? N : 1), sizeof(float));
    h->tt = (float*)xcalloc((size_t)(N > 0 ? N : 1), sizeof(float));
    return h;
}

static void f32_spmv(const sp_t* S, const float* v, const float* x, float* y) {
    for (int i = 0; i < S->nr; ++i) {
        float acc = 0;
        for (int k = S->rp[i]; k < S->rp[i + 1]; ++k) acc += v[k] * x[S->ci[k]];
        y[i] = acc;
    }
}

void orc_devcpr_apply(const orc_devcpr* h, const float* r, float* z) {
    const int n = h->n, nb = h->nb, b2 = nb * nb, L = h->L;
    const orc_amg* G = h->cpr->amg;
    const float omega = 0.6667f;
    for (int i = 0; i < n; ++i) {                                  /* W r */
        float acc = 0;
        for (int e = 0; e < nb; ++e) acc += h->w[(size_t)i * nb + e] * r[(size_t)i * nb + e];
        h->b[0][i] = acc;
    }
    for (int l = 0; l + 1 < L; ++l) {
        const sp_t* A = &G->lv[l].A;
        float *x = h->x[l], *b = h->b[l], *t = h->t[l];
        const float* dinv = h->dinv[l];
        for (int i = 0; i < A->nr; ++i) x[i] = omega * dinv[i] * b[i];   /* one sweep from x = 0 */
        f32_spmv(A, h->A[l], x, t);
        for (int i = 0; i < A->nr; ++i) t[i] = b[i] - t[i];
        f32_spmv(&G->lv[l].R, h->R[l], t, h->b[l + 1]);
    }
    {                                                              /* coarsest */
        const sp_t* A = &G->lv[L - 1].A;
        float *x = h->x[L - 1], *b = h->b[L - 1], *t = h->t[L - 1];
        const float* dinv = h->dinv[L - 1];
        if (h->cinv) {
            const int m = h->m;
            for (int i = 0; i < m; ++i) {
                float acc = 0;
                for (int j = 0; j < m; ++j) acc += h->cinv[(size_t)i * m + j] * b[j];
                x[i] = acc;
            }
        } else {
            for (int i = 0; i < A->nr; ++i) x[i] = omega * dinv[i] * b[i];
            for (int s = 0; s < 30; ++s) {
                f32_spmv(A, h->A[L - 1], x, t);
                for (int i = 0; i < A->nr; ++i) x[i] += omega * dinv[i] * (b[i] - t[i]);
            }
        }
    }
    for (int l = L - 2; l >= 0; --l) {
        const sp_t* A = &G->lv[l].A;
        float *x = h->x[l], *b = h->b[l], *t = h->t[l];
        const float* dinv = h->dinv[l];
        f32_spmv(&G->lv[l].P, h->P[l], h->x[l + 1], t);
        for (int i = 0; i < A->nr; ++i) x[i] += t[i];
        f32_spmv(A, h->A[l], x, t);                                /* one sweep after */
        for (int i = 0; i < A->nr; ++i) x[i] += omega * dinv[i] * (b[i] - t[i]);
    }
    for (int i = 0; i < n; ++i)                                    /* E x: the pressure of each block (a CSR row */
        for (int e = 0; e < nb; ++e)                               /* with one unit entry, or none)             */
            h->z1[(size_t)i * nb + e] = e == 0 ? 0.0f + 1.0f * h->x[0][i] : 0.0f;
    for (int i = 0; i < n; ++i) {                                  /* second stage: z = z1 + D^-1 (r - S z1) */
        float acc[KMAXB];
        for (int e = 0; e < nb; ++e) acc[e] = 0;
        for (int k = h->rowPtr[i]; k < h->rowPtr[i + 1]; ++k) {
            const float* B = h->Av + (size_t)k * b2;
            const float* xk = h->z1 + (size_t)h->col[k] * nb;
            for (int e = 0; e < nb; ++e)
                for (int f = 0; f < nb; ++f) acc[e] += B[e * nb + f] * xk[f];
        }
        for (int e = 0; e < nb; ++e) h->tt[(size_t)i * nb + e] = r[(size_t)i * nb + e] - acc[e];
    }
    for (int i = 0; i < n; ++i) {
        const float* D = h->bj + (size_t)i * b2;
        for (int e = 0; e < nb; ++e) {
            float s2 = 0;
            for (int f = 0; f < nb; ++f) s2 += D[e * nb + f] * h->tt[(size_t)i * nb + f];
            z[(size_t)i * nb + e] = h->z1[(size_t)i * nb + e] + s2;
        }
    }
}

int orc_devcpr_levels(const orc_devcpr* h) { return h ? h->L : 0; }
int orc_devcpr_has_inverse(const orc_devcpr* h) { return h && h->cinv ? 1 : 0; }

void orc_devcpr_free(orc_devcpr* h) {
    if (!h) return;
    orc_cpr_free(h->cpr);
    free(h->w); free(h->Av); free(h->bj); free(h->cinv); free(h->z1); free(h->tt);
    for (int l = 0; l < h->L; ++l) {
        free(h->A[l]); free(h->dinv[l]); free(h->x[l]); free(h->b[l]); free(h->t[l]);
        if (l + 1 < h->L) { free(h->P[l]); free(h->R[l]); }
    }
    free(h);
}

/* ================================================================== Krylov (engine/src/linsolve.cpp:147-273) */
static double dot(const double* a, const double* b, int n) {
    double s = 0;
    if (par(n > 20000)) {
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (int i = 0; i < n; ++i) s += a[i] * b[i];
    } else {
        for (int i = 0; i < n; ++i) s += a[i] * b[i];
    }
    return s;
}
static double norm2(const double* a, int n) { return sqrt(dot(a, a, n)); }

int orc_bicgstab(int n, orc_apply_fn A, void* actx, orc_apply_fn M, void* mctx, const double* b, double* x, double tol, int maxIt,
                 int* its, double* relres) {
    *its = 0;
    *relres = 0;
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    double* buf = (double*)xcalloc((size_t)n * 8, sizeof(double));
    double *r = buf, *rh = buf + n, *p = buf + 2 * (size_t)n, *v = buf + 3 * (size_t)n, *s = buf + 4 * (size_t)n,
           *t = buf + 5 * (size_t)n, *ph = buf + 6 * (size_t)n, *sh = buf + 7 * (size_t)n;
    memcpy(r, b, sizeof(double) * (size_t)n);
    memcpy(rh, b, sizeof(double) * (size_t)n);
    const double bn = norm2(b, n);
    int conv = 0;
    if (bn == 0) {
        free(buf);
        return 1;
    }
    const int pv = par(n > 20000);
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 1; it <= maxIt; ++it) {
        const double rhoN = dot(rh, r, n);
        if (fabs(rhoN) < 1e-300) break;
        const double beta = (rhoN / rho) * (alpha / omega);
        rho = rhoN;
#pragma omp parallel for schedule(static) if (pv)
        for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        M(mctx, p, ph);
        A(actx, ph, v);
        const double rv = dot(rh, v, n);
        if (fabs(rv) < 1e-300) break;
        alpha = rho / rv;
#pragma omp parallel for schedule(static) if (pv)
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        const double sn = norm2(s, n);
        if (sn / bn < tol) {
#pragma omp parallel for schedule(static) if (pv)
            for (int i = 0; i < n; ++i) x[i] += alpha * ph[i];
            conv = 1;
            *its = it;
            *relres = sn / bn;
            break;
        }
        M(mctx, s, sh);
        A(actx, sh, t);
        const double tt = dot(t, t, n);
        omega = tt > 0 ? dot(t, s, n) / tt : 0;
#pragma omp parallel for schedule(static) if (pv)
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * ph[i] + omega * sh[i];
            r[i] = s[i] - omega * t[i];
        }
        const double rn = norm2(r, n);
        *its = it;
        *relres = rn / bn;
        if (rn / bn < tol) {
            conv = 1;
            break;
        }
        if (omega == 0) break;
    }
    free(buf);
    return conv;
}

int orc_gmres(int n, orc_apply_fn A, void* actx, orc_apply_fn M, void* mctx, const double* b, double* x, double tol, int maxIt, int m,
              int* its, double* relres) {
    *its = 0;
    *relres = 0;
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    const double bn = norm2(b, n);
    if (bn == 0) return 1;
    double* V = (double*)xcalloc((size_t)(m + 1) * n, sizeof(double));
    double* Z = (double*)xcalloc((size_t)m * n, sizeof(double));
    double* H = (double*)xcalloc((size_t)(m + 1) * m, sizeof(double));
    double* cs = (double*)xcalloc((size_t)m, sizeof(double));
    double* sn = (double*)xcalloc((size_t)m, sizeof(double));
    double* g = (double*)xcalloc((size_t)m + 1, sizeof(double));
    double* y = (double*)xcalloc((size_t)m, sizeof(double));
    double* r = (double*)xmalloc(sizeof(double) * (size_t)n);
    double* w = (double*)xmalloc(sizeof(double) * (size_t)n);
#define HAT(i, j) H[(size_t)(i) * m + (j)]
    int total = 0, conv = 0;
    double rel = 0;
    while (total < maxIt) {
        A(actx, x, r);
        for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
        const double beta = norm2(r, n);
        rel = beta / bn;
        if (beta / bn < tol) {
            conv = 1;
            break;
        }
        for (int i = 0; i < n; ++i) V[i] = r[i] / beta;
        for (int i = 0; i <= m; ++i) g[i] = 0;
        g[0] = beta;
        int j = 0;
        for (; j < m && total < maxIt; ++j, ++total) {
            M(mctx, V + (size_t)j * n, Z + (size_t)j * n);
            A(actx, Z + (size_t)j * n, w);
            for (int i = 0; i <= j; ++i) {
                const double hh = dot(w, V + (size_t)i * n, n);
                HAT(i, j) = hh;
                for (int q = 0; q < n; ++q) w[q] -= hh * V[(size_t)i * n + q];
            }
            const double hn = norm2(w, n);
            HAT(j + 1, j) = hn;
            if (hn > 0)
                for (int q = 0; q < n; ++q) V[(size_t)(j + 1) * n + q] = w[q] / hn;
            for (int i = 0; i < j; ++i) {
                const double t = cs[i] * HAT(i, j) + sn[i] * HAT(i + 1, j);
                HAT(i + 1, j) = -sn[i] * HAT(i, j) + cs[i] * HAT(i + 1, j);
                HAT(i, j) = t;
            }
            const double den = hypot(HAT(j, j), HAT(j + 1, j));
            cs[j] = den > 0 ? HAT(j, j) / den : 1;
            sn[j] = den > 0 ? HAT(j + 1, j) / den : 0;
            HAT(j, j) = den;
            HAT(j + 1, j) = 0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            rel = fabs(g[j + 1]) / bn;
            if (rel < tol) {
                ++j;
                ++total;
                break;
            }
        }
        for (int i = j - 1; i >= 0; --i) {
            double s = g[i];
            for (int k = i + 1; k < j; ++k) s -= HAT(i, k) * y[k];
            y[i] = s / HAT(i, i);
        }
        for (int i = 0; i < j; ++i)
            for (int q = 0; q < n; ++q) x[q] += y[i] * Z[(size_t)i * n + q];
        if (rel < tol) {
            conv = 1;
            break;
        }
    }
#undef HAT
    *its = total;
    *relres = rel;
    free(V);
    free(Z);
    free(H);
    free(cs);
    free(sn);
    free(g);
    free(y);
    free(r);
    free(w);
    return conv;
}

/* ================================================================== drivers */
typedef struct {
    int n, nb;
    const int* rowPtr;
    const int* col;
    const double* val;
} bsr_ctx;
static void op_bsr(void* c, const double* x, double* y) {
    const bsr_ctx* b = (const bsr_ctx*)c;
    orc_bsr_spmv(b->n, b->nb, b->rowPtr, b->col, b->val, x, y);
}
typedef struct {
    int n, nb;
    const int* rowPtr;
    const int* col;
    double* lu;
    float* luf;
    orc_cpr* cpr;
} prec_ctx;
static void op_prec(void* c, const double* r, double* z) {
    const prec_ctx* p = (const prec_ctx*)c;
    if (p->cpr)
        orc_cpr_apply(p->cpr, r, z);
    else if (p->luf)
        orc_bilu0_apply_fd(p->n, p->nb, p->rowPtr, p->col, p->luf, r, z);
    else
        orc_bilu0_apply(p->n, p->nb, p->rowPtr, p->col, p->lu, r, z);
}
static void prec_build(prec_ctx* P, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec) {
    memset(P, 0, sizeof(*P));
    P->n = n;
    P->nb = nb;
    P->rowPtr = rowPtr;
    P->col = col;
    const size_t ne = (size_t)rowPtr[n] * nb * nb;
    if (prec == 1 || prec == 3)
        P->cpr = orc_cpr_setup(n, nb, rowPtr, col, val, acc, prec == 3);
    else if (prec == 2) {
        P->luf = (float*)xmalloc(sizeof(float) * (ne ? ne : 1));
        orc_bilu0_factor_lean(n, nb, rowPtr, col, val, P->luf);
    } else {
        P->lu = (double*)xmalloc(sizeof(double) * (ne ? ne : 1));
        orc_bilu0_factor(n, nb, rowPtr, col, val, P->lu);
    }
}
static void prec_free(prec_ctx* P) {
    orc_cpr_free(P->cpr);
    free(P->lu);
    free(P->luf);
}

int orc_prec_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, const double* r,
                   double* z) {
    prec_ctx P;
    prec_build(&P, n, nb, rowPtr, col, val, acc, prec);
    op_prec(&P, r, z);
    const int levels = P.cpr ? orc_amg_levels(P.cpr->amg) : 0;
    prec_free(&P);
    return levels;
}

int orc_solve_timed(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, int method,
                    int restart, const double* b, double* x, double tol, int maxIt, int* its, double* relres, double* setupSec,
                    double* solveSec) {
    const double t0 = wall();
    prec_ctx P;
    prec_build(&P, n, nb, rowPtr, col, val, acc, prec);
    const double t1 = wall();
    bsr_ctx A = {n, nb, rowPtr, col, val};
    const int N = n * nb;
    const int conv = method == 1 ? orc_gmres(N, op_bsr, &A, op_prec, &P, b, x, tol, maxIt, restart, its, relres)
                                 : orc_bicgstab(N, op_bsr, &A, op_prec, &P, b, x, tol, maxIt, its, relres);
    const double t2 = wall();
    prec_free(&P);
    if (setupSec) *setupSec = t1 - t0;
    if (solveSec) *solveSec = t2 - t1;
    return conv;
}

int orc_solve(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, int method, int restart,
              const double* b, double* x, double tol, int maxIt, int* its, double* relres) {
    return orc_solve_timed(n, nb, rowPtr, col, val, acc, prec, method, restart, b, x, tol, maxIt, its, relres, NULL, NULL);
}

/* ================================================================== float device emulation + refinement */
/* CpuFloatBlockSolver::solve, BILU0f preconditioner (engine/src/bsr.cpp:1130-1215) */
static int float_device_solve(int n, int nb, const int* rowPtr, const int* col, const double* val, const float* Av, const float* F,
                              const double* bd, double* xd, double tol, int maxIt, int* iterations) {
    const int N = n * nb;
    *iterations = 0;
    float* buf = (float*)xcalloc((size_t)N * 9, sizeof(float));
    float *x = buf, *r = buf + N, *r0 = buf + 2 * (size_t)N, *p = buf + 3 * (size_t)N, *v = buf + 4 * (size_t)N, *ph = buf + 5 * (size_t)N,
          *s = buf + 6 * (size_t)N, *sh = buf + 7 * (size_t)N, *t = buf + 8 * (size_t)N;
    double* tmpD = (double*)xmalloc(sizeof(double) * (size_t)N);
    double* tmpZ = (double*)xmalloc(sizeof(double) * (size_t)N);
    (void)val;
#define FDOT(u, w)                                                        \
    ({                                                                    \
        double acc_ = 0;                                                  \
        for (int e_ = 0; e_ < N; ++e_) acc_ += (double)(u)[e_] * (w)[e_]; \
        acc_;                                                             \
    })
#define PREC(in, out)                                                          \
    do {                                                                       \
        for (int e_ = 0; e_ < N; ++e_) tmpD[e_] = (in)[e_];                    \
        orc_bilu0_apply_ff(n, nb, rowPtr, col, F, tmpD, tmpZ);                 \
        for (int e_ = 0; e_ < N; ++e_) (out)[e_] = (float)tmpZ[e_];            \
    } while (0)
    for (int e = 0; e < N; ++e) r[e] = (float)bd[e];
    memcpy(r0, r, sizeof(float) * (size_t)N);
    const double bn = sqrt(FDOT(r, r));
    for (int e = 0; e < N; ++e) xd[e] = 0.0;
    if (!(bn > 0)) {
        free(buf);
        free(tmpD);
        free(tmpZ);
        return 1;
    }
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 1; it <= maxIt; ++it) {
        *iterations = it;
        const double rhoN = FDOT(r0, r);
        if (rhoN == 0 || !isfinite(rhoN)) break;
        const double beta = (rhoN / rho) * (alpha / omega);
        for (int e = 0; e < N; ++e) p[e] = (float)(r[e] + beta * (p[e] - omega * v[e]));
        PREC(p, ph);
        orc_bsr_spmv_f(n, nb, rowPtr, col, Av, ph, v);
        const double r0v = FDOT(r0, v);
        if (r0v == 0 || !isfinite(r0v)) break;
        alpha = rhoN / r0v;
        for (int e = 0; e < N; ++e) s[e] = (float)(r[e] - alpha * v[e]);
        if (sqrt(FDOT(s, s)) <= tol * bn) {
            for (int e = 0; e < N; ++e) x[e] += (float)(alpha * ph[e]);
            break;
        }
        PREC(s, sh);
        orc_bsr_spmv_f(n, nb, rowPtr, col, Av, sh, t);
        const double tt = FDOT(t, t);
        omega = tt > 0 ? FDOT(t, s) / tt : 0;
        for (int e = 0; e < N; ++e) {
            x[e] += (float)(alpha * ph[e] + omega * sh[e]);
            r[e] = (float)(s[e] - omega * t[e]);
        }
        rho = rhoN;
        if (sqrt(FDOT(r, r)) <= tol * bn || omega == 0) break;
    }
#undef FDOT
#undef PREC
    int ok = 1;
    for (int e = 0; e < N; ++e) {
        xd[e] = x[e];
        if (!isfinite(xd[e])) ok = 0;
    }
    free(buf);
    free(tmpD);
    free(tmpZ);
    return ok;
}

int orc_refine_float(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b, double* x, double tol,
                     int maxOuter, int innerIt, int* its, double* relres) {
    const int N = n * nb;
    const size_t ne = (size_t)rowPtr[n] * nb * nb;
    float* Av = (float*)xmalloc(sizeof(float) * (ne ? ne : 1));
    for (size_t e = 0; e < ne; ++e) Av[e] = (float)val[e];
    /* BILU0f: factor in double, store in float (engine/src/bsr.cpp:1087-1098) */
    double* lu = (double*)xmalloc(sizeof(double) * (ne ? ne : 1));
    orc_bilu0_factor(n, nb, rowPtr, col, val, lu);
    float* F = (float*)xmalloc(sizeof(float) * (ne ? ne : 1));
    for (size_t e = 0; e < ne; ++e) F[e] = (float)lu[e];
    free(lu);
    double* r = (double*)xmalloc(sizeof(double) * (size_t)N);
    double* d = (double*)xmalloc(sizeof(double) * (size_t)N);
    double* Ax = (double*)xmalloc(sizeof(double) * (size_t)N);
    memcpy(r, b, sizeof(double) * (size_t)N);
    for (int e = 0; e < N; ++e) x[e] = 0.0;
    *its = 0;
    *relres = 0;
    double bn = 0;
    for (int e = 0; e < N; ++e) bn += b[e] * b[e];
    bn = sqrt(bn);
    int conv = 0;
    if (!(bn > 0)) conv = 1;
    /* engine/src/bsr.cpp:1373-1396 */
    const double innerTol = fmax(1e-4, fmin(1e-2, tol * 10));
    int done = conv;
    for (int outer = 0; outer < maxOuter && !done; ++outer) {
        double rn = 0;
        for (int e = 0; e < N; ++e) rn += r[e] * r[e];
        rn = sqrt(rn);
        *relres = rn / bn;
        if (*relres <= tol) {
            conv = 1;
            done = 1;
            break;
        }
        int it = 0;
        if (!float_device_solve(n, nb, rowPtr, col, val, Av, F, r, d, innerTol, innerIt, &it)) {
            done = 1;
            break;
        }
        *its += it;
        for (int e = 0; e < N; ++e) x[e] += d[e];
        orc_bsr_spmv(n, nb, rowPtr, col, val, x, Ax);
        for (int e = 0; e < N; ++e) r[e] = b[e] - Ax[e];
    }
    if (!done) {
        double rn = 0;
        for (int e = 0; e < N; ++e) rn += r[e] * r[e];
        rn = sqrt(rn);
        *relres = rn / bn;
        conv = *relres <= tol;
    }
    free(Av);
    free(F);
    free(r);
    free(d);
    free(Ax);
    return conv;
}

/* ================================================================== well Schur complement (engine/src/bsr.cpp:733-840) */
typedef struct {
    int nc, nw;
    double* dInv;
    int *wcPtr, *wcCol;
    double* wcVal;
    int *cwPtr, *cwWell;
    double* cwVal;
} well_parts;

static void wp_free(well_parts* W) {
    free(W->dInv);
    free(W->wcPtr);
    free(W->wcCol);
    free(W->wcVal);
    free(W->cwPtr);
    free(W->cwWell);
    free(W->cwVal);
}

static int wp_build(well_parts* W, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw) {
    const int nc = na * nv;
    memset(W, 0, sizeof(*W));
    W->nc = nc;
    W->nw = nw;
    W->dInv = (double*)xcalloc((size_t)nw, sizeof(double));
    W->wcPtr = (int*)xcalloc((size_t)nw + 1, sizeof(int));
    const int nnz = rowPtr[nc + nw];
    W->wcCol = (int*)xmalloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    W->wcVal = (double*)xmalloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    int nwc = 0;
    for (int w = 0; w < nw; ++w) {
        const int r = nc + w;
        double d = 0, rowMax = 0;
        for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
            const int c = col[p];
            if (c == r)
                d = val[p];
            else if (c < nc) {
                W->wcCol[nwc] = c;
                W->wcVal[nwc] = val[p];
                ++nwc;
                rowMax = fmax(rowMax, fabs(val[p]));
            } else if (val[p] != 0.0)
                return 0; /* well-well coupling: not supported */
        }
        if (!(fabs(d) > 1e-12 * fmax(rowMax, 1e-300)) || !isfinite(d)) return 0;
        W->dInv[w] = 1.0 / d;
        W->wcPtr[w + 1] = nwc;
    }
    W->cwPtr = (int*)xcalloc((size_t)nc + 1, sizeof(int));
    W->cwWell = (int*)xmalloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    W->cwVal = (double*)xmalloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    int ncw = 0;
    for (int r = 0; r < nc; ++r) {
        for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
            if (col[p] >= nc && val[p] != 0.0) {
                W->cwWell[ncw] = col[p] - nc;
                W->cwVal[ncw] = val[p];
                ++ncw;
            }
        W->cwPtr[r + 1] = ncw;
    }
    return 1;
}

static int int_cmp(const void* a, const void* b) {
    const int x = *(const int*)a, y = *(const int*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int orc_wellschur(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                  int capBlocks, int* sRowPtr, int* sCol, double* sVal, double* bc) {
    (void)nrows;
    well_parts W;
    if (!wp_build(&W, rowPtr, col, val, na, nv, nw)) {
        wp_free(&W);
        return 0;
    }
    const int nc = na * nv, b2 = nv * nv;
    /* cells of each well (sorted, unique) */
    int** wellCells = (int**)xcalloc((size_t)(nw > 0 ? nw : 1), sizeof(int*));
    int* wellCount = (int*)xcalloc((size_t)(nw > 0 ? nw : 1), sizeof(int));
    for (int w = 0; w < nw; ++w) {
        const int m = W.wcPtr[w + 1] - W.wcPtr[w];
        wellCells[w] = (int*)xmalloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
        for (int p = W.wcPtr[w]; p < W.wcPtr[w + 1]; ++p) wellCells[w][p - W.wcPtr[w]] = W.wcCol[p] / nv;
        qsort(wellCells[w], (size_t)m, sizeof(int), int_cmp);
        int u = 0;
        for (int k = 0; k < m; ++k)
            if (u == 0 || wellCells[w][u - 1] != wellCells[w][k]) wellCells[w][u++] = wellCells[w][k];
        wellCount[w] = u;
    }
    /* block pattern: cell pattern plus couplings through shared wells */
    int* mark = (int*)xmalloc(sizeof(int) * (size_t)(na > 0 ? na : 1));
    for (int i = 0; i < na; ++i) mark[i] = -1;
    int cap = 64, cnt = 0;
    int* cols = (int*)xmalloc(sizeof(int) * (size_t)cap);
    int* wl = (int*)xmalloc(sizeof(int) * (size_t)(nw + 1) * (size_t)(nv + 1) + sizeof(int));
    int need = 0;
    int ok = 1;
    sRowPtr[0] = 0;
    for (int pass = 0; pass < 1; ++pass) {
        for (int i = 0; i < na; ++i) {
            cnt = 0;
            int nwl = 0;
            for (int e = 0; e < nv; ++e) {
                const int r = i * nv + e;
                for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
                    const int c = col[p];
                    if (c < nc) {
                        const int j = c / nv;
                        if (mark[j] != i) {
                            mark[j] = i;
                            if (cnt == cap) {
                                cap *= 2;
                                cols = (int*)realloc(cols, sizeof(int) * (size_t)cap);
                            }
                            cols[cnt++] = j;
                        }
                    }
                }
                for (int p = W.cwPtr[r]; p < W.cwPtr[r + 1]; ++p) wl[nwl++] = W.cwWell[p];
            }
            if (mark[i] != i) {
                mark[i] = i;
                if (cnt == cap) {
                    cap *= 2;
                    cols = (int*)realloc(cols, sizeof(int) * (size_t)cap);
                }
                cols[cnt++] = i;
            }
            qsort(wl, (size_t)nwl, sizeof(int), int_cmp);
            for (int k = 0; k < nwl; ++k) {
                if (k > 0 && wl[k] == wl[k - 1]) continue;
                const int w = wl[k];
                for (int q = 0; q < wellCount[w]; ++q) {
                    const int j = wellCells[w][q];
                    if (mark[j] != i) {
                        mark[j] = i;
                        if (cnt == cap) {
                            cap *= 2;
                            cols = (int*)realloc(cols, sizeof(int) * (size_t)cap);
                        }
                        cols[cnt++] = j;
                    }
                }
            }
            qsort(cols, (size_t)cnt, sizeof(int), int_cmp);
            if (need + cnt <= capBlocks)
                for (int k = 0; k < cnt; ++k) sCol[need + k] = cols[k];
            else
                ok = 0;
            need += cnt;
            sRowPtr[i + 1] = need;
        }
    }
    free(cols);
    free(wl);
    free(mark);
    if (!ok) {
        for (int w = 0; w < nw; ++w) free(wellCells[w]);
        free(wellCells);
        free(wellCount);
        wp_free(&W);
        return -need;
    }
    /* values: S = Acc - Acw Dww^-1 Awc, in the reference's order of operations */
    memset(sVal, 0, sizeof(double) * (size_t)need * b2);
    int* pos = (int*)xmalloc(sizeof(int) * (size_t)(na > 0 ? na : 1));
    for (int i = 0; i < na; ++i) pos[i] = -1;
    for (int i = 0; i < na; ++i) {
        for (int p = sRowPtr[i]; p < sRowPtr[i + 1]; ++p) pos[sCol[p]] = p;
        for (int e = 0; e < nv; ++e) {
            const int r = i * nv + e;
            for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
                const int c = col[p];
                if (c < nc) sVal[(size_t)pos[c / nv] * b2 + e * nv + c % nv] += val[p];
            }
            for (int p = W.cwPtr[r]; p < W.cwPtr[r + 1]; ++p) {
                const int w = W.cwWell[p];
                const double f = W.cwVal[p] * W.dInv[w];
                for (int q = W.wcPtr[w]; q < W.wcPtr[w + 1]; ++q) {
                    const int c = W.wcCol[q];
                    sVal[(size_t)pos[c / nv] * b2 + e * nv + c % nv] -= f * W.wcVal[q];
                }
            }
        }
    }
    free(pos);
    /* bc = b_c - Acw Dww^-1 b_w (engine/src/bsr.cpp:973-980) */
    if (b && bc)
        for (int r = 0; r < nc; ++r) {
            double s = b[r];
            for (int p = W.cwPtr[r]; p < W.cwPtr[r + 1]; ++p) s -= W.cwVal[p] * W.dInv[W.cwWell[p]] * b[nc + W.cwWell[p]];
            bc[r] = s;
        }
    for (int w = 0; w < nw; ++w) free(wellCells[w]);
    free(wellCells);
    free(wellCount);
    wp_free(&W);
    return need;
}

/* engine/src/bsr.cpp:982-990 */
int orc_wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                          const double* xc, double* x) {
    (void)nrows;
    well_parts W;
    if (!wp_build(&W, rowPtr, col, val, na, nv, nw)) {
        wp_free(&W);
        return 0;
    }
    const int nc = na * nv;
    if (x != xc) memcpy(x, xc, sizeof(double) * (size_t)nc);
    for (int w = 0; w < nw; ++w) {
        double s = b[nc + w];
        for (int p = W.wcPtr[w]; p < W.wcPtr[w + 1]; ++p) s -= W.wcVal[p] * xc[W.wcCol[p]];
        x[nc + w] = s * W.dInv[w];
    }
    wp_free(&W);
    return 1;
}

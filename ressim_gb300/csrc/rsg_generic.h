// Block-size-generic solve path: BSR systems with nb x nb blocks, 1 <= nb <= 16 (compositional blocks are nc + 1
// wide, thermal 4-5), one system per handle, FP64. It serves the engine's other callers of the same solver -- the
// compositional simulator (engine/src/compsim.cpp:1366-1449: BlockCPR + GMRES(60)) and the thermal one
// (engine/src/thermsim.cpp:1816-1828: BlockCPR + GMRES(80)) -- through the same C ABI as the black-oil path.
//
// Arithmetic follows the reference's generic block kernels (engine/src/bsr.cpp:12-57, 67-87, 183-215, 437-596,
// 993-1084) operation for operation with separately rounded products and sums: the BILU0 factors, the CPR weights,
// the pressure matrix and the AMG hierarchy are the reference's bit for bit; the Krylov inner products are reduced
// in a fixed tree order.
#pragma once
#include "rsg.h"

#include <cuda_runtime.h>

namespace rsg {

struct GenEngine;

constexpr int GEN_MAX_NB = 16;        // engine/include/ressim/bsr.h:21 (kMaxBlock)

GenEngine* gen_create(cudaStream_t st);
void gen_destroy(GenEngine* g);
// pattern (kept when unchanged: values only) and values of one system, host arrays
int gen_set_matrix(GenEngine* g, const rsg_options& o, int n, int nb, const int* rowPtr, const int* col, const double* val);
// values already on the device, in the caller's block order
int gen_set_values_device(GenEngine* g, const double* d_val);
int gen_setup(GenEngine* g, const rsg_options& o, const double* acc);
int gen_solve_device(GenEngine* g, const rsg_options& o, const double* d_b, double* d_x, double tol, int maxIt, int* its, double* relres);
// host vectors (staged through the engine's own device buffers)
int gen_solve_host(GenEngine* g, const rsg_options& o, const double* b, double* x, double tol, int maxIt, int* its, double* relres);
int gen_spmv_host(GenEngine* g, const double* x, double* y);
int gen_precond_host(GenEngine* g, const double* r, double* z);
int gen_spmv_device(GenEngine* g, const double* d_x, double* d_y);
int gen_precond_device(GenEngine* g, const double* d_r, double* d_z);
int gen_get_factors(GenEngine* g, double* lu);
void gen_stats(const GenEngine* g, rsg_stats* st);
int gen_rows(const GenEngine* g);          // n * nb
int gen_amg_level_sizes(const GenEngine* g, int maxlev, long long* rows, long long* nnz, long long* dense);
bool gen_ready(const GenEngine* g);        // a matrix is set
bool gen_have_setup(const GenEngine* g);

}  // namespace rsg

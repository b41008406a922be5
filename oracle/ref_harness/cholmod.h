/*
 * cholmod.h -- the subset of the CHOLMOD API that LF_DEM's StokesSolver.cpp
 * calls, declared so the reference's own sources compile unmodified into the
 * oracle/_ref harness.  TEST INFRASTRUCTURE ONLY.
 *
 * SuiteSparse CHOLMOD is not vendored with LF_DEM and is not installed here.
 * cholmod_compat.cpp implements these entry points with a plain dense FP64
 * Cholesky (row/column order as given, no fill-reducing ordering), which is
 * adequate for the N <= ~500 systems used to pin the CPU restatement.  It is
 * NOT SuiteSparse CHOLMOD.
 */
#ifndef LFG_CHOLMOD_COMPAT_H
#define LFG_CHOLMOD_COMPAT_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#define CHOLMOD_REAL 1
#define CHOLMOD_DOUBLE 0
#define CHOLMOD_A 0
#define CHOLMOD_P 7
#define CHOLMOD_Pt 8
#define CHOLMOD_SIMPLICIAL 0
#define CHOLMOD_AUTO 1
#define CHOLMOD_SUPERNODAL 2
#define CHOLMOD_NATURAL 0
#define CHOLMOD_AMD 2
#define CHOLMOD_METIS 3
#define CHOLMOD_OK 0
#define CHOLMOD_NOT_POSDEF 1

typedef struct { int ordering; } cholmod_method_struct;

typedef struct cholmod_common_struct {
	int supernodal;
	int nmethods;
	cholmod_method_struct method[10];
	int status;
	int final_ll;
	int useGPU;
} cholmod_common;

typedef struct cholmod_sparse_struct {
	size_t nrow, ncol, nzmax;
	void *p, *i, *nz, *x, *z;
	int stype, itype, xtype, dtype, sorted, packed;
} cholmod_sparse;

typedef struct cholmod_dense_struct {
	size_t nrow, ncol, nzmax, d;
	void *x, *z;
	int xtype, dtype;
} cholmod_dense;

typedef struct cholmod_factor_struct {
	size_t n;
	int is_ll;
	double *L; /* dense lower factor, column-major n x n (compat only) */
	void *blk; /* block mode: the oracle's factor of the 6x6-block matrix */
} cholmod_factor;

/* Block mode (compat only): factorise through the oracle's block-matrix
 * factor (supernodal with BLAS kernels when those are set) instead of the
 * dense stand-in; for LF_DEM's 6x6-block R_FU at sizes where a dense factor
 * does not fit.  Solves with CHOLMOD_A only. */
void cholmod_compat_use_blocks(int on);

int cholmod_start(cholmod_common *c);
int cholmod_finish(cholmod_common *c);
cholmod_dense *cholmod_allocate_dense(size_t nrow, size_t ncol, size_t d, int xtype, cholmod_common *c);
int cholmod_free_dense(cholmod_dense **X, cholmod_common *c);
cholmod_dense *cholmod_copy_dense(cholmod_dense *X, cholmod_common *c);
cholmod_sparse *cholmod_allocate_sparse(size_t nrow, size_t ncol, size_t nzmax, int sorted,
                                        int packed, int stype, int xtype, cholmod_common *c);
int cholmod_reallocate_sparse(size_t nznew, cholmod_sparse *A, cholmod_common *c);
int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *c);
cholmod_dense *cholmod_sparse_to_dense(cholmod_sparse *A, cholmod_common *c);
cholmod_sparse *cholmod_transpose(cholmod_sparse *A, int values, cholmod_common *c);
cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *c);
int cholmod_factorize(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c);
int cholmod_free_factor(cholmod_factor **L, cholmod_common *c);
cholmod_factor *cholmod_copy_factor(cholmod_factor *L, cholmod_common *c);
cholmod_sparse *cholmod_factor_to_sparse(cholmod_factor *L, cholmod_common *c);
int cholmod_solve2(int sys, cholmod_factor *L, cholmod_dense *B, cholmod_sparse *Bset,
                   cholmod_dense **X_Handle, cholmod_sparse **Xset_Handle,
                   cholmod_dense **Y_Handle, cholmod_dense **E_Handle, cholmod_common *c);
int cholmod_sdmult(cholmod_sparse *A, int transpose, double alpha[2], double beta[2],
                   cholmod_dense *X, cholmod_dense *Y, cholmod_common *c);

#ifdef __cplusplus
}
#endif
#endif

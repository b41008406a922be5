// cholmod_compat.cpp -- dense FP64 stand-in for the CHOLMOD calls made by
// LF_DEM's StokesSolver.cpp.  TEST INFRASTRUCTURE ONLY (see cholmod.h).
#include "cholmod.h"
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {

int cholmod_start(cholmod_common *c)
{
	std::memset(c, 0, sizeof *c);
	c->supernodal = CHOLMOD_AUTO;
	c->final_ll = 1;
	return 1;
}

int cholmod_finish(cholmod_common *) { return 1; }

cholmod_dense *cholmod_allocate_dense(size_t nrow, size_t ncol, size_t d, int xtype, cholmod_common *)
{
	cholmod_dense *X = (cholmod_dense *)std::calloc(1, sizeof(cholmod_dense));
	X->nrow = nrow; X->ncol = ncol; X->d = d < nrow ? nrow : d;
	X->nzmax = X->d*ncol; X->xtype = xtype;
	X->x = std::calloc(X->nzmax ? X->nzmax : 1, sizeof(double));
	return X;
}

int cholmod_free_dense(cholmod_dense **X, cholmod_common *)
{
	if (X && *X) { std::free((*X)->x); std::free(*X); *X = nullptr; }
	return 1;
}

cholmod_dense *cholmod_copy_dense(cholmod_dense *X, cholmod_common *c)
{
	cholmod_dense *Y = cholmod_allocate_dense(X->nrow, X->ncol, X->d, X->xtype, c);
	std::memcpy(Y->x, X->x, sizeof(double)*X->nzmax);
	return Y;
}

cholmod_sparse *cholmod_allocate_sparse(size_t nrow, size_t ncol, size_t nzmax, int sorted,
                                        int packed, int stype, int xtype, cholmod_common *)
{
	cholmod_sparse *A = (cholmod_sparse *)std::calloc(1, sizeof(cholmod_sparse));
	A->nrow = nrow; A->ncol = ncol; A->nzmax = nzmax ? nzmax : 1;
	A->sorted = sorted; A->packed = packed; A->stype = stype; A->xtype = xtype;
	A->p = std::calloc(ncol+1, sizeof(int));
	A->i = std::calloc(A->nzmax, sizeof(int));
	A->x = std::calloc(A->nzmax, sizeof(double));
	return A;
}

int cholmod_reallocate_sparse(size_t nznew, cholmod_sparse *A, cholmod_common *)
{
	A->i = std::realloc(A->i, sizeof(int)*nznew);
	A->x = std::realloc(A->x, sizeof(double)*nznew);
	A->nzmax = nznew;
	return 1;
}

int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *)
{
	if (A && *A) { std::free((*A)->p); std::free((*A)->i); std::free((*A)->x); std::free(*A); *A = nullptr; }
	return 1;
}

static void to_dense_sym(const cholmod_sparse *A, double *M)
{
	size_t n = A->nrow;
	const int *p = (const int *)A->p, *ii = (const int *)A->i;
	const double *x = (const double *)A->x;
	std::memset(M, 0, sizeof(double)*n*A->ncol);
	for (size_t j = 0; j < A->ncol; j++) {
		for (int k = p[j]; k < p[j+1]; k++) {
			size_t i = (size_t)ii[k];
			M[i+j*n] += x[k];
			if (A->stype != 0 && i != j) M[j+i*n] += x[k];
		}
	}
}

cholmod_dense *cholmod_sparse_to_dense(cholmod_sparse *A, cholmod_common *c)
{
	cholmod_dense *X = cholmod_allocate_dense(A->nrow, A->ncol, A->nrow, CHOLMOD_REAL, c);
	to_dense_sym(A, (double *)X->x);
	return X;
}

cholmod_sparse *cholmod_transpose(cholmod_sparse *A, int, cholmod_common *c)
{
	size_t m = A->nrow, n = A->ncol;
	const int *p = (const int *)A->p, *ii = (const int *)A->i;
	const double *x = (const double *)A->x;
	size_t nnz = (size_t)p[n];
	cholmod_sparse *T = cholmod_allocate_sparse(n, m, nnz, 1, 1, -A->stype, A->xtype, c);
	std::vector<int> cnt(m+1, 0);
	for (size_t k = 0; k < nnz; k++) cnt[ii[k]+1]++;
	for (size_t r = 0; r < m; r++) cnt[r+1] += cnt[r];
	int *tp = (int *)T->p, *ti = (int *)T->i;
	double *tx = (double *)T->x;
	for (size_t r = 0; r <= m; r++) tp[r] = cnt[r];
	std::vector<int> pos(cnt.begin(), cnt.end()-1);
	for (size_t j = 0; j < n; j++)
		for (int k = p[j]; k < p[j+1]; k++) {
			int d = pos[ii[k]]++;
			ti[d] = (int)j; tx[d] = x[k];
		}
	return T;
}

cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *)
{
	cholmod_factor *L = (cholmod_factor *)std::calloc(1, sizeof(cholmod_factor));
	L->n = A->nrow;
	L->is_ll = 1;
	L->L = (double *)std::calloc(L->n*L->n, sizeof(double));
	return L;
}

// dense right-looking Cholesky of the lower triangle, column-major
int cholmod_factorize(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c)
{
	size_t n = A->nrow;
	double *M = L->L;
	to_dense_sym(A, M);
	c->status = CHOLMOD_OK;
	for (size_t j = 0; j < n; j++) {
		double d = M[j+j*n];
		if (!(d > 0)) { c->status = CHOLMOD_NOT_POSDEF; return 0; }
		d = std::sqrt(d);
		M[j+j*n] = d;
		double inv = 1.0/d;
		for (size_t i = j+1; i < n; i++) M[i+j*n] *= inv;
		for (size_t k = j+1; k < n; k++) {
			double lkj = M[k+j*n];
			if (lkj == 0) continue;
			double *colk = &M[k*n];
			const double *colj = &M[j*n];
			for (size_t i = k; i < n; i++) colk[i] -= colj[i]*lkj;
		}
	}
	return 1;
}

int cholmod_free_factor(cholmod_factor **L, cholmod_common *)
{
	if (L && *L) { std::free((*L)->L); std::free(*L); *L = nullptr; }
	return 1;
}

cholmod_factor *cholmod_copy_factor(cholmod_factor *L, cholmod_common *)
{
	cholmod_factor *C = (cholmod_factor *)std::calloc(1, sizeof(cholmod_factor));
	C->n = L->n; C->is_ll = L->is_ll;
	C->L = (double *)std::malloc(sizeof(double)*L->n*L->n);
	std::memcpy(C->L, L->L, sizeof(double)*L->n*L->n);
	return C;
}

cholmod_sparse *cholmod_factor_to_sparse(cholmod_factor *L, cholmod_common *c)
{
	size_t n = L->n;
	size_t nnz = n*(n+1)/2;
	cholmod_sparse *S = cholmod_allocate_sparse(n, n, nnz, 1, 1, 0, CHOLMOD_REAL, c);
	int *p = (int *)S->p, *ii = (int *)S->i;
	double *x = (double *)S->x;
	size_t k = 0;
	for (size_t j = 0; j < n; j++) {
		p[j] = (int)k;
		for (size_t i = j; i < n; i++) { ii[k] = (int)i; x[k] = L->L[i+j*n]; k++; }
	}
	p[n] = (int)k;
	return S;
}

int cholmod_solve2(int sys, cholmod_factor *L, cholmod_dense *B, cholmod_sparse *,
                   cholmod_dense **X_Handle, cholmod_sparse **, cholmod_dense **,
                   cholmod_dense **, cholmod_common *c)
{
	size_t n = L->n;
	if (!*X_Handle || (*X_Handle)->nrow != B->nrow || (*X_Handle)->ncol != B->ncol) {
		cholmod_free_dense(X_Handle, c);
		*X_Handle = cholmod_allocate_dense(B->nrow, B->ncol, B->nrow, CHOLMOD_REAL, c);
	}
	for (size_t col = 0; col < B->ncol; col++) {
		const double *b = (const double *)B->x + col*B->d;
		double *x = (double *)(*X_Handle)->x + col*(*X_Handle)->d;
		std::memcpy(x, b, sizeof(double)*n);
		if (sys != CHOLMOD_A) continue; /* identity permutation: P, Pt are copies */
		const double *M = L->L;
		for (size_t j = 0; j < n; j++) {
			x[j] /= M[j+j*n];
			double xj = x[j];
			for (size_t i = j+1; i < n; i++) x[i] -= M[i+j*n]*xj;
		}
		for (size_t jj = n; jj-- > 0;) {
			double v = x[jj];
			for (size_t i = jj+1; i < n; i++) v -= M[i+jj*n]*x[i];
			x[jj] = v/M[jj+jj*n];
		}
	}
	return 1;
}

int cholmod_sdmult(cholmod_sparse *A, int transpose, double alpha[2], double beta[2],
                   cholmod_dense *X, cholmod_dense *Y, cholmod_common *)
{
	const int *p = (const int *)A->p, *ii = (const int *)A->i;
	const double *ax = (const double *)A->x;
	size_t ny = transpose && A->stype == 0 ? A->ncol : A->nrow;
	for (size_t col = 0; col < X->ncol; col++) {
		const double *x = (const double *)X->x + col*X->d;
		double *y = (double *)Y->x + col*Y->d;
		std::vector<double> acc(ny, 0.0);
		for (size_t j = 0; j < A->ncol; j++) {
			for (int k = p[j]; k < p[j+1]; k++) {
				size_t i = (size_t)ii[k];
				if (A->stype != 0) {
					acc[i] += ax[k]*x[j];
					if (i != j) acc[j] += ax[k]*x[i];
				} else if (!transpose) {
					acc[i] += ax[k]*x[j];
				} else {
					acc[j] += ax[k]*x[i];
				}
			}
		}
		for (size_t i = 0; i < ny; i++) y[i] = alpha[0]*acc[i] + beta[0]*y[i];
	}
	return 1;
}

} // extern "C"

// cholmod_compat.cpp -- dense FP64 stand-in for the CHOLMOD calls made by
// LF_DEM's StokesSolver.cpp.  TEST INFRASTRUCTURE ONLY (see cholmod.h).
#include "cholmod.h"
#include "../lfdem_oracle.h"
#include <cmath>
#include <cstdio>
#include <map>
#include <utility>
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

static int g_blocks = 0;
void cholmod_compat_use_blocks(int on) { g_blocks = on; }

cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *)
{
	cholmod_factor *L = (cholmod_factor *)std::calloc(1, sizeof(cholmod_factor));
	L->n = A->nrow;
	L->is_ll = 1;
	if (!g_blocks) L->L = (double *)std::calloc(L->n*L->n, sizeof(double));
	return L;
}

// block mode: the lower scalar CSC (stype -1) as 6x6 blocks, factored by the
// oracle (row-major blocks; off-diagonal ones with block row > block column)
static int factorize_blocks(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c)
{
	size_t n = A->nrow;
	if (n%6) { std::fprintf(stderr, "cholmod_compat: block mode needs 6 unknowns per particle\n"); std::abort(); }
	int nblk = (int)(n/6);
	const int *p = (const int *)A->p, *ii = (const int *)A->i;
	const double *x = (const double *)A->x;
	std::vector<double> diag((size_t)nblk*36, 0.0), off;
	std::vector<int> brow, bcol;
	std::map<std::pair<int, int>, int> index;
	for (size_t j = 0; j < A->ncol; j++) {
		int bj = (int)(j/6), cj = (int)(j%6);
		for (int k = p[j]; k < p[j+1]; k++) {
			int i = ii[k];
			if ((size_t)i < j) continue;   // lower part only
			int bi = i/6, ci = i%6;
			if (bi == bj) {
				diag[(size_t)bi*36+ci*6+cj] += x[k];
				if (ci != cj) diag[(size_t)bi*36+cj*6+ci] += x[k];
			} else {
				auto key = std::make_pair(bi, bj);
				auto it = index.find(key);
				int e;
				if (it == index.end()) {
					e = (int)brow.size();
					index[key] = e;
					brow.push_back(bi); bcol.push_back(bj);
					off.resize(off.size()+36, 0.0);
				} else {
					e = it->second;
				}
				off[(size_t)e*36+ci*6+cj] += x[k];
			}
		}
	}
	if (L->blk) lfo_factor_free((lfo_factor *)L->blk);
	int status = 0;
	L->blk = lfo_factor_create(nblk, diag.data(), (int)brow.size(), brow.data(), bcol.data(),
	                           off.empty() ? nullptr : off.data(), &status);
	c->status = status ? CHOLMOD_NOT_POSDEF : CHOLMOD_OK;
	return status ? 0 : 1;
}

// dense right-looking Cholesky of the lower triangle, column-major
int cholmod_factorize(cholmod_sparse *A, cholmod_factor *L, cholmod_common *c)
{
	if (g_blocks) return factorize_blocks(A, L, c);
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
	if (L && *L) {
		if ((*L)->blk) lfo_factor_free((lfo_factor *)(*L)->blk);
		std::free((*L)->L); std::free(*L); *L = nullptr;
	}
	return 1;
}

cholmod_factor *cholmod_copy_factor(cholmod_factor *L, cholmod_common *)
{
	if (L->blk) { std::fprintf(stderr, "cholmod_compat: no factor copy in block mode\n"); std::abort(); }
	cholmod_factor *C = (cholmod_factor *)std::calloc(1, sizeof(cholmod_factor));
	C->n = L->n; C->is_ll = L->is_ll;
	C->L = (double *)std::malloc(sizeof(double)*L->n*L->n);
	std::memcpy(C->L, L->L, sizeof(double)*L->n*L->n);
	return C;
}

cholmod_sparse *cholmod_factor_to_sparse(cholmod_factor *L, cholmod_common *c)
{
	if (L->blk) { std::fprintf(stderr, "cholmod_compat: no sparse factor in block mode\n"); std::abort(); }
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
	if (L->blk) {
		if (sys != CHOLMOD_A) { std::fprintf(stderr, "cholmod_compat: block mode solves CHOLMOD_A only\n"); std::abort(); }
		for (size_t col = 0; col < B->ncol; col++)
			lfo_factor_solve((const lfo_factor *)L->blk, 1, (const double *)B->x+col*B->d,
			                 (double *)(*X_Handle)->x+col*(*X_Handle)->d);
		return 1;
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

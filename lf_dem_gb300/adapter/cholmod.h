/*
 * cholmod.h -- the CHOLMOD type names that LF_DEM's StokesSolver.h and
 * System.h mention, for building LF_DEM with StokesSolverGB300.cpp in place
 * of StokesSolver.cpp without SuiteSparse.  StokesSolver.h keeps CHOLMOD
 * objects as private members (one by value), so the types must be complete;
 * the GB300 adapter never touches them and nothing from CHOLMOD is called or
 * linked.  A build that keeps SuiteSparse on its include path can use
 * SuiteSparse's own cholmod.h instead.
 */
#ifndef LFG_ADAPTER_CHOLMOD_TYPES_H
#define LFG_ADAPTER_CHOLMOD_TYPES_H
#include <stddef.h>

typedef struct { int unused; } cholmod_factor;
typedef struct { int unused; size_t nrow, ncol; void *x; } cholmod_dense;
typedef struct { int unused; size_t nrow, ncol; void *p, *i, *x; } cholmod_sparse;
typedef struct { int unused; } cholmod_common;

#endif

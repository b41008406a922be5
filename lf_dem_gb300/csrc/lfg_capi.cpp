// lfg_capi.cpp -- extern "C" entry points of include/lfdem_gb300.h for the
// resistance solver (lfg_solver_*) and library information.  C++ exceptions
// never cross this boundary: every entry point returns a status code.
#include <cstdio>
#include <cstring>
#include <new>

#include "lfg_solver.h"

using namespace lfg;

struct lfg_solver {
	cudaStream_t stream = nullptr;
	Solver *s = nullptr;
	int device = 0;
};

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg)
{
	if (st) {
		st->code = code;
		st->info = info;
		snprintf(st->msg, sizeof st->msg, "%s", msg);
	}
	return code;
}

int ok(lfg_status *st)
{
	if (st) {
		st->code = LFG_OK;
		st->info = 0;
		st->msg[0] = 0;
	}
	return LFG_OK;
}

int check_device(int device, lfg_status *st)
{
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0)
		return fail(st, LFG_ERR_NO_DEVICE, device, "no CUDA device");
	cudaDeviceProp p;
	if (cudaGetDeviceProperties(&p, device) != cudaSuccess)
		return fail(st, LFG_ERR_NO_DEVICE, device, "cannot query device");
	if (p.major != 10 || p.minor != 3)
		return fail(st, LFG_ERR_NO_DEVICE, p.major*10+p.minor,
		            "this build targets sm_103a (GB300); device has a different architecture");
	if (cudaSetDevice(device) != cudaSuccess) return fail(st, LFG_ERR_NO_DEVICE, device, "cudaSetDevice failed");
	return LFG_OK;
}
} // namespace lfg

#define LFG_GUARD_BEGIN try {
#define LFG_GUARD_END                                                              \
	}                                                                              \
	catch (const lfg::Error &e) { return fail(st, e.code, e.info, e.msg.c_str()); } \
	catch (const std::bad_alloc &) { return fail(st, LFG_ERR_OOM, 0, "host allocation failed"); } \
	catch (...) { return fail(st, LFG_ERR_CUDA, 0, "unexpected exception"); }

extern "C" {

void lfg_default_options(lfg_options *o)
{
	std::memset(o, 0, sizeof *o);
	o->precision = LFG_PREC_FP64;
	o->device = 0;
	o->refine_tol = 2e-10;
	o->refine_max_iter = 30;
	o->skin = 0.15;
	o->use_graphs = 1;
	o->leaf_size = 16;
	o->dof_2d = 3;
}

int lfg_device_info(int device, char *name, int name_len, int *sm_major, int *sm_minor, int *sm_count)
{
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || device >= n || device < 0) return LFG_ERR_NO_DEVICE;
	cudaDeviceProp p;
	if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return LFG_ERR_NO_DEVICE;
	if (name && name_len > 0) snprintf(name, name_len, "%s", p.name);
	if (sm_major) *sm_major = p.major;
	if (sm_minor) *sm_minor = p.minor;
	if (sm_count) *sm_count = p.multiProcessorCount;
	return (p.major == 10 && p.minor == 3) ? LFG_OK : LFG_ERR_NO_DEVICE;
}

int lfg_solver_create(int n_mobile, int dof, const lfg_options *opt, lfg_solver **out, lfg_status *st)
{
	if (!out || n_mobile <= 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	if (dof != 6 && dof != 3) return fail(st, LFG_ERR_BAD_ARG, dof, "degrees of freedom per particle must be 6 or 3");
	lfg_options o;
	if (opt) o = *opt; else lfg_default_options(&o);
	if (o.precision != LFG_PREC_FP64 && o.precision != LFG_PREC_FP32_REFINE)
		return fail(st, LFG_ERR_BAD_ARG, o.precision, "unknown precision");
	int rc = check_device(o.device, st);
	if (rc) return rc;
	lfg_solver *h = nullptr;
	LFG_GUARD_BEGIN
	h = new lfg_solver();
	h->device = o.device;
	LFG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
	h->s = new Solver(n_mobile, o, h->stream, dof);
	*out = h;
	return ok(st);
	}
	catch (const lfg::Error &e) {
		if (h) { delete h->s; if (h->stream) cudaStreamDestroy(h->stream); delete h; }
		return fail(st, e.code, e.info, e.msg.c_str());
	}
	catch (...) {
		if (h) { delete h->s; if (h->stream) cudaStreamDestroy(h->stream); delete h; }
		return fail(st, LFG_ERR_OOM, 0, "allocation failed");
	}
}

int lfg_solver_set_blocks(lfg_solver *h, const double *dblocks, int nb, const int32_t *od_row,
                          const int32_t *od_col, const double *odblocks, int pattern_changed,
                          const double *positions, lfg_status *st)
{
	if (!h || !dblocks || nb < 0 || (nb > 0 && (!od_row || !od_col || !odblocks)))
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	LFG_GUARD_BEGIN
	cudaSetDevice(h->device);
	if (pattern_changed || !h->s->analyzed() || nb != h->s->nb())
		h->s->set_pattern(nb, od_row, od_col, positions, 0, positions ? 1 : 0, 0, false);
	h->s->set_values_host(dblocks, odblocks);
	return ok(st);
	LFG_GUARD_END
}

int lfg_solver_factorize(lfg_solver *h, lfg_status *st)
{
	if (!h) return fail(st, LFG_ERR_BAD_ARG, 0, "null solver");
	LFG_GUARD_BEGIN
	cudaSetDevice(h->device);
	h->s->factorize_async();
	int rc = h->s->check_factor(st);
	if (rc) return rc;
	return ok(st);
	LFG_GUARD_END
}

int lfg_solver_multiply_factor(lfg_solver *h, int k, const double *rhs, double *x, lfg_status *st)
{
	if (!h || k < 0 || (k > 0 && (!rhs || !x))) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	LFG_GUARD_BEGIN
	cudaSetDevice(h->device);
	int rc = h->s->multiply_host(k, rhs, x, st);
	if (rc) return rc;
	return ok(st);
	LFG_GUARD_END
}

int lfg_solver_solve(lfg_solver *h, int k, const double *rhs, double *x, lfg_status *st)
{
	if (!h || k < 0 || (k > 0 && (!rhs || !x))) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	LFG_GUARD_BEGIN
	cudaSetDevice(h->device);
	int rc = h->s->solve_host(k, rhs, x, st);
	if (rc) return rc;
	int it = h->s->last_iters();
	double res = h->s->last_resid();
	ok(st);
	if (st) { st->refine_iters = it; st->refine_residual = res; }
	return LFG_OK;
	LFG_GUARD_END
}

int lfg_solver_solve_device(lfg_solver *h, int k, const double *d_rhs, double *d_x, lfg_status *st)
{
	if (!h || k < 0 || (k > 0 && (!d_rhs || !d_x))) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	LFG_GUARD_BEGIN
	cudaSetDevice(h->device);
	int rc = h->s->solve_device(k, d_rhs, d_x, st, true);
	if (rc) return rc;
	LFG_CUDA(cudaStreamSynchronize(h->stream));
	return ok(st);
	LFG_GUARD_END
}

int lfg_solver_get_stats(const lfg_solver *h, lfg_solver_stats *out)
{
	if (!h || !out) return LFG_ERR_BAD_ARG;
	h->s->stats(out);
	return LFG_OK;
}

void lfg_solver_destroy(lfg_solver *h)
{
	if (!h) return;
	cudaSetDevice(h->device);
	delete h->s;
	if (h->stream) cudaStreamDestroy(h->stream);
	delete h;
}

} // extern "C"

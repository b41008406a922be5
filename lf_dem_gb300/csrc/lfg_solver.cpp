// lfg_solver.cpp -- the resistance solve behind LF_DEM's StokesSolver
// (StokesSolver.h:198-285), as a device object: compact block matrix in HBM,
// symbolic analysis on pattern change only (StokesSolver.cpp:955-962),
// multifrontal factorisation in FP64 or FP32, solves with k right-hand sides,
// FP64 iterative refinement for the FP32 form.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "lfg_solver.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);

Solver::Solver(int n, const lfg_options &o, cudaStream_t st, int dof, bool analysis_only)
    : n_(n), dof_(dof), analysis_only_(analysis_only), opt_(o), st_(st)
{
	if (dof != 6 && dof != 3) throw Error{LFG_ERR_BAD_ARG, dof, "degrees of freedom per particle must be 6 or 3"};
	A_.n = n;
	A_.dof = dof;
	LFG_CUDA(cudaMalloc((void **)&A_.dblocks, sizeof(double)*15*(size_t)std::max(n, 1)));
	LFG_CUDA(cudaMalloc((void **)&A_.lo_ptr, sizeof(int)*(n+1)));
	LFG_CUDA(cudaMalloc((void **)&A_.up_ptr, sizeof(int)*(n+1)));
	LFG_CUDA(cudaMallocHost((void **)&h_norms_, sizeof(double)*64));
	LFG_CUDA(cudaMalloc((void **)&d_norms_, sizeof(double)*64));
	LFG_CUDA(cudaMallocHost((void **)&h_status_, sizeof(int)*4));
}

Solver::~Solver()
{
	dev_symbolic_free(D_);
	factor_free(F64_);
	factor_free(F32_);
	void *p[] = {A_.dblocks, A_.odblocks, A_.od_row, A_.od_col, A_.lo_ptr, A_.lo_idx, A_.up_ptr, A_.up_idx,
	             d_norms_, ref_x_, ref_r_, ref_d_, hb_, hx_, d_seg_};
	for (void *q : p) if (q) cudaFree(q);
	if (h_norms_) cudaFreeHost(h_norms_);
	if (h_status_) cudaFreeHost(h_status_);
	for (auto &g : graphs_) if (g.exec) cudaGraphExecDestroy(g.exec);
}

void Solver::set_pattern(int nb, const int32_t *row, const int32_t *col, const double *pos, double lx,
                         double ly, double lz, bool device_ptrs)
{
	std::vector<int32_t> r(nb), c(nb);
	if (device_ptrs) {
		if (nb) {
			LFG_CUDA(cudaMemcpyAsync(r.data(), row, sizeof(int32_t)*nb, cudaMemcpyDeviceToHost, st_));
			LFG_CUDA(cudaMemcpyAsync(c.data(), col, sizeof(int32_t)*nb, cudaMemcpyDeviceToHost, st_));
			LFG_CUDA(cudaStreamSynchronize(st_));
		}
	} else {
		std::copy(row, row+nb, r.begin());
		std::copy(col, col+nb, c.begin());
	}
	for (int e = 0; e < nb; e++)
		if (r[e] <= c[e] || r[e] >= n_ || c[e] < 0)
			throw Error{LFG_ERR_BAD_ARG, e, "off-diagonal block must have n > row > col >= 0"};
	nb_ = nb;
	pat_r_ = r;
	pat_c_ = c;
	pat_pos_.assign(pos ? pos : nullptr, pos ? pos+3*(size_t)n_ : nullptr);
	pat_box_[0] = lx; pat_box_[1] = ly; pat_box_[2] = lz;
	symbolic_analyze(S_, n_, nb, r.data(), c.data(), pos, lx, ly, lz, opt_.leaf_size, dof_);
	if (analysis_only_) {
		analyzed_ = true;
		symbolic_runs_++;
		return;
	}
	upload(r, c);
}

// A symbolic analysis made elsewhere (a joint analysis of several
// suspensions) for the pattern (row, col): upload and allocate as set_pattern.
void Solver::install(Symbolic &&S, int nb, const int32_t *row, const int32_t *col)
{
	if (S.nblk != n_ || S.dof != dof_) throw Error{LFG_ERR_BAD_ARG, S.nblk, "symbolic analysis of another system"};
	std::vector<int32_t> r(row, row+nb), c(col, col+nb);
	nb_ = nb;
	pat_r_ = r;
	pat_c_ = c;
	pat_pos_.clear();
	S_ = std::move(S);
	upload(r, c);
}

void Solver::upload(const std::vector<int32_t> &r, const std::vector<int32_t> &c)
{
	const int nb = nb_;
	dev_symbolic_upload(D_, S_, nb, factor_panel_width(opt_.precision), factor_tile_size(opt_.precision),
	                    factor_syrk_tile_size(opt_.precision), opt_.precision == LFG_PREC_FP32_REFINE, st_);
	if (opt_.precision == LFG_PREC_FP64) factor_alloc(F64_, D_, 4);
	else factor_alloc(F32_, D_, 4);
	// block matrix pattern + row adjacency for the residual
	if (A_.odblocks) cudaFree(A_.odblocks);
	if (A_.od_row) cudaFree(A_.od_row);
	if (A_.od_col) cudaFree(A_.od_col);
	if (A_.lo_idx) cudaFree(A_.lo_idx);
	if (A_.up_idx) cudaFree(A_.up_idx);
	A_.odblocks = nullptr; A_.od_row = A_.od_col = A_.lo_idx = A_.up_idx = nullptr;
	A_.nb = nb;
	size_t nbb = std::max(nb, 1);
	LFG_CUDA(cudaMalloc((void **)&A_.odblocks, sizeof(double)*18*nbb));
	LFG_CUDA(cudaMalloc((void **)&A_.od_row, sizeof(int)*nbb));
	LFG_CUDA(cudaMalloc((void **)&A_.od_col, sizeof(int)*nbb));
	LFG_CUDA(cudaMalloc((void **)&A_.lo_idx, sizeof(int)*nbb));
	LFG_CUDA(cudaMalloc((void **)&A_.up_idx, sizeof(int)*nbb));
	std::vector<int> lp(n_+1, 0), upp(n_+1, 0), li(nb), ui(nb);
	for (int e = 0; e < nb; e++) { lp[r[e]+1]++; upp[c[e]+1]++; }
	for (int i = 0; i < n_; i++) { lp[i+1] += lp[i]; upp[i+1] += upp[i]; }
	{
		std::vector<int> f1(lp.begin(), lp.end()-1), f2(upp.begin(), upp.end()-1);
		for (int e = 0; e < nb; e++) { li[f1[r[e]]++] = e; ui[f2[c[e]]++] = e; }
	}
	if (nb) {
		LFG_CUDA(cudaMemcpyAsync(A_.od_row, r.data(), sizeof(int)*nb, cudaMemcpyHostToDevice, st_));
		LFG_CUDA(cudaMemcpyAsync(A_.od_col, c.data(), sizeof(int)*nb, cudaMemcpyHostToDevice, st_));
		LFG_CUDA(cudaMemcpyAsync(A_.lo_idx, li.data(), sizeof(int)*nb, cudaMemcpyHostToDevice, st_));
		LFG_CUDA(cudaMemcpyAsync(A_.up_idx, ui.data(), sizeof(int)*nb, cudaMemcpyHostToDevice, st_));
	}
	LFG_CUDA(cudaMemcpyAsync(A_.lo_ptr, lp.data(), sizeof(int)*(n_+1), cudaMemcpyHostToDevice, st_));
	LFG_CUDA(cudaMemcpyAsync(A_.up_ptr, upp.data(), sizeof(int)*(n_+1), cudaMemcpyHostToDevice, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	for (auto &g : graphs_) if (g.exec) cudaGraphExecDestroy(g.exec);
	graphs_.clear();
	analyzed_ = true;
	symbolic_runs_++;
}

void Solver::reanalyze(int leaf_size)
{
	if (!analyzed_) throw Error{LFG_ERR_BAD_ARG, 0, "reanalyze before the first analysis"};
	if (leaf_size < 1) throw Error{LFG_ERR_BAD_ARG, leaf_size, "leaf size must be positive"};
	opt_.leaf_size = leaf_size;
	std::vector<int32_t> r = pat_r_, c = pat_c_;
	std::vector<double> pos = pat_pos_;
	set_pattern(nb_, r.data(), c.data(), pos.empty() ? nullptr : pos.data(), pat_box_[0], pat_box_[1], pat_box_[2],
	            false);
}

void Solver::set_values_host(const double *dblocks, const double *odblocks)
{
	LFG_CUDA(cudaMemcpyAsync(A_.dblocks, dblocks, sizeof(double)*15*n_, cudaMemcpyHostToDevice, st_));
	if (nb_) LFG_CUDA(cudaMemcpyAsync(A_.odblocks, odblocks, sizeof(double)*18*nb_, cudaMemcpyHostToDevice, st_));
}

// Launch the factorisation; with graphs, the launch sequence is captured once
// per symbolic analysis and replayed.
void Solver::factorize_async()
{
	if (!analyzed_) throw Error{LFG_ERR_BAD_ARG, 0, "factorize before set_blocks"};
	auto body = [&]() {
		if (opt_.precision == LFG_PREC_FP64) launches_factor_ = factor_numeric(F64_, D_, A_.dblocks, A_.odblocks, st_);
		else launches_factor_ = factor_numeric(F32_, D_, A_.dblocks, A_.odblocks, st_);
	};
	run_graph(0, 0, A_.dblocks, A_.odblocks, body);
}

void Solver::run_graph(int kind, int k, const void *b, const void *x, const std::function<void()> &body)
{
	if (!opt_.use_graphs) {
		body();
		kernels_ += kind == 0 ? launches_factor_ : launches_solve_+(kind == 2 ? 3 : 0);
		return;
	}
	for (auto &g : graphs_) {
		if (g.kind == kind && g.k == k && g.b == b && g.x == x) {
			LFG_CUDA(cudaGraphLaunch(g.exec, st_));
			kernels_ += g.nodes;
			return;
		}
	}
	auto t0 = std::chrono::steady_clock::now();
	cudaGraph_t graph;
	LFG_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
	try {
		body();
	} catch (...) {
		cudaStreamEndCapture(st_, &graph);
		throw;
	}
	LFG_CUDA(cudaStreamEndCapture(st_, &graph));
	GraphEntry e;
	e.kind = kind; e.k = k; e.b = b; e.x = x;
	size_t nn = 0;
	LFG_CUDA(cudaGraphGetNodes(graph, nullptr, &nn));
	std::vector<cudaGraphNode_t> nodes(nn);
	if (nn) LFG_CUDA(cudaGraphGetNodes(graph, nodes.data(), &nn));
	e.nodes = 0;   // kernel nodes only (memsets and copies are not launches)
	for (size_t q = 0; q < nn; q++) {
		cudaGraphNodeType t;
		LFG_CUDA(cudaGraphNodeGetType(nodes[q], &t));
		if (t == cudaGraphNodeTypeKernel) e.nodes++;
	}
	LFG_CUDA(cudaGraphInstantiate(&e.exec, graph, 0));
	cudaGraphDestroy(graph);
	graphs_.push_back(e);
	capture_ms_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now()-t0).count();
	LFG_CUDA(cudaGraphLaunch(e.exec, st_));
	kernels_ += e.nodes;
}

int Solver::check_factor(lfg_status *st)
{
	int *dst = opt_.precision == LFG_PREC_FP64 ? F64_.status : F32_.status;
	LFG_CUDA(cudaMemcpyAsync(h_status_, dst, sizeof(int), cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	if (*h_status_ == 0) return fail(st, LFG_ERR_TIMEOUT, 0, "a bounded device wait gave up");
	if (*h_status_ != 0x7fffffff) {
		int q = *h_status_-1;
		// scalar column of the caller's 6-per-particle numbering (dof 3:
		// components 0, 2, 4)
		int orig = dof_ == 6 ? S_.perm[q/6]*6+q%6 : S_.perm[q/3]*6+2*(q%3);
		if (st) {
			st->code = LFG_ERR_NOT_SPD;
			st->info = orig+1;
			snprintf(st->msg, sizeof st->msg, "non-positive pivot at column %d (particle %d)", orig, orig/6);
		}
		return LFG_ERR_NOT_SPD;
	}
	return LFG_OK;
}

void Solver::ensure_refine_ws(int k)
{
	int64_t need = (int64_t)6*n_*std::max(k, 1);
	if (ref_cap_ >= need) return;
	if (ref_x_) cudaFree(ref_x_);
	if (ref_r_) cudaFree(ref_r_);
	if (ref_d_) cudaFree(ref_d_);
	LFG_CUDA(cudaMalloc((void **)&ref_x_, sizeof(double)*need));
	LFG_CUDA(cudaMalloc((void **)&ref_r_, sizeof(double)*need));
	LFG_CUDA(cudaMalloc((void **)&ref_d_, sizeof(double)*need));
	ref_cap_ = need;
}

// k RHS on the device.  FP64: one direct solve.  FP32: x = 0, repeat
// { d = (L L^T)_32^-1 r ; x += d ; r = b - A x } until max relative residual
// <= refine_tol.
int Solver::solve_device(int k, const double *b, double *x, lfg_status *st, bool sync_check)
{
	if (k <= 0) return LFG_OK;
	if (opt_.precision == LFG_PREC_FP64) {
		run_graph(1, k, b, x, [&]() { launches_solve_ = factor_solve(F64_, D_, k, b, x, st_); });
		last_iters_ = 0;
		last_resid_ = 0;
		return LFG_OK;
	}
	refine_begin(k, b);
	int it = 0;
	double worst = 0;
	int batch = std::max(1, std::min(pred_iters_, opt_.refine_max_iter));
	while (it < opt_.refine_max_iter) {
		int j = std::min(batch, opt_.refine_max_iter-it);
		run_graph(2, k*64+j, b, nullptr, [&]() { refine_iterations(k, b, j); });
		it += j;
		worst = refine_worst(k);
		if (worst <= opt_.refine_tol) break;
		batch = 1;
	}
	pred_iters_ = it;
	return refine_finish(k, x, it, worst, st);
}

// FP32 refinement in pieces.  refine_begin: x = 0, r = b.  refine_iterations:
// j times { d = (L L^T)_32^-1 r in FP32; x += d; r = b - A x in FP64 }, then
// the squared norms of r and b per right-hand side (and per segment); these
// only launch work, so a caller may capture them in its own graph.
// refine_worst: waits and returns the largest relative residual.
// refine_finish: copies x out and records the counts.
void Solver::refine_begin(int k, const double *b)
{
	ensure_refine_ws(k);
	int64_t tot = (int64_t)6*n_*k;
	LFG_CUDA(cudaMemsetAsync(ref_x_, 0, sizeof(double)*tot, st_));
	LFG_CUDA(cudaMemcpyAsync(ref_r_, b, sizeof(double)*tot, cudaMemcpyDeviceToDevice, st_));
}

void Solver::refine_iterations(int k, const double *b, int j)
{
	for (int q = 0; q < j; q++) {
		launches_solve_ = factor_solve(F32_, D_, k, ref_r_, ref_d_, st_);
		axpy_vec(n_, k, ref_d_, ref_x_, st_);
		block_residual(A_, k, b, ref_x_, ref_r_, st_);
	}
	residual_norms(6*n_, k, ref_r_, b, d_norms_, st_, seg_.empty() ? nullptr : d_seg_, (int)seg_.size()-1);
}

double Solver::refine_worst(int k)
{
	int nseg = seg_.empty() ? 1 : (int)seg_.size()-1;
	LFG_CUDA(cudaMemcpyAsync(h_norms_, d_norms_, sizeof(double)*2*k*nseg, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	double worst = 0;
	for (int r = 0; r < k*nseg; r++) {
		double rb = h_norms_[2*r+1] > 0 ? std::sqrt(h_norms_[2*r]/h_norms_[2*r+1]) : std::sqrt(h_norms_[2*r]);
		if (!(rb == rb)) rb = INFINITY;
		worst = std::max(worst, rb);
	}
	return worst;
}

int Solver::refine_finish(int k, double *x, int iters, double worst, lfg_status *st)
{
	int64_t tot = (int64_t)6*n_*k;
	last_iters_ = iters;
	last_resid_ = worst;
	LFG_CUDA(cudaMemcpyAsync(x, ref_x_, sizeof(double)*tot, cudaMemcpyDeviceToDevice, st_));
	if (st) { st->refine_iters = last_iters_; st->refine_residual = worst; }
	if (!(worst <= opt_.refine_tol)) {
		if (st) {
			st->code = LFG_ERR_NOT_CONVERGED;
			snprintf(st->msg, sizeof st->msg, "FP32 refinement reached %.3e after %d iterations", worst, last_iters_);
		}
		return LFG_ERR_NOT_CONVERGED;
	}
	return LFG_OK;
}

// Per-suspension segments of a joint system (particle offsets, nseg + 1):
// the refinement's convergence test takes the largest relative residual over
// the segments, so every suspension meets the tolerance on its own.
void Solver::set_segments(const std::vector<int> &particle_off)
{
	seg_.resize(particle_off.size());
	for (size_t q = 0; q < particle_off.size(); q++) seg_[q] = 6*particle_off[q];
	if (d_seg_) cudaFree(d_seg_);
	d_seg_ = nullptr;
	LFG_CUDA(cudaMalloc((void **)&d_seg_, sizeof(int)*std::max<size_t>(seg_.size(), 1)));
	LFG_CUDA(cudaMemcpyAsync(d_seg_, seg_.data(), sizeof(int)*seg_.size(), cudaMemcpyHostToDevice, st_));
	size_t need = 2*8*std::max<size_t>(seg_.size(), 2);
	if (need > norms_cap_) {
		cudaFreeHost(h_norms_);
		cudaFree(d_norms_);
		h_norms_ = nullptr; d_norms_ = nullptr;
		LFG_CUDA(cudaMallocHost((void **)&h_norms_, sizeof(double)*need));
		LFG_CUDA(cudaMalloc((void **)&d_norms_, sizeof(double)*need));
		norms_cap_ = need;
	}
	LFG_CUDA(cudaStreamSynchronize(st_));
}

// StokesSolver::compute_LTRHS (StokesSolver.cpp:627-669): the Brownian
// force's L psi, with this factor's L (any L with L L^T = R gives the same
// statistics; the reference's CHOLMOD factor is another one)
void Solver::multiply_device(int k, const double *b, double *x)
{
	if (k <= 0) return;
	run_graph(3, k, b, x, [&]() {
		if (opt_.precision == LFG_PREC_FP64) factor_multiply(F64_, D_, k, b, x, st_);
		else factor_multiply(F32_, D_, k, b, x, st_);
	});
}

int Solver::multiply_host(int k, const double *rhs, double *x, lfg_status *st)
{
	int64_t tot = (int64_t)6*n_*k;
	if (hcap_ < tot) {
		if (hb_) cudaFree(hb_);
		if (hx_) cudaFree(hx_);
		LFG_CUDA(cudaMalloc((void **)&hb_, sizeof(double)*tot));
		LFG_CUDA(cudaMalloc((void **)&hx_, sizeof(double)*tot));
		hcap_ = tot;
	}
	LFG_CUDA(cudaMemcpyAsync(hb_, rhs, sizeof(double)*tot, cudaMemcpyHostToDevice, st_));
	multiply_device(k, hb_, hx_);
	LFG_CUDA(cudaMemcpyAsync(x, hx_, sizeof(double)*tot, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	(void)st;
	return LFG_OK;
}

int Solver::solve_host(int k, const double *rhs, double *x, lfg_status *st)
{
	int64_t tot = (int64_t)6*n_*k;
	if (hcap_ < tot) {
		if (hb_) cudaFree(hb_);
		if (hx_) cudaFree(hx_);
		LFG_CUDA(cudaMalloc((void **)&hb_, sizeof(double)*tot));
		LFG_CUDA(cudaMalloc((void **)&hx_, sizeof(double)*tot));
		hcap_ = tot;
	}
	LFG_CUDA(cudaMemcpyAsync(hb_, rhs, sizeof(double)*tot, cudaMemcpyHostToDevice, st_));
	int rc = solve_device(k, hb_, hx_, st, true);
	LFG_CUDA(cudaMemcpyAsync(x, hx_, sizeof(double)*tot, cudaMemcpyDeviceToHost, st_));
	int *dst = opt_.precision == LFG_PREC_FP64 ? F64_.status : F32_.status;
	LFG_CUDA(cudaMemcpyAsync(h_status_+1, dst, sizeof(int), cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	if (h_status_[1] == 0) return fail(st, LFG_ERR_TIMEOUT, 0, "a bounded device wait gave up");
	return rc;
}

void Solver::stats(lfg_solver_stats *o) const
{
	std::memset(o, 0, sizeof *o);
	o->n_blocks = S_.nblk;
	o->n_supernodes = S_.nsn;
	o->n_levels = S_.nlevels;
	o->max_front = S_.max_F;
	o->nnz_L = S_.nnz_L;
	o->flops_factor = S_.flops;
	o->front_bytes = S_.arena_elems*(opt_.precision == LFG_PREC_FP64 ? 8 : 4);
	o->n_factor_launches = launches_factor_;
	o->n_solve_launches = launches_solve_;
}

} // namespace lfg

// lfg_solver.h -- device resistance solver (C++ side of lfg_solver_*).
#pragma once
#include <functional>

#include "lfg_internal.h"

namespace lfg {

class Solver {
public:
	// dof: 6, or 3 for the in-plane unknowns (x, z translation, y rotation)
	// of a 2D system; right-hand sides and solutions keep 6 values per
	// particle either way
	// analysis_only: set_pattern keeps the symbolic analysis on the host and
	// allocates nothing on the device (the suspension's factor is part of a
	// joint solver's, see install)
	Solver(int n, const lfg_options &o, cudaStream_t st, int dof = 6, bool analysis_only = false);
	~Solver();
	// pattern of the lower off-diagonal blocks; re-runs the symbolic analysis
	void set_pattern(int nb, const int32_t *row, const int32_t *col, const double *pos, double lx,
	                 double ly, double lz, bool device_ptrs);
	void set_values_host(const double *dblocks, const double *odblocks);
	// a symbolic analysis made elsewhere (the concatenation of several
	// suspensions' analyses) for the lower blocks (row, col): upload, allocate
	void install(Symbolic &&S, int nb, const int32_t *row, const int32_t *col);
	const Symbolic &symbolic() const { return S_; }
	const std::vector<int32_t> &pattern_rows() const { return pat_r_; }
	const std::vector<int32_t> &pattern_cols() const { return pat_c_; }
	void set_segments(const std::vector<int> &particle_off);
	// the FP32 refinement in pieces (launch-only parts may be captured by the caller)
	void refine_begin(int k, const double *b);
	void refine_iterations(int k, const double *b, int j);
	double refine_worst(int k);
	int refine_finish(int k, double *x, int iters, double worst, lfg_status *st);
	void reserve_refine(int k) { ensure_refine_ws(k); }
	int pred_iters() const { return pred_iters_; }
	void set_pred_iters(int j) { pred_iters_ = j; }
	// re-run the symbolic analysis of the current pattern with another
	// nested-dissection leaf size (the batch autotuner's knob)
	void reanalyze(int leaf_size);
	// device arrays of the compact values (dblocks n x 15, odblocks nb x 18)
	double *d_dblocks() { return A_.dblocks; }
	double *d_odblocks() { return A_.odblocks; }
	void factorize_async();
	int check_factor(lfg_status *st);
	int solve_device(int k, const double *b, double *x, lfg_status *st, bool sync_check);
	int solve_host(int k, const double *rhs, double *x, lfg_status *st);
	// x = L b (R = L L^T, caller's order) with the current factor: device / host
	void multiply_device(int k, const double *b, double *x);
	int multiply_host(int k, const double *b, double *x, lfg_status *st);
	void stats(lfg_solver_stats *o) const;
	bool analyzed() const { return analyzed_; }
	int n() const { return n_; }
	int dof() const { return dof_; }
	int nb() const { return nb_; }
	int symbolic_runs() const { return symbolic_runs_; }
	int last_iters() const { return last_iters_; }
	double last_resid() const { return last_resid_; }
	double flops() const { return S_.flops; }
	int64_t nnz_L() const { return S_.nnz_L; }
	int launches_factor() const { return launches_factor_; }
	int launches_solve() const { return launches_solve_; }
	int64_t kernels_launched() const { return kernels_; }
	double capture_ms() const { return capture_ms_; }   // host time spent capturing + instantiating graphs
	const lfg_options &options() const { return opt_; }
	int *d_status() { return opt_.precision == LFG_PREC_FP64 ? F64_.status : F32_.status; }

private:
	struct GraphEntry {
		int kind = 0, k = 0;
		const void *b = nullptr;
		const void *x = nullptr;
		cudaGraphExec_t exec = nullptr;
		int64_t nodes = 0;
	};
	void run_graph(int kind, int k, const void *b, const void *x, const std::function<void()> &body);
	void ensure_refine_ws(int k);
	void upload(const std::vector<int32_t> &r, const std::vector<int32_t> &c);

	int n_ = 0, nb_ = 0, dof_ = 6;
	bool analysis_only_ = false;
	std::vector<int> seg_;       // scalar offsets of the segments (joint systems)
	int *d_seg_ = nullptr;
	size_t norms_cap_ = 64;
	lfg_options opt_;
	cudaStream_t st_;
	Symbolic S_;
	DevSymbolic D_;
	DevFactor<double> F64_;
	DevFactor<float> F32_;
	DevBlockMatrix A_;
	bool analyzed_ = false;
	int symbolic_runs_ = 0;
	double *h_norms_ = nullptr, *d_norms_ = nullptr;
	int *h_status_ = nullptr;
	double *ref_x_ = nullptr, *ref_r_ = nullptr, *ref_d_ = nullptr;
	int64_t ref_cap_ = 0;
	double *hb_ = nullptr, *hx_ = nullptr;
	int64_t hcap_ = 0;
	std::vector<GraphEntry> graphs_;
	std::vector<int32_t> pat_r_, pat_c_;   // the analysed pattern (for reanalyze)
	std::vector<double> pat_pos_;
	double pat_box_[3] = {0, 0, 0};
	int last_iters_ = 0;
	int pred_iters_ = 2;   // refinement iterations launched together (the last solve's count)
	double last_resid_ = 0;
	int launches_factor_ = 0, launches_solve_ = 0;
	int64_t kernels_ = 0;
	double capture_ms_ = 0;
};

} // namespace lfg

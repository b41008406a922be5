// lfg_sim.cpp -- host driver of the device-resident time step that replaces
// System::timeEvolution (LF_DEM/System.cpp:1203-1279), and the lfg_sim_* C ABI.
//
// All state lives on the device.  Per step the host only launches kernels
// (factorisation and solves are CUDA graphs) and synchronises once, after the
// corrector move, to read the clock and the "superset stale" flag.  The pair
// list is a superset of the interactions (every pair within range + skin);
// its sparsity pattern is the pattern of R_FU, so the nested-dissection
// analysis is redone only when a pair within range falls outside it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <new>

#include "lfg_physics.h"
#include "lfg_solver.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);
int ok(lfg_status *st);
int check_device(int device, lfg_status *st);

class Sim {
public:
	// fused: a member of a fused batch (its solver only analyses the pattern;
	// the batch's joint solver factors and solves)
	Sim(const lfg_params &p, const lfg_options &o, int n, const double *pos, const double *radius, double lx,
	    double ly, double lz, const double *le_disp, cudaStream_t st, bool fused = false);
	~Sim();
	void set_contacts(int ncs, const int32_t *p0, const int32_t *p1, const double *dt);
	void first_time();
	void step(int calc_stress, double time_end, double strain_end);
	void advance(double time_end, double strain_end);
	bool advance_partial(double time_end, double strain_end, int max_steps);
	void scalars(lfg_sim_scalars *o);
	void particles(double *pos, double *vel, double *ang, double *na_vel, double *na_ang);
	int num_pairs();
	int get_pairs(lfg_pair *out, int cap);
	int contact_states(int32_t *p0, int32_t *p1, double *dt, double *dr, int cap);
	int particle_stress(int comp, double *out);
	int velocity_component(int comp, double *out);
	int set_contact(int p0, int p1, int state, const double *disp_tan, const double *disp_roll = nullptr);
	void set_clock(double time, double strain, double dt, double rate, double maxv, double maxsv);
	void refresh();
	int assemble(double *dbl, int32_t *row, int32_t *col, double *odbl, int cap, int *nb_out);
	int force_component(int comp, double *out);
	void force_component_noalloc(int comp, double *d_out, int device);
	void timing(lfg_sim_timing *o) const;
	void run(int nsteps, double time_end, double strain_end);
	void set_leaf_size(int leaf) { solver_->reanalyze(leaf); symbolic_runs_++; }
	void output_snapshot(OutputSnapshot &o);
	void set_brownian_force(const double *fb);
	int64_t device_bytes() const;
	std::vector<double> step_ms;
	int64_t step_kernels = 0;
	double rebuild_ms_ = 0;   // host wall time of superset rebuilds (see lfg_sim_timing)
	int rebuilds_ = 0;
	double capture_mark_ = 0; // the solver's graph-capture time at the last clear
	void clear_timing() { step_ms.clear(); step_kernels = 0; rebuild_ms_ = 0; rebuilds_ = 0;
	                      capture_mark_ = solver_->capture_ms(); }
	int error_code = 0, error_info = 0;
	std::string error_msg;

	// stages of a step (see compute_velocities); used by step() and by the
	// lockstep driver of a fused batch
	void pc_pre_solve(double *dbl, double *odbl);
	int pc_forces_rhs(int calc_stress, int in_predictor, double **rhs, double **sol);
	void pc_post_solve(int calc_stress, int in_predictor);
	void pc_move_predictor(int calc_stress, double time_end, double strain_end, bool timed);
	void pc_move_corrector(int calc_stress, bool timed);
	void superset_check_launch();
	void rebuild_superset();
	DevSim &dev() { return S_; }
	DevClock *host_clock() { return h_clock_; }
	void pull_clock_public() { pull_clock(); }
	// the clock's copy to the host (pinned), ordered on this stream
	void queue_clock_copy()
	{
		LFG_CUDA(cudaMemcpyAsync(h_clock_, S_.clock, sizeof(DevClock), cudaMemcpyDeviceToHost, st_));
	}
	// right-hand sides solved for in a half step and where they and their
	// solutions live (as pc_forces_rhs, without launching anything)
	int rhs_count(int calc_stress, double **rhs, double **sol)
	{
		int divided = (calc_stress || prm_.control == 1) ? 1 : 0;
		*rhs = S_.rhs;
		*sol = divided ? S_.vc : S_.sol;
		return divided ? (S_.P.brownian_on ? NFC : NPFC) : 1;
	}
	Solver *solver() { return solver_; }
	const lfg_params &params() const { return prm_; }
	bool fused_ = false;      // member of a fused batch: no own factor, no own step
	cudaStream_t stream() const { return st_; }

private:
	void compute_velocities(int calc_stress, int in_predictor);
	void check_error();
	void pull_clock();
	void stage_begin(int s);
	void stage_end(int s);

	lfg_params prm_;
	lfg_options opt_;
	DevSim S_;
	Solver *solver_ = nullptr;
	cudaStream_t st_;
	bool firsttime_ = true;
	DevClock *h_clock_ = nullptr;
	int *d_err_ = nullptr, *h_err_ = nullptr;
	int *d_counts_ = nullptr;   // interaction counts (lfg_sim_scalars)
	std::vector<double> h_pos_;
	int symbolic_runs_ = 0;
	// Brownian force: draws so far, psi work vector, a force given for the
	// next predictor (set_brownian_force)
	unsigned long long brownian_draws_ = 0;
	double *psi_ = nullptr;
	bool fb_given_ = false;
	// System::avg_dt: mean dt over the loop steps of the last timeEvolution
	// (System.cpp:1234-1270); dt itself for a fixed time step (:609-611)
	double avg_dt_ = 0, avg_dt_sum_ = 0;
	int avg_dt_n_ = 0;
	bool adv_running_ = false;
	// stage timing
	struct Ev { cudaEvent_t a, b; int stage; };
	std::vector<Ev> evs_;
	size_t ev_used_ = 0;
	int cur_stage_ = -1;
	double stage_ms_[8] = {0};
	int64_t launches_mark_ = 0;
	int64_t last_launches_ = 0;
	cudaEvent_t step_a_ = nullptr, step_b_ = nullptr;
	cudaEvent_t run_a_ = nullptr, run_b_ = nullptr;   // around a whole run()
	double run_ms_ = 0;
	int run_steps_ = 0;
};

static DevParams make_dev_params(const lfg_params &p, int n, double lx, double ly, double lz, double skin)
{
	DevParams P;
	std::memset(&P, 0, sizeof P);
	P.n = n;
	P.friction = p.friction_model != 0;
	P.friction_model = p.friction_model;
	P.mu_s = P.friction ? p.mu_static : 0;
	P.mu_d = p.mu_dynamic < 0 ? P.mu_s : p.mu_dynamic;
	P.kn = p.kn; P.kt = p.kt;
	P.rolling = p.mu_rolling > 0;
	P.mu_r = p.mu_rolling; P.kr = p.kr;
	P.brownian_on = p.brownian > 0;
	P.brownian = p.brownian;
	P.critical_load = p.critical_load; P.ft_max = p.ft_max;
	P.repulsiveforce = p.repulsion_on && p.repulsive_length > 0;
	P.repulsion = p.repulsion; P.rep_len = p.repulsive_length; P.rep_max_len = p.repulsive_max_length;
	P.lub_on = p.lubrication_model != 0;
	P.tangential = p.lubrication_model == 2;
	P.lub_reduce = p.lub_reduce_parameter; P.lub_max_gap = p.lub_max_gap;
	P.interaction_range = p.interaction_range;
	P.sd_coeff = p.sd_coeff;
	// ContactDashpot::setDashpotResistanceCoeffs (ContactDashpot.cpp:65-105),
	// evaluated on the host as in the reference
	double rn = p.contact_relaxation_time, rt = p.contact_relaxation_time_tan;
	if (rn > 0) P.dp_normal_coeff = 4*p.kn*rn;
	else if (P.lub_on) P.dp_normal_coeff = 1/p.lub_reduce_parameter;
	else throw Error{LFG_ERR_BAD_ARG, 0, "normal relaxation time <= 0 without lubrication"};
	if (!P.friction && !P.tangential) P.dp_tan_coeff = 0;
	else if (rt > 0) {
		if (P.lub_on) throw Error{LFG_ERR_BAD_ARG, 0, "with lubrication the tangential relaxation time cannot be positive"};
		P.dp_tan_coeff = 6*p.kt*rt;
	} else {
		if (!P.lub_on) throw Error{LFG_ERR_BAD_ARG, 0, "tangential relaxation time <= 0 without lubrication"};
		P.dp_tan_coeff = p.lub_reduce_parameter < 1 ? std::log(1/p.lub_reduce_parameter) : 0;
	}
	P.lx = lx; P.ly = ly; P.lz = lz;
	P.lx_half = lx/2; P.ly_half = ly/2; P.lz_half = lz/2;
	P.twodim = ly == 0;
	for (int k = 0; k < 6; k++) P.Ehat[k] = p.Ehat[k];
	for (int k = 0; k < 3; k++) P.Ohat[k] = p.Ohat[k];
	P.disp_max = p.disp_max; P.dt_max = p.dt_max; P.dt_min = p.dt_min;
	P.fixed_dt = p.fixed_dt;
	P.control = p.control;
	P.integration_method = p.integration_method;
	P.target_stress = p.target_stress;
	P.init_strain_limit = p.init_strain_shear_rate_limit;
	P.init_rate_limit = p.init_shear_rate_limit;
	P.system_volume = P.twodim ? lx*lz : lx*ly*lz;
	P.skin = skin;
	return P;
}

// zero-filled device allocation, ordered on the simulation's stream (no
// device-wide synchronisation, so other suspensions keep running)
template <typename V> static void dalloc(V *&p, size_t count, cudaStream_t st)
{
	LFG_CUDA(cudaMalloc((void **)&p, sizeof(V)*std::max<size_t>(count, 1)));
	LFG_CUDA(cudaMemsetAsync(p, 0, sizeof(V)*std::max<size_t>(count, 1), st));
}

Sim::Sim(const lfg_params &p, const lfg_options &o, int n, const double *pos, const double *radius, double lx,
         double ly, double lz, const double *le_disp, cudaStream_t st, bool fused)
    : fused_(fused), prm_(p), opt_(o), st_(st)
{
	avg_dt_ = p.fixed_dt ? p.dt : 0;
	if (p.friction_model == 4 || p.friction_model < 0 || p.friction_model > 6)
		throw Error{LFG_ERR_BAD_ARG, p.friction_model, "unknown friction model"};
	if (p.lubrication_model < 0 || p.lubrication_model > 2)
		throw Error{LFG_ERR_BAD_ARG, p.lubrication_model, "unknown lubrication model"};
	if (p.mu_rolling > 0 && p.friction_model == 0)
		throw Error{LFG_ERR_BAD_ARG, 0, "rolling friction without sliding friction (System.cpp:386-391)"};
	if (p.lubrication_model == 2 && p.lub_max_gap >= 1)
		throw Error{LFG_ERR_BAD_ARG, 0, "lub_max_gap must be smaller than 1 (System.cpp:340-346)"};
	S_.n = n;
	S_.P = make_dev_params(p, n, lx, ly, lz, o.skin);
	dalloc(S_.clock, 1, st_);
	dalloc(S_.pos, 3*n, st_); dalloc(S_.radius, n, st_);
	dalloc(S_.vel, 3*n, st_); dalloc(S_.ang, 3*n, st_); dalloc(S_.vel_pred, 3*n, st_); dalloc(S_.ang_pred, 3*n, st_);
	dalloc(S_.u_inf, 3*n, st_); dalloc(S_.na, 6*n, st_);
	dalloc(S_.na_disp, 3*n, st_); dalloc(S_.angle, n, st_);
	if (p.brownian > 0) dalloc(psi_, 6*n, st_);
	dalloc(S_.vc, (size_t)NFC*6*n, st_); dalloc(S_.fc, (size_t)NFC*6*n, st_);
	dalloc(S_.rhs, (size_t)NFC*6*n, st_); dalloc(S_.sol, (size_t)NFC*6*n, st_);
	dalloc(S_.sc, (size_t)NSC*6*n, st_); dalloc(S_.sc_tot, (size_t)NSC*6+12*(size_t)n, st_);
	dalloc(S_.row_ptr, n+1, st_); dalloc(S_.col_ptr, n+1, st_);
	dalloc(d_err_, 1, st_);
	dalloc(d_counts_, 4, st_);
	LFG_CUDA(cudaMallocHost((void **)&h_clock_, sizeof(DevClock)));
	LFG_CUDA(cudaMallocHost((void **)&h_err_, sizeof(int)));
	LFG_CUDA(cudaMemcpyAsync(S_.pos, pos, sizeof(double)*3*n, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	LFG_CUDA(cudaMemcpyAsync(S_.radius, radius, sizeof(double)*n, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	int big = 0x7fffffff;
	LFG_CUDA(cudaMemcpyAsync(d_err_, &big, sizeof(int), cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	// clock: rate control starts at the imposed rate, stress control at 0
	// (SimulationInit.cpp:276); dt = p.dt (System.cpp:607)
	DevClock K;
	std::memset(&K, 0, sizeof K);
	K.dt = p.dt;
	if (le_disp) { K.shear_disp[0] = le_disp[0]; K.shear_disp[1] = le_disp[1]; }
	LFG_CUDA(cudaMemcpyAsync(S_.clock, &K, sizeof K, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	phys_set_shear_rate(S_, p.control == 0 ? p.shear_rate : 0.0, false, st_);
	// cells sized for the largest superset range
	double amax = 0;
	for (int i = 0; i < n; i++) amax = std::max(amax, radius[i]);
	double rc = (p.interaction_range < 0 ? 2+p.lub_max_gap+o.skin : p.interaction_range+o.skin)*amax;
	S_.ncx = std::max(1, (int)(lx/rc));
	S_.ncy = S_.P.twodim ? 1 : std::max(1, (int)(ly/rc));
	S_.ncz = std::max(1, (int)(lz/rc));
	S_.brute = (S_.ncx < 3 || S_.ncz < 3 || (!S_.P.twodim && S_.ncy < 3)) ? 1 : 0;
	S_.csx = lx/S_.ncx; S_.csy = S_.P.twodim ? 1.0 : ly/S_.ncy; S_.csz = lz/S_.ncz;
	int ncell = S_.ncx*S_.ncy*S_.ncz;
	dalloc(S_.cell_of, n, st_); dalloc(S_.cell_count, ncell, st_); dalloc(S_.cell_start, ncell+1, st_); dalloc(S_.cell_list, n, st_);
	dalloc(S_.cell_rec, 4*(size_t)n, st_);
	dalloc(S_.cell_rec32, 4*(size_t)n, st_);
	dalloc(S_.cand_count, std::max(n, ncell), st_); dalloc(S_.cand_ptr, n+1, st_);
	// a monolayer's in-plane unknowns (x, z, rotation about y) decouple from
	// the others: solve them alone unless asked for LF_DEM's 6x6 blocks
	int dof = (S_.P.twodim && !S_.P.brownian_on && o.dof_2d != 6) ? 3 : 6;
	solver_ = new Solver(n, opt_, st_, dof, fused);
	h_pos_.assign(pos, pos+3*n);
	rebuild_superset();
	// System::setupGenericConfiguration -> checkNewInteraction (System.cpp:517-519)
	phys_pairs_update(S_, 2, 0, true, st_);
}

Sim::~Sim()
{
	delete solver_;
	void *p[] = {S_.clock, S_.pos, S_.radius, S_.vel, S_.ang, S_.vel_pred, S_.ang_pred, S_.u_inf, S_.na, S_.na_disp,
	             S_.angle, psi_, S_.vc,
	             S_.fc, S_.rhs, S_.sol, S_.sc, S_.sc_tot, S_.pairs, S_.pconst, S_.row_ptr, S_.col_ptr, S_.col_idx,
	             S_.blk_scratch, S_.pair_scratch, S_.cell_of, S_.cell_start, S_.cell_count, S_.cell_list, S_.cell_rec, S_.cell_rec32,
	             S_.cand_count, S_.cand_ptr, S_.cand, d_err_, d_counts_};
	for (void *q : p) if (q) cudaFree(q);
	if (h_clock_) cudaFreeHost(h_clock_);
	if (h_err_) cudaFreeHost(h_err_);
	for (auto &e : evs_) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
	if (step_a_) cudaEventDestroy(step_a_);
	if (step_b_) cudaEventDestroy(step_b_);
	if (run_a_) cudaEventDestroy(run_a_);
	if (run_b_) cudaEventDestroy(run_b_);
}

// Build the pair superset at the current positions, carry the pair state of
// the previous superset over, and redo the symbolic analysis.
void Sim::rebuild_superset()
{
	phys_cells(S_, 0, st_);
	int total = 0;
	phys_candidates(S_, st_, &total);
	DPair *old = S_.pairs;
	int *old_row = nullptr;
	int old_n = old ? S_.n : 0;
	if (old) {
		LFG_CUDA(cudaMalloc((void **)&old_row, sizeof(int)*(S_.n+1)));
		LFG_CUDA(cudaMemcpyAsync(old_row, S_.row_ptr, sizeof(int)*(S_.n+1), cudaMemcpyDeviceToDevice, st_));
	}
	S_.npairs = total;
	if (total > S_.cap || !old) {
		S_.cap = std::max(total+total/4+256, S_.cap);
		if (S_.pconst) cudaFree(S_.pconst);
		if (S_.blk_scratch) cudaFree(S_.blk_scratch);
		if (S_.pair_scratch) cudaFree(S_.pair_scratch);
		if (S_.col_idx) cudaFree(S_.col_idx);
		S_.pconst = nullptr; S_.blk_scratch = S_.pair_scratch = nullptr; S_.col_idx = nullptr;
		dalloc(S_.pconst, S_.cap, st_);
		dalloc(S_.blk_scratch, (size_t)30*S_.cap, st_);
		dalloc(S_.pair_scratch, (size_t)12*NSC*S_.cap, st_);
		dalloc(S_.col_idx, S_.cap, st_);
	}
	DPair *fresh = nullptr;
	dalloc(fresh, S_.cap, st_);
	S_.pairs = fresh;
	phys_merge_pairs(S_, old, old_row, old_n, st_);
	LFG_CUDA(cudaMemcpyAsync(S_.row_ptr, S_.cand_ptr, sizeof(int)*(S_.n+1), cudaMemcpyDeviceToDevice, st_));
	phys_pair_constants(S_, st_);
	// host copies of the pattern: transpose lists and the symbolic analysis
	std::vector<int> rp(S_.n+1), cand(total);
	LFG_CUDA(cudaMemcpyAsync(rp.data(), S_.cand_ptr, sizeof(int)*(S_.n+1), cudaMemcpyDeviceToHost, st_));
	if (total) LFG_CUDA(cudaMemcpyAsync(cand.data(), S_.cand, sizeof(int)*total, cudaMemcpyDeviceToHost, st_));
	std::vector<double> pos(3*S_.n);
	LFG_CUDA(cudaMemcpyAsync(pos.data(), S_.pos, sizeof(double)*3*S_.n, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	if (old) cudaFree(old);
	if (old_row) cudaFree(old_row);
	std::vector<int32_t> od_row(total), od_col(total);
	std::vector<int> cp(S_.n+1, 0), ci(total);
	for (int i = 0; i < S_.n; i++)
		for (int t = rp[i]; t < rp[i+1]; t++) { od_col[t] = i; od_row[t] = cand[t]; cp[cand[t]+1]++; }
	for (int i = 0; i < S_.n; i++) cp[i+1] += cp[i];
	{
		std::vector<int> f(cp.begin(), cp.end()-1);
		for (int t = 0; t < total; t++) ci[f[od_row[t]]++] = t;   // ascending t = ascending p0 per p1
	}
	LFG_CUDA(cudaMemcpyAsync(S_.col_ptr, cp.data(), sizeof(int)*(S_.n+1), cudaMemcpyHostToDevice, st_));
	if (total) LFG_CUDA(cudaMemcpyAsync(S_.col_idx, ci.data(), sizeof(int)*total, cudaMemcpyHostToDevice, st_));
	solver_->set_pattern(total, od_row.data(), od_col.data(), pos.data(), S_.P.lx, S_.P.ly, S_.P.lz, false);
	symbolic_runs_++;
}

void Sim::set_contacts(int ncs, const int32_t *p0, const int32_t *p1, const double *dt)
{
	for (int c = 0; c < ncs; c++)
		if (set_contact(p0[c], p1[c], -1, dt+3*c) != 0)
			throw Error{LFG_ERR_BAD_ARG, c, "contact state for a pair that is not within interaction range"};
}

// System::timeEvolution first-time block (System.cpp:1216-1226); the
// interactions of the configuration are created here as well
// (System::setupGenericConfiguration, System.cpp:517-520).
void Sim::first_time()
{
	if (!firsttime_) return;
	phys_pairs_update(S_, 1, 1, true, st_);
	firsttime_ = false;
}

void Sim::stage_begin(int s)
{
	if (ev_used_ == evs_.size()) {
		Ev e;
		LFG_CUDA(cudaEventCreate(&e.a));
		LFG_CUDA(cudaEventCreate(&e.b));
		evs_.push_back(e);
	}
	evs_[ev_used_].stage = s;
	LFG_CUDA(cudaEventRecord(evs_[ev_used_].a, st_));
	cur_stage_ = s;
}

void Sim::stage_end(int)
{
	LFG_CUDA(cudaEventRecord(evs_[ev_used_].b, st_));
	ev_used_++;
	cur_stage_ = -1;
}

// Stages of a step, shared by step() (with this suspension's own solver) and
// the lockstep driver of a fused batch (one joint solver for all its
// suspensions, FusedGroup below).

// System::computeVelocities (System.cpp:2273-2319) up to the factorisation:
// the shear rate set to 1 under stress control, u_inf, the R_FU blocks
// (into dbl / odbl)
void Sim::pc_pre_solve(double *dbl, double *odbl)
{
	if (prm_.control == 1) phys_set_shear_rate(S_, 1.0, false, st_);
	phys_u_inf(S_, st_);
	phys_blocks(S_, dbl, odbl, st_);
}

// the force components and the right-hand sides; returns how many of them
// are solved for and where they and the solutions live
int Sim::pc_forces_rhs(int calc_stress, int in_predictor, double **rhs, double **sol)
{
	int divided = (calc_stress || prm_.control == 1) ? 1 : 0;
	phys_force_components(S_, st_);
	if (S_.P.brownian_on && in_predictor) {
		// System::setBrownianForceToParticle (System.cpp:1665-1710): F_B =
		// L (sqrt(2 kT/dt) psi) with the factor of this configuration, drawn
		// in the predictor only (the corrector keeps it)
		if (fused_) throw Error{LFG_ERR_BAD_ARG, 0, "Brownian forces in a fused batch"};
		double *fb = S_.fc+(size_t)FC_BROWNIAN*6*S_.n;
		if (fb_given_) {
			fb_given_ = false;
		} else {
			phys_brownian_psi(S_, prm_.seed, brownian_draws_++, std::sqrt(2*prm_.brownian/prm_.dt), psi_, st_);
			solver_->multiply_device(1, psi_, fb);
		}
	}
	phys_rhs(S_, divided, st_);
	int nrhs = S_.P.brownian_on ? NFC : NPFC;   // the Brownian component is the last
	*rhs = S_.rhs;
	*sol = divided ? S_.vc : S_.sol;
	return divided ? nrhs : 1;
}

// after the solve: stress control's stresslets and shear rate, velocities
void Sim::pc_post_solve(int calc_stress, int in_predictor)
{
	int divided = (calc_stress || prm_.control == 1) ? 1 : 0;
	if (divided && prm_.control == 1) {
		phys_stresslets(S_, in_predictor, st_);
		phys_shear_rate_from_stress(S_, st_);
	}
	phys_velocities(S_, divided, in_predictor, st_);
}

// the predictor's move (System::timeStepMovePredictor, System.cpp:1124-1162)
// and the interaction update at the moved positions
void Sim::pc_move_predictor(int calc_stress, double time_end, double strain_end, bool timed)
{
	if (calc_stress) { if (timed) stage_begin(4); phys_stresslets(S_, 1, st_); if (timed) stage_end(4); }
	if (timed) stage_begin(5);
	// no adaptive time step with Brownian forces (System.cpp:1129, 1243)
	if (!prm_.fixed_dt && !S_.P.brownian_on) phys_adapt_dt(S_, time_end, strain_end, st_);
	phys_boxing(S_, st_);
	phys_move(S_, 1, st_);
	if (timed) { stage_end(5); stage_begin(0); }
	phys_pairs_update(S_, 0, 1, false, st_);
	if (timed) stage_end(0);
	phys_save_pred(S_, st_);
}

// the corrector's move (System::timeStepMoveCorrector, System.cpp:1164-1187)
void Sim::pc_move_corrector(int calc_stress, bool timed)
{
	if (calc_stress) { if (timed) stage_begin(4); phys_stresslets(S_, 0, st_); if (timed) stage_end(4); }
	if (timed) stage_begin(5);
	phys_move(S_, 2, st_);
	if (timed) stage_end(5);
}

// checkNewInteraction: does the superset still hold every pair within range?
// (the flag is read on the host)
void Sim::superset_check_launch()
{
	LFG_CUDA(cudaMemsetAsync(&S_.clock->stale, 0, sizeof(int), st_));
	phys_cells(S_, 0, st_);
	phys_check_superset(S_, st_);
}

void Sim::compute_velocities(int calc_stress, int in_predictor)
{
	// System::computeVelocities (System.cpp:2273-2319)
	stage_begin(1);
	pc_pre_solve(solver_->d_dblocks(), solver_->d_odblocks());
	stage_end(1);
	stage_begin(2);
	solver_->factorize_async();
	stage_end(2);
	stage_begin(4);
	double *rhs = nullptr, *sol = nullptr;
	int k = pc_forces_rhs(calc_stress, in_predictor, &rhs, &sol);
	stage_end(4);
	stage_begin(3);
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	int rc = solver_->solve_device(k, rhs, sol, &st, false);
	// factor and solve status (a non-positive pivot, or a bounded wait that gave up)
	phys_sticky_status(solver_->d_status(), d_err_, st_);
	stage_end(3);
	if (rc == LFG_ERR_NOT_CONVERGED) { error_code = rc; error_msg = st.msg; }
	stage_begin(4);
	pc_post_solve(calc_stress, in_predictor);
	stage_end(4);
}

void Sim::pull_clock()
{
	LFG_CUDA(cudaMemcpyAsync(h_clock_, S_.clock, sizeof(DevClock), cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
}

void Sim::step(int calc_stress, double time_end, double strain_end)
{
	if (fused_) throw Error{LFG_ERR_BAD_ARG, 0, "a suspension of a fused batch steps with its batch"};
	first_time();
	ev_used_ = 0;
	int64_t l0 = S_.launches, k0 = solver_->kernels_launched();
	if (!step_a_) {
		LFG_CUDA(cudaEventCreate(&step_a_));
		LFG_CUDA(cudaEventCreate(&step_b_));
	}
	LFG_CUDA(cudaEventRecord(step_a_, st_));
	if (!prm_.fixed_dt && !S_.P.brownian_on) phys_adapt_dt(S_, time_end, strain_end, st_);
	if (prm_.integration_method == 0) {
		// System::timeEvolutionEulersMethod + timeStepMove (System.cpp:843-882, 1083-1122)
		compute_velocities(calc_stress, 1);
		if (calc_stress) { stage_begin(4); phys_stresslets(S_, 1, st_); stage_end(4); }
		stage_begin(5);
		if (!prm_.fixed_dt) phys_adapt_dt(S_, time_end, strain_end, st_);
		phys_boxing(S_, st_);
		phys_move(S_, 0, st_);
		stage_end(5);
	} else {
		// predictor (System.cpp:888-930, 1124-1162)
		compute_velocities(calc_stress, 1);
		pc_move_predictor(calc_stress, time_end, strain_end, true);
		// corrector (System.cpp:931-983, 1164-1187)
		compute_velocities(calc_stress, 0);
		pc_move_corrector(calc_stress, true);
	}
	// checkNewInteraction: the superset must hold every pair within range
	stage_begin(0);
	superset_check_launch();
	stage_end(0);
	pull_clock();
	if (h_clock_->stale) {
		auto t0 = std::chrono::steady_clock::now();
		rebuild_superset();
		LFG_CUDA(cudaStreamSynchronize(st_));
		rebuild_ms_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now()-t0).count();
		rebuilds_++;
	}
	stage_begin(0);
	phys_pairs_update(S_, 1, 0, false, st_);
	stage_end(0);
	LFG_CUDA(cudaMemcpyAsync(h_err_, d_err_, sizeof(int), cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaEventRecord(step_b_, st_));
	pull_clock();
	last_launches_ = S_.launches-l0+(solver_->kernels_launched()-k0);
	{
		float ms = 0;
		cudaEventElapsedTime(&ms, step_a_, step_b_);
		step_ms.push_back(ms);
		step_kernels += last_launches_;
	}
	for (int k = 0; k < 8; k++) stage_ms_[k] = 0;
	for (size_t e = 0; e < ev_used_; e++) {
		float ms = 0;
		cudaEventElapsedTime(&ms, evs_[e].a, evs_[e].b);
		stage_ms_[evs_[e].stage] += ms;
	}
	check_error();
}

void Sim::check_error()
{
	if (*h_err_ == 0) {
		error_code = LFG_ERR_TIMEOUT;
		error_info = 0;
		error_msg = "a bounded device wait in the resistance factorisation or solve gave up";
	} else if (*h_err_ != 0x7fffffff) {
		error_code = LFG_ERR_NOT_SPD;
		error_info = *h_err_;
		error_msg = "non-positive pivot in the resistance factorisation";
	}
}

void Sim::advance(double time_end, double strain_end)
{
	while (!advance_partial(time_end, strain_end, 1 << 30))
		if (error_code) return;
}

// System::timeEvolution loop and final stress step (System.cpp:1227-1279),
// resumable: at most max_steps loop steps; returns true once the end was
// reached and the final stress-computing step has run
bool Sim::advance_partial(double time_end, double strain_end, int max_steps)
{
	first_time();
	pull_clock();
	double adj = prm_.fixed_dt ? prm_.dt : 0;
	auto keep = [&](double te, double se) {
		if (h_clock_->strain > se-1e-8 && se >= 0) return false;
		if (h_clock_->time > te-1e-8 && te >= 0) return false;
		return true;
	};
	if (!adv_running_) {
		adv_running_ = true;
		avg_dt_sum_ = 0;
		avg_dt_n_ = 0;
	}
	for (int k = 0; k < max_steps && keep(time_end-adj, strain_end-adj); k++) {
		step(0, time_end, strain_end);
		if (error_code) { adv_running_ = false; return false; }
		avg_dt_sum_ += h_clock_->dt;
		avg_dt_n_++;
	}
	if (keep(time_end-adj, strain_end-adj)) return false;
	avg_dt_ = avg_dt_n_ > 0 ? avg_dt_sum_/avg_dt_n_ : h_clock_->dt;
	adv_running_ = false;
	step(1, time_end, strain_end);
	return error_code == 0;
}

void Sim::set_brownian_force(const double *fb)
{
	if (!S_.P.brownian_on) throw Error{LFG_ERR_BAD_ARG, 0, "the simulation has no Brownian force"};
	LFG_CUDA(cudaMemcpyAsync(S_.fc+(size_t)FC_BROWNIAN*6*S_.n, fb, sizeof(double)*6*S_.n, cudaMemcpyHostToDevice,
	                         st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	fb_given_ = true;
}

// The state the output writers read (Simulation::outputData,
// outputParFileTxt, outputIntFileTxt: Simulation.cpp:641-1006).
void Sim::output_snapshot(OutputSnapshot &o)
{
	lfg_sim_scalars sc;
	scalars(&sc);   // pulls the clock
	const DevClock &K = *h_clock_;
	const DevParams &P = S_.P;
	const int n = S_.n;
	o.n = n;
	o.twodim = P.twodim;
	o.lubrication = P.lub_on;
	o.repulsion = P.repulsiveforce;
	o.control = P.control;
	o.lx = P.lx; o.ly = P.ly; o.lz = P.lz;
	o.time = K.time; o.strain = K.strain; o.shear_rate = K.shear_rate; o.avg_dt = avg_dt_;
	o.max_velocity = K.max_velocity;
	o.shear_disp[0] = K.shear_disp[0]; o.shear_disp[1] = K.shear_disp[1];
	for (int k = 0; k < 3; k++) { o.shear_strain[k] = K.shear_strain[k]; o.vel_diff[k] = K.vel_diff[k]; }
	for (int k = 0; k < 6; k++) o.Einf[k] = K.Einf[k];
	o.kn = prm_.kn; o.kt = prm_.kt; o.kr = prm_.kr;
	o.interaction_range = prm_.interaction_range == -1 ? 2+prm_.lub_max_gap : prm_.interaction_range;
	// System::total_stress_groups (Stress.cpp:70-75, 342-358): the groups of
	// the declared components; "hydro" always (E_inf term), "dashpot" with the
	// velocity components (lubrication)
	std::vector<double> tot(NSC*6);
	LFG_CUDA(cudaMemcpyAsync(tot.data(), S_.sc_tot, sizeof(double)*6*NSC, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	bool has[NSC] = {(bool)P.lub_on, (bool)P.lub_on, (bool)P.lub_on, (bool)P.lub_on,
	                 P.lub_on && P.repulsiveforce, P.control == 0, P.control == 1, P.control == 1,
	                 (bool)P.repulsiveforce, P.lub_on && P.brownian_on, (bool)P.brownian_on};
	// groups: 0 contact, 1 dashpot, 2 hydro, 3 repulsion, 4 brownian
	const int group[NSC] = {2, 0, 1, 2, 3, 0, 0, 0, 3, 4, 4};
	double g[5][6] = {{0}};
	for (int c = 0; c < NSC; c++)
		if (has[c]) for (int e = 0; e < 6; e++) g[group[c]][e] += tot[6*c+e];
	for (int a = 0; a < 5; a++) for (int e = 0; e < 6; e++) g[a][e] /= P.system_volume;
	for (int e = 0; e < 6; e++) g[2][e] += 2*K.Einf[e]/(6*M_PI);
	// key order of System::total_stress_groups
	const char *names[5] = {"brownian", "contact", "dashpot", "hydro", "repulsion"};
	const int idx[5] = {4, 0, 1, 2, 3};
	const bool present[5] = {(bool)P.brownian_on, true, (bool)P.lub_on, true, (bool)P.repulsiveforce};
	if (o.want_particle_stress) {
		o.slot_declared.assign(has, has+NSC);
		o.particle_stress.resize((size_t)NSC*6*n);
		LFG_CUDA(cudaMemcpyAsync(o.particle_stress.data(), S_.sc, sizeof(double)*NSC*6*(size_t)n,
		                         cudaMemcpyDeviceToHost, st_));
	}
	o.groups.clear();
	o.group_stress.clear();
	for (int a = 0; a < 5; a++) {
		if (!present[a]) continue;
		o.groups.push_back(names[a]);
		std::array<double, 6> v;
		for (int e = 0; e < 6; e++) v[e] = g[idx[a]][e];
		o.group_stress.push_back(v);
	}
	// System::calcStress: total = sum of the groups in key order
	for (int e = 0; e < 6; e++) o.total_stress[e] = 0;
	for (const auto &v : o.group_stress)
		for (int e = 0; e < 6; e++) o.total_stress[e] += v[e];
	auto get = [&](std::vector<double> &h, const double *d, size_t cnt) {
		h.resize(cnt);
		if (cnt) LFG_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(double)*cnt, cudaMemcpyDeviceToHost, st_));
	};
	get(o.radius, S_.radius, n);
	get(o.pos, S_.pos, 3*(size_t)n);
	get(o.vel, S_.vel, 3*(size_t)n);
	get(o.ang, S_.ang, 3*(size_t)n);
	get(o.na, S_.na, 6*(size_t)n);
	get(o.na_disp, S_.na_disp, 3*(size_t)n);
	get(o.angle, S_.angle, n);
	o.out_w = OUT_W;
	std::vector<double> all;
	if (S_.npairs) {
		static_assert(OUT_W <= 12*NSC, "pair scratch too small for the output records");
		phys_pair_output(S_, S_.pair_scratch, st_);   // scratch holds 12*max(NFC, NSC) >= OUT_W doubles per pair
		get(all, S_.pair_scratch, (size_t)OUT_W*S_.npairs);
	}
	LFG_CUDA(cudaStreamSynchronize(st_));
	o.pairs.clear();
	for (int t = 0; t < S_.npairs; t++) {
		const double *r = all.data()+(size_t)OUT_W*t;
		if (!((int)r[0] & PF_INTER)) continue;
		o.pairs.insert(o.pairs.end(), r, r+OUT_W);
	}
}

void Sim::scalars(lfg_sim_scalars *o)
{
	// the clock, the per-component stress totals and the interaction counts,
	// read back with one synchronisation
	std::vector<double> tot(NSC*6);
	int cnt[4];
	LFG_CUDA(cudaMemcpyAsync(h_clock_, S_.clock, sizeof(DevClock), cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaMemcpyAsync(tot.data(), S_.sc_tot, sizeof(double)*6*NSC, cudaMemcpyDeviceToHost, st_));
	phys_pair_counts(S_, d_counts_, st_);
	LFG_CUDA(cudaMemcpyAsync(cnt, d_counts_, sizeof cnt, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	std::memset(o, 0, sizeof *o);
	const DevClock &K = *h_clock_;
	o->time = K.time; o->strain = K.strain; o->shear_rate = K.shear_rate; o->dt = K.dt;
	o->shear_disp[0] = K.shear_disp[0]; o->shear_disp[1] = K.shear_disp[1];
	o->max_velocity = K.max_velocity; o->max_sliding_velocity = K.max_sliding_velocity;
	o->rate_prop_shearstress = K.rate_prop; o->rate_indep_shearstress = K.rate_indep;
	o->total_num_timesteps = K.steps;
	// System::calcStress (Stress.cpp:342-384) from the per-component totals
	const DevParams &P = S_.P;
	bool has[NSC] = {(bool)P.lub_on, (bool)P.lub_on, (bool)P.lub_on, (bool)P.lub_on,
	                 P.lub_on && P.repulsiveforce, P.control == 0, P.control == 1, P.control == 1,
	                 (bool)P.repulsiveforce, P.lub_on && P.brownian_on, (bool)P.brownian_on};
	// groups: 0 contact, 1 dashpot, 2 hydro, 3 repulsion, 4 brownian
	const int group[NSC] = {2, 0, 1, 2, 3, 0, 0, 0, 3, 4, 4};
	double g[5][6] = {{0}};
	for (int c = 0; c < NSC; c++)
		if (has[c]) for (int e = 0; e < 6; e++) g[group[c]][e] += tot[6*c+e];
	double inv = 1.0/P.system_volume;
	for (int a = 0; a < 5; a++) for (int e = 0; e < 6; e++) g[a][e] *= inv;
	for (int e = 0; e < 6; e++) g[2][e] += 2*K.Einf[e]/(6*M_PI);
	// in the groups' key order (brownian, contact, dashpot, hydro, repulsion)
	for (int e = 0; e < 6; e++) o->total_stress[e] = g[4][e]+g[0][e]+g[1][e]+g[2][e]+g[3][e];
	const double *E = K.Einf;
	double EE = E[0]*E[0]+2*E[1]*E[1]+2*E[2]*E[2]+2*E[3]*E[3]+E[4]*E[4]+E[5]*E[5];
	if (K.shear_rate != 0 && EE != 0) {
		const double *s = o->total_stress;
		double sE = s[0]*E[0]+2*s[1]*E[1]+2*s[2]*E[2]+2*s[3]*E[3]+s[4]*E[4]+s[5]*E[5];
		o->viscosity = 0.5*sE/EE;
		o->N1 = (s[0]-s[5])/K.shear_rate;
		o->N2 = (s[5]-s[4])/K.shear_rate;
	}
	// interaction counts, counted on the device (not the pair records copied here)
	o->n_pairs = cnt[0];
	o->n_contacts = cnt[1];
	o->n_lub = cnt[2];
	o->n_resistance_pairs = cnt[3];
	o->n_superset_pairs = S_.npairs;
	o->n_symbolic_runs = symbolic_runs_;
	o->last_refine_iters = solver_->last_iters();
	o->last_refine_residual = solver_->last_resid();
}

void Sim::particles(double *pos, double *vel, double *ang, double *na_vel, double *na_ang)
{
	int n = S_.n;
	// the copies share one synchronisation
	if (pos) LFG_CUDA(cudaMemcpyAsync(pos, S_.pos, sizeof(double)*3*n, cudaMemcpyDeviceToHost, st_));
	if (vel) LFG_CUDA(cudaMemcpyAsync(vel, S_.vel, sizeof(double)*3*n, cudaMemcpyDeviceToHost, st_));
	if (ang) LFG_CUDA(cudaMemcpyAsync(ang, S_.ang, sizeof(double)*3*n, cudaMemcpyDeviceToHost, st_));
	std::vector<double> na;
	if (na_vel || na_ang) {
		na.resize(6*(size_t)n);
		LFG_CUDA(cudaMemcpyAsync(na.data(), S_.na, sizeof(double)*6*n, cudaMemcpyDeviceToHost, st_));
	}
	LFG_CUDA(cudaStreamSynchronize(st_));
	if (na_vel || na_ang) {
		for (int i = 0; i < n; i++)
			for (int e = 0; e < 3; e++) {
				if (na_vel) na_vel[3*i+e] = na[6*i+e];
				if (na_ang) na_ang[3*i+e] = na[6*i+3+e];
			}
	}
}

int Sim::num_pairs()
{
	int cnt[4];
	phys_pair_counts(S_, d_counts_, st_);
	LFG_CUDA(cudaMemcpyAsync(cnt, d_counts_, sizeof cnt, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	return cnt[0];
}

// active contacts with their springs (System::getContacts, System.cpp:306-320),
// sorted by (p0, p1)
int Sim::contact_states(int32_t *p0, int32_t *p1, double *dt, double *dr, int cap)
{
	std::vector<DPair> pairs(S_.npairs);
	if (S_.npairs) LFG_CUDA(cudaMemcpyAsync(pairs.data(), S_.pairs, sizeof(DPair)*S_.npairs, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	int c = 0;
	for (const DPair &q : pairs) {
		if (!(q.flags & PF_INTER) || !(q.flags & PF_CONTACT)) continue;
		if (c < cap) {
			if (p0) p0[c] = q.p0;
			if (p1) p1[c] = q.p1;
			for (int k = 0; k < 3; k++) {
				if (dt) dt[3*c+k] = q.disp_tan[k];
				if (dr) dr[3*c+k] = q.disp_roll[k];
			}
		}
		c++;
	}
	return c;
}

int Sim::get_pairs(lfg_pair *out, int cap)
{
	std::vector<DPair> pairs(S_.npairs);
	if (S_.npairs) LFG_CUDA(cudaMemcpyAsync(pairs.data(), S_.pairs, sizeof(DPair)*S_.npairs, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	int c = 0;
	for (const DPair &q : pairs) {
		if (!(q.flags & PF_INTER)) continue;
		if (c < cap) {
			lfg_pair &o = out[c];
			std::memset(&o, 0, sizeof o);
			o.p0 = q.p0; o.p1 = q.p1; o.z_offset = q.zoff;
			o.contact_active = (q.flags & PF_CONTACT) ? 1 : 0;
			o.state = q.state;
			o.lub_active = (q.flags & PF_LUB) ? 1 : 0;
			o.r = q.r; o.reduced_gap = q.gap;
			for (int k = 0; k < 3; k++) {
				o.nvec[k] = q.nvec[k]; o.rvec[k] = q.rvec[k]; o.disp_tan[k] = q.disp_tan[k];
				o.f_spring_total[k] = q.fs_total[k]; o.rep_force[k] = q.rep_force[k];
			}
			o.lub_coeff = q.lub_coeff; o.log_lub_coeff = q.log_lub_coeff;
		}
		c++;
	}
	return c;
}

int Sim::particle_stress(int comp, double *out)
{
	static const int map[10] = {SC_GU_CONTACT, SC_GU_DASHPOT, SC_GU_HYDRO, SC_GU_REPULSION, SC_ME,
	                            SC_XF_CONTACT, SC_XF_RATEINDEP, SC_XF_REPULSION, SC_GU_BROWNIAN, SC_BROWNIAN_PRED};
	if (comp < 0 || comp >= 10) return LFG_ERR_BAD_ARG;
	int c = map[comp];
	if (comp == 5 && S_.P.control == 1) c = SC_XF_RATEPROP;
	LFG_CUDA(cudaMemcpyAsync(out, S_.sc+(size_t)c*6*S_.n, sizeof(double)*6*S_.n, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	return LFG_OK;
}

int Sim::velocity_component(int comp, double *out)
{
	if (comp < 0 || comp >= NFC) return LFG_ERR_BAD_ARG;
	LFG_CUDA(cudaMemcpyAsync(out, S_.vc+(size_t)comp*6*S_.n, sizeof(double)*6*S_.n, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	return LFG_OK;
}

int Sim::set_contact(int p0, int p1, int state, const double *disp_tan, const double *disp_roll)
{
	if (p0 > p1) std::swap(p0, p1);
	std::vector<int> rp(S_.n+1);
	LFG_CUDA(cudaMemcpyAsync(rp.data(), S_.row_ptr, sizeof(int)*(S_.n+1), cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	if (p0 < 0 || p1 >= S_.n) return LFG_ERR_BAD_ARG;
	for (int t = rp[p0]; t < rp[p0+1]; t++) {
		DPair q;
		LFG_CUDA(cudaMemcpyAsync(&q, S_.pairs+t, sizeof q, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
		if (q.p1 != p1) continue;
		if (disp_tan) for (int k = 0; k < 3; k++) q.disp_tan[k] = disp_tan[k];
		if (disp_roll) for (int k = 0; k < 3; k++) q.disp_roll[k] = disp_roll[k];
		if (state >= 0 && (q.flags & PF_CONTACT)) q.state = state;
		LFG_CUDA(cudaMemcpyAsync(S_.pairs+t, &q, sizeof q, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
		return LFG_OK;
	}
	return LFG_ERR_BAD_ARG;
}

void Sim::set_clock(double time, double strain, double dt, double rate, double maxv, double maxsv)
{
	first_time();
	pull_clock();
	DevClock K = *h_clock_;
	K.time = time; K.strain = strain; K.dt = dt;
	K.max_velocity = maxv; K.max_sliding_velocity = maxsv;
	LFG_CUDA(cudaMemcpyAsync(S_.clock, &K, sizeof K, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	phys_set_shear_rate(S_, rate, false, st_);
	LFG_CUDA(cudaStreamSynchronize(st_));
}

void Sim::refresh()
{
	first_time();
	pull_clock();
	double msv = h_clock_->max_sliding_velocity;
	phys_pairs_update(S_, 0, 1, true, st_);
	pull_clock();
	DevClock K = *h_clock_;
	K.max_sliding_velocity = msv;
	LFG_CUDA(cudaMemcpyAsync(S_.clock, &K, sizeof K, cudaMemcpyHostToDevice, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
}

int Sim::assemble(double *dbl, int32_t *row, int32_t *col, double *odbl, int cap, int *nb_out)
{
	first_time();
	phys_blocks(S_, solver_->d_dblocks(), solver_->d_odblocks(), st_);
	LFG_CUDA(cudaStreamSynchronize(st_));
	if (dbl) LFG_CUDA(cudaMemcpyAsync(dbl, solver_->d_dblocks(), sizeof(double)*15*S_.n, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	std::vector<DPair> pairs(S_.npairs);
	std::vector<double> od(18*(size_t)S_.npairs);
	if (S_.npairs) {
		LFG_CUDA(cudaMemcpyAsync(pairs.data(), S_.pairs, sizeof(DPair)*S_.npairs, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
		LFG_CUDA(cudaMemcpyAsync(od.data(), solver_->d_odblocks(), sizeof(double)*18*S_.npairs, cudaMemcpyDeviceToHost, st_)); LFG_CUDA(cudaStreamSynchronize(st_));
	}
	int c = 0;
	const DevParams &P = S_.P;
	for (int t = 0; t < S_.npairs; t++) {
		const DPair &q = pairs[t];
		if (!(q.flags & PF_INTER)) continue;
		bool res = P.lub_on ? ((q.flags & PF_DASHPOT) || (q.flags & PF_LUB)) : (q.flags & PF_DASHPOT);
		if (!res) continue;
		if (c < cap) {
			if (row) row[c] = q.p1;
			if (col) col[c] = q.p0;
			if (odbl) std::memcpy(odbl+18*(size_t)c, &od[18*(size_t)t], sizeof(double)*18);
		}
		c++;
	}
	if (nb_out) *nb_out = c;
	return LFG_OK;
}

int Sim::force_component(int comp, double *out)
{
	if (comp < 0 || comp >= NFC) return LFG_ERR_BAD_ARG;
	first_time();
	phys_u_inf(S_, st_);
	phys_force_components(S_, st_);
	LFG_CUDA(cudaMemcpyAsync(out, S_.fc+(size_t)comp*6*S_.n, sizeof(double)*6*S_.n, cudaMemcpyDeviceToHost, st_));
	LFG_CUDA(cudaStreamSynchronize(st_));
	return LFG_OK;
}

// Same kernels and summation order as force_component, with the per-pair
// intermediate in the static no-allocation scratch and the result written to
// the caller's device buffer; nothing is allocated.
void Sim::force_component_noalloc(int comp, double *d_out, int device)
{
	// the pair-force components only: the Brownian one (FC_BROWNIAN) is not a
	// sum over pairs and has no slot in the scratch
	if (comp < 0 || comp >= NPFC) throw Error{LFG_ERR_BAD_ARG, comp, "component must be 0..3"};
	if (S_.npairs > NOALLOC_MAX_PAIRS)
		throw Error{LFG_ERR_BAD_ARG, S_.npairs, "pair slots exceed the no-allocation scratch (32768)"};
	double *scr = noalloc_pair_scratch(device);
	first_time();
	phys_u_inf(S_, st_);
	phys_force_component_into(S_, comp, scr, d_out, st_);
	LFG_CUDA(cudaGetLastError());
	LFG_CUDA(cudaStreamSynchronize(st_));
}

// device memory held by this suspension: fronts (the dominant term), pair
// records and their scratch, per-particle vectors, the compact R_FU values
int64_t Sim::device_bytes() const
{
	lfg_solver_stats ss;
	solver_->stats(&ss);
	int64_t pair = sizeof(DPair)+sizeof(DPairConst)+sizeof(double)*(30+12*NSC)+2*sizeof(int);
	int64_t part = sizeof(double)*(3*7+6*(1+4*NFC+NSC)+15)+sizeof(int)*8;
	int64_t w = opt_.precision == LFG_PREC_FP64 ? 8 : 4;
	int64_t sol = (int64_t)6*S_.n*4*w*4 + (int64_t)18*8*S_.cap;
	return ss.front_bytes+(int64_t)S_.cap*pair+(int64_t)S_.n*part+sol;
}

void Sim::timing(lfg_sim_timing *o) const
{
	std::memset(o, 0, sizeof *o);
	for (int k = 0; k < 8; k++) o->ms[k] = stage_ms_[k];
	o->launches = last_launches_;
	o->factor_flops = solver_->flops();
	o->solve_bytes = 2.0*(double)solver_->nnz_L()*(opt_.precision == LFG_PREC_FP64 ? 8 : 4);
	o->rebuild_ms = rebuild_ms_+(solver_->capture_ms()-capture_mark_);
	o->rebuilds = rebuilds_;
	o->run_steps = run_steps_;
	o->run_ms = run_ms_;
}

// nsteps loop steps (lfg_sim_run), timed as a whole on the device: one event
// before the first step's work and one after the last step's, so the host's
// part between steps (the end-of-step read of the clock, the next step's
// launches) counts as well
void Sim::run(int nsteps, double time_end, double strain_end)
{
	first_time();
	if (!run_a_) {
		LFG_CUDA(cudaEventCreate(&run_a_));
		LFG_CUDA(cudaEventCreate(&run_b_));
	}
	run_ms_ = 0;
	run_steps_ = 0;
	LFG_CUDA(cudaEventRecord(run_a_, st_));
	for (int k = 0; k < nsteps; k++) {
		step(0, time_end, strain_end);
		run_steps_++;
		if (error_code) break;
	}
	LFG_CUDA(cudaEventRecord(run_b_, st_));
	LFG_CUDA(cudaEventSynchronize(run_b_));
	float ms = 0;
	LFG_CUDA(cudaEventElapsedTime(&ms, run_a_, run_b_));
	run_ms_ = ms;
}


// ---------------------------------------------------------------------------
// Fused batch: independent suspensions advanced in lockstep through one joint
// solver.  The joint system is the block-diagonal matrix of all of them
// (symbolic_concat): every factorisation and solve launch serves every
// suspension, level by level of the merged assembly forest.  Each half step
// runs as CUDA graphs captured once per joint analysis: the suspensions'
// own kernels on parallel branches (one stream each), joined before the
// joint factorisation and solve.  The host synchronises three times per step:
// after each of the two solves (the FP32 refinement's convergence test, per
// suspension) and after the corrector (the pair supersets' staleness).
// Predictor-corrector steps only, no Brownian force; all suspensions share
// the precision and the number of unknowns per particle.
// ---------------------------------------------------------------------------
class FusedGroup {
public:
	FusedGroup(int device, int precision) : device_(device), prec_(precision)
	{
		LFG_CUDA(cudaSetDevice(device));
		LFG_CUDA(cudaStreamCreateWithFlags(&main_, cudaStreamNonBlocking));
		LFG_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
		LFG_CUDA(cudaMallocHost((void **)&h_status_, sizeof(int)));
	}
	~FusedGroup()
	{
		clear_graphs();
		delete joint_;
		for (cudaEvent_t e : join_) cudaEventDestroy(e);
		if (fork_) cudaEventDestroy(fork_);
		if (d_rhs_) cudaFree(d_rhs_);
		if (d_sol_) cudaFree(d_sol_);
		if (h_status_) cudaFreeHost(h_status_);
		if (main_) cudaStreamDestroy(main_);
	}
	void add(Sim *s)
	{
		const lfg_params &p = s->params();
		if (p.integration_method != 1) throw Error{LFG_ERR_BAD_ARG, 0, "a fused batch needs the predictor-corrector method"};
		if (p.brownian > 0) throw Error{LFG_ERR_BAD_ARG, 0, "a fused batch takes no Brownian forces"};
		if (!sims_.empty() && s->solver()->dof() != sims_[0]->solver()->dof())
			throw Error{LFG_ERR_BAD_ARG, 0, "a fused batch needs one kind of system (all 3D or all 2D)"};
		sims_.push_back(s);
		cudaEvent_t e;
		LFG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
		join_.push_back(e);
		dirty_ = true;
	}
	int size() const { return (int)sims_.size(); }
	// nsteps lockstep steps of every suspension (no stress output)
	void run(int nsteps)
	{
		std::vector<double> te(sims_.size(), -1.0), se(sims_.size(), 1e300);
		std::vector<char> act(sims_.size(), 1);
		for (int k = 0; k < nsteps; k++) step(0, te, se, act);
	}
	// System::timeEvolution of every suspension to its own strain: lockstep
	// steps while any suspension is short of its target (the others wait,
	// unchanged), then one stress-computing step of all of them
	void advance(const double *strain_end)
	{
		std::vector<double> te(sims_.size(), -1.0), se(strain_end, strain_end+sims_.size());
		for (;;) {
			std::vector<char> act(sims_.size(), 0);
			bool any = false;
			for (size_t i = 0; i < sims_.size(); i++) {
				sims_[i]->pull_clock_public();
				act[i] = sims_[i]->host_clock()->strain <= se[i]-1e-8;
				any = any || act[i];
			}
			if (!any) break;
			step(0, te, se, act);
		}
		std::vector<char> all(sims_.size(), 1);
		step(1, te, se, all);
	}
	int64_t kernels() const { return kernels_; }
	int symbolic_joint_runs() const { return joint_runs_; }
	double factor_flops() const { return joint_ ? joint_->flops() : 0; }
	int last_refine_iters() const { return last_iters_; }
	// nested-dissection leaf size of every suspension (the autotuner's knob)
	void set_leaf_size(int leaf)
	{
		for (Sim *s : sims_) s->set_leaf_size(leaf);
		dirty_ = true;
	}

private:
	void clear_graphs()
	{
		for (auto &g : graphs_) if (g.second) cudaGraphExecDestroy(g.second);
		graphs_.clear();
	}
	// the joint analysis: after additions and pattern changes
	void build_joint()
	{
		std::vector<const Symbolic *> parts;
		std::vector<int32_t> row, col;
		pbase_.assign(sims_.size()+1, 0);
		obase_.assign(sims_.size()+1, 0);
		for (size_t i = 0; i < sims_.size(); i++) {
			const Solver *v = sims_[i]->solver();
			parts.push_back(&v->symbolic());
			for (size_t e = 0; e < v->pattern_rows().size(); e++) {
				row.push_back(pbase_[i]+v->pattern_rows()[e]);
				col.push_back(pbase_[i]+v->pattern_cols()[e]);
			}
			pbase_[i+1] = pbase_[i]+v->n();
			obase_[i+1] = obase_[i]+(int)v->pattern_rows().size();
		}
		Symbolic J;
		symbolic_concat(J, parts);
		int ntot = pbase_.back();
		if (!joint_ || joint_->n() != ntot) {
			delete joint_;
			joint_ = nullptr;
			lfg_options o;
			lfg_default_options(&o);
			o.precision = prec_;
			o.device = device_;
			o.use_graphs = 0;   // the group captures the joint launches in its own graphs
			joint_ = new Solver(ntot, o, main_, sims_[0]->solver()->dof());
			if (d_rhs_) cudaFree(d_rhs_);
			if (d_sol_) cudaFree(d_sol_);
			d_rhs_ = d_sol_ = nullptr;
			// right-hand sides every suspension does not use stay zero
			LFG_CUDA(cudaMalloc((void **)&d_rhs_, sizeof(double)*6*(size_t)ntot*NPFC));
			LFG_CUDA(cudaMalloc((void **)&d_sol_, sizeof(double)*6*(size_t)ntot*NPFC));
			LFG_CUDA(cudaMemsetAsync(d_rhs_, 0, sizeof(double)*6*(size_t)ntot*NPFC, main_));
			LFG_CUDA(cudaMemsetAsync(d_sol_, 0, sizeof(double)*6*(size_t)ntot*NPFC, main_));
		}
		joint_->install(std::move(J), (int)row.size(), row.data(), col.data());
		joint_->set_segments(pbase_);
		joint_->reserve_refine(NPFC);   // no allocation inside the captured segments
		clear_graphs();
		joint_runs_++;
		dirty_ = false;
	}
	void fork()
	{
		LFG_CUDA(cudaEventRecord(fork_, main_));
		for (Sim *s : sims_) LFG_CUDA(cudaStreamWaitEvent(s->stream(), fork_, 0));
	}
	void join()
	{
		for (size_t i = 0; i < sims_.size(); i++) {
			LFG_CUDA(cudaEventRecord(join_[i], sims_[i]->stream()));
			LFG_CUDA(cudaStreamWaitEvent(main_, join_[i], 0));
		}
	}
	// the suspensions' right-hand sides into the joint one (6 n_i values of
	// each of their k_i right-hand sides at offset 6 pbase_i), and back
	void gather(size_t i, int k, const double *rhs)
	{
		int n6 = 6*sims_[i]->solver()->n(), N6 = 6*pbase_.back();
		LFG_CUDA(cudaMemcpy2DAsync(d_rhs_+6*(size_t)pbase_[i], sizeof(double)*N6, rhs, sizeof(double)*n6,
		                           sizeof(double)*n6, k, cudaMemcpyDeviceToDevice, sims_[i]->stream()));
	}
	void scatter(size_t i, int k, double *sol)
	{
		int n6 = 6*sims_[i]->solver()->n(), N6 = 6*pbase_.back();
		LFG_CUDA(cudaMemcpy2DAsync(sol, sizeof(double)*n6, d_sol_+6*(size_t)pbase_[i], sizeof(double)*N6,
		                           sizeof(double)*n6, k, cudaMemcpyDeviceToDevice, sims_[i]->stream()));
	}
	// launches of one graph segment: captured on first use, then replayed
	void segment(int key, const std::function<void()> &body)
	{
		auto it = graphs_.find(key);
		if (it == graphs_.end()) {
			cudaGraph_t g;
			LFG_CUDA(cudaStreamBeginCapture(main_, cudaStreamCaptureModeThreadLocal));
			try {
				body();
			} catch (...) {
				cudaStreamEndCapture(main_, &g);
				throw;
			}
			LFG_CUDA(cudaStreamEndCapture(main_, &g));
			size_t nn = 0;
			LFG_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
			std::vector<cudaGraphNode_t> nodes(nn);
			if (nn) LFG_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
			int64_t kn = 0;
			for (size_t q = 0; q < nn; q++) {
				cudaGraphNodeType t;
				LFG_CUDA(cudaGraphNodeGetType(nodes[q], &t));
				if (t == cudaGraphNodeTypeKernel) kn++;
			}
			cudaGraphExec_t ex;
			LFG_CUDA(cudaGraphInstantiate(&ex, g, 0));
			cudaGraphDestroy(g);
			it = graphs_.emplace(key, ex).first;
			graph_kernels_[key] = kn;
		}
		LFG_CUDA(cudaGraphLaunch(it->second, main_));
		kernels_ += graph_kernels_[key];
	}
	// one half step's solve: launched in a graph segment (refinement
	// iterations as many as the last solve needed), completed here
	void solve_finish(int k)
	{
		if (prec_ == LFG_PREC_FP64) return;
		int it = iters_planned_;
		double worst = joint_->refine_worst(k);
		lfg_options o;
		lfg_default_options(&o);
		while (!(worst <= o.refine_tol) && it < o.refine_max_iter) {
			joint_->refine_iterations(k, d_rhs_, 1);
			kernels_ += joint_->launches_solve()+3;   // sweeps, x += d, residual, norms
			it++;
			worst = joint_->refine_worst(k);
		}
		lfg_status st;
		std::memset(&st, 0, sizeof st);
		int rc = joint_->refine_finish(k, d_sol_, it, worst, &st);
		last_iters_ = it;
		joint_->set_pred_iters(it);
		if (rc) throw Error{rc, it, st.msg};
	}
	void solve_launch(int k)
	{
		if (prec_ == LFG_PREC_FP64) {
			joint_->solve_device(k, d_rhs_, d_sol_, nullptr, false);
			return;
		}
		joint_->refine_begin(k, d_rhs_);
		joint_->refine_iterations(k, d_rhs_, iters_planned_);
	}
	void step(int calc_stress, const std::vector<double> &te, const std::vector<double> &se,
	          const std::vector<char> &act)
	{
		cudaSetDevice(device_);
		if (dirty_) build_joint();
		std::vector<double> key_args(te);
		key_args.insert(key_args.end(), se.begin(), se.end());
		for (char a : act) key_args.push_back(a);
		if (key_args != graph_args_) { clear_graphs(); graph_args_ = key_args; }
		const size_t m = sims_.size();
		std::vector<int> k(m, 1);
		std::vector<double *> rhs(m, nullptr), sol(m, nullptr);
		const int kmax = kmax_of(calc_stress, act);
		double *dbl = joint_->d_dblocks(), *odbl = joint_->d_odblocks();
		if (prec_ != LFG_PREC_FP64) iters_planned_ = std::max(1, joint_->pred_iters());
		const int ip = iters_planned_;
		auto forces = [&](int in_pred) {
			fork();
			for (size_t i = 0; i < m; i++) {
				if (!act[i]) continue;
				k[i] = sims_[i]->pc_forces_rhs(calc_stress, in_pred, &rhs[i], &sol[i]);
				gather(i, k[i], rhs[i]);
			}
			join();
		};
		// predictor: time step, blocks, joint factorisation, forces, solve
		segment(key(0, calc_stress, ip), [&]() {
			fork();
			for (size_t i = 0; i < m; i++) {
				if (!act[i]) continue;
				Sim *s = sims_[i];
				if (!s->params().fixed_dt) phys_adapt_dt(s->dev(), te[i], se[i], s->stream());
				s->pc_pre_solve(dbl+15*(size_t)pbase_[i], odbl+18*(size_t)obase_[i]);
			}
			join();
			joint_->factorize_async();
			forces(1);
			solve_launch(kmax);
		});
		solve_finish(kmax);
		// predictor's velocities and move, corrector's blocks, factorisation, solve
		segment(key(1, calc_stress, ip), [&]() {
			fork();
			for (size_t i = 0; i < m; i++) {
				if (!act[i]) continue;
				Sim *s = sims_[i];
				double *r = nullptr, *x = nullptr;
				int ki = s->rhs_count(calc_stress, &r, &x);
				scatter(i, ki, x);
				s->pc_post_solve(calc_stress, 1);
				s->pc_move_predictor(calc_stress, te[i], se[i], false);
				s->pc_pre_solve(dbl+15*(size_t)pbase_[i], odbl+18*(size_t)obase_[i]);
			}
			join();
			joint_->factorize_async();
			forces(0);
			solve_launch(kmax);
		});
		solve_finish(kmax);
		// corrector's velocities and move, the supersets' check, clocks to the host
		segment(key(2, calc_stress, ip), [&]() {
			fork();
			for (size_t i = 0; i < m; i++) {
				if (!act[i]) continue;
				Sim *s = sims_[i];
				double *r = nullptr, *x = nullptr;
				int ki = s->rhs_count(calc_stress, &r, &x);
				scatter(i, ki, x);
				s->pc_post_solve(calc_stress, 0);
				s->pc_move_corrector(calc_stress, false);
				s->superset_check_launch();
				s->queue_clock_copy();
			}
			join();
			LFG_CUDA(cudaMemcpyAsync(h_status_, joint_->d_status(), sizeof(int), cudaMemcpyDeviceToHost, main_));
		});
		LFG_CUDA(cudaStreamSynchronize(main_));
		if (*h_status_ == 0) throw Error{LFG_ERR_TIMEOUT, 0, "a bounded device wait in the joint factorisation gave up"};
		if (*h_status_ != 0x7fffffff) throw Error{LFG_ERR_NOT_SPD, *h_status_, "non-positive pivot in the joint factorisation"};
		bool changed = false;
		for (size_t i = 0; i < m; i++) {
			if (!act[i] || !sims_[i]->host_clock()->stale) continue;
			sims_[i]->rebuild_superset();
			changed = true;
		}
		if (changed) { build_joint(); graph_args_.clear(); }
		segment(key(3, calc_stress, ip), [&]() {
			fork();
			for (size_t i = 0; i < m; i++)
				if (act[i]) phys_pairs_update(sims_[i]->dev(), 1, 0, false, sims_[i]->stream());
			join();
		});
		LFG_CUDA(cudaStreamSynchronize(main_));
	}
	int kmax_of(int calc_stress, const std::vector<char> &act)
	{
		int km = 1;
		for (size_t i = 0; i < sims_.size(); i++) {
			if (!act[i]) continue;
			double *r, *x;
			km = std::max(km, sims_[i]->rhs_count(calc_stress, &r, &x));
		}
		return km;
	}
	static int key(int seg, int calc_stress, int iters) { return (iters*2+calc_stress)*4+seg; }

	int device_, prec_;
	cudaStream_t main_ = nullptr;
	cudaEvent_t fork_ = nullptr;
	std::vector<cudaEvent_t> join_;
	std::vector<Sim *> sims_;
	std::vector<int> pbase_, obase_;
	Solver *joint_ = nullptr;
	double *d_rhs_ = nullptr, *d_sol_ = nullptr;
	int *h_status_ = nullptr;
	std::map<int, cudaGraphExec_t> graphs_;
	std::map<int, int64_t> graph_kernels_;
	std::vector<double> graph_args_;
	bool dirty_ = true;
	int iters_planned_ = 2, last_iters_ = 0;
	int joint_runs_ = 0;
	int64_t kernels_ = 0;
};

} // namespace lfg

using namespace lfg;

struct lfg_sim {
	cudaStream_t stream = nullptr;
	Sim *s = nullptr;
	int device = 0;
};

#define SIM_GUARD_BEGIN try {
#define SIM_GUARD_END                                                                   \
	}                                                                                   \
	catch (const lfg::Error &e) { return fail(st, e.code, e.info, e.msg.c_str()); }      \
	catch (const std::bad_alloc &) { return fail(st, LFG_ERR_OOM, 0, "host allocation failed"); } \
	catch (...) { return fail(st, LFG_ERR_CUDA, 0, "unexpected exception"); }

static int sim_status(lfg_sim *h, lfg_status *st)
{
	if (h->s->error_code) {
		int c = h->s->error_code;
		int rc = fail(st, c, h->s->error_info, h->s->error_msg.c_str());
		h->s->error_code = 0;
		return rc;
	}
	return ok(st);
}

namespace lfg {
int sim_output_snapshot(lfg_sim *h, OutputSnapshot &o)
{
	h->s->output_snapshot(o);
	return LFG_OK;
}
} // namespace lfg

extern "C" {

static int sim_new(const lfg_params *p, const lfg_options *opt, int n, const double *pos, const double *radius,
                   double lx, double ly, double lz, const double *le_disp, int ncs, const int32_t *cs_p0,
                   const int32_t *cs_p1, const double *cs_disp_tan, lfg_sim **out, lfg_status *st, bool fused);

int lfg_sim_create(const lfg_params *p, const lfg_options *opt, int n, const double *pos, const double *radius,
                   double lx, double ly, double lz, const double *le_disp, int ncs, const int32_t *cs_p0,
                   const int32_t *cs_p1, const double *cs_disp_tan, lfg_sim **out, lfg_status *st)
{
	return sim_new(p, opt, n, pos, radius, lx, ly, lz, le_disp, ncs, cs_p0, cs_p1, cs_disp_tan, out, st, false);
}

} // extern "C"

static int sim_new(const lfg_params *p, const lfg_options *opt, int n, const double *pos, const double *radius,
                   double lx, double ly, double lz, const double *le_disp, int ncs, const int32_t *cs_p0,
                   const int32_t *cs_p1, const double *cs_disp_tan, lfg_sim **out, lfg_status *st, bool fused)
{
	if (!p || !out || n <= 1 || !pos || !radius || lx <= 0 || lz <= 0 || ly < 0 || ncs < 0 ||
	    (ncs > 0 && (!cs_p0 || !cs_p1 || !cs_disp_tan)))
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	if (p->brownian > 0 && (p->integration_method != 1 || p->control != 0))
		return fail(st, LFG_ERR_BAD_ARG, 0,
		            "Brownian forces need the predictor-corrector method and rate control (System.cpp:423-436)");
	lfg_options o;
	if (opt) o = *opt; else lfg_default_options(&o);
	int rc = check_device(o.device, st);
	if (rc) return rc;
	lfg_sim *h = new (std::nothrow) lfg_sim();
	if (!h) return fail(st, LFG_ERR_OOM, 0, "host allocation failed");
	h->device = o.device;
	try {
		LFG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
		h->s = new Sim(*p, o, n, pos, radius, lx, ly, lz, le_disp, h->stream, fused);
		if (ncs) h->s->set_contacts(ncs, cs_p0, cs_p1, cs_disp_tan);   // System::setContacts
		h->s->first_time();
		*out = h;
		return ok(st);
	} catch (const lfg::Error &e) {
		delete h->s;
		if (h->stream) cudaStreamDestroy(h->stream);
		delete h;
		return fail(st, e.code, e.info, e.msg.c_str());
	} catch (...) {
		delete h->s;
		if (h->stream) cudaStreamDestroy(h->stream);
		delete h;
		return fail(st, LFG_ERR_OOM, 0, "allocation failed");
	}
}

namespace lfg {
FusedGroup *fused_create(int device, int precision) { return new FusedGroup(device, precision); }
void fused_destroy(FusedGroup *g) { delete g; }
int fused_add(FusedGroup *g, const lfg_params *p, const lfg_options *opt, int n, const double *pos,
              const double *radius, double lx, double ly, double lz, const double *le_disp, lfg_sim **out,
              lfg_status *st)
{
	int rc = sim_new(p, opt, n, pos, radius, lx, ly, lz, le_disp, 0, nullptr, nullptr, nullptr, out, st, true);
	if (rc) return rc;
	try {
		g->add((*out)->s);
	} catch (const Error &e) {
		lfg_sim_destroy(*out);
		*out = nullptr;
		return fail(st, e.code, e.info, e.msg.c_str());
	}
	return ok(st);
}
void fused_run(FusedGroup *g, int nsteps) { g->run(nsteps); }
void fused_advance(FusedGroup *g, const double *strain_end) { g->advance(strain_end); }
void fused_set_leaf_size(FusedGroup *g, int leaf) { g->set_leaf_size(leaf); }
void fused_stats(const FusedGroup *g, int64_t *kernels, int *joint_runs, double *flops, int *iters)
{
	*kernels = g->kernels();
	*joint_runs = g->symbolic_joint_runs();
	*flops = g->factor_flops();
	*iters = g->last_refine_iters();
}
} // namespace lfg

extern "C" {

int lfg_sim_advance(lfg_sim *h, double time_end, double strain_end, lfg_status *st)
{
	if (!h) return fail(st, LFG_ERR_BAD_ARG, 0, "null sim");
	SIM_GUARD_BEGIN
	cudaSetDevice(h->device);
	h->s->advance(time_end, strain_end);
	return sim_status(h, st);
	SIM_GUARD_END
}

int lfg_sim_advance_partial(lfg_sim *h, double time_end, double strain_end, int max_steps, int *done,
                            lfg_status *st)
{
	if (!h || max_steps < 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	SIM_GUARD_BEGIN
	cudaSetDevice(h->device);
	bool d = h->s->advance_partial(time_end, strain_end, max_steps);
	if (done) *done = d ? 1 : 0;
	return sim_status(h, st);
	SIM_GUARD_END
}

int lfg_sim_step(lfg_sim *h, int calc_stress, double time_end, double strain_end, lfg_status *st)
{
	if (!h) return fail(st, LFG_ERR_BAD_ARG, 0, "null sim");
	SIM_GUARD_BEGIN
	cudaSetDevice(h->device);
	h->s->step(calc_stress, time_end, strain_end);
	return sim_status(h, st);
	SIM_GUARD_END
}

int lfg_sim_run(lfg_sim *h, int nsteps, double time_end, double strain_end, lfg_status *st)
{
	if (!h || nsteps < 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	SIM_GUARD_BEGIN
	cudaSetDevice(h->device);
	h->s->run(nsteps, time_end, strain_end);
	return sim_status(h, st);
	SIM_GUARD_END
}

int lfg_sim_get_scalars(lfg_sim *h, lfg_sim_scalars *o)
{
	lfg_status *st = nullptr;
	if (!h || !o) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	h->s->scalars(o);
	return LFG_OK;
	SIM_GUARD_END
}

int lfg_sim_get_particles(lfg_sim *h, double *pos, double *vel, double *ang, double *na_vel, double *na_ang)
{
	lfg_status *st = nullptr;
	if (!h) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	h->s->particles(pos, vel, ang, na_vel, na_ang);
	return LFG_OK;
	SIM_GUARD_END
}

int lfg_sim_get_num_pairs(lfg_sim *h)
{
	if (!h) return -1;
	try { return h->s->num_pairs(); } catch (...) { return -1; }
}

int lfg_sim_get_pairs(lfg_sim *h, lfg_pair *out, int cap)
{
	if (!h || (cap > 0 && !out)) return -1;
	try { return h->s->get_pairs(out, cap); } catch (...) { return -1; }
}

int lfg_sim_get_particle_stress(lfg_sim *h, int comp, double *out)
{
	lfg_status *st = nullptr;
	if (!h || !out) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->particle_stress(comp, out);
	SIM_GUARD_END
}

int lfg_sim_set_brownian_force(lfg_sim *h, const double *fb, lfg_status *st)
{
	if (!h || !fb) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	SIM_GUARD_BEGIN
	h->s->set_brownian_force(fb);
	return ok(st);
	SIM_GUARD_END
}

int lfg_sim_get_velocity_component(lfg_sim *h, int comp, double *out)
{
	lfg_status *st = nullptr;
	if (!h || !out) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->velocity_component(comp, out);
	SIM_GUARD_END
}

int lfg_sim_set_contact(lfg_sim *h, int p0, int p1, int state, const double *disp_tan)
{
	lfg_status *st = nullptr;
	if (!h || !disp_tan) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->set_contact(p0, p1, state, disp_tan);
	SIM_GUARD_END
}

int lfg_sim_get_contact_states(lfg_sim *h, int32_t *p0, int32_t *p1, double *disp_tan, double *disp_rolling,
                               int cap)
{
	lfg_status *st = nullptr;
	if (!h || cap < 0) return -LFG_ERR_BAD_ARG;
	try {
		cudaSetDevice(h->device);
		return h->s->contact_states(p0, p1, disp_tan, disp_rolling, cap);
	} catch (...) {
		(void)st;
		return -LFG_ERR_CUDA;
	}
}

int lfg_sim_set_contact_rolling(lfg_sim *h, int p0, int p1, const double *disp_rolling)
{
	lfg_status *st = nullptr;
	if (!h || !disp_rolling) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->set_contact(p0, p1, -1, nullptr, disp_rolling);
	SIM_GUARD_END
}

int lfg_sim_set_clock(lfg_sim *h, double time, double strain, double dt, double shear_rate, double maxv,
                      double maxsv)
{
	lfg_status *st = nullptr;
	if (!h) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	h->s->set_clock(time, strain, dt, shear_rate, maxv, maxsv);
	return LFG_OK;
	SIM_GUARD_END
}

int lfg_sim_refresh(lfg_sim *h)
{
	lfg_status *st = nullptr;
	if (!h) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	h->s->refresh();
	return LFG_OK;
	SIM_GUARD_END
}

int lfg_sim_assemble(lfg_sim *h, double *dblocks, int32_t *od_row, int32_t *od_col, double *odblocks, int cap,
                     int *nb_out)
{
	lfg_status *st = nullptr;
	if (!h) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->assemble(dblocks, od_row, od_col, odblocks, cap, nb_out);
	SIM_GUARD_END
}

int lfg_sim_force_component(lfg_sim *h, int comp, double *out)
{
	lfg_status *st = nullptr;
	if (!h || !out) return LFG_ERR_BAD_ARG;
	SIM_GUARD_BEGIN
	return h->s->force_component(comp, out);
	SIM_GUARD_END
}

int lfg_sim_force_component_noalloc(lfg_sim *h, int comp, double *d_out, lfg_status *st)
{
	if (!h || !d_out) return fail(st, LFG_ERR_BAD_ARG, 0, "null simulation or output");
	SIM_GUARD_BEGIN
	LFG_CUDA(cudaSetDevice(h->device));
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, d_out) != cudaSuccess ||
	    !(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == h->device))) {
		cudaGetLastError();
		return fail(st, LFG_ERR_BAD_ARG, 0, "d_out must be device memory on the simulation's device");
	}
	h->s->force_component_noalloc(comp, d_out, h->device);
	return ok(st);
	SIM_GUARD_END
}

int lfg_sim_set_leaf_size(lfg_sim *h, int leaf_size, lfg_status *st)
{
	if (!h || leaf_size < 1) return fail(st, LFG_ERR_BAD_ARG, leaf_size, "bad arguments");
	SIM_GUARD_BEGIN
	LFG_CUDA(cudaSetDevice(h->device));
	h->s->set_leaf_size(leaf_size);
	return ok(st);
	SIM_GUARD_END
}

int64_t lfg_sim_device_bytes(lfg_sim *h)
{
	if (!h) return 0;
	try { return h->s->device_bytes(); } catch (...) { return 0; }
}

int lfg_sim_get_timing(lfg_sim *h, lfg_sim_timing *o)
{
	if (!h || !o) return LFG_ERR_BAD_ARG;
	h->s->timing(o);
	return LFG_OK;
}

int lfg_sim_get_step_times(lfg_sim *h, double *ms, int cap, int64_t *kernels)
{
	if (!h) return -1;
	int n = (int)h->s->step_ms.size();
	for (int k = 0; k < n && k < cap && ms; k++) ms[k] = h->s->step_ms[k];
	if (kernels) *kernels = h->s->step_kernels;
	return n;
}

void lfg_sim_clear_step_times(lfg_sim *h)
{
	if (!h) return;
	h->s->clear_timing();
}

void lfg_sim_destroy(lfg_sim *h)
{
	if (!h) return;
	cudaSetDevice(h->device);
	delete h->s;
	if (h->stream) cudaStreamDestroy(h->stream);
	delete h;
}

} // extern "C"

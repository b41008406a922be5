// lfg_physics.h -- device data layout and launchers of the per-step physics
// (lfg_physics.cu).  Internal to the engine.
#pragma once
#include "lfg_internal.h"

namespace lfg {

// Flat parameters as the kernels read them (passed by value).
struct DevParams {
	double kn, kt, mu_s, mu_d, critical_load, ft_max;
	double repulsion, rep_len, rep_max_len;
	double lub_reduce, lub_max_gap, interaction_range;
	double sd_coeff;
	double dp_normal_coeff, dp_tan_coeff;   // ContactDashpot.cpp:65-103, computed on the host
	double lx, ly, lz, lx_half, ly_half, lz_half;
	double Ehat[6], Ohat[3];
	double disp_max, dt_max, dt_min;
	double target_stress, init_strain_limit, init_rate_limit;
	double system_volume;
	double skin;
	double mu_r, kr;                       // rolling friction (Contact.cpp:35-45, 283-305)
	double brownian;                       // kT in internal units (0: no Brownian force)
	int friction_model, friction, rolling, repulsiveforce, lub_on, tangential, twodim, brownian_on;
	int fixed_dt, control, integration_method, n;
};

// Clocks and flow state, device resident (one per suspension).
struct DevClock {
	double time, strain, dt, shear_rate;
	double Einf[6], Omega[3], vel_diff[3], shear_disp[3];
	double max_velocity, max_sliding_velocity;
	double rate_prop, rate_indep;
	unsigned long long sq_max_sliding_bits;  // atomicMax accumulator (non-negative doubles)
	unsigned long long sq_max_vel_bits;
	long long steps;
	int stale;       // a pair within range is missing from the superset
	int pad_;
	double shear_strain[3];   // System::shear_strain: unwrapped sum of 2 Einf.ez dt (System.cpp:681-683)
};

// Pair state (one record per superset pair, sorted by (p0, p1)).
// PF_CHANGED: the contact opened or closed in the predictor's update of a
// Brownian step (Interaction::contact_state_changed_after_predictor)
enum { PF_INTER = 1, PF_CONTACT = 2, PF_LUB = 4, PF_DASHPOT = 8, PF_CHANGED = 16 };
struct DPair {
	double rvec[3], nvec[3], r, gap;
	double disp_tan[3], prev_disp_tan[3];
	double fs_total[3], fs_tan[3], fsn_norm, normal_load, rsv_sq;
	double lub_coeff, log_lub_coeff;
	double rep_force[3], rep_reduced;
	double disp_roll[3], prev_disp_roll[3], f_roll[3];   // rolling spring (Contact.h:33-70)
	double xf_contact[6];   // Contact::contact_stresslet_XF as of the last stress computation that set it
	int p0, p1, zoff, flags, state, pad_;
};

// Radius-dependent pair constants (Lubrication.cpp:165-294,
// ContactDashpot.cpp:107-183, Contact.cpp:35-45, RepulsiveForce.cpp:23-40).
enum { NLUB = 36, NDP = 16 };
struct DPairConst {
	double lc[NLUB];  // cXA cYA cYB cYC cXG cYG cYH cXM cYM (4 each)
	double dc[NDP];   // dashpot XA YA YB YC (4 each)
	double range, lub_range, a0, a1, ro, kn_s, kt_s, rep_geo, kr_s;
};

// Component slots.
// The pair-force components come first (NPFC of them, gathered from the
// pair scratch); the Brownian force (System::setBrownianForceToParticle) is
// generated per particle.  Sums over components run in the reference's
// std::map order: brownian, contact, dashpot, hydro, repulsion.
enum { FC_CONTACT = 0, FC_DASHPOT = 1, FC_HYDRO = 2, FC_REPULSION = 3, FC_BROWNIAN = 4, NFC = 5 };
constexpr int NPFC = 4;
enum { SC_ME = 0, SC_GU_CONTACT, SC_GU_DASHPOT, SC_GU_HYDRO, SC_GU_REPULSION,
       SC_XF_CONTACT, SC_XF_RATEINDEP, SC_XF_RATEPROP, SC_XF_REPULSION,
       SC_GU_BROWNIAN, SC_BROWNIAN_PRED, NSC };
// GU stress slot of force component c
__host__ __device__ inline int sc_gu_slot(int c) { return c == FC_BROWNIAN ? SC_GU_BROWNIAN : SC_GU_CONTACT+c; }

struct DevSim {
	int n = 0;
	DevParams P;
	DevClock *clock = nullptr;
	double *pos = nullptr, *radius = nullptr;
	double *vel = nullptr, *ang = nullptr, *vel_pred = nullptr, *ang_pred = nullptr, *u_inf = nullptr;
	double *na = nullptr;              // 6n
	double *na_disp = nullptr;         // 3n: System::na_disp (System.cpp:877, 981)
	double *angle = nullptr;           // n: System::angle (2D only, System.cpp:1113, 1151, 1178)
	double *vc = nullptr;              // NFC x 6n
	double *fc = nullptr;              // NFC x 6n
	double *rhs = nullptr, *sol = nullptr;  // NFC x 6n
	double *sc = nullptr;              // NSC x 6n
	double *sc_tot = nullptr;          // NSC x 6
	// superset pairs
	int npairs = 0, cap = 0;
	DPair *pairs = nullptr;
	DPairConst *pconst = nullptr;
	int *row_ptr = nullptr;            // n+1: pairs with p0 == i
	int *col_ptr = nullptr, *col_idx = nullptr;  // n+1 / P: pairs with p1 == i (ascending p0)
	double *blk_scratch = nullptr;     // P x 30 (b0, b1)
	double *pair_scratch = nullptr;    // P x 12 x max(NFC, NSC)
	// cells
	int ncx = 0, ncy = 0, ncz = 0, brute = 0;
	double csx = 0, csy = 0, csz = 0;
	int *cell_of = nullptr, *cell_start = nullptr, *cell_count = nullptr, *cell_list = nullptr;
	double *cell_rec = nullptr;        // 4n: (x, y, z, radius) of cell_list[k] at 4k (cell order)
	float *cell_rec32 = nullptr;       // 4n: the same rounded to FP32 (neighbour-test prefilter)
	int *cand_count = nullptr, *cand_ptr = nullptr, *cand = nullptr;
	int cand_cap = 0;
	int ncell_cap = 0;
	unsigned int *flag = nullptr;
	int64_t launches = 0;
};

// launchers
void phys_set_shear_rate(DevSim &S, double rate, bool from_device_value, cudaStream_t st);
void phys_u_inf(DevSim &S, cudaStream_t st);
void phys_cells(DevSim &S, double range_scale, cudaStream_t st);
// count (pass 1) / fill (pass 2) candidate pairs within the superset range
void phys_candidates(DevSim &S, cudaStream_t st, int *h_total);
void phys_check_superset(DevSim &S, cudaStream_t st);
void phys_pair_constants(DevSim &S, cudaStream_t st);
// mode 0: update interactions; 1: create (checkNewInteraction) then update;
// 2: create only
void phys_pairs_update(DevSim &S, int mode, int in_predictor, bool zero_dt, cudaStream_t st);
void phys_blocks(DevSim &S, double *d_dblocks, double *d_odblocks, cudaStream_t st);
void phys_force_components(DevSim &S, cudaStream_t st);
// force component comp into out (6n) through the static no-allocation scratch
constexpr int NOALLOC_MAX_PAIRS = 32768;
constexpr int NOALLOC_MAX_DEVICES = 64;
double *noalloc_pair_scratch(int device);
void phys_force_component_into(DevSim &S, int comp, double *scr, double *out, cudaStream_t st);
// divided = 1: one RHS per component (setSolverRHS); 0: their sum (addToSolverRHS)
void phys_rhs(DevSim &S, int divided, cudaStream_t st);
// in_predictor: the Brownian stress of the mid-point scheme (Stress.cpp:270-286)
void phys_stresslets(DevSim &S, int in_predictor, cudaStream_t st);
// psi: amp * standard normal deviates (6n), Philox4x32-10 keyed by seed,
// counter draw (one draw per Brownian force)
void phys_brownian_psi(DevSim &S, unsigned long long seed, unsigned long long draw, double amp, double *psi,
                       cudaStream_t st);
void phys_shear_rate_from_stress(DevSim &S, cudaStream_t st);
void phys_velocities(DevSim &S, int divided, int in_predictor, cudaStream_t st);
void phys_adapt_dt(DevSim &S, double time_end, double strain_end, cudaStream_t st);
// mode 0: Euler move (then na_disp), 1: predictor move, 2: corrector move (then na_disp)
void phys_move(DevSim &S, int mode, cudaStream_t st);
// per-pair output record (OUT_W doubles per superset pair): see k_pair_output
constexpr int OUT_W = 40;
void phys_pair_output(DevSim &S, double *out, cudaStream_t st);
void phys_boxing(DevSim &S, cudaStream_t st);
void phys_save_pred(DevSim &S, cudaStream_t st);
void phys_clear_sliding(DevSim &S, cudaStream_t st);
void phys_finish_sliding(DevSim &S, cudaStream_t st);
void phys_set_dt(DevSim &S, double dt, cudaStream_t st);
// fold a factorisation status word (first failing column + 1, INT_MAX = ok)
// into a sticky per-simulation error word
void phys_sticky_status(const int *status, int *err, cudaStream_t st);
// merge: for each new superset pair find the old record (binary search in the
// old row) and copy it, else initialise an empty record
// interactions, contacts, lubricated pairs, pairs with a resistance of the current state (4 ints)
void phys_pair_counts(DevSim &S, int *d_out, cudaStream_t st);
void phys_merge_pairs(DevSim &S, const DPair *old_pairs, const int *old_row_ptr, int old_n,
                      cudaStream_t st);

} // namespace lfg

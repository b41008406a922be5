/*
 * lfdem_gb300.h -- C ABI of the GB300 (sm_103a) engine for LF_DEM's
 * per-timestep hydrodynamic core.
 *
 * Two nested boundaries, both plain C (pointers and sizes, no CUDA or torch
 * types), every call returns an int status (LFG_OK = 0) and never throws:
 *
 *  1. lfg_solver_*  replaces the linear algebra behind LF_DEM's StokesSolver
 *     (LF_DEM/StokesSolver.h:198-285): block fill, CHOLMOD analyse/factorise
 *     (StokesSolver.cpp:937-978) and cholmod_solve2 (StokesSolver.cpp:671-703).
 *
 *  2. lfg_sim_*     replaces System::timeEvolution (LF_DEM/System.cpp:1203-1279)
 *     with a device-resident step loop: Lees-Edwards cell lists and pair
 *     discovery (System.cpp:1328-1373, BoxSet.cpp), Interaction::updateState
 *     (Interaction.cpp:171-236), resistance assembly (System.cpp:1429-1473),
 *     the resistance solve, RHS force components (System.cpp:1727-1828),
 *     stress-controlled shear rate (System.cpp:2017-2055), stresslets
 *     (Stress.cpp:77-287) and the predictor-corrector integrator
 *     (System.cpp:888-1187).
 *
 * Conventions: particle-major vectors of 6 doubles per particle (Fx Fy Fz Tx
 * Ty Tz, or Ux Uy Uz Wx Wy Wz), as in StokesSolver's RHS layout
 * (StokesSolver.h:31-45).  Resistance blocks are passed in LF_DEM's compact
 * forms: a DBlock is 15 doubles (col0[5] col1[3] col2[1] col3[3] col4[2]
 * col5[1]) and an ODBlock 18 doubles (col0[5] col1[3] col2[1] col3[5]
 * col4[3] col5[1]), MatrixBlocks.h:5-122.  An off-diagonal block (row r,
 * column c) has r > c.
 */
#ifndef LFDEM_GB300_H
#define LFDEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
	LFG_OK = 0,
	LFG_ERR_BAD_ARG = 1,   /* invalid argument or unsupported option */
	LFG_ERR_OOM = 2,       /* device or host allocation failed */
	LFG_ERR_NOT_SPD = 3,   /* non-positive pivot; lfg_status.info = scalar column + 1 */
	LFG_ERR_TIMEOUT = 4,   /* a bounded device wait gave up */
	LFG_ERR_CUDA = 5,      /* CUDA runtime error; lfg_status.msg has the text */
	LFG_ERR_NO_DEVICE = 6, /* no usable sm_103 device */
	LFG_ERR_NOT_CONVERGED = 7 /* FP32 + refinement did not reach the tolerance */
};

enum {
	LFG_PREC_FP64 = 0,        /* FP64 multifrontal Cholesky ("plain form") */
	LFG_PREC_FP32_REFINE = 1  /* FP32 factor + FP64 iterative refinement */
};

typedef struct {
	int code;
	int info;
	int refine_iters;      /* last solve's refinement iterations (FP32 form) */
	int pad_;
	double refine_residual; /* last solve's relative residual (FP32 form) */
	char msg[200];
} lfg_status;

/* Flat, already non-dimensionalised parameters (the subset of LF_DEM's
 * ParameterSet.h + System flags the step reads). */
typedef struct {
	double kn, kt;
	double mu_static, mu_dynamic;    /* mu_dynamic < 0 -> mu_static (System.cpp:370-372) */
	double critical_load;
	double ft_max;
	int friction_model;              /* 0,1,2,3,5,6 (Contact.cpp:10-33) */
	int repulsion_on;                /* "repulsion" present in the unit system */
	double repulsion;
	double repulsive_length;         /* <= 0 disables repulsion (System.cpp:415-418) */
	double repulsive_max_length;     /* -1: no tanh cutoff */
	int lubrication_model;           /* 0 none, 1 normal, 2 tangential */
	double lub_reduce_parameter;
	double lub_max_gap;
	double interaction_range;        /* -1: lubrication range (System.cpp:405-410) */
	double sd_coeff;
	double contact_relaxation_time;
	double contact_relaxation_time_tan;
	double disp_max, dt, dt_max, dt_min;
	int fixed_dt;
	int integration_method;          /* 0 Euler, 1 predictor-corrector */
	int control;                     /* 0 rate, 1 stress */
	double shear_rate;               /* rate control: imposed rate in internal units */
	double target_stress;            /* stress control: sigma/(6 pi), internal units */
	double Ehat[6];                  /* (xx,xy,xz,yz,yy,zz) at unit rate */
	double Ohat[3];
	double init_strain_shear_rate_limit;
	double init_shear_rate_limit;
	double mu_rolling;               /* > 0 enables rolling friction (System.cpp:386-388) */
	double kr;                       /* rolling spring constant (Contact.cpp:35-45) */
	double brownian;                 /* > 0: Brownian force with kT = brownian (internal units;
	                                    System::setBrownianForceToParticle, System.cpp:1665-1710):
	                                    rate control, predictor-corrector, fixed dt */
	uint64_t seed;                   /* random stream of the Brownian force (Philox4x32-10) */
} lfg_params;

/* LF_DEM's Parameter_File (the text of the file) and command-line control
 * ('r' with e.g. "1r" for `-r 1r`, 's' with e.g. "10cl" for `-s 10cl`)
 * resolved by the reference's own rules (SimulationInit.cpp:156-1014:
 * defaults, keyword parsing, unit suffixes, non-dimensionalisation; then
 * System.cpp:348-414) into the flat parameters above.  time_end / strain_end
 * are System::timeEvolution's arguments (the one not given is -1).  Brownian
 * and cohesive forces are refused (LFG_ERR_BAD_ARG, message in st). */
int lfg_config_resolve(const char *parameter_text, char control, const char *control_value,
                       lfg_params *out, double *time_end, double *strain_end, lfg_status *st);

/* The output side of the same resolution (SimulationInit.cpp:287-295,
 * 392-402, 455-472): the output unit (the control value's scale), the factor
 * from internal to output force units (Simulation::outputData's
 * force_ratios[internal/output], Simulation.cpp:654-663), the control value's
 * number (Simulation::input_rate / target_stress_input) and the output
 * switches of the Parameter_File. */
typedef struct {
	char unit[32];
	double internal_to_output;
	double input_value;
	int out_data_particle, out_data_interaction, origin_zero_flow, pad_;
	char out_particle_stress[32];   /* the out_particle_stress letters, quotes removed ("" by default) */
} lfg_output_units;
int lfg_config_output(const char *parameter_text, char control, const char *control_value, lfg_output_units *out,
                      lfg_status *st);

/* LF_DEM's checkpoint files (Simulation::checkpoint, Simulation.cpp:602-611).
 * Binary configuration conf_*.dat (Simulation.cpp:513-600, Configuration.h:
 * 67-120): written in the labelled format 2; read in format 2 and in the old
 * unlabelled format (unsigned-short contact particle numbers recognised as
 * the reference does).  lfg_conf_read_binary: call with NULL arrays to get
 * *np and *ncont, then with arrays of 3np (pos), np (radius), ncont (p0, p1)
 * and 3ncont (disp_tan, disp_rolling); meta = vf, lx, ly, lz, le_disp x, y.
 * State file chk_*.dat (States.cpp:9-66): format 1, strain, time, time in
 * simulation units.  Host I/O only. */
int lfg_conf_write_binary(const char *path, int np, double vf, double lx, double ly, double lz,
                          const double *le_disp, const double *pos, const double *radius, int ncont,
                          const int32_t *p0, const int32_t *p1, const double *disp_tan,
                          const double *disp_rolling, lfg_status *st);
int lfg_conf_read_binary(const char *path, int *np, int *ncont, int *format, double *meta, double *pos,
                         double *radius, int32_t *p0, int32_t *p1, double *disp_tan, double *disp_rolling,
                         lfg_status *st);
int lfg_checkpoint_write(const char *path, double strain, double time, double time_in_simulation_units,
                         lfg_status *st);
int lfg_checkpoint_read(const char *path, double *strain, double *time, double *time_in_simulation_units,
                        lfg_status *st);

/* Engine options (not physics). */
typedef struct {
	int precision;          /* LFG_PREC_* */
	int device;             /* CUDA device ordinal */
	double refine_tol;      /* relative residual target of the FP32 form (default 2e-10: two
	                           iterations at N=4096, velocities within ~1e-11 of the FP64 form) */
	int refine_max_iter;    /* default 30 */
	double skin;            /* pair superset skin, units of (a_i+a_j)/2 (default 0.15) */
	int use_graphs;         /* capture factor/solve launch sequences in CUDA graphs (default 1) */
	int leaf_size;          /* nested-dissection leaf size in particles (default 16) */
	int dof_2d;             /* unknowns per particle of a 2D run (ly = 0) without Brownian force:
	                           3 (default) solves only the in-plane x, z translation and y rotation,
	                           which the 6x6 blocks of a monolayer decouple exactly from the others
	                           (their out-of-plane velocities are 0); 6 keeps LF_DEM's 6x6 blocks
	                           (System.cpp:478-491, StokesSolver.cpp:87-100).  3D and Brownian runs
	                           always use 6. */
} lfg_options;

void lfg_default_options(lfg_options *opt);

/* Library / device information.  Returns LFG_OK if an sm_103 device is usable. */
int lfg_device_info(int device, char *name, int name_len, int *sm_major, int *sm_minor, int *sm_count);

/* ------------------------------------------------------------------ */
/* 1. Inner boundary: the resistance solve (StokesSolver replacement). */
/* ------------------------------------------------------------------ */
typedef struct lfg_solver lfg_solver;

/* StokesSolver::init (StokesSolver.cpp:77-106): n_mobile particles, dof 6;
 * or dof 3 for a 2D system (ly = 0), whose 6x6 blocks couple the in-plane
 * unknowns (x, z translation, y rotation: components 0, 2, 4) only among
 * themselves: the solver then factors those alone.  Blocks, right-hand sides
 * and solutions keep LF_DEM's 6-per-particle layout either way; with dof 3
 * the other components of a right-hand side are not read and those of a
 * solution are 0.  LF_DEM itself has no 3-unknown variant. */
int lfg_solver_create(int n_mobile, int dof, const lfg_options *opt, lfg_solver **out,
                      lfg_status *st);

/* StokesSolver::resetResistanceMatrix + addResistanceBlocks + matrixFillingDone
 * (StokesSolver.cpp:121-152, 474-511, 937-948): the complete lower block
 * matrix.  dblocks: n x 15; od_row/od_col/odblocks: nb entries of 18.
 * pattern_changed = 1 re-runs the symbolic analysis (cholmod_analyze,
 * StokesSolver.cpp:955-962); 0 reuses it (the (row,col) list must then be
 * identical to the previous call's).  positions (3n, may be NULL) guide the
 * nested-dissection ordering; without them a graph ordering is used. */
int lfg_solver_set_blocks(lfg_solver *s, const double *dblocks, int nb, const int32_t *od_row,
                          const int32_t *od_col, const double *odblocks, int pattern_changed,
                          const double *positions, lfg_status *st);

/* cholmod_factorize (StokesSolver.cpp:950-978).  LFG_ERR_NOT_SPD carries the
 * failing scalar column (original numbering) + 1 in st->info. */
int lfg_solver_factorize(lfg_solver *s, lfg_status *st);

/* cholmod_solve2(CHOLMOD_A) for k right-hand sides (StokesSolver.cpp:671-703):
 * rhs and x are k x 6n host arrays (x may alias rhs). */
int lfg_solver_solve(lfg_solver *s, int k, const double *rhs, double *x, lfg_status *st);

/* x = L rhs for k right-hand sides (k x 6n host arrays, x must not alias rhs)
 * with the current factor, L L^T = R in the caller's numbering:
 * StokesSolver::compute_LTRHS (StokesSolver.cpp:627-669), used for the
 * Brownian force.  L is this engine's factor (nested-dissection order); the
 * reference's CHOLMOD L is another square root of R. */
int lfg_solver_multiply_factor(lfg_solver *s, int k, const double *rhs, double *x, lfg_status *st);

/* Device-pointer variant: rhs and x are k x 6n device arrays. */
int lfg_solver_solve_device(lfg_solver *s, int k, const double *d_rhs, double *d_x,
                            lfg_status *st);

/* Symbolic statistics of the current analysis. */
typedef struct {
	int n_blocks, n_supernodes, n_levels, max_front;
	int64_t nnz_L;          /* scalar nonzeros of L (dense supernodal panels) */
	double flops_factor;    /* sum_s n^3/3 + n^2 m + n m^2 (scalar columns) */
	int64_t front_bytes;    /* device bytes of the front arena */
	int n_factor_launches, n_solve_launches;
} lfg_solver_stats;
int lfg_solver_get_stats(const lfg_solver *s, lfg_solver_stats *out);

void lfg_solver_destroy(lfg_solver *s);

/* ------------------------------------------------------------------ */
/* 2. Outer boundary: the per-timestep core (System::timeEvolution).   */
/* ------------------------------------------------------------------ */
typedef struct lfg_sim lfg_sim;

/* System::setupConfiguration (System.cpp:468-521) + the first-time block of
 * timeEvolution.  pos: 3n, radius: n, le_disp: 2 (may be NULL), contact
 * states (ncs entries of p0 < p1 with disp_tan, System::setContacts
 * System.cpp:266-285). */
int lfg_sim_create(const lfg_params *p, const lfg_options *opt, int n, const double *pos,
                   const double *radius, double lx, double ly, double lz, const double *le_disp,
                   int ncs, const int32_t *cs_p0, const int32_t *cs_p1, const double *cs_disp_tan,
                   lfg_sim **out, lfg_status *st);

/* System::timeEvolution(time_end, strain_end), System.cpp:1203-1279: steps
 * until the end (negative = unused), then one stress-computing step. */
int lfg_sim_advance(lfg_sim *s, double time_end, double strain_end, lfg_status *st);

/* One timeEvolutionDt call (System.cpp:843-983) preceded by the loop's
 * adaptTimeStep (System.cpp:1243-1245). */
int lfg_sim_step(lfg_sim *s, int calc_stress, double time_end, double strain_end, lfg_status *st);

/* nsteps steps without stress output (the throughput loop). */
int lfg_sim_run(lfg_sim *s, int nsteps, double time_end, double strain_end, lfg_status *st);

/* lfg_sim_advance in slices: at most max_steps loop steps of
 * System::timeEvolution; when the end is reached, also the final
 * stress-computing step, and *done = 1. */
int lfg_sim_advance_partial(lfg_sim *s, double time_end, double strain_end, int max_steps, int *done,
                            lfg_status *st);

typedef struct {
	double time, strain, shear_rate, dt;
	double shear_disp[2];
	double max_velocity, max_sliding_velocity;
	double total_stress[6];
	double viscosity, N1, N2;
	double rate_prop_shearstress, rate_indep_shearstress;
	int64_t total_num_timesteps;
	int n_pairs, n_contacts, n_lub, n_resistance_pairs;
	int n_superset_pairs, n_symbolic_runs;
	int last_refine_iters, pad_;
	double last_refine_residual;
} lfg_sim_scalars;
int lfg_sim_get_scalars(lfg_sim *s, lfg_sim_scalars *out);

/* pos, vel, angvel, na_vel, na_angvel: 3n each, any may be NULL. */
int lfg_sim_get_particles(lfg_sim *s, double *pos, double *vel, double *angvel, double *na_vel,
                          double *na_angvel);

/* Interactions (pairs with an Interaction object), sorted by (p0, p1). */
typedef struct {
	int32_t p0, p1, z_offset, contact_active, state, lub_active, pad0_, pad1_;
	double r, reduced_gap;
	double nvec[3], rvec[3], disp_tan[3], f_spring_total[3];
	double lub_coeff, log_lub_coeff;
	double rep_force[3];
} lfg_pair;
int lfg_sim_get_num_pairs(lfg_sim *s);
int lfg_sim_get_pairs(lfg_sim *s, lfg_pair *out, int cap);

/* Per-particle stress of one component (6n, Sym2Tensor order xx xy xz yz yy
 * zz): 0 GU contact, 1 GU dashpot, 2 GU hydro, 3 GU repulsion, 4 M_E_hydro,
 * 5 xF_contact (rate) / xF_contact_rateprop (stress), 6 xF_contact_rateindep,
 * 7 xF_repulsion.  Valid after a stress-computing step. */
int lfg_sim_get_particle_stress(lfg_sim *s, int comp, double *out);
/* Non-affine velocity component (6n): 0 contact 1 dashpot 2 hydro 3 repulsion. */
int lfg_sim_get_velocity_component(lfg_sim *s, int comp, double *out);

/* Restart hooks (parity tests and checkpoint restore): set pair (p0,p1)'s
 * tangential spring and friction state; set clocks; recompute every pair's
 * forces at the current positions with dt = 0 (System.cpp:1216-1226). */
int lfg_sim_set_contact(lfg_sim *s, int p0, int p1, int state, const double *disp_tan);
/* The rolling spring of that contact (contact_state.disp_rolling, Contact.h:150-162).
 * On restart, set the rolling springs after lfg_sim_create and then call
 * lfg_sim_refresh, so the first step starts from forces that include them. */
int lfg_sim_set_contact_rolling(lfg_sim *s, int p0, int p1, const double *disp_rolling);
/* Active contacts and their springs (System::getContacts, System.cpp:306-320),
 * sorted by (p0, p1): returns the count and copies up to cap of them
 * (disp_tan, disp_rolling: 3 per contact; any array may be NULL); a negative
 * value is an error code. */
int lfg_sim_get_contact_states(lfg_sim *s, int32_t *p0, int32_t *p1, double *disp_tan,
                               double *disp_rolling, int cap);
int lfg_sim_set_clock(lfg_sim *s, double time, double strain, double dt, double shear_rate,
                      double max_velocity, double max_sliding_velocity);
int lfg_sim_refresh(lfg_sim *s);

/* Stage-level entry points (kernel parity tests): assemble R_FU for the
 * current state and copy it out (dblocks n x 15; odblocks for the nb
 * resistance pairs, sorted by (col,row)); force component comp at the current
 * state (6n). */
int lfg_sim_assemble(lfg_sim *s, double *dblocks, int32_t *od_row, int32_t *od_col,
                     double *odblocks, int cap, int *nb_out);
int lfg_sim_force_component(lfg_sim *s, int comp, double *out);

/* Pair-force component comp (0 contact, 1 dashpot, 2 hydro, 3 repulsion; 4,
 * the Brownian force, is refused with LFG_ERR_BAD_ARG) at the current state,
 * like lfg_sim_force_component, written to DEVICE memory d_out (6n doubles on
 * the simulation's device),
 * allocating nothing: no cudaMalloc/cudaFree and no pinned staging.  This
 * entry point has no counterpart in the reference (LF_DEM keeps no device
 * memory).  It is for callers that may not allocate device memory while they
 * run: an application that owns every device allocation through its own pool
 * or arena, or one on a path where the implicit device synchronisation of
 * cudaMalloc/cudaFree is not allowed.
 *  - The per-pair intermediate of the requested component goes to a fixed
 *    scratch in static device memory with room for LFG_NOALLOC_MAX_PAIRS
 *    pair slots (12 doubles each, 3.1 MB per device).  A simulation whose candidate-pair list is longer
 *    gets LFG_ERR_BAD_ARG; use lfg_sim_force_component there.
 *  - Neither the scratch nor d_out needs to start at zero: every value read
 *    is written earlier in the same call, and all 6n outputs are written.
 *  - The first call on a device does set-up (it resolves the scratch's device
 *    address with cudaGetSymbolAddress, with that device current); make that
 *    first call before any stream capture.
 *  - All calls on one device share the scratch.  Calls that overlap in time
 *    (from several threads, or for several simulations on one device) race
 *    and corrupt each other's results: the caller must serialise them.
 * Returns when the result is in d_out. */
#define LFG_NOALLOC_MAX_PAIRS 32768
int lfg_sim_force_component_noalloc(lfg_sim *s, int comp, double *d_out, lfg_status *st);

/* Timing of the last lfg_sim_run / lfg_sim_step, device milliseconds by stage
 * (0 pairs, 1 assembly, 2 factorisation, 3 solves, 4 forces+stress, 5 move)
 * and kernels launched. */
typedef struct {
	double ms[8];
	int64_t launches;
	double factor_flops;     /* algorithmic flops of one factorisation */
	double solve_bytes;      /* algorithmic bytes of one forward+backward solve, 1 RHS */
	double rebuild_ms;       /* host wall time of the pair-superset rebuilds since the last
	                            lfg_sim_clear_step_times: candidate pairs, symbolic analysis
	                            (cholmod_analyze's counterpart, StokesSolver.cpp:955-962) and
	                            upload, plus the capture of the new factorisation and solve
	                            graphs after them */
	int rebuilds;            /* number of those rebuilds */
	int run_steps;           /* steps of the last lfg_sim_run */
	double run_ms;           /* device duration of the last lfg_sim_run as a whole: CUDA
	                            events on the simulation's stream before its first step and
	                            after its last, the gaps between the steps included */
} lfg_sim_timing;
int lfg_sim_get_timing(lfg_sim *s, lfg_sim_timing *out);

/* Device duration (ms, CUDA events on the simulation's stream) of every step
 * since the last lfg_sim_clear_step_times; returns the number recorded and
 * copies up to cap of them.  Also the number of kernels launched in them. */
int lfg_sim_get_step_times(lfg_sim *s, double *ms, int cap, int64_t *kernels);
void lfg_sim_clear_step_times(lfg_sim *s);

void lfg_sim_destroy(lfg_sim *s);

/* Test and restart hook (Brownian runs): the next step's predictor uses this
 * Brownian force (6n host doubles, (F, T) per particle) instead of drawing
 * one -- the force a reference run drew, for a step-by-step comparison. */
int lfg_sim_set_brownian_force(lfg_sim *s, const double *fb, lfg_status *st);

/* LF_DEM's text output files for a simulation (Simulation::openOutputFiles,
 * SimulationInit.cpp:1034-1074; Simulation::generateOutput with "data" and
 * "config", Simulation.cpp:145-163): data_<name>.dat and st_<name>.dat
 * (Simulation::outputData, Simulation.cpp:641-792), par_<name>.dat and
 * int_<name>.dat (outputParFileTxt / outputIntFileTxt, Simulation.cpp:
 * 884-1006), column for column, OutputData's format (OutputData.h:27-209).
 * unit / internal_to_output / input_value as lfg_config_output gives them;
 * version goes into the "# LF_DEM version" header line; volume_fraction into
 * "# VF".  Existing files are an error unless force_overwrite.  Rows of int_
 * are sorted by particle pair.  Simple shear, no walls (what the engine runs).
 * With out_particle_stress letters (the Parameter_File keyword, e.g. "tc";
 * NULL or "" for none) each output event also writes a pst_<name>.dat block
 * (Simulation::outputPstFileTxt, Simulation.cpp:823-852): per particle, for
 * each group the letters name (l hydro, c contact, r repulsion, b brownian,
 * d dashpot, t total; any other letter the unnamed empty group, all zeros),
 * in group-name order, the sum of its stress components' per-particle
 * stresslets (Simulation::getParticleStressGroup, Simulation.cpp:628-639). */
typedef struct lfg_output lfg_output;
typedef struct {
	const char *directory;          /* NULL or "": the working directory */
	const char *simu_name;
	const char *version;
	const char *unit;
	double internal_to_output;
	double input_value;
	double volume_fraction;
	int out_data_particle, out_data_interaction, origin_zero_flow, diminish_output, force_overwrite;
	const char *out_particle_stress;  /* NULL or "": no pst_ file */
} lfg_output_config;
int lfg_output_open(lfg_sim *s, const lfg_output_config *cfg, lfg_output **out, lfg_status *st);
/* One output event at the current state: a data_ / st_ line, a par_, an
 * int_ and a pst_ block. */
int lfg_output_write(lfg_output *o, lfg_status *st);
void lfg_output_close(lfg_output *o);

/* Re-run the symbolic analysis of the current pattern with another
 * nested-dissection leaf size (supernode size at the leaves). */
int lfg_sim_set_leaf_size(lfg_sim *s, int leaf_size, lfg_status *st);
/* Device bytes held by the simulation (fronts, pair records, vectors). */
int64_t lfg_sim_device_bytes(lfg_sim *s);

/* ------------------------------------------------------------------ */
/* 3. Many suspensions on one GPU (a rheology sweep, and a server).    */
/* These have no single counterpart in the reference, which runs one   */
/* System per process; each suspension behaves exactly like one        */
/* simulation of its own: the same results alone or together.        */
/* ------------------------------------------------------------------ */

/* Estimated device bytes of one suspension of n particles (phi 0.45-0.58)
 * before it exists: the factor's front arena (~N^1.55) plus pair records. */
int64_t lfg_footprint_estimate(int n, int precision);

/* Batch: suspensions of uneven N advanced together; nthreads host workers
 * (0: one per core, at most 16) step them in slices on their own streams. */
typedef struct lfg_batch lfg_batch;
int lfg_batch_create(int device, int nthreads, lfg_batch **out, lfg_status *st);
/* Same arguments as lfg_sim_create (no contact states); *slot = its index. */
int lfg_batch_add(lfg_batch *b, const lfg_params *p, const lfg_options *opt, int n, const double *pos,
                  const double *radius, double lx, double ly, double lz, const double *le_disp, int *slot,
                  lfg_status *st);
int lfg_batch_size(const lfg_batch *b);
/* The slot's simulation, for the lfg_sim_get_* calls (owned by the batch). */
lfg_sim *lfg_batch_sim(lfg_batch *b, int slot);
/* Every suspension nsteps steps (lfg_sim_run). */
int lfg_batch_run(lfg_batch *b, int nsteps, lfg_status *st);
/* Every suspension to its own strain_end[slot] (lfg_sim_advance). */
int lfg_batch_advance(lfg_batch *b, const double *strain_end, lfg_status *st);
/* Autotuner: per size class (half-octaves of N, precision), time `steps`
 * steps of one member with each candidate leaf size and keep the fastest
 * for the class (and for suspensions added later). */
int lfg_batch_autotune(lfg_batch *b, const int *leaf_sizes, int count, int steps, lfg_status *st);
/* The leaf size chosen for (n, precision), 0 if none. */
int lfg_batch_tuned_leaf(const lfg_batch *b, int n, int precision);
void lfg_batch_destroy(lfg_batch *b);

/* Fused batch: the suspensions advance in lockstep through ONE joint
 * factorisation and solve of the block-diagonal system of all of them (the
 * assembly trees merged level by level from the leaves), so each launch of
 * the factorisation and of the solve serves every suspension; each half step
 * is a CUDA graph (the suspensions' own kernels on parallel branches) that
 * is captured once per joint analysis and replayed.  The FP32 refinement
 * stops when every suspension's own relative residual meets the tolerance.
 * Each suspension's results are those it gets alone, to the solve's
 * tolerance (1e-10 relative in FP64, 1e-8 with FP32 + refinement).  The
 * host waits three times per step (after each solve and after the
 * corrector's superset check); a pattern change of any suspension redoes
 * its analysis and the joint one.  Same calls as a batch: lfg_batch_add
 * (predictor-corrector, no Brownian force, all 3D or all 2D; the options'
 * precision is replaced by the batch's), lfg_batch_run, lfg_batch_advance
 * (lockstep until each suspension reaches its strain, the finished ones
 * waiting, then one stress-computing step of all), lfg_batch_autotune (the
 * leaf size of all suspensions, timed on the fused step), lfg_batch_sim (to
 * read a suspension's state; it cannot step on its own). */
int lfg_batch_create_fused(int device, int precision, lfg_batch **out, lfg_status *st);

/* Counters of a batch: kernels launched so far (graph kernel nodes counted
 * per replay), joint analyses (fused), factorisation flops of the joint
 * system (fused), refinement iterations of the last solve (fused FP32). */
typedef struct {
	int64_t kernels;
	int joint_analyses, last_refine_iters;
	double factor_flops;
	int fused, pad_;
} lfg_batch_stats;
int lfg_batch_get_stats(const lfg_batch *b, lfg_batch_stats *out);

/* Server: requests admitted while fewer than max_active run and their
 * estimated footprint fits in hbm_budget_bytes next to the running ones
 * (first fit in arrival order; one request always runs when nothing else
 * does); each runs to strain_end on its own stream and worker thread, and
 * newly arrived requests join as others finish. */
typedef struct lfg_server lfg_server;
typedef struct {
	int64_t id;
	const lfg_params *params;
	const lfg_options *options;     /* may be NULL (defaults) */
	int n;
	const double *pos, *radius;     /* copied by lfg_server_submit */
	double lx, ly, lz;
	double strain_end;
} lfg_request;
typedef struct {
	int64_t id;
	int status, n;                  /* status: LFG_OK or the error code */
	int64_t steps;
	double t_submit, t_admit, t_done;   /* seconds since lfg_server_create */
	double strain, shear_rate, viscosity, N1, N2;
	int64_t footprint_est, footprint_bytes;
	char msg[120];
} lfg_result;
typedef struct {
	int64_t submitted, admitted;
	int active, queued, peak_active, pad_;
	int64_t reserved_bytes, peak_reserved_bytes, budget_bytes;
} lfg_server_stats;
int lfg_server_create(int device, int max_active, int64_t hbm_budget_bytes, lfg_server **out,
                      lfg_status *st);
int lfg_server_submit(lfg_server *s, const lfg_request *r, lfg_status *st);
/* Copies up to cap finished results (each returned once); returns the count. */
int lfg_server_poll(lfg_server *s, lfg_result *out, int cap);
/* Until every submitted request has finished (timeout_s <= 0: no limit). */
int lfg_server_wait(lfg_server *s, double timeout_s, lfg_status *st);
/* Final positions (3n) of a finished request. */
int lfg_server_final_positions(lfg_server *s, int64_t id, double *pos, int n);
int lfg_server_get_stats(lfg_server *s, lfg_server_stats *out);
void lfg_server_destroy(lfg_server *s);

#ifdef __cplusplus
}
#endif
#endif

/*
 * lfdem_oracle.h -- CPU restatement (plain C, FP64) of LF_DEM's per-timestep
 * hydrodynamic core.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * engine in lf_dem_gb300/.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  The product path
 * never links, loads or calls it.
 *
 * Every function cites the reference file:line whose behaviour it restates
 * (paths relative to the LF_DEM project root).  The restatement is pinned
 * against the reference's own C++ sources, compiled here into oracle/_ref by
 * oracle/Makefile, through the fixtures in tests/golden/.
 *
 * Scope: simple shear (Lees-Edwards), rate or stress control, lubrication
 * models none/normal/tangential, friction models 0/1/2/3/5/6, repulsion
 * (exp, optional tanh cutoff), contact dashpots, Stokes drag, predictor-
 * corrector or Euler integration, 3D or 2D (ly = 0).  Not covered (as in the
 * GPU engine): Brownian forces, cohesion, rolling friction, vdW, fixed
 * particles, extensional flow.
 */
#ifndef LFDEM_ORACLE_H
#define LFDEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Flat, already non-dimensionalised parameter set (the subset of
 * ParameterSet.h that the hot path reads). */
typedef struct {
	double kn, kt;                   /* contact stiffnesses */
	double mu_static, mu_dynamic;    /* mu_dynamic < 0 -> = mu_static (System.cpp:370) */
	double critical_load;            /* friction_model 2/3 */
	double ft_max;                   /* friction_model 5/6 */
	int friction_model;              /* 0,1,2,3,5,6 */
	int repulsion_on;                /* "repulsion" present in the unit system */
	double repulsion;                /* amplitude in internal units */
	double repulsive_length;         /* <= 0 disables repulsion (System.cpp:415) */
	double repulsive_max_length;     /* -1 = no tanh cutoff */
	int lubrication_model;           /* 0 none, 1 normal, 2 tangential */
	double lub_reduce_parameter;     /* lambda regularisation */
	double lub_max_gap;
	double interaction_range;        /* -1 -> lubrication range */
	double sd_coeff;                 /* Stokes drag coefficient */
	double contact_relaxation_time;
	double contact_relaxation_time_tan;
	double disp_max, dt, dt_max, dt_min;
	int fixed_dt;
	int integration_method;          /* 0 Euler, 1 predictor-corrector */
	int control;                     /* 0 rate, 1 stress */
	double shear_rate;               /* rate control: imposed rate */
	double target_stress;            /* stress control: sigma/(6 pi) in internal units */
	double Ehat[6];                  /* (xx,xy,xz,yz,yy,zz) at unit rate */
	double Ohat[3];
	double init_strain_shear_rate_limit; /* System.cpp:90 default 0 */
	double init_shear_rate_limit;        /* System.cpp:91 default 999 */
	double mu_rolling;               /* > 0 enables rolling friction (System.cpp:386-388) */
	double kr;                       /* rolling spring constant */
} lfo_params;

typedef struct lfo_sim lfo_sim;

/* Pair record exported by lfo_get_pairs (sorted by (p0,p1)). */
typedef struct {
	int p0, p1;
	int z_offset;
	int contact_active;
	int state;              /* friction state 0..3 (Contact.h:110-116) */
	int lub_active;
	int dashpot_active;
	int pad_;
	double r, reduced_gap;
	double nvec[3];
	double rvec[3];
	double disp_tan[3];
	double f_spring_total[3];
	double lub_coeff, log_lub_coeff;
	double rep_force[3];
} lfo_pair_out;

/* Scalars exported by lfo_get_scalars. */
typedef struct {
	double time, strain, shear_rate, dt;
	double shear_disp[2];
	double max_velocity, max_sliding_velocity;
	double total_stress[6];
	double viscosity, N1, N2;
	double rate_prop_shearstress, rate_indep_shearstress;
	long long total_num_timesteps;
	int n_pairs, n_contacts, n_lub;
	int n_resistance_pairs;
	int pad_;
} lfo_scalars;

/* Create a system from a configuration (System::setupGenericConfiguration,
 * System.cpp:468-521).  Contact states (p0<p1, disp_tan) come from a
 * configuration file (System::setContacts, System.cpp:266-285). */
lfo_sim *lfo_create(const lfo_params *p, int np,
                    const double *pos /*3np*/, const double *radius,
                    double lx, double ly, double lz,
                    const double *le_disp /*2*/,
                    int ncs, const int *cs_p0, const int *cs_p1,
                    const double *cs_disp_tan /*3 ncs*/);
void lfo_destroy(lfo_sim *s);

/* System::timeEvolution (System.cpp:1203-1279): loops steps until
 * time_end/strain_end (negative = unused) then one calc_stress step. */
int lfo_time_evolution(lfo_sim *s, double time_end, double strain_end);

/* One call of timeEvolutionDt (System.cpp:843-983) with calc_stress given;
 * performs the one-off "firsttime" set-up (System.cpp:1216-1226) first if
 * needed. */
int lfo_step(lfo_sim *s, int calc_stress, double time_end, double strain_end);

/* Only the first-time set-up of System::timeEvolution. */
void lfo_first_time(lfo_sim *s);

/* ---- restart from a dumped state (one-step parity tests) ---- */
/* Set the tangential spring and friction state of pair (p0,p1) (Contact.h
 * setState, :161-167).  Returns -1 if no such pair exists. */
int lfo_set_contact(lfo_sim *s, int p0, int p1, int state, const double *disp_tan);
int lfo_set_contact_rolling(lfo_sim *s, int p0, int p1, const double *disp_rolling);
/* Set the clocks and rate (System::clk, shear_rate, dt, max velocities) and
 * mark the first-time set-up of timeEvolution as done or not. */
void lfo_set_clock(lfo_sim *s, double time, double strain, double dt, double shear_rate,
                   double max_velocity, double max_sliding_velocity, int firsttime_done);
/* Recompute every pair's forces for the current positions without moving the
 * tangential springs (updateInteractions with dt = 0, as in
 * System.cpp:1216-1226). */
void lfo_refresh(lfo_sim *s);

void lfo_get_scalars(const lfo_sim *s, lfo_scalars *out);
/* positions, velocities, ang velocities, na velocities, na ang velocities:
 * each 3np, any pointer may be NULL. */
void lfo_get_particles(const lfo_sim *s, double *pos, double *vel, double *angvel,
                       double *na_vel, double *na_angvel);
int lfo_get_num_pairs(const lfo_sim *s);
void lfo_get_pairs(const lfo_sim *s, lfo_pair_out *out);
/* Per-particle stress by component: comp = 0 contact(GU), 1 dashpot(GU),
 * 2 hydro(GU), 3 repulsion(GU), 4 M_E_hydro, 5 xF_contact (rate) or
 * xF_contact_rateprop (stress), 6 xF_contact_rateindep (stress only),
 * 7 xF_repulsion.  out is 6np.  Returns 0 if the component exists. */
int lfo_get_particle_stress(const lfo_sim *s, int comp, double *out);
/* na velocity components, comp 0 contact 1 dashpot 2 hydro 3 repulsion;
 * out 6np (vx,vy,vz,ox,oy,oz per particle). */
int lfo_get_velocity_component(const lfo_sim *s, int comp, double *out);

/* ---- stage-level entry points used by the kernel parity tests ---- */

/* Assemble R_FU for the current interaction state (System.cpp:1429-1473).
 * Returns number of off-diagonal blocks nb.  If the output pointers are
 * non-NULL: dblocks (np x 15, MatrixBlocks.h DBlock order col0..col5),
 * odrow/odcol (nb, row particle > column particle), odblocks (nb x 18,
 * ODBlock order col0..col5). */
int lfo_assemble(lfo_sim *s, double *dblocks, int *odrow, int *odcol, double *odblocks);

/* Solve R_FU x = b for the matrix last assembled by lfo_assemble, k RHS of
 * length 6np each (particle-major, F then T). */
int lfo_solve_assembled(lfo_sim *s, int k, const double *b, double *x);

/* Force components for the current state (System.cpp:1727-1828):
 * comp 0 contact, 1 dashpot, 2 hydro, 3 repulsion; out 6np (F,T). */
int lfo_force_component(lfo_sim *s, int comp, double *out);

/* Sparse Cholesky stand-alone: lower BSR (diag + off-diag 6x6 dense blocks,
 * row-major within a block) -> solve.  Used to check solver parity on
 * arbitrary SPD block matrices. */
int lfo_bsr_solve(int nblk, const double *diag36, int nb, const int *row, const int *col,
                  const double *off36, int k, const double *b, double *x);

/* Number of host threads the oracle's factorisation uses (OpenMP). */
int lfo_num_threads(void);
void lfo_set_num_threads(int n);   /* OpenMP threads of later parallel regions */

/* Factorisation statistics for baseline reporting: out4 = {factorisations so
 * far, algorithmic flops of the last one (sum over block columns of
 * n^3/3 + n^2 m + n m^2 with n = 6, m = 6 x its off-diagonal blocks), wall
 * seconds spent in ordering + symbolic analysis, wall seconds in the numeric
 * factorisation}. */
void lfo_factor_stats(const lfo_sim *s, double *out4);

/* Dense kernels for the supernodal factorisation (the method of CHOLMOD's
 * supernodal factorisation, which the reference calls): LAPACK dpotrf and
 * BLAS dtrsm, dsyrk, dgemm with the Fortran calling convention (32-bit
 * integers), and optionally the BLAS library's thread-count setter and the
 * thread count to use for the large fronts.  Once set, every later
 * factorisation is supernodal; without them the block factorisation runs. */
void lfo_set_blas(void *potrf, void *trsm, void *syrk, void *gemm, void *set_threads, int threads);
int lfo_blas_ready(void);

/* A factor of an SPD block matrix on its own (6x6 blocks: diag36 n x 36
 * row-major, nb lower off-diagonal blocks (row > col) off36 row-major):
 * supernodal when the BLAS kernels are set, block otherwise; *status 0 or
 * the failing column + 1.  Solve: k right-hand sides of 6n. */
typedef struct lfo_factor lfo_factor;
lfo_factor *lfo_factor_create(int nblk, const double *diag36, int nb, const int *row, const int *col,
                              const double *off36, int *status);
void lfo_factor_solve(const lfo_factor *f, int k, const double *b, double *x);
void lfo_factor_free(lfo_factor *f);

/* Block (compact -> dense 6x6 row-major) reconstructions of
 * StokesSolver.cpp:154-231 (rows of the lower block, columns of the column
 * particle). */
void lfo_dblock_to_dense(const double *d15, double *m36);
void lfo_odblock_to_dense(const double *od18, double *m36);

#ifdef __cplusplus
}
#endif
#endif

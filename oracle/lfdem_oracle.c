/*
 * lfdem_oracle.c -- CPU restatement (plain C99, FP64) of LF_DEM's per-timestep
 * hydrodynamic core.  TEST INFRASTRUCTURE ONLY (see lfdem_oracle.h).
 *
 * Compiled with -ffp-contract=off so that every expression rounds the way
 * the reference's scalar C++ does.  Pair records are kept sorted by (p0,p1);
 * the reference keeps them in a swap-removed vector, so per-particle sums may
 * differ from it in the last bits (a 1e-16 relative effect).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "lfdem_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

int lfo_num_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

void lfo_set_num_threads(int n)
{
#ifdef _OPENMP
	if (n > 0) omp_set_num_threads(n);
#else
	(void)n;
#endif
}

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* small vector helpers (vec3d.h, Sym2Tensor.h)                        */
/* ------------------------------------------------------------------ */
typedef struct { double x, y, z; } v3;
static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x+b.x, a.y+b.y, a.z+b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x-b.x, a.y-b.y, a.z-b.z); }
static inline v3 vscale(double s, v3 a) { return V(s*a.x, s*a.y, s*a.z); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline double vdot(v3 a, v3 b) { return a.x*b.x+a.y*b.y+a.z*b.z; }
static inline double vsq(v3 a) { return a.x*a.x+a.y*a.y+a.z*a.z; }
/* vec3d.h:277-283 */
static inline v3 vcross(v3 a, v3 b) {
	return V(a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x);
}
static inline v3 vzero(void) { return V(0, 0, 0); }

typedef struct { double e[6]; } s2; /* (xx,xy,xz,yz,yy,zz) Sym2Tensor.h:28-31 */
static inline s2 szero(void) { s2 r; memset(&r, 0, sizeof r); return r; }
static inline void sadd_to(s2 *a, s2 b) { for (int i = 0; i < 6; i++) a->e[i] += b.e[i]; }
static inline s2 sscale(double c, s2 a) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = c*a.e[i]; return r; }
static inline s2 ssub(s2 a, s2 b) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = a.e[i]-b.e[i]; return r; }
static inline s2 saddv(s2 a, s2 b) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = a.e[i]+b.e[i]; return r; }
/* Sym2Tensor.h:256-264 */
static inline s2 outer_sym(v3 a, v3 b) {
	s2 r;
	r.e[0] = a.x*b.x;
	r.e[1] = 0.5*(a.x*b.y+a.y*b.x);
	r.e[2] = 0.5*(a.x*b.z+a.z*b.x);
	r.e[3] = 0.5*(a.y*b.z+a.z*b.y);
	r.e[4] = a.y*b.y;
	r.e[5] = a.z*b.z;
	return r;
}
/* Sym2Tensor.h:266-274 */
static inline s2 outer(v3 a) {
	s2 r;
	r.e[0] = a.x*a.x; r.e[1] = a.x*a.y; r.e[2] = a.x*a.z;
	r.e[3] = a.y*a.z; r.e[4] = a.y*a.y; r.e[5] = a.z*a.z;
	return r;
}
/* Sym2Tensor.h:227-234 */
static inline v3 sdot(const double *s, v3 v) {
	return V(s[0]*v.x + s[1]*v.y + s[2]*v.z,
	         s[1]*v.x + s[4]*v.y + s[3]*v.z,
	         s[2]*v.x + s[3]*v.y + s[5]*v.z);
}
/* Sym2Tensor.h:246-254 */
static inline double doubledot(const double *a, const double *b) {
	return a[0]*b[0] + 2*a[1]*b[1] + 2*a[2]*b[2] + 2*a[3]*b[3] + a[4]*b[4] + a[5]*b[5];
}

/* ------------------------------------------------------------------ */
/* lubrication scalar functions (LubricationFunctions.h:12-90)         */
/* ------------------------------------------------------------------ */
static double g1_XA(double l) { double p = l+1; return 2*l*l/(p*p*p); }
static double g2_YA(double l) { double p = l+1; return (4./15)*l*(2+l+2*l*l)/(p*p*p); }
static double g2_YB(double l) { double p = l+1; return -(1./5)*l*(4+l)/(p*p); }
static double g2_YC(double l) { return (2./5)*l/(l+1); }
static double g4_YC(double l) { double p = l+1; return (4./5)*l*l/(p*p*p*p); }
static double g1_XG(double l) { double p = l+1; return 3*l*l/(p*p*p); }
static double g2_YG(double l) { double p = l+1; return (1./10)*l*(4-l+7*l*l)/(p*p*p); }
static double g2_YH(double l) { double p = l+1; return (1./10)*l*(2-l)/(p*p); }
static double g5_YH(double l) { double p = l+1; return (1./20)*l*l*(1+7*l)/(p*p); }
static double g1_XM(double l) { double p = l+1; return (6./5)*l*l/(p*p*p); }
static double g4_XM(double l) { double p = l+1; return (6./5)*l*l*l/(p*p*p); }
static double g2_YM(double l) { double p = l+1; return (6./25)*l*(1-l+4*l*l)/(p*p*p); }
static double g5_YM(double l) { double p = l+1; return (3./50)*l*l*(7-10*l+7*l*l)/(p*p*p); }

enum { CXA = 0, CYA, CYB, CYC, CXG, CYG, CYH, CXM, CYM, NLUBC };

/* Lubrication::calcLubConstants, Lubrication.cpp:165-294 */
static void lub_constants(double a0, double a1, double c[NLUBC][4])
{
	double ro = a0+a1;
	double ro_12 = ro/2;
	double lambda = a1/a0;
	double invlambda = 1/lambda;
	double lambda_square = lambda*lambda;
	double lambda_cubic = lambda*lambda*lambda;
	double lambda_p_1 = 1+lambda;
	double lambda_p_1_square = lambda_p_1*lambda_p_1;
	double lambda_p_1_cubic = lambda_p_1_square*lambda_p_1;
	double a0a0_23 = a0*a0*(2.0/3);
	double a1a1_23 = a1*a1*(2.0/3);
	double roro_16 = ro*ro*(1.0/6);
	double a0a0a0 = a0*a0*a0;
	double a1a1a1 = a1*a1*a1;
	double rororo = ro*ro*ro;
	double a0a0a0_43 = a0a0a0*(4.0/3);
	double a1a1a1_43 = a1a1a1*(4.0/3);
	double rororo_16 = rororo*(1.0/6);
	double a0a0a0_109 = a0a0a0*(10.0/9);
	double a1a1a1_109 = a1a1a1*(10.0/9);
	double rororo_536 = rororo*(5.0/36);
	double g;
	g = g1_XA(lambda);
	c[CXA][0] = a0*g;
	c[CXA][1] = ro_12*(-2/lambda_p_1)*g;
	c[CXA][2] = c[CXA][1];
	c[CXA][3] = a1*g1_XA(invlambda);
	g = g2_YA(lambda);
	c[CYA][0] = a0*g;
	c[CYA][1] = ro_12*(-2/lambda_p_1)*g;
	c[CYA][2] = c[CYA][1];
	c[CYA][3] = a1*g2_YA(invlambda);
	g = g2_YB(lambda);
	c[CYB][0] = a0a0_23*g;
	c[CYB][1] = roro_16*(-4/lambda_p_1_square)*g;
	c[CYB][2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YB(invlambda);
	c[CYB][3] = -a1a1_23*g2_YB(invlambda);
	c[CYC][0] = a0a0a0_43*g2_YC(lambda);
	c[CYC][1] = rororo_16*g4_YC(lambda);
	c[CYC][2] = c[CYC][1];
	c[CYC][3] = a1a1a1_43*g2_YC(invlambda);
	g = g1_XG(lambda);
	c[CXG][0] = a0a0_23*g;
	c[CXG][1] = roro_16*(-4/lambda_p_1_square)*g;
	c[CXG][2] = roro_16*(4*lambda_square/lambda_p_1_square)*g1_XG(invlambda);
	c[CXG][3] = -a1a1_23*g1_XG(invlambda);
	g = g2_YG(lambda);
	c[CYG][0] = a0a0_23*g;
	c[CYG][1] = roro_16*(-4/lambda_p_1_square)*g;
	c[CYG][2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YG(invlambda);
	c[CYG][3] = -a1a1_23*g2_YG(invlambda);
	c[CYH][0] = a0a0a0_43*g2_YH(lambda);
	c[CYH][1] = rororo_16*(8/lambda_p_1_cubic)*g5_YH(lambda);
	c[CYH][2] = rororo_16*(8*lambda_cubic/lambda_p_1_cubic)*g5_YH(invlambda);
	c[CYH][3] = a1a1a1_43*g2_YH(invlambda);
	c[CXM][0] = a0a0a0_109*g1_XM(lambda);
	c[CXM][1] = rororo_536*(8/lambda_p_1_cubic)*g4_XM(lambda);
	c[CXM][2] = c[CXM][1];
	c[CXM][3] = a1a1a1_109*g1_XM(invlambda);
	c[CYM][0] = a0a0a0_109*g2_YM(lambda);
	c[CYM][1] = rororo_536*(8/lambda_p_1_cubic)*g5_YM(lambda);
	c[CYM][2] = c[CYM][1];
	c[CYM][3] = a1a1a1_109*g2_YM(invlambda);
}

/* ------------------------------------------------------------------ */
/* data structures                                                     */
/* ------------------------------------------------------------------ */
typedef struct {
	int p0, p1;
	double a0, a1, ro;
	double range;        /* interaction range (Interaction.cpp:13-36) */
	double lub_range;    /* Lubrication::range (Lubrication.cpp:121) */
	v3 rvec, nvec;
	double r, gap;       /* gap = reduced gap 2r/ro-2 */
	int z_offset;
	/* contact (Contact.h) */
	int c_active, state;
	double kn_s, kt_s, mu_s, mu_d;
	v3 disp_tan, prev_disp_tan;
	double kr_s, mu_r;                 /* rolling friction (Contact.cpp:35-45, 60-67) */
	v3 disp_roll, prev_disp_roll, f_roll;
	double fsn_norm, normal_load;
	v3 fs_normal, fs_tan, fs_total;
	double rsv_sq;
	/* dashpot (ContactDashpot.h) */
	int dp_active;
	double dXA[4], dYA[4], dYB[4], dYC[4], dp_tan_coeff;
	/* lubrication */
	int lub_active;
	double lub_coeff, log_lub_coeff;
	double lc[NLUBC][4];
	/* repulsion */
	double rep_geo, rep_reduced, rep_norm;
	v3 rep_force;
	int dead;
} opair;

enum { FC_CONTACT = 0, FC_DASHPOT, FC_HYDRO, FC_REPULSION, NFC };
/* stress component slots, listed in std::map key order (Stress.cpp:16-75):
 * "M_E_hydro" < "contact" < "dashpot" < "hydro" < "repulsion" <
 * "xF_contact" / "xF_contact_rateindep" < "xF_contact_rateprop" < "xF_repulsion" */
enum { SC_ME = 0, SC_GU_CONTACT, SC_GU_DASHPOT, SC_GU_HYDRO, SC_GU_REPULSION,
       SC_XF_CONTACT, SC_XF_RATEINDEP, SC_XF_RATEPROP, SC_XF_REPULSION, NSC };
enum { RATE_INDEP = 0, RATE_PROP, RATE_DEP };

struct lfo_sim {
	lfo_params p;
	int np, twodim;
	double lx, ly, lz, lx_half, ly_half, lz_half;
	double system_volume;
	int friction, rolling, lubrication, tangential, repulsiveforce, pairwise_resistance;
	int has_fc[NFC], fc_torque[NFC], fc_rate[NFC];
	int has_sc[NSC], sc_rate[NSC], sc_group[NSC];
	v3 *pos, *vel, *ang, *na_vel, *na_ang, *vel_pred, *ang_pred, *u_inf;
	double *radius;
	v3 shear_disp, vel_difference, shear_strain;
	double Einf[6], Omega[3], shear_rate;
	double dt, time, strain, time_sim;
	double max_velocity, max_sliding_velocity;
	long long total_num_timesteps;
	int in_predictor, in_corrector, firsttime;
	/* pairs */
	opair *pairs; int npairs, cap;
	/* per-component data */
	double *fc_force[NFC]; /* 6np each (F,T interleaved per particle) */
	double *vc[NFC];       /* 6np each: na velocity components */
	s2 *sc[NSC];           /* np each */
	/* assembled matrix */
	double *dblocks; /* np x 18 */
	int nod; int *odrow, *odcol; double *odblocks; int odcap;
	/* solver */
	void *fact;
	double rate_prop_shearstress, rate_indep_shearstress;
	/* factorisation statistics (baseline reporting): count, ordering flops
	 * of the last one, wall seconds of analysis and numeric phases */
	long long n_factor; double last_factor_flops, analyze_s, factor_s;
};

/* ------------------------------------------------------------------ */
/* periodic boundaries (System.cpp:2478-2548)                          */
/* ------------------------------------------------------------------ */
static int periodize(lfo_sim *s, v3 *pos)
{
	int z_shift = 0;
	if (pos->z >= s->lz) {
		pos->z -= s->lz;
		*pos = vsub(*pos, s->shear_disp);
		z_shift = -1;
	} else if (pos->z < 0) {
		pos->z += s->lz;
		*pos = vadd(*pos, s->shear_disp);
		z_shift = 1;
	}
	while (pos->x >= s->lx) pos->x -= s->lx;
	while (pos->x < 0) pos->x += s->lx;
	if (!s->twodim) {
		if (pos->y >= s->ly) pos->y -= s->ly;
		else if (pos->y < 0) pos->y += s->ly;
	}
	return z_shift;
}

static int periodize_diff(const lfo_sim *s, v3 *d)
{
	int zshift = 0;
	if (d->z > s->lz_half) {
		d->z -= s->lz;
		*d = vsub(*d, s->shear_disp);
		zshift = -1;
	} else if (d->z < -s->lz_half) {
		d->z += s->lz;
		*d = vadd(*d, s->shear_disp);
		zshift = 1;
	}
	while (d->x > s->lx_half) d->x -= s->lx;
	while (d->x < -s->lx_half) d->x += s->lx;
	if (!s->twodim) {
		if (d->y > s->ly_half) d->y -= s->ly;
		else if (d->y < -s->ly_half) d->y += s->ly;
	}
	return zshift;
}

/* System::calcLubricationRange, System.cpp:2665-2674 */
static double lub_range(const lfo_sim *s, int i, int j)
{
	double ri = s->radius[i], rj = s->radius[j];
	double rad_ratio = ri/rj;
	if (rad_ratio < 2 && rad_ratio > 0.5) {
		return (2+s->p.lub_max_gap)*0.5*(ri+rj);
	} else {
		double minradius = (ri < rj ? ri : rj);
		return ri+rj+s->p.lub_max_gap*minradius;
	}
}
/* System::calcInteractionRangeDefault, System.cpp:2660-2663 */
static double interaction_range(const lfo_sim *s, int i, int j)
{
	if (s->p.interaction_range == -1 || s->p.interaction_range < 0)
		return lub_range(s, i, j);
	return s->p.interaction_range*0.5*(s->radius[i]+s->radius[j]);
}

/* ------------------------------------------------------------------ */
/* set-up                                                              */
/* ------------------------------------------------------------------ */
static void set_shear_rate(lfo_sim *s, double rate)
{
	/* System::set_shear_rate, System.cpp:1972-1982; setVelocityDifference :1967-1970 */
	s->shear_rate = rate;
	for (int k = 0; k < 3; k++) s->Omega[k] = s->p.Ohat[k]*rate;
	for (int k = 0; k < 6; k++) s->Einf[k] = s->p.Ehat[k]*rate;
	s->vel_difference = vscale(2, sdot(s->Einf, V(0, 0, s->lz)));
}

static void declare_components(lfo_sim *s)
{
	/* System::declareForceComponents, System.cpp:169-215 */
	memset(s->has_fc, 0, sizeof s->has_fc);
	s->has_fc[FC_CONTACT] = 1; s->fc_torque[FC_CONTACT] = s->friction; s->fc_rate[FC_CONTACT] = RATE_INDEP;
	if (s->lubrication) {
		/* "hydro" exists for normal/tangential models */
		s->has_fc[FC_HYDRO] = 1; s->fc_torque[FC_HYDRO] = s->tangential; s->fc_rate[FC_HYDRO] = RATE_PROP;
	}
	s->has_fc[FC_DASHPOT] = 1; s->fc_torque[FC_DASHPOT] = 1; s->fc_rate[FC_DASHPOT] = RATE_PROP;
	if (s->repulsiveforce) {
		s->has_fc[FC_REPULSION] = 1; s->fc_torque[FC_REPULSION] = 0; s->fc_rate[FC_REPULSION] = RATE_INDEP;
	}
	/* System::declareStressComponents, Stress.cpp:16-75 */
	memset(s->has_sc, 0, sizeof s->has_sc);
	if (s->lubrication) {
		s->has_sc[SC_GU_CONTACT] = 1; s->sc_rate[SC_GU_CONTACT] = RATE_INDEP; s->sc_group[SC_GU_CONTACT] = 0;
		s->has_sc[SC_GU_DASHPOT] = 1; s->sc_rate[SC_GU_DASHPOT] = RATE_PROP; s->sc_group[SC_GU_DASHPOT] = 1;
		s->has_sc[SC_GU_HYDRO] = 1; s->sc_rate[SC_GU_HYDRO] = RATE_PROP; s->sc_group[SC_GU_HYDRO] = 2;
		if (s->repulsiveforce) {
			s->has_sc[SC_GU_REPULSION] = 1; s->sc_rate[SC_GU_REPULSION] = RATE_INDEP; s->sc_group[SC_GU_REPULSION] = 3;
		}
		s->has_sc[SC_ME] = 1; s->sc_rate[SC_ME] = RATE_PROP; s->sc_group[SC_ME] = 2;
	}
	if (s->p.control == 0) {
		s->has_sc[SC_XF_CONTACT] = 1; s->sc_rate[SC_XF_CONTACT] = RATE_DEP; s->sc_group[SC_XF_CONTACT] = 0;
	} else {
		s->has_sc[SC_XF_RATEPROP] = 1; s->sc_rate[SC_XF_RATEPROP] = RATE_PROP; s->sc_group[SC_XF_RATEPROP] = 0;
		s->has_sc[SC_XF_RATEINDEP] = 1; s->sc_rate[SC_XF_RATEINDEP] = RATE_INDEP; s->sc_group[SC_XF_RATEINDEP] = 0;
	}
	if (s->repulsiveforce) {
		s->has_sc[SC_XF_REPULSION] = 1; s->sc_rate[SC_XF_REPULSION] = RATE_INDEP; s->sc_group[SC_XF_REPULSION] = 3;
	}
}

/* ------------------------------------------------------------------ */
/* pair (Interaction) life cycle                                       */
/* ------------------------------------------------------------------ */
/* Interaction::calcNormalVectorDistanceGap, Interaction.cpp:124-135 */
static void pair_geometry(lfo_sim *s, opair *q)
{
	q->rvec = vsub(s->pos[q->p1], s->pos[q->p0]);
	q->z_offset = periodize_diff(s, &q->rvec);
	q->r = sqrt(vsq(q->rvec));
	q->nvec = V(q->rvec.x/q->r, q->rvec.y/q->r, q->rvec.z/q->r);
	q->gap = 2*q->r/q->ro-2;
}

/* ContactDashpot::setDashpotResistanceCoeffs + calcDashpotResistances,
 * ContactDashpot.cpp:65-183 */
static int dashpot_coeffs(lfo_sim *s, opair *q)
{
	double kn = s->p.kn, kt = s->p.kt;
	double rn = s->p.contact_relaxation_time, rt = s->p.contact_relaxation_time_tan;
	double normal_coeff, tangential_coeff;
	if (rn > 0) {
		normal_coeff = 4*kn*rn;
	} else {
		if (s->lubrication) normal_coeff = 1/s->p.lub_reduce_parameter;
		else return -1;
	}
	if (!s->friction && !s->tangential) {
		tangential_coeff = 0;
	} else {
		if (rt > 0) {
			if (s->lubrication) return -1;
			tangential_coeff = 6*kt*rt;
		} else {
			if (s->lubrication) {
				if (s->p.lub_reduce_parameter < 1) tangential_coeff = log(1/s->p.lub_reduce_parameter);
				else tangential_coeff = 0;
			} else return -1;
		}
	}
	q->dp_tan_coeff = tangential_coeff;
	double a0 = q->a0, a1 = q->a1, ro = q->ro, ro_12 = ro/2;
	double lambda = a1/a0;
	double invlambda = 1/lambda;
	double lambda_square = lambda*lambda;
	double lambda_p_1 = 1+lambda;
	double lambda_p_1_square = lambda_p_1*lambda_p_1;
	double a0a0_23 = a0*a0*(2.0/3);
	double a1a1_23 = a1*a1*(2.0/3);
	double roro_16 = ro*ro*(1.0/6);
	double a0a0a0_43 = a0*a0*a0*(4.0/3);
	double a1a1a1_43 = a1*a1*a1*(4.0/3);
	double rororo_16 = ro*ro*ro*(1.0/6);
	q->dXA[0] = a0*g1_XA(lambda);
	q->dXA[1] = ro_12*(-2/lambda_p_1)*g1_XA(lambda);
	q->dXA[2] = ro_12*q->dXA[1];
	q->dXA[3] = a1*g1_XA(invlambda);
	for (int j = 0; j < 4; j++) q->dXA[j] *= normal_coeff;
	for (int j = 0; j < 4; j++) q->dYA[j] = q->dYB[j] = q->dYC[j] = 0;
	if (tangential_coeff == 0) return 0;
	q->dYA[0] = a0*g2_YA(lambda);
	q->dYA[1] = ro_12*(-2/lambda_p_1)*g2_YA(lambda);
	q->dYA[2] = ro_12*q->dYA[1];
	q->dYA[3] = a1*g2_YA(invlambda);
	for (int j = 0; j < 4; j++) q->dYA[j] *= tangential_coeff;
	q->dYB[0] = a0a0_23*g2_YB(lambda);
	q->dYB[1] = roro_16*(-4/lambda_p_1_square)*g2_YB(lambda);
	q->dYB[2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YB(invlambda);
	q->dYB[3] = -a1a1_23*g2_YB(invlambda);
	for (int j = 0; j < 4; j++) q->dYB[j] *= tangential_coeff;
	q->dYC[0] = a0a0a0_43*g2_YC(lambda);
	q->dYC[1] = rororo_16*g4_YC(lambda);
	q->dYC[2] = rororo_16*q->dYC[1];
	q->dYC[3] = a1a1a1_43*g2_YC(invlambda);
	for (int j = 0; j < 4; j++) q->dYC[j] *= tangential_coeff;
	return 0;
}

/* Contact::activate, Contact.cpp:73-96 */
static void contact_activate(lfo_sim *s, opair *q)
{
	q->c_active = 1;
	q->fsn_norm = 0;
	q->fs_normal = vzero();
	q->normal_load = 0;
	q->fs_total = vzero();
	if (s->friction) {
		if (s->p.friction_model == 2 || s->p.friction_model == 3) q->state = 1;
		else q->state = 2;
		q->disp_tan = vzero();
		q->prev_disp_tan = vzero();
		q->disp_roll = vzero();
		q->prev_disp_roll = vzero();
		q->f_roll = vzero();
	} else {
		q->state = 1;
	}
	q->dp_active = 1;
}

/* Contact::deactivate, Contact.cpp:98-112 */
static void contact_deactivate(lfo_sim *s, opair *q)
{
	q->state = 0;
	q->c_active = 0;
	q->fsn_norm = 0;
	q->fs_normal = vzero();
	q->fs_total = vzero();
	if (s->friction) {
		q->disp_tan = vzero();
		q->disp_roll = vzero();
		q->fs_tan = vzero();
	}
	q->dp_active = 0;
}

/* Lubrication::updateResistanceCoeff, Lubrication.cpp:696-706 */
static void lub_update_coeff(lfo_sim *s, opair *q)
{
	if (q->gap > 0) {
		double coeff = 1/(q->gap+s->p.lub_reduce_parameter);
		q->lub_coeff = coeff;
		q->log_lub_coeff = coeff > 1. ? log(coeff) : 0.;
	}
}

/* Lubrication::updateActivationState, Lubrication.cpp:137-146 */
static void lub_update_activation(opair *q)
{
	int in_range = q->r < q->lub_range && q->r > q->ro;
	if (!q->lub_active && in_range) q->lub_active = 1;
	if (q->lub_active && !in_range) q->lub_active = 0;
}

/* Interaction ctor + activateForceMembers, Interaction.cpp:13-36, 137-156,
 * Contact::setInteractionData Contact.cpp:47-71, RepulsiveForce::activate
 * RepulsiveForce.cpp:23-40 */
static int pair_create(lfo_sim *s, opair *q, int i, int j, double range)
{
	memset(q, 0, sizeof *q);
	if (j > i) { q->p0 = i; q->p1 = j; } else { q->p0 = j; q->p1 = i; }
	q->a0 = s->radius[q->p0];
	q->a1 = s->radius[q->p1];
	q->ro = q->a0+q->a1;
	q->range = range;
	if (s->repulsiveforce) {
		q->rep_geo = q->a0*q->a1/(q->a0+q->a1);
		q->rep_force = vzero(); q->rep_norm = 0; q->rep_reduced = 0;
	}
	pair_geometry(s, q);
	/* Contact::setInteractionData */
	double ro_12 = (q->a0+q->a1)/2;
	q->kn_s = ro_12*ro_12*s->p.kn;
	if (s->friction) {
		q->kt_s = ro_12*s->p.kt;
		q->mu_s = s->p.mu_static;
		q->mu_d = s->p.mu_dynamic;
		if (s->rolling) {
			q->kr_s = ro_12*s->p.kr;
			q->mu_r = s->p.mu_rolling;
		}
	}
	if (dashpot_coeffs(s, q)) return -1;
	if (q->gap <= 0) contact_activate(s, q);
	if (s->lubrication) {
		lub_constants(q->a0, q->a1, q->lc);
		q->lub_range = lub_range(s, q->p0, q->p1);
		lub_update_activation(q);
		if (q->lub_active) lub_update_coeff(s, q);
	}
	return 0;
}

static inline void set_tan_norm(opair *q, double current, double target)
{
	/* Contact::setTangentialForceNorm, Contact.cpp:293-299 */
	q->disp_tan = vscale(target/current, q->disp_tan);
	q->fs_tan = vscale(q->kt_s, q->disp_tan);
}

/* friction laws, Contact.cpp:235-408 */
static void friction_law(lfo_sim *s, opair *q)
{
	int fm = s->p.friction_model;
	if (fm == 1) {
		double supportable = 0;
		double sq_f_tan = vsq(q->fs_tan);
		q->normal_load = q->fsn_norm;
		if (q->state == 2) supportable = q->mu_s*q->normal_load;
		else supportable = q->mu_d*q->normal_load;
		if (sq_f_tan > supportable*supportable) {
			q->state = 3;
			supportable = q->mu_d*q->normal_load;
		} else {
			q->state = 2;
		}
		if (q->state == 3) set_tan_norm(q, sqrt(sq_f_tan), supportable);
		if (s->rolling) {
			/* Contact::setRollingForceNorm, Contact.cpp:283-305 */
			double sup_r = q->mu_r*q->normal_load;
			double sq_f_roll = vsq(q->f_roll);
			if (sq_f_roll > sup_r*sup_r) {
				q->disp_roll = vscale(sup_r/sqrt(sq_f_roll), q->disp_roll);
				q->f_roll = vscale(q->kr_s, q->disp_roll);
			}
		}
	} else if (fm == 2) {
		double supportable = q->fsn_norm-s->p.critical_load;
		if (supportable < 0) {
			q->state = 1;
			q->disp_tan = vzero();
			q->fs_tan = vzero();
		} else {
			supportable *= q->mu_s;
			double sq_f_tan = vsq(q->fs_tan);
			if (sq_f_tan > supportable*supportable) {
				q->state = 3;
				set_tan_norm(q, sqrt(sq_f_tan), supportable);
			} else {
				q->state = 2;
			}
		}
	} else if (fm == 3) {
		double supportable = q->fsn_norm-s->p.critical_load;
		if (supportable < 0) {
			q->state = 1;
			q->disp_tan = vzero();
			q->fs_tan = vzero();
		} else {
			q->state = 2;
		}
	} else if (fm == 5) {
		double sq_f_tan = vsq(q->fs_tan);
		if (sq_f_tan > s->p.ft_max*s->p.ft_max) {
			q->state = 3;
			set_tan_norm(q, sqrt(sq_f_tan), s->p.ft_max);
		} else {
			q->state = 2;
		}
	} else if (fm == 6) {
		double supportable = 0;
		q->normal_load = q->fsn_norm;
		if (q->state == 2) supportable = q->mu_s*q->normal_load;
		else supportable = q->mu_d*q->normal_load;
		if (supportable > s->p.ft_max) supportable = s->p.ft_max;
		double sq_f_tan = vsq(q->fs_tan);
		if (sq_f_tan > supportable*supportable) {
			q->state = 3;
			set_tan_norm(q, sqrt(sq_f_tan), supportable);
		} else {
			q->state = 2;
		}
	}
}

/* Contact::calcContactSpringForce, Contact.cpp:200-233 */
static void contact_spring(lfo_sim *s, opair *q)
{
	if (!q->c_active) return;
	q->fsn_norm = -q->kn_s*q->gap;
	q->fs_normal = vscale(-q->fsn_norm, q->nvec);
	if (s->friction) {
		q->disp_tan = vsub(q->disp_tan, vscale(vdot(q->disp_tan, q->nvec), q->nvec));
		q->fs_tan = vscale(q->kt_s, q->disp_tan);
		if (s->rolling) q->f_roll = vscale(q->kr_s, q->disp_roll);
		friction_law(s, q);
	}
	if (q->state <= 1) q->fs_total = q->fs_normal;
	else q->fs_total = vadd(q->fs_normal, q->fs_tan);
}

/* Contact::incrementTangentialDisplacement, Contact.cpp:125-160 */
static void contact_increment(lfo_sim *s, opair *q)
{
	if (!s->friction) return;
	v3 vel_offset = vscale((double)q->z_offset, s->vel_difference);
	v3 tdv = vadd(vsub(s->vel[q->p1], s->vel[q->p0]), vel_offset);
	v3 rdv = vneg(vcross(vadd(vscale(q->a0, s->ang[q->p0]), vscale(q->a1, s->ang[q->p1])), q->nvec));
	v3 rsv = vadd(tdv, rdv);
	rsv = vsub(rsv, vscale(vdot(rsv, q->nvec), q->nvec));
	q->rsv_sq = vsq(rsv);
	if (s->in_predictor) q->prev_disp_tan = q->disp_tan;
	q->disp_tan = vadd(q->prev_disp_tan, vscale(s->dt, rsv));
	if (s->rolling) {
		/* Contact::calcRollingVelocities + incrementRollingDisplacement, Contact.cpp:162-180 */
		double a_red = q->a0*q->a1/(q->a0+q->a1);
		v3 rv = vscale(2*a_red, vcross(vsub(s->ang[q->p1], s->ang[q->p0]), q->nvec));
		if (s->in_predictor) q->prev_disp_roll = q->disp_roll;
		q->disp_roll = vadd(q->prev_disp_roll, vscale(s->dt, rv));
	}
}

/* RepulsiveForce::calcReducedForceNorm + calcScaledForce,
 * RepulsiveForce.cpp:42-95 */
static void repulsion_force(lfo_sim *s, opair *q)
{
	double gap = q->r-q->ro;
	if (gap > 0) {
		if (s->p.repulsive_max_length == -1) {
			q->rep_reduced = exp(-gap/s->p.repulsive_length);
		} else {
			q->rep_reduced = exp(-gap/s->p.repulsive_length)*0.5*(1+tanh(-(gap-s->p.repulsive_max_length)/1e-3));
		}
		q->rep_reduced *= q->rep_geo;
	} else {
		q->rep_reduced = q->rep_geo;
	}
	q->rep_norm = s->p.repulsion*q->rep_reduced;
	q->rep_force = vscale(-q->rep_norm, q->nvec);
}

/* Interaction::updateState + updateContactState, Interaction.cpp:171-236 */
static void pair_update(lfo_sim *s, opair *q, int *deactivated)
{
	if (q->c_active) contact_increment(s, q);
	pair_geometry(s, q);
	if (q->r > q->range) {
		if (q->c_active) contact_deactivate(s, q);
		if (s->lubrication && q->lub_active) q->lub_active = 0;
		*deactivated = 1;
		return;
	}
	if (q->c_active) {
		if (q->gap > 0) contact_deactivate(s, q);
	} else {
		if (q->gap <= 0) contact_activate(s, q);
	}
	if (q->c_active) contact_spring(s, q);
	if (s->lubrication) {
		lub_update_activation(q);
		if (q->lub_active) lub_update_coeff(s, q);
	}
	if (s->repulsiveforce) repulsion_force(s, q);
}

static int pair_cmp(const void *a, const void *b)
{
	const opair *x = a, *y = b;
	if (x->p0 != y->p0) return x->p0 < y->p0 ? -1 : 1;
	if (x->p1 != y->p1) return x->p1 < y->p1 ? -1 : 1;
	return 0;
}

static int find_pair(const lfo_sim *s, int i, int j)
{
	int lo = 0, hi = s->npairs-1;
	while (lo <= hi) {
		int m = (lo+hi)/2;
		const opair *q = &s->pairs[m];
		if (q->p0 == i && q->p1 == j) return m;
		if (q->p0 < i || (q->p0 == i && q->p1 < j)) lo = m+1; else hi = m-1;
	}
	return -1;
}

/* System::checkNewInteraction, System.cpp:1328-1373 (all-pairs search; the
 * reference's Lees-Edwards cell list returns a superset of the pairs within
 * range, so the created set is the same). */
static int check_new_interaction(lfo_sim *s)
{
	int n = s->np;
	int added = 0;
	int base = s->npairs;
	for (int i = 0; i < n-1; i++) {
		for (int j = i+1; j < n; j++) {
			v3 d = vsub(s->pos[j], s->pos[i]);
			periodize_diff(s, &d);
			double sq_dist = vsq(d);
			double range = interaction_range(s, i, j);
			double lim = range*range;
			if (sq_dist < lim) {
				if (find_pair(s, i, j) >= 0) continue;
				if (s->npairs == s->cap) {
					s->cap = s->cap ? 2*s->cap : 1024;
					s->pairs = realloc(s->pairs, sizeof(opair)*s->cap);
				}
				if (pair_create(s, &s->pairs[s->npairs], i, j, range)) return -1;
				s->npairs++;
				added++;
			}
		}
	}
	(void)base;
	if (added) qsort(s->pairs, s->npairs, sizeof(opair), pair_cmp);
	return 0;
}

/* System::updateInteractions, System.cpp:1375-1403 */
static void update_interactions(lfo_sim *s)
{
	double sq_max = 0;
	int removed = 0;
	for (int k = 0; k < s->npairs; k++) {
		opair *q = &s->pairs[k];
		int deact = 0;
		pair_update(s, q, &deact);
		if (s->friction && q->c_active) {
			if (q->rsv_sq > sq_max) sq_max = q->rsv_sq;
		}
		if (deact) { q->dead = 1; removed++; }
	}
	if (removed) {
		int w = 0;
		for (int k = 0; k < s->npairs; k++) if (!s->pairs[k].dead) s->pairs[w++] = s->pairs[k];
		s->npairs = w;
	}
	s->max_sliding_velocity = sqrt(sq_max);
}

/* ------------------------------------------------------------------ */
/* resistance blocks                                                   */
/* ------------------------------------------------------------------ */
/* 18 DBlock entries: col0[5] col1[3] col2[1] col3[3] col4[2] col5[1]
 * 18 ODBlock entries: col0[5] col1[3] col2[1] col3[5] col4[3] col5[1]
 * (MatrixBlocks.h:5-122) */
static void lub_blocks(const lfo_sim *s, const opair *q, double *od, double *b0, double *b1)
{
	double XA[4], YA[4], YB[4], YC[4];
	for (int j = 0; j < 4; j++) {
		XA[j] = q->lc[CXA][j]*q->lub_coeff;
		YA[j] = q->lc[CYA][j]*q->log_lub_coeff;
		YB[j] = q->lc[CYB][j]*q->log_lub_coeff;
		YC[j] = q->lc[CYC][j]*q->log_lub_coeff;
	}
	double nx = q->nvec.x, ny = q->nvec.y, nz = q->nvec.z;
	if (!s->tangential) {
		/* Lubrication::RFU_ODBlock_squeeze / RFU_DBlocks_squeeze, Lubrication.cpp:406-517 */
		memset(od, 0, 18*sizeof(double));
		od[0] = XA[1]*nx*nx; od[1] = XA[1]*nx*ny; od[2] = XA[1]*nx*nz;
		od[5] = XA[1]*ny*ny; od[6] = XA[1]*ny*nz;
		od[8] = XA[1]*nz*nz;
		memset(b0, 0, 15*sizeof(double)); memset(b1, 0, 15*sizeof(double));
		b0[0] = XA[0]*nx*nx; b0[1] = XA[0]*nx*ny; b0[2] = XA[0]*nx*nz;
		b0[5] = XA[0]*ny*ny; b0[6] = XA[0]*ny*nz; b0[8] = XA[0]*nz*nz;
		b1[0] = XA[3]*nx*nx; b1[1] = XA[3]*nx*ny; b1[2] = XA[3]*nx*nz;
		b1[5] = XA[3]*ny*ny; b1[6] = XA[3]*ny*nz; b1[8] = XA[3]*nz*nz;
		return;
	}
	/* Lubrication::RFU_ODBlock_squeeze_tangential, Lubrication.cpp:437-467 */
	double XA1_YA1 = XA[1]-YA[1];
	od[0] = YA[1] + XA1_YA1*nx*nx;
	od[1] = XA1_YA1*nx*ny;
	od[2] = XA1_YA1*nx*nz;
	od[3] = -YB[2]*nz;
	od[4] = YB[2]*ny;
	od[5] = YA[1] + XA1_YA1*ny*ny;
	od[6] = XA1_YA1*ny*nz;
	od[7] = -YB[2]*nx;
	od[8] = YA[1] + XA1_YA1*nz*nz;
	od[9] = YB[1]*nz;
	od[10] = -YB[1]*ny;
	od[11] = YC[1]*(1-nx*nx);
	od[12] = -YC[1]*nx*ny;
	od[13] = -YC[1]*nx*nz;
	od[14] = YB[1]*nx;
	od[15] = YC[1]*(1-ny*ny);
	od[16] = -YC[1]*ny*nz;
	od[17] = YC[1]*(1-nz*nz);
	/* Lubrication::RFU_DBlocks_squeeze_tangential, Lubrication.cpp:520-580 */
	double n0n0 = nx*nx, n0n1 = nx*ny, n0n2 = nx*nz, n1n1 = ny*ny, n1n2 = ny*nz, n2n2 = nz*nz;
	double one_n0n0 = 1-n0n0, one_n1n1 = 1-n1n1, one_n2n2 = 1-n2n2;
	double XA0mYA0 = XA[0]-YA[0];
	b0[0] = XA[0]*n0n0+YA[0]*one_n0n0;
	b0[1] = XA0mYA0*n0n1;
	b0[2] = XA0mYA0*n0n2;
	b0[3] = -YB[0]*nz;
	b0[4] = YB[0]*ny;
	b0[5] = XA[0]*n1n1+YA[0]*one_n1n1;
	b0[6] = XA0mYA0*n1n2;
	b0[7] = -YB[0]*nx;
	b0[8] = XA[0]*n2n2+YA[0]*one_n2n2;
	b0[9] = YC[0]*one_n0n0;
	b0[10] = -YC[0]*n0n1;
	b0[11] = -YC[0]*n0n2;
	b0[12] = YC[0]*one_n1n1;
	b0[13] = -YC[0]*n1n2;
	b0[14] = YC[0]*one_n2n2;
	double XA3mYA3 = XA[3]-YA[3];
	b1[0] = XA[3]*n0n0+YA[3]*one_n0n0;
	b1[1] = XA3mYA3*n0n1;
	b1[2] = XA3mYA3*n0n2;
	b1[3] = -YB[3]*nz;
	b1[4] = YB[3]*ny;
	b1[5] = XA[3]*n1n1+YA[3]*one_n1n1;
	b1[6] = XA3mYA3*n1n2;
	b1[7] = -YB[3]*nx;
	b1[8] = XA[3]*n2n2+YA[3]*one_n2n2;
	b1[9] = YC[3]*one_n0n0;
	b1[10] = -YC[3]*n0n1;
	b1[11] = -YC[3]*n0n2;
	b1[12] = YC[3]*one_n1n1;
	b1[13] = -YC[3]*n1n2;
	b1[14] = YC[3]*one_n2n2;
}

/* ContactDashpot::RFU_ODBlock / RFU_DBlocks, ContactDashpot.cpp:186-340 */
static void dashpot_blocks(const opair *q, double *od, double *b0, double *b1)
{
	const double *XA = q->dXA, *YA = q->dYA, *YB = q->dYB, *YC = q->dYC;
	double nx = q->nvec.x, ny = q->nvec.y, nz = q->nvec.z;
	if (q->dp_tan_coeff > 0) {
		double XA1_YA1 = XA[1]-YA[1];
		od[0] = YA[1] + XA1_YA1*nx*nx;
		od[1] = XA1_YA1*nx*ny;
		od[2] = XA1_YA1*nx*nz;
		od[3] = -YB[2]*nz;
		od[4] = YB[2]*ny;
		od[5] = YA[1] + XA1_YA1*ny*ny;
		od[6] = XA1_YA1*ny*nz;
		od[7] = -YB[2]*nx;
		od[8] = YA[1] + XA1_YA1*nz*nz;
		od[9] = YB[1]*nz;
		od[10] = -YB[1]*ny;
		od[11] = YC[1]*(1-nx*nx);
		od[12] = -YC[1]*nx*ny;
		od[13] = -YC[1]*nx*nz;
		od[14] = YB[1]*nx;
		od[15] = YC[1]*(1-ny*ny);
		od[16] = -YC[1]*ny*nz;
		od[17] = YC[1]*(1-nz*nz);
		double XA0_YA0 = XA[0] - YA[0];
		b0[0] = YA[0] + XA0_YA0*nx*nx;
		b0[1] = XA0_YA0*nx*ny;
		b0[2] = XA0_YA0*nx*nz;
		b0[3] = -YB[0]*nz;
		b0[4] = YB[0]*ny;
		b0[5] = YA[0] + XA0_YA0*ny*ny;
		b0[6] = XA0_YA0*ny*nz;
		b0[7] = -YB[0]*nx;
		b0[8] = YA[0] + XA0_YA0*nz*nz;
		b0[9] = YC[0]*(1-nx*nx);
		b0[10] = -YC[0]*nx*ny;
		b0[11] = -YC[0]*nx*nz;
		b0[12] = YC[0]*(1-ny*ny);
		b0[13] = -YC[0]*ny*nz;
		b0[14] = YC[0]*(1-nz*nz);
		double XA3_YA3 = XA[3] - YA[3];
		b1[0] = YA[3] + XA3_YA3*nx*nx;
		b1[1] = XA3_YA3*nx*ny;
		b1[2] = XA3_YA3*nx*nz;
		b1[3] = -YB[3]*nz;
		b1[4] = YB[3]*ny;
		b1[5] = YA[3] + XA3_YA3*ny*ny;
		b1[6] = XA3_YA3*ny*nz;
		b1[7] = -YB[3]*nx;
		b1[8] = YA[3] + XA3_YA3*nz*nz;
		b1[9] = YC[3]*(1-nx*nx);
		b1[10] = -YC[3]*nx*ny;
		b1[11] = -YC[3]*nx*nz;
		b1[12] = YC[3]*(1-ny*ny);
		b1[13] = -YC[3]*ny*nz;
		b1[14] = YC[3]*(1-nz*nz);
	} else {
		memset(od, 0, 18*sizeof(double));
		od[0] = XA[1]*nx*nx; od[1] = XA[1]*nx*ny; od[2] = XA[1]*nx*nz;
		od[5] = XA[1]*ny*ny; od[6] = XA[1]*ny*nz; od[8] = XA[1]*nz*nz;
		memset(b0, 0, 15*sizeof(double)); memset(b1, 0, 15*sizeof(double));
		b0[0] = XA[0]*nx*nx; b0[1] = XA[0]*nx*ny; b0[2] = XA[0]*nx*nz;
		b0[5] = XA[0]*ny*ny; b0[6] = XA[0]*ny*nz; b0[8] = XA[0]*nz*nz;
		b1[0] = XA[3]*nx*nx; b1[1] = XA[3]*nx*ny; b1[2] = XA[3]*nx*nz;
		b1[5] = XA[3]*ny*ny; b1[6] = XA[3]*ny*nz; b1[8] = XA[3]*nz*nz;
	}
}

/* Compact storage: a DBlock is 15 doubles (col0[5], col1[3], col2[1],
 * col3[3], col4[2], col5[1]) and an ODBlock 18 doubles (col0[5], col1[3],
 * col2[1], col3[5], col4[3], col5[1]), MatrixBlocks.h:40-45, 86-91.  The
 * reference's CSC stores 18 and 30 nonzeros for them because it writes the
 * anti-symmetric mirrors explicitly (StokesSolver.cpp:154-231). */

/* Interaction::hasPairwiseResistance, Interaction.cpp:238-245 */
static int has_resistance(const lfo_sim *s, const opair *q)
{
	if (s->lubrication) return q->dp_active || q->lub_active;
	return q->dp_active;
}

/* Interaction::RFU_ODBlock / RFU_DBlocks selection, Interaction.cpp:247-311
 * (non-Brownian: contact_state_changed_after_predictor is always false). */
static void pair_blocks(const lfo_sim *s, const opair *q, double *od, double *b0, double *b1)
{
	if (q->dp_active) { dashpot_blocks(q, od, b0, b1); return; }
	if (s->lubrication && q->lub_active) { lub_blocks(s, q, od, b0, b1); return; }
	memset(od, 0, 18*sizeof(double)); memset(b0, 0, 15*sizeof(double)); memset(b1, 0, 15*sizeof(double));
}

/* dense reconstructions, StokesSolver.cpp:154-231 (row-major m[r*6+c]) */
void lfo_dblock_to_dense(const double *d, double *m)
{
	memset(m, 0, 36*sizeof(double));
	/* column 0 rows {0,1,2,4,5} */
	m[0*6+0] = d[0]; m[1*6+0] = d[1]; m[2*6+0] = d[2]; m[4*6+0] = d[3]; m[5*6+0] = d[4];
	/* column 1 rows {1,2,3,5} */
	m[1*6+1] = d[5]; m[2*6+1] = d[6]; m[3*6+1] = -d[3]; m[5*6+1] = d[7];
	/* column 2 rows {2,3,4} */
	m[2*6+2] = d[8]; m[3*6+2] = -d[4]; m[4*6+2] = -d[7];
	/* column 3 rows {3,4,5} */
	m[3*6+3] = d[9]; m[4*6+3] = d[10]; m[5*6+3] = d[11];
	/* column 4 rows {4,5} */
	m[4*6+4] = d[12]; m[5*6+4] = d[13];
	/* column 5 row {5} */
	m[5*6+5] = d[14];
	/* symmetric upper part */
	for (int r = 0; r < 6; r++) for (int c = r+1; c < 6; c++) m[r*6+c] = m[c*6+r];
}

void lfo_odblock_to_dense(const double *o, double *m)
{
	memset(m, 0, 36*sizeof(double));
	/* col0 rows {0,1,2,4,5} */
	m[0*6+0] = o[0]; m[1*6+0] = o[1]; m[2*6+0] = o[2]; m[4*6+0] = o[3]; m[5*6+0] = o[4];
	/* col1 rows {0,1,2,3,5} */
	m[0*6+1] = o[1]; m[1*6+1] = o[5]; m[2*6+1] = o[6]; m[3*6+1] = -o[3]; m[5*6+1] = o[7];
	/* col2 rows {0,1,2,3,4} */
	m[0*6+2] = o[2]; m[1*6+2] = o[6]; m[2*6+2] = o[8]; m[3*6+2] = -o[4]; m[4*6+2] = -o[7];
	/* col3 rows {1,2,3,4,5} */
	m[1*6+3] = o[9]; m[2*6+3] = o[10]; m[3*6+3] = o[11]; m[4*6+3] = o[12]; m[5*6+3] = o[13];
	/* col4 rows {0,2,3,4,5} */
	m[0*6+4] = -o[9]; m[2*6+4] = o[14]; m[3*6+4] = o[12]; m[4*6+4] = o[15]; m[5*6+4] = o[16];
	/* col5 rows {0,1,3,4,5} */
	m[0*6+5] = -o[10]; m[1*6+5] = -o[14]; m[3*6+5] = o[13]; m[4*6+5] = o[16]; m[5*6+5] = o[17];
}

/* System::buildResistanceMatrix + StokesSolver fill, System.cpp:1429-1473,
 * StokesSolver.cpp:121-152, 474-511.  Diagonal blocks start from the Stokes
 * drag (System.cpp:558-575) and accumulate in column-traversal order. */
static int assemble(lfo_sim *s)
{
	int n = s->np;
	if (!s->dblocks) s->dblocks = calloc((size_t)n*15, sizeof(double));
	for (int i = 0; i < n; i++) {
		double *d = &s->dblocks[i*15];
		memset(d, 0, 15*sizeof(double));
		double a = s->radius[i];
		double FU = s->p.sd_coeff*a;
		double TW = s->p.sd_coeff*pow(a, 3)*4.0/3;
		d[0] = FU; d[5] = FU; d[8] = FU;
		d[9] = TW; d[12] = TW; d[14] = TW;
	}
	int cnt = 0;
	for (int k = 0; k < s->npairs; k++) if (has_resistance(s, &s->pairs[k])) cnt++;
	if (cnt > s->odcap) {
		s->odcap = cnt+1024;
		s->odrow = realloc(s->odrow, sizeof(int)*s->odcap);
		s->odcol = realloc(s->odcol, sizeof(int)*s->odcap);
		s->odblocks = realloc(s->odblocks, sizeof(double)*18*s->odcap);
	}
	s->nod = 0;
	/* pairs are sorted by (p0,p1): this is the column-major traversal order
	 * "for i: for inter in interaction_list[i] (partner-sorted), j > i". */
	for (int k = 0; k < s->npairs; k++) {
		opair *q = &s->pairs[k];
		if (!has_resistance(s, q)) continue;
		double b0[15], b1[15];
		double *od = &s->odblocks[18*s->nod];
		memset(od, 0, 18*sizeof(double));
		pair_blocks(s, q, od, b0, b1);
		double *d0 = &s->dblocks[q->p0*15], *d1 = &s->dblocks[q->p1*15];
		for (int e = 0; e < 15; e++) d0[e] += b0[e];
		for (int e = 0; e < 15; e++) d1[e] += b1[e];
		s->odrow[s->nod] = q->p1;
		s->odcol[s->nod] = q->p0;
		s->nod++;
	}
	return 0;
}

/* ------------------------------------------------------------------ */
/* sparse block Cholesky (stand-in for CHOLMOD's analyze/factorize/solve) */
/* Minimum-degree ordering on the block graph (bitset elimination graph),  */
/* right-looking block factorisation with dense 6x6 blocks.                */
/* ------------------------------------------------------------------ */
typedef struct {
	int n;            /* blocks */
	int *perm;        /* perm[k] = original block eliminated k-th */
	int *iperm;       /* iperm[orig] = k */
	int *colptr;      /* per eliminated column k: row list [colptr[k], colptr[k+1]) */
	int *rowidx;      /* elimination indices > k, sorted */
	double *Lblk;     /* 36 per (k,row) entry, row-major */
	double *Ldiag;    /* 36 per k: lower Cholesky factor of the diagonal block */
} bfact;

static void bfact_free(bfact *f)
{
	if (!f) return;
	free(f->perm); free(f->iperm); free(f->colptr); free(f->rowidx); free(f->Lblk); free(f->Ldiag);
	free(f);
}

static int popcount64(uint64_t x) { return __builtin_popcountll(x); }

/* symbolic: minimum degree with elimination-graph bitsets */
static bfact *bfact_analyze_ex(int n, int nb, const int *row, const int *col, int numeric);
static bfact *bfact_analyze(int n, int nb, const int *row, const int *col)
{
	return bfact_analyze_ex(n, nb, row, col, 1);
}

static bfact *bfact_analyze_ex(int n, int nb, const int *row, const int *col, int numeric)
{
	int W = (n+63)/64;
	uint64_t *adj = calloc((size_t)n*W, sizeof(uint64_t));
	uint64_t *elim = calloc(W, sizeof(uint64_t));
	int *deg = calloc(n, sizeof(int));
	if (!adj || !elim || !deg) return NULL;
	for (int e = 0; e < nb; e++) {
		int i = row[e], j = col[e];
		if (i == j) continue;
		adj[(size_t)i*W + j/64] |= 1ull << (j%64);
		adj[(size_t)j*W + i/64] |= 1ull << (i%64);
	}
	for (int i = 0; i < n; i++) {
		int d = 0;
		for (int w = 0; w < W; w++) d += popcount64(adj[(size_t)i*W+w]);
		deg[i] = d;
	}
	bfact *f = calloc(1, sizeof(bfact));
	f->n = n;
	f->perm = malloc(sizeof(int)*n);
	f->iperm = malloc(sizeof(int)*n);
	/* column structures are recorded in original labels and mapped afterwards */
	int cap = 1024, used = 0;
	int *rows_orig = malloc(sizeof(int)*cap);
	int *cstart = malloc(sizeof(int)*(n+1));
	uint64_t *nb_set = malloc(sizeof(uint64_t)*W);
	char *done = calloc(n, 1);
	for (int k = 0; k < n; k++) {
		int best = -1, bd = 0x7fffffff;
		for (int i = 0; i < n; i++) if (!done[i] && deg[i] < bd) { bd = deg[i]; best = i; }
		int v = best;
		f->perm[k] = v; f->iperm[v] = k; done[v] = 1;
		elim[v/64] |= 1ull << (v%64);
		for (int w = 0; w < W; w++) nb_set[w] = adj[(size_t)v*W+w] & ~elim[w];
		cstart[k] = used;
		for (int w = 0; w < W; w++) {
			uint64_t m = nb_set[w];
			while (m) {
				int b = __builtin_ctzll(m); m &= m-1;
				int u = w*64+b;
				if (used == cap) { cap *= 2; rows_orig = realloc(rows_orig, sizeof(int)*cap); }
				rows_orig[used++] = u;
			}
		}
		for (int t = cstart[k]; t < used; t++) {
			int u = rows_orig[t];
			uint64_t *au = &adj[(size_t)u*W];
			int d = 0;
			for (int w = 0; w < W; w++) { au[w] = (au[w] | nb_set[w]) & ~elim[w]; }
			au[u/64] &= ~(1ull << (u%64));
			for (int w = 0; w < W; w++) d += popcount64(au[w]);
			deg[u] = d;
		}
	}
	cstart[n] = used;
	f->colptr = malloc(sizeof(int)*(n+1));
	f->rowidx = malloc(sizeof(int)*(used > 0 ? used : 1));
	for (int k = 0; k <= n; k++) f->colptr[k] = cstart[k];
	for (int k = 0; k < n; k++) {
		int a = cstart[k], b = cstart[k+1];
		for (int t = a; t < b; t++) f->rowidx[t] = f->iperm[rows_orig[t]];
		/* sort ascending (insertion sort; lists are short) */
		for (int t = a+1; t < b; t++) {
			int x = f->rowidx[t], u = t-1;
			while (u >= a && f->rowidx[u] > x) { f->rowidx[u+1] = f->rowidx[u]; u--; }
			f->rowidx[u+1] = x;
		}
	}
	if (numeric) {
		f->Lblk = calloc((size_t)(used > 0 ? used : 1)*36, sizeof(double));
		f->Ldiag = calloc((size_t)n*36, sizeof(double));
	}
	free(adj); free(elim); free(deg); free(rows_orig); free(cstart); free(nb_set); free(done);
	return f;
}

static double *find_blk(bfact *f, int k, int r)
{
	int lo = f->colptr[k], hi = f->colptr[k+1]-1;
	while (lo <= hi) {
		int m = (lo+hi)/2;
		if (f->rowidx[m] == r) return &f->Lblk[(size_t)m*36];
		if (f->rowidx[m] < r) lo = m+1; else hi = m-1;
	}
	return NULL;
}

/* numeric: A given as full diag blocks (36) and lower off-diagonal blocks
 * (row > col in original labels, row-major 36). */
static int bfact_factorize(bfact *f, const double *diag36, int nb, const int *row, const int *col,
                           const double *off36)
{
	int n = f->n;
	size_t nnzb = (size_t)f->colptr[n];
	memset(f->Lblk, 0, nnzb*36*sizeof(double));
	for (int k = 0; k < n; k++) memcpy(&f->Ldiag[(size_t)k*36], &diag36[(size_t)f->perm[k]*36], 36*sizeof(double));
	for (int e = 0; e < nb; e++) {
		int pi = f->iperm[row[e]], pj = f->iperm[col[e]];
		const double *B = &off36[(size_t)e*36];
		if (pi > pj) {
			double *t = find_blk(f, pj, pi);
			if (!t) return -2;
			for (int u = 0; u < 36; u++) t[u] += B[u];
		} else {
			double *t = find_blk(f, pi, pj);
			if (!t) return -2;
			for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) t[r*6+c] += B[c*6+r];
		}
	}
	for (int k = 0; k < n; k++) {
		double *D = &f->Ldiag[(size_t)k*36];
		/* dense Cholesky of the 6x6 block, lower */
		for (int j = 0; j < 6; j++) {
			double d = D[j*6+j];
			for (int t = 0; t < j; t++) d -= D[j*6+t]*D[j*6+t];
			if (!(d > 0)) return k*6+j+1;
			d = sqrt(d);
			D[j*6+j] = d;
			for (int i = j+1; i < 6; i++) {
				double v = D[i*6+j];
				for (int t = 0; t < j; t++) v -= D[i*6+t]*D[j*6+t];
				D[i*6+j] = v/d;
			}
			for (int c = j+1; c < 6; c++) D[j*6+c] = 0;
		}
		/* L_rk = A_rk D^-T : solve X D^T = A for each row block */
		int a = f->colptr[k], b = f->colptr[k+1];
		for (int t = a; t < b; t++) {
			double *X = &f->Lblk[(size_t)t*36];
			for (int r = 0; r < 6; r++) {
				for (int j = 0; j < 6; j++) {
					double v = X[r*6+j];
					for (int u = 0; u < j; u++) v -= X[r*6+u]*D[j*6+u];
					X[r*6+j] = v/D[j*6+j];
				}
			}
		}
		/* trailing update: A(r1,r2) -= L_r1k L_r2k^T for r1 >= r2; each t2
		 * writes only column r2, so the loop runs in parallel */
		int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) if (b-a > 16) reduction(|:bad)
		for (int t2 = a; t2 < b; t2++) {
			int r2 = f->rowidx[t2];
			const double *L2 = &f->Lblk[(size_t)t2*36];
			/* diagonal block of r2 */
			double *Dr = &f->Ldiag[(size_t)r2*36];
			for (int i = 0; i < 6; i++) for (int j = 0; j <= i; j++) {
				double v = 0;
				for (int u = 0; u < 6; u++) v += L2[i*6+u]*L2[j*6+u];
				Dr[i*6+j] -= v;
				if (i != j) Dr[j*6+i] -= v;
			}
			int p = f->colptr[r2], pe = f->colptr[r2+1];
			for (int t1 = t2+1; t1 < b; t1++) {
				int r1 = f->rowidx[t1];
				while (p < pe && f->rowidx[p] < r1) p++;
				if (p >= pe || f->rowidx[p] != r1) { bad = 1; break; }
				double *T = &f->Lblk[(size_t)p*36];
				const double *L1 = &f->Lblk[(size_t)t1*36];
				for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) {
					double v = 0;
					for (int u = 0; u < 6; u++) v += L1[i*6+u]*L2[j*6+u];
					T[i*6+j] -= v;
				}
			}
		}
		if (bad) return -3;
	}
	return 0;
}

/* x = A^-1 b for one RHS (6n) */
static void bfact_solve(const bfact *f, const double *b, double *x, double *w)
{
	int n = f->n;
	for (int k = 0; k < n; k++) memcpy(&w[k*6], &b[f->perm[k]*6], 6*sizeof(double));
	/* forward: L y = b */
	for (int k = 0; k < n; k++) {
		const double *D = &f->Ldiag[(size_t)k*36];
		double *y = &w[k*6];
		for (int i = 0; i < 6; i++) {
			double v = y[i];
			for (int u = 0; u < i; u++) v -= D[i*6+u]*y[u];
			y[i] = v/D[i*6+i];
		}
		for (int t = f->colptr[k]; t < f->colptr[k+1]; t++) {
			const double *L = &f->Lblk[(size_t)t*36];
			double *z = &w[f->rowidx[t]*6];
			for (int i = 0; i < 6; i++) {
				double v = 0;
				for (int u = 0; u < 6; u++) v += L[i*6+u]*y[u];
				z[i] -= v;
			}
		}
	}
	/* backward: L^T x = y */
	for (int k = n-1; k >= 0; k--) {
		double *y = &w[k*6];
		for (int t = f->colptr[k]; t < f->colptr[k+1]; t++) {
			const double *L = &f->Lblk[(size_t)t*36];
			const double *z = &w[f->rowidx[t]*6];
			for (int u = 0; u < 6; u++) {
				double v = 0;
				for (int i = 0; i < 6; i++) v += L[i*6+u]*z[i];
				y[u] -= v;
			}
		}
		const double *D = &f->Ldiag[(size_t)k*36];
		for (int i = 5; i >= 0; i--) {
			double v = y[i];
			for (int u = i+1; u < 6; u++) v -= D[u*6+i]*y[u];
			y[i] = v/D[i*6+i];
		}
	}
	for (int k = 0; k < n; k++) memcpy(&x[f->perm[k]*6], &w[k*6], 6*sizeof(double));
}

/* ------------------------------------------------------------------ */
/* Supernodal multifrontal factorisation with dense BLAS-3 kernels: the   */
/* method of CHOLMOD's supernodal cholmod_factorize / cholmod_solve2,     */
/* which LF_DEM calls (StokesSolver.cpp:671-703, 950-978).  Same ordering */
/* and column structure as the block factorisation above (minimum degree  */
/* on the 6x6 blocks); consecutive columns whose structures nest form a   */
/* supernode (a fundamental supernode), factored as a dense front:        */
/*   front = A's entries + the children's update matrices (extend-add);   */
/*   L11 = chol(F11) (dpotrf), L21 = F21 L11^-T (dtrsm),                   */
/*   update = F22 - L21 L21^T (dsyrk), passed to the parent.               */
/* The dense kernels come from the caller (lfo_set_blas: LAPACK dpotrf,   */
/* BLAS dtrsm, dsyrk, dgemm, Fortran calling convention, e.g. scipy's     */
/* OpenBLAS).  Levels of the supernode tree with many fronts run them in  */
/* parallel (OpenMP, one BLAS thread each); the top levels run one front  */
/* at a time with every BLAS thread.  Without lfo_set_blas the block      */
/* factorisation is used.                                                 */
/* ------------------------------------------------------------------ */
typedef void (*potrf_fn)(const char *, const int *, double *, const int *, int *);
typedef void (*trsm_fn)(const char *, const char *, const char *, const char *, const int *, const int *,
                        const double *, const double *, const int *, double *, const int *);
typedef void (*syrk_fn)(const char *, const char *, const int *, const int *, const double *, const double *,
                        const int *, const double *, double *, const int *);
typedef void (*gemm_fn)(const char *, const char *, const int *, const int *, const int *, const double *,
                        const double *, const int *, const double *, const int *, const double *, double *,
                        const int *);
typedef void (*threads_fn)(int);
static struct {
	potrf_fn potrf; trsm_fn trsm; syrk_fn syrk; gemm_fn gemm; threads_fn set_threads;
	int threads;
} g_blas;

void lfo_set_blas(void *potrf, void *trsm, void *syrk, void *gemm, void *set_threads, int threads)
{
	g_blas.potrf = (potrf_fn)potrf;
	g_blas.trsm = (trsm_fn)trsm;
	g_blas.syrk = (syrk_fn)syrk;
	g_blas.gemm = (gemm_fn)gemm;
	g_blas.set_threads = (threads_fn)set_threads;
	g_blas.threads = threads > 0 ? threads : 1;
}

int lfo_blas_ready(void) { return g_blas.potrf && g_blas.trsm && g_blas.syrk && g_blas.gemm; }

static void blas_threads(int t)
{
	if (g_blas.set_threads) g_blas.set_threads(t);
}

typedef struct {
	bfact *sym;            /* ordering and block column structures */
	int nsn;
	int *first, *width;    /* supernode: first eliminated block column, width in blocks */
	int *rows_off;         /* below-diagonal block rows of supernode q: sym->rowidx[rows_off[q] ..] */
	int *nrows;
	int *parent;           /* supernode parent, -1 at a root */
	int *child_off, *child;
	int *level, nlevels, *level_off, *level_sn;
	double **L;            /* 6F x 6w, column-major, ld 6F (F = w + nrows) */
	double **U;            /* update matrices (6 nrows)^2, freed by the parent */
	/* A's off-diagonal blocks by lower eliminated column */
	int *acol_ptr, *arow, *aidx, *atr;
} snfact;

static void sn_free(snfact *f)
{
	if (!f) return;
	for (int q = 0; q < f->nsn; q++) { free(f->L ? f->L[q] : NULL); free(f->U ? f->U[q] : NULL); }
	free(f->L); free(f->U);
	free(f->first); free(f->width); free(f->rows_off); free(f->nrows); free(f->parent);
	free(f->child_off); free(f->child); free(f->level); free(f->level_off); free(f->level_sn);
	free(f->acol_ptr); free(f->arow); free(f->aidx); free(f->atr);
	bfact_free(f->sym);
	free(f);
}

static snfact *sn_analyze(int n, int nb, const int *row, const int *col)
{
	bfact *b = bfact_analyze_ex(n, nb, row, col, 0);
	if (!b) return NULL;
	snfact *f = calloc(1, sizeof(snfact));
	f->sym = b;
	int *sn_of = malloc(sizeof(int)*(n > 0 ? n : 1));
	f->first = malloc(sizeof(int)*(n+1));
	f->width = malloc(sizeof(int)*(n+1));
	int q = -1;
	for (int k = 0; k < n; k++) {
		int cnt = b->colptr[k+1]-b->colptr[k];
		int merge = 0;
		if (k > 0) {
			int pc = b->colptr[k]-b->colptr[k-1];
			/* column k-1's structure is {k} plus column k's: nested */
			merge = pc == cnt+1 && pc > 0 && b->rowidx[b->colptr[k-1]] == k;
		}
		if (!merge) { q++; f->first[q] = k; f->width[q] = 0; }
		f->width[q]++;
		sn_of[k] = q;
	}
	int nsn = q+1;
	/* relaxed amalgamation (CHOLMOD's rule, cholmod_super.c defaults nrelax
	 * 4/16/48, zrelax 0.8/0.1/0.05): a supernode whose parent is the next
	 * one merges into it when the dense front adds few explicit zeros */
	{
		int *par = malloc(sizeof(int)*(nsn > 0 ? nsn : 1));
		int *nr = malloc(sizeof(int)*(nsn > 0 ? nsn : 1));
		for (q = 0; q < nsn; q++) {
			int last = f->first[q]+f->width[q]-1;
			nr[q] = b->colptr[last+1]-b->colptr[last];
			par[q] = nr[q] > 0 ? sn_of[b->rowidx[b->colptr[last]]] : -1;
		}
		int out = 0;
		double extra_acc = 0;   /* explicit zeros already merged into the supernode being built */
		for (q = 0; q < nsn; q++) {
			int p = q+1;
			if (p < nsn && par[q] == p) {
				double wq = f->width[q], wp = f->width[p], mq = nr[q], mp = nr[p];
				double w = wq+wp;
				double nnz = w*(w+1)/2+w*mp;
				double extra = extra_acc+wq*(wp+mp-mq);
				double z = extra/nnz, cols = 6*w;
				int merge = cols <= 4*6 || (cols <= 16*6 && z < 0.8) || (cols <= 48*6 && z < 0.1) || z < 0.05;
				if (merge) {
					f->first[p] = f->first[q];
					f->width[p] += f->width[q];
					extra_acc = extra;
					continue;
				}
			}
			f->first[out] = f->first[q];
			f->width[out] = f->width[q];
			out++;
			extra_acc = 0;
		}
		nsn = out;
		for (q = 0; q < nsn; q++)
			for (int k = f->first[q]; k < f->first[q]+f->width[q]; k++) sn_of[k] = q;
		free(par);
		free(nr);
	}
	f->nsn = nsn;
	f->rows_off = malloc(sizeof(int)*(nsn+1));
	f->nrows = malloc(sizeof(int)*(nsn+1));
	f->parent = malloc(sizeof(int)*(nsn+1));
	for (q = 0; q < nsn; q++) {
		int last = f->first[q]+f->width[q]-1;
		f->rows_off[q] = b->colptr[last];
		f->nrows[q] = b->colptr[last+1]-b->colptr[last];
		f->parent[q] = f->nrows[q] > 0 ? sn_of[b->rowidx[b->colptr[last]]] : -1;
	}
	f->child_off = calloc(nsn+1, sizeof(int));
	f->child = malloc(sizeof(int)*(nsn > 0 ? nsn : 1));
	for (q = 0; q < nsn; q++) if (f->parent[q] >= 0) f->child_off[f->parent[q]+1]++;
	for (q = 0; q < nsn; q++) f->child_off[q+1] += f->child_off[q];
	{
		int *fill = malloc(sizeof(int)*(nsn+1));
		memcpy(fill, f->child_off, sizeof(int)*(nsn+1));
		for (q = 0; q < nsn; q++) if (f->parent[q] >= 0) f->child[fill[f->parent[q]]++] = q;
		free(fill);
	}
	/* levels from the leaves (children have lower numbers) */
	f->level = calloc(nsn+1, sizeof(int));
	f->nlevels = 0;
	for (q = 0; q < nsn; q++) {
		int l = 0;
		for (int c = f->child_off[q]; c < f->child_off[q+1]; c++)
			if (f->level[f->child[c]]+1 > l) l = f->level[f->child[c]]+1;
		f->level[q] = l;
		if (l+1 > f->nlevels) f->nlevels = l+1;
	}
	f->level_off = calloc(f->nlevels+1, sizeof(int));
	f->level_sn = malloc(sizeof(int)*(nsn > 0 ? nsn : 1));
	for (q = 0; q < nsn; q++) f->level_off[f->level[q]+1]++;
	for (int l = 0; l < f->nlevels; l++) f->level_off[l+1] += f->level_off[l];
	{
		int *fill = malloc(sizeof(int)*(f->nlevels+1));
		memcpy(fill, f->level_off, sizeof(int)*(f->nlevels+1));
		for (q = 0; q < nsn; q++) f->level_sn[fill[f->level[q]]++] = q;
		free(fill);
	}
	/* A's off-diagonal blocks by their lower eliminated column */
	f->acol_ptr = calloc(n+1, sizeof(int));
	f->arow = malloc(sizeof(int)*(nb > 0 ? nb : 1));
	f->aidx = malloc(sizeof(int)*(nb > 0 ? nb : 1));
	f->atr = malloc(sizeof(int)*(nb > 0 ? nb : 1));
	for (int e = 0; e < nb; e++) {
		int pi = b->iperm[row[e]], pj = b->iperm[col[e]];
		f->acol_ptr[(pi < pj ? pi : pj)+1]++;
	}
	for (int k = 0; k < n; k++) f->acol_ptr[k+1] += f->acol_ptr[k];
	{
		int *fill = malloc(sizeof(int)*(n+1));
		memcpy(fill, f->acol_ptr, sizeof(int)*(n+1));
		for (int e = 0; e < nb; e++) {
			int pi = b->iperm[row[e]], pj = b->iperm[col[e]];
			int lo = pi < pj ? pi : pj, hi = pi < pj ? pj : pi;
			int t = fill[lo]++;
			f->arow[t] = hi;
			f->aidx[t] = e;
			f->atr[t] = pi < pj;   /* the stored block is the transpose of the lower one */
		}
		free(fill);
	}
	f->L = calloc(nsn, sizeof(double *));
	f->U = calloc(nsn, sizeof(double *));
	free(sn_of);
	return f;
}

/* one front: assemble, factor, update; fpos is a per-thread block -> front
 * position map (entries of other fronts are never read) */
static int sn_front(snfact *f, int q, const double *diag36, const double *off36, int *fpos)
{
	bfact *b = f->sym;
	int w = f->width[q], m = f->nrows[q], F = w+m, k0 = f->first[q];
	int nf = 6*F, n6 = 6*w, m6 = 6*m;
	/* the copies run on one thread: OpenMP threads next to the BLAS
	 * library's own (spinning) threads were measured slower */
	const int par = 0;
	double *A = malloc(sizeof(double)*(size_t)nf*nf);
	if (!A) return -4;
#pragma omp parallel for schedule(static) if (par)
	for (int c = 0; c < nf; c++) memset(&A[(size_t)c*nf], 0, sizeof(double)*nf);
	for (int j = 0; j < w; j++) fpos[k0+j] = j;
	for (int t = 0; t < m; t++) fpos[b->rowidx[f->rows_off[q]+t]] = w+t;
	/* A's blocks of the supernode's columns (lower part) */
	for (int j = 0; j < w; j++) {
		int k = k0+j;
		const double *D = &diag36[(size_t)b->perm[k]*36];
		for (int c = 0; c < 6; c++)
			for (int r = c; r < 6; r++) A[(size_t)(6*j+c)*nf+6*j+r] += D[r*6+c];
		for (int t = f->acol_ptr[k]; t < f->acol_ptr[k+1]; t++) {
			int fr = fpos[f->arow[t]];
			const double *B = &off36[(size_t)f->aidx[t]*36];
			for (int c = 0; c < 6; c++)
				for (int r = 0; r < 6; r++)
					A[(size_t)(6*j+c)*nf+6*fr+r] += f->atr[t] ? B[c*6+r] : B[r*6+c];
		}
	}
	/* extend-add of the children's update matrices */
	for (int cc = f->child_off[q]; cc < f->child_off[q+1]; cc++) {
		int c = f->child[cc];
		int mc = f->nrows[c], mc6 = 6*mc;
		double *Uc = f->U[c];
		const int *rc = &b->rowidx[f->rows_off[c]];
#pragma omp parallel for schedule(dynamic, 8) if (par)
		for (int bj = 0; bj < mc; bj++) {
			int pj = fpos[rc[bj]];
			for (int bi = bj; bi < mc; bi++) {
				int pi = fpos[rc[bi]];
				for (int c6 = 0; c6 < 6; c6++)
					for (int r6 = (bi == bj ? c6 : 0); r6 < 6; r6++)
						A[(size_t)(6*pj+c6)*nf+6*pi+r6] += Uc[(size_t)(6*bj+c6)*mc6+6*bi+r6];
			}
		}
		free(Uc);
		f->U[c] = NULL;
	}
	int info = 0;
	g_blas.potrf("L", &n6, A, &nf, &info);
	if (info > 0) { free(A); return 6*k0+info; }
	if (m > 0) {
		const double one = 1.0, mone = -1.0;
		g_blas.trsm("R", "L", "T", "N", &m6, &n6, &one, A, &nf, A+n6, &nf);
		g_blas.syrk("L", "N", &m6, &n6, &mone, A+n6, &nf, &one, A+(size_t)n6*nf+n6, &nf);
		double *U = malloc(sizeof(double)*(size_t)m6*m6);
#pragma omp parallel for schedule(static) if (par)
		for (int c = 0; c < m6; c++) memcpy(&U[(size_t)c*m6], &A[(size_t)(n6+c)*nf+n6], sizeof(double)*m6);
		f->U[q] = U;
	}
	/* keep the supernode's columns (L11 over L21) */
	double *L = malloc(sizeof(double)*(size_t)nf*n6);
#pragma omp parallel for schedule(static) if (par)
	for (int c = 0; c < n6; c++) memcpy(&L[(size_t)c*nf], &A[(size_t)c*nf], sizeof(double)*nf);
	free(A);
	f->L[q] = L;
	return 0;
}

static int sn_factorize(snfact *f, const double *diag36, const double *off36)
{
	int n = f->sym->n;
	int nthr = lfo_num_threads();
	int bad = 0;
	int *fpos_all = malloc(sizeof(int)*(size_t)n*(nthr > 0 ? nthr : 1));
	for (int l = 0; l < f->nlevels && !bad; l++) {
		int a = f->level_off[l], z = f->level_off[l+1];
		if (z-a >= 2*nthr && nthr > 1) {
			/* many fronts: one per thread, single-threaded BLAS */
			blas_threads(1);
#pragma omp parallel for schedule(dynamic, 1) reduction(|:bad)
			for (int t = a; t < z; t++) {
				int tid = 0;
#ifdef _OPENMP
				tid = omp_get_thread_num();
#endif
				int st = sn_front(f, f->level_sn[t], diag36, off36, fpos_all+(size_t)tid*n);
				if (st) bad |= 1;
			}
			blas_threads(g_blas.threads);
		} else {
			blas_threads(g_blas.threads);
			for (int t = a; t < z && !bad; t++) {
				int st = sn_front(f, f->level_sn[t], diag36, off36, fpos_all);
				if (st) bad = 1;
			}
		}
	}
	free(fpos_all);
	return bad ? -5 : 0;
}

/* x = A^-1 b for k right-hand sides (6n each) */
static void sn_solve(const snfact *f, int k, const double *b, double *x)
{
	const bfact *s = f->sym;
	int n = s->n, n6t = 6*n;
	double *y = malloc(sizeof(double)*(size_t)n6t*k);
	for (int r = 0; r < k; r++)
		for (int kk = 0; kk < n; kk++) memcpy(&y[(size_t)r*n6t+6*kk], &b[(size_t)r*n6t+6*s->perm[kk]], 6*sizeof(double));
	int cap = 0;
	double *tmp = NULL;
	const double one = 1.0, mone = -1.0;
	blas_threads(g_blas.threads);
	/* forward: L y = b */
	for (int q = 0; q < f->nsn; q++) {
		int w = f->width[q], m = f->nrows[q], nf = 6*(w+m), n6 = 6*w, m6 = 6*m;
		double *yq = y+6*(size_t)f->first[q];
		g_blas.trsm("L", "L", "N", "N", &n6, &k, &one, f->L[q], &nf, yq, &n6t);
		if (!m) continue;
		if (cap < m6*k) { free(tmp); cap = m6*k; tmp = malloc(sizeof(double)*cap); }
		const int *rr = &s->rowidx[f->rows_off[q]];
		for (int r = 0; r < k; r++)
			for (int t = 0; t < m; t++)
				memcpy(&tmp[(size_t)r*m6+6*t], &y[(size_t)r*n6t+6*rr[t]], 6*sizeof(double));
		g_blas.gemm("N", "N", &m6, &k, &n6, &mone, f->L[q]+n6, &nf, yq, &n6t, &one, tmp, &m6);
		for (int r = 0; r < k; r++)
			for (int t = 0; t < m; t++)
				memcpy(&y[(size_t)r*n6t+6*rr[t]], &tmp[(size_t)r*m6+6*t], 6*sizeof(double));
	}
	/* backward: L^T x = y */
	for (int q = f->nsn-1; q >= 0; q--) {
		int w = f->width[q], m = f->nrows[q], nf = 6*(w+m), n6 = 6*w, m6 = 6*m;
		double *yq = y+6*(size_t)f->first[q];
		if (m) {
			if (cap < m6*k) { free(tmp); cap = m6*k; tmp = malloc(sizeof(double)*cap); }
			const int *rr = &s->rowidx[f->rows_off[q]];
			for (int r = 0; r < k; r++)
				for (int t = 0; t < m; t++)
					memcpy(&tmp[(size_t)r*m6+6*t], &y[(size_t)r*n6t+6*rr[t]], 6*sizeof(double));
			g_blas.gemm("T", "N", &n6, &k, &m6, &mone, f->L[q]+n6, &nf, tmp, &m6, &one, yq, &n6t);
		}
		g_blas.trsm("L", "L", "T", "N", &n6, &k, &one, f->L[q], &nf, yq, &n6t);
	}
	for (int r = 0; r < k; r++)
		for (int kk = 0; kk < n; kk++) memcpy(&x[(size_t)r*n6t+6*s->perm[kk]], &y[(size_t)r*n6t+6*kk], 6*sizeof(double));
	free(tmp);
	free(y);
}

/* the factor a system holds: the block factorisation or the supernodal one */
typedef struct { bfact *b; snfact *sn; } factor_t;

static void fact_free(void *p)
{
	factor_t *f = p;
	if (!f) return;
	bfact_free(f->b);
	sn_free(f->sn);
	free(f);
}

static void fact_solve(const void *p, const double *b, double *x, double *w)
{
	const factor_t *f = p;
	if (f->sn) sn_solve(f->sn, 1, b, x);
	else bfact_solve(f->b, b, x, w);
}

/* A factor of a block matrix on its own (the reference harness's CHOLMOD
 * stand-in): supernodal when the BLAS kernels are set, block otherwise. */
struct lfo_factor { factor_t f; int n; };

lfo_factor *lfo_factor_create(int nblk, const double *diag36, int nb, const int *row, const int *col,
                              const double *off36, int *status)
{
	lfo_factor *h = calloc(1, sizeof(lfo_factor));
	h->n = nblk;
	int st;
	if (lfo_blas_ready()) {
		h->f.sn = sn_analyze(nblk, nb, row, col);
		st = h->f.sn ? sn_factorize(h->f.sn, diag36, off36) : -1;
	} else {
		h->f.b = bfact_analyze(nblk, nb, row, col);
		st = h->f.b ? bfact_factorize(h->f.b, diag36, nb, row, col, off36) : -1;
	}
	if (status) *status = st;
	return h;
}

void lfo_factor_solve(const lfo_factor *h, int k, const double *b, double *x)
{
	if (h->f.sn) { sn_solve(h->f.sn, k, b, x); return; }
	double *w = malloc(sizeof(double)*6*(size_t)h->n);
	for (int r = 0; r < k; r++) bfact_solve(h->f.b, &b[(size_t)r*6*h->n], &x[(size_t)r*6*h->n], w);
	free(w);
}

void lfo_factor_free(lfo_factor *h)
{
	if (!h) return;
	bfact_free(h->f.b);
	sn_free(h->f.sn);
	free(h);
}

int lfo_bsr_solve(int nblk, const double *diag36, int nb, const int *row, const int *col,
                  const double *off36, int k, const double *b, double *x)
{
	bfact *f = bfact_analyze(nblk, nb, row, col);
	if (!f) return -1;
	int st = bfact_factorize(f, diag36, nb, row, col, off36);
	if (st) { bfact_free(f); return st; }
	double *w = malloc(sizeof(double)*6*nblk);
	for (int r = 0; r < k; r++) bfact_solve(f, &b[(size_t)r*6*nblk], &x[(size_t)r*6*nblk], w);
	free(w);
	bfact_free(f);
	return 0;
}

/* assemble -> dense blocks -> analyse + factorise (StokesSolver::
 * matrixFillingDone / factorizeResistanceMatrix, StokesSolver.cpp:937-978) */
/* algorithmic flops of a factorisation with this ordering: every block
 * column is 6 scalar columns with 6c rows below them (c off-diagonal
 * blocks), counted as n^3/3 + n^2 m + n m^2 with n = 6, m = 6c */
static double bfact_flops(const bfact *f)
{
	double fl = 0;
	for (int k = 0; k < f->n; k++) {
		double m = 6.0*(f->colptr[k+1]-f->colptr[k]);
		fl += 72.0+36.0*m+6.0*m*m;
	}
	return fl;
}

static double wall_s(void)
{
#ifdef _OPENMP
	return omp_get_wtime();
#else
	return 0.0;
#endif
}

static int factorize_current(lfo_sim *s)
{
	int n = s->np;
	double *diag36 = malloc(sizeof(double)*36*n);
	double *off36 = malloc(sizeof(double)*36*(s->nod > 0 ? s->nod : 1));
	for (int i = 0; i < n; i++) lfo_dblock_to_dense(&s->dblocks[i*15], &diag36[i*36]);
	for (int e = 0; e < s->nod; e++) lfo_odblock_to_dense(&s->odblocks[e*18], &off36[e*36]);
	if (s->fact) { fact_free(s->fact); s->fact = NULL; }
	factor_t *F = calloc(1, sizeof(factor_t));
	double t0 = wall_s(), t1, t2;
	int st;
	if (lfo_blas_ready()) {
		F->sn = sn_analyze(n, s->nod, s->odrow, s->odcol);
		t1 = wall_s();
		st = F->sn ? sn_factorize(F->sn, diag36, off36) : -1;
		t2 = wall_s();
		if (F->sn) s->last_factor_flops = bfact_flops(F->sn->sym);
	} else {
		F->b = bfact_analyze(n, s->nod, s->odrow, s->odcol);
		t1 = wall_s();
		st = F->b ? bfact_factorize(F->b, diag36, s->nod, s->odrow, s->odcol, off36) : -1;
		t2 = wall_s();
		if (F->b) s->last_factor_flops = bfact_flops(F->b);
	}
	s->n_factor++;
	s->analyze_s += t1-t0;
	s->factor_s += t2-t1;
	free(diag36); free(off36);
	s->fact = F;
	return st;
}

int lfo_assemble(lfo_sim *s, double *dblocks, int *odrow, int *odcol, double *odblocks)
{
	assemble(s);
	if (dblocks) memcpy(dblocks, s->dblocks, sizeof(double)*15*s->np);
	if (odrow) memcpy(odrow, s->odrow, sizeof(int)*s->nod);
	if (odcol) memcpy(odcol, s->odcol, sizeof(int)*s->nod);
	if (odblocks) memcpy(odblocks, s->odblocks, sizeof(double)*18*s->nod);
	return s->nod;
}

int lfo_solve_assembled(lfo_sim *s, int k, const double *b, double *x)
{
	int st = factorize_current(s);
	if (st) return st;
	double *w = malloc(sizeof(double)*6*s->np);
	for (int r = 0; r < k; r++) fact_solve(s->fact, &b[(size_t)r*6*s->np], &x[(size_t)r*6*s->np], w);
	free(w);
	return 0;
}

static void compute_u_inf(lfo_sim *s);

/* ------------------------------------------------------------------ */
/* force components (System.cpp:1727-1828)                              */
/* ------------------------------------------------------------------ */
static inline void addF(double *f, int i, v3 v) { f[6*i] += v.x; f[6*i+1] += v.y; f[6*i+2] += v.z; }
static inline void addT(double *f, int i, v3 v) { f[6*i+3] += v.x; f[6*i+4] += v.y; f[6*i+5] += v.z; }

/* ContactDashpot::getForceOnP0, ContactDashpot.cpp:342-385 */
static v3 dashpot_force_p0(const lfo_sim *s, const opair *q, v3 vi, v3 vj, v3 oi, v3 oj, int affine)
{
	if (!q->dp_active) return vzero();
	if (affine) vj = vadd(vj, vscale((double)q->z_offset, s->vel_difference));
	v3 n = q->nvec;
	v3 f = vscale(-vdot(vadd(vscale(q->dXA[0], vi), vscale(q->dXA[1], vj)), n), n);
	if (q->dp_tan_coeff > 0) {
		v3 t1 = vsub(vscale(-q->dYA[0], vsub(vi, vscale(vdot(n, vi), n))),
		             vscale(q->dYA[1], vsub(vj, vscale(vdot(n, vj), n))));
		f = vadd(f, t1);
		v3 t2 = vsub(vscale(-q->dYB[0], vcross(n, oi)), vscale(q->dYB[2], vcross(n, oj)));
		f = vadd(f, t2);
	}
	return f;
}

static void force_component(lfo_sim *s, int comp, double *out)
{
	int n = s->np;
	memset(out, 0, sizeof(double)*6*n);
	if (comp == FC_CONTACT) {
		/* setContactForceToParticle + Contact::addUpForceTorque, Contact.cpp:410-437 */
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			if (!q->c_active) continue;
			addF(out, q->p0, q->fs_total);
			addF(out, q->p1, vneg(q->fs_total));
			if (q->state >= 2) {
				v3 t = vcross(q->nvec, q->fs_tan);
				addT(out, q->p0, vscale(q->a0, t));
				addT(out, q->p1, vscale(q->a1, t));
				if (s->rolling) {
					v3 tr = vcross(q->nvec, q->f_roll);
					addT(out, q->p0, vscale(q->a0, tr));
					addT(out, q->p1, vneg(vscale(q->a1, tr)));
				}
			}
		}
	} else if (comp == FC_DASHPOT) {
		/* setDashpotForceToParticle + ContactDashpot::getRFU_Uinf, ContactDashpot.cpp:426-441 */
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			if (!(q->c_active && q->dp_active)) continue;
			v3 om = V(s->Omega[0], s->Omega[1], s->Omega[2]);
			v3 f0 = dashpot_force_p0(s, q, s->u_inf[q->p0], s->u_inf[q->p1], om, om, 1);
			v3 t0 = vzero();
			if (q->dp_tan_coeff > 0) t0 = vscale(q->a0, vcross(q->nvec, f0));
			addF(out, q->p0, f0);
			addF(out, q->p1, vneg(f0));
			addT(out, q->p0, t0);
			addT(out, q->p1, vscale(q->a1/q->a0, t0));
		}
	} else if (comp == FC_HYDRO) {
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			if (!q->lub_active) continue;
			double XG[4], YG[4], YH[4];
			for (int j = 0; j < 4; j++) {
				XG[j] = q->lc[CXG][j]*q->lub_coeff;
				YG[j] = q->lc[CYG][j]*q->log_lub_coeff;
				YH[j] = q->lc[CYH][j]*q->log_lub_coeff;
			}
			v3 n = q->nvec;
			double nnE = vdot(n, sdot(s->Einf, n));
			if (!s->tangential) {
				/* Lubrication::calcGE_squeeze, Lubrication.cpp:332-356 */
				double ci = (XG[0]+XG[2])*nnE, cj = (XG[1]+XG[3])*nnE;
				addF(out, q->p0, V(ci*n.x, ci*n.y, ci*n.z));
				addF(out, q->p1, V(cj*n.x, cj*n.y, cj*n.z));
			} else {
				/* Lubrication::calcGEHE_squeeze_tangential, Lubrication.cpp:378-403 */
				double YG0_YG2 = YG[0]+YG[2];
				double YG1_YG3 = YG[1]+YG[3];
				double cGE_i = (XG[0]+XG[2]-2*YG0_YG2)*nnE;
				double cGE_j = (XG[1]+XG[3]-2*YG1_YG3)*nnE;
				double cHE_i = YH[0]+YH[2];
				double cHE_j = YH[1]+YH[3];
				v3 En = sdot(s->Einf, n);
				v3 GEi = vadd(vscale(cGE_i, n), vscale(YG0_YG2*2, En));
				v3 GEj = vadd(vscale(cGE_j, n), vscale(YG1_YG3*2, En));
				v3 nExn = vcross(En, n);
				v3 HEi = vscale(-2*cHE_i, nExn);
				v3 HEj = vscale(-2*cHE_j, nExn);
				addF(out, q->p0, GEi); addF(out, q->p1, GEj);
				addT(out, q->p0, HEi); addT(out, q->p1, HEj);
			}
		}
	} else if (comp == FC_REPULSION) {
		/* setRepulsiveForceToParticle + RepulsiveForce::addUpForce, RepulsiveForce.cpp:101-105 */
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			addF(out, q->p0, q->rep_force);
			addF(out, q->p1, vneg(q->rep_force));
		}
	}
}

int lfo_force_component(lfo_sim *s, int comp, double *out)
{
	if (comp < 0 || comp >= NFC || !s->has_fc[comp]) return -1;
	compute_u_inf(s);
	force_component(s, comp, out);
	return 0;
}

/* ------------------------------------------------------------------ */
/* velocities (System.cpp:1932-1965, 2236-2392)                          */
/* ------------------------------------------------------------------ */
static void compute_u_inf(lfo_sim *s)
{
	/* System::computeUInf, System.cpp:2357-2367 */
	v3 om = V(s->Omega[0], s->Omega[1], s->Omega[2]);
	for (int i = 0; i < s->np; i++) s->u_inf[i] = vadd(sdot(s->Einf, s->pos[i]), vcross(om, s->pos[i]));
}

static void rhs_set(const lfo_sim *s, int comp, const double *fc, double *rhs)
{
	/* System::setSolverRHS, System.cpp:1858-1871 */
	for (int i = 0; i < s->np; i++) {
		rhs[6*i] = fc[6*i]; rhs[6*i+1] = fc[6*i+1]; rhs[6*i+2] = fc[6*i+2];
		if (s->fc_torque[comp]) { rhs[6*i+3] = fc[6*i+3]; rhs[6*i+4] = fc[6*i+4]; rhs[6*i+5] = fc[6*i+5]; }
		else { rhs[6*i+3] = 0; rhs[6*i+4] = 0; rhs[6*i+5] = 0; }
	}
}
static void rhs_add(const lfo_sim *s, int comp, const double *fc, double *rhs)
{
	/* System::addToSolverRHS, System.cpp:1873-1885 */
	for (int i = 0; i < s->np; i++) {
		rhs[6*i] += fc[6*i]; rhs[6*i+1] += fc[6*i+1]; rhs[6*i+2] += fc[6*i+2];
		if (s->fc_torque[comp]) { rhs[6*i+3] += fc[6*i+3]; rhs[6*i+4] += fc[6*i+4]; rhs[6*i+5] += fc[6*i+5]; }
	}
}

static void calc_stress_per_particle(lfo_sim *s);

static int compute_velocities(lfo_sim *s, int divided)
{
	/* System::computeVelocities, System.cpp:2273-2319 */
	int n = s->np;
	double *rhs = calloc((size_t)6*n, sizeof(double));
	double *x = malloc(sizeof(double)*6*n);
	double *w = malloc(sizeof(double)*6*n);
	int st;
	if (divided || s->p.control == 1) {
		if (s->p.control == 1) set_shear_rate(s, 1);
		compute_u_inf(s);
		assemble(s);
		if ((st = factorize_current(s))) goto out;
		for (int c = 0; c < NFC; c++) {
			if (!s->has_fc[c]) continue;
			force_component(s, c, s->fc_force[c]);
			rhs_set(s, c, s->fc_force[c], rhs);
			fact_solve(s->fact, rhs, s->vc[c], w);
		}
		if (s->p.control == 1) {
			/* System::computeShearRate, System.cpp:2017-2055 */
			calc_stress_per_particle(s);
			double prop[6] = {0}, indep[6] = {0};
			for (int c = 0; c < NSC; c++) {
				if (!s->has_sc[c]) continue;
				double tot[6] = {0};
				for (int i = 0; i < n; i++) for (int e = 0; e < 6; e++) tot[e] += s->sc[c][i].e[e];
				if (s->sc_rate[c] == RATE_INDEP) for (int e = 0; e < 6; e++) indep[e] += tot[e];
				if (s->sc_rate[c] == RATE_PROP) for (int e = 0; e < 6; e++) prop[e] += tot[e];
			}
			double inv = 1.0/s->system_volume;
			for (int e = 0; e < 6; e++) { prop[e] *= inv; indep[e] *= inv; }
			for (int e = 0; e < 6; e++) prop[e] += 2*s->Einf[e]/(6*M_PI);
			double rp = doubledot(prop, s->Einf);
			double ri = doubledot(indep, s->Einf);
			s->rate_prop_shearstress = rp;
			s->rate_indep_shearstress = ri;
			if (rp != 0) set_shear_rate(s, (s->p.target_stress-ri)/rp);
			if (s->strain < s->p.init_strain_shear_rate_limit && s->shear_rate > s->p.init_shear_rate_limit)
				set_shear_rate(s, s->p.init_shear_rate_limit);
			/* System::rescaleVelHydroStressControlled, System.cpp:2264-2271 */
			for (int c = 0; c < NFC; c++)
				if (s->has_fc[c] && s->fc_rate[c] == RATE_PROP)
					for (int e = 0; e < 6*n; e++) s->vc[c][e] *= s->shear_rate;
		}
		/* System::sumUpVelocityComponents, System.cpp:2236-2250 */
		for (int i = 0; i < n; i++) { s->na_vel[i] = vzero(); s->na_ang[i] = vzero(); }
		for (int c = 0; c < NFC; c++) {
			if (!s->has_fc[c]) continue;
			for (int i = 0; i < n; i++) {
				s->na_vel[i] = vadd(s->na_vel[i], V(s->vc[c][6*i], s->vc[c][6*i+1], s->vc[c][6*i+2]));
				s->na_ang[i] = vadd(s->na_ang[i], V(s->vc[c][6*i+3], s->vc[c][6*i+4], s->vc[c][6*i+5]));
			}
		}
	} else {
		compute_u_inf(s);
		/* System::computeVelocityWithoutComponents, System.cpp:1932-1945 */
		assemble(s);
		if ((st = factorize_current(s))) goto out;
		for (int c = 0; c < NFC; c++) {
			if (!s->has_fc[c]) continue;
			force_component(s, c, s->fc_force[c]);
			rhs_add(s, c, s->fc_force[c], rhs);
		}
		fact_solve(s->fact, rhs, x, w);
		for (int i = 0; i < n; i++) {
			s->na_vel[i] = V(x[6*i], x[6*i+1], x[6*i+2]);
			s->na_ang[i] = V(x[6*i+3], x[6*i+4], x[6*i+5]);
		}
	}
	if (!s->p.fixed_dt && s->in_predictor) {
		/* System::computeMaxNAVelocity, System.cpp:1887-1930 */
		double m = 0;
		for (int i = 0; i < n; i++) { double v = vsq(s->na_vel[i]); if (v > m) m = v; }
		s->max_velocity = sqrt(m);
	}
	/* System::adjustVelocityPeriodicBoundary, System.cpp:2369-2392 */
	if (s->p.control == 1) compute_u_inf(s);
	v3 om = V(s->Omega[0], s->Omega[1], s->Omega[2]);
	for (int i = 0; i < n; i++) {
		s->vel[i] = vadd(s->na_vel[i], s->u_inf[i]);
		s->ang[i] = vadd(s->na_ang[i], om);
	}
	st = 0;
out:
	free(rhs); free(x); free(w);
	return st;
}

/* ------------------------------------------------------------------ */
/* stresslets (Stress.cpp:77-287)                                       */
/* ------------------------------------------------------------------ */
static void lub_XYM(const opair *q, double *XG, double *YG, double *XM, double *YM)
{
	for (int j = 0; j < 4; j++) {
		XG[j] = q->lc[CXG][j]*q->lub_coeff;
		YG[j] = q->lc[CYG][j]*q->log_lub_coeff;
		XM[j] = q->lc[CXM][j]*q->lub_coeff;
		YM[j] = q->lc[CYM][j]*q->log_lub_coeff;
	}
}

/* Lubrication::addGUStresslet, Lubrication.cpp:587-615 */
static void gu_stresslet(const lfo_sim *s, const opair *q, v3 vi, v3 vj, v3 oi, v3 oj, s2 *Si, s2 *Sj)
{
	double XG[4], YG[4], XM[4], YM[4];
	lub_XYM(q, XG, YG, XM, YM);
	v3 n = q->nvec;
	double nvi = vdot(n, vi), nvj = vdot(n, vj);
	s2 nn = outer(n);
	sadd_to(Si, sscale(-(XG[0]*nvi+XG[1]*nvj), nn));
	sadd_to(Sj, sscale(-(XG[2]*nvi+XG[3]*nvj), nn));
	if (!s->tangential) return;
	s2 ti = ssub(outer_sym(n, vi), sscale(nvi, nn));
	s2 tj = ssub(outer_sym(n, vj), sscale(nvj, nn));
	sadd_to(Si, sscale(-2, saddv(sscale(YG[0], ti), sscale(YG[1], tj))));
	sadd_to(Sj, sscale(-2, saddv(sscale(YG[2], ti), sscale(YG[3], tj))));
	s2 t2i = outer_sym(n, vcross(oi, n));
	s2 t2j = outer_sym(n, vcross(oj, n));
	sadd_to(Si, sscale(-2, saddv(sscale(YM[0], t2i), sscale(YM[1], t2j))));
	sadd_to(Sj, sscale(-2, saddv(sscale(YM[2], t2i), sscale(YM[3], t2j))));
}

/* Lubrication::addMEStresslet, Lubrication.cpp:617-650 */
static void me_stresslet(const lfo_sim *s, const opair *q, s2 *Si, s2 *Sj)
{
	double XG[4], YG[4], XM[4], YM[4];
	lub_XYM(q, XG, YG, XM, YM);
	v3 n = q->nvec;
	double nnE = vdot(n, sdot(s->Einf, n));
	s2 nn = outer(n);
	double coeff = 1.5*nnE;
	sadd_to(Si, sscale(coeff*(XM[0]+XM[1]), nn));
	sadd_to(Sj, sscale(coeff*(XM[2]+XM[3]), nn));
	if (s->tangential) {
		v3 En = sdot(s->Einf, n);
		s2 nEn = outer_sym(n, En);
		s2 T = sscale(2, ssub(nEn, sscale(nnE, nn)));
		sadd_to(Si, sscale(YM[0]+YM[1], T));
		sadd_to(Sj, sscale(YM[2]+YM[3], T));
	}
}

/* System::calcStressPerParticle, Stress.cpp:194-287 */
static void calc_stress_per_particle(lfo_sim *s)
{
	int n = s->np;
	for (int c = 0; c < NSC; c++) if (s->has_sc[c]) memset(s->sc[c], 0, sizeof(s2)*n);
	/* GU per velocity component, ME */
	static const int gu_slot[NFC] = {SC_GU_CONTACT, SC_GU_DASHPOT, SC_GU_HYDRO, SC_GU_REPULSION};
	if (s->lubrication) {
		for (int c = 0; c < NFC; c++) {
			if (!s->has_fc[c] || !s->has_sc[gu_slot[c]]) continue;
			s2 *S = s->sc[gu_slot[c]];
			const double *v = s->vc[c];
			for (int k = 0; k < s->npairs; k++) {
				const opair *q = &s->pairs[k];
				if (!q->lub_active) continue;
				int i = q->p0, j = q->p1;
				gu_stresslet(s, q, V(v[6*i], v[6*i+1], v[6*i+2]), V(v[6*j], v[6*j+1], v[6*j+2]),
				             V(v[6*i+3], v[6*i+4], v[6*i+5]), V(v[6*j+3], v[6*j+4], v[6*j+5]),
				             &S[i], &S[j]);
			}
		}
		s2 *S = s->sc[SC_ME];
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			if (!q->lub_active) continue;
			me_stresslet(s, q, &S[q->p0], &S[q->p1]);
		}
	}
	if (s->p.control == 0) {
		/* Contact::addUpStress, Contact.cpp:439-458 (total velocities) */
		s2 *S = s->sc[SC_XF_CONTACT];
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			if (!q->c_active) continue;
			v3 F = vadd(q->fs_total, dashpot_force_p0(s, q, s->vel[q->p0], s->vel[q->p1],
			                                          s->ang[q->p0], s->ang[q->p1], 1));
			s2 XF = outer_sym(q->rvec, F);
			double r_ij = q->a0+q->a1;
			sadd_to(&S[q->p0], sscale(q->a0/r_ij, XF));
			sadd_to(&S[q->p1], sscale(q->a1/r_ij, XF));
		}
	} else {
		/* System::calcContactXFPerParticleStressControlled, Stress.cpp:150-192 */
		v3 *pv = malloc(sizeof(v3)*n), *pa = malloc(sizeof(v3)*n);
		v3 *iv = malloc(sizeof(v3)*n), *ia = malloc(sizeof(v3)*n);
		for (int i = 0; i < n; i++) { pv[i] = pa[i] = iv[i] = ia[i] = vzero(); }
		for (int c = 0; c < NFC; c++) {
			if (!s->has_fc[c]) continue;
			const double *v = s->vc[c];
			if (s->fc_rate[c] == RATE_PROP) {
				for (int i = 0; i < n; i++) {
					pv[i] = vadd(pv[i], V(v[6*i], v[6*i+1], v[6*i+2]));
					pa[i] = vadd(pa[i], V(v[6*i+3], v[6*i+4], v[6*i+5]));
				}
			}
			if (s->fc_rate[c] == RATE_INDEP) {
				for (int i = 0; i < n; i++) {
					iv[i] = vadd(iv[i], V(v[6*i], v[6*i+1], v[6*i+2]));
					ia[i] = vadd(ia[i], V(v[6*i+3], v[6*i+4], v[6*i+5]));
				}
			}
		}
		v3 om = V(s->Omega[0], s->Omega[1], s->Omega[2]);
		for (int i = 0; i < n; i++) { pv[i] = vadd(pv[i], s->u_inf[i]); pa[i] = vadd(pa[i], om); }
		s2 *Sp = s->sc[SC_XF_RATEPROP], *Si = s->sc[SC_XF_RATEINDEP];
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			int i = q->p0, j = q->p1;
			double r_ij = s->radius[i]+s->radius[j];
			if (q->c_active) {
				/* Contact::addUpStressSpring, Contact.cpp:460-467 */
				s2 sp = outer_sym(q->rvec, q->fs_total);
				sadd_to(&Si[i], sscale(q->a0/r_ij, sp));
				sadd_to(&Si[j], sscale(q->a1/r_ij, sp));
			}
			if (q->dp_active) {
				s2 rp = outer_sym(q->rvec, dashpot_force_p0(s, q, pv[i], pv[j], pa[i], pa[j], 1));
				sadd_to(&Sp[i], sscale(s->radius[i]/r_ij, rp));
				sadd_to(&Sp[j], sscale(s->radius[j]/r_ij, rp));
				s2 ri = outer_sym(q->rvec, dashpot_force_p0(s, q, iv[i], iv[j], ia[i], ia[j], 0));
				sadd_to(&Si[i], sscale(s->radius[i]/r_ij, ri));
				sadd_to(&Si[j], sscale(s->radius[j]/r_ij, ri));
			}
		}
		free(pv); free(pa); free(iv); free(ia);
	}
	if (s->repulsiveforce) {
		/* RepulsiveForce::addUpStressXF, RepulsiveForce.cpp:122-131 */
		s2 *S = s->sc[SC_XF_REPULSION];
		for (int k = 0; k < s->npairs; k++) {
			const opair *q = &s->pairs[k];
			v3 F = vscale(-(s->p.repulsion*q->rep_reduced), q->nvec);
			s2 sc = sscale(0.5, outer_sym(q->rvec, F));
			sadd_to(&S[q->p0], sc);
			sadd_to(&S[q->p1], sc);
		}
	}
}

/* System::calcStress, Stress.cpp:342-384 */
static void calc_stress(const lfo_sim *s, double *total, double groups[4][6])
{
	for (int g = 0; g < 4; g++) for (int e = 0; e < 6; e++) groups[g][e] = 0;
	for (int c = 0; c < NSC; c++) {
		if (!s->has_sc[c]) continue;
		double tot[6] = {0};
		for (int i = 0; i < s->np; i++) for (int e = 0; e < 6; e++) tot[e] += s->sc[c][i].e[e];
		for (int e = 0; e < 6; e++) groups[s->sc_group[c]][e] += tot[e];
	}
	double inv = 1.0/s->system_volume;
	for (int g = 0; g < 4; g++) for (int e = 0; e < 6; e++) groups[g][e] *= inv;
	for (int e = 0; e < 6; e++) groups[2][e] += 2*s->Einf[e]/(6*M_PI);
	/* std::map<string> order: contact, dashpot, hydro, repulsion */
	for (int e = 0; e < 6; e++) total[e] = 0;
	for (int g = 0; g < 4; g++) for (int e = 0; e < 6; e++) total[e] += groups[g][e];
}

/* ------------------------------------------------------------------ */
/* integrator (System.cpp:672-717, 843-1187, 1013-1066, 2418-2443)      */
/* ------------------------------------------------------------------ */
static void adapt_time_step(lfo_sim *s, double time_end, double strain_end)
{
	/* System::adaptTimeStep(), System.cpp:1013-1046 */
	if (s->max_velocity > 0 || s->max_sliding_velocity > 0) {
		if (s->max_velocity > s->max_sliding_velocity) s->dt = s->p.disp_max/s->max_velocity;
		else s->dt = s->p.disp_max/s->max_sliding_velocity;
	} else {
		s->dt = s->p.disp_max/s->shear_rate;
	}
	if (s->dt*s->shear_rate > s->p.disp_max) s->dt = s->p.disp_max/s->shear_rate;
	if (s->p.dt_max > 0 && s->dt > s->p.dt_max) s->dt = s->p.dt_max;
	if (s->p.dt_min > 0 && s->dt < s->p.dt_min) s->dt = s->p.dt_min;
	/* System::adaptTimeStep(time_end, strain_end), System.cpp:1048-1066 */
	if (strain_end >= 0) {
		if (fabs(s->dt*s->shear_rate) > strain_end-s->strain)
			s->dt = fabs((strain_end-s->strain)/s->shear_rate);
	}
	if (time_end >= 0) {
		if (s->time+s->dt > time_end) s->dt = time_end-s->time;
	}
}

static void time_step_boxing(lfo_sim *s)
{
	/* System::timeStepBoxing, System.cpp:672-717 (simple shear) */
	double strain_increment = s->shear_rate*s->dt;
	s->strain += strain_increment;
	/* 2*dot(E,{0,0,1})*dt evaluates as (2*E.z)*dt */
	v3 inc = V(2*sdot(s->Einf, V(0, 0, 1)).x*s->dt, 2*sdot(s->Einf, V(0, 0, 1)).y*s->dt,
	        2*sdot(s->Einf, V(0, 0, 1)).z*s->dt);
	s->shear_strain = vadd(s->shear_strain, inc);
	s->shear_disp = vadd(s->shear_disp, vscale(s->lz, inc));
	int m = (int)(s->shear_disp.x/s->lx);
	if (s->shear_disp.x < 0) m--;
	s->shear_disp.x = s->shear_disp.x-m*s->lx;
	if (!s->twodim) {
		m = (int)(s->shear_disp.y/s->ly);
		if (s->shear_disp.y < 0) m--;
		s->shear_disp.y = s->shear_disp.y-m*s->ly;
	}
}

static void displacement(lfo_sim *s, int i, v3 dr)
{
	/* System::displacement, System.cpp:2418-2443 */
	s->pos[i] = vadd(s->pos[i], dr);
	int z_shift = periodize(s, &s->pos[i]);
	if (z_shift != 0) s->vel[i] = vadd(s->vel[i], vscale((double)z_shift, s->vel_difference));
}

static int step_pc(lfo_sim *s, int calc_stress, double time_end, double strain_end)
{
	/* System::timeEvolutionPredictorCorrectorMethod, System.cpp:888-983 */
	int n = s->np, st;
	s->in_predictor = 1; s->in_corrector = 0;
	if ((st = compute_velocities(s, calc_stress))) return st;
	if (calc_stress) calc_stress_per_particle(s);
	/* timeStepMovePredictor, System.cpp:1124-1162 */
	if (!s->p.fixed_dt) adapt_time_step(s, time_end, strain_end);
	s->time += s->dt;
	s->time_sim += s->dt;
	s->total_num_timesteps++;
	time_step_boxing(s);
	for (int i = 0; i < n; i++) displacement(s, i, vscale(s->dt, s->vel[i]));
	update_interactions(s);
	for (int i = 0; i < n; i++) { s->vel_pred[i] = s->vel[i]; s->ang_pred[i] = s->ang[i]; }
	/* corrector */
	s->in_predictor = 0; s->in_corrector = 1;
	if ((st = compute_velocities(s, calc_stress))) return st;
	if (calc_stress) calc_stress_per_particle(s);
	/* timeStepMoveCorrector, System.cpp:1164-1187 */
	for (int i = 0; i < n; i++) {
		s->vel[i] = vscale(0.5, vadd(s->vel[i], s->vel_pred[i]));
		s->ang[i] = vscale(0.5, vadd(s->ang[i], s->ang_pred[i]));
	}
	for (int i = 0; i < n; i++) displacement(s, i, vscale(s->dt, vsub(s->vel[i], s->vel_pred[i])));
	if (check_new_interaction(s)) return -1;
	update_interactions(s);
	return 0;
}

static int step_euler(lfo_sim *s, int calc_stress, double time_end, double strain_end)
{
	/* System::timeEvolutionEulersMethod + timeStepMove, System.cpp:843-882, 1083-1122 */
	int n = s->np, st;
	s->in_predictor = 1; s->in_corrector = 1;
	if ((st = compute_velocities(s, calc_stress))) return st;
	if (calc_stress) calc_stress_per_particle(s);
	if (!s->p.fixed_dt) adapt_time_step(s, time_end, strain_end);
	s->time += s->dt;
	s->time_sim += s->dt;
	s->total_num_timesteps++;
	time_step_boxing(s);
	for (int i = 0; i < n; i++) displacement(s, i, vscale(s->dt, s->vel[i]));
	if (check_new_interaction(s)) return -1;
	update_interactions(s);
	return 0;
}

void lfo_first_time(lfo_sim *s)
{
	/* System::timeEvolution first-time block, System.cpp:1216-1226 */
	if (!s->firsttime) return;
	double dt_bak = s->dt;
	s->dt = 0;
	check_new_interaction(s);
	s->in_predictor = 1;
	update_interactions(s);
	s->in_predictor = 0;
	s->dt = dt_bak;
	s->firsttime = 0;
}

int lfo_set_contact(lfo_sim *s, int p0, int p1, int state, const double *disp_tan)
{
	int k = find_pair(s, p0, p1);
	if (k < 0) return -1;
	opair *q = &s->pairs[k];
	q->disp_tan = V(disp_tan[0], disp_tan[1], disp_tan[2]);
	if (q->c_active) q->state = state;
	return 0;
}

/* rolling spring of an existing contact (contact_state.disp_rolling,
 * Contact.h:150-162) */
int lfo_set_contact_rolling(lfo_sim *s, int p0, int p1, const double *disp_rolling)
{
	int k = find_pair(s, p0, p1);
	if (k < 0) return -1;
	s->pairs[k].disp_roll = V(disp_rolling[0], disp_rolling[1], disp_rolling[2]);
	return 0;
}

void lfo_set_clock(lfo_sim *s, double time, double strain, double dt, double shear_rate,
                   double max_velocity, double max_sliding_velocity, int firsttime_done)
{
	s->time = time;
	s->strain = strain;
	s->dt = dt;
	set_shear_rate(s, shear_rate);
	s->max_velocity = max_velocity;
	s->max_sliding_velocity = max_sliding_velocity;
	s->firsttime = !firsttime_done;
}

void lfo_refresh(lfo_sim *s)
{
	double dt_bak = s->dt;
	double msv = s->max_sliding_velocity;
	s->dt = 0;
	s->in_predictor = 1;
	update_interactions(s);
	s->in_predictor = 0;
	s->dt = dt_bak;
	s->max_sliding_velocity = msv;
}

int lfo_step(lfo_sim *s, int calc_stress, double time_end, double strain_end)
{
	lfo_first_time(s);
	if (!s->p.fixed_dt) {
		/* the loop's own adaptTimeStep, System.cpp:1243-1245 */
		adapt_time_step(s, time_end, strain_end);
	}
	if (s->p.integration_method == 0) return step_euler(s, calc_stress, time_end, strain_end);
	return step_pc(s, calc_stress, time_end, strain_end);
}

static int keep_running(const lfo_sim *s, double time_end, double strain_end)
{
	/* System::keepRunning, System.cpp:1189-1201 */
	if (s->strain > strain_end-1e-8 && strain_end >= 0) return 0;
	if (s->time > time_end-1e-8 && time_end >= 0) return 0;
	return 1;
}

int lfo_time_evolution(lfo_sim *s, double time_end, double strain_end)
{
	lfo_first_time(s);
	double adj = s->p.fixed_dt ? s->dt : 0;
	int st;
	while (keep_running(s, time_end-adj, strain_end-adj)) {
		if (!s->p.fixed_dt) adapt_time_step(s, time_end, strain_end);
		st = (s->p.integration_method == 0) ? step_euler(s, 0, time_end, strain_end)
		                                     : step_pc(s, 0, time_end, strain_end);
		if (st) return st;
	}
	if (!s->p.fixed_dt) adapt_time_step(s, time_end, strain_end);
	return (s->p.integration_method == 0) ? step_euler(s, 1, time_end, strain_end)
	                                       : step_pc(s, 1, time_end, strain_end);
}

/* ------------------------------------------------------------------ */
/* create / destroy / getters                                          */
/* ------------------------------------------------------------------ */
lfo_sim *lfo_create(const lfo_params *p, int np, const double *pos, const double *radius,
                    double lx, double ly, double lz, const double *le_disp,
                    int ncs, const int *cs_p0, const int *cs_p1, const double *cs_disp_tan)
{
	if (p->mu_rolling > 0 && p->friction_model == 0) return NULL;   /* System.cpp:386-391 */
	lfo_sim *s = calloc(1, sizeof(lfo_sim));
	s->p = *p;
	s->np = np;
	s->lx = lx; s->ly = ly; s->lz = lz;
	s->lx_half = lx/2; s->ly_half = ly/2; s->lz_half = lz/2;
	s->twodim = (ly == 0);
	s->system_volume = s->twodim ? lx*lz : lx*ly*lz;
	/* System::setupParameters*, System.cpp:394-440, 348-392 */
	s->lubrication = p->lubrication_model != 0;
	s->tangential = p->lubrication_model == 2;
	s->friction = p->friction_model != 0;
	s->rolling = p->mu_rolling > 0;
	if (!s->friction) s->p.mu_static = 0;
	if (s->p.mu_dynamic < 0) s->p.mu_dynamic = s->p.mu_static;
	s->repulsiveforce = p->repulsion_on && p->repulsive_length > 0;
	s->pairwise_resistance = s->lubrication || p->contact_relaxation_time != 0 || p->contact_relaxation_time_tan != 0;
	declare_components(s);
	size_t n = (size_t)np;
	s->pos = calloc(n, sizeof(v3)); s->vel = calloc(n, sizeof(v3)); s->ang = calloc(n, sizeof(v3));
	s->na_vel = calloc(n, sizeof(v3)); s->na_ang = calloc(n, sizeof(v3));
	s->vel_pred = calloc(n, sizeof(v3)); s->ang_pred = calloc(n, sizeof(v3)); s->u_inf = calloc(n, sizeof(v3));
	s->radius = calloc(n, sizeof(double));
	for (int c = 0; c < NFC; c++) { s->fc_force[c] = calloc(6*n, sizeof(double)); s->vc[c] = calloc(6*n, sizeof(double)); }
	for (int c = 0; c < NSC; c++) s->sc[c] = calloc(n, sizeof(s2));
	for (int i = 0; i < np; i++) {
		s->pos[i] = V(pos[3*i], pos[3*i+1], pos[3*i+2]);
		s->radius[i] = radius[i];
	}
	s->shear_disp = V(le_disp ? le_disp[0] : 0, le_disp ? le_disp[1] : 0, 0);
	s->shear_strain = vzero();
	/* shear rate: rate control sets it in exportForceAmplitudes; stress
	 * control starts from 0 (SimulationInit.cpp:276) */
	set_shear_rate(s, p->control == 0 ? p->shear_rate : 0);
	s->dt = p->dt;
	s->firsttime = 1;
	/* initializeBoxing + checkNewInteraction + setContacts, System.cpp:517-520 */
	if (check_new_interaction(s)) { lfo_destroy(s); return NULL; }
	for (int c = 0; c < ncs; c++) {
		int k = find_pair(s, cs_p0[c], cs_p1[c]);
		if (k < 0) { lfo_destroy(s); return NULL; }
		s->pairs[k].disp_tan = V(cs_disp_tan[3*c], cs_disp_tan[3*c+1], cs_disp_tan[3*c+2]);
	}
	return s;
}

void lfo_destroy(lfo_sim *s)
{
	if (!s) return;
	free(s->pos); free(s->vel); free(s->ang); free(s->na_vel); free(s->na_ang);
	free(s->vel_pred); free(s->ang_pred); free(s->u_inf); free(s->radius);
	for (int c = 0; c < NFC; c++) { free(s->fc_force[c]); free(s->vc[c]); }
	for (int c = 0; c < NSC; c++) free(s->sc[c]);
	free(s->pairs); free(s->dblocks); free(s->odrow); free(s->odcol); free(s->odblocks);
	fact_free(s->fact);
	free(s);
}

void lfo_get_scalars(const lfo_sim *s, lfo_scalars *o)
{
	memset(o, 0, sizeof *o);
	o->time = s->time; o->strain = s->strain; o->shear_rate = s->shear_rate; o->dt = s->dt;
	o->shear_disp[0] = s->shear_disp.x; o->shear_disp[1] = s->shear_disp.y;
	o->max_velocity = s->max_velocity; o->max_sliding_velocity = s->max_sliding_velocity;
	double groups[4][6];
	calc_stress(s, o->total_stress, groups);
	/* Simulation::outputData, Simulation.cpp:661-706 */
	double E[6];
	for (int e = 0; e < 6; e++) E[e] = s->Einf[e];
	double EE = doubledot(E, E);
	if (s->shear_rate != 0 && EE != 0) {
		o->viscosity = 0.5*doubledot(o->total_stress, E)/EE;
		o->N1 = (o->total_stress[0]-o->total_stress[5])/s->shear_rate;
		o->N2 = (o->total_stress[5]-o->total_stress[4])/s->shear_rate;
	}
	o->rate_prop_shearstress = s->rate_prop_shearstress;
	o->rate_indep_shearstress = s->rate_indep_shearstress;
	o->total_num_timesteps = s->total_num_timesteps;
	o->n_pairs = s->npairs;
	for (int k = 0; k < s->npairs; k++) {
		o->n_contacts += s->pairs[k].c_active;
		o->n_lub += s->pairs[k].lub_active;
		o->n_resistance_pairs += has_resistance(s, &s->pairs[k]);
	}
}

void lfo_get_particles(const lfo_sim *s, double *pos, double *vel, double *angvel,
                       double *na_vel, double *na_angvel)
{
	for (int i = 0; i < s->np; i++) {
		if (pos) { pos[3*i] = s->pos[i].x; pos[3*i+1] = s->pos[i].y; pos[3*i+2] = s->pos[i].z; }
		if (vel) { vel[3*i] = s->vel[i].x; vel[3*i+1] = s->vel[i].y; vel[3*i+2] = s->vel[i].z; }
		if (angvel) { angvel[3*i] = s->ang[i].x; angvel[3*i+1] = s->ang[i].y; angvel[3*i+2] = s->ang[i].z; }
		if (na_vel) { na_vel[3*i] = s->na_vel[i].x; na_vel[3*i+1] = s->na_vel[i].y; na_vel[3*i+2] = s->na_vel[i].z; }
		if (na_angvel) { na_angvel[3*i] = s->na_ang[i].x; na_angvel[3*i+1] = s->na_ang[i].y; na_angvel[3*i+2] = s->na_ang[i].z; }
	}
}

int lfo_get_num_pairs(const lfo_sim *s) { return s->npairs; }

void lfo_get_pairs(const lfo_sim *s, lfo_pair_out *out)
{
	for (int k = 0; k < s->npairs; k++) {
		const opair *q = &s->pairs[k];
		lfo_pair_out *o = &out[k];
		memset(o, 0, sizeof *o);
		o->p0 = q->p0; o->p1 = q->p1; o->z_offset = q->z_offset;
		o->contact_active = q->c_active; o->state = q->state;
		o->lub_active = q->lub_active; o->dashpot_active = q->dp_active;
		o->r = q->r; o->reduced_gap = q->gap;
		o->nvec[0] = q->nvec.x; o->nvec[1] = q->nvec.y; o->nvec[2] = q->nvec.z;
		o->rvec[0] = q->rvec.x; o->rvec[1] = q->rvec.y; o->rvec[2] = q->rvec.z;
		o->disp_tan[0] = q->disp_tan.x; o->disp_tan[1] = q->disp_tan.y; o->disp_tan[2] = q->disp_tan.z;
		o->f_spring_total[0] = q->fs_total.x; o->f_spring_total[1] = q->fs_total.y; o->f_spring_total[2] = q->fs_total.z;
		o->lub_coeff = q->lub_coeff; o->log_lub_coeff = q->log_lub_coeff;
		o->rep_force[0] = q->rep_force.x; o->rep_force[1] = q->rep_force.y; o->rep_force[2] = q->rep_force.z;
	}
}

int lfo_get_particle_stress(const lfo_sim *s, int comp, double *out)
{
	static const int map[8] = {SC_GU_CONTACT, SC_GU_DASHPOT, SC_GU_HYDRO, SC_GU_REPULSION, SC_ME,
	                           SC_XF_CONTACT, SC_XF_RATEINDEP, SC_XF_REPULSION};
	if (comp < 0 || comp >= 8) return -1;
	int c = map[comp];
	if (comp == 5 && s->p.control == 1) c = SC_XF_RATEPROP;
	if (!s->has_sc[c]) return -1;
	for (int i = 0; i < s->np; i++) for (int e = 0; e < 6; e++) out[6*i+e] = s->sc[c][i].e[e];
	return 0;
}

int lfo_get_velocity_component(const lfo_sim *s, int comp, double *out)
{
	if (comp < 0 || comp >= NFC || !s->has_fc[comp]) return -1;
	memcpy(out, s->vc[comp], sizeof(double)*6*s->np);
	return 0;
}

void lfo_factor_stats(const lfo_sim *s, double *out4)
{
	out4[0] = (double)s->n_factor;
	out4[1] = s->last_factor_flops;
	out4[2] = s->analyze_s;
	out4[3] = s->factor_s;
}

// lfdem_ref_harness.cpp -- drives LF_DEM's own System (compiled unmodified
// from the reference sources) one time step at a time and dumps its state, so
// that the CPU restatement in oracle/lfdem_oracle.c can be pinned against the
// reference.  TEST INFRASTRUCTURE ONLY; built into oracle/_ref by
// oracle/Makefile, never shipped.
//
// usage: lfdem_ref_harness CONF PARAMS r|s VALUE SUFFIX NSTEPS OUTDIR [CALC_STRESS]
//   Runs Simulation::setupSimulation (SimulationInit.cpp:620-743) exactly as
//   the LF_DEM binary does for "-r VALUE SUFFIX" / "-s VALUE SUFFIX", then for
//   each step k writes OUTDIR/step_<k>.bin with the state before the step,
//   the reference's R_FU, force / velocity / stress components at that state
//   (System::computeVelocities(true) + calcStressPerParticle, which leave the
//   trajectory untouched), and the state after
//   System::timeEvolutionPredictorCorrectorMethod (System.cpp:888-983).
//
// Private members are read through the "#define private public" test idiom
// below; no reference source is modified.
#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <map>
#include <memory>
#include <queue>
#include <random>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>
#include <csignal>
#include <getopt.h>
#include <unistd.h>
#include <climits>
#define private public
#define protected public
#include "Simulation.h"
#include "States.h"
#undef private
#undef protected

#include "../lfdem_oracle.h"
#include <chrono>

// main.cpp:25 defines this flag; the harness replaces main.cpp.
volatile sig_atomic_t sig_caught = 0;

// scipy's OpenBLAS (linked by oracle/Makefile's ref target)
extern "C" {
void scipy_dpotrf_(const char *, const int *, double *, const int *, int *);
void scipy_dtrsm_(const char *, const char *, const char *, const char *, const int *, const int *, const double *,
                  const double *, const int *, double *, const int *);
void scipy_dsyrk_(const char *, const char *, const int *, const int *, const double *, const double *, const int *,
                  const double *, double *, const int *);
void scipy_dgemm_(const char *, const char *, const int *, const int *, const int *, const double *, const double *,
                  const int *, const double *, const int *, const double *, double *, const int *);
void scipy_openblas_set_num_threads(int);
}

static FILE *g_out = nullptr;

static void put(const char *name, const double *v, size_t n)
{
	uint32_t l = (uint32_t)strlen(name);
	fwrite(&l, 4, 1, g_out); fwrite(name, 1, l, g_out);
	char t = 'd'; fwrite(&t, 1, 1, g_out);
	uint64_t c = n; fwrite(&c, 8, 1, g_out);
	if (n) fwrite(v, sizeof(double), n, g_out);
}
static void puti(const char *name, const int *v, size_t n)
{
	uint32_t l = (uint32_t)strlen(name);
	fwrite(&l, 4, 1, g_out); fwrite(name, 1, l, g_out);
	char t = 'i'; fwrite(&t, 1, 1, g_out);
	uint64_t c = n; fwrite(&c, 8, 1, g_out);
	if (n) fwrite(v, sizeof(int), n, g_out);
}
static void put1(const char *name, double v) { put(name, &v, 1); }

static void put_vec3(const char *name, const std::vector<vec3d> &v)
{
	std::vector<double> a(3*v.size());
	for (size_t i = 0; i < v.size(); i++) { a[3*i] = v[i].x; a[3*i+1] = v[i].y; a[3*i+2] = v[i].z; }
	put(name, a.data(), a.size());
}

static void dump_pairs(System &sys, const char *prefix)
{
	size_t n = sys.interaction.size();
	std::vector<int> ip(n*6);
	std::vector<double> dp(n*23);
	for (size_t k = 0; k < n; k++) {
		Interaction &in = sys.interaction[k];
		auto pr = in.get_par_num();
		ip[6*k+0] = (int)pr.first;
		ip[6*k+1] = (int)pr.second;
		ip[6*k+2] = in.contact.is_active();
		ip[6*k+3] = in.contact.getFrictionState();
		ip[6*k+4] = sys.lubrication ? in.lubrication.is_active() : 0;
		ip[6*k+5] = in.z_offset;
		double *d = &dp[23*k];
		d[0] = in.separation_distance();
		d[1] = in.get_reduced_gap();
		d[2] = in.nvec.x; d[3] = in.nvec.y; d[4] = in.nvec.z;
		d[5] = in.contact.disp_tan.x; d[6] = in.contact.disp_tan.y; d[7] = in.contact.disp_tan.z;
		d[8] = in.contact.f_spring_total.x; d[9] = in.contact.f_spring_total.y; d[10] = in.contact.f_spring_total.z;
		d[11] = sys.lubrication ? in.lubrication.lub_coeff : 0;
		d[12] = sys.lubrication ? in.lubrication.log_lub_coeff : 0;
		vec3d rf = in.repulsion.getForceVector();
		d[13] = rf.x; d[14] = rf.y; d[15] = rf.z;
		d[16] = in.rvec.x; d[17] = in.rvec.y; d[18] = in.rvec.z;
		d[19] = in.contact.relative_surface_velocity_sqnorm;
		d[20] = in.contact.disp_rolling.x; d[21] = in.contact.disp_rolling.y; d[22] = in.contact.disp_rolling.z;
	}
	std::string a = std::string(prefix)+"pairs_i", b = std::string(prefix)+"pairs_d";
	puti(a.c_str(), ip.data(), ip.size());
	put(b.c_str(), dp.data(), dp.size());
}

static void dump_scalars(System &sys, const char *prefix)
{
	std::string p(prefix);
	put1((p+"time").c_str(), sys.get_time());
	put1((p+"strain").c_str(), sys.get_cumulated_strain());
	put1((p+"shear_rate").c_str(), sys.get_shear_rate());
	put1((p+"dt").c_str(), sys.dt);
	put1((p+"max_velocity").c_str(), sys.max_velocity);
	put1((p+"max_sliding_velocity").c_str(), sys.max_sliding_velocity);
	double sd[2] = {sys.shear_disp.x, sys.shear_disp.y};
	put((p+"shear_disp").c_str(), sd, 2);
	put_vec3((p+"position").c_str(), sys.position);
	put_vec3((p+"velocity").c_str(), sys.velocity);
	put_vec3((p+"ang_velocity").c_str(), sys.ang_velocity);
	put_vec3((p+"na_velocity").c_str(), sys.na_velocity);
	put_vec3((p+"na_ang_velocity").c_str(), sys.na_ang_velocity);
}

static void dump_components(System &sys, const char *prefix)
{
	std::string p(prefix);
	for (auto &fc : sys.force_components) {
		std::vector<double> a(6*sys.np);
		for (int i = 0; i < sys.np; i++) {
			a[6*i] = fc.second.force[i].x; a[6*i+1] = fc.second.force[i].y; a[6*i+2] = fc.second.force[i].z;
			a[6*i+3] = fc.second.torque[i].x; a[6*i+4] = fc.second.torque[i].y; a[6*i+5] = fc.second.torque[i].z;
		}
		put((p+"force_"+fc.first).c_str(), a.data(), a.size());
	}
	for (auto &vc : sys.na_velo_components) {
		std::vector<double> a(6*sys.np);
		for (int i = 0; i < sys.np; i++) {
			a[6*i] = vc.second.vel[i].x; a[6*i+1] = vc.second.vel[i].y; a[6*i+2] = vc.second.vel[i].z;
			a[6*i+3] = vc.second.ang_vel[i].x; a[6*i+4] = vc.second.ang_vel[i].y; a[6*i+5] = vc.second.ang_vel[i].z;
		}
		put((p+"velcomp_"+vc.first).c_str(), a.data(), a.size());
	}
	for (auto &sc : sys.stress_components) {
		std::vector<double> a(6*sys.np);
		for (int i = 0; i < sys.np; i++)
			for (int e = 0; e < 6; e++) a[6*i+e] = sc.second.particle_stress[i].elm[e];
		put((p+"stress_"+sc.first).c_str(), a.data(), a.size());
	}
}

static void dump_matrix(System &sys, const char *prefix)
{
	cholmod_sparse *A = sys.stokes_solver.chol_res_matrix;
	std::string p(prefix);
	if (!A) return;
	size_t n = A->ncol;
	const int *ap = (const int *)A->p;
	puti((p+"csc_p").c_str(), ap, n+1);
	puti((p+"csc_i").c_str(), (const int *)A->i, (size_t)ap[n]);
	put((p+"csc_x").c_str(), (const double *)A->x, (size_t)ap[n]);
}

int main(int argc, char **argv)
{
	if (argc < 8) {
		fprintf(stderr, "usage: %s CONF PARAMS r|s VALUE SUFFIX NSTEPS OUTDIR [CALC_STRESS] [STAGE]\n", argv[0]);
		return 2;
	}
	char buf[4096];
	std::string conf = realpath(argv[1], buf) ? std::string(buf) : std::string(argv[1]);
	std::string params = realpath(argv[2], buf) ? std::string(buf) : std::string(argv[2]);
	bool stress = argv[3][0] == 's';
	double value = atof(argv[4]);
	std::string suffix = argv[5];
	int nsteps = atoi(argv[6]);
	std::string outdir = realpath(argv[7], buf) ? std::string(buf) : std::string(argv[7]);
	// the reference opens its output files in the working directory
	if (chdir(outdir.c_str()) != 0) { perror("chdir"); return 2; }
	int calc_stress = argc > 8 ? atoi(argv[8]) : 0;
	int stage = argc > 9 ? atoi(argv[9]) : 1;

	// HARNESS_SUPERNODAL: CHOLMOD's calls go to the oracle's supernodal
	// block factorisation with OpenBLAS kernels (the method of CHOLMOD's
	// supernodal factorisation) instead of the dense stand-in
	if (getenv("HARNESS_SUPERNODAL")) {
		lfo_set_blas((void *)scipy_dpotrf_, (void *)scipy_dtrsm_, (void *)scipy_dsyrk_, (void *)scipy_dgemm_,
		             (void *)scipy_openblas_set_num_threads, lfo_num_threads());
		cholmod_compat_use_blocks(1);
	}
	std::cout.setstate(std::ios_base::failbit);
	Simulation sim;
	sim.sys.ext_flow = false;
	sim.control_var = stress ? ControlVariable::stress : ControlVariable::rate;
	std::vector<std::string> files = {conf, params, "not_given", "not_given"};
	bool binary_conf = conf.size() > 4 && conf.substr(conf.size()-4) == ".bin";
	sim.setupSimulation("harness", files, binary_conf, value, suffix, "shear", "");
	std::cout.clear();
	System &sys = sim.getSys();
	// Prevent std::vector<Interaction> reallocation: its copy path re-runs
	// Interaction::activateForceMembers on every interaction
	// (Interaction.cpp:38-55), which would reset all tangential springs.
	sys.interaction.reserve(64*(size_t)sys.np+1024);

	// resolved, non-dimensionalised parameters
	{
		std::string f = outdir+"/params.bin";
		g_out = fopen(f.c_str(), "wb");
		ParameterSet &p = sys.p;
		put1("kn", p.kn); put1("kt", p.kt); put1("mu_static", p.mu_static); put1("mu_dynamic", p.mu_dynamic);
		put1("critical_load", p.critical_load); put1("ft_max", p.ft_max); put1("friction_model", p.friction_model);
		put1("repulsion_on", sys.repulsiveforce ? 1 : 0); put1("repulsion", p.repulsion);
		put1("repulsive_length", p.repulsive_length); put1("repulsive_max_length", p.repulsive_max_length);
		double lm = p.lubrication_model == "none" ? 0 : (p.lubrication_model == "normal" ? 1 : 2);
		put1("lubrication_model", lm);
		put1("lub_reduce_parameter", p.lub_reduce_parameter); put1("lub_max_gap", p.lub_max_gap);
		put1("interaction_range", p.interaction_range); put1("sd_coeff", p.sd_coeff);
		put1("contact_relaxation_time", p.contact_relaxation_time);
		put1("contact_relaxation_time_tan", p.contact_relaxation_time_tan);
		put1("disp_max", p.disp_max); put1("dt", p.dt); put1("dt_max", p.dt_max); put1("dt_min", p.dt_min);
		put1("fixed_dt", p.fixed_dt ? 1 : 0); put1("integration_method", p.integration_method);
		put1("control", stress ? 1 : 0); put1("shear_rate", sys.get_shear_rate());
		put1("target_stress", sys.target_stress);
		put("Ehat", sys.Ehat_infinity.elm, 6);
		double oh[3] = {sys.omegahat_inf.x, sys.omegahat_inf.y, sys.omegahat_inf.z};
		put("Ohat", oh, 3);
		put1("init_strain_shear_rate_limit", sys.init_strain_shear_rate_limit);
		put1("init_shear_rate_limit", sys.init_shear_rate_limit);
		put1("mu_rolling", sys.rolling_friction ? p.mu_rolling : 0.0);
		put1("kr", sys.rolling_friction ? p.kr : 0.0);
		put1("brownian", sys.brownian ? p.brownian : 0.0);
		put1("lx", sys.get_lx()); put1("ly", sys.get_ly()); put1("lz", sys.get_lz());
		put("radius", sys.radius.data(), sys.radius.size());
		put_vec3("position0", sys.position);
		double sd[2] = {sys.shear_disp.x, sys.shear_disp.y};
		put("shear_disp0", sd, 2);
		put1("time_end", sim.time_end); put1("strain_end", sim.strain_end);
		fclose(g_out);
	}

	// Output mode: with HARNESS_OUTPUT_DSTRAIN set, the reference's own
	// System::timeEvolution runs to strains k * DSTRAIN (k = 1..NSTEPS), each
	// followed by Simulation::generateOutput with "data" and "config"
	// (Simulation.cpp:145-163), which writes data_/st_/par_/int_ into OUTDIR
	// (the files Simulation::setupSimulation opened there).
	if (const char *ods = getenv("HARNESS_OUTPUT_DSTRAIN")) {
		double ds = atof(ods);
		int counter = 0;
		std::cout.setstate(std::ios_base::failbit);
		for (int k = 1; k <= nsteps; k++) {
			sys.timeEvolution(-1, k*ds);
			std::set<std::string> ev = {"data", "config"};
			sim.generateOutput(ev, counter);
		}
		std::cout.clear();
		return 0;
	}
	// Timing mode: with HARNESS_TIME_STEPS set, the reference's own time
	// step (System::adaptTimeStep + timeEvolutionPredictorCorrectorMethod,
	// the loop of System::timeEvolution, System.cpp:1243-1250) runs
	// HARNESS_WARMUP steps (default 1), then HARNESS_TIME_STEPS steps are
	// timed (wall clock) and reported on stdout in one line.
	if (const char *ts = getenv("HARNESS_TIME_STEPS")) {
		int K = atoi(ts), W = getenv("HARNESS_WARMUP") ? atoi(getenv("HARNESS_WARMUP")) : 1;
		std::cout.setstate(std::ios_base::failbit);
		sys.timeEvolution(-1, 0);   // the first-time set-up (and one stress step)
		auto loop = [&](int nsteps) {
			for (int k = 0; k < nsteps; k++) {
				if (!sys.brownian && !sys.p.fixed_dt) sys.adaptTimeStep(-1, 1e9);
				if (sys.p.integration_method == 0) sys.timeEvolutionEulersMethod(false, -1, 1e9);
				else sys.timeEvolutionPredictorCorrectorMethod(false, -1, 1e9);
			}
		};
		loop(W);
		auto t0 = std::chrono::steady_clock::now();
		loop(K);
		double sec = std::chrono::duration<double>(std::chrono::steady_clock::now()-t0).count();
		std::cout.clear();
		printf("steps %d seconds %.3f particle_steps_per_s %.1f np %d threads %d supernodal %d\n", K, sec,
		       (double)sys.np*K/sec, sys.np, lfo_num_threads(), getenv("HARNESS_SUPERNODAL") ? 1 : 0);
		return 0;
	}
	// System::timeEvolution first-time block (System.cpp:1216-1226)
	{
		double dt_bak = sys.dt;
		sys.dt = 0;
		sys.checkNewInteraction();
		sys.in_predictor = true;
		sys.updateInteractions();
		sys.in_predictor = false;
		sys.dt = dt_bak;
	}
	const double time_end = -1, strain_end = 1e9;
	for (int k = 0; k < nsteps; k++) {
		char fn[512];
		snprintf(fn, sizeof fn, "%s/step_%04d.bin", outdir.c_str(), k);
		g_out = fopen(fn, "wb");
		dump_scalars(sys, "pre_");
		dump_pairs(sys, "pre_");
		if (stage) {
			sys.in_predictor = false; sys.in_corrector = false;
			sys.computeVelocities(true);
			dump_matrix(sys, "stage_");
			sys.calcStressPerParticle();
			dump_components(sys, "stage_");
			dump_scalars(sys, "stage_");
		}
		// System::timeEvolution's loop (System.cpp:1243-1245): no adaptive step
		// with Brownian forces
		if (!sys.brownian && !sys.p.fixed_dt) sys.adaptTimeStep(time_end, strain_end);
		if (sys.p.integration_method == 0) sys.timeEvolutionEulersMethod(calc_stress, time_end, strain_end);
		else sys.timeEvolutionPredictorCorrectorMethod(calc_stress, time_end, strain_end);
		dump_scalars(sys, "post_");
		dump_pairs(sys, "post_");
		if (sys.brownian) {
			// the Brownian force of this step (drawn in the predictor, kept for
			// the corrector: System::setBrownianForceToParticle)
			const auto &fcb = sys.force_components["brownian"];
			std::vector<double> fb(6*(size_t)sys.np);
			for (int i = 0; i < sys.np; i++) {
				fb[6*i] = fcb.force[i].x; fb[6*i+1] = fcb.force[i].y; fb[6*i+2] = fcb.force[i].z;
				fb[6*i+3] = fcb.torque[i].x; fb[6*i+4] = fcb.torque[i].y; fb[6*i+5] = fcb.torque[i].z;
			}
			put("post_brownian_force", fb.data(), fb.size());
		}
		if (calc_stress) {
			dump_components(sys, "post_");
			sys.calcStress();
			put("post_total_stress", sys.total_stress.elm, 6);
		}
		fclose(g_out);
	}
	// checkpoint of the final state in the reference's own formats
	// (Simulation::checkpoint, Simulation.cpp:602-611)
	sim.outputConfigurationBinary(outdir+"/conf.bin");
	State::outputStateBinary(outdir+"/chk.bin", sys);
	return 0;
}

// StokesSolverGB300.cpp -- LF_DEM's StokesSolver backed by the GB300 engine.
//
// Compiled into LF_DEM in place of StokesSolver.cpp (the class declaration in
// StokesSolver.h is kept as it is; it still names CHOLMOD types in its
// private members, so a cholmod.h must be on the include path, but none of
// those members is used and nothing from CHOLMOD is called).  Every method
// that the rest of LF_DEM calls (StokesSolver.h:198-285) is defined here on
// top of the C ABI of include/lfdem_gb300.h:
//
//   init                       lfg_solver_create (6 unknowns per particle)
//   resetResistanceMatrix,     host copies of the compact blocks (DBlock: 15
//   startNewColumn,            doubles, ODBlock: 18, in MatrixBlocks.h's
//   addResistanceBlocks        column order)
//   matrixFillingDone          lfg_solver_set_blocks + lfg_solver_factorize
//   resetRHS ... setRHSTorque  a host right-hand side, 6 values per particle
//   solve                      lfg_solver_solve
//   compute_LTRHS              lfg_solver_multiply_factor
//
// The solver state lives in a table keyed by the StokesSolver object, since
// the unmodified class declaration has no member for it.  Errors of the
// engine are thrown as std::runtime_error, which LF_DEM's main catches.
// Only mobile particles are supported: the mixed problem (fixed-velocity
// particles, walls) and the testing helpers throw.
//
// Environment: LFDEM_GB300_PRECISION=fp32 selects the FP32 factor with FP64
// refinement (default: the FP64 factor); LFDEM_GB300_DEVICE picks the device.
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "StokesSolver.h"
#include "lfdem_gb300.h"

namespace {

struct GpuState {
	lfg_solver *h = nullptr;
	int n = 0;
	bool pattern_changed = true;
	bool analysed = false;
	std::vector<double> dblocks;     // n x 15
	std::vector<int32_t> od_row, od_col;
	std::vector<double> odblocks;    // 18 per off-diagonal block
	std::vector<double> rhs, x;      // 6 n
};

std::mutex g_mu;
std::map<const StokesSolver *, GpuState> g_state;

GpuState &state(const StokesSolver *s)
{
	std::lock_guard<std::mutex> lk(g_mu);
	return g_state[s];
}

void check(int rc, const lfg_status &st, const char *what)
{
	if (rc != LFG_OK)
		throw std::runtime_error(std::string("StokesSolver (GB300) ") + what + ": " + st.msg +
		                         " (status " + std::to_string(rc) + ")");
}

// MatrixBlocks.h column order: col0[5] col1[3] col2[1] col3[3] col4[2] col5[1]
void add_dblock(const DBlock &b, double *d)
{
	int k = 0;
	for (double v : b.col0) d[k++] += v;
	for (double v : b.col1) d[k++] += v;
	for (double v : b.col2) d[k++] += v;
	for (double v : b.col3) d[k++] += v;
	for (double v : b.col4) d[k++] += v;
	for (double v : b.col5) d[k++] += v;
}

// col0[5] col1[3] col2[1] col3[5] col4[3] col5[1]
void push_odblock(const ODBlock &b, std::vector<double> &o)
{
	o.insert(o.end(), b.col0.begin(), b.col0.end());
	o.insert(o.end(), b.col1.begin(), b.col1.end());
	o.insert(o.end(), b.col2.begin(), b.col2.end());
	o.insert(o.end(), b.col3.begin(), b.col3.end());
	o.insert(o.end(), b.col4.begin(), b.col4.end());
	o.insert(o.end(), b.col5.begin(), b.col5.end());
}

[[noreturn]] void unsupported(const char *what)
{
	throw std::runtime_error(std::string("StokesSolver (GB300): ") + what +
	                         " is not supported by the GB300 engine (mobile particles only)");
}

} // namespace

StokesSolver::StokesSolver() : np(0), mobile_particle_nb(0), fixed_particle_nb(0), mobile_matrix_done(false),
                               to_be_factorized(false), chol_L(nullptr), chol_rhs(nullptr),
                               chol_res_matrix(nullptr), chol_res_matrix_mf(nullptr), chol_res_matrix_ff(nullptr),
                               chol_solution(nullptr), chol_solveE_workspace(nullptr),
                               chol_solveY_workspace(nullptr), chol_vel_mob(nullptr), chol_vel_fix(nullptr),
                               chol_force_mob(nullptr), chol_force_fix(nullptr), chol_Psolution(nullptr),
                               dblocks_size(0), current_column(0)
{
}

StokesSolver::~StokesSolver()
{
	std::lock_guard<std::mutex> lk(g_mu);
	auto it = g_state.find(this);
	if (it != g_state.end()) {
		if (it->second.h) lfg_solver_destroy(it->second.h);
		g_state.erase(it);
	}
}

void StokesSolver::init(chol_int np_total, chol_int np_mobile)
{
	np = np_total;
	mobile_particle_nb = np_mobile;
	fixed_particle_nb = np_total-np_mobile;
	if (fixed_particle_nb != 0) unsupported("the mixed problem (fixed-velocity particles)");
	GpuState &g = state(this);
	if (g.h) lfg_solver_destroy(g.h);
	lfg_options opt;
	lfg_default_options(&opt);
	const char *prec = std::getenv("LFDEM_GB300_PRECISION");
	if (prec && std::string(prec) == "fp32") opt.precision = LFG_PREC_FP32_REFINE;
	const char *dev = std::getenv("LFDEM_GB300_DEVICE");
	if (dev) opt.device = std::atoi(dev);
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	check(lfg_solver_create((int)np_mobile, 6, &opt, &g.h, &st), st, "create");
	g.n = (int)np_mobile;
	g.dblocks.assign(15*(size_t)g.n, 0.0);
	g.rhs.assign(6*(size_t)g.n, 0.0);
	g.x.assign(6*(size_t)g.n, 0.0);
	g.analysed = false;
}

void StokesSolver::resetResistanceMatrix(chol_int nb_of_interactions_mm, chol_int nb_of_interactions_mf,
                                         chol_int nb_of_interactions_ff,
                                         const std::vector<struct DBlock> &reset_resmat_dblocks,
                                         bool matrix_pattern_changed)
{
	if (nb_of_interactions_mf != 0 || nb_of_interactions_ff != 0) unsupported("the mixed problem");
	GpuState &g = state(this);
	g.pattern_changed = matrix_pattern_changed || !g.analysed;
	std::fill(g.dblocks.begin(), g.dblocks.end(), 0.0);
	for (int i = 0; i < g.n && i < (int)reset_resmat_dblocks.size(); i++)
		add_dblock(reset_resmat_dblocks[i], &g.dblocks[15*(size_t)i]);
	g.od_row.clear();
	g.od_col.clear();
	g.odblocks.clear();
	g.od_row.reserve(nb_of_interactions_mm);
	g.od_col.reserve(nb_of_interactions_mm);
	g.odblocks.reserve(18*(size_t)nb_of_interactions_mm);
	current_column = -1;
	mobile_matrix_done = false;
}

void StokesSolver::startNewColumn()
{
	current_column++;
}

void StokesSolver::addResistanceBlocks(chol_int i, chol_int j,
                                       const std::pair<struct DBlock, struct DBlock> &DiagBlocks_i_and_j,
                                       const struct ODBlock &ODBlock_ij)
{
	GpuState &g = state(this);
	if (i >= j || j >= g.n) throw std::runtime_error("StokesSolver (GB300): addResistanceBlocks needs i < j < np");
	add_dblock(DiagBlocks_i_and_j.first, &g.dblocks[15*(size_t)i]);
	add_dblock(DiagBlocks_i_and_j.second, &g.dblocks[15*(size_t)j]);
	g.od_row.push_back((int32_t)j);
	g.od_col.push_back((int32_t)i);
	push_odblock(ODBlock_ij, g.odblocks);
}

void StokesSolver::matrixFillingDone()
{
	GpuState &g = state(this);
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	check(lfg_solver_set_blocks(g.h, g.dblocks.data(), (int)g.od_row.size(), g.od_row.data(), g.od_col.data(),
	                            g.odblocks.data(), g.pattern_changed ? 1 : 0, nullptr, &st), st, "set_blocks");
	check(lfg_solver_factorize(g.h, &st), st, "factorize");
	g.analysed = true;
	mobile_matrix_done = true;
}

void StokesSolver::resetRHS()
{
	GpuState &g = state(this);
	std::fill(g.rhs.begin(), g.rhs.end(), 0.0);
}

void StokesSolver::resetRHStorque()
{
	GpuState &g = state(this);
	for (int i = 0; i < g.n; i++)
		for (int d = 3; d < 6; d++) g.rhs[6*(size_t)i+d] = 0.0;
}

void StokesSolver::addToRHSForce(chol_int i, const vec3d &force_i)
{
	GpuState &g = state(this);
	if (i >= g.n) return;
	g.rhs[6*i] += force_i.x; g.rhs[6*i+1] += force_i.y; g.rhs[6*i+2] += force_i.z;
}

void StokesSolver::addToRHSTorque(chol_int i, const vec3d &torque_i)
{
	GpuState &g = state(this);
	if (i >= g.n) return;
	g.rhs[6*i+3] += torque_i.x; g.rhs[6*i+4] += torque_i.y; g.rhs[6*i+5] += torque_i.z;
}

void StokesSolver::addToRHS(double *rhs)
{
	GpuState &g = state(this);
	for (size_t k = 0; k < g.rhs.size(); k++) g.rhs[k] += rhs[k];
}

void StokesSolver::addToRHS(const std::vector<double> &force)
{
	GpuState &g = state(this);
	for (size_t k = 0; k < force.size() && k < g.rhs.size(); k++) g.rhs[k] += force[k];
}

void StokesSolver::addToRHS(chol_int first_particle, const std::vector<double> &force)
{
	GpuState &g = state(this);
	size_t shift = 6*(size_t)first_particle;
	for (size_t k = 0; k < force.size() && shift+k < g.rhs.size(); k++) g.rhs[shift+k] += force[k];
}

// forces and torques interleaved as vec3d pairs (F_0, T_0, F_1, T_1, ...)
void StokesSolver::setRHS(const std::vector<vec3d> &force_and_torque)
{
	GpuState &g = state(this);
	for (int i = 0; i < 2*g.n; i++) {
		g.rhs[3*(size_t)i] = force_and_torque[i].x;
		g.rhs[3*(size_t)i+1] = force_and_torque[i].y;
		g.rhs[3*(size_t)i+2] = force_and_torque[i].z;
	}
}

void StokesSolver::setRHS(const std::vector<vec3d> &force, const std::vector<vec3d> &torque)
{
	GpuState &g = state(this);
	vec3dToDouble(g.rhs.data(), force, torque);
}

void StokesSolver::setRHSForce(chol_int i, const vec3d &force_i)
{
	GpuState &g = state(this);
	if (i >= g.n) return;
	g.rhs[6*i] = force_i.x; g.rhs[6*i+1] = force_i.y; g.rhs[6*i+2] = force_i.z;
}

void StokesSolver::setRHSTorque(chol_int i, const vec3d &torque_i)
{
	GpuState &g = state(this);
	if (i >= g.n) return;
	g.rhs[6*i+3] = torque_i.x; g.rhs[6*i+4] = torque_i.y; g.rhs[6*i+5] = torque_i.z;
}

void StokesSolver::solve(std::vector<vec3d> &velocity, std::vector<vec3d> &ang_velocity)
{
	GpuState &g = state(this);
	if ((size_t)g.n > velocity.size() || (size_t)g.n > ang_velocity.size())
		throw std::runtime_error(" StokesSolver::solve: allocated solution vector too small");
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	check(lfg_solver_solve(g.h, 1, g.rhs.data(), g.x.data(), &st), st, "solve");
	for (int i = 0; i < g.n; i++) {
		velocity[i].x = g.x[6*(size_t)i];
		velocity[i].y = g.x[6*(size_t)i+1];
		velocity[i].z = g.x[6*(size_t)i+2];
		ang_velocity[i].x = g.x[6*(size_t)i+3];
		ang_velocity[i].y = g.x[6*(size_t)i+4];
		ang_velocity[i].z = g.x[6*(size_t)i+5];
	}
}

void StokesSolver::solve(vec3d *velocity, vec3d *ang_velocity)
{
	GpuState &g = state(this);
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	check(lfg_solver_solve(g.h, 1, g.rhs.data(), g.x.data(), &st), st, "solve");
	for (int i = 0; i < g.n; i++) {
		velocity[i].set(g.x[6*(size_t)i], g.x[6*(size_t)i+1], g.x[6*(size_t)i+2]);
		ang_velocity[i].set(g.x[6*(size_t)i+3], g.x[6*(size_t)i+4], g.x[6*(size_t)i+5]);
	}
}

// The Brownian force's L psi with this engine's factor (another square root
// of R than CHOLMOD's permuted one; the covariance L L^T = R is the same)
void StokesSolver::compute_LTRHS(std::vector<vec3d> &F, std::vector<vec3d> &T)
{
	GpuState &g = state(this);
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	check(lfg_solver_multiply_factor(g.h, 1, g.rhs.data(), g.x.data(), &st), st, "multiply_factor");
	doubleToVec3d(g.x.data(), F, T);
}

void StokesSolver::solvingIsDone()
{
	// the factor stays on the device until the next matrixFillingDone
}

void StokesSolver::vec3dToDouble(double *a, const std::vector<vec3d> &b, const std::vector<vec3d> &c)
{
	for (size_t i = 0; i < b.size(); i++) {
		a[6*i] = b[i].x; a[6*i+1] = b[i].y; a[6*i+2] = b[i].z;
		a[6*i+3] = c[i].x; a[6*i+4] = c[i].y; a[6*i+5] = c[i].z;
	}
}

void StokesSolver::doubleToVec3d(double *a, std::vector<vec3d> &b, std::vector<vec3d> &c)
{
	for (size_t i = 0; i < b.size(); i++) {
		b[i].set(a[6*i], a[6*i+1], a[6*i+2]);
		c[i].set(a[6*i+3], a[6*i+4], a[6*i+5]);
	}
}

void StokesSolver::printResistanceMatrix(std::ostream &out, std::string)
{
	lfg_solver_stats s;
	GpuState &g = state(this);
	if (g.h && lfg_solver_get_stats(g.h, &s) == LFG_OK)
		out << "# GB300 resistance solver: " << s.n_blocks << " particles, " << g.od_row.size()
		    << " off-diagonal blocks, " << s.n_supernodes << " supernodes, nnz(L) " << s.nnz_L << "\n";
}

void StokesSolver::printFactor(std::ostream &out)
{
	printResistanceMatrix(out, "");
}

void StokesSolver::printRHS()
{
	GpuState &g = state(this);
	for (double v : g.rhs) std::cout << v << "\n";
}

void StokesSolver::convertDirectToIterative() { unsupported("convertDirectToIterative"); }
void StokesSolver::multiply_by_RFU_mm(std::vector<double> &, std::vector<double> &) { unsupported("multiply_by_RFU_mm"); }
void StokesSolver::multiply_by_RFU_mf(std::vector<double> &, std::vector<double> &) { unsupported("multiply_by_RFU_mf"); }
void StokesSolver::multiply_by_RFU_fm(std::vector<double> &, std::vector<double> &) { unsupported("multiply_by_RFU_fm"); }
void StokesSolver::multiply_by_RFU_fm(std::vector<vec3d> &, std::vector<vec3d> &, std::vector<vec3d> &,
                                      std::vector<vec3d> &)
{
	unsupported("multiply_by_RFU_fm");
}
void StokesSolver::multiply_by_RFU_ff(std::vector<double> &, std::vector<double> &) { unsupported("multiply_by_RFU_ff"); }
void StokesSolver::multiply_by_RFU_ff(std::vector<vec3d> &, std::vector<vec3d> &, std::vector<vec3d> &,
                                      std::vector<vec3d> &)
{
	unsupported("multiply_by_RFU_ff");
}
void StokesSolver::multiplyByResMat(double *) { unsupported("multiplyByResMat (a testing function)"); }
void StokesSolver::multiplySolutionByResMat(double *) { unsupported("multiplySolutionByResMat (a testing function)"); }

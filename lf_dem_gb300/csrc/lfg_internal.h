// lfg_internal.h -- internal declarations shared by the host driver (C++) and
// the CUDA translation units of the GB300 engine.  Not part of the C ABI.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/lfdem_gb300.h"

namespace lfg {

// ---------------------------------------------------------------------------
// error handling: every CUDA call in the host driver goes through LFG_CUDA,
// which throws lfg::Error; the C-ABI layer converts it to a status code.
// ---------------------------------------------------------------------------
struct Error {
	int code;
	int info;
	std::string msg;
};

#define LFG_CUDA(call)                                                                     \
	do {                                                                                   \
		cudaError_t e_ = (call);                                                       \
		if (e_ != cudaSuccess)                                                         \
			throw ::lfg::Error{e_ == cudaErrorMemoryAllocation ? LFG_ERR_OOM : LFG_ERR_CUDA, \
			                   (int)e_, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
	} while (0)

// ---------------------------------------------------------------------------
// Symbolic analysis of the block matrix (nested dissection + multifrontal
// assembly tree).  Computed on the host, mirrored to the device.
// ---------------------------------------------------------------------------
struct Symbolic {
	int nblk = 0;                 // particles (dof x dof blocks)
	int dof = 6;                  // scalar unknowns per particle: 6, or 3 for the in-plane part of a 2D system
	std::vector<int> perm;        // perm[k] = particle at permuted position k
	std::vector<int> iperm;       // iperm[particle] = permuted position
	// supernodes, in postorder (children before parents)
	int nsn = 0;
	std::vector<int> sn_first, sn_n, sn_m, sn_parent, sn_level;
	std::vector<int> sn_rows_off;     // into rows[] (m entries each, permuted block ids)
	std::vector<int> rows;
	std::vector<int64_t> sn_off;      // front arena offsets (elements)
	std::vector<int> sn_ld;           // front leading dimension = 6F + 6n
	std::vector<int64_t> sn_woff;     // forward-solve update vector offsets (elements)
	// children and inverse maps: for child c of parent p, inv[cinv_off[c] + b]
	// (b in [0, F_p)) = child front block index or -1
	std::vector<int> child_off, children;   // CSR over supernodes
	std::vector<int64_t> cinv_off;
	std::vector<int> cinv;
	// cfwd[sn_rows_off[c] + t]: parent front block of child c's update block t
	std::vector<int> cfwd;
	// levels (0 = leaves)
	int nlevels = 0;
	std::vector<int> level_off, level_sn;   // CSR: supernodes of each level
	// A-block scatter: for each particle (D block) and each off-diagonal
	// block e (in the caller's order): target supernode, front block row/col,
	// transpose flag.
	std::vector<int> d_sn, d_bc;
	std::vector<int> od_sn, od_br, od_bc, od_tr;
	std::vector<int> level_d_off, level_d;     // D blocks per level
	std::vector<int> level_od_off, level_od;   // OD blocks per level
	int64_t arena_elems = 0;
	int64_t w_elems = 0;
	int max_F = 0;
	int64_t nnz_L = 0;
	double flops = 0;
};

// Build the symbolic analysis.  od_row/od_col: nb lower off-diagonal blocks
// (the pattern).  pos (3 * nblk, may be null) drives a geometric nested
// dissection; otherwise a breadth-first level-set dissection is used.
// dof: scalar unknowns per particle (6; 3 for the in-plane x, z translation
// and y rotation of a 2D system); it scales the front sizes only.
void symbolic_analyze(Symbolic &S, int nblk, int nb, const int32_t *od_row,
                      const int32_t *od_col, const double *pos, double lx, double ly, double lz,
                      int leaf_size, int dof = 6);

// The joint analysis of independent systems (the block-diagonal matrix of
// all of them): parts concatenated, levels of their assembly trees merged
// from the leaves.
void symbolic_concat(Symbolic &J, const std::vector<const Symbolic *> &parts);

// ---------------------------------------------------------------------------
// Device-side multifrontal factor (one precision per instance).
// ---------------------------------------------------------------------------
// One phase of a solve sweep: gx x gy x gz work units of one type over the
// supernodes level_sn[lev_off ...] of one level (gy of them).
enum { SP_PERM_IN, SP_GATHER, SP_COLS0, SP_ROWS0, SP_COLS1, SP_ROWS1, SP_PERM_OUT, SP_PERM_IN_Y, SP_MUL_TOP,
       SP_MUL_UPD, SP_COLS0W, SP_COLS1W };
struct SolvePhase { int type, lev_off, gx, gy, gz, nchunk; };

struct DevSymbolic {
	int nblk = 0, nsn = 0, nlevels = 0, nb = 0;
	int dof = 6;                   // scalar unknowns per particle (6 or 3)
	int *perm = nullptr, *iperm = nullptr;
	int *sn_first = nullptr, *sn_n = nullptr, *sn_m = nullptr, *sn_ld = nullptr;
	int *sn_rows_off = nullptr, *rows = nullptr;
	int64_t *sn_off = nullptr, *sn_woff = nullptr;
	int *child_off = nullptr, *children = nullptr;
	int64_t *cinv_off = nullptr;
	int *cinv = nullptr;
	int *cfwd = nullptr;
	int *level_sn = nullptr;
	int *d_sn = nullptr, *d_bc = nullptr;
	int *od_sn = nullptr, *od_br = nullptr, *od_bc = nullptr, *od_tr = nullptr;
	int *level_d = nullptr, *level_od = nullptr;
	// per-level / per-panel task lists
	int *col_tasks = nullptr;      // (sn, col) pairs for the assembly kernel
	int4 *panel_tasks = nullptr;   // (sn, row0, k, nrows)
	int4 *tile_tasks = nullptr;    // (sn, row0, col0, k)
	int4 *diag_tasks = nullptr;    // (sn, col0, k, width) of each panel's diagonal block
	std::vector<SolvePhase> h_solve_phases;   // phase table of a solve sweep
	std::vector<SolvePhase> h_mul_phases;     // ... of the product with L
	// host-side launch plan
	struct Launch { int kind; int level; int k; int64_t off; int count; };
	std::vector<Launch> factor_plan;
	std::vector<int> h_level_off, h_level_d_off, h_level_od_off;
	std::vector<int> h_level_maxn6, h_level_maxm6;   // per-level maxima of dof n and dof m (scalar)
	std::vector<int> h_level_maxF6;                  // per-level maximum front order dof (n + m) (scalar)
	std::vector<int64_t> h_col_task_off;
	int64_t arena_elems = 0, w_elems = 0;
	int max_F = 0;
	int max_n6 = 0;
	double flops = 0;
	int64_t nnz_L = 0;
};

// Tile edge and panel width the factor kernels use for a precision; the
// launch plan built by dev_symbolic_upload must use the same values.
int factor_tile_size(int precision);
int factor_syrk_tile_size(int precision);
int factor_panel_width(int precision);
int factor_panel_rows();

void dev_symbolic_upload(DevSymbolic &D, const Symbolic &S, int nb, int panel_nb, int tile, int syrk_tile,
                         bool tensor_cores, cudaStream_t st);
void dev_symbolic_free(DevSymbolic &D);
// builds and uploads the phase table of the solve sweep (lfg_factor.cu)
void solve_plan_build(DevSymbolic &D, cudaStream_t st);

// Factor arenas and launchers (lfg_factor.cu).
template <typename T> struct DevFactor {
	T *arena = nullptr;   // fronts
	T *w = nullptr;       // forward-solve update vectors
	T *xp = nullptr, *yp = nullptr; // permuted solve workspaces (k * 6n)
	T *linv = nullptr;    // per supernode: Linv^T of its current panel's diagonal block
	T *part = nullptr;    // solve: partial row sums per column chunk
	int *tally = nullptr; // solve: chunks done per row block of a row-product phase (0 between phases)
	int64_t pstride = 0;
	int64_t arena_cap = 0, w_cap = 0, x_cap = 0, linv_cap = 0, part_cap = 0, tally_cap = 0;
	int *status = nullptr; // device: first non-positive pivot column + 1; 0 = a bounded wait gave up;
	                       // 0x7fffffff = ok
};

template <typename T> void factor_alloc(DevFactor<T> &F, const DevSymbolic &D, int kmax);
template <typename T> void factor_free(DevFactor<T> &F);

// Numeric factorisation from compact blocks (dblocks n x 15, odblocks nb x 18,
// both FP64 device arrays).  Launches only; status left in F.status.
template <typename T>
int factor_numeric(DevFactor<T> &F, const DevSymbolic &D, const double *d_dblocks,
                   const double *d_odblocks, cudaStream_t st);

// Solve with k right-hand sides: b, x device arrays k x 6n, FP64 (x may alias b).
template <typename T>
int factor_solve(DevFactor<T> &F, const DevSymbolic &D, int k, const double *b, double *x,
                 cudaStream_t st);
// x = P^T L P b (k vectors; x may not alias b)
template <typename T>
int factor_multiply(DevFactor<T> &F, const DevSymbolic &D, int k, const double *b, double *x,
                    cudaStream_t st);

// y = A x for the compact block matrix (FP64), k vectors, and r = b - A x.
// Lower/upper adjacency lists for the per-block-row gather.
struct DevBlockMatrix {
	int n = 0, nb = 0;
	int dof = 6;                 // unknowns per particle of the solved system (6, or 3: components 0, 2, 4)
	double *dblocks = nullptr;   // n x 15
	double *odblocks = nullptr;  // nb x 18
	int *od_row = nullptr, *od_col = nullptr;
	int *lo_ptr = nullptr, *lo_idx = nullptr;   // for row block i: OD entries with row == i
	int *up_ptr = nullptr, *up_idx = nullptr;   // OD entries with col == i
};
void block_residual(const DevBlockMatrix &A, int k, const double *b, const double *x, double *r,
                    cudaStream_t st);

// Everything the output writers read from a simulation (lfg_output.cpp),
// gathered by sim_output_snapshot (lfg_sim.cpp) at the current state.
struct OutputSnapshot {
	int n = 0, twodim = 0, lubrication = 0, repulsion = 0, control = 0;
	double lx = 0, ly = 0, lz = 0;
	double time = 0, strain = 0, shear_rate = 0, avg_dt = 0, max_velocity = 0;
	double shear_disp[2] = {0, 0}, shear_strain[3] = {0, 0, 0}, Einf[6] = {0}, vel_diff[3] = {0, 0, 0};
	double kn = 0, kt = 0, kr = 0, interaction_range = 0;
	double total_stress[6] = {0};
	std::vector<std::string> groups;          // System::total_stress_groups, in key order
	std::vector<std::array<double, 6>> group_stress;
	std::vector<double> radius, pos, vel, ang, na, na_disp, angle;   // n, 3n, 3n, 3n, 6n, 3n, n
	std::vector<double> pairs;                // OUT_W doubles per interaction, sorted by (p0, p1)
	int out_w = 0;
	// per-particle stresslets of every stress slot (NSC x 6n) and which slots
	// the run declares; filled only when want_particle_stress is set
	bool want_particle_stress = false;
	std::vector<double> particle_stress;
	std::vector<char> slot_declared;
};

// Fused batch (lfg_sim.cpp): suspensions stepping in lockstep through one
// joint solver.  fused_add creates a member simulation (owned by the caller,
// destroyed with lfg_sim_destroy after the group).
class FusedGroup;
FusedGroup *fused_create(int device, int precision);
void fused_destroy(FusedGroup *g);
int fused_add(FusedGroup *g, const lfg_params *p, const lfg_options *opt, int n, const double *pos,
              const double *radius, double lx, double ly, double lz, const double *le_disp, lfg_sim **out,
              lfg_status *st);
void fused_run(FusedGroup *g, int nsteps);
void fused_advance(FusedGroup *g, const double *strain_end);
void fused_set_leaf_size(FusedGroup *g, int leaf);
void fused_stats(const FusedGroup *g, int64_t *kernels, int *joint_runs, double *flops, int *iters);

void axpy_vec(int n, int k, const double *d, double *x, cudaStream_t st);
// per-RHS squared norms of r and b, written to out[2k] (device); with a
// segment table seg (nseg + 1 offsets into each right-hand side, device), per
// right-hand side and segment: out[2 (rh nseg + q)]
void residual_norms(int n6, int k, const double *r, const double *b, double *out, cudaStream_t st,
                    const int *seg = nullptr, int nseg = 1);

} // namespace lfg

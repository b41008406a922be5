// lfg_factor.cu -- device multifrontal Cholesky of R_FU (replaces CHOLMOD's
// supernodal cholmod_factorize / cholmod_solve2, LF_DEM/StokesSolver.cpp:
// 671-703, 950-978), in FP64 ("plain form") or FP32 (factor of the FP32 +
// FP64-refinement form).
//
// Front layout: supernode s with n (own) and m (below) block columns has a
// dense column-major front of 6F x ... (F = n + m) with leading dimension
// ld = 6F + 6n.  Rows [6F, 6F + 6n) are an appended identity block: the same
// panel triangular solves that produce L21 = A21 L11^-T turn it into
// E = L11^-T, so both triangular solves become parallel matrix-vector
// products.  Columns [0, 6n) hold L after factorisation; the lower triangle
// of rows/columns [6n, 6F) holds the update (Schur complement) matrix that the
// parent gathers.
//
// Per level of the assembly tree (leaves first):
//   assemble  : zero + gather children's update matrices (fixed child order),
//   scatter   : add the compact D / OD blocks of the level's columns,
//   diag      : factor and invert panel 0's diagonal block (one CTA per front);
//               panel k + 1's is done inside update k by the tile that holds it,
//   trsm k    : rows below it (real rows and identity rows) times Linv^T,
//   update k  : trailing rank-w update of the front's own columns (tiles),
//   syrk      : the update (Schur complement) matrix, one deep-K product.
// Nothing uses atomics except the failure flag, so results are bitwise
// reproducible run to run.
#include <atomic>
#include <type_traits>
#include <cstdio>
#include <mutex>
#include <cuda_runtime.h>

#include "lfg_internal.h"

namespace lfg {

enum { PLAN_ASSEMBLE = 0, PLAN_SCATTER = 1, PLAN_PANEL = 3, PLAN_UPDATE = 4, PLAN_SYRK = 5, PLAN_DIAG = 6,
       PLAN_SYRK_TC = 8 };
constexpr int PANEL_ROWS = 64;   // rows per panel (k_trsm) task (must match the plan)
constexpr int SOLVE_WARPS = 8;
constexpr int SOLVE_CB = 8;      // columns per CTA of the solve's column kernels
constexpr int SOLVE_JC = 256;    // columns per chunk of the solve's row kernels
constexpr int SOLVE_WARP_ROWS = 256;   // column products with at most this many rows: one warp per unit
constexpr unsigned FULL_MASK = 0xffffffffu;

template <typename T> struct Cfg;
// NB: panel width; TILE/TPT: trailing-update tile edge / outputs per thread
// per dimension; STILE/STPT: the same for the deep-K Schur complement SYRK
template <> struct Cfg<double> { static constexpr int NB = 32, TILE = 64, TPT = 4, STILE = 64, STPT = 4; };
template <> struct Cfg<float>  { static constexpr int NB = 64, TILE = 64, TPT = 4, STILE = 128, STPT = 8; };

// ---------------------------------------------------------------------------
// compact blocks -> dense (StokesSolver.cpp:154-231), m[r*6+c]
// ---------------------------------------------------------------------------
__device__ inline void d15_to_dense(const double *d, double *m)
{
#pragma unroll
	for (int i = 0; i < 36; i++) m[i] = 0;
	m[0*6+0] = d[0]; m[1*6+0] = d[1]; m[2*6+0] = d[2]; m[4*6+0] = d[3]; m[5*6+0] = d[4];
	m[1*6+1] = d[5]; m[2*6+1] = d[6]; m[3*6+1] = -d[3]; m[5*6+1] = d[7];
	m[2*6+2] = d[8]; m[3*6+2] = -d[4]; m[4*6+2] = -d[7];
	m[3*6+3] = d[9]; m[4*6+3] = d[10]; m[5*6+3] = d[11];
	m[4*6+4] = d[12]; m[5*6+4] = d[13];
	m[5*6+5] = d[14];
}

__device__ inline void od18_to_dense(const double *o, double *m)
{
#pragma unroll
	for (int i = 0; i < 36; i++) m[i] = 0;
	m[0*6+0] = o[0]; m[1*6+0] = o[1]; m[2*6+0] = o[2]; m[4*6+0] = o[3]; m[5*6+0] = o[4];
	m[0*6+1] = o[1]; m[1*6+1] = o[5]; m[2*6+1] = o[6]; m[3*6+1] = -o[3]; m[5*6+1] = o[7];
	m[0*6+2] = o[2]; m[1*6+2] = o[6]; m[2*6+2] = o[8]; m[3*6+2] = -o[4]; m[4*6+2] = -o[7];
	m[1*6+3] = o[9]; m[2*6+3] = o[10]; m[3*6+3] = o[11]; m[4*6+3] = o[12]; m[5*6+3] = o[13];
	m[0*6+4] = -o[9]; m[2*6+4] = o[14]; m[3*6+4] = o[12]; m[4*6+4] = o[15]; m[5*6+4] = o[16];
	m[0*6+5] = -o[10]; m[1*6+5] = -o[14]; m[3*6+5] = o[13]; m[4*6+5] = o[16]; m[5*6+5] = o[17];
}

// ---------------------------------------------------------------------------
// assembly: one CTA per (supernode, scalar column)
// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The factor and solve kernels are launched
// with programmatic stream serialisation (launch_pdl) and call pdl_wait --
// which returns once the previous launch has finished and its writes are
// visible -- before their first access to data an earlier launch writes;
// task lists and indices (written by the symbolic upload, before any of these
// launches) may be read before it.  The solve phases also call pdl_trigger
// first, so the next phase is scheduled as soon as all their CTAs run, and so
// does the panel solve k_trsm (a short launch: the next update's CTAs, the
// diagonal tiles first, are resident when it completes).  The other factor
// kernels do not (their successors would sit resident next to the
// diagonal-block CTA on the critical path: measured slower), so theirs start
// when they finish, overlapping only the final flush.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Scalar index r of a front or vector with dof unknowns per particle (6, or
// 3 for the in-plane part of a 2D system): its particle (block) and component.
__device__ __forceinline__ int bdiv(int r, int dof) { return dof == 6 ? r/6 : r/3; }
__device__ __forceinline__ int bmod(int r, int dof) { return dof == 6 ? r%6 : r%3; }

template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
	cudaLaunchConfig_t cfg = {};
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	LFG_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
}

// Column c of front s (rows [c, 6F) and, for own columns, the identity rows):
// the sum over s's children, in child order, of their update-matrix entries
// that land there.  Child-driven: for each child whose update contains
// column c, its column is read contiguously (rows from the diagonal down)
// and added into a shared-memory copy of the parent column through cfwd
// (child update block -> parent front block; monotone, so the child's lower
// triangle lands on the parent's).  The children's parameters are fetched
// by one thread each, up to ASM_CHILDREN at a time.
constexpr int ASM_CHILDREN = 32;
constexpr int ASM_BATCH = 8;       // rows per thread and pass of a child's column
constexpr int ASM_THREADS = 128;   // threads of the CTA-per-column form

template <typename T>
__global__ void __launch_bounds__(ASM_THREADS) k_assemble(const int *__restrict__ col_tasks, const int *__restrict__ sn_n,
                                                  const int *__restrict__ sn_m, const int *__restrict__ sn_ld,
                                                  const int64_t *__restrict__ sn_off,
                                                  const int *__restrict__ child_off,
                                                  const int *__restrict__ children,
                                                  const int64_t *__restrict__ cinv_off,
                                                  const int *__restrict__ cinv, const int *__restrict__ sn_rows_off,
                                                  const int *__restrict__ cfwd, T *__restrict__ arena, int dof)
{
	extern __shared__ __align__(16) unsigned char smem_asm[];
	T *buf = reinterpret_cast<T *>(smem_asm);   // buf[r - c], r in [c, 6F)
	__shared__ int c_jc[ASM_CHILDREN], c_n6[ASM_CHILDREN], c_F6[ASM_CHILDREN], c_ld[ASM_CHILDREN],
		c_ro[ASM_CHILDREN];
	__shared__ int64_t c_off[ASM_CHILDREN];
	int s = col_tasks[2*blockIdx.x], c = col_tasks[2*blockIdx.x+1];
	int n6 = dof*sn_n[s], F6 = n6+dof*sn_m[s], ld = sn_ld[s];
	T *col = arena+sn_off[s]+(int64_t)c*ld;
	int cb = bdiv(c, dof), cr = bmod(c, dof);
	int ca = child_off[s], cz = child_off[s+1];
	for (int r = c+threadIdx.x; r < F6; r += blockDim.x) buf[r-c] = T(0);
	pdl_wait();
	for (int q0 = ca; q0 < cz; q0 += ASM_CHILDREN) {
		int nq = min(ASM_CHILDREN, cz-q0);
		__syncthreads();   // the previous chunk's parameters are no longer read
		if (threadIdx.x < nq) {
			int ch = children[q0+threadIdx.x];
			int ic = cinv[cinv_off[ch]+cb];
			c_jc[threadIdx.x] = ic < 0 ? -1 : dof*ic+cr;
			c_n6[threadIdx.x] = sn_n[ch];   // in particles
			c_F6[threadIdx.x] = dof*(sn_n[ch]+sn_m[ch]);
			c_ld[threadIdx.x] = sn_ld[ch];
			c_ro[threadIdx.x] = sn_rows_off[ch];
			c_off[threadIdx.x] = sn_off[ch];
		}
		__syncthreads();
		for (int u = 0; u < nq; u++) {
			int jc = c_jc[u];
			if (jc < 0) continue;   // uniform: column c is not in this child's update
			int nbc = c_n6[u], F6c = c_F6[u];
			// child fronts are complete and not written here: read-only loads
			const T *src = arena+c_off[u]+(int64_t)jc*c_ld[u];
			const int *fw = cfwd+c_ro[u];
			// ASM_BATCH rows per thread and pass, their loads issued first
			// (within a child the parent rows are distinct)
			for (int i0 = jc+threadIdx.x; i0 < F6c; i0 += ASM_BATCH*blockDim.x) {
				T v[ASM_BATCH];
				int pr[ASM_BATCH];
#pragma unroll
				for (int b = 0; b < ASM_BATCH; b++) {
					int i = i0+b*blockDim.x;
					pr[b] = -1;
					v[b] = T(0);
					if (i < F6c) {
						pr[b] = dof*__ldg(&fw[bdiv(i, dof)-nbc])+bmod(i, dof);
						v[b] = __ldg(&src[i]);
					}
				}
#pragma unroll
				for (int b = 0; b < ASM_BATCH; b++)
					if (pr[b] >= 0) buf[pr[b]-c] += v[b];
			}
			__syncthreads();   // adds of one child complete before the next child's
		}
	}
	__syncthreads();
	for (int r = c+threadIdx.x; r < F6; r += blockDim.x) col[r] = buf[r-c];
	if (c < n6)
		for (int r = threadIdx.x; r < n6; r += blockDim.x) col[F6+r] = (r == c) ? T(1) : T(0);
}

// The same column assembly with one warp per column, ASM_WARPS columns per
// CTA, for levels of short fronts (the CTA-per-column form leaves most of its
// threads idle there and is bound by CTA turnover).  Each warp owns a
// shared-memory column buffer of bufw entries (>= the level's largest front
// order); the children's parameters are loaded by one lane each and
// broadcast.  Within a child the parent rows are distinct (cfwd is
// injective), so each lane adds ASM_BATCH rows per pass with all their loads
// issued first; children follow one another in the same fixed order as in
// k_assemble, so every entry is the same sum, bit for bit.
constexpr int ASM_WARPS = 8;
constexpr int ASM_WARP_MAXF = 1536;   // levels whose fronts are at most this order use the warp form

template <typename T>
__global__ void __launch_bounds__(32*ASM_WARPS) k_assemble_warp(const int *__restrict__ col_tasks, int ncols, int bufw,
                                                                const int *__restrict__ sn_n,
                                                                const int *__restrict__ sn_m,
                                                                const int *__restrict__ sn_ld,
                                                                const int64_t *__restrict__ sn_off,
                                                                const int *__restrict__ child_off,
                                                                const int *__restrict__ children,
                                                                const int64_t *__restrict__ cinv_off,
                                                                const int *__restrict__ cinv,
                                                                const int *__restrict__ sn_rows_off,
                                                                const int *__restrict__ cfwd, T *__restrict__ arena,
                                                                int dof)
{
	extern __shared__ __align__(16) unsigned char smem_asm[];
	const int warp = threadIdx.x/32, lane = threadIdx.x%32;
	const int task = blockIdx.x*ASM_WARPS+warp;
	if (task >= ncols) return;   // whole warps only; nothing below synchronises the CTA
	T *buf = reinterpret_cast<T *>(smem_asm)+(size_t)warp*bufw;   // buf[r - c], r in [c, 6F)
	const int s = col_tasks[2*task], c = col_tasks[2*task+1];
	const int n6 = dof*sn_n[s], F6 = n6+dof*sn_m[s], ld = sn_ld[s];
	T *col = arena+sn_off[s]+(int64_t)c*ld;
	const int cb = bdiv(c, dof), cr = bmod(c, dof);
	const int ca = child_off[s], cz = child_off[s+1];
	for (int r = lane; r < F6-c; r += 32) buf[r] = T(0);
	pdl_wait();
	for (int q0 = ca; q0 < cz; q0 += 32) {
		const int nq = min(32, cz-q0);
		int jc = -1, nbc = 0, F6c = 0, cld = 0, cro = 0;
		int64_t coff = 0;
		if (lane < nq) {
			int ch = children[q0+lane];
			int ic = cinv[cinv_off[ch]+cb];
			jc = ic < 0 ? -1 : dof*ic+cr;
			nbc = sn_n[ch];   // in particles
			F6c = dof*(sn_n[ch]+sn_m[ch]);
			cld = sn_ld[ch];
			cro = sn_rows_off[ch];
			coff = sn_off[ch];
		}
		for (int u = 0; u < nq; u++) {
			const int ju = __shfl_sync(FULL_MASK, jc, u);
			if (ju < 0) continue;   // uniform: column c is not in this child's update
			const int nbu = __shfl_sync(FULL_MASK, nbc, u), Fu = __shfl_sync(FULL_MASK, F6c, u);
			const int ldu = __shfl_sync(FULL_MASK, cld, u), rou = __shfl_sync(FULL_MASK, cro, u);
			const int64_t offu = __shfl_sync(FULL_MASK, coff, u);
			// child fronts are complete and not written here: read-only loads
			const T *src = arena+offu+(int64_t)ju*ldu;
			const int *fw = cfwd+rou;
			for (int i0 = ju+lane; i0 < Fu; i0 += 32*ASM_BATCH) {
				T v[ASM_BATCH];
				int pr[ASM_BATCH];
#pragma unroll
				for (int b = 0; b < ASM_BATCH; b++) {
					int i = i0+32*b;
					pr[b] = -1;
					v[b] = T(0);
					if (i < Fu) {
						pr[b] = dof*__ldg(&fw[bdiv(i, dof)-nbu])+bmod(i, dof);
						v[b] = __ldg(&src[i]);
					}
				}
#pragma unroll
				for (int b = 0; b < ASM_BATCH; b++)
					if (pr[b] >= 0) buf[pr[b]-c] += v[b];
			}
			__syncwarp();   // adds of one child complete before the next child's
		}
	}
	__syncwarp();
	for (int r = c+lane; r < F6; r += 32) col[r] = buf[r-c];
	if (c < n6)
		for (int r = lane; r < n6; r += 32) col[F6+r] = (r == c) ? T(1) : T(0);
}

// R_FU blocks of one level added into its fronts, one thread per block: the
// level's diagonal blocks (threads < nd), then its off-diagonal blocks.  The
// two kinds never share a front entry (an off-diagonal block joins two
// different particles), so one launch adds both.
template <typename T>
__global__ void k_scatter(int nd, int nod, const int *__restrict__ dlist, const int *__restrict__ odlist,
                          const double *__restrict__ dblocks, const double *__restrict__ odblocks,
                          const int *__restrict__ d_sn, const int *__restrict__ d_bc, const int *__restrict__ od_sn,
                          const int *__restrict__ od_br, const int *__restrict__ od_bc, const int *__restrict__ od_tr,
                          const int *__restrict__ sn_ld, const int64_t *__restrict__ sn_off, T *__restrict__ arena,
                          int dof)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= nd+nod) return;
	double m[36];
	if (dof == 3) {
		// in-plane part of a 2D system: unknowns x, z translation and y
		// rotation, components 0, 2, 4 of the 6x6 block
		if (t < nd) {
			int i = dlist[t];
			int s = d_sn[i], b = d_bc[i], ld = sn_ld[s];
			T *base = arena+sn_off[s];
			pdl_wait();
			d15_to_dense(dblocks+15*(int64_t)i, m);
			T old[6];
#pragma unroll
			for (int c = 0, e = 0; c < 3; c++)
#pragma unroll
				for (int r = c; r < 3; r++, e++) old[e] = base[(int64_t)(3*b+c)*ld+3*b+r];
#pragma unroll
			for (int c = 0, e = 0; c < 3; c++)
#pragma unroll
				for (int r = c; r < 3; r++, e++) base[(int64_t)(3*b+c)*ld+3*b+r] = old[e]+(T)m[(2*r)*6+2*c];
		} else {
			int e = odlist[t-nd];
			int s = od_sn[e], br = od_br[e], bc = od_bc[e], ld = sn_ld[s];
			T *base = arena+sn_off[s];
			bool tr = od_tr[e];
			pdl_wait();
			od18_to_dense(odblocks+18*(int64_t)e, m);
			T old[9];
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) old[3*c+r] = base[(int64_t)(3*bc+c)*ld+3*br+r];
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++)
					base[(int64_t)(3*bc+c)*ld+3*br+r] =
						old[3*c+r]+(T)(tr ? m[(2*c)*6+2*r] : m[(2*r)*6+2*c]);
		}
		return;
	}
	if (t < nd) {
		int i = dlist[t];
		int s = d_sn[i], b = d_bc[i], ld = sn_ld[s];
		T *base = arena+sn_off[s];
		pdl_wait();
		d15_to_dense(dblocks+15*(int64_t)i, m);
		// all 21 old values are loaded before the first store (a store between
		// them would serialise the loads: the addresses may alias)
		T old[21];
#pragma unroll
		for (int c = 0, e = 0; c < 6; c++)
#pragma unroll
			for (int r = c; r < 6; r++, e++) old[e] = base[(int64_t)(6*b+c)*ld+6*b+r];
#pragma unroll
		for (int c = 0, e = 0; c < 6; c++)
#pragma unroll
			for (int r = c; r < 6; r++, e++) base[(int64_t)(6*b+c)*ld+6*b+r] = old[e]+(T)m[r*6+c];
	} else {
		int e = odlist[t-nd];
		int s = od_sn[e], br = od_br[e], bc = od_bc[e], ld = sn_ld[s];
		T *base = arena+sn_off[s];
		bool tr = od_tr[e];
		pdl_wait();
		od18_to_dense(odblocks+18*(int64_t)e, m);
		T old[36];
#pragma unroll
		for (int c = 0; c < 6; c++)
#pragma unroll
			for (int r = 0; r < 6; r++) old[6*c+r] = base[(int64_t)(6*bc+c)*ld+6*br+r];
#pragma unroll
		for (int c = 0; c < 6; c++)
#pragma unroll
			for (int r = 0; r < 6; r++)
				base[(int64_t)(6*bc+c)*ld+6*br+r] = old[6*c+r]+(T)(tr ? m[c*6+r] : m[r*6+c]);
	}
}

// ---------------------------------------------------------------------------
// diagonal block of panel k (k_diag): one CTA (256 threads) per front.  The
// NB x NB block (NB = 32 or 64) is factored by 32 x 32 sub-blocks, each by
// one warp holding its rows in registers (lane = row), then inverted:
// Linv = L_kk^-1 (lower triangular).  k_diag writes L_kk back into the front
// and Linv^T (row-major, NB x NB, zeros below the diagonal) to the front's
// slot of the Linv workspace, so the rows below the block are solved by
// k_trsm as a product with Linv^T.  Rows and columns past the panel width w
// are padded with the identity.  A non-positive pivot is replaced by 1 and
// reported through *fail (first global scalar column + 1).
// ---------------------------------------------------------------------------

// Warp routines on 32 x 32 blocks in shared memory (row-major, stride ld),
// one row or column per lane in registers.  The step loops are not fully
// unrolled (the code stays small: it runs once per launch, so a fully
// unrolled body would be fetched cold every time); register indices stay
// static because every step shifts the lane's values down by one, so the
// current column is always element 0.
//
// Lsh (32 x 32, 16-byte aligned): Lsh[32 j + q] = L[j + q][j] for q >= 1
// (zero past the block) and Lsh[32 j] = 1 / L[j][j] (the pivot's rsqrt),
// column j of L from the diagonal down, written by warp_potrf32 and read by
// the solves with vector loads.
//
// The steps are latency chains; each routine keeps only what the next step
// needs on the chain: in warp_potrf32 the next pivot's lane updates its
// own diagonal entry and broadcasts it, and its rsqrt is issued before the
// column updates, which wait for Lsh; the solves take the reciprocal from
// Lsh (no shuffle, no division) and load two columns per iteration ahead of
// their updates.

// the 32 entries Lsh[32 j + q], q < 32
template <typename T> __device__ inline void lsh_column(const T *Lsh, int j, T (&c)[32])
{
	if constexpr (sizeof(T) == 4) {
		const float4 *p = reinterpret_cast<const float4 *>(Lsh+32*j);
#pragma unroll
		for (int u = 0; u < 8; u++) {
			float4 v = p[u];
			c[4*u] = v.x; c[4*u+1] = v.y; c[4*u+2] = v.z; c[4*u+3] = v.w;
		}
	} else {
		const double2 *p = reinterpret_cast<const double2 *>(Lsh+32*j);
#pragma unroll
		for (int u = 0; u < 16; u++) {
			double2 v = p[u];
			c[2*u] = v.x; c[2*u+1] = v.y;
		}
	}
}

// pivot reciprocal square root: the hardware approximation for FP32 (the
// FP32 factor is refined in FP64 anyway; no denormal handling on the chain),
// the library rsqrt for FP64
__device__ __forceinline__ float pivot_rsqrt(float x)
{
	float r;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ double pivot_rsqrt(double x) { return rsqrt(x); }

// Progress flags of the FP32 diagonal-block pipeline (shared memory): the
// producer warp publishes "columns [0, v) are in Lsh" with a release store
// after the __syncwarp that follows its lanes' stores; a follower warp polls
// with acquire loads.  The wait is bounded: past the limit it records status 0
// (LFG_ERR_TIMEOUT) and goes on, so a broken pipeline cannot hang the SM.
__device__ __forceinline__ void flag_publish(int *p, int v)
{
	asm volatile("st.release.cta.shared::cta.u32 [%0], %1;"
	             :: "r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}
__device__ __forceinline__ int flag_read(const int *p)
{
	int v;
	asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];"
	             : "=r"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
	return v;
}
constexpr int FLAG_SPIN_LIMIT = 1 << 22;   // ~0.1 s of polls
__device__ __forceinline__ void flag_wait(const int *p, int need, int *fail)
{
	if (!p) return;
	for (int it = 0; it < FLAG_SPIN_LIMIT; it++)
		if (flag_read(p) >= need) return;
	if (fail) atomicMin(fail, 0);
}

// Cholesky of S (lower part), lane = row; S's lower part becomes L and its
// upper part zero; Lsh receives L's columns, and *flag (if given) the number
// of columns already there.  Two steps per loop iteration: the second step's
// chain can start while the first step's updates of later columns issue.
template <typename T>
__device__ void warp_potrf32(T *S, int ld, T *Lsh, int lane, int jlim, int gcol0, int *fail, int *flag)
{
	T a[32];   // at step j: a[q] = S[lane][j + q]
#pragma unroll
	for (int l = 0; l < 32; l++) a[l] = S[lane*ld+l];
	T djj = __shfl_sync(FULL_MASK, a[0], 0);
	if (!(djj > T(0))) {
		if (lane == 0 && jlim > 0 && fail) atomicMin(fail, gcol0+1);
		djj = T(1);
	}
	T rs = pivot_rsqrt(djj);
#pragma unroll 2
	for (int j = 0; j < 32; j++) {
		T lij = a[0]*rs;
		// the next pivot first: lane j + 1 updates its own diagonal entry with
		// its own L[j + 1][j] and broadcasts it (one shuffle on the chain)
		T dn = __shfl_sync(FULL_MASK, a[1]-lij*lij, (j+1) & 31);
		S[lane*ld+j] = lane > j ? lij : (lane == j ? djj*rs : T(0));
		Lsh[32*j+((lane-j) & 31)] = lane > j ? lij : (lane == j ? rs : T(0));
		__syncwarp();
		T c[32];
		lsh_column<T>(Lsh, j, c);   // in flight during the pivot's check and rsqrt
		bool bad = !(dn > T(0));
		if (bad && lane == 0 && j+1 < 32 && j+1 < jlim && fail) atomicMin(fail, gcol0+j+2);
		dn = bad ? T(1) : dn;
		T rsn = pivot_rsqrt(dn);
#pragma unroll
		for (int q = 1; q < 32; q++) a[q-1] = a[q]-lij*c[q];   // entries past the block are dead
		djj = dn;
		rs = rsn;
		if (flag && lane == 0) flag_publish(flag, j+1);
	}
	__syncwarp();
}

// X L^T = A for 32 rows (lane = row) of X (stride ldx), L lower given by its
// columns in Lsh; X replaces A.  Columns alternate between two register
// buffers, each loaded one step before its use.  With a flag the routine
// follows a warp_potrf32 still producing Lsh (each column is loaded once the
// flag shows it), and with pub it publishes its own solved columns of X.
template <typename T>
__device__ void warp_trsm32(T *X, int ldx, const T *Lsh, int lane, const int *flag = nullptr, int *fail = nullptr,
                            int *pub = nullptr)
{
	T x[32];   // at step t: x[q] = X[lane][t + q]
#pragma unroll
	for (int l = 0; l < 32; l++) x[l] = X[lane*ldx+l];
	T c[32], d[32];
	flag_wait(flag, 1, fail);
	lsh_column<T>(Lsh, 0, c);
#pragma unroll 1
	for (int t = 0; t < 32; t += 2) {
		flag_wait(flag, t+2, fail);
		lsh_column<T>(Lsh, t+1, d);
		T xt = x[0]*c[0];
		X[lane*ldx+t] = xt;
#pragma unroll
		for (int q = 1; q < 32; q++) x[q-1] = x[q]-xt*c[q];
		flag_wait(flag, min(t+3, 32), fail);
		lsh_column<T>(Lsh, (t+2) & 31, c);   // after the last pair: column 0 again, unused
		xt = x[0]*d[0];
		X[lane*ldx+t+1] = xt;
		if (pub) {
			__syncwarp();
			if (lane == 0) flag_publish(pub, t+2);
		}
#pragma unroll
		for (int q = 1; q < 32; q++) x[q-1] = x[q]-xt*d[q];
	}
	__syncwarp();
}

// V = L^-1 (lower; lane = column), V row-major with stride ldv; L's columns
// in Lsh (loaded as in warp_trsm32, following the producer when flag is given)
template <typename T>
__device__ void warp_trtri32(const T *Lsh, T *V, int ldv, int lane, const int *flag = nullptr, int *fail = nullptr,
                             int *pub = nullptr)
{
	T y[32];   // at step t: y[q] = V[t + q][lane]
#pragma unroll
	for (int i = 0; i < 32; i++) y[i] = (i == lane) ? T(1) : T(0);
	T c[32], d[32];
	flag_wait(flag, 1, fail);
	lsh_column<T>(Lsh, 0, c);
#pragma unroll 1
	for (int t = 0; t < 32; t += 2) {
		flag_wait(flag, t+2, fail);
		lsh_column<T>(Lsh, t+1, d);
		T yt = y[0]*c[0];
		V[t*ldv+lane] = yt;
#pragma unroll
		for (int q = 1; q < 32; q++) y[q-1] = y[q]-c[q]*yt;
		flag_wait(flag, min(t+3, 32), fail);
		lsh_column<T>(Lsh, (t+2) & 31, c);
		yt = y[0]*d[0];
		V[(t+1)*ldv+lane] = yt;
		if (pub) {   // rows t and t + 1 of V are complete
			__syncwarp();
			if (lane == 0) flag_publish(pub, t+2);
		}
#pragma unroll
		for (int q = 1; q < 32; q++) y[q-1] = y[q]-d[q]*yt;
	}
	__syncwarp();
}

// Fully unrolled forms of the same three routines (lane = row or column,
// every step's updates limited to the live entries), used for FP64: FP64
// multiply-adds are scarce (the compact forms do twice as many, half of them
// on dead entries), so the shorter arithmetic beats the cost of fetching the
// larger code cold; in FP32 the compact forms are faster.
// Cholesky of S (lower part), lane = row; S's lower part becomes L and its
// upper part zero
template <typename T>
__device__ void warp_potrf32_unrolled(T *S, int ld, int lane, int jlim, int gcol0, int *fail)
{
	T a[32];
#pragma unroll
	for (int l = 0; l < 32; l++) a[l] = S[lane*ld+l];
#pragma unroll
	for (int j = 0; j < 32; j++) {
		T djj = __shfl_sync(FULL_MASK, a[j], j);
		if (!(djj > T(0))) {
			if (lane == 0 && j < jlim && fail) atomicMin(fail, gcol0+j+1);
			djj = T(1);
		}
		T rs = rsqrt(djj);
		T lij = a[j]*rs;
		a[j] = (lane == j) ? djj*rs : lij;
#pragma unroll
		for (int l = j+1; l < 32; l++) a[l] -= lij*__shfl_sync(FULL_MASK, lij, l);
	}
#pragma unroll
	for (int l = 0; l < 32; l++) S[lane*ld+l] = (l <= lane) ? a[l] : T(0);
	__syncwarp();
}

// X L^T = A for 32 rows (lane = row) of X (stride ldx), L lower (stride ldl);
// X replaces A
template <typename T>
__device__ void warp_trsm32_unrolled(T *X, int ldx, const T *L, int ldl, int lane)
{
	T rd = T(1)/L[lane*ldl+lane];
	T x[32];
#pragma unroll
	for (int l = 0; l < 32; l++) x[l] = X[lane*ldx+l];
#pragma unroll
	for (int t = 0; t < 32; t++) {
		x[t] *= __shfl_sync(FULL_MASK, rd, t);
#pragma unroll
		for (int l = t+1; l < 32; l++) x[l] -= x[t]*L[l*ldl+t];
	}
#pragma unroll
	for (int l = 0; l < 32; l++) X[lane*ldx+l] = x[l];
	__syncwarp();
}

// V = L^-1 (lower; lane = column), V row-major with stride ldv
template <typename T>
__device__ void warp_trtri32_unrolled(const T *L, int ldl, T *V, int ldv, int lane)
{
	T rd = T(1)/L[lane*ldl+lane];
	T y[32];
#pragma unroll
	for (int i = 0; i < 32; i++) y[i] = (i == lane) ? T(1) : T(0);
#pragma unroll
	for (int t = 0; t < 32; t++) {
		y[t] *= __shfl_sync(FULL_MASK, rd, t);
#pragma unroll
		for (int i = t+1; i < 32; i++) y[i] -= L[i*ldl+t]*y[t];
	}
#pragma unroll
	for (int i = 0; i < 32; i++) V[i*ldv+lane] = y[i];
	__syncwarp();
}


// c8[q] = sum_{t < 32} A[i][t] B[t][c] for row i = tid / 4 and columns
// c = tid % 4 + 4q (128 threads, tid < 128, cover a 32 x 32 product);
// B[t][c] is read at B[t*ldb_t + c*ldb_c]
template <typename T>
__device__ void cta_gemm32(T (&c8)[8], const T *A, int lda, const T *B, int ldb_t, int ldb_c, int tid)
{
	int i = tid/4, c0 = tid%4;
#pragma unroll
	for (int q = 0; q < 8; q++) c8[q] = T(0);
#pragma unroll 8
	for (int t = 0; t < 32; t++) {
		T av = A[i*lda+t];
#pragma unroll
		for (int q = 0; q < 8; q++) c8[q] += av*B[t*ldb_t+(c0+4*q)*ldb_c];
	}
}

// Factor and invert the NB x NB diagonal block at (p0, p0) of a front (width
// w, identity-padded past it), with the calling CTA (256 threads).  L_kk
// goes back into the front, Linv_kk^T (row-major NB x NB) to vt.  Ls, Vs:
// NB x (NB + 1), Ts: 32 x 33 and Lsh: 2 x 32 x 32 (16-byte aligned) shared
// arrays of the caller.
// diag_load: the block into Ls (lower part, identity-padded past w) and
// zeros into Vs; diag_factor: the rest, from there
template <typename T>
__device__ void diag_load(const T *base, int ld, int p0, int w, T *Ls, T *Vs)
{
	constexpr int NB = Cfg<T>::NB, LD = NB+1;
	// batches of 16 loads per thread in flight, then their shared stores
	for (int e0 = threadIdx.x; e0 < NB*NB; e0 += 16*blockDim.x) {
		T v[16];
#pragma unroll
		for (int u = 0; u < 16; u++) {
			int e = e0+u*blockDim.x;
			int i = e%NB, j = e/NB;    // coalesced over i (column-major front)
			v[u] = T(0);
			if (e < NB*NB && j <= i) {
				if (i < w) v[u] = base[(int64_t)(p0+j)*ld+p0+i];
				else if (i == j) v[u] = T(1);
			}
		}
#pragma unroll
		for (int u = 0; u < 16; u++) {
			int e = e0+u*blockDim.x;
			if (e < NB*NB) {
				int i = e%NB, j = e/NB;
				Ls[i*LD+j] = v[u];
				Vs[i*LD+j] = T(0);
			}
		}
	}
}

// Stores of the factored block for rows [ilo, ihi) and columns [jlo, jhi):
// L's lower part (rows below w excluded) back into the front, Linv^T to vt
// (vt[j NB + i] = Linv[i][j]); batches of 8 per thread, shared loads first.
template <typename T>
__device__ void diag_store(T *base, int ld, int p0, int w, const T *Ls, const T *Vs, T *vt, int ilo, int ihi,
                           int jlo, int jhi, bool store_l, bool store_v, int tid, int nthr)
{
	constexpr int NB = Cfg<T>::NB, LD = NB+1;
	const int ni = ihi-ilo, cnt = ni*(jhi-jlo);
	for (int e0 = tid; e0 < cnt; e0 += 8*nthr) {
		T lv[8], vv[8];
#pragma unroll
		for (int u = 0; u < 8; u++) {
			int e = e0+u*nthr;
			if (e < cnt) {
				int i = ilo+e%ni, j = jlo+e/ni;
				lv[u] = Ls[i*LD+j];
				vv[u] = Vs[i*LD+j];
			}
		}
#pragma unroll
		for (int u = 0; u < 8; u++) {
			int e = e0+u*nthr;
			if (e < cnt) {
				int i = ilo+e%ni, j = jlo+e/ni;
				if (store_l && j <= i && i < w) base[(int64_t)(p0+j)*ld+p0+i] = lv[u];
				if (store_v) vt[j*NB+i] = vv[u];
			}
		}
	}
}

// A11 -= L21 L21^T (the 32 x 32 lower-right quadrant of a 64 x 64 block in
// Ls, stride LD), accumulated while warp_trsm32 still produces L21: it runs
// behind the published columns, four at a time (128 threads: row i = tid / 4,
// columns tid % 4 + 4 q).  The sum over t runs in increasing t, as in
// cta_gemm32.
template <typename T>
__device__ void syrk32_follow(T *Ls, int LD, int tid, const int *flag, int *fail)
{
	int i = tid/4, c0 = tid%4;
	T acc[8];
#pragma unroll
	for (int q = 0; q < 8; q++) acc[q] = T(0);
	const T *L21 = Ls+32*LD;
#pragma unroll 1
	for (int t0 = 0; t0 < 32; t0 += 4) {
		flag_wait(flag, t0+4, fail);
#pragma unroll
		for (int t = t0; t < t0+4; t++) {
			T av = L21[i*LD+t];
#pragma unroll
			for (int q = 0; q < 8; q++) acc[q] += av*L21[(c0+4*q)*LD+t];
		}
	}
#pragma unroll
	for (int q = 0; q < 8; q++)
		if (c0+4*q <= i) Ls[(32+i)*LD+32+c0+4*q] -= acc[q];
}

// flags: 4 ints of shared memory, zeroed by the caller before a
// __syncthreads that precedes the call.  FP32 needs 256 threads.
template <typename T>
__device__ void diag_factor(T *base, int ld, int p0, int w, int gcol0, int *fail, T *Ls, T *Vs, T *Ts, T *Lsh,
                            T *vt, int *flags)
{
	constexpr int NB = Cfg<T>::NB, LD = NB+1;
	static_assert(NB == 32 || NB == 64, "panel width");
	int warp = threadIdx.x/32, lane = threadIdx.x%32;
	if constexpr (sizeof(T) == 4) {
		static_assert(NB == 64, "FP32 panels are 64 wide");
		// FP32, one pipeline over the two 32 x 32 halves.  First half: warp 0
		// factors A00 and publishes L00's columns; warp 1 solves L21 = A21
		// L00^-T and warp 2 inverts L00 as the columns appear; warps 3-6
		// accumulate A11 -= L21 L21^T behind warp 1.  Second half: warp 0
		// factors A11, warp 1 inverts L11 behind it and publishes its rows,
		// warps 2-3 store what is final, warps 4-7 form T1 = L21 Linv00 and
		// then Linv21 = -Linv11 T1 row by row behind warp 1.
		if (warp == 0) warp_potrf32<T>(Ls, LD, Lsh, lane, w, gcol0, fail, flags);
		else if (warp == 1) warp_trsm32<T>(Ls+32*LD, LD, Lsh, lane, flags, fail, flags+2);
		else if (warp == 2) warp_trtri32<T>(Lsh, Vs, LD, lane, flags, fail);
		else if (warp < 7) syrk32_follow<T>(Ls, LD, threadIdx.x-96, flags+2, fail);
		__syncthreads();
		if (warp == 0) warp_potrf32<T>(Ls+32*LD+32, LD, Lsh+1024, lane, w-32, gcol0+32, fail, flags+1);
		else if (warp == 1) warp_trtri32<T>(Lsh+1024, Vs+32*LD+32, LD, lane, flags+1, fail, flags+3);
		else if (warp < 4) {
			// what is final already: L00, L21, Linv00 and the zero upper-right of Linv^T
			diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 0, 32, 0, 32, true, true, threadIdx.x-64, 64);
			diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 32, 64, 0, 32, true, false, threadIdx.x-64, 64);
			diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 0, 32, 32, 64, false, true, threadIdx.x-64, 64);
		} else {
			T c8[8];
			int t2 = threadIdx.x-128, i = t2/4, c0 = t2%4;
			cta_gemm32<T>(c8, Ls+32*LD, LD, Vs, LD, 1, t2);                    // T1 = L21 Linv00
#pragma unroll
			for (int q = 0; q < 8; q++) Ts[i*33+c0+4*q] = c8[q];
			asm volatile("bar.sync 1, 128;" ::: "memory");                     // T1 complete (warps 4-7)
			// Linv21 = -Linv11 T1, row i once row i of Linv11 is published
			flag_wait(flags+3, i+1, fail);
			cta_gemm32<T>(c8, Vs+32*LD+32, LD, Ts, 33, 1, t2);
#pragma unroll
			for (int q = 0; q < 8; q++) Vs[(32+i)*LD+c0+4*q] = -c8[q];
		}
		__syncthreads();
		diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 32, 64, 0, 32, false, true, threadIdx.x, blockDim.x);
		diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 32, 64, 32, 64, true, true, threadIdx.x, blockDim.x);
		return;
	} else {
		// FP64: NB = 32, one half (fully unrolled routines)
		(void)Ts; (void)flags;
		if (warp == 0) warp_potrf32_unrolled<T>(Ls, LD, lane, w, gcol0, fail);
		__syncthreads();
		if (warp == 0) warp_trtri32_unrolled<T>(Ls, LD, Vs, LD, lane);
		__syncthreads();
	}
	diag_store<T>(base, ld, p0, w, Ls, Vs, vt, 0, NB, 0, NB, true, true, threadIdx.x, blockDim.x);
}

template <typename T>
__device__ void diag_block(T *base, int ld, int p0, int w, int gcol0, int *fail, T *Ls, T *Vs, T *Ts, T *Lsh, T *vt,
                           int *flags)
{
	diag_load<T>(base, ld, p0, w, Ls, Vs);
	if (threadIdx.x < 4) flags[threadIdx.x] = 0;
	__syncthreads();
	diag_factor<T>(base, ld, p0, w, gcol0, fail, Ls, Vs, Ts, Lsh, vt, flags);
}

// Linv slot of supernode s for panel k: two slots per supernode, by the
// parity of k, so the update launch of panel k can write panel k + 1's while
// the panel-k solve of other fronts still reads panel k's
template <typename T>
__device__ inline T *linv_slot(T *linv, int nsn, int s, int k)
{
	constexpr int NB = Cfg<T>::NB;
	return linv+((int64_t)(k & 1)*nsn+s)*NB*NB;
}

// diagonal block of panel 0 of every front of a level (later panels' blocks
// are factored by the update launch of the previous panel)
template <typename T>
__global__ void __launch_bounds__(256) k_diag(const int4 *__restrict__ tasks, const int *__restrict__ sn_first,
                                              const int *__restrict__ sn_ld, const int64_t *__restrict__ sn_off,
                                              T *__restrict__ arena, T *__restrict__ linv, int nsn, int *fail, int dof)
{
	constexpr int NB = Cfg<T>::NB, LD = NB+1;
	__shared__ T Ls[NB*LD];
	__shared__ T Vs[NB*LD];
	__shared__ T Ts[32*33];
	__shared__ __align__(16) T Lsh[2*32*32];
	__shared__ int flags[4];
	int4 tk = tasks[blockIdx.x];
	int s = tk.x, p0 = tk.y, k = tk.z, w = tk.w;
	pdl_wait();
	diag_block<T>(arena+sn_off[s], sn_ld[s], p0, w, dof*sn_first[s]+p0, fail, Ls, Vs, Ts, Lsh,
	              linv_slot<T>(linv, nsn, s, k), flags);
}

// ---------------------------------------------------------------------------
// rows below the diagonal block of panel k (k_trsm): X = A Linv_kk^T for up
// to PANEL_ROWS rows per CTA (real rows [t0, 6F) and identity rows [6F,
// 6F + t0)), in place.  256 threads: thread (g, r) computes row r for two
// column chunks of width NB/8, chunks g and 7 - g (equal work, since column
// j needs t <= j).  Linv^T sits in shared memory row-major, so a
// chunk's coefficients for one t are one or two vector loads (a broadcast).
// ---------------------------------------------------------------------------
template <typename T> struct Vec2;
template <> struct Vec2<float> { typedef float4 V; static constexpr int W = 4; };
template <> struct Vec2<double> { typedef double2 V; static constexpr int W = 2; };

template <typename T, int CW>
__device__ inline void lds_chunk(const T *p, T (&v)[CW])
{
	typedef typename Vec2<T>::V V;
	constexpr int W = Vec2<T>::W;
	static_assert(CW % W == 0, "chunk width");
#pragma unroll
	for (int q = 0; q < CW/W; q++) {
		V x = reinterpret_cast<const V *>(p)[q];
		const T *xs = reinterpret_cast<const T *>(&x);
#pragma unroll
		for (int u = 0; u < W; u++) v[q*W+u] = xs[u];
	}
}

template <typename T>
__global__ void __launch_bounds__(256) k_trsm(const int4 *__restrict__ tasks, const int *__restrict__ sn_n,
                                              const int *__restrict__ sn_ld, const int64_t *__restrict__ sn_off,
                                              T *__restrict__ arena, T *__restrict__ linv, int nsn, int dof)
{
	constexpr int NB = Cfg<T>::NB, CW = NB/8;
	__shared__ __align__(16) T Vt[NB*NB];
	__shared__ T As[PANEL_ROWS*NB];   // row r, column t at r*NB + (t ^ (r & 31)): a warp's rows on distinct banks
	static_assert(PANEL_ROWS == 64, "one row per thread");
	int4 tk = tasks[blockIdx.x];
	int s = tk.x, row0 = tk.y, k = tk.z, nrows = tk.w;
	int ld = sn_ld[s];
	int p0 = k*NB;
	int w = min(NB, dof*sn_n[s]-p0);   // panel width: columns p0 + w and later are not touched
	T *base = arena+sn_off[s];
	const T *vt = linv_slot<T>(linv, nsn, s, k);
	pdl_trigger();   // the next update's CTAs wait resident while this short launch runs
	pdl_wait();
	// all of a thread's loads are issued before its shared stores (256
	// threads: NB*NB/256 entries of Linv^T, PANEL_ROWS*NB/256 of the panel)
	{
		constexpr int PV = NB*NB/256, PA = PANEL_ROWS*NB/256;
		T lv[PV], av[PA];
#pragma unroll
		for (int u = 0; u < PV; u++) lv[u] = vt[threadIdx.x+256*u];
#pragma unroll
		for (int u = 0; u < PA; u++) {
			int e = threadIdx.x+256*u;
			int r = e%PANEL_ROWS, t = e/PANEL_ROWS;   // coalesced over rows
			av[u] = (r < nrows && t < w) ? base[(int64_t)(p0+t)*ld+row0+r] : T(0);
		}
#pragma unroll
		for (int u = 0; u < PV; u++) Vt[threadIdx.x+256*u] = lv[u];
#pragma unroll
		for (int u = 0; u < PA; u++) {
			int e = threadIdx.x+256*u;
			int r = e%PANEL_ROWS, t = e/PANEL_ROWS;
			As[r*NB+(t ^ (r & 31))] = av[u];
		}
	}
	__syncthreads();
	// thread: row r, column chunks g and 7 - g (equal work per thread:
	// chunk c has (c + 1) CW terms per entry)
	int g = threadIdx.x/64, r = threadIdx.x%64;
	const T *a0 = As+r*NB;
	const int sw = r & 31;
#pragma unroll
	for (int h = 0; h < 2; h++) {
		int c = h ? 7-g : g;
		int j0 = c*CW;
		T x0[CW];
#pragma unroll
		for (int q = 0; q < CW; q++) x0[q] = T(0);
#pragma unroll 4
		for (int t = 0; t < j0+CW; t++) {
			T v[CW];
			lds_chunk<T, CW>(Vt+t*NB+j0, v);
			T u0 = a0[t ^ sw];
#pragma unroll
			for (int q = 0; q < CW; q++) x0[q] += u0*v[q];
		}
#pragma unroll
		for (int q = 0; q < CW; q++) {
			if (j0+q >= w) continue;
			if (r < nrows) base[(int64_t)(p0+j0+q)*ld+row0+r] = x0[q];
		}
	}
}

// trailing update: CTA = one tile (sn, r0, c0, k) of the front's own columns.
// The tile at (t0, t0) holds panel k + 1's diagonal block: after its update it
// factors and inverts that block (diag_factor), so the next panel needs no
// separate diagonal launch.  (Solving panel k + 1's rows in this launch as
// well -- column-t0 tiles waiting on a flag the diagonal CTA publishes, tasks
// in ticket order -- was measured slower than the separate solve launch.)
template <typename T>
__global__ void __launch_bounds__(256, 2) k_update(const int4 *__restrict__ tasks, const int *__restrict__ sn_first,
                                                const int *__restrict__ sn_n, const int *__restrict__ sn_m,
                                                const int *__restrict__ sn_ld, const int64_t *__restrict__ sn_off,
                                                T *__restrict__ arena, T *__restrict__ linv, int nsn, int *fail,
                                                int dof)
{
	constexpr int NB = Cfg<T>::NB, TL = Cfg<T>::TILE, TPT = Cfg<T>::TPT;
	constexpr int TD = TL/TPT; // threads per dimension (16)
	extern __shared__ __align__(16) unsigned char smem_upd[];
	T (*As)[TL] = reinterpret_cast<T (*)[TL]>(smem_upd);
	T (*Bs)[TL] = reinterpret_cast<T (*)[TL]>(smem_upd+sizeof(T)*NB*TL);
	int4 tk = tasks[blockIdx.x];
	int s = tk.x, r0 = tk.y, cc0 = tk.z, k = tk.w;
	int n6 = dof*sn_n[s], F6 = n6+dof*sn_m[s], ld = sn_ld[s];
	int p0 = k*NB, w = min(NB, n6-p0), t0 = p0+w;
	T *base = arena+sn_off[s];
	bool extra = r0 >= F6;
	int rlim = extra ? F6+t0 : F6;
	int clim = n6;   // own columns only; the update matrix is k_syrk's
	int tx = threadIdx.x%TD, ty = threadIdx.x/TD;
	pdl_wait();
	// the tile's old values, loaded first: their latency overlaps the panel
	// loads and the products
	T old[TPT][TPT];
#pragma unroll
	for (int b = 0; b < TPT; b++) {
		int c = cc0+ty+TD*b;
#pragma unroll
		for (int a = 0; a < TPT; a++) {
			int r = r0+tx+TD*a;
			bool in = c < clim && r < rlim && (extra || r >= c);
			old[a][b] = in ? base[(int64_t)c*ld+r] : T(0);
		}
	}
	// load panel rows of the tile rows and tile columns
	{
		constexpr int PU = NB*TL/256;   // entries of each panel per thread, all loaded before the stores
		T av[PU], bv[PU];
#pragma unroll
		for (int u = 0; u < PU; u++) {
			int e = threadIdx.x+256*u;
			int t = e/TL, i = e%TL;
			int ra = r0+i, rb = cc0+i;
			av[u] = (t < w && ra < rlim) ? base[(int64_t)(p0+t)*ld+ra] : T(0);
			bv[u] = (t < w && rb < clim) ? base[(int64_t)(p0+t)*ld+rb] : T(0);
		}
		// row i = x + TD a of the tile (thread x's a-th row) goes to position
		// TPT x + a, so a thread's TPT values of one t are one vector load
#pragma unroll
		for (int u = 0; u < PU; u++) {
			int e = threadIdx.x+256*u;
			int i = e%TL, pi = TPT*(i%TD)+i/TD;
			As[e/TL][pi] = av[u];
			Bs[e/TL][pi] = bv[u];
		}
	}
	__syncthreads();
	T acc[TPT][TPT];
#pragma unroll
	for (int a = 0; a < TPT; a++)
#pragma unroll
		for (int b = 0; b < TPT; b++) acc[a][b] = 0;
	for (int t = 0; t < w; t++) {
		T av[TPT], bv[TPT];
		lds_chunk<T, TPT>(&As[t][TPT*tx], av);
		lds_chunk<T, TPT>(&Bs[t][TPT*ty], bv);
#pragma unroll
		for (int a = 0; a < TPT; a++)
#pragma unroll
			for (int b = 0; b < TPT; b++) acc[a][b] += av[a]*bv[b];
	}
	const bool diag = !extra && r0 == t0 && cc0 == t0;
	constexpr int LD = NB+1;
	T *Lsh = reinterpret_cast<T *>(smem_upd);   // diagonal-block work space (over As, Bs): Lsh first, 16-byte aligned
	T *Ls = Lsh+2*32*32;
	T *Vs = Ls+NB*LD;
	T *Ts = Vs+NB*LD;
	int *flags = reinterpret_cast<int *>(Ts+32*33);
	const int w1 = min(NB, n6-t0);   // width of panel k + 1
	// With NB == TL the diagonal tile is panel k + 1's diagonal block: its
	// entries in the block's rows go to Ls directly (diag_factor writes them
	// back), the rows below it to the front.
	const bool handoff = NB == TL && diag;
	if (handoff) __syncthreads();   // As, Bs are no longer read
#pragma unroll
	for (int b = 0; b < TPT; b++) {
		int c = cc0+ty+TD*b;
#pragma unroll
		for (int a = 0; a < TPT; a++) {
			int r = r0+tx+TD*a;
			T v = old[a][b]-acc[a][b];
			if (handoff) {
				int i = tx+TD*a, j = ty+TD*b;
				if (i < NB && j < NB) {
					T l = T(0);
					if (j <= i) {
						if (i < w1) l = v;
						else if (i == j) l = T(1);
					}
					Ls[i*LD+j] = l;
					Vs[i*LD+j] = T(0);
				}
				if (i < w1) continue;
			}
			if (c < clim && r < rlim && (extra || r >= c)) base[(int64_t)c*ld+r] = v;
		}
	}
	if (diag) {
		__syncthreads();   // this CTA's updates of the block are visible to all its threads
		if (!handoff) diag_load<T>(base, ld, t0, w1, Ls, Vs);
		if (threadIdx.x < 4) flags[threadIdx.x] = 0;
		__syncthreads();
		diag_factor<T>(base, ld, t0, w1, dof*sn_first[s]+t0, fail, Ls, Vs, Ts, Lsh, linv_slot<T>(linv, nsn, s, k+1),
		               flags);
	}
}


// Schur complement of a supernode: U[r][c] -= sum_{t < 6n} L[r][t] L[c][t]
// for 6n <= c <= r < 6F (tile (r0, c0) per CTA).  Deep-K loop over the
// supernode's columns in chunks of KC, next chunk prefetched into registers
// while the current one is multiplied from shared memory.
template <typename T>
__global__ void __launch_bounds__(256) k_syrk(const int4 *__restrict__ tasks, const int *__restrict__ sn_n,
                                              const int *__restrict__ sn_m, const int *__restrict__ sn_ld,
                                              const int64_t *__restrict__ sn_off, T *__restrict__ arena, int dof)
{
	constexpr int TL = Cfg<T>::STILE, TPT = Cfg<T>::STPT, TD = TL/TPT;
	constexpr int KC = 16;
	constexpr int PER = KC*TL/256;   // elements of A (and of B) each thread loads per chunk
	__shared__ T As[KC][TL];
	__shared__ T Bs[KC][TL];
	int4 tk = tasks[blockIdx.x];
	int s = tk.x, r0 = tk.y, c0 = tk.z;
	int n6 = dof*sn_n[s], F6 = n6+dof*sn_m[s], ld = sn_ld[s];
	T *base = arena+sn_off[s];
	pdl_wait();
	int tx = threadIdx.x%TD, ty = threadIdx.x/TD;
	T acc[TPT][TPT];
#pragma unroll
	for (int a = 0; a < TPT; a++)
#pragma unroll
		for (int b = 0; b < TPT; b++) acc[a][b] = 0;
	T pa[PER], pb[PER];
	auto load = [&](int t0) {
#pragma unroll
		for (int u = 0; u < PER; u++) {
			int e = threadIdx.x+256*u;
			int t = e/TL, i = e%TL;
			int col = t0+t;
			int ra = r0+i, rb = c0+i;
			pa[u] = (col < n6 && ra < F6) ? base[(int64_t)col*ld+ra] : T(0);
			pb[u] = (col < n6 && rb < F6) ? base[(int64_t)col*ld+rb] : T(0);
		}
	};
	load(0);
	for (int t0 = 0; t0 < n6; t0 += KC) {
		__syncthreads();
#pragma unroll
		for (int u = 0; u < PER; u++) {
			int e = threadIdx.x+256*u;
			As[e/TL][e%TL] = pa[u];
			Bs[e/TL][e%TL] = pb[u];
		}
		__syncthreads();
		if (t0+KC < n6) load(t0+KC);
#pragma unroll
		for (int t = 0; t < KC; t++) {
			T av[TPT], bv[TPT];
#pragma unroll
			for (int a = 0; a < TPT; a++) av[a] = As[t][tx+TD*a];
#pragma unroll
			for (int b = 0; b < TPT; b++) bv[b] = Bs[t][ty+TD*b];
#pragma unroll
			for (int a = 0; a < TPT; a++)
#pragma unroll
				for (int b = 0; b < TPT; b++) acc[a][b] += av[a]*bv[b];
		}
	}
	// old values loaded before the stores (as in k_update)
	T old[TPT][TPT];
#pragma unroll
	for (int b = 0; b < TPT; b++) {
		int c = c0+ty+TD*b;
#pragma unroll
		for (int a = 0; a < TPT; a++) {
			int r = r0+tx+TD*a;
			old[a][b] = (c < F6 && r < F6 && r >= c) ? base[(int64_t)c*ld+r] : T(0);
		}
	}
#pragma unroll
	for (int b = 0; b < TPT; b++) {
		int c = c0+ty+TD*b;
#pragma unroll
		for (int a = 0; a < TPT; a++) {
			int r = r0+tx+TD*a;
			if (c < F6 && r < F6 && r >= c) base[(int64_t)c*ld+r] = old[a][b]-acc[a][b];
		}
	}
}

// ---------------------------------------------------------------------------
// FP32 Schur complement on the tensor cores: k_syrk_tc.  tcgen05.mma
// (kind::tf32) with a 3xTF32 split: x = hi + lo with hi the TF32 part of x
// (the MMA reads only the upper 19 bits, so hi is x itself) and lo = x -
// hi exactly, so A B^T ~ Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T keeps FP32-level
// accuracy for the refinement.  One CTA (256 threads) per 128 x 128 tile of
// the update matrix; the accumulator lives in tensor memory (128 columns).
// K is walked in chunks of 32 (one 128-byte row of TF32): the threads
// transpose the chunk's column-major front data into K-major,
// 128-byte-swizzled shared-memory tiles in a ring of 3 stages, one thread
// issues 4 K-steps x 3 MMAs per chunk and commits them to the stage's
// mbarrier, and staging of the next chunks overlaps the MMAs.  Every mbarrier
// wait is bounded: on a timeout the CTA stops issuing, waits (bounded) for
// what it issued, frees its tensor memory and records the timeout (status 0)
// in *fail.
// ---------------------------------------------------------------------------
namespace umma {
constexpr int M = 128, N = 128, KC = 32, STAGES = 4;
constexpr int GROUP = 256;                // threads of a producer group (8 warps)
constexpr int GROUPS = 2;                 // group g stages the chunks ch = g (mod GROUPS)
constexpr int PRODUCERS = GROUPS*GROUP;   // warps 0-15: staging and epilogue
constexpr int THREADS = PRODUCERS+32;     // + warp 16: MMA issue
constexpr int TILE_BYTES = M*KC*4;           // one operand part (16 KB)
constexpr int STAGE_BYTES = 2*TILE_BYTES;    // B hi, B lo (A's parts are in tensor memory)
constexpr int SMEM_BYTES = STAGES*STAGE_BYTES+1024;
// tensor memory: the accumulator in columns [0, N), stage b's A hi / lo in
// columns ACOL + 2 KC b + [0, KC) / + KC + [0, KC)
constexpr int ACOL = N;
constexpr int TMEM_COLS = 512;
static_assert(ACOL+STAGES*2*KC <= TMEM_COLS, "tensor memory columns");
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__device__ inline uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1
__device__ inline uint64_t sdesc(uint32_t a)
{
	return (uint64_t)((a >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
	       ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = 128, M = 128
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
                           ((uint32_t)(M >> 4) << 24);

__device__ inline float tf32_lo(float x) { return x-__uint_as_float(__float_as_uint(x) & 0xffffe000u); }

__device__ inline bool mbar_wait(uint32_t bar, uint32_t parity)
{
	for (uint32_t it = 0; it < WAIT_LIMIT; it++) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
		             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		             "selp.u32 %0, 1, 0, p;\n\t}\n"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
	}
	return false;
}

// D (tensor memory) += A (tensor memory, lane = row, one column per K
// element) B^T (shared memory descriptor)
__device__ inline void mma_tf32(uint32_t dt, uint32_t at, uint64_t b, uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "setp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n"
	             :: "r"(dt), "r"(at), "l"(b), "r"(IDESC), "r"(accumulate));
}
__device__ inline void tmem_st16(uint32_t ta, const uint32_t (&v)[16])
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
	             "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};"
	             :: "r"(ta), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]),
	                "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
	                "r"(v[15]) : "memory");
}

__device__ inline void mbar_init(uint64_t *b, int count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(saddr(b)), "r"(count));
}
__device__ inline void mbar_arrive(uint64_t *b)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" :: "r"(saddr(b)) : "memory");
}
__device__ inline void mma_commit(uint64_t *b)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
	             :: "r"(saddr(b)) : "memory");
}
} // namespace umma

// Barriers of a tensor-core tile: per ring stage "full" (the producers'
// stores are in) and "empty" (the stage's MMAs are complete), and "done" (all
// MMAs complete).
struct TcBars { uint64_t full[umma::STAGES], empty[umma::STAGES], done; };

// One 128 x 128 tile C -= A B^T on the tensor cores, for the calling CTA
// (umma::THREADS threads): rows r0 + [0, 128) of A and c0 + [0, 128) of B
// taken from the front's columns [k0, k1) (A and B are rows of the same
// column-major front), C[r][c] at base[c ld + r] for r < rlim, c < clim and,
// when lower_only, r >= c.  tmem: this CTA's tensor memory; bars: fresh
// (phase 0).  Returns false if a wait timed out.
//
// Warp-specialised: two producer groups of 8 warps take alternate K chunks.
// A producer thread (row m, K half h) loads its chunk's values of A row m
// and B row m into registers one chunk of its group ahead, writes A's TF32
// hi / lo parts to tensor memory (tcgen05.st: a warp owns the 32 lanes =
// rows of its quarter) and B's parts to the swizzled shared stage, then
// arrives on the stage's full barrier.  The MMA warp waits on that, issues
// the stage's three products per K step (A hi B hi, A hi B lo, A lo B hi)
// and commits them to the stage's empty barrier, which the producers wait on
// before they reuse the stage.  No CTA-wide barrier in the K loop.  Then the
// producer warps run the epilogue (old values first, TMEM, stores).
__device__ bool tc_tile_update(float *base, int ld, int r0, int c0, int k0, int k1, int rlim, int clim,
                               bool lower_only, unsigned char *sm, TcBars &bars, uint32_t tmem)
{
	using namespace umma;
	const int tid = threadIdx.x, warp = tid/32, lane = tid%32;
	const int nchunk = (k1-k0+KC-1)/KC;
	constexpr int PW = PRODUCERS/32;
	bool ok = true;
	if (warp < PW) {
		const int g = warp/(GROUP/32), gt = tid-GROUP*g;
		const int m = gt & (M-1), h = gt >> 7, q = warp & 3;
		const int ra = r0+m, rb = c0+m;
		const bool va = ra < rlim, vb = rb < clim;
		auto load = [&](int ch, float (&a)[16], float (&b)[16]) {
			int tb = k0+ch*KC+16*h;
			const float *pa = base+(int64_t)tb*ld+ra, *pb = base+(int64_t)tb*ld+rb;
			int nk = ch < nchunk ? min(16, k1-tb) : 0;
#pragma unroll
			for (int k = 0; k < 16; k++) {
				a[k] = (k < nk && va) ? *pa : 0.f;
				b[k] = (k < nk && vb) ? *pb : 0.f;
				pa += ld;
				pb += ld;
			}
		};
		float av[16], bv[16];
		load(g, av, bv);
		for (int ch = g; ch < nchunk; ch += GROUPS) {
			int b = ch % STAGES;
			if (ch >= STAGES && !mbar_wait(saddr(&bars.empty[b]), ((ch/STAGES)-1) & 1)) ok = false;
			// B: 16-byte chunks (4 consecutive K); the 8 lanes of a quarter
			// warp (consecutive m) land on 8 distinct rows and swizzled chunk
			// columns, i.e. on all 32 banks
			unsigned char *stg = sm+b*STAGE_BYTES;
#pragma unroll
			for (int c4 = 0; c4 < 4; c4++) {
				int ck = 4*h+c4;
				uint32_t off = (uint32_t)((m >> 3)*1024+(m & 7)*128+((ck ^ (m & 7)) << 4));
				const float *bq = bv+4*c4;
				*reinterpret_cast<float4 *>(stg+0*TILE_BYTES+off) = make_float4(bq[0], bq[1], bq[2], bq[3]);
				*reinterpret_cast<float4 *>(stg+1*TILE_BYTES+off) =
					make_float4(tf32_lo(bq[0]), tf32_lo(bq[1]), tf32_lo(bq[2]), tf32_lo(bq[3]));
			}
			// A: lane = row of the warp's quarter, 16 columns = this K half
			uint32_t hi[16], lo[16];
#pragma unroll
			for (int k = 0; k < 16; k++) {
				hi[k] = __float_as_uint(av[k]);
				lo[k] = __float_as_uint(tf32_lo(av[k]));
			}
			uint32_t ta = tmem+((uint32_t)(32*q) << 16)+(uint32_t)(ACOL+2*KC*b+16*h);
			tmem_st16(ta, hi);
			tmem_st16(ta+KC, lo);
			asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // B visible to the tensor cores
			asm volatile("tcgen05.fence::before_thread_sync;");
			mbar_arrive(&bars.full[b]);
			load(ch+GROUPS, av, bv);
		}
	} else if (warp == PW && lane == 0) {
		for (int ch = 0; ch < nchunk; ch++) {
			int b = ch % STAGES;
			if (!mbar_wait(saddr(&bars.full[b]), (ch/STAGES) & 1)) { ok = false; break; }
			asm volatile("tcgen05.fence::after_thread_sync;");
			uint32_t sa = saddr(sm+b*STAGE_BYTES);
			uint32_t at = tmem+(uint32_t)(ACOL+2*KC*b);
#pragma unroll
			for (int kk = 0; kk < KC/8; kk++) {
				uint64_t bhi = sdesc(sa+0*TILE_BYTES+32*kk), blo = sdesc(sa+1*TILE_BYTES+32*kk);
				mma_tf32(tmem, at+8*kk, bhi, (ch > 0 || kk > 0) ? 1u : 0u);
				mma_tf32(tmem, at+8*kk, blo, 1u);
				mma_tf32(tmem, at+KC+8*kk, bhi, 1u);
			}
			mma_commit(&bars.empty[b]);
		}
		mma_commit(&bars.done);   // every MMA issued above is complete
	}
	if (warp < PW) {
		if (!mbar_wait(saddr(&bars.done), 0)) ok = false;
		asm volatile("tcgen05.fence::after_thread_sync;");
	}
	ok = __syncthreads_and(ok);
	if (ok && nchunk > 0 && warp < PW) {
		// warp w reads TMEM lanes 32 (w % 4) .. +32 (rows) and CPW columns
		constexpr int CPW = N/(PW/4);
		int q = warp & 3, grp = warp >> 2;
		int r = r0+32*q+lane;
		// the thread's old values, loaded before any store (the stores
		// would otherwise serialise the loads: the addresses may alias)
		float old[CPW];
		const float *po = base+(int64_t)(c0+CPW*grp)*ld+r;
#pragma unroll
		for (int j = 0; j < CPW; j++) {
			int c = c0+CPW*grp+j;
			old[j] = (r < rlim && c < clim && (!lower_only || r >= c)) ? *po : 0.f;
			po += ld;
		}
#pragma unroll
		for (int cb = CPW*grp; cb < CPW*grp+CPW; cb += 16) {
			uint32_t v[16];
			uint32_t ta = tmem+((uint32_t)(32*q) << 16)+(uint32_t)cb;
			asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
			             "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
			             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
			               "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
			               "=r"(v[14]), "=r"(v[15])
			             : "r"(ta));
			asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
			for (int j = 0; j < 16; j++) {
				int c = c0+cb+j;
				if (r < rlim && c < clim && (!lower_only || r >= c))
					base[(int64_t)c*ld+r] = old[cb-CPW*grp+j]-__uint_as_float(v[j]);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	return ok;
}

// tensor memory (all TMEM_COLS columns: one CTA per SM) and the barriers of a
// tensor-core CTA
__device__ inline uint32_t tc_setup(uint32_t *tmem_slot, TcBars &bars)
{
	using namespace umma;
	if (threadIdx.x/32 == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		             :: "r"(saddr(tmem_slot)), "r"(TMEM_COLS));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
		asm volatile("tcgen05.fence::before_thread_sync;");
	}
	if (threadIdx.x == 0) {
		for (int q = 0; q < STAGES; q++) {
			mbar_init(&bars.full[q], GROUP);
			mbar_init(&bars.empty[q], 1);
		}
		mbar_init(&bars.done, 1);
		asm volatile("fence.mbarrier_init.release.cluster;");
	}
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;");
	return *tmem_slot;
}

__device__ inline void tc_teardown(uint32_t tmem)
{
	if (threadIdx.x/32 == 0)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(umma::TMEM_COLS));
}

// Schur complement tile: U[r][c] -= sum_{t < 6n} L[r][t] L[c][t], lower part of [6n, 6F)^2
__global__ void __launch_bounds__(umma::THREADS, 1) k_syrk_tc(const int4 *__restrict__ tasks,
                                                              const int *__restrict__ sn_n,
                                                              const int *__restrict__ sn_m,
                                                              const int *__restrict__ sn_ld,
                                                              const int64_t *__restrict__ sn_off,
                                                              float *__restrict__ arena, int *fail, int dof)
{
	extern __shared__ unsigned char smem_tc[];
	__shared__ __align__(8) TcBars bars;
	__shared__ uint32_t tmem_slot;
	unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_tc)+1023) &
	                                                      ~static_cast<uintptr_t>(1023));
	int4 tk = tasks[blockIdx.x];
	int s = tk.x, r0 = tk.y, c0 = tk.z;
	int n6 = dof*sn_n[s], F6 = n6+dof*sn_m[s], ld = sn_ld[s];
	pdl_wait();   // before the tensor-memory allocation, too
	uint32_t tmem = tc_setup(&tmem_slot, bars);
	bool ok = tc_tile_update(arena+sn_off[s], ld, r0, c0, 0, n6, F6, F6, true, sm, bars, tmem);
	tc_teardown(tmem);
	if (!ok && threadIdx.x == 0 && fail) atomicMin(fail, 0);
}

// ---------------------------------------------------------------------------
// allocation and launch
// ---------------------------------------------------------------------------


template <typename T> static size_t update_smem()
{
	// the tile's two panels, or diag_factor's Lsh, Ls, Vs, Ts and flags
	constexpr int NB = Cfg<T>::NB;
	return std::max(sizeof(T)*2*NB*Cfg<T>::TILE, sizeof(T)*(2*32*32+2*NB*(NB+1)+32*33)+4*sizeof(int));
}

// assembly: one column of the largest front
template <typename T> static size_t assemble_smem(const DevSymbolic &D) { return sizeof(T)*(size_t)D.max_F; }

template <typename T> static void set_assemble_smem(const DevSymbolic &D)
{
	static std::once_flag warp_once;
	std::call_once(warp_once, [] {
		LFG_CUDA(cudaFuncSetAttribute(k_assemble_warp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                              (int)(sizeof(T)*ASM_WARP_MAXF*ASM_WARPS)));
	});
	static std::mutex mu;
	static size_t set = 48*1024;
	size_t need = assemble_smem<T>(D);
	std::lock_guard<std::mutex> g(mu);
	if (need <= set) return;
	if (need > 227*1024) throw Error{LFG_ERR_BAD_ARG, (int)D.max_F, "front too large for the assembly kernel"};
	LFG_CUDA(cudaFuncSetAttribute(k_assemble<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
	set = need;
}

// FP32 update launches of at most UPDATE_SOLO_TILES tiles (about three waves
// at one CTA per SM) ask for more shared memory than two CTAs can share, so
// the CTA that factors the next diagonal block -- the launch's critical path
// -- has its SM to itself.  Measured at N = 4096 over thresholds 0 to 1000:
// 480 was best, 7.58 -> 7.53 ms per step; at 1000 the tiles' waves outlast
// the diagonal block (7.89 ms).
constexpr int UPDATE_SOLO_TILES = 480;
constexpr size_t UPDATE_SOLO_SMEM = 120*1024;

template <typename T> static void set_update_smem()
{
	static std::once_flag once;
	std::call_once(once, [] {
		LFG_CUDA(cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                              (int)std::max(update_smem<T>(), UPDATE_SOLO_SMEM)));
		LFG_CUDA(cudaFuncSetAttribute(k_syrk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, umma::SMEM_BYTES));
	});
}

template <typename T> void factor_alloc(DevFactor<T> &F, const DevSymbolic &D, int kmax)
{
	if (F.arena_cap < D.arena_elems) {
		if (F.arena) cudaFree(F.arena);
		F.arena = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.arena, sizeof(T)*D.arena_elems));
		F.arena_cap = D.arena_elems;
	}
	int64_t wneed = D.w_elems*kmax;
	if (F.w_cap < wneed) {
		if (F.w) cudaFree(F.w);
		F.w = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.w, sizeof(T)*wneed));
		F.w_cap = wneed;
	}
	int64_t xneed = (int64_t)6*D.nblk*kmax;
	if (F.x_cap < xneed) {
		if (F.xp) cudaFree(F.xp);
		if (F.yp) cudaFree(F.yp);
		F.xp = F.yp = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.xp, sizeof(T)*xneed));
		LFG_CUDA(cudaMalloc((void **)&F.yp, sizeof(T)*xneed));
		F.x_cap = xneed;
	}
	int64_t lneed = (int64_t)2*D.nsn*Cfg<T>::NB*Cfg<T>::NB;
	if (F.linv_cap < lneed) {
		if (F.linv) cudaFree(F.linv);
		F.linv = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.linv, sizeof(T)*lneed));
		F.linv_cap = lneed;
	}
	F.pstride = std::max<int64_t>(D.w_elems, (int64_t)6*D.nblk);
	int64_t pneed = (int64_t)kmax*((D.max_n6+SOLVE_JC-1)/SOLVE_JC)*F.pstride;
	if (F.part_cap < pneed) {
		if (F.part) cudaFree(F.part);
		F.part = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.part, sizeof(T)*pneed));
		F.part_cap = pneed;
	}
	int64_t tneed = 1;
	for (const auto *tab : {&D.h_solve_phases, &D.h_mul_phases})
		for (const SolvePhase &p : *tab)
			if (p.nchunk > 1) tneed = std::max<int64_t>(tneed, (int64_t)p.gx*p.gy);
	if (F.tally_cap < tneed) {
		if (F.tally) cudaFree(F.tally);
		F.tally = nullptr;
		LFG_CUDA(cudaMalloc((void **)&F.tally, sizeof(int)*tneed));
		LFG_CUDA(cudaMemset(F.tally, 0, sizeof(int)*tneed));
		F.tally_cap = tneed;
	}
	if (!F.status) LFG_CUDA(cudaMalloc((void **)&F.status, sizeof(int)*4));
	set_update_smem<T>();
	set_assemble_smem<T>(D);
}

template <typename T> void factor_free(DevFactor<T> &F)
{
	if (F.arena) cudaFree(F.arena);
	if (F.w) cudaFree(F.w);
	if (F.xp) cudaFree(F.xp);
	if (F.yp) cudaFree(F.yp);
	if (F.status) cudaFree(F.status);
	if (F.linv) cudaFree(F.linv);
	if (F.part) cudaFree(F.part);
	if (F.tally) cudaFree(F.tally);
	F = DevFactor<T>();
}

__global__ void k_set_int(int *p, int v) { *p = v; }

template <typename T>
int factor_numeric(DevFactor<T> &F, const DevSymbolic &D, const double *dbl, const double *odbl,
                   cudaStream_t st)
{
	int launches = 0;
	k_set_int<<<1, 1, 0, st>>>(F.status, 0x7fffffff);
	launches++;
	for (const auto &L : D.factor_plan) {
		if (L.count <= 0) continue;
		switch (L.kind) {
		case PLAN_ASSEMBLE: {
			const int fmax = D.h_level_maxF6[L.level];
			if (fmax <= ASM_WARP_MAXF) {
				const int bufw = (fmax+3) & ~3;   // 16-byte aligned per-warp buffers
				launch_pdl(k_assemble_warp<T>, (L.count+ASM_WARPS-1)/ASM_WARPS, 32*ASM_WARPS,
				           sizeof(T)*(size_t)bufw*ASM_WARPS, st, (const int *)D.col_tasks+2*L.off, L.count, bufw,
				           (const int *)D.sn_n, (const int *)D.sn_m, (const int *)D.sn_ld,
				           (const int64_t *)D.sn_off, (const int *)D.child_off, (const int *)D.children,
				           (const int64_t *)D.cinv_off, (const int *)D.cinv, (const int *)D.sn_rows_off,
				           (const int *)D.cfwd, F.arena, D.dof);
			} else {
				launch_pdl(k_assemble<T>, L.count, ASM_THREADS, assemble_smem<T>(D), st,
				           (const int *)D.col_tasks+2*L.off,
				           (const int *)D.sn_n, (const int *)D.sn_m, (const int *)D.sn_ld,
				           (const int64_t *)D.sn_off, (const int *)D.child_off, (const int *)D.children,
				           (const int64_t *)D.cinv_off, (const int *)D.cinv, (const int *)D.sn_rows_off,
				           (const int *)D.cfwd, F.arena, D.dof);
			}
			break;
		}
		case PLAN_SCATTER: {
			int d0 = D.h_level_d_off[L.level], nd = D.h_level_d_off[L.level+1]-d0;
			int o0 = D.h_level_od_off[L.level], nod = D.h_level_od_off[L.level+1]-o0;
			launch_pdl(k_scatter<T>, (nd+nod+127)/128, 128, 0, st, nd, nod, (const int *)D.level_d+d0,
			           (const int *)D.level_od+o0, dbl, odbl, (const int *)D.d_sn, (const int *)D.d_bc,
			           (const int *)D.od_sn, (const int *)D.od_br, (const int *)D.od_bc, (const int *)D.od_tr,
			           (const int *)D.sn_ld, (const int64_t *)D.sn_off, F.arena, D.dof);
			break;
		}
		case PLAN_DIAG:
			launch_pdl(k_diag<T>, L.count, 256, 0, st, (const int4 *)D.diag_tasks+L.off, (const int *)D.sn_first,
			           (const int *)D.sn_ld, (const int64_t *)D.sn_off, F.arena, F.linv, D.nsn, F.status, D.dof);
			break;
		case PLAN_PANEL:
			launch_pdl(k_trsm<T>, L.count, 256, 0, st, (const int4 *)D.panel_tasks+L.off, (const int *)D.sn_n,
			           (const int *)D.sn_ld, (const int64_t *)D.sn_off, F.arena, F.linv, D.nsn, D.dof);
			break;
		case PLAN_UPDATE:
			launch_pdl(k_update<T>, L.count, 256,
			           std::is_same<T, float>::value && L.count <= UPDATE_SOLO_TILES ? UPDATE_SOLO_SMEM : update_smem<T>(),
			           st, (const int4 *)D.tile_tasks+L.off,
			           (const int *)D.sn_first, (const int *)D.sn_n, (const int *)D.sn_m, (const int *)D.sn_ld,
			           (const int64_t *)D.sn_off, F.arena, F.linv, D.nsn, F.status, D.dof);
			break;
		case PLAN_SYRK:
			launch_pdl(k_syrk<T>, L.count, 256, 0, st, (const int4 *)D.tile_tasks+L.off, (const int *)D.sn_n,
			           (const int *)D.sn_m, (const int *)D.sn_ld, (const int64_t *)D.sn_off, F.arena, D.dof);
			break;
		case PLAN_SYRK_TC:
			if (!std::is_same<T, float>::value) throw Error{LFG_ERR_BAD_ARG, 0, "tensor-core plan for FP64"};
			launch_pdl(k_syrk_tc, L.count, umma::THREADS, umma::SMEM_BYTES, st, (const int4 *)D.tile_tasks+L.off,
			           (const int *)D.sn_n, (const int *)D.sn_m, (const int *)D.sn_ld, (const int64_t *)D.sn_off,
			           reinterpret_cast<float *>(F.arena), F.status, D.dof);
			break;
		}
		launches++;
	}
	LFG_CUDA(cudaGetLastError());
	return launches;
}

// ---------------------------------------------------------------------------
// solves (k <= 4 right-hand sides, RHS-major: v[r*6n + i])
// ---------------------------------------------------------------------------
// Solve: forward (leaves first) and backward (root first) sweeps over the
// levels of the assembly tree, for K <= 4 right-hand sides (RHS-major:
// v[r*6n + i], permuted order).  Per level, forward:
//   gather  : v_top (own columns, in xp) += children's update vectors;
//             w_s (update rows) = children's update vectors
//   cols 0  : y = E^T v_top            (E = L11^-T, upper triangular)
//   rows 0  : w_s -= L21 y              (+ ordered sum of column chunks)
// backward:
//   cols 1  : z = y - L21^T x[rows of s]
//   rows 1  : x = E z                   (+ ordered sum of column chunks)
// A phase table built with the symbolic analysis lists the phases of a
// sweep; each runs as one launch of k_solve_phase with one CTA per work
// unit.  Column products take SOLVE_CB columns per unit (8 warps split the
// rows), row products 32 rows x SOLVE_JC columns (lanes own rows, warps
// split the columns; the last chunk of a row block to finish, found with a
// per-block counter, adds the chunks' partial sums).  Every sum runs in a
// fixed order: results are bitwise reproducible.  (One persistent kernel with grid barriers between phases
// was measured slower: the barriers cost more than the launch gaps.)

// Solve phases read their indices and the first batch of their factor
// entries before pdl_wait, overlapping the previous phase: the factor is
// complete before the second phase starts (the first phase does not trigger
// early and waits for the factorisation, whether both run as graphs or as
// plain launches in one stream) and constant during the solve; every other
// access follows the wait.

template <typename T> struct SolveArgs {
	const int *lev_sn, *sn_first, *sn_n, *sn_m, *sn_ld, *sn_rows_off, *rows;
	const int64_t *sn_off, *sn_woff, *cinv_off;
	const int *child_off, *children, *cinv, *iperm;
	const T *arena;
	T *w, *xp, *yp, *part;
	int *tally;
	int64_t wstride, pstride;
	int n, n6tot, dof;   // particles, scalar unknowns (dof n), unknowns per particle
	const double *b;
	double *x;
};

template <typename T> struct SolveShared {
	T red_c[SOLVE_WARPS][SOLVE_CB][4];
	T red_r[SOLVE_WARPS][4][32];
	int last;
};

template <typename T, int K>
__device__ void unit_gather(const SolveArgs<T> &A, const int *lev, int bx, int by)
{
	int s = lev[by];
	const int dof = A.dof;
	int n6 = dof*A.sn_n[s], F6 = n6+dof*A.sn_m[s];
	int r = bx*blockDim.x+threadIdx.x;
	if (r >= F6) return;
	int ca = A.child_off[s], cz = A.child_off[s+1];
	int rb = bdiv(r, dof), rr = bmod(r, dof);
	// the first children's source positions (symbolic) before the wait
	constexpr int CPRE = 4;
	int64_t src[CPRE];
#pragma unroll
	for (int c = 0; c < CPRE; c++) {
		src[c] = -1;
		if (ca+c < cz) {
			int ch = A.children[ca+c];
			int ic = A.cinv[A.cinv_off[ch]+rb];
			if (ic >= 0) src[c] = A.sn_woff[ch]+dof*(ic-A.sn_n[ch])+rr;
		}
	}
	T acc[K];
#pragma unroll
	for (int q = 0; q < K; q++) acc[q] = 0;
	pdl_wait();
#pragma unroll
	for (int c = 0; c < CPRE; c++)
		if (src[c] >= 0)
#pragma unroll
			for (int q = 0; q < K; q++) acc[q] += A.w[q*A.wstride+src[c]];
	for (int c = ca+CPRE; c < cz; c++) {
		int ch = A.children[c];
		int ic = A.cinv[A.cinv_off[ch]+rb];
		if (ic < 0) continue;
		int64_t sc = A.sn_woff[ch]+dof*(ic-A.sn_n[ch])+rr;
#pragma unroll
		for (int q = 0; q < K; q++) acc[q] += A.w[q*A.wstride+sc];
	}
	if (r < n6) {
		int g = dof*A.sn_first[s]+r;
#pragma unroll
		for (int q = 0; q < K; q++) A.xp[(int64_t)q*A.n6tot+g] += acc[q];
	} else {
		int64_t d = A.sn_woff[s]+(r-n6);
#pragma unroll
		for (int q = 0; q < K; q++) A.w[q*A.wstride+d] = acc[q];
	}
}

// MODE 0: y_j = sum_{i <= j} E[i][j] x_i;  MODE 1: z_j -= sum_t L21[t][j] x[rows(t)]
// The row loop takes SolveUnroll<T>::U rows of a thread per batch: all their loads are
// issued before the first multiply-add (the phases are latency-bound, one
// round trip per batch instead of per row); each thread still adds its rows
// in increasing order.
template <typename T> struct SolveUnroll { static constexpr int U = sizeof(T) == 4 ? 4 : 2; };

// one batch of a column product's rows: their positions (g < 0 past the
// rows) and factor entries
template <typename T, int U, int MODE>
__device__ __forceinline__ void cols_batch(int i0, int nrow, int f6, const int *R, const T *M, int ld, int j0, int jn,
                                           int dof, int64_t (&g)[U], T (&e)[U][SOLVE_CB], int stride)
{
#pragma unroll
	for (int u = 0; u < U; u++) {
		int i = i0+u*stride;
		g[u] = i >= nrow ? -1 : MODE == 0 ? f6+i : dof*R[bdiv(i, dof)]+bmod(i, dof);
#pragma unroll
		for (int c = 0; c < SOLVE_CB; c++)
			e[u][c] = (i >= nrow || c >= jn || (MODE == 0 && i > j0+c)) ? T(0) : __ldg(&M[(int64_t)c*ld+i]);
	}
}

template <typename T, int K, int MODE>
__device__ void unit_cols(const SolveArgs<T> &A, const int *lev, int bx, int by, SolveShared<T> &sh)
{
	constexpr int U = SolveUnroll<T>::U;
	int s = lev[by];
	const int dof = A.dof;
	int n6 = dof*A.sn_n[s], m6 = dof*A.sn_m[s], ld = A.sn_ld[s];
	int j0 = bx*SOLVE_CB;
	if (j0 >= n6 || (MODE == 1 && m6 == 0)) return;
	int jn = min(SOLVE_CB, n6-j0);
	int f6 = dof*A.sn_first[s];
	const T *M = A.arena+A.sn_off[s]+(MODE == 0 ? n6+m6 : n6)+(int64_t)j0*ld;
	const int *R = A.rows+A.sn_rows_off[s];
	int nrow = MODE == 0 ? j0+jn : m6;
	T acc[SOLVE_CB][K];
#pragma unroll
	for (int c = 0; c < SOLVE_CB; c++)
#pragma unroll
		for (int q = 0; q < K; q++) acc[c][q] = 0;
	int64_t g[U];
	T e[U][SOLVE_CB];
	cols_batch<T, U, MODE>(threadIdx.x, nrow, f6, R, M, ld, j0, jn, dof, g, e, blockDim.x);   // before the wait
	pdl_wait();
	for (int i0 = threadIdx.x; i0 < nrow; i0 += U*blockDim.x) {
		T v[U][K];
#pragma unroll
		for (int u = 0; u < U; u++)
#pragma unroll
			for (int q = 0; q < K; q++) v[u][q] = g[u] < 0 ? T(0) : A.xp[(int64_t)q*A.n6tot+g[u]];
#pragma unroll
		for (int u = 0; u < U; u++) {
			if (g[u] < 0) continue;
			int i = i0+u*blockDim.x;
#pragma unroll
			for (int c = 0; c < SOLVE_CB; c++) {
				if (c >= jn || (MODE == 0 && i > j0+c)) continue;
#pragma unroll
				for (int q = 0; q < K; q++) acc[c][q] += e[u][c]*v[u][q];
			}
		}
		int i1 = i0+U*blockDim.x;
		if (i1 < nrow) cols_batch<T, U, MODE>(i1, nrow, f6, R, M, ld, j0, jn, dof, g, e, blockDim.x);
	}
	int warp = threadIdx.x/32, lane = threadIdx.x%32;
#pragma unroll
	for (int c = 0; c < SOLVE_CB; c++)
#pragma unroll
		for (int q = 0; q < K; q++) {
			T a = acc[c][q];
			for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
			if (lane == 0) sh.red_c[warp][c][q] = a;
		}
	__syncthreads();
	if (threadIdx.x < SOLVE_CB*K) {
		int c = threadIdx.x/K, q = threadIdx.x%K;
		if (c < jn) {
			T a = 0;
			for (int u = 0; u < SOLVE_WARPS; u++) a += sh.red_c[u][c][q];
			T *o = A.yp+(int64_t)q*A.n6tot+f6+j0+c;
			if (MODE == 0) *o = a;
			else *o -= a;
		}
	}
}

// The same column products with one warp per unit (SOLVE_CB columns of one
// front), for levels whose products have few rows (at most SOLVE_WARP_ROWS):
// eight units per CTA instead of one, so a level of many small fronts fits
// in one wave.  Lanes take rows lane, lane + 32, ...; the SOLVE_CB x K
// partial sums are combined by a butterfly reduce-scatter (lane l ends with
// sum number l).
template <typename T, int K, int MODE>
__device__ void unit_cols_warp(const SolveArgs<T> &A, const int *lev, int units_x, int nfronts)
{
	constexpr int U = SolveUnroll<T>::U;
	constexpr int NV = SOLVE_CB*K;                            // sums of the unit
	constexpr int NVP = NV <= 8 ? 8 : NV <= 16 ? 16 : 32;     // padded to a power of two
	static_assert(NV <= 32, "one sum per lane");
	const int lane = threadIdx.x%32;
	const int unit = blockIdx.x*(blockDim.x/32)+threadIdx.x/32;
	const int bx = unit%units_x, by = unit/units_x;
	if (by >= nfronts) return;
	int s = lev[by];
	const int dof = A.dof;
	int n6 = dof*A.sn_n[s], m6 = dof*A.sn_m[s], ld = A.sn_ld[s];
	int j0 = bx*SOLVE_CB;
	if (j0 >= n6 || (MODE == 1 && m6 == 0)) return;
	int jn = min(SOLVE_CB, n6-j0);
	int f6 = dof*A.sn_first[s];
	const T *M = A.arena+A.sn_off[s]+(MODE == 0 ? n6+m6 : n6)+(int64_t)j0*ld;
	const int *R = A.rows+A.sn_rows_off[s];
	int nrow = MODE == 0 ? j0+jn : m6;
	T acc[NVP];
#pragma unroll
	for (int v = 0; v < NVP; v++) acc[v] = 0;
	int64_t g[U];
	T e[U][SOLVE_CB];
	cols_batch<T, U, MODE>(lane, nrow, f6, R, M, ld, j0, jn, dof, g, e, 32);   // before the wait
	pdl_wait();
	for (int i0 = lane; i0 < nrow; i0 += U*32) {
		T v[U][K];
#pragma unroll
		for (int u = 0; u < U; u++)
#pragma unroll
			for (int q = 0; q < K; q++) v[u][q] = g[u] < 0 ? T(0) : A.xp[(int64_t)q*A.n6tot+g[u]];
#pragma unroll
		for (int u = 0; u < U; u++) {
			if (g[u] < 0) continue;
			int i = i0+u*32;
#pragma unroll
			for (int c = 0; c < SOLVE_CB; c++) {
				if (c >= jn || (MODE == 0 && i > j0+c)) continue;
#pragma unroll
				for (int q = 0; q < K; q++) acc[c*K+q] += e[u][c]*v[u][q];
			}
		}
		int i1 = i0+U*32;
		if (i1 < nrow) cols_batch<T, U, MODE>(i1, nrow, f6, R, M, ld, j0, jn, dof, g, e, 32);
	}
	// reduce-scatter: halving steps over the lane bits below NVP; at each step
	// a lane keeps the half of its values whose index bit matches its lane
	// bit; then sums over the lane bits above
#pragma unroll
	for (int w = NVP/2; w >= 1; w /= 2) {
		const bool upper = (lane & w) != 0;
#pragma unroll
		for (int v = 0; v < w; v++) {
			T mine = upper ? acc[v+w] : acc[v];
			T other = upper ? acc[v] : acc[v+w];
			acc[v] = mine+__shfl_xor_sync(0xffffffffu, other, w);
		}
	}
#pragma unroll
	for (int w = NVP; w < 32; w *= 2) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], w);
	// lane l holds sum l % NVP
	if (lane < NV) {
		int c = lane/K, q = lane%K;
		if (c < jn) {
			T *o = A.yp+(int64_t)q*A.n6tot+f6+j0+c;
			if (MODE == 0) *o = acc[0];
			else *o -= acc[0];
		}
	}
}

// a row product's result for row `row` of right-hand side q
template <typename T, int MODE>
__device__ inline void rows_apply(const SolveArgs<T> &A, int q, int64_t row, T a)
{
	if (MODE == 0) A.w[q*A.wstride+row] -= a;
	else if (MODE == 3) A.w[q*A.wstride+row] += a;
	else if (MODE == 2) A.xp[(int64_t)q*A.n6tot+row] += a;
	else A.xp[(int64_t)q*A.n6tot+row] = a;
}

// MODE 0: w_t -= sum_j L21[t][j] y_j;  MODE 1: x_i = sum_{j >= i} E[i][j] z_j
// (product with L, y in yp): MODE 2: x_i += sum_{j <= i} L11[i][j] y_j;
// MODE 3: w_t += sum_j L21[t][j] y_j
template <typename T, int K, int MODE>
__device__ void unit_rows(const SolveArgs<T> &A, const int *lev, int bx, int by, int bz, int nchunk,
                          SolveShared<T> &sh)
{
	constexpr bool UPD = MODE == 0 || MODE == 3;   // rows of the update block (w)
	int s = lev[by];
	const int dof = A.dof;
	int n6 = dof*A.sn_n[s], m6 = dof*A.sn_m[s], ld = A.sn_ld[s];
	int nrows = UPD ? m6 : n6;
	int r0 = bx*32;
	if (r0 >= nrows) return;
	int warp = threadIdx.x/32, lane = threadIdx.x%32;
	int f6 = dof*A.sn_first[s];
	int jlo = (MODE == 1 ? r0 : 0)+bz*SOLVE_JC;
	int jhi = min(n6, jlo+SOLVE_JC);
	const T *M = A.arena+A.sn_off[s]+(UPD ? n6 : MODE == 1 ? n6+m6 : 0);
	int r = r0+lane;
	T acc[K];
#pragma unroll
	for (int q = 0; q < K; q++) acc[q] = 0;
	// RU columns of a warp per batch, the factor entries of the first batch
	// before the wait, loads ahead of the multiply-adds (see unit_cols).
	// Unmasked by the triangle: column j < n6 of a front is allocated down
	// to its last row (the masked product skips it).
	constexpr int RU = 2*SolveUnroll<T>::U;
	T e[RU];
	int jb = jlo+warp;
#pragma unroll
	for (int u = 0; u < RU; u++) {
		int j = jb+u*SOLVE_WARPS;
		e[u] = (r < nrows && j < jhi) ? __ldg(&M[(int64_t)j*ld+r]) : T(0);
	}
	pdl_wait();
	if (r < nrows) {
		for (int j0 = jb; j0 < jhi; j0 += RU*SOLVE_WARPS) {
			T y[RU][K];
#pragma unroll
			for (int u = 0; u < RU; u++) {
				int j = j0+u*SOLVE_WARPS;
#pragma unroll
				for (int q = 0; q < K; q++) y[u][q] = j < jhi ? A.yp[(int64_t)q*A.n6tot+f6+j] : T(0);
			}
#pragma unroll
			for (int u = 0; u < RU; u++) {
				int j = j0+u*SOLVE_WARPS;
				if (j >= jhi || (MODE == 1 && j < r) || (MODE == 2 && j > r)) continue;
#pragma unroll
				for (int q = 0; q < K; q++) acc[q] += e[u]*y[u][q];
			}
			int j1 = j0+RU*SOLVE_WARPS;
			if (j1 < jhi)
#pragma unroll
				for (int u = 0; u < RU; u++) {
					int j = j1+u*SOLVE_WARPS;
					e[u] = j < jhi ? __ldg(&M[(int64_t)j*ld+r]) : T(0);
				}
		}
	}
#pragma unroll
	for (int q = 0; q < K; q++) sh.red_r[warp][q][lane] = acc[q];
	__syncthreads();
	if (warp == 0 && r < nrows) {
		int64_t row = UPD ? A.sn_woff[s]+r : (int64_t)f6+r;
#pragma unroll
		for (int q = 0; q < K; q++) {
			T a = 0;
			for (int u = 0; u < SOLVE_WARPS; u++) a += sh.red_r[u][q][lane];
			if (nchunk == 1) rows_apply<T, MODE>(A, q, row, a);
			else A.part[((int64_t)q*nchunk+bz)*A.pstride+row] = a;
		}
	}
	if (nchunk == 1) return;
	// The chunk that completes this row block adds the chunks' partial sums
	// in chunk order (the same sum a separate launch would form).  The
	// fence orders each chunk's partial stores before its count.
	__threadfence();
	__syncthreads();
	int *cnt = A.tally+(int64_t)by*gridDim.x+bx;
	if (threadIdx.x == 0) sh.last = atomicAdd(cnt, 1) == nchunk-1;
	__syncthreads();
	if (!sh.last) return;
	__threadfence();
	if (warp == 0 && r < nrows) {
		int64_t row = UPD ? A.sn_woff[s]+r : (int64_t)f6+r;
#pragma unroll
		for (int q = 0; q < K; q++) {
			T a = 0;
			for (int c = 0; c < nchunk; c++) a += __ldcg(&A.part[((int64_t)q*nchunk+c)*A.pstride+row]);
			rows_apply<T, MODE>(A, q, row, a);
		}
	}
	if (threadIdx.x == 0) *cnt = 0;   // ready for the next row-product phase
}

// in: b (permuted) into xp; in_y (product with L): b into yp and xp zeroed;
// out: xp (unpermuted) into x.  b and x keep 6 values per particle; with
// dof 3 only components 0, 2, 4 (x, z translation, y rotation) are unknowns:
// the others of b are not read and those of x are written as 0.
template <typename T, int K>
__device__ void unit_permute(const SolveArgs<T> &A, int bx, bool in, bool in_y = false)
{
	int t = bx*blockDim.x+threadIdx.x;
	if (t >= 6*A.n) return;
	int i = t/6, d = t%6;
	const int64_t n6 = A.n6tot;
	int q;
	if (A.dof == 6) q = 6*A.iperm[i]+d;
	else q = (d & 1) ? -1 : 3*A.iperm[i]+d/2;
	pdl_wait();
	if (q < 0) {
		if (!in && !in_y)
			for (int r = 0; r < K; r++) A.x[(int64_t)r*6*A.n+t] = 0.0;
		return;
	}
	if (in_y) {
		for (int r = 0; r < K; r++) {
			A.yp[(int64_t)r*n6+q] = (T)A.b[(int64_t)r*6*A.n+t];
			A.xp[(int64_t)r*n6+q] = T(0);
		}
	} else if (in)
		for (int r = 0; r < K; r++) A.xp[(int64_t)r*n6+q] = (T)A.b[(int64_t)r*6*A.n+t];
	else
		for (int r = 0; r < K; r++) A.x[(int64_t)r*6*A.n+t] = (double)A.xp[(int64_t)r*n6+q];
}

// one phase as its own launch: one CTA per work unit; one instantiation per
// phase type, so each gets its own register budget
template <typename T, int K, int TYPE>
__global__ void __launch_bounds__(256) k_solve_phase(SolveArgs<T> A, SolvePhase ph)
{
	__shared__ SolveShared<T> sh;
	// The first phase (permutation in) lets the next one start only when it
	// has finished, i.e. after the factorisation it waits for: the later
	// phases read factor entries before their wait.
	if (TYPE != SP_PERM_IN && TYPE != SP_PERM_IN_Y) pdl_trigger();
	const int *lev = A.lev_sn+ph.lev_off;
	int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
	if (TYPE == SP_PERM_IN) unit_permute<T, K>(A, bx, true);
	if (TYPE == SP_GATHER) unit_gather<T, K>(A, lev, bx, by);
	if (TYPE == SP_COLS0) unit_cols<T, K, 0>(A, lev, bx, by, sh);
	if (TYPE == SP_ROWS0) unit_rows<T, K, 0>(A, lev, bx, by, bz, ph.nchunk, sh);
	if (TYPE == SP_COLS1) unit_cols<T, K, 1>(A, lev, bx, by, sh);
	if (TYPE == SP_COLS0W) unit_cols_warp<T, K, 0>(A, lev, ph.gx, ph.gy);
	if (TYPE == SP_COLS1W) unit_cols_warp<T, K, 1>(A, lev, ph.gx, ph.gy);
	if (TYPE == SP_ROWS1) unit_rows<T, K, 1>(A, lev, bx, by, bz, ph.nchunk, sh);
	if (TYPE == SP_PERM_OUT) unit_permute<T, K>(A, bx, false);
	if (TYPE == SP_PERM_IN_Y) unit_permute<T, K>(A, bx, true, true);
	if (TYPE == SP_MUL_TOP) unit_rows<T, K, 2>(A, lev, bx, by, bz, ph.nchunk, sh);
	if (TYPE == SP_MUL_UPD) unit_rows<T, K, 3>(A, lev, bx, by, bz, ph.nchunk, sh);
}

template <typename T, int K>
static void launch_phase(const SolveArgs<T> &A, const SolvePhase &p, cudaStream_t st)
{
	dim3 g(p.gx, p.gy, p.gz);
	switch (p.type) {
	case SP_PERM_IN: launch_pdl(k_solve_phase<T, K, SP_PERM_IN>, g, 256, 0, st, A, p); break;
	case SP_GATHER: launch_pdl(k_solve_phase<T, K, SP_GATHER>, g, 256, 0, st, A, p); break;
	case SP_COLS0: launch_pdl(k_solve_phase<T, K, SP_COLS0>, g, 256, 0, st, A, p); break;
	case SP_ROWS0: launch_pdl(k_solve_phase<T, K, SP_ROWS0>, g, 256, 0, st, A, p); break;
	case SP_COLS1: launch_pdl(k_solve_phase<T, K, SP_COLS1>, g, 256, 0, st, A, p); break;
	case SP_ROWS1: launch_pdl(k_solve_phase<T, K, SP_ROWS1>, g, 256, 0, st, A, p); break;
	case SP_PERM_IN_Y: launch_pdl(k_solve_phase<T, K, SP_PERM_IN_Y>, g, 256, 0, st, A, p); break;
	case SP_MUL_TOP: launch_pdl(k_solve_phase<T, K, SP_MUL_TOP>, g, 256, 0, st, A, p); break;
	case SP_MUL_UPD: launch_pdl(k_solve_phase<T, K, SP_MUL_UPD>, g, 256, 0, st, A, p); break;
	case SP_COLS0W: case SP_COLS1W: {
		dim3 gw((p.gx*p.gy+7)/8, 1, 1);   // eight warp units per CTA
		if (p.type == SP_COLS0W) launch_pdl(k_solve_phase<T, K, SP_COLS0W>, gw, 256, 0, st, A, p);
		else launch_pdl(k_solve_phase<T, K, SP_COLS1W>, gw, 256, 0, st, A, p);
		break;
	}
	default: launch_pdl(k_solve_phase<T, K, SP_PERM_OUT>, g, 256, 0, st, A, p); break;
	}
}

// Phase table of one sweep (forward levels leaves first, backward levels
// root first); the grid extents are those of the former per-phase launches.
void solve_plan_build(DevSymbolic &D, cudaStream_t st)
{
	std::vector<SolvePhase> P;
	auto add = [&](int type, int lev_off, int gx, int gy, int gz, int nchunk) {
		P.push_back(SolvePhase{type, lev_off, gx, gy, gz, nchunk});
	};
	int n = D.nblk;
	add(SP_PERM_IN, 0, (6*n+255)/256, 1, 1, 1);
	for (int l = 0; l < D.nlevels; l++) {
		int off = D.h_level_off[l], cnt = D.h_level_off[l+1]-off;
		if (!cnt) continue;
		int n6 = D.h_level_maxn6[l], m6 = D.h_level_maxm6[l];
		add(SP_GATHER, off, (n6+m6+255)/256, cnt, 1, 1);
		add(n6 <= SOLVE_WARP_ROWS ? SP_COLS0W : SP_COLS0, off, (n6+SOLVE_CB-1)/SOLVE_CB, cnt, 1, 1);
		if (m6 > 0) {
			int nch = (n6+SOLVE_JC-1)/SOLVE_JC;
			add(SP_ROWS0, off, (m6+31)/32, cnt, nch, nch);
		}
	}
	for (int l = D.nlevels-1; l >= 0; l--) {
		int off = D.h_level_off[l], cnt = D.h_level_off[l+1]-off;
		if (!cnt) continue;
		int n6 = D.h_level_maxn6[l], m6 = D.h_level_maxm6[l];
		if (m6 > 0) add(m6 <= SOLVE_WARP_ROWS ? SP_COLS1W : SP_COLS1, off, (n6+SOLVE_CB-1)/SOLVE_CB, cnt, 1, 1);
		int nch = (n6+SOLVE_JC-1)/SOLVE_JC;
		add(SP_ROWS1, off, (n6+31)/32, cnt, nch, nch);
	}
	add(SP_PERM_OUT, 0, (6*n+255)/256, 1, 1, 1);
	D.h_solve_phases = P;
	// product y = P^T L P b (compute_LTRHS): per level leaves first, gather
	// the children's update vectors, x_top += L11 b_top, w += L21 b_top
	std::vector<SolvePhase> M;
	P.swap(M);
	add(SP_PERM_IN_Y, 0, (6*n+255)/256, 1, 1, 1);
	for (int l = 0; l < D.nlevels; l++) {
		int off = D.h_level_off[l], cnt = D.h_level_off[l+1]-off;
		if (!cnt) continue;
		int n6 = D.h_level_maxn6[l], m6 = D.h_level_maxm6[l];
		int nch = (n6+SOLVE_JC-1)/SOLVE_JC;
		add(SP_GATHER, off, (n6+m6+255)/256, cnt, 1, 1);
		add(SP_MUL_TOP, off, (n6+31)/32, cnt, nch, nch);
		if (m6 > 0) {
			add(SP_MUL_UPD, off, (m6+31)/32, cnt, nch, nch);
		}
	}
	add(SP_PERM_OUT, 0, (6*n+255)/256, 1, 1, 1);
	D.h_mul_phases = P;
	P.swap(M);
	(void)st;
}

template <typename T, int K>
static int solve_k(DevFactor<T> &F, const DevSymbolic &D, const std::vector<SolvePhase> &phases,
                   const double *b, double *x, cudaStream_t st)
{
	SolveArgs<T> A;
	A.lev_sn = D.level_sn; A.sn_first = D.sn_first; A.sn_n = D.sn_n; A.sn_m = D.sn_m; A.sn_ld = D.sn_ld;
	A.sn_rows_off = D.sn_rows_off; A.rows = D.rows; A.sn_off = D.sn_off; A.sn_woff = D.sn_woff;
	A.cinv_off = D.cinv_off; A.child_off = D.child_off; A.children = D.children; A.cinv = D.cinv;
	A.iperm = D.iperm; A.arena = F.arena; A.w = F.w; A.xp = F.xp; A.yp = F.yp; A.part = F.part; A.tally = F.tally;
	A.wstride = D.w_elems; A.pstride = F.pstride; A.n = D.nblk; A.n6tot = D.dof*D.nblk; A.dof = D.dof;
	A.b = b; A.x = x;
	for (const SolvePhase &p : phases) launch_phase<T, K>(A, p, st);
	LFG_CUDA(cudaGetLastError());
	return (int)phases.size();
}

template <typename T>
static int run_sweeps(DevFactor<T> &F, const DevSymbolic &D, const std::vector<SolvePhase> &ph, int k,
                      const double *b, double *x, cudaStream_t st)
{
	int launches = 0;
	for (int r0 = 0; r0 < k; r0 += 4) {
		int kk = std::min(4, k-r0);
		const double *bb = b+(int64_t)r0*6*D.nblk;
		double *xx = x+(int64_t)r0*6*D.nblk;
		switch (kk) {
		case 1: launches += solve_k<T, 1>(F, D, ph, bb, xx, st); break;
		case 2: launches += solve_k<T, 2>(F, D, ph, bb, xx, st); break;
		case 3: launches += solve_k<T, 3>(F, D, ph, bb, xx, st); break;
		default: launches += solve_k<T, 4>(F, D, ph, bb, xx, st); break;
		}
	}
	return launches;
}

template <typename T>
int factor_solve(DevFactor<T> &F, const DevSymbolic &D, int k, const double *b, double *x, cudaStream_t st)
{
	return run_sweeps(F, D, D.h_solve_phases, k, b, x, st);
}

// y = L b with the factor (R = L L^T in the caller's order): StokesSolver::
// compute_LTRHS (StokesSolver.cpp:627-669) for the Brownian force
template <typename T>
int factor_multiply(DevFactor<T> &F, const DevSymbolic &D, int k, const double *b, double *x, cudaStream_t st)
{
	return run_sweeps(F, D, D.h_mul_phases, k, b, x, st);
}

// ---------------------------------------------------------------------------
// FP64 block residual r = b - A x (row-block gather, deterministic)
// ---------------------------------------------------------------------------
// Dense position r*6+c of a compact block: 0 = structural zero, otherwise
// +-(index+1) into the compact storage.  DSYM is the full symmetric diagonal
// block of the 15-value storage, ODENSE the 18-value off-diagonal block; both
// follow d15_to_dense / od18_to_dense above.
__constant__ signed char c_dsym[36] = {1, 2, 3, 0, 4, 5, 2, 6, 7, -4, 0, 8, 3, 7, 9, -5, -8, 0,
                                       0, -4, -5, 10, 11, 12, 4, 0, -8, 11, 13, 14, 5, 8, 0, 12, 14, 15};
__constant__ signed char c_odense[36] = {1, 2, 3, 0, -10, -11, 2, 6, 7, 10, 0, -15, 3, 7, 9, 11, 15, 0,
                                         0, -4, -5, 12, 13, 14, 4, 0, -8, 13, 16, 17, 5, 8, 0, 14, 17, 18};

__device__ inline void warp_expand(const double *src, const signed char *tab, double *m, int lane)
{
	for (int p = lane; p < 36; p += 32) {
		int t = tab[p];
		m[p] = t == 0 ? 0.0 : (t > 0 ? src[t-1] : -src[-t-1]);
	}
	__syncwarp();
}

// r = b - A x, one warp per block row i: lane = 6 * rhs + a owns output entry
// a of right-hand side rhs (up to 4 right-hand sides per pass).  Each block
// is expanded once into the warp's shared 6x6 buffer.  Blocks are visited in
// a fixed order (diagonal, row i's lower blocks, then its upper blocks), so
// the result is reproducible.
__global__ void __launch_bounds__(256) k_residual(int n, int k, const double *__restrict__ dbl,
                           const double *__restrict__ odbl, const int *__restrict__ od_row,
                           const int *__restrict__ od_col, const int *__restrict__ lo_ptr,
                           const int *__restrict__ lo_idx, const int *__restrict__ up_ptr,
                           const int *__restrict__ up_idx, const double *__restrict__ b,
                           const double *__restrict__ x, double *__restrict__ r, int dof)
{
	__shared__ double sm[8][36];
	int w = threadIdx.x/32, lane = threadIdx.x%32;
	int i = blockIdx.x*8+w;
	if (i >= n) return;
	double *m = sm[w];
	for (int q0 = 0; q0 < k; q0 += 4) {
		int q = q0+lane/6, a = lane%6;
		bool act = lane < 24 && q < k;
		const double *xv = x+(int64_t)(act ? q : 0)*6*n;
		double acc = 0;
		warp_expand(dbl+15*(int64_t)i, c_dsym, m, lane);
		if (act)
			for (int c = 0; c < 6; c++) acc += m[a*6+c]*xv[6*i+c];
		for (int t = lo_ptr[i]; t < lo_ptr[i+1]; t++) {
			int e = lo_idx[t];
			__syncwarp();
			warp_expand(odbl+18*(int64_t)e, c_odense, m, lane);
			if (act) {
				int j = od_col[e];
				for (int c = 0; c < 6; c++) acc += m[a*6+c]*xv[6*j+c];
			}
		}
		for (int t = up_ptr[i]; t < up_ptr[i+1]; t++) {
			int e = up_idx[t];
			__syncwarp();
			warp_expand(odbl+18*(int64_t)e, c_odense, m, lane);
			if (act) {
				int j = od_row[e];
				for (int c = 0; c < 6; c++) acc += m[c*6+a]*xv[6*j+c];
			}
		}
		// dof 3: only components 0, 2, 4 are unknowns of the system (the
		// out-of-plane ones are neither solved nor part of the residual)
		if (act) r[(int64_t)q*6*n+6*i+a] = (dof == 3 && (a & 1)) ? 0.0 : b[(int64_t)q*6*n+6*i+a]-acc;
		__syncwarp();
	}
}

void block_residual(const DevBlockMatrix &A, int k, const double *b, const double *x, double *r,
                    cudaStream_t st)
{
	k_residual<<<(A.n+7)/8, 256, 0, st>>>(A.n, k, A.dblocks, A.odblocks, A.od_row, A.od_col, A.lo_ptr,
	                                      A.lo_idx, A.up_ptr, A.up_idx, b, x, r, A.dof);
}

__global__ void k_axpy(int64_t total, const double *__restrict__ d, double *__restrict__ x)
{
	int64_t t = blockIdx.x*(int64_t)blockDim.x+threadIdx.x;
	if (t < total) x[t] += d[t];
}

void axpy_vec(int n, int k, const double *d, double *x, cudaStream_t st)
{
	int64_t total = (int64_t)6*n*k;
	k_axpy<<<(int)((total+255)/256), 256, 0, st>>>(total, d, x);
}

// per-RHS sums of squares of r and b, single CTA per RHS (fixed order)
// squared norms of r and b per right-hand side (one CTA of 1024 threads each;
// a fixed reduction order: per thread, then warps by shuffles, then warps)
// squared norms of r and b per right-hand side and segment: segment q of a
// right-hand side is entries [seg[q], seg[q+1]) (one segment, [0, n6), when
// seg is null); out[2 (rh nseg + q)] = |r|^2, then |b|^2
__global__ void __launch_bounds__(1024) k_norms(int n6, const double *__restrict__ r, const double *__restrict__ b,
                                                const int *__restrict__ seg, double *out)
{
	__shared__ double sr[32], sb[32];
	int rh = blockIdx.x, q = blockIdx.y, nseg = gridDim.y;
	int lo = seg ? seg[q] : 0, hi = seg ? seg[q+1] : n6;
	double a = 0, c = 0;
#pragma unroll 4
	for (int i = lo+threadIdx.x; i < hi; i += blockDim.x) {
		double u = r[(int64_t)rh*n6+i], v = b[(int64_t)rh*n6+i];
		a += u*u;
		c += v*v;
	}
	for (int o = 16; o > 0; o >>= 1) {
		a += __shfl_down_sync(FULL_MASK, a, o);
		c += __shfl_down_sync(FULL_MASK, c, o);
	}
	int w = threadIdx.x/32, l = threadIdx.x%32;
	if (l == 0) { sr[w] = a; sb[w] = c; }
	__syncthreads();
	if (w == 0) {
		a = l < (int)blockDim.x/32 ? sr[l] : 0.0;
		c = l < (int)blockDim.x/32 ? sb[l] : 0.0;
		for (int o = 16; o > 0; o >>= 1) {
			a += __shfl_down_sync(FULL_MASK, a, o);
			c += __shfl_down_sync(FULL_MASK, c, o);
		}
		if (l == 0) { out[2*(rh*nseg+q)] = a; out[2*(rh*nseg+q)+1] = c; }
	}
}

void residual_norms(int n6, int k, const double *r, const double *b, double *out, cudaStream_t st,
                    const int *seg, int nseg)
{
	k_norms<<<dim3(k, seg ? nseg : 1), 1024, 0, st>>>(n6, r, b, seg, out);
}

int factor_tile_size(int precision) { return precision == LFG_PREC_FP64 ? Cfg<double>::TILE : Cfg<float>::TILE; }
int factor_syrk_tile_size(int precision) { return precision == LFG_PREC_FP64 ? Cfg<double>::STILE : Cfg<float>::STILE; }
int factor_panel_rows() { return PANEL_ROWS; }
int factor_panel_width(int precision) { return precision == LFG_PREC_FP64 ? Cfg<double>::NB : Cfg<float>::NB; }

template void factor_alloc<double>(DevFactor<double> &, const DevSymbolic &, int);
template void factor_alloc<float>(DevFactor<float> &, const DevSymbolic &, int);
template void factor_free<double>(DevFactor<double> &);
template void factor_free<float>(DevFactor<float> &);
template int factor_numeric<double>(DevFactor<double> &, const DevSymbolic &, const double *, const double *, cudaStream_t);
template int factor_numeric<float>(DevFactor<float> &, const DevSymbolic &, const double *, const double *, cudaStream_t);
template int factor_multiply<double>(DevFactor<double> &, const DevSymbolic &, int, const double *, double *,
                                     cudaStream_t);
template int factor_multiply<float>(DevFactor<float> &, const DevSymbolic &, int, const double *, double *,
                                    cudaStream_t);
template int factor_solve<double>(DevFactor<double> &, const DevSymbolic &, int, const double *, double *, cudaStream_t);
template int factor_solve<float>(DevFactor<float> &, const DevSymbolic &, int, const double *, double *, cudaStream_t);

} // namespace lfg

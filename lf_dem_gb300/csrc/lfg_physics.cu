// lfg_physics.cu -- per-step physics of LF_DEM's hydrodynamic core on the
// device: Lees-Edwards cell lists and pair discovery, Interaction updates
// (contact springs, friction laws, lubrication coefficients, repulsion),
// R_FU block assembly, RHS force components, stresslets, stress-controlled
// shear rate, velocity assembly and the predictor-corrector moves.
//
// Compiled with --fmad=false: geometry and contact tests round exactly like
// LF_DEM's scalar C++ (System.cpp:2517-2548, Interaction.cpp:124-135), so the
// pair list and the contact states are bit-identical on identical inputs.
// Every per-particle sum is a gather over the pair list in a fixed order (no
// floating-point atomics), so the engine is bitwise reproducible.
#include <cstdio>
#include <mutex>

#include "lfg_physics.h"

namespace lfg {

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

// ---------------------------------------------------------------------------
// small vector / tensor helpers (vec3d.h, Sym2Tensor.h)
// ---------------------------------------------------------------------------
struct v3 { double x, y, z; };
__device__ __forceinline__ v3 V(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return V(a.x+b.x, a.y+b.y, a.z+b.z); }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return V(a.x-b.x, a.y-b.y, a.z-b.z); }
__device__ __forceinline__ v3 vscale(double s, v3 a) { return V(s*a.x, s*a.y, s*a.z); }
__device__ __forceinline__ v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
__device__ __forceinline__ double vdot(v3 a, v3 b) { return a.x*b.x+a.y*b.y+a.z*b.z; }
__device__ __forceinline__ double vsq(v3 a) { return a.x*a.x+a.y*a.y+a.z*a.z; }
__device__ __forceinline__ v3 vcross(v3 a, v3 b) { return V(a.y*b.z-a.z*b.y, a.z*b.x-a.x*b.z, a.x*b.y-a.y*b.x); }
__device__ __forceinline__ v3 vzero() { return V(0, 0, 0); }
__device__ __forceinline__ v3 ld3(const double *p) { return V(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(double *p, v3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
// Sym2Tensor.h:227-234
__device__ __forceinline__ v3 sdot(const double *s, v3 v)
{
	return V(s[0]*v.x + s[1]*v.y + s[2]*v.z, s[1]*v.x + s[4]*v.y + s[3]*v.z, s[2]*v.x + s[3]*v.y + s[5]*v.z);
}
struct s2 { double e[6]; };
__device__ __forceinline__ s2 szero() { s2 r; for (int i = 0; i < 6; i++) r.e[i] = 0; return r; }
__device__ __forceinline__ void sadd_to(s2 &a, const s2 &b) { for (int i = 0; i < 6; i++) a.e[i] += b.e[i]; }
__device__ __forceinline__ s2 sscale(double c, const s2 &a) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = c*a.e[i]; return r; }
__device__ __forceinline__ s2 ssub(const s2 &a, const s2 &b) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = a.e[i]-b.e[i]; return r; }
__device__ __forceinline__ s2 saddv(const s2 &a, const s2 &b) { s2 r; for (int i = 0; i < 6; i++) r.e[i] = a.e[i]+b.e[i]; return r; }
__device__ __forceinline__ s2 outer_sym(v3 a, v3 b)
{
	s2 r;
	r.e[0] = a.x*b.x; r.e[1] = 0.5*(a.x*b.y+a.y*b.x); r.e[2] = 0.5*(a.x*b.z+a.z*b.x);
	r.e[3] = 0.5*(a.y*b.z+a.z*b.y); r.e[4] = a.y*b.y; r.e[5] = a.z*b.z;
	return r;
}
__device__ __forceinline__ s2 outer(v3 a)
{
	s2 r;
	r.e[0] = a.x*a.x; r.e[1] = a.x*a.y; r.e[2] = a.x*a.z; r.e[3] = a.y*a.z; r.e[4] = a.y*a.y; r.e[5] = a.z*a.z;
	return r;
}
__device__ __forceinline__ double doubledot(const double *a, const double *b)
{
	return a[0]*b[0] + 2*a[1]*b[1] + 2*a[2]*b[2] + 2*a[3]*b[3] + a[4]*b[4] + a[5]*b[5];
}
__device__ __forceinline__ double dmax_atomic_value(unsigned long long bits) { return __longlong_as_double((long long)bits); }

static inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n+t-1)/t); }

// ---------------------------------------------------------------------------
// periodic boundaries, System.cpp:2478-2548
// ---------------------------------------------------------------------------
__device__ int periodize(const DevParams &P, const double *sd, v3 &p)
{
	int z_shift = 0;
	if (p.z >= P.lz) {
		p.z -= P.lz;
		p = vsub(p, V(sd[0], sd[1], sd[2]));
		z_shift = -1;
	} else if (p.z < 0) {
		p.z += P.lz;
		p = vadd(p, V(sd[0], sd[1], sd[2]));
		z_shift = 1;
	}
	while (p.x >= P.lx) p.x -= P.lx;
	while (p.x < 0) p.x += P.lx;
	if (!P.twodim) {
		if (p.y >= P.ly) p.y -= P.ly;
		else if (p.y < 0) p.y += P.ly;
	}
	return z_shift;
}

__device__ int periodize_diff(const DevParams &P, const double *sd, v3 &d)
{
	int zshift = 0;
	if (d.z > P.lz_half) {
		d.z -= P.lz;
		d = vsub(d, V(sd[0], sd[1], sd[2]));
		zshift = -1;
	} else if (d.z < -P.lz_half) {
		d.z += P.lz;
		d = vadd(d, V(sd[0], sd[1], sd[2]));
		zshift = 1;
	}
	while (d.x > P.lx_half) d.x -= P.lx;
	while (d.x < -P.lx_half) d.x += P.lx;
	if (!P.twodim) {
		if (d.y > P.ly_half) d.y -= P.ly;
		else if (d.y < -P.ly_half) d.y += P.ly;
	}
	return zshift;
}

// System::calcLubricationRange (System.cpp:2665-2674) and the interaction
// range (System.cpp:2660-2663, 405-410)
__device__ __forceinline__ double lub_range(const DevParams &P, double ri, double rj)
{
	double rad_ratio = ri/rj;
	if (rad_ratio < 2 && rad_ratio > 0.5) return (2+P.lub_max_gap)*0.5*(ri+rj);
	double minradius = ri < rj ? ri : rj;
	return ri+rj+P.lub_max_gap*minradius;
}
__device__ __forceinline__ double inter_range(const DevParams &P, double ri, double rj)
{
	if (P.interaction_range < 0) return lub_range(P, ri, rj);
	return P.interaction_range*0.5*(ri+rj);
}

// ---------------------------------------------------------------------------
// pair constants (LubricationFunctions.h:12-90, Lubrication.cpp:165-294,
// ContactDashpot.cpp:107-183)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double g1_XA(double l) { double p = l+1; return 2*l*l/(p*p*p); }
__device__ __forceinline__ double g2_YA(double l) { double p = l+1; return (4./15)*l*(2+l+2*l*l)/(p*p*p); }
__device__ __forceinline__ double g2_YB(double l) { double p = l+1; return -(1./5)*l*(4+l)/(p*p); }
__device__ __forceinline__ double g2_YC(double l) { return (2./5)*l/(l+1); }
__device__ __forceinline__ double g4_YC(double l) { double p = l+1; return (4./5)*l*l/(p*p*p*p); }
__device__ __forceinline__ double g1_XG(double l) { double p = l+1; return 3*l*l/(p*p*p); }
__device__ __forceinline__ double g2_YG(double l) { double p = l+1; return (1./10)*l*(4-l+7*l*l)/(p*p*p); }
__device__ __forceinline__ double g2_YH(double l) { double p = l+1; return (1./10)*l*(2-l)/(p*p); }
__device__ __forceinline__ double g5_YH(double l) { double p = l+1; return (1./20)*l*l*(1+7*l)/(p*p); }
__device__ __forceinline__ double g1_XM(double l) { double p = l+1; return (6./5)*l*l/(p*p*p); }
__device__ __forceinline__ double g4_XM(double l) { double p = l+1; return (6./5)*l*l*l/(p*p*p); }
__device__ __forceinline__ double g2_YM(double l) { double p = l+1; return (6./25)*l*(1-l+4*l*l)/(p*p*p); }
__device__ __forceinline__ double g5_YM(double l) { double p = l+1; return (3./50)*l*l*(7-10*l+7*l*l)/(p*p*p); }

enum { CXA = 0, CYA = 4, CYB = 8, CYC = 12, CXG = 16, CYG = 20, CYH = 24, CXM = 28, CYM = 32 };
enum { DXA = 0, DYA = 4, DYB = 8, DYC = 12 };

__global__ void k_pair_constants(DevParams P, int np, const DPair *__restrict__ pairs,
                                 const double *__restrict__ radius, DPairConst *__restrict__ pc)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= np) return;
	int i = pairs[t].p0, j = pairs[t].p1;
	DPairConst c;
	double a0 = radius[i], a1 = radius[j];
	c.a0 = a0; c.a1 = a1;
	double ro = a0+a1;
	c.ro = ro;
	c.range = inter_range(P, a0, a1);
	c.lub_range = lub_range(P, a0, a1);
	double ro_12 = (a0+a1)/2;
	c.kn_s = ro_12*ro_12*P.kn;
	c.kt_s = P.friction ? ro_12*P.kt : 0;
	c.kr_s = (P.friction && P.rolling) ? ro_12*P.kr : 0;
	c.rep_geo = a0*a1/(a0+a1);
	// Lubrication::calcLubConstants
	double r12 = ro/2;
	double lambda = a1/a0, invlambda = 1/lambda;
	double lambda_square = lambda*lambda, lambda_cubic = lambda*lambda*lambda;
	double lambda_p_1 = 1+lambda, lambda_p_1_square = lambda_p_1*lambda_p_1;
	double lambda_p_1_cubic = lambda_p_1_square*lambda_p_1;
	double a0a0_23 = a0*a0*(2.0/3), a1a1_23 = a1*a1*(2.0/3), roro_16 = ro*ro*(1.0/6);
	double a0a0a0 = a0*a0*a0, a1a1a1 = a1*a1*a1, rororo = ro*ro*ro;
	double a0a0a0_43 = a0a0a0*(4.0/3), a1a1a1_43 = a1a1a1*(4.0/3), rororo_16 = rororo*(1.0/6);
	double a0a0a0_109 = a0a0a0*(10.0/9), a1a1a1_109 = a1a1a1*(10.0/9), rororo_536 = rororo*(5.0/36);
	double *L = c.lc;
	double g = g1_XA(lambda);
	L[CXA+0] = a0*g; L[CXA+1] = r12*(-2/lambda_p_1)*g; L[CXA+2] = L[CXA+1]; L[CXA+3] = a1*g1_XA(invlambda);
	g = g2_YA(lambda);
	L[CYA+0] = a0*g; L[CYA+1] = r12*(-2/lambda_p_1)*g; L[CYA+2] = L[CYA+1]; L[CYA+3] = a1*g2_YA(invlambda);
	g = g2_YB(lambda);
	L[CYB+0] = a0a0_23*g; L[CYB+1] = roro_16*(-4/lambda_p_1_square)*g;
	L[CYB+2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YB(invlambda); L[CYB+3] = -a1a1_23*g2_YB(invlambda);
	L[CYC+0] = a0a0a0_43*g2_YC(lambda); L[CYC+1] = rororo_16*g4_YC(lambda); L[CYC+2] = L[CYC+1];
	L[CYC+3] = a1a1a1_43*g2_YC(invlambda);
	g = g1_XG(lambda);
	L[CXG+0] = a0a0_23*g; L[CXG+1] = roro_16*(-4/lambda_p_1_square)*g;
	L[CXG+2] = roro_16*(4*lambda_square/lambda_p_1_square)*g1_XG(invlambda); L[CXG+3] = -a1a1_23*g1_XG(invlambda);
	g = g2_YG(lambda);
	L[CYG+0] = a0a0_23*g; L[CYG+1] = roro_16*(-4/lambda_p_1_square)*g;
	L[CYG+2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YG(invlambda); L[CYG+3] = -a1a1_23*g2_YG(invlambda);
	L[CYH+0] = a0a0a0_43*g2_YH(lambda); L[CYH+1] = rororo_16*(8/lambda_p_1_cubic)*g5_YH(lambda);
	L[CYH+2] = rororo_16*(8*lambda_cubic/lambda_p_1_cubic)*g5_YH(invlambda); L[CYH+3] = a1a1a1_43*g2_YH(invlambda);
	L[CXM+0] = a0a0a0_109*g1_XM(lambda); L[CXM+1] = rororo_536*(8/lambda_p_1_cubic)*g4_XM(lambda);
	L[CXM+2] = L[CXM+1]; L[CXM+3] = a1a1a1_109*g1_XM(invlambda);
	L[CYM+0] = a0a0a0_109*g2_YM(lambda); L[CYM+1] = rororo_536*(8/lambda_p_1_cubic)*g5_YM(lambda);
	L[CYM+2] = L[CYM+1]; L[CYM+3] = a1a1a1_109*g2_YM(invlambda);
	// ContactDashpot::calcDashpotResistances
	double *D = c.dc;
	double nc = P.dp_normal_coeff, tc = P.dp_tan_coeff;
	D[DXA+0] = a0*g1_XA(lambda);
	D[DXA+1] = ro_12*(-2/lambda_p_1)*g1_XA(lambda);
	D[DXA+2] = ro_12*D[DXA+1];
	D[DXA+3] = a1*g1_XA(invlambda);
	for (int k = 0; k < 4; k++) D[DXA+k] *= nc;
	for (int k = 0; k < 12; k++) D[DYA+k] = 0;
	if (tc != 0) {
		D[DYA+0] = a0*g2_YA(lambda);
		D[DYA+1] = ro_12*(-2/lambda_p_1)*g2_YA(lambda);
		D[DYA+2] = ro_12*D[DYA+1];
		D[DYA+3] = a1*g2_YA(invlambda);
		for (int k = 0; k < 4; k++) D[DYA+k] *= tc;
		D[DYB+0] = a0a0_23*g2_YB(lambda);
		D[DYB+1] = roro_16*(-4/lambda_p_1_square)*g2_YB(lambda);
		D[DYB+2] = roro_16*(4*lambda_square/lambda_p_1_square)*g2_YB(invlambda);
		D[DYB+3] = -a1a1_23*g2_YB(invlambda);
		for (int k = 0; k < 4; k++) D[DYB+k] *= tc;
		D[DYC+0] = a0a0a0_43*g2_YC(lambda);
		D[DYC+1] = rororo_16*g4_YC(lambda);
		D[DYC+2] = rororo_16*D[DYC+1];
		D[DYC+3] = a1a1a1_43*g2_YC(invlambda);
		for (int k = 0; k < 4; k++) D[DYC+k] *= tc;
	}
	pc[t] = c;
}

// ---------------------------------------------------------------------------
// cell lists with Lees-Edwards shifted neighbour rows (BoxSet.cpp)
// ---------------------------------------------------------------------------
struct CellView {
	int ncx, ncy, ncz, brute, n;
	double csx, csy, csz;
	const int *start, *count, *list;
};

__device__ __forceinline__ int wrapc(int c, int nc) { c %= nc; return c < 0 ? c+nc : c; }
__device__ __forceinline__ int cell_coord(double x, double L, double cs, int nc)
{
	double w = x-floor(x/L)*L;
	int c = (int)(w/cs);
	return c < 0 ? 0 : (c >= nc ? nc-1 : c);
}

template <typename F>
__device__ void for_neighbours(const CellView &C, const DevParams &P, const double *sd, int i, v3 pi, F f)
{
	if (C.brute) {
		for (int j = i+1; j < C.n; j++) f(j);
		return;
	}
	int cz = cell_coord(pi.z, P.lz, C.csz, C.ncz);
	for (int dz = -1; dz <= 1; dz++) {
		int zc = cz+dz;
		double sx = 0, sy = 0;
		if (zc < 0) { zc += C.ncz; sx = sd[0]; sy = sd[1]; }
		else if (zc >= C.ncz) { zc -= C.ncz; sx = -sd[0]; sy = -sd[1]; }
		int xc = cell_coord(pi.x+sx, P.lx, C.csx, C.ncx);
		int yc = P.twodim ? 0 : cell_coord(pi.y+sy, P.ly, C.csy, C.ncy);
		int ylo = P.twodim ? 0 : -1, yhi = P.twodim ? 0 : 1;
		for (int dy = ylo; dy <= yhi; dy++) {
			int yy = P.twodim ? 0 : wrapc(yc+dy, C.ncy);
			for (int dx = -1; dx <= 1; dx++) {
				int xx = wrapc(xc+dx, C.ncx);
				int cell = (zc*C.ncy+yy)*C.ncx+xx;
				int s = C.start[cell], e = s+C.count[cell];
				for (int k = s; k < e; k++) {
					int j = C.list[k];
					if (j > i) f(j);
				}
			}
		}
	}
}

__global__ void k_cell_assign(DevParams P, CellView C, const double *__restrict__ pos, int *__restrict__ cell_of,
                              int *__restrict__ count)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= C.n) return;
	int cx = cell_coord(pos[3*i], P.lx, C.csx, C.ncx);
	int cy = P.twodim ? 0 : cell_coord(pos[3*i+1], P.ly, C.csy, C.ncy);
	int cz = cell_coord(pos[3*i+2], P.lz, C.csz, C.ncz);
	int c = (cz*C.ncy+cy)*C.ncx+cx;
	cell_of[i] = c;
	atomicAdd(&count[c], 1);
}

// exclusive scan of n ints by one CTA of 1024 threads (cell counts, candidate
// counts: n up to a few 10^5): tiles of 4096 entries, four consecutive
// entries per thread (one vector load), warp-shuffle scans of the thread and
// warp sums, the tile total carried to the next tile; out[n] = total.
constexpr unsigned PFULL = 0xffffffffu;
__global__ void __launch_bounds__(1024) k_scan(int n, const int *__restrict__ in, int *__restrict__ out, int *total)
{
	__shared__ int wsum[32];
	const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
	int carry = 0;
	for (int base = 0; base < n; base += 4*1024) {
		const int i0 = base+4*t;
		int v[4];
		if (i0+3 < n) {
			int4 q = *reinterpret_cast<const int4 *>(in+i0);   // base and i0 are multiples of 4
			v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
		} else {
#pragma unroll
			for (int k = 0; k < 4; k++) v[k] = i0+k < n ? in[i0+k] : 0;
		}
		const int sum = v[0]+v[1]+v[2]+v[3];
		int x = sum;   // inclusive scan over the warp
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			int y = __shfl_up_sync(PFULL, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) wsum[wid] = x;
		__syncthreads();
		if (wid == 0) {
			int w = wsum[lane];
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				int y = __shfl_up_sync(PFULL, w, o);
				if (lane >= o) w += y;
			}
			wsum[lane] = w;
		}
		__syncthreads();
		int excl = carry+(wid ? wsum[wid-1] : 0)+x-sum;
#pragma unroll
		for (int k = 0; k < 4; k++) {
			if (i0+k < n) out[i0+k] = excl;
			excl += v[k];
		}
		carry += wsum[31];
		__syncthreads();   // wsum is rewritten by the next tile
	}
	if (t == 0) {
		out[n] = carry;
		if (total) *total = carry;
	}
}

// ascending sort of 32 values, one per lane (bitonic network over shuffles)
__device__ __forceinline__ int warp_sort32(int v, int lane)
{
#pragma unroll
	for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
		for (int j = k >> 1; j > 0; j >>= 1) {
			int o = __shfl_xor_sync(PFULL, v, j);
			bool up = (lane & k) == 0, lower = (lane & j) == 0;
			v = (lower == up) ? min(v, o) : max(v, o);
		}
	return v;
}

__global__ void k_cell_fill(int n, const int *__restrict__ cell_of, const int *__restrict__ start,
                            int *__restrict__ fill, int *__restrict__ list)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	int c = cell_of[i];
	int k = atomicAdd(&fill[c], 1);
	list[start[c]+k] = i;
}

// A particle's cell-ordered FP64 record: position and radius (32 bytes)
struct __align__(32) PRec { double x, y, z, w; };

// Each cell's particle list sorted (deterministic neighbour order), one warp
// per cell: up to 32 members sorted in registers (bitonic), larger cells by
// lane 0 in place.  The warp then writes the cell-ordered records (x, y, z,
// radius) of its members, in FP64 and rounded to FP32, so the neighbour
// searches read a cell's particles as contiguous records (one 16-byte vector
// load each for the FP32 prefilter, two for the FP64 test).
__global__ void k_cell_sort(int ncell, const int *__restrict__ start, const int *__restrict__ count,
                            int *__restrict__ list, const double *__restrict__ pos, const double *__restrict__ radius,
                            double *__restrict__ rec, float *__restrict__ rec32)
{
	const int c = (blockIdx.x*blockDim.x+threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (c >= ncell) return;   // whole warps
	const int s = start[c], m = count[c];
	if (m <= 32) {
		int v = lane < m ? list[s+lane] : 0x7fffffff;
		v = warp_sort32(v, lane);
		if (lane < m) list[s+lane] = v;
	} else {
		if (lane == 0)
			for (int a = s+1; a < s+m; a++) {
				int x = list[a], b = a-1;
				while (b >= s && list[b] > x) { list[b+1] = list[b]; b--; }
				list[b+1] = x;
			}
		__syncwarp();
	}
	for (int k = s+lane; k < s+m; k += 32) {
		int j = list[k];
		const PRec r = {pos[3*j], pos[3*j+1], pos[3*j+2], radius[j]};
		reinterpret_cast<PRec *>(rec)[k] = r;
		reinterpret_cast<float4 *>(rec32)[k] = make_float4((float)r.x, (float)r.y, (float)r.z, (float)r.w);
	}
}

// FP32 prefilter of the neighbour tests.  The decision "|d|^2 < range^2"
// must be the FP64 one bit for bit, and the FP64 arithmetic (periodic wrap,
// range, squares) runs on GB300's narrow FP64 pipe.  So each test is first
// made from FP32-rounded records: every component of d is then within 8
// roundings of the box size of its FP64 value (positions, the wrap and the
// Lees-Edwards shift), so |d|^2 is within 2 sqrt(3) r e + O(e^2) of it near
// |d| = r, and the FP32 range within a few roundings of r; prefilter_tol
// bounds both with a factor 4 to spare.  Outside [r^2 - tol, r^2 + tol] the
// FP32 answer is the FP64 one; inside, the exact FP64 test decides.  (A
// different wrap decision in FP32 only happens at |d_x| ~ L/2, far beyond
// any range: out either way.)
struct Box32 { float lx, ly, lz, lxh, lyh, lzh, sx, sy, sz, lmax; int twodim; };
__device__ __forceinline__ Box32 box32(const DevParams &P, const double *sd)
{
	Box32 B;
	B.lx = (float)P.lx; B.ly = (float)P.ly; B.lz = (float)P.lz;
	B.lxh = (float)P.lx_half; B.lyh = (float)P.ly_half; B.lzh = (float)P.lz_half;
	B.sx = (float)sd[0]; B.sy = (float)sd[1]; B.sz = (float)sd[2];
	B.lmax = fmaxf(fmaxf(B.lx, fmaxf(B.ly, B.lz)), fmaxf(fabsf(B.sx), fmaxf(fabsf(B.sy), fabsf(B.sz))));
	B.twodim = P.twodim;
	return B;
}
// periodize_diff in FP32, then |d|^2
__device__ __forceinline__ float dist2_32(const Box32 &B, float dx, float dy, float dz)
{
	if (dz > B.lzh) { dz -= B.lz; dx -= B.sx; dy -= B.sy; dz -= B.sz; }
	else if (dz < -B.lzh) { dz += B.lz; dx += B.sx; dy += B.sy; dz += B.sz; }
	while (dx > B.lxh) dx -= B.lx;
	while (dx < -B.lxh) dx += B.lx;
	if (!B.twodim) {
		if (dy > B.lyh) dy -= B.ly;
		else if (dy < -B.lyh) dy += B.ly;
	}
	return dx*dx+dy*dy+dz*dz;
}
// FP32 bounds [lo, hi] of inter_range(ri, rj) + extra: both branches of the
// radius-ratio test when the ratio is within 1e-5 of a branch point
__device__ __forceinline__ void range32(const DevParams &P, float ri, float rj, float extra, float &lo, float &hi)
{
	if (P.interaction_range >= 0) {
		lo = hi = (float)P.interaction_range*0.5f*(ri+rj)+extra;
		return;
	}
	const float g = (float)P.lub_max_gap;
	const float a = (2.0f+g)*0.5f*(ri+rj), b = ri+rj+g*fminf(ri, rj);
	const float q = ri/rj;
	const bool ina = q < 2.0f && q > 0.5f;
	const bool near = fabsf(q-2.0f) < 2e-5f || fabsf(q-0.5f) < 1e-5f;
	const float r = ina ? a : b;
	lo = (near ? fminf(a, b) : r)+extra;
	hi = (near ? fmaxf(a, b) : r)+extra;
}
// -1: out, 1: in, 0: undecided (the FP64 test decides)
__device__ __forceinline__ int prefilter(const Box32 &B, float d2, float lo, float hi)
{
	const float tol = 1.6e-5f*B.lmax*hi+1e-6f*hi*hi;
	if (d2 < lo*lo-tol) return 1;
	if (d2 > hi*hi+tol) return -1;
	return 0;
}

// Candidate pairs within the superset range (range + skin (a_i+a_j)/2), one
// warp per particle i: the lanes take the members of each neighbour cell (the
// cells for_neighbours visits, in its order) as contiguous cell-ordered
// records, a ballot compacts the hits in visit order, and the row is sorted
// in registers (bitonic; rows longer than 32 by lane 0 in place).  Pass 1
// (ptr null) counts, pass 2 fills.  Systems too small for cells (brute) take
// every j > i from the particle arrays.
__global__ void k_candidates(DevParams P, CellView C, const DevClock *__restrict__ clk,
                             const double *__restrict__ pos, const double *__restrict__ radius,
                             const double *__restrict__ rec, const float *__restrict__ rec32,
                             int *__restrict__ count, const int *__restrict__ ptr, int *__restrict__ cand)
{
	const int i = (int)(((int64_t)blockIdx.x*blockDim.x+threadIdx.x) >> 5), lane = threadIdx.x & 31;
	if (i >= C.n) return;   // whole warps
	const double *sd = clk->shear_disp;
	const v3 pi = ld3(pos+3*i);
	const double ri = radius[i];
	const Box32 B = box32(P, sd);
	const float pxf = (float)pi.x, pyf = (float)pi.y, pzf = (float)pi.z, rif = (float)ri, skf = (float)P.skin;
	const int base = ptr ? ptr[i] : 0;
	int c = 0;   // hits so far (the same in every lane)
	auto scan = [&](int s, int e, bool brute) {
		for (int k0 = s; k0 < e; k0 += 32) {
			const int k = k0+lane;
			bool hit = false;
			int j = -1;
			if (k < e) {
				v3 pj;
				double rj;
				if (brute) {
					j = k;
					pj = ld3(pos+3*j);
					rj = radius[j];
				} else {
					j = C.list[k];
					if (j > i) {
						// FP32 prefilter; the FP64 record only when it cannot decide
						const float4 f = reinterpret_cast<const float4 *>(rec32)[k];
						float lo, hi;
						range32(P, rif, f.w, skf*0.5f*(rif+f.w), lo, hi);
						const int v = prefilter(B, dist2_32(B, f.x-pxf, f.y-pyf, f.z-pzf), lo, hi);
						if (v != 0) {
							hit = v > 0;
							j = v > 0 ? j : -1;
						} else {
							const PRec r = reinterpret_cast<const PRec *>(rec)[k];
							pj = V(r.x, r.y, r.z);
							rj = r.w;
						}
					}
				}
				if (j > i && (brute || !hit)) {
					v3 d = vsub(pj, pi);
					periodize_diff(P, sd, d);
					double rs = inter_range(P, ri, rj)+P.skin*0.5*(ri+rj);
					hit = vsq(d) < rs*rs;
				}
			}
			const unsigned b = __ballot_sync(PFULL, hit);
			if (ptr && hit) cand[base+c+__popc(b & ((1u << lane)-1))] = j;
			c += __popc(b);
		}
	};
	if (C.brute) {
		scan(i+1, C.n, true);
	} else {
		const int cz = cell_coord(pi.z, P.lz, C.csz, C.ncz);
		for (int dz = -1; dz <= 1; dz++) {
			int zc = cz+dz;
			double sx = 0, sy = 0;
			if (zc < 0) { zc += C.ncz; sx = sd[0]; sy = sd[1]; }
			else if (zc >= C.ncz) { zc -= C.ncz; sx = -sd[0]; sy = -sd[1]; }
			const int xc = cell_coord(pi.x+sx, P.lx, C.csx, C.ncx);
			const int yc = P.twodim ? 0 : cell_coord(pi.y+sy, P.ly, C.csy, C.ncy);
			const int ylo = P.twodim ? 0 : -1, yhi = P.twodim ? 0 : 1;
			for (int dy = ylo; dy <= yhi; dy++) {
				const int yy = P.twodim ? 0 : wrapc(yc+dy, C.ncy);
				for (int dx = -1; dx <= 1; dx++) {
					const int cell = (zc*C.ncy+yy)*C.ncx+wrapc(xc+dx, C.ncx);
					const int s0 = C.start[cell];
					scan(s0, s0+C.count[cell], false);
				}
			}
		}
	}
	if (!ptr) {
		if (lane == 0) count[i] = c;
		return;
	}
	__syncwarp();   // the row's stores are visible to the warp
	if (c <= 32) {
		int v = lane < c ? cand[base+lane] : 0x7fffffff;
		v = warp_sort32(v, lane);
		if (lane < c) cand[base+lane] = v;
	} else if (lane == 0) {
		for (int a = base+1; a < base+c; a++) {
			int x = cand[a], q = a-1;
			while (q >= base && cand[q] > x) { cand[q+1] = cand[q]; q--; }
			cand[q+1] = x;
		}
	}
}

// System::checkNewInteraction's test (System.cpp:1328-1373): every pair
// (i, j > i) within the interaction range must be in the superset.  One CTA
// per home cell: the records of the cells its particles search are staged in
// shared memory (in passes of CHK_CAP), and one warp per home particle i
// tests them (FP32 prefilter, FP64 where it cannot decide), its superset row
// (the sorted candidate list) held in lanes and matched by shuffles.  The staged cells are a superset of those
// for_neighbours visits from any particle of the home cell: a Lees-Edwards
// shifted row takes five x (and, with a y shift, five y) cells around the
// shifted cell of the home cell's centre, since a particle's shifted cell is
// at most one away from it.  Extra or repeated cells only repeat tests.
constexpr int CHK_CAP = 640;   // staged records per pass
constexpr int CHK_SLOTS = 75;  // 3 rows x 5 x 5 cells at most
__global__ void __launch_bounds__(128) k_check_cells(DevParams P, CellView C, DevClock *__restrict__ clk,
                                                     const double *__restrict__ rec, const float *__restrict__ rec32,
                                                     const int *__restrict__ row_ptr, const int *__restrict__ cand)
{
	__shared__ float4 srec[CHK_CAP];
	__shared__ int sidx[CHK_CAP], skey[CHK_CAP];
	__shared__ int cs[CHK_SLOTS], cpre[CHK_SLOTS+1];
	const int h = blockIdx.x;
	const int hs = C.start[h], hn = C.count[h];
	if (hn == 0) return;   // the same in every thread
	const int hx = h%C.ncx, hy = (h/C.ncx)%C.ncy, hz = h/(C.ncx*C.ncy);
	const double *sd = clk->shear_disp;
	const Box32 B = box32(P, sd);
	const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
	if (t < CHK_SLOTS) {
		// slot (row dz, y offset, x offset) -> cell and member count (0 if unused)
		const int dz = t/25-1, yq = (t/5)%5, xq = t%5;
		int zc = hz+dz;
		double sx = 0, sy = 0;
		bool sh = false;
		if (zc < 0) { zc += C.ncz; sx = sd[0]; sy = sd[1]; sh = true; }
		else if (zc >= C.ncz) { zc -= C.ncz; sx = -sd[0]; sy = -sd[1]; sh = true; }
		int xa = hx-1, xn = 3;
		if (sh && sx != 0) { xa = cell_coord((hx+0.5)*C.csx+sx, P.lx, C.csx, C.ncx)-2; xn = 5; }
		int ya = 0, yn = 1;
		if (!P.twodim) {
			ya = hy-1; yn = 3;
			if (sh && sy != 0) { ya = cell_coord((hy+0.5)*C.csy+sy, P.ly, C.csy, C.ncy)-2; yn = 5; }
		}
		int cnt = 0, st0 = 0;
		if (xq < xn && yq < yn) {
			const int yy = P.twodim ? 0 : wrapc(ya+yq, C.ncy);
			const int cell = (zc*C.ncy+yy)*C.ncx+wrapc(xa+xq, C.ncx);
			st0 = C.start[cell];
			cnt = C.count[cell];
		}
		cs[t] = st0;
		cpre[t+1] = cnt;
	}
	__syncthreads();
	if (warp == 0) {
		// inclusive prefix of the slot counts: lane l sums slots 3l .. 3l + 2
		int v[3], sum = 0;
#pragma unroll
		for (int u = 0; u < 3; u++) { int q = 3*lane+u; v[u] = q < CHK_SLOTS ? cpre[q+1] : 0; sum += v[u]; }
		int x = sum;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			int y = __shfl_up_sync(PFULL, x, o);
			if (lane >= o) x += y;
		}
		int run = x-sum;
#pragma unroll
		for (int u = 0; u < 3; u++) {
			int q = 3*lane+u;
			run += v[u];
			if (q < CHK_SLOTS) cpre[q+1] = run;
		}
		if (lane == 0) cpre[0] = 0;
	}
	__syncthreads();
	const int R = cpre[CHK_SLOTS];
	for (int f0 = 0; f0 < R; f0 += CHK_CAP) {
		const int fn = min(CHK_CAP, R-f0);
		for (int f = t; f < fn; f += blockDim.x) {
			const int g = f0+f;
			int lo = 0, hi = CHK_SLOTS-1;   // last slot with cpre <= g
			while (lo < hi) {
				int mid = (lo+hi+1) >> 1;
				if (cpre[mid] <= g) lo = mid; else hi = mid-1;
			}
			const int k = cs[lo]+g-cpre[lo];
			srec[f] = reinterpret_cast<const float4 *>(rec32)[k];
			sidx[f] = C.list[k];
			skey[f] = k;
		}
		__syncthreads();
		for (int hp = warp; hp < hn; hp += blockDim.x >> 5) {
			const int i = C.list[hs+hp];
			const float4 p4 = reinterpret_cast<const float4 *>(rec32)[hs+hp];
			const int lo = row_ptr[i], len = row_ptr[i+1]-lo;
			const int rv0 = lane < len ? cand[lo+lane] : -2;
			for (int fb = 0; fb < fn; fb += 32) {
				const int f = fb+lane;
				int need = -1;
				if (f < fn) {
					const int j = sidx[f];
					if (j > i) {
						// FP32 prefilter; the FP64 records only when it cannot decide
						const float4 q = srec[f];
						float rlo, rhi;
						range32(P, p4.w, q.w, 0.0f, rlo, rhi);
						const int v = prefilter(B, dist2_32(B, q.x-p4.x, q.y-p4.y, q.z-p4.z), rlo, rhi);
						if (v > 0) {
							need = j;
						} else if (v == 0) {
							const PRec a = reinterpret_cast<const PRec *>(rec)[hs+hp];
							const PRec r = reinterpret_cast<const PRec *>(rec)[skey[f]];
							v3 d = vsub(V(r.x, r.y, r.z), V(a.x, a.y, a.z));
							periodize_diff(P, sd, d);
							double range = inter_range(P, a.w, r.w);
							if (vsq(d) < range*range) need = j;
						}
					}
				}
				if (!__any_sync(PFULL, need >= 0)) continue;
				bool found = false;
				for (int e0 = 0; e0 < len; e0 += 32) {
					const int rv = e0 == 0 ? rv0 : (e0+lane < len ? cand[lo+e0+lane] : -2);
					const int m = min(32, len-e0);
					for (int e = 0; e < m; e++) found |= __shfl_sync(PFULL, rv, e) == need;
				}
				if (need >= 0 && !found) atomicOr(&clk->stale, 1);
			}
		}
		__syncthreads();   // srec is restaged by the next pass
	}
}

// every pair within the interaction range must be in the superset
// (System::checkNewInteraction's test, System.cpp:1328-1373)
// one thread per (particle i, neighbour cell): every pair (i, j > i) within
// interaction range must be in the superset row of i
__global__ void k_check_superset(DevParams P, CellView C, DevClock *__restrict__ clk,
                                 const double *__restrict__ pos, const double *__restrict__ radius,
                                 const int *__restrict__ row_ptr, const DPair *__restrict__ pairs)
{
	const int ncell = P.twodim ? 9 : 27;
	int64_t t = (int64_t)blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= (int64_t)C.n*ncell) return;
	int i = (int)(t/ncell), q = (int)(t%ncell);
	if (C.brute && q != 0) return;
	const double *sd = clk->shear_disp;
	v3 pi = ld3(pos+3*i);
	double ri = radius[i];
	int lo0 = row_ptr[i], hi0 = row_ptr[i+1];
	auto check = [&](int j) {
		v3 d = vsub(ld3(pos+3*j), pi);
		periodize_diff(P, sd, d);
		double range = inter_range(P, ri, radius[j]);
		if (vsq(d) < range*range) {
			int lo = lo0, hi = hi0-1;
			while (lo <= hi) {
				int m = (lo+hi) >> 1;
				int pj = pairs[m].p1;
				if (pj == j) return;
				if (pj < j) lo = m+1; else hi = m-1;
			}
			atomicOr(&clk->stale, 1);
		}
	};
	if (C.brute) {
		for (int j = i+1; j < C.n; j++) check(j);
		return;
	}
	// the neighbour cell of index q, located as for_neighbours does
	int dz = q/(P.twodim ? 3 : 9)-1;
	int dy = P.twodim ? 0 : (q/3)%3-1;
	int dx = q%3-1;
	int zc = cell_coord(pi.z, P.lz, C.csz, C.ncz)+dz;
	double sx = 0, sy = 0;
	if (zc < 0) { zc += C.ncz; sx = sd[0]; sy = sd[1]; }
	else if (zc >= C.ncz) { zc -= C.ncz; sx = -sd[0]; sy = -sd[1]; }
	int xc = cell_coord(pi.x+sx, P.lx, C.csx, C.ncx);
	int yy = P.twodim ? 0 : wrapc(cell_coord(pi.y+sy, P.ly, C.csy, C.ncy)+dy, C.ncy);
	int xx = wrapc(xc+dx, C.ncx);
	int cell = (zc*C.ncy+yy)*C.ncx+xx;
	int s0 = C.start[cell], e0 = s0+C.count[cell];
	for (int k = s0; k < e0; k++) {
		int j = C.list[k];
		if (j > i) check(j);
	}
}

// ---------------------------------------------------------------------------
// Interaction life cycle (Interaction.cpp, Contact.cpp, Lubrication.cpp,
// RepulsiveForce.cpp)
// ---------------------------------------------------------------------------
__device__ void pair_geometry(const DevParams &P, const double *sd, const double *pos, DPair &q, const DPairConst &c)
{
	v3 rv = vsub(ld3(pos+3*q.p1), ld3(pos+3*q.p0));
	q.zoff = periodize_diff(P, sd, rv);
	double r = sqrt(vsq(rv));
	q.r = r;
	st3(q.rvec, rv);
	q.nvec[0] = rv.x/r; q.nvec[1] = rv.y/r; q.nvec[2] = rv.z/r;
	q.gap = 2*r/c.ro-2;
}

__device__ void contact_activate(const DevParams &P, DPair &q)
{
	q.flags |= PF_CONTACT | PF_DASHPOT;
	q.fsn_norm = 0;
	q.normal_load = 0;
	for (int k = 0; k < 3; k++) q.fs_total[k] = 0;
	if (P.friction) {
		q.state = (P.friction_model == 2 || P.friction_model == 3) ? 1 : 2;
		for (int k = 0; k < 3; k++) { q.disp_tan[k] = 0; q.prev_disp_tan[k] = 0; }
		for (int k = 0; k < 3; k++) { q.disp_roll[k] = 0; q.prev_disp_roll[k] = 0; q.f_roll[k] = 0; }
	} else {
		q.state = 1;
	}
}

__device__ void contact_deactivate(const DevParams &P, DPair &q)
{
	q.state = 0;
	q.flags &= ~(PF_CONTACT | PF_DASHPOT);
	q.fsn_norm = 0;
	for (int k = 0; k < 3; k++) q.fs_total[k] = 0;
	if (P.friction)
		for (int k = 0; k < 3; k++) { q.disp_tan[k] = 0; q.disp_roll[k] = 0; q.fs_tan[k] = 0; }
}

__device__ void lub_update(const DevParams &P, DPair &q, const DPairConst &c)
{
	if (!P.lub_on) return;
	bool in_range = q.r < c.lub_range && q.r > c.ro;
	bool act = q.flags & PF_LUB;
	if (!act && in_range) { q.flags |= PF_LUB; act = true; }
	if (act && !in_range) { q.flags &= ~PF_LUB; act = false; }
	if (act && q.gap > 0) {
		double coeff = 1/(q.gap+P.lub_reduce);
		q.lub_coeff = coeff;
		q.log_lub_coeff = coeff > 1. ? log(coeff) : 0.;
	}
}

__device__ void set_tan_norm(DPair &q, const DPairConst &c, double cur, double target)
{
	double s = target/cur;
	for (int k = 0; k < 3; k++) q.disp_tan[k] = s*q.disp_tan[k];
	for (int k = 0; k < 3; k++) q.fs_tan[k] = c.kt_s*q.disp_tan[k];
}

__device__ void friction_law(const DevParams &P, DPair &q, const DPairConst &c)
{
	int fm = P.friction_model;
	v3 ft = ld3(q.fs_tan);
	if (fm == 1) {
		double sup;
		double sq = vsq(ft);
		q.normal_load = q.fsn_norm;
		sup = (q.state == 2) ? P.mu_s*q.normal_load : P.mu_d*q.normal_load;
		if (sq > sup*sup) { q.state = 3; sup = P.mu_d*q.normal_load; }
		else q.state = 2;
		if (q.state == 3) set_tan_norm(q, c, sqrt(sq), sup);
		if (P.rolling) {
			// Contact::setRollingForceNorm (Contact.cpp:283-305)
			double sup_r = P.mu_r*q.normal_load;
			double sq_r = vsq(ld3(q.f_roll));
			if (sq_r > sup_r*sup_r) {
				double sc = sup_r/sqrt(sq_r);
				for (int k = 0; k < 3; k++) q.disp_roll[k] = sc*q.disp_roll[k];
				for (int k = 0; k < 3; k++) q.f_roll[k] = c.kr_s*q.disp_roll[k];
			}
		}
	} else if (fm == 2) {
		double sup = q.fsn_norm-P.critical_load;
		if (sup < 0) {
			q.state = 1;
			for (int k = 0; k < 3; k++) { q.disp_tan[k] = 0; q.fs_tan[k] = 0; }
		} else {
			sup *= P.mu_s;
			double sq = vsq(ft);
			if (sq > sup*sup) { q.state = 3; set_tan_norm(q, c, sqrt(sq), sup); }
			else q.state = 2;
		}
	} else if (fm == 3) {
		double sup = q.fsn_norm-P.critical_load;
		if (sup < 0) {
			q.state = 1;
			for (int k = 0; k < 3; k++) { q.disp_tan[k] = 0; q.fs_tan[k] = 0; }
		} else q.state = 2;
	} else if (fm == 5) {
		double sq = vsq(ft);
		if (sq > P.ft_max*P.ft_max) { q.state = 3; set_tan_norm(q, c, sqrt(sq), P.ft_max); }
		else q.state = 2;
	} else if (fm == 6) {
		q.normal_load = q.fsn_norm;
		double sup = (q.state == 2) ? P.mu_s*q.normal_load : P.mu_d*q.normal_load;
		if (sup > P.ft_max) sup = P.ft_max;
		double sq = vsq(ft);
		if (sq > sup*sup) { q.state = 3; set_tan_norm(q, c, sqrt(sq), sup); }
		else q.state = 2;
	}
}

__device__ void contact_spring(const DevParams &P, DPair &q, const DPairConst &c)
{
	if (!(q.flags & PF_CONTACT)) return;
	q.fsn_norm = -c.kn_s*q.gap;
	v3 n = ld3(q.nvec);
	v3 fn = vscale(-q.fsn_norm, n);
	if (P.friction) {
		v3 d = ld3(q.disp_tan);
		d = vsub(d, vscale(vdot(d, n), n));
		st3(q.disp_tan, d);
		st3(q.fs_tan, vscale(c.kt_s, d));
		if (P.rolling) st3(q.f_roll, vscale(c.kr_s, ld3(q.disp_roll)));
		friction_law(P, q, c);
	}
	if (q.state <= 1) st3(q.fs_total, fn);
	else st3(q.fs_total, vadd(fn, ld3(q.fs_tan)));
}

__device__ void contact_increment(const DevParams &P, const DevClock &K, const double *vel, const double *ang,
                                  DPair &q, const DPairConst &c, double dt, int in_predictor)
{
	if (!P.friction) return;
	v3 off = vscale((double)q.zoff, ld3(K.vel_diff));
	v3 tdv = vadd(vsub(ld3(vel+3*q.p1), ld3(vel+3*q.p0)), off);
	v3 n = ld3(q.nvec);
	v3 rdv = vneg(vcross(vadd(vscale(c.a0, ld3(ang+3*q.p0)), vscale(c.a1, ld3(ang+3*q.p1))), n));
	v3 rsv = vadd(tdv, rdv);
	rsv = vsub(rsv, vscale(vdot(rsv, n), n));
	q.rsv_sq = vsq(rsv);
	if (in_predictor) for (int k = 0; k < 3; k++) q.prev_disp_tan[k] = q.disp_tan[k];
	st3(q.disp_tan, vadd(ld3(q.prev_disp_tan), vscale(dt, rsv)));
	if (P.rolling) {
		// Contact::calcRollingVelocities + incrementRollingDisplacement (Contact.cpp:162-180)
		double a_red = c.a0*c.a1/(c.a0+c.a1);
		v3 rv = vscale(2*a_red, vcross(vsub(ld3(ang+3*q.p1), ld3(ang+3*q.p0)), n));
		if (in_predictor) for (int k = 0; k < 3; k++) q.prev_disp_roll[k] = q.disp_roll[k];
		st3(q.disp_roll, vadd(ld3(q.prev_disp_roll), vscale(dt, rv)));
	}
}

__device__ void repulsion_force(const DevParams &P, DPair &q, const DPairConst &c)
{
	double gap = q.r-c.ro;
	double red;
	if (gap > 0) {
		if (P.rep_max_len == -1) red = exp(-gap/P.rep_len);
		else red = exp(-gap/P.rep_len)*0.5*(1+tanh(-(gap-P.rep_max_len)/1e-3));
		red *= c.rep_geo;
	} else {
		red = c.rep_geo;
	}
	q.rep_reduced = red;
	double fn = P.repulsion*red;
	st3(q.rep_force, vscale(-fn, ld3(q.nvec)));
}

__global__ void k_pairs_update(DevParams P, int np, DevClock *__restrict__ clk, const double *__restrict__ pos,
                               const double *__restrict__ vel, const double *__restrict__ ang,
                               DPair *__restrict__ pairs, const DPairConst *__restrict__ pc, int mode,
                               int in_predictor, int zero_dt)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	double sq_local = 0;
	if (t < np) {
		DPair q = pairs[t];
		const DPairConst &c = pc[t];
		DevClock K = *clk;
		const double *sd = K.shear_disp;
		double dt = zero_dt ? 0.0 : K.dt;
		if (mode >= 1 && !(q.flags & PF_INTER)) {
			v3 d = vsub(ld3(pos+3*q.p1), ld3(pos+3*q.p0));
			periodize_diff(P, sd, d);
			double range = c.range;
			if (vsq(d) < range*range) {
				// Interaction ctor + activateForceMembers (Interaction.cpp:13-36, 137-156)
				int p0 = q.p0, p1 = q.p1;
				memset(&q, 0, sizeof q);
				q.p0 = p0; q.p1 = p1;
				q.flags = PF_INTER;
				for (int k = 0; k < 6; k++) q.xf_contact[k] = 0;   // a new Interaction (Contact.h)
				pair_geometry(P, sd, pos, q, c);
				if (q.gap <= 0) contact_activate(P, q);
				lub_update(P, q, c);
			}
		}
		if (mode != 2 && (q.flags & PF_INTER)) {
			// Interaction::updateState (Interaction.cpp:171-198)
			if (q.flags & PF_CONTACT) contact_increment(P, K, vel, ang, q, c, dt, in_predictor);
			pair_geometry(P, sd, pos, q, c);
			if (q.r > c.range) {
				if (q.flags & PF_CONTACT) contact_deactivate(P, q);
				q.flags = 0;   // interaction removed (System.cpp:1395-1400)
			} else {
				// Interaction::updateContactState (Interaction.cpp:199-235)
				q.flags &= ~PF_CHANGED;
				const bool mark = in_predictor && P.brownian_on;
				if (q.flags & PF_CONTACT) {
					if (q.gap > 0) {
						contact_deactivate(P, q);
						if (mark) q.flags |= PF_CHANGED;
					}
				} else if (q.gap <= 0) {
					contact_activate(P, q);
					if (mark) q.flags |= PF_CHANGED;
				}
				if (q.flags & PF_CONTACT) contact_spring(P, q, c);
				lub_update(P, q, c);
				if (P.repulsiveforce) repulsion_force(P, q, c);
				if (P.friction && (q.flags & PF_CONTACT)) sq_local = q.rsv_sq;
			}
		}
		pairs[t] = q;
	}
	// block max of the sliding velocity, then one atomic per block
	__shared__ double red[256];
	red[threadIdx.x] = sq_local;
	__syncthreads();
	for (int o = blockDim.x/2; o > 0; o >>= 1) {
		if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x+o]);
		__syncthreads();
	}
	if (threadIdx.x == 0 && red[0] > 0)
		atomicMax(&clk->sq_max_sliding_bits, (unsigned long long)__double_as_longlong(red[0]));
}

__global__ void k_clear_sliding(DevClock *clk) { clk->sq_max_sliding_bits = 0; }
__global__ void k_finish_sliding(DevClock *clk)
{
	clk->max_sliding_velocity = sqrt(dmax_atomic_value(clk->sq_max_sliding_bits));
}

// ---------------------------------------------------------------------------
// resistance blocks (Lubrication.cpp:406-580, ContactDashpot.cpp:186-340,
// Interaction.cpp:238-311) and diagonal accumulation (System.cpp:1429-1473)
// ---------------------------------------------------------------------------
__device__ void xa_blocks(double XA0, double XA1, double XA3, v3 n, double *od, double *b0, double *b1)
{
	for (int k = 0; k < 18; k++) od[k] = 0;
	for (int k = 0; k < 15; k++) { b0[k] = 0; b1[k] = 0; }
	od[0] = XA1*n.x*n.x; od[1] = XA1*n.x*n.y; od[2] = XA1*n.x*n.z;
	od[5] = XA1*n.y*n.y; od[6] = XA1*n.y*n.z; od[8] = XA1*n.z*n.z;
	b0[0] = XA0*n.x*n.x; b0[1] = XA0*n.x*n.y; b0[2] = XA0*n.x*n.z;
	b0[5] = XA0*n.y*n.y; b0[6] = XA0*n.y*n.z; b0[8] = XA0*n.z*n.z;
	b1[0] = XA3*n.x*n.x; b1[1] = XA3*n.x*n.y; b1[2] = XA3*n.x*n.z;
	b1[5] = XA3*n.y*n.y; b1[6] = XA3*n.y*n.z; b1[8] = XA3*n.z*n.z;
}

// full (squeeze + tangential) blocks; the lubrication and dashpot forms
// share this algebra (the dashpot writes YA+(XA-YA)nn where lubrication
// writes XA nn + YA(1-nn) for the diagonal blocks, handled by `dp`).
__device__ void full_blocks(const double *XA, const double *YA, const double *YB, const double *YC, v3 n,
                            bool dp, double *od, double *b0, double *b1)
{
	double nx = n.x, ny = n.y, nz = n.z;
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
	for (int s = 0; s < 2; s++) {
		int a = s == 0 ? 0 : 3;
		double *b = s == 0 ? b0 : b1;
		if (dp) {
			double XmY = XA[a]-YA[a];
			b[0] = YA[a] + XmY*nx*nx;
			b[1] = XmY*nx*ny;
			b[2] = XmY*nx*nz;
			b[3] = -YB[a]*nz;
			b[4] = YB[a]*ny;
			b[5] = YA[a] + XmY*ny*ny;
			b[6] = XmY*ny*nz;
			b[7] = -YB[a]*nx;
			b[8] = YA[a] + XmY*nz*nz;
			b[9] = YC[a]*(1-nx*nx);
			b[10] = -YC[a]*nx*ny;
			b[11] = -YC[a]*nx*nz;
			b[12] = YC[a]*(1-ny*ny);
			b[13] = -YC[a]*ny*nz;
			b[14] = YC[a]*(1-nz*nz);
		} else {
			double n0n0 = nx*nx, n0n1 = nx*ny, n0n2 = nx*nz, n1n1 = ny*ny, n1n2 = ny*nz, n2n2 = nz*nz;
			double one_n0n0 = 1-n0n0, one_n1n1 = 1-n1n1, one_n2n2 = 1-n2n2;
			double XmY = XA[a]-YA[a];
			b[0] = XA[a]*n0n0+YA[a]*one_n0n0;
			b[1] = XmY*n0n1;
			b[2] = XmY*n0n2;
			b[3] = -YB[a]*nz;
			b[4] = YB[a]*ny;
			b[5] = XA[a]*n1n1+YA[a]*one_n1n1;
			b[6] = XmY*n1n2;
			b[7] = -YB[a]*nx;
			b[8] = XA[a]*n2n2+YA[a]*one_n2n2;
			b[9] = YC[a]*one_n0n0;
			b[10] = -YC[a]*n0n1;
			b[11] = -YC[a]*n0n2;
			b[12] = YC[a]*one_n1n1;
			b[13] = -YC[a]*n1n2;
			b[14] = YC[a]*one_n2n2;
		}
	}
}

__device__ __forceinline__ bool has_resistance(const DevParams &P, int flags)
{
	if (!(flags & PF_INTER)) return false;
	if (P.lub_on) return (flags & PF_DASHPOT) || (flags & PF_LUB);
	return flags & PF_DASHPOT;
}

__global__ void k_pair_blocks(DevParams P, int np, const DPair *__restrict__ pairs, const DPairConst *__restrict__ pc,
                              double *__restrict__ odb, double *__restrict__ bscr)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= np) return;
	const DPair &q = pairs[t];
	double od[18], b0[15], b1[15];
	if (!has_resistance(P, q.flags)) {
		for (int k = 0; k < 18; k++) od[k] = 0;
		for (int k = 0; k < 15; k++) { b0[k] = 0; b1[k] = 0; }
	} else {
		const DPairConst &c = pc[t];
		v3 n = ld3(q.nvec);
		// Interaction::RFU_ODBlock / RFU_DBlocks (Interaction.cpp:247-300): in the
		// corrector of a Brownian step, a pair whose contact opened or closed in
		// the predictor keeps the resistance it had before (lubrication for a
		// new contact, the dashpot for a broken one)
		const bool dp = q.flags & PF_DASHPOT, ch = q.flags & PF_CHANGED;
		const bool use_dashpot = !P.lub_on ? dp : (dp ? !ch : ch);
		if (use_dashpot) {
			const double *D = c.dc;
			if (P.dp_tan_coeff > 0) full_blocks(D+DXA, D+DYA, D+DYB, D+DYC, n, true, od, b0, b1);
			else xa_blocks(D[DXA+0], D[DXA+1], D[DXA+3], n, od, b0, b1);
		} else {
			double XA[4], YA[4], YB[4], YC[4];
			for (int k = 0; k < 4; k++) {
				XA[k] = c.lc[CXA+k]*q.lub_coeff;
				YA[k] = c.lc[CYA+k]*q.log_lub_coeff;
				YB[k] = c.lc[CYB+k]*q.log_lub_coeff;
				YC[k] = c.lc[CYC+k]*q.log_lub_coeff;
			}
			if (P.tangential) full_blocks(XA, YA, YB, YC, n, false, od, b0, b1);
			else xa_blocks(XA[0], XA[1], XA[3], n, od, b0, b1);
		}
	}
	for (int k = 0; k < 18; k++) odb[18*(int64_t)t+k] = od[k];
	for (int k = 0; k < 15; k++) { bscr[30*(int64_t)t+k] = b0[k]; bscr[30*(int64_t)t+15+k] = b1[k]; }
}

// DBlock of particle i: Stokes drag (System.cpp:558-575), then the b1 blocks
// of the pairs where i is the larger index (ascending partner), then the b0
// blocks of the pairs where i is the smaller index -- the reference's
// column-by-column accumulation order.
__global__ void k_dblocks(DevParams P, int n, const double *__restrict__ radius, const int *__restrict__ row_ptr,
                          const int *__restrict__ col_ptr, const int *__restrict__ col_idx,
                          const double *__restrict__ bscr, double *__restrict__ dbl)
{
	// one thread per (particle, entry of its 15-value block): the pairs'
	// contributions to that entry in the reference's order (p1 == i first,
	// then p0 == i); adjacent threads read adjacent entries of a record
	int64_t tt = (int64_t)blockIdx.x*blockDim.x+threadIdx.x;
	if (tt >= 15*(int64_t)n) return;
	int i = (int)(tt/15), e = (int)(tt%15);
	double a = radius[i];
	double d = 0;
	if (e == 0 || e == 5 || e == 8) d = P.sd_coeff*a;
	else if (e == 9 || e == 12 || e == 14) d = P.sd_coeff*pow(a, 3)*4.0/3;
	for (int k = col_ptr[i]; k < col_ptr[i+1]; k++) d += bscr[30*(int64_t)col_idx[k]+15+e];
	for (int t = row_ptr[i]; t < row_ptr[i+1]; t++) d += bscr[30*(int64_t)t+e];
	dbl[15*(int64_t)i+e] = d;
}

// ---------------------------------------------------------------------------
// force components (System.cpp:1727-1828)
// ---------------------------------------------------------------------------
// ContactDashpot::getForceOnP0 (ContactDashpot.cpp:342-385)
__device__ v3 dashpot_force_p0(const DevParams &P, const double *vel_diff, const DPair &q, const DPairConst &c,
                               v3 vi, v3 vj, v3 oi, v3 oj, bool affine)
{
	if (!(q.flags & PF_DASHPOT)) return vzero();
	if (affine) vj = vadd(vj, vscale((double)q.zoff, ld3(vel_diff)));
	v3 n = ld3(q.nvec);
	const double *D = c.dc;
	v3 f = vscale(-vdot(vadd(vscale(D[DXA+0], vi), vscale(D[DXA+1], vj)), n), n);
	if (P.dp_tan_coeff > 0) {
		v3 t1 = vsub(vscale(-D[DYA+0], vsub(vi, vscale(vdot(n, vi), n))), vscale(D[DYA+1], vsub(vj, vscale(vdot(n, vj), n))));
		f = vadd(f, t1);
		v3 t2 = vsub(vscale(-D[DYB+0], vcross(n, oi)), vscale(D[DYB+2], vcross(n, oj)));
		f = vadd(f, t2);
	}
	return f;
}

// per pair: 4 components x (F0, T0, F1, T1) (only < 0, 48 values per pair),
// or the one component `only` (12 values per pair)
__global__ void k_pair_forces(DevParams P, int np, const DevClock *__restrict__ clk, const DPair *__restrict__ pairs,
                              const DPairConst *__restrict__ pc, const double *__restrict__ u_inf,
                              double *__restrict__ scr, int only)
{
	// one thread per (force component, pair), component-major (a warp's pairs
	// share the component's branch): it writes the component's 12 values (the
	// pair's p0 and p1 force and torque), zero where it does not apply
	int64_t tt = (int64_t)blockIdx.x*blockDim.x+threadIdx.x;
	if (tt >= (int64_t)np*(only < 0 ? NPFC : 1)) return;
	int t = (int)(tt%np), comp = only < 0 ? (int)(tt/np) : only;
	double *dst = only < 0 ? scr+48*(int64_t)t+12*comp : scr+12*(int64_t)t;
	double ov[12];
	for (int k = 0; k < 12; k++) ov[k] = 0;
	const DPair &q = pairs[t];
	if (!(q.flags & PF_INTER)) {
		for (int k = 0; k < 12; k++) dst[k] = 0;
		return;
	}
	const DPairConst &c = pc[t];
	v3 n = ld3(q.nvec);
	// contact (Contact::addUpForceTorque, Contact.cpp:419-437)
	if (comp == FC_CONTACT && (q.flags & PF_CONTACT)) {
		v3 f = ld3(q.fs_total);
		st3(ov+0, f);
		st3(ov+6, vneg(f));
		if (q.state >= 2) {
			v3 tq = vcross(n, ld3(q.fs_tan));
			v3 t0 = vscale(c.a0, tq), t1 = vscale(c.a1, tq);
			if (P.rolling) {
				// Contact::addUpForceTorque (Contact.cpp:431-435): +a0 n x f_r on p0, -a1 n x f_r on p1
				v3 tr = vcross(n, ld3(q.f_roll));
				t0 = vadd(t0, vscale(c.a0, tr));
				t1 = vsub(t1, vscale(c.a1, tr));
			}
			st3(ov+3, t0);
			st3(ov+9, t1);
		}
	}
	// dashpot R_FU U_inf (ContactDashpot::getRFU_Uinf, :426-441)
	if (comp == FC_DASHPOT && (q.flags & PF_CONTACT) && (q.flags & PF_DASHPOT)) {
		v3 om = V(clk->Omega[0], clk->Omega[1], clk->Omega[2]);
		v3 f0 = dashpot_force_p0(P, clk->vel_diff, q, c, ld3(u_inf+3*q.p0), ld3(u_inf+3*q.p1), om, om, true);
		v3 t0 = vzero();
		if (P.dp_tan_coeff > 0) t0 = vscale(c.a0, vcross(n, f0));
		st3(ov+0, f0);
		st3(ov+3, t0);
		st3(ov+6, vneg(f0));
		st3(ov+9, vscale(c.a1/c.a0, t0));
	}
	// hydro (Lubrication::calcGEHE_squeeze_tangential / calcGE_squeeze, :332-403)
	if (comp == FC_HYDRO && P.lub_on && (q.flags & PF_LUB)) {
		double XG[4], YG[4], YH[4];
		for (int k = 0; k < 4; k++) {
			XG[k] = c.lc[CXG+k]*q.lub_coeff;
			YG[k] = c.lc[CYG+k]*q.log_lub_coeff;
			YH[k] = c.lc[CYH+k]*q.log_lub_coeff;
		}
		double nnE = vdot(n, sdot(clk->Einf, n));
		if (!P.tangential) {
			double ci = (XG[0]+XG[2])*nnE, cj = (XG[1]+XG[3])*nnE;
			st3(ov+0, V(ci*n.x, ci*n.y, ci*n.z));
			st3(ov+6, V(cj*n.x, cj*n.y, cj*n.z));
		} else {
			double YG0_YG2 = YG[0]+YG[2], YG1_YG3 = YG[1]+YG[3];
			double cGE_i = (XG[0]+XG[2]-2*YG0_YG2)*nnE;
			double cGE_j = (XG[1]+XG[3]-2*YG1_YG3)*nnE;
			double cHE_i = YH[0]+YH[2], cHE_j = YH[1]+YH[3];
			v3 En = sdot(clk->Einf, n);
			st3(ov+0, vadd(vscale(cGE_i, n), vscale(YG0_YG2*2, En)));
			st3(ov+6, vadd(vscale(cGE_j, n), vscale(YG1_YG3*2, En)));
			v3 nExn = vcross(En, n);
			st3(ov+3, vscale(-2*cHE_i, nExn));
			st3(ov+9, vscale(-2*cHE_j, nExn));
		}
	}
	// repulsion (RepulsiveForce::addUpForce, :101-105)
	if (comp == FC_REPULSION && P.repulsiveforce) {
		v3 f = ld3(q.rep_force);
		st3(ov+0, f);
		st3(ov+6, vneg(f));
	}
	for (int k = 0; k < 12; k++) dst[k] = ov[k];
}

// per particle gather: components c with stride 12 in scratch of width W
__global__ void k_gather_pairs(int n, int ncomp, int width, const int *__restrict__ row_ptr,
                               const int *__restrict__ col_ptr, const int *__restrict__ col_idx,
                               const double *__restrict__ scr, double *__restrict__ out)
{
	// one thread per (particle, component, element): pairs with p1 == i first
	// (ascending p0), then pairs with p0 == i (ascending p1)
	int64_t t = (int64_t)blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= (int64_t)n*ncomp*6) return;
	int e = (int)(t%6), c = (int)((t/6)%ncomp), i = (int)(t/(6*ncomp));
	double a = 0;
	for (int k = col_ptr[i]; k < col_ptr[i+1]; k++) a += scr[width*(int64_t)col_idx[k]+12*c+6+e];
	for (int q = row_ptr[i]; q < row_ptr[i+1]; q++) a += scr[width*(int64_t)q+12*c+e];
	out[(int64_t)c*6*n+6*i+e] = a;
}

// torque mask per component: contact (friction), dashpot (1), hydro (tangential), repulsion (0)
__global__ void k_rhs(DevParams P, int n, int divided, const double *__restrict__ fc, double *__restrict__ rhs)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= 6*n) return;
	int d = t%6;
	bool has[NFC] = {true, true, (bool)P.lub_on, (bool)P.repulsiveforce, (bool)P.brownian_on};
	bool tq[NFC] = {(bool)P.friction, true, (bool)P.tangential, false, true};
	const int order[NFC] = {FC_BROWNIAN, FC_CONTACT, FC_DASHPOT, FC_HYDRO, FC_REPULSION};
	if (divided) {
		for (int c = 0; c < NFC; c++)
			rhs[(int64_t)c*6*n+t] = (!has[c] || (d >= 3 && !tq[c])) ? 0.0 : fc[(int64_t)c*6*n+t];
	} else {
		double s = 0;
		for (int u = 0; u < NFC; u++) {
			int c = order[u];
			if (has[c] && (d < 3 || tq[c])) s += fc[(int64_t)c*6*n+t];
		}
		rhs[t] = s;
	}
}

// ---------------------------------------------------------------------------
// stresslets (Stress.cpp:77-287, Lubrication.cpp:587-650, Contact.cpp:439-467,
// RepulsiveForce.cpp:108-131)
// ---------------------------------------------------------------------------
__global__ void k_rate_split(int n, const DevParams P, const DevClock *__restrict__ clk, const double *__restrict__ vc,
                             const double *__restrict__ u_inf, double *__restrict__ split)
{
	// split[12 i + 0..5] = rate-proportional (v, w) incl. u_inf, Omega;
	// split[12 i + 6..11] = rate-independent (v, w)  (Stress.cpp:112-148)
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	double pv[6] = {0, 0, 0, 0, 0, 0}, iv[6] = {0, 0, 0, 0, 0, 0};
	bool has[NFC] = {true, true, (bool)P.lub_on, (bool)P.repulsiveforce, false};
	bool prop[NFC] = {false, true, true, false, false};
	for (int c = 0; c < NFC; c++) {
		if (!has[c]) continue;
		const double *v = vc+(int64_t)c*6*n+6*i;
		for (int e = 0; e < 6; e++) {
			if (prop[c]) pv[e] += v[e];
			else iv[e] += v[e];
		}
	}
	for (int e = 0; e < 3; e++) pv[e] += u_inf[3*i+e];
	for (int e = 0; e < 3; e++) pv[3+e] += clk->Omega[e];
	for (int e = 0; e < 6; e++) { split[12*i+e] = pv[e]; split[12*i+6+e] = iv[e]; }
}

__global__ void k_pair_stress(DevParams P, int np, const DevClock *__restrict__ clk, DPair *__restrict__ pairs,
                              const DPairConst *__restrict__ pc, const double *__restrict__ vc,
                              const double *__restrict__ vel, const double *__restrict__ ang,
                              const double *__restrict__ split, int n, double *__restrict__ scr)
{
	// one thread per (stresslet slot, pair), slot-major (a warp's pairs share
	// the slot's branch): it writes the slot's 12 values (the pair's p0 and p1
	// parts), zero where the slot does not apply
	int64_t tt = (int64_t)blockIdx.x*blockDim.x+threadIdx.x;
	if (tt >= (int64_t)np*NSC) return;
	int t = (int)(tt%np), slot = (int)(tt/np);
	double *o = scr+12*NSC*(int64_t)t+12*slot;
	s2 Si = szero(), Sj = szero();
	DPair &q = pairs[t];
	const int flags = q.flags;
	if (flags & PF_INTER) {
		const DPairConst &c = pc[t];
		int i = q.p0, j = q.p1;
		v3 nv = ld3(q.nvec);
		const bool lub = P.lub_on && (flags & PF_LUB);
		int cc = -1;   // force component of a GU slot
		for (int u = 0; u < NFC; u++)
			if (sc_gu_slot(u) == slot) cc = u;
		bool has[NFC] = {true, true, (bool)P.lub_on, (bool)P.repulsiveforce, (bool)P.brownian_on};
		if (lub && cc >= 0 && has[cc]) {
			// GU of one velocity component (Lubrication::addGUStresslet)
			double XG[4], YG[4], YM[4];
			for (int k = 0; k < 4; k++) {
				XG[k] = c.lc[CXG+k]*q.lub_coeff;
				YG[k] = c.lc[CYG+k]*q.log_lub_coeff;
				YM[k] = c.lc[CYM+k]*q.log_lub_coeff;
			}
			s2 nn = outer(nv);
			const double *v = vc+(int64_t)cc*6*n;
			v3 vi = ld3(v+6*i), vj = ld3(v+6*j), oi = ld3(v+6*i+3), oj = ld3(v+6*j+3);
			double nvi = vdot(nv, vi), nvj = vdot(nv, vj);
			Si = sscale(-(XG[0]*nvi+XG[1]*nvj), nn);
			Sj = sscale(-(XG[2]*nvi+XG[3]*nvj), nn);
			if (P.tangential) {
				s2 ti = ssub(outer_sym(nv, vi), sscale(nvi, nn));
				s2 tj = ssub(outer_sym(nv, vj), sscale(nvj, nn));
				sadd_to(Si, sscale(-2, saddv(sscale(YG[0], ti), sscale(YG[1], tj))));
				sadd_to(Sj, sscale(-2, saddv(sscale(YG[2], ti), sscale(YG[3], tj))));
				s2 t2i = outer_sym(nv, vcross(oi, nv));
				s2 t2j = outer_sym(nv, vcross(oj, nv));
				sadd_to(Si, sscale(-2, saddv(sscale(YM[0], t2i), sscale(YM[1], t2j))));
				sadd_to(Sj, sscale(-2, saddv(sscale(YM[2], t2i), sscale(YM[3], t2j))));
			}
		} else if (lub && slot == SC_ME) {
			// ME (Lubrication::addMEStresslet)
			double XM[4], YM[4];
			for (int k = 0; k < 4; k++) {
				XM[k] = c.lc[CXM+k]*q.lub_coeff;
				YM[k] = c.lc[CYM+k]*q.log_lub_coeff;
			}
			s2 nn = outer(nv);
			double nnE = vdot(nv, sdot(clk->Einf, nv));
			double coeff = 1.5*nnE;
			Si = sscale(coeff*(XM[0]+XM[1]), nn);
			Sj = sscale(coeff*(XM[2]+XM[3]), nn);
			if (P.tangential) {
				v3 En = sdot(clk->Einf, nv);
				s2 T = sscale(2, ssub(outer_sym(nv, En), sscale(nnE, nn)));
				sadd_to(Si, sscale(YM[0]+YM[1], T));
				sadd_to(Sj, sscale(YM[2]+YM[3], T));
			}
		} else if (slot == SC_XF_CONTACT || slot == SC_XF_RATEINDEP || slot == SC_XF_RATEPROP) {
			v3 rv = ld3(q.rvec);
			double r_ij = c.a0+c.a1;
			if (P.control == 0) {
				if (slot == SC_XF_CONTACT && (flags & PF_CONTACT)) {
					// Contact::addUpStress with total velocities
					v3 F = vadd(ld3(q.fs_total), dashpot_force_p0(P, clk->vel_diff, q, c, ld3(vel+3*i),
					                                             ld3(vel+3*j), ld3(ang+3*i), ld3(ang+3*j), true));
					s2 XF = outer_sym(rv, F);
					for (int e = 0; e < 6; e++) q.xf_contact[e] = XF.e[e];   // Contact::calcContactStress (Contact.cpp:439-450)
					Si = sscale(c.a0/r_ij, XF);
					Sj = sscale(c.a1/r_ij, XF);
				}
			} else if (slot == SC_XF_RATEINDEP) {
				if (flags & PF_CONTACT) {
					s2 sp = outer_sym(rv, ld3(q.fs_total));
					sadd_to(Si, sscale(c.a0/r_ij, sp));
					sadd_to(Sj, sscale(c.a1/r_ij, sp));
				}
				if (flags & PF_DASHPOT) {
					const double *si = split+12*i, *sj = split+12*j;
					s2 ri = outer_sym(rv, dashpot_force_p0(P, clk->vel_diff, q, c, ld3(si+6), ld3(sj+6), ld3(si+9),
					                                       ld3(sj+9), false));
					sadd_to(Si, sscale(c.a0/r_ij, ri));
					sadd_to(Sj, sscale(c.a1/r_ij, ri));
				}
			} else if (slot == SC_XF_RATEPROP && (flags & PF_DASHPOT)) {
				const double *si = split+12*i, *sj = split+12*j;
				s2 rp = outer_sym(rv, dashpot_force_p0(P, clk->vel_diff, q, c, ld3(si), ld3(sj), ld3(si+3), ld3(sj+3),
				                                       true));
				sadd_to(Si, sscale(c.a0/r_ij, rp));
				sadd_to(Sj, sscale(c.a1/r_ij, rp));
			}
		} else if (slot == SC_XF_REPULSION && P.repulsiveforce) {
			v3 rv = ld3(q.rvec);
			v3 F = vscale(-(P.repulsion*q.rep_reduced), nv);
			Si = sscale(0.5, outer_sym(rv, F));
			Sj = Si;
		}
	}
	for (int e = 0; e < 6; e++) { o[e] = Si.e[e]; o[6+e] = Sj.e[e]; }
}

// Per-pair quantities of the output files (Simulation::outputData,
// outputIntFileTxt: Simulation.cpp:641-809, 967-1006), at the current state.
// Record of OUT_W doubles per superset pair:
//   0 flags, 1 p0, 2 p1, 3 contact state, 4 reduced gap, 5-7 nvec,
//   8-10 Lubrication::getTotalForce (Lubrication.cpp:659-690; non-affine
//        velocities, the pair's current coefficients, + GE),
//   11-13 Contact::getTotalForce (Contact.cpp:235-250; spring + dashpot with
//        the total velocities; zero when not in contact),
//   14 RepulsiveForce force_norm (RepulsiveForce.cpp:76-83),
//   15-20 Contact::contact_stresslet_XF as last set (Contact.cpp:439-450),
//   21 Contact::calcEnergy (Contact.cpp:469-485) when in contact,
//   22 RepulsiveForce::calcEnergy (RepulsiveForce.cpp:133-150) with repulsion,
//   23-25 disp_tan, 26-28 disp_rolling.
__global__ void k_pair_output(DevParams P, int np, const DevClock *__restrict__ clk, const DPair *__restrict__ pairs,
                              const DPairConst *__restrict__ pc, const double *__restrict__ vel,
                              const double *__restrict__ ang, const double *__restrict__ na, double *__restrict__ out)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= np) return;
	const DPair &q = pairs[t];
	double *o = out+OUT_W*(int64_t)t;
	for (int k = 0; k < OUT_W; k++) o[k] = 0;
	o[0] = q.flags; o[1] = q.p0; o[2] = q.p1; o[3] = q.state; o[4] = q.gap;
	if (!(q.flags & PF_INTER)) return;
	const DPairConst &c = pc[t];
	int i = q.p0, j = q.p1;
	v3 n = ld3(q.nvec);
	st3(o+5, n);
	if (P.lub_on) {
		double XA[4], YA[4], YB[4], XG[4], YG[4];
		for (int k = 0; k < 4; k++) {
			XA[k] = c.lc[CXA+k]*q.lub_coeff;
			YA[k] = c.lc[CYA+k]*q.log_lub_coeff;
			YB[k] = c.lc[CYB+k]*q.log_lub_coeff;
			XG[k] = c.lc[CXG+k]*q.lub_coeff;
			YG[k] = c.lc[CYG+k]*q.log_lub_coeff;
		}
		v3 vi = ld3(na+6*i), vj = ld3(na+6*j);
		v3 f = vscale(-vdot(vadd(vscale(XA[0], vi), vscale(XA[1], vj)), n), n);
		if (P.tangential) {
			v3 oi = ld3(na+6*i+3), oj = ld3(na+6*j+3);
			f = vadd(f, vsub(vscale(-YA[0], vsub(vi, vscale(vdot(n, vi), n))),
			                 vscale(YA[1], vsub(vj, vscale(vdot(n, vj), n)))));
			f = vadd(f, vsub(vscale(-YB[0], vcross(n, oi)), vscale(YB[2], vcross(n, oj))));
		}
		// GE_i (Lubrication::calcGE_squeeze / calcGE_squeeze_tangential)
		double nnE = vdot(n, sdot(clk->Einf, n));
		if (!P.tangential) {
			double ci = (XG[0]+XG[2])*nnE;
			f = vadd(f, V(ci*n.x, ci*n.y, ci*n.z));
		} else {
			double YG0_YG2 = YG[0]+YG[2];
			double cGE_i = (XG[0]+XG[2]-2*YG0_YG2)*nnE;
			v3 En = sdot(clk->Einf, n);
			f = vadd(f, vadd(vscale(cGE_i, n), vscale(YG0_YG2*2, En)));
		}
		st3(o+8, f);
	}
	if (q.flags & PF_CONTACT) {
		v3 F = vadd(ld3(q.fs_total), dashpot_force_p0(P, clk->vel_diff, q, c, ld3(vel+3*i), ld3(vel+3*j),
		                                             ld3(ang+3*i), ld3(ang+3*j), true));
		st3(o+11, F);
		double overlap = -q.gap;
		double e = 0.5*c.kn_s*overlap*overlap;
		if (q.state >= 2) {
			e += 0.5*c.kt_s*vsq(ld3(q.disp_tan));
			if (P.rolling) e += 0.5*c.kr_s*vsq(ld3(q.disp_roll));
		}
		o[21] = e;
	}
	if (P.repulsiveforce) {
		o[14] = P.repulsion*q.rep_reduced;
		double gap = q.r-c.ro, e;
		if (gap > 0) {
			if (P.rep_max_len == -1) e = c.rep_geo*P.rep_len*exp(-gap/P.rep_len);
			else e = c.rep_geo*P.rep_len*exp(-gap/P.rep_len)*0.5*(1+tanh(-(gap-P.rep_max_len)/1e-3));
		} else {
			e = c.rep_geo*P.rep_len*(1-gap);
		}
		o[22] = e;
	}
	for (int e = 0; e < 6; e++) o[15+e] = q.xf_contact[e];
	st3(o+23, ld3(q.disp_tan));
	st3(o+26, ld3(q.disp_roll));
}

// per-component totals over particles (fixed-order tree reduction)
// per stresslet component, the sum over particles (one CTA of 1024 threads
// each; a fixed reduction order: per thread, then warps by shuffles, then
// warps)
__global__ void __launch_bounds__(1024) k_stress_totals(int n, const double *__restrict__ sc,
                                                        double *__restrict__ tot)
{
	__shared__ double red[32][6];
	int c = blockIdx.x;
	double a[6] = {0, 0, 0, 0, 0, 0};
	for (int i = threadIdx.x; i < n; i += blockDim.x)
		for (int e = 0; e < 6; e++) a[e] += sc[(int64_t)c*6*n+6*i+e];
	for (int o = 16; o > 0; o >>= 1)
		for (int e = 0; e < 6; e++) a[e] += __shfl_down_sync(0xffffffffu, a[e], o);
	int w = threadIdx.x/32, l = threadIdx.x%32;
	if (l == 0)
		for (int e = 0; e < 6; e++) red[w][e] = a[e];
	__syncthreads();
	if (w == 0) {
		for (int e = 0; e < 6; e++) a[e] = l < (int)blockDim.x/32 ? red[l][e] : 0.0;
		for (int o = 16; o > 0; o >>= 1)
			for (int e = 0; e < 6; e++) a[e] += __shfl_down_sync(0xffffffffu, a[e], o);
		if (l == 0)
			for (int e = 0; e < 6; e++) tot[6*c+e] = a[e];
	}
}

__device__ void set_rate(const DevParams &P, DevClock &K, double rate)
{
	// System::set_shear_rate + setVelocityDifference (System.cpp:1967-1982)
	K.shear_rate = rate;
	for (int k = 0; k < 3; k++) K.Omega[k] = P.Ohat[k]*rate;
	for (int k = 0; k < 6; k++) K.Einf[k] = P.Ehat[k]*rate;
	v3 vd = vscale(2, sdot(K.Einf, V(0, 0, P.lz)));
	K.vel_diff[0] = vd.x; K.vel_diff[1] = vd.y; K.vel_diff[2] = vd.z;
}

__global__ void k_set_rate(DevParams P, DevClock *clk, double rate) { set_rate(P, *clk, rate); }

// System::computeShearRate (System.cpp:2017-2055) from the component totals
__global__ void k_shear_rate(DevParams P, DevClock *clk, const double *__restrict__ tot, int has_mask)
{
	DevClock &K = *clk;
	const int rate_of[NSC] = {1, 0, 1, 1, 0, 2, 0, 1, 0, 0, 0};  // 0 indep 1 prop 2 dependent
	double prop[6] = {0, 0, 0, 0, 0, 0}, indep[6] = {0, 0, 0, 0, 0, 0};
	for (int c = 0; c < NSC; c++) {
		if (!(has_mask & (1 << c))) continue;
		for (int e = 0; e < 6; e++) {
			if (rate_of[c] == 0) indep[e] += tot[6*c+e];
			if (rate_of[c] == 1) prop[e] += tot[6*c+e];
		}
	}
	double inv = 1.0/P.system_volume;
	for (int e = 0; e < 6; e++) { prop[e] *= inv; indep[e] *= inv; }
	for (int e = 0; e < 6; e++) prop[e] += 2*K.Einf[e]/(6*M_PI);
	double rp = doubledot(prop, K.Einf), ri = doubledot(indep, K.Einf);
	K.rate_prop = rp;
	K.rate_indep = ri;
	if (rp != 0) set_rate(P, K, (P.target_stress-ri)/rp);
	if (K.strain < P.init_strain_limit && K.shear_rate > P.init_rate_limit) set_rate(P, K, P.init_rate_limit);
}

// rescale rate-proportional components (System.cpp:2264-2271), sum
// components into na (System.cpp:2236-2250) and the max |U_na|
__global__ void k_velocities(DevParams P, int n, int divided, int stress_ctl, int want_max, DevClock *__restrict__ clk,
                             double *__restrict__ vc, const double *__restrict__ sol, double *__restrict__ na)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	double sq = 0;
	if (i < n) {
		double v[6];
		// System::sumUpVelocityComponents in map order (brownian first);
		// 2D Brownian: rushWorkFor2DBrownian (System.cpp:2394-2416) on the
		// Brownian component (divided) or the total
		bool rush = P.brownian_on && P.twodim;
		if (divided) {
			bool has[NFC] = {true, true, (bool)P.lub_on, (bool)P.repulsiveforce, (bool)P.brownian_on};
			bool prop[NFC] = {false, true, true, false, false};
			const int order[NFC] = {FC_BROWNIAN, FC_CONTACT, FC_DASHPOT, FC_HYDRO, FC_REPULSION};
			double rate = clk->shear_rate;
			for (int e = 0; e < 6; e++) v[e] = 0;
			for (int u = 0; u < NFC; u++) {
				int c = order[u];
				if (!has[c]) continue;
				double *x = vc+(int64_t)c*6*n+6*i;
				if (stress_ctl && prop[c])
					for (int e = 0; e < 6; e++) x[e] *= rate;
				if (rush && c == FC_BROWNIAN) { x[1] = 0; x[3] = 0; x[5] = 0; }
				for (int e = 0; e < 6; e++) v[e] += x[e];
			}
		} else {
			for (int e = 0; e < 6; e++) v[e] = sol[6*i+e];
			if (rush) { v[1] = 0; v[3] = 0; v[5] = 0; }
		}
		for (int e = 0; e < 6; e++) na[6*i+e] = v[e];
		sq = v[0]*v[0]+v[1]*v[1]+v[2]*v[2];
	}
	if (!want_max) return;
	__shared__ double red[256];
	red[threadIdx.x] = sq;
	__syncthreads();
	for (int o = blockDim.x/2; o > 0; o >>= 1) {
		if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x+o]);
		__syncthreads();
	}
	if (threadIdx.x == 0 && red[0] > 0)
		atomicMax(&clk->sq_max_vel_bits, (unsigned long long)__double_as_longlong(red[0]));
}

__global__ void k_clear_maxvel(DevClock *clk) { clk->sq_max_vel_bits = 0; }
__global__ void k_finish_maxvel(DevClock *clk) { clk->max_velocity = sqrt(dmax_atomic_value(clk->sq_max_vel_bits)); }

// System::computeUInf (System.cpp:2357-2367)
__global__ void k_u_inf(int n, const DevClock *__restrict__ clk, const double *__restrict__ pos, double *__restrict__ u)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	v3 p = ld3(pos+3*i);
	v3 om = V(clk->Omega[0], clk->Omega[1], clk->Omega[2]);
	st3(u+3*i, vadd(sdot(clk->Einf, p), vcross(om, p)));
}

// System::adjustVelocityPeriodicBoundary (System.cpp:2369-2392)
__global__ void k_total_velocity(int n, const DevClock *__restrict__ clk, const double *__restrict__ na,
                                 const double *__restrict__ u_inf, double *__restrict__ vel, double *__restrict__ ang)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	st3(vel+3*i, vadd(ld3(na+6*i), ld3(u_inf+3*i)));
	st3(ang+3*i, vadd(ld3(na+6*i+3), V(clk->Omega[0], clk->Omega[1], clk->Omega[2])));
}

// System::adaptTimeStep(time_end, strain_end) (System.cpp:1013-1066)
__global__ void k_adapt_dt(DevParams P, DevClock *clk, double time_end, double strain_end)
{
	DevClock &K = *clk;
	double dt;
	if (K.max_velocity > 0 || K.max_sliding_velocity > 0) {
		if (K.max_velocity > K.max_sliding_velocity) dt = P.disp_max/K.max_velocity;
		else dt = P.disp_max/K.max_sliding_velocity;
	} else {
		dt = P.disp_max/K.shear_rate;
	}
	if (dt*K.shear_rate > P.disp_max) dt = P.disp_max/K.shear_rate;
	if (P.dt_max > 0 && dt > P.dt_max) dt = P.dt_max;
	if (P.dt_min > 0 && dt < P.dt_min) dt = P.dt_min;
	if (strain_end >= 0) {
		if (fabs(dt*K.shear_rate) > strain_end-K.strain) dt = fabs((strain_end-K.strain)/K.shear_rate);
	}
	if (time_end >= 0) {
		if (K.time+dt > time_end) dt = time_end-K.time;
	}
	K.dt = dt;
}

// clocks + System::timeStepBoxing (System.cpp:672-717)
__global__ void k_boxing(DevParams P, DevClock *clk)
{
	DevClock &K = *clk;
	K.time += K.dt;
	K.steps++;
	K.strain += K.shear_rate*K.dt;
	v3 ez = sdot(K.Einf, V(0, 0, 1));
	v3 inc = V(2*ez.x*K.dt, 2*ez.y*K.dt, 2*ez.z*K.dt);
	for (int k = 0; k < 3; k++) K.shear_disp[k] += P.lz*(k == 0 ? inc.x : (k == 1 ? inc.y : inc.z));
	K.shear_strain[0] += inc.x;
	K.shear_strain[1] += inc.y;
	K.shear_strain[2] += inc.z;
	int m = (int)(K.shear_disp[0]/P.lx);
	if (K.shear_disp[0] < 0) m--;
	K.shear_disp[0] = K.shear_disp[0]-m*P.lx;
	if (!P.twodim) {
		m = (int)(K.shear_disp[1]/P.ly);
		if (K.shear_disp[1] < 0) m--;
		K.shear_disp[1] = K.shear_disp[1]-m*P.ly;
	}
}

// System::displacement (System.cpp:2418-2443); corrector: the velocity
// average of timeStepMoveCorrector (System.cpp:1164-1187) first.  mode 0
// (Euler) and 2 (corrector) then add na_velocity dt to na_disp (System.cpp:
// 877, 981); in 2D the angle follows the y angular velocity (System.cpp:1113,
// 1151, 1178).
__global__ void k_move(DevParams P, int n, int mode, const DevClock *__restrict__ clk, double *__restrict__ pos,
                       double *__restrict__ vel, double *__restrict__ ang, const double *__restrict__ vel_pred,
                       const double *__restrict__ ang_pred, const double *__restrict__ na,
                       double *__restrict__ na_disp, double *__restrict__ angle)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	double dt = clk->dt;
	v3 v = ld3(vel+3*i);
	v3 dr;
	if (mode == 2) {
		v3 vp = ld3(vel_pred+3*i);
		v = vscale(0.5, vadd(v, vp));
		double wy = 0.5*(ang[3*i+1]+ang_pred[3*i+1]);
		st3(ang+3*i, vscale(0.5, vadd(ld3(ang+3*i), ld3(ang_pred+3*i))));
		dr = vscale(dt, vsub(v, vp));
		if (P.twodim) angle[i] += (wy-ang_pred[3*i+1])*dt;
	} else {
		dr = vscale(dt, v);
		if (P.twodim) angle[i] += ang[3*i+1]*dt;
	}
	if (mode != 1) {
		na_disp[3*i+0] += na[6*i+0]*dt;
		na_disp[3*i+1] += na[6*i+1]*dt;
		na_disp[3*i+2] += na[6*i+2]*dt;
	}
	v3 p = vadd(ld3(pos+3*i), dr);
	int zs = periodize(P, clk->shear_disp, p);
	if (zs != 0) v = vadd(v, vscale((double)zs, ld3(clk->vel_diff)));
	st3(pos+3*i, p);
	st3(vel+3*i, v);
}

__global__ void k_copy(int64_t n, const double *__restrict__ a, double *__restrict__ b)
{
	int64_t t = blockIdx.x*(int64_t)blockDim.x+threadIdx.x;
	if (t < n) b[t] = a[t];
}

__global__ void k_set_dt(DevClock *clk, double dt) { clk->dt = dt; }

__global__ void k_sticky(const int *status, int *err)
{
	if (*status != 0x7fffffff) atomicMin(err, *status);
}

// merge pair state from the previous superset (rows sorted by p1)
__global__ void k_merge(int np, int n, const int *__restrict__ new_row_ptr, const int *__restrict__ new_cand,
                        const DPair *__restrict__ old_pairs, const int *__restrict__ old_row_ptr, int old_n,
                        DPair *__restrict__ out)
{
	int i = blockIdx.x*blockDim.x+threadIdx.x;
	if (i >= n) return;
	for (int t = new_row_ptr[i]; t < new_row_ptr[i+1]; t++) {
		int j = new_cand[t];
		int found = -1;
		if (old_pairs && i < old_n) {
			int lo = old_row_ptr[i], hi = old_row_ptr[i+1]-1;
			while (lo <= hi) {
				int m = (lo+hi) >> 1;
				int pj = old_pairs[m].p1;
				if (pj == j) { found = m; break; }
				if (pj < j) lo = m+1; else hi = m-1;
			}
		}
		DPair q;
		if (found >= 0) q = old_pairs[found];
		else {
			memset(&q, 0, sizeof q);
			q.p0 = i; q.p1 = j;
		}
		out[t] = q;
	}
	(void)np;
}

// Interaction counts of the current state (lfg_sim_scalars: interactions,
// contacts, lubricated pairs, pairs with a resistance): one thread per pair
// slot, a warp sum by ballot, one atomic per warp and count.  out[4] must
// start at zero.
__global__ void k_pair_counts(int np, int lub_on, const DPair *__restrict__ pairs, int *__restrict__ out)
{
	const int t = blockIdx.x*blockDim.x+threadIdx.x;
	const int f = t < np ? pairs[t].flags : 0;
	const bool inter = f & PF_INTER;
	const bool res = lub_on ? ((f & PF_DASHPOT) || (f & PF_LUB)) : (f & PF_DASHPOT);
	const unsigned b0 = __ballot_sync(PFULL, inter), b1 = __ballot_sync(PFULL, inter && (f & PF_CONTACT));
	const unsigned b2 = __ballot_sync(PFULL, inter && (f & PF_LUB)), b3 = __ballot_sync(PFULL, inter && res);
	if ((threadIdx.x & 31) == 0) {
		if (b0) atomicAdd(out, __popc(b0));
		if (b1) atomicAdd(out+1, __popc(b1));
		if (b2) atomicAdd(out+2, __popc(b2));
		if (b3) atomicAdd(out+3, __popc(b3));
	}
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static CellView view(const DevSim &S)
{
	CellView C;
	C.ncx = S.ncx; C.ncy = S.ncy; C.ncz = S.ncz; C.brute = S.brute; C.n = S.n;
	C.csx = S.csx; C.csy = S.csy; C.csz = S.csz;
	C.start = S.cell_start; C.count = S.cell_count; C.list = S.cell_list;
	return C;
}

void phys_set_shear_rate(DevSim &S, double rate, bool, cudaStream_t st)
{
	k_set_rate<<<1, 1, 0, st>>>(S.P, S.clock, rate);
	S.launches++;
}

void phys_u_inf(DevSim &S, cudaStream_t st)
{
	k_u_inf<<<blocks_for(S.n, 128), 128, 0, st>>>(S.n, S.clock, S.pos, S.u_inf);
	S.launches++;
}

void phys_cells(DevSim &S, double, cudaStream_t st)
{
	if (S.brute) return;
	int ncell = S.ncx*S.ncy*S.ncz;
	LFG_CUDA(cudaMemsetAsync(S.cell_count, 0, sizeof(int)*ncell, st));
	CellView C = view(S);
	k_cell_assign<<<blocks_for(S.n, 128), 128, 0, st>>>(S.P, C, S.pos, S.cell_of, S.cell_count);
	k_scan<<<1, 1024, 0, st>>>(ncell, S.cell_count, S.cell_start, nullptr);
	// reuse cand_count as the fill counter
	LFG_CUDA(cudaMemsetAsync(S.cand_count, 0, sizeof(int)*ncell, st));
	k_cell_fill<<<blocks_for(S.n, 128), 128, 0, st>>>(S.n, S.cell_of, S.cell_start, S.cand_count, S.cell_list);
	k_cell_sort<<<blocks_for((int64_t)32*ncell, 128), 128, 0, st>>>(ncell, S.cell_start, S.cell_count, S.cell_list,
	                                                                 S.pos, S.radius, S.cell_rec, S.cell_rec32);
	S.launches += 4;
}

void phys_candidates(DevSim &S, cudaStream_t st, int *h_total)
{
	CellView C = view(S);
	k_candidates<<<blocks_for((int64_t)32*S.n, 128), 128, 0, st>>>(S.P, C, S.clock, S.pos, S.radius, S.cell_rec,
	                                                                S.cell_rec32, S.cand_count, nullptr, nullptr);
	k_scan<<<1, 1024, 0, st>>>(S.n, S.cand_count, S.cand_ptr, nullptr);
	LFG_CUDA(cudaMemcpyAsync(h_total, S.cand_ptr+S.n, sizeof(int), cudaMemcpyDeviceToHost, st));
	LFG_CUDA(cudaStreamSynchronize(st));
	if (*h_total > S.cand_cap) {
		if (S.cand) cudaFree(S.cand);
		S.cand_cap = *h_total+*h_total/4+1024;
		LFG_CUDA(cudaMalloc((void **)&S.cand, sizeof(int)*S.cand_cap));
	}
	k_candidates<<<blocks_for((int64_t)32*S.n, 128), 128, 0, st>>>(S.P, C, S.clock, S.pos, S.radius, S.cell_rec,
	                                                                S.cell_rec32, S.cand_count, S.cand_ptr, S.cand);
	S.launches += 3;
}

void phys_check_superset(DevSim &S, cudaStream_t st)
{
	CellView C = view(S);
	if (S.brute)
		k_check_superset<<<blocks_for((S.P.twodim ? 9 : 27)*S.n, 256), 256, 0, st>>>(S.P, C, S.clock, S.pos, S.radius,
		                                                                           S.row_ptr, S.pairs);
	else
		k_check_cells<<<S.ncx*S.ncy*S.ncz, 128, 0, st>>>(S.P, C, S.clock, S.cell_rec, S.cell_rec32, S.row_ptr,
		                                                 S.cand);
	S.launches++;
}

void phys_pair_constants(DevSim &S, cudaStream_t st)
{
	if (!S.npairs) return;
	k_pair_constants<<<blocks_for(S.npairs, 128), 128, 0, st>>>(S.P, S.npairs, S.pairs, S.radius, S.pconst);
	S.launches++;
}

void phys_clear_sliding(DevSim &S, cudaStream_t st) { k_clear_sliding<<<1, 1, 0, st>>>(S.clock); S.launches++; }
void phys_finish_sliding(DevSim &S, cudaStream_t st) { k_finish_sliding<<<1, 1, 0, st>>>(S.clock); S.launches++; }

void phys_pairs_update(DevSim &S, int mode, int in_predictor, bool zero_dt, cudaStream_t st)
{
	k_clear_sliding<<<1, 1, 0, st>>>(S.clock);
	if (S.npairs)
		// 64 threads per CTA: one thread per pair holds a whole pair record, so
		// small CTAs spread the ~10^4 pairs over every SM
		k_pairs_update<<<blocks_for(S.npairs, 64), 64, 0, st>>>(S.P, S.npairs, S.clock, S.pos, S.vel, S.ang, S.pairs,
		                                                        S.pconst, mode, in_predictor, zero_dt ? 1 : 0);
	k_finish_sliding<<<1, 1, 0, st>>>(S.clock);
	S.launches += 3;
}

void phys_blocks(DevSim &S, double *dbl, double *odbl, cudaStream_t st)
{
	if (S.npairs)
		k_pair_blocks<<<blocks_for(S.npairs, 64), 64, 0, st>>>(S.P, S.npairs, S.pairs, S.pconst, odbl, S.blk_scratch);
	k_dblocks<<<blocks_for(15*(int64_t)S.n, 128), 128, 0, st>>>(S.P, S.n, S.radius, S.row_ptr, S.col_ptr, S.col_idx,
	                                                S.blk_scratch, dbl);
	S.launches += 2;
}

void phys_force_components(DevSim &S, cudaStream_t st)
{
	if (S.npairs)
		k_pair_forces<<<blocks_for((int64_t)S.npairs*NPFC, 128), 128, 0, st>>>(S.P, S.npairs, S.clock, S.pairs, S.pconst,
		                                                                       S.u_inf, S.pair_scratch, -1);
	k_gather_pairs<<<blocks_for(6*NPFC*S.n, 256), 256, 0, st>>>(S.n, NPFC, 12*NPFC, S.row_ptr, S.col_ptr,
	                                                      S.col_idx, S.pair_scratch, S.fc);
	S.launches += 2;
}

// ---------------------------------------------------------------------------
// Force components into caller memory without allocating (backs
// lfg_sim_force_component_noalloc).  Some callers may not allocate device
// memory while they run: a host application that owns every device
// allocation through its own pool, or one on a path where the implicit device
// synchronisation of cudaMalloc/cudaFree is not allowed.  For them the
// per-pair intermediate of k_pair_forces, computed for the requested
// component only (12 doubles per pair slot), goes to a fixed scratch in static
// device memory instead of DevSim::pair_scratch.  k_pair_forces writes all 12
// values of every slot it covers before k_gather_pairs reads them, so the
// scratch need not start at zero.  All calls on one device share it: calls
// that overlap in time race.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_noalloc_pair_scratch[(size_t)NOALLOC_MAX_PAIRS*12];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[NOALLOC_MAX_DEVICES];

double *noalloc_pair_scratch(int device)
{
	if (device < 0 || device >= NOALLOC_MAX_DEVICES)
		throw Error{LFG_ERR_BAD_ARG, device, "device ordinal beyond the no-allocation scratch table"};
	std::lock_guard<std::mutex> lock(g_noalloc_mu);
	if (!g_noalloc_ptr[device]) {
		// set-up, once per device, with that device current
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_pair_scratch);
		if (e != cudaSuccess)
			throw Error{LFG_ERR_CUDA, (int)e,
			            std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ")+
			            cudaGetErrorString(e)};
		g_noalloc_ptr[device] = static_cast<double *>(p);
	}
	return g_noalloc_ptr[device];
}

void phys_force_component_into(DevSim &S, int comp, double *scr, double *out, cudaStream_t st)
{
	if (comp < 0 || comp >= NPFC)
		throw Error{LFG_ERR_BAD_ARG, comp, "pair-force component must be 0..3"};
	if (S.npairs > NOALLOC_MAX_PAIRS)
		throw Error{LFG_ERR_BAD_ARG, S.npairs, "pair slots exceed the no-allocation scratch (32768)"};
	if (S.npairs)
		k_pair_forces<<<blocks_for((int64_t)S.npairs, 128), 128, 0, st>>>(S.P, S.npairs, S.clock, S.pairs, S.pconst,
		                                                                  S.u_inf, scr, comp);
	k_gather_pairs<<<blocks_for(6*S.n, 256), 256, 0, st>>>(S.n, 1, 12, S.row_ptr, S.col_ptr, S.col_idx, scr, out);
	S.launches += 2;
}

void phys_rhs(DevSim &S, int divided, cudaStream_t st)
{
	k_rhs<<<blocks_for(6*S.n, 256), 256, 0, st>>>(S.P, S.n, divided, S.fc, S.rhs);
	S.launches++;
}

// System::calcStressPerParticle's Brownian part (Stress.cpp:270-286): every
// component is reset first, so the predictor keeps a copy of the Brownian GU
// stress in brownian_predictor, and the corrector halves its own Brownian GU
// stress with the (just reset, zero) predictor copy
__global__ void k_brownian_stress(int n6, int in_predictor, double *__restrict__ sc)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (t >= n6) return;
	double *b = sc+(int64_t)SC_GU_BROWNIAN*n6, *bp = sc+(int64_t)SC_BROWNIAN_PRED*n6;
	if (in_predictor) bp[t] = b[t];
	else b[t] = 0.5*(b[t]-bp[t]);
}

// Standard normal deviates for the Brownian force: Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC11),
// counter (thread, draw), key = seed; Box-Muller on the two pairs of each
// 4-word output.  Thread t writes psi[4t .. 4t+3].
__device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
	for (int r = 0; r < 10; r++) {
		uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u*c[0];
		uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u*c[2];
		uint32_t n0 = hi1^c[1]^k0, n1 = lo1, n2 = hi0^c[3]^k1, n3 = lo0;
		c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
}

__global__ void k_brownian_psi(int n6, uint32_t k0, uint32_t k1, uint32_t d0, uint32_t d1, double amp,
                               double *__restrict__ psi)
{
	int t = blockIdx.x*blockDim.x+threadIdx.x;
	if (4*t >= n6) return;
	uint32_t c[4] = {(uint32_t)t, d0, d1, 0x4C464744u};
	philox4x32_10(c, k0, k1);
	double z[4];
	for (int h = 0; h < 2; h++) {
		// u1 in (0, 1], u2 in [0, 1)
		double u1 = ((double)c[2*h]+1.0)*2.3283064365386963e-10;
		double u2 = (double)c[2*h+1]*2.3283064365386963e-10;
		double r = sqrt(-2.0*log(u1));
		double sn, cs;
		sincospi(2.0*u2, &sn, &cs);
		z[2*h] = r*cs;
		z[2*h+1] = r*sn;
	}
	for (int q = 0; q < 4; q++)
		if (4*t+q < n6) psi[4*t+q] = amp*z[q];
}

void phys_brownian_psi(DevSim &S, unsigned long long seed, unsigned long long draw, double amp, double *psi,
                       cudaStream_t st)
{
	int n6 = 6*S.n;
	int threads = (n6+3)/4;
	k_brownian_psi<<<blocks_for(threads, 256), 256, 0, st>>>(n6, (uint32_t)seed, (uint32_t)(seed >> 32),
	                                                          (uint32_t)draw, (uint32_t)(draw >> 32), amp, psi);
	S.launches++;
}

void phys_stresslets(DevSim &S, int in_predictor, cudaStream_t st)
{
	double *split = S.sc_tot+6*NSC;  // n x 12 region after the totals
	if (S.P.control == 1) {
		k_rate_split<<<blocks_for(S.n, 128), 128, 0, st>>>(S.n, S.P, S.clock, S.vc, S.u_inf, split);
		S.launches++;
	}
	if (S.npairs)
		k_pair_stress<<<blocks_for(S.npairs*NSC, 128), 128, 0, st>>>(S.P, S.npairs, S.clock, S.pairs, S.pconst, S.vc,
		                                                             S.vel, S.ang, split, S.n, S.pair_scratch);
	k_gather_pairs<<<blocks_for(6*NSC*S.n, 256), 256, 0, st>>>(S.n, NSC, 12*NSC, S.row_ptr, S.col_ptr, S.col_idx,
	                                                     S.pair_scratch, S.sc);
	if (S.P.brownian_on) {
		k_brownian_stress<<<blocks_for(6*S.n, 256), 256, 0, st>>>(6*S.n, in_predictor, S.sc);
		S.launches++;
	}
	k_stress_totals<<<NSC, 1024, 0, st>>>(S.n, S.sc, S.sc_tot);
	S.launches += 3;
}

static int sc_mask(const DevParams &P)
{
	int m = 0;
	if (P.lub_on) {
		m |= 1 << SC_ME;
		m |= 1 << SC_GU_CONTACT;
		m |= 1 << SC_GU_DASHPOT;
		m |= 1 << SC_GU_HYDRO;
		if (P.repulsiveforce) m |= 1 << SC_GU_REPULSION;
		if (P.brownian_on) m |= 1 << SC_GU_BROWNIAN;
	}
	if (P.brownian_on) m |= 1 << SC_BROWNIAN_PRED;
	if (P.control == 0) m |= 1 << SC_XF_CONTACT;
	else m |= (1 << SC_XF_RATEPROP) | (1 << SC_XF_RATEINDEP);
	if (P.repulsiveforce) m |= 1 << SC_XF_REPULSION;
	return m;
}

void phys_shear_rate_from_stress(DevSim &S, cudaStream_t st)
{
	k_shear_rate<<<1, 1, 0, st>>>(S.P, S.clock, S.sc_tot, sc_mask(S.P));
	S.launches++;
}

void phys_velocities(DevSim &S, int divided, int in_predictor, cudaStream_t st)
{
	int want_max = (!S.P.fixed_dt && in_predictor) ? 1 : 0;
	if (want_max) { k_clear_maxvel<<<1, 1, 0, st>>>(S.clock); S.launches++; }
	k_velocities<<<blocks_for(S.n, 256), 256, 0, st>>>(S.P, S.n, divided, S.P.control == 1, want_max, S.clock, S.vc,
	                                                   S.sol, S.na);
	S.launches++;
	if (want_max) { k_finish_maxvel<<<1, 1, 0, st>>>(S.clock); S.launches++; }
	if (S.P.control == 1) phys_u_inf(S, st);
	k_total_velocity<<<blocks_for(S.n, 128), 128, 0, st>>>(S.n, S.clock, S.na, S.u_inf, S.vel, S.ang);
	S.launches++;
}

void phys_adapt_dt(DevSim &S, double time_end, double strain_end, cudaStream_t st)
{
	k_adapt_dt<<<1, 1, 0, st>>>(S.P, S.clock, time_end, strain_end);
	S.launches++;
}

void phys_boxing(DevSim &S, cudaStream_t st)
{
	k_boxing<<<1, 1, 0, st>>>(S.P, S.clock);
	S.launches++;
}

void phys_pair_output(DevSim &S, double *out, cudaStream_t st)
{
	if (!S.npairs) return;
	k_pair_output<<<blocks_for(S.npairs, 128), 128, 0, st>>>(S.P, S.npairs, S.clock, S.pairs, S.pconst, S.vel, S.ang,
	                                                         S.na, out);
	S.launches++;
}

void phys_move(DevSim &S, int mode, cudaStream_t st)
{
	k_move<<<blocks_for(S.n, 128), 128, 0, st>>>(S.P, S.n, mode, S.clock, S.pos, S.vel, S.ang, S.vel_pred, S.ang_pred,
	                                             S.na, S.na_disp, S.angle);
	S.launches++;
}

void phys_save_pred(DevSim &S, cudaStream_t st)
{
	k_copy<<<blocks_for(3*S.n, 256), 256, 0, st>>>(3*(int64_t)S.n, S.vel, S.vel_pred);
	k_copy<<<blocks_for(3*S.n, 256), 256, 0, st>>>(3*(int64_t)S.n, S.ang, S.ang_pred);
	S.launches += 2;
}

void phys_set_dt(DevSim &S, double dt, cudaStream_t st)
{
	k_set_dt<<<1, 1, 0, st>>>(S.clock, dt);
	S.launches++;
}

void phys_sticky_status(const int *status, int *err, cudaStream_t st)
{
	k_sticky<<<1, 1, 0, st>>>(status, err);
}

void phys_merge_pairs(DevSim &S, const DPair *old_pairs, const int *old_row_ptr, int old_n, cudaStream_t st)
{
	k_merge<<<blocks_for(S.n, 128), 128, 0, st>>>(S.npairs, S.n, S.cand_ptr, S.cand, old_pairs, old_row_ptr, old_n, S.pairs);
	S.launches++;
}

void phys_pair_counts(DevSim &S, int *d_out, cudaStream_t st)
{
	LFG_CUDA(cudaMemsetAsync(d_out, 0, 4*sizeof(int), st));
	if (S.npairs)
		k_pair_counts<<<blocks_for(S.npairs, 256), 256, 0, st>>>(S.npairs, S.P.lub_on ? 1 : 0, S.pairs, d_out);
	S.launches++;
}

} // namespace lfg

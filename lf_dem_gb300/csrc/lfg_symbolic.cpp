// lfg_symbolic.cpp -- symbolic analysis for the device multifrontal Cholesky
// that replaces CHOLMOD's cholmod_analyze (LF_DEM/StokesSolver.cpp:950-962).
//
// The matrix is R_FU in 6x6 blocks (one block row/column per particle).  The
// ordering is a nested dissection of the block graph: recursive bisection
// (coordinate cuts at several quantiles when particle positions are given,
// breadth-first level sets otherwise).  With positions, the separator is the
// minimum vertex cover of the cut edges (Koenig's theorem), about a third
// fewer factorisation flops than a one-sided boundary.
// The dissection tree is used directly as the multifrontal assembly tree:
// each separator (and each leaf sub-domain) is one supernode whose columns are
// contiguous in the ordering, and whose front is dense.  The row structure of
// a supernode is the union of its columns' adjacency and its children's row
// structures, restricted to later columns -- every such row belongs to an
// ancestor, so a child's update matrix always fits in its parent's front.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <numeric>
#include <queue>
#include <thread>

#include "lfg_internal.h"

namespace lfg {
namespace {

struct Graph {
	std::vector<int> ptr, adj;
};

Graph build_graph(int n, int nb, const int32_t *r, const int32_t *c)
{
	Graph g;
	std::vector<int> deg(n, 0);
	for (int e = 0; e < nb; e++) {
		if (r[e] == c[e]) continue;
		deg[r[e]]++;
		deg[c[e]]++;
	}
	g.ptr.assign(n+1, 0);
	for (int i = 0; i < n; i++) g.ptr[i+1] = g.ptr[i] + deg[i];
	g.adj.resize(g.ptr[n]);
	std::vector<int> fill(g.ptr.begin(), g.ptr.end()-1);
	for (int e = 0; e < nb; e++) {
		if (r[e] == c[e]) continue;
		g.adj[fill[r[e]]++] = c[e];
		g.adj[fill[c[e]]++] = r[e];
	}
	for (int i = 0; i < n; i++) {
		std::sort(g.adj.begin()+g.ptr[i], g.adj.begin()+g.ptr[i+1]);
		auto end = std::unique(g.adj.begin()+g.ptr[i], g.adj.begin()+g.ptr[i+1]);
		// keep duplicates out of the degree count (pattern lists are unique
		// pairs; this only guards against repeated entries)
		for (auto it = end; it != g.adj.begin()+g.ptr[i+1]; ++it) *it = -1;
	}
	return g;
}

struct TNode {
	std::vector<int> cols;
	std::vector<int> kids;
};

// work arrays of the separator search (one set per thread); side and level
// are indexed by vertex (a candidate cut's labelling and ranks)
struct CoverWork {
	std::vector<int> eptr, eadj, m0, m1, seen, stk, it, via, q, side, level;
	std::vector<char> z0, z1;
	void reserve(int n)
	{
		if ((int)side.size() < n) {
			side.assign(n, 0);
			level.assign(n, -1);
		}
	}
};

// the best cut along one axis
struct AxisCut {
	bool have = false;
	double cost = 0;
	int mid = 0;
	std::vector<int> sep;
	std::vector<std::pair<double,int>> key;   // S sorted along the axis
};

// The two halves of a cut are dissected by separate threads near the top of
// the tree: they touch disjoint vertex sets of side[], level[] and stamp[]
// (stamp[] is also read for the neighbours of a set, hence relaxed atomics),
// and node ids are only labels (the tree and its postorder come from the
// kids lists), so the result does not depend on the thread schedule.
struct Dissector {
	const Graph &g;
	const double *pos;
	bool twod;
	int leaf;
	std::vector<TNode> nodes;
	std::mutex nodes_mu;
	std::unique_ptr<std::atomic<int>[]> stamp;
	std::vector<int> side, level;
	std::atomic<int> cur{0};

	Dissector(const Graph &g_, const double *pos_, bool twod_, int leaf_, int n)
	    : g(g_), pos(pos_), twod(twod_), leaf(leaf_), stamp(new std::atomic<int>[n]), side(n, 0), level(n, -1)
	{
		for (int i = 0; i < n; i++) stamp[i].store(-1, std::memory_order_relaxed);
	}

	bool in(int u, int st) const { return u >= 0 && stamp[u].load(std::memory_order_relaxed) == st; }

	int add_node(TNode &&t)
	{
		std::lock_guard<std::mutex> lk(nodes_mu);
		nodes.push_back(std::move(t));
		return (int)nodes.size()-1;
	}

	// Minimum vertex cover of the cut edges (edges between side 0 and side 1
	// of S), by Koenig's theorem: maximum bipartite matching (augmenting
	// paths), then the alternating-path labelling from the unmatched side-0
	// vertices; cover = (side-0 vertices not reached) + (side-1 vertices
	// reached).  Removing the cover disconnects the two sides.
	std::vector<int> min_cover(int st, const std::vector<int> &b0, const std::vector<int> &b1, CoverWork &w)
	{
		auto &eptr = w.eptr, &eadj = w.eadj, &m0 = w.m0, &m1 = w.m1, &seen = w.seen, &stk = w.stk, &it = w.it;
		auto &via = w.via, &q = w.q, &side = w.side, &level = w.level;
		auto &z0 = w.z0, &z1 = w.z1;
		int n0 = (int)b0.size(), n1 = (int)b1.size();
		for (int t = 0; t < n0; t++) level[b0[t]] = t;
		for (int t = 0; t < n1; t++) level[b1[t]] = t;
		eptr.assign(n0+1, 0);
		eadj.clear();
		for (int t = 0; t < n0; t++) {
			int v = b0[t];
			for (int k = g.ptr[v]; k < g.ptr[v+1]; k++) {
				int u = g.adj[k];
				if (!in(u, st) || side[u] != 1) continue;
				eadj.push_back(level[u]);
			}
			eptr[t+1] = (int)eadj.size();
		}
		m0.assign(n0, -1);
		m1.assign(n1, -1);
		seen.assign(n1, -1);
		// greedy start (each side-0 vertex takes its first free neighbour);
		// augmenting paths then extend it to a maximum matching
		for (int x = 0; x < n0; x++)
			for (int k = eptr[x]; k < eptr[x+1]; k++)
				if (m1[eadj[k]] < 0) {
					m0[x] = eadj[k];
					m1[eadj[k]] = x;
					break;
				}
		// via: side-1 vertex taken at each depth of the search
		for (int r = 0; r < n0; r++) {
			if (m0[r] >= 0) continue;
			// iterative DFS for an augmenting path from r
			stk.assign(1, r);
			it.assign(1, eptr[r]);
			via.clear();
			bool found = false;
			while (!stk.empty() && !found) {
				int x = stk.back();
				int &k = it.back();
				if (k == eptr[x+1]) { stk.pop_back(); it.pop_back(); if (!via.empty()) via.pop_back(); continue; }
				int y = eadj[k++];
				if (seen[y] == r) continue;
				seen[y] = r;
				if (m1[y] < 0) {
					via.push_back(y);
					found = true;
				} else {
					via.push_back(y);
					stk.push_back(m1[y]);
					it.push_back(eptr[m1[y]]);
				}
			}
			if (found) {
				// flip the path: stk[d] matched to via[d]
				for (size_t d = 0; d < stk.size(); d++) {
					m0[stk[d]] = via[d];
					m1[via[d]] = stk[d];
				}
			}
		}
		z0.assign(n0, 0);
		z1.assign(n1, 0);
		q.clear();
		for (int x = 0; x < n0; x++) if (m0[x] < 0) { z0[x] = 1; q.push_back(x); }
		for (size_t h = 0; h < q.size(); h++) {
			int x = q[h];
			for (int k = eptr[x]; k < eptr[x+1]; k++) {
				int y = eadj[k];
				if (z1[y] || m0[x] == y) continue;
				z1[y] = 1;
				int x2 = m1[y];
				if (x2 >= 0 && !z0[x2]) { z0[x2] = 1; q.push_back(x2); }
			}
		}
		std::vector<int> cover;
		for (int x = 0; x < n0; x++) if (!z0[x] && eptr[x+1] > eptr[x]) cover.push_back(b0[x]);
		for (int y = 0; y < n1; y++) if (z1[y]) cover.push_back(b1[y]);
		for (int v : b0) level[v] = -1;
		for (int v : b1) level[v] = -1;
		return cover;
	}

	// coordinate cuts along each axis at several quantiles; the separator is
	// the minimum vertex cover of the cut edges; the cut with the smallest
	// ratio |separator| / (|side 0| |side 1|) wins (the first one, in axis
	// then quantile order, among equals)
	void cut_axis(int ax, const std::vector<int> &S, int st, CoverWork &w, AxisCut &out)
	{
		static const double fracs[] = {0.5, 0.47, 0.53, 0.44, 0.56, 0.41, 0.59, 0.38, 0.62};
		auto &side = w.side, &level = w.level;
		std::vector<int> b0, b1;
		std::vector<std::pair<double,int>> key(S.size());
		// each vertex's rank along the axis and the lowest and highest rank
		// of its neighbours in S: the boundary of a cut at rank mid (side 0 =
		// rank < mid) is read off without walking the adjacency again
		std::vector<int> rk(S.size()), lo(S.size()), hi(S.size());
		for (size_t t = 0; t < S.size(); t++) key[t] = {pos[3*S[t]+ax], S[t]};
		std::sort(key.begin(), key.end());
		for (size_t t = 0; t < S.size(); t++) level[key[t].second] = (int)t;   // rank (scratch)
		for (size_t t = 0; t < S.size(); t++) {
			int v = S[t];
			rk[t] = level[v];
			int a = INT32_MAX, b = -1;
			for (int k = g.ptr[v]; k < g.ptr[v+1]; k++) {
				int u = g.adj[k];
				if (!in(u, st)) continue;
				a = std::min(a, level[u]);
				b = std::max(b, level[u]);
			}
			lo[t] = a;
			hi[t] = b;
		}
		for (int v : S) level[v] = -1;
		for (double f : fracs) {
			int mid = (int)(f*S.size());
			if (mid == 0 || mid >= (int)S.size()) continue;
			for (size_t t = 0; t < S.size(); t++) side[key[t].second] = (int)t < mid ? 0 : 1;
			b0.clear(); b1.clear();
			for (size_t t = 0; t < S.size(); t++) {
				if (rk[t] < mid) { if (hi[t] >= mid) b0.push_back(S[t]); }
				else if (lo[t] < mid) b1.push_back(S[t]);
			}
			std::vector<int> sep = min_cover(st, b0, b1, w);
			double cost = (double)sep.size()/((double)mid*(double)(S.size()-mid));
			if (!out.have || cost < out.cost) {
				out.have = true;
				out.cost = cost;
				out.mid = mid;
				out.sep = std::move(sep);
			}
		}
		if (out.have) out.key = std::move(key);
	}

	std::vector<int> split_geometric(const std::vector<int> &S, int st, CoverWork &w)
	{
		int n = (int)side.size();
		std::vector<int> axes = twod ? std::vector<int>{0, 2} : std::vector<int>{0, 1, 2};
		std::vector<AxisCut> cut(axes.size());
		w.reserve(n);
		if (S.size() >= 1024) {
			// large sets: the axes on separate threads, each with its own
			// labelling and rank arrays
			std::vector<CoverWork> wk(axes.size()-1);
			std::vector<std::exception_ptr> err(axes.size(), nullptr);
			std::vector<std::thread> th;
			for (size_t a = 1; a < axes.size(); a++)
				th.emplace_back([&, a] {
					try {
						wk[a-1].reserve(n);
						cut_axis(axes[a], S, st, wk[a-1], cut[a]);
					} catch (...) {
						err[a] = std::current_exception();
					}
				});
			try {
				cut_axis(axes[0], S, st, w, cut[0]);
			} catch (...) {
				err[0] = std::current_exception();
			}
			for (auto &t : th) t.join();
			for (auto &e : err) if (e) std::rethrow_exception(e);
		} else {
			for (size_t a = 0; a < axes.size(); a++) cut_axis(axes[a], S, st, w, cut[a]);
		}
		int b = -1;
		for (size_t a = 0; a < axes.size(); a++)
			if (cut[a].have && (b < 0 || cut[a].cost < cut[b].cost)) b = (int)a;
		if (b < 0) {   // (sets of one vertex do not reach this)
			for (int v : S) side[v] = 0;
			return {};
		}
		const AxisCut &c = cut[b];
		for (size_t t = 0; t < S.size(); t++) side[c.key[t].second] = (int)t < c.mid ? 0 : 1;
		return c.sep;
	}

	// breadth-first level structure from a pseudo-peripheral vertex; the
	// level holding the median vertex is the separator
	std::vector<int> split_bfs(const std::vector<int> &S, int st)
	{
		auto bfs = [&](int src, std::vector<int> &order) {
			for (int v : S) level[v] = -1;
			order.clear();
			std::queue<int> q;
			q.push(src); level[src] = 0;
			while (!q.empty()) {
				int v = q.front(); q.pop(); order.push_back(v);
				for (int k = g.ptr[v]; k < g.ptr[v+1]; k++) {
					int u = g.adj[k];
					if (!in(u, st) || level[u] >= 0) continue;
					level[u] = level[v]+1;
					q.push(u);
				}
			}
		};
		std::vector<int> order;
		int src = S[0];
		for (int it = 0; it < 3; it++) {
			bfs(src, order);
			src = order.back();
		}
		bfs(src, order);
		if (order.size() < S.size()) {
			// disconnected: reachable part vs the rest, empty separator
			for (int v : S) side[v] = level[v] >= 0 ? 0 : 1;
			return {};
		}
		int lmid = level[order[order.size()/2]];
		std::vector<int> sep;
		for (int v : S) {
			if (level[v] < lmid) side[v] = 0;
			else if (level[v] > lmid) side[v] = 1;
			else { side[v] = 2; sep.push_back(v); }
		}
		return sep;
	}

	std::vector<int> dissect(std::vector<int> S, int depth, CoverWork &w)
	{
		if ((int)S.size() <= leaf) return {add_node(TNode{S, {}})};
		int st = cur++;
		for (int v : S) stamp[v].store(st, std::memory_order_relaxed);
		std::vector<int> sep = pos ? split_geometric(S, st, w) : split_bfs(S, st);
		for (int v : sep) side[v] = 2;
		std::vector<int> L, R;
		for (int v : S) {
			if (side[v] == 0) L.push_back(v);
			else if (side[v] == 1) R.push_back(v);
		}
		std::vector<int> roots;
		if (L.size() == S.size() || R.size() == S.size()) {
			// no progress (should not happen); make a leaf
			return {add_node(TNode{S, {}})};
		}
		std::vector<int> kl, kr;
		if (depth < 4 && L.size() >= 256 && R.size() >= 256) {
			std::exception_ptr err;
			std::thread t([&] {
				try {
					CoverWork wl;
					kl = dissect(L, depth+1, wl);
				} catch (...) {
					err = std::current_exception();
				}
			});
			kr = dissect(R, depth+1, w);
			t.join();
			if (err) std::rethrow_exception(err);
		} else {
			if (!L.empty()) kl = dissect(L, depth+1, w);
			if (!R.empty()) kr = dissect(R, depth+1, w);
		}
		if (sep.empty()) {
			roots = kl;
			roots.insert(roots.end(), kr.begin(), kr.end());
			return roots;
		}
		TNode nd;
		nd.cols = sep;
		nd.kids = kl;
		nd.kids.insert(nd.kids.end(), kr.begin(), kr.end());
		return {add_node(std::move(nd))};
	}
};

} // namespace

void symbolic_analyze(Symbolic &S, int n, int nb, const int32_t *od_row, const int32_t *od_col,
                      const double *pos, double lx, double ly, double lz, int leaf_size, int dof)
{
	(void)lx; (void)lz;
	if (dof != 6 && dof != 3) throw Error{LFG_ERR_BAD_ARG, dof, "degrees of freedom per particle must be 6 or 3"};
	S = Symbolic();
	S.nblk = n;
	S.dof = dof;
	Graph g = build_graph(n, nb, od_row, od_col);
	Dissector D(g, pos, ly == 0, std::max(1, leaf_size), n);
	std::vector<int> all(n);
	std::iota(all.begin(), all.end(), 0);
	CoverWork work;
	std::vector<int> roots = D.dissect(all, 0, work);

	// postorder numbering of tree nodes -> supernodes
	std::vector<int> post;                 // tree node ids in postorder
	std::vector<int> sn_of_node(D.nodes.size(), -1);
	{
		std::vector<std::pair<int,int>> stk;
		for (auto it = roots.rbegin(); it != roots.rend(); ++it) stk.push_back({*it, 0});
		while (!stk.empty()) {
			auto &top = stk.back();
			TNode &t = D.nodes[top.first];
			if (top.second < (int)t.kids.size()) {
				int kid = t.kids[top.second++];
				stk.push_back({kid, 0});
			} else {
				sn_of_node[top.first] = (int)post.size();
				post.push_back(top.first);
				stk.pop_back();
			}
		}
	}
	int nsn = (int)post.size();
	S.nsn = nsn;
	S.perm.resize(n);
	S.iperm.resize(n);
	S.sn_first.resize(nsn); S.sn_n.resize(nsn); S.sn_m.resize(nsn);
	S.sn_parent.assign(nsn, -1); S.sn_level.assign(nsn, 0);
	int k = 0;
	for (int s = 0; s < nsn; s++) {
		TNode &t = D.nodes[post[s]];
		S.sn_first[s] = k;
		S.sn_n[s] = (int)t.cols.size();
		for (int v : t.cols) { S.perm[k] = v; S.iperm[v] = k; k++; }
		for (int kid : t.kids) S.sn_parent[sn_of_node[kid]] = s;
	}
	std::vector<int> colsn(n);
	for (int s = 0; s < nsn; s++)
		for (int q = S.sn_first[s]; q < S.sn_first[s]+S.sn_n[s]; q++) colsn[q] = s;
	// children CSR (in postorder, i.e. increasing supernode id)
	S.child_off.assign(nsn+1, 0);
	for (int s = 0; s < nsn; s++) if (S.sn_parent[s] >= 0) S.child_off[S.sn_parent[s]+1]++;
	for (int s = 0; s < nsn; s++) S.child_off[s+1] += S.child_off[s];
	S.children.resize(S.child_off[nsn]);
	{
		std::vector<int> fill(S.child_off.begin(), S.child_off.end()-1);
		for (int s = 0; s < nsn; s++) if (S.sn_parent[s] >= 0) S.children[fill[S.sn_parent[s]]++] = s;
	}
	// row structures (bottom-up)
	std::vector<std::vector<int>> R(nsn);
	for (int s = 0; s < nsn; s++) {
		int last = S.sn_first[s]+S.sn_n[s]-1;
		std::vector<int> tmp;
		for (int q = S.sn_first[s]; q <= last; q++) {
			int v = S.perm[q];
			for (int e = g.ptr[v]; e < g.ptr[v+1]; e++) {
				int u = g.adj[e];
				if (u < 0) continue;
				int qu = S.iperm[u];
				if (qu > last) tmp.push_back(qu);
			}
		}
		for (int c = S.child_off[s]; c < S.child_off[s+1]; c++)
			for (int r : R[S.children[c]]) if (r > last) tmp.push_back(r);
		std::sort(tmp.begin(), tmp.end());
		tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
		R[s] = std::move(tmp);
		S.sn_m[s] = (int)R[s].size();
		int lev = 0;
		for (int c = S.child_off[s]; c < S.child_off[s+1]; c++)
			lev = std::max(lev, S.sn_level[S.children[c]]+1);
		S.sn_level[s] = lev;
	}
	S.sn_rows_off.resize(nsn+1);
	S.sn_rows_off[0] = 0;
	for (int s = 0; s < nsn; s++) S.sn_rows_off[s+1] = S.sn_rows_off[s]+S.sn_m[s];
	S.rows.resize(S.sn_rows_off[nsn]);
	for (int s = 0; s < nsn; s++)
		std::copy(R[s].begin(), R[s].end(), S.rows.begin()+S.sn_rows_off[s]);
	// front sizes, arena offsets, flops
	S.sn_off.resize(nsn); S.sn_ld.resize(nsn); S.sn_woff.resize(nsn);
	int64_t off = 0, woff = 0;
	S.max_F = 0; S.nnz_L = 0; S.flops = 0;
	for (int s = 0; s < nsn; s++) {
		int n6 = dof*S.sn_n[s], m6 = dof*S.sn_m[s], F6 = n6+m6;
		S.sn_ld[s] = F6+n6;
		S.sn_off[s] = off;
		off += (int64_t)S.sn_ld[s]*F6;
		off = (off+31)/32*32;
		S.sn_woff[s] = woff;
		woff += m6;
		S.max_F = std::max(S.max_F, F6);
		S.nnz_L += (int64_t)n6*(n6+1)/2 + (int64_t)n6*m6;
		double dn = n6, dm = m6;
		S.flops += dn*dn*dn/3 + dn*dn*dm + dn*dm*dm;
	}
	S.arena_elems = off;
	S.w_elems = std::max<int64_t>(woff, 1);
	// inverse maps child -> parent front
	S.cinv_off.assign(nsn+1, 0);
	for (int c = 0; c < nsn; c++) {
		int p = S.sn_parent[c];
		S.cinv_off[c+1] = S.cinv_off[c] + (p >= 0 ? S.sn_n[p]+S.sn_m[p] : 0);
	}
	S.cinv.assign(S.cinv_off[nsn], -1);
	S.cfwd.assign(S.rows.size(), -1);
	auto front_index = [&](int s, int q) -> int {
		int f = S.sn_first[s];
		if (q >= f && q < f+S.sn_n[s]) return q-f;
		const int *b = &S.rows[S.sn_rows_off[s]], *e = b+S.sn_m[s];
		const int *it = std::lower_bound(b, e, q);
		if (it == e || *it != q) return -1;
		return S.sn_n[s]+(int)(it-b);
	};
	for (int c = 0; c < nsn; c++) {
		int p = S.sn_parent[c];
		if (p < 0) continue;
		for (int t = 0; t < S.sn_m[c]; t++) {
			int fi = front_index(p, S.rows[S.sn_rows_off[c]+t]);
			if (fi < 0) throw Error{LFG_ERR_BAD_ARG, 0, "symbolic: child row outside parent front"};
			S.cinv[S.cinv_off[c]+fi] = S.sn_n[c]+t;
			S.cfwd[S.sn_rows_off[c]+t] = fi;
		}
	}
	// levels
	S.nlevels = 0;
	for (int s = 0; s < nsn; s++) S.nlevels = std::max(S.nlevels, S.sn_level[s]+1);
	S.level_off.assign(S.nlevels+1, 0);
	for (int s = 0; s < nsn; s++) S.level_off[S.sn_level[s]+1]++;
	for (int l = 0; l < S.nlevels; l++) S.level_off[l+1] += S.level_off[l];
	S.level_sn.resize(nsn);
	{
		std::vector<int> fill(S.level_off.begin(), S.level_off.end()-1);
		for (int s = 0; s < nsn; s++) S.level_sn[fill[S.sn_level[s]]++] = s;
	}
	// A-block scatter maps
	S.d_sn.resize(n); S.d_bc.resize(n);
	for (int i = 0; i < n; i++) {
		int q = S.iperm[i], s = colsn[q];
		S.d_sn[i] = s;
		S.d_bc[i] = q-S.sn_first[s];
	}
	S.od_sn.resize(nb); S.od_br.resize(nb); S.od_bc.resize(nb); S.od_tr.resize(nb);
	for (int e = 0; e < nb; e++) {
		int qr = S.iperm[od_row[e]], qc = S.iperm[od_col[e]];
		int lo = std::min(qr, qc), hi = std::max(qr, qc);
		int s = colsn[lo];
		S.od_sn[e] = s;
		S.od_bc[e] = lo-S.sn_first[s];
		int fi = front_index(s, hi);
		if (fi < 0) throw Error{LFG_ERR_BAD_ARG, 0, "symbolic: matrix entry outside its front"};
		S.od_br[e] = fi;
		S.od_tr[e] = qr > qc ? 0 : 1;
	}
	S.level_d_off.assign(S.nlevels+1, 0);
	S.level_od_off.assign(S.nlevels+1, 0);
	for (int i = 0; i < n; i++) S.level_d_off[S.sn_level[S.d_sn[i]]+1]++;
	for (int e = 0; e < nb; e++) S.level_od_off[S.sn_level[S.od_sn[e]]+1]++;
	for (int l = 0; l < S.nlevels; l++) {
		S.level_d_off[l+1] += S.level_d_off[l];
		S.level_od_off[l+1] += S.level_od_off[l];
	}
	S.level_d.resize(n); S.level_od.resize(nb);
	{
		std::vector<int> f1(S.level_d_off.begin(), S.level_d_off.end()-1);
		for (int i = 0; i < n; i++) S.level_d[f1[S.sn_level[S.d_sn[i]]]++] = i;
		std::vector<int> f2(S.level_od_off.begin(), S.level_od_off.end()-1);
		for (int e = 0; e < nb; e++) S.level_od[f2[S.sn_level[S.od_sn[e]]]++] = e;
	}
}

// Joint analysis of independent systems: the block-diagonal matrix of all of
// them, whose assembly forest is the union of their trees.  Each part's
// particles, supernodes, rows, fronts, update vectors and off-diagonal blocks
// follow the previous parts'; level l of the forest holds every part's level
// l (levels count from the leaves), so one launch per level and stage serves
// all parts.
void symbolic_concat(Symbolic &J, const std::vector<const Symbolic *> &parts)
{
	J = Symbolic();
	if (parts.empty()) throw Error{LFG_ERR_BAD_ARG, 0, "joint analysis of no system"};
	J.dof = parts[0]->dof;
	for (const Symbolic *P : parts) {
		if (P->dof != J.dof) throw Error{LFG_ERR_BAD_ARG, P->dof, "joint analysis of systems with different dof"};
		J.nlevels = std::max(J.nlevels, P->nlevels);
	}
	int B = 0, SB = 0, RB = 0, CHB = 0, OB = 0;
	int64_t AB = 0, WB = 0, CB = 0;
	for (const Symbolic *P : parts) {
		for (int k = 0; k < P->nblk; k++) {
			J.perm.push_back(B+P->perm[k]);
			J.iperm.push_back(B+P->iperm[k]);
		}
		for (int q = 0; q < P->nsn; q++) {
			J.sn_first.push_back(B+P->sn_first[q]);
			J.sn_n.push_back(P->sn_n[q]);
			J.sn_m.push_back(P->sn_m[q]);
			J.sn_parent.push_back(P->sn_parent[q] >= 0 ? SB+P->sn_parent[q] : -1);
			J.sn_level.push_back(P->sn_level[q]);
			J.sn_rows_off.push_back(RB+P->sn_rows_off[q]);
			J.sn_off.push_back(AB+P->sn_off[q]);
			J.sn_ld.push_back(P->sn_ld[q]);
			J.sn_woff.push_back(WB+P->sn_woff[q]);
			J.child_off.push_back(CHB+P->child_off[q]);
			J.cinv_off.push_back(CB+P->cinv_off[q]);
		}
		for (int r : P->rows) J.rows.push_back(B+r);
		J.cfwd.insert(J.cfwd.end(), P->cfwd.begin(), P->cfwd.end());
		for (int c : P->children) J.children.push_back(SB+c);
		J.cinv.insert(J.cinv.end(), P->cinv.begin(), P->cinv.end());
		for (int i = 0; i < P->nblk; i++) {
			J.d_sn.push_back(SB+P->d_sn[i]);
			J.d_bc.push_back(P->d_bc[i]);
		}
		for (size_t e = 0; e < P->od_sn.size(); e++) {
			J.od_sn.push_back(SB+P->od_sn[e]);
			J.od_br.push_back(P->od_br[e]);
			J.od_bc.push_back(P->od_bc[e]);
			J.od_tr.push_back(P->od_tr[e]);
		}
		J.max_F = std::max(J.max_F, P->max_F);
		J.nnz_L += P->nnz_L;
		J.flops += P->flops;
		B += P->nblk;
		SB += P->nsn;
		RB += (int)P->rows.size();
		CHB += (int)P->children.size();
		OB += (int)P->od_sn.size();
		AB += P->arena_elems;
		WB += P->w_elems;
		CB += P->cinv_off[P->nsn];
	}
	J.nblk = B;
	J.nsn = SB;
	J.sn_rows_off.push_back(RB);
	J.child_off.push_back(CHB);
	J.cinv_off.push_back(CB);
	J.arena_elems = AB;
	J.w_elems = std::max<int64_t>(WB, 1);
	// levels: every part's level l, parts in order
	J.level_off.assign(J.nlevels+1, 0);
	J.level_d_off.assign(J.nlevels+1, 0);
	J.level_od_off.assign(J.nlevels+1, 0);
	for (int l = 0; l < J.nlevels; l++) {
		int sb = 0, b = 0, ob = 0;
		for (const Symbolic *P : parts) {
			if (l < P->nlevels) {
				for (int t = P->level_off[l]; t < P->level_off[l+1]; t++) J.level_sn.push_back(sb+P->level_sn[t]);
				for (int t = P->level_d_off[l]; t < P->level_d_off[l+1]; t++) J.level_d.push_back(b+P->level_d[t]);
				for (int t = P->level_od_off[l]; t < P->level_od_off[l+1]; t++)
					J.level_od.push_back(ob+P->level_od[t]);
			}
			sb += P->nsn;
			b += P->nblk;
			ob += (int)P->od_sn.size();
		}
		J.level_off[l+1] = (int)J.level_sn.size();
		J.level_d_off[l+1] = (int)J.level_d.size();
		J.level_od_off[l+1] = (int)J.level_od.size();
	}
}

// ---------------------------------------------------------------------------
// device mirror + launch plan
// ---------------------------------------------------------------------------
template <typename V> static void up(V *&d, const std::vector<V> &h, cudaStream_t st)
{
	size_t bytes = std::max<size_t>(h.size(), 1)*sizeof(V);
	LFG_CUDA(cudaMalloc((void **)&d, bytes));
	if (!h.empty()) LFG_CUDA(cudaMemcpyAsync(d, h.data(), h.size()*sizeof(V), cudaMemcpyHostToDevice, st));
}

void dev_symbolic_free(DevSymbolic &D)
{
	void *ptrs[] = {D.perm, D.iperm, D.sn_first, D.sn_n, D.sn_m, D.sn_ld, D.sn_rows_off, D.rows,
	                D.sn_off, D.sn_woff, D.child_off, D.children, D.cinv_off, D.cinv, D.cfwd, D.level_sn,
	                D.d_sn, D.d_bc, D.od_sn, D.od_br, D.od_bc, D.od_tr, D.level_d, D.level_od,
	                D.col_tasks, D.panel_tasks, D.tile_tasks, D.diag_tasks};
	for (void *p : ptrs) if (p) cudaFree(p);
	D = DevSymbolic();
}

// Launch kinds of the factor plan (interpreted by factor_numeric).
enum { PLAN_ASSEMBLE = 0, PLAN_SCATTER = 1, PLAN_PANEL = 3, PLAN_UPDATE = 4, PLAN_SYRK = 5, PLAN_DIAG = 6,
       PLAN_SYRK_TC = 8 };

// levels whose largest front has at least this many pivot columns compute the
// Schur complement on the tensor cores: all of them in FP32 (at N = 4096 the
// tensor-core kernel was faster down to 6n = 64 and no slower below); FP64
// uses the CUDA-core kernel.  (The in-front
// update of a panel step has K = 64 only: on the tensor cores its tiles cost
// the same staging and read-modify-write and ran slower, so it stays on the
// CUDA cores.)
constexpr int TC_SYRK_MIN_N6 = 0;

void dev_symbolic_upload(DevSymbolic &D, const Symbolic &S, int nb, int panel_nb, int tile, int syrk_tile,
                         bool tensor_cores, cudaStream_t st)
{
	dev_symbolic_free(D);
	D.nblk = S.nblk; D.nsn = S.nsn; D.nlevels = S.nlevels; D.nb = nb;
	const int dof = S.dof;
	D.dof = dof;
	D.arena_elems = S.arena_elems; D.w_elems = S.w_elems; D.max_F = S.max_F;
	D.flops = S.flops; D.nnz_L = S.nnz_L;
	up(D.perm, S.perm, st); up(D.iperm, S.iperm, st);
	up(D.sn_first, S.sn_first, st); up(D.sn_n, S.sn_n, st); up(D.sn_m, S.sn_m, st);
	up(D.sn_ld, S.sn_ld, st); up(D.sn_rows_off, S.sn_rows_off, st); up(D.rows, S.rows, st);
	up(D.sn_off, S.sn_off, st); up(D.sn_woff, S.sn_woff, st);
	up(D.child_off, S.child_off, st); up(D.children, S.children, st);
	up(D.cinv_off, S.cinv_off, st); up(D.cinv, S.cinv, st); up(D.cfwd, S.cfwd, st);
	up(D.level_sn, S.level_sn, st);
	up(D.d_sn, S.d_sn, st); up(D.d_bc, S.d_bc, st);
	up(D.od_sn, S.od_sn, st); up(D.od_br, S.od_br, st); up(D.od_bc, S.od_bc, st); up(D.od_tr, S.od_tr, st);
	up(D.level_d, S.level_d, st); up(D.level_od, S.level_od, st);
	D.h_level_off = S.level_off;
	D.h_level_d_off = S.level_d_off;
	D.h_level_od_off = S.level_od_off;
	D.max_n6 = 0;
	for (int s = 0; s < S.nsn; s++) D.max_n6 = std::max(D.max_n6, dof*S.sn_n[s]);
	D.h_level_maxn6.assign(S.nlevels, 0);
	D.h_level_maxm6.assign(S.nlevels, 0);
	D.h_level_maxF6.assign(S.nlevels, 0);
	for (int s = 0; s < S.nsn; s++) {
		int l = S.sn_level[s];
		D.h_level_maxn6[l] = std::max(D.h_level_maxn6[l], dof*S.sn_n[s]);
		D.h_level_maxm6[l] = std::max(D.h_level_maxm6[l], dof*S.sn_m[s]);
		D.h_level_maxF6[l] = std::max(D.h_level_maxF6[l], dof*(S.sn_n[s]+S.sn_m[s]));
	}
	// assembly column tasks, panel tasks and update tiles, level by level
	std::vector<int> col_tasks;
	std::vector<int4> panel_tasks, tile_tasks, diag_tasks;
	const int RC = factor_panel_rows();  // rows per panel task
	D.factor_plan.clear();
	for (int l = 0; l < S.nlevels; l++) {
		int64_t c0 = (int64_t)col_tasks.size()/2;
		int kmax = 0;
		for (int t = S.level_off[l]; t < S.level_off[l+1]; t++) {
			int s = S.level_sn[t];
			int F6 = dof*(S.sn_n[s]+S.sn_m[s]);
			for (int c = 0; c < F6; c++) { col_tasks.push_back(s); col_tasks.push_back(c); }
			kmax = std::max(kmax, (dof*S.sn_n[s]+panel_nb-1)/panel_nb);
		}
		D.factor_plan.push_back({PLAN_ASSEMBLE, l, 0, c0, (int)((int64_t)col_tasks.size()/2-c0)});
		// one launch for the level's diagonal and off-diagonal blocks (ranges
		// from h_level_d_off / h_level_od_off)
		D.factor_plan.push_back({PLAN_SCATTER, l, 0, 0,
		                         (S.level_d_off[l+1]-S.level_d_off[l])+(S.level_od_off[l+1]-S.level_od_off[l])});
		// diagonal blocks of panel 0 (later panels' are factored by the update
		// launch of the panel before)
		{
			int64_t d0 = (int64_t)diag_tasks.size();
			for (int t = S.level_off[l]; t < S.level_off[l+1]; t++) {
				int s = S.level_sn[t];
				int n6 = dof*S.sn_n[s];
				if (n6 > 0) diag_tasks.push_back(make_int4(s, 0, 0, std::min(panel_nb, n6)));
			}
			D.factor_plan.push_back({PLAN_DIAG, l, 0, d0, (int)((int64_t)diag_tasks.size()-d0)});
		}
		for (int k = 0; k < kmax; k++) {
			int64_t p0 = (int64_t)panel_tasks.size(), t0i = (int64_t)tile_tasks.size();
			// every front's diagonal tile first: its CTA factors the next
			// panel's diagonal block (the launch's critical path), so it is
			// dispatched in the first wave
			for (int t = S.level_off[l]; t < S.level_off[l+1]; t++) {
				int s = S.level_sn[t];
				int n6 = dof*S.sn_n[s];
				if (n6 <= k*panel_nb) continue;
				int t0 = k*panel_nb+std::min(panel_nb, n6-k*panel_nb);
				if (t0 < n6) tile_tasks.push_back(make_int4(s, t0, t0, k));
			}
			for (int t = S.level_off[l]; t < S.level_off[l+1]; t++) {
				int s = S.level_sn[t];
				int n6 = dof*S.sn_n[s], F6 = n6+dof*S.sn_m[s];
				if (n6 <= k*panel_nb) continue;
				int w = std::min(panel_nb, n6-k*panel_nb);
				int t0 = k*panel_nb+w;
				// panel rows: real [t0, F6), extra [F6, F6+t0)
				for (int r = t0; r < F6; r += RC) panel_tasks.push_back(make_int4(s, r, k, std::min(RC, F6-r)));
				for (int r = F6; r < F6+t0; r += RC) panel_tasks.push_back(make_int4(s, r, k, std::min(RC, F6+t0-r)));
				// trailing tiles of the supernode's own columns (the
				// update-matrix block is one SYRK after the panels)
				for (int r = t0; r < F6; r += tile)
					for (int c = t0; c <= r && c < n6; c += tile)
						if (r != t0 || c != t0) tile_tasks.push_back(make_int4(s, r, c, k));
				for (int r = F6; r < F6+t0; r += tile)
					for (int c = t0; c < n6; c += tile)
						tile_tasks.push_back(make_int4(s, r, c, k));
			}
			D.factor_plan.push_back({PLAN_PANEL, l, k, p0, (int)((int64_t)panel_tasks.size()-p0)});
			D.factor_plan.push_back({PLAN_UPDATE, l, k, t0i, (int)((int64_t)tile_tasks.size()-t0i)});
		}
		// Schur complement U -= L21 L21^T, depth 6n, lower triangle of [6n, 6F)^2
		int64_t s0 = (int64_t)tile_tasks.size();
		for (int t = S.level_off[l]; t < S.level_off[l+1]; t++) {
			int s = S.level_sn[t];
			int n6 = dof*S.sn_n[s], F6 = n6+dof*S.sn_m[s];
			for (int r = n6; r < F6; r += syrk_tile)
				for (int c = n6; c <= r; c += syrk_tile)
					tile_tasks.push_back(make_int4(s, r, c, 0));
		}
		if ((int64_t)tile_tasks.size() > s0)
			D.factor_plan.push_back({tensor_cores && D.h_level_maxn6[l] >= TC_SYRK_MIN_N6 ? PLAN_SYRK_TC : PLAN_SYRK,
			                         l, 0, s0, (int)((int64_t)tile_tasks.size()-s0)});
	}
	up(D.col_tasks, col_tasks, st);
	up(D.panel_tasks, panel_tasks, st);
	up(D.tile_tasks, tile_tasks, st);
	up(D.diag_tasks, diag_tasks, st);
	solve_plan_build(D, st);
}

} // namespace lfg

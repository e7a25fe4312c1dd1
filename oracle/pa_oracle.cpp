// CPU oracle for the batched alignment solve -- TEST INFRASTRUCTURE ONLY.
//
// A plain scalar C++ restatement of the recurrences, tie rules, seeds, traceback walk,
// path compression and all-optimal DFS of pyalign's DP core (pyalign/algorithm/solver.h,
// pyalign 0.4.4).  It checks the CUDA path: only tests/, the smoke check and
// the CPU-baseline leg of bench.py load it.  Nothing in the product links or calls it.
//
// Parity pin: the reference's own known-answer tests (pyalign/tests/*.py) run on this
// oracle through oracle/algorithm.py (tests/golden/make_golden.py); global/local linear,
// affine (max and min), general (log) gap and lane batching are pinned that way.
// Semiglobal, DTW, score-only and the Solution codomain are pinned only by this
// restatement (the reference's tests do not cover them).
//
// Every value is a float32, as in the reference (module.cpp:11-14 instantiates
// Options<float, int16_t/int32_t>); both optimisation directions are implemented natively
// (no negation trick), so the oracle independently checks the GPU path's
// "minimize == -maximize(-x)" rewrite.

#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <cstring>
#include <limits>
#include <memory>
#include <stack>
#include <unordered_set>
#include <vector>

namespace {

constexpr int32_t NO_TB = std::numeric_limits<int32_t>::min();  // solver.h:182-185

struct Pt {
	int32_t u, v;
	bool operator==(const Pt &o) const { return u == o.u && v == o.v; }
};

enum { DIR_MIN = 0, DIR_MAX = 1 };                       // enum.h:13-16
enum { LOC_LOCAL = 0, LOC_GLOBAL = 1, LOC_SEMIGLOBAL = 2 };  // enum.h:28-32
enum { GAP_LINEAR = 0, GAP_AFFINE = 1, GAP_GENERAL = 2 };
enum { TYPE_ALIGNMENT = 0, TYPE_DTW = 1 };
enum { GOAL_SCORE = 0, GOAL_ONE = 1, GOAL_ALL = 2 };     // solver.h:13-39

}  // namespace

extern "C" {

// Options as resolved by the reference's FactoryCreator (factory.h:1036-1241).
typedef struct {
	int32_t type;        // 0 alignment, 1 dtw
	int32_t direction;   // 0 minimize, 1 maximize
	int32_t detail;      // 0 score, 1 alignment, 2 solution
	int32_t count;       // 0 one, 1 all
	int32_t locality;    // 0 local, 1 global, 2 semiglobal
	int32_t remove_dup;  // options.h:21 (= not return_dup)
	int32_t gap_kind;    // 0 linear, 1 affine, 2 general (factory.h:1112-1135)
	float linear_s, linear_t;
	float affine_u_s, affine_v_s, affine_u_t, affine_v_t;  // Gotoh w(k) = u k + v (solver.h:2858-2881)
	const float *general_s;  // cap_s + 1 costs (GapCost.costs(n), factory.h:20-31)
	const float *general_t;  // cap_t + 1 costs
	int32_t cap_s, cap_t;    // solver capacity (create_solver max_len_s/max_len_t)
} pao_options;

}  // extern "C"

namespace {

// T is float (the reference's Value, module.cpp:11-14) or double (the FP64 twin used to
// check float results and gradients).
template <typename T>
struct Dir {
	bool maximize;
	T worst() const {  // solver.h:62-65, 88-91
		return maximize ? -std::numeric_limits<T>::infinity() : std::numeric_limits<T>::infinity();
	}
	bool is_opt(T a, T b) const { return maximize ? (a > b) : (a < b); }  // solver.h:53-56, 79-82
	T opt(T a, T b) const { return is_opt(a, b) ? a : b; }
	T sgn() const { return maximize ? T(-1) : T(1); }  // gap_sgn, solver.h:2807
};

// One traceback cell.  In "one" mode (traceback_1, solver.h:196-278) the list holds at most
// one point and a cleared cell is {NO_TB, NO_TB} with size 0; in "all" mode (traceback_n,
// solver.h:280-374) it is a list that can hold {NO_TB, NO_TB} as a real entry (the local
// zero candidate, solver.h:2006-2011).
struct TB {
	int32_t n = 0;
	Pt p0{NO_TB, NO_TB};
	std::vector<Pt> rest;  // entries 1..n-1 (all-optimal mode only; never allocated otherwise)
	void clear() { n = 0; rest.clear(); }
	void push(Pt p) {
		if (n == 0) p0 = p;
		else rest.push_back(p);
		n++;
	}
	Pt at(int32_t k) const { return k == 0 ? p0 : rest[size_t(k - 1)]; }
	void assign(const TB &o) {
		n = o.n;
		p0 = o.p0;
		if (o.n > 1 || !rest.empty()) rest = o.rest;
	}
	void append(const TB &o) {
		for (int32_t k = 0; k < o.n; k++) push(o.at(k));
	}
};

// A layer of values and traceback cells with the reference's (-1)-shifted indexing.
template <typename T>
struct Layer {
	int32_t ls = 0, lt = 0;
	std::vector<T> val;
	std::vector<TB> tb;
	void init(int32_t s, int32_t t, T fill) {
		ls = s; lt = t;
		val.assign(size_t(s + 1) * size_t(t + 1), fill);
		tb.assign(size_t(s + 1) * size_t(t + 1), TB());
	}
	size_t idx(int32_t i, int32_t j) const { return size_t(i + 1) * size_t(lt + 1) + size_t(j + 1); }
	T &V(int32_t i, int32_t j) { return val[idx(i, j)]; }
	T V(int32_t i, int32_t j) const { return val[idx(i, j)]; }
	TB &Tb(int32_t i, int32_t j) { return tb[idx(i, j)]; }
	const TB &Tb(int32_t i, int32_t j) const { return tb[idx(i, j)]; }
};

// The accumulators of solver.h:1226-1427: the first push initialises, later pushes replace
// only when strictly better (direction::opt_q); in "all" mode, equal values append.
template <typename T>
struct Acc {
	const Dir<T> &dir;
	int goal;
	T &val;
	TB &tb;

	void init(T v, Pt p) {
		val = v;
		if (goal != GOAL_SCORE) {
			tb.clear();
			if (goal == GOAL_ALL || p.u != NO_TB) tb.push(p);
		}
	}
	void init(T v, const TB &t) {
		val = v;
		if (goal != GOAL_SCORE) tb.assign(t);
	}
	void push(T v, Pt p) {
		if (goal == GOAL_SCORE) {
			val = dir.opt(v, val);
			return;
		}
		if (dir.is_opt(v, val)) {
			init(v, p);
		} else if (goal == GOAL_ALL && v == val) {
			tb.push(p);
		}
	}
	void push(T v, const TB &t) {
		if (goal == GOAL_SCORE) {
			val = dir.opt(v, val);
			return;
		}
		if (dir.is_opt(v, val)) {
			init(v, t);
		} else if (goal == GOAL_ALL && v == val) {
			tb.append(t);
		}
	}
};

// xt::linspace<float>(start, stop, n): start + step * i, step = (stop - start) / (n - 1).
// This is the assumed semantics of the xtensor generator used by AffineCost::vector
// (solver.h:2876-2880); it is exact for integer costs.
template <typename T>
std::vector<T> affine_vector(T u, T v, size_t n) {
	std::vector<T> w(n);
	const T stop = T(n - 1) * u;
	const T step = n > 1 ? (stop - T(0)) / T(n - 1) : T(0);
	for (size_t i = 0; i < n; i++) w[i] = (T(0) + step * T(i)) + v;
	if (n > 0) w[0] = 0;
	return w;
}

struct Alignment {
	bool has = false;    // false when the traceback iterator produced nothing
	int32_t ls = 0, lt = 0;
	float score = 0;
	std::vector<int32_t> map;  // s_to_t if ls <= lt else t_to_s (factory.h:149-170)
	std::vector<Pt> path;      // build_path (solver.h:858-938)
};

// path_compressor (solver.h:809-847): emits the previous point when a step changes both
// coordinates and that point is non-negative.
void compress_path(const std::vector<Pt> &path, Alignment &a) {
	a.map.assign(a.ls <= a.lt ? size_t(a.ls) : size_t(a.lt), -1);
	bool empty = true;
	Pt last{0, 0};
	for (const auto &p : path) {
		if (empty) {
			empty = false;
		} else if (p.u != last.u && p.v != last.v) {
			if (last.u >= 0 && last.v >= 0) {
				if (a.ls <= a.lt) a.map[size_t(last.u)] = last.v;
				else a.map[size_t(last.v)] = last.u;
			}
		}
		last = p;
	}
}

std::vector<Pt> compressed_points(const std::vector<Pt> &path) {
	std::vector<Pt> out;
	bool empty = true;
	Pt last{0, 0};
	for (const auto &p : path) {
		if (empty) {
			empty = false;
		} else if (p.u != last.u && p.v != last.v) {
			if (last.u >= 0 && last.v >= 0) out.push_back(last);
		}
		last = p;
	}
	return out;
}

struct PathHash {
	size_t operator()(const std::vector<Pt> &v) const {
		size_t seed = 0;
		for (const auto &p : v) {
			seed ^= std::hash<int32_t>()(p.u) + 0x9e3779b9 + (seed << 6) + (seed >> 2);
			seed ^= std::hash<int32_t>()(p.v) + 0x9e3779b9 + (seed << 6) + (seed >> 2);
		}
		return seed;
	}
};

template <typename T>
struct Problem {
	pao_options o;
	Dir<T> dir;
	int goal;
	int32_t ls, lt;
	std::vector<T> sim;  // ls x lt row-major
	std::vector<T> gen_s, gen_t;
	T lin_s = 0, lin_t = 0, au_s = 0, av_s = 0, au_t = 0, av_t = 0;  // gap costs
	std::vector<Layer<T>> layers;  // D (, P, Q)

	// traceback strategy (solver.h:2094-2124, 2190-2220, 2296-2326)
	bool cont1(int32_t u, int32_t v) const { return u >= 0 && v >= 0; }
	bool cont2(T val) const {
		if (o.type == TYPE_ALIGNMENT && o.locality == LOC_LOCAL) return dir.is_opt(val, T(0));
		return true;
	}
	bool has_trace() const { return goal != GOAL_SCORE; }
	T s(int32_t i, int32_t j) const { return sim[size_t(i) * size_t(lt) + size_t(j)]; }

	// seeds pushed onto a LIFO stack (solver.h:1937-2092, 2174-2188, 2266-2294)
	std::vector<Pt> seeds() const {
		std::vector<Pt> out;
		const Layer<T> &D = layers[0];
		const int loc = o.type == TYPE_DTW ? LOC_GLOBAL : o.locality;
		if (loc == LOC_GLOBAL) {
			out.push_back(Pt{ls - 1, lt - 1});
		} else if (loc == LOC_LOCAL && goal == GOAL_ALL) {
			T best = T(0);
			for (int32_t i = ls - 1; i >= 0; i--)
				for (int32_t j = lt - 1; j >= 0; j--) best = dir.opt(D.V(i, j), best);
			for (int32_t i = ls - 1; i >= 0; i--)
				for (int32_t j = lt - 1; j >= 0; j--) {
					const T x = D.V(i, j);
					if (x == best && dir.is_opt(x, T(0))) out.push_back(Pt{i, j});
				}
		} else {
			// Optima: strict replacement in scan order
			T best = dir.worst();
			Pt bp{0, 0};
			auto add = [&](int32_t i, int32_t j) {
				const T x = D.V(i, j);
				if (dir.is_opt(x, best)) { best = x; bp = Pt{i, j}; }
			};
			if (loc == LOC_LOCAL) {
				for (int32_t i = ls - 1; i >= 0; i--)
					for (int32_t j = lt - 1; j >= 0; j--) add(i, j);
			} else {
				for (int32_t j = 0; j < lt; j++) add(ls - 1, j);
				for (int32_t i = 0; i < ls; i++) add(i, lt - 1);
			}
			if (dir.is_opt(best, dir.worst())) out.push_back(bp);
		}
		return out;
	}

	void build_layers() {
		const bool dtw = o.type == TYPE_DTW;
		const int loc = dtw ? LOC_GLOBAL : o.locality;
		const T sgn = dir.sgn();
		const T worst = dir.worst();
		const int nlayers = (!dtw && o.gap_kind == GAP_AFFINE) ? 3 : 1;
		layers.assign(size_t(nlayers), Layer<T>());
		for (auto &L : layers) L.init(ls, lt, T(0));
		Layer<T> &D = layers[0];

		if (dtw) {  // solver.h:3205-3210
			for (auto &x : D.val) x = worst;
			D.V(-1, -1) = T(0);
		} else if (o.gap_kind == GAP_LINEAR) {  // solver.h:2806-2814
			for (int32_t i = -1; i < ls; i++)
				D.V(i, -1) = loc == LOC_GLOBAL ? (T(i + 1) * lin_s) * sgn : T(0);
			for (int32_t j = -1; j < lt; j++)
				D.V(-1, j) = loc == LOC_GLOBAL ? (T(j + 1) * lin_t) * sgn : T(0);
		} else if (o.gap_kind == GAP_AFFINE) {  // solver.h:2918-2967
			Layer<T> &P = layers[1], &Q = layers[2];
			const auto ws = affine_vector<T>(au_s, av_s, size_t(o.cap_s) + 1);
			const auto wt = affine_vector<T>(au_t, av_t, size_t(o.cap_t) + 1);
			for (int32_t i = -1; i < ls; i++) Q.V(i, -1) = worst;
			for (int32_t j = -1; j < lt; j++) P.V(-1, j) = worst;
			for (int32_t i = -1; i < ls; i++) {
				const T x = loc == LOC_GLOBAL ? ws[size_t(i + 1)] * sgn : T(0);
				D.V(i, -1) = x;
				P.V(i, -1) = x;
			}
			for (int32_t j = -1; j < lt; j++) {
				const T x = loc == LOC_GLOBAL ? wt[size_t(j + 1)] * sgn : T(0);
				D.V(-1, j) = x;
				Q.V(-1, j) = x;
			}
		} else {  // solver.h:3116-3125
			for (int32_t i = -1; i < ls; i++)
				D.V(i, -1) = loc == LOC_GLOBAL ? gen_s[size_t(i + 1)] * sgn : T(0);
			for (int32_t j = -1; j < lt; j++)
				D.V(-1, j) = loc == LOC_GLOBAL ? gen_t[size_t(j + 1)] * sgn : T(0);
		}
	}

	void solve() {
		build_layers();
		const bool dtw = o.type == TYPE_DTW;
		const bool local = !dtw && o.locality == LOC_LOCAL;
		const T sgn = dir.sgn();
		Layer<T> &D = layers[0];

		auto start = [&](T &val, TB &tb) {
			Acc<T> a{dir, goal, val, tb};
			return a;
		};

		for (int32_t u = 0; u < ls; u++) {
			for (int32_t v = 0; v < lt; v++) {
				if (dtw) {  // solver.h:3233-3250
					Acc<T> a = start(D.V(u, v), D.Tb(u, v));
					a.init(D.V(u - 1, v - 1), Pt{u - 1, v - 1});
					a.push(D.V(u - 1, v), Pt{u - 1, v});
					a.push(D.V(u, v - 1), Pt{u, v - 1});
					D.V(u, v) += s(u, v);
				} else if (o.gap_kind == GAP_LINEAR) {  // solver.h:2837-2854
					Acc<T> a = start(D.V(u, v), D.Tb(u, v));
					bool first = true;
					if (local) { a.init(T(0), Pt{NO_TB, NO_TB}); first = false; }
					const T dg = D.V(u - 1, v - 1) + s(u, v);
					if (first) a.init(dg, Pt{u - 1, v - 1}); else a.push(dg, Pt{u - 1, v - 1});
					a.push(D.V(u - 1, v) + lin_s * sgn, Pt{u - 1, v});
					a.push(D.V(u, v - 1) + lin_t * sgn, Pt{u, v - 1});
				} else if (o.gap_kind == GAP_AFFINE) {  // solver.h:2989-3035
					Layer<T> &P = layers[1], &Q = layers[2];
					const T w1s = au_s + av_s;
					const T w1t = au_t + av_t;
					{
						Acc<T> a = start(P.V(u, v), P.Tb(u, v));
						a.init(D.V(u - 1, v) + w1s * sgn, Pt{u - 1, v});
						a.push(P.V(u - 1, v) + au_s * sgn, P.Tb(u - 1, v));
					}
					{
						Acc<T> a = start(Q.V(u, v), Q.Tb(u, v));
						a.init(D.V(u, v - 1) + w1t * sgn, Pt{u, v - 1});
						a.push(Q.V(u, v - 1) + au_t * sgn, Q.Tb(u, v - 1));
					}
					{
						Acc<T> a = start(D.V(u, v), D.Tb(u, v));
						bool first = true;
						if (local) { a.init(T(0), Pt{NO_TB, NO_TB}); first = false; }
						const T dg = D.V(u - 1, v - 1) + s(u, v);
						if (first) a.init(dg, Pt{u - 1, v - 1}); else a.push(dg, Pt{u - 1, v - 1});
						a.push(P.V(u, v), P.Tb(u, v));
						a.push(Q.V(u, v), Q.Tb(u, v));
					}
				} else {  // solver.h:3153-3182
					Acc<T> a = start(D.V(u, v), D.Tb(u, v));
					bool first = true;
					if (local) { a.init(T(0), Pt{NO_TB, NO_TB}); first = false; }
					const T dg = D.V(u - 1, v - 1) + s(u, v);
					if (first) a.init(dg, Pt{u - 1, v - 1}); else a.push(dg, Pt{u - 1, v - 1});
					for (int32_t k = -1; k < u; k++)
						a.push(D.V(k, v) + gen_s[size_t(u - k)] * sgn, Pt{k, v});
					for (int32_t k = -1; k < v; k++)
						a.push(D.V(u, k) + gen_t[size_t(v - k)] * sgn, Pt{u, k});
				}
			}
		}
	}

	// TracebackIterators<false>::Iterator::next (solver.h:1497-1536) for one seed.
	bool walk_one(Pt seed, T &score, std::vector<Pt> &path) const {
		const Layer<T> &D = layers[0];
		int32_t u = seed.u, v = seed.v;
		score = D.V(u, v);
		path.clear();
		if (!has_trace()) return true;
		path.push_back(Pt{u, v});
		while (cont1(u, v) && cont2(D.V(u, v))) {
			const TB &t = D.Tb(u, v);
			const int32_t nu = t.n == 0 ? NO_TB : t.p0.u;
			const int32_t nv = t.n == 0 ? NO_TB : t.p0.v;
			u = nu; v = nv;
			path.push_back(Pt{u, v});
		}
		return true;
	}

	// --- all-optimal DFS state (solver.h:1582-1716) ---
	struct Entry {
		T path_val;
		Pt cur;
		int32_t path_len;
	};
	std::stack<Entry> stk;
	std::vector<Pt> dfs_path;
	std::unordered_set<std::vector<Pt>, PathHash> emitted;
	bool iter_one_done = false;   // for max-degree-1 iterators (TracebackIterators<false>)
	std::vector<Pt> one_seeds;

	void init_iterator() {
		const auto sd = seeds();
		if (goal == GOAL_ALL) {
			for (const auto &p : sd) stk.push(Entry{layers[0].V(p.u, p.v), p, 0});
		} else {
			one_seeds = sd;  // Stack1 keeps only the last pushed seed (solver.h:1429-1449)
			if (one_seeds.size() > 1) one_seeds.erase(one_seeds.begin(), one_seeds.end() - 1);
		}
	}

	bool next(T &score, std::vector<Pt> &path) {
		if (goal != GOAL_ALL) {
			if (one_seeds.empty()) return false;
			const Pt sd = one_seeds.back();
			one_seeds.pop_back();
			walk_one(sd, score, path);
			return true;
		}
		const Layer<T> &D = layers[0];
		while (!stk.empty()) {
			const Entry e = stk.top();
			stk.pop();
			if (e.path_len == 0) dfs_path.clear();
			else dfs_path.resize(size_t(e.path_len));
			dfs_path.push_back(e.cur);
			const int32_t u1 = e.cur.u, v1 = e.cur.v;
			if (cont1(u1, v1) && cont2(D.V(u1, v1))) {
				const TB &t = D.Tb(u1, v1);
				const int32_t psize = int32_t(dfs_path.size());
				if (t.n > 0) {
					for (int32_t q = 0; q < t.n; q++) stk.push(Entry{e.path_val, t.at(q), psize});
				} else {
					stk.push(Entry{e.path_val, Pt{NO_TB, NO_TB}, psize});
				}
			} else {
				if (o.remove_dup) {
					auto cp = compressed_points(dfs_path);
					if (emitted.count(cp)) continue;
					emitted.insert(std::move(cp));
				}
				score = e.path_val;
				path = dfs_path;
				return true;
			}
		}
		return false;
	}
};

}  // namespace

extern "C" {

struct pao_result {
	Problem<float> p;
	// result of the one-shot codomains
	Alignment one;
	float score = 0;
	bool iterator = false;
	// last iterator result
	Alignment cur;
	// solution data: values and traceback of the reported layers
	int32_t sol_layers = 0;
};

// Solve one pair.  `sim` is the ls x lt similarity (or distance) matrix, row-major.
pao_result *pao_solve(const pao_options *o, int32_t ls, int32_t lt, const float *sim) {
	auto *r = new pao_result();
	Problem<float> &p = r->p;
	p.o = *o;
	p.dir = Dir<float>{o->direction == DIR_MAX};
	p.lin_s = o->linear_s;
	p.lin_t = o->linear_t;
	p.au_s = o->affine_u_s;
	p.av_s = o->affine_v_s;
	p.au_t = o->affine_u_t;
	p.av_t = o->affine_v_t;
	if (o->type == TYPE_DTW) p.goal = GOAL_ONE;  // factory.h:1055-1099
	else if (o->count == 1) p.goal = GOAL_ALL;   // factory.h:1219-1233
	else p.goal = o->detail == 0 ? GOAL_SCORE : GOAL_ONE;  // factory.h:1198-1216
	p.ls = ls;
	p.lt = lt;
	p.sim.assign(sim, sim + size_t(ls) * size_t(lt));
	if (o->type == TYPE_ALIGNMENT && o->gap_kind == GAP_GENERAL) {
		p.gen_s.assign(o->general_s, o->general_s + o->cap_s + 1);
		p.gen_t.assign(o->general_t, o->general_t + o->cap_t + 1);
	}
	p.solve();
	p.init_iterator();
	return r;
}

void pao_free(pao_result *r) { delete r; }

int32_t pao_goal(const pao_result *r) { return r->p.goal; }
int32_t pao_layer_count(const pao_result *r) { return int32_t(r->p.layers.size()); }

// Advance the traceback iterator of this pair.  Returns 1 and fills score, the alignment
// map (min(ls, lt) entries) and the full path (path_len points, up to ls + lt + 2) when a
// result exists, 0 when exhausted.  For Score/Alignment/Solution (count ONE) this is the
// single next() of Solver::score/alignment/solution (solver.h:2593-2705).
int32_t pao_next(pao_result *r, float *score, int32_t *map, int32_t *path, int32_t *path_len) {
	float sc = 0;
	std::vector<Pt> pth;
	if (!r->p.next(sc, pth)) return 0;
	Alignment a;
	a.ls = r->p.ls;
	a.lt = r->p.lt;
	compress_path(pth, a);
	*score = sc;
	if (map) std::memcpy(map, a.map.data(), a.map.size() * sizeof(int32_t));
	if (path) {
		for (size_t k = 0; k < pth.size(); k++) { path[2 * k] = pth[k].u; path[2 * k + 1] = pth[k].v; }
	}
	if (path_len) *path_len = int32_t(pth.size());
	return 1;
}

float pao_worst(const pao_result *r) { return r->p.dir.worst(); }

// Values of layer k, (ls+1) x (lt+1) row-major, including the border row/column.
void pao_values(const pao_result *r, int32_t k, float *out) {
	const auto &L = r->p.layers[size_t(k)];
	std::memcpy(out, L.val.data(), L.val.size() * sizeof(float));
}

// First traceback entry per cell of layer k ((ls+1) x (lt+1) x 2), NO_TB where empty
// (solver.h:2413-2431).
void pao_tb_matrix(const pao_result *r, int32_t k, int32_t *out) {
	const auto &L = r->p.layers[size_t(k)];
	for (size_t c = 0; c < L.tb.size(); c++) {
		const auto &t = L.tb[c];
		out[2 * c] = t.n == 0 ? NO_TB : t.p0.u;
		out[2 * c + 1] = t.n == 0 ? NO_TB : t.p0.v;
	}
}

// All traceback entries of layer k as (n, 2, 2) edges ((i-1, j-1) -> (u, v)), in the
// order of solver.h:2445-2479.  Call with out == nullptr to get n.
int64_t pao_tb_edges(const pao_result *r, int32_t k, int32_t *out) {
	const auto &L = r->p.layers[size_t(k)];
	int64_t n = 0;
	for (int32_t i = 0; i <= L.ls; i++) {
		for (int32_t j = 0; j <= L.lt; j++) {
			const auto &t = L.tb[size_t(i) * size_t(L.lt + 1) + size_t(j)];
			for (int32_t q = 0; q < t.n; q++) {
				const Pt p = t.at(q);
				if (out) {
					out[4 * n + 0] = i - 1;
					out[4 * n + 1] = j - 1;
					out[4 * n + 2] = p.u;
					out[4 * n + 3] = p.v;
				}
				n++;
			}
		}
	}
	return n;
}

}  // extern "C"

extern "C" {

// Timed CPU baseline: solves `npairs` problems of the indexed form (codes a/b, a similarity
// table A x A) on `nthreads` threads, each pair like one lane of Solver::alignment
// (solver.h:2610-2630): DP with traceback, seed, walk, alignment map.  Returns the cell
// count; writes scores and maps (concatenated at map_off).
int64_t pao_batch_alignments(const pao_options *o, int32_t npairs, const int32_t *ls, const int32_t *lt,
                             const uint32_t *a, int64_t a_stride, const uint32_t *b, int64_t b_stride,
                             const float *table, int32_t A, int32_t nthreads, float *scores, int32_t *maps,
                             const int64_t *map_off) {
	std::atomic<int32_t> next{0};
	auto work = [&]() {
		std::vector<float> sim;
		for (;;) {
			const int32_t k = next.fetch_add(1);
			if (k >= npairs) break;
			const int32_t s_len = ls[k], t_len = lt[k];
			sim.assign(size_t(s_len) * size_t(t_len), 0.0f);
			for (int32_t i = 0; i < s_len; i++) {
				const uint32_t x = a[int64_t(k) * a_stride + i];
				for (int32_t j = 0; j < t_len; j++)
					sim[size_t(i) * size_t(t_len) + size_t(j)] = table[size_t(x) * size_t(A) + b[int64_t(k) * b_stride + j]];
			}
			pao_result *r = pao_solve(o, s_len, t_len, sim.data());
			float sc = 0;
			if (!pao_next(r, &sc, maps ? maps + map_off[k] : nullptr, nullptr, nullptr)) sc = pao_worst(r);
			scores[k] = sc;
			pao_free(r);
		}
	};
	std::vector<std::thread> th;
	for (int32_t t = 0; t < std::max(1, nthreads); t++) th.emplace_back(work);
	for (auto &t : th) t.join();
	int64_t cells = 0;
	for (int32_t k = 0; k < npairs; k++) cells += int64_t(ls[k]) * lt[k];
	return cells;
}

}  // extern "C"

extern "C" {

// FP64 twin of pao_solve + pao_next for one pair (the same recurrences with every value a
// double): gaps = {linear_s, linear_t, affine_u_s, affine_v_s, affine_u_t, affine_v_t} in
// double, general costs (cap + 1 entries) in double when o->gap_kind is general.  Returns
// 1 and fills the score and the one-optimal path (path_len points) when a result exists.
int32_t pao_solve_f64(const pao_options *o, const double *gaps, const double *gen_s, const double *gen_t,
                      int32_t ls, int32_t lt, const double *sim, double *score, int32_t *path, int32_t *path_len) {
	Problem<double> p;
	p.o = *o;
	p.dir = Dir<double>{o->direction == DIR_MAX};
	if (o->type == TYPE_DTW) p.goal = GOAL_ONE;
	else if (o->count == 1) p.goal = GOAL_ALL;
	else p.goal = o->detail == 0 ? GOAL_SCORE : GOAL_ONE;
	p.ls = ls;
	p.lt = lt;
	p.lin_s = gaps[0];
	p.lin_t = gaps[1];
	p.au_s = gaps[2];
	p.av_s = gaps[3];
	p.au_t = gaps[4];
	p.av_t = gaps[5];
	p.sim.assign(sim, sim + size_t(ls) * size_t(lt));
	if (o->type == TYPE_ALIGNMENT && o->gap_kind == GAP_GENERAL) {
		p.gen_s.assign(gen_s, gen_s + o->cap_s + 1);
		p.gen_t.assign(gen_t, gen_t + o->cap_t + 1);
	}
	p.solve();
	p.init_iterator();
	double sc = 0;
	std::vector<Pt> pth;
	if (!p.next(sc, pth)) return 0;
	*score = sc;
	if (path)
		for (size_t k = 0; k < pth.size(); k++) { path[2 * k] = pth[k].u; path[2 * k + 1] = pth[k].v; }
	if (path_len) *path_len = int32_t(pth.size());
	return 1;
}

}  // extern "C"

namespace {

// Score only, two rows per layer: the recurrences of LinearGapCostSolver::solve
// (solver.h:2825-2855) and AffineGapCostSolver::solve (solver.h:2970-3036) with the same
// float operations in the same order as Problem::solve above, the borders of build_layers
// (solver.h:2806-2814, 2918-2967), and the score of Solver::score (solver.h:2593-2608): the
// value at the seed -- global (ls-1, lt-1) (solver.h:2174-2188), semiglobal the optimum of
// the last row then the last column (solver.h:2266-2294), local the optimum over every cell
// (solver.h:2035-2056; only the value matters for a score, not which tied cell holds it).
// Memory is O(lt), so pairs of 5000 x 10000 cells fit; pairs with an empty side go through
// the full solver.
float score_lean(const pao_options &o, int32_t ls, int32_t lt, const uint32_t *a, const uint32_t *b,
                 const float *table, int32_t A) {
	typedef float T;
	const Dir<T> dir{o.direction == DIR_MAX};
	const T sgn = dir.sgn();
	const T worst = dir.worst();
	const bool local = o.locality == LOC_LOCAL, global = o.locality == LOC_GLOBAL;
	const bool affine = o.gap_kind == GAP_AFFINE;
	std::vector<T> ws, wt;
	if (affine) {
		ws = affine_vector<T>(o.affine_u_s, o.affine_v_s, size_t(o.cap_s) + 1);
		wt = affine_vector<T>(o.affine_u_t, o.affine_v_t, size_t(o.cap_t) + 1);
	}
	const T w1s = T(o.affine_u_s) + T(o.affine_v_s), w1t = T(o.affine_u_t) + T(o.affine_v_t);
	// row u - 1 and row u of D and P, index j + 1 (column -1 at index 0)
	std::vector<T> Dp(size_t(lt) + 1), Dc(size_t(lt) + 1), Pp(size_t(lt) + 1), Pc(size_t(lt) + 1);
	for (int32_t j = -1; j < lt; j++) {
		T x;
		if (affine) x = global ? wt[size_t(j + 1)] * sgn : T(0);
		else x = global ? (T(j + 1) * o.linear_t) * sgn : T(0);
		Dp[size_t(j + 1)] = x;
		Pp[size_t(j + 1)] = worst;  // P(-1, j)
	}
	T best = worst;  // local: optimum over all cells; semiglobal: over the last column
	std::vector<T> last_row;
	for (int32_t u = 0; u < ls; u++) {
		T left;
		if (affine) left = global ? ws[size_t(u + 1)] * sgn : T(0);
		else left = global ? (T(u + 1) * o.linear_s) * sgn : T(0);
		Dc[0] = left;
		Pc[0] = left;     // P(u, -1) = D(u, -1)
		T Q = worst;      // Q(u, -1)
		const float *trow = table + size_t(a[u]) * size_t(A);
		for (int32_t v = 0; v < lt; v++) {
			const T s = trow[b[v]];
			T d;
			if (affine) {
				T P = Dp[size_t(v + 1)] + w1s * sgn;
				P = dir.opt(Pp[size_t(v + 1)] + T(o.affine_u_s) * sgn, P);
				T Qn = Dc[size_t(v)] + w1t * sgn;
				Qn = dir.opt(Q + T(o.affine_u_t) * sgn, Qn);
				Q = Qn;
				Pc[size_t(v + 1)] = P;
				const T dg = Dp[size_t(v)] + s;
				d = local ? dir.opt(dg, T(0)) : dg;
				d = dir.opt(P, d);
				d = dir.opt(Q, d);
			} else {
				const T dg = Dp[size_t(v)] + s;
				d = local ? dir.opt(dg, T(0)) : dg;
				d = dir.opt(Dp[size_t(v + 1)] + T(o.linear_s) * sgn, d);
				d = dir.opt(Dc[size_t(v)] + T(o.linear_t) * sgn, d);
			}
			Dc[size_t(v + 1)] = d;
			if (local) best = dir.opt(d, best);
		}
		if (o.locality == LOC_SEMIGLOBAL) best = dir.opt(Dc[size_t(lt)], best);
		std::swap(Dp, Dc);
		std::swap(Pp, Pc);
	}
	// Dp now holds row ls - 1
	if (global) return Dp[size_t(lt)];
	if (o.locality == LOC_SEMIGLOBAL) {
		// last row first (j ascending), then the last column: the optimum's value is the same
		// whichever cell of a tie the scan keeps
		T r = worst;
		for (int32_t j = 0; j < lt; j++) r = dir.opt(Dp[size_t(j + 1)], r);
		return dir.opt(best, r);
	}
	return best;
}

}  // namespace

extern "C" {

// Scores of `npairs` problems of the indexed form on `nthreads` threads with the memory-lean
// score_lean above (linear or affine gaps, any locality, either direction, alignment type).
// Pairs with an empty side are solved by the full solver.  Returns the cell count.
int64_t pao_batch_scores_lean(const pao_options *o, int32_t npairs, const int32_t *ls, const int32_t *lt,
                              const uint32_t *a, int64_t a_stride, const uint32_t *b, int64_t b_stride,
                              const float *table, int32_t A, int32_t nthreads, float *scores) {
	std::atomic<int32_t> next{0};
	auto work = [&]() {
		for (;;) {
			const int32_t k = next.fetch_add(1);
			if (k >= npairs) break;
			const uint32_t *ak = a + int64_t(k) * a_stride, *bk = b + int64_t(k) * b_stride;
			if (ls[k] > 0 && lt[k] > 0 && o->gap_kind != GAP_GENERAL && o->type == TYPE_ALIGNMENT) {
				scores[k] = score_lean(*o, ls[k], lt[k], ak, bk, table, A);
				continue;
			}
			std::vector<float> sim(static_cast<size_t>(ls[k]) * static_cast<size_t>(lt[k]));
			for (int32_t i = 0; i < ls[k]; i++)
				for (int32_t j = 0; j < lt[k]; j++) sim[size_t(i) * size_t(lt[k]) + size_t(j)] = table[size_t(ak[i]) * size_t(A) + bk[j]];
			pao_result *r = pao_solve(o, ls[k], lt[k], sim.data());
			float sc = 0;
			if (!pao_next(r, &sc, nullptr, nullptr, nullptr)) sc = pao_worst(r);
			scores[k] = sc;
			pao_free(r);
		}
	};
	std::vector<std::thread> th;
	for (int32_t t = 0; t < std::max(1, nthreads); t++) th.emplace_back(work);
	for (auto &t : th) t.join();
	int64_t cells = 0;
	for (int32_t k = 0; k < npairs; k++) cells += int64_t(ls[k]) * lt[k];
	return cells;
}

}  // extern "C"

extern "C" {

// FP64 twin on a batch of float32 similarity (or distance) matrices, `nthreads` host
// threads: pair k reads S + k * pair_stride, row i at + i * row_stride, converted to double.
// Writes the FP64 score of each pair and the magnitude of the terms it sums along its
// optimal path -- sum |S| over the cells the score adds (aligned cells; every visited cell
// for DTW) plus |score - sum S| (the gap costs) -- the denominator for scores near zero.
void pao_batch_f64(const pao_options *o, const double *gaps, int32_t npairs, const int32_t *ls, const int32_t *lt,
                   const float *S, int64_t pair_stride, int64_t row_stride, int32_t nthreads, double *scores,
                   double *scales) {
	std::atomic<int32_t> next{0};
	auto work = [&]() {
		std::vector<double> sim;
		std::vector<int32_t> path;
		for (;;) {
			const int32_t k = next.fetch_add(1);
			if (k >= npairs) break;
			const int32_t n_s = ls[k], n_t = lt[k];
			sim.resize(size_t(n_s) * size_t(n_t));
			const float *Sk = S + int64_t(k) * pair_stride;
			for (int32_t i = 0; i < n_s; i++)
				for (int32_t j = 0; j < n_t; j++) sim[size_t(i) * size_t(n_t) + size_t(j)] = double(Sk[int64_t(i) * row_stride + j]);
			path.assign(2 * (size_t(n_s) + size_t(n_t) + 4), 0);
			double sc = 0;
			int32_t np = 0;
			if (!pao_solve_f64(o, gaps, nullptr, nullptr, n_s, n_t, sim.data(), &sc, path.data(), &np)) {
				scores[k] = std::nan("");
				scales[k] = std::nan("");
				continue;
			}
			double tot = 0, mag = 0;
			for (int32_t q = 0; q + 1 < np; q++) {
				const int32_t u0 = path[2 * q], v0 = path[2 * q + 1], u1 = path[2 * q + 2], v1 = path[2 * q + 3];
				if (u0 < 0 || v0 < 0) break;
				if (o->type == TYPE_DTW || (u1 == u0 - 1 && v1 == v0 - 1)) {
					const double x = sim[size_t(u0) * size_t(n_t) + size_t(v0)];
					tot += x;
					mag += std::fabs(x);
				}
			}
			scores[k] = sc;
			scales[k] = mag + std::fabs(tot - sc);
		}
	};
	std::vector<std::thread> th;
	for (int32_t t = 0; t < std::max(1, nthreads); t++) th.emplace_back(work);
	for (auto &t : th) t.join();
}

}  // extern "C"

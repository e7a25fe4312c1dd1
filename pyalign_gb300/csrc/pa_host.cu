// Host runtime and C ABI of the GB300 alignment solve (include/pyalign_gb300.h).
//
// One pa_solver per reference Solver (factory.h:682-973): it owns the options, the border
// vectors of its capacity (computed exactly as the reference's constructors do), a CUDA
// stream and a set of growable device buffers.  A solve call uploads one batch, runs the
// DP kernels and the traceback kernel on the stream, downloads the results and wraps
// them in a pa_result that outlives later calls.  There is no CPU fallback: without a
// device every solve fails with PA_ERR_NO_DEVICE.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <stack>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pyalign_gb300.h"
#include "pa_dp.cuh"
#include "pa_enum.h"
#include "pa_launch.h"
#include "pa_wsb.h"

using namespace pa;

namespace {

thread_local std::string g_err;

pa_status fail(pa_status st, const std::string &msg) {
	g_err = msg;
	return st;
}

#define PA_CUDA(call)                                                                       \
	do {                                                                                    \
		cudaError_t e_ = (call);                                                            \
		if (e_ != cudaSuccess)                                                              \
			return fail(PA_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e_) + \
			                             " at " #call);                                     \
	} while (0)

constexpr int32_t NO_TB = INT32_MIN;

struct DevBuf {
	void *p = nullptr;
	size_t cap = 0;
	~DevBuf() {
		if (p) cudaFree(p);
	}
	cudaError_t ensure(size_t n) {
		if (n <= cap && p) return cudaSuccess;
		if (p) cudaFree(p);
		p = nullptr;
		cap = 0;
		const size_t want = std::max<size_t>(n + n / 4, 256);
		cudaError_t e = cudaMalloc(&p, want);
		if (e == cudaSuccess) cap = want;
		return e;
	}
	template <typename T>
	T *as() const { return reinterpret_cast<T *>(p); }
};

struct PinBuf {
	void *p = nullptr;
	size_t cap = 0;
	~PinBuf() {
		if (p) cudaFreeHost(p);
	}
	cudaError_t ensure(size_t n) {
		if (n <= cap && p) return cudaSuccess;
		if (p) cudaFreeHost(p);
		p = nullptr;
		cap = 0;
		const size_t want = std::max<size_t>(n + n / 4, 256);
		cudaError_t e = cudaMallocHost(&p, want);
		if (e == cudaSuccess) cap = want;
		return e;
	}
	template <typename T>
	T *as() const { return reinterpret_cast<T *>(p); }
};

// Goals of solver.h:13-39 as selected by FactoryCreator (factory.h:1195-1240).
enum Goal { GOAL_SCORE = 0, GOAL_ONE = 1, GOAL_ALL = 2 };
// Output shapes of the 15 solve methods (factory.h:699-808).
enum Method { M_SCORE = 0, M_ALIGNMENT = 1, M_ALIGNMENT_ITER = 2, M_SOLUTION = 3, M_SOLUTION_ITER = 4, M_PATHS = 5 };
enum Form { F_DENSE = 0, F_INDEXED = 1, F_BINARY = 2, F_SERIES = 3 };  // F_SERIES: S = |x_i - y_j| of two series

struct Input {
	int form;
	int location;  // where a/b/sim/table live
	int64_t batch, n_s, n_t;
	const uint32_t *a, *b;
	const float *sim;
	const float *table;
	int64_t table_rows, table_cols;
	float eq, ne;
	const int32_t *length;  // host (2, batch)
	// dense form with explicit layout: S(k, i, j) = sim[dense_off[k] + i * dense_si + j * dense_sj]
	const int64_t *dense_off_host = nullptr;
	int64_t dense_si = 0, dense_sj = 0;
	// series form: S(k, i, j) = |x[k * x_stride + i] - y[k * y_stride + j]| (device)
	const float *sx = nullptr, *sy = nullptr;
	int64_t sx_stride = 0, sy_stride = 0;
};

// Device buffers of the caller that receive the one-optimal paths (M_PATHS).
struct UserPaths {
	int32_t *paths = nullptr;          // 2 ints per point, |s| + |t| + 2 points per pair
	const int64_t *path_off = nullptr;  // host, in ints
	int32_t *path_len = nullptr;
	float *scores = nullptr;
};

// xt::linspace<float>(0, (n-1)*u, n) + v with w[0] = 0 -- AffineCost::vector
// (solver.h:2876-2880), assuming the generator start + step * i, step = (stop - start)/(n-1).
std::vector<float> affine_vector(float u, float v, size_t n) {
	std::vector<float> w(n);
	const float stop = float(n - 1) * u;
	const float step = n > 1 ? (stop - 0.0f) / float(n - 1) : 0.0f;
	for (size_t i = 0; i < n; i++) w[i] = (0.0f + step * float(i)) + v;
	if (n) w[0] = 0.0f;
	return w;
}

bool integral(float x) { return std::isfinite(x) && std::nearbyint(x) == x; }

}  // namespace

// ---------------------------------------------------------------------------------------
// Results

struct ResultData {
	int64_t batch = 0;
	std::vector<int32_t> ls, lt;
	int goal = GOAL_ONE, gap = GAP_LINEAR, loc = LOC_GLOBAL, type = PA_TYPE_ALIGNMENT;
	int remove_dup = 1;
	int layers = 1;
	int method = 0;
	float sign = 1.0f;
	int G = 32;
	float worst = -INFINITY;
	std::vector<float> scores;
	std::vector<int32_t> has;     // has_alignment per lane
	std::vector<int32_t> seeds;   // 2 per lane
	std::vector<int64_t> map_off;
	std::vector<int32_t> maps;
	bool maps_external = false;  // the maps went to the caller's buffer (pa_solve_batch_result)
	std::vector<int64_t> path_off;
	std::vector<int32_t> paths, path_len;
	std::vector<int64_t> mask_off;
	std::vector<uint32_t> masks_one;  // TB_ONE words (solutions)
	bool matrices = false;  // the cell matrices (masks or general-gap codes) are readable
	// TB_ALL: 4 words per lane-step, left on the device (the result owns the buffer) and
	// read by the host DFS in 64 KB chunks on demand: the DFS touches the cells near the
	// optimal paths only, a few MB of masks that can be 16 bytes per cell in total
	void *dev_masks_all = nullptr;
	int64_t dev_masks_words = 0;
	static constexpr int64_t CHUNK = 16384;  // words per chunk
	mutable std::unordered_map<int64_t, std::vector<uint32_t>> mchunks;
	mutable int64_t mchunk_bytes = 0;
	ResultData() = default;
	ResultData(const ResultData &) = delete;  // owns dev_masks_all
	ResultData &operator=(const ResultData &) = delete;
	~ResultData() {
		if (dev_masks_all) cudaFree(dev_masks_all);
	}
	uint32_t mask_word(int64_t w) const {
		const int64_t c = w / CHUNK;
		auto it = mchunks.find(c);
		if (it == mchunks.end()) {
			if (mchunk_bytes > (int64_t(256) << 20)) {  // bound the cache
				mchunks.clear();
				mchunk_bytes = 0;
			}
			const int64_t n = std::min(CHUNK, dev_masks_words - c * CHUNK);
			std::vector<uint32_t> buf(size_t(std::max<int64_t>(n, 1)), 0u);
			if (n > 0 &&
			    cudaMemcpy(buf.data(), static_cast<const uint32_t *>(dev_masks_all) + c * CHUNK, size_t(n) * 4,
			               cudaMemcpyDeviceToHost) != cudaSuccess)
				std::fill(buf.begin(), buf.end(), 0u);
			mchunk_bytes += n * 4;
			it = mchunks.emplace(c, std::move(buf)).first;
		}
		return it->second[size_t(w - c * CHUNK)];
	}
	std::vector<int64_t> val_off;
	std::vector<float> values;
	mutable std::vector<uint64_t> path_counts;  // all-optimal: co-optimal path count per lane, once computed
	// general (WSB) gap: traceback codes and values per lane
	std::vector<int64_t> wsb_off;
	std::vector<int32_t> wsb_tb;
	std::vector<float> wsb_vals;
	std::vector<float> gen_s, gen_t;  // normalised gap costs for all-optimal WSB ties
	bool has_algorithm = true;
	std::string alg[3];

	// ---- mask access
	uint32_t nib(int64_t lane, int i, int j) const {
		const int rpp = G * R;
		const int q = i / rpp, rem = i - q * rpp, sb = rem / R, r = rem - sb * R;
		const int64_t S = lt[lane] + G - 1;
		const uint32_t w = masks_one[size_t(mask_off[lane] + (int64_t(q) * S + (j + sb)) * G + sb)];
		// row r's nibble: D source code | P-extend << 2 | Q-extend << 3, at bits 4(R-1-r)
		return (w >> (4 * (R - 1 - r))) & 15u;
	}
	uint32_t cell(int64_t lane, int i, int j) const {
		const int rpp = G * R;
		const int q = i / rpp, rem = i - q * rpp, sb = rem / R, r = rem - sb * R;
		const int64_t S = lt[lane] + G - 1;
		const size_t e = size_t(mask_off[lane] + (int64_t(q) * S + (j + sb)) * G + sb);
		const uint32_t w = mask_word(int64_t(4 * e) + (r >> 1));
		return (w >> (16 * (r & 1))) & 0xffffu;
	}
	// WSB one-optimal traceback code of D(i, j): kind (0 none, 1 diag, 2 vertical k, 3 horizontal k)
	int32_t wsb(int64_t lane, int i, int j) const {
		return wsb_tb[size_t(wsb_off[lane] + int64_t(i) * lt[lane] + j)];
	}
	float wsb_val(int64_t lane, int i, int j) const {  // normalised D(i, j), i, j >= -1
		return wsb_vals[size_t(wsb_voff[lane] + int64_t(i + 1) * (lt[lane] + 1) + (j + 1))];
	}
	std::vector<int64_t> wsb_voff;

	// traceback list of D(i, j) in push order (solver.h:1328-1369): all-optimal masks
	void tb_list_all(int64_t lane, int i, int j, std::vector<std::pair<int, int>> &out, int layer = 0) const {
		out.clear();
		if (gap == GAP_GENERAL) {
			wsb_list(lane, i, j, out);
			return;
		}
		const uint32_t c0 = cell(lane, i, j);
		// layer 1 (P) / 2 (Q): only that gap's own list (solver.h:2995-3016)
		const uint32_t c = layer == 0 ? c0 : (layer == 1 ? 4u : 8u);
		if (c & 1u) out.push_back({NO_TB, NO_TB});
		if (c & 2u) out.push_back({i - 1, j - 1});
		if (c & 4u) {
			if (gap == GAP_AFFINE) {
				for (int k = i;; k--) {
					const uint32_t ck = cell(lane, k, j);
					if (ck & 16u) out.push_back({k - 1, j});
					if ((ck & 32u) && k > 0) continue;
					break;
				}
			} else {
				out.push_back({i - 1, j});
			}
		}
		if (c & 8u) {
			if (gap == GAP_AFFINE) {
				for (int k = j;; k--) {
					const uint32_t ck = cell(lane, i, k);
					if (ck & 64u) out.push_back({i, k - 1});
					if ((ck & 128u) && k > 0) continue;
					break;
				}
			} else {
				out.push_back({i, j - 1});
			}
		}
	}
	// WSB ties recomputed from the device values with the reference's float operations
	// (solver.h:3157-3180)
	void wsb_list(int64_t lane, int i, int j, std::vector<std::pair<int, int>> &out) const {
		const float d = wsb_val(lane, i, j);
		const bool local = loc == LOC_LOCAL;
		if (local && d == 0.0f) out.push_back({NO_TB, NO_TB});
		const float dg = wsb_val(lane, i - 1, j - 1) + wsb_diag(lane, i, j);
		if (dg == d) out.push_back({i - 1, j - 1});
		for (int k = -1; k < i; k++)
			if (wsb_val(lane, k, j) + (-gen_s[size_t(i - k)]) == d) out.push_back({k, j});
		for (int k = -1; k < j; k++)
			if (wsb_val(lane, i, k) + (-gen_t[size_t(j - k)]) == d) out.push_back({i, k});
	}
	std::vector<float> wsb_sub;  // normalised similarity per lane cell (all-optimal WSB)
	std::vector<int64_t> wsb_sub_off;
	float wsb_diag(int64_t lane, int i, int j) const {
		return wsb_sub[size_t(wsb_sub_off[lane] + int64_t(i) * lt[lane] + j)];
	}

	bool cont2_all(int64_t lane, int i, int j) const {
		if (loc != LOC_LOCAL) return true;
		if (gap == GAP_GENERAL) return wsb_val(lane, i, j) > 0.0f;
		return !(cell(lane, i, j) & 1u);
	}
};

struct pa_result {
	std::shared_ptr<ResultData> d;
};

struct pa_iterator {
	std::shared_ptr<ResultData> d;
	int64_t lane = 0;
	bool one_done = false;
	// DFS state (solver.h:1582-1716)
	struct Entry {
		int u, v;
		int32_t path_len;
	};
	std::stack<Entry> stk;
	std::vector<std::pair<int, int>> path;
	struct Hash {
		size_t operator()(const std::vector<int32_t> &v) const {
			size_t seed = 0;
			for (auto x : v) seed ^= std::hash<int32_t>()(x) + 0x9e3779b9 + (seed << 6) + (seed >> 2);
			return seed;
		}
	};
	std::unordered_set<std::vector<int32_t>, Hash> emitted;
	std::vector<std::pair<int, int>> scratch;
};

// Length buckets of |s| that can get a group width of their own (Plan::bucket_G): rows up to
// 128, 256, 512 and more.
constexpr int PA_BUCKETS = PA_MAX_SEG;
constexpr int PA_MAX_CHUNKS = 12;  // pipeline chunks of a repeated host-buffer solve
inline int bucket_of(int64_t ls) { return ls <= 128 ? 0 : ls <= 256 ? 1 : ls <= 512 ? 2 : 3; }
// "g0,g1,g2,g3": a group width (1, 2, 4, 8, 16 or 32) per length bucket
bool parse_bucket_widths(const char *e, int *g) {
	int v[PA_BUCKETS];
	for (int k = 0; k < PA_BUCKETS; k++) {
		char *end = nullptr;
		const long x = std::strtol(e, &end, 10);
		if (end == e || x < 1 || x > 32 || (x & (x - 1))) return false;
		v[k] = int(x);
		e = end;
		if (k + 1 < PA_BUCKETS) {
			if (*e != ',') return false;
			e++;
		}
	}
	if (*e) return false;
	for (int k = 0; k < PA_BUCKETS; k++) g[k] = v[k];
	return true;
}

// The segments of one DP launch's order with length buckets: segment k has group width G[k],
// units (twins) unit[k] .. unit[k + 1] - 1 and warp tasks task[k] .. task[k + 1] - 1.
struct SegInfo {
	int nseg = 0, Gmin = 32;
	int G[PA_MAX_SEG] = {}, unit[PA_MAX_SEG + 1] = {}, task[PA_MAX_SEG + 1] = {};
};

// ---------------------------------------------------------------------------------------
// Solver

struct pa_solver {
	pa_options opt{};
	std::vector<float> gen_s, gen_t;  // general gap costs (reference domain)
	int64_t cap_s = 0, cap_t = 0;
	int32_t batch_size = 1;
	int gap = GAP_LINEAR;  // GapKind, or GAP_GENERAL
	int goal = GOAL_ONE;
	int loc = LOC_GLOBAL;
	float sign = 1.0f;     // +1 maximize, -1 minimize
	// normalised (maximize-form) borders, float: index k = cell -1 + k
	std::vector<float> left_D, left_P, top_D, top_Q;
	std::string alg[3];

	int device = -1;
	int sm_count = 0;
	cudaStream_t own_stream = nullptr;
	cudaStream_t stream = nullptr;
	bool stream_set = false;  // pa_solver_set_stream was called (stream may be NULL then)
	cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	float last_ms[4] = {0, 0, 0, 0};
	bool dp_timing_pending = false;  // a device-resident paths solve: read ev[1] -> ev[2] on demand
	int32_t last_launches = 0;
	int32_t last_plan[4] = {0, 0, 0, 0};  // kernel family, G, arithmetic, graph replay
	int32_t last_widths[4] = {0, 0, 0, 0};  // group width per length bucket (0: one width)
	int64_t bytes_h2d = 0, bytes_d2h = 0;

	DevBuf d_a, d_b, d_tab, d_dense, d_dense_off, d_ls, d_lt, d_order, d_mask_off, d_score, d_seed, d_has,
	    d_masks, d_scratch, d_counter, d_status, d_border, d_maps, d_map_off, d_paths, d_path_off,
	    d_path_len, d_vals, d_val_off, d_best, d_gen, d_wsb_off, d_wsb_tb, d_wsb_vals, d_wsb_vals_t, d_wsb_sub,
	    d_wsb_sub_off, d_codes_max, d_progress, d_chain;
	PinBuf h_stage, h_out;
	// per-call pair metadata, staged in one pinned buffer and sent with one copy
	DevBuf d_meta;
	PinBuf h_meta;
	cudaEvent_t meta_ev = nullptr;    // the staging buffer is free again once this completes
	bool meta_pending = false;
	struct {
		int32_t *ls, *lt, *order, *level_start;
		int64_t *mask_off, *map_off, *path_off, *val_off, *dense_off;
		int8_t *pair_G;  // per pair group width (length buckets)
	} m{};
	std::vector<std::pair<uint64_t, int>> occ_cache;  // (kernel variant, smem) -> blocks per SM
	DevBuf d_border_mode[4];          // borders per arithmetic mode: float, int tagged, int plain, packed 16-bit
	bool border_ready[4] = {false, false, false, false};
	std::vector<unsigned char> h_tab;  // staging of the converted similarity table
	// the per-pair lengths of the current call, kept across calls: a fresh vector of that size
	// per call would be new pages (allocator mmap) faulted in on every call
	std::vector<int32_t> h_ls, h_lt;

	// Repeated solves: the signature of the last device-resident solve and, once the same
	// solve came twice in a row, a CUDA graph of its device work (see solve_impl).
	struct Repeat {
		bool valid = false;
		int method = -1, form = -1;
		int64_t B = 0, n_s = 0, n_t = 0, trows = 0, tcols = 0, dsi = 0, dsj = 0;
		const void *a = nullptr, *b = nullptr, *sim = nullptr, *table = nullptr, *sx = nullptr, *sy = nullptr;
		int64_t sxs = 0, sys = 0;
		float eq = 0, ne = 0;
		int32_t *maps_out = nullptr, *paths = nullptr, *path_len = nullptr;
		float *scores = nullptr;
		cudaStream_t stream = nullptr;
		std::vector<int32_t> ls, lt;
		std::vector<float> table_host;
		std::vector<int64_t> user_map_off, user_path_off, dense_off;
		// the plan and what the downloads need from it
		int G = 0, C = 1, launches = 0, key_shift = 0, ntickets = 0, nlevels = 0;
		bool units = false, use_int = false, h16 = false, blk = false, seg = false;
		int bucket_G[PA_BUCKETS] = {};
		SegInfo segs[PA_MAX_CHUNKS];
		int32_t h_neg = 0;
		int nchunks = 1;
		std::vector<int64_t> mask_off, map_off, path_off, val_off;
		cudaGraphExec_t exec = nullptr;
	} rep;
	cudaStream_t cap_stream = nullptr;  // private stream the graph is captured on
	bool capturing = false;
	cudaStream_t copy_stream = nullptr;   // uploads and downloads of a pipelined host-buffer repeat
	cudaStream_t cmp2 = nullptr;          // its second compute stream (odd chunks)
	DevBuf d_counter2, d_scratch2;        // work counter and scratch rows of DP launches on cmp2
	std::vector<cudaEvent_t> ev_chunk;    // its per-chunk ordering events
	bool skip_table = false;              // run_dp: the converted table is already on the device
	cudaEvent_t table_ev = nullptr;       // run_dp: recorded once the converted table is copied

	void drop_graph() {
		if (rep.exec) cudaGraphExecDestroy(rep.exec);
		rep.exec = nullptr;
		rep.valid = false;
	}

	~pa_solver() {
		drop_graph();
		for (auto &e : ev)
			if (e) cudaEventDestroy(e);
		if (meta_ev) cudaEventDestroy(meta_ev);
		if (cap_stream) cudaStreamDestroy(cap_stream);
		for (auto &e : ev_chunk) cudaEventDestroy(e);
		if (copy_stream) cudaStreamDestroy(copy_stream);
		if (cmp2) cudaStreamDestroy(cmp2);
		if (own_stream) cudaStreamDestroy(own_stream);
	}
};

namespace {

// page-locked (pinned or registered) host memory: copies from or to it run asynchronously
bool host_pinned(const void *p) {
	if (!p) return true;
	cudaPointerAttributes a{};
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeHost;
}

// every host<->device copy of a solve goes through here, so the solver can report bytes
cudaError_t pa_copy(pa_solver *s, void *dst, const void *src, size_t n, cudaMemcpyKind kind, cudaStream_t st) {
	if (kind == cudaMemcpyHostToDevice) s->bytes_h2d += int64_t(n);
	else if (kind == cudaMemcpyDeviceToHost) s->bytes_d2h += int64_t(n);
	return cudaMemcpyAsync(dst, src, n, kind, st);
}

pa_status ensure_device(pa_solver *s) {
	if (s->device >= 0) return PA_OK;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
		cudaGetLastError();
		return fail(PA_ERR_NO_DEVICE, "no CUDA device: pyalign_gb300 has no CPU fallback");
	}
	PA_CUDA(cudaGetDevice(&s->device));
	PA_CUDA(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
	PA_CUDA(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
	if (!s->stream_set) s->stream = s->own_stream;
	for (auto &e : s->ev) PA_CUDA(cudaEventCreate(&e));
	PA_CUDA(cudaEventCreateWithFlags(&s->meta_ev, cudaEventDisableTiming));
	return PA_OK;
}

// Per-call plan of the DP launch.
struct Plan {
	bool use_int = false;
	int tb = TB_ONE;
	int G = 32;
	int key_shift = 0;
	int64_t max_ls = 0, max_lt = 0;
	bool units = false;        // stripe-chained mode (G = 32): one ticket per stripe
	int32_t ntickets = 0, nlevels = 0;
	int C = 1;                 // columns per lane step: 2 = dp2_kernel (int32 tagged, no values)
	bool h16 = false;          // packed 16-bit twin pairs (dp16_kernel); h_neg is its sentinel
	bool blk = false;          // with h16: the 4 x 4 block kernel (dp16b_kernel: 4 rows per lane, C = 4)
	// with h16 (dp16_kernel): a group width per length bucket of |s| (bucket_of), the pairs of
	// one launch ordered bucket by bucket; stage() cuts each pipeline chunk's order into
	// segments of one width (segs[chunk])
	bool seg = false;
	int bucket_G[PA_BUCKETS] = {16, 16, 16, 16};
	SegInfo segs[PA_MAX_CHUNKS];
	int32_t h_neg = 0;
	int C32 = 1;               // columns per lane step of the int32/float kernels for this launch
	int nchunks = 1;           // repeated host-buffer solves: pipeline of this many pair ranges
};

// The packed 16-bit twin kernel (pa_dp16.cuh) computes a launch exactly when every value
// it forms fits an int16 as value * 16 + tag, with room below the smallest real value for
// the sentinel and the addends applied to it.  Bounds, in value units: no D exceeds the
// largest similarity times the shorter length (plus the largest border); no real D, P or Q
// falls below the smallest border minus the costs of one gap down and one gap across the
// whole matrix (local alignment: below minus one gap opening and extension, the zero floor
// holds the rest).  It also needs an indexed form with at most 4 letters of t (int8
// profiles of 4 bytes, one prmt per two cells), similarities in [-8, 7] (int8 after the
// scaling), gap costs of at least 1 (rows past a pair's |s| must stay below its optimum),
// lengths of t below 65536 (16-bit column field), local or global alignment and no
// all-optimal masks or Solution values.  PA_DP16=0 turns it off.
bool h16_plan(const pa_solver *s, const Input &in, const float *host_table, const std::vector<int32_t> &ls,
              const std::vector<int32_t> &lt, int tb, bool want_values, bool use_int, int32_t *neg_out) {
	if (const char *e = std::getenv("PA_DP16"))
		if (std::strcmp(e, "0") == 0) return false;
	if (!use_int || want_values || tb == TB_ALL || in.form != F_INDEXED) return false;
	if (in.table_cols > 4 || in.table_rows > MAX_SMEM_TABLE || in.table_cols < 1) return false;
	if (s->loc != LOC_LOCAL && s->loc != LOC_GLOBAL) return false;
	if (s->gap != GAP_LINEAR && s->gap != GAP_AFFINE) return false;
	const pa_options &o = s->opt;
	double us, ut, w1s, w1t;
	if (s->gap == GAP_LINEAR) {
		us = w1s = o.linear_s;
		ut = w1t = o.linear_t;
	} else {
		us = o.affine_u_s;
		ut = o.affine_u_t;
		w1s = double(o.affine_u_s) + o.affine_v_s;
		w1t = double(o.affine_u_t) + o.affine_v_t;
	}
	if (!(us >= 1 && ut >= 1 && w1s >= 1 && w1t >= 1)) return false;
	double smax = -INFINITY;
	for (int64_t k = 0; k < in.table_rows * in.table_cols; k++) {
		const double v = double(host_table[k]) * s->sign;
		if (v * 16 + 8 < -128 || v * 16 + 8 > 127) return false;
		smax = std::max(smax, v);
	}
	int64_t mshort = 0, mls = 0, mlt = 0;
	for (size_t k = 0; k < ls.size(); k++) {
		if (ls[k] == 0 || lt[k] == 0) continue;
		mshort = std::max<int64_t>(mshort, std::min(ls[k], lt[k]));
		mls = std::max<int64_t>(mls, ls[k]);
		mlt = std::max<int64_t>(mlt, lt[k]);
	}
	if (mlt >= 65536) return false;
	double bmin = 0, bmax = 0;
	for (int64_t k = 0; k <= mls && k < int64_t(s->left_D.size()); k++) {
		if (!std::isfinite(s->left_D[size_t(k)])) return false;
		bmin = std::min(bmin, double(s->left_D[size_t(k)]));
		bmax = std::max(bmax, double(s->left_D[size_t(k)]));
	}
	for (int64_t k = 0; k <= mlt && k < int64_t(s->top_D.size()); k++) {
		if (!std::isfinite(s->top_D[size_t(k)])) return false;
		bmin = std::min(bmin, double(s->top_D[size_t(k)]));
		bmax = std::max(bmax, double(s->top_D[size_t(k)]));
	}
	// a twin computes the larger of its two pairs' shapes: bound the upper side over the
	// launch's whole rectangle (at least the largest shorter length of one pair)
	const double hi = std::max(0.0, smax) * double(std::max(mshort, std::min(mls, mlt))) + bmax;
	const double one_step = std::max({w1s + us, w1t + ut, 8.0});
	const double lo = s->loc == LOC_LOCAL ? -one_step
	                                      : bmin - (w1s + us * double(mls)) - (w1t + ut * double(mlt)) - one_step;
	const double neg = 16.0 * std::ceil(std::max(w1s, w1t) + std::max(us, ut) + 10.0) - 32768.0;
	if (hi * 16.0 + 15.0 > 32767.0 || lo * 16.0 <= neg + 16.0) return false;
	*neg_out = int32_t(neg);
	return true;
}

// Pair range [k0, k1) of chunk c of a pipelined solve of B pairs in K chunks: sizes grow as
// 1 : 2 : 4 : ..., so each chunk's upload (about 4x faster per pair than its DP) is hidden
// behind the previous chunk's DP and only the small first chunk's upload is exposed.
void chunk_range(int64_t B, int K, int c, int64_t &k0, int64_t &k1) {
	const int64_t den = (int64_t(1) << K) - 1;
	k0 = B * ((int64_t(1) << c) - 1) / den;
	k1 = B * ((int64_t(1) << (c + 1)) - 1) / den;
}

// a 16-bit addend in both halves
uint32_t h16_pack(int32_t v) { return (uint32_t(uint16_t(int16_t(v))) * 0x10001u); }
// a value (value * 16 + tag) in both halves, biased by 32768
uint32_t h16_value(int32_t v) { return uint32_t(uint16_t(v + 32768)) * 0x10001u; }
// a negative addend c as a 32-bit constant: adding it to a biased value always carries out
// of the low half (the value exceeds -c), so the high half takes c - 1
uint32_t h16_addk(int32_t c) { return (uint32_t(uint16_t(c - 1)) << 16) | uint32_t(uint16_t(c)); }

// Rows per lane and traceback words per lane step of a plan's DP kernel: 8 rows and C
// words (one per column) for dp_kernel / dp2_kernel / dp16_kernel, 4 rows and two words (a
// 4 x 4 block) for dp16b_kernel.
int plan_rows(const Plan &pl) { return pl.blk ? 4 : R; }
int plan_words(const Plan &pl) { return pl.blk ? 2 : pl.C; }

// Launches the two-column kernel can run: int32 tagged scoring without all-optimal masks
// or Solution values.
bool cols2_ok(const Plan &plan, bool want_values) { return plan.use_int && plan.tb != TB_ALL && !want_values; }

// Group width G (lanes per pair, R = 8 rows each; G = 1 is a lane per pair) that minimises the cells a launch
// computes: the real cells plus the padding rows of each pair's last stripe and the G-1
// skew steps of every stripe.  Narrower groups share a warp with other pairs and pay more
// per-stripe overhead: a 6% penalty per halving (measured: G = 8 beats G = 4 on uniform
// lengths in [100, 1000] although it computes 3% more cells) keeps G from shrinking for no
// gain.
int choose_G(const std::vector<int32_t> &ls, const std::vector<int32_t> &lt, int sm_count) {
	if (const char *e = std::getenv("PA_GROUP_WIDTH")) {  // experiments and tuning
		const int g = std::atoi(e);
		if (g == 1 || g == 2 || g == 4 || g == 8 || g == 16 || g == 32) return g;
	}
	static const int cand[6] = {32, 16, 8, 4, 2, 1};  // 1: a lane per pair
	int64_t pairs = 0;
	for (size_t k = 0; k < ls.size(); k++) pairs += (ls[k] > 0 && lt[k] > 0);
	double best = 0;
	int bestG = 32;
	for (int c = 0; c < 6; c++) {
		const int G = cand[c];
		const int64_t rpp = int64_t(G) * R;
		double cells = 0;
		for (size_t k = 0; k < ls.size(); k++) {
			if (ls[k] == 0 || lt[k] == 0) continue;
			const int64_t npass = (ls[k] + rpp - 1) / rpp;
			cells += double(npass * rpp) * double(lt[k] + G - 1);
		}
		cells *= 1.0 + 0.06 * c;
		// keep at least 4 warps per SM busy: narrower groups pack more pairs per warp (below
		// that the launch is latency-bound; at 4096 pairs of 64 x 64 one 64-row stripe per
		// pair, G = 8 with 7 warps per SM, beats G = 32 with 27 per SM, 3 of 4 lanes idle, 3x)
		const int64_t warps = (pairs + 32 / G - 1) / (32 / G);
		if (c > 0 && warps < int64_t(sm_count) * 4) break;
		if (c == 0 || cells < best) {
			best = cells;
			bestG = G;
		}
	}
	return bestG;
}

// Group mode (a group of G lanes sweeps all stripes of its pair) or stripe-chained mode (a
// warp per stripe, consecutive stripes of a pair on different warps, each waiting on the
// boundary row of the one above).  Both are estimated in warp-steps: the work spread over
// the resident warps, or the longest dependent chain, whichever is larger.  Group mode's
// chain is a whole pair; the stripe-chained chain is one sweep plus a PUB_CHUNK + 32 column
// lag per stripe.  Chaining pays when a launch has too few pairs to fill the GPU.
bool choose_units(const std::vector<int32_t> &ls, const std::vector<int32_t> &lt, int sm_count, int G) {
	if (const char *e = std::getenv("PA_DP_MODE")) {  // experiments and tests
		if (std::strcmp(e, "units") == 0) return true;
		if (std::strcmp(e, "groups") == 0) return false;
	}
	if (std::getenv("PA_GROUP_WIDTH")) return false;  // a forced group width means group mode
	const double slots = double(sm_count) * 16.0;
	const int64_t rg = int64_t(G) * R, ru = 32 * R;
	double work_g = 0, work_u = 0, chain_g = 0, chain_u = 0;
	for (size_t k = 0; k < ls.size(); k++) {
		if (ls[k] == 0 || lt[k] == 0) continue;
		const int64_t ng = (ls[k] + rg - 1) / rg, nu = (ls[k] + ru - 1) / ru;
		work_g += double(ng) * double(lt[k] + G - 1) * double(G) / 32.0;
		work_u += double(nu) * double(lt[k] + 31);
		chain_g = std::max(chain_g, double(ng) * double(lt[k] + G - 1));
		chain_u = std::max(chain_u, double(lt[k] + 31) + double(nu) * double(PUB_CHUNK + 32));
	}
	const double tg = std::max(work_g / slots, chain_g), tu = std::max(work_u / slots, chain_u);
	return tu < 0.8 * tg;
}

template <typename V>
V cvt(float x, bool use_int, int scale, int tag) {
	if (use_int) {
		if (!std::isfinite(x)) return V(-(1 << 29));
		return V(int32_t(std::nearbyint(x)) * scale + tag);
	}
	return V(x);
}

// The kernel family of a (value type, gap kind, mode).
template <typename V>
cudaError_t dp_launch(int gk, bool chain, int loc, int tb, bool vals, const DpParams<V> &p, int grid, size_t smem,
                      cudaStream_t st, int cols = 1) {
	if constexpr (std::is_same<V, int32_t>::value) {
		if (cols == 2)
			return gk == GAP_LINEAR ? launch_dp2_linear(loc, tb, chain, p, grid, smem, st)
			       : gk == GAP_AFFINE ? launch_dp2_affine(loc, tb, chain, p, grid, smem, st)
			                          : launch_dp2_dtw(loc, tb, chain, p, grid, smem, st);
		if (chain)
			return gk == GAP_LINEAR ? launch_dp_i_linear_chain(loc, tb, vals, p, grid, smem, st)
			       : gk == GAP_AFFINE ? launch_dp_i_affine_chain(loc, tb, vals, p, grid, smem, st)
			                          : launch_dp_i_dtw_chain(loc, tb, vals, p, grid, smem, st);
		return gk == GAP_LINEAR ? launch_dp_i_linear(loc, tb, vals, p, grid, smem, st)
		       : gk == GAP_AFFINE ? launch_dp_i_affine(loc, tb, vals, p, grid, smem, st)
		                          : launch_dp_i_dtw(loc, tb, vals, p, grid, smem, st);
	} else {
		if (chain)
			return gk == GAP_LINEAR ? launch_dp_f_linear_chain(loc, tb, vals, p, grid, smem, st)
			       : gk == GAP_AFFINE ? launch_dp_f_affine_chain(loc, tb, vals, p, grid, smem, st)
			                          : launch_dp_f_dtw_chain(loc, tb, vals, p, grid, smem, st);
		return gk == GAP_LINEAR ? launch_dp_f_linear(loc, tb, vals, p, grid, smem, st)
		       : gk == GAP_AFFINE ? launch_dp_f_affine(loc, tb, vals, p, grid, smem, st)
		                          : launch_dp_f_dtw(loc, tb, vals, p, grid, smem, st);
	}
}

template <typename V>
cudaError_t dp_occupancy(int gk, bool chain, int loc, int tb, bool vals, size_t smem, int *bps, int cols = 1) {
	if constexpr (std::is_same<V, int32_t>::value) {
		if (cols == 2)
			return gk == GAP_LINEAR ? occupancy_dp2_linear(loc, tb, chain, smem, bps)
			       : gk == GAP_AFFINE ? occupancy_dp2_affine(loc, tb, chain, smem, bps)
			                          : occupancy_dp2_dtw(loc, tb, chain, smem, bps);
		if (chain)
			return gk == GAP_LINEAR ? occupancy_dp_i_linear_chain(loc, tb, vals, smem, bps)
			       : gk == GAP_AFFINE ? occupancy_dp_i_affine_chain(loc, tb, vals, smem, bps)
			                          : occupancy_dp_i_dtw_chain(loc, tb, vals, smem, bps);
		return gk == GAP_LINEAR ? occupancy_dp_i_linear(loc, tb, vals, smem, bps)
		       : gk == GAP_AFFINE ? occupancy_dp_i_affine(loc, tb, vals, smem, bps)
		                          : occupancy_dp_i_dtw(loc, tb, vals, smem, bps);
	} else {
		if (chain)
			return gk == GAP_LINEAR ? occupancy_dp_f_linear_chain(loc, tb, vals, smem, bps)
			       : gk == GAP_AFFINE ? occupancy_dp_f_affine_chain(loc, tb, vals, smem, bps)
			                          : occupancy_dp_f_dtw_chain(loc, tb, vals, smem, bps);
		return gk == GAP_LINEAR ? occupancy_dp_f_linear(loc, tb, vals, smem, bps)
		       : gk == GAP_AFFINE ? occupancy_dp_f_affine(loc, tb, vals, smem, bps)
		                          : occupancy_dp_f_dtw(loc, tb, vals, smem, bps);
	}
}

template <typename V>
pa_status run_dp(pa_solver *s, const Input &in, const Plan &plan, int tb, const float *host_table,
                 int64_t npairs, bool want_values, const float *best_in_dev, int *launches, int64_t first = 0,
                 int codes_slot = 0, int side = 0, int seg_slot = -1) {
	if (seg_slot < 0) seg_slot = codes_slot;  // the pipeline chunk whose segments this launch runs
	const bool ISINT = std::is_same<V, int32_t>::value;
	const bool tag = ISINT && tb != TB_ALL;
	const int scale = tag ? 4 : 1;
	// side 1: a pipeline chunk on the second compute stream, with its own counter and scratch
	cudaStream_t st = side ? s->cmp2 : s->stream;
	DevBuf &counter = side ? s->d_counter2 : s->d_counter;
	DevBuf &scratch = side ? s->d_scratch2 : s->d_scratch;
	DpParams<V> p{};
	p.npairs = int32_t(npairs);
	p.order = s->m.order + first;  // a pipeline chunk: its pairs occupy order[first, first + npairs)
	p.len_s = s->m.ls;
	p.len_t = s->m.lt;
	p.sub_kind = in.form == F_DENSE ? SUB_DENSE
	             : in.form == F_SERIES ? SUB_SERIES
	             : (in.form == F_BINARY ? SUB_BINARY : SUB_TABLE);
	p.neg_inf = ISINT ? V(-(1 << 29)) : V(-INFINITY);
	p.G = plan.G;
	p.slots_per_warp = 32 / plan.G;
	// length buckets (16-bit two-column kernel): the segments of this chunk's order
	const bool segd = ISINT && plan.h16 && !plan.blk && plan.seg && plan.segs[seg_slot].nseg > 0;
	if (segd) {
		const SegInfo &sg = plan.segs[seg_slot];
		p.nseg = sg.nseg;
		for (int k = 0; k < sg.nseg; k++) p.seg_G[k] = sg.G[k];
		for (int k = 0; k <= sg.nseg; k++) {
			p.seg_unit[k] = sg.unit[k];
			p.seg_task[k] = sg.task[k];
		}
		p.slots_per_warp = 32 / sg.Gmin;
	}
	p.key_shift = plan.key_shift;
	p.one = 1;
	p.minus_one = -1;
	p.minus_four = -4;
	p.minus_eight = -8;
	p.sixteen = 16;
	p.two = 2;
	p.bit16 = 65536;
	p.out_sign = s->sign;
	const int gk = s->gap;  // GAP_LINEAR / GAP_AFFINE / GAP_DTW
	const int diag_tag = (tag && gk != GAP_DTW) ? 2 : 0;
	const bool h16 = ISINT && plan.h16;

	// ---- sequences and substitution
	if (in.form == F_SERIES) {
		// the series travel through the code paths as raw 32-bit words
		p.a = reinterpret_cast<const uint32_t *>(in.sx);
		p.b = reinterpret_cast<const uint32_t *>(in.sy);
		p.a_stride = in.sx_stride;
		p.b_stride = in.sy_stride;
		p.dense_sign = s->sign;
	} else if (in.form != F_DENSE) {
		p.a = in.location == PA_DEVICE ? in.a : s->d_a.as<uint32_t>();
		p.b = in.location == PA_DEVICE ? in.b : s->d_b.as<uint32_t>();
		p.a_stride = in.n_s;
		p.b_stride = in.n_t;
	}
	if (in.form == F_SERIES) {
		// nothing more: S is computed in the kernel
	} else if (in.form == F_INDEXED) {
		p.table_rows = int32_t(in.table_rows);
		p.table_cols = int32_t(in.table_cols);
		p.table = s->d_tab.as<V>();
	} else if (in.form == F_BINARY) {
		p.eq = cvt<V>(in.eq * s->sign, ISINT, scale, diag_tag);
		p.ne = cvt<V>(in.ne * s->sign, ISINT, scale, diag_tag);
	} else {
		p.dense = in.location == PA_DEVICE ? in.sim : s->d_dense.as<float>();
		p.dense_off = s->m.dense_off;
		p.dense_si = in.dense_si ? in.dense_si : in.n_t * in.batch;
		p.dense_sj = in.dense_si ? in.dense_sj : in.batch;
		p.dense_sign = s->sign;
	}
	// ---- gaps (negative addends, maximize form)
	const pa_options &o = s->opt;
	if (gk == GAP_LINEAR) {
		p.c_up = cvt<V>(-o.linear_s, ISINT, scale, tag ? 1 : 0);
		p.c_left = cvt<V>(-o.linear_t, ISINT, scale, 0);
	} else if (gk == GAP_AFFINE) {
		const float w1s = o.affine_u_s + o.affine_v_s, w1t = o.affine_u_t + o.affine_v_t;
		p.c_open_s = cvt<V>(-w1s, ISINT, scale, tag ? 1 : 0);
		p.c_ext_s = cvt<V>(-o.affine_u_s, ISINT, scale, 0);
		p.c_open_t = cvt<V>(-w1t, ISINT, scale, 0);
		p.c_ext_t = cvt<V>(-o.affine_u_t, ISINT, scale, 0);
	}
	if (h16) {
		// value * 16 + tag: P's open candidate carries code 1 (bits 2-3) and its open bit 0,
		// Q's carries code 0 and its open bit 1
		auto raw = [](float x, int tg) { return int32_t(std::nearbyint(x)) * 16 + tg; };
		if (gk == GAP_LINEAR) {
			p.k_up = h16_addk(raw(-o.linear_s, 4));
			p.k_left = h16_addk(raw(-o.linear_t, 0));
		} else {
			p.k_open_s = h16_addk(raw(-(o.affine_u_s + o.affine_v_s), 5));
			p.h_ext_s = h16_pack(raw(-o.affine_u_s, 0));
			p.k_open_t = h16_addk(raw(-(o.affine_u_t + o.affine_v_t), 2));
			p.h_ext_t = h16_pack(raw(-o.affine_u_t, 0));
		}
		p.h_neg = h16_value(plan.h_neg);
	}
	// ---- borders: converted once per solver and arithmetic mode, then kept on the device
	{
		const size_t ns = s->left_D.size(), nt = s->top_D.size();
		const int mode = ISINT ? (tag ? 1 : 2) : 0;
		if (!s->border_ready[mode]) {
			std::vector<V> bv(2 * ns + 2 * nt);
			for (size_t k = 0; k < ns; k++) {
				bv[k] = cvt<V>(s->left_D[k], ISINT, scale, 0);
				bv[ns + k] = cvt<V>(s->left_P[k], ISINT, scale, tag ? 1 : 0);
			}
			for (size_t k = 0; k < nt; k++) {
				bv[2 * ns + k] = cvt<V>(s->top_D[k], ISINT, scale, 0);
				bv[2 * ns + nt + k] = cvt<V>(s->top_Q[k], ISINT, scale, 0);
			}
			PA_CUDA(s->d_border_mode[mode].ensure(bv.size() * sizeof(V)));
			PA_CUDA(cudaMemcpy(s->d_border_mode[mode].p, bv.data(), bv.size() * sizeof(V), cudaMemcpyHostToDevice));
			s->border_ready[mode] = true;
		}
		V *b = s->d_border_mode[mode].as<V>();
		p.left_D = b;
		p.left_P = b + ns;
		p.top_D = b + 2 * ns;
		p.top_Q = b + 2 * ns + nt;
		if (h16) {
			// packed borders of the 16-bit kernel (its launches have finite borders)
			if (!s->border_ready[3]) {
				std::vector<uint32_t> hb(ns + nt);
				// (borders beyond the launch's bounds are never read; clamped to stay encodable)
				auto bv16 = [](float x) {
					const double v = std::isfinite(x) ? std::nearbyint(double(x)) * 16.0 : -30000.0;
					return h16_value(int32_t(std::min(30000.0, std::max(-30000.0, v))));
				};
				for (size_t k = 0; k < ns; k++) hb[k] = bv16(s->left_D[k]);
				for (size_t k = 0; k < nt; k++) hb[ns + k] = bv16(s->top_D[k]);
				PA_CUDA(s->d_border_mode[3].ensure(hb.size() * 4));
				PA_CUDA(cudaMemcpy(s->d_border_mode[3].p, hb.data(), hb.size() * 4, cudaMemcpyHostToDevice));
				s->border_ready[3] = true;
			}
			p.left16 = s->d_border_mode[3].as<uint32_t>();
			p.top16 = p.left16 + ns;
		}
		if (in.form == F_INDEXED) {
			// the table (small) is converted on the host: scaled, tagged, direction-normalised;
			// the staging buffer belongs to the solver, so the copy needs no synchronisation
			const size_t nt_ = size_t(in.table_rows * in.table_cols);
			s->h_tab.resize(nt_ * sizeof(V));
			V *tabv = reinterpret_cast<V *>(s->h_tab.data());
			bool fits_int8 = ISINT && tag && in.table_cols <= 8 && in.table_rows <= MAX_SMEM_TABLE;
			for (size_t k = 0; k < nt_; k++) {
				tabv[k] = h16 ? V(int32_t(std::nearbyint(host_table[k] * s->sign)) * 16 + 8)
				              : cvt<V>(host_table[k] * s->sign, ISINT, scale, diag_tag);
				if (ISINT && (int64_t(tabv[k]) < -128 || int64_t(tabv[k]) > 127)) fits_int8 = false;
			}
			// int8 profiles read with one prmt per cell: per row in registers (alphabets of
			// <= 8 letters) or per letter in shared memory (<= 32 letters)
			bool colprof_ok = ISINT && tag && in.table_cols <= MAX_COLPROF && in.table_rows <= MAX_SMEM_TABLE;
			for (size_t k = 0; k < nt_ && colprof_ok; k++)
				if (int64_t(tabv[k]) < -128 || int64_t(tabv[k]) > 127) colprof_ok = false;
			const char *sk = std::getenv("PA_SUBST");  // experiments: "table", "colprof"
			if (fits_int8) p.sub_kind = SUB_PROFILE;
			else if (colprof_ok) p.sub_kind = SUB_COLPROF;
			if (sk && std::strcmp(sk, "table") == 0) p.sub_kind = SUB_TABLE;
			if (sk && std::strcmp(sk, "colprof") == 0 && colprof_ok) p.sub_kind = SUB_COLPROF;
			PA_CUDA(s->d_tab.ensure(nt_ * sizeof(V)));
			if (!s->capturing && !s->skip_table)
				PA_CUDA(pa_copy(s, s->d_tab.p, tabv, nt_ * sizeof(V), cudaMemcpyHostToDevice, st));
			if (s->table_ev) PA_CUDA(cudaEventRecord(s->table_ev, st));
			p.table = s->d_tab.as<V>();
		}
	}
	// ---- outputs
	p.score = s->d_score.as<float>();
	p.seed = s->d_seed.as<int32_t>();
	p.has_seed = s->d_has.as<int32_t>();
	p.masks = s->d_masks.p;
	p.mask_off = s->m.mask_off;
	p.best_in = best_in_dev;
	p.values = want_values ? s->d_vals.as<float>() : nullptr;
	p.val_off = s->m.val_off;
	PA_CUDA(counter.ensure(4));
	p.work_counter = counter.as<int32_t>();
	p.status = s->d_status.as<int32_t>();
	if (in.form == F_INDEXED) {
		p.codes_max = s->d_codes_max.as<uint32_t>() + 2 * codes_slot;
		p.code_lim_a = (in.batch * in.n_s > 0) ? uint32_t(in.table_rows) : 0xFFFFFFFFu;
		p.code_lim_b = (in.batch * in.n_t > 0) ? uint32_t(in.table_cols) : 0xFFFFFFFFu;
	}

	// ---- grid and scratch
	size_t smem = (in.form == F_INDEXED && in.table_rows <= MAX_SMEM_TABLE && in.table_cols <= MAX_SMEM_TABLE)
	                  ? size_t(in.table_rows * in.table_cols) * sizeof(V)
	                  : 0;
	if (p.sub_kind == SUB_COLPROF) smem = ((smem + 15) & ~size_t(15)) + size_t(in.table_cols) * BLOCK * 8;
	if (p.sub_kind == SUB_DENSE) smem = size_t(BLOCK) * DENSE_RING * 32;  // the dense S ring (pa_dp.cuh)
	int bps = 0;
	cudaError_t e = cudaSuccess;
	const int loc = s->loc;
	const uint64_t okey = (uint64_t(ISINT) << 60) | (uint64_t(gk) << 56) | (uint64_t(loc) << 52) |
	                      (uint64_t(tb) << 48) | (uint64_t(want_values) << 44) | uint64_t(smem);
	const bool ch = plan.units;
	const int cols = (ISINT && plan.C == 2 && tb != TB_ALL && !want_values) ? 2 : 1;
	const bool blk = h16 && plan.blk;
	const uint64_t ckey = okey | (uint64_t(ch) << 40) | (uint64_t(cols == 2) << 41) | (uint64_t(h16) << 42) |
	                      (uint64_t(blk) << 43);
	for (const auto &kv : s->occ_cache)
		if (kv.first == ckey) bps = kv.second;
	if (bps == 0) {
		if (blk) e = gk == GAP_LINEAR ? occupancy_dp16b_linear(loc, tb, smem, &bps)
		                              : occupancy_dp16b_affine(loc, tb, smem, &bps);
		else if (h16) e = gk == GAP_LINEAR ? occupancy_dp16_linear(loc, tb, cols, smem, &bps)
		                                   : occupancy_dp16_affine(loc, tb, cols, smem, &bps);
		else e = dp_occupancy<V>(gk, ch, loc, tb, want_values, smem, &bps, cols);
	}
	PA_CUDA(e);
	bps = std::max(bps, 1);
	if (s->occ_cache.size() < 64) s->occ_cache.push_back({ckey, bps});
	const int gpw = segd ? p.slots_per_warp : 32 / plan.G;
	const int64_t units_needed = h16 ? (npairs + 1) / 2 : npairs;  // twins or pairs
	const int64_t groups_needed = plan.units ? plan.ntickets
	                              : segd     ? p.seg_task[p.nseg]  // warp tasks of the segments
	                                         : (units_needed + gpw - 1) / gpw;  // warps needed
	int64_t grid = int64_t(s->sm_count) * bps;
	grid = std::min<int64_t>(grid, (groups_needed + WARPS - 1) / WARPS);
	// PA_GRID=exact: one block per WARPS work units, each warp takes one unit and exits -- the
	// non-persistent launch of a plain per-bucket solve, kept for that comparison
	if (const char *ge = std::getenv("PA_GRID"))
		if (std::strcmp(ge, "exact") == 0) grid = (groups_needed + WARPS - 1) / WARPS;
	grid = std::max<int64_t>(grid, 1);
	// scratch rows: per group slot, or per pair in the stripe-chained mode
	const int64_t slots = plan.units ? std::max<int64_t>(npairs, 1) : grid * WARPS * gpw;
	p.scratch_stride = 2 * std::max<int64_t>(plan.max_lt, 1);
	PA_CUDA(scratch.ensure(size_t(slots * p.scratch_stride) * 2 * sizeof(V)));
	p.scratch = scratch.p;
	if (plan.units) {
		p.units = 1;
		p.ntickets = plan.ntickets;
		p.nlevels = plan.nlevels;
		p.level_start = s->m.level_start;
		PA_CUDA(s->d_progress.ensure(size_t(plan.ntickets) * 4));
		PA_CUDA(s->d_chain.ensure(size_t(plan.ntickets) * 16));
		p.progress = s->d_progress.as<int32_t>();
		p.chain = s->d_chain.as<int4>();
		PA_CUDA(cudaMemsetAsync(s->d_progress.p, 0, size_t(plan.ntickets) * 4, st));
	}

	PA_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(int32_t), st));
	if constexpr (std::is_same<V, int32_t>::value) {
		if (blk) e = gk == GAP_LINEAR ? launch_dp16b_linear(loc, tb, p, int(grid), smem, st)
		                              : launch_dp16b_affine(loc, tb, p, int(grid), smem, st);
		else if (h16) e = gk == GAP_LINEAR ? launch_dp16_linear(loc, tb, cols, p, int(grid), smem, st)
		                                   : launch_dp16_affine(loc, tb, cols, p, int(grid), smem, st);
		else e = dp_launch<V>(gk, ch, loc, tb, want_values, p, int(grid), smem, st, cols);
	} else {
		e = dp_launch<V>(gk, ch, loc, tb, want_values, p, int(grid), smem, st, cols);
	}
	PA_CUDA(e);
	(*launches)++;
	return PA_OK;
}

// Validation shared by all entry points (factory.h:387-394, 526-533, 602-614;
// solver.h:487-503, 719-728).
pa_status validate(pa_solver *s, const Input &in) {
	if (in.batch != s->batch_size)
		return fail(PA_ERR_INVALID_ARGUMENT, "problem of batch size " + std::to_string(in.batch) +
		                                         " given to solver that was configured to batch size " +
		                                         std::to_string(s->batch_size));
	if (in.n_s > s->cap_s)
		return fail(PA_ERR_LENGTH, "sequence s of length " + std::to_string(in.n_s) +
		                               " exceeds configured maximum length " + std::to_string(s->cap_s));
	if (in.n_t > s->cap_t)
		return fail(PA_ERR_LENGTH, "sequence t of length " + std::to_string(in.n_t) +
		                               " exceeds configured maximum length " + std::to_string(s->cap_t));
	if (!in.length) return fail(PA_ERR_INVALID_ARGUMENT, "length array missing");
	return PA_OK;
}

// Decide int32 (exact, faster) vs float32 arithmetic.  Integer mode is used when every
// similarity, gap cost and border is an integer and every reachable value stays below
// 2^23 in magnitude, which also means the reference's float32 arithmetic is exact.
bool int_mode_ok(const pa_solver *s, const Input &in, const float *host_table, int64_t max_ls, int64_t max_lt,
                 double *bound_out) {
	if (in.form == F_DENSE || in.form == F_SERIES) return false;
	if (s->gap == GAP_GENERAL) return false;
	double m = 0;
	auto chk = [&](float x) {
		if (!integral(x)) return false;
		m = std::max(m, double(std::fabs(x)));
		return true;
	};
	const pa_options &o = s->opt;
	if (s->gap == GAP_LINEAR && !(chk(o.linear_s) && chk(o.linear_t))) return false;
	if (s->gap == GAP_AFFINE &&
	    !(chk(o.affine_u_s) && chk(o.affine_v_s) && chk(o.affine_u_t) && chk(o.affine_v_t) &&
	      chk(o.affine_u_s + o.affine_v_s) && chk(o.affine_u_t + o.affine_v_t)))
		return false;
	if (in.form == F_BINARY) {
		if (!(chk(in.eq) && chk(in.ne))) return false;
	} else {
		for (int64_t k = 0; k < in.table_rows * in.table_cols; k++)
			if (!chk(host_table[k])) return false;
	}
	double mb = 0;
	for (size_t k = 0; k <= size_t(std::min<int64_t>(max_ls, int64_t(s->left_D.size()) - 1)); k++) {
		if (std::isfinite(s->left_D[k])) {
			if (!integral(s->left_D[k])) return false;
			mb = std::max(mb, double(std::fabs(s->left_D[k])));
		}
	}
	for (size_t k = 0; k <= size_t(std::min<int64_t>(max_lt, int64_t(s->top_D.size()) - 1)); k++) {
		if (std::isfinite(s->top_D[k])) {
			if (!integral(s->top_D[k])) return false;
			mb = std::max(mb, double(std::fabs(s->top_D[k])));
		}
	}
	const double bound = double(max_ls + max_lt + 2) * m + mb;
	*bound_out = bound;
	return bound < double(1 << 23);
}

// General gap costs: one CTA per pair (pa_wsb.cu).  With `maps` (device, at the staged map
// offsets) the one-optimal alignments are walked on the device too; otherwise the values,
// traceback codes and similarity of every cell are downloaded for the host's traceback
// (download_wsb).
pa_status run_wsb(pa_solver *s, const Input &in, const std::vector<int32_t> &ls, const std::vector<int32_t> &lt,
                  int *launches, ResultData &res, int32_t *maps) {
	cudaStream_t st = s->stream;
	const int64_t B = in.batch;
	std::vector<int64_t> voff(size_t(B) + 1, 0), toff(size_t(B) + 1, 0);
	for (int64_t k = 0; k < B; k++) {
		voff[size_t(k) + 1] = voff[size_t(k)] + int64_t(ls[size_t(k)] + 1) * (lt[size_t(k)] + 1);
		toff[size_t(k) + 1] = toff[size_t(k)] + int64_t(ls[size_t(k)]) * lt[size_t(k)];
	}
	res.wsb_voff = voff;
	res.wsb_off = toff;
	res.wsb_sub_off = toff;
	const size_t ns = s->left_D.size(), nt = s->top_D.size();
	std::vector<float> host(2 * ns + 2 * nt);
	std::copy(s->left_D.begin(), s->left_D.end(), host.begin());
	std::copy(s->top_D.begin(), s->top_D.end(), host.begin() + ns);
	std::copy(s->gen_s.begin(), s->gen_s.end(), host.begin() + ns + nt);
	std::copy(s->gen_t.begin(), s->gen_t.end(), host.begin() + 2 * ns + nt);
	PA_CUDA(s->d_gen.ensure(host.size() * 4));
	PA_CUDA(pa_copy(s, s->d_gen.p, host.data(), host.size() * 4, cudaMemcpyHostToDevice, st));
	PA_CUDA(s->d_wsb_off.ensure(voff.size() * 8));
	PA_CUDA(pa_copy(s, s->d_wsb_off.p, voff.data(), voff.size() * 8, cudaMemcpyHostToDevice, st));
	PA_CUDA(s->d_wsb_sub_off.ensure(toff.size() * 8));
	PA_CUDA(pa_copy(s, s->d_wsb_sub_off.p, toff.data(), toff.size() * 8, cudaMemcpyHostToDevice, st));
	// (+64 bytes: the kernel copies the 16-byte blocks that hold a run of values)
	PA_CUDA(s->d_wsb_vals.ensure(size_t(voff[size_t(B)]) * 4 + 64));
	PA_CUDA(s->d_wsb_vals_t.ensure(size_t(voff[size_t(B)]) * 4 + 64));
	PA_CUDA(s->d_wsb_tb.ensure(size_t(std::max<int64_t>(toff[size_t(B)], 1)) * 4));
	PA_CUDA(s->d_wsb_sub.ensure(size_t(std::max<int64_t>(toff[size_t(B)], 1)) * 4));
	std::vector<float> tab;
	WsbParams w{};
	w.npairs = int32_t(B);
	w.len_s = s->m.ls;
	w.len_t = s->m.lt;
	w.local = s->loc;
	w.sub_kind = in.form == F_DENSE ? SUB_DENSE : (in.form == F_BINARY ? SUB_BINARY : SUB_TABLE);
	if (in.form != F_DENSE) {
		w.a = in.location == PA_DEVICE ? in.a : s->d_a.as<uint32_t>();
		w.b = in.location == PA_DEVICE ? in.b : s->d_b.as<uint32_t>();
		w.a_stride = in.n_s;
		w.b_stride = in.n_t;
	}
	if (in.form == F_INDEXED) {
		const size_t n = size_t(in.table_rows * in.table_cols) * 4;
		PA_CUDA(s->d_tab.ensure(n));
		PA_CUDA(pa_copy(s, s->d_tab.p, in.table, n, in.location == PA_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
		w.table = s->d_tab.as<float>();
		w.table_rows = int32_t(in.table_rows);
		w.table_cols = int32_t(in.table_cols);
	}
	w.eq = in.eq;
	w.ne = in.ne;
	if (in.form == F_DENSE) {
		w.dense = in.location == PA_DEVICE ? in.sim : s->d_dense.as<float>();
		w.dense_si = in.n_t * in.batch;
		w.dense_sj = in.batch;
	}
	w.sign = s->sign;
	const float *g = s->d_gen.as<float>();
	w.left_D = g;
	w.top_D = g + ns;
	w.gap_s = g + ns + nt;
	w.gap_t = g + 2 * ns + nt;
	w.vals = s->d_wsb_vals.as<float>();
	w.vals_t = s->d_wsb_vals_t.as<float>();
	w.vals_off = s->d_wsb_off.as<int64_t>();
	w.tb = s->d_wsb_tb.as<int32_t>();
	w.tb_off = s->d_wsb_sub_off.as<int64_t>();
	w.sub = s->d_wsb_sub.as<float>();
	w.score = s->d_score.as<float>();
	w.seed = s->d_seed.as<int32_t>();
	w.has_seed = s->d_has.as<int32_t>();
	w.status = s->d_status.as<int32_t>();
	// about four cells per warp on a pair's longest diagonal, 128 to 1024 threads; a cluster
	// of 4 or 2 CTAs per pair when the clusters of all pairs fit the SMs at once and the pairs
	// are long enough to keep them busy (pairs of 200 x 200: one CTA 1.84 ms, two 1.99 ms;
	// 300 x 300: 4.9 and 4.2 ms).  PA_WSB_THREADS, PA_WSB_WARP_CELLS, PA_WSB_CLUSTER:
	// experiments and tests.
	int64_t diag = 0;
	for (int64_t k = 0; k < B; k++) diag = std::max<int64_t>(diag, std::min(ls[size_t(k)], lt[size_t(k)]));
	int threads = int(std::min<int64_t>(1024, std::max<int64_t>(128, 32 * ((diag + 3) / 4))));
	threads = (threads + 31) / 32 * 32;
	if (const char *e = std::getenv("PA_WSB_THREADS")) threads = std::min(1024, std::max(32, std::atoi(e) / 32 * 32));
	int cluster = 1;
	if (B * 4 <= s->sm_count && diag >= 512) cluster = 4;
	else if (B * 2 <= s->sm_count && diag >= 256) cluster = 2;
	const char *cenv = std::getenv("PA_WSB_CLUSTER");
	if (cenv) {
		const int c = std::atoi(cenv);
		cluster = c >= 4 ? 4 : c >= 2 ? 2 : 1;
	}
	// one CTA per pair: the pair's rows in its shared memory too when they fit 200 KB (3% on
	// 128 pairs of 200 x 200; the rows of a cluster's pair spread over its CTAs measured slower
	// than L2).  PA_WSB_SMEM=0: global memory only, for tests.
	int64_t max_ls = 0, max_lt = 0;
	for (int64_t k = 0; k < B; k++) {
		max_ls = std::max<int64_t>(max_ls, ls[size_t(k)]);
		max_lt = std::max<int64_t>(max_lt, lt[size_t(k)]);
	}
	const int64_t lds = (max_lt + 1) | 1;
	w.lds = 0;
	w.max_ls = int32_t(max_ls);
	const char *menv = std::getenv("PA_WSB_SMEM");
	if (cluster == 1 && !(menv && std::strcmp(menv, "0") == 0) && (max_ls + 1) * lds * 4 <= 200 * 1024)
		w.lds = int32_t(lds);
	// a warp per cell on every diagonal (one thread per cell measured 3.5x slower on pairs of
	// 1000 x 1000 and only loses more as scans grow); PA_WSB_WARP_CELLS=0 keeps the thread per cell
	w.warp_cells = 1 << 20;
	if (const char *e = std::getenv("PA_WSB_WARP_CELLS")) w.warp_cells = std::min(1 << 20, std::max(0, std::atoi(e)));
	PA_CUDA(launch_wsb(w, threads, cluster, st));
	(*launches)++;
	if (maps) {
		WsbWalkParams wk{};
		wk.npairs = int32_t(B);
		wk.len_s = s->m.ls;
		wk.len_t = s->m.lt;
		wk.local = s->loc;
		wk.vals = w.vals;
		wk.vals_off = w.vals_off;
		wk.tb = w.tb;
		wk.tb_off = w.tb_off;
		wk.seed = w.seed;
		wk.has_seed = w.has_seed;
		wk.map_off = s->m.map_off;
		wk.maps = maps;
		PA_CUDA(launch_wsb_walk(wk, st));
		(*launches)++;
	}
	PA_CUDA(cudaStreamSynchronize(st));  // host vectors above are temporaries
	return PA_OK;
}

pa_status download_wsb(pa_solver *s, ResultData &res) {
	cudaStream_t st = s->stream;
	const int64_t B = res.batch;
	res.wsb_vals.resize(size_t(res.wsb_voff[size_t(B)]));
	res.wsb_tb.resize(size_t(res.wsb_off[size_t(B)]));
	res.wsb_sub.resize(size_t(res.wsb_off[size_t(B)]));
	if (!res.wsb_vals.empty())
		PA_CUDA(pa_copy(s, res.wsb_vals.data(), s->d_wsb_vals.p, res.wsb_vals.size() * 4, cudaMemcpyDeviceToHost, st));
	if (!res.wsb_tb.empty()) {
		PA_CUDA(pa_copy(s, res.wsb_tb.data(), s->d_wsb_tb.p, res.wsb_tb.size() * 4, cudaMemcpyDeviceToHost, st));
		PA_CUDA(pa_copy(s, res.wsb_sub.data(), s->d_wsb_sub.p, res.wsb_sub.size() * 4, cudaMemcpyDeviceToHost, st));
	}
	return PA_OK;
}

// ---------------------------------------------------------------------------------------
// Autotuner.  A DP launch runs in group mode with G = 4, 8, 16 or 32 lanes per pair or in
// the stripe-chained mode; which is fastest depends on how many pairs there are and how
// long they are (measured on GB300: 12,288 pairs of lengths in [100, 1000] run 1.8x faster
// with G = 16 than with G = 8, 65,536 such pairs run fastest with G = 8, 256 pairs of
// 5000 x 10000 4x faster chained).  The first call with a new workload signature -- pair
// count, mean and largest lengths in half-octave/octave buckets, gap kind, locality,
// traceback kind, arithmetic, input form -- times each candidate on the real input and
// keeps the fastest for every later call with that signature, process-wide.  Every plan
// computes the same results (the order of pairs and the grouping never change a value).
// PA_TUNE=0 turns the timing off (the analytic choice stands), as do the experiment
// overrides PA_DP_MODE, PA_GROUP_WIDTH and PA_BUCKET_WIDTHS.
//
// When the 16-bit twin kernel wins and the pairs fall into more than one length bucket of
// |s| (bucket_of), the tuner also tries a group width per bucket, by timing: one launch with
// the buckets in segments of one width each, starting from the uniform width, each bucket in
// turn at half (then a quarter ...) or twice the width, a change kept only when the launch
// runs at least 1% faster.
struct TuneEntry {
	uint64_t key;
	int G;
	bool units;
	bool h16;
	int C;
	bool blk;
	bool seg;
	int bucket_G[PA_BUCKETS];
};
std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;
constexpr double TUNE_MIN_CELLS = 4e6;  // smaller launches keep the analytic choice

uint64_t tune_key(const pa_solver *s, const Input &in, const Plan &plan, const std::vector<int32_t> &ls,
                  const std::vector<int32_t> &lt, double *cells) {
	int64_t n = 0, mls = 0, mlt = 0;
	double sls = 0, slt = 0, c = 0;
	for (size_t k = 0; k < ls.size(); k++) {
		if (ls[k] == 0 || lt[k] == 0) continue;
		n++;
		sls += ls[k];
		slt += lt[k];
		c += double(ls[k]) * double(lt[k]);
		mls = std::max<int64_t>(mls, ls[k]);
		mlt = std::max<int64_t>(mlt, lt[k]);
	}
	*cells = c;
	auto oct = [](double x) -> uint64_t { return x < 1 ? 0 : uint64_t(std::floor(std::log2(x))) & 63; };
	auto half = [](double x) -> uint64_t { return x < 1 ? 0 : uint64_t(std::floor(2 * std::log2(x))) & 63; };
	const uint64_t tabk = in.form != F_INDEXED ? 0 : in.table_cols <= 8 ? 1 : in.table_cols <= MAX_COLPROF ? 2 : 3;
	return oct(double(n)) | (half(n ? sls / n : 0) << 6) | (half(n ? slt / n : 0) << 12) | (oct(double(mls)) << 18) |
	       (oct(double(mlt)) << 24) | (uint64_t(s->gap & 3) << 30) | (uint64_t(s->loc & 3) << 32) |
	       (uint64_t(plan.tb & 3) << 34) | (uint64_t(plan.use_int) << 36) | (uint64_t(in.form & 3) << 37) |
	       (tabk << 39) | (uint64_t(s->sm_count & 1023) << 41) | (uint64_t(s->device & 63) << 51);
}

template <typename Stage, typename Dp>
pa_status tune_plan(pa_solver *s, const std::vector<int32_t> &ls, const std::vector<int32_t> &lt, const Input &in,
                    Plan &plan, Stage &stage, Dp &dp) {
	const char *te = std::getenv("PA_TUNE");
	if ((te && std::strcmp(te, "0") == 0) || std::getenv("PA_DP_MODE") || std::getenv("PA_GROUP_WIDTH") ||
	    std::getenv("PA_BUCKET_WIDTHS"))
		return PA_OK;
	double cells = 0;
	const uint64_t key = tune_key(s, in, plan, ls, lt, &cells);
	{
		std::lock_guard<std::mutex> lk(g_tune_mu);
		for (const auto &t : g_tune)
			if (t.key == key) {
				plan.G = t.G;
				plan.units = t.units;
				plan.h16 = plan.h16 && t.h16;  // the 16-bit kernel still needs this launch's bounds
				plan.blk = plan.h16 && t.blk;
				plan.C = plan.h16 ? t.C : plan.C32;
				plan.seg = plan.h16 && !plan.blk && t.seg;
				for (int k = 0; k < PA_BUCKETS; k++) plan.bucket_G[k] = t.bucket_G[k];
				return PA_OK;
			}
	}
	if (cells < TUNE_MIN_CELLS) return PA_OK;
	// candidates: every group width whose stripe is not far taller than the pairs, and the
	// stripe-chained mode when the longest pairs span several 256-row stripes
	// (G, chained, 16-bit twins, columns per step): the 16-bit kernel, with one or two columns
	// per step, where this launch's bounds admit it
	const int C0 = plan.C32;
	struct Cand {
		int G;
		bool units, h16;
		int C;
		bool blk;
	};
	std::vector<Cand> cand;
	for (int G : {32, 16, 8, 4, 2, 1})
		if (G == 4 || (int64_t(G) * R <= 2 * plan.max_ls && (G >= 4 || plan.max_ls <= 256))) {
			cand.push_back({G, false, false, C0, false});
			if (plan.h16) {
				cand.push_back({G, false, true, 1, false});
				if (C0 == 2) cand.push_back({G, false, true, 2, false});
			}
		}
	// the 16-bit 4 x 4 block kernel (stripes of 4 G rows: the tile height 4 instead of 8)
	if (plan.h16 && C0 == 2)
		for (int G : {32, 16, 8})
			if (int64_t(G) * 4 <= 2 * plan.max_ls) cand.push_back({G, false, true, 4, true});
	if (plan.max_ls > 2 * 32 * R) cand.push_back({32, true, false, C0, false});
	if (cand.size() < 2) return PA_OK;
	cudaStream_t st = s->stream;
	float best = INFINITY;
	int bestG = plan.G, bestC = plan.C;
	bool bestU = plan.units, bestH = plan.h16, bestB = plan.blk;
	auto time_plan = [&](Plan &pl, int reps, float *ms) -> pa_status {
		if (pa_status e = stage(pl)) return e;
		*ms = INFINITY;
		for (int rep = 0; rep < reps; rep++) {
			PA_CUDA(cudaEventRecord(s->ev[1], st));
			if (pa_status e = dp(pl, pl.tb, false, nullptr)) return e;
			PA_CUDA(cudaEventRecord(s->ev[2], st));
			PA_CUDA(cudaEventSynchronize(s->ev[2]));
			float t = 0;
			PA_CUDA(cudaEventElapsedTime(&t, s->ev[1], s->ev[2]));
			*ms = std::min(*ms, t);
		}
		return PA_OK;
	};
	std::vector<float> cand_ms(cand.size(), INFINITY);
	auto plan_of = [&](const Cand &c) {
		Plan pl = plan;
		pl.G = c.G;
		pl.units = c.units;
		pl.h16 = c.h16;
		pl.C = c.C;
		pl.blk = c.blk;
		pl.seg = false;
		return pl;
	};
	// untimed runs first, at least 3 and 30 ms of them (clocks and caches leave their idle
	// state: a first candidate timed on a cold GPU loses to a slower one timed warm), then
	// each candidate timed twice, keeping its faster run, and the two fastest timed twice
	// more, alternately, so neither is judged on one stretch of clock
	{
		Plan pl = plan_of(cand[0]);
		float spent = 0;
		for (int w = 0; w < 16 && (w < 3 || spent < 30.0f); w++) {
			float ms = INFINITY;
			if (pa_status e = time_plan(pl, 1, &ms)) return e;
			spent += ms;
		}
	}
	for (size_t ci = 0; ci < cand.size(); ci++) {
		Plan pl = plan_of(cand[ci]);
		if (pa_status e = time_plan(pl, 2, &cand_ms[ci])) return e;
	}
	if (cand.size() >= 2) {
		size_t a = 0, b = 1;
		if (cand_ms[b] < cand_ms[a]) std::swap(a, b);
		for (size_t ci = 2; ci < cand.size(); ci++) {
			if (cand_ms[ci] < cand_ms[a]) {
				b = a;
				a = ci;
			} else if (cand_ms[ci] < cand_ms[b]) {
				b = ci;
			}
		}
		for (int rep = 0; rep < 2; rep++)
			for (size_t ci : {a, b}) {
				Plan pl = plan_of(cand[ci]);
				float ms = INFINITY;
				if (pa_status e = time_plan(pl, 1, &ms)) return e;
				cand_ms[ci] = std::min(cand_ms[ci], ms);
			}
	}
	for (size_t ci = 0; ci < cand.size(); ci++) {
		if (cand_ms[ci] < best) {
			best = cand_ms[ci];
			bestG = cand[ci].G;
			bestU = cand[ci].units;
			bestH = cand[ci].h16;
			bestC = cand[ci].C;
			bestB = cand[ci].blk;
		}
	}
	plan.G = bestG;
	plan.units = bestU;
	plan.h16 = bestH;
	plan.C = bestC;
	plan.blk = bestB;
	plan.seg = false;
	if (bestH && !bestB && !bestU) {
		// a width per length bucket, by measurement: from the uniform plan, each populated
		// bucket in turn tries half the width (and half again while that helps), else twice
		// the width, keeping a change only when the whole launch runs at least 1% faster
		int bpop[PA_BUCKETS] = {};
		int64_t bmax[PA_BUCKETS] = {};
		for (size_t k = 0; k < ls.size(); k++) {
			if (ls[k] == 0 || lt[k] == 0) continue;
			const int b = bucket_of(ls[k]);
			bpop[b]++;
			bmax[b] = std::max<int64_t>(bmax[b], ls[k]);
		}
		int nb = 0;
		for (int b = 0; b < PA_BUCKETS; b++) nb += bpop[b] > 0;
		if (nb > 1) {
			Plan pl = plan;
			pl.seg = true;
			for (int b = 0; b < PA_BUCKETS; b++) pl.bucket_G[b] = bestG;
			float cur = best;
			bool changed = false;
			for (int b = 0; b < PA_BUCKETS; b++) {
				if (!bpop[b]) continue;
				// the widths the uniform candidates allow for this bucket's longest pair
				auto ok = [&](int g) {
					return g >= 1 && g <= 32 && (g == 4 || (int64_t(g) * R <= 2 * bmax[b] && (g >= 4 || bmax[b] <= 256)));
				};
				for (int dir : {-1, 1}) {
					for (int g = dir < 0 ? pl.bucket_G[b] / 2 : pl.bucket_G[b] * 2; ok(g); g = dir < 0 ? g / 2 : g * 2) {
						Plan t = pl;
						t.bucket_G[b] = g;
						float ms = INFINITY;
						if (pa_status e = time_plan(t, 2, &ms)) return e;
						if (!(ms < cur * 0.99f)) break;
						cur = ms;
						pl = t;
						changed = true;
					}
					if (pl.bucket_G[b] != bestG) break;  // narrower helped: no need to try wider
				}
			}
			if (changed) {
				best = cur;
				plan.seg = true;
				for (int b = 0; b < PA_BUCKETS; b++) plan.bucket_G[b] = pl.bucket_G[b];
			}
		}
	}
	std::lock_guard<std::mutex> lk(g_tune_mu);
	if (g_tune.size() < 4096) {
		TuneEntry t{key, bestG, bestU, bestH, bestC, bestB, plan.seg, {}};
		for (int b = 0; b < PA_BUCKETS; b++) t.bucket_G[b] = plan.bucket_G[b];
		g_tune.push_back(t);
	}
	return PA_OK;
}

pa_status solve_impl(pa_solver *s, const Input &in, int method, float *scores_out, pa_result **out,
                     int32_t *maps_out = nullptr, const int64_t *map_offsets = nullptr,
                     const UserPaths *user_paths = nullptr) {
	if (pa_status st = ensure_device(s)) return st;
	if (pa_status st = validate(s, in)) return st;
	cudaStream_t st = s->stream;
	s->bytes_h2d = s->bytes_d2h = 0;
	const int64_t B = in.batch;

	// per-lane lengths, clamped to the batch arrays (stale lanes of a partial batch carry
	// lengths beyond the master shape; the reference computes them from padding and the
	// Python layer discards them, solve.py:382-396, 554-560)
	std::vector<int32_t> &ls = s->h_ls, &lt = s->h_lt;
	ls.resize(size_t(B));  // every entry is written below
	lt.resize(size_t(B));
	int64_t max_ls = 0, max_lt = 0;
	{
		// int32 throughout, so the compiler vectorises the clamp and the maxima
		const int32_t cs = int32_t(std::min<int64_t>(in.n_s, INT32_MAX)), ct = int32_t(std::min<int64_t>(in.n_t, INT32_MAX));
		const int32_t *l0 = in.length, *l1 = in.length + B;
		int32_t *ps = ls.data(), *pt = lt.data();
		int32_t ms = 0, mt = 0;
		for (int64_t k = 0; k < B; k++) {
			const int32_t a = std::min(std::max(l0[k], 0), cs), b = std::min(std::max(l1[k], 0), ct);
			ps[k] = a;
			pt[k] = b;
			ms = std::max(ms, a);
			mt = std::max(mt, b);
		}
		max_ls = ms;
		max_lt = mt;
	}

	if (maps_out && map_offsets && in.location == PA_HOST) {
		// host maps are staged in a packed device buffer: the offsets must be the packed ones
		int64_t o = 0;
		for (int64_t k = 0; k < B; k++) {
			if (map_offsets[k] != o)
				return fail(PA_ERR_INVALID_ARGUMENT, "map_offsets must be the prefix sums of min(|s|, |t|)");
			o += std::min(ls[size_t(k)], lt[size_t(k)]);
		}
	}

	auto R_ = std::make_shared<ResultData>();
	ResultData &res = *R_;
	res.batch = B;  // (the lengths join the result at the end, when a result is returned)
	res.goal = s->goal;
	res.gap = s->gap;
	res.loc = s->loc;
	res.type = s->opt.type;
	res.remove_dup = s->opt.remove_dup;
	res.layers = s->gap == GAP_AFFINE ? 3 : 1;
	res.worst = -INFINITY * s->sign;
	res.method = method;
	res.sign = s->sign;
	for (int k = 0; k < 3; k++) res.alg[k] = s->alg[k];
	res.gen_s = s->gen_s;
	res.gen_t = s->gen_t;

	// what the method needs from the goal (factory.h:699-808, solver.h:2593-2740)
	const int goal = s->goal;
	int tb;
	if (goal == GOAL_SCORE) tb = TB_NONE;
	else if (goal == GOAL_ONE || method == M_PATHS) tb = (method == M_SCORE) ? TB_NONE : TB_ONE;
	else tb = method == M_SCORE ? TB_NONE : TB_ALL;
	const bool want_values = (method == M_SOLUTION || method == M_SOLUTION_ITER) && s->gap != GAP_GENERAL;
	const bool want_paths = method == M_SOLUTION || (goal == GOAL_ONE && method == M_SOLUTION_ITER) ||
	                        (goal == GOAL_ONE && method == M_ALIGNMENT_ITER) || method == M_PATHS;
	if (method == M_PATHS && s->gap == GAP_GENERAL)
		return fail(PA_ERR_UNSUPPORTED, "paths of general (WSB) gap costs are not produced on the device");

	cudaEventRecord(s->ev[0], st);
	int launches = 0;

	// the similarity table is small: keep a host copy (device-resident tables are read back)
	std::vector<float> host_table;
	if (in.form == F_INDEXED) {
		host_table.resize(size_t(in.table_rows * in.table_cols));
		if (in.location == PA_DEVICE) {
			// through the solver's pinned block (a pageable destination makes CUDA stage the copy)
			const size_t nb = host_table.size() * 4;
			PA_CUDA(s->h_out.ensure(nb + 16));
			PA_CUDA(pa_copy(s, s->h_out.p, in.table, nb, cudaMemcpyDeviceToHost, st));
			PA_CUDA(cudaStreamSynchronize(st));
			std::memcpy(host_table.data(), s->h_out.p, nb);
		} else if (!host_table.empty()) {
			std::memcpy(host_table.data(), in.table, host_table.size() * 4);
		}
	}

	// ---- repeated solves: the same solve as the last call on this solver (same lengths,
	// shapes, buffers, options, table, offsets and stream) skips planning and staging -- the
	// device metadata, converted table and plan of that call are still in place.  A repeated
	// device-resident solve runs, from its second repetition on, as one CUDA graph of the
	// device work, captured on a private stream; with host buffers the inputs are copied in
	// as always and the work is launched directly.  Any other call first drops the cached
	// state, since it rewrites the buffers the repeat reads.  PA_GRAPHS=0 turns this off.
	const char *genv = std::getenv("PA_GRAPHS");
	const bool repeatable = s->gap != GAP_GENERAL && tb != TB_ALL && !want_values &&
	                        (method == M_SCORE || method == M_ALIGNMENT || method == M_PATHS) &&
	                        !(genv && std::strcmp(genv, "0") == 0);
	const bool paths_to_user = method == M_PATHS && user_paths;
	auto same_rep = [&]() -> bool {
		const pa_solver::Repeat &r = s->rep;
		if (!r.valid || r.method != method || r.form != in.form || r.B != B || r.n_s != in.n_s || r.n_t != in.n_t)
			return false;
		if (r.sx != in.sx || r.sy != in.sy || r.sxs != in.sx_stride || r.sys != in.sy_stride) return false;
		if (r.a != in.a || r.b != in.b || r.sim != in.sim || r.table != in.table || r.trows != in.table_rows ||
		    r.tcols != in.table_cols || r.dsi != in.dense_si || r.dsj != in.dense_sj || r.stream != st)
			return false;
		if (std::memcmp(&r.eq, &in.eq, 4) || std::memcmp(&r.ne, &in.ne, 4)) return false;
		// device maps are written by the captured graph, so the buffer must be the same one;
		// host maps are copied out per call (any buffer with the same offsets will do)
		if ((in.location == PA_DEVICE && r.maps_out != maps_out) || r.ls != ls || r.lt != lt ||
		    r.table_host != host_table)
			return false;
		if (r.scores != (paths_to_user ? user_paths->scores : nullptr)) return false;
		if (paths_to_user && (r.paths != user_paths->paths || r.path_len != user_paths->path_len ||
		                      std::memcmp(r.user_path_off.data(), user_paths->path_off, size_t(B) * 8)))
			return false;
		if (maps_out && map_offsets && (r.user_map_off.size() != size_t(B) ||
		                                std::memcmp(r.user_map_off.data(), map_offsets, size_t(B) * 8)))
			return false;
		if (in.dense_off_host && (r.dense_off.size() != size_t(B) ||
		                          std::memcmp(r.dense_off.data(), in.dense_off_host, size_t(B) * 8)))
			return false;
		return true;
	};
	const bool hit = repeatable && same_rep();
	if (!hit) s->drop_graph();
	// a repeated solve with host buffers and many pairs runs as a pipeline of chunks (see
	// below): its uploads and index checks happen chunk by chunk there
	const bool chunked = hit && in.location == PA_HOST && s->rep.nchunks > 1;

	// ---- upload inputs
	if (in.location == PA_HOST && !chunked) {
		if (in.form == F_DENSE) {
			const size_t n = size_t(in.n_s * in.n_t * B) * sizeof(float);
			PA_CUDA(s->d_dense.ensure(n));
			if (n) PA_CUDA(pa_copy(s, s->d_dense.p, in.sim, n, cudaMemcpyHostToDevice, st));
		} else {
			const size_t na = size_t(B * in.n_s) * sizeof(uint32_t), nb = size_t(B * in.n_t) * sizeof(uint32_t);
			PA_CUDA(s->d_a.ensure(na));
			PA_CUDA(s->d_b.ensure(nb));
			if (na) PA_CUDA(pa_copy(s, s->d_a.p, in.a, na, cudaMemcpyHostToDevice, st));
			if (nb) PA_CUDA(pa_copy(s, s->d_b.p, in.b, nb, cudaMemcpyHostToDevice, st));
		}
	}
	if (in.form == F_INDEXED && !chunked) {
		// codes must index the table (factory.h:602-614); checked on the device
		PA_CUDA(s->d_codes_max.ensure(8));
		PA_CUDA(cudaMemsetAsync(s->d_codes_max.p, 0, 8, st));
		const uint32_t *da = in.location == PA_DEVICE ? in.a : s->d_a.as<uint32_t>();
		const uint32_t *db = in.location == PA_DEVICE ? in.b : s->d_b.as<uint32_t>();
		const int grid = std::max(1, std::min(s->sm_count * 4, int((B * std::max(in.n_s, in.n_t) + 255) / 256)));
		if (B * in.n_s > 0) codes_max_kernel<<<grid, 256, 0, st>>>(da, B * in.n_s, s->d_codes_max.as<uint32_t>());
		if (B * in.n_t > 0) codes_max_kernel<<<grid, 256, 0, st>>>(db, B * in.n_t, s->d_codes_max.as<uint32_t>() + 1);
		PA_CUDA(cudaGetLastError());
		launches += int(B * in.n_s > 0) + int(B * in.n_t > 0);
		// no wait here: the DP kernels read the maxima at launch and do nothing (ST_BAD_CODE)
		// when a code is out of bounds; the error is raised after the solve's one sync
	}


	// ---- plan: group width and mode, arithmetic; the tuner may try several plans
	// (a repeated solve takes the plan of the call it repeats: no planning)
	Plan plan;
	plan.max_ls = max_ls;
	plan.max_lt = max_lt;
	plan.tb = tb;
	if (!hit) plan.G = choose_G(ls, lt, s->sm_count);
	if (!hit && s->gap != GAP_GENERAL) {
		plan.units = choose_units(ls, lt, s->sm_count, plan.G);
		if (plan.units) plan.G = 32;
		double bound = 0;
		bool use_int = int_mode_ok(s, in, host_table.data(), max_ls, max_lt, &bound);
		if (use_int && s->loc == LOC_LOCAL && tb == TB_ONE) {
			// local seeds are packed as value * 2^shift + j in an int32
			int shift = 1;
			while ((int64_t(1) << shift) <= max_lt) shift++;
			plan.key_shift = shift;
			if ((bound * 4.0 + 4.0) * double(int64_t(1) << shift) >= 2147483647.0) use_int = false;
		}
		plan.use_int = use_int;
		plan.C = cols2_ok(plan, want_values) ? 2 : 1;
		if (const char *e = std::getenv("PA_DP_COLS"))  // experiments and tests
			if (std::atoi(e) == 1) plan.C = 1;
		int32_t hneg = 0;
		plan.C32 = plan.C;
		plan.h16 = !plan.units && h16_plan(s, in, host_table.data(), ls, lt, tb, want_values, use_int, &hneg);
		plan.h_neg = hneg;
		if (plan.h16) plan.C = plan.C32;  // two columns per step unless PA_DP_COLS=1
		if (const char *e = std::getenv("PA_DP_BLOCK"))  // experiments and tests: the 4 x 4 block kernel
			if (plan.h16 && std::strcmp(e, "1") == 0) {
				plan.blk = true;
				plan.C = 4;
			}
		if (const char *e = std::getenv("PA_BUCKET_WIDTHS"))  // experiments and tests: "g0,g1,g2,g3"
			if (plan.h16 && !plan.blk && parse_bucket_widths(e, plan.bucket_G)) plan.seg = true;
	}
	std::vector<int32_t> order, level_start;
	std::vector<int8_t> pair_g;  // group width per pair (length buckets)
	std::vector<int64_t> mask_off, map_off, path_off, val_off, dense_off;
	struct Lend {  // a repeat's offsets lent to this call, returned however the call ends
		pa_solver::Repeat *r = nullptr;
		std::vector<int64_t> *mo, *mp, *po, *vo;
		~Lend() {
			if (!r) return;
			r->mask_off.swap(*mo);
			r->map_off.swap(*mp);
			r->path_off.swap(*po);
			r->val_off.swap(*vo);
		}
	} lend{nullptr, &mask_off, &map_off, &path_off, &val_off};
	// per-pair metadata of a plan: processing order, stripe tickets, output offsets, staged
	// to the device; output buffers sized
	auto stage = [&](Plan &plan) -> pa_status {
		// processing order: by number of stripes, then |t|, largest first (a counting sort), so
		// the groups that share a warp get pairs of the same shape and long pairs start early
		// (a pipelined solve sorts each chunk's pair range on its own: chunk c's pairs occupy
		// order[k0, k1) for its pair indices [k0, k1))
		order.assign(size_t(B), 0);
		pair_g.assign(size_t(B), int8_t(plan.G));
		if (!plan.seg) {
			{
				const int64_t rpp = int64_t(plan.G) * plan_rows(plan);
				const int64_t kt = max_lt + 1;
				const int64_t nkeys = ((max_ls + rpp - 1) / rpp + 1) * kt;
				std::vector<int32_t> count(size_t(nkeys) + 1);
				auto key = [&](int64_t k) {
					const int64_t np = (ls[size_t(k)] + rpp - 1) / rpp;
					return nkeys - 1 - (np * kt + lt[size_t(k)]);  // descending
				};
				for (int c = 0; c < plan.nchunks; c++) {
					int64_t k0, k1;
					chunk_range(B, plan.nchunks, c, k0, k1);
					std::fill(count.begin(), count.end(), 0);
					for (int64_t k = k0; k < k1; k++) count[size_t(key(k)) + 1]++;
					count[0] = int32_t(k0);
					for (int64_t c2 = 0; c2 < nkeys; c2++) count[size_t(c2) + 1] += count[size_t(c2)];
					for (int64_t k = k0; k < k1; k++) order[size_t(count[size_t(key(k))]++)] = int32_t(k);
				}
			}
		} else {
			// length buckets: within each chunk the pairs bucket by bucket (the longest first),
			// each bucket by its stripe count at the bucket's width and |t|, largest first; a
			// segment of one width per bucket, starting at an even position (a twin never
			// straddles two widths: an odd bucket lends the next bucket's first pair)
			std::vector<int32_t> idx;
			for (int c = 0; c < plan.nchunks; c++) {
				int64_t k0, k1;
				chunk_range(B, plan.nchunks, c, k0, k1);
				idx.resize(size_t(k1 - k0));
				for (int64_t k = k0; k < k1; k++) idx[size_t(k - k0)] = int32_t(k);
				auto np_of = [&](int32_t k) {
					const int64_t g = plan.bucket_G[bucket_of(ls[size_t(k)])], rpp = g * plan_rows(plan);
					return (ls[size_t(k)] + rpp - 1) / rpp;
				};
				std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) {
					const int bx = bucket_of(ls[size_t(x)]), by = bucket_of(ls[size_t(y)]);
					if (bx != by) return bx > by;
					const int64_t nx = np_of(x), ny = np_of(y);
					if (nx != ny) return nx > ny;
					return lt[size_t(x)] > lt[size_t(y)];
				});
				for (size_t i = 0; i < idx.size(); i++) order[size_t(k0) + i] = idx[i];
				SegInfo &sg = plan.segs[c];
				sg = SegInfo();
				const int64_t n = k1 - k0;
				int64_t pos = 0;
				while (pos < n) {
					const int bk = bucket_of(ls[size_t(idx[size_t(pos)])]);
					const int g = plan.bucket_G[bk];
					int64_t e = pos;
					while (e < n && bucket_of(ls[size_t(idx[size_t(e)])]) == bk) e++;
					if (e < n && (e & 1)) e++;
					for (int64_t i = pos; i < e; i++) pair_g[size_t(idx[size_t(i)])] = int8_t(g);
					const int64_t units = (e + 1) / 2 - pos / 2, per = 32 / g;
					sg.G[sg.nseg] = g;
					sg.unit[sg.nseg] = int(pos / 2);
					sg.task[sg.nseg + 1] = sg.task[sg.nseg] + int((units + per - 1) / per);
					sg.Gmin = std::min(sg.Gmin, g);
					sg.nseg++;
					pos = e;
				}
				sg.unit[sg.nseg] = int((n + 1) / 2);
			}
		}
		// stripe-chained tickets: level q holds stripe q of every pair with more than q stripes
		// (an empty pair counts as one stripe, which writes its border result); the order puts
		// those pairs first, so stripe q of rank w is ticket level_start[q] + w
		level_start.clear();
		if (plan.units) {
			const int64_t rpp_u = int64_t(plan.G) * R;
			std::vector<int64_t> hist;
			for (int64_t k = 0; k < B; k++) {
				const int64_t np = std::max<int64_t>(1, (ls[size_t(k)] + rpp_u - 1) / rpp_u);
				if (int64_t(hist.size()) <= np) hist.resize(size_t(np) + 1, 0);
				hist[size_t(np)]++;
			}
			const int64_t nlev = int64_t(hist.size()) - 1;
			level_start.assign(size_t(nlev) + 1, 0);
			int64_t above = B;  // pairs with more than q stripes
			for (int64_t q = 0; q < nlev; q++) {
				level_start[size_t(q) + 1] = int32_t(level_start[size_t(q)] + above);
				above -= hist[size_t(q) + 1];
			}
			if (int64_t(level_start.back()) >= (int64_t(1) << 31) - 64) return fail(PA_ERR_LENGTH, "too many stripes in one launch");
			plan.nlevels = int32_t(nlev);
			plan.ntickets = level_start.back();
		}
		mask_off.assign(size_t(B) + 1, 0);
		map_off.assign(size_t(B) + 1, 0);
		path_off.assign(size_t(B) + 1, 0);
		val_off.assign(size_t(B) + 1, 0);
		dense_off.assign(size_t(B), 0);
		for (int64_t k = 0; k < B; k++) {
			const int64_t a = ls[size_t(k)], b = lt[size_t(k)];
			const int64_t gk = pair_g[size_t(k)], rpp = gk * plan_rows(plan);
			const int64_t npass = (a == 0 || b == 0) ? 0 : (a + rpp - 1) / rpp;
			const int64_t steps = (b + plan.C - 1) / plan.C + gk - 1;
			mask_off[size_t(k) + 1] = mask_off[size_t(k)] + npass * steps * gk * plan_words(plan);
			map_off[size_t(k) + 1] = map_off[size_t(k)] + std::min(a, b);
			path_off[size_t(k) + 1] = path_off[size_t(k)] + 2 * (a + b + 2);
			val_off[size_t(k) + 1] = val_off[size_t(k)] + int64_t(res.layers) * (a + 1) * (b + 1);
			dense_off[size_t(k)] = in.dense_off_host ? in.dense_off_host[k] : k;
		}
		// pair metadata: packed into one pinned staging buffer, one host-to-device copy
		{
			const size_t n32 = size_t(B), n64 = size_t(B) + 1;
			const size_t bytes = ((3 * n32 * 4 + level_start.size() * 4 + 7) & ~size_t(7)) + 5 * n64 * 8 + 16 + n32 + 8;
			if (s->meta_pending) {
				PA_CUDA(cudaEventSynchronize(s->meta_ev));  // the previous call's copy has read it
				s->meta_pending = false;
			}
			PA_CUDA(s->h_meta.ensure(bytes));
			PA_CUDA(s->d_meta.ensure(bytes));
			unsigned char *h = s->h_meta.as<unsigned char>();
			unsigned char *d = s->d_meta.as<unsigned char>();
			size_t o = 0;
			auto put = [&](const void *src, size_t nbytes, size_t align) {
				o = (o + align - 1) & ~(align - 1);
				if (nbytes) std::memcpy(h + o, src, nbytes);
				unsigned char *dp = d + o;
				o += nbytes;
				return dp;
			};
			s->m.ls = reinterpret_cast<int32_t *>(put(ls.data(), n32 * 4, 4));
			s->m.lt = reinterpret_cast<int32_t *>(put(lt.data(), n32 * 4, 4));
			s->m.order = reinterpret_cast<int32_t *>(put(order.data(), n32 * 4, 4));
			s->m.level_start = reinterpret_cast<int32_t *>(put(level_start.data(), level_start.size() * 4, 4));
			s->m.mask_off = reinterpret_cast<int64_t *>(put(mask_off.data(), n64 * 8, 8));
			// the caller's output offsets replace the internal ones when results go to its buffers
			const int64_t *mo = (maps_out && map_offsets) ? map_offsets : map_off.data();
			s->m.map_off = reinterpret_cast<int64_t *>(put(mo, (maps_out && map_offsets ? n32 : n64) * 8, 8));
			o += (maps_out && map_offsets) ? 8 : 0;
			const int64_t *po = (method == M_PATHS && user_paths) ? user_paths->path_off : path_off.data();
			s->m.path_off = reinterpret_cast<int64_t *>(put(po, (method == M_PATHS && user_paths ? n32 : n64) * 8, 8));
			o += (method == M_PATHS && user_paths) ? 8 : 0;
			s->m.val_off = reinterpret_cast<int64_t *>(put(val_off.data(), n64 * 8, 8));
			s->m.dense_off = reinterpret_cast<int64_t *>(put(dense_off.data(), n32 * 8, 8));
			o += 8;
			s->m.pair_G = reinterpret_cast<int8_t *>(put(pair_g.data(), n32, 1));
			PA_CUDA(pa_copy(s, d, h, o, cudaMemcpyHostToDevice, st));
			PA_CUDA(cudaEventRecord(s->meta_ev, st));
			s->meta_pending = true;
		}
		PA_CUDA(s->d_score.ensure(size_t(B) * 4));
		PA_CUDA(s->d_seed.ensure(size_t(B) * 8));
		PA_CUDA(s->d_has.ensure(size_t(B) * 4));
		PA_CUDA(s->d_counter.ensure(4));
		PA_CUDA(s->d_status.ensure(4));
		PA_CUDA(cudaMemsetAsync(s->d_status.p, 0, 4, st));
		const size_t mask_elem = tb == TB_ALL ? 16 : 4;
		if (tb != TB_NONE) PA_CUDA(s->d_masks.ensure(size_t(mask_off[size_t(B)]) * mask_elem));
		if (want_values) PA_CUDA(s->d_vals.ensure(size_t(val_off[size_t(B)]) * 4));
		return PA_OK;
	};
	auto dp = [&](const Plan &pl, int tbk, bool vals, const float *best_in) -> pa_status {
		if (pl.seg && pl.h16 && !pl.blk && pl.nchunks > 1) {
			// length buckets of a chunk-major order: one launch per chunk, each over its own
			// segments (a whole-bag launch has none: segments do not cross chunks)
			for (int c = 0; c < pl.nchunks; c++) {
				int64_t k0, k1;
				chunk_range(B, pl.nchunks, c, k0, k1);
				if (k1 > k0)
					if (pa_status e = run_dp<int32_t>(s, in, pl, tbk, host_table.data(), k1 - k0, vals, best_in,
					                                  &launches, k0, 0, 0, c))
						return e;
			}
			return PA_OK;
		}
		return pl.use_int ? run_dp<int32_t>(s, in, pl, tbk, host_table.data(), B, vals, best_in, &launches)
		                  : run_dp<float>(s, in, pl, tbk, host_table.data(), B, vals, best_in, &launches);
	};

	const bool need_walk = tb == TB_ONE && s->gap != GAP_GENERAL &&
	                       (method == M_ALIGNMENT || method == M_ALIGNMENT_ITER || method == M_SOLUTION ||
	                        method == M_SOLUTION_ITER || method == M_PATHS);
	// general gap costs, one alignment per pair: walked on the device (wsb_walk_kernel); the
	// cell matrices stay there, as they do for a score-only solve (the iterators, solutions and
	// all-optimal searches walk them on the host)
	const bool wsb_maps = s->gap == GAP_GENERAL && tb == TB_ONE && method == M_ALIGNMENT;
	const bool wsb_host = s->gap == GAP_GENERAL && !(goal != GOAL_ALL && (method == M_SCORE || wsb_maps));
	// the device work after staging: status reset, DP, traceback walk, the scores of the
	// device-resident path form.  The phase events are recorded in it; inside a capture they
	// become external event nodes of the graph, so the timings stay exact on replays.
	auto record = [&](cudaEvent_t e, cudaStream_t sw) -> cudaError_t {
		return s->capturing ? cudaEventRecordWithFlags(e, sw, cudaEventRecordExternal) : cudaEventRecord(e, sw);
	};
	// the traceback walk of all pairs (pair0 / npairs select a range)
	auto walk_params = [&]() -> WalkParams {
		const bool to_user = maps_out && in.location == PA_DEVICE;
		WalkParams w{};
		w.npairs = int32_t(B);
		w.len_s = s->m.ls;
		w.len_t = s->m.lt;
		w.seed = s->d_seed.as<int32_t>();
		w.has_seed = s->d_has.as<int32_t>();
		w.masks = s->d_masks.as<uint32_t>();
		w.mask_off = s->m.mask_off;
		w.G = plan.G;
		w.cols = plan.C;
		w.fmt16 = plan.h16 ? 1 : 0;
		w.rows4 = plan.blk ? 1 : 0;
		w.pair_G = plan.seg ? s->m.pair_G : nullptr;
		w.status = s->d_status.as<int32_t>();
		w.gap = s->gap;
		w.local = s->loc == LOC_LOCAL;
		w.maps = to_user ? maps_out : s->d_maps.as<int32_t>();
		w.map_off = s->m.map_off;
		w.paths = want_paths ? s->d_paths.as<int32_t>() : nullptr;
		w.path_off = s->m.path_off;
		w.path_len = want_paths ? s->d_path_len.as<int32_t>() : nullptr;
		if (paths_to_user) {
			w.maps = nullptr;
			w.paths = user_paths->paths;
			w.path_len = user_paths->path_len;
		}
		return w;
	};
	auto ensure_walk_buffers = [&]() -> cudaError_t {
		cudaError_t e = s->d_maps.ensure(size_t(map_off[size_t(B)]) * 4);
		if (e == cudaSuccess && want_paths) e = s->d_paths.ensure(size_t(path_off[size_t(B)]) * 4);
		if (e == cudaSuccess && want_paths) e = s->d_path_len.ensure(size_t(B) * 4);
		return e;
	};
	auto device_work = [&](cudaStream_t sw, bool timed) -> pa_status {
		PA_CUDA(cudaMemsetAsync(s->d_status.p, 0, 4, sw));
		if (timed) PA_CUDA(record(s->ev[1], sw));
		if (s->gap == GAP_GENERAL) {
			int32_t *wmaps = nullptr;
			if (wsb_maps) {
				if (maps_out && in.location == PA_DEVICE) {
					wmaps = maps_out;
				} else {
					PA_CUDA(s->d_maps.ensure(size_t(std::max<int64_t>(map_off[size_t(B)], 1)) * 4));
					wmaps = s->d_maps.as<int32_t>();
				}
			}
			if (pa_status e = run_wsb(s, in, ls, lt, &launches, res, wmaps)) return e;
		} else {
			if (tb == TB_ALL && s->loc == LOC_LOCAL) {
				// the optimum is needed to mark the seeds (solver.h:2066-2091): a score pass first
				if (pa_status e2 = dp(plan, TB_NONE, false, nullptr)) return e2;
				PA_CUDA(s->d_best.ensure(size_t(B) * 4));
				PA_CUDA(pa_copy(s, s->d_best.p, s->d_score.p, size_t(B) * 4, cudaMemcpyDeviceToDevice, sw));
			}
			if (pa_status e2 = dp(plan, tb, want_values, s->d_best.as<float>())) return e2;
		}
		if (timed) PA_CUDA(record(s->ev[2], sw));
		if (need_walk) {
		PA_CUDA(ensure_walk_buffers());
		WalkParams w = walk_params();
		walk_kernel<<<int((B + 3) / 4), 128, 0, sw>>>(w);  // a warp per pair
		PA_CUDA(cudaGetLastError());
		launches++;
		}
		if (paths_to_user && user_paths->scores)
			PA_CUDA(cudaMemcpyAsync(user_paths->scores, s->d_score.p, size_t(B) * 4, cudaMemcpyDeviceToDevice, sw));
		return PA_OK;
	};
	// A repeated solve with host buffers and many pairs, as a pipeline of nchunks pair ranges
	// (the staged order is chunk-major: chunk c's pairs [k0, k1) occupy order[k0, k1)).  The
	// copy stream uploads each chunk's codes; the solver's stream, per chunk once its codes
	// are in, checks their range and runs the DP and the walk over the chunk's pairs; the copy
	// stream then downloads the chunk's alignment maps.  Uploads of later chunks and downloads
	// of earlier ones overlap the computation.  Per-chunk index checks write their own maxima
	// slot, which that chunk's DP launch reads.
	auto pipeline = [&]() -> pa_status {
		const int K = plan.nchunks;
		if (!s->copy_stream) PA_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
		if (!s->cmp2) PA_CUDA(cudaStreamCreateWithFlags(&s->cmp2, cudaStreamNonBlocking));
		while (int(s->ev_chunk.size()) < 2 * K + 4) {
			cudaEvent_t e = nullptr;
			PA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
			s->ev_chunk.push_back(e);
		}
		cudaStream_t cs = s->copy_stream;
		const cudaStream_t side_stream[2] = {st, s->cmp2};
		cudaEvent_t *ev = s->ev_chunk.data();  // uploads 0..K-1, walks K..2K-1, then 4 joins
		cudaEvent_t ev_start = ev[2 * K], ev_table = ev[2 * K + 1], ev_cmp2 = ev[2 * K + 2], ev_copy = ev[2 * K + 3];
		PA_CUDA(s->d_a.ensure(size_t(B * in.n_s) * 4));
		PA_CUDA(s->d_b.ensure(size_t(B * in.n_t) * 4));
		PA_CUDA(s->d_codes_max.ensure(size_t(8 * K)));
		if (need_walk) PA_CUDA(ensure_walk_buffers());
		int32_t *maps_host = nullptr;
		if (need_walk) {
			if (!maps_out) res.maps.resize(size_t(map_off[size_t(B)]));
			maps_host = maps_out ? maps_out : res.maps.data();
		}
		auto range = [&](int c, int64_t &k0, int64_t &k1) { chunk_range(B, K, c, k0, k1); };
		// page-locked codes are all queued for upload at once; a copy from pageable codes holds
		// this thread until the copy engine has them, so each chunk's upload is issued just
		// before that chunk's work (the GPU computes the chunks before it meanwhile).  Maps
		// go to a page-locked buffer chunk by chunk behind each walk; to pageable memory (or
		// while uploads still follow on the copy stream) in one copy at the end.
		const bool pin_in = host_pinned(in.a) && host_pinned(in.b);
		const bool defer_maps = need_walk && (!pin_in || !host_pinned(maps_host));
		auto upload = [&](int c) -> cudaError_t {
			int64_t k0, k1;
			range(c, k0, k1);
			cudaError_t e = cudaSuccess;
			if (in.n_s && k1 > k0)
				e = pa_copy(s, s->d_a.as<uint32_t>() + k0 * in.n_s, in.a + k0 * in.n_s, size_t((k1 - k0) * in.n_s) * 4,
				            cudaMemcpyHostToDevice, cs);
			if (e == cudaSuccess && in.n_t && k1 > k0)
				e = pa_copy(s, s->d_b.as<uint32_t>() + k0 * in.n_t, in.b + k0 * in.n_t, size_t((k1 - k0) * in.n_t) * 4,
				            cudaMemcpyHostToDevice, cs);
			if (e == cudaSuccess) e = cudaEventRecord(ev[c], cs);
			return e;
		};
		// the copy stream and the second compute stream start after the work already queued on
		// the solver's stream, and after this call's status reset
		PA_CUDA(cudaMemsetAsync(s->d_status.p, 0, 4, st));
		PA_CUDA(cudaEventRecord(ev_start, st));
		PA_CUDA(cudaStreamWaitEvent(cs, ev_start, 0));
		PA_CUDA(cudaStreamWaitEvent(s->cmp2, ev_start, 0));
		if (pin_in)
			for (int c = 0; c < K; c++) PA_CUDA(upload(c));
		PA_CUDA(cudaEventRecord(s->ev[1], st));
		// even chunks on the solver's stream, odd ones on the second compute stream: a chunk's
		// launch fills the SMs that the previous chunk's tail leaves idle
		pa_status err = PA_OK;
		for (int c = 0; c < K && err == PA_OK; c++) {
			int64_t k0, k1;
			range(c, k0, k1);
			const int side = c & 1;
			const cudaStream_t sc = side_stream[side];
			if (!pin_in) PA_CUDA(upload(c));
			PA_CUDA(cudaStreamWaitEvent(sc, ev[c], 0));
			if (in.form == F_INDEXED) {
				uint32_t *mx = s->d_codes_max.as<uint32_t>() + 2 * c;
				PA_CUDA(cudaMemsetAsync(mx, 0, 8, sc));
				const int64_t na = (k1 - k0) * in.n_s, nb = (k1 - k0) * in.n_t;
				const int grid = std::max(1, std::min(s->sm_count * 4, int((std::max(na, nb) + 255) / 256)));
				if (na > 0) codes_max_kernel<<<grid, 256, 0, sc>>>(s->d_a.as<uint32_t>() + k0 * in.n_s, na, mx);
				if (nb > 0) codes_max_kernel<<<grid, 256, 0, sc>>>(s->d_b.as<uint32_t>() + k0 * in.n_t, nb, mx + 1);
				PA_CUDA(cudaGetLastError());
				launches += int(na > 0) + int(nb > 0);
			}
			if (c == 1) PA_CUDA(cudaStreamWaitEvent(sc, ev_table, 0));  // the table chunk 0 uploaded
			if (k1 > k0) {
				// chunk 0 converts and uploads the table; the others reuse it
				s->table_ev = c == 0 ? ev_table : nullptr;
				s->skip_table = c > 0;
				err = plan.use_int ? run_dp<int32_t>(s, in, plan, tb, host_table.data(), k1 - k0, false, nullptr,
				                                     &launches, k0, c, side)
				                   : run_dp<float>(s, in, plan, tb, host_table.data(), k1 - k0, false, nullptr,
				                                   &launches, k0, c, side);
				s->table_ev = nullptr;
				s->skip_table = false;
				if (err) break;
			} else if (c == 0) {
				PA_CUDA(cudaEventRecord(ev_table, sc));
			}
			if (need_walk && k1 > k0) {
				WalkParams w = walk_params();
				w.pair0 = int32_t(k0);
				w.npairs = int32_t(k1 - k0);
				walk_kernel<<<int((k1 - k0 + 3) / 4), 128, 0, sc>>>(w);
				PA_CUDA(cudaGetLastError());
				launches++;
				if (!defer_maps) {
					PA_CUDA(cudaEventRecord(ev[K + c], sc));
					PA_CUDA(cudaStreamWaitEvent(cs, ev[K + c], 0));
					const int64_t m0 = map_off[size_t(k0)], m1 = map_off[size_t(k1)];
					if (m1 > m0)
						PA_CUDA(pa_copy(s, maps_host + m0, s->d_maps.as<int32_t>() + m0, size_t(m1 - m0) * 4,
						                cudaMemcpyDeviceToHost, cs));
				}
			}
		}
		// join: the solver's stream continues after the second compute stream and the copies
		PA_CUDA(cudaEventRecord(ev_cmp2, s->cmp2));
		PA_CUDA(cudaStreamWaitEvent(st, ev_cmp2, 0));
		PA_CUDA(cudaEventRecord(s->ev[2], st));
		PA_CUDA(cudaEventRecord(ev_copy, cs));
		PA_CUDA(cudaStreamWaitEvent(st, ev_copy, 0));
		if (err == PA_OK && defer_maps && map_off[size_t(B)] > 0)
			PA_CUDA(pa_copy(s, maps_host, s->d_maps.as<int32_t>(), size_t(map_off[size_t(B)]) * 4,
			                cudaMemcpyDeviceToHost, st));
		return err;
	};

	if (hit) {
		pa_solver::Repeat &r = s->rep;
		plan.G = r.G;
		plan.C = r.C;
		plan.h16 = r.h16;
		plan.blk = r.blk;
		plan.seg = r.seg;
		for (int k = 0; k < PA_BUCKETS; k++) plan.bucket_G[k] = r.bucket_G[k];
		for (int c = 0; c < PA_MAX_CHUNKS; c++) plan.segs[c] = r.segs[c];
		plan.h_neg = r.h_neg;
		plan.nchunks = r.nchunks;
		plan.units = r.units;
		plan.use_int = r.use_int;
		plan.key_shift = r.key_shift;
		plan.ntickets = r.ntickets;
		plan.nlevels = r.nlevels;
		// the staged offsets of the last call, lent to this one (swapped back on every return)
		mask_off.swap(r.mask_off);
		map_off.swap(r.map_off);
		path_off.swap(r.path_off);
		val_off.swap(r.val_off);
		lend.r = &r;
		if (chunked) {
			if (pa_status e = pipeline()) return e;
		} else if (in.location == PA_HOST) {
			// host buffers: the inputs were copied to the solver's own buffers above; the plan
			// and the staged metadata of the last call are reused, the work is launched as is
			if (pa_status e = device_work(st, true)) return e;
		} else if (!r.exec) {
			// second identical solve: capture its device work once, then launch it as a graph
			if (!s->cap_stream) PA_CUDA(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
			cudaGraph_t graph = nullptr;
			const cudaStream_t saved = s->stream;
			int before = launches;
			PA_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
			s->stream = s->cap_stream;
			s->capturing = true;
			pa_status e = device_work(s->cap_stream, true);
			s->capturing = false;
			s->stream = saved;
			const cudaError_t ce = cudaStreamEndCapture(s->cap_stream, &graph);
			if (e == PA_OK && ce == cudaSuccess && graph) {
				if (cudaGraphInstantiate(&r.exec, graph, 0) != cudaSuccess) r.exec = nullptr;
			}
			if (graph) cudaGraphDestroy(graph);
			cudaGetLastError();  // a failed capture leaves no sticky error
			r.launches = launches - before;
			launches = before;
			if (!r.exec) {
				s->drop_graph();
				return fail(PA_ERR_CUDA, "capturing the repeated solve as a CUDA graph failed (PA_GRAPHS=0 disables it)");
			}
		}
		if (in.location == PA_DEVICE) {
			PA_CUDA(cudaGraphLaunch(r.exec, st));  // records ev[1], ev[2] around the DP
			launches += r.launches;
		}
	} else {
		if (s->gap != GAP_GENERAL && tb != TB_ALL && !want_values) {
			if (pa_status e = tune_plan(s, ls, lt, in, plan, stage, dp)) return e;
		}
		// host buffers and many pairs: the repeats of this solve run as a pipeline of chunks
		// (3 chunks from 32K pairs, 2 from 8K; PA_CHUNKS overrides, up to 12); host maps use
		// the packed offsets (checked above)
		plan.nchunks = 1;
		if (repeatable && in.location == PA_HOST && in.form != F_DENSE && !plan.units && !want_paths) {
			int K = B >= 32768 ? 3 : B >= 8192 ? 2 : 1;
			if (const char *e = std::getenv("PA_CHUNKS")) K = std::atoi(e);
			K = std::min(K, 12);
			if (K > 1 && B >= (int64_t(1) << K)) plan.nchunks = K;
		}
		if (pa_status e = stage(plan)) return e;
		if (pa_status e = device_work(st, true)) return e;
	}
	res.G = plan.G;
	s->last_plan[0] = s->gap == GAP_GENERAL ? 4
	                  : plan.h16  ? (plan.blk ? 6 : plan.C == 2 ? 5 : 3)
	                  : plan.units ? 2
	                  : plan.C == 2 ? 1
	                               : 0;
	s->last_plan[1] = plan.G;
	s->last_plan[2] = plan.h16 ? 2 : plan.use_int ? 1 : 0;
	s->last_plan[3] = hit && s->rep.exec ? 1 : 0;
	for (int k = 0; k < PA_BUCKETS; k++) s->last_widths[k] = plan.seg ? plan.bucket_G[k] : 0;
	PA_CUDA(cudaEventRecord(s->ev[3], st));
	if (repeatable && !hit) {
		// remember this solve for the next call
		pa_solver::Repeat &r = s->rep;
		r.valid = true;
		r.method = method;
		r.form = in.form;
		r.B = B;
		r.n_s = in.n_s;
		r.n_t = in.n_t;
		r.trows = in.table_rows;
		r.tcols = in.table_cols;
		r.dsi = in.dense_si;
		r.dsj = in.dense_sj;
		r.a = in.a;
		r.b = in.b;
		r.sim = in.sim;
		r.sx = in.sx;
		r.sy = in.sy;
		r.sxs = in.sx_stride;
		r.sys = in.sy_stride;
		r.table = in.table;
		r.eq = in.eq;
		r.ne = in.ne;
		r.stream = st;
		r.maps_out = maps_out;
		r.scores = paths_to_user ? user_paths->scores : nullptr;
		r.paths = paths_to_user ? user_paths->paths : nullptr;
		r.path_len = paths_to_user ? user_paths->path_len : nullptr;
		r.ls = ls;
		r.lt = lt;
		r.table_host = host_table;
		r.user_map_off.assign(maps_out && map_offsets ? map_offsets : nullptr,
		                      maps_out && map_offsets ? map_offsets + B : nullptr);
		r.user_path_off.assign(paths_to_user ? user_paths->path_off : nullptr,
		                       paths_to_user ? user_paths->path_off + B : nullptr);
		r.dense_off.assign(in.dense_off_host ? in.dense_off_host : nullptr,
		                   in.dense_off_host ? in.dense_off_host + B : nullptr);
		r.G = plan.G;
		r.C = plan.C;
		r.h16 = plan.h16;
		r.blk = plan.blk;
		r.seg = plan.seg;
		for (int k = 0; k < PA_BUCKETS; k++) r.bucket_G[k] = plan.bucket_G[k];
		for (int c = 0; c < PA_MAX_CHUNKS; c++) r.segs[c] = plan.segs[c];
		r.h_neg = plan.h_neg;
		r.nchunks = plan.nchunks;
		r.units = plan.units;
		r.use_int = plan.use_int;
		r.key_shift = plan.key_shift;
		r.ntickets = plan.ntickets;
		r.nlevels = plan.nlevels;
		r.mask_off = mask_off;
		r.map_off = map_off;
		r.path_off = path_off;
		r.val_off = val_off;
		r.exec = nullptr;
	}

	if (paths_to_user) {
		// device-resident form: results stay on the device, nothing to wait for here
		s->last_launches = launches;
		for (auto &ms : s->last_ms) ms = 0.0f;
		s->dp_timing_pending = true;  // the DP's phase events, read without a wait here
		if (out) *out = nullptr;
		return PA_OK;
	}

	// ---- download: the status word, and the per-pair scores and seeds where the host needs
	// them (a result object, or host scores), through the solver's pinned block
	const bool host_scores = out != nullptr || scores_out != nullptr || (goal == GOAL_ALL && method == M_SCORE);
	const size_t hb = 16 + (host_scores ? size_t(B) * 4 : 0) + (out ? size_t(B) * 12 : 0);
	PA_CUDA(s->h_out.ensure(hb));
	unsigned char *hp = s->h_out.as<unsigned char>();
	PA_CUDA(pa_copy(s, hp, s->d_status.p, 4, cudaMemcpyDeviceToHost, st));
	if (host_scores) PA_CUDA(pa_copy(s, hp + 16, s->d_score.p, size_t(B) * 4, cudaMemcpyDeviceToHost, st));
	if (out) {
		PA_CUDA(pa_copy(s, hp + 16 + size_t(B) * 4, s->d_has.p, size_t(B) * 4, cudaMemcpyDeviceToHost, st));
		PA_CUDA(pa_copy(s, hp + 16 + size_t(B) * 8, s->d_seed.p, size_t(B) * 8, cudaMemcpyDeviceToHost, st));
	}
	if (out) {
		res.map_off = map_off;
		res.mask_off = mask_off;
	}
	if (need_walk || wsb_maps) {
		if ((maps_out && in.location == PA_DEVICE) || paths_to_user || chunked) {
			// results stay on the device, or the pipeline downloaded them chunk by chunk
		} else if (maps_out) {
			PA_CUDA(pa_copy(s, maps_out, s->d_maps.p, size_t(map_off[size_t(B)]) * 4, cudaMemcpyDeviceToHost, st));
		} else {
			res.maps.resize(size_t(map_off[size_t(B)]));
			PA_CUDA(pa_copy(s, res.maps.data(), s->d_maps.p, res.maps.size() * 4, cudaMemcpyDeviceToHost, st));
		}
		if (want_paths) {
			res.path_off = path_off;
			res.paths.resize(size_t(path_off[size_t(B)]));
			res.path_len.resize(size_t(B));
			PA_CUDA(pa_copy(s, res.paths.data(), s->d_paths.p, res.paths.size() * 4, cudaMemcpyDeviceToHost, st));
			PA_CUDA(pa_copy(s, res.path_len.data(), s->d_path_len.p, size_t(B) * 4, cudaMemcpyDeviceToHost, st));
		}
	}
	if (tb == TB_ALL && s->gap != GAP_GENERAL) {
		// the result takes the mask buffer over (the solver allocates a new one next time)
		res.dev_masks_all = s->d_masks.p;
		res.matrices = true;
		res.dev_masks_words = mask_off[size_t(B)] * 4;
		s->d_masks.p = nullptr;
		s->d_masks.cap = 0;
	}
	if (tb == TB_ONE && want_values && s->gap != GAP_GENERAL) {
		res.masks_one.resize(size_t(mask_off[size_t(B)]));
		res.matrices = true;
		PA_CUDA(pa_copy(s, res.masks_one.data(), s->d_masks.p, res.masks_one.size() * 4, cudaMemcpyDeviceToHost, st));
	}
	if (want_values) {
		res.val_off = val_off;
		res.values.resize(size_t(val_off[size_t(B)]));
		PA_CUDA(pa_copy(s, res.values.data(), s->d_vals.p, res.values.size() * 4, cudaMemcpyDeviceToHost, st));
	}
	if (wsb_host) {
		if (pa_status e = download_wsb(s, res)) return e;
		res.matrices = true;
	}
	PA_CUDA(cudaEventRecord(s->ev[4], st));
	PA_CUDA(cudaStreamSynchronize(st));
	for (int k = 0; k < 4; k++) cudaEventElapsedTime(&s->last_ms[k], s->ev[k], s->ev[k + 1]);
	s->dp_timing_pending = false;
	s->last_launches = launches;
	int32_t status = 0;
	std::memcpy(&status, hp, 4);
	if (host_scores) {
		res.scores.resize(size_t(B));
		std::memcpy(res.scores.data(), hp + 16, size_t(B) * 4);
	}
	if (out) {
		res.has.resize(size_t(B));
		res.seeds.resize(size_t(2 * B));
		std::memcpy(res.has.data(), hp + 16 + size_t(B) * 4, size_t(B) * 4);
		std::memcpy(res.seeds.data(), hp + 16 + size_t(B) * 8, size_t(B) * 8);
	}
	if ((status & ST_BAD_CODE) && in.form == F_INDEXED && s->gap != GAP_GENERAL) {
		uint32_t mx[2] = {0, 0};
		PA_CUDA(cudaMemcpy(mx, s->d_codes_max.p, 8, cudaMemcpyDeviceToHost));
		if (B * in.n_s > 0 && int64_t(mx[0]) >= in.table_rows) return fail(PA_ERR_INVALID_ARGUMENT, "out of bounds index in a");
		return fail(PA_ERR_INVALID_ARGUMENT, "out of bounds index in b");
	}
	if (status & ST_BAD_CODE) return fail(PA_ERR_INVALID_ARGUMENT, "out of bounds index in a or b");
	if (status & ST_TIMEOUT) return fail(PA_ERR_TIMEOUT, "a chained stripe timed out waiting for the stripe above it");

	// ---- codomain semantics on the host side
	if (goal == GOAL_ALL && method == M_SCORE) {
		// Solver::score with all-optimal goal: first DFS result (solver.h:2593-2608);
		// local problems without a positive optimum have no seed -> worst value
		for (int64_t k = 0; k < B; k++) {
			const bool pos = s->loc != LOC_LOCAL || (res.scores[size_t(k)] * s->sign > 0.0f);
			if (!pos || ls[size_t(k)] == 0 || lt[size_t(k)] == 0) {
				if (s->loc == LOC_LOCAL) res.scores[size_t(k)] = res.worst;
			}
		}
	}
	if (scores_out) std::memcpy(scores_out, res.scores.data(), size_t(B) * 4);
	if (out) {
		res.ls = ls;
		res.lt = lt;
		*out = new pa_result{R_};
	}
	return PA_OK;
}

// ---- host DFS over all-optimal masks (TracebackIterators<true>, solver.h:1647-1716)

void iterator_init(pa_iterator *it) {
	const ResultData &d = *it->d;
	const int64_t k = it->lane;
	const int ls = d.ls[size_t(k)], lt = d.lt[size_t(k)];
	if (d.goal != GOAL_ALL) return;
	if (d.loc == LOC_LOCAL) {
		// all cells equal to a strictly positive optimum, pushed in reverse scan order
		// (solver.h:2066-2091)
		const float best = d.scores[size_t(k)] * d.sign;  // normalised optimum
		if (!(best > 0.0f) || ls == 0 || lt == 0) return;
		for (int i = ls - 1; i >= 0; i--)
			for (int j = lt - 1; j >= 0; j--) {
				bool seed;
				if (d.gap == GAP_GENERAL) seed = d.wsb_val(k, i, j) == best;
				else seed = (d.cell(k, i, j) & 256u) != 0;
				if (seed) it->stk.push({i, j, 0});
			}
	} else {
		if (d.has[size_t(k)]) it->stk.push({d.seeds[size_t(2 * k)], d.seeds[size_t(2 * k + 1)], 0});
	}
}

// compressed path = the points emitted by path_compressor (solver.h:809-847)
void compress(const std::vector<std::pair<int, int>> &path, std::vector<int32_t> &cp) {
	cp.clear();
	bool empty = true;
	int lu = 0, lv = 0;
	for (const auto &pt : path) {
		if (empty) empty = false;
		else if (pt.first != lu && pt.second != lv) {
			if (lu >= 0 && lv >= 0) {
				cp.push_back(lu);
				cp.push_back(lv);
			}
		}
		lu = pt.first;
		lv = pt.second;
	}
}

bool iterator_next_all(pa_iterator *it, std::vector<std::pair<int, int>> &path_out) {
	const ResultData &d = *it->d;
	const int64_t k = it->lane;
	std::vector<int32_t> cp;
	while (!it->stk.empty()) {
		const auto e = it->stk.top();
		it->stk.pop();
		if (e.path_len == 0) it->path.clear();
		else it->path.resize(size_t(e.path_len));
		it->path.push_back({e.u, e.v});
		if (e.u >= 0 && e.v >= 0 && d.cont2_all(k, e.u, e.v)) {
			d.tb_list_all(k, e.u, e.v, it->scratch);
			const int32_t psize = int32_t(it->path.size());
			if (!it->scratch.empty()) {
				for (const auto &pt : it->scratch) it->stk.push({pt.first, pt.second, psize});
			} else {
				it->stk.push({NO_TB, NO_TB, psize});
			}
		} else {
			if (d.remove_dup) {
				compress(it->path, cp);
				if (it->emitted.count(cp)) continue;
				it->emitted.insert(cp);
			}
			path_out = it->path;
			return true;
		}
	}
	return false;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// WSB (general gap) glue lives in pa_wsb.cu; it needs these accessors.
namespace pa {
pa_status wsb_fail(pa_status st, const std::string &m) { return fail(st, m); }
}  // namespace pa

// ---------------------------------------------------------------------------------------
// C ABI

extern "C" {

const char *pa_last_error(void) { return g_err.c_str(); }

const char *pa_version(void) { return "pyalign_gb300 0.1 (sm_103a)"; }

int32_t pa_device_count(void) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return n;
}

pa_status pa_solver_create(const pa_options *o, int64_t max_len_s, int64_t max_len_t, pa_solver **out) {
	if (!o || !out) return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	const int bits = o->index_bits == 16 ? 16 : 32;
	const int64_t lim = (bits == 16 ? int64_t(INT16_MAX) : int64_t(INT32_MAX)) >> 1;  // solver.h:496-503
	if (max_len_s < 0 || max_len_t < 0) return fail(PA_ERR_INVALID_ARGUMENT, "negative maximum length");
	if (max_len_s > lim)
		return fail(PA_ERR_LENGTH, "requested maximum length " + std::to_string(max_len_s) +
		                               " for s exceeds maximum supported sequence length in this implementation " +
		                               std::to_string(lim));
	if (max_len_t > lim)
		return fail(PA_ERR_LENGTH, "requested maximum length " + std::to_string(max_len_t) +
		                               " for t exceeds maximum supported sequence length in this implementation " +
		                               std::to_string(lim));
	if (o->direction != PA_MINIMIZE && o->direction != PA_MAXIMIZE)
		return fail(PA_ERR_INVALID_ARGUMENT, "illegal direction");
	if (o->type != PA_TYPE_ALIGNMENT && o->type != PA_TYPE_DTW)
		return fail(PA_ERR_INVALID_ARGUMENT, "illegal solver type");
	if (o->type == PA_TYPE_ALIGNMENT) {
		if (o->locality < 0 || o->locality > 2) return fail(PA_ERR_INVALID_ARGUMENT, "invalid locality");
		if (o->count < 0 || o->count > 1) return fail(PA_ERR_INVALID_ARGUMENT, "invalid count");
		if (o->detail < 0 || o->detail > 2) return fail(PA_ERR_INVALID_ARGUMENT, "invalid detail");
		if (o->gap_kind < 0 || o->gap_kind > 2) return fail(PA_ERR_INVALID_ARGUMENT, "invalid gap cost kind");
	}
	auto s = std::make_unique<pa_solver>();
	s->opt = *o;
	s->opt.general_s = nullptr;
	s->opt.general_t = nullptr;
	s->cap_s = max_len_s;
	s->cap_t = max_len_t;
	s->batch_size = o->batch ? (o->batch_size > 0 ? o->batch_size : 2048) : 1;
	s->sign = o->direction == PA_MAXIMIZE ? 1.0f : -1.0f;
	const float sgn = o->direction == PA_MINIMIZE ? 1.0f : -1.0f;  // gap_sgn (solver.h:2807)
	const size_t ns = size_t(max_len_s) + 1, nt = size_t(max_len_t) + 1;
	s->left_D.assign(ns, 0.0f);
	s->left_P.assign(ns, 0.0f);
	s->top_D.assign(nt, 0.0f);
	s->top_Q.assign(nt, 0.0f);
	// normalised value = sign * reference value
	auto norm = [&](float ref) { return ref * s->sign; };
	if (o->type == PA_TYPE_DTW) {
		s->gap = GAP_DTW;
		s->goal = GOAL_ONE;  // factory.h:1055-1099
		s->loc = LOC_GLOBAL;
		const float worst = -INFINITY;  // normalised
		std::fill(s->left_D.begin(), s->left_D.end(), worst);
		std::fill(s->top_D.begin(), s->top_D.end(), worst);
		s->left_D[0] = s->top_D[0] = 0.0f;  // solver.h:3205-3210
		s->alg[0] = "DTW";
		s->alg[1] = "n^2";
		s->alg[2] = "n^2";
	} else {
		s->gap = o->gap_kind == PA_GAP_LINEAR ? GAP_LINEAR : o->gap_kind == PA_GAP_AFFINE ? GAP_AFFINE : GAP_GENERAL;
		s->goal = o->count == PA_COUNT_ALL ? GOAL_ALL : (o->detail == PA_DETAIL_SCORE ? GOAL_SCORE : GOAL_ONE);
		s->loc = o->locality == PA_LOCAL ? LOC_LOCAL : o->locality == PA_GLOBAL ? LOC_GLOBAL : LOC_SEMI;
		const bool global = s->loc == LOC_GLOBAL;
		if (s->gap == GAP_LINEAR) {  // solver.h:2806-2814: arange(0, n) * g * gap_sgn
			for (size_t k = 0; k < ns; k++) s->left_D[k] = global ? norm((float(int64_t(k)) * o->linear_s) * sgn) : 0.0f;
			for (size_t k = 0; k < nt; k++) s->top_D[k] = global ? norm((float(int64_t(k)) * o->linear_t) * sgn) : 0.0f;
			s->alg[0] = global ? "Needleman-Wunsch" : "Smith-Waterman";
			s->alg[1] = "n^2";
			s->alg[2] = "n^2";
		} else if (s->gap == GAP_AFFINE) {  // solver.h:2918-2967
			const auto ws = affine_vector(o->affine_u_s, o->affine_v_s, ns);
			const auto wt = affine_vector(o->affine_u_t, o->affine_v_t, nt);
			for (size_t k = 0; k < ns; k++) s->left_D[k] = s->left_P[k] = global ? norm(ws[k] * sgn) : 0.0f;
			for (size_t k = 0; k < nt; k++) s->top_D[k] = s->top_Q[k] = global ? norm(wt[k] * sgn) : 0.0f;
			s->alg[0] = "Gotoh";
			s->alg[1] = "n^2";
			s->alg[2] = "n^2";
		} else {  // solver.h:3095-3126
			if (!o->general_s || !o->general_t)
				return fail(PA_ERR_INVALID_ARGUMENT, "general gap cost needs cost vectors");
			s->gen_s.assign(o->general_s, o->general_s + ns);
			s->gen_t.assign(o->general_t, o->general_t + nt);
			for (size_t k = 0; k < ns; k++) s->left_D[k] = global ? norm(s->gen_s[k] * sgn) : 0.0f;
			for (size_t k = 0; k < nt; k++) s->top_D[k] = global ? norm(s->gen_t[k] * sgn) : 0.0f;
			s->alg[0] = "Waterman-Smith-Beyer";
			s->alg[1] = "n^3";
			s->alg[2] = "n^2";
		}
	}
	*out = s.release();
	return PA_OK;
}

void pa_solver_destroy(pa_solver *s) { delete s; }

int32_t pa_solver_batch_size(const pa_solver *s) { return s ? s->batch_size : 0; }

pa_status pa_solver_set_stream(pa_solver *s, void *stream) {
	if (!s) return fail(PA_ERR_INVALID_ARGUMENT, "null solver");
	if (pa_status st = ensure_device(s)) return st;
	s->stream = reinterpret_cast<cudaStream_t>(stream);  // NULL: CUDA's default stream
	s->stream_set = true;
	return PA_OK;
}

pa_status pa_solver_last_bytes(const pa_solver *s, int64_t *h2d, int64_t *d2h) {
	if (!s) return fail(PA_ERR_INVALID_ARGUMENT, "null solver");
	if (h2d) *h2d = s->bytes_h2d;
	if (d2h) *d2h = s->bytes_d2h;
	return PA_OK;
}

pa_status pa_solver_last_plan(const pa_solver *s, int32_t *plan4) {
	if (!s) return fail(PA_ERR_INVALID_ARGUMENT, "null solver");
	if (plan4)
		for (int k = 0; k < 4; k++) plan4[k] = s->last_plan[k];
	return PA_OK;
}

pa_status pa_solver_last_bucket_widths(const pa_solver *s, int32_t *widths4) {
	if (!s) return fail(PA_ERR_INVALID_ARGUMENT, "null solver");
	if (widths4)
		for (int k = 0; k < PA_BUCKETS; k++) widths4[k] = s->last_widths[k];
	return PA_OK;
}

pa_status pa_solver_last_timings(const pa_solver *s, float *ms4, int32_t *kernel_launches) {
	if (!s) return fail(PA_ERR_INVALID_ARGUMENT, "null solver");
	if (s->dp_timing_pending) {
		// a device-resident paths solve returned without waiting: its DP time is read here,
		// once the DP's end event has completed (the other phases stay 0)
		pa_solver *m = const_cast<pa_solver *>(s);
		m->dp_timing_pending = false;
		if (cudaEventSynchronize(m->ev[2]) != cudaSuccess ||
		    cudaEventElapsedTime(&m->last_ms[1], m->ev[1], m->ev[2]) != cudaSuccess) {
			cudaGetLastError();
			m->last_ms[1] = 0.0f;
		}
	}
	if (ms4)
		for (int k = 0; k < 4; k++) ms4[k] = s->last_ms[k];
	if (kernel_launches) *kernel_launches = s->last_launches;
	return PA_OK;
}

#define PA_DENSE_INPUT                                                                            \
	Input in{};                                                                                   \
	in.form = F_DENSE;                                                                            \
	in.location = PA_HOST;                                                                        \
	in.batch = batch;                                                                             \
	in.n_s = n_s;                                                                                 \
	in.n_t = n_t;                                                                                 \
	in.sim = sim;                                                                                 \
	in.length = length;
#define PA_INDEXED_INPUT                                                                          \
	Input in{};                                                                                   \
	in.form = F_INDEXED;                                                                          \
	in.location = PA_HOST;                                                                        \
	in.batch = batch;                                                                             \
	in.n_s = n_s;                                                                                 \
	in.n_t = n_t;                                                                                 \
	in.a = a;                                                                                     \
	in.b = b;                                                                                     \
	in.table = table;                                                                             \
	in.table_rows = table_rows;                                                                   \
	in.table_cols = table_cols;                                                                   \
	in.length = length;
#define PA_BINARY_INPUT                                                                           \
	Input in{};                                                                                   \
	in.form = F_BINARY;                                                                           \
	in.location = PA_HOST;                                                                        \
	in.batch = batch;                                                                             \
	in.n_s = n_s;                                                                                 \
	in.n_t = n_t;                                                                                 \
	in.a = a;                                                                                     \
	in.b = b;                                                                                     \
	in.eq = eq;                                                                                   \
	in.ne = ne;                                                                                   \
	in.length = length;

pa_status pa_solve_for_score(pa_solver *s, const float *sim, int64_t n_s, int64_t n_t, int64_t batch,
                             const int32_t *length, float *scores) {
	PA_DENSE_INPUT return solve_impl(s, in, M_SCORE, scores, nullptr);
}
pa_status pa_solve_indexed_for_score(pa_solver *s, const uint32_t *a, const uint32_t *b, int64_t batch, int64_t n_s,
                                     int64_t n_t, const float *table, int64_t table_rows, int64_t table_cols,
                                     const int32_t *length, float *scores) {
	PA_INDEXED_INPUT return solve_impl(s, in, M_SCORE, scores, nullptr);
}
pa_status pa_solve_binary_for_score(pa_solver *s, const uint32_t *a, const uint32_t *b, int64_t batch, int64_t n_s,
                                    int64_t n_t, float eq, float ne, const int32_t *length, float *scores) {
	PA_BINARY_INPUT return solve_impl(s, in, M_SCORE, scores, nullptr);
}

#define PA_METHODS(NAME, M)                                                                               \
	pa_status pa_solve_for_##NAME(pa_solver *s, const float *sim, int64_t n_s, int64_t n_t, int64_t batch, \
	                              const int32_t *length, pa_result **out) {                              \
		PA_DENSE_INPUT return solve_impl(s, in, M, nullptr, out);                                        \
	}                                                                                                    \
	pa_status pa_solve_indexed_for_##NAME(pa_solver *s, const uint32_t *a, const uint32_t *b, int64_t batch, \
	                                      int64_t n_s, int64_t n_t, const float *table, int64_t table_rows,  \
	                                      int64_t table_cols, const int32_t *length, pa_result **out) {      \
		PA_INDEXED_INPUT return solve_impl(s, in, M, nullptr, out);                                      \
	}                                                                                                    \
	pa_status pa_solve_binary_for_##NAME(pa_solver *s, const uint32_t *a, const uint32_t *b, int64_t batch, \
	                                     int64_t n_s, int64_t n_t, float eq, float ne, const int32_t *length, \
	                                     pa_result **out) {                                              \
		PA_BINARY_INPUT return solve_impl(s, in, M, nullptr, out);                                       \
	}

PA_METHODS(alignment, M_ALIGNMENT)
PA_METHODS(alignment_iterator, M_ALIGNMENT_ITER)
PA_METHODS(solution, M_SOLUTION)
PA_METHODS(solution_iterator, M_SOLUTION_ITER)

pa_status pa_solve_batch(pa_solver *s, const pa_batch *b, float *scores, int32_t *maps, const int64_t *map_offsets) {
	if (!s || !b) return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	Input in{};
	in.form = b->form;
	in.location = b->location;
	in.batch = b->batch;
	in.n_s = b->n_s;
	in.n_t = b->n_t;
	in.a = b->a;
	in.b = b->b;
	in.sim = b->sim;
	in.table = b->table;
	in.table_rows = b->table_rows;
	in.table_cols = b->table_cols;
	in.eq = b->eq;
	in.ne = b->ne;
	in.length = b->length;
	if (s->goal == GOAL_ALL) return fail(PA_ERR_UNSUPPORTED, "pa_solve_batch returns one alignment per pair");
	const bool dev = b->location == PA_DEVICE;
	// no result object: only the scores (and the maps, written in place) leave the call
	pa_status st = solve_impl(s, in, maps ? M_ALIGNMENT : M_SCORE, dev ? nullptr : scores, nullptr, maps, map_offsets);
	if (st) return st;
	if (dev && scores) {
		cudaError_t e = pa_copy(s, scores, s->d_score.p, size_t(b->batch) * 4, cudaMemcpyDeviceToDevice, s->stream);
		if (e != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
	}
	return PA_OK;
}

pa_status pa_solve_batch_result(pa_solver *s, const pa_batch *b, int32_t *maps, const int64_t *map_offsets,
                                pa_result **out) {
	if (!s || !b || !maps || !map_offsets || !out) return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	if (b->location != PA_HOST) return fail(PA_ERR_INVALID_ARGUMENT, "pa_solve_batch_result takes host buffers");
	if (s->goal != GOAL_ONE || s->gap == GAP_GENERAL)
		return fail(PA_ERR_UNSUPPORTED, "pa_solve_batch_result: one optimal alignment per pair, linear, affine or DTW");
	Input in{};
	in.form = b->form;
	in.location = PA_HOST;
	in.batch = b->batch;
	in.n_s = b->n_s;
	in.n_t = b->n_t;
	in.a = b->a;
	in.b = b->b;
	in.sim = b->sim;
	in.table = b->table;
	in.table_rows = b->table_rows;
	in.table_cols = b->table_cols;
	in.eq = b->eq;
	in.ne = b->ne;
	in.length = b->length;
	pa_result *r = nullptr;
	if (pa_status st = solve_impl(s, in, M_ALIGNMENT, nullptr, &r, maps, map_offsets)) return st;
	r->d->maps_external = true;
	*out = r;
	return PA_OK;
}

pa_status pa_solve_dense_paths(pa_solver *s, const float *sim, const int64_t *offsets, int64_t stride_s,
                               int64_t stride_t, int64_t batch, int64_t n_s, int64_t n_t, const int32_t *length,
                               float *scores, int32_t *paths, const int64_t *path_offsets, int32_t *path_len) {
	if (!s || !sim || !offsets || !length || !paths || !path_offsets || !path_len)
		return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	Input in{};
	in.form = F_DENSE;
	in.location = PA_DEVICE;
	in.batch = batch;
	in.n_s = n_s;
	in.n_t = n_t;
	in.sim = sim;
	in.length = length;
	in.dense_off_host = offsets;
	in.dense_si = stride_s;
	in.dense_sj = stride_t;
	UserPaths up_{};
	up_.paths = paths;
	up_.path_off = path_offsets;
	up_.path_len = path_len;
	up_.scores = scores;
	pa_result *r = nullptr;
	pa_status st = solve_impl(s, in, M_PATHS, nullptr, &r, nullptr, nullptr, &up_);
	if (r) pa_result_destroy(r);
	return st;
}

pa_status pa_solve_series_paths(pa_solver *s, const float *x, int64_t x_stride, const float *y, int64_t y_stride,
                                int64_t batch, int64_t n_s, int64_t n_t, const int32_t *length, float *scores,
                                int32_t *paths, const int64_t *path_offsets, int32_t *path_len) {
	if (!s || !x || !y || !length || !paths || !path_offsets || !path_len)
		return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	if (x_stride < n_s || y_stride < n_t) return fail(PA_ERR_INVALID_ARGUMENT, "series stride below its length");
	if (s->gap == GAP_GENERAL) return fail(PA_ERR_UNSUPPORTED, "series form: linear, affine or DTW gap costs only");
	Input in{};
	in.form = F_SERIES;
	in.location = PA_DEVICE;
	in.batch = batch;
	in.n_s = n_s;
	in.n_t = n_t;
	in.sx = x;
	in.sy = y;
	in.sx_stride = x_stride;
	in.sy_stride = y_stride;
	in.length = length;
	UserPaths up_{};
	up_.paths = paths;
	up_.path_off = path_offsets;
	up_.path_len = path_len;
	up_.scores = scores;
	pa_result *r = nullptr;
	pa_status st = solve_impl(s, in, M_PATHS, nullptr, &r, nullptr, nullptr, &up_);
	if (r) pa_result_destroy(r);
	return st;
}

void pa_result_destroy(pa_result *r) { delete r; }
int64_t pa_result_size(const pa_result *r) { return r ? r->d->batch : 0; }
int64_t pa_result_len_s(const pa_result *r, int64_t lane) { return r->d->ls[size_t(lane)]; }
int64_t pa_result_len_t(const pa_result *r, int64_t lane) { return r->d->lt[size_t(lane)]; }
pa_status pa_result_lengths(const pa_result *r, int32_t *len_s, int32_t *len_t) {
	if (!r || !len_s || !len_t) return fail(PA_ERR_INVALID_ARGUMENT, "null argument");
	std::memcpy(len_s, r->d->ls.data(), r->d->ls.size() * 4);
	std::memcpy(len_t, r->d->lt.data(), r->d->lt.size() * 4);
	return PA_OK;
}

int32_t pa_result_has_alignment(const pa_result *r, int64_t lane) {
	const ResultData &d = *r->d;
	if (d.goal == GOAL_ALL) {
		pa_iterator it;
		it.d = r->d;
		it.lane = lane;
		iterator_init(&it);
		return it.stk.empty() ? 0 : 1;
	}
	return d.has[size_t(lane)];
}

float pa_result_score(const pa_result *r, int64_t lane) {
	const ResultData &d = *r->d;
	if (!pa_result_has_alignment(r, lane)) return d.worst;
	return d.scores[size_t(lane)];
}

}  // extern "C"

static void map_from_path(const ResultData &d, int64_t lane, const std::vector<std::pair<int, int>> &path,
                          int32_t *map) {
	const int ls = d.ls[size_t(lane)], lt = d.lt[size_t(lane)];
	const int n = std::min(ls, lt);
	for (int k = 0; k < n; k++) map[k] = -1;
	std::vector<int32_t> cp;
	compress(path, cp);
	for (size_t k = 0; k + 1 < cp.size(); k += 2) {
		if (ls <= lt) map[cp[k]] = cp[k + 1];
		else map[cp[k + 1]] = cp[k];
	}
}

// The one-path walk of a lane from the device results or (all-optimal goal) the first
// result of the DFS.
static bool lane_walk(const pa_result *r, int64_t lane, std::vector<std::pair<int, int>> *path, int32_t *map) {
	const ResultData &d = *r->d;
	if (d.goal == GOAL_ALL) {
		pa_iterator it;
		it.d = r->d;
		it.lane = lane;
		iterator_init(&it);
		std::vector<std::pair<int, int>> p;
		if (!iterator_next_all(&it, p)) return false;
		if (map) map_from_path(d, lane, p, map);
		if (path) *path = p;
		return true;
	}
	if (!d.has[size_t(lane)]) return false;
	const int n = std::min(d.ls[size_t(lane)], d.lt[size_t(lane)]);
	if (d.gap == GAP_GENERAL && !d.wsb_tb.empty()) {
		// WSB one-optimal walk over the device traceback codes (solver.h:1497-1536); a
		// solve for alignments walked on the device and kept only the maps
		std::vector<std::pair<int, int>> p;
		int u = d.seeds[size_t(2 * lane)], v = d.seeds[size_t(2 * lane + 1)];
		p.push_back({u, v});
		while (u >= 0 && v >= 0) {
			if (d.loc == LOC_LOCAL && !(d.wsb_val(lane, u, v) > 0.0f)) break;
			const int32_t c = d.wsb(lane, u, v);
			const int kind = c & 3, kk = (c >> 2) - 1;
			if (kind == 0) { u = NO_TB; v = NO_TB; }
			else if (kind == 1) { u--; v--; }
			else if (kind == 2) u = kk;
			else v = kk;
			p.push_back({u, v});
		}
		if (map) map_from_path(d, lane, p, map);
		if (path) *path = p;
		return true;
	}
	if (map) {
		if (d.maps.empty()) {
			for (int k = 0; k < n; k++) map[k] = -1;
		} else {
			std::memcpy(map, d.maps.data() + d.map_off[size_t(lane)], size_t(n) * 4);
		}
	}
	if (path && !d.path_len.empty()) {
		path->clear();
		const int32_t *pp = d.paths.data() + d.path_off[size_t(lane)];
		for (int k = 0; k < d.path_len[size_t(lane)]; k++) path->push_back({pp[2 * k], pp[2 * k + 1]});
	}
	return true;
}

extern "C" {

pa_status pa_result_alignment(const pa_result *r, int64_t lane, int32_t *map) {
	if (!r || lane < 0 || lane >= r->d->batch) return fail(PA_ERR_INVALID_ARGUMENT, "bad lane");
	const ResultData &d = *r->d;
	if (d.maps_external) return fail(PA_ERR_INVALID_ARGUMENT, "this result's maps are in the caller's buffer");
	const int n = std::min(d.ls[size_t(lane)], d.lt[size_t(lane)]);
	if (!lane_walk(r, lane, nullptr, map))
		for (int k = 0; k < n; k++) map[k] = -1;
	return PA_OK;
}

pa_status pa_result_export(const pa_result *r, float *scores, int32_t *maps, const int64_t *map_offsets) {
	if (!r) return fail(PA_ERR_INVALID_ARGUMENT, "null result");
	if (maps && r->d->maps_external)
		return fail(PA_ERR_INVALID_ARGUMENT, "this result's maps are in the caller's buffer");
	for (int64_t k = 0; k < r->d->batch; k++) {
		if (scores) scores[k] = pa_result_score(r, k);
		if (maps) pa_result_alignment(r, k, maps + map_offsets[k]);
	}
	return PA_OK;
}

int32_t pa_result_layers(const pa_result *r, int64_t) {
	// Solver::solution copies every layer; the iterators detach layer D only
	// (solver.h:2644-2651, 2680, 2720-2721)
	const ResultData &d = *r->d;
	return d.method == M_SOLUTION ? d.layers : 1;
}

int32_t pa_result_max_degree_1(const pa_result *r) { return r->d->goal != GOAL_ALL ? 1 : 0; }

pa_status pa_result_values(const pa_result *r, int64_t lane, float *values) {
	const ResultData &d = *r->d;
	const int ls = d.ls[size_t(lane)], lt = d.lt[size_t(lane)];
	const size_t n = size_t(ls + 1) * size_t(lt + 1) * size_t(pa_result_layers(r, lane));
	if (d.gap == GAP_GENERAL) {
		if (d.wsb_vals.empty()) return fail(PA_ERR_INVALID_ARGUMENT, "no values in this result");
		const float *v = d.wsb_vals.data() + d.wsb_voff[size_t(lane)];
		for (size_t k = 0; k < n; k++) values[k] = v[k] * d.sign;
		return PA_OK;
	}
	if (d.values.empty()) return fail(PA_ERR_INVALID_ARGUMENT, "no values in this result");
	std::memcpy(values, d.values.data() + d.val_off[size_t(lane)], n * 4);
	return PA_OK;
}

}  // extern "C"

// traceback of one cell and layer as a list (one- or all-optimal), storage indices
// i, j >= 0 meaning cell (i-1, j-1).
static void cell_tb(const ResultData &d, int64_t lane, int layer, int i, int j, std::vector<std::pair<int, int>> &out,
                    std::vector<int32_t> &colP, std::vector<int32_t> &rowQ) {
	out.clear();
	if (i == 0 || j == 0) return;  // borders are cleared (solver.h:530-537, 2953-2967)
	const int u = i - 1, v = j - 1;
	if (d.goal == GOAL_ALL) {
		d.tb_list_all(lane, u, v, out, layer);
		return;
	}
	if (d.gap == GAP_GENERAL) {
		const int32_t c = d.wsb(lane, u, v);
		const int kind = c & 3, kk = (c >> 2) - 1;
		if (kind == 1) out.push_back({u - 1, v - 1});
		else if (kind == 2) out.push_back({kk, v});
		else if (kind == 3) out.push_back({u, kk});
		return;
	}
	const uint32_t nb = d.nib(lane, u, v);
	const int lt = d.lt[size_t(lane)];
	(void)lt;
	if (layer == 1) {  // P: (u-1, v) or tb_P(u-1, v) -- colP holds tb_P row index per column
		out.push_back({colP[size_t(v)], v});
		return;
	}
	if (layer == 2) {
		out.push_back({u, rowQ[size_t(u)]});
		return;
	}
	const uint32_t code = nb & 3u;
	if (code == 3u && d.loc == LOC_LOCAL) return;  // the zero candidate: traceback_1 of size 0
	if (code == 2u) out.push_back({u - 1, v - 1});
	else if (code == 1u) out.push_back({d.gap == GAP_AFFINE ? colP[size_t(v)] : u - 1, v});
	else out.push_back({u, d.gap == GAP_AFFINE ? rowQ[size_t(u)] : v - 1});
}

// Iterate the cells in storage order, maintaining tb_P (per column) and tb_Q (per row)
// gap-open coordinates for one-optimal affine masks.
template <typename F>
static void for_each_cell_tb(const ResultData &d, int64_t lane, int layer, F f) {
	const int ls = d.ls[size_t(lane)], lt = d.lt[size_t(lane)];
	std::vector<int32_t> colP(size_t(std::max(lt, 1)), 0), rowQ(size_t(std::max(ls, 1)), 0);
	std::vector<std::pair<int, int>> lst;
	const bool affine_one = d.gap == GAP_AFFINE && d.goal != GOAL_ALL && d.gap != GAP_GENERAL;
	for (int i = 0; i <= ls; i++) {
		for (int j = 0; j <= lt; j++) {
			if (affine_one && i > 0 && j > 0) {
				const int u = i - 1, v = j - 1;
				const uint32_t nb = d.nib(lane, u, v);
				colP[size_t(v)] = (nb & 4u) ? colP[size_t(v)] : u - 1;  // tb_P(u, v)
				rowQ[size_t(u)] = (nb & 8u) ? rowQ[size_t(u)] : v - 1;  // tb_Q(u, v)
			}
			cell_tb(d, lane, layer, i, j, lst, colP, rowQ);
			f(i, j, lst);
		}
	}
}

extern "C" {

pa_status pa_result_tb_matrix(const pa_result *r, int64_t lane, int32_t *tb) {
	const ResultData &d = *r->d;
	if (!d.matrices) return fail(PA_ERR_INVALID_ARGUMENT, "no traceback matrix in this result");
	const int ls = d.ls[size_t(lane)], lt = d.lt[size_t(lane)];
	const int layers = pa_result_layers(r, lane);
	for (int layer = 0; layer < layers; layer++) {
		int32_t *t = tb + size_t(layer) * size_t(ls + 1) * size_t(lt + 1) * 2;
		for_each_cell_tb(d, lane, layer, [&](int i, int j, const std::vector<std::pair<int, int>> &l) {
			const size_t c = size_t(i) * size_t(lt + 1) + size_t(j);
			t[2 * c] = l.empty() ? NO_TB : l[0].first;
			t[2 * c + 1] = l.empty() ? NO_TB : l[0].second;
		});
	}
	return PA_OK;
}

int64_t pa_result_tb_edges(const pa_result *r, int64_t lane, int32_t layer, int32_t *edges) {
	const ResultData &d = *r->d;
	if (!d.matrices) return -1;  // no traceback matrix in this result
	int64_t n = 0;
	for_each_cell_tb(d, lane, layer, [&](int i, int j, const std::vector<std::pair<int, int>> &l) {
		for (const auto &pt : l) {
			if (edges) {
				edges[4 * n + 0] = i - 1;
				edges[4 * n + 1] = j - 1;
				edges[4 * n + 2] = pt.first;
				edges[4 * n + 3] = pt.second;
			}
			n++;
		}
	});
	return n;
}

int64_t pa_result_path(const pa_result *r, int64_t lane, int32_t *path) {
	std::vector<std::pair<int, int>> p;
	if (!lane_walk(r, lane, &p, nullptr)) return -1;
	if (path)
		for (size_t k = 0; k < p.size(); k++) {
			path[2 * k] = p[k].first;
			path[2 * k + 1] = p[k].second;
		}
	return int64_t(p.size());
}

const char *pa_result_algorithm(const pa_result *r, int32_t field) {
	if (!r || field < 0 || field > 2) return "";
	return r->d->alg[field].c_str();
}

pa_status pa_result_iterator(pa_result *r, int64_t lane, pa_iterator **out) {
	if (!r || lane < 0 || lane >= r->d->batch) return fail(PA_ERR_INVALID_ARGUMENT, "bad lane");
	auto *it = new pa_iterator();
	it->d = r->d;
	it->lane = lane;
	iterator_init(it);
	*out = it;
	return PA_OK;
}

int32_t pa_iterator_next(pa_iterator *it, float *score, int32_t *map, int32_t *path, int64_t *path_len) {
	const ResultData &d = *it->d;
	const int64_t lane = it->lane;
	std::vector<std::pair<int, int>> p;
	if (d.goal != GOAL_ALL) {
		// TracebackIterators<false>: a single result (solver.h:1497-1536)
		if (it->one_done) return 0;
		it->one_done = true;
		pa_result tmp{it->d};
		if (!lane_walk(&tmp, lane, &p, map)) return 0;
		if (score) *score = d.scores[size_t(lane)];
	} else {
		if (!iterator_next_all(it, p)) return 0;
		if (map) map_from_path(d, lane, p, map);
		if (score) *score = d.scores[size_t(lane)];
	}
	if (path)
		for (size_t k = 0; k < p.size(); k++) {
			path[2 * k] = p[k].first;
			path[2 * k + 1] = p[k].second;
		}
	if (path_len) *path_len = int64_t(p.size());
	return 1;
}

void pa_iterator_destroy(pa_iterator *it) { delete it; }

}  // extern "C"

namespace pa {
cudaError_t path_count_solve(int32_t npairs, int32_t G, int32_t local, int32_t affine, const int32_t *len_s,
                             const int32_t *len_t, const int64_t *mask_off, const void *masks, const int32_t *seed,
                             unsigned long long *counts, unsigned long long *scratch, int64_t scratch_stride,
                             int32_t *work_counter, int grid, cudaStream_t st, int32_t ntickets,
                             int32_t nlevels, const int32_t *level_start, const int32_t *order, int32_t *progress,
                             int32_t *status, unsigned long long *partial);
}  // namespace pa

extern "C" {

// Number of co-optimal traceback paths per lane of an all-optimal result: the count of
// results the reference's depth-first enumeration (solver.h:1647-1716) produces without
// de-duplication, computed on the device over the result's masks (path_count_kernel,
// pa_count.cu), uint64 saturating at 2^64 - 1.  Blocks until the counts are on the host.
pa_status pa_result_path_counts(const pa_result *r, uint64_t *counts) {
	if (!r || !counts) return fail(PA_ERR_INVALID_ARGUMENT, "pa_result_path_counts: null argument");
	const ResultData &d = *r->d;
	if (d.goal != GOAL_ALL || !d.dev_masks_all || d.gap == GAP_GENERAL)
		return fail(PA_ERR_UNSUPPORTED, "path counts need an all-optimal result with linear or affine gap costs");
	const int64_t B = d.batch;
	if (d.path_counts.size() != size_t(B)) {
		const bool local = d.loc == LOC_LOCAL;
		std::vector<int32_t> seed(size_t(2 * B), -1);
		int64_t max_lt = 1;
		for (int64_t k = 0; k < B; k++) {
			max_lt = std::max<int64_t>(max_lt, d.lt[size_t(k)]);
			if (!local && d.has[size_t(k)]) {
				seed[size_t(2 * k)] = d.seeds[size_t(2 * k)];
				seed[size_t(2 * k + 1)] = d.seeds[size_t(2 * k + 1)];
			}
		}
		int dev = 0, sms = 1;
		PA_CUDA(cudaGetDevice(&dev));
		PA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
		DevBuf dl, dm, dseed, dcnt, dscr, dctr, dord, dlev, dprog, dpart, dstat;
		PA_CUDA(dl.ensure(size_t(2 * B) * 4));
		PA_CUDA(dm.ensure(size_t(B) * 8));
		PA_CUDA(dseed.ensure(size_t(2 * B) * 4));
		PA_CUDA(dcnt.ensure(size_t(B) * 8));
		PA_CUDA(dctr.ensure(4));
		PA_CUDA(cudaMemcpy(dl.p, d.ls.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dl.as<int32_t>() + B, d.lt.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dm.p, d.mask_off.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dseed.p, seed.data(), size_t(2 * B) * 4, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemset(dctr.p, 0, 4));
		// few long pairs written with G = 32: a warp per 256-row stripe, stripes chained
		const int64_t rpp32 = 32 * R;
		int64_t max_np = 0;
		for (int64_t k = 0; k < B; k++)
			if (d.ls[size_t(k)] > 0 && d.lt[size_t(k)] > 0)
				max_np = std::max<int64_t>(max_np, (d.ls[size_t(k)] + rpp32 - 1) / rpp32);
		bool chain = d.G == 32 && max_np >= 3;
		if (const char *e = std::getenv("PA_COUNT_MODE"))  // tests: "group" or "chain" (G = 32 only)
			chain = std::strcmp(e, "chain") == 0 ? d.G == 32 : std::strcmp(e, "group") == 0 ? false : chain;
		std::vector<uint64_t> c(static_cast<size_t>(B), 0);
		if (chain) {
			// tickets stripe-major: level q holds stripe q of every pair with more than q stripes
			// (an empty pair counts as one), the pairs with the most stripes first
			std::vector<int32_t> np(static_cast<size_t>(B)), order(static_cast<size_t>(B)), rank(static_cast<size_t>(B));
			for (int64_t k = 0; k < B; k++) {
				const int64_t a = d.ls[size_t(k)], b = d.lt[size_t(k)];
				np[size_t(k)] = int32_t(std::max<int64_t>(1, (a == 0 || b == 0) ? 1 : (a + rpp32 - 1) / rpp32));
				order[size_t(k)] = int32_t(k);
			}
			std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return np[size_t(x)] > np[size_t(y)]; });
			for (int64_t w = 0; w < B; w++) rank[size_t(order[size_t(w)])] = int32_t(w);
			const int64_t nlev = np[size_t(order[0])];
			std::vector<int32_t> level_start(static_cast<size_t>(nlev) + 1, 0);
			for (int64_t q = 0; q < nlev; q++) {
				int64_t above = 0;  // pairs with more than q stripes
				for (int64_t k = 0; k < B; k++) above += np[size_t(k)] > q;
				level_start[size_t(q) + 1] = int32_t(level_start[size_t(q)] + above);
			}
			const int64_t nt = level_start.back();
			const int64_t stride = 4 * max_lt;
			PA_CUDA(dord.ensure(size_t(B) * 4));
			PA_CUDA(dlev.ensure(level_start.size() * 4));
			PA_CUDA(dprog.ensure(size_t(nt) * 4));
			PA_CUDA(dpart.ensure(size_t(nt) * 8));
			PA_CUDA(dstat.ensure(4));
			PA_CUDA(dscr.ensure(size_t(B * stride) * 8));
			PA_CUDA(cudaMemcpy(dord.p, order.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
			PA_CUDA(cudaMemcpy(dlev.p, level_start.data(), level_start.size() * 4, cudaMemcpyHostToDevice));
			PA_CUDA(cudaMemset(dprog.p, 0, size_t(nt) * 4));
			PA_CUDA(cudaMemset(dstat.p, 0, 4));
			const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(int64_t(sms) * 4, (nt + WARPS - 1) / WARPS));
			PA_CUDA(pa::path_count_solve(int32_t(B), 32, local ? 1 : 0, d.gap == GAP_AFFINE ? 1 : 0, dl.as<int32_t>(),
			                             dl.as<int32_t>() + B, dm.as<int64_t>(), d.dev_masks_all, dseed.as<int32_t>(),
			                             dcnt.as<unsigned long long>(), dscr.as<unsigned long long>(), stride,
			                             dctr.as<int32_t>(), int(grid), nullptr, int32_t(nt), int32_t(nlev),
			                             dlev.as<int32_t>(), dord.as<int32_t>(), dprog.as<int32_t>(),
			                             dstat.as<int32_t>(), dpart.as<unsigned long long>()));
			std::vector<uint64_t> part(static_cast<size_t>(nt));
			int32_t status = 0;
			PA_CUDA(cudaMemcpy(part.data(), dpart.p, size_t(nt) * 8, cudaMemcpyDeviceToHost));
			PA_CUDA(cudaMemcpy(&status, dstat.p, 4, cudaMemcpyDeviceToHost));
			if (status & ST_TIMEOUT)
				return fail(PA_ERR_TIMEOUT, "a chained stripe of the path count timed out waiting for the stripe above it");
			for (int64_t k = 0; k < B; k++)
				for (int32_t q = 0; q < np[size_t(k)]; q++) {
					const uint64_t x = part[size_t(level_start[size_t(q)] + rank[size_t(k)])];
					const uint64_t y = c[size_t(k)] + x;
					c[size_t(k)] = y < x ? ~uint64_t(0) : y;
				}
		} else {
			const int gpw = 32 / d.G;
			const int64_t warps = (B + gpw - 1) / gpw;
			const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(int64_t(sms) * 8, (warps + WARPS - 1) / WARPS));
			const int64_t slots = grid * WARPS * gpw;
			const int64_t stride = 4 * max_lt;
			PA_CUDA(dscr.ensure(size_t(slots * stride) * 8));
			PA_CUDA(pa::path_count_solve(int32_t(B), d.G, local ? 1 : 0, d.gap == GAP_AFFINE ? 1 : 0, dl.as<int32_t>(),
			                             dl.as<int32_t>() + B, dm.as<int64_t>(), d.dev_masks_all, dseed.as<int32_t>(),
			                             dcnt.as<unsigned long long>(), dscr.as<unsigned long long>(), stride,
			                             dctr.as<int32_t>(), int(grid), nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr,
			                             nullptr));
			PA_CUDA(cudaMemcpy(c.data(), dcnt.p, size_t(B) * 8, cudaMemcpyDeviceToHost));
		}
		for (int64_t k = 0; k < B; k++) {
			const int ls = d.ls[size_t(k)], lt = d.lt[size_t(k)];
			if (local) {
				// seeds exist only for a strictly positive optimum (solver.h:2060-2091)
				if (!(d.scores[size_t(k)] * d.sign > 0.0f) || ls == 0 || lt == 0) c[size_t(k)] = 0;
			} else if (ls == 0 || lt == 0) {
				c[size_t(k)] = d.has[size_t(k)] ? 1 : 0;  // the seed itself has a negative coordinate
			} else if (!d.has[size_t(k)]) {
				c[size_t(k)] = 0;
			}
		}
		d.path_counts.swap(c);
	}
	std::memcpy(counts, d.path_counts.data(), size_t(B) * 8);
	return PA_OK;
}

// The first k optimal alignments of every lane of an all-optimal result, enumerated on the
// device (enum_kernel, pa_enum.cu) in the order and with the de-duplication of the
// reference's depth-first search (solver.h:1647-1716).  Blocks until the results are in the
// caller's host buffers.
pa_status pa_result_first_alignments(const pa_result *r, int32_t k, int32_t *counts, int32_t *maps, int32_t *paths,
                                     int32_t *path_len) {
	if (!r || !counts || k < 1) return fail(PA_ERR_INVALID_ARGUMENT, "pa_result_first_alignments: bad argument");
	if ((paths == nullptr) != (path_len == nullptr))
		return fail(PA_ERR_INVALID_ARGUMENT, "pa_result_first_alignments: paths and path_len go together");
	const ResultData &d = *r->d;
	if (d.goal != GOAL_ALL || !d.dev_masks_all || d.gap == GAP_GENERAL)
		return fail(PA_ERR_UNSUPPORTED, "device enumeration needs an all-optimal result with linear or affine gap costs");
	const int64_t B = d.batch;
	if (B == 0) return PA_OK;
	const bool local = d.loc == LOC_LOCAL;
	const int64_t K = k;
	// per-lane regions: maps k x min(|s|, |t|), paths k x (|s| + |t| + 2), the search's path
	std::vector<int64_t> moff(size_t(B) + 1, 0), poff(size_t(B) + 1, 0), woff(size_t(B) + 1, 0);
	std::vector<int32_t> has(static_cast<size_t>(B), 0), seed(static_cast<size_t>(2 * B), 0);
	std::vector<int32_t> all(static_cast<size_t>(B));
	for (int64_t L = 0; L < B; L++) {
		const int64_t ls = d.ls[size_t(L)], lt = d.lt[size_t(L)];
		moff[size_t(L) + 1] = moff[size_t(L)] + K * std::min(ls, lt);
		poff[size_t(L) + 1] = poff[size_t(L)] + (paths ? K * (ls + lt + 2) : 0);
		woff[size_t(L) + 1] = woff[size_t(L)] + ls + lt + 2;
		all[size_t(L)] = int32_t(L);
		if (!local) {
			has[size_t(L)] = d.has[size_t(L)];
			seed[size_t(2 * L)] = d.seeds[size_t(2 * L)];
			seed[size_t(2 * L + 1)] = d.seeds[size_t(2 * L + 1)];
		}
	}
	DevBuf dl, dm, dhas, dseed, dwork, dpath, dmaps, dpaths, dplen, dhash, dnpts, dcnt, dstat;
	PA_CUDA(dl.ensure(size_t(2 * B) * 4));
	PA_CUDA(dm.ensure(size_t(B) * 8));
	PA_CUDA(dhas.ensure(size_t(B) * 4));
	PA_CUDA(dseed.ensure(size_t(2 * B) * 4));
	PA_CUDA(dwork.ensure(size_t(B) * 4));
	PA_CUDA(cudaMemcpy(dl.p, d.ls.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dl.as<int32_t>() + B, d.lt.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dm.p, d.mask_off.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dhas.p, has.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dseed.p, seed.data(), size_t(2 * B) * 4, cudaMemcpyHostToDevice));
	int dev = 0, sms = 1;
	PA_CUDA(cudaGetDevice(&dev));
	PA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

	// ---- local seeds: every cell with the seed bit, in the stack's pop order (increasing row,
	// then column: the reverse of the push order, solver.h:2066-2091); only lanes with a
	// strictly positive optimum have any
	DevBuf dsd, dsoff, dsn, dscap;
	if (local) {
		std::vector<int32_t> cand;
		for (int64_t L = 0; L < B; L++)
			if (d.ls[size_t(L)] > 0 && d.lt[size_t(L)] > 0 && d.scores[size_t(L)] * d.sign > 0.0f)
				cand.push_back(int32_t(L));
		std::vector<int32_t> cap(static_cast<size_t>(B), 0), n(static_cast<size_t>(B), 0);
		int seed_cap0 = 16;
		if (const char *e = std::getenv("PA_ENUM_SEEDS")) seed_cap0 = std::max(1, std::atoi(e));  // tests
		for (int32_t L : cand) cap[size_t(L)] = seed_cap0;
		std::vector<std::vector<std::pair<int32_t, int32_t>>> found(static_cast<size_t>(B));
		std::vector<int32_t> work = cand;
		for (int round = 0; !work.empty(); round++) {
			if (round > 1) return fail(PA_ERR_INTERNAL, "local seed scan did not settle");
			std::vector<int64_t> off(size_t(B) + 1, 0);
			for (int64_t L = 0; L < B; L++) off[size_t(L) + 1] = off[size_t(L)] + cap[size_t(L)];
			PA_CUDA(dsd.ensure(size_t(std::max<int64_t>(off[size_t(B)], 1)) * 8));
			PA_CUDA(dsoff.ensure(size_t(B) * 8));
			PA_CUDA(dscap.ensure(size_t(B) * 4));
			PA_CUDA(dsn.ensure(size_t(B) * 4));
			PA_CUDA(cudaMemcpy(dsoff.p, off.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
			PA_CUDA(cudaMemcpy(dscap.p, cap.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
			PA_CUDA(cudaMemset(dsn.p, 0, size_t(B) * 4));
			PA_CUDA(cudaMemcpy(dwork.p, work.data(), work.size() * 4, cudaMemcpyHostToDevice));
			pa::SeedScanParams sp{};
			sp.nwork = int32_t(work.size());
			sp.work = dwork.as<int32_t>();
			sp.G = d.G;
			sp.len_s = dl.as<int32_t>();
			sp.len_t = dl.as<int32_t>() + B;
			sp.mask_off = dm.as<int64_t>();
			sp.masks = static_cast<const uint4 *>(d.dev_masks_all);
			sp.seeds = dsd.as<int2>();
			sp.seed_off = dsoff.as<int64_t>();
			sp.seed_cap = dscap.as<int32_t>();
			sp.seed_n = dsn.as<int32_t>();
			const int grid = int(std::min<int64_t>(int64_t(work.size()), int64_t(sms) * 8));
			PA_CUDA(pa::enum_seed_scan(sp, grid, nullptr));
			std::vector<int32_t> got(static_cast<size_t>(B));
			std::vector<int2> buf(size_t(std::max<int64_t>(off[size_t(B)], 1)));
			PA_CUDA(cudaMemcpy(got.data(), dsn.p, size_t(B) * 4, cudaMemcpyDeviceToHost));
			PA_CUDA(cudaMemcpy(buf.data(), dsd.p, size_t(off[size_t(B)]) * 8, cudaMemcpyDeviceToHost));
			std::vector<int32_t> again;
			for (int32_t L : work) {
				if (got[size_t(L)] > cap[size_t(L)]) {  // more seeds than room: scan this lane again
					again.push_back(L);
					continue;
				}
				auto &f = found[size_t(L)];
				f.clear();
				for (int32_t x = 0; x < got[size_t(L)]; x++) {
					const int2 c = buf[size_t(off[size_t(L)] + x)];
					f.push_back({c.x, c.y});
				}
				std::sort(f.begin(), f.end());
				n[size_t(L)] = got[size_t(L)];
			}
			std::fill(cap.begin(), cap.end(), 0);
			for (int32_t L : again) cap[size_t(L)] = got[size_t(L)];
			work.swap(again);
		}
		std::vector<int64_t> off(size_t(B) + 1, 0);
		for (int64_t L = 0; L < B; L++) off[size_t(L) + 1] = off[size_t(L)] + n[size_t(L)];
		std::vector<int2> flat(size_t(std::max<int64_t>(off[size_t(B)], 1)));
		for (int64_t L = 0; L < B; L++)
			for (size_t x = 0; x < found[size_t(L)].size(); x++)
				flat[size_t(off[size_t(L)]) + x] = make_int2(found[size_t(L)][x].first, found[size_t(L)][x].second);
		PA_CUDA(dsd.ensure(flat.size() * 8));
		PA_CUDA(dsoff.ensure(size_t(B) * 8));
		PA_CUDA(dsn.ensure(size_t(B) * 4));
		PA_CUDA(cudaMemcpy(dsd.p, flat.data(), flat.size() * 8, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dsoff.p, off.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dsn.p, n.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
	}

	// ---- the search
	PA_CUDA(dpath.ensure(size_t(woff[size_t(B)]) * 8));
	PA_CUDA(dmaps.ensure(size_t(std::max<int64_t>(moff[size_t(B)], 1)) * 4));
	if (paths) {
		PA_CUDA(dpaths.ensure(size_t(std::max<int64_t>(poff[size_t(B)], 1)) * 8));
		PA_CUDA(dplen.ensure(size_t(B * K) * 4));
	}
	PA_CUDA(dhash.ensure(size_t(B * K) * 8));
	PA_CUDA(dnpts.ensure(size_t(B * K) * 4));
	PA_CUDA(dcnt.ensure(size_t(B) * 4));
	PA_CUDA(dstat.ensure(size_t(B) * 4));
	DevBuf dmo, dpo, dwo;
	PA_CUDA(dmo.ensure(size_t(B) * 8));
	PA_CUDA(dpo.ensure(size_t(B) * 8));
	PA_CUDA(dwo.ensure(size_t(B) * 8));
	PA_CUDA(cudaMemcpy(dmo.p, moff.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dpo.p, poff.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
	PA_CUDA(cudaMemcpy(dwo.p, woff.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
	// stacks: |s| + |t| + 66 entries per lane at first; a lane that fills its stack is
	// enumerated again with four times the room
	std::vector<int32_t> scap(static_cast<size_t>(B), 0);
	int64_t stack0 = -1;
	if (const char *e = std::getenv("PA_ENUM_STACK")) stack0 = std::max(1, std::atoi(e));  // tests
	for (int64_t L = 0; L < B; L++)
		scap[size_t(L)] = int32_t(stack0 > 0 ? stack0 : d.ls[size_t(L)] + d.lt[size_t(L)] + 66);
	std::vector<int32_t> work = all, status(static_cast<size_t>(B), 0);
	DevBuf dstk, dsto, dscp;
	PA_CUDA(dsto.ensure(size_t(B) * 8));
	PA_CUDA(dscp.ensure(size_t(B) * 4));
	for (int round = 0; !work.empty(); round++) {
		std::vector<int64_t> so(static_cast<size_t>(B), 0);
		int64_t tot = 0;
		for (int32_t L : work) {
			so[size_t(L)] = tot;
			tot += scap[size_t(L)];
		}
		if (tot > (int64_t(1) << 31))
			return fail(PA_ERR_INTERNAL, "device enumeration: the search stacks outgrow the device");
		PA_CUDA(dstk.ensure(size_t(std::max<int64_t>(tot, 1)) * 16));
		PA_CUDA(cudaMemcpy(dsto.p, so.data(), size_t(B) * 8, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dscp.p, scap.data(), size_t(B) * 4, cudaMemcpyHostToDevice));
		PA_CUDA(cudaMemcpy(dwork.p, work.data(), work.size() * 4, cudaMemcpyHostToDevice));
		pa::EnumParams ep{};
		ep.nwork = int32_t(work.size());
		ep.work = dwork.as<int32_t>();
		ep.G = d.G;
		ep.local = local ? 1 : 0;
		ep.affine = d.gap == GAP_AFFINE ? 1 : 0;
		ep.remove_dup = d.remove_dup ? 1 : 0;
		ep.k = k;
		ep.len_s = dl.as<int32_t>();
		ep.len_t = dl.as<int32_t>() + B;
		ep.mask_off = dm.as<int64_t>();
		ep.masks = static_cast<const uint4 *>(d.dev_masks_all);
		ep.has = dhas.as<int32_t>();
		ep.seed = dseed.as<int32_t>();
		ep.seeds = local ? dsd.as<int2>() : nullptr;
		ep.seed_off = local ? dsoff.as<int64_t>() : nullptr;
		ep.seed_n = local ? dsn.as<int32_t>() : nullptr;
		ep.stack = dstk.as<int4>();
		ep.stack_off = dsto.as<int64_t>();
		ep.stack_cap = dscp.as<int32_t>();
		ep.path = dpath.as<int2>();
		ep.path_off = dwo.as<int64_t>();
		ep.maps = dmaps.as<int32_t>();
		ep.map_off = dmo.as<int64_t>();
		ep.paths = paths ? dpaths.as<int2>() : nullptr;
		ep.paths_off = dpo.as<int64_t>();
		ep.path_len = paths ? dplen.as<int32_t>() : nullptr;
		ep.hash = dhash.as<unsigned long long>();
		ep.npts = dnpts.as<int32_t>();
		ep.count = dcnt.as<int32_t>();
		ep.status = dstat.as<int32_t>();
		PA_CUDA(pa::enum_solve(ep, nullptr));
		PA_CUDA(cudaMemcpy(status.data(), dstat.p, size_t(B) * 4, cudaMemcpyDeviceToHost));
		std::vector<int32_t> again;
		for (int32_t L : work) {
			if (status[size_t(L)] == pa::ENUM_BAD_PATH)
				return fail(PA_ERR_INTERNAL, "device enumeration: a path outgrew |s| + |t| + 2 points");
			if (status[size_t(L)] == pa::ENUM_OVERFLOW) {
				if (scap[size_t(L)] > (1 << 28)) return fail(PA_ERR_INTERNAL, "device enumeration: stack limit");
				scap[size_t(L)] *= 4;
				again.push_back(L);
			}
		}
		work.swap(again);
	}
	PA_CUDA(cudaMemcpy(counts, dcnt.p, size_t(B) * 4, cudaMemcpyDeviceToHost));
	if (maps && moff[size_t(B)] > 0)
		PA_CUDA(cudaMemcpy(maps, dmaps.p, size_t(moff[size_t(B)]) * 4, cudaMemcpyDeviceToHost));
	if (paths) {
		if (poff[size_t(B)] > 0)
			PA_CUDA(cudaMemcpy(paths, dpaths.p, size_t(poff[size_t(B)]) * 8, cudaMemcpyDeviceToHost));
		PA_CUDA(cudaMemcpy(path_len, dplen.p, size_t(B * K) * 4, cudaMemcpyDeviceToHost));
	}
	return PA_OK;
}

}  // extern "C"

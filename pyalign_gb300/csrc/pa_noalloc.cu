// Score-only batched solve that allocates no memory (pa_solve_indexed_for_score_noalloc).
//
// Some callers cannot allocate device memory while they run: a caller that owns every byte
// of the GPU through its own pool (a serving process that reserved HBM up front), a caller
// inside a context where cudaMalloc would synchronise the device and stall other streams,
// or a caller that simply must not fail on allocation half-way through a request.  This
// entry point takes device-resident inputs and outputs from the caller and keeps all of
// its scratch -- the per-group boundary rows of the wavefront, the direction-normalised
// similarity table, the border vectors, the pair order, the per-pair seed slots and the
// work counter -- in one file-scope device array of PA_NOALLOC_SCRATCH_BYTES.  It calls no
// cudaMalloc/cudaFree and no allocating library routine; only a rejected call stores its
// error text (read with pa_last_error) in host memory.
//
// The array is shared by every call on a device and keeps the last call's contents; the
// parts that must start at zero (the work counter, the kernel's status word, the code
// maxima) are cleared by each call.  Each call waits on `stream` for the check that every
// code indexes the table (the host reads the maxima back), so the call returns only after
// the work queued on `stream` before it has finished; the DP itself is left running.  Calls whose
// GPU work overlaps (two streams, or two threads on one stream without ordering) race on
// the array and give wrong results.  The first call on a device looks up the array's device
// address with cudaGetSymbolAddress, once per device, with that device current; make that
// first call before any stream capture.

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/pyalign_gb300.h"
#include "pa_dp.cuh"
#include "pa_launch.h"

using namespace pa;

namespace {

constexpr size_t SCRATCH_BYTES = size_t(PA_NOALLOC_SCRATCH_BYTES);
constexpr int64_t MAX_BATCH = PA_NOALLOC_MAX_BATCH;
constexpr int64_t MAX_LEN = PA_NOALLOC_MAX_LEN;
constexpr int64_t MAX_TABLE = 64;  // alphabet size (the table is staged in shared memory)

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void *g_addr[MAX_DEVICES] = {};


struct Prep {
	int64_t batch, n_s, n_t, rows, cols;
	const float *table;  // caller's (reference-domain) table
	float *table_out;    // direction-normalised copy
	float *left_D, *top_D;
	int32_t *order;
	int32_t *counter;
	int32_t *status;     // the DP kernel's status word (progress timeouts, bad codes)
	const int32_t *len_s_in, *len_t_in;  // caller's lengths
	int32_t *len_s, *len_t;              // clamped to [0, n_s] x [0, n_t]
	int32_t global;      // 1: global borders -w(k), else 0
	int32_t gap_kind;
	float sign, gsgn;    // +1/-1 maximize/minimize; gap_sgn of the reference
	float lin_s, lin_t, u_s, v_s, u_t, v_t;
};

// Gotoh border w(k) = u k + v via the xtensor linspace of AffineCost::vector
// (solver.h:2876-2880), in IEEE round-to-nearest operations as the host computes it.
__device__ float affine_w(float u, float v, int64_t n, int64_t k) {
	if (k == 0) return 0.0f;
	const float stop = __fmul_rn(float(n - 1), u);
	const float step = n > 1 ? __fdiv_rn(__fsub_rn(stop, 0.0f), float(n - 1)) : 0.0f;
	return __fadd_rn(__fadd_rn(0.0f, __fmul_rn(step, float(k))), v);
}

__global__ void noalloc_prep_kernel(Prep p) {
	const int64_t stride = int64_t(gridDim.x) * blockDim.x;
	const int64_t t0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t0 == 0) {
		*p.counter = 0;
		*p.status = 0;
	}
	for (int64_t k = t0; k < p.batch; k += stride) {
		p.order[k] = int32_t(k);
		p.len_s[k] = int32_t(min(max(int64_t(p.len_s_in[k]), int64_t(0)), p.n_s));
		p.len_t[k] = int32_t(min(max(int64_t(p.len_t_in[k]), int64_t(0)), p.n_t));
	}
	for (int64_t k = t0; k < p.rows * p.cols; k += stride) p.table_out[k] = __fmul_rn(p.table[k], p.sign);
	for (int64_t k = t0; k <= p.n_s; k += stride) {
		float w = 0.0f;
		if (p.global) {
			const float ref = p.gap_kind == PA_GAP_LINEAR ? __fmul_rn(__fmul_rn(float(k), p.lin_s), p.gsgn)
			                                              : __fmul_rn(affine_w(p.u_s, p.v_s, p.n_s + 1, k), p.gsgn);
			w = __fmul_rn(ref, p.sign);
		}
		p.left_D[k] = w;
	}
	for (int64_t k = t0; k <= p.n_t; k += stride) {
		float w = 0.0f;
		if (p.global) {
			const float ref = p.gap_kind == PA_GAP_LINEAR ? __fmul_rn(__fmul_rn(float(k), p.lin_t), p.gsgn)
			                                              : __fmul_rn(affine_w(p.u_t, p.v_t, p.n_t + 1, k), p.gsgn);
			w = __fmul_rn(ref, p.sign);
		}
		p.top_D[k] = w;
	}
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

namespace pa {
pa_status wsb_fail(pa_status st, const std::string &m);  // the library's error slot (pa_last_error)
}  // namespace pa

namespace {

// Rejections record their message in the library's error slot, read by pa_last_error().
pa_status reject(pa_status st, const char *msg) { return pa::wsb_fail(st, msg); }

}  // namespace

extern "C" pa_status pa_solve_indexed_for_score_noalloc(const pa_options *o, const uint32_t *a, const uint32_t *b,
                                                        int64_t batch, int64_t n_s, int64_t n_t, const float *table,
                                                        int64_t table_rows, int64_t table_cols, const int32_t *len_s,
                                                        const int32_t *len_t, float *scores, void *stream) {
	if (!o || !a || !b || !table || !len_s || !len_t || !scores)
		return reject(PA_ERR_INVALID_ARGUMENT, "pa_solve_indexed_for_score_noalloc: null argument");
	if (o->type != PA_TYPE_ALIGNMENT || (o->gap_kind != PA_GAP_LINEAR && o->gap_kind != PA_GAP_AFFINE))
		return reject(PA_ERR_UNSUPPORTED, "pa_solve_indexed_for_score_noalloc: linear or affine gap costs only");
	if (o->locality < 0 || o->locality > 2 || (o->direction != PA_MINIMIZE && o->direction != PA_MAXIMIZE))
		return reject(PA_ERR_INVALID_ARGUMENT, "pa_solve_indexed_for_score_noalloc: invalid locality or direction");
	if (batch < 0 || batch > MAX_BATCH)
		return reject(PA_ERR_LENGTH, "pa_solve_indexed_for_score_noalloc: batch exceeds PA_NOALLOC_MAX_BATCH (65536)");
	if (n_s < 0 || n_t < 0 || n_s > MAX_LEN || n_t > MAX_LEN)
		return reject(PA_ERR_LENGTH, "pa_solve_indexed_for_score_noalloc: sequence length exceeds PA_NOALLOC_MAX_LEN (4096)");
	if (table_rows < 1 || table_cols < 1 || table_rows > MAX_TABLE || table_cols > MAX_TABLE)
		return reject(PA_ERR_LENGTH, "pa_solve_indexed_for_score_noalloc: similarity table larger than 64 x 64");
	if (batch == 0) return PA_OK;

	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
		cudaGetLastError();
		return reject(PA_ERR_NO_DEVICE, "pa_solve_indexed_for_score_noalloc: no usable CUDA device");
	}
	void *base = nullptr;
	{
		std::lock_guard<std::mutex> lock(g_mu);
		if (!g_addr[dev]) {
			// once per device, with the device current
			if (cudaGetSymbolAddress(&g_addr[dev], g_noalloc_scratch) != cudaSuccess) {
				cudaGetLastError();
				g_addr[dev] = nullptr;
				return reject(PA_ERR_CUDA, "pa_solve_indexed_for_score_noalloc: cudaGetSymbolAddress failed");
			}
		}
		base = g_addr[dev];
	}
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

	// scratch layout
	unsigned char *cur = static_cast<unsigned char *>(base);
	auto take = [&](size_t n) {
		unsigned char *x = cur;
		cur += align256(n);
		return x;
	};
	int32_t *counter = reinterpret_cast<int32_t *>(take(8));
	int32_t *status = reinterpret_cast<int32_t *>(take(8));
	uint32_t *codes_max = reinterpret_cast<uint32_t *>(take(8));
	int32_t *order = reinterpret_cast<int32_t *>(take(size_t(batch) * 4));
	int32_t *seeds = reinterpret_cast<int32_t *>(take(size_t(batch) * 8));
	int32_t *has = reinterpret_cast<int32_t *>(take(size_t(batch) * 4));
	int32_t *cls = reinterpret_cast<int32_t *>(take(size_t(batch) * 4));
	int32_t *clt = reinterpret_cast<int32_t *>(take(size_t(batch) * 4));
	float *tab = reinterpret_cast<float *>(take(size_t(table_rows * table_cols) * 4));
	float *left_D = reinterpret_cast<float *>(take(size_t(n_s + 1) * 4));
	float *top_D = reinterpret_cast<float *>(take(size_t(n_t + 1) * 4));
	const size_t used = size_t(cur - static_cast<unsigned char *>(base));
	const size_t row_bytes = size_t(2) * size_t(std::max<int64_t>(n_t, 1)) * sizeof(float2);  // per group slot
	const int G = 32;
	const int64_t slots_fit = int64_t((SCRATCH_BYTES - used) / row_bytes);
	int sms = 0;
	if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
		cudaGetLastError();
		return reject(PA_ERR_CUDA, "pa_solve_indexed_for_score_noalloc: cannot read the SM count of the device");
	}
	int64_t blocks = std::min<int64_t>(int64_t(sms) * 4, slots_fit / WARPS);
	blocks = std::min<int64_t>(blocks, (batch + WARPS - 1) / WARPS);
	if (blocks < 1) return reject(PA_ERR_LENGTH, "pa_solve_indexed_for_score_noalloc: scratch too small for this length");
	float2 *rows = reinterpret_cast<float2 *>(cur);

	// codes must index the table (factory.h:602-614)
	if (cudaMemsetAsync(codes_max, 0, 8, st) != cudaSuccess) return reject(PA_ERR_CUDA, "cudaMemsetAsync failed");
	const int cgrid = std::max(1, std::min(sms * 4, int((batch * std::max(n_s, n_t) + 255) / 256)));
	if (batch * n_s > 0) codes_max_kernel<<<cgrid, 256, 0, st>>>(a, batch * n_s, codes_max);
	if (batch * n_t > 0) codes_max_kernel<<<cgrid, 256, 0, st>>>(b, batch * n_t, codes_max + 1);
	uint32_t mx[2] = {0, 0};
	if (cudaMemcpyAsync(mx, codes_max, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	    cudaStreamSynchronize(st) != cudaSuccess)
		return reject(PA_ERR_CUDA, "pa_solve_indexed_for_score_noalloc: CUDA error in the code check");
	if (batch * n_s > 0 && int64_t(mx[0]) >= table_rows)
		return reject(PA_ERR_INVALID_ARGUMENT, "out of bounds index in a");
	if (batch * n_t > 0 && int64_t(mx[1]) >= table_cols)
		return reject(PA_ERR_INVALID_ARGUMENT, "out of bounds index in b");

	const float sign = o->direction == PA_MAXIMIZE ? 1.0f : -1.0f;
	Prep pr{};
	pr.batch = batch;
	pr.n_s = n_s;
	pr.n_t = n_t;
	pr.rows = table_rows;
	pr.cols = table_cols;
	pr.table = table;
	pr.table_out = tab;
	pr.left_D = left_D;
	pr.top_D = top_D;
	pr.order = order;
	pr.counter = counter;
	pr.status = status;
	pr.len_s_in = len_s;
	pr.len_t_in = len_t;
	pr.len_s = cls;
	pr.len_t = clt;
	pr.global = o->locality == PA_GLOBAL;
	pr.gap_kind = o->gap_kind;
	pr.sign = sign;
	pr.gsgn = o->direction == PA_MINIMIZE ? 1.0f : -1.0f;
	pr.lin_s = o->linear_s;
	pr.lin_t = o->linear_t;
	pr.u_s = o->affine_u_s;
	pr.v_s = o->affine_v_s;
	pr.u_t = o->affine_u_t;
	pr.v_t = o->affine_v_t;
	noalloc_prep_kernel<<<std::max(1, sms), 256, 0, st>>>(pr);

	DpParams<float> p{};
	p.npairs = int32_t(batch);
	p.order = order;
	p.len_s = cls;
	p.len_t = clt;
	p.a = a;
	p.b = b;
	p.a_stride = n_s;
	p.b_stride = n_t;
	p.sub_kind = SUB_TABLE;
	p.table = tab;
	p.table_rows = int32_t(table_rows);
	p.table_cols = int32_t(table_cols);
	if (o->gap_kind == PA_GAP_LINEAR) {
		p.c_up = -o->linear_s;
		p.c_left = -o->linear_t;
	} else {
		p.c_open_s = -(o->affine_u_s + o->affine_v_s);
		p.c_ext_s = -o->affine_u_s;
		p.c_open_t = -(o->affine_u_t + o->affine_v_t);
		p.c_ext_t = -o->affine_u_t;
	}
	p.left_D = left_D;
	p.top_D = top_D;
	p.left_P = left_D;
	p.top_Q = top_D;
	p.neg_inf = -INFINITY;
	p.G = G;
	p.one = 1;
	p.minus_one = -1;
	p.minus_four = -4;
	p.minus_eight = -8;
	p.sixteen = 16;
	p.two = 2;
	p.bit16 = 65536;
	p.score = scores;
	p.seed = seeds;
	p.has_seed = has;
	p.out_sign = sign;
	p.scratch = rows;
	p.scratch_stride = 2 * std::max<int64_t>(n_t, 1);
	p.work_counter = counter;
	p.status = status;
	const int loc = o->locality == PA_LOCAL ? LOC_LOCAL : o->locality == PA_GLOBAL ? LOC_GLOBAL : LOC_SEMI;
	const size_t smem = size_t(table_rows * table_cols) * sizeof(float);
	cudaError_t e = o->gap_kind == PA_GAP_LINEAR ? launch_dp_f_linear(loc, TB_NONE, false, p, int(blocks), smem, st)
	                                              : launch_dp_f_affine(loc, TB_NONE, false, p, int(blocks), smem, st);
	if (e != cudaSuccess) return reject(PA_ERR_CUDA, "pa_solve_indexed_for_score_noalloc: kernel launch failed");
	return PA_OK;
}

// Backward of the optimal alignment score: the max-plus subgradient along the optimal path.
//
// The score of an alignment is the sum of the similarities of its aligned cells minus the
// costs of its gaps (maximize; plus for minimize), so its derivative is 1 for every
// aligned (diagonal-step) cell of the optimal path, 0 elsewhere, and -(number of gaps) /
// -(sum of gap lengths - 1) for the open / extend costs, w(k) = open + extend (k - 1)
// (pyalign/gaps.py:164-193 with solver.h:2858-2881).  For DTW the score is the sum of the
// distances of every visited cell (solver.h:3233-3250).  Global alignments also pay the
// border gap their path ends in (solver.h:2918-2951).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/pyalign_gb300.h"

namespace {

struct GradParams {
	int64_t batch;
	int32_t dtw, global;
	float gap_sign;  // -1 maximize, +1 minimize (gap_sgn of solver.h:2807)
	const int32_t *paths;
	const int64_t *path_off;
	const int32_t *path_len;
	const float *grad;
	float *dS;
	const int64_t *ds_off;
	int64_t ss, st;
	float *dgap;  // 4 per pair: open_s, extend_s, open_t, extend_t
};

__global__ void path_grad_kernel(GradParams p) {
	const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (k >= p.batch) return;
	const float g = p.grad[k];
	const int n = p.path_len[k];
	const int32_t *P = p.paths + p.path_off[k];
	float *d = p.dS ? p.dS + p.ds_off[k] : nullptr;
	int open_s = 0, ext_s = 0, open_t = 0, ext_t = 0;
	for (int q = 0; q + 1 < n; q++) {
		const int u0 = P[2 * q], v0 = P[2 * q + 1], u1 = P[2 * q + 2], v1 = P[2 * q + 3];
		if (u0 < 0 || v0 < 0) break;
		if (p.dtw) {
			if (d) d[int64_t(u0) * p.ss + int64_t(v0) * p.st] += g;
		} else if (u1 == u0 - 1 && v1 == v0 - 1) {
			if (d) d[int64_t(u0) * p.ss + int64_t(v0) * p.st] += g;
		} else if (v1 == v0 && u1 < u0) {
			open_s += 1;
			ext_s += u0 - u1 - 1;
		} else if (u1 == u0 && v1 < v0) {
			open_t += 1;
			ext_t += v0 - v1 - 1;
		}
	}
	if (n > 0 && p.global && !p.dtw) {
		const int ul = P[2 * (n - 1)], vl = P[2 * (n - 1) + 1];
		if (ul < 0 && vl >= 0) {  // D(-1, vl) = w_t(vl + 1)
			open_t += 1;
			ext_t += vl;
		} else if (vl < 0 && ul >= 0) {  // D(ul, -1) = w_s(ul + 1)
			open_s += 1;
			ext_s += ul;
		}
	}
	if (p.dgap) {
		const float c = p.gap_sign * g;
		p.dgap[4 * k + 0] = c * float(open_s);
		p.dgap[4 * k + 1] = c * float(ext_s);
		p.dgap[4 * k + 2] = c * float(open_t);
		p.dgap[4 * k + 3] = c * float(ext_t);
	}
}

}  // namespace

extern "C" pa_status pa_path_gradients(int32_t type, int32_t locality, int32_t direction, int64_t batch,
                                       const int32_t *paths, const int64_t *path_offsets, const int32_t *path_len,
                                       const float *grad_scores, float *dS, const int64_t *ds_offsets,
                                       int64_t stride_s, int64_t stride_t, float *dgap, void *stream) {
	if (batch < 0 || !paths || !path_offsets || !path_len || !grad_scores || (dS && !ds_offsets))
		return PA_ERR_INVALID_ARGUMENT;
	if (batch == 0) return PA_OK;
	GradParams p{};
	p.batch = batch;
	p.dtw = type == PA_TYPE_DTW;
	p.global = type == PA_TYPE_DTW || locality == PA_GLOBAL;
	p.gap_sign = direction == PA_MINIMIZE ? 1.0f : -1.0f;
	p.paths = paths;
	p.path_off = path_offsets;
	p.path_len = path_len;
	p.grad = grad_scores;
	p.dS = dS;
	p.ds_off = ds_offsets;
	p.ss = stride_s;
	p.st = stride_t;
	p.dgap = dgap;
	path_grad_kernel<<<int((batch + 127) / 128), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(p);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

// ---------------------------------------------------------------------------------------
// Similarity-matrix problems built from per-token embeddings, S(i, j) = <en_s[i], en_t[j]>
// with en = E / |E| (cosine) or en = E (dot), multiplied in BF16 with FP32 accumulation.
//
// normalize_rows_bf16_kernel: one warp per row writes the BF16 factor and 1/|E| in one
// pass over E.  path_embedding_grad_kernel: dScore/dE[i] for the aligned cells (i, j) of
// each pair's optimal path only -- the gradient of S w.r.t. en_s[i] is g * en_t_bf16[j]
// (the BF16 cast passes gradients through), then the normalisation backward
// (g - (g . en) en) / |E| -- without materialising dS.  In one path the aligned cells
// have distinct i and distinct j, so a warp per pair writes without atomics.

namespace {

__global__ void normalize_rows_bf16_kernel(const float *E, int64_t rows, int32_t dim, int32_t normalize,
                                           __nv_bfloat16 *out, float *inv_norm) {
	const int64_t r = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (r >= rows) return;
	const float *x = E + r * dim;
	float ss = 0.0f;
	for (int c = lane; c < dim; c += 32) ss += x[c] * x[c];
	for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
	const float inv = normalize ? 1.0f / fmaxf(sqrtf(ss), 1e-12f) : 1.0f;
	for (int c = lane; c < dim; c += 32) out[r * dim + c] = __float2bfloat16_rn(x[c] * inv);
	if (lane == 0) inv_norm[r] = inv;
}

// The same with each pair's length: rows past it get a zero factor and 1/|E| = 0 without
// reading E (the product's padding rows must be zero, and their values are never used);
// rows of a width that is a multiple of 4 are read as 16-byte words.
__global__ void normalize_rows_bf16_len_kernel(const float *E, int64_t batch, int64_t n, int32_t dim,
                                               int32_t normalize, const int32_t *len, int32_t tile,
                                               __nv_bfloat16 *out, float *inv_norm) {
	const int64_t r = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (r >= batch * n) return;
	const int64_t k = r / n, i = r - k * n;
	__nv_bfloat16 *o = out + r * dim;
	if (tile > 0 && i >= (int64_t(len[k]) + tile - 1) / tile * tile) return;  // past the last tile: not written
	if (i >= len[k]) {
		for (int c = lane; c < dim; c += 32) o[c] = __float2bfloat16_rn(0.0f);
		if (lane == 0) inv_norm[r] = 0.0f;
		return;
	}
	const float *x = E + r * dim;
	const bool vec = (dim & 3) == 0;
	float ss = 0.0f;
	if (vec) {
		for (int c = 4 * lane; c < dim; c += 128) {
			const float4 v = *reinterpret_cast<const float4 *>(x + c);
			ss += v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
		}
	} else {
		for (int c = lane; c < dim; c += 32) ss += x[c] * x[c];
	}
	for (int o2 = 16; o2 > 0; o2 >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o2);
	const float inv = normalize ? 1.0f / fmaxf(sqrtf(ss), 1e-12f) : 1.0f;
	if (vec) {
		for (int c = 4 * lane; c < dim; c += 128) {
			const float4 v = *reinterpret_cast<const float4 *>(x + c);
			__nv_bfloat162 w[2] = {__floats2bfloat162_rn(v.x * inv, v.y * inv), __floats2bfloat162_rn(v.z * inv, v.w * inv)};
			*reinterpret_cast<uint2 *>(o + c) = *reinterpret_cast<const uint2 *>(w);  // 8-byte store
		}
	} else {
		for (int c = lane; c < dim; c += 32) o[c] = __float2bfloat16_rn(x[c] * inv);
	}
	if (lane == 0) inv_norm[r] = inv;
}

// The same for widths that are a multiple of 4 up to 512, the common case: a warp takes RPW
// rows at once -- every lane issues its NV 16-byte loads of all RPW rows before any sum is
// reduced, so a warp keeps RPW * NV loads in flight instead of one row's -- holds the rows
// in registers (one read of E), and writes each lane's four BF16 values as one 8-byte store,
// zeros included.  The sums run in the order of the kernel above, so the factors and 1/|E|
// are the same bit for bit.
// tile > 0: rows from each length rounded up to a multiple of tile on are not written.
template <int NV, int RPW>
__global__ void __launch_bounds__(256) normalize_rows_bf16_rows_kernel(const float *E, int64_t batch, int64_t n,
                                                                      int32_t dim, int32_t normalize,
                                                                      const int32_t *len, int32_t tile,
                                                                      __nv_bfloat16 *out, float *inv_norm) {
	const int lane = threadIdx.x & 31;
	const int64_t rows = batch * n;
	const int64_t r0 = ((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * RPW;
	if (r0 >= rows) return;  // whole warps
	float4 v[RPW][NV];
	bool has[RPW], put[RPW];
	// (pair, row) of the warp's first row by one division, then stepped (a 64-bit division
	// per row would dominate this kernel's instructions)
	int64_t k = r0 / n, i = r0 - k * n;
#pragma unroll
	for (int q = 0; q < RPW; q++) {
		const int64_t r = r0 + q;
		if (q > 0) {
			if (++i == n) {
				i = 0;
				k++;
			}
		}
		bool h = r < rows, w = h;
		if (h) {
			const int32_t m = len[k];
			h = i < m;
			w = tile <= 0 || i < (int64_t(m) + tile - 1) / tile * tile;
		}
		has[q] = h;
		put[q] = w;
#pragma unroll
		for (int j = 0; j < NV; j++) {
			const int c = 4 * lane + 128 * j;
			v[q][j] = (h && c < dim) ? *reinterpret_cast<const float4 *>(E + r * dim + c) : make_float4(0.f, 0.f, 0.f, 0.f);
		}
	}
#pragma unroll
	for (int q = 0; q < RPW; q++) {
		const int64_t r = r0 + q;
		float ss = 0.0f;
#pragma unroll
		for (int j = 0; j < NV; j++)
			if (4 * lane + 128 * j < dim) {
				const float4 x = v[q][j];
				ss += x.x * x.x + x.y * x.y + x.z * x.z + x.w * x.w;
			}
		for (int o2 = 16; o2 > 0; o2 >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o2);
		const float inv = has[q] ? (normalize ? 1.0f / fmaxf(sqrtf(ss), 1e-12f) : 1.0f) : 0.0f;
		if (r < rows && put[q]) {
#pragma unroll
			for (int j = 0; j < NV; j++) {
				const int c = 4 * lane + 128 * j;
				if (c < dim) {
					const float4 x = v[q][j];
					__nv_bfloat162 w[2] = {__floats2bfloat162_rn(x.x * inv, x.y * inv), __floats2bfloat162_rn(x.z * inv, x.w * inv)};
					*reinterpret_cast<uint2 *>(out + r * dim + c) = *reinterpret_cast<const uint2 *>(w);
				}
			}
			if (lane == 0) inv_norm[r] = inv;
		}
	}
}

struct EmbGradParams {
	int64_t batch;
	int32_t dim, normalize;
	const int32_t *paths;
	const int64_t *path_off;
	const int32_t *path_len;
	const float *grad;
	const float *Es, *Et;                 // raw embeddings (batch, n, dim)
	const __nv_bfloat16 *Esb, *Etb;       // the BF16 factors of the product
	const float *inv_s, *inv_t;           // 1/|E| per row (1 when not normalising)
	float *dEs, *dEt;                     // zero except on aligned rows
	int64_t n_s, n_t;
	int32_t zero_rest;                    // vector kernel: also write the zero rows (see there)
};

__device__ __forceinline__ float warp_sum(float x) {
	for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
	return x;
}

__global__ void path_embedding_grad_kernel(EmbGradParams p) {
	const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (k >= p.batch) return;
	const float g = p.grad[k];
	const int n = p.path_len[k];
	const int32_t *P = p.paths + p.path_off[k];
	const int64_t bs = k * p.n_s, bt = k * p.n_t;
	for (int q = 0; q + 1 < n; q++) {
		const int u0 = P[2 * q], v0 = P[2 * q + 1];
		if (u0 < 0 || v0 < 0) break;
		const int u1 = P[2 * q + 2], v1 = P[2 * q + 3];
		if (!(u1 == u0 - 1 && v1 == v0 - 1)) continue;
		const int64_t ri = (bs + u0) * p.dim, rj = (bt + v0) * p.dim;
		const float is = p.inv_s[bs + u0], it = p.inv_t[bt + v0];
		float dots = 0.0f, dott = 0.0f;
		for (int c = lane; c < p.dim; c += 32) {
			dots += g * __bfloat162float(p.Etb[rj + c]) * p.Es[ri + c] * is;
			dott += g * __bfloat162float(p.Esb[ri + c]) * p.Et[rj + c] * it;
		}
		if (p.normalize) {
			dots = warp_sum(dots);
			dott = warp_sum(dott);
		}
		for (int c = lane; c < p.dim; c += 32) {
			const float gs = g * __bfloat162float(p.Etb[rj + c]);
			const float gt = g * __bfloat162float(p.Esb[ri + c]);
			if (p.normalize) {
				p.dEs[ri + c] = (gs - dots * p.Es[ri + c] * is) * is;
				p.dEt[rj + c] = (gt - dott * p.Et[rj + c] * it) * it;
			} else {
				p.dEs[ri + c] = gs;
				p.dEt[rj + c] = gt;
			}
		}
	}
}

// The same gradients, four aligned cells at a time per warp (widths that are a multiple of
// 32): lanes examine 32 path steps at once and a ballot lists the aligned ones (the scan
// stops at the first point with a negative coordinate, as above); each 8-lane quarter of
// the warp then takes one listed cell, reads its rows with 16-byte loads (lane l holds
// elements 4l + 32t) and reduces over its 8 lanes.  Four independent cells in flight per
// warp instead of one dependent chain of row loads.
__device__ __forceinline__ float quarter_sum(float x) {
	for (int o = 4; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
	return x;
}

__device__ __forceinline__ float4 bf16x4(const __nv_bfloat16 *p4) {
	const uint2 w = *reinterpret_cast<const uint2 *>(p4);
	return make_float4(__uint_as_float(w.x << 16), __uint_as_float(w.x & 0xffff0000u), __uint_as_float(w.y << 16),
	                   __uint_as_float(w.y & 0xffff0000u));
}

// With zero_rest the kernel writes every row of the pair's dE itself, so dE needs no
// zeroing beforehand (which would write the aligned rows twice): the warp first marks the
// rows of its aligned cells in a bitmap in shared memory (ceil(n_s / 32) + ceil(n_t / 32)
// words per warp, dynamic), stores zeros to the unmarked rows -- padding rows included --
// and then writes the aligned rows below.
__global__ void path_embedding_grad_vec_kernel(EmbGradParams p) {
	const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (k >= p.batch) return;
	const float g = p.grad[k];
	const int n = p.path_len[k];
	const int32_t *P = p.paths + p.path_off[k];
	const int64_t bs = k * p.n_s, bt = k * p.n_t;
	if (p.zero_rest) {
		extern __shared__ uint32_t row_marks[];
		const int ws = int((p.n_s + 31) >> 5), wt = int((p.n_t + 31) >> 5);
		uint32_t *ms = row_marks + (threadIdx.x >> 5) * (ws + wt), *mt = ms + ws;
		for (int w = lane; w < ws + wt; w += 32) ms[w] = 0u;
		__syncwarp();
		for (int q0 = 0; q0 + 1 < n; q0 += 32) {
			const int q = q0 + lane;
			int u0 = -1, v0 = -1;
			bool neg = false, al = false;
			if (q + 1 < n) {
				u0 = P[2 * q];
				v0 = P[2 * q + 1];
				neg = u0 < 0 || v0 < 0;
				al = !neg && P[2 * q + 2] == u0 - 1 && P[2 * q + 3] == v0 - 1;
			}
			const uint32_t negm = __ballot_sync(0xffffffffu, neg);
			const int stop = negm ? __ffs(int(negm)) - 1 : 32;
			if (al && lane < stop && u0 < p.n_s && v0 < p.n_t) {
				atomicOr(ms + (u0 >> 5), 1u << (u0 & 31));
				atomicOr(mt + (v0 >> 5), 1u << (v0 & 31));
			}
			if (negm) break;
		}
		__syncwarp();
		const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
		for (int64_t i = 0; i < p.n_s; i++)
			if (!((ms[i >> 5] >> (i & 31)) & 1u))
				for (int c = 4 * lane; c < p.dim; c += 128) *reinterpret_cast<float4 *>(p.dEs + (bs + i) * p.dim + c) = z;
		for (int64_t j = 0; j < p.n_t; j++)
			if (!((mt[j >> 5] >> (j & 31)) & 1u))
				for (int c = 4 * lane; c < p.dim; c += 128) *reinterpret_cast<float4 *>(p.dEt + (bt + j) * p.dim + c) = z;
	}
	const int quarter = lane >> 3, ql = lane & 7;
	const int chunks = p.dim >> 5;
	for (int q0 = 0; q0 + 1 < n; q0 += 32) {
		const int q = q0 + lane;
		int u0 = -1, v0 = -1;
		bool neg = false, al = false;
		if (q + 1 < n) {
			u0 = P[2 * q];
			v0 = P[2 * q + 1];
			neg = u0 < 0 || v0 < 0;
			al = !neg && P[2 * q + 2] == u0 - 1 && P[2 * q + 3] == v0 - 1;
		}
		const uint32_t negm = __ballot_sync(0xffffffffu, neg);
		const int stop = negm ? __ffs(int(negm)) - 1 : 32;  // steps from the first negative point on are not visited
		uint32_t am = __ballot_sync(0xffffffffu, al && lane < stop);
		while (am) {
			// this quarter's cell: the (quarter + 1)-th listed step; every lane runs every shuffle
			// below in the same order (a quarter without a cell only skips the memory accesses)
			uint32_t m = am;
			for (int c = 0; c < quarter; c++) m &= m - 1;
			const int src = m ? __ffs(int(m)) - 1 : 32;
			const int u = __shfl_sync(0xffffffffu, u0, src < 32 ? src : 0);
			const int v = __shfl_sync(0xffffffffu, v0, src < 32 ? src : 0);
			for (int c = 0; c < 4 && am; c++) am &= am - 1;  // the four cells of this pass
			const bool has = src < 32 && u >= 0 && u < p.n_s && v >= 0 && v < p.n_t;
			const int64_t ri = (bs + (has ? u : 0)) * p.dim, rj = (bt + (has ? v : 0)) * p.dim;
			const float is = has ? p.inv_s[bs + u] : 0.0f, it = has ? p.inv_t[bt + v] : 0.0f;
			float dots = 0.0f, dott = 0.0f;
			if (has) {
				for (int t = 0; t < chunks; t++) {
					const int e = 4 * ql + 32 * t;
					const float4 es = *reinterpret_cast<const float4 *>(p.Es + ri + e);
					const float4 et = *reinterpret_cast<const float4 *>(p.Et + rj + e);
					const float4 tb = bf16x4(p.Etb + rj + e), sb = bf16x4(p.Esb + ri + e);
					dots += g * tb.x * es.x * is + g * tb.y * es.y * is + g * tb.z * es.z * is + g * tb.w * es.w * is;
					dott += g * sb.x * et.x * it + g * sb.y * et.y * it + g * sb.z * et.z * it + g * sb.w * et.w * it;
				}
			}
			if (p.normalize) {
				dots = quarter_sum(dots);
				dott = quarter_sum(dott);
			}
			if (has) {
				for (int t = 0; t < chunks; t++) {
					const int e = 4 * ql + 32 * t;
					const float4 tb = bf16x4(p.Etb + rj + e), sb = bf16x4(p.Esb + ri + e);
					float4 os, ot;
					if (p.normalize) {
						const float4 es = *reinterpret_cast<const float4 *>(p.Es + ri + e);
						const float4 et = *reinterpret_cast<const float4 *>(p.Et + rj + e);
						os = make_float4((g * tb.x - dots * es.x * is) * is, (g * tb.y - dots * es.y * is) * is,
						                 (g * tb.z - dots * es.z * is) * is, (g * tb.w - dots * es.w * is) * is);
						ot = make_float4((g * sb.x - dott * et.x * it) * it, (g * sb.y - dott * et.y * it) * it,
						                 (g * sb.z - dott * et.z * it) * it, (g * sb.w - dott * et.w * it) * it);
					} else {
						os = make_float4(g * tb.x, g * tb.y, g * tb.z, g * tb.w);
						ot = make_float4(g * sb.x, g * sb.y, g * sb.z, g * sb.w);
					}
					*reinterpret_cast<float4 *>(p.dEs + ri + e) = os;
					*reinterpret_cast<float4 *>(p.dEt + rj + e) = ot;
				}
			}
		}
		if (negm) break;
	}
}

// DTW on two series with d(u, v) = |x_u - y_v|: every visited cell adds
// g * sign(x_u - y_v) to dx_u and subtracts it from dy_v.
//
// One warp per pair, 32 path points per step.  A DTW path is monotone (every step lowers u,
// v or both), so the points of one row u -- and those of one column v -- are consecutive: a
// segmented warp scan of the signs gives each run's count, and the run's last lane adds
// g * count to dx[u] (dy[v]).  A run that reaches the end of a step is carried into the next
// one.  Each dx[u], dy[v] thus has one writer, and the sum is g times an exact integer
// count, independent of the order of the points.
struct SeriesGradParams {
	int64_t batch;
	const int32_t *paths;
	const int64_t *path_off;
	const int32_t *path_len;
	const float *grad;
	const float *x, *y;
	float *dx, *dy;
	int64_t n_s, n_t;
};

// inclusive scan of a over the lanes' runs of equal key (runs are contiguous)
__device__ __forceinline__ int run_scan(int a, int key, int lane) {
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const int t = __shfl_up_sync(0xffffffffu, a, o);
		const int tk = __shfl_up_sync(0xffffffffu, key, o);
		if (lane >= o && tk == key) a += t;
	}
	return a;
}

__global__ void path_series_grad_kernel(SeriesGradParams p) {
	const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (k >= p.batch) return;  // whole warps
	const float g = p.grad[k];
	const int n = p.path_len[k];
	const int32_t *P = p.paths + p.path_off[k];
	const float *x = p.x + k * p.n_s;
	const float *y = p.y + k * p.n_t;
	float *dx = p.dx + k * p.n_s;
	float *dy = p.dy + k * p.n_t;
	int cu = -1, cv = -1, cx = 0, cy = 0;  // the runs carried from the last step (warp-uniform)
	for (int q0 = 0; q0 < n; q0 += 32) {
		const int q = q0 + lane;
		int u = -1, v = -1, sg = 0;
		if (q < n) {
			u = P[2 * q];
			v = P[2 * q + 1];
		}
		if (u >= 0 && v >= 0 && u < p.n_s && v < p.n_t) {  // a walk's final point may be (-1, -1)
			const float d = x[u] - y[v];
			sg = d > 0.0f ? 1 : (d < 0.0f ? -1 : 0);
		} else {
			u = v = -1;
		}
		// the carried runs: continued by lane 0, else complete
		if (lane == 0) {
			if (cu >= 0 && u != cu) dx[cu] += g * float(cx);
			if (cv >= 0 && v != cv) dy[cv] -= g * float(cy);
		}
		const int ax = run_scan(sg + ((lane == 0 && u == cu) ? cx : 0), u, lane);
		const int ay = run_scan(sg + ((lane == 0 && v == cv) ? cy : 0), v, lane);
		const int nu = __shfl_down_sync(0xffffffffu, u, 1), nv = __shfl_down_sync(0xffffffffu, v, 1);
		if (lane < 31 && u >= 0 && nu != u) dx[u] += g * float(ax);
		if (lane < 31 && v >= 0 && nv != v) dy[v] -= g * float(ay);
		cu = __shfl_sync(0xffffffffu, u, 31);
		cv = __shfl_sync(0xffffffffu, v, 31);
		cx = __shfl_sync(0xffffffffu, ax, 31);
		cy = __shfl_sync(0xffffffffu, ay, 31);
	}
	if (lane == 0) {
		if (cu >= 0) dx[cu] += g * float(cx);
		if (cv >= 0) dy[cv] -= g * float(cy);
	}
}

}  // namespace

extern "C" pa_status pa_normalize_rows_bf16(const float *E, int64_t rows, int32_t dim, int32_t normalize,
                                            void *out_bf16, float *inv_norm, void *stream) {
	if (rows < 0 || dim <= 0 || !E || !out_bf16 || !inv_norm) return PA_ERR_INVALID_ARGUMENT;
	if (rows == 0) return PA_OK;
	normalize_rows_bf16_kernel<<<int((rows * 32 + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
	    E, rows, dim, normalize, reinterpret_cast<__nv_bfloat16 *>(out_bf16), inv_norm);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

namespace {

pa_status normalize_lengths(const float *E, int64_t batch, int64_t n, int32_t dim, int32_t normalize,
                            const int32_t *lengths, int32_t tile, void *out_bf16, float *inv_norm, void *stream) {
	if (batch < 0 || n < 0 || dim <= 0 || tile < 0 || !E || !lengths || !out_bf16 || !inv_norm)
		return PA_ERR_INVALID_ARGUMENT;
	if (batch * n == 0) return PA_OK;
	const bool aligned = ((reinterpret_cast<uintptr_t>(E)) & 15) == 0 && ((reinterpret_cast<uintptr_t>(out_bf16)) & 7) == 0;
	if (!aligned && (dim & 3) == 0) return PA_ERR_INVALID_ARGUMENT;  // 16-byte rows need aligned bases
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	__nv_bfloat16 *o = reinterpret_cast<__nv_bfloat16 *>(out_bf16);
	constexpr int RPW = 4;
	const int64_t blocks = (batch * n + 8 * RPW - 1) / (8 * RPW);  // 8 warps of RPW rows per block
	if ((dim & 3) == 0 && dim <= 512) {
		const int nv = (dim + 127) / 128;
		if (nv == 1) normalize_rows_bf16_rows_kernel<1, RPW><<<int(blocks), 256, 0, st>>>(E, batch, n, dim, normalize, lengths, tile, o, inv_norm);
		else if (nv == 2) normalize_rows_bf16_rows_kernel<2, RPW><<<int(blocks), 256, 0, st>>>(E, batch, n, dim, normalize, lengths, tile, o, inv_norm);
		else if (nv == 3) normalize_rows_bf16_rows_kernel<3, RPW><<<int(blocks), 256, 0, st>>>(E, batch, n, dim, normalize, lengths, tile, o, inv_norm);
		else normalize_rows_bf16_rows_kernel<4, RPW><<<int(blocks), 256, 0, st>>>(E, batch, n, dim, normalize, lengths, tile, o, inv_norm);
	} else {
		normalize_rows_bf16_len_kernel<<<int((batch * n * 32 + 255) / 256), 256, 0, st>>>(E, batch, n, dim, normalize,
		                                                                              lengths, tile, o, inv_norm);
	}
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

}  // namespace

extern "C" pa_status pa_normalize_rows_bf16_lengths(const float *E, int64_t batch, int64_t n, int32_t dim,
                                                    int32_t normalize, const int32_t *lengths, void *out_bf16,
                                                    float *inv_norm, void *stream) {
	return normalize_lengths(E, batch, n, dim, normalize, lengths, 0, out_bf16, inv_norm, stream);
}

extern "C" pa_status pa_normalize_rows_bf16_tiled(const float *E, int64_t batch, int64_t n, int32_t dim,
                                                  int32_t normalize, const int32_t *lengths, int32_t tile,
                                                  void *out_bf16, float *inv_norm, void *stream) {
	if (tile <= 0) return PA_ERR_INVALID_ARGUMENT;
	return normalize_lengths(E, batch, n, dim, normalize, lengths, tile, out_bf16, inv_norm, stream);
}

namespace {

pa_status embedding_gradients(int64_t batch, int32_t dim, int32_t normalize, const int32_t *paths,
                              const int64_t *path_offsets, const int32_t *path_len, const float *grad_scores,
                              const float *Es, const float *Et, const void *Es_bf16, const void *Et_bf16,
                              const float *inv_s, const float *inv_t, int64_t n_s, int64_t n_t, float *dEs,
                              float *dEt, bool full, void *stream) {
	if (batch < 0 || dim <= 0 || n_s < 0 || n_t < 0 || !paths || !path_offsets || !path_len || !grad_scores || !Es ||
	    !Et || !Es_bf16 || !Et_bf16 || !inv_s || !inv_t || !dEs || !dEt)
		return PA_ERR_INVALID_ARGUMENT;
	if (batch == 0) return PA_OK;
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	EmbGradParams p{batch, dim, normalize, paths, path_offsets, path_len, grad_scores, Es, Et,
	                reinterpret_cast<const __nv_bfloat16 *>(Es_bf16), reinterpret_cast<const __nv_bfloat16 *>(Et_bf16),
	                inv_s, inv_t, dEs, dEt, n_s, n_t, 0};
	const int64_t threads = batch * 32;
	// 16-byte rows (the vector kernel) when the width is a multiple of 32 and the rows aligned
	const bool vec = dim % 32 == 0 &&
	                 ((reinterpret_cast<uintptr_t>(Es) | reinterpret_cast<uintptr_t>(Et) | reinterpret_cast<uintptr_t>(dEs) |
	                   reinterpret_cast<uintptr_t>(dEt)) & 15) == 0 &&
	                 ((reinterpret_cast<uintptr_t>(Es_bf16) | reinterpret_cast<uintptr_t>(Et_bf16)) & 7) == 0;
	// the row marks of the 8 warps of a block in shared memory
	const size_t marks = size_t(8) * size_t((n_s + 31) / 32 + (n_t + 31) / 32) * 4;
	if (full && vec && marks <= 48 * 1024) {
		p.zero_rest = 1;
		path_embedding_grad_vec_kernel<<<int((threads + 255) / 256), 256, marks, st>>>(p);
		return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
	}
	if (full) {
		if (cudaMemsetAsync(dEs, 0, size_t(batch * n_s * dim) * 4, st) != cudaSuccess ||
		    cudaMemsetAsync(dEt, 0, size_t(batch * n_t * dim) * 4, st) != cudaSuccess)
			return PA_ERR_CUDA;
	}
	if (vec)
		path_embedding_grad_vec_kernel<<<int((threads + 255) / 256), 256, 0, st>>>(p);
	else
		path_embedding_grad_kernel<<<int((threads + 255) / 256), 256, 0, st>>>(p);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

}  // namespace

extern "C" pa_status pa_path_embedding_gradients(int64_t batch, int32_t dim, int32_t normalize, const int32_t *paths,
                                                 const int64_t *path_offsets, const int32_t *path_len,
                                                 const float *grad_scores, const float *Es, const float *Et,
                                                 const void *Es_bf16, const void *Et_bf16, const float *inv_s,
                                                 const float *inv_t, int64_t n_s, int64_t n_t, float *dEs, float *dEt,
                                                 void *stream) {
	return embedding_gradients(batch, dim, normalize, paths, path_offsets, path_len, grad_scores, Es, Et, Es_bf16,
	                           Et_bf16, inv_s, inv_t, n_s, n_t, dEs, dEt, false, stream);
}

extern "C" pa_status pa_path_embedding_gradients_full(int64_t batch, int32_t dim, int32_t normalize,
                                                      const int32_t *paths, const int64_t *path_offsets,
                                                      const int32_t *path_len, const float *grad_scores,
                                                      const float *Es, const float *Et, const void *Es_bf16,
                                                      const void *Et_bf16, const float *inv_s, const float *inv_t,
                                                      int64_t n_s, int64_t n_t, float *dEs, float *dEt, void *stream) {
	return embedding_gradients(batch, dim, normalize, paths, path_offsets, path_len, grad_scores, Es, Et, Es_bf16,
	                           Et_bf16, inv_s, inv_t, n_s, n_t, dEs, dEt, true, stream);
}

extern "C" pa_status pa_path_series_gradients(int64_t batch, const int32_t *paths, const int64_t *path_offsets,
                                              const int32_t *path_len, const float *grad_scores, const float *x,
                                              const float *y, int64_t n_s, int64_t n_t, float *dx, float *dy,
                                              void *stream) {
	if (batch < 0 || !paths || !path_offsets || !path_len || !grad_scores || !x || !y || !dx || !dy)
		return PA_ERR_INVALID_ARGUMENT;
	if (batch == 0) return PA_OK;
	SeriesGradParams p{batch, paths, path_offsets, path_len, grad_scores, x, y, dx, dy, n_s, n_t};
	path_series_grad_kernel<<<int((batch + 7) / 8), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(p);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

// ---------------------------------------------------------------------------------------
// FP64 replay of a recovered path's score.  The float32 DP accumulates its score in float32
// along the path; for long alignments that sum drifts from the exact value.  Re-evaluating
// the same path in float64 -- aligned cells' similarities (every visited cell for DTW), gap
// runs as w(k) = open + extend (k - 1), border gaps of global paths as in the backward
// above -- gives the float64 score of that path, and its distance to the DP's score is the
// DP's accumulation error.

namespace {

struct ReplayParams {
	int64_t batch;
	int32_t dtw, global;
	double gap_sign;  // -1 maximize, +1 minimize
	const int32_t *paths;
	const int64_t *path_off;
	const int32_t *path_len;
	const float *sim;
	const int64_t *sim_off;
	int64_t ss, st;
	double open_s, ext_s, open_t, ext_t;
	double *out;
	double *scale;
};

__global__ void path_replay_f64_kernel(ReplayParams p) {
	const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (k >= p.batch) return;
	const int n = p.path_len[k];
	const int32_t *P = p.paths + p.path_off[k];
	const float *S = p.sim + p.sim_off[k];
	double sum = 0.0, gaps = 0.0, mag = 0.0;
	for (int q = 0; q + 1 < n; q++) {
		const int u0 = P[2 * q], v0 = P[2 * q + 1], u1 = P[2 * q + 2], v1 = P[2 * q + 3];
		if (u0 < 0 || v0 < 0) break;
		if (p.dtw || (u1 == u0 - 1 && v1 == v0 - 1)) {
			const double x = double(S[int64_t(u0) * p.ss + int64_t(v0) * p.st]);
			sum += x;
			mag += fabs(x);
		} else if (v1 == v0 && u1 < u0) {
			gaps += p.open_s + p.ext_s * double(u0 - u1 - 1);
		} else if (u1 == u0 && v1 < v0) {
			gaps += p.open_t + p.ext_t * double(v0 - v1 - 1);
		}
	}
	if (n > 0 && p.global && !p.dtw) {
		const int ul = P[2 * (n - 1)], vl = P[2 * (n - 1) + 1];
		if (ul < 0 && vl >= 0) gaps += p.open_t + p.ext_t * double(vl);
		else if (vl < 0 && ul >= 0) gaps += p.open_s + p.ext_s * double(ul);
	}
	p.out[k] = n > 0 ? sum + p.gap_sign * gaps : 0.0;
	if (p.scale) p.scale[k] = mag + fabs(gaps);
}

}  // namespace

extern "C" pa_status pa_path_scores_f64(int32_t type, int32_t locality, int32_t direction, int64_t batch,
                                        const int32_t *paths, const int64_t *path_offsets, const int32_t *path_len,
                                        const float *sim, const int64_t *sim_offsets, int64_t stride_s,
                                        int64_t stride_t, const double *gaps, double *scores, double *scale,
                                        void *stream) {
	if (batch < 0 || !paths || !path_offsets || !path_len || !sim || !sim_offsets || !scores ||
	    (type != PA_TYPE_DTW && !gaps))
		return PA_ERR_INVALID_ARGUMENT;
	if (batch == 0) return PA_OK;
	ReplayParams p{};
	p.batch = batch;
	p.dtw = type == PA_TYPE_DTW;
	p.global = type == PA_TYPE_DTW || locality == PA_GLOBAL;
	p.gap_sign = direction == PA_MINIMIZE ? 1.0 : -1.0;
	p.paths = paths;
	p.path_off = path_offsets;
	p.path_len = path_len;
	p.sim = sim;
	p.sim_off = sim_offsets;
	p.ss = stride_s;
	p.st = stride_t;
	if (gaps) {
		p.open_s = gaps[0];
		p.ext_s = gaps[1];
		p.open_t = gaps[2];
		p.ext_t = gaps[3];
	}
	p.out = scores;
	p.scale = scale;
	path_replay_f64_kernel<<<int((batch + 127) / 128), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(p);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

// General gap cost solve (GeneralGapCostSolver, solver.h:3056-3184): O(n m (n + m)).
//
// One CTA per pair sweeps anti-diagonals; every cell scans its whole column and row
// history, so D is kept in global memory (L2-resident for the small problems this
// cubic recurrence is used for), twice: row-major for the column scans and transposed for
// the row scans, so that the threads of an anti-diagonal (consecutive rows u, columns
// d - u) read consecutive words at every step k of either scan.  Candidates are pushed in
// the reference's order -- (local zero), diagonal, vertical gaps k = -1..u-1, horizontal
// gaps k = -1..v-1 -- and a later candidate wins only when strictly better.  The seed scans
// (solver.h:2035-2058, 2174-2188, 2266-2294) run over the CTA with a block reduction that
// keeps the scan order's winner.
#include <cmath>
#include "pa_dp.cuh"
#include "pa_wsb.h"

namespace pa {

__global__ void __launch_bounds__(256) wsb_kernel(WsbParams p) {
	const int pair = blockIdx.x;
	if (pair >= p.npairs) return;
	const int ls = p.len_s[pair], lt = p.len_t[pair];
	float *D = p.vals + p.vals_off[pair];
	float *DT = p.vals_t + p.vals_off[pair];  // DT[(j + 1) * (ls + 1) + (i + 1)] = D(i, j)
	int32_t *T = p.tb + p.tb_off[pair];
	float *SUB = p.sub + p.tb_off[pair];
	const int64_t ld = lt + 1, ldt = ls + 1;
	// borders
	for (int j = threadIdx.x; j <= lt; j += blockDim.x) {
		D[j] = p.top_D[j];
		DT[int64_t(j) * ldt] = p.top_D[j];
	}
	for (int i = threadIdx.x; i <= ls; i += blockDim.x) {
		D[int64_t(i) * ld] = p.left_D[i];
		DT[i] = p.left_D[i];
	}
	__syncthreads();
	const uint32_t *arow = p.a ? p.a + int64_t(pair) * p.a_stride : nullptr;
	const uint32_t *brow = p.b ? p.b + int64_t(pair) * p.b_stride : nullptr;
	for (int d = 0; d <= ls + lt - 2; d++) {
		const int u0 = max(0, d - (lt - 1)), u1 = min(ls - 1, d);
		for (int u = u0 + threadIdx.x; u <= u1; u += blockDim.x) {
			const int v = d - u;
			float s;
			if (p.sub_kind == SUB_DENSE) {
				s = p.dense[int64_t(pair) + int64_t(u) * p.dense_si + int64_t(v) * p.dense_sj] * p.sign;
			} else if (p.sub_kind == SUB_BINARY) {
				s = (arow[u] == brow[v] ? p.eq : p.ne) * p.sign;
			} else {
				const uint32_t x = arow[u], y = brow[v];
				if (int(x) >= p.table_rows || int(y) >= p.table_cols) {
					atomicOr(p.status, ST_BAD_CODE);
					s = 0.0f;
				} else {
					s = p.table[x * p.table_cols + y] * p.sign;
				}
			}
			SUB[int64_t(u) * lt + v] = s;
			const float dg = D[int64_t(u) * ld + v] + s;  // D(u-1, v-1) + s(u, v)
			float best;
			int kind, kk = -2;
			if (p.local == LOC_LOCAL) {
				best = 0.0f;
				kind = 0;
				if (dg > best) { best = dg; kind = 1; }
			} else {
				best = dg;
				kind = 1;
			}
			for (int k = -1; k < u; k++) {
				const float c = D[int64_t(k + 1) * ld + (v + 1)] + (-p.gap_s[u - k]);
				if (c > best) { best = c; kind = 2; kk = k; }
			}
			for (int k = -1; k < v; k++) {
				const float c = DT[int64_t(k + 1) * ldt + (u + 1)] + (-p.gap_t[v - k]);
				if (c > best) { best = c; kind = 3; kk = k; }
			}
			D[int64_t(u + 1) * ld + (v + 1)] = best;
			DT[int64_t(v + 1) * ldt + (u + 1)] = best;
			T[int64_t(u) * lt + v] = kind | ((kk + 1) << 2);
		}
		__syncthreads();
	}
	// seeds (Local 2035-2058, Global 2174-2188, Semiglobal 2266-2294): each is the first
	// strict optimum of a scan, i.e. the optimum with the smallest scan position; every
	// thread scans a strided share, then the block keeps (largest value, smallest position)
	auto V = [&](int i, int j) { return D[int64_t(i + 1) * ld + (j + 1)]; };
	float best = -INFINITY;
	int64_t bpos = INT64_MAX;  // scan position of this thread's optimum
	int si = -1, sj = -1, has = 0;
	if (p.local == LOC_LOCAL) {
		// scan i = ls-1 .. 0, j = lt-1 .. 0: position (ls-1-i) * lt + (lt-1-j)
		const int64_t n = int64_t(ls) * lt;
		for (int64_t x = threadIdx.x; x < n; x += blockDim.x) {
			const int i = ls - 1 - int(x / lt), j = lt - 1 - int(x % lt);
			const float val = V(i, j);
			if (val > best) { best = val; bpos = x; }
		}
	} else if (p.local == LOC_SEMI) {
		// the last row (j ascending), then the last column (i ascending)
		for (int64_t x = threadIdx.x; x < int64_t(lt) + ls; x += blockDim.x) {
			const float val = x < lt ? V(ls - 1, int(x)) : V(int(x - lt), lt - 1);
			if (val > best) { best = val; bpos = x; }
		}
	}
	__shared__ float rb[256];
	__shared__ long long rp[256];
	rb[threadIdx.x] = best;
	rp[threadIdx.x] = bpos;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			const float ov = rb[threadIdx.x + o];
			const long long op = rp[threadIdx.x + o];
			if (ov > rb[threadIdx.x] || (ov == rb[threadIdx.x] && op < rp[threadIdx.x])) {
				rb[threadIdx.x] = ov;
				rp[threadIdx.x] = op;
			}
		}
		__syncthreads();
	}
	if (threadIdx.x != 0) return;
	if (p.local == LOC_GLOBAL) {
		si = ls - 1; sj = lt - 1; has = 1; best = V(si, sj);
	} else {
		best = rb[0];
		const long long x = rp[0];
		has = best > -INFINITY;
		if (has && p.local == LOC_LOCAL) {
			si = ls - 1 - int(x / lt);
			sj = lt - 1 - int(x % lt);
		} else if (has) {
			si = x < lt ? ls - 1 : int(x - lt);
			sj = x < lt ? int(x) : lt - 1;
		}
	}
	p.score[pair] = has ? best * p.sign : -INFINITY * p.sign;
	p.seed[2 * pair] = si;
	p.seed[2 * pair + 1] = sj;
	p.has_seed[pair] = has;
}

cudaError_t launch_wsb(const WsbParams &p, cudaStream_t st) {
	if (p.npairs == 0) return cudaSuccess;
	wsb_kernel<<<p.npairs, 256, 0, st>>>(p);
	return cudaGetLastError();
}

}  // namespace pa

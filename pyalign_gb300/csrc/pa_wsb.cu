// General gap cost solve (GeneralGapCostSolver, solver.h:3056-3184): O(n m (n + m)).
//
// A CTA, or a cluster of 2 or 4 CTAs when there are fewer pairs than SMs, per pair sweeps
// anti-diagonals.  Cell (u, v) takes the best of its head candidates -- (local zero), the
// diagonal -- and of u + v + 2 scan candidates: the vertical gaps k = -1..u-1,
// D(k, v) - w_s(u - k), then the horizontal gaps k = -1..v-1, D(u, k) - w_t(v - k).  A later
// candidate wins only when strictly better, so the winner is the first maximum in that
// order.  Numbering the scan candidates q = 0..u+v+1 (vertical k = q - 1 while q <= u,
// horizontal k = q - u - 2 after), the scan's winner is its largest value at the smallest q:
// any split of the scan finds it by keeping a (value, q) pair per part and combining parts by
// (larger value, then smaller q); the scan's winner replaces the head's only when strictly
// better.
//
// D is kept in global memory (L2-resident at the sizes this cubic recurrence is used for),
// twice: row-major and transposed.  Every cell of anti-diagonal d scans d + 2 candidates.
// The warps of the pair split a diagonal one of two ways:
//  * a warp per cell (diagonals of at most warp_cells cells per warp): the lanes take the
//    positions of both scans 32 apart -- the vertical scan reads a row of the transposed
//    copy, the horizontal scan a row of the row-major copy, 32 consecutive words per step,
//    four steps of both in flight together -- and two warp reductions combine the lanes.
//    Per 32 cells of a warp, lane j loads cell j's similarity and diagonal value before the
//    scans and stores its result after them.
//  * a thread per cell (diagonals of more than warp_cells cells per warp; the host keeps the
//    warp per cell everywhere and this split for tests): the threads of a warp hold
//    consecutive cells and at step k read row k of the row-major copy (vertical scans) or of
//    the transposed copy (horizontal scans), again 32 consecutive words.
// The CTAs of a cluster meet at a cluster barrier (release / acquire) after every diagonal
// and read the values of D through L2, where the other CTAs' writes are.  With one CTA per
// pair and rows that fit (at most 200 KB), the scans read D from a copy in shared memory.  The seed scans
// (solver.h:2035-2058, 2174-2188, 2266-2294) run over the first CTA with a block reduction
// that keeps the scan order's winner.
#include <climits>
#include <cmath>
#include <mutex>
#include "pa_dp.cuh"
#include "pa_wsb.h"

namespace pa {

namespace {

constexpr int32_t WSB_NO_TB = INT32_MIN;  // "no traceback" coordinates of a local zero

// a value of D: through L2 when the pair's CTAs form a cluster (another SM wrote it)
template <bool CL>
__device__ __forceinline__ float wsb_ld(const float *a) {
	if constexpr (CL) return __ldcg(a);
	else return *a;
}

// every thread of the pair (its CTA, or its cluster) has finished the previous diagonal and
// its writes are visible
template <bool CL>
__device__ __forceinline__ void wsb_sync() {
	if constexpr (CL) {
		asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
		asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
	} else {
		__syncthreads();
	}
}

// similarity of cell (u, v), normalised (multiplied by the direction's sign)
__device__ __forceinline__ float wsb_similarity(const WsbParams &p, int pair, const uint32_t *arow,
                                                const uint32_t *brow, int u, int v) {
	if (p.sub_kind == SUB_DENSE)
		return p.dense[int64_t(pair) + int64_t(u) * p.dense_si + int64_t(v) * p.dense_sj] * p.sign;
	if (p.sub_kind == SUB_BINARY) return (arow[u] == brow[v] ? p.eq : p.ne) * p.sign;
	const uint32_t x = arow[u], y = brow[v];
	if (x >= uint32_t(p.table_rows) || y >= uint32_t(p.table_cols)) {
		atomicOr(p.status, ST_BAD_CODE);
		return 0.0f;
	}
	return p.table[size_t(x) * size_t(p.table_cols) + y] * p.sign;
}

// combine two parts of a scan: the larger value, on a tie the smaller position
template <typename Q>
__device__ __forceinline__ void wsb_keep(float &bv, Q &bq, float ov, Q oq) {
	if (ov > bv || (ov == bv && oq < bq)) {
		bv = ov;
		bq = oq;
	}
}

// order-preserving key of a float that is not NaN, with -0 and +0 equal
__device__ __forceinline__ uint32_t wsb_order(float f) {
	const uint32_t b = __float_as_uint(f == 0.0f ? 0.0f : f);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// the scan of cell (u, v) by one warp.  The vertical positions q = p (p = 0..u) and the
// horizontal ones q = u + 1 + p (p = 0..v) are read in the same batches: lane l takes
// p = l, l + 32, l + 64, l + 96 of both phases, sixteen loads in flight, and keeps each
// phase's first maximum (the vertical one wins a tie, coming first).  Every lane returns the
// scan's first maximum: the largest key by one reduction, the smallest position holding it
// by another, its value from the lane that scanned that position.
template <bool CL>
__device__ __forceinline__ void wsb_scan_warp(const WsbParams &p, const float *D, const float *DT, int64_t ld,
                                              int64_t ldt, int u, int v, int lane, float &bv, int &bq) {
	// D(p - 1, v) = DT[(v + 1) * ldt + p], w_s(u - k) = gap_s[u + 1 - p]
	const float *xv = DT + int64_t(v + 1) * ldt + lane, *gv = p.gap_s + (u + 1) - lane;
	// D(u, p - 1) = D[(u + 1) * ld + p], w_t(v - k) = gap_t[v + 1 - p]
	const float *xh = D + int64_t(u + 1) * ld + lane, *gh = p.gap_t + (v + 1) - lane;
	float bvv = -INFINITY, bvh = -INFINITY;
	int bqv = INT_MAX, bqh = INT_MAX;
	const int pend = max(u, v);
	for (int p0 = 0; p0 <= pend; p0 += 128, xv += 128, gv -= 128, xh += 128, gh -= 128) {
		float a[4], ga[4], b[4], gb[4];
#pragma unroll
		for (int r = 0; r < 4; r++) {
			const int pp = p0 + lane + 32 * r;
			a[r] = pp <= u ? wsb_ld<CL>(xv + 32 * r) : -INFINITY;
			ga[r] = pp <= u ? __ldg(gv - 32 * r) : 0.0f;
			b[r] = pp <= v ? wsb_ld<CL>(xh + 32 * r) : -INFINITY;
			gb[r] = pp <= v ? __ldg(gh - 32 * r) : 0.0f;
		}
#pragma unroll
		for (int r = 0; r < 4; r++) {
			const int pp = p0 + lane + 32 * r;
			const float cv = a[r] + (-ga[r]), ch = b[r] + (-gb[r]);
			if (cv > bvv) {
				bvv = cv;
				bqv = pp;
			}
			if (ch > bvh) {
				bvh = ch;
				bqh = u + 1 + pp;
			}
		}
	}
	bv = bvh > bvv ? bvh : bvv;
	bq = bvh > bvv ? bqh : bqv;
	const uint32_t key = wsb_order(bv);
	const uint32_t m = __reduce_max_sync(0xffffffffu, key);
	const int qw = __reduce_min_sync(0xffffffffu, key == m ? bq : INT_MAX);
	// the lane that scanned position qw: p = qw or qw - u - 1, lane p mod 32
	bv = __shfl_sync(0xffffffffu, bv, (qw <= u ? qw : qw - u - 1) & 31);
	bq = qw;
}

// the scan of cell (u, v) by one thread, in order
template <bool CL>
__device__ __forceinline__ void wsb_scan_thread(const WsbParams &p, const float *D, const float *DT, int64_t ld,
                                                int64_t ldt, int u, int v, float &bv, int &bq) {
	bv = -INFINITY;
	bq = INT_MAX;
	const float *gs = p.gap_s + (u + 1);
	int64_t o = v + 1;  // D(q - 1, v) = D[q * ld + v + 1]
	for (int q = 0; q <= u; q++, o += ld) {
		const float c = wsb_ld<CL>(D + o) + (-__ldg(gs - q));
		if (c > bv) {
			bv = c;
			bq = q;
		}
	}
	const float *gt = p.gap_t + (u + v + 2);
	o = u + 1;  // D(u, q - u - 2) = DT[(q - u - 1) * ldt + u + 1]
	for (int q = u + 1; q <= u + v + 1; q++, o += ldt) {
		const float c = wsb_ld<CL>(DT + o) + (-__ldg(gt - q));
		if (c > bv) {
			bv = c;
			bq = q;
		}
	}
}

// the cell's result: the head candidates -- (local zero), the diagonal (dprev = D(u-1, v-1))
// -- then the scan's first maximum (bv at position bq), which replaces the head's only when
// strictly better
template <bool WRITE_DT = true>
__device__ __forceinline__ float wsb_store(const WsbParams &p, float *D, float *DT, int32_t *T, float *SUB, int64_t ld,
                                          int64_t ldt, int lt, int u, int v, float s, float dprev, float bv, int bq) {
	const float dg = dprev + s;
	float best;
	int kind, kk = -2;
	if (p.local == LOC_LOCAL) {
		best = 0.0f;
		kind = 0;
		if (dg > best) {
			best = dg;
			kind = 1;
		}
	} else {
		best = dg;
		kind = 1;
	}
	if (bv > best) {
		best = bv;
		if (bq <= u) {
			kind = 2;
			kk = bq - 1;
		} else {
			kind = 3;
			kk = bq - u - 2;
		}
	}
	SUB[int64_t(u) * lt + v] = s;
	D[int64_t(u + 1) * ld + (v + 1)] = best;
	if (WRITE_DT) DT[int64_t(v + 1) * ldt + (u + 1)] = best;
	T[int64_t(u) * lt + v] = int32_t(uint32_t(kk + 1) << 2) | kind;
	return best;
}

// The scan of cell (u, v) by one warp with the pair's D in the CTA's shared memory (bordered
// row i, i.e. D(i - 1, .), at sD[i * lds]): the same lane split and reductions as
// wsb_scan_warp.  Position p of the vertical scan is col[p * lds] (col: column v + 1), of the
// horizontal scan row[p] (row: bordered row u + 1).  lds is odd, so the lanes' column reads
// fall in distinct banks.
__device__ __forceinline__ void wsb_scan_warp_sm(const WsbParams &p, const float *col, const float *row, int lds,
                                                 int u, int v, int lane, float &bv, int &bq) {
	const float *gv = p.gap_s + (u + 1) - lane, *gh = p.gap_t + (v + 1) - lane;
	float bvv = -INFINITY, bvh = -INFINITY;
	int bqv = INT_MAX, bqh = INT_MAX;
	const int pend = max(u, v);
	for (int p0 = 0; p0 <= pend; p0 += 128, gv -= 128, gh -= 128) {
		float a[4], ga[4], b[4], gb[4];
#pragma unroll
		for (int r = 0; r < 4; r++) {
			const int pp = p0 + lane + 32 * r;
			a[r] = pp <= u ? col[pp * lds] : -INFINITY;
			ga[r] = pp <= u ? __ldg(gv - 32 * r) : 0.0f;
			b[r] = pp <= v ? row[pp] : -INFINITY;
			gb[r] = pp <= v ? __ldg(gh - 32 * r) : 0.0f;
		}
#pragma unroll
		for (int r = 0; r < 4; r++) {
			const int pp = p0 + lane + 32 * r;
			const float cv = a[r] + (-ga[r]), ch = b[r] + (-gb[r]);
			if (cv > bvv) {
				bvv = cv;
				bqv = pp;
			}
			if (ch > bvh) {
				bvh = ch;
				bqh = u + 1 + pp;
			}
		}
	}
	bv = bvh > bvv ? bvh : bvv;
	bq = bvh > bvv ? bqh : bqv;
	const uint32_t key = wsb_order(bv);
	const uint32_t m = __reduce_max_sync(0xffffffffu, key);
	const int qw = __reduce_min_sync(0xffffffffu, key == m ? bq : INT_MAX);
	bv = __shfl_sync(0xffffffffu, bv, (qw <= u ? qw : qw - u - 1) & 31);
	bq = qw;
}

// CL: the pair's CTAs form a cluster (its size from %cluster_nctarank, 2 or 4).  SM (one CTA
// per pair): the pair's D is also held in the CTA's shared memory (p.lds floats a row) and the
// scans read it there; the global copy serves the walk, the seeds and the host.
template <bool CL, bool SM>
__global__ void __launch_bounds__(1024) wsb_kernel(WsbParams p) {
	static_assert(!(CL && SM), "shared-memory rows: one CTA per pair");
	extern __shared__ float4 wsb_smem4[];
	float *sD = reinterpret_cast<float *>(wsb_smem4);
	uint32_t rank = 0, csize = 1;
	if constexpr (CL) {
		asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
		asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(csize));
	}
	const int pair = int(blockIdx.x / csize);
	if (pair >= p.npairs) return;  // cluster-uniform
	const int ls = p.len_s[pair], lt = p.len_t[pair];
	float *D = p.vals + p.vals_off[pair];
	float *DT = p.vals_t + p.vals_off[pair];  // DT[(j + 1) * (ls + 1) + (i + 1)] = D(i, j)
	int32_t *T = p.tb + p.tb_off[pair];
	float *SUB = p.sub + p.tb_off[pair];
	const int64_t ld = lt + 1, ldt = ls + 1;
	const int lds = p.lds;
	// borders (the first CTA's; in shared memory too with SM)
	if (rank == 0) {
		for (int j = threadIdx.x; j <= lt; j += blockDim.x) {
			D[j] = p.top_D[j];
			if (SM) sD[j] = p.top_D[j];
			else DT[int64_t(j) * ldt] = p.top_D[j];
		}
		for (int i = threadIdx.x; i <= ls; i += blockDim.x) {
			D[int64_t(i) * ld] = p.left_D[i];
			if (SM) {
				if (i > 0) sD[i * lds] = p.left_D[i];
			} else {
				DT[i] = p.left_D[i];
			}
		}
	}
	wsb_sync<CL>();
	const uint32_t *arow = p.a ? p.a + int64_t(pair) * p.a_stride : nullptr;
	const uint32_t *brow = p.b ? p.b + int64_t(pair) * p.b_stride : nullptr;
	const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
	const int gw = int(rank) * nwarps + (threadIdx.x >> 5), GW = int(csize) * nwarps;  // the pair's warps
	const int gt = int(rank * blockDim.x + threadIdx.x), GT = int(csize * blockDim.x);  // and threads
	for (int d = 0; d <= ls + lt - 2; d++) {
		const int u0 = max(0, d - (lt - 1)), u1 = min(ls - 1, d);
		const int ncell = u1 - u0 + 1;
		if constexpr (SM) {
			// the same split as below over the CTA's warps, D read from shared memory
			const int w = threadIdx.x >> 5;
			const int nw = ncell > w ? (ncell - w + nwarps - 1) / nwarps : 0;
			for (int j0 = 0; j0 < nw; j0 += 32) {
				const bool mine = j0 + lane < nw;
				const int um = u0 + w + nwarps * (j0 + lane), vm = d - um;
				float s = 0.0f, dprev = 0.0f, kv = -INFINITY;
				int kq = INT_MAX;
				if (mine) {
					s = wsb_similarity(p, pair, arow, brow, um, vm);
					dprev = sD[um * lds + vm];
				}
				const int jn = min(32, nw - j0);
				for (int jj = 0; jj < jn; jj++) {  // warp-uniform
					const int u = u0 + w + nwarps * (j0 + jj), v = d - u;
					float bv;
					int bq;
					wsb_scan_warp_sm(p, sD + (v + 1), sD + (u + 1) * lds, lds, u, v, lane, bv, bq);
					if (lane == jj) {
						kv = bv;
						kq = bq;
					}
				}
				if (mine)
					sD[(um + 1) * lds + (vm + 1)] = wsb_store<false>(p, D, DT, T, SUB, ld, ldt, lt, um, vm, s, dprev, kv, kq);
			}
		} else if (ncell <= GW * p.warp_cells) {
			// this warp's cells c = gw + GW * j, 32 at a time: lane l loads the similarity and
			// D(u-1, v-1) of cell j0 + l before the scans and stores its result after them
			const int nw = ncell > gw ? (ncell - gw + GW - 1) / GW : 0;
			for (int j0 = 0; j0 < nw; j0 += 32) {
				const bool mine = j0 + lane < nw;
				const int um = u0 + gw + GW * (j0 + lane), vm = d - um;
				float s = 0.0f, dprev = 0.0f, kv = -INFINITY;
				int kq = INT_MAX;
				if (mine) {
					s = wsb_similarity(p, pair, arow, brow, um, vm);
					dprev = wsb_ld<CL>(D + int64_t(um) * ld + vm);
				}
				const int jn = min(32, nw - j0);
				for (int jj = 0; jj < jn; jj++) {  // warp-uniform
					const int u = u0 + gw + GW * (j0 + jj);
					float bv;
					int bq;
					wsb_scan_warp<CL>(p, D, DT, ld, ldt, u, d - u, lane, bv, bq);
					if (lane == jj) {
						kv = bv;
						kq = bq;
					}
				}
				if (mine) wsb_store(p, D, DT, T, SUB, ld, ldt, lt, um, vm, s, dprev, kv, kq);
			}
		} else {
			for (int u = u0 + gt; u <= u1; u += GT) {
				const int v = d - u;
				const float s = wsb_similarity(p, pair, arow, brow, u, v);
				float bv;
				int bq;
				wsb_scan_thread<CL>(p, D, DT, ld, ldt, u, v, bv, bq);
				wsb_store(p, D, DT, T, SUB, ld, ldt, lt, u, v, s, wsb_ld<CL>(D + int64_t(u) * ld + v), bv, bq);
			}
		}
		wsb_sync<CL>();
	}
	if (rank != 0) return;
	// seeds (Local 2035-2058, Global 2174-2188, Semiglobal 2266-2294): each is the first
	// strict optimum of a scan, i.e. the optimum with the smallest scan position; every
	// thread scans a strided share, then the block keeps (largest value, smallest position)
	auto V = [&](int i, int j) { return wsb_ld<CL>(D + int64_t(i + 1) * ld + (j + 1)); };
	float best = -INFINITY;
	long long bpos = LLONG_MAX;  // scan position of this thread's optimum
	if (p.local == LOC_LOCAL) {
		// scan i = ls-1 .. 0, j = lt-1 .. 0: position (ls-1-i) * lt + (lt-1-j)
		const int64_t n = int64_t(ls) * lt;
		for (int64_t x = threadIdx.x; x < n; x += blockDim.x) {
			const int i = ls - 1 - int(x / lt), j = lt - 1 - int(x % lt);
			const float val = V(i, j);
			if (val > best) {
				best = val;
				bpos = x;
			}
		}
	} else if (p.local == LOC_SEMI) {
		// the last row (j ascending), then the last column (i ascending)
		for (int64_t x = threadIdx.x; x < int64_t(lt) + ls; x += blockDim.x) {
			const float val = x < lt ? V(ls - 1, int(x)) : V(int(x - lt), lt - 1);
			if (val > best) {
				best = val;
				bpos = x;
			}
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		const float ov = __shfl_xor_sync(0xffffffffu, best, o);
		const long long op = __shfl_xor_sync(0xffffffffu, bpos, o);
		wsb_keep(best, bpos, ov, op);
	}
	__shared__ float rb[32];
	__shared__ long long rp[32];
	const int warp = threadIdx.x >> 5;
	if (lane == 0) {
		rb[warp] = best;
		rp[warp] = bpos;
	}
	__syncthreads();
	if (threadIdx.x != 0) return;
	for (int w = 1; w < nwarps; w++) wsb_keep(best, bpos, rb[w], rp[w]);
	int si = -1, sj = -1, has = 0;
	if (p.local == LOC_GLOBAL) {
		si = ls - 1;
		sj = lt - 1;
		has = 1;
		best = V(si, sj);
	} else {
		const long long x = bpos;
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

// a warp per pair: the lanes clear the map, lane 0 follows the codes from the seed and
// writes the aligned pairs (a step that changes both coordinates aligns the cell it leaves)
__global__ void __launch_bounds__(128) wsb_walk_kernel(WsbWalkParams p) {
	const int pair = blockIdx.x * 4 + int(threadIdx.x >> 5);
	const int lane = threadIdx.x & 31;
	if (pair >= p.npairs) return;
	const int ls = p.len_s[pair], lt = p.len_t[pair];
	int32_t *map = p.maps + p.map_off[pair];
	const int n = min(ls, lt);
	for (int k = lane; k < n; k += 32) map[k] = -1;
	__syncwarp();
	if (lane != 0 || !p.has_seed[pair]) return;
	const float *D = p.vals + p.vals_off[pair];
	const int32_t *T = p.tb + p.tb_off[pair];
	const int64_t ld = lt + 1;
	int u = p.seed[2 * pair], v = p.seed[2 * pair + 1];
	while (u >= 0 && v >= 0 && u < ls && v < lt) {
		if (p.local == LOC_LOCAL && !(D[int64_t(u + 1) * ld + (v + 1)] > 0.0f)) break;
		const int32_t c = T[int64_t(u) * lt + v];
		const int kind = c & 3, kk = (c >> 2) - 1;
		int nu = u, nv = v;
		if (kind == 0) {
			nu = WSB_NO_TB;
			nv = WSB_NO_TB;
		} else if (kind == 1) {
			nu = u - 1;
			nv = v - 1;
		} else if (kind == 2 && kk < u) {
			nu = kk;
		} else if (kind == 3 && kk < v) {
			nv = kk;
		} else {
			break;  // not a code of wsb_kernel
		}
		if (nu != u && nv != v) {
			if (ls <= lt) map[u] = v;
			else map[v] = u;
		}
		u = nu;
		v = nv;
	}
}

// opens a kernel for `smem` bytes of dynamic shared memory on the current device (the
// attribute belongs to the device's copy of the kernel): once per device and larger size,
// under a lock so that threads solving at once each see an opened kernel
template <bool CL, bool SM>
cudaError_t wsb_open(int smem) {
	static std::mutex mu;
	static int opened[64] = {};
	int dev = 0;
	if (cudaError_t e = cudaGetDevice(&dev)) return e;
	const bool known = dev >= 0 && dev < 64;
	std::lock_guard<std::mutex> lock(mu);
	if (known && smem <= opened[dev]) return cudaSuccess;
	const cudaError_t e = cudaFuncSetAttribute(wsb_kernel<CL, SM>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
	if (e == cudaSuccess && known) opened[dev] = smem;
	return e;
}

template <bool SM>
cudaError_t launch_wsb_as(const WsbParams &p, int threads, int cluster, int smem, cudaStream_t st) {
	if (SM || cluster <= 1) {
		if (cudaError_t e = wsb_open<false, SM>(smem)) return e;
		wsb_kernel<false, SM><<<p.npairs, threads, smem, st>>>(p);
		return cudaGetLastError();
	}
	if (cudaError_t e = wsb_open<true, false>(smem)) return e;
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3(unsigned(p.npairs) * unsigned(cluster));
	cfg.blockDim = dim3(unsigned(threads));
	cfg.dynamicSmemBytes = size_t(smem);
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = unsigned(cluster);
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	int active = 0;
	if (cudaOccupancyMaxActiveClusters(&active, wsb_kernel<true, false>, &cfg) != cudaSuccess || active < 1) {
		cudaGetLastError();
		return cudaErrorNotSupported;
	}
	return cudaLaunchKernelEx(&cfg, wsb_kernel<true, false>, p);
}

}  // namespace

cudaError_t launch_wsb(const WsbParams &p, int threads, int cluster, cudaStream_t st) {
	if (p.npairs == 0) return cudaSuccess;
	if (p.lds > 0)  // the pair's rows in the CTA's shared memory: max |s| + 1 rows
		return launch_wsb_as<true>(p, threads, 1, (p.max_ls + 1) * p.lds * int(sizeof(float)), st);
	const cudaError_t e = launch_wsb_as<false>(p, threads, cluster, 0, st);
	if (e != cudaErrorNotSupported) return e;
	return launch_wsb_as<false>(p, threads, 1, 0, st);  // one CTA per pair
}

cudaError_t launch_wsb_walk(const WsbWalkParams &p, cudaStream_t st) {
	if (p.npairs == 0) return cudaSuccess;
	wsb_walk_kernel<<<(p.npairs + 3) / 4, 128, 0, st>>>(p);
	return cudaGetLastError();
}

}  // namespace pa

// Co-optimal traceback path counts over the all-optimal masks (sm_103a).
//
// The reference enumerates every optimal alignment with a depth-first search over the
// traceback lists (TracebackIterators<true>::Iterator::next, solver.h:1647-1716): from each
// seed it follows every entry of a cell's list -- the zero candidate of local alignment, the
// diagonal, and for affine gaps the P/Q lists, which hold the cells where a vertical or
// horizontal gap was opened (solver.h:2995-3016) -- until a point with a negative coordinate
// or (local) a value that is not strictly positive.  Without de-duplication every leaf of
// that search is one result, so the number of results is a sum over the traceback graph:
//
//   N(u, v)  = 1                                    u < 0, v < 0, or local with D(u, v) = 0
//            = max(1, [zero] + [diag] N(u-1, v-1) + [P] Pc(u, v) + [Q] Qc(u, v))   otherwise
//   Pc(u, v) = [P open] N(u-1, v) + [P extend, u > 0] Pc(u-1, v)     (linear gaps: N(u-1, v))
//   Qc(u, v) = [Q open] N(u, v-1) + [Q extend, v > 0] Qc(u, v-1)     (linear gaps: N(u, v-1))
//
// (an empty list pushes one terminal entry, hence the max), and the count of a pair is N
// summed over its seeds: every cell equal to a strictly positive optimum for local
// alignment, the one seed of Global/Semiglobal otherwise.  N depends only on cells above
// and to the left, so it runs in the DP's own wavefront order, over the DP's own mask layout
// (pa_dp.cuh: per pair, stripe q, step s, lane k one uint4 holding 8 rows of 16-bit cells):
// a group of G lanes per pair, lane k owning 8 rows of each G * 8-row stripe, column
// s - k in step s; (N, Pc) of a lane's last row reach the next lane by a shuffle, the last
// lane's row crosses to the next stripe through a double-buffered boundary row in global
// memory, and (N, Qc) of each row stay in registers along the row.  Counts are uint64,
// exact below 2^64 and saturating at 2^64 - 1.
//
// Few long pairs (masks written with G = 32): path_count_chain_kernel gives every 256-row
// stripe of every pair to its own warp, like the DP's stripe-chained mode -- tickets numbered
// stripe-major (stripe q of the pair at rank w is ticket level_start[q] + w), the warp of
// stripe q reading the boundary row of stripe q - 1 while that stripe's warp still writes
// it, behind a progress counter published every 32 columns (bounded waits: past the limit
// the kernel flags ST_TIMEOUT and finishes).  Each ticket writes its own partial count (the
// seeds inside its stripe); the host adds a pair's partials.
#include "pa_dp.cuh"

namespace pa {

struct CountParams {
	int32_t npairs;
	int32_t G;                 // group width of the DP launch that wrote the masks
	int32_t local, affine;
	const int32_t *len_s, *len_t;
	const int64_t *mask_off;   // per pair, in uint4 units
	const uint4 *masks;
	const int32_t *seed;       // (i, j) per pair: the single seed of Global/Semiglobal
	unsigned long long *counts;
	unsigned long long *scratch;  // per group slot: 2 buffers x (N, Pc) x max |t|
	int64_t scratch_stride;       // uint64 per slot (per pair in the chained kernel)
	int32_t *work_counter;
	// stripe-chained kernel
	int32_t ntickets, nlevels;
	const int32_t *level_start;   // nlevels + 1 ticket offsets
	const int32_t *order;         // pairs by stripe count, most first
	int32_t *progress;            // per ticket: columns of its boundary row written
	int32_t *status;              // ST_TIMEOUT
	unsigned long long *partial;  // per ticket: the count of the seeds in its stripe
};

__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
	const unsigned long long c = a + b;
	return c < a ? ~0ull : c;
}

__device__ __forceinline__ unsigned long long shfl_up64(unsigned long long x, int G) {
	const uint32_t lo = __shfl_up_sync(0xffffffffu, uint32_t(x), 1, G);
	const uint32_t hi = __shfl_up_sync(0xffffffffu, uint32_t(x >> 32), 1, G);
	return (unsigned long long)(hi) << 32 | lo;
}

// One lane's R rows in column j: N, Pc from the row above (uN, uP) and the diagonal dN,
// N and Qc of each row to the left (Nl, Ql, updated in place); the seed counts of its cells
// add into acc.  Returns (N, Pc) of the last row in uN, uP.
__device__ __forceinline__ void count_rows(const CountParams &p, const uint32_t (&ws)[4], int row0, int j, int ls,
                                           int si, int sj, unsigned long long dN, unsigned long long &uN,
                                           unsigned long long &uP, unsigned long long (&Nl)[R],
                                           unsigned long long (&Ql)[R], unsigned long long &acc) {
#pragma unroll
	for (int r = 0; r < R; r++) {
		const int i = row0 + r;
		const uint32_t c = (ws[r >> 1] >> (16 * (r & 1))) & 0xffffu;
		const unsigned long long lN = Nl[r], lQ = Ql[r];
		unsigned long long Pc, Qc;
		if (p.affine) {
			Pc = sat_add((c & 16u) ? uN : 0ull, ((c & 32u) && i > 0) ? uP : 0ull);
			Qc = sat_add((c & 64u) ? lN : 0ull, ((c & 128u) && j > 0) ? lQ : 0ull);
		} else {
			Pc = uN;
			Qc = lN;
		}
		unsigned long long N;
		if (p.local && (c & 1u)) {
			N = 1ull;  // D = 0: the search stops here
		} else {
			unsigned long long t = (c & 1u) ? 1ull : 0ull;
			t = sat_add(t, (c & 2u) ? dN : 0ull);
			t = sat_add(t, (c & 4u) ? Pc : 0ull);
			t = sat_add(t, (c & 8u) ? Qc : 0ull);
			N = t ? t : 1ull;
		}
		if (i < ls) {
			if (p.local ? (c & 256u) != 0 : (i == si && j == sj)) acc = sat_add(acc, N);
		}
		dN = lN;  // N(i, j - 1) is the diagonal of row i + 1
		Nl[r] = N;
		Ql[r] = Qc;
		uN = N;
		uP = Pc;
	}
}

__global__ void __launch_bounds__(BLOCK) path_count_kernel(CountParams p) {
	const int G = p.G;
	const int lane = threadIdx.x & 31;
	const int sub = lane % G, grp = lane / G, gpw = 32 / G;
	const int warp_global = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
	const int slot = warp_global * gpw + grp;
	const int rpp = G * R;
	const int64_t half = p.scratch_stride / 2;
	for (;;) {
		int base = 0;
		if (lane == 0) base = atomicAdd(p.work_counter, gpw);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= p.npairs) break;
		const int pair = base + grp;
		const bool have = pair < p.npairs;
		const int ls = have ? p.len_s[pair] : 0, lt = have ? p.len_t[pair] : 0;
		const int npass = (ls == 0 || lt == 0) ? 0 : (ls + rpp - 1) / rpp;
		const int nsteps = npass ? lt + G - 1 : 0;
		int wpass = npass, wsteps = nsteps;
		for (int o = 16; o > 0; o >>= 1) {
			wpass = max(wpass, __shfl_xor_sync(0xffffffffu, wpass, o));
			wsteps = max(wsteps, __shfl_xor_sync(0xffffffffu, wsteps, o));
		}
		const int si = (have && !p.local) ? p.seed[2 * pair] : -1;
		const int sj = (have && !p.local) ? p.seed[2 * pair + 1] : -1;
		const uint4 *M = p.masks + (have ? p.mask_off[pair] : 0);
		const int64_t S = int64_t(lt) + G - 1;
		unsigned long long acc = 0;
		unsigned long long *slot_rows = p.scratch + int64_t(slot) * p.scratch_stride;
		for (int q = 0; q < wpass; q++) {
			const bool pass_active = q < npass;
			const int row0 = q * rpp + sub * R;
			const unsigned long long *bin = slot_rows + (q & 1) * half;
			unsigned long long *bout = slot_rows + ((q + 1) & 1) * half;
			const bool write_boundary = sub == G - 1 && q + 1 < npass;
			unsigned long long Nl[R], Ql[R];
#pragma unroll
			for (int r = 0; r < R; r++) {
				Nl[r] = 1ull;  // N(i, -1): a leaf
				Ql[r] = 0ull;  // no Q list at column -1
			}
			unsigned long long outN = 1ull, outP = 0ull;  // this lane's last row, previous column
			unsigned long long prev_up = 1ull;            // N(row0 - 1, j - 1); column -1 is a leaf
			// the mask words of the next four steps and (lane 0) the boundary row of the next two
			// columns, loaded ahead: one pair's steps are a chain of dependent cells, so a load
			// used in its own step would cost a memory round trip per step
			const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
			auto load = [&](int st) -> uint4 {
				const int jj = st - sub;
				return (pass_active && jj >= 0 && jj < lt) ? __ldg(M + (int64_t(q) * S + st) * G + sub) : zero4;
			};
			auto load_row = [&](int col) -> ulonglong2 {
				if (sub != 0 || !pass_active || col >= lt) return make_ulonglong2(1ull, 0ull);
				if (q == 0) return make_ulonglong2(1ull, 0ull);  // N(-1, j): a leaf; no P list above
				return make_ulonglong2(bin[2 * col], bin[2 * col + 1]);
			};
			uint4 w0 = load(0), w1 = load(1), w2 = load(2), w3 = load(3);
			ulonglong2 b0 = load_row(0), b1 = load_row(1);
			for (int s = 0; s < wsteps; s++) {
				const uint4 w = w0;
				w0 = w1;
				w1 = w2;
				w2 = w3;
				w3 = load(s + 4);
				const ulonglong2 bcur = b0;  // lane 0: (N, Pc) above row 0 in column s
				b0 = b1;
				b1 = load_row(s + 2);
				const int j = s - sub;
				unsigned long long upN = shfl_up64(outN, G);
				unsigned long long upP = shfl_up64(outP, G);
				const bool act = pass_active && j >= 0 && j < lt;
				if (act) {
					if (sub == 0) {
						upN = bcur.x;
						upP = bcur.y;
					}
					const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
					unsigned long long uN = upN, uP = upP;
					count_rows(p, ws, row0, j, ls, si, sj, prev_up, uN, uP, Nl, Ql, acc);
					outN = uN;
					outP = uP;
					if (write_boundary) {
						bout[2 * j] = outN;
						bout[2 * j + 1] = outP;
					}
				}
				prev_up = upN;
			}
			__syncwarp();
		}
		// the group's sum
		for (int o = 1; o < G; o <<= 1) {
			const uint32_t lo = __shfl_xor_sync(0xffffffffu, uint32_t(acc), o, G);
			const uint32_t hi = __shfl_xor_sync(0xffffffffu, uint32_t(acc >> 32), o, G);
			acc = sat_add(acc, (unsigned long long)(hi) << 32 | lo);
		}
		if (have && sub == 0) p.counts[pair] = acc;
	}
}

__global__ void __launch_bounds__(BLOCK) path_count_chain_kernel(CountParams p) {
	constexpr int G = 32, rpp = G * R;
	const int lane = threadIdx.x & 31;
	const int sub = lane;
	for (;;) {
		int t = 0;
		if (lane == 0) t = atomicAdd(p.work_counter, 1);
		t = __shfl_sync(0xffffffffu, t, 0);
		if (t >= p.ntickets) break;
		int q = 0;
		while (q + 1 < p.nlevels && p.level_start[q + 1] <= t) q++;
		const int w = t - p.level_start[q];
		const int pair = p.order[w];
		const int prod = q > 0 ? p.level_start[q - 1] + w : -1;  // the stripe above: an earlier ticket
		const int ls = p.len_s[pair], lt = p.len_t[pair];
		const int npass = (ls == 0 || lt == 0) ? 0 : (ls + rpp - 1) / rpp;
		const int si = p.local ? -1 : p.seed[2 * pair], sj = p.local ? -1 : p.seed[2 * pair + 1];
		const uint4 *M = p.masks + p.mask_off[pair];
		const int64_t S = int64_t(lt) + G - 1;
		unsigned long long acc = 0;
		const bool pass_active = q < npass;
		unsigned long long *rows = p.scratch + int64_t(pair) * p.scratch_stride;
		const unsigned long long *bin = rows + (q & 1) * (p.scratch_stride / 2);
		unsigned long long *bout = rows + ((q + 1) & 1) * (p.scratch_stride / 2);
		const bool write_boundary = sub == G - 1 && q + 1 < npass;
		const int32_t *prog_in = q > 0 ? p.progress + prod : nullptr;
		int32_t avail = 0;  // lane 0: columns of bin known to be written
		const int row0 = q * rpp + sub * R;
		unsigned long long Nl[R], Ql[R];
#pragma unroll
		for (int r = 0; r < R; r++) {
			Nl[r] = 1ull;
			Ql[r] = 0ull;
		}
		unsigned long long outN = 1ull, outP = 0ull, prev_up = 1ull;
		const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
		auto load = [&](int st) -> uint4 {
			const int jj = st - sub;
			return (pass_active && jj >= 0 && jj < lt) ? __ldg(M + (int64_t(q) * S + st) * G + sub) : zero4;
		};
		// lane 0: the boundary row of column col, once the stripe above has published it
		auto load_row = [&](int col) -> ulonglong2 {
			if (sub != 0 || !pass_active || col >= lt || q == 0) return make_ulonglong2(1ull, 0ull);
			if (avail < col + 1) avail = wait_progress(prog_in, col + 1, p.status);
			return make_ulonglong2(__ldcg(bin + 2 * col), __ldcg(bin + 2 * col + 1));
		};
		uint4 w0 = load(0), w1 = load(1), w2 = load(2), w3 = load(3);
		ulonglong2 b0 = load_row(0), b1 = load_row(1);
		int pub_next = PUB_CHUNK;
		const int nsteps = pass_active ? lt + G - 1 : 0;
		for (int s = 0; s < nsteps; s++) {
			const uint4 wcur = w0;
			w0 = w1;
			w1 = w2;
			w2 = w3;
			w3 = load(s + 4);
			const ulonglong2 bcur = b0;
			b0 = b1;
			b1 = load_row(s + 2);
			const int j = s - sub;
			unsigned long long upN = shfl_up64(outN, G);
			unsigned long long upP = shfl_up64(outP, G);
			if (j >= 0 && j < lt) {
				if (sub == 0) {
					upN = bcur.x;
					upP = bcur.y;
				}
				const uint32_t ws[4] = {wcur.x, wcur.y, wcur.z, wcur.w};
				unsigned long long uN = upN, uP = upP;
				count_rows(p, ws, row0, j, ls, si, sj, prev_up, uN, uP, Nl, Ql, acc);
				outN = uN;
				outP = uP;
				if (write_boundary) {
					bout[2 * j] = outN;
					bout[2 * j + 1] = outP;
					if (j + 1 == pub_next && j + 1 < lt) {  // columns < j + 1 are written
						st_release(p.progress + t, j + 1);
						pub_next += PUB_CHUNK;
					}
				}
			}
			prev_up = upN;
		}
		if (write_boundary) st_release(p.progress + t, lt);  // every column
		for (int o = 1; o < G; o <<= 1) {
			const uint32_t lo = __shfl_xor_sync(0xffffffffu, uint32_t(acc), o);
			const uint32_t hi = __shfl_xor_sync(0xffffffffu, uint32_t(acc >> 32), o);
			acc = sat_add(acc, (unsigned long long)(hi) << 32 | lo);
		}
		if (lane == 0) p.partial[t] = acc;
	}
}

cudaError_t launch_path_count(const CountParams &p, int grid, cudaStream_t st) {
	if (p.ntickets > 0) path_count_chain_kernel<<<grid, BLOCK, 0, st>>>(p);
	else path_count_kernel<<<grid, BLOCK, 0, st>>>(p);
	return cudaGetLastError();
}

}  // namespace pa

// host-side declaration for pa_host.cu
namespace pa {
cudaError_t path_count_solve(int32_t npairs, int32_t G, int32_t local, int32_t affine, const int32_t *len_s,
                             const int32_t *len_t, const int64_t *mask_off, const void *masks, const int32_t *seed,
                             unsigned long long *counts, unsigned long long *scratch, int64_t scratch_stride,
                             int32_t *work_counter, int grid, cudaStream_t st, int32_t ntickets,
                             int32_t nlevels, const int32_t *level_start, const int32_t *order, int32_t *progress,
                             int32_t *status, unsigned long long *partial) {
	CountParams p{};
	p.ntickets = ntickets;
	p.nlevels = nlevels;
	p.level_start = level_start;
	p.order = order;
	p.progress = progress;
	p.status = status;
	p.partial = partial;
	p.npairs = npairs;
	p.G = G;
	p.local = local;
	p.affine = affine;
	p.len_s = len_s;
	p.len_t = len_t;
	p.mask_off = mask_off;
	p.masks = static_cast<const uint4 *>(masks);
	p.seed = seed;
	p.counts = counts;
	p.scratch = scratch;
	p.scratch_stride = scratch_stride;
	p.work_counter = work_counter;
	return launch_path_count(p, grid, st);
}
}  // namespace pa

// Traceback walk over the one-optimal-path masks (see pa_dp.cuh).
#include "pa_dp.cuh"

namespace pa {

// One warp per pair.  Steps follow TracebackIterators<false>::Iterator::next
// (solver.h:1497-1536): record the point, stop when u < 0 or v < 0 or (local) the value is
// not strictly positive -- which is exactly the "zero" source code 3 -- else follow the
// traceback: diagonal, vertical or horizontal; for affine gaps the P/Q tracebacks jump to
// the cell where the gap was opened (tb_P = tb_P(i-1, j) while the P-extend bit is set,
// solver.h:2995-3016).  Diagonal steps are the alignment edges (solver.h:809-847).
//
// The walk is a chain of dependent mask reads, so its speed is the latency of one read.
// The warp therefore caches a window of the masks in shared memory: lane l loads the words
// of the 8-row blocks (u >> 3) - r, r = 0..3, at column v - l -- 32 columns and the 25-32
// rows up-left of the cell where the window was placed, four independent loads in one round
// trip; a cell outside the window re-places it there.  Runs are resolved 32 cells at a time:
// for a run of diagonal steps lane k decodes cell (u - k, v - k) and one ballot gives the
// run's length (lanes then write their map entries and path points in parallel), and the
// start of an affine gap -- the first cell up or left whose extend bit is clear -- is found
// the same way.  A diagonal or gap run thus costs one memory round trip per 25-32 cells and a
// few instructions per 32 cells instead of per cell.
constexpr int WALK_WARPS = 4;  // warps per block of walk_kernel (128 threads)
constexpr int WIN_BLOCKS = 4;  // 8-row blocks per window
__global__ void __launch_bounds__(WALK_WARPS * 32) walk_kernel(WalkParams p) {
	__shared__ uint32_t wins[WALK_WARPS][WIN_BLOCKS][32];
	const int wid = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	uint32_t(*const win)[32] = wins[threadIdx.x >> 5];  // [row block ub - r][column vb - c]
	if (wid >= p.npairs) return;  // whole warps
	const int pair = p.pair0 + wid;
	if (p.status && (*p.status & ST_BAD_CODE)) return;  // the DP did not run: no seeds, no masks
	const int ls = p.len_s[pair], lt = p.len_t[pair];
	const int nmap = min(ls, lt);
	int32_t *map = p.maps ? p.maps + p.map_off[pair] : nullptr;
	if (map)
		for (int k = lane; k < nmap; k += 32) map[k] = -1;
	__syncwarp();  // the fill is ordered before lane 0's writes below
	int32_t *path = p.paths ? p.paths + p.path_off[pair] : nullptr;
	if (!p.has_seed[pair]) {
		if (p.path_len && lane == 0) p.path_len[pair] = 0;
		return;
	}
	int u = p.seed[2 * pair], v = p.seed[2 * pair + 1];
	if (path && lane == 0) { path[0] = u; path[1] = v; }
	int np = 1;
	const uint32_t *W = p.masks + p.mask_off[pair];
	const int G = p.pair_G ? int(p.pair_G[pair]) : p.G;
	const bool two = p.cols == 2;  // dp2_kernel layout: a uint2 per lane and step, columns j, j + 1
	const bool fmt16 = p.fmt16 != 0;
	const bool rows4 = p.rows4 != 0;  // dp16b_kernel records: 4-row lanes, 4 columns per step
	const int S = rows4 ? ((lt + 3) >> 2) + G - 1 : two ? ((lt + 1) >> 1) + G - 1 : lt + G - 1;
	const int npass4 = rows4 ? (ls + 4 * G - 1) / (4 * G) : 0;  // stripes of the 4-row layout
	const bool s2t = ls <= lt;
	const bool affine = p.gap == GAP_AFFINE;
	int ub = -1000000, vb = -1000000;  // window: row blocks ub-3..ub, columns vb-31..vb
	// place the window with cell (i, j) at its bottom-right corner (warp-uniform i, j)
	auto place = [&](int i, int j) {
		ub = i >> 3;
		vb = j;
		const int col = vb - lane;
		uint32_t w[WIN_BLOCKS];
#pragma unroll
		for (int r = 0; r < WIN_BLOCKS; r++) {
			const int rb = ub - r;
			w[r] = 0u;
			if (rb >= 0 && col >= 0) {
				if (rows4) {
					// the 8-row word of column col joins the 16-bit columns of the 4-row lanes
					// 2 rb (rows 0-3: high half) and 2 rb + 1 (rows 4-7: low half)
					uint32_t h[2] = {0u, 0u};
#pragma unroll
					for (int e = 0; e < 2; e++) {
						const int b4 = 2 * rb + e, q = b4 / G, sb = b4 - q * G;
						if (q < npass4) {
							const uint32_t word = W[((int64_t(q) * S + ((col >> 2) + sb)) * G + sb) * 2 + ((col >> 1) & 1)];
							h[e] = (word >> (16 * (col & 1))) & 0xffffu;
						}
					}
					w[r] = (h[0] << 16) | h[1];
				} else {
					const int q = rb / G, sb = rb - q * G;
					w[r] = two ? W[((int64_t(q) * S + ((col >> 1) + sb)) * G + sb) * 2 + (col & 1)]
					           : W[(int64_t(q) * S + (col + sb)) * G + sb];
				}
			}
		}
		__syncwarp();  // every lane is done reading the previous window
#pragma unroll
		for (int r = 0; r < WIN_BLOCKS; r++) win[r][lane] = w[r];
		__syncwarp();
	};
	auto inwin = [&](int i, int j) {
		const int dr = ub - (i >> 3), dc = vb - j;
		return i >= 0 && j >= 0 && dr >= 0 && dr < WIN_BLOCKS && dc >= 0 && dc <= 31;
	};
	// nibble of this lane's cell (i, j), valid where ok (the cell lies in the window).  Row
	// r's nibble (D source code | P-extend << 2 | Q-extend << 3) sits at bits 4(R-1-r); the
	// 16-bit kernel's nibbles hold the code in bits 2-3 and the open bits in 0-1.
	auto nib_at = [&](int i, int j, bool ok) -> uint32_t {
		const uint32_t w = ok ? win[ub - (i >> 3)][vb - j] : 0u;
		const uint32_t n = (w >> (4 * (R - 1 - (i & (R - 1))))) & 15u;
		return fmt16 ? ((n >> 2) | ((~n & 3u) << 2)) : n;
	};
	// index of the lowest clear bit of a ballot (32 when all are set)
	auto first_clear = [](uint32_t b) { return b == 0xffffffffu ? 32 : __ffs(int(~b)) - 1; };
	// first cell of a gap run: from (i, j) up (di = 1) or left (dj = 1) while the cell's
	// extend bit (mask) is set and the index is positive; lane m looks m cells ahead, one
	// ballot resolves up to 32 cells (the scalar loop: k = i; while (k > 0 && ext(k)) k--)
	auto gap_start = [&](int i, int j, int di, int dj, uint32_t mask) -> int {
		for (;;) {
			if (!inwin(i, j)) place(i, j);
			const int r = i - di * lane, c = j - dj * lane;
			const bool ok = inwin(r, c);
			const uint32_t n = nib_at(r, c, ok);
			const bool stop = ok && ((di ? r : c) == 0 || !(n & mask));
			const uint32_t bs = __ballot_sync(0xffffffffu, stop);
			const uint32_t bo = __ballot_sync(0xffffffffu, ok);
			const int first_stop = bs ? __ffs(int(bs)) - 1 : 32;
			const int first_out = first_clear(bo);  // >= 1: lane 0's cell (i, j) is in the window
			if (first_stop < first_out) return (di ? i : j) - first_stop;
			i -= di * first_out;
			j -= dj * first_out;
		}
	};
	while (u >= 0 && v >= 0) {
		if (!inwin(u, v)) place(u, v);
		// a run of diagonal steps: lane k looks at (u - k, v - k), one ballot finds how many
		// consecutive cells from (u, v) have the diagonal code
		const int iu = u - lane, iv = v - lane;
		const bool ok = inwin(iu, iv);
		const uint32_t n = nib_at(iu, iv, ok);
		const uint32_t bal = __ballot_sync(0xffffffffu, ok && (n & 3u) == 2u);
		const int run = first_clear(bal);
		if (run > 0) {
			if (lane < run) {
				if (map) {
					if (s2t) map[iu] = iv;
					else map[iv] = iu;
				}
				if (path) {
					path[2 * (np + lane)] = iu - 1;
					path[2 * (np + lane) + 1] = iv - 1;
				}
			}
			u -= run;
			v -= run;
			np += run;
			continue;
		}
		const uint32_t code = __shfl_sync(0xffffffffu, n, 0) & 3u;  // (u, v) is lane 0's cell
		if (p.local && code == 3u) break;
		int nu = u, nv = v;
		if (code == 1u) {
			nu = (affine ? gap_start(u, v, 1, 0, 4u) : u) - 1;
		} else {
			nv = (affine ? gap_start(u, v, 0, 1, 8u) : v) - 1;
		}
		u = nu;
		v = nv;
		if (path && lane == 0) { path[2 * np] = u; path[2 * np + 1] = v; }
		np++;
	}
	if (p.path_len && lane == 0) p.path_len[pair] = np;
}

// Largest code of an array, folded into *out with atomicMax.  Streams 16-byte words with
// four loads in flight per thread (the reads are the whole cost: 4 bytes per code), after a
// scalar head up to the first 16-byte boundary and before a scalar tail.
__global__ void codes_max_kernel(const uint32_t *x, int64_t n, uint32_t *out) {
	const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	const int64_t nth = int64_t(gridDim.x) * blockDim.x;
	const int64_t head = min(n, int64_t(((16 - (reinterpret_cast<uintptr_t>(x) & 15)) & 15) >> 2));
	uint32_t m = 0;
	if (tid < head) m = x[tid];
	const uint4 *v = reinterpret_cast<const uint4 *>(x + head);
	const int64_t nv = (n - head) >> 2;
	for (int64_t k = tid; k < nv; k += 4 * nth) {
		uint4 q[4];
#pragma unroll
		for (int u = 0; u < 4; u++) q[u] = k + u * nth < nv ? __ldcs(v + k + u * nth) : make_uint4(0, 0, 0, 0);
#pragma unroll
		for (int u = 0; u < 4; u++) m = max(m, max(max(q[u].x, q[u].y), max(q[u].z, q[u].w)));
	}
	const int64_t t0 = head + 4 * nv;
	if (t0 + tid < n) m = max(m, x[t0 + tid]);  // at most 3 tail codes
	for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace pa

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
// The warp therefore caches a window of the masks: lane l holds the word of the 8-row block
// (u >> 3) - (l >> 4) at column v - (l & 15), i.e. 16 rows x 16 columns up-left of the cell
// where the window was placed, loaded in one round trip.  Every lane runs the same walk
// (all values are warp-uniform) and takes a cell's word from its lane with a shuffle; a
// cell outside the window re-places it there.  A diagonal or gap run thus costs one memory
// round trip per 8-16 steps instead of one per step.
__global__ void walk_kernel(WalkParams p) {
	const int pair = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (pair >= p.npairs) return;  // whole warps
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
	const int G = p.G;
	const bool two = p.cols == 2;  // dp2_kernel layout: a uint2 per lane and step, columns j, j + 1
	const int S = two ? ((lt + 1) >> 1) + G - 1 : lt + G - 1;
	const bool s2t = ls <= lt;
	const bool affine = p.gap == GAP_AFFINE;
	int ub = -1000000, vb = -1000000;  // window: row blocks ub-1..ub, columns vb-15..vb
	uint32_t win = 0;
	// nibble of cell (i, j), i, j >= 0 and warp-uniform (R = 8 rows per block)
	auto nib = [&](int i, int j) -> uint32_t {
		int dr = ub - (i >> 3), dc = vb - j;
		if (dr < 0 || dr > 1 || dc < 0 || dc > 15) {
			ub = i >> 3;
			vb = j;
			dr = 0;
			dc = 0;
			const int rb = ub - (lane >> 4), col = vb - (lane & 15);
			win = 0u;
			if (rb >= 0 && col >= 0) {
				const int q = rb / G, sb = rb - q * G;
				win = two ? W[((int64_t(q) * S + ((col >> 1) + sb)) * G + sb) * 2 + (col & 1)]
				          : W[(int64_t(q) * S + (col + sb)) * G + sb];
			}
		}
		const uint32_t w = __shfl_sync(0xffffffffu, win, dr * 16 + dc);
		// row r's nibble (D source code | P-extend << 2 | Q-extend << 3) at bits 4(R-1-r)
		return (w >> (4 * (R - 1 - (i & (R - 1))))) & 15u;
	};
	while (u >= 0 && v >= 0) {
		const uint32_t code = nib(u, v) & 3u;
		if (p.local && code == 3u) break;
		int nu = u, nv = v;
		if (code == 2u) {
			if (map && lane == 0) {
				if (s2t) map[u] = v;
				else map[v] = u;
			}
			nu = u - 1;
			nv = v - 1;
		} else if (code == 1u) {
			if (affine) {
				int k = u;
				while (k > 0 && (nib(k, v) & 4u)) k--;
				nu = k - 1;
			} else {
				nu = u - 1;
			}
		} else {
			if (affine) {
				int k = v;
				while (k > 0 && (nib(u, k) & 8u)) k--;
				nv = k - 1;
			} else {
				nv = v - 1;
			}
		}
		u = nu;
		v = nv;
		if (path && lane == 0) { path[2 * np] = u; path[2 * np + 1] = v; }
		np++;
	}
	if (p.path_len && lane == 0) p.path_len[pair] = np;
}

__global__ void codes_max_kernel(const uint32_t *x, int64_t n, uint32_t *out) {
	uint32_t m = 0;
	const int64_t stride = int64_t(gridDim.x) * blockDim.x;
	for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) m = max(m, x[k]);
	for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace pa

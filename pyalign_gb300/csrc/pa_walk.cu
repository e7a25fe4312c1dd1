// Traceback walk over the one-optimal-path masks (see pa_dp.cuh).
#include "pa_dp.cuh"

namespace pa {

__device__ __forceinline__ uint32_t nibble_at(const uint32_t *W, int i, int j, int G, int S) {
	const int rpp = G * R;
	const int q = i / rpp;
	const int rem = i - q * rpp;
	const int sb = rem / R;
	const int r = rem - sb * R;
	const uint32_t w = W[(int64_t(q) * S + (j + sb)) * G + sb];
	// row r's nibble (D source code | P-extend << 2 | Q-extend << 3) at bits 4(R-1-r)
	return (w >> (4 * (R - 1 - r))) & 15u;
}

// One thread per pair.  Steps follow TracebackIterators<false>::Iterator::next
// (solver.h:1497-1536): record the point, stop when u < 0 or v < 0 or (local) the value is
// not strictly positive -- which is exactly the "zero" source code 3 -- else follow the
// traceback: diagonal, vertical or horizontal; for affine gaps the P/Q tracebacks jump to
// the cell where the gap was opened (tb_P = tb_P(i-1, j) while the P-extend bit is set,
// solver.h:2995-3016).  Diagonal steps are the alignment edges (solver.h:809-847).
__global__ void walk_kernel(WalkParams p) {
	const int pair = blockIdx.x * blockDim.x + threadIdx.x;
	if (pair >= p.npairs) return;
	const int ls = p.len_s[pair], lt = p.len_t[pair];
	const int nmap = min(ls, lt);
	int32_t *map = p.maps ? p.maps + p.map_off[pair] : nullptr;
	if (map)
		for (int k = 0; k < nmap; k++) map[k] = -1;
	int32_t *path = p.paths ? p.paths + p.path_off[pair] : nullptr;
	if (!p.has_seed[pair]) {
		if (p.path_len) p.path_len[pair] = 0;
		return;
	}
	int u = p.seed[2 * pair], v = p.seed[2 * pair + 1];
	int np = 0;
	if (path) { path[0] = u; path[1] = v; }
	np = 1;
	const uint32_t *W = p.masks + p.mask_off[pair];
	const int G = p.G;
	const int S = lt + G - 1;
	const bool s2t = ls <= lt;
	const bool affine = p.gap == GAP_AFFINE;
	while (u >= 0 && v >= 0) {
		const uint32_t code = nibble_at(W, u, v, G, S) & 3u;
		if (p.local && code == 3u) break;
		int nu = u, nv = v;
		if (code == 2u) {
			if (map) {
				if (s2t) map[u] = v;
				else map[v] = u;
			}
			nu = u - 1;
			nv = v - 1;
		} else if (code == 1u) {
			if (affine) {
				int k = u;
				while (k > 0 && (nibble_at(W, k, v, G, S) & 4u)) k--;
				nu = k - 1;
			} else {
				nu = u - 1;
			}
		} else {
			if (affine) {
				int k = v;
				while (k > 0 && (nibble_at(W, u, k, G, S) & 8u)) k--;
				nv = k - 1;
			} else {
				nv = v - 1;
			}
		}
		u = nu;
		v = nv;
		if (path) { path[2 * np] = u; path[2 * np + 1] = v; }
		np++;
	}
	if (p.path_len) p.path_len[pair] = np;
}

__global__ void codes_max_kernel(const uint32_t *x, int64_t n, uint32_t *out) {
	uint32_t m = 0;
	const int64_t stride = int64_t(gridDim.x) * blockDim.x;
	for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) m = max(m, x[k]);
	for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace pa

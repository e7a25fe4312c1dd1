// The first k optimal alignments of every pair of an all-optimal result, enumerated on the
// device (sm_103a).
//
// The reference yields all optimal alignments of a pair one at a time from a depth-first
// search over the traceback lists (TracebackIterators<true>::Iterator::next,
// solver.h:1647-1716): a LIFO stack of (u, v, path length) entries, seeded with the one
// optimum of Global/Semiglobal or, for local alignment, every cell equal to a strictly
// positive optimum pushed in reverse scan order (solver.h:2060-2091); popping an entry
// truncates the path to its length and appends its point; a point with both coordinates
// >= 0 that continues (local: its value is not 0) pushes its traceback list in stored order
// -- the zero candidate, the diagonal, then the P list (the rows where the vertical gap was
// opened, scanned up its column while the gap extends) and the Q list (solver.h:1328-1369,
// 2995-3016), or one terminal entry when the list is empty -- and any other point ends a
// path, which is yielded unless de-duplication (remove_dup) has already yielded the same
// compressed path (CompressedPath, solver.h:730-760).
//
// enum_kernel runs exactly that search, one warp per pair, over the all-optimal masks the
// DP wrote (pa_dp.cuh layout: stripe q, step s, lane k, one uint4 of 8 rows of 16-bit cells).
// The control flow is warp-uniform: every lane follows the same search, lane 0 alone reads
// and writes the stack and the path (so it always sees its own writes), and the lanes
// cooperate where the work is wide -- a 32-row x 32-column window of mask cells loaded into
// shared memory (one uint4 per lane and row block; the search walks up and left, so a
// diagonal path reloads it every 32 steps), and at each yielded path the compression, the
// map (s_to_t or t_to_s, the reference's build_alignment from the compressed points,
// solver.h:940-1086) and the de-duplication test, 32 path points per lane step.  The last
// entry a point pushes is the next one popped, so it stays in registers and only the others
// are written to the stack.  Local seeds come from enum_seed_kernel (every cell with the
// seed bit, one block per pair), sorted on the host in the order the reference's stack
// pops them: increasing row, then increasing column.
//
// De-duplication: the compressed points of a path decrease strictly in both coordinates,
// so two compressed paths are equal exactly when their maps are.  Each yielded map carries
// a 64-bit order-free hash and its point count; a new path is compared in full with every
// earlier yield of equal hash and count, so the test is exact.
//
// Bounded memory: the stack of a pair has a fixed capacity; a pair that would exceed it
// stops, flags ENUM_OVERFLOW and is enumerated again from the start with a larger stack by
// the host.  The seed lists are sized the same way (the scan counts every seed).
#include "pa_dp.cuh"
#include "pa_enum.h"

namespace pa {

// every cell of a pair with the local seed bit (256), in any order
__global__ void __launch_bounds__(256) enum_seed_kernel(SeedScanParams p) {
	for (int w = blockIdx.x; w < p.nwork; w += gridDim.x) {
		const int L = p.work[w];
		const int ls = p.len_s[L], lt = p.len_t[L];
		if (ls == 0 || lt == 0) continue;
		const int G = p.G, rpp = G * R, lg = __ffs(G) - 1;  // G is a power of two
		const int64_t S = int64_t(lt) + G - 1, per = S * G;
		const int npass = (ls + rpp - 1) / rpp;
		const uint4 *m = p.masks + p.mask_off[L];
		int2 *out = p.seeds + p.seed_off[L];
		const int cap = p.seed_cap[L];
		for (int q = 0; q < npass; q++)
		for (int64_t e = threadIdx.x; e < per; e += blockDim.x) {
			const int k = int(e & (G - 1));
			const int64_t s = e >> lg;
			const int64_t j = s - k;
			const int i0 = q * rpp + k * R;
			if (j < 0 || j >= lt || i0 >= ls) continue;
			const uint4 c = m[int64_t(q) * per + e];
			const uint32_t wv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
			for (int r = 0; r < R; r++) {
				if (i0 + r >= ls) break;
				if ((wv[r >> 1] >> (16 * (r & 1))) & 256u) {
					const int x = atomicAdd(&p.seed_n[L], 1);
					if (x < cap) out[x] = make_int2(i0 + r, int(j));
				}
			}
		}
	}
}

struct Window {
	int gb0, j0;  // row blocks [gb0, gb0 + 4), columns [j0, j0 + 32)
};

// cell (i, j) of the pair's masks through the warp's shared window (warp-uniform call)
__device__ __forceinline__ uint32_t enum_cell(const EnumParams &p, uint4 (*win)[32], Window &w, const uint4 *m,
                                              int64_t S, int ls, int lt, int i, int j, int lane) {
	const int gb = i >> 3;
	if (gb < w.gb0 || gb >= w.gb0 + 4 || j < w.j0 || j >= w.j0 + 32) {
		w.gb0 = max(0, gb - 3);
		w.j0 = max(0, j - 31);
		__syncwarp();  // every lane is done with the old window
		const int jj = w.j0 + lane;
		if (jj < lt) {
#pragma unroll
			for (int r = 0; r < 4; r++) {
				const int g = w.gb0 + r;
				if (g * R < ls) {
					const int q = g / p.G, sb = g - q * p.G;
					win[r][lane] = m[(int64_t(q) * S + jj + sb) * p.G + sb];
				}
			}
		}
		__syncwarp();
	}
	const uint4 e = win[gb - w.gb0][j - w.j0];
	const int r = i & 7, h = r >> 1;
	const uint32_t word = h == 0 ? e.x : h == 1 ? e.y : h == 2 ? e.z : e.w;
	return (word >> (16 * (r & 1))) & 0xffffu;
}

__device__ __forceinline__ unsigned long long enum_mix(int u, int v) {
	// splitmix64 finaliser of the point: an order-free sum of these hashes a point set
	unsigned long long x = (static_cast<unsigned long long>(static_cast<uint32_t>(u)) << 32) | static_cast<uint32_t>(v);
	x += 0x9e3779b97f4a7c15ull;
	x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
	x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
	return x ^ (x >> 31);
}

__global__ void __launch_bounds__(WARPS * 32) enum_kernel(EnumParams p) {
	__shared__ uint4 win_all[WARPS][4][32];
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	uint4 (*win)[32] = win_all[wib];
	const int wi = blockIdx.x * WARPS + wib;
	if (wi >= p.nwork) return;
	const int L = p.work[wi];
	const int ls = p.len_s[L], lt = p.len_t[L];
	const int m = min(ls, lt);
	const bool s_side = ls <= lt;  // the map is s_to_t, else t_to_s
	const int64_t S = int64_t(lt) + p.G - 1;
	const uint4 *mk = p.masks + p.mask_off[L];
	int4 *stk = p.stack + p.stack_off[L];
	const int cap = p.stack_cap[L];
	int2 *path = p.path + p.path_off[L];
	int32_t *maps = p.maps + p.map_off[L];
	unsigned long long *hash = p.hash + int64_t(L) * p.k;
	int32_t *npts = p.npts + int64_t(L) * p.k;
	const int plen_cap = ls + lt + 2;
	Window w{-16, -64};

	int count = 0, sp = 0, si = 0, status = 0;
	const int nseed = p.local ? p.seed_n[L] : 0;
	const int2 *seeds = p.local ? p.seeds + p.seed_off[L] : nullptr;
	bool have = false;
	int eu = 0, ev = 0, epl = 0;
	if (!p.local && p.has[L]) {
		eu = p.seed[2 * L];
		ev = p.seed[2 * L + 1];
		have = true;
	}
	while (count < p.k) {
		if (!have) {
			if (sp > 0) {
				int4 t = make_int4(0, 0, 0, 0);
				if (lane == 0) t = stk[sp - 1];
				eu = __shfl_sync(0xffffffffu, t.x, 0);
				ev = __shfl_sync(0xffffffffu, t.y, 0);
				epl = __shfl_sync(0xffffffffu, t.z, 0);
				sp--;
			} else if (si < nseed) {
				const int2 s = seeds[si++];
				eu = s.x;
				ev = s.y;
				epl = 0;
			} else {
				break;  // exhausted
			}
		}
		have = false;
		int plen = epl;
		if (plen >= plen_cap) {  // cannot happen: every step lowers u + v
			status = ENUM_BAD_PATH;
			break;
		}
		if (lane == 0) path[plen] = make_int2(eu, ev);
		plen++;
		bool cont = eu >= 0 && ev >= 0;
		uint32_t c = 0;
		if (cont) {
			c = enum_cell(p, win, w, mk, S, ls, lt, eu, ev, lane);
			if (p.local && (c & 1u)) cont = false;
		}
		if (cont) {
			// the list in push order; every entry but the last goes to the stack, the last is
			// popped next and stays in registers
			int nu = ENUM_NO_TB, nv = ENUM_NO_TB;
			bool pend = false;
			bool over = false;
			auto add = [&](int u, int v) {
				if (pend) {
					if (sp >= cap) over = true;
					else {
						if (lane == 0) stk[sp] = make_int4(nu, nv, plen, 0);
						sp++;
					}
				}
				nu = u;
				nv = v;
				pend = true;
			};
			if (c & 1u) add(ENUM_NO_TB, ENUM_NO_TB);
			if (c & 2u) add(eu - 1, ev - 1);
			if (c & 4u) {
				if (p.affine) {
					for (int k = eu;; k--) {
						const uint32_t ck = k == eu ? c : enum_cell(p, win, w, mk, S, ls, lt, k, ev, lane);
						if (ck & 16u) add(k - 1, ev);
						if ((ck & 32u) && k > 0) continue;
						break;
					}
				} else {
					add(eu - 1, ev);
				}
			}
			if (c & 8u) {
				if (p.affine) {
					for (int k = ev;; k--) {
						const uint32_t ck = k == ev ? c : enum_cell(p, win, w, mk, S, ls, lt, eu, k, lane);
						if (ck & 64u) add(eu, k - 1);
						if ((ck & 128u) && k > 0) continue;
						break;
					}
				} else {
					add(eu, ev - 1);
				}
			}
			if (over) {
				status = ENUM_OVERFLOW;
				break;
			}
			eu = nu;
			ev = nv;
			epl = plen;
			have = true;
			continue;
		}

		// ---- a complete path: path[0, plen).  Its map, hash and point count, 32 points per step
		__syncwarp();  // lane 0's path writes are visible to the warp
		int32_t *mp = maps + int64_t(count) * m;
		for (int x = lane; x < m; x += 32) mp[x] = -1;
		__syncwarp();
		unsigned long long h = 0;
		int n = 0;
		for (int t = lane; t + 1 < plen; t += 32) {
			const int2 a = path[t], b = path[t + 1];
			if (b.x != a.x && b.y != a.y && a.x >= 0 && a.y >= 0) {
				if (s_side) mp[a.x] = a.y;
				else mp[a.y] = a.x;
				h += enum_mix(a.x, a.y);
				n++;
			}
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			h += __shfl_xor_sync(0xffffffffu, h, o);
			n += __shfl_xor_sync(0xffffffffu, n, o);
		}
		__syncwarp();  // the map is complete
		bool dup = false;
		if (p.remove_dup) {
			for (int r = 0; r < count && !dup; r++) {
				if (hash[r] != h || npts[r] != n) continue;
				const int32_t *mr = maps + int64_t(r) * m;
				bool same = true;
				for (int x = lane; x < m; x += 32) same &= mr[x] == mp[x];
				dup = __all_sync(0xffffffffu, same);
			}
		}
		if (dup) continue;
		if (lane == 0) {
			hash[count] = h;
			npts[count] = n;
		}
		if (p.paths) {
			int2 *po = p.paths + p.paths_off[L] + int64_t(count) * plen_cap;
			for (int t = lane; t < plen; t += 32) po[t] = path[t];
			if (lane == 0) p.path_len[int64_t(L) * p.k + count] = plen;
		}
		count++;
	}
	// the slots past the last result hold no data of an earlier, abandoned search: -1 maps,
	// empty walks
	for (int64_t x = int64_t(count) * m + lane; x < int64_t(p.k) * m; x += 32) maps[x] = -1;
	if (p.paths)
		for (int j = count + lane; j < p.k; j += 32) p.path_len[int64_t(L) * p.k + j] = 0;
	if (lane == 0) {
		p.count[L] = count;
		p.status[L] = status;
	}
}

cudaError_t enum_seed_scan(const SeedScanParams &p, int grid, cudaStream_t st) {
	enum_seed_kernel<<<grid, 256, 0, st>>>(p);
	return cudaGetLastError();
}

cudaError_t enum_solve(const EnumParams &p, cudaStream_t st) {
	const int grid = (p.nwork + WARPS - 1) / WARPS;
	if (grid > 0) enum_kernel<<<grid, WARPS * 32, 0, st>>>(p);
	return cudaGetLastError();
}

}  // namespace pa

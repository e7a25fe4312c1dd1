// Two-column variant of the integer DP kernel (sm_103a).
//
// Same recurrences, tie rules and seeds as dp_kernel (pa_dp.cuh; solver.h:2825-2855,
// 2970-3036, 3213-3251, 1226-1427, 1980-2327) for int32 tagged scoring without the
// all-optimal masks or Solution values.  The difference is the work of a lane per step:
// dp_kernel updates its R = 8 rows in one column, a dependent chain of max operations down
// the rows that leaves the issue slots idle while each result is awaited; here a lane updates
// its rows in two adjacent columns j, j + 1 per step.  Cell (r, j + 1) needs only (r, j),
// (r - 1, j + 1) and (r - 1, j), so the two columns form two chains offset by one row that
// the scheduler interleaves, and the per-step work (shuffles of the boundary row, code
// loads, the traceback store) is shared by 16 cells instead of 8.
//
// Lane k of a group works on columns 2(s - k) and 2(s - k) + 1 in step s.  The traceback
// words of a step are stored as one uint2 per lane (column j in .x, j + 1 in .y) at
// ((q * S2 + s) * G + k) in uint2 units, S2 = ceil(|t| / 2) + G - 1: a coalesced G * 8-byte
// line per step; the walker maps cell (i, j) to word 2 * ((q * S2 + j / 2 + k) * G + k) +
// j % 2.
#pragma once

#include "pa_dp.cuh"

namespace pa {

// One tagged cell: value and tie winner from one max chain (see dp_kernel), the 4-bit
// traceback nibble shifted into mword.  Qrow holds Q of the cell to the left on entry and
// this cell's Q on return (affine only).
template <int GAP, int LOC, int TB>
__device__ __forceinline__ void cell_tag(const DpParams<int32_t> &p, int32_t S, int32_t dsave, int32_t old,
                                         int32_t &Qrow, int32_t uD, int32_t uP, int32_t &D, int32_t &P,
                                         uint32_t &mword) {
	int32_t key;
	if (GAP == GAP_AFFINE) {
		const int32_t oP = imad(uD, p.one, p.c_open_s);
		P = addmax(uP, p.c_ext_s, oP);
		const int32_t oQ = imad(old, p.one, p.c_open_t);
		const int32_t Q = addmax(Qrow, p.c_ext_t, oQ);
		key = addmax(dsave, S, vmax(P, Q));
		if (LOC == LOC_LOCAL) key = vmax(key, 3);
		const int32_t code = key & 3;
		D = imad(code, p.minus_one, key);
		if (TB == TB_ONE) {
			int32_t nb = imad(int32_t(gt_mask(P, oP)), p.minus_four, code);
			nb = imad(int32_t(gt_mask(Q, oQ)), p.minus_eight, nb);
			mword = uint32_t(imad(int32_t(mword), p.sixteen, nb));
		}
		Qrow = Q;
	} else if (GAP == GAP_LINEAR) {
		key = addmax(dsave, S, addmax(uD, p.c_up, imad(old, p.one, p.c_left)));
		if (LOC == LOC_LOCAL) key = vmax(key, 3);
		const int32_t code = key & 3;
		D = imad(code, p.minus_one, key);
		if (TB == TB_ONE) mword = uint32_t(imad(int32_t(mword), p.sixteen, code));
	} else {  // DTW
		key = addmax(dsave, 2, addmax(uD, 1, old));
		const int32_t code = key & 3;
		D = imad(code, p.minus_one, key) + S;
		if (TB == TB_ONE) mword = uint32_t(imad(int32_t(mword), p.sixteen, code));
	}
}

template <int GAP, int LOC, int TB, bool CHAIN>
__global__ void __launch_bounds__(BLOCK, 4) dp2_kernel(DpParams<int32_t> p) {
	typedef int32_t V;
	typedef int2 V2;
	constexpr bool TAG = true;
	constexpr bool KEYSEED = TB == TB_ONE && LOC == LOC_LOCAL;
	static_assert(TB != TB_ALL, "all-optimal masks use dp_kernel");
	if (!codes_valid(p)) return;

	extern __shared__ __align__(16) unsigned char smem_raw[];
	V *stab = reinterpret_cast<V *>(smem_raw);
	const bool table_in_smem = (p.sub_kind == SUB_TABLE || p.sub_kind == SUB_PROFILE || p.sub_kind == SUB_COLPROF) &&
	                           p.table_rows <= MAX_SMEM_TABLE && p.table_cols <= MAX_SMEM_TABLE;
	if (table_in_smem) {
		const int n = p.table_rows * p.table_cols;
		for (int k = threadIdx.x; k < n; k += blockDim.x) stab[k] = p.table[k];
	}
	__syncthreads();
	const V *tab = table_in_smem ? stab : p.table;
	uint2 *colprof = reinterpret_cast<uint2 *>(
	    smem_raw + ((size_t(table_in_smem ? p.table_rows * p.table_cols : 0) * sizeof(V) + 15) & ~size_t(15)));

	const int G = p.G;
	const int lane = threadIdx.x & 31;
	const int sub = lane % G;
	const int grp = lane / G;
	const int gpw = 32 / G;
	const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int slot = warp_global * gpw + grp;
	const int64_t half = p.scratch_stride / 2;
	const V NEG = p.neg_inf;
	const int rpp = G * R;
	const int sub_kind = p.sub_kind;
	const int ntickets = CHAIN ? p.ntickets : p.npairs;

	for (;;) {
		int base = 0;
		if (lane == 0) base = atomicAdd(p.work_counter, gpw);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= ntickets) break;
		int w = base + grp, q_lo = 0, prod = -1;
		if constexpr (CHAIN) {
			int lo = 0, hi = p.nlevels - 1;
			while (lo < hi) {
				const int mid = (lo + hi + 1) >> 1;
				if (p.level_start[mid] <= base) lo = mid;
				else hi = mid - 1;
			}
			q_lo = lo;
			w = base - p.level_start[lo];
			if (lo > 0) prod = p.level_start[lo - 1] + w;
		}
		V2 *scr = reinterpret_cast<V2 *>(p.scratch) + int64_t(CHAIN ? w : slot) * p.scratch_stride;
		const int pair = w < p.npairs ? p.order[w] : -1;
		const int ls = pair >= 0 ? p.len_s[pair] : 0;
		const int lt = pair >= 0 ? p.len_t[pair] : 0;
		const bool empty = ls == 0 || lt == 0;
		const int npass = empty ? 0 : (ls + rpp - 1) / rpp;
		const int nsteps_pair = ((lt + 1) >> 1) + G - 1;
		int wpass = npass, wsteps = empty ? 0 : nsteps_pair;
		for (int o = 16; o > 0; o >>= 1) {
			wpass = max(wpass, __shfl_xor_sync(0xffffffffu, wpass, o));
			wsteps = max(wsteps, __shfl_xor_sync(0xffffffffu, wsteps, o));
		}
		const uint32_t *arow = p.a + int64_t(pair < 0 ? 0 : pair) * p.a_stride;
		const uint32_t *brow = p.b + int64_t(pair < 0 ? 0 : pair) * p.b_stride;

		V l_best = NEG;
		int l_bi = -1, l_bj = -1;
		V row_best = NEG;
		int row_bj = -1;
		V col_best = NEG;
		int col_bi = -1;
		V glob = NEG;
		bool have_glob = false;

		const int q_hi = CHAIN ? min(q_lo + 1, npass) : wpass;
		for (int q = q_lo; q < q_hi; q++) {
			const bool pass_active = q < npass;
			const int row0 = q * rpp + sub * R;
			const int nvalid = ls - row0;
			const V2 *bin = scr + (q & 1) * half;
			V2 *bout = scr + ((q + 1) & 1) * half;
			const bool write_boundary = sub == G - 1 && q + 1 < npass;
			const int32_t *prog_in = (CHAIN && q > 0) ? p.progress + prod : nullptr;
			int32_t avail = 0;
			int pub_next = PUB_CHUNK;
			// lane 0: (D, P) above the next step's two columns, read one step ahead -- the top
			// border in the first stripe, else the boundary row of the stripe above
			V2 bn0, bn1;
			bn0.x = bn0.y = bn1.x = bn1.y = NEG;
			if (sub == 0 && pass_active) {
				if (q == 0) {
					bn0.x = p.top_D[1];
					if (lt > 1) bn1.x = p.top_D[2];
				} else if (CHAIN) {
					avail = wait_progress(prog_in, min(2, lt), p.status);
					bn0 = __ldcg(bin);
					if (lt > 1) bn1 = __ldcg(bin + 1);
				} else {  // group mode: written by this warp's last lane in the previous pass
					bn0 = bin[0];
					if (lt > 1) bn1 = bin[1];
				}
			}

			uint32_t qa[R];
			uint32_t plo[R], phi[R];
#pragma unroll
			for (int r = 0; r < R; r++) {
				const int i = row0 + r;
				qa[r] = (pass_active && i < ls) ? arow[i] : 0u;
				plo[r] = phi[r] = 0u;
			}
			if (sub_kind == SUB_COLPROF) {
				const int cols = p.table_cols;
				for (int c = 0; c < cols; c++) {
					uint32_t lo = 0, hi = 0;
#pragma unroll
					for (int r = 0; r < R; r++) {
						const uint32_t byte = uint32_t(tab[qa[r] * cols + c]) & 0xffu;
						if (r < 4) lo |= byte << (8 * r);
						else hi |= byte << (8 * (r - 4));
					}
					colprof[c * BLOCK + threadIdx.x] = make_uint2(lo, hi);
				}
			} else if (sub_kind == SUB_PROFILE) {
				const int cols = p.table_cols;
#pragma unroll
				for (int r = 0; r < R; r++) {
					uint32_t lo = 0, hi = 0;
					for (int c = 0; c < cols; c++) {
						const uint32_t byte = uint32_t(tab[qa[r] * cols + c]) & 0xffu;
						if (c < 4) lo |= byte << (8 * c);
						else hi |= byte << (8 * (c - 4));
					}
					plo[r] = lo;
					phi[r] = hi;
				}
			}

			V Dl[R], Ql[R];
#pragma unroll
			for (int r = 0; r < R; r++) {
				const int i = row0 + r;
				Dl[r] = (pass_active && i < ls) ? p.left_D[i + 1] : NEG;
				Ql[r] = NEG;
			}
			// (D, P) of this lane's last row in both columns as seen by the next lane; before the
			// lane starts they stand for column -1, whose D is the border D(row0 + 7, -1)
			V outD0 = Dl[R - 1], outP0 = NEG, outD1 = Dl[R - 1], outP1 = NEG;
			V prev_up = (pass_active && row0 <= ls) ? p.left_D[row0] : NEG;  // D(row0-1, j0-1)

			constexpr int NB = KEYSEED ? R : 1;
			V bv[NB];
#pragma unroll
			for (int r = 0; r < NB; r++) bv[r] = -1;
			const int kshift = p.key_shift;
			const int kmul = 1 << kshift;
			const bool last_row_lane = pass_active && nvalid >= 1 && nvalid <= R;
			const int r_last = nvalid - 1;

			uint32_t tn0 = pass_active ? brow[0] : 0u;
			uint32_t tn1 = (pass_active && lt > 1) ? brow[1] : 0u;
			uint2 *mrow = nullptr;
			if (TB == TB_ONE && pass_active)
				mrow = reinterpret_cast<uint2 *>(p.masks) + p.mask_off[pair] / 2 + int64_t(q) * nsteps_pair * G + sub;

			for (int s = 0; s < wsteps; s++) {
				const int j0 = 2 * (s - sub), j1 = j0 + 1;
				V upD0 = __shfl_up_sync(0xffffffffu, outD0, 1, G);
				V upP0 = __shfl_up_sync(0xffffffffu, outP0, 1, G);
				V upD1 = __shfl_up_sync(0xffffffffu, outD1, 1, G);
				V upP1 = __shfl_up_sync(0xffffffffu, outP1, 1, G);
				const bool act = pass_active && j0 >= 0 && j0 < lt;
				const bool act1 = act && j1 < lt;
				const uint32_t tc0 = tn0, tc1 = tn1;
				if (act && j0 + 2 < lt) tn0 = brow[j0 + 2];
				if (act && j0 + 3 < lt) tn1 = brow[j0 + 3];
				if (sub == 0 && act) {
					if (q == 0) {
						upD0 = bn0.x;
						upP0 = NEG;
						upD1 = act1 ? bn1.x : NEG;
						upP1 = NEG;
						if (j0 + 2 < lt) {  // prefetch the next step's two columns
							bn0.x = p.top_D[j0 + 3];
							if (j0 + 3 < lt) bn1.x = p.top_D[j0 + 4];
						}
					} else if constexpr (CHAIN) {
						upD0 = bn0.x;
						upP0 = bn0.y;
						upD1 = bn1.x;
						upP1 = bn1.y;
						if (j0 + 2 < lt) {  // prefetch the next step's two columns
							const int need = min(j0 + 4, lt);
							if (avail < need) avail = wait_progress(prog_in, need, p.status);
							bn0 = __ldcg(bin + j0 + 2);
							if (j0 + 3 < lt) bn1 = __ldcg(bin + j0 + 3);
						}
					} else {
						upD0 = bn0.x;
						upP0 = bn0.y;
						upD1 = bn1.x;
						upP1 = bn1.y;
						if (j0 + 2 < lt) {
							bn0 = bin[j0 + 2];
							if (j0 + 3 < lt) bn1 = bin[j0 + 3];
						}
					}
				}
				if (act) {
					uint32_t sel0 = 0, sel1 = 0;
					uint2 pr0 = make_uint2(0, 0), pr1 = make_uint2(0, 0);
					if (sub_kind == SUB_PROFILE) {
						sel0 = sext_selector(tc0);
						sel1 = sext_selector(tc1);
					} else if (sub_kind == SUB_COLPROF) {
						pr0 = colprof[tc0 * BLOCK + threadIdx.x];
						pr1 = colprof[tc1 * BLOCK + threadIdx.x];
					}
					uint32_t mw0 = 0, mw1 = 0;
					V dsave0 = prev_up, dsave1 = upD0;  // D(i-1, j0-1), D(i-1, j0) for row 0
					V uD0 = upD0, uP0 = upP0, uD1 = upD1, uP1 = upP1;
					V x0 = NEG, x1 = NEG;  // the last valid row's values (semiglobal / global)
#pragma unroll
					for (int r = 0; r < R; r++) {
						V S0, S1;
						if (sub_kind == SUB_PROFILE) {
							S0 = prmt(plo[r], phi[r], sel0);
							S1 = prmt(plo[r], phi[r], sel1);
						} else if (sub_kind == SUB_COLPROF) {
							S0 = prmt(pr0.x, pr0.y, sext_selector(uint32_t(r)));
							S1 = prmt(pr1.x, pr1.y, sext_selector(uint32_t(r)));
						} else if (sub_kind == SUB_BINARY) {
							S0 = (qa[r] == tc0) ? p.eq : p.ne;
							S1 = (qa[r] == tc1) ? p.eq : p.ne;
						} else {
							S0 = tab[qa[r] * p.table_cols + tc0];
							S1 = tab[qa[r] * p.table_cols + tc1];
						}
						const V old = Dl[r];
						V Q = Ql[r];
						V D0, P0 = NEG, D1, P1 = NEG;
						cell_tag<GAP, LOC, TB>(p, S0, dsave0, old, Q, uD0, uP0, D0, P0, mw0);
						cell_tag<GAP, LOC, TB>(p, S1, dsave1, D0, Q, uD1, uP1, D1, P1, mw1);
						if (KEYSEED) {
							bv[r] = vmax(bv[r], imad(D0, kmul, j0));
							if (act1) bv[r] = vmax(bv[r], imad(D1, kmul, j1));
						} else if (LOC == LOC_LOCAL && TB == TB_NONE) {
							if (r < nvalid) l_best = vmax(l_best, act1 ? vmax(D0, D1) : D0);
						}
						if (LOC != LOC_LOCAL && r == r_last) {
							x0 = D0;
							x1 = D1;
						}
						dsave0 = old;
						dsave1 = D0;
						Dl[r] = act1 ? D1 : D0;  // the values at the lane's last real column
						Ql[r] = Q;
						uD0 = D0;
						uP0 = P0;
						uD1 = D1;
						uP1 = P1;
					}
					outD0 = uD0;
					outP0 = uP0;
					outD1 = uD1;
					outP1 = uP1;
					if (write_boundary) {
						bout[j0] = V2{outD0, outP0};
						if (act1) bout[j1] = V2{outD1, outP1};
						if (CHAIN && j1 + 1 == pub_next) {  // columns < j1 + 1 are written
							if (j1 + 1 < lt) st_release(p.progress + base, j1 + 1);
							pub_next += PUB_CHUNK;
						}
					}
					if (TB == TB_ONE) mrow[s * G] = make_uint2(mw0, mw1);

					if (LOC == LOC_SEMI || LOC == LOC_GLOBAL) {
						if (last_row_lane && q == npass - 1) {
							if (LOC == LOC_SEMI) {
								if (x0 > row_best) { row_best = x0; row_bj = j0; }
								if (act1 && x1 > row_best) { row_best = x1; row_bj = j1; }
							} else if (j0 == lt - 1) {
								glob = x0;
								have_glob = true;
							} else if (j1 == lt - 1) {
								glob = x1;
								have_glob = true;
							}
						}
						if (LOC == LOC_SEMI && (j0 == lt - 1 || j1 == lt - 1)) {
#pragma unroll
							for (int r = 0; r < R; r++)
								if (r < nvalid && Dl[r] > col_best) { col_best = Dl[r]; col_bi = row0 + r; }
						}
					}
				}
				prev_up = upD1;
			}
			if (KEYSEED) {
				// fold the per-row bests of valid rows: larger value, then larger i, then the
				// row's own largest j (solver.h:2048-2056)
#pragma unroll
				for (int r = 0; r < NB; r++) {
					if (r >= nvalid || bv[r] < 0) continue;
					const V v = bv[r] >> kshift;
					const int jj = bv[r] & (kmul - 1);
					if (v >= l_best) { l_best = v; l_bi = row0 + r; l_bj = jj; }
				}
			}
			__syncwarp();
		}
		finish_pair<V, LOC, TB, TAG, CHAIN>(p, G, sub, pair, ls, lt, empty, npass, q_lo, prod, base, NEG, l_best, l_bi,
		                                    l_bj, row_best, row_bj, col_best, col_bi, glob, have_glob);
	}
}

}  // namespace pa

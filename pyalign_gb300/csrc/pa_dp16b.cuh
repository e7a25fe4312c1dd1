// Packed 16-bit twin-pair DP kernel on 4 x 4 cell blocks (sm_103a).
//
// The same cells, recurrences, tie rules and 16-bit encoding as dp16_kernel (pa_dp16.cuh;
// solver.h:2825-2855, 2970-3036, 1226-1427, seeds 1980-2124), with another tile shape: a
// lane owns RB = 4 rows of each stripe of G * 4 rows and updates CB = 4 adjacent columns
// per step (lane k at columns 4 (s - k) .. 4 (s - k) + 3 in step s), a 4 x 4 block of cells
// of both pairs of its twin.  The block is computed by anti-diagonals -- cells (r, c) with
// r + c = d are independent -- so one step's dependent chain is 7 cells long for 16 cells
// (the 8-row, two-column kernel: 9 cells for 16), and a stripe is half as tall, which
// halves the padding rows of each pair's last stripe at equal G.
//
// Traceback records: per pair, stripe q, step s and lane k one uint2 at
// (q * S4 + s) * G + k, S4 = ceil(|t| / 4) + G - 1: word w holds columns 2w and 2w + 1 of
// the block, column c in bits 16 (c & 1) .. 16 (c & 1) + 15, row r's nibble at bits
// 4 (3 - r) of its column -- so an 8-row block of one column is two such 16-bit columns of
// lanes 2m and 2m + 1, which the walker joins (WalkParams.rows4).
//
// Local seeds: a cell's key carries its row (bits 2-3) and its column within the block
// (bits 0-1), so a step's best key is the largest value, then the largest row, then the
// largest column; across steps the later step wins a tie of (value, row), the column bits
// ignored (seed16b).
#pragma once

#include "pa_dp16.cuh"

namespace pa {

constexpr int RB = 4;  // rows per lane
constexpr int CB = 4;  // columns per lane step

// Local seeds, once per step: as seed16 with the block's column in tag bits 0-1.
template <int TB>
__device__ __forceinline__ void seed16b(uint32_t sv, int j, uint32_t &lm, uint32_t &pos) {
	if (TB == TB_NONE) {
		lm = h_max(lm, sv);
	} else {
		constexpr uint32_t par = 0x00030003u;
		const uint32_t s1 = sv | par;
		const uint32_t mx = h_max(s1, lm | par);
		const uint32_t below = h_minu(mx ^ s1, 0x00010001u);  // 1 where the step's key < best
		const uint32_t keep = below * 0xFFFFu;
		pos = (pos & keep) | ((uint32_t(j) * 0x10001u) & ~keep);
		lm = (lm & keep) | (sv & ~keep);
	}
}

template <int GAP, int LOC, int TB>
__global__ void __launch_bounds__(BLOCK, 4) dp16b_kernel(DpParams<int32_t> p) {
	static_assert(GAP == GAP_LINEAR || GAP == GAP_AFFINE, "linear or affine gaps");
	static_assert(LOC == LOC_LOCAL || LOC == LOC_GLOBAL, "local or global");
	static_assert(TB != TB_ALL, "one traceback or none");
	constexpr uint32_t HMIN = 0u;              // below every biased value
	constexpr uint32_t INVALID_ROW = 0x80808080u;
	constexpr bool SEED = LOC == LOC_LOCAL;
	if (!codes_valid(p)) return;

	extern __shared__ __align__(16) unsigned char smem_raw[];
	int32_t *stab = reinterpret_cast<int32_t *>(smem_raw);
	const int cols = p.table_cols;
	for (int k = threadIdx.x; k < p.table_rows * cols; k += blockDim.x) stab[k] = p.table[k];
	__syncthreads();

	const int G = p.G;
	const int lane = threadIdx.x & 31;
	const int sub = lane % G;
	const int grp = lane / G;
	const int gpw = 32 / G;
	const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int slot = warp_global * gpw + grp;
	const int64_t half = p.scratch_stride / 2;
	const int rpp = G * RB;
	const int ntwins = (p.npairs + 1) >> 1;
	const uint32_t NEG = p.h_neg;
	const int32_t NEG32 = p.neg_inf;

	for (;;) {
		int base = 0;
		if (lane == 0) base = atomicAdd(p.work_counter, gpw);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= ntwins) break;
		const int w = base + grp;
		const int pa = w < ntwins ? p.order[2 * w] : -1;
		const int pb = (w < ntwins && 2 * w + 1 < p.npairs) ? p.order[2 * w + 1] : -1;
		const int lsA = pa >= 0 ? p.len_s[pa] : 0, ltA = pa >= 0 ? p.len_t[pa] : 0;
		const int lsB = pb >= 0 ? p.len_s[pb] : 0, ltB = pb >= 0 ? p.len_t[pb] : 0;
		const bool emptyA = lsA == 0 || ltA == 0, emptyB = lsB == 0 || ltB == 0;
		const int npA = emptyA ? 0 : (lsA + rpp - 1) / rpp;
		const int npB = emptyB ? 0 : (lsB + rpp - 1) / rpp;
		const int rsA = emptyA ? 0 : lsA, rsB = emptyB ? 0 : lsB;
		const int ctA = emptyA ? 0 : ltA, ctB = emptyB ? 0 : ltB;
		const int ls = max(rsA, rsB), lt = max(ctA, ctB), ctmin = min(ctA, ctB);
		const int npass = max(npA, npB);
		const int nsteps = ((lt + CB - 1) / CB) + G - 1;
		int wpass = npass, wsteps = npass ? nsteps : 0;
		for (int o = 16; o > 0; o >>= 1) {
			wpass = max(wpass, __shfl_xor_sync(0xffffffffu, wpass, o));
			wsteps = max(wsteps, __shfl_xor_sync(0xffffffffu, wsteps, o));
		}
		const uint32_t *arowA = p.a + int64_t(pa < 0 ? 0 : pa) * p.a_stride;
		const uint32_t *arowB = p.a + int64_t(pb < 0 ? 0 : pb) * p.a_stride;
		const uint32_t *browA = p.b + int64_t(pa < 0 ? 0 : pa) * p.b_stride;
		const uint32_t *browB = p.b + int64_t(pb < 0 ? 0 : pb) * p.b_stride;

		int32_t bestA = NEG32, biA = -1, bjA = -1, bestB = NEG32, biB = -1, bjB = -1;
		int32_t globA = NEG32, globB = NEG32;
		bool haveA = false, haveB = false;

		for (int q = 0; q < wpass; q++) {
			const bool pass_active = q < npass;
			const int row0 = q * rpp + sub * RB;
			const int2 *bin = reinterpret_cast<const int2 *>(p.scratch) + int64_t(slot) * p.scratch_stride + (q & 1) * half;
			int2 *bout = reinterpret_cast<int2 *>(p.scratch) + int64_t(slot) * p.scratch_stride + ((q + 1) & 1) * half;
			const bool write_boundary = sub == G - 1 && q + 1 < npass;

			// int8 score profiles of this lane's rows, their floors, the left border
			uint32_t prA[RB], prB[RB], fl[RB], Dl[RB], Ql[RB];
#pragma unroll
			for (int r = 0; r < RB; r++) {
				const int i = row0 + r;
				const bool vA = pass_active && i < rsA, vB = pass_active && i < rsB;
				uint32_t xa = INVALID_ROW, xb = INVALID_ROW;
				if (vA) {
					const int32_t *t = stab + arowA[i] * cols;
					xa = 0x80808080u;
					for (int c = 0; c < cols; c++) xa = (xa & ~(0xffu << (8 * c))) | ((uint32_t(t[c]) & 0xffu) << (8 * c));
				}
				if (vB) {
					const int32_t *t = stab + arowB[i] * cols;
					xb = 0x80808080u;
					for (int c = 0; c < cols; c++) xb = (xb & ~(0xffu << (8 * c))) | ((uint32_t(t[c]) & 0xffu) << (8 * c));
				}
				prA[r] = xa;
				prB[r] = xb;
				fl[r] = LOC == LOC_LOCAL
				            ? ((vA ? 0x0000800Cu : (NEG & 0x0000FFFFu)) | (vB ? 0x800C0000u : (NEG & 0xFFFF0000u)))
				            : NEG;
				Dl[r] = (pass_active && i < ls) ? p.left16[i + 1] : NEG;
				Ql[r] = NEG;
			}
			// (D, P) of this lane's last row in each column of a step as the next lane sees them;
			// before the lane starts they stand for column -1 (the last column's D is the next
			// lane's diagonal at its first step)
			uint32_t outD[CB], outP[CB];
#pragma unroll
			for (int c = 0; c < CB; c++) {
				outD[c] = Dl[RB - 1];
				outP[c] = NEG;
			}
			uint32_t prev_up = (pass_active && row0 <= ls) ? p.left16[row0] : NEG;  // D(row0-1, j0-1)
			uint32_t lm = HMIN, pos = 0;
			const int nvA = rsA - row0, nvB = rsB - row0;

			uint2 *mA = nullptr, *mB = nullptr;  // this lane's traceback records of step 0
			if (TB == TB_ONE) {
				uint2 *m = reinterpret_cast<uint2 *>(p.masks);
				const int64_t sA = ((ltA + CB - 1) / CB) + G - 1, sB = ((ltB + CB - 1) / CB) + G - 1;
				if (pass_active && q < npA) mA = m + p.mask_off[pa] / 2 + int64_t(q) * sA * G + sub;
				if (pass_active && q < npB) mB = m + p.mask_off[pb] / 2 + int64_t(q) * sB * G + sub;
			}
			// lane 0: (D, P) above the pass's first row in the next step's columns, read a step
			// ahead -- the border row, or the boundary row of the previous pass
			auto fetch = [&](int col) -> int2 {
				if (col >= lt) return make_int2(int32_t(NEG), int32_t(NEG));
				return q == 0 ? make_int2(int32_t(p.top16[col + 1]), int32_t(NEG)) : bin[col];
			};
			int2 bn[CB];
#pragma unroll
			for (int c = 0; c < CB; c++) bn[c] = (sub == 0 && pass_active) ? fetch(c) : make_int2(int32_t(NEG), int32_t(NEG));
			// letters of t of the next step's columns
			uint32_t tnA[CB], tnB[CB];
#pragma unroll
			for (int c = 0; c < CB; c++) {
				tnA[c] = (pass_active && c < lt) ? browA[c] : 0u;
				tnB[c] = (pass_active && c < lt) ? browB[c] : 0u;
			}

			for (int s = 0; s < wsteps; s++) {
				const int j0 = CB * (s - sub);
				uint32_t upD[CB], upP[CB];
#pragma unroll
				for (int c = 0; c < CB; c++) {
					upD[c] = __shfl_up_sync(0xffffffffu, outD[c], 1, G);
					upP[c] = GAP == GAP_AFFINE ? __shfl_up_sync(0xffffffffu, outP[c], 1, G) : 0u;
				}
				const bool act = pass_active && j0 >= 0 && j0 < lt;
				uint32_t tcA[CB], tcB[CB];
#pragma unroll
				for (int c = 0; c < CB; c++) {
					tcA[c] = tnA[c];
					tcB[c] = tnB[c];
					if (act && j0 + CB + c < lt) {
						tnA[c] = browA[j0 + CB + c];
						tnB[c] = browB[j0 + CB + c];
					}
				}
				if (sub == 0 && act) {
#pragma unroll
					for (int c = 0; c < CB; c++) {
						upD[c] = uint32_t(bn[c].x);
						upP[c] = uint32_t(bn[c].y);
						bn[c] = fetch(j0 + CB + c);
					}
				}
				if (act) {
					uint32_t sel[CB];
#pragma unroll
					for (int c = 0; c < CB; c++) sel[c] = tcA[c] * 0x11u + tcB[c] * 0x1100u + 0xC480u;
					uint32_t Db[RB][CB], Pb[RB][CB], Qb[RB][CB];
					uint32_t mc[CB], sm[CB], ev[CB];
#pragma unroll
					for (int c = 0; c < CB; c++) {
						mc[c] = 0u;
						sm[c] = HMIN;
						ev[c] = HMIN;
					}
					// the block by anti-diagonals: (r, c) needs (r - 1, c), (r, c - 1), (r - 1, c - 1)
#pragma unroll
					for (int d = 0; d < RB + CB - 1; d++) {
#pragma unroll
						for (int c = 0; c < CB; c++) {
							const int r = d - c;
							if (r < 0 || r >= RB) continue;
							const uint32_t uD = r == 0 ? upD[c] : Db[r - 1][c];
							const uint32_t uP = r == 0 ? upP[c] : Pb[r - 1][c];
							const uint32_t old = c == 0 ? Dl[r] : Db[r][c - 1];
							const uint32_t Qleft = c == 0 ? Ql[r] : Qb[r][c - 1];
							const uint32_t dsave = r == 0 ? (c == 0 ? prev_up : upD[c - 1]) : (c == 0 ? Dl[r - 1] : Db[r - 1][c - 1]);
							const uint32_t S = uint32_t(prmt(prA[r], prB[r], sel[c]));
							uint32_t D, P, Q;
							const uint32_t key = cell16<GAP, LOC>(p, S, dsave, old, Qleft, uD, uP, fl[r], D, P, Q);
							Db[r][c] = D;
							Pb[r][c] = P;
							Qb[r][c] = Q;
							if (TB == TB_ONE) mc[c] = uint32_t(imad(int32_t(mc[c]), p.sixteen, int32_t(nib16<GAP>(key, P, Q))));
							if (SEED) {
								const uint32_t k = TB == TB_ONE ? h_addk(D, p.one, uint32_t(r * CB + c) * 0x10001u) : D;
								if ((r & 1) == 0) ev[c] = k;
								else sm[c] = h_max3(sm[c], ev[c], k);
							}
						}
					}
#pragma unroll
					for (int r = 0; r < RB; r++) {
						Dl[r] = Db[r][CB - 1];
						if (GAP == GAP_AFFINE) Ql[r] = Qb[r][CB - 1];
					}
#pragma unroll
					for (int c = 0; c < CB; c++) {
						outD[c] = Db[RB - 1][c];
						outP[c] = Pb[RB - 1][c];
					}
					if (write_boundary) {
#pragma unroll
						for (int c = 0; c < CB; c++)
							if (j0 + c < lt) bout[j0 + c] = make_int2(int32_t(outD[c]), int32_t(outP[c]));
					}
					if (TB == TB_ONE) {
						// pair A's columns in the low halves, pair B's in the high halves
						if (mA && j0 < ctA)
							mA[int64_t(s) * G] = make_uint2(__byte_perm(mc[0], mc[1], 0x5410), __byte_perm(mc[2], mc[3], 0x5410));
						if (mB && j0 < ctB)
							mB[int64_t(s) * G] = make_uint2(__byte_perm(mc[0], mc[1], 0x7632), __byte_perm(mc[2], mc[3], 0x7632));
					}
					if (SEED) {
						uint32_t sv;
						if (j0 + CB <= ctmin) {
							sv = h_max3(sm[0], sm[1], h_max(sm[2], sm[3]));
						} else {
							// a column inside one pair only: masked per half
							sv = HMIN;
#pragma unroll
							for (int c = 0; c < CB; c++) {
								const uint32_t cm = colmask16(j0 + c, ctA, ctB);
								sv = h_max(sv, (sm[c] & cm) | (HMIN & ~cm));
							}
						}
						seed16b<TB>(sv, j0, lm, pos);
					}
					if (LOC == LOC_GLOBAL) {
						// D(|s|-1, |t|-1) of a half: this lane's row |s|-1 in the step holding column |t|-1
						const int cA = ltA - 1 - j0, cBc = ltB - 1 - j0;
						if (q == npA - 1 && nvA >= 1 && nvA <= RB && cA >= 0 && cA < CB) {
							uint32_t v = 0u;
#pragma unroll
							for (int r = 0; r < RB; r++)
#pragma unroll
								for (int c = 0; c < CB; c++)
									if (r == nvA - 1 && c == cA) v = Db[r][c];
							globA = (h_lo(v) >> 4) * 4;
							haveA = true;
						}
						if (q == npB - 1 && nvB >= 1 && nvB <= RB && cBc >= 0 && cBc < CB) {
							uint32_t v = 0u;
#pragma unroll
							for (int r = 0; r < RB; r++)
#pragma unroll
								for (int c = 0; c < CB; c++)
									if (r == nvB - 1 && c == cBc) v = Db[r][c];
							globB = (h_hi(v) >> 4) * 4;
							haveB = true;
						}
					}
				}
				prev_up = upD[CB - 1];
			}
			if (SEED) {
				// fold the pass into the lane's running best (x4 tagged domain of finish_pair):
				// a later pass has larger rows, so it wins a tie of values
				const int32_t kA = h_lo(lm), kB = h_hi(lm);
				if (kA != -32768) {
					const int32_t v = (kA >> 4) * 4;
					if (v >= bestA) {
						bestA = v;
						biA = row0 + ((kA >> 2) & 3);
						bjA = int32_t(pos & 0xffffu) + (kA & 3);
					}
				}
				if (kB != -32768) {
					const int32_t v = (kB >> 4) * 4;
					if (v >= bestB) {
						bestB = v;
						biB = row0 + ((kB >> 2) & 3);
						bjB = int32_t(pos >> 16) + (kB & 3);
					}
				}
			}
			__syncwarp();
		}
		finish_pair<int32_t, LOC, TB, true, false>(p, G, sub, pa, lsA, ltA, emptyA, npA, 0, -1, 0, NEG32, bestA, biA,
		                                           bjA, NEG32, -1, NEG32, -1, globA, haveA);
		finish_pair<int32_t, LOC, TB, true, false>(p, G, sub, pb, lsB, ltB, emptyB, npB, 0, -1, 0, NEG32, bestB, biB,
		                                           bjB, NEG32, -1, NEG32, -1, globB, haveB);
	}
}

}  // namespace pa

// Packed 16-bit DP kernel for twin pairs (sm_103a).
//
// Same recurrences and tie rules as dp_kernel (pa_dp.cuh; solver.h:2825-2855, 2970-3036,
// 1226-1427) and the same Local / Global seeds (solver.h:1980-2124), for integer scoring
// whose values provably fit in 16 bits.  Every 32-bit register holds the same cell of two
// pairs -- the "twin" of two consecutive pairs in the processing order, which the host sorts
// by stripe count and |t| so twins have nearly the same shape -- one per 16-bit half, and
// every add and max is one packed instruction (add.s16x2 / max.s16x2, fused to one
// add-max or three-way max where the hardware has it) that updates both cells.
//
// Value encoding: value * 16 + tag, offset by 32768 (offset binary, compared as unsigned
// 16-bit numbers, so the order is the signed order).  Bits 2-3 of the tag are the push priority of the
// candidate as in the int32 kernels (zero 3 > diag 2 > P/up 1 > Q/left 0), so one max
// chain yields the value and the reference's tie winner.  Bit 0 is set on P's "open"
// candidate (from D above) and bit 1 on Q's (from D to the left); the "extend" candidates
// are formed from P and Q with that bit cleared, so among equal values the open candidate
// wins -- the extend bit of the int32 kernels (P > open strictly) is its complement -- and
// D = key with the four tag bits cleared.  The traceback nibble of a cell is
// (key & 12) | ((P | Q) & 3): code in bits 2-3, P-open in bit 0, Q-open in bit 1; the
// walker reads it with that layout (WalkParams.fmt16).
//
// Lanes and layout follow dp_kernel: a group of G lanes per twin, R = 8 rows per lane, one
// column per step.  The traceback words of each pair of the twin are stored in that pair's
// own dp_kernel layout ((q * S + s) * G + k, S = |t| + G - 1), so the walker needs no
// knowledge of twins.  A pair's cells beyond its own |s| or |t| (the twin computes the
// larger shape of the two) are never stored; for local seeds they are kept out as follows:
// columns beyond |t| are masked per step, and rows beyond |s| get an int8 score of -128
// (-8 in value units) and no zero floor, which -- with gap costs of at least 1, which the
// host requires -- keeps their values strictly below the pair's optimum, so they can
// neither win nor tie.
//
// The host admits a launch only when bounds on every value (largest similarity times the
// shorter length, the borders, the gap costs) fit the 16-bit range with room for the
// sentinel, so the results equal the int32 kernels' bit for bit.
//
// Adds of a constant to a packed value run as one 32-bit IMAD on the FMA pipe instead of a
// packed add on the ALU pipe, which the max chains keep busy: every biased value stays above
// the sentinel margin, which exceeds the magnitude of any negative gap addend, so adding such
// an addend always carries out of the low half, and the host folds that carry into the high
// half of the constant (k_open_s and friends).  The bounds hold in every cell a launch
// computes -- the padding rows and columns of twins included (a zero or sentinel floor on
// every row, the upper bound over the launch's whole rectangle) -- because a wrapped half
// would carry into its neighbour.
#pragma once

#include "pa_dp.cuh"

namespace pa {

__device__ __forceinline__ uint32_t h_add(uint32_t a, uint32_t b) {
	uint32_t d;
	asm("add.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

__device__ __forceinline__ uint32_t h_max(uint32_t a, uint32_t b) {
	uint32_t d;
	asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

// max(a + b, c) per half
__device__ __forceinline__ uint32_t h_addmax(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm("{.reg .b32 t;\n\tadd.u16x2 t, %1, %2;\n\tmax.u16x2 %0, t, %3;}" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

__device__ __forceinline__ uint32_t h_max3(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm("{.reg .b32 t;\n\tmax.u16x2 t, %1, %2;\n\tmax.u16x2 %0, t, %3;}" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

__device__ __forceinline__ uint32_t h_minu(uint32_t a, uint32_t b) {
	uint32_t d;
	asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

// the (value * 16 + tag) of the low or high half, bias removed
__device__ __forceinline__ int32_t h_lo(uint32_t x) { return int32_t(x & 0xffffu) - 32768; }
__device__ __forceinline__ int32_t h_hi(uint32_t x) { return int32_t(x >> 16) - 32768; }
// x + k as one IMAD (FMA pipe); k carries the low half's carry (see above)
__device__ __forceinline__ uint32_t h_addk(uint32_t x, int32_t one, uint32_t k) {
	return uint32_t(imad(int32_t(x), one, int32_t(k)));
}

// One cell of each half: (D, P) from above, the D to the left and its Q, the diagonal D, the
// score S; returns the tagged key, writes D, P, Q (see the encoding above).
template <int GAP, int LOC>
__device__ __forceinline__ uint32_t cell16(const DpParams<int32_t> &p, uint32_t S, uint32_t dsave, uint32_t old,
                                           uint32_t Qleft, uint32_t uD, uint32_t uP, uint32_t floor_, uint32_t &D,
                                           uint32_t &P, uint32_t &Q) {
	constexpr uint32_t CLR_TAG = 0xFFF0FFF0u;  // D: the value bits
	constexpr uint32_t CLR_PF = 0xFFFEFFFEu;   // P without its open bit
	constexpr uint32_t CLR_QF = 0xFFFDFFFDu;   // Q without its open bit
	if (GAP == GAP_AFFINE) {
		P = h_addmax(uP & CLR_PF, p.h_ext_s, h_addk(uD, p.one, p.k_open_s));
		Q = h_addmax(Qleft & CLR_QF, p.h_ext_t, h_addk(old, p.one, p.k_open_t));
	} else {
		P = h_addk(uD, p.one, p.k_up);
		Q = h_addk(old, p.one, p.k_left);
	}
	const uint32_t m = h_max3(P, Q, floor_);  // zero floor (local) or sentinel floor
	const uint32_t key = h_addmax(dsave, S, m);
	D = key & CLR_TAG;
	return key;
}

// The traceback nibbles of a cell in both halves: code in bits 2-3, P-open bit 0, Q-open bit 1.
template <int GAP>
__device__ __forceinline__ uint32_t nib16(uint32_t key, uint32_t P, uint32_t Q) {
	constexpr uint32_t FLAGS = 0x00030003u, CODES = 0x000C000Cu;
	return GAP == GAP_AFFINE ? (((P | Q) & FLAGS) | (key & CODES)) : (key & CODES);
}

// Local seeds, once per step: fold the step's best (value | tag) key per half -- masked to the
// half's own columns -- into the lane's best of the pass; a key whose (value, row) is >= that
// best's moves the best, and its column, to this step (the later column wins a tie).  With two
// columns per step the tag's bit 0 is the column parity: it orders the step's two columns but
// not steps, so the comparison with the best ignores it.
template <int TB, int C>
__device__ __forceinline__ void seed16(uint32_t sv, int j, uint32_t &lm, uint32_t &pos) {
	if (TB == TB_NONE) {
		lm = h_max(lm, sv);
	} else {
		const uint32_t par = C == 2 ? 0x00010001u : 0u;
		const uint32_t s1 = sv | par;
		const uint32_t mx = h_max(s1, lm | par);
		const uint32_t below = h_minu(mx ^ s1, 0x00010001u);  // 1 where the step's key < best
		const uint32_t keep = below * 0xFFFFu;
		pos = (pos & keep) | ((uint32_t(j) * 0x10001u) & ~keep);
		lm = (lm & keep) | (sv & ~keep);
	}
}

__device__ __forceinline__ uint32_t colmask16(int j, int ctA, int ctB) {
	return (j < ctA ? 0x0000FFFFu : 0u) | (j < ctB ? 0xFFFF0000u : 0u);
}

// C = 1: a lane updates its R rows in one column per step.  C = 2: in two adjacent columns
// j, j + 1 per step (two dependency chains offset by one row that the scheduler interleaves;
// the step's shuffles, letter loads, stores and seed update serve 32 cells), with the
// traceback words of a pair stored as one uint2 per lane and step in the dp2_kernel layout
// ((q * S2 + s) * G + k, S2 = ceil(|t| / 2) + G - 1).  The local seed keys carry the row in
// tag bits 0-2 (C = 1) or 1-3 with the column parity in bit 0 (C = 2): a larger row wins a tie
// of values, then the later column.
template <int GAP, int LOC, int TB, int C>
__global__ void __launch_bounds__(BLOCK, 4) dp16_kernel(DpParams<int32_t> p) {
	static_assert(GAP == GAP_LINEAR || GAP == GAP_AFFINE, "linear or affine gaps");
	static_assert(LOC == LOC_LOCAL || LOC == LOC_GLOBAL, "local or global");
	static_assert(TB != TB_ALL, "one traceback or none");
	static_assert(C == 1 || C == 2, "one or two columns per step");
	constexpr uint32_t HMIN = 0u;              // below every biased value
	constexpr uint32_t INVALID_ROW = 0x80808080u;
	constexpr bool SEED = LOC == LOC_LOCAL;
	if (!codes_valid(p)) return;

	extern __shared__ __align__(16) unsigned char smem_raw[];
	int32_t *stab = reinterpret_cast<int32_t *>(smem_raw);
	const int cols = p.table_cols;
	for (int k = threadIdx.x; k < p.table_rows * cols; k += blockDim.x) stab[k] = p.table[k];
	__syncthreads();

	const int lane = threadIdx.x & 31;
	const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int64_t half = p.scratch_stride / 2;
	const int ntwins = (p.npairs + 1) >> 1;
	const uint32_t NEG = p.h_neg;
	const int32_t NEG32 = p.neg_inf;

	for (;;) {
		// the next warp task: 32 / G twins of one width -- the launch's G, or with length
		// buckets the width of the segment the task falls in
		int G = p.G, base = 0, end = ntwins;
		if (p.nseg > 0) {
			int t = 0;
			if (lane == 0) t = atomicAdd(p.work_counter, 1);
			t = __shfl_sync(0xffffffffu, t, 0);
			if (t >= p.seg_task[p.nseg]) break;
			int k = 0;
			while (k + 1 < p.nseg && p.seg_task[k + 1] <= t) k++;
			G = p.seg_G[k];
			base = p.seg_unit[k] + (t - p.seg_task[k]) * (32 / G);
			end = p.seg_unit[k + 1];
		} else {
			if (lane == 0) base = atomicAdd(p.work_counter, 32 / G);
			base = __shfl_sync(0xffffffffu, base, 0);
			if (base >= ntwins) break;
		}
		const int sub = lane % G;
		const int grp = lane / G;
		const int slot = warp_global * p.slots_per_warp + grp;
		const int rpp = G * R;
		const int w = base + grp;
		const int pa = w < end ? p.order[2 * w] : -1;
		const int pb = (w < end && 2 * w + 1 < p.npairs) ? p.order[2 * w + 1] : -1;
		const int lsA = pa >= 0 ? p.len_s[pa] : 0, ltA = pa >= 0 ? p.len_t[pa] : 0;
		const int lsB = pb >= 0 ? p.len_s[pb] : 0, ltB = pb >= 0 ? p.len_t[pb] : 0;
		const bool emptyA = lsA == 0 || ltA == 0, emptyB = lsB == 0 || ltB == 0;
		const int npA = emptyA ? 0 : (lsA + rpp - 1) / rpp;
		const int npB = emptyB ? 0 : (lsB + rpp - 1) / rpp;
		// rows and columns of each pair that hold cells (none for an empty pair), and the
		// shape the twin computes
		const int rsA = emptyA ? 0 : lsA, rsB = emptyB ? 0 : lsB;
		const int ctA = emptyA ? 0 : ltA, ctB = emptyB ? 0 : ltB;
		const int ls = max(rsA, rsB), lt = max(ctA, ctB), ctmin = min(ctA, ctB);
		const int npass = max(npA, npB);
		const int nsteps = C == 2 ? ((lt + 1) >> 1) + G - 1 : lt + G - 1;
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
			const int row0 = q * rpp + sub * R;
			const int2 *bin = reinterpret_cast<const int2 *>(p.scratch) + int64_t(slot) * p.scratch_stride + (q & 1) * half;
			int2 *bout = reinterpret_cast<int2 *>(p.scratch) + int64_t(slot) * p.scratch_stride + ((q + 1) & 1) * half;
			const bool write_boundary = sub == G - 1 && q + 1 < npass;

			// int8 score profiles of this lane's rows (bytes = letters of t), the zero floor of
			// local alignment per row (none on rows beyond a pair's |s|), the left border
			uint32_t prA[R], prB[R], fl[R], Dl[R], Ql[R];
#pragma unroll
			for (int r = 0; r < R; r++) {
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
				// zero (tag 12, biased) on local rows, else the sentinel: no value falls below it
				fl[r] = LOC == LOC_LOCAL
				            ? ((vA ? 0x0000800Cu : (NEG & 0x0000FFFFu)) | (vB ? 0x800C0000u : (NEG & 0xFFFF0000u)))
				            : NEG;
				Dl[r] = (pass_active && i < ls) ? p.left16[i + 1] : NEG;
				Ql[r] = NEG;
			}
			// (D, P) of this lane's last row in each column of a step as the next lane sees them;
			// before the lane starts they stand for column -1
			uint32_t outD0 = Dl[R - 1], outP0 = NEG, outD1 = Dl[R - 1], outP1 = NEG;
			uint32_t prev_up = (pass_active && row0 <= ls) ? p.left16[row0] : NEG;  // D(row0-1, j-1)
			uint32_t lm = HMIN, pos = 0;  // the lane's best (value | tag) per half in this pass, its column
			const int nvA = rsA - row0, nvB = rsB - row0;

			uint32_t *mA = nullptr, *mB = nullptr;  // this lane's traceback words of step 0
			if (TB == TB_ONE) {
				uint32_t *m = reinterpret_cast<uint32_t *>(p.masks);
				const int64_t sA = C == 2 ? ((ltA + 1) >> 1) + G - 1 : ltA + G - 1;
				const int64_t sB = C == 2 ? ((ltB + 1) >> 1) + G - 1 : ltB + G - 1;
				if (pass_active && q < npA) mA = m + p.mask_off[pa] + (int64_t(q) * sA * G + sub) * C;
				if (pass_active && q < npB) mB = m + p.mask_off[pb] + (int64_t(q) * sB * G + sub) * C;
			}
			// lane 0: the (D, P) above this pass's first row in the next step's columns, read one
			// step ahead -- the border row, or the boundary row the group's last lane wrote in the
			// previous pass (complete before this pass: same warp, __syncwarp between passes)
			int2 bn0 = make_int2(int32_t(NEG), int32_t(NEG)), bn1 = bn0;
			if (sub == 0 && pass_active) {
				if (q == 0) {
					bn0.x = int32_t(p.top16[1]);
					if (C == 2 && lt > 1) bn1.x = int32_t(p.top16[2]);
				} else {
					bn0 = bin[0];
					if (C == 2 && lt > 1) bn1 = bin[1];
				}
			}
			uint32_t tnA0 = pass_active ? browA[0] : 0u, tnB0 = pass_active ? browB[0] : 0u;
			uint32_t tnA1 = (C == 2 && pass_active && lt > 1) ? browA[1] : 0u;
			uint32_t tnB1 = (C == 2 && pass_active && lt > 1) ? browB[1] : 0u;

			for (int s = 0; s < wsteps; s++) {
				const int j0 = C * (s - sub), j1 = j0 + 1;
				uint32_t upD0 = __shfl_up_sync(0xffffffffu, outD0, 1, G);
				uint32_t upP0 = GAP == GAP_AFFINE ? __shfl_up_sync(0xffffffffu, outP0, 1, G) : 0u;
				uint32_t upD1 = 0u, upP1 = 0u;
				if (C == 2) {
					upD1 = __shfl_up_sync(0xffffffffu, outD1, 1, G);
					if (GAP == GAP_AFFINE) upP1 = __shfl_up_sync(0xffffffffu, outP1, 1, G);
				}
				const bool act = pass_active && j0 >= 0 && j0 < lt;
				const bool act1 = C == 2 && act && j1 < lt;
				const uint32_t tcA0 = tnA0, tcB0 = tnB0, tcA1 = tnA1, tcB1 = tnB1;
				if (act && j0 + C < lt) {
					tnA0 = browA[j0 + C];
					tnB0 = browB[j0 + C];
				}
				if (C == 2 && act && j0 + 3 < lt) {
					tnA1 = browA[j0 + 3];
					tnB1 = browB[j0 + 3];
				}
				if (sub == 0 && act) {
					upD0 = uint32_t(bn0.x);
					upP0 = uint32_t(bn0.y);
					upD1 = uint32_t(bn1.x);
					upP1 = uint32_t(bn1.y);
					const int n0 = j0 + C, n1 = j0 + 3;  // the next step's columns
					if (n0 < lt) bn0 = q == 0 ? make_int2(int32_t(p.top16[n0 + 1]), int32_t(NEG)) : bin[n0];
					if (C == 2 && n1 < lt) bn1 = q == 0 ? make_int2(int32_t(p.top16[n1 + 1]), int32_t(NEG)) : bin[n1];
				}
				if (act) {
					// prmt selectors: half A = byte tcA of prA sign-extended, half B = byte tcB of prB
					const uint32_t sel0 = tcA0 * 0x11u + tcB0 * 0x1100u + 0xC480u;
					const uint32_t sel1 = tcA1 * 0x11u + tcB1 * 0x1100u + 0xC480u;
					uint32_t dsave0 = prev_up, dsave1 = upD0;  // D(i-1, j0-1), D(i-1, j0) for row 0
					uint32_t uD0 = upD0, uP0 = upP0, uD1 = upD1, uP1 = upP1;
					uint32_t mlo0 = 0, mhi0 = 0, mlo1 = 0, mhi1 = 0;
					uint32_t smax0 = HMIN, smax1 = HMIN, even0 = HMIN, even1 = HMIN;
					uint32_t x0 = 0, x1 = 0;  // global: column j0's D of this lane's rows (C = 2)
					// the traceback nibble of a cell into the row's word (rows 0-3: lo, 4-7: hi)
					auto put_nib = [&](uint32_t &lo, uint32_t &hi, int r, uint32_t n) {
						uint32_t &w = r < 4 ? lo : hi;
						w = uint32_t(imad(int32_t(w), p.sixteen, int32_t(n)));  // on the FMA pipe
					};
					// local seeds: the row's key (D | row tag) into the step's best, two rows per max3
					auto put_seed = [&](uint32_t &best, uint32_t &even, int r, uint32_t D, uint32_t t) {
						const uint32_t k = TB == TB_ONE ? h_addk(D, p.one, t) : D;  // D | t
						if ((r & 1) == 0) even = k;
						else best = h_max3(best, even, k);
					};
					// column j0 of row r: its D and Q feed column j1 of the same row
					uint32_t c0D[R], c0Q[R];
					auto col0 = [&](int r) {
						const uint32_t old = Dl[r];
						uint32_t D0, P0, Q0;
						const uint32_t S0 = uint32_t(prmt(prA[r], prB[r], sel0));  // sign-replicating prmt
						const uint32_t key0 = cell16<GAP, LOC>(p, S0, dsave0, old, Ql[r], uD0, uP0, fl[r], D0, P0, Q0);
						if (TB == TB_ONE) put_nib(mlo0, mhi0, r, nib16<GAP>(key0, P0, Q0));
						if (SEED) put_seed(smax0, even0, r, D0, TB == TB_ONE ? uint32_t(r * C) * 0x10001u : 0u);
						if (LOC == LOC_GLOBAL && C == 2) {
							if (r == nvA - 1) x0 = (x0 & 0xFFFF0000u) | (D0 & 0x0000FFFFu);
							if (r == nvB - 1) x0 = (x0 & 0x0000FFFFu) | (D0 & 0xFFFF0000u);
						}
						dsave0 = old;
						uD0 = D0;
						uP0 = P0;
						c0D[r] = D0;
						c0Q[r] = Q0;
						if (C == 1) {
							Dl[r] = D0;
							if (GAP == GAP_AFFINE) Ql[r] = Q0;
						}
					};
					// column j1 of row r (C = 2)
					auto col1 = [&](int r) {
						uint32_t D1, P1, Q1;
						const uint32_t S1 = uint32_t(prmt(prA[r], prB[r], sel1));
						const uint32_t key1 = cell16<GAP, LOC>(p, S1, dsave1, c0D[r], c0Q[r], uD1, uP1, fl[r], D1, P1, Q1);
						if (TB == TB_ONE) put_nib(mlo1, mhi1, r, nib16<GAP>(key1, P1, Q1));
						if (SEED) put_seed(smax1, even1, r, D1, TB == TB_ONE ? uint32_t(r * C + 1) * 0x10001u : 0u);
						dsave1 = c0D[r];
						Dl[r] = D1;
						if (GAP == GAP_AFFINE) Ql[r] = Q1;
						uD1 = D1;
						uP1 = P1;
					};
					if (C == 1) {
#pragma unroll
						for (int r = 0; r < R; r++) col0(r);
					} else {
						// column j0 of row r + 1 before column j1 of row r: row r's old D (the
						// diagonal of row r + 1, column j0) is dead before column j1 of row r
						// replaces it, so the new values can take the old ones' registers
#pragma unroll
						for (int r = 0; r <= R; r++) {
							if (r < R) col0(r);
							if (r >= 1) col1(r - 1);
						}
					}
					outD0 = uD0;
					outP0 = uP0;
					outD1 = uD1;
					outP1 = uP1;
					if (write_boundary) {
						bout[j0] = make_int2(int32_t(outD0), int32_t(outP0));
						if (act1) bout[j1] = make_int2(int32_t(outD1), int32_t(outP1));
					}
					if (TB == TB_ONE) {
						// rows 0-3 of each half in mlo, 4-7 in mhi, row r at bits 4 (R - 1 - r) of the word
						if (C == 2) {
							if (mA && j0 < ctA)
								reinterpret_cast<uint2 *>(mA)[int64_t(s) * G] =
								    make_uint2(__byte_perm(mhi0, mlo0, 0x5410), __byte_perm(mhi1, mlo1, 0x5410));
							if (mB && j0 < ctB)
								reinterpret_cast<uint2 *>(mB)[int64_t(s) * G] =
								    make_uint2(__byte_perm(mhi0, mlo0, 0x7632), __byte_perm(mhi1, mlo1, 0x7632));
						} else {
							if (mA && j0 < ctA) mA[int64_t(s) * G] = __byte_perm(mhi0, mlo0, 0x5410);
							if (mB && j0 < ctB) mB[int64_t(s) * G] = __byte_perm(mhi0, mlo0, 0x7632);
						}
					}
					if (SEED) {
						// a step's columns lie inside both pairs until the shorter pair's end
						uint32_t sv = C == 2 ? h_max(smax0, smax1) : smax0;
						if (j0 + C > ctmin) {
							const uint32_t cm0 = colmask16(j0, ctA, ctB);
							sv = (smax0 & cm0) | (HMIN & ~cm0);
							if (C == 2) {
								const uint32_t cm1 = colmask16(j1, ctA, ctB);
								sv = h_max(sv, (smax1 & cm1) | (HMIN & ~cm1));
							}
						}
						seed16<TB, C>(sv, j0, lm, pos);
					}
					if (LOC == LOC_GLOBAL) {
						// D(|s|-1, |t|-1) of a half: this lane's row |s|-1 in the pass's last step
						if (q == npA - 1 && nvA >= 1 && nvA <= R && (j0 == ltA - 1 || (C == 2 && j1 == ltA - 1))) {
							uint32_t v = x0;
							if (C == 1 || j1 == ltA - 1) {
#pragma unroll
								for (int r = 0; r < R; r++)
									if (r == nvA - 1) v = Dl[r];
							}
							globA = (h_lo(v) >> 4) * 4;
							haveA = true;
						}
						if (q == npB - 1 && nvB >= 1 && nvB <= R && (j0 == ltB - 1 || (C == 2 && j1 == ltB - 1))) {
							uint32_t v = x0;
							if (C == 1 || j1 == ltB - 1) {
#pragma unroll
								for (int r = 0; r < R; r++)
									if (r == nvB - 1) v = Dl[r];
							}
							globB = (h_hi(v) >> 4) * 4;
							haveB = true;
						}
					}
				}
				prev_up = C == 2 ? upD1 : upD0;
			}
			if (SEED) {
				// fold the pass into the lane's running best (x4 tagged domain of finish_pair):
				// a later pass has larger rows, so it wins a tie of values
				const int32_t kA = h_lo(lm), kB = h_hi(lm);
				const int rsh = C == 2 ? 1 : 0;
				if (kA != -32768) {  // the lane saw a cell of the pair
					const int32_t v = (kA >> 4) * 4;
					if (v >= bestA) {
						bestA = v;
						biA = row0 + ((kA >> rsh) & 7);
						bjA = int32_t(pos & 0xffffu) + (C == 2 ? (kA & 1) : 0);
					}
				}
				if (kB != -32768) {
					const int32_t v = (kB >> 4) * 4;
					if (v >= bestB) {
						bestB = v;
						biB = row0 + ((kB >> rsh) & 7);
						bjB = int32_t(pos >> 16) + (C == 2 ? (kB & 1) : 0);
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

// Wavefront DP kernels for the batched alignment solve (sm_103a).
//
// Recurrences restated from pyalign/algorithm/solver.h (pyalign 0.4.4):
//   linear  (NW/SW)  LinearGapCostSolver::solve   solver.h:2825-2855
//   affine  (Gotoh)  AffineGapCostSolver::solve   solver.h:2970-3036
//   DTW              DynamicTimeSolver::solve     solver.h:3213-3251
// with the tie rule of Accumulator/TracingAccumulator (solver.h:1226-1427): the first
// candidate pushed wins unless a later one is strictly better; "all optimal" keeps every
// candidate equal to the maximum.  Seeds follow Local/Global/Semiglobal
// (solver.h:1980-2327).
//
// Everything runs in the "maximize" form: the host negates similarities for minimize
// problems (min f == -max(-f) exactly in IEEE arithmetic), and gap costs enter as
// negative addends.
//
// Mapping to the GPU.  A pair is solved by a group of G lanes (G = 4..32) of one warp;
// each lane owns R = 8 consecutive rows of a stripe of G*R rows and the group sweeps the
// columns of t as a skewed wavefront (lane k works on column s-k at step s).  The
// boundary (D, P) of a lane's last row travels to the next lane by __shfl_up_sync; the
// last lane writes it to a per-group scratch row that feeds the next stripe.  Per cell,
// the traceback is a 4-bit nibble (one optimal path: 2-bit D source, P-extend bit,
// Q-extend bit) or a 16-bit word (all optimal paths: every tied predecessor), stored
// as one coalesced 32-bit (or 128-bit) word per lane per step.
//
// Integer scoring runs on int32 "tagged" values: every value is scaled by 4 and the low
// two bits of each candidate carry its push priority (zero 3 > diag 2 > P/up 1 > Q/left
// 0), so a single max chain yields the value and the reference's tie winner at once.

#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace pa {

enum GapKind { GAP_LINEAR = 0, GAP_AFFINE = 1, GAP_DTW = 2, GAP_GENERAL = 3 };
enum LocKind { LOC_LOCAL = 0, LOC_GLOBAL = 1, LOC_SEMI = 2 };
enum TbKind { TB_NONE = 0, TB_ONE = 1, TB_ALL = 2 };
enum SubKind { SUB_TABLE = 0, SUB_BINARY = 1, SUB_DENSE = 2, SUB_PROFILE = 3, SUB_COLPROF = 4, SUB_SERIES = 5 };
// SUB_SERIES: S(i, j) = |x_i - y_j| of two float32 series, computed per cell; the series travel
// in the code registers as raw 32-bit words (a = x, b = y), scaled by dense_sign.

// SUB_COLPROF: per thread and letter c, the int8 scores of the thread's R rows against c,
// kept in shared memory after the table as colprof[c * BLOCK + thread] (8 bytes): one
// conflict-free 64-bit load per step replaces R table lookups (alphabets up to 32 letters).
constexpr int MAX_COLPROF = 32;

constexpr int R = 8;              // rows per lane
constexpr int BLOCK = 128;        // threads per block
constexpr int WARPS = BLOCK / 32;
constexpr int MAX_SMEM_TABLE = 64;  // alphabet size kept in shared memory

// status bits written by kernels (host turns them into errors)
constexpr int ST_BAD_CODE = 1;
constexpr int ST_TIMEOUT = 2;   // a chained stripe waited too long for the stripe above it

// Stripe-chained mode: columns a stripe publishes at a time, and the bound of one wait.
constexpr int PUB_CHUNK = 32;
constexpr int WAIT_LIMIT = 1 << 23;

constexpr int PA_MAX_SEG = 4;  // length buckets of one launch (|s| <= 128, 256, 512, more)

template <typename V>
struct DpParams {
	int32_t npairs;
	const int32_t *order;   // processing order (host sorted by cost)
	const int32_t *len_s;   // per pair
	const int32_t *len_t;
	// sequences (SUB_TABLE / SUB_BINARY)
	const uint32_t *a;
	const uint32_t *b;
	int64_t a_stride, b_stride;
	// substitution
	int32_t sub_kind;
	const V *table;         // table_rows x table_cols, prepared by the host (scaled/tagged)
	int32_t table_rows, table_cols;
	V eq, ne;               // binary, prepared
	const float *dense;     // S(k,i,j) = dense[dense_off[k] + i*dense_si + j*dense_sj]
	const int64_t *dense_off;
	int64_t dense_si, dense_sj;
	float dense_sign;       // +1 maximize, -1 minimize
	// gap addends (negative), prepared by the host
	V c_up, c_left;         // linear: vertical / horizontal step
	V c_open_s, c_ext_s;    // affine P (vertical): from D, from P
	V c_open_t, c_ext_t;    // affine Q (horizontal)
	// borders: left_D[i+1] = D(i,-1), top_D[j+1] = D(-1,j)  (i, j >= -1)
	const V *left_D;
	const V *top_D;
	const V *left_P;        // values output only: P(i,-1)
	const V *top_Q;         // values output only: Q(-1,j)
	V neg_inf;
	int32_t G;              // lanes per pair group
	// length buckets with their own group width (16-bit twin kernel): the processing order is
	// cut into nseg segments, segment k holding units seg_unit[k] .. seg_unit[k + 1] - 1 and warp
	// tasks seg_task[k] .. seg_task[k + 1] - 1 (one group of seg_G[k] lanes per unit, 32 /
	// seg_G[k] units per task); nseg = 0: one width, G, for the whole launch
	int32_t nseg;
	int32_t seg_G[PA_MAX_SEG];
	int32_t seg_unit[PA_MAX_SEG + 1];
	int32_t seg_task[PA_MAX_SEG + 1];
	int32_t slots_per_warp; // group slots of scratch per warp (32 / the narrowest width)
	int32_t key_shift;      // local seeds: key = value * 2^key_shift + j
	int32_t one, minus_one, minus_four, minus_eight, sixteen;  // IMAD multipliers (see imad)
	int32_t two, bit16;  // 2, 65536
	// outputs
	float *score;           // reference-domain score
	int32_t *seed;          // (i, j) per pair
	int32_t *has_seed;
	float out_sign;         // +1 maximize, -1 minimize
	void *masks;            // TB_ONE: uint32 words; TB_ALL: uint4
	const int64_t *mask_off;  // per pair, in store elements
	const float *best_in;   // TB_ALL + local: optimum per pair (reference domain)
	// solution values (optional): per pair layers x (ls+1) x (lt+1) floats
	float *values;
	const int64_t *val_off;
	// scratch: per group slot, 2 buffers of max_lt (D, P) pairs
	void *scratch;
	int64_t scratch_stride;  // elements per slot
	int32_t *work_counter;
	int32_t *status;
	// stripe-chained mode (units != 0): a ticket is one stripe of one pair; tickets are
	// numbered stripe-major, level_start[q] is the first ticket of stripe q (nlevels + 1
	// entries), and stripe q of the pair at rank w in the order is ticket level_start[q] + w.
	// A stripe reads the boundary row of the stripe above it once that stripe's progress
	// counter (columns finished) covers the column; the scratch rows are per pair rank.
	int32_t units;          // informational: the kernel variant decides
	int32_t ntickets;
	int32_t nlevels;
	const int32_t *level_start;
	int32_t *progress;      // per ticket, zeroed before the launch
	int4 *chain;            // per ticket: running seed of the stripes so far (value bits, i, j)
	// packed 16-bit twin kernel (dp16_kernel, pa_dp16.cuh): the extend addends (value * 16,
	// both halves), the opening / linear addends as 32-bit IMAD constants (value * 16 + tag,
	// the low half's carry folded into the high half), the sentinel and the borders as biased
	// values (value * 16 + 32768; left16[i+1] = D(i,-1), top16[j+1] = D(-1,j)); the table
	// holds value * 16 + 8
	uint32_t h_ext_s, h_ext_t, h_neg;
	uint32_t k_open_s, k_open_t, k_up, k_left;
	const uint32_t *left16;
	const uint32_t *top16;
	// indexed form: the largest code of a and of b (written by codes_max_kernel earlier in
	// the stream) and the bounds they must stay below; a launch with a code out of bounds
	// does no work and sets ST_BAD_CODE (codes_valid)
	const uint32_t *codes_max;
	uint32_t code_lim_a, code_lim_b;
};

// False (and ST_BAD_CODE set) when a code of the launch lies outside the similarity table:
// every thread reads the same two words, so a whole launch returns before any table access.
template <typename P>
__device__ __forceinline__ bool codes_valid(const P &p) {
	if (!p.codes_max) return true;
	const bool ok = p.codes_max[0] < p.code_lim_a && p.codes_max[1] < p.code_lim_b;
	if (!ok && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(p.status, ST_BAD_CODE);
	return ok;
}

__device__ __forceinline__ int32_t ld_acquire(const int32_t *a) {
	int32_t v;
	asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
	return v;
}

__device__ __forceinline__ void st_release(int32_t *a, int32_t v) {
	asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}

// Wait until *prog >= need; returns the value seen.  The wait is bounded: past WAIT_LIMIT
// polls (or once another wait gave up) it sets ST_TIMEOUT and returns INT32_MAX, so the
// kernel finishes with flagged, meaningless results instead of hanging.
static __device__ __noinline__ int32_t wait_progress(const int32_t *prog, int32_t need, int32_t *status) {
	for (int it = 0; it < WAIT_LIMIT; it++) {
		const int32_t v = ld_acquire(prog);
		if (v >= need) return v;
		if (it >= 64) {
			if ((it & 63) == 0 && (*reinterpret_cast<volatile int32_t *>(status) & ST_TIMEOUT)) return INT32_MAX;
			__nanosleep(256);
		}
	}
	atomicOr(status, ST_TIMEOUT);
	return INT32_MAX;
}

template <typename V>
__device__ __forceinline__ int32_t vbits(V x) {
	if constexpr (std::is_same<V, float>::value) return __float_as_int(x);
	else return x;
}

template <typename V>
__device__ __forceinline__ V vfrom(int32_t x) {
	if constexpr (std::is_same<V, float>::value) return __int_as_float(x);
	else return x;
}

template <typename V>
struct V2T;
template <>
struct V2T<int32_t> { typedef int2 type; };
template <>
struct V2T<float> { typedef float2 type; };

__device__ __forceinline__ int32_t vmax(int32_t a, int32_t b) { return max(a, b); }
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }

template <typename V>
__device__ __forceinline__ float to_ref(V x, bool tagged, float sign);

template <>
__device__ __forceinline__ float to_ref<int32_t>(int32_t x, bool tagged, float sign) {
	if (x < -(1 << 28)) return -INFINITY * sign;
	const int32_t v = tagged ? (x >> 2) : x;
	return float(v) * sign;
}

template <>
__device__ __forceinline__ float to_ref<float>(float x, bool, float sign) {
	return x * sign;
}

// Substitution value of (query code qa at row i, subject code tb at column j).
template <typename V>
struct SubCtx {
	const V *table;  // shared or global
	int32_t cols;
	V eq, ne;
};

// prmt.b32 in its default mode: byte k of the result is source byte sel[4k+2:4k] of {b, a},
// sign-replicated when bit 4k+3 is set.  Used to read an int8 substitution profile.
__device__ __forceinline__ int32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
	uint32_t d;
	asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
	return int32_t(d);
}

// Selector that extracts byte t (0..7) of {hi, lo} sign-extended to 32 bits:
// nibbles t, t|8, t|8, t|8, i.e. t * 0x1111 + 0x8880 for t < 8.
__device__ __forceinline__ uint32_t sext_selector(uint32_t t) { return t * 0x1111u + 0x8880u; }

// max(a + b, c) in one DPX instruction.
__device__ __forceinline__ int32_t addmax(int32_t a, int32_t b, int32_t c) { return __viaddmax_s32(a, b, c); }

// a * b + c on the FMA pipe.  Callers pass multipliers that come from kernel parameters, so
// the compiler keeps the IMAD instead of turning it into an ALU add/shift: the DP cell
// update is ALU-pipe bound and this moves part of it to the otherwise idle FMA pipe.
__device__ __forceinline__ int32_t imad(int32_t a, int32_t b, int32_t c) {
	int32_t d;
	asm("mad.lo.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

// Asynchronous 16-byte global -> shared copies (cp.async): commit closes a group, wait<N>
// returns once at most N of this thread's groups are still in flight.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
	const uint32_t sa = uint32_t(__cvta_generic_to_shared(smem));
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Dense S with stride 1 along s: each lane keeps the next DENSE_RING - 1 columns of its 8
// rows in flight in a shared-memory ring (2 x 16 bytes per column), DENSE_RING * 32 bytes per
// thread at the start of the dynamic shared memory.
constexpr int DENSE_RING = 4;

// 0xffffffff when a > b, else 0.
__device__ __forceinline__ uint32_t gt_mask(int32_t a, int32_t b) {
	uint32_t d;
	asm("set.gt.u32.s32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

// 0xffffffff when a == b, else 0.
__device__ __forceinline__ uint32_t eq_mask(int32_t a, int32_t b) {
	uint32_t d;
	asm("set.eq.u32.s32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

// End of a pair (group mode) or of a stripe ticket (stripe-chained mode): reduce the seed
// candidates over the group, fold in and pass on the seed of the stripes above (chained),
// and -- for the last stripe -- write the score and the traceback seed (solver.h:2035-2124,
// 2174-2220, 2266-2326).
template <typename V, int LOC, int TB, bool TAG, bool CHAIN>
__device__ __forceinline__ void finish_pair(const DpParams<V> &p, int G, int sub, int pair, int ls, int lt, bool empty,
                                            int npass, int q_lo, int prod, int base, V NEG, V l_best, int l_bi,
                                            int l_bj, V row_best, int row_bj, V col_best, int col_bi, V glob,
                                            bool have_glob) {
	// ---- group reductions and outputs
	if (LOC == LOC_LOCAL) {
		for (int o = 1; o < G; o <<= 1) {
			const V ov = __shfl_xor_sync(0xffffffffu, l_best, o, G);
			const int oi = __shfl_xor_sync(0xffffffffu, l_bi, o, G);
			const int oj = __shfl_xor_sync(0xffffffffu, l_bj, o, G);
			const bool take = ov > l_best || (ov == l_best && (oi > l_bi || (oi == l_bi && oj > l_bj)));
			if (take) { l_best = ov; l_bi = oi; l_bj = oj; }
		}
	} else if (LOC == LOC_SEMI) {
		for (int o = 1; o < G; o <<= 1) {
			const V orv = __shfl_xor_sync(0xffffffffu, row_best, o, G);
			const int orj = __shfl_xor_sync(0xffffffffu, row_bj, o, G);
			if (orj >= 0 && (row_bj < 0 || orv > row_best)) { row_best = orv; row_bj = orj; }
			const V ocv = __shfl_xor_sync(0xffffffffu, col_best, o, G);
			const int oci = __shfl_xor_sync(0xffffffffu, col_bi, o, G);
			if (oci >= 0 && (col_bi < 0 || ocv > col_best || (ocv == col_best && oci < col_bi))) {
				col_best = ocv; col_bi = oci;
			}
		}
	} else {
		for (int o = 1; o < G; o <<= 1) {
			const V og = __shfl_xor_sync(0xffffffffu, glob, o, G);
			const int oh = __shfl_xor_sync(0xffffffffu, int(have_glob), o, G);
			if (oh && !have_glob) { glob = og; have_glob = true; }
		}
	}

	// ---- stripe-chained: fold in the seed of the stripes above, pass it on
	bool last_unit = true;
	if (CHAIN && pair >= 0) {
		last_unit = q_lo >= npass - 1;
		if (q_lo > 0 && (LOC == LOC_LOCAL || LOC == LOC_SEMI) && !(LOC == LOC_LOCAL && TB == TB_ALL)) {
			const int32_t *pi = p.progress + prod;
			if (ld_acquire(pi) < lt) wait_progress(pi, lt, p.status);
			const int4 rc = __ldcg(p.chain + prod);
			const V ov = vfrom<V>(rc.x);
			if (LOC == LOC_LOCAL) {
				if (ov > l_best || (ov == l_best && (rc.y > l_bi || (rc.y == l_bi && rc.z > l_bj)))) {
					l_best = ov; l_bi = rc.y; l_bj = rc.z;
				}
			} else if (rc.y >= 0 && (col_bi < 0 || ov > col_best || (ov == col_best && rc.y < col_bi))) {
				col_best = ov; col_bi = rc.y;
			}
		}
		if (!last_unit && sub == G - 1) {
			int4 rc;
			if (LOC == LOC_LOCAL) rc = make_int4(vbits(l_best), l_bi, l_bj, 0);
			else rc = make_int4(vbits(col_best), col_bi, -1, 0);
			p.chain[base] = rc;
			st_release(p.progress + base, lt);  // every column, and the record
		}
	}

	if (sub == 0 && pair >= 0 && last_unit) {
		int si = -1, sj = -1, has = 0;
		float sc = -INFINITY * p.out_sign;
		if (!empty) {
			if (LOC == LOC_LOCAL) {
				if (TB == TB_ALL) {
					has = 1;
					sc = p.best_in[pair];
				} else if (l_best > NEG) {
					has = 1; si = l_bi; sj = l_bj;
					sc = to_ref(l_best, TAG, p.out_sign);
				}
			} else if (LOC == LOC_SEMI) {
				has = 1;
				if (row_bj >= 0 && (col_bi < 0 || !(col_best > row_best))) {
					si = ls - 1; sj = row_bj; sc = to_ref(row_best, TAG, p.out_sign);
				} else {
					si = col_bi; sj = lt - 1; sc = to_ref(col_best, TAG, p.out_sign);
				}
			} else {
				has = 1; si = ls - 1; sj = lt - 1;
				sc = to_ref(glob, TAG, p.out_sign);
			}
		} else {
			// no cells: the seed is a border cell or does not exist
			if (LOC == LOC_GLOBAL) {
				has = 1; si = ls - 1; sj = lt - 1;
				const V x = ls == 0 ? p.top_D[lt] : p.left_D[ls];
				sc = to_ref(x, TAG, p.out_sign);
			} else if (LOC == LOC_SEMI) {
				// Optima over D(ls-1, 0..lt-1) then D(0..ls-1, lt-1) (solver.h:2284-2292)
				V b = NEG;
				for (int jj = 0; jj < lt; jj++) {
					const V x = p.top_D[jj + 1];
					if (x > b) { b = x; si = ls - 1; sj = jj; }
				}
				for (int ii = 0; ii < ls; ii++) {
					const V x = p.left_D[ii + 1];
					if (x > b) { b = x; si = ii; sj = lt - 1; }
				}
				if (b > NEG) { has = 1; sc = to_ref(b, TAG, p.out_sign); }
			}
		}
		p.score[pair] = sc;
		p.seed[2 * pair] = si;
		p.seed[2 * pair + 1] = sj;
		p.has_seed[pair] = has;
	}
}

template <typename V, int GAP, int LOC, int TB, bool VALS, bool CHAIN>
__global__ void __launch_bounds__(BLOCK, 4) dp_kernel(DpParams<V> p) {
	constexpr bool ISINT = std::is_same<V, int32_t>::value;
	constexpr bool TAG = ISINT && TB != TB_ALL;  // int32 tagged values
	constexpr bool KEYSEED = TAG && TB == TB_ONE && LOC == LOC_LOCAL;  // packed (value, j) seed keys
	typedef typename V2T<V>::type V2;
	if (!codes_valid(p)) return;

	extern __shared__ __align__(16) unsigned char smem_raw[];
	V *stab = reinterpret_cast<V *>(smem_raw);
	const bool table_in_smem = (p.sub_kind == SUB_TABLE || p.sub_kind == SUB_PROFILE) &&
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
	const int sub = lane % G;          // lane within the group
	const int grp = lane / G;          // group within the warp
	const int gpw = 32 / G;            // groups per warp
	const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int slot = warp_global * gpw + grp;
	const int64_t half = p.scratch_stride / 2;
	const V NEG = p.neg_inf;
	const int rpp = G * R;  // rows per pass
	const int sub_kind = p.sub_kind;
	constexpr bool units = CHAIN;  // stripe-chained mode (G == 32)
	const int ntickets = units ? p.ntickets : p.npairs;

	for (;;) {
		int base = 0;
		if (lane == 0) base = atomicAdd(p.work_counter, gpw);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= ntickets) break;
		// group mode: the pair at rank base + grp, all of its stripes.  Stripe-chained mode:
		// stripe q_lo of the pair at rank w, waiting on ticket prod (stripe q_lo - 1).
		int w = base + grp, q_lo = 0, prod = -1;
		if constexpr (units) {
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
		V2 *scr = reinterpret_cast<V2 *>(p.scratch) + int64_t(units ? w : slot) * p.scratch_stride;
		const int pair = w < p.npairs ? p.order[w] : -1;
		const int ls = pair >= 0 ? p.len_s[pair] : 0;
		const int lt = pair >= 0 ? p.len_t[pair] : 0;
		const bool empty = ls == 0 || lt == 0;
		const int npass = empty ? 0 : (ls + rpp - 1) / rpp;
		const int nsteps_pair = lt + G - 1;
		int wpass = npass, wsteps = empty ? 0 : nsteps_pair;
		for (int o = 16; o > 0; o >>= 1) {
			wpass = max(wpass, __shfl_xor_sync(0xffffffffu, wpass, o));
			wsteps = max(wsteps, __shfl_xor_sync(0xffffffffu, wsteps, o));
		}

		const uint32_t *arow = p.a ? p.a + int64_t(pair < 0 ? 0 : pair) * p.a_stride : nullptr;
		const uint32_t *brow = p.b ? p.b + int64_t(pair < 0 ? 0 : pair) * p.b_stride : nullptr;
		const float *drow = p.dense ? p.dense + (pair >= 0 ? p.dense_off[pair] : 0) : nullptr;
		const V best_in = (TB == TB_ALL && LOC == LOC_LOCAL && pair >= 0) ? V(p.best_in[pair] * p.out_sign) : V(0);
		float *vals = (VALS && pair >= 0) ? p.values + p.val_off[pair] : nullptr;
		const int64_t lstride = int64_t(lt + 1);
		const int64_t layer_sz = int64_t(ls + 1) * lstride;

		// --- solution values: borders (solver.h:2806-2814, 2918-2967, 3116-3125, 3205-3210)
		if (VALS && vals && q_lo == 0) {
			for (int j = sub - 1; j < lt; j += G) {
				vals[j + 1] = to_ref(p.top_D[j + 1], TAG, p.out_sign);
				if (GAP == GAP_AFFINE) {
					vals[layer_sz + (j + 1)] = (j < 0) ? to_ref(p.left_P[0], TAG, p.out_sign) : -INFINITY * p.out_sign;
					vals[2 * layer_sz + (j + 1)] = to_ref(p.top_Q[j + 1], TAG, p.out_sign);
				}
			}
			for (int i = sub; i < ls; i += G) {
				vals[int64_t(i + 1) * lstride] = to_ref(p.left_D[i + 1], TAG, p.out_sign);
				if (GAP == GAP_AFFINE) {
					vals[layer_sz + int64_t(i + 1) * lstride] = to_ref(p.left_P[i + 1], TAG, p.out_sign);
					vals[2 * layer_sz + int64_t(i + 1) * lstride] = -INFINITY * p.out_sign;
				}
			}
		}

		// seed tracking state
		V l_best = NEG;              // local: best value of this lane
		int l_bi = -1, l_bj = -1;
		V row_best = NEG;            // semiglobal: last row (first max in ascending j)
		int row_bj = -1;
		V col_best = NEG;            // semiglobal: last column (first max in ascending i)
		int col_bi = -1;
		V glob = NEG;                // global: D(ls-1, lt-1)
		bool have_glob = false;

		const int q_hi = units ? min(q_lo + 1, npass) : wpass;
		for (int q = q_lo; q < q_hi; q++) {
			const bool pass_active = q < npass;
			const int row0 = q * rpp + sub * R;
			const int nvalid = ls - row0;  // rows of this lane that are < ls (may be <= 0 or >= R)
			const V2 *bin = scr + (q & 1) * half;
			V2 *bout = scr + ((q + 1) & 1) * half;
			const bool write_boundary = sub == G - 1 && q + 1 < npass;
			// stripe-chained: the boundary row comes from another warp, column by column
			const int32_t *prog_in = (units && q > 0) ? p.progress + prod : nullptr;
			int32_t avail = 0;        // columns of bin known to be written
			int pub_next = PUB_CHUNK;  // next progress value to publish
			// lane 0: (D, P) above the next column, read one step ahead -- the top border in the
			// first stripe, else the boundary row of the stripe above
			V2 bnext;
			bnext.x = NEG;
			bnext.y = NEG;
			if (sub == 0 && pass_active) {
				if (q == 0) {
					bnext.x = p.top_D[1];
				} else if (units) {
					avail = wait_progress(prog_in, 1, p.status);
					bnext = __ldcg(bin);
				} else {
					bnext = bin[0];  // group mode: written by this warp's last lane in the previous pass
				}
			}

			// query codes, and the int8 substitution profile of each row (SUB_PROFILE)
			uint32_t qa[R];
			uint32_t plo[R], phi[R];
#pragma unroll
			for (int r = 0; r < R; r++) {
				const int i = row0 + r;
				qa[r] = (pass_active && i < ls && arow) ? arow[i] : 0u;
				plo[r] = phi[r] = 0u;
			}
			if (sub_kind == SUB_COLPROF) {
				const int cols = p.table_cols;
				for (int c = 0; c < cols; c++) {
					uint32_t lo = 0, hi = 0;
#pragma unroll
					for (int r = 0; r < R; r++) {
						const uint32_t byte = uint32_t(int32_t(tab[qa[r] * cols + c])) & 0xffu;
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
						const uint32_t byte = uint32_t(int32_t(tab[qa[r] * cols + c])) & 0xffu;
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
			// (D, P) of this lane's last row as seen by the next lane; column -1 initially
			V outD = Dl[R - 1], outP = NEG;
			V prev_up = (pass_active && row0 <= ls) ? p.left_D[row0] : NEG;  // D(row0-1, -1)

			// best cell per row for local one-optimal seeds (solver.h:2048-2056)
			constexpr int NB = (TB == TB_ONE && LOC == LOC_LOCAL) ? R : 1;
			V bv[NB];
			int bj[NB];
#pragma unroll
			for (int r = 0; r < NB; r++) { bv[r] = KEYSEED ? V(-1) : NEG; bj[r] = -1; }
			const int kshift = p.key_shift;
			const int kmul = 1 << kshift;
			const bool last_row_lane = pass_active && nvalid >= 1 && nvalid <= R;
			const int r_last = nvalid - 1;

			uint32_t tnext = (pass_active && brow) ? brow[0] : 0u;  // code of column 0 (lt >= 1 here)
			// dense S with stride 1 along s: a lane whose 8 rows all lie in the pair reads them as
			// two 16-byte loads, one column ahead of its use (drow + row0 + j * sj)
			const bool dvec = sub_kind == SUB_DENSE && pass_active && nvalid >= R && p.dense_si == 1 &&
			                  (p.dense_sj & 3) == 0 && ((reinterpret_cast<uintptr_t>(drow) & 15) == 0);
			const float *dcol = dvec ? drow + row0 : nullptr;
			// column jj's 8 rows into ring slot jj % DENSE_RING, one commit group per column (an
			// empty group past the last column keeps the count)
			float4 *ring = reinterpret_cast<float4 *>(smem_raw) + threadIdx.x * (2 * DENSE_RING);
			auto fetch = [&](int jj) {
				if (jj < lt) {
					const float *src = dcol + int64_t(jj) * p.dense_sj;
					float4 *dst = ring + 2 * (jj & (DENSE_RING - 1));
					cp_async16(dst, src);
					cp_async16(dst + 1, src + 4);
				}
				cp_async_commit();
			};
			if (dvec)
				for (int k = 0; k < DENSE_RING - 1; k++) fetch(k);
			// this lane's traceback word of step s is mrow[s * G] (hoisted out of the step loop)
			uint32_t *mrow1 = nullptr;
			uint4 *mrow4 = nullptr;
			if (TB == TB_ONE && pass_active)
				mrow1 = reinterpret_cast<uint32_t *>(p.masks) + p.mask_off[pair] + int64_t(q) * nsteps_pair * G + sub;
			if (TB == TB_ALL && pass_active)
				mrow4 = reinterpret_cast<uint4 *>(p.masks) + p.mask_off[pair] + int64_t(q) * nsteps_pair * G + sub;
			for (int s = 0; s < wsteps; s++) {
				const int j = s - sub;
				V upD = __shfl_up_sync(0xffffffffu, outD, 1, G);
				V upP = __shfl_up_sync(0xffffffffu, outP, 1, G);
				const bool act = pass_active && j >= 0 && j < lt;
				const uint32_t tcode = tnext;
				if (act && brow && j + 1 < lt) tnext = brow[j + 1];
				if (sub == 0 && act) {
					upD = bnext.x;
					upP = bnext.y;
					if (j + 1 < lt) {  // prefetch the next column's
						if (q == 0) {
							bnext.x = p.top_D[j + 2];
						} else if constexpr (units) {
							if (avail < j + 2) avail = wait_progress(prog_in, j + 2, p.status);
							bnext = __ldcg(bin + j + 1);
						} else {
							bnext = bin[j + 1];
						}
					}
				}
				if (act) {
					// substitution values of the R rows at column j
					V S[R];
					if (sub_kind == SUB_COLPROF) {
						const uint2 pr = colprof[tcode * BLOCK + threadIdx.x];
#pragma unroll
						for (int r = 0; r < R; r++) S[r] = V(prmt(pr.x, pr.y, sext_selector(uint32_t(r))));
					} else if (sub_kind == SUB_PROFILE) {
						const uint32_t sel = sext_selector(tcode);
#pragma unroll
						for (int r = 0; r < R; r++) S[r] = V(prmt(plo[r], phi[r], sel));
					} else if (sub_kind == SUB_BINARY) {
#pragma unroll
						for (int r = 0; r < R; r++) S[r] = (qa[r] == tcode) ? p.eq : p.ne;
					} else if (sub_kind == SUB_TABLE) {
#pragma unroll
						for (int r = 0; r < R; r++) S[r] = tab[qa[r] * p.table_cols + tcode];
					} else if (sub_kind == SUB_SERIES) {
						const float yj = __int_as_float(int(tcode));
#pragma unroll
						for (int r = 0; r < R; r++) S[r] = V(fabsf(__int_as_float(int(qa[r])) - yj) * p.dense_sign);
					} else if (dvec) {
						// column j's group is complete once at most DENSE_RING - 2 newer ones remain;
						// the refill goes to the slot read in the previous step
						cp_async_wait<DENSE_RING - 2>();
						const float4 dn0 = ring[2 * (j & (DENSE_RING - 1))], dn1 = ring[2 * (j & (DENSE_RING - 1)) + 1];
						fetch(j + DENSE_RING - 1);
						S[0] = V(dn0.x * p.dense_sign);
						S[1] = V(dn0.y * p.dense_sign);
						S[2] = V(dn0.z * p.dense_sign);
						S[3] = V(dn0.w * p.dense_sign);
						S[4] = V(dn1.x * p.dense_sign);
						S[5] = V(dn1.y * p.dense_sign);
						S[6] = V(dn1.z * p.dense_sign);
						S[7] = V(dn1.w * p.dense_sign);
					} else {
#pragma unroll
						for (int r = 0; r < R; r++) {
							const int i = min(row0 + r, ls - 1);
							S[r] = V(drow[int64_t(i) * p.dense_si + int64_t(j) * p.dense_sj] * p.dense_sign);
						}
					}

					uint32_t mword = 0;  // one-optimal traceback nibbles of the R rows
					uint32_t mall[4] = {0, 0, 0, 0};
					V dsave = prev_up;  // D(i-1, j-1) for the first row
					V uD = upD, uP = upP;
#pragma unroll
					for (int r = 0; r < R; r++) {
						const V old = Dl[r];
						V D, P = NEG, Q = NEG;
						if (TAG) {
							// ---- int32 tagged: one max chain gives value and tie winner
							int32_t key;
							if (GAP == GAP_AFFINE) {
								// P = max(D(i-1,j) - open, P(i-1,j) - extend); extend only when strictly better
								const V oP = imad(uD, p.one, p.c_open_s);
								P = addmax(uP, p.c_ext_s, oP);
								const V oQ = imad(old, p.one, p.c_open_t);
								Q = addmax(Ql[r], p.c_ext_t, oQ);
								key = addmax(dsave, S[r], vmax(P, Q));
								if (LOC == LOC_LOCAL) key = vmax(key, 3);
								const int32_t code = key & 3;
								D = imad(code, p.minus_one, key);
								if (TB == TB_ONE) {
									// nibble code | P-extend << 2 | Q-extend << 3, row r at bits 4(R-1-r)
									int32_t nb = imad(int32_t(gt_mask(P, oP)), p.minus_four, code);
									nb = imad(int32_t(gt_mask(Q, oQ)), p.minus_eight, nb);
									mword = uint32_t(imad(int32_t(mword), p.sixteen, nb));
								}
							} else if (GAP == GAP_LINEAR) {
								key = addmax(dsave, S[r], addmax(uD, p.c_up, imad(old, p.one, p.c_left)));
								if (LOC == LOC_LOCAL) key = vmax(key, 3);
								const int32_t code = key & 3;
								D = imad(code, p.minus_one, key);
								if (TB == TB_ONE) mword = uint32_t(imad(int32_t(mword), p.sixteen, code));
							} else {  // DTW
								key = addmax(dsave, 2, addmax(uD, 1, old));
								const int32_t code = key & 3;
								D = imad(code, p.minus_one, key) + S[r];
								if (TB == TB_ONE) mword = uint32_t(imad(int32_t(mword), p.sixteen, code));
							}
						} else {
							// ---- explicit compares (float, or int32 for all-optimal masks)
							uint32_t cell = 0;
							V best;
							int code;
							if constexpr (ISINT && TB == TB_ALL && GAP == GAP_AFFINE) {
								// all-optimal int32: the maxima by max instructions, the eight tie
								// flags as 0 / -1 masks folded into the cell word by IMAD (FMA
								// pipe), highest bit first: nacc = -(flag bits)
								const V oP = imad(uD, p.one, p.c_open_s), eP = imad(uP, p.one, p.c_ext_s);
								P = vmax(oP, eP);
								const V oQ = imad(old, p.one, p.c_open_t), eQ = imad(Ql[r], p.one, p.c_ext_t);
								Q = vmax(oQ, eQ);
								const V dg = imad(S[r], p.one, dsave);
								best = vmax(vmax(dg, P), Q);
								if (LOC == LOC_LOCAL) best = vmax(best, V(0));
								D = best;
								int32_t nacc = int32_t(eq_mask(eQ, Q));
								nacc = imad(nacc, p.two, int32_t(eq_mask(oQ, Q)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(eP, P)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(oP, P)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(Q, best)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(P, best)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(dg, best)));
								nacc = imad(nacc, p.two, LOC == LOC_LOCAL ? int32_t(eq_mask(best, 0)) : 0);
								cell = uint32_t(imad(nacc, p.minus_one, 0));
								code = 0;
							} else if (GAP == GAP_AFFINE) {
								const V oP = uD + p.c_open_s, eP = uP + p.c_ext_s;
								const bool bP = eP > oP;
								P = bP ? eP : oP;
								const V oQ = old + p.c_open_t, eQ = Ql[r] + p.c_ext_t;
								const bool bQ = eQ > oQ;
								Q = bQ ? eQ : oQ;
								const V dg = dsave + S[r];
								if (LOC == LOC_LOCAL) {
									best = V(0); code = 3;
									if (dg > best) { best = dg; code = 2; }
								} else {
									best = dg; code = 2;
								}
								if (P > best) { best = P; code = 1; }
								if (Q > best) { best = Q; code = 0; }
								D = best;
								if (TB == TB_ONE) {
									mword = (mword << 4) | uint32_t(code) | (bP ? 4u : 0u) | (bQ ? 8u : 0u);
								} else if (TB == TB_ALL) {
									cell = (LOC == LOC_LOCAL && best == V(0) ? 1u : 0u) | (dg == best ? 2u : 0u) |
									       (P == best ? 4u : 0u) | (Q == best ? 8u : 0u) |
									       (oP == P ? 16u : 0u) | (eP == P ? 32u : 0u) |
									       (oQ == Q ? 64u : 0u) | (eQ == Q ? 128u : 0u);
								}
							} else if constexpr (ISINT && TB == TB_ALL && GAP == GAP_LINEAR) {
								// all-optimal int32, linear gaps: as the affine form above
								const V dg = imad(S[r], p.one, dsave);
								const V up = imad(uD, p.one, p.c_up);
								const V lf = imad(old, p.one, p.c_left);
								best = vmax(vmax(dg, up), lf);
								if (LOC == LOC_LOCAL) best = vmax(best, V(0));
								D = best;
								int32_t nacc = int32_t(eq_mask(lf, best));
								nacc = imad(nacc, p.two, int32_t(eq_mask(up, best)));
								nacc = imad(nacc, p.two, int32_t(eq_mask(dg, best)));
								nacc = imad(nacc, p.two, LOC == LOC_LOCAL ? int32_t(eq_mask(best, 0)) : 0);
								cell = uint32_t(imad(nacc, p.minus_one, 0));
								code = 0;
							} else if (GAP == GAP_LINEAR) {
								const V dg = dsave + S[r];
								const V up = uD + p.c_up;
								const V lf = old + p.c_left;
								if (LOC == LOC_LOCAL) {
									best = V(0); code = 3;
									if (dg > best) { best = dg; code = 2; }
								} else {
									best = dg; code = 2;
								}
								if (up > best) { best = up; code = 1; }
								if (lf > best) { best = lf; code = 0; }
								D = best;
								if (TB == TB_ONE) {
									mword = (mword << 4) | uint32_t(code);
								} else if (TB == TB_ALL) {
									cell = (LOC == LOC_LOCAL && best == V(0) ? 1u : 0u) | (dg == best ? 2u : 0u) |
									       (up == best ? 4u : 0u) | (lf == best ? 8u : 0u);
								}
							} else {  // DTW
								best = dsave; code = 2;
								if (uD > best) { best = uD; code = 1; }
								if (old > best) { best = old; code = 0; }
								if (TB == TB_ALL) {
									cell = (dsave == best ? 2u : 0u) | (uD == best ? 4u : 0u) | (old == best ? 8u : 0u);
								}
								D = best + S[r];
								if (TB == TB_ONE) mword = (mword << 4) | uint32_t(code);
							}
							if (TB == TB_ALL) {
								if (LOC == LOC_LOCAL && r < nvalid && best_in > V(0) && D == best_in) cell |= 256u;
								// the odd row's cell into the high half by IMAD (FMA pipe): the
								// halves are disjoint, so the add is the OR
								if (r & 1) mall[r >> 1] = uint32_t(imad(int32_t(cell), p.bit16, int32_t(mall[r >> 1])));
								else mall[r >> 1] |= cell;
							}
						}

						// seeds
						if (LOC == LOC_LOCAL) {
							if constexpr (KEYSEED) {
								// D >= 0 here; key = D * 2^kshift + j orders by value, then j
								bv[r] = vmax(bv[r], V(D * kmul + j));
							} else if (TB == TB_ONE) {
								if (r < nvalid && D >= bv[r]) { bv[r] = D; bj[r] = j; }
							} else if (TB == TB_NONE) {
								if (r < nvalid) l_best = vmax(l_best, D);
							}
						}
						if (VALS && vals && r < nvalid) {
							const int64_t c = int64_t(row0 + r + 1) * lstride + (j + 1);
							vals[c] = to_ref(D, TAG, p.out_sign);
							if (GAP == GAP_AFFINE) {
								vals[layer_sz + c] = to_ref(P, TAG, p.out_sign);
								vals[2 * layer_sz + c] = to_ref(Q, TAG, p.out_sign);
							}
						}
						dsave = old;
						Dl[r] = D;
						if (GAP == GAP_AFFINE) Ql[r] = Q;
						uD = D;
						uP = P;
					}
					outD = uD;
					outP = uP;
					if (write_boundary) {
						bout[j] = V2{outD, outP};
						if (units && j + 1 == pub_next) {  // columns < j + 1 are written
							if (j + 1 < lt) st_release(p.progress + base, j + 1);
							pub_next += PUB_CHUNK;
						}
					}

					if (TB == TB_ONE) {
						mrow1[s * G] = mword;
					} else if (TB == TB_ALL) {
						mrow4[s * G] = make_uint4(mall[0], mall[1], mall[2], mall[3]);
					}

					if (LOC == LOC_SEMI || LOC == LOC_GLOBAL) {
						if (last_row_lane && q == npass - 1) {
							V x = Dl[0];
#pragma unroll
							for (int r = 1; r < R; r++)
								if (r == r_last) x = Dl[r];
							if (LOC == LOC_SEMI) {
								if (x > row_best) { row_best = x; row_bj = j; }
							} else if (j == lt - 1) {
								glob = x;
								have_glob = true;
							}
						}
						if (LOC == LOC_SEMI && j == lt - 1) {
#pragma unroll
							for (int r = 0; r < R; r++)
								if (r < nvalid && Dl[r] > col_best) { col_best = Dl[r]; col_bi = row0 + r; }
						}
					}
				}
				prev_up = upD;
			}
			if (TB == TB_ONE && LOC == LOC_LOCAL) {
				// fold the per-row bests of valid rows: larger value, then larger i (rows
				// ascend), then the row's own largest j (solver.h:2048-2056 scans i, j
				// descending with strict replacement)
#pragma unroll
				for (int r = 0; r < NB; r++) {
					if (r >= nvalid) continue;
					V v;
					int jj;
					if constexpr (KEYSEED) {
						if (bv[r] < 0) continue;
						v = bv[r] >> kshift;
						jj = bv[r] & (kmul - 1);
					} else {
						if (bj[r] < 0) continue;
						v = bv[r];
						jj = bj[r];
					}
					if (v >= l_best) { l_best = v; l_bi = row0 + r; l_bj = jj; }
				}
			}
			__syncwarp();
		}

		finish_pair<V, LOC, TB, TAG, CHAIN>(p, G, sub, pair, ls, lt, empty, npass, q_lo, prod, base, NEG, l_best, l_bi,
		                                    l_bj, row_best, row_bj, col_best, col_bi, glob, have_glob);
	}
}

// Largest code in a batch of sequences (host validation of the indexed form,
// factory.h:602-614, done on the device for device-resident inputs).
__global__ void codes_max_kernel(const uint32_t *x, int64_t n, uint32_t *out);

// ---------------------------------------------------------------------------------------
// Traceback walk for one optimal path (TracebackIterators<false>::Iterator::next,
// solver.h:1497-1536), one thread per pair, over the 4-bit masks.  The walk emits the
// alignment map: a point is an edge when the next step moves diagonally
// (path_compressor, solver.h:809-847); P/Q steps jump to the gap-open cell.
struct WalkParams {
	int32_t npairs;  // pairs pair0 .. pair0 + npairs - 1, a warp each
	int32_t pair0;
	const int32_t *len_s;
	const int32_t *len_t;
	const int32_t *seed;
	const int32_t *has_seed;
	const uint32_t *masks;
	const int64_t *mask_off;
	int32_t G;
	int32_t cols;   // columns per lane step of the DP that wrote the masks (1: dp_kernel, 2: dp2_kernel)
	int32_t fmt16;  // 1: nibbles of dp16_kernel (code in bits 2-3, P-open bit 0, Q-open bit 1)
	const int8_t *pair_G;  // per pair group width of a launch with length buckets (else G)
	int32_t rows4;  // 1: records of dp16b_kernel (4 rows x 4 columns per lane step, cols = 4)
	const int32_t *status;  // the DP's status: a launch that flagged ST_BAD_CODE has no masks
	int32_t gap;    // GapKind
	int32_t local;  // 1: stop at value-0 cells
	int32_t *maps;  // min(ls, lt) per pair at map_off
	const int64_t *map_off;
	int32_t *paths;  // optional: 2 ints per point, ls + lt + 2 points per pair at path_off
	const int64_t *path_off;
	int32_t *path_len;
};

__global__ void walk_kernel(WalkParams p);

}  // namespace pa

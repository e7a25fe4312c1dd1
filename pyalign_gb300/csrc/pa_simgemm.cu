// Ragged batched similarity product on the 5th-generation tensor cores (sm_103a):
//   St[k][j][i] = beta + alpha * <Et[k][j], Es[k][i]>   for j < len_t[k], i < len_s[k]
// BF16 operands, FP32 accumulation in tensor memory.  This is the similarity matrix of
// per-token embeddings that the dense (MatrixForm) alignment problems read, written as S^T
// so that the DP kernel reads it with stride 1 along s.
//
// One CTA of 128 threads computes a 128 x 128 tile of one pair at a time (persistent grid,
// tiles numbered pair by pair through tile_start).  Per K chunk of up to 128 elements the
// threads copy both operand tiles into shared memory in the canonical K-major layout without
// swizzle -- 8-row x 16-byte core matrices, 128 bytes apart along K (leading byte offset)
// and (K chunk / 8) * 128 bytes apart along M/N (stride byte offset) -- and one thread
// issues K/16 tcgen05.mma (M = 128, N = 128, K = 16) into a 128-column TMEM accumulator and
// commits them to an mbarrier.  The four warps then read their 32 TMEM lanes (tile rows)
// with tcgen05.ld and store the rows that fall inside the pair.  Three CTAs share an SM
// (64 KB of operands each, 3 x 128 of the 512 TMEM columns), so one CTA's copies overlap
// another's MMAs and epilogue.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is reached through the runtime)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include "../../include/pyalign_gb300.h"

namespace {

constexpr int TM = 128;           // tile rows (t positions): MMA M, TMEM lanes
constexpr int TN = 128;           // tile columns (s positions): MMA N, TMEM columns
constexpr int KC = 128;           // K elements staged per chunk
constexpr int THREADS = 128;
constexpr int OPBYTES = TM * KC * 2;             // one operand tile: 32 KB
constexpr int SMEM_BYTES = 2 * OPBYTES + 1024;   // operands + barrier/TMEM slot, 1 KB aligned
constexpr int ST_TIMEOUT = 2;

struct SimParams {
	const __nv_bfloat16 *Es;  // (batch, n_s, dim)
	const __nv_bfloat16 *Et;  // (batch, n_t, dim)
	int64_t n_s, n_t;
	int32_t dim;
	const int32_t *len_s, *len_t;  // device
	const int32_t *tile_start;     // device, batch + 1
	int64_t batch, total_tiles;
	float *St;
	int64_t pitch_pair, pitch_row;
	float alpha, beta;  // epilogue: beta + alpha * dot (1 - cos for DTW distances)
	int32_t *status;
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, leading and stride byte offsets (all >> 4),
// descriptor version 1 at bit 46, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
	return uint64_t((addr >> 4) & 0x3fff) | (uint64_t((lbo >> 4) & 0x3fff) << 16) |
	       (uint64_t((sbo >> 4) & 0x3fff) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(TN >> 3) << 17) | (uint32_t(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
	    "l"(da), "l"(db), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Bounded wait for the mbarrier phase with the given parity: false after about two seconds.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
	const long long t0 = clock64();
	for (;;) {
		uint32_t done;
		asm volatile(
		    "{\n\t.reg .pred p;\n\t"
		    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}\n"
		    : "=r"(done)
		    : "r"(bar), "r"(parity)
		    : "memory");
		if (done) return true;
		if (clock64() - t0 > (1ll << 32)) return false;
	}
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
	    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
	    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
	    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
	      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
	      "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
	      "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
	    : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Copy rows [r0, r0 + 128) x K elements [kc, kc + kw) of X (rows of `dim` BF16, `rows`
// valid, zero beyond) into the canonical K-major layout: 16-byte piece (r, c) at
// (r / 8) * (kw / 8) * 128 + c * 128 + (r % 8) * 16.  Eight consecutive threads fill one
// 128-byte core matrix.
__device__ __forceinline__ void stage(unsigned char *dst, const __nv_bfloat16 *X, int64_t r0, int64_t rows, int dim,
                                      int kc, int kw) {
	const int nkc = kw >> 3;  // pieces per thread: TM * nkc / THREADS = nkc (TM == THREADS)
	constexpr int BATCH = 8;  // loads in flight per thread before their stores
	for (int c0 = 0; c0 < nkc; c0 += BATCH) {
		uint4 v[BATCH];
#pragma unroll
		for (int u = 0; u < BATCH; u++) {
			const int c = (c0 + u) * THREADS + threadIdx.x;
			const int r8 = c & 7, rest = c >> 3;
			const int kq = rest % nkc, g = rest / nkc;
			const int r = g * 8 + r8;
			v[u] = make_uint4(0, 0, 0, 0);
			if (c0 + u < nkc && r0 + r < rows)
				v[u] = __ldg(reinterpret_cast<const uint4 *>(X + (r0 + r) * int64_t(dim) + kc + kq * 8));
		}
#pragma unroll
		for (int u = 0; u < BATCH; u++) {
			const int c = (c0 + u) * THREADS + threadIdx.x;
			const int r8 = c & 7, rest = c >> 3;
			const int kq = rest % nkc, g = rest / nkc;
			if (c0 + u < nkc) *reinterpret_cast<uint4 *>(dst + (g * nkc + kq) * 128 + r8 * 16) = v[u];
		}
	}
}

// The pair of tile t -- the last k with tile_start[k] <= t -- and the tile's origin, by a
// 32-way search of the whole warp (every lane probes one candidate per round, a ballot
// picks the bracket): 3 rounds of dependent loads for 8192 pairs instead of 13 for a
// binary search, which otherwise dominates the time per tile.  Call with all 32 lanes.
__device__ __forceinline__ void tile_of(const SimParams &p, int64_t t, int64_t &k, int64_t &m0, int64_t &n0,
                                        int64_t &ls, int64_t &lt) {
	const int lane = threadIdx.x & 31;
	int64_t lo = 0, hi = p.batch - 1;  // tile_start[lo] <= t always holds (tile_start[0] = 0)
	while (lo < hi) {
		const int64_t step = (hi - lo + 32) / 32;  // ceil((hi - lo + 1) / 32)
		const int64_t idx = lo + int64_t(lane) * step;
		const bool le = idx <= hi && p.tile_start[idx] <= t;
		const uint32_t m = __ballot_sync(0xffffffffu, le);
		const int top = 31 - __clz(m);  // lane 0 always qualifies
		lo = lo + int64_t(top) * step;
		hi = min(hi, lo + step - 1);
	}
	k = lo;
	ls = p.len_s[k];
	lt = p.len_t[k];
	const int64_t tiles_n = (ls + TN - 1) / TN;
	const int64_t local = t - p.tile_start[k];
	m0 = (local / tiles_n) * TM;
	n0 = (local % tiles_n) * TN;
}

__global__ void __launch_bounds__(THREADS, 3) sim_bf16_kernel(SimParams p) {
	extern __shared__ __align__(1024) unsigned char smem[];
	unsigned char *sA = smem;
	unsigned char *sB = smem + OPBYTES;
	uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * OPBYTES);
	uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + 2 * OPBYTES + 16);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
		             "r"(TN)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (threadIdx.x == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tslot;
	const uint32_t bar_a = smem_addr(bar);
	uint32_t phase = 0;
	bool ok = true;

	for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
		int64_t k, m0, n0, ls, lt;
		tile_of(p, t, k, m0, n0, ls, lt);
		const __nv_bfloat16 *A = p.Et + k * p.n_t * p.dim;
		const __nv_bfloat16 *B = p.Es + k * p.n_s * p.dim;

		for (int kc = 0; kc < p.dim && ok; kc += KC) {
			const int kw = min(KC, p.dim - kc);
			stage(sA, A, m0, lt, p.dim, kc, kw);
			stage(sB, B, n0, ls, p.dim, kc, kw);
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			__syncthreads();
			if (threadIdx.x == 0) {
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				const uint32_t sbo = uint32_t(kw >> 3) * 128u;
				for (int kk = 0; kk < kw / 16; kk++) {
					const uint64_t da = smem_desc(smem_addr(sA) + kk * 256, 128, sbo);
					const uint64_t db = smem_desc(smem_addr(sB) + kk * 256, 128, sbo);
					mma_bf16(tmem, da, db, (kc > 0 || kk > 0) ? 1u : 0u);
				}
				mma_commit(bar_a);
			}
			// every thread takes the same decision, so the barriers below stay matched
			if (!__syncthreads_and(mbar_wait(bar_a, phase) ? 1 : 0)) {
				if (threadIdx.x == 0) atomicOr(p.status, ST_TIMEOUT);
				ok = false;
			}
			phase ^= 1u;
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		}
		if (ok && m0 + warp * 32 < lt) {
			// epilogue: warp w holds tile rows 32w..32w+31 (TMEM lanes), one row per thread.
			// Per 32 columns each thread parks its row in shared memory (the A operand's
			// space, free once the MMAs completed; row pitch 33 words, conflict-free both
			// ways) and the warp writes the rows back one at a time as 128-byte segments.
			float *buf = reinterpret_cast<float *>(sA) + warp * 32 * 33;
			const int64_t ncols = ls - n0;  // valid columns of this tile (> 0)
			const int rows = int(min(int64_t(32), lt - (m0 + warp * 32)));
			float *out = p.St + k * p.pitch_pair + (m0 + warp * 32) * p.pitch_row + n0;
			for (int cc = 0; cc < TN && cc < ncols; cc += 32) {
				uint32_t v[32];
				tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(cc), v);
#pragma unroll
				for (int q = 0; q < 32; q++) buf[lane * 33 + q] = __fmaf_rn(p.alpha, __uint_as_float(v[q]), p.beta);
				__syncwarp();
				if (cc + lane < ncols) {
					for (int rr = 0; rr < rows; rr++) out[rr * p.pitch_row + cc + lane] = buf[rr * 33 + lane];
				}
				__syncwarp();
			}
		}
		asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
		__syncthreads();
	}
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN) : "memory");
	}
}

// ---------------------------------------------------------------------------------------
// The pipelined form (default).  One persistent CTA per SM, 192 threads in three roles:
//   warp 0    producer: per 64-element K chunk, 16 TMA loads (cp.async.bulk.tensor) of
//             8-element x 128-row boxes into a 4-stage ring, completing on the stage's
//             "full" mbarrier;
//   warp 1    MMA issuer: waits "full", issues 4 tcgen05.mma (K = 16) into one of two
//             128-column TMEM accumulators, commits the stage back to its "empty" mbarrier
//             and, after a tile's last chunk, the accumulator to its "ready" mbarrier;
//   warps 2-5 epilogue: wait "ready", read their 32 TMEM lanes, write the rows inside the
//             pair through a shared-memory transpose as 128-byte segments, then release
//             the accumulator ("free", 4 arrivals).
// So the loads of chunk c + 1..c + 3, the MMAs of chunk c and the stores of the previous
// tile run at the same time.  A 64-element K chunk of a 128-row operand tile is one TMA box
// of 128 rows x 128 bytes written with the 128-byte swizzle (16-byte pieces of each row
// XOR-permuted within 8-row, 1 KB atoms) -- the canonical K-major SWIZZLE_128B layout the
// MMA descriptors name (8-row groups 1 KB apart; the K = 16 steps start 32 bytes apart in
// the row).  One request per 128-byte row: full sectors, 4x fewer requests than 16-byte
// boxes.  Rows past the tensor read as zero (TMA fill);
// rows of a neighbouring pair are multiplied but never stored.  Every wait is bounded: on a
// timeout the role sets the status bit and stops, and the others stop at their own.
constexpr int PK = 64;                       // K elements per stage: one 128-byte row
constexpr int PSTAGES = 4;
constexpr int PTILE = TM * PK * 2;           // one operand tile of a stage: 16 KB
constexpr int PSTAGE_BYTES = 2 * PTILE;      // A and B: 32 KB
constexpr int PEPI_BYTES = 4 * 32 * 33 * 4;  // transpose buffers of the 4 epilogue warps
constexpr int PSMEM = PSTAGES * PSTAGE_BYTES + PEPI_BYTES + 256 + 1024;
constexpr int PTHREADS = 192;

__device__ __forceinline__ bool pwait(uint32_t bar, uint32_t parity) { return mbar_wait(bar, parity); }

// Shared-memory descriptor of a K-major SWIZZLE_128B operand: start (>> 4), leading byte
// offset 16 (unused for this layout), stride byte offset 1024 (8-row groups), version 1 at
// bit 46, layout type 2 (128-byte swizzle) at bits 61-63.  The tile base is 1 KB aligned.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
	return uint64_t((addr >> 4) & 0x3fff) | (uint64_t(16 >> 4) << 16) | (uint64_t(1024 >> 4) << 32) |
	       (uint64_t(1) << 46) | (uint64_t(2) << 61);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
	        dst),
	    "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
	    : "memory");
}

// The tiles of one CTA, a contiguous range [t0, t1), walked pair by pair: one warp-wide
// search for the pair of t0, then per tile only a counter, and per pair three loads
// (its tile count and lengths).  All three roles walk the same sequence.
struct TileWalk {
	int64_t t, t1, k, local, ntiles_k, tiles_n, ls, lt;
	__device__ __forceinline__ void load_pair(const SimParams &p) {
		ntiles_k = p.tile_start[k + 1] - p.tile_start[k];
		ls = p.len_s[k];
		lt = p.len_t[k];
		tiles_n = (ls + TN - 1) / TN;
	}
	__device__ __forceinline__ void begin(const SimParams &p, int64_t t0, int64_t tend) {
		t = t0;
		t1 = tend;
		if (t >= t1) return;
		int64_t m0_, n0_, ls_, lt_;
		tile_of(p, t, k, m0_, n0_, ls_, lt_);  // warp-wide search
		local = t - p.tile_start[k];
		load_pair(p);
	}
	__device__ __forceinline__ bool valid() const { return t < t1; }
	__device__ __forceinline__ int64_t m0() const { return (local / tiles_n) * TM; }
	__device__ __forceinline__ int64_t n0() const { return (local % tiles_n) * TN; }
	__device__ __forceinline__ void next(const SimParams &p) {
		if (++t >= t1) return;
		if (++local >= ntiles_k) {  // next pair with tiles
			do {
				k++;
				local = 0;
				load_pair(p);
			} while (ntiles_k == 0);
		}
	}
};

__global__ void __launch_bounds__(PTHREADS, 1)
    sim_bf16_tma_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                        SimParams p) {
	extern __shared__ __align__(1024) unsigned char smem_raw[];
	// 1024-byte aligned base for the stages
	unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
	float *epi = reinterpret_cast<float *>(smem + PSTAGES * PSTAGE_BYTES);
	uint64_t *bars = reinterpret_cast<uint64_t *>(smem + PSTAGES * PSTAGE_BYTES + PEPI_BYTES);
	// bars: full[0..3], empty[4..7], ready[8..9], free[10..11]; TMEM address at bars + 12
	uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 12);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const uint32_t bar0 = smem_addr(bars);
	auto full = [&](int s) { return bar0 + 8u * s; };
	auto empty = [&](int s) { return bar0 + 8u * (4 + s); };
	auto ready = [&](int a) { return bar0 + 8u * (8 + a); };
	auto freed = [&](int a) { return bar0 + 8u * (10 + a); };

	if (threadIdx.x == 0) {
		for (int s = 0; s < PSTAGES; s++) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full(s)) : "memory");
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(empty(s)) : "memory");
		}
		for (int a = 0; a < 2; a++) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ready(a)) : "memory");
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(freed(a)) : "memory");
		}
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
		             "r"(2 * TN)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tslot;
	const int nchunks = (p.dim + PK - 1) / PK;
	const int64_t per = (p.total_tiles + gridDim.x - 1) / gridDim.x;
	const int64_t t_begin = min(int64_t(blockIdx.x) * per, p.total_tiles);
	const int64_t t_end = min(t_begin + per, p.total_tiles);
	TileWalk tw;
	tw.begin(p, t_begin, t_end);  // every warp, all lanes

	if (warp == 0) {
		// ---- producer (the warp decodes tiles, lane 0 issues the copies)
		int s = 0;
		uint32_t ph = 0;
		bool ok = true;
		for (; tw.valid() && ok; tw.next(p)) {
			if (lane == 0) {
				const int ya = int(tw.k * p.n_t + tw.m0()), yb = int(tw.k * p.n_s + tw.n0());
				for (int c = 0; c < nchunks; c++) {
					if (!pwait(empty(s), ph ^ 1u)) { atomicOr(p.status, ST_TIMEOUT); ok = false; break; }
					asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full(s)),
					             "r"(PSTAGE_BYTES)
					             : "memory");
					const uint32_t sa = smem_addr(smem + s * PSTAGE_BYTES), sb = sa + PTILE;
					tma_load_2d(sa, &mapA, c * PK, ya, full(s));
					tma_load_2d(sb, &mapB, c * PK, yb, full(s));
					if (++s == PSTAGES) { s = 0; ph ^= 1u; }
				}
			}
			ok = __shfl_sync(0xffffffffu, ok, 0);
		}
	} else if (warp == 1) {
		// ---- MMA issuer (lane 0; the warp only iterates the tiles with it)
		int s = 0, a = 0;
		uint32_t ph = 0, aph = 0;
		bool ok = true;
		for (; tw.valid() && ok; tw.next(p)) {
			if (lane == 0) {
				if (!pwait(freed(a), aph ^ 1u)) {
					atomicOr(p.status, ST_TIMEOUT);
					ok = false;
				} else {
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
					const uint32_t dacc = tmem + uint32_t(a * TN);
					for (int c = 0; c < nchunks; c++) {
						if (!pwait(full(s), ph)) { atomicOr(p.status, ST_TIMEOUT); ok = false; break; }
						asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
						const uint32_t sa = smem_addr(smem + s * PSTAGE_BYTES), sb = sa + PTILE;
#pragma unroll
						for (int kk = 0; kk < PK / 16; kk++) {
							const uint64_t da = desc_sw128(sa + kk * 32);
							const uint64_t db = desc_sw128(sb + kk * 32);
							mma_bf16(dacc, da, db, (c > 0 || kk > 0) ? 1u : 0u);
						}
						mma_commit(empty(s));  // the stage is free once these MMAs have read it
						if (++s == PSTAGES) { s = 0; ph ^= 1u; }
					}
					if (ok) mma_commit(ready(a));
				}
				if (++a == 2) { a = 0; aph ^= 1u; }
			}
			ok = __shfl_sync(0xffffffffu, ok, 0);
		}
	} else {
		// ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (tile rows)
		const int rq = warp & 3;
		float *buf = epi + (warp - 2) * 32 * 33;
		int a = 0;
		uint32_t aph = 0;
		for (; tw.valid(); tw.next(p)) {
			const int64_t k = tw.k, m0 = tw.m0(), n0 = tw.n0(), ls = tw.ls, lt = tw.lt;
			if (!__all_sync(0xffffffffu, pwait(ready(a), aph))) {
				if (lane == 0) atomicOr(p.status, ST_TIMEOUT);
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const int64_t r0 = m0 + rq * 32;
			if (r0 < lt) {
				const int64_t ncols = ls - n0;
				const int rows = int(min(int64_t(32), lt - r0));
				float *out = p.St + k * p.pitch_pair + r0 * p.pitch_row + n0;
				for (int cc = 0; cc < TN && cc < ncols; cc += 32) {
					uint32_t v[32];
					tmem_ld32(tmem + (uint32_t(rq * 32) << 16) + uint32_t(a * TN + cc), v);
#pragma unroll
					for (int q = 0; q < 32; q++) buf[lane * 33 + q] = __fmaf_rn(p.alpha, __uint_as_float(v[q]), p.beta);
					__syncwarp();
					if (cc + lane < ncols)
						for (int rr = 0; rr < rows; rr++) out[rr * p.pitch_row + cc + lane] = buf[rr * 33 + lane];
					__syncwarp();
				}
			}
			asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
			__syncwarp();
			if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(freed(a)) : "memory");
			if (++a == 2) { a = 0; aph ^= 1u; }
		}
	}
	__syncthreads();
	if (warp == 1) {
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TN) : "memory");
	}
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
	static std::once_flag once;
	static EncodeTiledFn fn = nullptr;
	std::call_once(once, [] {
		void *f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
		        cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<EncodeTiledFn>(f);
	});
	return fn;
}

// 2-D map of a (rows x dim) BF16 matrix, boxes of 64 elements x 128 rows written with the
// 128-byte swizzle, zero fill.
bool make_map(CUtensorMap *m, const void *base, int64_t rows, int32_t dim) {
	EncodeTiledFn fn = encode_fn();
	if (!fn) return false;
	const cuuint64_t gdim[2] = {cuuint64_t(dim), cuuint64_t(rows)};
	const cuuint64_t gstride[1] = {cuuint64_t(dim) * 2};
	const cuuint32_t box[2] = {cuuint32_t(PK), cuuint32_t(TM)};
	const cuuint32_t estride[2] = {1, 1};
	return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), gdim, gstride, box, estride,
	          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

extern "C" pa_status pa_similarity_bf16(const void *Es, const void *Et, int64_t batch, int64_t n_s, int64_t n_t,
                                        int32_t dim, const int32_t *len_s, const int32_t *len_t,
                                        const int32_t *tile_start, int64_t total_tiles, float *St,
                                        int64_t pitch_pair, int64_t pitch_row, float alpha, float beta,
                                        int32_t *status, void *stream) {
	if (batch < 0 || n_s < 0 || n_t < 0 || total_tiles < 0) return PA_ERR_INVALID_ARGUMENT;
	if (batch == 0 || total_tiles == 0) return PA_OK;
	if (!Es || !Et || !len_s || !len_t || !tile_start || !St || !status) return PA_ERR_INVALID_ARGUMENT;
	if (dim <= 0 || dim % 16 != 0) return PA_ERR_INVALID_ARGUMENT;  // K steps of 16, 16-byte rows
	if ((reinterpret_cast<uintptr_t>(Es) | reinterpret_cast<uintptr_t>(Et)) & 15) return PA_ERR_INVALID_ARGUMENT;
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return PA_ERR_NO_DEVICE;
	if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PA_ERR_CUDA;
	static bool attr_set[64] = {};
	if (dev < 64 && !attr_set[dev]) {
		if (cudaFuncSetAttribute(sim_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
		    cudaSuccess)
			return PA_ERR_CUDA;
		attr_set[dev] = true;
	}
	SimParams p;
	p.Es = static_cast<const __nv_bfloat16 *>(Es);
	p.Et = static_cast<const __nv_bfloat16 *>(Et);
	p.n_s = n_s;
	p.n_t = n_t;
	p.dim = dim;
	p.len_s = len_s;
	p.len_t = len_t;
	p.tile_start = tile_start;
	p.batch = batch;
	p.total_tiles = total_tiles;
	p.St = St;
	p.pitch_pair = pitch_pair;
	p.pitch_row = pitch_row;
	p.alpha = alpha;
	p.beta = beta;
	p.status = status;
	const char *kind = std::getenv("PA_SIM_KERNEL");  // "plain": the unpipelined kernel (comparisons)
	CUtensorMap ma, mb;
	const bool piped = !(kind && std::strcmp(kind, "plain") == 0) && batch * n_t < (int64_t(1) << 31) &&
	                   batch * n_s < (int64_t(1) << 31) && make_map(&ma, Et, batch * n_t, dim) &&
	                   make_map(&mb, Es, batch * n_s, dim);
	if (piped) {
		static bool pattr_set[64] = {};
		if (dev < 64 && !pattr_set[dev]) {
			if (cudaFuncSetAttribute(sim_bf16_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, PSMEM) !=
			    cudaSuccess)
				return PA_ERR_CUDA;
			pattr_set[dev] = true;
		}
		const int64_t grid = total_tiles < int64_t(sms) ? total_tiles : int64_t(sms);
		sim_bf16_tma_kernel<<<int(grid), PTHREADS, PSMEM, static_cast<cudaStream_t>(stream)>>>(ma, mb, p);
		return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
	}
	const int64_t grid = total_tiles < int64_t(3) * sms ? total_tiles : int64_t(3) * sms;
	sim_bf16_kernel<<<int(grid), THREADS, SMEM_BYTES, static_cast<cudaStream_t>(stream)>>>(p);
	return cudaGetLastError() == cudaSuccess ? PA_OK : PA_ERR_CUDA;
}

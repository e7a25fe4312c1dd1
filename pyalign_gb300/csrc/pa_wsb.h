// General gap cost (Waterman-Smith-Beyer) kernel interface.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pa {

struct WsbParams {
	int32_t npairs;
	const int32_t *len_s;
	const int32_t *len_t;
	int32_t local;         // locality: 0 local, 1 global, 2 semiglobal
	int32_t sub_kind;      // SubKind
	const uint32_t *a;
	const uint32_t *b;
	int64_t a_stride, b_stride;
	const float *table;
	int32_t table_rows, table_cols;
	float eq, ne;
	const float *dense;
	int64_t dense_si, dense_sj;
	float sign;            // +1 maximize, -1 minimize (similarities are multiplied by it)
	const float *gap_s;    // reference-domain costs w_s(k), k = 0..cap_s
	const float *gap_t;
	const float *left_D;   // normalised borders, index i+1 for row i
	const float *top_D;
	float *vals;           // normalised D, (ls+1) x (lt+1) per pair at vals_off
	float *vals_t;         // the same values transposed, (lt+1) x (ls+1)
	const int64_t *vals_off;
	int32_t *tb;           // ls x lt traceback codes per pair at tb_off: kind | (k+1) << 2
	const int64_t *tb_off;
	float *sub;            // ls x lt normalised similarity per pair at tb_off (for tie replay)
	float *score;          // reference domain
	int32_t *seed;
	int32_t *has_seed;
	int32_t *status;
	int32_t warp_cells;    // a warp per cell on diagonals of at most warp_cells x warps cells
	int32_t lds;           // > 0 (one CTA per pair): the rows also in shared memory, lds (odd) floats a row
	int32_t max_ls;        // the launch's largest |s| (sizes that shared memory)
};

// One optimal alignment per pair from the traceback codes (TracebackIterators<false>,
// solver.h:1497-1536, compressed as path_compressor does, solver.h:809-847): the map of
// min(|s|, |t|) entries at map_off (s_to_t when |s| <= |t|, else t_to_s, -1 = unaligned).
struct WsbWalkParams {
	int32_t npairs;
	const int32_t *len_s;
	const int32_t *len_t;
	int32_t local;
	const float *vals;
	const int64_t *vals_off;
	const int32_t *tb;
	const int64_t *tb_off;
	const int32_t *seed;
	const int32_t *has_seed;
	const int64_t *map_off;
	int32_t *maps;
};

// threads: the block size, a multiple of 32 up to 1024; cluster: CTAs per pair (1, 2 or 4)
cudaError_t launch_wsb(const WsbParams &p, int threads, int cluster, cudaStream_t st);
cudaError_t launch_wsb_walk(const WsbWalkParams &p, cudaStream_t st);

}  // namespace pa

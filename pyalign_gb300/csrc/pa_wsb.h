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
	float *vals_t;         // the same values transposed, (lt+1) x (ls+1): the row scans read it
	const int64_t *vals_off;
	int32_t *tb;           // ls x lt traceback codes per pair at tb_off: kind | (k+1) << 2
	const int64_t *tb_off;
	float *sub;            // ls x lt normalised similarity per pair at tb_off (for tie replay)
	float *score;          // reference domain
	int32_t *seed;
	int32_t *has_seed;
	int32_t *status;
};

cudaError_t launch_wsb(const WsbParams &p, cudaStream_t st);

}  // namespace pa

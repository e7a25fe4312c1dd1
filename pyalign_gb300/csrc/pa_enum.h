// Device enumeration of the first k optimal alignments per pair (pa_enum.cu): parameters
// shared with the host glue in pa_host.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pa {

constexpr int32_t ENUM_NO_TB = INT32_MIN;  // the terminal point of an empty list
constexpr int32_t ENUM_OVERFLOW = 1;  // the stack was full: enumerate again with a larger one
constexpr int32_t ENUM_BAD_PATH = 2;  // a path longer than |s| + |t| + 2 points (not reachable)

struct EnumParams {
	int32_t nwork;
	const int32_t *work;        // pairs to enumerate
	int32_t G;                  // group width of the DP launch that wrote the masks
	int32_t local, affine, remove_dup, k;
	const int32_t *len_s, *len_t;
	const int64_t *mask_off;    // per pair, uint4 units
	const uint4 *masks;
	const int32_t *has;         // Global/Semiglobal: the pair has its seed
	const int32_t *seed;        // (i, j) per pair
	const int2 *seeds;          // local: seed cells per pair, in pop order
	const int64_t *seed_off;
	const int32_t *seed_n;
	int4 *stack;                // (u, v, path length, -) entries
	const int64_t *stack_off;
	const int32_t *stack_cap;
	int2 *path;                 // ls + lt + 2 points per pair
	const int64_t *path_off;
	int32_t *maps;              // k maps of min(ls, lt) per pair
	const int64_t *map_off;
	int2 *paths;                // optional: k paths of ls + lt + 2 points per pair
	const int64_t *paths_off;
	int32_t *path_len;          // optional: k per pair
	unsigned long long *hash;   // k per pair
	int32_t *npts;              // k per pair
	int32_t *count;             // per pair: paths yielded (<= k)
	int32_t *status;            // per pair: ENUM_OVERFLOW
};

struct SeedScanParams {
	int32_t nwork;
	const int32_t *work;
	int32_t G;
	const int32_t *len_s, *len_t;
	const int64_t *mask_off;
	const uint4 *masks;
	int2 *seeds;
	const int64_t *seed_off;
	const int32_t *seed_cap;
	int32_t *seed_n;            // every seed is counted; only seed_cap are stored
};

cudaError_t enum_seed_scan(const SeedScanParams &p, int grid, cudaStream_t st);
cudaError_t enum_solve(const EnumParams &p, cudaStream_t st);

}  // namespace pa

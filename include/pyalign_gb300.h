/*
 * pyalign_gb300 -- C ABI of the GB300 (sm_103a) batched alignment solve.
 *
 * This library replaces the native core of pyalign 0.4.4: the pybind11 module
 * `pyalign.algorithm.<variant>.algorithm` (pyalign/algorithm/module.cpp:7-18), whose
 * Solver interface is declared in pyalign/algorithm/factory.h:414-508 and registered in
 * pyalign/algorithm/pyalign.h:17-77.  Each entry point below names the reference
 * function it replaces.  All arguments are plain pointers and sizes; no torch or numpy
 * types cross this boundary.  The Python binding (pyalign_gb300/algorithm.py, ctypes)
 * re-exports the reference's Python names on top of it.
 *
 * Conventions
 *  - Every function that can fail returns a pa_status; pa_last_error() gives the
 *    message of the last failure on the calling thread.  PA_ERR_INVALID_ARGUMENT maps
 *    to the reference's std::invalid_argument (Python ValueError); PA_ERR_LENGTH to its
 *    exceeded_*_length exceptions (solver.h:95-152, Python RuntimeError).
 *  - Arrays follow the reference's layouts: codes a/b are (batch, n_s) and (batch, n_t)
 *    uint32 row-major (solve.py:402-404); a dense similarity is (n_s, n_t, batch) float32,
 *    lane-minor (solve.py:349); lengths are (2, batch) int32: row 0 = |s|, row 1 = |t|.
 *  - Values are float32 as in the reference (module.cpp:11-14); alignment maps, paths
 *    and traceback matrices are int32 (the Python layer narrows them for m16).
 *  - A solver is not re-entrant (like the reference, factory.h:682-973); results and
 *    iterators own their data and stay valid after later solve calls.
 *  - All device work of a solver runs on its CUDA stream (pa_solver_set_stream).  A
 *    device-resident solve that repeats the solver's previous one exactly (lengths, shapes,
 *    buffers, options) reuses its plan and, from the second repetition on, runs as a CUDA
 *    graph captured on a private stream; inputs are read at every launch (PA_GRAPHS=0
 *    disables the cache).
 */
#ifndef PYALIGN_GB300_H
#define PYALIGN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t pa_status;
#define PA_OK 0
#define PA_ERR_INVALID_ARGUMENT 1
#define PA_ERR_LENGTH 2
#define PA_ERR_CUDA 3
#define PA_ERR_NO_DEVICE 4
#define PA_ERR_INTERNAL 5
#define PA_ERR_TIMEOUT 6
#define PA_ERR_UNSUPPORTED 7

/* enums: values identical to pyalign/algorithm/enum.h:8-33 */
#define PA_TYPE_ALIGNMENT 0
#define PA_TYPE_DTW 1
#define PA_MINIMIZE 0
#define PA_MAXIMIZE 1
#define PA_DETAIL_SCORE 0
#define PA_DETAIL_ALIGNMENT 1
#define PA_DETAIL_SOLUTION 2
#define PA_COUNT_ONE 0
#define PA_COUNT_ALL 1
#define PA_LOCAL 0
#define PA_GLOBAL 1
#define PA_SEMIGLOBAL 2

/* gap cost kinds, as resolved by FactoryCreator::resolve_gap_type (factory.h:1106-1136) */
#define PA_GAP_LINEAR 0
#define PA_GAP_AFFINE 1
#define PA_GAP_GENERAL 2

/* where caller buffers live */
#define PA_HOST 0
#define PA_DEVICE 1

typedef struct pa_options {
	int32_t type;        /* PA_TYPE_* (options.h:14-21) */
	int32_t direction;   /* PA_MINIMIZE / PA_MAXIMIZE */
	int32_t detail;      /* PA_DETAIL_* (options.h:25-36) */
	int32_t count;       /* PA_COUNT_* */
	int32_t locality;    /* PA_LOCAL / PA_GLOBAL / PA_SEMIGLOBAL */
	int32_t remove_dup;  /* = not return_dup (options.h:21) */
	int32_t batch;       /* options "batch" (solve.py:181) */
	int32_t batch_size;  /* lanes per solve call when batch != 0; 0 = library default */
	int32_t index_bits;  /* 16 for m16, 32 for m32 (module.cpp:10-14) */
	int32_t gap_kind;    /* PA_GAP_*; ignored for DTW */
	float linear_s, linear_t;                 /* linear: w(k) = g k */
	float affine_u_s, affine_v_s;             /* affine, Gotoh form w(k) = u k + v (solver.h:2858-2881) */
	float affine_u_t, affine_v_t;
	const float *general_s;  /* general: GapCost.costs(max_len_s + 1) (factory.h:20-31), copied */
	const float *general_t;  /* general: GapCost.costs(max_len_t + 1), copied */
} pa_options;

typedef struct pa_solver pa_solver;
typedef struct pa_result pa_result;
typedef struct pa_iterator pa_iterator;

/* Last error message of the calling thread ("" if none). */
const char *pa_last_error(void);

/* Library version string. */
const char *pa_version(void);

/* Number of usable CUDA devices (0 when none: every solve then fails with
 * PA_ERR_NO_DEVICE -- there is no CPU fallback). */
int32_t pa_device_count(void);

/* Replaces create_solver<Options> (factory.h:1268-1278): a solver for sequences up to
 * max_len_s x max_len_t.  Fails with PA_ERR_LENGTH past the index type's limit
 * (solver.h:496-503). */
pa_status pa_solver_create(const pa_options *options, int64_t max_len_s, int64_t max_len_t,
                           pa_solver **out);
void pa_solver_destroy(pa_solver *solver);

/* Replaces Solver::batch_size (factory.h:422, pyalign.h:25). */
int32_t pa_solver_batch_size(const pa_solver *solver);

/* Run the solver's device work on `stream`, a cudaStream_t; NULL is CUDA's default stream,
 * as for a kernel launch, so work on it is ordered with the caller's work on that stream.
 * Until this is called the solver uses a non-blocking stream of its own (its calls that
 * return host results synchronise it before returning). */
pa_status pa_solver_set_stream(pa_solver *solver, void *stream);

/* ---- the 15 solve entry points (factory.h:424-507; pyalign.h:26-40) ----
 * sim (dense): n_s x n_t x batch float32; a: batch x n_s, b: batch x n_t uint32;
 * table: table_rows x table_cols float32; length: 2 x batch int32 (host memory).
 * Score variants write `batch` float32 scores; all others return a pa_result.     */

pa_status pa_solve_for_score(pa_solver *s, const float *sim, int64_t n_s, int64_t n_t,
                             int64_t batch, const int32_t *length, float *scores);
pa_status pa_solve_indexed_for_score(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                     int64_t batch, int64_t n_s, int64_t n_t,
                                     const float *table, int64_t table_rows, int64_t table_cols,
                                     const int32_t *length, float *scores);
pa_status pa_solve_binary_for_score(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                    int64_t batch, int64_t n_s, int64_t n_t, float eq, float ne,
                                    const int32_t *length, float *scores);

pa_status pa_solve_for_alignment(pa_solver *s, const float *sim, int64_t n_s, int64_t n_t,
                                 int64_t batch, const int32_t *length, pa_result **out);
pa_status pa_solve_indexed_for_alignment(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                         int64_t batch, int64_t n_s, int64_t n_t,
                                         const float *table, int64_t table_rows,
                                         int64_t table_cols, const int32_t *length,
                                         pa_result **out);
pa_status pa_solve_binary_for_alignment(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                        int64_t batch, int64_t n_s, int64_t n_t, float eq,
                                        float ne, const int32_t *length, pa_result **out);

pa_status pa_solve_for_alignment_iterator(pa_solver *s, const float *sim, int64_t n_s,
                                          int64_t n_t, int64_t batch, const int32_t *length,
                                          pa_result **out);
pa_status pa_solve_indexed_for_alignment_iterator(pa_solver *s, const uint32_t *a,
                                                  const uint32_t *b, int64_t batch, int64_t n_s,
                                                  int64_t n_t, const float *table,
                                                  int64_t table_rows, int64_t table_cols,
                                                  const int32_t *length, pa_result **out);
pa_status pa_solve_binary_for_alignment_iterator(pa_solver *s, const uint32_t *a,
                                                 const uint32_t *b, int64_t batch, int64_t n_s,
                                                 int64_t n_t, float eq, float ne,
                                                 const int32_t *length, pa_result **out);

pa_status pa_solve_for_solution(pa_solver *s, const float *sim, int64_t n_s, int64_t n_t,
                                int64_t batch, const int32_t *length, pa_result **out);
pa_status pa_solve_indexed_for_solution(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                        int64_t batch, int64_t n_s, int64_t n_t,
                                        const float *table, int64_t table_rows,
                                        int64_t table_cols, const int32_t *length,
                                        pa_result **out);
pa_status pa_solve_binary_for_solution(pa_solver *s, const uint32_t *a, const uint32_t *b,
                                       int64_t batch, int64_t n_s, int64_t n_t, float eq,
                                       float ne, const int32_t *length, pa_result **out);

pa_status pa_solve_for_solution_iterator(pa_solver *s, const float *sim, int64_t n_s,
                                         int64_t n_t, int64_t batch, const int32_t *length,
                                         pa_result **out);
pa_status pa_solve_indexed_for_solution_iterator(pa_solver *s, const uint32_t *a,
                                                 const uint32_t *b, int64_t batch, int64_t n_s,
                                                 int64_t n_t, const float *table,
                                                 int64_t table_rows, int64_t table_cols,
                                                 const int32_t *length, pa_result **out);
pa_status pa_solve_binary_for_solution_iterator(pa_solver *s, const uint32_t *a,
                                                const uint32_t *b, int64_t batch, int64_t n_s,
                                                int64_t n_t, float eq, float ne,
                                                const int32_t *length, pa_result **out);

/* ---- results: one per solve call, `batch` lanes ---- */
void pa_result_destroy(pa_result *r);
int64_t pa_result_size(const pa_result *r);
int64_t pa_result_len_s(const pa_result *r, int64_t lane);
int64_t pa_result_len_t(const pa_result *r, int64_t lane);
/* All lanes' lengths at once (len_s, len_t: pa_result_size entries each): the per-lane
 * shapes pyalign reads for every result object (solve.py:376-379), in one call. */
pa_status pa_result_lengths(const pa_result *r, int32_t *len_s, int32_t *len_t);

/* Alignment of a lane (codomain Alignment or Solution): Alignment::score/s_to_t/t_to_s
 * (factory.h:130-193).  `map` receives min(|s|, |t|) entries: s_to_t when |s| <= |t|,
 * else t_to_s, -1 where unaligned.  has_alignment is 0 when the reference's traceback
 * iterator yields nothing (local/semiglobal problems without cells); the score is then
 * the direction's worst value. */
int32_t pa_result_has_alignment(const pa_result *r, int64_t lane);
float pa_result_score(const pa_result *r, int64_t lane);
pa_status pa_result_alignment(const pa_result *r, int64_t lane, int32_t *map);

/* Bulk export of all lanes: scores[batch]; maps concatenated at map_offsets[lane]
 * (caller-computed prefix sums of min(|s|, |t|)). */
pa_status pa_result_export(const pa_result *r, float *scores, int32_t *maps,
                           const int64_t *map_offsets);

/* Solution of a lane (core::Solution, solver.h:2329-2507; SolutionImpl factory.h:284-352).
 * values: layers x (|s|+1) x (|t|+1) float32, the border row/column included.
 * tb_matrix: layers x (|s|+1) x (|t|+1) x 2, first traceback entry per cell, INT32_MIN
 * where none.  tb_edges: (n, 2, 2) per layer ((i-1, j-1) -> (u, v)); pass NULL to get n.
 * path: (n, 2) points of the traceback walk (build_path, solver.h:858-938). */
int32_t pa_result_layers(const pa_result *r, int64_t lane);
int32_t pa_result_max_degree_1(const pa_result *r);
pa_status pa_result_values(const pa_result *r, int64_t lane, float *values);
pa_status pa_result_tb_matrix(const pa_result *r, int64_t lane, int32_t *tb);
int64_t pa_result_tb_edges(const pa_result *r, int64_t lane, int32_t layer, int32_t *edges);
int64_t pa_result_path(const pa_result *r, int64_t lane, int32_t *path);

/* Solver metadata (AlgorithmMetaData, solver.h:154-177): name, runtime, memory. */
const char *pa_result_algorithm(const pa_result *r, int32_t field);

/* ---- iterators over all optimal alignments of a lane (AlignmentIterator,
 * SolutionIterator: solver.h:1783-1888; TracebackIterators<true> 1568-1743).
 * The iterator keeps the result alive.  next() returns 1 and fills score, map
 * (min(|s|,|t|) entries) and, if path != NULL, the walk (path_len points, at most
 * |s| + |t| + 2); 0 when exhausted. */
pa_status pa_result_iterator(pa_result *r, int64_t lane, pa_iterator **out);
int32_t pa_iterator_next(pa_iterator *it, float *score, int32_t *map, int32_t *path,
                         int64_t *path_len);
void pa_iterator_destroy(pa_iterator *it);

/* Number of co-optimal traceback paths of every lane of an all-optimal result (count ALL,
 * linear or affine gaps): how many alignments the reference's depth-first enumeration
 * (TracebackIterators<true>::Iterator::next, solver.h:1647-1716) yields with return_dup set,
 * i.e. before de-duplication of identical alignments.  Computed on the device from the
 * result's masks in one wavefront pass; `counts` (batch uint64, host) saturate at
 * 2^64 - 1.  The reference has no counterpart: its enumeration is the only way to count. */
pa_status pa_result_path_counts(const pa_result *r, uint64_t *counts);

/* The first k optimal alignments of every lane of an all-optimal result (count ALL, linear or
 * affine gaps), enumerated on the device in the order and with the de-duplication of the
 * reference's depth-first search (TracebackIterators<true>::Iterator::next,
 * solver.h:1647-1716; remove_dup as the solver's options say): the same results, in the same
 * order, as the first k calls of pa_iterator_next on each lane, for all lanes in one pass.
 * Host outputs: counts (batch int32) = results of each lane, <= k (< k: the lane has no
 * more); maps (may be NULL) = lane L's results at k * sum_{l < L} min(|s_l|, |t_l|), result j
 * at + j * min(|s_L|, |t_L|), each an s_to_t map when |s| <= |t| and a t_to_s map otherwise,
 * -1 where unaligned; paths and path_len (both or neither) = each result's walk, lane L's
 * at k * sum_{l < L} (|s_l| + |t_l| + 2) points (x, y int32), result j at
 * + j * (|s_L| + |t_L| + 2) points, path_len[L * k + j] points long; the slots past a lane's
 * count hold -1 maps and 0 path lengths.  The scores are the
 * lane's score (pa_result_score).  Blocks until the outputs are written.  No counterpart in
 * the reference: it enumerates one lane at a time. */
pa_status pa_result_first_alignments(const pa_result *r, int32_t k, int32_t *counts, int32_t *maps,
                                     int32_t *paths, int32_t *path_len);

/* ---- batched form: the whole bag in one call (no per-lane objects) ----
 * Score plus one optimal traceback for `batch` pairs of uneven lengths, the throughput
 * path behind ProblemBatch.  Inputs and outputs are host or device memory
 * (`location`); lengths (2 x batch int32) are always host memory.  Outputs: scores
 * (batch) and the maps concatenated at map_offsets (host array of batch entries,
 * prefix sums of min(|s|, |t|)); maps may be NULL for score only. */
typedef struct pa_batch {
	int32_t form;       /* 0 dense, 1 indexed, 2 binary */
	int32_t location;   /* PA_HOST or PA_DEVICE for a, b, table, sim, scores, maps */
	int64_t batch, n_s, n_t;
	const uint32_t *a;
	const uint32_t *b;
	const float *sim;   /* dense (n_s, n_t, batch) */
	const float *table; /* indexed */
	int64_t table_rows, table_cols;
	float eq, ne;       /* binary */
	const int32_t *length;  /* host (2, batch) */
} pa_batch;

pa_status pa_solve_batch(pa_solver *s, const pa_batch *batch, float *scores, int32_t *maps,
                         const int64_t *map_offsets);

/* The alignment codomain of the solve_*_for_alignment methods (factory.h:699-808) with the
 * maps written straight into the caller's host buffer: host inputs (`location` PA_HOST), maps
 * at map_offsets (host, batch entries, the prefix sums of min(|s|, |t|) of the lengths
 * clamped to [0, n_s] and [0, n_t]), and a result object for the rest of each lane's
 * Alignment (pa_result_score: the score, or the worst value where the lane has no
 * alignment; pa_result_has_alignment).  pa_result_alignment / pa_result_export of maps refuse
 * such a result (its maps are the caller's).  One-optimal solvers (count ONE, detail ALIGNMENT
 * or SOLUTION, or DTW) with linear, affine or DTW costs; others get PA_ERR_UNSUPPORTED.  No
 * counterpart in the reference: the module's solve_*_for_alignment methods use it to skip a
 * copy of every map. */
pa_status pa_solve_batch_result(pa_solver *s, const pa_batch *batch, int32_t *maps, const int64_t *map_offsets,
                                pa_result **out);

/* ---- differentiation (the fwd+bwd form) ----
 * Forward: score plus one optimal path per pair for a dense similarity held in device
 * memory with an explicit layout, S(k, i, j) = sim[offsets[k] + i*stride_s + j*stride_t]
 * (offsets: host array).  Writes scores (device, batch), the traceback walk of each pair
 * (device, 2 ints per point, |s| + |t| + 2 points at path_offsets[k] ints; host array of
 * offsets) and path_len (device).  The solver must be a one-optimal-path solver
 * (linear, affine or DTW).  No counterpart in the reference, which has no gradients; the
 * path is the one Solver::solution reports (solver.h:2665-2705). */
pa_status pa_solve_dense_paths(pa_solver *s, const float *sim, const int64_t *offsets, int64_t stride_s,
                               int64_t stride_t, int64_t batch, int64_t n_s, int64_t n_t, const int32_t *length,
                               float *scores, int32_t *paths, const int64_t *path_offsets, int32_t *path_len);

/* The same for two float32 series per pair (device memory): S(i, j) = |x[k * x_stride + i] -
 * y[k * y_stride + j]| computed in the DP kernel, never stored -- the cost matrix of DTW on
 * series (pyalign/problems/factory.py's distance-based problems with the absolute difference).
 * Replaces materialising the batch * n_s * n_t matrix for pa_solve_dense_paths; results are
 * identical (the kernel computes the same float32 difference).  Linear, affine or DTW solvers. */
pa_status pa_solve_series_paths(pa_solver *s, const float *x, int64_t x_stride, const float *y, int64_t y_stride,
                                int64_t batch, int64_t n_s, int64_t n_t, const int32_t *length, float *scores,
                                int32_t *paths, const int64_t *path_offsets, int32_t *path_len);

/* Backward: the max-plus subgradient of the optimal score.  Adds grad_scores[k] to dS at
 * every aligned (diagonal-step) cell of pair k's path -- every visited cell for DTW -- and
 * writes dgap[4k..4k+3] = d score / d (open_s, extend_s, open_t, extend_t) times
 * grad_scores[k], for w(len) = open + extend * (len - 1), border gaps of global paths
 * included.  paths/path_offsets/path_len as produced by pa_solve_dense_paths but ALL in
 * device memory, as are grad_scores, dS, ds_offsets and dgap (dS and dgap may be NULL).
 * Allocates nothing; runs on `stream`. */
pa_status pa_path_gradients(int32_t type, int32_t locality, int32_t direction, int64_t batch,
                            const int32_t *paths, const int64_t *path_offsets, const int32_t *path_len,
                            const float *grad_scores, float *dS, const int64_t *ds_offsets, int64_t stride_s,
                            int64_t stride_t, float *dgap, void *stream);

/* Embedding similarity S(i, j) = <en_s[i], en_t[j]> with en = E / |E| (normalize != 0,
 * cosine) or en = E (dot).  pa_normalize_rows_bf16 writes the BF16 factor en (rows x dim)
 * and 1/|E| per row (1 when not normalising) in one pass over E (rows x dim float32).
 * pa_path_embedding_gradients is the fused backward: for every aligned cell (i, j) of pair
 * k's path it writes dEs[i] and dEt[j] (the gradients w.r.t. the raw E, through the
 * normalisation), without materialising dS; other rows are left untouched (pass zeros).
 * Es/Et (batch, n, dim) float32, Es_bf16/Et_bf16 their BF16 factors, inv_s/inv_t the
 * inverse norms.  Device memory; allocates nothing. */
pa_status pa_normalize_rows_bf16(const float *E, int64_t rows, int32_t dim, int32_t normalize, void *out_bf16,
                                 float *inv_norm, void *stream);

/* pa_normalize_rows_bf16 for batch x n rows of a (batch, n, dim) tensor with each pair's
 * length (lengths: device, batch int32): rows i >= lengths[k] of pair k get a zero BF16 row
 * and 1/|E| = 0 without reading E (the padding rows of the product are zero).  E must be
 * 16-byte aligned when dim is a multiple of 4 (its rows are then read as 16-byte words). */
pa_status pa_normalize_rows_bf16_lengths(const float *E, int64_t batch, int64_t n, int32_t dim, int32_t normalize,
                                         const int32_t *lengths, void *out_bf16, float *inv_norm, void *stream);

/* pa_normalize_rows_bf16_lengths writing only the rows a product of `tile`-row tiles reads:
 * rows below each length as above, the rows from the length up to the next multiple of
 * `tile` zero, and the rows (and 1/|E| entries) beyond left unwritten. */
pa_status pa_normalize_rows_bf16_tiled(const float *E, int64_t batch, int64_t n, int32_t dim, int32_t normalize,
                                       const int32_t *lengths, int32_t tile, void *out_bf16, float *inv_norm,
                                       void *stream);

pa_status pa_path_embedding_gradients(int64_t batch, int32_t dim, int32_t normalize, const int32_t *paths,
                                      const int64_t *path_offsets, const int32_t *path_len,
                                      const float *grad_scores, const float *Es, const float *Et,
                                      const void *Es_bf16, const void *Et_bf16, const float *inv_s,
                                      const float *inv_t, int64_t n_s, int64_t n_t, float *dEs, float *dEt,
                                      void *stream);

/* pa_path_embedding_gradients writing every row of dEs and dEt: the rows without an aligned
 * cell (padding rows included) are set to zero, so the caller need not zero them first. */
pa_status pa_path_embedding_gradients_full(int64_t batch, int32_t dim, int32_t normalize, const int32_t *paths,
                                           const int64_t *path_offsets, const int32_t *path_len,
                                           const float *grad_scores, const float *Es, const float *Et,
                                           const void *Es_bf16, const void *Et_bf16, const float *inv_s,
                                           const float *inv_t, int64_t n_s, int64_t n_t, float *dEs, float *dEt,
                                           void *stream);

/* Fused backward of DTW on two series with d(u, v) = |x_u - y_v| (x: (batch, n_s),
 * y: (batch, n_t) float32): every visited cell adds grad * sign(x_u - y_v) to dx_u and
 * subtracts it from dy_v (per row and column: grad times the exact count of signs, adding to
 * dx and dy, which the caller zeroes).  Device memory; allocates nothing. */
pa_status pa_path_series_gradients(int64_t batch, const int32_t *paths, const int64_t *path_offsets,
                                   const int32_t *path_len, const float *grad_scores, const float *x,
                                   const float *y, int64_t n_s, int64_t n_t, float *dx, float *dy, void *stream);

/* Similarity matrices of per-token embeddings on the tensor cores (tcgen05, BF16 operands,
 * FP32 accumulation): St[k * pitch_pair + j * pitch_row + i] = beta + alpha * <Et[k, j],
 * Es[k, i]> (one rounding; alpha = 1, beta = 0 for the similarity itself, alpha = -1,
 * beta = 1 for the distance 1 - cos) for j < len_t[k], i < len_s[k]; other elements are not
 * written.  Es (batch, n_s, dim) and
 * Et (batch, n_t, dim) are row-major BF16 (16-byte aligned, dim a multiple of 16);
 * tile_start (batch + 1) holds the prefix sums of ceil(len_t / 128) * ceil(len_s / 128)
 * and total_tiles its last entry.  The dense similarity of MatrixForm problems
 * (pyalign/solve.py:342-379, factory.h:573-576), written transposed (S^T) so the DP reads it
 * with stride 1 along s; the oracle is a float64 product.  len_s, len_t, tile_start, St and
 * status are device memory; a wait that times out ORs 2 into *status.  Allocates nothing;
 * runs on `stream`. */
pa_status pa_similarity_bf16(const void *Es, const void *Et, int64_t batch, int64_t n_s, int64_t n_t, int32_t dim,
                             const int32_t *len_s, const int32_t *len_t, const int32_t *tile_start,
                             int64_t total_tiles, float *St, int64_t pitch_pair, int64_t pitch_row, float alpha,
                             float beta, int32_t *status, void *stream);

/* Score of each pair's recovered path re-evaluated in FP64: the similarities of its aligned
 * cells (every visited cell for DTW) plus or minus its gap costs w(k) = open + extend (k - 1),
 * border gaps of global paths included -- the float64 restatement of the score that the
 * float32 DP accumulated along the same path.  paths as from pa_solve_dense_paths (device);
 * sim read as sim[sim_offsets[k] + u * stride_s + v * stride_t]; gaps[4] = open_s, extend_s,
 * open_t, extend_t (host).  scale (device, may be NULL) receives the magnitude of the terms
 * the score sums -- sum |S| over those cells plus the path's total gap cost -- the natural
 * denominator of an error for scores near zero.  Allocates nothing; runs on `stream`. */
pa_status pa_path_scores_f64(int32_t type, int32_t locality, int32_t direction, int64_t batch, const int32_t *paths,
                             const int64_t *path_offsets, const int32_t *path_len, const float *sim,
                             const int64_t *sim_offsets, int64_t stride_s, int64_t stride_t, const double *gaps,
                             double *scores, double *scale, void *stream);

/* Device time of the phases of the last solve on this solver, in milliseconds
 * (0: upload, 1: DP kernels, 2: traceback kernels, 3: download), and the number of
 * kernels launched.  Measured with CUDA events on the solver's stream.  After a
 * device-resident paths solve (pa_solve_dense_paths, pa_solve_series_paths), which returns
 * without waiting, only the DP time is reported, and this call waits for the DP to end. */
pa_status pa_solver_last_timings(const pa_solver *s, float *ms4, int32_t *kernel_launches);

/* The DP plan of the last solve on this solver (diagnostic): plan4[0] = kernel family
 * (0: one column per lane step, 1: two columns per lane step, 2: stripe-chained, 3: packed
 * 16-bit twin pairs, one column per step, 4: general gap costs, 5: packed 16-bit twin pairs,
 * two columns per step, 6: packed 16-bit twin pairs on 4 x 4 blocks), plan4[1] = lanes per
 * pair group G, plan4[2] = arithmetic (0: float32, 1: int32, 2: packed int16), plan4[3] = 1
 * when the solve ran as a replayed CUDA graph.  No counterpart in the reference. */
pa_status pa_solver_last_plan(const pa_solver *s, int32_t *plan4);

/* The group width per length bucket of |s| (widths4[0..3] for |s| <= 128, <= 256, <= 512 and
 * longer) of the last solve on this solver, when its 16-bit twin launch gave each bucket a
 * width of its own; all four 0 when one width G (pa_solver_last_plan) served every pair.
 * Diagnostic; no counterpart in the reference. */
pa_status pa_solver_last_bucket_widths(const pa_solver *s, int32_t *widths4);

/* Bytes copied host->device and device->host by the last solve call of this solver
 * (inputs, per-pair metadata, results). */
pa_status pa_solver_last_bytes(const pa_solver *s, int64_t *h2d, int64_t *d2h);

/* Batch encoding of byte-alphabet sequences (replaces the per-problem encoding of pyalign's
 * prepare step, pyalign/solve.py:382-396 -> AlphabetProblem.build_index_sequences,
 * problems/factory.py:87-90 -> ByteAlphabetEncoder.encode, factory.py:114-127).  count
 * strings of latin1 bytes, string k = text[offsets[k] .. offsets[k+1]) (host), are mapped
 * through lut (256 entries, host; 0xff = not in the alphabet -- ByteAlphabetEncoder._index)
 * into row k of codes (row k at codes + k * row_stride, uint32), zero-padded to width.
 * location PA_HOST: codes is host memory, encoded by worker threads; PA_DEVICE: codes is
 * device memory, the bytes are uploaded once and encoded by a kernel on `stream`, and the
 * call waits for it.  Returns PA_ERR_INVALID_ARGUMENT ("item not in alphabet") when a byte
 * is not in the alphabet, PA_ERR_LENGTH when a string is longer than width.  No counterpart
 * in the reference's native module. */
pa_status pa_encode_latin1(const uint8_t *text, const int64_t *offsets, int64_t count, const uint8_t *lut, int64_t width,
                           int64_t row_stride, uint32_t *codes, int32_t location, void *stream);

/* Diagnostic: measured int32 throughput of this GPU (Gop/s) for the add/add/max mix of the
 * DP cell update, used as the denominator of the DP kernels' roofline.  No counterpart in
 * the reference (it has no GPU code). */
pa_status pa_measure_int32_peak(float *gops, float *ms);

/* Diagnostic: the same mix on packed 16-bit pairs (add.s16x2 / max.s16x2), counted as two
 * operations per instruction: the roofline denominator of the packed 16-bit twin kernel. */
pa_status pa_measure_int16x2_peak(float *gops, float *ms);

/* Diagnostic: the same mix in float32 (FADD, FADD, FMNMX): the roofline denominator of the
 * float DP kernels of the similarity-matrix and DTW forms. */
pa_status pa_measure_f32_peak(float *gops, float *ms);

/* ---- allocation-free score solve ----
 * No counterpart in the reference (its solver allocates its matrices on the host).
 * For callers that cannot allocate device memory while they run -- a process that owns
 * all of its HBM through a preallocated pool, or code where a cudaMalloc would stall or
 * fail mid-request.  Scores only (Solver::score, solver.h:2593-2608) of `batch` pairs in
 * the indexed form with linear or affine gap costs (o: type ALIGNMENT, direction,
 * locality, gap_kind and its costs; other fields ignored; the gap border vectors use the
 * capacity n_s x n_t).  Inputs a (batch x n_s), b (batch x n_t), table, len_s, len_t
 * (batch int32 each) and the output scores (batch float32) are device memory of the
 * caller; the work runs on `stream` (a cudaStream_t, NULL = default stream) and is
 * complete when the stream is.  The call blocks the calling thread until `stream` has run
 * the check that every code indexes the table (it synchronises `stream` once, after the
 * two index-range kernels, and then queues the DP without waiting for it), so an out-of-
 * range code is reported by the call itself (PA_ERR_INVALID_ARGUMENT).
 * All scratch lives in one static device array of PA_NOALLOC_SCRATCH_BYTES per device
 * (held until the process exits): batch <= PA_NOALLOC_MAX_BATCH, n_s, n_t <=
 * PA_NOALLOC_MAX_LEN and a table of at most 64 x 64; larger sizes are rejected with
 * PA_ERR_LENGTH.  Every call shares that array: calls whose GPU work overlaps race and
 * give wrong results.  The first call on a device looks up the array's address (once per
 * device, that device current) and so should come before any stream capture. */
#define PA_NOALLOC_SCRATCH_BYTES (32 * 1024 * 1024)
#define PA_NOALLOC_MAX_BATCH 65536
#define PA_NOALLOC_MAX_LEN 4096
pa_status pa_solve_indexed_for_score_noalloc(const pa_options *o, const uint32_t *a, const uint32_t *b,
                                             int64_t batch, int64_t n_s, int64_t n_t, const float *table,
                                             int64_t table_rows, int64_t table_cols, const int32_t *len_s,
                                             const int32_t *len_t, float *scores, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYALIGN_GB300_H */

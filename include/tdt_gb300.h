/*
 * tdt_gb300.h — C ABI of the GB300 (sm_103a) truss-decomposition library
 * (libtdt_gb300.so).
 *
 * Conventions
 *   - Every pointer argument is a DEVICE pointer unless its comment says host.
 *   - The caller allocates every buffer, as with the reference's `trusstensor`
 *     operators (the ops write their outputs in place and return nothing
 *     there); here each call returns an int status (TDT_OK == 0) and never
 *     allocates device memory itself.  Whole-path entry points take a
 *     caller-provided workspace whose size the matching *_workspace_bytes()
 *     query returns.
 *   - Work is enqueued on `stream` (a cudaStream_t; NULL = the legacy default
 *     stream, which is where the reference launches).  Calls are asynchronous;
 *     device-side failures (a bounded wait that expired) are reported in the
 *     device `stats` words described below.
 *   - Graph layout: the degree-oriented CSRCOO of the reference
 *     (src/type/CSRCOO.py:9-33): `rows`/`cols` int32[E] (edge i = rows[i] ->
 *     cols[i]), columns sorted within each row, `row_ptr` of the rows.  The
 *     drop-in operators take the reference's int32 tiled row_ptr
 *     (int32[V*n_cut+1], singlegpu_truss.py:160-169); the whole-path entry
 *     points take int64 row offsets int64[V+1] and require rows[i] < cols[i].
 */
#ifndef TDT_GB300_H
#define TDT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *tdt_stream_t; /* == cudaStream_t */

enum tdt_status {
    TDT_OK = 0,
    TDT_ERR_INVALID = 1,     /* bad argument (size, null pointer, n_cut < 1, ...) */
    TDT_ERR_CUDA = 2,        /* a CUDA runtime call failed                       */
    TDT_ERR_WORKSPACE = 3,   /* workspace smaller than *_workspace_bytes()       */
    TDT_ERR_TIMEOUT = 4,     /* a bounded device-side wait expired               */
    TDT_ERR_CAPACITY = 5,    /* an output capacity (e.g. ptr_truss_cap) too small */
    TDT_ERR_UNSUPPORTED = 6, /* device or configuration not supported            */
    TDT_ERR_NOT_ORIENTED = 7 /* an edge with rows[i] >= cols[i]                  */
};

/* Human-readable text of a status code, and detail of the last error raised
 * on the calling host thread. */
const char *tdt_status_string(int status);
const char *tdt_last_error(void);
int tdt_version(void);
/* Number of kernels this library has launched in the process so far. */
unsigned long long tdt_launch_count(void);

/* Phase timing of the whole-path calls: after tdt_profile_start(n), the next
 * n calls record CUDA events on their stream; tdt_profile_stop() waits for
 * them and writes the summed milliseconds of four phases to ms_phase[4]
 * (host): [0] the support pass, [1] the triangle-listing pass, [2] the peel
 * (in-adjacency build and the persistent peel kernel), [3] the outputs; and
 * the number of calls recorded to *ncalls.  The recording is process-wide:
 * start and stop it while no other thread makes whole-path calls. */
int tdt_profile_start(int max_calls);
int tdt_profile_stop(float *ms_phase, int *ncalls);

/* Block 0's clock of the last decomposition or k-truss search run in
 * `workspace` (diagnostic): ns[0] candidate processing, ns[1] grid-barrier
 * waits after processing, ns[2] level changes, ns[3] the whole persistent
 * peel kernel.  Synchronises `stream`.  The phases also appear as NVTX
 * ranges ("tdt support", "tdt listing", "tdt peel", "tdt outputs") when a
 * profiler is attached.  The reference times its phases with host clocks
 * around synchronize calls (demo_truss/singlegpu_truss.py:69-77, :153-157). */
int tdt_peel_clock(const void *workspace, long long *ns, cudaStream_t stream);

/* Testing knob of the support/listing kernels: rows with out-degree <=
 * warp_cap are processed by one warp, heavier rows by a block with the row
 * staged in shared memory up to heavy_cap entries, and beyond that in place.
 * Lower values let small graphs exercise every path; 0 restores the
 * defaults.  Affects calls launched afterwards from any thread. */
void tdt_set_support_caps(int warp_cap, int heavy_cap);

/* Testing knob of the support/listing kernels: 0 makes their wedge walk load
 * one column index per lane and step, 1 (the default) four at a time from
 * 16-byte chunks (used when the columns array is 16-byte aligned and the
 * graph has fewer than 2^30 edges).  Results do not depend on it.  Affects
 * calls launched afterwards from any thread. */
void tdt_set_vector_walk(int on);

/* Knob of the support/listing kernels: 1 stages the rows that a whole block
 * walks (out-degree above 256) into shared memory by one bulk copy
 * (cp.async.bulk, tracked by an mbarrier with a bounded wait) plus plain
 * loads of the ragged ends; 0 (the default) loads them with plain loads.
 * Needs the vectorised walk.  Results do not depend on it.  Affects calls
 * launched afterwards from any thread. */
void tdt_set_bulk_staging(int on);

/* Knob of the persistent peel (no counterpart in the reference): its grid in
 * units of half the SM count (1 = one block per two SMs, 2 = one per SM, 4 =
 * two per SM, capped by what stays resident); 0 (the default) restores the
 * size heuristic (half the SMs under 2^18 edges with lists, one block per SM
 * under 2^22, otherwise every resident block).  The autotuner's launch-shape
 * dimension.  Results do not depend on it.  Affects calls launched
 * afterwards from any thread. */
void tdt_set_peel_grid(int half_sms);

/* Testing knobs of the failure paths (no counterpart in the reference, which
 * has no bounded waits).  tdt_set_peel_deadline_ns: wall-clock budget of the
 * peel launches that follow (<= 0 restores the default of 120 s); a run past
 * it stops between sub-rounds with TDT_ERR_TIMEOUT in its stats.
 * tdt_test_barrier_timeout: launches 8 blocks at a grid barrier that one of
 * them never reaches; the others give up after limit_ns (1 ms .. 2 s) and the
 * call returns the device status, TDT_ERR_TIMEOUT.  workspace: >= 4096 bytes
 * of device memory.  Blocks the calling thread until the kernel ends. */
void tdt_set_peel_deadline_ns(long long ns);

/* Testing knob of tdt_ktruss_search: the low-support edges that start the
 * peel are queued in batches of at most `items` edges and `cands` candidate
 * slots per sub-round (defaults 2^27 and 2^35, for graphs whose low-support
 * edges outnumber the queue); lower values let small graphs run several
 * batches.  <= 0 restores a default.  Results do not depend on it. */
void tdt_set_ktruss_batch_caps(long long items, long long cands);
/* Testing knob of the peel without triangle lists (no counterpart in the
 * reference): sub-rounds of at least `slots` candidate slots are split among
 * the warps in 256-slot ranges taken from a shared cursor instead of one
 * equal range per warp (default 2^20; lower values take the dynamic split on
 * small graphs).  <= 0 restores the default.  Results do not depend on it. */
void tdt_set_peel_dynamic_min(long long slots);
int tdt_test_barrier_timeout(void *workspace, long long limit_ns, cudaStream_t stream);

/* =====================================================================
 * Drop-in `trusstensor` operators.
 * Each replaces the pybind op of the same name in
 * demo_truss/myops/mysrc/hpu_extension/myhpu_extension.cpp:572-593; the
 * argument order is the reference's, with sizes made explicit.
 * ===================================================================== */

/* segment_add (myhpu_extension.cpp:8-16; kernel.cu:5-26):
 * output[r] = sum(col_indices[col_ptr[r]:col_ptr[r+1]]) for every non-empty
 * row r < num_rows; rows with an empty segment are left untouched.
 * num_values = length of col_indices (segments are clamped to it). */
int tdt_segment_add(const int32_t *col_indices, int64_t num_values, const int32_t *col_ptr,
                    int32_t *output, int64_t num_rows, tdt_stream_t stream);

/* segment_isin2 (myhpu_extension.cpp:24-34; kernel.cu:28-79) and
 * segment_isin2tile (myhpu_extension.cpp:43-56; kernel.cu:81-141):
 * output[i] += number of triangles containing edge i (its support).
 * ACCUMULATES into output, as the reference does.  b_row_ptr holds
 * row_ptr_len = V*n_cut+1 entries (n_cut = 1 for segment_isin2).
 * Input contract (the reference's): a valid CSRCOO without -1 sentinels. */
int tdt_segment_isin2(const int32_t *a_rows, const int32_t *b_col_indices,
                      const int32_t *b_row_ptr, int64_t row_ptr_len, int32_t *output,
                      int64_t num_edges, tdt_stream_t stream);
int tdt_segment_isin2tile(const int32_t *a_rows, const int32_t *b_col_indices,
                          const int32_t *b_row_ptr, int64_t row_ptr_len, int32_t n_cut,
                          int32_t *output, int64_t num_edges, tdt_stream_t stream);

/* sub_AllAffectedSupport (myhpu_extension.cpp:70-86; kernel.cu:144-191) and
 * sub_AllAffectedSupport_tile (myhpu_extension.cpp:162-177; kernel.cu:407-456):
 * `mark` = deleted edges.  For each affected edge e and each triangle of e
 * whose third column is live (not -1) and that has a deleted edge: the two
 * wedge edges still above l are decremented and flagged in n_mark; e, when
 * not deleted, is decremented by the number of such triangles and flagged. */
int tdt_sub_all_affected_support(const int32_t *e_affect, int64_t num_affect,
                                 const int32_t *a_rows, const int32_t *b_col_indices,
                                 const int32_t *b_row_ptr, int64_t row_ptr_len,
                                 const uint8_t *mark, int32_t l, uint8_t *n_mark,
                                 int32_t *output, int64_t num_edges, tdt_stream_t stream);
int tdt_sub_all_affected_support_tile(const int32_t *e_affect, int64_t num_affect,
                                      const int32_t *a_rows, const int32_t *b_col_indices,
                                      const int32_t *b_row_ptr, int64_t row_ptr_len, int32_t n_cut,
                                      const uint8_t *mark, int32_t l, uint8_t *n_mark,
                                      int32_t *output, int64_t num_edges, tdt_stream_t stream);

/* sub_AllAffectedSupport_not (myhpu_extension.cpp:93-106; kernel.cu:220-273)
 * and sub_AllAffectedSupport_tilenot (myhpu_extension.cpp:191-205;
 * kernel.cu:492-547), the peel update of the `--cuda` flow:
 * `mark` = alive and not peeled this round.  A triangle of affected edge e
 * with a live third column is destroyed when not all of its three edges are
 * in `mark`: each wedge edge above l loses one and is flagged in n_mark when
 * it reaches l; e, when in `mark`, loses the number of destroyed triangles
 * and is flagged when it ends at or below l.  Supports that end at or below l
 * are racy in the reference and here alike; n_mark and supports above l are
 * exact. */
int tdt_sub_all_affected_support_not(const int32_t *e_affect, int64_t num_affect,
                                     const int32_t *a_rows, const int32_t *b_col_indices,
                                     const int32_t *b_row_ptr, int64_t row_ptr_len,
                                     const uint8_t *mark, int32_t l, uint8_t *n_mark,
                                     int32_t *output, int64_t num_edges, tdt_stream_t stream);
int tdt_sub_all_affected_support_tilenot(const int32_t *e_affect, int64_t num_affect,
                                         const int32_t *a_rows, const int32_t *b_col_indices,
                                         const int32_t *b_row_ptr, int64_t row_ptr_len,
                                         int32_t n_cut, const uint8_t *mark, int32_t l,
                                         uint8_t *n_mark, int32_t *output, int64_t num_edges,
                                         tdt_stream_t stream);

/* sub_AllAffectedSupport_notwin (myhpu_extension.cpp:123-140; kernel.cu:302-370)
 * and _tilenotwin (myhpu_extension.cpp:224-242; kernel.cu:578-648): the _not
 * update that also flags, in in_windows_mask, every edge whose support
 * crosses below windows_high and appends its index to buff_index at
 * atomicAdd(buf_size, 1).  buff_index must hold num_edges entries. */
int tdt_sub_all_affected_support_notwin(const int32_t *e_affect, int64_t num_affect,
                                        const int32_t *a_rows, const int32_t *b_col_indices,
                                        const int32_t *b_row_ptr, int64_t row_ptr_len,
                                        const uint8_t *mark, int32_t l, uint8_t *n_mark,
                                        int32_t *output, int32_t windows_high,
                                        uint8_t *in_windows_mask, int32_t *buff_index,
                                        int32_t *buf_size, int64_t num_edges,
                                        tdt_stream_t stream);
int tdt_sub_all_affected_support_tilenotwin(const int32_t *e_affect, int64_t num_affect,
                                            const int32_t *a_rows, const int32_t *b_col_indices,
                                            const int32_t *b_row_ptr, int64_t row_ptr_len,
                                            int32_t n_cut, const uint8_t *mark, int32_t l,
                                            uint8_t *n_mark, int32_t *output,
                                            int32_t windows_high, uint8_t *in_windows_mask,
                                            int32_t *buff_index, int32_t *buf_size,
                                            int64_t num_edges, tdt_stream_t stream);

/* k-truss search operators.  The reference launches these from pycuda
 * (ktruss_search/ktruss_cuda.py:316-343); they are not in its trusstensor
 * module.  Mapping: run_kernel_two_k -> tdt_segment_isin2_k,
 * run_kernel_two_tile_k -> tdt_segment_isin2tile_k, run_affect_support ->
 * tdt_sub_affected_support, run_affect_support_tile ->
 * tdt_sub_affected_support_tile.
 *
 * segment_isin2_k (ktruss_cuda.py:121-200): the support count that stops
 * incrementing a target once it has reached k (accumulates into output).
 * sub_affected_support (ktruss_cuda.py:201-286): on an extracted subgraph,
 * every unmarked edge loses one per triangle that has a marked edge. */
int tdt_segment_isin2_k(const int32_t *a_rows, const int32_t *b_col_indices,
                        const int32_t *b_row_ptr, int64_t row_ptr_len, int32_t k,
                        int32_t *output, int64_t num_edges, tdt_stream_t stream);
int tdt_segment_isin2tile_k(const int32_t *a_rows, const int32_t *b_col_indices,
                            const int32_t *b_row_ptr, int64_t row_ptr_len, int32_t n_cut,
                            int32_t k, int32_t *output, int64_t num_edges, tdt_stream_t stream);
int tdt_sub_affected_support(const int32_t *sub_rows, const int32_t *sub_columns,
                             const int32_t *sub_row_ptr, int64_t row_ptr_len,
                             const uint8_t *mark, int32_t *sub_support, int64_t num_edges,
                             tdt_stream_t stream);
int tdt_sub_affected_support_tile(const int32_t *sub_rows, const int32_t *sub_columns,
                                  const int32_t *sub_row_ptr, int64_t row_ptr_len, int32_t n_cut,
                                  const uint8_t *mark, int32_t *sub_support, int64_t num_edges,
                                  tdt_stream_t stream);

/* Research-variant operators (the reference's `tensor_original` and
 * `undirected` drivers; none is on the `--cuda` flow).  Row-pointer arrays are
 * int32, as the reference's ops read them.  Two lists pair up exactly as the
 * reference's two-pointer merge pairs them, whatever their order: strictly
 * increasing lists take a shared-memory hash path, any others a one-lane
 * merge walk.
 *
 * segment_isinis_m (myhpu_extension.cpp:255-265; kernel.cu:687-737): for each
 * row r < num_rows, the positions of the values rows r of a and b share, -1
 * excepted, are set in mask1 (over a_columns) and mask2 (over b_columns).
 * Both row-pointer arrays hold num_rows + 1 entries.
 * segment_isinmm (myhpu_extension.cpp:555-565; kernel.cu:1555-1607): the same
 * without the -1 exception. */
int tdt_segment_isinis_m(const int32_t *a_columns, int64_t a_len, const int32_t *a_row_ptr,
                         const int32_t *b_columns, int64_t b_len, const int32_t *b_row_ptr,
                         int64_t num_rows, uint8_t *mask1, uint8_t *mask2, tdt_stream_t stream);
int tdt_segment_isinmm(const int32_t *u_clos, int64_t u_len, const int32_t *v_clos, int64_t v_len,
                       const int32_t *uptr, const int32_t *vptr, int64_t num_rows, uint8_t *u_mask,
                       uint8_t *v_mask, tdt_stream_t stream);

/* sub_suppport_affect (myhpu_extension.cpp:284-296; kernel.cu:739-805): for
 * triangle i of a current edge e_curr_rep[i] with partner edges left_nbr[i]
 * and right_nbr[i] (mask1/mask2: that partner takes part): both flagged ->
 * both lose one; left only -> left loses one when e_curr_rep[i] < right;
 * right only -> right loses one when e_curr_rep[i] < left.  Every decremented
 * edge is set in e_affect_mask.  l is accepted and unused, as in the
 * reference. */
int tdt_sub_suppport_affect(const int32_t *left_nbr, const int32_t *right_nbr, const int32_t *e_curr_rep,
                            int64_t num_triangles, int32_t *support, int64_t num_edges,
                            const uint8_t *mask1, const uint8_t *mask2, uint8_t *e_affect_mask,
                            int32_t l, tdt_stream_t stream);

/* Oriented / undirected peel updates (myhpu_extension.cpp:316-539;
 * kernel.cu:808-1551).  For each current edge e = (rows[e], columns[e]) and
 * tile k < n_cut (1 for the untiled forms), the third vertices of its
 * triangles are the keys two lists share:
 *   peeling_undirect  symmetric adjacency of both ends (columns_g, edge ids
 *                     edges_id_nbr, offsets row_ptr[v * n_cut + k]);
 *   peeling_direct_oo out-lists of both ends (columns, offsets row_ptr);
 *   peeling_direct_ii in-lists of both ends (edge ids r_edges grouped by head,
 *                     keys rows[r_edges[i]], offsets re_ptr);
 *   peeling_direct_oi out-list of the tail, in-list of the head.
 * A shared key whose two edges e2 (first list) and e3 (second) are both in
 * e_mask: neither in in_curr -> both lose one; only e3 in in_curr -> e2 loses
 * one (undirect: when e < e3; ii: never); only e2 in in_curr -> e3 loses one
 * (oo always; undirect when e < e2; ii, oi never).  An edge whose support
 * goes from l + 1 to l is set in n_mark (the reference's op hands l + 1 to its
 * kernel; pass the level l here as there).  Decrements are exact atomics, so
 * supports and n_mark do not depend on thread order. */
int tdt_peeling_undirect(const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                         const int32_t *columns, const int32_t *columns_g, const int32_t *row_ptr,
                         int64_t row_ptr_len, const int32_t *edges_id_nbr, int64_t g_len,
                         int32_t *support, const uint8_t *e_mask, uint8_t *n_mark,
                         const uint8_t *in_curr, int32_t l, int64_t num_edges, tdt_stream_t stream);
int tdt_peeling_undirect_tile(const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                              const int32_t *columns, const int32_t *columns_g, const int32_t *row_ptr,
                              int64_t row_ptr_len, const int32_t *edges_id_nbr, int64_t g_len,
                              int32_t *support, const uint8_t *e_mask, uint8_t *n_mark,
                              const uint8_t *in_curr, int32_t l, int32_t n_cut, int64_t num_edges,
                              tdt_stream_t stream);
int tdt_peeling_direct_oo(const int32_t *e_curr, int64_t n_curr, const int32_t *rows, const int32_t *columns,
                          const int32_t *row_ptr, int64_t row_ptr_len, int32_t *support,
                          const uint8_t *e_mask, uint8_t *n_mark, const uint8_t *in_curr, int32_t l,
                          int64_t num_edges, tdt_stream_t stream);
int tdt_peeling_direct_tile_oo(const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                               const int32_t *columns, const int32_t *row_ptr, int64_t row_ptr_len,
                               int32_t *support, const uint8_t *e_mask, uint8_t *n_mark,
                               const uint8_t *in_curr, int32_t l, int32_t n_cut, int64_t num_edges,
                               tdt_stream_t stream);
int tdt_peeling_direct_ii(const int32_t *e_curr, int64_t n_curr, const int32_t *rows, const int32_t *columns,
                          const int32_t *r_edges, const int32_t *re_ptr, int64_t re_ptr_len,
                          int32_t *support, const uint8_t *e_mask, uint8_t *n_mark,
                          const uint8_t *in_curr, int32_t l, int64_t num_edges, tdt_stream_t stream);
int tdt_peeling_direct_tile_ii(const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                               const int32_t *columns, const int32_t *r_edges, const int32_t *re_ptr,
                               int64_t re_ptr_len, int32_t *support, const uint8_t *e_mask,
                               uint8_t *n_mark, const uint8_t *in_curr, int32_t l, int32_t n_cut,
                               int64_t num_edges, tdt_stream_t stream);
int tdt_peeling_direct_oi(const int32_t *e_curr, int64_t n_curr, const int32_t *rows, const int32_t *columns,
                          const int32_t *row_ptr, int64_t row_ptr_len, const int32_t *r_edges,
                          const int32_t *re_ptr, int64_t re_ptr_len, int32_t *support,
                          const uint8_t *e_mask, uint8_t *n_mark, const uint8_t *in_curr, int32_t l,
                          int64_t num_edges, tdt_stream_t stream);
int tdt_peeling_direct_tile_oi(const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                               const int32_t *columns, const int32_t *row_ptr, int64_t row_ptr_len,
                               const int32_t *r_edges, const int32_t *re_ptr, int64_t re_ptr_len,
                               int32_t *support, const uint8_t *e_mask, uint8_t *n_mark,
                               const uint8_t *in_curr, int32_t l, int32_t n_cut, int64_t num_edges,
                               tdt_stream_t stream);

/* =====================================================================
 * Whole-path entry points (the device-resident hot path).
 * ===================================================================== */

/* Preprocessing: raw edge list -> degree-oriented CSRCOO on the device.
 * Restates read_prepro_save (singlegpu_truss.py:172-178): Graph.read_edgelist
 * (src/type/Graph_Truss.py:177-213: drop self-loops, dedup unordered pairs,
 * rank vertices by degree) + CSRCOO.edge_list_to_Graph / counter_sort
 * (src/type/CSRCOO.py:128-177: relabel by rank, orient low->high, CSR sorted
 * by (row, column)).  Degree ties go to the smaller id (the reference's numpy
 * argsort is unstable); with vertex_group (int32[num_ids], may be NULL) the
 * rank key is (group, degree, id), so a batch of graphs keeps contiguous
 * ranges.  Inputs: src/dst int32[num_draws] with ids in [0, num_ids).
 * Outputs: rows/cols int32[num_draws] (first E_out used), row_ptr
 * int64[num_ids+1] (first V_out+1 used), vertices int32[num_ids] (original id
 * of each rank), counts int64[3] = {E_out, V_out, status} (device).  No host
 * synchronisation inside. */
size_t tdt_preprocess_workspace_bytes(int64_t num_draws, int64_t num_ids);
int tdt_preprocess(const int32_t *src, const int32_t *dst, int64_t num_draws, int64_t num_ids,
                   const int32_t *vertex_group, int32_t num_groups, int32_t *rows, int32_t *cols,
                   int64_t *row_ptr, int32_t *vertices, int64_t *counts, void *workspace,
                   size_t workspace_bytes, tdt_stream_t stream);

/* Layout of the int64 `stats` words the whole-path calls write (device). */
enum tdt_stat_index {
    TDT_STAT_STATUS = 0,     /* 0 = ok, else a tdt_status raised on the device */
    TDT_STAT_KMAX = 1,       /* maximum truss number (2 for a triangle-free graph) */
    TDT_STAT_NPTR = 2,       /* entries written to ptr_truss                   */
    TDT_STAT_ROUNDS = 3,     /* peel sub-rounds executed                       */
    TDT_STAT_TRIANGLES = 4,  /* triangle count                                 */
    TDT_STAT_NETRUSS = 5,    /* entries written to e_truss                     */
    TDT_STAT_ALIVE = 6,      /* k-truss search: edges left in the k-truss      */
    TDT_STAT_LISTED = 7,     /* how the peel found each peeled edge's triangles: 0 by search in
                                the adjacency; per-edge triangle lists, 1 written by a second walk,
                                2 packed from the one walk that also counted them */
    TDT_STAT_COUNT = 8
};

/* Workspace for tdt_truss_decompose / tdt_ktruss_search / tdt_triangle_count.
 * Workspace bytes beyond this size (rounded up to 256), the list tail, hold
 * per-edge triangle lists: when 24 * T bytes fit there (T = triangle count),
 * the peel reads each peeled edge's triangles from its list; otherwise it
 * finds them by binary search in the adjacency.  When the tail also holds the
 * staging area of the one walk (8 bytes per slot of the per-edge bounds
 * min(d+(u)-i-1, d+(v)) + min(i, d-(v)-1), edge (u,v) at position i of row
 * u), one walk counts the triangles and writes the lists; otherwise a
 * count-only walk runs first and a second walk writes them.  Results are
 * identical every way. */
size_t tdt_decompose_workspace_bytes(int64_t num_vertices, int64_t num_edges);

/* Full truss decomposition: the single-call replacement of the `--cuda` flow
 * k_truss (singlegpu_truss.py:67-158) together with its support pass
 * (:38-45).  Outputs:
 *   truss[E]      per-edge truss number (2 = in no triangle);
 *   e_truss[E]    the reference's peel order: edges of level 1, 2, ... with,
 *                 within each sub-round, ascending edge index (support-0 edges
 *                 are not listed, as in the reference) — may be NULL;
 *   ptr_truss     per-level offsets into e_truss (ptr_truss[0] = 0; level i
 *                 = truss i+2 spans ptr_truss[i-1]..ptr_truss[i]); capacity
 *                 ptr_truss_cap entries, may be NULL;
 *   stats[8]      see tdt_stat_index (kmax = truss number of the last level).
 * `rows` may be NULL (derived from row_ptr).  Requires rows[i] < cols[i]. */
int tdt_truss_decompose(const int32_t *rows, const int32_t *cols, const int64_t *row_ptr,
                        int64_t num_vertices, int64_t num_edges, int32_t *truss,
                        int32_t *e_truss, int32_t *ptr_truss, int64_t ptr_truss_cap,
                        int64_t *stats, void *workspace, size_t workspace_bytes,
                        tdt_stream_t stream);

/* Triangle count: support[E] (overwritten, may be NULL) and
 * stats[TDT_STAT_TRIANGLES] = sum(support) / 3 (kernel.cu:28-79 semantics;
 * the reference derives the count as support.sum() // 3). */
int tdt_triangle_count(const int32_t *cols, const int64_t *row_ptr, int64_t num_vertices,
                       int64_t num_edges, int32_t *support, int64_t *stats, void *workspace,
                       size_t workspace_bytes, tdt_stream_t stream);

/* Triangle count that allocates no device memory.  It has no counterpart in
 * the reference; it is for callers that cannot call cudaMalloc where they
 * need the count (another component owns the device allocator, or the path
 * must not stall on an allocation).  Same outputs as tdt_triangle_count
 * (support may be NULL; stats[TDT_STAT_TRIANGLES], stats[TDT_STAT_STATUS]),
 * but the scratch is a fixed 40 MiB array inside the library, held on every
 * GPU that loads it until the process exits.  Limit: at most 2^18 vertices
 * and 2^18 edges; larger graphs return TDT_ERR_INVALID (use
 * tdt_triangle_count).  The first call on a device looks up that array's
 * address (cudaGetSymbolAddress) with the device current; make that first
 * call before any stream capture, and do not call it across a
 * cudaDeviceReset (the cached address would be stale).  All calls share the
 * array and each call re-initialises what it uses, so two calls that overlap
 * on the same GPU (for example on two streams) race on it and must be
 * serialised by the caller. */
int tdt_triangle_count_noalloc(const int32_t *cols, const int64_t *row_ptr, int64_t num_vertices,
                               int64_t num_edges, int32_t *support, int64_t *stats, tdt_stream_t stream);

/* k-truss search (ktruss_search/ktruss_cuda.py:383-463 with l = k-2):
 * in_ktruss[i] = 1 when edge i belongs to the k-truss, else 0;
 * stats[TDT_STAT_ALIVE] = its edge count. */
int tdt_ktruss_search(const int32_t *rows, const int32_t *cols, const int64_t *row_ptr,
                      int64_t num_vertices, int64_t num_edges, int32_t k, uint8_t *in_ktruss,
                      int64_t *stats, void *workspace, size_t workspace_bytes,
                      tdt_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* TDT_GB300_H */

/*
 * TEST INFRASTRUCTURE ONLY — the oracle.
 *
 * A plain-C (OpenMP) restatement of the TDT reference's CPU/CUDA algorithm for
 * the truss-decomposition hot path.  It exists to check the GPU path, never to
 * be the product: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg / `--impl reference` arm may load it.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).  The operators follow the reference's
 * one-work-item-per-edge merge loops; the drivers follow the Python flows
 * step by step (same frontier selection, same compaction threshold), so the
 * timed CPU baseline pays the reference algorithm's own costs.
 *
 * Racy reads in the reference kernels (`if (output[x] > l) atomicSub(...)`)
 * are OpenMP atomic reads here; the results that are deterministic in the
 * reference (n_mark, supports > l, peel sets) are deterministic here too.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* Operators                                                            */
/* ------------------------------------------------------------------ */

/* myhpu_extension_opmp.cpp:4-24 (segment_add_cpu): out[r] = sum of
 * col_indices[col_ptr[r]:col_ptr[r+1]]; rows with an empty segment are left
 * untouched. */
ORC_API void orc_segment_add(const int32_t *col_indices, const int32_t *col_ptr,
                             int32_t *out, int64_t num_rows) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < num_rows; r++) {
        int32_t s = col_ptr[r], e = col_ptr[r + 1];
        if (s < e) {
            int32_t sum = 0;
            for (int32_t i = s; i < e; i++) sum += col_indices[i];
            out[r] = sum;
        }
    }
}

/* Merge of two sorted adjacency ranges; for every common column calls the
 * body.  Shared by the support/peel restatements below (kernel.cu:43-57). */
#define ORC_MERGE(COLS, A0, A1, B0, B1, ...)                                  \
    do {                                                                      \
        int64_t ia_ = (A0), ea_ = (A1), ib_ = (B0), eb_ = (B1);               \
        while (ia_ < ea_ && ib_ < eb_) {                                      \
            int32_t ca_ = (COLS)[ia_], cb_ = (COLS)[ib_];                     \
            if (ca_ == cb_) {                                                 \
                int64_t pa = ia_, pb = ib_;                                   \
                int32_t cw = ca_;                                             \
                (void)cw; (void)pa; (void)pb;                                 \
                __VA_ARGS__;                                                  \
                ia_++; ib_++;                                                 \
            } else if (ca_ < cb_) {                                           \
                ia_++;                                                        \
            } else {                                                          \
                ib_++;                                                        \
            }                                                                 \
        }                                                                     \
    } while (0)

static inline void atomic_add_i32(int32_t *p, int32_t v) {
#pragma omp atomic
    *p += v;
}
static inline int32_t atomic_read_i32(const int32_t *p) {
    int32_t v;
#pragma omp atomic read
    v = *p;
    return v;
}
static inline int32_t atomic_fetch_sub_i32(int32_t *p, int32_t v) {
    int32_t old;
#pragma omp atomic capture
    { old = *p; *p -= v; }
    return old;
}
static inline int32_t atomic_fetch_add_i32(int32_t *p, int32_t v) {
    int32_t old;
#pragma omp atomic capture
    { old = *p; *p += v; }
    return old;
}

/* Tiled addressing (kernel.cu:86-95): work item `row` = edge i = row / n_cut,
 * tile j = row % n_cut; A = tile j of the head vertex, B = tile j of the tail.
 * n_cut == 1 is the untiled operator (kernel.cu:33-40). */
#define ORC_TILE_BOUNDS(I, J)                                                 \
    int64_t colv_ = (int64_t)cols[(I)] * n_cut + (J);                         \
    int64_t rowv_ = (int64_t)a_rows[(I)] * n_cut + (J);                       \
    int64_t a0 = rp[colv_], a1 = rp[colv_ + 1];                               \
    int64_t b0 = rp[rowv_], b1 = rp[rowv_ + 1];

/* myhpu_extension_opmp.cpp:26-59 (n_cut == 1) and :61-97 (tiled):
 * for edge i and every common out-neighbour w of its endpoints, +1 on the two
 * wedge edges and +count on i.  Accumulates into out. */
ORC_API void orc_segment_isin2tile(const int32_t *a_rows, const int32_t *cols,
                                   const int32_t *rp, int32_t n_cut,
                                   int32_t *out, int64_t num_edges) {
    int64_t n = num_edges * n_cut;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t row = 0; row < n; row++) {
        int64_t i = row / n_cut;
        int32_t j = (int32_t)(row % n_cut);
        ORC_TILE_BOUNDS(i, j)
        int32_t count = 0;
        ORC_MERGE(cols, a0, a1, b0, b1, {
            atomic_add_i32(&out[pa], 1);
            atomic_add_i32(&out[pb], 1);
            count++;
        });
        atomic_add_i32(&out[i], count);
    }
}

/* ktruss_search/ktruss_cuda.py:121-200 (checkElementsTwoPtr_k / ..Tile_k):
 * the support count saturating at k: increments only while the target is
 * below k; the edge's own count is added only while it is below k. */
ORC_API void orc_segment_isin2tile_k(const int32_t *a_rows, const int32_t *cols,
                                     const int32_t *rp, int32_t n_cut, int32_t k,
                                     int32_t *out, int64_t num_edges) {
    int64_t n = num_edges * n_cut;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t row = 0; row < n; row++) {
        int64_t i = row / n_cut;
        int32_t j = (int32_t)(row % n_cut);
        ORC_TILE_BOUNDS(i, j)
        int32_t count = 0;
        ORC_MERGE(cols, a0, a1, b0, b1, {
            if (atomic_read_i32(&out[pa]) < k) atomic_add_i32(&out[pa], 1);
            if (atomic_read_i32(&out[pb]) < k) atomic_add_i32(&out[pb], 1);
            count++;
        });
        if (count > 0 && atomic_read_i32(&out[i]) < k) atomic_add_i32(&out[i], count);
    }
}

/* myhpu_extension_opmp.cpp:99-152 (n_cut == 1) and :154-209 (tiled):
 * `mark` = deleted.  For a triangle of affected edge e with a live third
 * column and any deleted edge, decrement the wedge edges still above l and
 * mark them; decrement e by the count of such triangles when e is not
 * deleted, and mark it. */
ORC_API void orc_all_affected_support_tile(const int32_t *e_affect, int64_t n_affect,
                                           const int32_t *a_rows, const int32_t *cols,
                                           const int32_t *rp, int32_t n_cut,
                                           const uint8_t *mark, int32_t l,
                                           uint8_t *n_mark, int32_t *out) {
    int64_t n = n_affect * n_cut;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t row = 0; row < n; row++) {
        int64_t i = row / n_cut;
        int32_t j = (int32_t)(row % n_cut);
        int64_t e = e_affect[i];
        ORC_TILE_BOUNDS(e, j)
        int32_t count = 0;
        ORC_MERGE(cols, a0, a1, b0, b1, {
            if (cw != -1 && (mark[e] || mark[pa] || mark[pb])) {
                if (atomic_read_i32(&out[pa]) > l) { atomic_add_i32(&out[pa], -1); n_mark[pa] = 1; }
                if (atomic_read_i32(&out[pb]) > l) { atomic_add_i32(&out[pb], -1); n_mark[pb] = 1; }
                if (!mark[e]) count++;
            }
        });
        if (count > 0) { atomic_add_i32(&out[e], -count); n_mark[e] = 1; }
    }
}

/* myhpu_extension_kernel.cu:220-273 (n_cut == 1) and :492-547 (tiled), the
 * optimised peel update.  `mark` = alive and not being peeled this round.
 * A triangle is destroyed when not all three edges are in `mark`; wedge
 * edges above l lose one and are marked when they reach l; e (if in mark)
 * loses its count and is marked when it ends at or below l.
 * With windows (kernel.cu:302-370, :578-648): crossings of windows_high also
 * set in_windows_mask and append to buff_index. */
static void orc_affected_not_impl(const int32_t *e_affect, int64_t n_affect,
                                  const int32_t *a_rows, const int32_t *cols,
                                  const int32_t *rp, int32_t n_cut,
                                  const uint8_t *mark, int32_t l, uint8_t *n_mark,
                                  int32_t *out, int use_win, int32_t windows_high,
                                  uint8_t *in_win, int32_t *buff_index, int32_t *buf_size) {
    int64_t n = n_affect * n_cut;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t row = 0; row < n; row++) {
        int64_t i = row / n_cut;
        int32_t j = (int32_t)(row % n_cut);
        int64_t e = e_affect[i];
        ORC_TILE_BOUNDS(e, j)
        int32_t count = 0;
        ORC_MERGE(cols, a0, a1, b0, b1, {
            if (cw != -1 && !(mark[e] && mark[pa] && mark[pb])) {
                int64_t wedge[2] = {pa, pb};
                for (int q = 0; q < 2; q++) {
                    int64_t x = wedge[q];
                    if (atomic_read_i32(&out[x]) > l) {
                        int32_t temp = atomic_fetch_sub_i32(&out[x], 1);
                        if (temp - 1 == l) n_mark[x] = 1;
                        if (use_win && temp == windows_high) {
                            in_win[x] = 1;
                            int32_t slot = atomic_fetch_add_i32(buf_size, 1);
                            buff_index[slot] = (int32_t)x;
                        }
                    }
                }
                if (mark[e]) count++;
            }
        });
        if (count > 0) {
            int32_t temp = atomic_fetch_sub_i32(&out[e], count);
            if (temp - count <= l) n_mark[e] = 1;
            if (use_win && temp - count < windows_high && temp >= windows_high) {
                in_win[e] = 1;
                int32_t slot = atomic_fetch_add_i32(buf_size, 1);
                buff_index[slot] = (int32_t)e;
            }
        }
    }
}

ORC_API void orc_all_affected_support_tilenot(const int32_t *e_affect, int64_t n_affect,
                                              const int32_t *a_rows, const int32_t *cols,
                                              const int32_t *rp, int32_t n_cut,
                                              const uint8_t *mark, int32_t l,
                                              uint8_t *n_mark, int32_t *out) {
    orc_affected_not_impl(e_affect, n_affect, a_rows, cols, rp, n_cut, mark, l, n_mark,
                          out, 0, 0, NULL, NULL, NULL);
}

ORC_API void orc_all_affected_support_tilenotwin(const int32_t *e_affect, int64_t n_affect,
                                                 const int32_t *a_rows, const int32_t *cols,
                                                 const int32_t *rp, int32_t n_cut,
                                                 const uint8_t *mark, int32_t l,
                                                 uint8_t *n_mark, int32_t *out,
                                                 int32_t windows_high, uint8_t *in_win,
                                                 int32_t *buff_index, int32_t *buf_size) {
    orc_affected_not_impl(e_affect, n_affect, a_rows, cols, rp, n_cut, mark, l, n_mark,
                          out, 1, windows_high, in_win, buff_index, buf_size);
}

/* ktruss_search/ktruss_cuda.py:201-286 (subAffectedSupport / _tile): on an
 * extracted subgraph, for every triangle with a marked (deleted) edge,
 * decrement each unmarked edge once.  Unconditional, hence deterministic. */
ORC_API void orc_sub_affected_support_tile(const int32_t *a_rows, const int32_t *cols,
                                           const int32_t *rp, int32_t n_cut,
                                           const uint8_t *mark, int32_t *out,
                                           int64_t num_edges) {
    int64_t n = num_edges * n_cut;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t row = 0; row < n; row++) {
        int64_t i = row / n_cut;
        int32_t j = (int32_t)(row % n_cut);
        ORC_TILE_BOUNDS(i, j)
        int32_t count = 0;
        ORC_MERGE(cols, a0, a1, b0, b1, {
            if (mark[i] || mark[pa] || mark[pb]) {
                if (!mark[pa]) atomic_add_i32(&out[pa], -1);
                if (!mark[pb]) atomic_add_i32(&out[pb], -1);
                if (!mark[i]) count++;
            }
        });
        if (count > 0) atomic_add_i32(&out[i], -count);
    }
}

/* ------------------------------------------------------------------ */
/* Drivers                                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    int32_t *data;
    int64_t n, cap;
} ivec;

static void iv_push(ivec *v, int32_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 64;
        v->data = (int32_t *)realloc(v->data, (size_t)v->cap * sizeof(int32_t));
    }
    v->data[v->n++] = x;
}

/* Indices i (ascending) with pred true, like torch.where(mask)[0]. */
static int64_t where_u8(const uint8_t *m, int64_t n, int32_t *idx) {
    int64_t c = 0;
    for (int64_t i = 0; i < n; i++)
        if (m[i]) idx[c++] = (int32_t)i;
    return c;
}

/* row_ptr after keeping the edges with keep[e] (update_row_ptr,
 * singlegpu_truss.py:60-64 = segment_add + cumsum). */
static void update_row_ptr(const uint8_t *keep, int32_t *rp, int64_t nseg, int32_t *tmp_i32) {
    int32_t *vals = (int32_t *)calloc((size_t)nseg, sizeof(int32_t));
    /* segment_add over the int mask (opmp.cpp:4-24) */
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < nseg; r++) {
        int32_t s = rp[r], e = rp[r + 1];
        int32_t sum = 0;
        for (int32_t i = s; i < e; i++) sum += keep[i];
        if (s < e) vals[r] = sum;
    }
    (void)tmp_i32;
    rp[0] = 0;
    for (int64_t r = 0; r < nseg; r++) rp[r + 1] = rp[r] + vals[r];
    free(vals);
}

/* Keep-compaction of the per-edge arrays (support[e_mask], columns[e_mask],
 * rows[e_mask], edges[e_mask]). */
static int64_t compact_edges(const uint8_t *keep, int64_t n, int32_t *support,
                             int32_t *cols, int32_t *rows, int32_t *edges) {
    int64_t c = 0;
    for (int64_t i = 0; i < n; i++) {
        if (keep[i]) {
            support[c] = support[i];
            cols[c] = cols[i];
            rows[c] = rows[i];
            edges[c] = edges[i];
            c++;
        }
    }
    return c;
}

/* singlegpu_truss.py:67-158 (k_truss, the `--cuda` flow) with the peel update
 * sub_AllAffectedSupport_(tile)not (kernel.cu:220-273, :492-547), or, with
 * cpu_flow != 0, demo_truss/test/truss_setup.py:61-154 (the CPU-capable flow
 * with sub_AllAffectedSupport(_tile), opmp.cpp:99-209).
 *
 * Inputs are the oriented CSRCOO: rows/cols int32[E], tiled row_ptr
 * int32[V*n_cut+1] (csr_to_tilingcsr, singlegpu_truss.py:160-169).  They are
 * copied, not modified.  Outputs: e_truss int32[E] (peel order, original
 * CSR positions), ptr_truss int32[cap] (per-level offsets; ptr_truss[i] ..
 * ptr_truss[i+1] is level i+1, truss number i+3), *n_ptr = entries written.
 * Returns kmax = l + 2, or -1 if ptr_cap is too small.
 *
 * Divergence, documented: the reference loops forever when no edge lies in a
 * triangle (it searches for support == l with l growing without bound); the
 * restatement returns kmax = 2 with ptr_truss = [0] in that case. */
ORC_API int32_t orc_k_truss(const int32_t *rows_in, const int32_t *cols_in,
                            const int32_t *rp_in, int64_t num_v, int64_t num_e,
                            int32_t n_cut, int32_t cpu_flow,
                            int32_t *e_truss, int64_t *n_etruss,
                            int32_t *ptr_truss, int64_t ptr_cap, int64_t *n_ptr) {
    int64_t nseg = num_v * n_cut;
    int64_t E = num_e;
    int32_t *rows = (int32_t *)malloc((size_t)(E ? E : 1) * 4);
    int32_t *cols = (int32_t *)malloc((size_t)(E ? E : 1) * 4);
    int32_t *rp = (int32_t *)malloc((size_t)(nseg + 1) * 4);
    int32_t *support = (int32_t *)calloc((size_t)(E ? E : 1), 4);
    int32_t *edges = (int32_t *)malloc((size_t)(E ? E : 1) * 4);
    uint8_t *e_mask = (uint8_t *)malloc((size_t)(E ? E : 1));
    uint8_t *n_mark = (uint8_t *)malloc((size_t)(E ? E : 1));
    uint8_t *mask = (uint8_t *)malloc((size_t)(E ? E : 1));
    uint8_t *mask_v = (uint8_t *)malloc((size_t)(num_v ? num_v : 1));
    int32_t *e_curr = (int32_t *)malloc((size_t)(E ? E : 1) * 4);
    int32_t *e_affect = (int32_t *)malloc((size_t)(E ? E : 1) * 4);
    memcpy(rows, rows_in, (size_t)E * 4);
    memcpy(cols, cols_in, (size_t)E * 4);
    memcpy(rp, rp_in, (size_t)(nseg + 1) * 4);
    int64_t et = 0, np = 0;
    int32_t kmax = -1;

    /* support_computing (singlegpu_truss.py:38-45) */
    orc_segment_isin2tile(rows, cols, rp, n_cut, support, E);
    /* drop support-0 edges (:83-90) */
    for (int64_t i = 0; i < E; i++) { edges[i] = (int32_t)i; e_mask[i] = support[i] != 0; }
    update_row_ptr(e_mask, rp, nseg, NULL);
    int64_t Ecur = compact_edges(e_mask, E, support, cols, rows, edges);

    ptr_truss[np++] = 0;
    int32_t l = 1;
    if (Ecur == 0) { kmax = 2; goto done; }
    int64_t ncurr;
#define SCAN_EQ(LV)                                                            \
    do { ncurr = 0;                                                            \
         for (int64_t i_ = 0; i_ < Ecur; i_++) if (support[i_] == (LV)) e_curr[ncurr++] = (int32_t)i_; \
    } while (0)
    SCAN_EQ(l);
    while (ncurr == 0) {
        if (np >= ptr_cap) { kmax = -1; goto done; }
        ptr_truss[np] = ptr_truss[np - 1]; np++;
        l++;
        SCAN_EQ(l);
    }
    int64_t peeled = 0;
    /* e_mask: _not flow = alive (ones); CPU flow = deleted (zeros) */
    memset(e_mask, cpu_flow ? 0 : 1, (size_t)Ecur);
    for (;;) {
        for (int64_t i = 0; i < ncurr; i++) e_truss[et++] = edges[e_curr[i]];
        /* p = unique(rows[e_curr]); mask = mask_v[columns] (:102-105) */
        memset(mask_v, 0, (size_t)num_v);
        for (int64_t i = 0; i < ncurr; i++) mask_v[rows[e_curr[i]]] = 1;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < Ecur; i++) {
            int64_t c = cols[i] < 0 ? cols[i] + num_v : cols[i]; /* index -1 = last */
            mask[i] = mask_v[c];
        }
        /* mask[p_c] = e_mask[p_c] (or ~e_mask in the CPU flow) for all out-edges
         * of p over all tiles (batched_csr_selection_opt2, helper.py:102-121) */
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t p = 0; p < num_v; p++) {
            if (!mask_v[p]) continue;
            for (int32_t q = rp[p * n_cut]; q < rp[p * n_cut + n_cut]; q++)
                mask[q] = cpu_flow ? !e_mask[q] : e_mask[q];
        }
        int64_t naff = where_u8(mask, Ecur, e_affect);
        for (int64_t i = 0; i < ncurr; i++) e_mask[e_curr[i]] = cpu_flow ? 1 : 0;
        memset(n_mark, 0, (size_t)Ecur);
        if (cpu_flow)
            orc_all_affected_support_tile(e_affect, naff, rows, cols, rp, n_cut, e_mask, l, n_mark, support);
        else
            orc_all_affected_support_tilenot(e_affect, naff, rows, cols, rp, n_cut, e_mask, l, n_mark, support);
        for (int64_t i = 0; i < ncurr; i++) cols[e_curr[i]] = -1;
        peeled += ncurr;
        if (peeled > 1000000) {
            /* compaction (:120-134 / truss_setup.py:105-120) */
            if (cpu_flow) for (int64_t i = 0; i < Ecur; i++) e_mask[i] = !e_mask[i];
            update_row_ptr(e_mask, rp, nseg, NULL);
            Ecur = compact_edges(e_mask, Ecur, support, cols, rows, edges);
            peeled = 0;
            ncurr = 0;
            for (int64_t i = 0; i < Ecur; i++) if (support[i] <= l) e_curr[ncurr++] = (int32_t)i;
            memset(e_mask, cpu_flow ? 0 : 1, (size_t)Ecur);
        } else {
            ncurr = 0;
            for (int64_t i = 0; i < Ecur; i++)
                if (n_mark[i] && support[i] <= l) e_curr[ncurr++] = (int32_t)i;
        }
        if (peeled + ncurr == Ecur) {
            for (int64_t i = 0; i < ncurr; i++) e_truss[et++] = edges[e_curr[i]];
            if (np >= ptr_cap) { kmax = -1; goto done; }
            ptr_truss[np++] = (int32_t)et;
            break;
        }
        if (ncurr == 0) {
            if (np >= ptr_cap) { kmax = -1; goto done; }
            ptr_truss[np++] = (int32_t)et;
            l++;
            SCAN_EQ(l);
            while (ncurr == 0) {
                if (np >= ptr_cap) { kmax = -1; goto done; }
                ptr_truss[np] = ptr_truss[np - 1]; np++;
                l++;
                SCAN_EQ(l);
            }
        }
    }
    kmax = l + 2;
#undef SCAN_EQ
done:
    *n_etruss = et;
    *n_ptr = np;
    free(rows); free(cols); free(rp); free(support); free(edges);
    free(e_mask); free(n_mark); free(mask); free(mask_v); free(e_curr); free(e_affect);
    return kmax;
}

/* Per-edge truss numbers from the driver outputs (the reference never
 * materialises them; singlegpu_truss.py:158 returns kmax only): edges of
 * e_truss[ptr[i]:ptr[i+1]] have truss i+3, all others (support 0) truss 2. */
ORC_API void orc_truss_from_levels(const int32_t *e_truss, const int32_t *ptr_truss,
                                   int64_t n_ptr, int64_t num_e, int32_t *truss) {
    for (int64_t i = 0; i < num_e; i++) truss[i] = 2;
    for (int64_t lv = 0; lv + 1 < n_ptr; lv++)
        for (int32_t q = ptr_truss[lv]; q < ptr_truss[lv + 1]; q++)
            truss[e_truss[q]] = (int32_t)(lv + 3);
}

ORC_API int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Research-variant operators (sequential merge walks)                  */
/* ------------------------------------------------------------------ */
/* The decrements of these operators commute, so one thread walking the work
 * items in order ends in the same supports and marks as the reference's
 * thread-per-item kernels. */

/* myhpu_extension_kernel.cu:687-713 (checkElementsTwoPtrIsInIs, skip_neg1 = 1)
 * and :1555-1583 (segmentIsinmmKernel, skip_neg1 = 0): per row, a merge walk of
 * the two sorted rows flags the positions of equal values. */
ORC_API void orc_rows_isin_mask(const int32_t *a, const int32_t *ap, const int32_t *b, const int32_t *bp,
                                int64_t rows, uint8_t *m1, uint8_t *m2, int skip_neg1) {
    for (int64_t r = 0; r < rows; r++) {
        int32_t i = ap[r], ie = ap[r + 1], j = bp[r], je = bp[r + 1];
        while (i < ie && j < je) {
            int32_t x = a[i], y = b[j];
            if (x == y && !(skip_neg1 && x == -1)) {
                m1[i++] = 1;
                m2[j++] = 1;
            } else if (x < y) {
                i++;
            } else {
                j++;
            }
        }
    }
}

/* myhpu_extension_kernel.cu:739-779 (checkTriangleSupportSub). */
ORC_API void orc_support_affect(const int32_t *left, const int32_t *right, const int32_t *cur, int64_t n,
                                int32_t *support, const uint8_t *m1, const uint8_t *m2, uint8_t *affect) {
    for (int64_t i = 0; i < n; i++) {
        int32_t a = left[i], b = right[i], c = cur[i];
        if (m1[i] && m2[i]) {
            support[a]--; support[b]--; affect[a] = 1; affect[b] = 1;
        } else if (m1[i]) {
            if (c < b) { support[a]--; affect[a] = 1; }
        } else if (m2[i]) {
            if (c < a) { support[b]--; affect[b] = 1; }
        }
    }
}

static void orc_dec_mark(int32_t *support, uint8_t *n_mark, int32_t x, int32_t lp1) {
    if (support[x]-- == lp1) n_mark[x] = 1;
}

/* myhpu_extension_kernel.cu:808-1551 (peeling_edges_undirect, _direct_oo,
 * _direct_ii, _direct_oi and their _tile forms).  variant: 0 undirect, 1 oo,
 * 2 ii, 3 oi; lp1 = the level + 1 (what the reference's op hands its kernel);
 * n_cut = 1 for the untiled forms.  List A belongs to the tail rows[e], list B
 * to the head columns[e]. */
ORC_API void orc_peel_op(int variant, const int32_t *e_curr, int64_t n_curr, const int32_t *rows,
                         const int32_t *columns, const int32_t *row_ptr, const int32_t *r_edges,
                         const int32_t *re_ptr, const int32_t *columns_g, const int32_t *edges_id_nbr,
                         int32_t *support, const uint8_t *e_mask, uint8_t *n_mark, const uint8_t *in_curr,
                         int32_t lp1, int32_t n_cut) {
    for (int64_t t = 0; t < n_curr * n_cut; t++) {
        int32_t e = e_curr[t / n_cut], k = (int32_t)(t % n_cut);
        int64_t u = (int64_t)rows[e] * n_cut + k, v = (int64_t)columns[e] * n_cut + k;
        /* list A: out (oo, oi), in (ii) or symmetric (undirect); list B: out (oo), in (ii, oi) or symmetric */
        const int32_t *pa = variant == 2 ? re_ptr : row_ptr;
        const int32_t *pb = (variant == 2 || variant == 3) ? re_ptr : row_ptr;
        int32_t i = pa[u], ie = pa[u + 1], j = pb[v], je = pb[v + 1];
        while (i < ie && j < je) {
            int32_t ka, kb, e2, e3;
            if (variant == 0) { ka = columns_g[i]; e2 = edges_id_nbr[i]; }
            else if (variant == 2) { e2 = r_edges[i]; ka = rows[e2]; }
            else { ka = columns[i]; e2 = i; }
            if (variant == 0) { kb = columns_g[j]; e3 = edges_id_nbr[j]; }
            else if (variant == 1) { kb = columns[j]; e3 = j; }
            else { e3 = r_edges[j]; kb = rows[e3]; }
            if (ka == kb) {
                if (e_mask[e2] && e_mask[e3]) {
                    int f2 = in_curr[e2], f3 = in_curr[e3];
                    if (!f2 && !f3) {
                        orc_dec_mark(support, n_mark, e2, lp1);
                        orc_dec_mark(support, n_mark, e3, lp1);
                    } else if (!f2 && f3) {
                        if (variant == 1 || variant == 3 || (variant == 0 && e < e3))
                            orc_dec_mark(support, n_mark, e2, lp1);
                    } else if (f2 && !f3) {
                        if (variant == 1 || (variant == 0 && e < e2))
                            orc_dec_mark(support, n_mark, e3, lp1);
                    }
                }
                i++;
                j++;
            } else if (ka < kb) {
                i++;
            } else {
                j++;
            }
        }
    }
}

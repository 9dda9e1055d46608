// Test infrastructure only: C entry points over the reference's own OpenMP
// operators (demo_truss/myops/mysrc/hpu_extension/myhpu_extension_opmp.cpp),
// compiled together with that file by oracle/build.py into oracle/_ref/.
// The declarations below restate the reference's signatures
// (myhpu_extension.cpp:4, :21, :39-40, :63-68, :154-160) so the functions can
// be called from ctypes; no reference code is copied.
#include <cstdint>

void segment_add_cpu(const int *col_indices, const int *col_ptr, int *output, const int numRows);
void segment_isin2_cpu(const int *a_rows, const int *b_col_indices, const int *b_row_ptr,
                       int *output, const int numRows);
void segment_isin2tile_cpu(const int *a_rows, const int *b_col_indices, const int *b_row_ptr,
                           const int n_cut, int *output, const int numRows);
void AllAffectedSupport_cpu(const int *e_affect, const int *a_rows, const int *b_col_indices,
                            const int *b_row_ptr, const bool *mark, const int l, bool *n_mark,
                            int *output, const int numRows);
void AllAffectedSupport_tile_cpu(const int *e_affect, const int *a_rows, const int *b_col_indices,
                                 const int *b_row_ptr, const int n_cut, const bool *mark,
                                 const int l, bool *n_mark, int *output, const int numRows);

extern "C" {
__attribute__((visibility("default"))) void ref_segment_add(const int *c, const int *p, int *o, int n) {
    segment_add_cpu(c, p, o, n);
}
__attribute__((visibility("default"))) void ref_segment_isin2(const int *r, const int *c, const int *p, int *o, int n) {
    segment_isin2_cpu(r, c, p, o, n);
}
// numRows = number of work items = E * n_cut, as the binding passes it
// (myhpu_extension.cpp:54).
__attribute__((visibility("default"))) void ref_segment_isin2tile(const int *r, const int *c, const int *p, int n_cut,
                                                                  int *o, int n_items) {
    segment_isin2tile_cpu(r, c, p, n_cut, o, n_items);
}
__attribute__((visibility("default"))) void ref_all_affected_support(const int *ea, const int *r, const int *c,
                                                                     const int *p, const uint8_t *mark, int l,
                                                                     uint8_t *n_mark, int *o, int n) {
    AllAffectedSupport_cpu(ea, r, c, p, reinterpret_cast<const bool *>(mark), l,
                           reinterpret_cast<bool *>(n_mark), o, n);
}
__attribute__((visibility("default"))) void ref_all_affected_support_tile(const int *ea, const int *r, const int *c,
                                                                          const int *p, int n_cut,
                                                                          const uint8_t *mark, int l,
                                                                          uint8_t *n_mark, int *o, int n_items) {
    AllAffectedSupport_tile_cpu(ea, r, c, p, n_cut, reinterpret_cast<const bool *>(mark), l,
                                reinterpret_cast<bool *>(n_mark), o, n_items);
}
}

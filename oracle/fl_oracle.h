/*
 * fl_oracle.h -- CPU oracle for the FastLoad CSC SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * CPU path (src/coo2csc.h, src/FastLoad_CPU.h, src/main.cu golden loops) used
 * as the parity checker by the tests, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py.  Nothing in the fastload_gb300 package links
 * or calls it; the product path is the CUDA library and fails loudly when
 * that library is missing.
 *
 * Parity pin: checked against the reference's own CPU functions compiled from
 * their sources (oracle/ref_shim.cpp -> oracle/_ref) and against the golden
 * fixtures in tests/golden/ that those produced.  The one deliberate
 * difference from src/coo2csc.h is the column sort: the reference's CPU
 * col_sort uses std::sort (unstable, coo2csc.h:100) while its GPU ColSort
 * (the path main.cu runs, ColSort_GPU.h:101) uses thrust::sort_by_key, a
 * stable radix sort.  This oracle reproduces the GPU order: ascending nnz per
 * column, ties in ascending original column id.
 *
 * All indices are 32-bit like the reference (nnz < 2^31).
 */
#ifndef FL_ORACLE_H
#define FL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* CSR -> CSC by counting sort; rows ascending within a column, CSR order for
 * duplicates.  Follows src/coo2csc.h:11-72.  Returns 0, or -1 when the
 * column indices do not add up to nnz. */
int fo_csr2csc(int m, int n, int nnz, const int *rowptr, const int *colidx,
               const double *val, int *cscptr, int *cscrow, double *cscval,
               int *nnzpercol);

/* Stable column sort by nonzeros per column.  Follows src/coo2csc.h:75-129
 * with the GPU's stable order (src/ColSort_GPU.h:93-125).  perm[i] is the
 * original column at sorted position i. */
int fo_col_sort(int n, const int *nnzpercol, const int *cscptr,
                const int *cscrow, const double *cscval, const double *x,
                int *perm, int *sortrowidx_tmp, double *sortval_tmp,
                int *sortnnz, double *sortx);

/* Number of steps (h_count) and tiles of the sorted staircase.  Follows
 * src/coo2csc.h:142-205 (and formatTransform_GPU.h:21-98). */
int fo_count_tiles(int n, const int *sortnnz, int *h_count, int *tilenum);

/* Tile layout: tile_ptr (tilenum+1), tile_len, tile_colidx, tile_tall
 * (all zero, as the reference CPU path leaves it) and the tile-ordered
 * sortrowidx/sortval (nnz).  Follows src/coo2csc.h:132-312. */
int fo_format_transform(int n, int nnz, const int *sortnnz,
                        const int *sortrowidx_tmp, const double *sortval_tmp,
                        int tilenum, int *tile_ptr, int *tile_len,
                        int *tile_colidx, int *tile_tall, int *sortrowidx,
                        double *sortval);

/* Runs of equal consecutive rows per tile: tile_format (0/1/2),
 * countrow (tilenum+1, exclusive scan of runs), segmentoffset (run lengths,
 * caller gives nnz+1 slots), sortrowindex (nnz) and segsum.  Follows
 * src/coo2csc.h:314-448. */
int fo_tile_classification(int nnz, int tilenum, const int *tile_ptr,
                           const int *tile_len, const int *sortrowidx,
                           int *tile_format, int *countrow,
                           int *segmentoffset, int *sortrowindex,
                           int *segsum);

/* y += A x over the tile layout, serial, in tile order.  Follows
 * src/FastLoad_CPU.h:19-31. */
void fo_fastload_spmv(int tilenum, const int *tile_ptr, const int *tile_len,
                      const int *tile_colidx, const int *sortrowidx,
                      const double *sortval, const double *sortx, double *y);

/* The same tile loop spread over nthreads OpenMP threads with atomic
 * updates of y, the pattern of the reference's multi-core CPU CSC SpMV
 * (test.cu:46-57).  Returns the thread count used. */
int fo_fastload_spmv_omp(int tilenum, const int *tile_ptr,
                         const int *tile_len, const int *tile_colidx,
                         const int *sortrowidx, const double *sortval,
                         const double *sortx, double *y, int nthreads);

/* y += A x column by column (src/main.cu:110-120). */
void fo_csc_spmv(int n, const int *cscptr, const int *cscrow,
                 const double *cscval, const double *x, double *y);

/* y = A x row by row (src/main.cu:98-108). */
void fo_csr_spmv(int m, const int *rowptr, const int *colidx,
                 const double *val, const double *x, double *y);

/* Compensated y = A x (double-double accumulation per row with an
 * fma-based exact product), rounded to double: the FP64 reference that
 * error statements are made against.  k right-hand sides, x and y stored
 * row-interleaved (x[col*k + r], y[row*k + r]). */
void fo_csc_spmv_dd(int m, int n, int k, const int *cscptr,
                    const int *cscrow, const double *cscval, const double *x,
                    double *y);

/* MatrixMarket coordinate file -> CSR, restating mmio_allinone
 * (src/auxiliary.h:64-232) with the banner / size-line rules of
 * src/mmio.h:142-259: entries read by fscanf in file order ("%d %d %lg",
 * "%d %d %d", "%d %d", or two values for complex keeping the real part),
 * symmetric and hermitian entries mirrored, rows filled in file order.
 * Call with rowptr == NULL for the sizes (m, n, expanded nnz, symmetric
 * flag), then again with arrays of m+1 / nnz / nnz entries.  Returns 0, -1
 * (cannot open), -2 (banner), -4 (size line), -5 (an entry that does not
 * scan or lies outside the matrix: the reference would read garbage or
 * write out of bounds there). */
int fo_mmio_read(const char *path, int *m, int *n, int *nnz, int *is_symmetric,
                 int *rowptr, int *colidx, double *val);

#ifdef __cplusplus
}
#endif
#endif

/*
 * fastload.h -- C ABI of the FastLoad GB300 CSC SpMV engine.
 *
 * Plain C: pointers, sizes and int status codes; no C++ or PyTorch types.
 * Two groups of entry points:
 *
 *  1. Reference-compatible calls with HOST buffers that replace the calls
 *     the reference's src/main.cu makes (csr_to_csc, ColSort,
 *     formatTransform, FastLoad_spmv).  They are synchronous, produce the
 *     reference's outputs bit for bit (layout) and fill the reference's
 *     slide_matrix struct.  include/fastload_compat.h wraps them under the
 *     reference's own names and C++ signatures.
 *
 *  2. A device-resident plan API: build the FastLoad layout once from device
 *     CSR/CSC arrays, keep it in HBM and run y = A x on caller streams
 *     (graph-capturable launches, no host round trips).
 *
 * Status codes are 0 on success and negative on failure; fl_last_error()
 * returns the message of the last failure on the calling thread.  All
 * indices are 32-bit, as in the reference (nnz < 2^31).
 *
 * Threads: different plans may be used from different host threads at
 * once; one plan is used by one host thread at a time (its host-buffer
 * calls keep staging buffers, streams and a pipelining slot counter).
 */
#ifndef FASTLOAD_GB300_H
#define FASTLOAD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The library is built with hidden visibility: the functions declared here
 * are its only exports, so its internal C++ symbols (and the static state of
 * its templates) never bind to another library's in the same process.  The
 * opaque handle types are declared before the default-visibility region, so
 * their members stay internal too. */
struct fl_plan;
struct fl_mtx;
struct fl_cusparse;
struct fl_batch;
struct fl_mlp;
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define FL_SUCCESS 0
#define FL_ERR_ARG (-1)       /* bad argument, malformed or inconsistent input */
#define FL_ERR_CUDA (-2)      /* CUDA runtime error */
#define FL_ERR_ALLOC (-3)     /* device or host allocation failed */
#define FL_ERR_OVERFLOW (-4)  /* a count does not fit the 32-bit index space */
#define FL_ERR_INTERNAL (-5)  /* internal consistency check failed */
#define FL_ERR_NOT_READY (-6) /* bounded device wait expired */
#define FL_ERR_IO (-7)        /* file missing, unreadable, truncated or corrupt */
#define FL_ERR_UNAVAILABLE (-8) /* optional component missing (cuSPARSE comparator) */

/* Same members, order and types as the reference's slide_matrix
 * (src/format.h:6-20), so a pointer to either can be passed. */
typedef struct fl_slide_matrix {
    double *sortval;
    int *sortrowidx;
    int *tile_ptr;
    int *tile_len;
    int *tile_colidx;
    int *tile_tall;
    int *tile_format;
    int *countrow;
    int *segmentoffset;
    int *sortrowindex;
    int tilenum;
    int segsum;
} fl_slide_matrix;

/* Message of the last failed call on this thread ("" if none). */
const char *fl_last_error(void);
/* Library version string. */
const char *fl_version(void);
/* Number of visible CUDA devices (0 when there is none). */
int fl_device_count(void);

/* ---- 1. reference-compatible host calls ------------------------------ */

/* Replaces csr_to_csc (src/csr2csc_cuda.h:51-135; CPU twin
 * src/coo2csc.h:11-72).  CSR (m x n) in, CSC out: rows ascending inside
 * each column (CSR order for duplicate entries), csc_col_ptr has n+1
 * entries, nnzpercol n.  *time_ms gets the device time of the transpose. */
int fl_csr_to_csc(double *time_ms, int m, int n, int nnz, const double *csr_val,
                  const int *csr_row_ptr, const int *csr_col_ind,
                  double *csc_val, int *csc_row_ind, int *csc_col_ptr,
                  int *nnzpercol);

/* Replaces ColSort (src/ColSort_GPU.h:46-136).  Stable ascending sort of the
 * columns by nonzero count (ties keep ascending column id, the order of
 * thrust::sort_by_key at ColSort_GPU.h:101); writes the column-sorted CSC
 * (sortrowidxTmp, sortvalTmp: nnz), the sorted counts (sortnnzTmp: colA) and
 * the permuted x (sortx: colA).  Reads only colA entries of each per-column
 * array. */
int fl_col_sort(double *time_ms, int rowA, int colA, int nnz,
                const int *nnzPerCol, const int *cscColPtr,
                const int *cscRowIdx, const double *cscVal,
                int *sortrowidxTmp, double *sortvalTmp, int *sortnnzTmp,
                const double *x, double *sortx);

/* Replaces formatTransform (src/formatTransform_GPU.h:289-596).  Builds the
 * FastLoad tile layout from the column-sorted CSC and fills *matrix with
 * malloc'd arrays the caller frees (fl_tile_destroy or the reference's
 * Tile_destroy).  Unlike the reference's GPU path, every member is defined:
 * tile_tall is zero-filled, countrow (tilenum+1), segmentoffset (segsum+1)
 * and segsum are set as the reference's CPU path sets them
 * (src/coo2csc.h:132-448).  *h_count gets the number of staircase steps. */
int fl_format_transform(double *time_tran_ms, double *time_class_ms,
                        fl_slide_matrix *matrix, const int *sortrowidx_tmp,
                        const double *sortval_tmp, const int *sortnnz_tmp,
                        int nnz, int rowA, int colA, int *h_count);

/* Replaces FastLoad_spmv (src/FastLoad_GPU.h:275-409).  Uploads the layout
 * and x_sorted, runs one untimed SpMV then `reps` timed ones (CUDA events,
 * y zeroed before each), copies y = A x back (original row order) and, when
 * y_golden is non-null, counts entries with |y_golden - y| > 0.01 |y|
 * (the reference's check, FastLoad_GPU.h:383-389) into *mismatches.
 * *ms_per_spmv gets the mean device time of one SpMV.  Any of the output
 * pointers may be NULL. */
int fl_fastload_spmv(const fl_slide_matrix *matrix, int nnz, int colA,
                     int rowA, const double *x_sorted, double *y,
                     const double *y_golden, int reps, double *ms_per_spmv,
                     int *mismatches);

/* Frees the arrays of a slide_matrix filled by fl_format_transform
 * (src/format.h:29-42) and clears the pointers. */
void fl_tile_destroy(fl_slide_matrix *matrix);

/* ---- 2. device-resident plan API ------------------------------------- */

typedef struct fl_plan *fl_plan_t;

typedef struct fl_plan_info {
    int m, n, nnz;
    int tilenum;     /* tiles of the reference layout */
    int steps;       /* staircase steps (h_count) */
    int segsum;      /* runs of equal rows over all tiles */
    int regions;     /* work regions of the streaming kernel */
    int items;       /* work items of the streaming kernel */
    size_t device_bytes; /* HBM held by the plan */
    int heavy_cols;  /* bucketed form: width of the heavy band (0: none) */
    int heavy_nnz;   /* nonzeros in the heavy band */
    int heavy_slices;/* 32-row slices of the heavy band */
    int heavy_padded;/* slice entries including padding */
    int spmv_launches; /* kernels one fl_plan_spmv(accumulate 0, FL_KERNEL_AUTO)
                          launches: the y zeroing (skipped when the band owns
                          every row) and the SpMV kernel */
} fl_plan_info;

/* Plan build options (NULL = defaults: no reference arrays, automatic
 * heavy band). */
typedef struct fl_plan_opts {
    int with_reference_arrays; /* keep the reference per-tile arrays */
    int heavy_band;  /* bucketed form: -1 off (FastLoad stream only),
                        0 automatic (the densest columns with >= 32 nonzeros,
                        at most 16384, when they hold >= 1/4 of the matrix;
                        with none, every column as row slices when x gathers
                        have locality, rows are skewed or the matrix has 1M+
                        nonzeros and 4+ a column; else off), > 0 that
                        many of the densest columns (even, at most
                        fl_plan_max_heavy_band()) */
    int reserved[6];
} fl_plan_opts;

#define FL_INPUT_CSR 0
#define FL_INPUT_CSC 1

/* Builds a plan from a device CSR (input_format FL_INPUT_CSR: ptr = row
 * pointer m+1, idx = column indices) or CSC (FL_INPUT_CSC: ptr = column
 * pointer n+1, idx = row indices, rows ascending per column) matrix. */
int fl_plan_create(fl_plan_t *plan, int input_format, int m, int n, int nnz,
                   const int *d_ptr, const int *d_idx, const double *d_val,
                   const fl_plan_opts *opts, void *stream);
/* Widest heavy band the bucketed kernel can stage in shared memory. */
int fl_plan_max_heavy_band(void);

/* Builds a plan from a device CSR matrix (m x n) with the default heavy
 * band.  stream may be NULL (legacy default stream).  Synchronises the
 * stream a few times to size the layout.  with_reference_arrays != 0 also
 * keeps the reference per-tile arrays on the device (needed by
 * fl_plan_export and the tile kernel). */
int fl_plan_create_csr(fl_plan_t *plan, int m, int n, int nnz,
                       const int *d_rowptr, const int *d_colidx,
                       const double *d_val, int with_reference_arrays,
                       void *stream);
/* Same from a device CSC matrix (rows ascending within each column). */
int fl_plan_create_csc(fl_plan_t *plan, int m, int n, int nnz,
                       const int *d_colptr, const int *d_rowidx,
                       const double *d_val, int with_reference_arrays,
                       void *stream);
int fl_plan_info_get(fl_plan_t plan, fl_plan_info *info);
/* Copies the reference layout into *matrix (malloc'd arrays, freed with
 * fl_tile_destroy) and the column permutation into perm (n entries, may be
 * NULL).  Needs a plan built with reference arrays. */
int fl_plan_export(fl_plan_t plan, fl_slide_matrix *matrix, int *perm);
/* xs[i] = x[perm[i]]: x in original column order -> sorted order. */
int fl_plan_permute_x(fl_plan_t plan, const double *d_x, double *d_xs,
                      void *stream);

/* SpMV kernels of the plan (variant argument of fl_plan_spmv). */
#define FL_KERNEL_AUTO 0     /* bucketed kernel when the plan has a heavy band, else streaming */
#define FL_KERNEL_TILE 1     /* one warp per reference tile (reference-style) */
#define FL_KERNEL_STREAM 2   /* streaming kernel, one block in flight per warp */
#define FL_KERNEL_STREAM2 3  /* streaming kernel, two blocks in flight per warp */
#define FL_KERNEL_BUCKET 4   /* light columns streamed + heavy band in row slices */

/* y = A xs (y zeroed first) or y += A xs when accumulate != 0; xs is in
 * sorted column order (fl_plan_permute_x), y in original row order.
 * Asynchronous on `stream`. */
int fl_plan_spmv(fl_plan_t plan, const double *d_xs, double *d_y,
                 int accumulate, int variant, void *stream);
/* Host-buffer SpMV through the plan: copies xs (n doubles) to the device,
 * runs y = A xs and copies y (m doubles) back; synchronous on `stream`.
 * Pinned host buffers give the fastest copies.  On an error return no copy
 * from h_xs or into h_y is still running. */
int fl_plan_spmv_host(fl_plan_t plan, const double *h_xs, double *h_y,
                      int variant, void *stream);
/* Pipelined host-buffer SpMV: enqueues the copy of xs to the device, y = A xs
 * and the copy of y back, and returns without waiting; `stream` waits for
 * the result, so synchronising it (or an event recorded on it after this
 * call) makes h_y valid.  Consecutive calls overlap: the upload of one x and
 * the download of an earlier y run while a kernel computes (three internal
 * streams, two device staging slots reused in turn once the call that used
 * a slot two calls earlier has finished with it).  The upload does not wait
 * for earlier work on `stream`: h_xs must hold x when the call is made, and
 * may be reused, like h_y read, only after that synchronisation.  Both
 * should be pinned (page-locked) host memory, otherwise the copies are
 * synchronous and nothing overlaps.  On an error return the call has waited
 * for what it had queued: no copy from h_xs or into h_y is still running. */
int fl_plan_spmv_host_async(fl_plan_t plan, const double *h_xs, double *h_y,
                            int variant, void *stream);
int fl_plan_destroy(fl_plan_t plan);
/* Reads and clears the device status word of the plan's kernels (0 when no
 * bounded wait expired); synchronises the device. */
int fl_plan_check(fl_plan_t plan);

/* ---- persistent plan files ------------------------------------------- */

/* Writes the plan's preprocessed FastLoad format to `path`: the column
 * permutation, nonzeros per sorted column, the tile-ordered row and value
 * streams (the reference's sortrowidx / sortval), the plan options and the
 * list of forms, with checksums.  Replaces rebuilding (and re-uploading,
 * src/FastLoad_GPU.h:318-327) the format on every run of the reference's
 * src/main.cu:314.  Synchronises the device. */
int fl_plan_save(fl_plan_t plan, const char *path);
/* Reads a plan file into a new device plan equal to the saved one (same
 * layout, heavy band and forms).  FL_ERR_IO for a missing, truncated or
 * corrupt file (checksums), FL_ERR_ARG when the content is not a valid
 * FastLoad format (permutation, ascending column counts, row range). */
int fl_plan_load(fl_plan_t *plan, const char *path, void *stream);

/* ---- MatrixMarket ingest on the GPU ------------------------------------ */

/* Data type and storage scheme of a .mtx file (banner fields 4 and 5). */
#define FL_MTX_REAL 0
#define FL_MTX_INTEGER 1
#define FL_MTX_PATTERN 2
#define FL_MTX_COMPLEX 3
#define FL_MTX_GENERAL 0
#define FL_MTX_SYMMETRIC 1
#define FL_MTX_HERMITIAN 2
#define FL_MTX_SKEW 3

typedef struct fl_mtx *fl_mtx_t;

typedef struct fl_mtx_info {
    int m, n;
    int nnz;          /* CSR nonzeros after symmetric expansion (mmio_allinone's *nnz) */
    int nnz_file;     /* entries stored in the file */
    int field;        /* FL_MTX_REAL / INTEGER / PATTERN / COMPLEX */
    int symmetry;     /* FL_MTX_GENERAL / SYMMETRIC / HERMITIAN / SKEW */
    int is_symmetric; /* mmio_allinone's *isSymmetric: symmetric or hermitian */
    int exact_path_values; /* values decided by the big-integer comparison */
    size_t file_bytes;
} fl_mtx_info;

/* Reads a coordinate .mtx file into device CSR: the banner and size line on
 * the host, the entries tokenised, converted and assembled on the GPU.
 * Produces exactly the CSR of the reference's mmio_allinone
 * (src/auxiliary.h:64-232): rows in file order, symmetric / hermitian
 * entries mirrored, values correctly rounded as strtod rounds them.
 * Synchronous on `stream`.  FL_ERR_IO for unreadable files, FL_ERR_ARG for
 * malformed or unsupported content (array files, indices out of range, too
 * few entries, hexadecimal floats, NaN payloads). */
int fl_mtx_read(fl_mtx_t *mtx, const char *path, void *stream);
int fl_mtx_info_get(fl_mtx_t mtx, fl_mtx_info *info);
/* Device CSR of the file (row pointer m+1, column indices and values nnz),
 * owned by the handle and valid until fl_mtx_destroy.  Any output may be
 * NULL. */
int fl_mtx_csr(fl_mtx_t mtx, const int **d_rowptr, const int **d_colidx,
               const double **d_val);
/* Copies the CSR into caller device buffers (m+1, nnz, nnz entries; any
 * may be NULL), asynchronously on `stream`. */
int fl_mtx_copy_csr(fl_mtx_t mtx, int *d_rowptr, int *d_colidx, double *d_val,
                    void *stream);
int fl_mtx_destroy(fl_mtx_t mtx);
/* Replaces mmio_allinone (src/auxiliary.h:64-232) with the same outputs:
 * host arrays from malloc (freed by the caller), parsed on the GPU.
 * Returns 0 or a negative FL_ERR_* status. */
int fl_mmio_allinone(int *m, int *n, int *nnz, int *isSymmetric,
                     int **csrrowptr, int **csrcolidx, double **csrval,
                     const char *filename);

/* ---- comparators (context lines for reports, never a fallback) --------- */

/* y = A x (y zeroed first unless accumulate) with the reference's naive CSC
 * kernel: one thread per column, one atomic per nonzero, 32 blocks of 64
 * threads per SM (src/CSCSpMV.h:4-27, launch at :68).  Device CSC in
 * original column order, x in original order.  Asynchronous on `stream`. */
int fl_csc_spmv_naive(int m, int n, int nnz, const int *d_colptr,
                      const int *d_rowidx, const double *d_val,
                      const double *d_x, double *d_y, int accumulate,
                      void *stream);

typedef struct fl_cusparse *fl_cusparse_t;
/* cuSPARSE CSR FP64 SpMV, the reference's second comparator
 * (src/cusparse_cuda.h:27-155), prepared once (buffer + preprocess) so that
 * fl_cusparse_spmv times the steady state.  alg: 0 CUSPARSE_SPMV_ALG_DEFAULT,
 * 1 CSR_ALG1, 2 CSR_ALG2.  The device CSR must outlive the handle.
 * libcusparse is loaded on first use; FL_ERR_UNAVAILABLE without it. */
int fl_cusparse_create(fl_cusparse_t *h, int m, int n, int nnz,
                       const int *d_rowptr, const int *d_colidx,
                       const double *d_val, int alg, void *stream);
/* y = A x, asynchronous on `stream`. */
int fl_cusparse_spmv(fl_cusparse_t h, const double *d_x, double *d_y,
                     void *stream);
int fl_cusparse_destroy(fl_cusparse_t h);
/* The two comparators on host buffers (device memory internal to the call):
 * y = A x, *mean_ms = mean kernel time over `reps` launches (CUDA events,
 * y zeroing outside the timed region).  CSC in original column order for the
 * naive kernel, CSR for cuSPARSE (CUSPARSE_SPMV_ALG_DEFAULT). */
int fl_csc_spmv_naive_host(int m, int n, int nnz, const int *csc_ptr,
                           const int *csc_rowidx, const double *csc_val,
                           const double *x, double *y, int reps,
                           double *mean_ms);
int fl_cusparse_spmv_host(int m, int n, int nnz, const int *csr_rowptr,
                          const int *csr_colidx, const double *csr_val,
                          const double *x, double *y, int reps,
                          double *mean_ms);

/* ---- storage / right-hand-side forms ---------------------------------- */

/* Value storage of a form. */
#define FL_VALUES_F64 0    /* FP64 values, FP64 products (x and y FP64) */
#define FL_VALUES_F32 1    /* FP32 values, FP32 x, FP32 products */
#define FL_VALUES_BF16X2 2 /* BF16 hi+lo split, FP32 x, FP32 products: the high
                              half of each 4-byte value is hi = bf16(v), the low
                              half a signed 16-bit correction d relative to hi
                              (v ~ hi (1 + d 2^-22)); 23 significant bits */
/* Heavy band of a form (columns handled in 32-row slices, one lane per row). */
#define FL_BAND_AUTO 0     /* automatic: the densest columns (>= 32 nonzeros, up to 128 KB of x: 16,384 FP64 / 32,768 FP32 columns) when they hold >= 1/4 of the matrix; else every column when x gathers have locality, rows are skewed or the matrix has 1M+ nonzeros and 4+ a column; else none */
#define FL_BAND_NONE (-1)  /* pure FastLoad tile stream (one atomic per run) */
#define FL_BAND_ALL (-2)   /* every column: rows owned by one lane, no atomics */

typedef struct fl_form_info {
    int value_type, heavy_cols, heavy_nnz, light_nnz, y_f32;
    size_t device_bytes;
} fl_form_info;

/* Adds a form to the plan: values stored as value_type, the given heavy band
 * (FL_BAND_* or a column count), y accumulated in FP32 when y_f32 != 0 (FP32
 * values only) else FP64.  *form_id receives the form's index.  Products and
 * per-row sums are FP32 for FP32/BF16 forms and FP64 for FP64 forms. */
int fl_plan_add_form(fl_plan_t plan, int value_type, int heavy_band, int y_f32,
                     int *form_id);
int fl_plan_form_info(fl_plan_t plan, int form_id, fl_form_info *info);

/* Heavy-band loop of a form (fl_form_opts.heavy_loop). */
#define FL_HEAVY_AUTO 0  /* the ring where it applies, else loads held in registers */
#define FL_HEAVY_RING 1  /* band values and columns streamed through shared-memory
                            rings by cp.async (needs the band's x in shared memory
                            and room for the rings beside it; else as REGS) */
#define FL_HEAVY_REGS 2  /* band loads held in registers, a group ahead */
/* Where the heavy band reads x (fl_form_opts.x_stage). */
#define FL_XSTAGE_AUTO 0   /* staged in shared memory (TMA bulk copy) when it fits */
#define FL_XSTAGE_GLOBAL 1 /* read through the cache, never staged */

/* Build and launch options of a form.  Fields after y_f32 at 0 take the
 * automatic choice; fl_plan_add_form is fl_plan_add_form_opts with them 0. */
typedef struct fl_form_opts {
    int value_type; /* FL_VALUES_* */
    int heavy_band; /* FL_BAND_* or a column count */
    int y_f32;      /* y accumulated in FP32 (FP32 values only) */
    int light_item; /* nonzeros per work item of the light columns' FastLoad
                       stream: 0 automatic (about two items per warp of the
                       GPU, 128..2048), else 128..8192 in steps of 128 */
    int heavy_loop; /* FL_HEAVY_* */
    int x_stage;    /* FL_XSTAGE_* */
    int unit_warps; /* heavy-band work units per resident warp: 0 automatic
                       (2 when the band holds every column, else 4),
                       else 1..64 */
    int reserved;   /* must be 0 */
} fl_form_opts;

/* Adds a form built with the given options (FL_ERR_ARG for values out of
 * range); *form_id receives its index. */
int fl_plan_add_form_opts(fl_plan_t plan, const fl_form_opts *opts,
                          int *form_id);
/* The options a form was built with (automatic choices left at 0). */
int fl_plan_form_opts_get(fl_plan_t plan, int form_id, fl_form_opts *opts);
/* Changes the launch options of a built form (heavy loop, x staging);
 * nothing is rebuilt.  Not to be called while the form's SpMVs may be
 * enqueued from another thread. */
int fl_plan_form_set_launch(fl_plan_t plan, int form_id, int heavy_loop,
                            int x_stage);
/* y = A xs (or += when accumulate) for k right-hand sides (k = 1 or 8):
 * xs[(sorted column)*k + r] (double for FP64 forms, float otherwise; see
 * fl_plan_permute_x_k), y[row*k + r] (double, or float for y_f32 forms).
 * For k > 1 both must be 16-byte aligned.  Asynchronous on `stream`. */
int fl_plan_spmv_form(fl_plan_t plan, int form_id, int k, const void *d_xs,
                      void *d_y, int accumulate, void *stream);
/* xs[i*k + r] = x[perm[i]*k + r], converted to float when to_f32 != 0. */
int fl_plan_permute_x_k(fl_plan_t plan, int k, int to_f32, const double *d_x,
                        void *d_xs, void *stream);

/* Converts n FP64 values to a form's storage type on the device, exactly as
 * forms store their values: FL_VALUES_F32 (d_out: n floats, round to
 * nearest) or FL_VALUES_BF16X2 (d_out: n 32-bit words, high half bf16(v),
 * low half the 16-bit correction).  Asynchronous on `stream`. */
int fl_convert_values(int value_type, long n, const double *d_in, void *d_out,
                      void *stream);

/* ---- batches: many matrices, one persistent launch ---------------------- */

typedef struct fl_batch *fl_batch_t;

/* Stacks the FastLoad layouts of `count` plans (which may be destroyed
 * afterwards) into one work list: y and x of the matrices are stacked in
 * plan order (offsets from fl_batch_offsets), values stored as value_type,
 * y accumulated in FP32 when y_f32 (FP32 values only) else FP64. */
int fl_batch_create(fl_batch_t *batch, int count, const fl_plan_t *plans,
                    int value_type, int y_f32);
int fl_batch_info(fl_batch_t batch, int *count, long *m_total, long *n_total,
                  long *nnz_total, int *items);
/* m_off, n_off: count+1 entries each (stacked row / column offsets). */
int fl_batch_offsets(fl_batch_t batch, int *m_off, int *n_off);
/* Stacked x in original column order -> stacked sorted x (float unless the
 * batch stores FP64 values). */
int fl_batch_permute_x(fl_batch_t batch, const double *d_x, void *d_xs,
                       void *stream);
/* y = A xs for every matrix of the batch in one launch (asynchronous). */
int fl_batch_spmv(fl_batch_t batch, const void *d_xs, void *d_y, void *stream);
/* The same through a CUDA graph captured on the first call (and again when
 * d_xs or d_y change) and replayed on `stream`. */
int fl_batch_spmv_graph(fl_batch_t batch, const void *d_xs, void *d_y,
                        void *stream);
int fl_batch_destroy(fl_batch_t batch);

/* ---- tuner: synthetic matrices, features, network ----------------------- */

/* Fills rows and values of a device CSC whose column pointer (degrees) the
 * caller chose: family 0 uniform rows, 1 uniform rows (Zipf degrees), 2
 * banded (window of `param` rows about the diagonal), 3 block-diagonal
 * (blocks of `param`), 4 row-skewed (row = m u^param).  Rows ascend within a
 * column (repeats possible when a degree nears its window); values uniform
 * in [-1, 1).  Deterministic in seed. */
int fl_gen_fill(int family, int m, int n, const int *d_colptr, int *d_rowidx,
                double *d_val, double param, unsigned long long seed,
                void *stream);
/* 24 features of the plan's matrix (log sizes, column-degree moments and
 * log2 histogram, nonzero share of the densest 2048/8192/24576 columns,
 * distance from the diagonal, row-degree spread, value type). */
int fl_plan_features(fl_plan_t plan, int value_type, float *out24);

typedef struct fl_mlp *fl_mlp_t;
/* MLP in -> h1 -> h2 -> out, ReLU hidden layers, He-uniform init from seed. */
int fl_mlp_create(fl_mlp_t *mlp, int in, int h1, int h2, int out,
                  unsigned long long seed);
long fl_mlp_num_params(fl_mlp_t mlp);
/* Parameters flat: W1 (in x h1, row-major), b1, W2, b2, W3, b3. */
int fl_mlp_get_params(fl_mlp_t mlp, float *params);
int fl_mlp_set_params(fl_mlp_t mlp, const float *params);
/* Host buffers: X (B x in), Y (B x out). */
int fl_mlp_forward(fl_mlp_t mlp, const float *X, int B, float *Y);
/* Masked mean-squared error against T (mask M, NULL = all ones) and its
 * gradient with respect to every parameter (flat, same order). */
int fl_mlp_grad(fl_mlp_t mlp, const float *X, const float *T, const float *M,
                int B, float *loss, float *grad);
/* `epochs` full-batch Adam steps on the GPU; losses[e] gets each epoch's
 * loss (may be NULL). */
int fl_mlp_train(fl_mlp_t mlp, const float *X, const float *T, const float *M,
                 int B, int epochs, float lr, float *losses);
int fl_mlp_destroy(fl_mlp_t mlp);

/* ---- tuned forms --------------------------------------------------------- */

/* value_type of a tuner variant that takes the caller's value type. */
#define FL_TUNE_REQUESTED (-1)

/* The tuner's variant table: the form options the autotuner times and the
 * network chooses among, in the order of the network's outputs.  Copies up
 * to `max` entries into out (may be NULL) and returns the table's length.
 * value_type is FL_TUNE_REQUESTED (the caller's value type) or
 * FL_VALUES_BF16X2 (BF16 hi+lo storage, offered to callers asking for FP32
 * values: both meet the same 1e-6 error bar). */
int fl_tuner_variants(fl_form_opts *out, int max);

/* Adds the form the learned tuner predicts fastest for this plan's matrix:
 * the plan's 24 features (fl_plan_features) go through the network stored
 * in model_path (written by the tuner's training, its variant table equal
 * to fl_tuner_variants) on the GPU, and the variant with the lowest
 * predicted time among those allowed is built.  Allowed: for value_type
 * FL_VALUES_F64 the FP64 variants; for FL_VALUES_F32 the FP32 and the BF16
 * hi+lo variants (FP32 only when y_f32).  *form_id receives the form,
 * *variant (may be NULL) the chosen row of the variant table.  FL_ERR_IO
 * for a missing or malformed model file, FL_ERR_ARG for a model trained on
 * another variant table.  Synchronises the device. */
int fl_plan_add_tuned_form(fl_plan_t plan, const char *model_path,
                           int value_type, int y_f32, int *form_id,
                           int *variant);

/* ---- allocation-free column sort -------------------------------------- */

/* Largest column count fl_col_sort_noalloc accepts (its scratch array holds
 * about 3.3 MB of device memory for this many columns). */
#define FL_NOALLOC_MAX_COLS 262144

/* No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory -- for example a plugin whose host
 * application has already reserved the whole GPU in its own pool and refuses
 * further allocations, or a latency-critical caller that cannot afford the
 * device-wide synchronisation cudaMalloc/cudaFree bring.  It computes what
 * fl_col_sort computes (stable sort of the columns by nonzero count, the
 * column-sorted CSC and the permuted x) but on DEVICE arrays the caller
 * provides, and it calls no cudaMalloc, cudaFree or other allocating
 * routine.  Its scratch is one statically sized device array in the library,
 * present on every GPU that loads the library until the process exits.
 *
 *  - n must be at most FL_NOALLOC_MAX_COLS; larger n returns FL_ERR_ARG
 *    with a message (use fl_col_sort or a plan instead).
 *  - The first call on a device looks up the scratch array's device address
 *    (with that device current) and keeps it for the life of the process;
 *    make that first call before any stream capture.  The kept address does
 *    not survive a reset of the device's context (cudaDeviceReset): do not
 *    call this entry point on a device after resetting it.
 *  - With CUDA's lazy module loading, the scratch array (about 3.3 MB) is
 *    created on a device when this library's module is first loaded there,
 *    which may be that first call.  An application that reserves the whole
 *    GPU for its own pool should make the first call on each device (or any
 *    other call of this library on it) before reserving the pool.
 *  - All calls share the one scratch array, which keeps the last call's
 *    contents (the entry point zeroes what must start at zero).  Calls that
 *    overlap on the GPU -- on different streams or from different host
 *    threads -- race on it; serialise them.
 *  - Synchronises `stream` once (to read the validation result); the rest is
 *    asynchronous on `stream` (NULL = legacy default stream).
 * Inputs: d_nnzpercol (n), d_colptr (n+1), d_rowidx, d_val (nnz), d_x (n,
 * may be NULL).  Outputs: d_perm, d_sortnnz (n), d_sortrowidx_tmp,
 * d_sortval_tmp (nnz), d_sortx (n, when d_x is given). */
int fl_col_sort_noalloc(int n, int nnz, const int *d_nnzpercol,
                        const int *d_colptr, const int *d_rowidx,
                        const double *d_val, const double *d_x, int *d_perm,
                        int *d_sortnnz, int *d_sortrowidx_tmp,
                        double *d_sortval_tmp, double *d_sortx, void *stream);

/* ---- test hooks ------------------------------------------------------- */

/* Makes the `countdown`-th device allocation from now fail with
 * FL_ERR_ALLOC (0 disables).  For error-path tests. */
void fl_debug_fail_alloc_after(int countdown);

/* hold != 0: fl_plan_spmv_host stops signalling that the light columns' x
 * has arrived, so the kernel's bounded wait for it runs out (about a second)
 * and the call returns FL_ERR_NOT_READY.  For the failure-detection test. */
void fl_debug_hold_x_upload(int hold);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif

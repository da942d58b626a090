// fl_api.cu -- extern "C" entry points of the FastLoad GB300 library.
//
// Reference-compatible host-buffer calls (csr_to_csc, ColSort,
// formatTransform, FastLoad_spmv) and the device-resident plan API.
// Every call validates its arguments, returns an int status and never
// falls back to a CPU path.
#include "fl_internal.cuh"

#include <cuda.h>

#include <atomic>
#include <mutex>

#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>

namespace fl {
const char *last_error_cstr();
void debug_fail_alloc_after(int n);
// test hook: fl_plan_spmv_host leaves out the epoch copy that releases the
// kernel's light items
static std::atomic<bool> g_hold_x_flag{false};

// *flag = *epoch_host once the work queued on s before it is done: a stream
// memory write (cuStreamWriteValue32, from the driver entry point) where the
// driver offers it -- it needs no copy engine and lands about a microsecond
// after the copy before it -- else a 4-byte copy from the pinned word.
typedef CUresult (*write_value32_fn)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
static int signal_epoch(cudaStream_t s, int *flag, const int *epoch_host) {
    static std::once_flag once;
    static write_value32_fn fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (write_value32_fn)f;
        cudaGetLastError();
    });
    if (fn && fn((CUstream)s, (CUdeviceptr)(uintptr_t)flag, (cuuint32_t)*epoch_host, CU_STREAM_WRITE_VALUE_DEFAULT) ==
                  CUDA_SUCCESS)
        return FL_SUCCESS;
    FL_CUDA(cudaMemcpyAsync(flag, epoch_host, sizeof(int), cudaMemcpyHostToDevice, s));
    return FL_SUCCESS;
}
}  // namespace fl

using namespace fl;

namespace {

constexpr long kMaxNnz = 0x7fffffffL - 65536;  // headroom for padding and item rounding

int check_sizes(const char *who, int m, int n, int nnz) {
    if (m < 0 || n < 0 || nnz < 0)
        return fail(FL_ERR_ARG, "%s: negative size (m=%d n=%d nnz=%d)", who, m, n, nnz);
    if ((long)nnz > kMaxNnz) return fail(FL_ERR_OVERFLOW, "%s: nnz=%d exceeds the 32-bit index space", who, nnz);
    return FL_SUCCESS;
}

template <typename T>
int upload(DevBuf<T> &d, const T *h, size_t count, cudaStream_t s) {
    FL_TRY(d.alloc(count, s));
    if (count) FL_CUDA(cudaMemcpyAsync(d.get(), h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return FL_SUCCESS;
}
template <typename T>
int download(T *h, const T *d, size_t count, cudaStream_t s) {
    if (count) FL_CUDA(cudaMemcpyAsync(h, d, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    return FL_SUCCESS;
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    int start(cudaStream_t s) {
        FL_CUDA(cudaEventCreate(&a));
        FL_CUDA(cudaEventCreate(&b));
        FL_CUDA(cudaEventRecord(a, s));
        return FL_SUCCESS;
    }
    int stop(cudaStream_t s, double *ms) {
        FL_CUDA(cudaEventRecord(b, s));
        FL_CUDA(cudaEventSynchronize(b));
        float f = 0;
        FL_CUDA(cudaEventElapsedTime(&f, a, b));
        if (ms) *ms = f;
        return FL_SUCCESS;
    }
    ~Timer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// On an error return of a host-buffer call, waits for the work the call has
// already queued on its streams, so that no copy from or into the caller's
// (possibly pinned) host buffers is still running once the call returns.
// Disarmed on success: the pipelined call returns with its copies in flight
// by design.
struct DrainOnError {
    cudaStream_t st[4];
    int n = 0;
    bool ok = false;
    void add(cudaStream_t s) {
        if (n < 4) st[n++] = s;
    }
    ~DrainOnError() {
        if (ok) return;
        for (int i = 0; i < n; i++) cudaStreamSynchronize(st[i]);
    }
};

template <typename T>
T *host_alloc(size_t count) {
    return (T *)calloc(count ? count : 1, sizeof(T));
}

// D2H of the reference layout into malloc'd arrays of *out.
int export_layout(const Layout &L, fl_slide_matrix *out, cudaStream_t s) {
    fl_slide_matrix m;
    memset(&m, 0, sizeof m);
    const int T = L.tilenum, S = L.segsum, Z = L.nnz;
    m.sortval = host_alloc<double>(Z);
    m.sortrowidx = host_alloc<int>(Z);
    m.tile_ptr = host_alloc<int>((size_t)T + 1);
    m.tile_len = host_alloc<int>(T);
    m.tile_colidx = host_alloc<int>(T);
    m.tile_tall = host_alloc<int>(T);
    m.tile_format = host_alloc<int>(T);
    m.countrow = host_alloc<int>((size_t)T + 1);
    m.segmentoffset = host_alloc<int>((size_t)S + 1);
    m.sortrowindex = host_alloc<int>(Z);
    m.tilenum = T;
    m.segsum = S;
    if (!m.sortval || !m.sortrowidx || !m.tile_ptr || !m.tile_len || !m.tile_colidx || !m.tile_tall ||
        !m.tile_format || !m.countrow || !m.segmentoffset || !m.sortrowindex) {
        fl_tile_destroy(&m);
        return fail(FL_ERR_ALLOC, "formatTransform: host allocation failed");
    }
    int rc = FL_SUCCESS;
    if (Z) {
        if ((rc = download(m.sortval, L.val.get(), Z, s))) goto bad;
        if ((rc = download(m.sortrowidx, L.row.get(), Z, s))) goto bad;
        if ((rc = download(m.sortrowindex, L.sortrowindex.get(), Z, s))) goto bad;
    }
    if ((rc = download(m.tile_ptr, L.tile_ptr.get(), (size_t)T + 1, s))) goto bad;
    if ((rc = download(m.countrow, L.countrow.get(), (size_t)T + 1, s))) goto bad;
    if ((rc = download(m.segmentoffset, L.segmentoffset.get(), (size_t)S + 1, s))) goto bad;
    if (T) {
        if ((rc = download(m.tile_len, L.tile_len.get(), T, s))) goto bad;
        if ((rc = download(m.tile_colidx, L.tile_colidx.get(), T, s))) goto bad;
        if ((rc = download(m.tile_format, L.tile_format.get(), T, s))) goto bad;
    }
    {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = fail(FL_ERR_CUDA, "formatTransform: copy-back failed: %s", cudaGetErrorString(e));
            goto bad;
        }
    }
    *out = m;
    return FL_SUCCESS;
bad:
    fl_tile_destroy(&m);
    return rc;
}

// Uploads a host slide_matrix into a device layout (for FastLoad_spmv).
// The step table the streaming kernel needs is re-derived from the tile
// arrays: sorted column c has as many nonzeros as tiles that cover it, and
// those counts determine the staircase.  check_tile_meta then confirms the
// uploaded tile arrays are exactly the staircase's, so deriving columns
// arithmetically is valid for this matrix.
__global__ void k_cover_count(int tilenum, const int *tile_colidx, const int *tile_len, int *cnt) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < tilenum; t += (long)gridDim.x * blockDim.x) {
        int c = tile_colidx[t], len = tile_len[t];
        for (int i = 0; i < len; i++) atomicAdd(cnt + c + i, 1);
    }
}

__global__ void k_check_layout(int tilenum, int n, int m, int nnz, const int *tile_ptr, const int *tile_len,
                               const int *tile_colidx, const int *row, int *err) {
    long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, stride = (long)gridDim.x * blockDim.x;
    int e = 0;
    for (long t = tid; t < tilenum; t += stride) {
        int len = tile_len[t], c = tile_colidx[t];
        if (len < 1 || len > 32 || c < 0 || c + len > n) e |= 1;
        if (tile_ptr[t + 1] - tile_ptr[t] != len) e |= 2;
    }
    for (long p = tid; p < nnz; p += stride) {
        int r = row[p];
        if (r < 0 || r >= m) e |= 4;
    }
    if (tid == 0 && (tile_ptr[0] != 0 || tile_ptr[tilenum] != nnz)) e |= 8;
    if (e) atomicOr(err, e);
}

int upload_layout(Layout &L, const fl_slide_matrix *mat, int m, int n, int nnz, cudaStream_t s) {
    const int T = mat->tilenum;
    if (T < 0) return fail(FL_ERR_ARG, "FastLoad_spmv: tilenum=%d", T);
    if (nnz > 0 && (!mat->sortval || !mat->sortrowidx || !mat->tile_ptr || !mat->tile_len || !mat->tile_colidx))
        return fail(FL_ERR_ARG, "FastLoad_spmv: slide_matrix has NULL arrays");
    L.m = m;
    L.n = n;
    L.nnz = nnz;
    L.tilenum = T;
    size_t np = padded(nnz);
    FL_TRY(L.row.alloc(np, s));
    FL_TRY(L.val.alloc(np, s));
    FL_CUDA(cudaMemsetAsync(L.row.get() + nnz, 0xff, (np - nnz) * sizeof(int), s));
    FL_CUDA(cudaMemsetAsync(L.val.get() + nnz, 0, (np - nnz) * sizeof(double), s));
    if (nnz) {
        FL_CUDA(cudaMemcpyAsync(L.row.get(), mat->sortrowidx, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice, s));
        FL_CUDA(cudaMemcpyAsync(L.val.get(), mat->sortval, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    DevBuf<int> tptr, tlen, tcol, cnt, err;
    FL_TRY(upload(tptr, mat->tile_ptr, (size_t)T + 1, s));
    FL_TRY(upload(tlen, mat->tile_len, T, s));
    FL_TRY(upload(tcol, mat->tile_colidx, T, s));
    FL_TRY(err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), s));
    k_check_layout<<<256, 256, 0, s>>>(T, n, m, nnz, tptr.get(), tlen.get(), tcol.get(), L.row.get(), err.get());
    FL_CUDA(cudaGetLastError());
    int herr = 0;
    FL_TRY(download(&herr, err.get(), 1, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (herr) return fail(FL_ERR_ARG, "FastLoad_spmv: slide_matrix is not a valid FastLoad layout for "
                                      "colA=%d rowA=%d nnz=%d (flags 0x%x)", n, m, nnz, herr);
    // nnz per sorted column from tile coverage, then the step table
    FL_TRY(cnt.alloc((size_t)n + 1, s));
    if (n) FL_CUDA(cudaMemsetAsync(cnt.get(), 0, (size_t)n * sizeof(int), s));
    if (T) {
        k_cover_count<<<256, 256, 0, s>>>(T, tcol.get(), tlen.get(), cnt.get());
        FL_CUDA(cudaGetLastError());
    }
    FL_TRY(build_steps(L, m, n, nnz, cnt.get(), s));
    if (L.tilenum != T) return fail(FL_ERR_ARG, "FastLoad_spmv: tilenum=%d but the tiles imply %d", T, L.tilenum);
    FL_TRY(check_tile_meta(L, tptr.get(), tlen.get(), tcol.get(), s));
    L.sortnnz = std::move(cnt);  // nnz per sorted column (the staircase the tiles were checked against)
    return FL_SUCCESS;
}

}  // namespace

extern "C" {

const char *fl_last_error(void) { return last_error_cstr(); }
const char *fl_version(void) { return "fastload_gb300 0.1 (sm_103a)"; }
int fl_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
void fl_debug_fail_alloc_after(int countdown) { debug_fail_alloc_after(countdown); }
void fl_debug_hold_x_upload(int hold) { g_hold_x_flag = hold != 0; }

int fl_csr_to_csc(double *time_ms, int m, int n, int nnz, const double *csr_val, const int *csr_row_ptr,
                  const int *csr_col_ind, double *csc_val, int *csc_row_ind, int *csc_col_ptr, int *nnzpercol) {
    clear_error();
    FL_TRY(check_sizes("csr_to_csc", m, n, nnz));
    if (!csr_row_ptr || !csc_col_ptr || !nnzpercol || (nnz && (!csr_val || !csr_col_ind || !csc_val || !csc_row_ind)))
        return fail(FL_ERR_ARG, "csr_to_csc: NULL array");
    cudaStream_t s = 0;
    SyncAtExit drain{s};
    DevBuf<int> rp, ci, cp, cr, npc;
    DevBuf<double> v, cv;
    FL_TRY(upload(rp, csr_row_ptr, (size_t)m + 1, s));
    FL_TRY(upload(ci, csr_col_ind, nnz, s));
    FL_TRY(upload(v, csr_val, nnz, s));
    FL_TRY(cp.alloc((size_t)n + 1, s));
    FL_TRY(cr.alloc(nnz, s));
    FL_TRY(cv.alloc(nnz, s));
    FL_TRY(npc.alloc(n, s));
    Timer t;
    FL_TRY(t.start(s));
    FL_TRY(csr_to_csc_device(m, n, nnz, rp.get(), ci.get(), v.get(), cp.get(), cr.get(), cv.get(), npc.get(), s));
    FL_TRY(t.stop(s, time_ms));
    FL_TRY(download(csc_col_ptr, cp.get(), (size_t)n + 1, s));
    FL_TRY(download(nnzpercol, npc.get(), n, s));
    FL_TRY(download(csc_row_ind, cr.get(), nnz, s));
    FL_TRY(download(csc_val, cv.get(), nnz, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

int fl_col_sort(double *time_ms, int rowA, int colA, int nnz, const int *nnzPerCol, const int *cscColPtr,
                const int *cscRowIdx, const double *cscVal, int *sortrowidxTmp, double *sortvalTmp, int *sortnnzTmp,
                const double *x, double *sortx) {
    clear_error();
    FL_TRY(check_sizes("ColSort", rowA, colA, nnz));
    if ((colA && (!nnzPerCol || !cscColPtr || !sortnnzTmp)) ||
        (nnz && (!cscRowIdx || !cscVal || !sortrowidxTmp || !sortvalTmp)) || (colA && x && !sortx))
        return fail(FL_ERR_ARG, "ColSort: NULL array");
    cudaStream_t s = 0;
    SyncAtExit drain{s};
    DevBuf<int> cnt, cp, cr, perm, snnz, srow;
    DevBuf<double> cv, dx, dxs, sval;
    FL_TRY(upload(cnt, nnzPerCol, colA, s));
    FL_TRY(upload(cp, cscColPtr, (size_t)colA + 1, s));
    FL_TRY(upload(cr, cscRowIdx, nnz, s));
    FL_TRY(upload(cv, cscVal, nnz, s));
    if (x) {
        FL_TRY(upload(dx, x, colA, s));
        FL_TRY(dxs.alloc(colA, s));
    }
    FL_TRY(perm.alloc(colA, s));
    FL_TRY(snnz.alloc(colA, s));
    FL_TRY(srow.alloc(nnz, s));
    FL_TRY(sval.alloc(nnz, s));
    Timer t;
    FL_TRY(t.start(s));
    FL_TRY(col_sort_device(colA, nnz, cnt.get(), cp.get(), cr.get(), cv.get(), x ? dx.get() : nullptr, perm.get(),
                           snnz.get(), srow.get(), sval.get(), x ? dxs.get() : nullptr, s));
    FL_TRY(t.stop(s, time_ms));
    FL_TRY(download(sortnnzTmp, snnz.get(), colA, s));
    FL_TRY(download(sortrowidxTmp, srow.get(), nnz, s));
    FL_TRY(download(sortvalTmp, sval.get(), nnz, s));
    if (x) FL_TRY(download(sortx, dxs.get(), colA, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

int fl_format_transform(double *time_tran_ms, double *time_class_ms, fl_slide_matrix *matrix,
                        const int *sortrowidx_tmp, const double *sortval_tmp, const int *sortnnz_tmp, int nnz,
                        int rowA, int colA, int *h_count) {
    clear_error();
    FL_TRY(check_sizes("formatTransform", rowA, colA, nnz));
    if (!matrix || (colA && !sortnnz_tmp) || (nnz && (!sortrowidx_tmp || !sortval_tmp)))
        return fail(FL_ERR_ARG, "formatTransform: NULL argument");
    cudaStream_t s = 0;
    SyncAtExit drain{s};
    DevBuf<int> snnz, srow;
    DevBuf<double> sval;
    FL_TRY(upload(snnz, sortnnz_tmp, colA, s));
    FL_TRY(upload(srow, sortrowidx_tmp, nnz, s));
    FL_TRY(upload(sval, sortval_tmp, nnz, s));
    Layout L;
    float a = 0, b = 0;
    FL_TRY(build_layout_device(L, rowA, colA, nnz, snnz.get(), srow.get(), sval.get(), true, s, &a, &b));
    if (time_tran_ms) *time_tran_ms = a;
    if (time_class_ms) *time_class_ms = b;
    if (h_count) *h_count = L.st.steps;
    return export_layout(L, matrix, s);
}

int fl_fastload_spmv(const fl_slide_matrix *matrix, int nnz, int colA, int rowA, const double *x_sorted, double *y,
                     const double *y_golden, int reps, double *ms_per_spmv, int *mismatches) {
    clear_error();
    FL_TRY(check_sizes("FastLoad_spmv", rowA, colA, nnz));
    if (!matrix || (colA && !x_sorted) || (rowA && !y)) return fail(FL_ERR_ARG, "FastLoad_spmv: NULL argument");
    if (reps < 0) return fail(FL_ERR_ARG, "FastLoad_spmv: reps=%d", reps);
    cudaStream_t s = 0;
    SyncAtExit drain{s};
    Layout L;
    FL_TRY(upload_layout(L, matrix, rowA, colA, nnz, s));
    // The bucketed split of the uploaded layout when it has a band of dense
    // columns (the plans' first rule; their second, rows as slices for local
    // or row-skewed matrices, needs the column permutation, which a
    // slide_matrix does not carry): the densest columns as row slices, the
    // rest as the FastLoad stream; else the FastLoad stream kernel.
    Bucket B;
    int nh = 0;
    if (nnz > 0) {
        nh = bucket_auto_band(L.sortnnz.get(), colA, nnz, s);
        if (nh < 0) return nh;
    }
    if (nh > 0) {
        DevBuf<int> srow;
        DevBuf<double> sval;
        FL_TRY(untile_layout(L, srow, sval, s));
        FL_TRY(build_bucket(B, rowA, colA, nnz, L.sortnnz.get(), srow.get(), sval.get(), nh, s));
    }
    DevBuf<double> dx, dy;
    FL_TRY(upload(dx, x_sorted, colA, s));
    FL_TRY(dy.alloc(rowA, s));
    auto run = [&]() -> int {
        return nh > 0 ? spmv_bucket_f64(B, dx.get(), dy.get(), 1, s)
                      : spmv_stream_f64(L, dx.get(), dy.get(), FL_KERNEL_AUTO, s);
    };
    if (rowA) FL_CUDA(cudaMemsetAsync(dy.get(), 0, (size_t)rowA * sizeof(double), s));
    FL_TRY(run());  // untimed first run
    double total = 0;
    for (int r = 0; r < reps; r++) {
        if (rowA) FL_CUDA(cudaMemsetAsync(dy.get(), 0, (size_t)rowA * sizeof(double), s));
        Timer t;
        double ms = 0;
        FL_TRY(t.start(s));
        FL_TRY(run());
        FL_TRY(t.stop(s, &ms));
        total += ms;
    }
    if (reps == 0 && rowA) {
        FL_CUDA(cudaMemsetAsync(dy.get(), 0, (size_t)rowA * sizeof(double), s));
        FL_TRY(run());
    }
    FL_TRY(download(y, dy.get(), rowA, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (nh > 0) {
        int h = 0;
        FL_CUDA(cudaMemcpy(&h, B.err.get(), sizeof(int), cudaMemcpyDeviceToHost));
        if (h) return fail(FL_ERR_NOT_READY, "FastLoad_spmv: a bounded device wait expired (0x%x)", h);
    }
    if (ms_per_spmv) *ms_per_spmv = reps ? total / reps : 0.0;
    if (mismatches) {
        int bad = 0;
        if (y_golden)
            for (int i = 0; i < rowA; i++) {
                double d = y_golden[i] - y[i];
                if (d < 0) d = -d;
                double a = y[i] < 0 ? -y[i] : y[i];
                if (d > 0.01 * a) bad++;
            }
        *mismatches = bad;
    }
    return FL_SUCCESS;
}

void fl_tile_destroy(fl_slide_matrix *m) {
    if (!m) return;
    free(m->sortval);
    free(m->sortrowidx);
    free(m->tile_ptr);
    free(m->tile_len);
    free(m->tile_colidx);
    free(m->tile_tall);
    free(m->tile_format);
    free(m->countrow);
    free(m->segmentoffset);
    free(m->sortrowindex);
    memset(m, 0, sizeof *m);
}

// ------------------------------------------------------------ plan API --
static int plan_from_csc(fl_plan_t *out, int m, int n, int nnz, const int *colptr, const int *rowidx,
                         const double *val, const fl_plan_opts &o, cudaStream_t s) {
    std::unique_ptr<fl_plan> p(new (std::nothrow) fl_plan());
    if (!p) return fail(FL_ERR_ALLOC, "plan: host allocation failed");
    DevBuf<int> cnt, srow;
    DevBuf<double> sval;
    FL_TRY(cnt.alloc(n, s));
    FL_TRY(p->L.perm.alloc(n, s));
    FL_TRY(p->L.sortnnz.alloc(n, s));
    FL_TRY(srow.alloc(nnz, s));
    FL_TRY(sval.alloc(nnz, s));
    FL_TRY(counts_from_ptr(colptr, n, cnt.get(), s));
    FL_TRY(col_sort_device(n, nnz, cnt.get(), colptr, rowidx, val, nullptr, p->L.perm.get(), p->L.sortnnz.get(),
                           srow.get(), sval.get(), nullptr, s));
    FL_TRY(build_layout_device(p->L, m, n, nnz, p->L.sortnnz.get(), srow.get(), sval.get(),
                               o.with_reference_arrays != 0, s, nullptr, nullptr));
    p->has_ref = o.with_reference_arrays != 0;
    if (o.heavy_band >= 0) {
        int nh = o.heavy_band;
        bool wide = false;
        if (nh == 0) {
            nh = auto_layout_band(p->L, 8, &wide, s);
            if (nh < 0) return nh;
        } else if (nh > bucket_max_band() || nh > n) {
            return fail(FL_ERR_ARG, "plan: heavy_band=%d exceeds min(n=%d, %d)", nh, n, bucket_max_band());
        }
        if (nh > 0) {
            p->bucket.reset(new (std::nothrow) Bucket());
            if (!p->bucket) return fail(FL_ERR_ALLOC, "plan: host allocation failed");
            FL_TRY(build_bucket(*p->bucket, m, n, nnz, p->L.sortnnz.get(), srow.get(), sval.get(), nh, s, wide));
        }
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(FL_ERR_CUDA, "plan: %s", cudaGetErrorString(e));
    *out = p.release();
    return FL_SUCCESS;
}

static fl_plan_opts default_opts(int with_ref) {
    fl_plan_opts o;
    memset(&o, 0, sizeof o);
    o.with_reference_arrays = with_ref;
    return o;
}

int fl_plan_max_heavy_band(void) { return bucket_max_band(); }

int fl_plan_create(fl_plan_t *plan, int input_format, int m, int n, int nnz, const int *d_ptr, const int *d_idx,
                   const double *d_val, const fl_plan_opts *opts, void *stream) {
    clear_error();
    if (!plan) return fail(FL_ERR_ARG, "plan_create: NULL plan pointer");
    *plan = nullptr;
    FL_TRY(check_sizes("plan_create", m, n, nnz));
    if (!d_ptr || (nnz && (!d_idx || !d_val))) return fail(FL_ERR_ARG, "plan_create: NULL array");
    if (input_format != FL_INPUT_CSR && input_format != FL_INPUT_CSC)
        return fail(FL_ERR_ARG, "plan_create: unknown input format %d", input_format);
    const fl_plan_opts o = opts ? *opts : default_opts(0);
    if (o.heavy_band < -1) return fail(FL_ERR_ARG, "plan_create: heavy_band=%d", o.heavy_band);
    cudaStream_t s = (cudaStream_t)stream;
    if (input_format == FL_INPUT_CSC) {
        FL_TRY(check_index_range(d_idx, nnz, m, "plan_create: row index", s));
        return plan_from_csc(plan, m, n, nnz, d_ptr, d_idx, d_val, o, s);
    }
    DevBuf<int> cp, cr, npc;
    DevBuf<double> cv;
    FL_TRY(cp.alloc((size_t)n + 1, s));
    FL_TRY(cr.alloc(nnz, s));
    FL_TRY(cv.alloc(nnz, s));
    FL_TRY(npc.alloc(n, s));
    FL_TRY(csr_to_csc_device(m, n, nnz, d_ptr, d_idx, d_val, cp.get(), cr.get(), cv.get(), npc.get(), s));
    return plan_from_csc(plan, m, n, nnz, cp.get(), cr.get(), cv.get(), o, s);
}

int fl_plan_create_csc(fl_plan_t *plan, int m, int n, int nnz, const int *d_colptr, const int *d_rowidx,
                       const double *d_val, int with_reference_arrays, void *stream) {
    const fl_plan_opts o = default_opts(with_reference_arrays);
    return fl_plan_create(plan, FL_INPUT_CSC, m, n, nnz, d_colptr, d_rowidx, d_val, &o, stream);
}

int fl_plan_create_csr(fl_plan_t *plan, int m, int n, int nnz, const int *d_rowptr, const int *d_colidx,
                       const double *d_val, int with_reference_arrays, void *stream) {
    const fl_plan_opts o = default_opts(with_reference_arrays);
    return fl_plan_create(plan, FL_INPUT_CSR, m, n, nnz, d_rowptr, d_colidx, d_val, &o, stream);
}

int fl_plan_info_get(fl_plan_t p, fl_plan_info *info) {
    clear_error();
    if (!p || !info) return fail(FL_ERR_ARG, "plan_info: NULL argument");
    const Layout &L = p->L;
    info->m = L.m;
    info->n = L.n;
    info->nnz = L.nnz;
    info->tilenum = L.tilenum;
    info->steps = L.st.steps;
    info->segsum = p->has_ref ? L.segsum : -1;
    info->regions = L.regions.nregions;
    info->items = L.regions.nitems;
    size_t b = L.row.n * 4 + L.val.n * 8 + L.perm.n * 4 + L.sortnnz.n * 4 + L.tile_ptr.n * 4 + L.tile_len.n * 4 +
               L.tile_colidx.n * 4 + L.tile_format.n * 4 + L.sortrowindex.n * 4 + L.countrow.n * 4 +
               L.segmentoffset.n * 4 + L.regions.region.n * sizeof(RegionDesc) +
               L.regions.item.n * sizeof(ItemDesc) + 5 * (size_t)(L.st.steps + 1) * 4;
    info->heavy_cols = 0;
    info->heavy_nnz = 0;
    info->heavy_slices = 0;
    info->heavy_padded = 0;
    info->spmv_launches = (L.m > 0) + (L.regions.nitems > 0);
    if (p->bucket) {
        const Bucket &B = *p->bucket;
        const HeavyBand &H = B.heavy;
        const bool owned = B.light.regions.nitems == 0 && !H.split && H.nrows == L.m;
        info->spmv_launches = (L.m > 0 && !owned) + (B.light.regions.nitems > 0 || (H.nnz > 0 && H.nunits > 0));
        info->heavy_cols = H.nh;
        info->heavy_nnz = (int)H.nnz;
        info->heavy_slices = H.nslices;
        info->heavy_padded = (int)H.padded;
        const Layout &Q = B.light;
        b += Q.row.n * 4 + Q.val.n * 8 + Q.regions.region.n * sizeof(RegionDesc) +
             Q.regions.item.n * sizeof(ItemDesc) + 5 * (size_t)(Q.st.steps + 1) * 4;
        b += H.val.n * 8 + H.col.n * 2 + H.col32.n * 4 + H.slice_ptr.n * 4 + H.row.n * 4 + H.len.n * 4;
    }
    info->device_bytes = b;
    return FL_SUCCESS;
}

int fl_plan_export(fl_plan_t p, fl_slide_matrix *matrix, int *perm) {
    clear_error();
    if (!p || !matrix) return fail(FL_ERR_ARG, "plan_export: NULL argument");
    if (!p->has_ref) return fail(FL_ERR_ARG, "plan_export: plan was built without reference arrays");
    cudaStream_t s = 0;
    FL_CUDA(cudaDeviceSynchronize());
    if (perm && p->L.n) {
        FL_TRY(download(perm, p->L.perm.get(), p->L.n, s));
        FL_CUDA(cudaStreamSynchronize(s));
    }
    return export_layout(p->L, matrix, s);
}

int fl_plan_permute_x(fl_plan_t p, const double *d_x, double *d_xs, void *stream) {
    clear_error();
    if (!p || (p->L.n && (!d_x || !d_xs))) return fail(FL_ERR_ARG, "plan_permute_x: NULL argument");
    return permute_x(p->L.perm.get(), p->L.n, d_x, d_xs, (cudaStream_t)stream);
}

int fl_plan_spmv(fl_plan_t p, const double *d_xs, double *d_y, int accumulate, int variant, void *stream) {
    if (!p || (p->L.n && !d_xs) || (p->L.m && !d_y)) return fail(FL_ERR_ARG, "plan_spmv: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (variant == FL_KERNEL_AUTO && p->bucket) variant = FL_KERNEL_BUCKET;
    if (variant == FL_KERNEL_BUCKET) {
        if (!p->bucket) return fail(FL_ERR_ARG, "plan_spmv: the plan has no heavy band");
        return spmv_bucket_f64(*p->bucket, d_xs, d_y, accumulate, s);
    }
    if (!accumulate) FL_TRY(zero_device(d_y, (size_t)p->L.m * sizeof(double), s));
    switch (variant) {
        case FL_KERNEL_AUTO: return spmv_stream_f64(p->L, d_xs, d_y, FL_KERNEL_STREAM, s);
        case FL_KERNEL_STREAM:
        case FL_KERNEL_STREAM2: return spmv_stream_f64(p->L, d_xs, d_y, variant, s);
        case FL_KERNEL_TILE: return spmv_tile_f64(p->L, d_xs, d_y, s);
        default: return fail(FL_ERR_ARG, "plan_spmv: unknown kernel variant %d", variant);
    }
}

int fl_plan_spmv_host(fl_plan_t p, const double *h_xs, double *h_y, int variant, void *stream) {
    clear_error();
    if (!p || (p->L.n && !h_xs) || (p->L.m && !h_y)) return fail(FL_ERR_ARG, "plan_spmv_host: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    DrainOnError drain;
    drain.add(s);
    if (p->stage_x.n < (size_t)p->L.n) FL_TRY(p->stage_x.alloc(p->L.n, s));
    if (p->stage_y.n < (size_t)p->L.m) FL_TRY(p->stage_y.alloc(p->L.m, s));
    double *dx = p->stage_x.get();
    const Bucket *B = p->bucket.get();
    const bool overlap = B && (variant == FL_KERNEL_AUTO || variant == FL_KERNEL_BUCKET) && bucket_overlap_ok(*B);
    if (!overlap) {
        if (p->L.n)
            FL_CUDA(cudaMemcpyAsync(dx, h_xs, (size_t)p->L.n * sizeof(double), cudaMemcpyHostToDevice, s));
        FL_TRY(fl_plan_spmv(p, dx, p->stage_y.get(), 0, variant, stream));
    } else {
        // The heavy band reads x only in [H0, n): upload that (at most 128 KB)
        // on s and launch.  The light columns' x [0, H0) follows on the side
        // stream, then the call's epoch into x_flag.  The kernel runs the
        // band while that copy is in flight and takes the light items once
        // the epoch is in.
        const int H0 = B->heavy.H0;
        if (!B->light_fine_built) {
            // the light items of this call run after most of the band, on
            // every warp: cut finer than the device-resident kernel's
            Bucket *Bm = p->bucket.get();
            FL_TRY(build_regions_sized(Bm->light, item_nnz_for(Bm->light.nnz), Bm->light_fine, s));
            Bm->light_fine_built = true;
        }
        if (!p->side) FL_CUDA(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
        if (!p->fork) FL_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        if (!p->join) FL_CUDA(cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming));
        drain.add(p->side);
        if (!p->epoch_host) {
            // [0] the epoch word, [1] the kernel's status word (written by the
            // kernel through the mapping only when a wait expires)
            FL_CUDA(cudaHostAlloc((void **)&p->epoch_host, 2 * sizeof(int), cudaHostAllocMapped));
            p->epoch_host[0] = p->epoch_host[1] = 0;
            FL_CUDA(cudaHostGetDevicePointer((void **)&p->epoch_dev, p->epoch_host, 0));
        }
        if (!p->x_flag.get()) {
            FL_TRY(p->x_flag.alloc(1, s));
            FL_CUDA(cudaMemsetAsync(p->x_flag.get(), 0, sizeof(int), s));
        }
        // the previous call has finished (this call is synchronous), so the
        // pinned words are free to rewrite
        p->epoch = (int)((unsigned)p->epoch + 1u);  // compared modulo 2^32 by the kernel
        p->epoch_host[0] = p->epoch;
        p->epoch_host[1] = 0;
        // the band's x first: host-to-device copies share a copy engine, so
        // a band copy queued behind the light columns' would wait for it
        FL_CUDA(cudaMemcpyAsync(dx + H0, h_xs + H0, (size_t)(p->L.n - H0) * sizeof(double),
                                cudaMemcpyHostToDevice, s));
        // the side stream follows earlier work on s that reads stage_x or
        // x_flag, but not this call's kernel (which waits for it)
        FL_CUDA(cudaEventRecord(p->fork, s));
        // launched first, so the host's remaining calls overlap the band
        const XUpload xu{p->x_flag.get(), p->epoch, p->epoch_dev + 1};
        FL_TRY(spmv_bucket_f64(*B, dx, p->stage_y.get(), 0, s, &xu));
        // nothing queued after the kernel is issued before these, so no copy
        // the kernel waits for sits behind one that waits for the kernel
        FL_CUDA(cudaStreamWaitEvent(p->side, p->fork, 0));
        FL_CUDA(cudaMemcpyAsync(dx, h_xs, (size_t)H0 * sizeof(double), cudaMemcpyHostToDevice, p->side));
        if (!g_hold_x_flag) FL_TRY(signal_epoch(p->side, p->x_flag.get(), p->epoch_host));
        FL_CUDA(cudaEventRecord(p->join, p->side));
        FL_CUDA(cudaStreamWaitEvent(s, p->join, 0));
    }
    FL_TRY(download(h_y, p->stage_y.get(), p->L.m, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (overlap && *(volatile int *)(p->epoch_host + 1)) {
        const int h = p->epoch_host[1];
        p->epoch_host[1] = 0;
        FL_CUDA(cudaMemsetAsync(B->err.get(), 0, sizeof(int), s));
        FL_CUDA(cudaStreamSynchronize(s));
        return fail(FL_ERR_NOT_READY, "plan_spmv_host: a bounded device wait expired (0x%x); y is incomplete", h);
    }
    drain.ok = true;
    return FL_SUCCESS;
}

int fl_plan_spmv_host_async(fl_plan_t p, const double *h_xs, double *h_y, int variant, void *stream) {
    clear_error();
    if (!p || (p->L.n && !h_xs) || (p->L.m && !h_y)) return fail(FL_ERR_ARG, "plan_spmv_host_async: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    // each handle on its own, so a call after a failed creation makes only
    // what is still missing
    for (cudaStream_t *st : {&p->up_s, &p->comp_s, &p->down_s})
        if (!*st) FL_CUDA(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    for (fl_plan::AsyncSlot &a : p->slot)
        for (cudaEvent_t *ev : {&a.up, &a.kdone, &a.down})
            if (!*ev) FL_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
    DrainOnError drain;
    drain.add(p->up_s);
    drain.add(p->comp_s);
    drain.add(p->down_s);
    fl_plan::AsyncSlot &S = p->slot[p->slot_next];
    // stream-ordered allocations on the upload stream: every later use of
    // the slot (compute, download) is ordered after the upload
    if (S.x.n < (size_t)p->L.n) FL_TRY(S.x.alloc(p->L.n, p->up_s));
    if (S.y.n < (size_t)p->L.m) FL_TRY(S.y.alloc(p->L.m, p->up_s));
    // The upload does not wait for earlier work on `stream`: that stream
    // waits for every earlier call's result, so ordering after it would
    // serialise the pipeline.  h_xs is read as it stands at the call.
    // upload: into the slot once the kernel two calls back has read it
    if (S.used) FL_CUDA(cudaStreamWaitEvent(p->up_s, S.kdone, 0));
    if (p->L.n)
        FL_CUDA(cudaMemcpyAsync(S.x.get(), h_xs, (size_t)p->L.n * sizeof(double), cudaMemcpyHostToDevice, p->up_s));
    FL_CUDA(cudaEventRecord(S.up, p->up_s));
    // compute: once x is in and the download two calls back has read y
    FL_CUDA(cudaStreamWaitEvent(p->comp_s, S.up, 0));
    if (S.used) FL_CUDA(cudaStreamWaitEvent(p->comp_s, S.down, 0));
    FL_TRY(fl_plan_spmv(p, S.x.get(), S.y.get(), 0, variant, p->comp_s));
    FL_CUDA(cudaEventRecord(S.kdone, p->comp_s));
    // download, and the caller's stream waits for it
    FL_CUDA(cudaStreamWaitEvent(p->down_s, S.kdone, 0));
    if (p->L.m)
        FL_CUDA(cudaMemcpyAsync(h_y, S.y.get(), (size_t)p->L.m * sizeof(double), cudaMemcpyDeviceToHost, p->down_s));
    FL_CUDA(cudaEventRecord(S.down, p->down_s));
    FL_CUDA(cudaStreamWaitEvent(s, S.down, 0));
    S.used = true;
    p->slot_next ^= 1;
    drain.ok = true;
    return FL_SUCCESS;
}

int fl_plan_add_form_opts(fl_plan_t p, const fl_form_opts *opts, int *form_id) {
    clear_error();
    if (!p || !opts || !form_id) return fail(FL_ERR_ARG, "add_form: NULL argument");
    std::unique_ptr<Form> F(new (std::nothrow) Form());
    if (!F) return fail(FL_ERR_ALLOC, "add_form: host allocation failed");
    FL_CUDA(cudaDeviceSynchronize());
    FL_TRY(build_form(*F, p->L, *opts, 0));
    p->forms.push_back(std::move(F));
    *form_id = (int)p->forms.size() - 1;
    return FL_SUCCESS;
}

int fl_plan_add_form(fl_plan_t p, int value_type, int heavy_band, int y_f32, int *form_id) {
    fl_form_opts o = {};
    o.value_type = value_type;
    o.heavy_band = heavy_band;
    o.y_f32 = y_f32 != 0;
    return fl_plan_add_form_opts(p, &o, form_id);
}

int fl_plan_form_opts_get(fl_plan_t p, int form_id, fl_form_opts *opts) {
    clear_error();
    if (!p || !opts || form_id < 0 || form_id >= (int)p->forms.size())
        return fail(FL_ERR_ARG, "form_opts_get: bad plan or form id");
    *opts = p->forms[form_id]->opts;
    return FL_SUCCESS;
}

int fl_plan_form_set_launch(fl_plan_t p, int form_id, int heavy_loop, int x_stage) {
    clear_error();
    if (!p || form_id < 0 || form_id >= (int)p->forms.size())
        return fail(FL_ERR_ARG, "form_set_launch: bad plan or form id");
    fl_form_opts o = p->forms[form_id]->opts;
    o.heavy_loop = heavy_loop;
    o.x_stage = x_stage;
    FL_TRY(check_form_opts(o));
    p->forms[form_id]->opts = o;
    return FL_SUCCESS;
}

int fl_plan_form_info(fl_plan_t p, int form_id, fl_form_info *info) {
    clear_error();
    if (!p || !info || form_id < 0 || form_id >= (int)p->forms.size())
        return fail(FL_ERR_ARG, "form_info: bad plan or form id");
    const Form &F = *p->forms[form_id];
    info->value_type = F.vtype;
    info->heavy_cols = F.B.heavy.nnz > 0 ? F.B.heavy.nh : 0;
    info->heavy_nnz = (int)F.B.heavy.nnz;
    info->light_nnz = F.B.light.nnz;
    info->y_f32 = F.yf32;
    const size_t vs = F.vtype == FL_VALUES_F64 ? 8 : 4;
    info->device_bytes = F.B.light.row.n * 4 + F.B.light.row.n * vs + F.B.heavy.padded * (vs + (F.wide ? 4 : 2)) +
                         F.B.heavy.row.n * 8 + F.B.light.regions.item.n * sizeof(ItemDesc);
    return FL_SUCCESS;
}

int fl_plan_spmv_form(fl_plan_t p, int form_id, int k, const void *d_xs, void *d_y, int accumulate, void *stream) {
    if (!p || form_id < 0 || form_id >= (int)p->forms.size()) return fail(FL_ERR_ARG, "spmv_form: bad plan or form id");
    if ((p->L.n && !d_xs) || (p->L.m && !d_y)) return fail(FL_ERR_ARG, "spmv_form: NULL argument");
    return spmv_form(*p->forms[form_id], k, d_xs, d_y, accumulate, (cudaStream_t)stream);
}

int fl_plan_permute_x_k(fl_plan_t p, int k, int to_f32, const double *d_x, void *d_xs, void *stream) {
    clear_error();
    if (!p || (p->L.n && (!d_x || !d_xs))) return fail(FL_ERR_ARG, "permute_x_k: NULL argument");
    if (k < 1) return fail(FL_ERR_ARG, "permute_x_k: k=%d", k);
    return permute_x_k(p->L.perm.get(), p->L.n, k, d_x, d_xs, to_f32, (cudaStream_t)stream);
}

int fl_plan_check(fl_plan_t p) {
    clear_error();
    if (!p) return fail(FL_ERR_ARG, "plan_check: NULL plan");
    FL_CUDA(cudaDeviceSynchronize());
    std::vector<const Bucket *> all;
    if (p->bucket) all.push_back(p->bucket.get());
    for (auto &f : p->forms) all.push_back(&f->B);
    for (const Bucket *b : all) {
        if (!b->err.get()) continue;
        int h = 0;
        FL_CUDA(cudaMemcpy(&h, b->err.get(), sizeof(int), cudaMemcpyDeviceToHost));
        FL_CUDA(cudaMemset(b->err.get(), 0, sizeof(int)));
        if (h)
            return fail(FL_ERR_NOT_READY,
                        "a bounded device wait expired (0x%x: 1, 2 staging of the heavy band's x; 4 the upload of "
                        "the light columns' x)", h);
    }
    return FL_SUCCESS;
}

int fl_plan_destroy(fl_plan_t p) {
    if (!p) return FL_SUCCESS;
    cudaDeviceSynchronize();  // no launch of this plan may still be reading it
    delete p;
    return FL_SUCCESS;
}

}  // extern "C"

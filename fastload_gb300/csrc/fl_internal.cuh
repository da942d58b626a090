// fl_internal.cuh -- shared internals of the FastLoad GB300 library:
// status handling, device buffers, the device-resident matrix layout and
// the launchers each translation unit exports to the others.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/fastload.h"

namespace fl {

// ---------------------------------------------------------------- status --
// Every entry point returns an int status (FL_SUCCESS or a negative code)
// and leaves a message readable through fl_last_error() on the same thread.
void set_error(int code, const std::string &msg);
int fail(int code, const char *fmt, ...);
void clear_error();

#define FL_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return ::fl::fail(FL_ERR_CUDA, "%s failed: %s (%s:%d)", #call,     \
                              cudaGetErrorString(e_), __FILE__, __LINE__);     \
    } while (0)

#define FL_TRY(expr)                                                           \
    do {                                                                       \
        int s_ = (expr);                                                       \
        if (s_ != FL_SUCCESS) return s_;                                       \
    } while (0)

// Allocation hook: tests install a countdown that makes the N-th device
// allocation fail, to exercise the error paths without touching the GPU.
int dev_alloc(void **p, size_t bytes, cudaStream_t s);
void dev_free(void *p, cudaStream_t s);

// Owning stream-ordered device buffer.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    int alloc(size_t count, cudaStream_t stream) {
        release();
        s = stream;
        n = count;
        if (count == 0) return FL_SUCCESS;
        return dev_alloc((void **)&p, count * sizeof(T), stream);
    }
    void release() {
        if (p) dev_free(p, s);
        p = nullptr;
        n = 0;
    }
    T *get() const { return p; }
};

// Synchronises a stream when it goes out of scope.  Declared before a
// synchronous host-buffer call's device buffers, it makes the call return,
// on every path, only after the copies it queued from or into the caller's
// host buffers (possibly pinned) have finished.
struct SyncAtExit {
    cudaStream_t s;
    ~SyncAtExit() { cudaStreamSynchronize(s); }
};

// ---------------------------------------------------------------- layout --
// Device-resident FastLoad layout of one matrix.  The tile-ordered value and
// row streams are the reference's sortval/sortrowidx (bit-identical); the
// step table replaces the per-tile metadata for the streaming kernels.
struct Regions;

struct StepTable {
    int steps = 0;              // h_count
    DevBuf<int> col;            // first sorted column of step s
    DevBuf<int> base;           // level of the step's first tile row
    DevBuf<int> tall;           // levels in the step
    DevBuf<int> tile_off;       // exclusive scan of tiles per step (steps+1)
    DevBuf<int> nnz_off;        // exclusive scan of nonzeros per step (steps+1)
};

// Work items for the streaming SpMV kernels.  A region is the full-chunk
// part or the partial-chunk part of one step; items cut regions into pieces
// of at most item_nnz_for(nnz) nonzeros whose interior boundaries sit on multiples of
// four, so 128-bit loads stay aligned.
struct RegionDesc {
    int start;     // first nonzero of the region (stream position)
    int col_base;  // first sorted column of the region
    int div;       // 32*tall for a full region, len for a partial region
    int full;      // 1: full 32-wide chunks, 0: the partial last chunk
};
struct ItemDesc {
    int begin;     // first nonzero of the piece
    int end;       // one past the last
    int region;    // index into the region table
    int pad;
};

struct Regions {
    int nregions = 0;
    int nitems = 0;
    DevBuf<RegionDesc> region;
    DevBuf<ItemDesc> item;
};

struct Layout {
    int m = 0, n = 0, nnz = 0;
    int tilenum = 0, segsum = 0;
    StepTable st;
    DevBuf<int> perm;           // sorted position -> original column
    DevBuf<int> sortnnz;        // nnz per sorted column
    // tile-ordered streams, padded to a multiple of FL_PAD entries
    DevBuf<int> row;            // sortrowidx (-1 in the padding)
    DevBuf<double> val;         // sortval (0 in the padding)
    // reference per-tile arrays (kept for export and the tile kernel)
    DevBuf<int> tile_ptr, tile_len, tile_colidx, tile_format;
    DevBuf<int> sortrowindex;
    DevBuf<int> countrow, segmentoffset;
    Regions regions;
    // nonzeros the work-item size is chosen for (item_nnz_for): the whole
    // matrix's, also for the light part of a bucketed split (0: nnz)
    long item_basis = 0;
};

// Heavy band of the bucketed form: the nh densest sorted columns, stored as
// slices of 32 rows (rows sorted by their band nonzero count, longest
// first); slice s holds width_s entries per lane, entry j of lane l at
// slice_ptr[s] + 32*j + l.  Columns are local (sorted column - H0) so they
// fit 16 bits and index the band's x staged in shared memory.
struct HeavyBand {
    int H0 = 0, nh = 0;         // first sorted column of the band, its width
    int nslices = 0, nrows = 0; // slices; rows with band nonzeros
    long nnz = 0;               // band nonzeros (no padding)
    long padded = 0;            // slice entries including padding
    DevBuf<double> val;
    DevBuf<uint16_t> col;       // local columns when nh <= 65535
    DevBuf<int> col32;          // local columns of wider bands
    DevBuf<int> slice_ptr;      // nslices+1
    DevBuf<int> row;            // 32*nslices, -1 for an empty lane
    DevBuf<int> len;            // 32*nslices
    // Work units are ranges of 32-entry steps (step t = entries 32t..32t+31;
    // the slices are contiguous, so a range may run over several short
    // slices or cover part of a long one).
    int nunits = 0;
    DevBuf<int> unit_step;      // nunits+1 step bounds
    DevBuf<int> unit_slice;     // nunits: the slice holding each unit's first step
    bool split = false;         // a slice is cut across units: its rows' sums meet in y by atomics
};

// Work units over slices whose entry offsets are sp (nslices+1, multiples
// of 32): consecutive short slices grouped to about per_unit entries (at
// least 256), slices longer than twice that cut into pieces of about
// per_unit entries.
// Returns true when a slice was cut.
bool make_units(const std::vector<int> &sp, long per_unit, std::vector<int> &unit_step,
                std::vector<int> &unit_slice);

// Bucketed form: light columns [0, H0) keep the FastLoad tile stream, the
// heavy band [H0, n) uses row slices.
struct Bucket {
    Layout light;
    HeavyBand heavy;
    DevBuf<int> err;            // device status word of the bucket kernel
    // the light part cut into finer work items (about two per warp of the
    // GPU for the light part alone) for the overlapped host call, whose
    // light items run once the band is mostly done; built on first use
    Regions light_fine;
    bool light_fine_built = false;
};

// A storage / right-hand-side form of a plan: its own bucketed split (light
// FastLoad stream + heavy band in row slices) with values in the form's
// storage type.  FP64 forms use the bucket's FP64 arrays directly.
struct Form {
    int vtype = 0;             // FL_VALUES_F64 / F32 / BF16X2
    int yf32 = 0;              // y accumulated in FP32 instead of FP64
    int band = 0;              // heavy band requested (FL_BAND_*)
    fl_form_opts opts = {};    // the options it was built with (launch options current)
    bool wide = false;         // band columns stored as 32-bit indices
    Bucket B;
    DevBuf<unsigned char> lval, hval;  // converted values (F32 / BF16X2 forms)
};

// Step table as raw pointers for kernels.
struct StepView {
    const int *col, *base, *tall, *tile_off, *nnz_off;
    int steps;
};

// Largest i in [0, cnt) with a[i] <= v (a non-decreasing, a[0] <= v).
__device__ __forceinline__ int upper_index(const int *__restrict__ a, int cnt, int v) {
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(a + mid) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr int FL_PAD = 512;     // stream padding granularity (entries)
constexpr int FL_ITEM = 2048;   // largest work item of the stream kernel (nonzeros)
// Work item size of a layout with nnz nonzeros (item_nnz_for in fl_prep.cu).
int item_nnz_for(long nnz);

inline size_t padded(size_t n) { return ((n + FL_PAD - 1) / FL_PAD + 1) * FL_PAD; }

// ---------------------------------------------------------- prep launchers --
// Device-wide exclusive scan of n ints; out may alias in.  When total is
// non-null the sum is written to total[0] (device memory).
int scan_exclusive(const int *in, int *out, long n, int *total, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
int radix_sort_pairs(unsigned *keys, unsigned *vals, long n, int bits, cudaStream_t s);
int max_reduce(const int *in, long n, int *out_dev, cudaStream_t s);

// CSR -> CSC transpose on the device (rows ascending per column).
int csr_to_csc_device(int m, int n, int nnz, const int *rowptr, const int *colidx,
                      const double *val, int *cscptr, int *cscrow, double *cscval,
                      int *nnzpercol, cudaStream_t s);
// Stable column sort; outputs are device arrays of the caller.
int col_sort_device(int n, int nnz, const int *nnzpercol, const int *cscptr,
                    const int *cscrow, const double *cscval, const double *x,
                    int *perm, int *sortnnz, int *sortrowidx_tmp, double *sortval_tmp,
                    double *sortx, cudaStream_t s);
// Builds the full layout from column-sorted CSC arrays (device pointers).
// with_reference_arrays: also build tile arrays, sortrowindex, countrow and
// segmentoffset (needed by the reference export and the tile kernel).
int build_layout_device(Layout &L, int m, int n, int nnz, const int *sortnnz,
                        const int *sortrowidx_tmp, const double *sortval_tmp,
                        bool with_reference_arrays, cudaStream_t s,
                        float *ms_tran, float *ms_class);
// Step table, tilenum and work items only (no payload): validates that
// sortnnz is non-negative, ascending and sums to nnz.
int build_steps(Layout &L, int m, int n, int nnz, const int *sortnnz, cudaStream_t s);
int build_regions(Layout &L, cudaStream_t s);
// Regions and work items of `item` nonzeros (a multiple of 4) over L's
// step table, into R.
int build_regions_sized(const Layout &L, int item, Regions &R, cudaStream_t s);
// Checks that host-provided per-tile arrays equal the ones the step table
// implies (so the streaming kernels may derive columns arithmetically).
int check_tile_meta(const Layout &L, const int *tile_ptr, const int *tile_len,
                    const int *tile_colidx, cudaStream_t s);
// cnt[c] = ptr[c+1] - ptr[c]
int counts_from_ptr(const int *ptr, int n, int *cnt, cudaStream_t s);
// FL_ERR_ARG unless every idx[i] is in [0, bound)
int check_index_range(const int *idx, long count, int bound, const char *what,
                      cudaStream_t s);
// xs[i] = x[perm[i]]
int permute_x(const int *perm, int n, const double *x, double *xs, cudaStream_t s);

// ---------------------------------------------------------- spmv launchers --
int spmv_stream_f64(const Layout &L, const double *xs, double *y, int variant,
                    cudaStream_t s);
int spmv_tile_f64(const Layout &L, const double *xs, double *y, cudaStream_t s);
// bytes (a multiple of 4) of zeros at p, by a kernel that the SpMV kernel
// launched behind it on s may overlap (programmatic dependent launch)
int zero_device(void *p, size_t bytes, cudaStream_t s);
// Bucketed form: build from the column-sorted CSC (device) and run.
// wide: allow a band of up to all n columns (x then read from global memory
// by the form kernels); otherwise the band is capped at bucket_max_band().
// unit_warps: heavy work units per resident warp (0: 4).
int build_bucket(Bucket &B, int m, int n, int nnz, const int *sortnnz, const int *srow_tmp,
                 const double *sval_tmp, int nh, cudaStream_t s, bool wide = false, int unit_warps = 0);
// The light columns' x (xs[0, H0)) still arriving while the bucket kernel
// runs (the overlapped host call): it is in once *flag reaches epoch;
// err_host is the device view of a host-mapped word that receives the
// status bits of an expired wait.
struct XUpload {
    const int *flag;
    int epoch;
    int *err_host;
};
// Whether the overlapped upload applies to B: light and heavy parts, the
// band's x staged in shared memory.
bool bucket_overlap_ok(const Bucket &B);
// y = A xs (accumulate 0) or y += A xs; xu: see XUpload (nullptr: x complete).
int spmv_bucket_f64(const Bucket &B, const double *xs, double *y, int accumulate, cudaStream_t s,
                    const XUpload *xu = nullptr);
// Largest heavy band the bucket kernel can stage in shared memory.
int bucket_max_band();
// Heavy band width chosen from the sorted column counts (device array):
// the densest columns with at least `min_degree` nonzeros, at most the
// shared-memory limit, or 0 when the band would hold little of the matrix.
int bucket_auto_band(const int *sortnnz, int n, int nnz, cudaStream_t s, int x_bytes = 8);
// The 24 tuner features of a layout (host array out[24]; out[23] left 0).
int plan_features(const Layout &L, float *out, cudaStream_t s);
// The automatic heavy band of a layout: the densest columns when they hold
// enough of the matrix; with none, every column as row slices when x
// gathers have locality, rows are skewed, or the matrix has 1M+ nonzeros and
// 4+ a column; else no band (0).  *wide is set when the band is wider than
// shared memory holds x for.
int auto_layout_band(const Layout &L, int x_bytes, bool *wide, cudaStream_t s);

int num_sms();

// Column-sorted CSC (rows, values) of a layout, recovered from its tile
// streams; needs L.sortnnz and the step table.
int untile_layout(const Layout &L, DevBuf<int> &srow, DevBuf<double> &sval, cudaStream_t s);

// Forms (fl_form.cu): build from a plan's FP64 layout, run.
int build_form(Form &F, const Layout &L, const fl_form_opts &o, cudaStream_t s);
// Range checks of form options (FL_ERR_ARG with a message).
int check_form_opts(const fl_form_opts &o);
int spmv_form(Form &F, int k, const void *xs, void *y, int accumulate, cudaStream_t s);
int permute_x_k(const int *perm, int n, int k, const double *x, void *xs, int to_f32, cudaStream_t s);

}  // namespace fl

// The plan object behind fl_plan_t.
#include <memory>
#include <vector>
struct fl_plan {
    fl::Layout L;
    bool has_ref = false;
    std::unique_ptr<fl::Bucket> bucket;           // bucketed FP64 form (heavy band), optional
    std::vector<std::unique_ptr<fl::Form>> forms; // storage / rhs forms
    fl::DevBuf<double> stage_x, stage_y;          // device staging of fl_plan_spmv_host
    // fl_plan_spmv_host overlaps the upload of the light columns' x with the
    // heavy band: that copy runs on a side stream, followed by a write of the
    // call's epoch into x_flag, on which the kernel's light items wait
    // (bounded)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    fl::DevBuf<int> x_flag;
    int *epoch_host = nullptr;                   // pinned, mapped: [0] epoch, [1] status
    int *epoch_dev = nullptr;                    // device view of epoch_host
    int epoch = 0;
    // fl_plan_spmv_host_async: two device staging slots used in turn, an
    // upload, a compute and a download stream.  A slot's x is overwritten
    // once the kernel that read it is done (kdone), its y once the copy that
    // read it is done (down).
    struct AsyncSlot {
        fl::DevBuf<double> x, y;
        cudaEvent_t up = nullptr, kdone = nullptr, down = nullptr;
        bool used = false;
    };
    AsyncSlot slot[2];
    int slot_next = 0;
    cudaStream_t up_s = nullptr, comp_s = nullptr, down_s = nullptr;
    fl_plan() = default;
    fl_plan(const fl_plan &) = delete;
    fl_plan &operator=(const fl_plan &) = delete;
    ~fl_plan() {
        // the device is idle here (fl_plan_destroy synchronises): free the
        // host-call staging on the legacy stream, before the streams they
        // were allocated on are destroyed (the caller's may be gone already)
        for (fl::DevBuf<double> *b : {&stage_x, &stage_y, &slot[0].x, &slot[0].y, &slot[1].x, &slot[1].y}) {
            b->s = 0;
            b->release();
        }
        x_flag.s = 0;
        x_flag.release();
        if (side) cudaStreamDestroy(side);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (epoch_host) cudaFreeHost(epoch_host);
        for (AsyncSlot &a : slot)
            for (cudaEvent_t e : {a.up, a.kdone, a.down})
                if (e) cudaEventDestroy(e);
        for (cudaStream_t st : {up_s, comp_s, down_s})
            if (st) cudaStreamDestroy(st);
    }
};

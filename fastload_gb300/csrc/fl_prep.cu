// fl_prep.cu -- GPU preprocessing of the FastLoad layout.
//
// Replaces the reference's csr_to_csc (src/csr2csc_cuda.h:51-135),
// ColSort (src/ColSort_GPU.h:46-136) and formatTransform
// (src/formatTransform_GPU.h:289-596) with device-resident map / scan /
// stable radix sort / gather passes.  No pass is quadratic: the reference's
// serial prefix loops (Pre4SortIdxVal, prepare, auxiliaryTrans) become
// scans, and the per-tile descriptors are computed arithmetically from a
// step table.  Outputs are bit-identical to the reference's layout.
#include "fl_internal.cuh"

#include <algorithm>
#include <cstring>
#include <cstdarg>
#include <cstdio>
#include <mutex>

namespace fl {

// ------------------------------------------------------------- errors ----
// the message of the calling thread's last failure (the code is the
// call's return value)
static thread_local std::string g_last_error;

void set_error(int, const std::string &msg) { g_last_error = msg; }
int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error(code, buf);
    return code;
}
void clear_error() { g_last_error.clear(); }
const char *last_error_cstr() { return g_last_error.c_str(); }

// ---------------------------------------------------------- allocation ---
static int g_fail_countdown = 0;
static std::mutex g_alloc_mu;

int dev_alloc(void **p, size_t bytes, cudaStream_t s) {
    {
        std::lock_guard<std::mutex> lk(g_alloc_mu);
        if (g_fail_countdown > 0 && --g_fail_countdown == 0) {
            *p = nullptr;
            return fail(FL_ERR_ALLOC, "injected device allocation failure (%zu bytes)", bytes);
        }
    }
    cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(FL_ERR_ALLOC, "cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    return FL_SUCCESS;
}
void dev_free(void *p, cudaStream_t s) {
    if (!p) return;
    // the stream it was allocated on may be gone (a caller's stream destroyed
    // before the plan): free synchronously then
    if (cudaFreeAsync(p, s) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(p);
    }
}
void debug_fail_alloc_after(int n) {
    std::lock_guard<std::mutex> lk(g_alloc_mu);
    g_fail_countdown = n;
}

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

static inline int grid_for(long n, int threads, int cap_per_sm = 8) {
    long b = (n + threads - 1) / threads;
    long cap = (long)num_sms() * cap_per_sm;
    if (b > cap) b = cap;
    return (int)std::max<long>(b, 1);
}

// ---------------------------------------------------------------- scan ---
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int warp_incl_scan(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; *total gets the block sum.
__device__ __forceinline__ int block_excl_scan(int v, int *sm, int *total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) sm[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s = lane < nw ? sm[lane] : 0;
        int si = warp_incl_scan(s);
        if (lane < nw) sm[lane] = si - s;
        if (lane == 31) sm[32] = si;
    }
    __syncthreads();
    int r = sm[w] + inc - v;
    *total = sm[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int *in, long n, int *sums) {
    __shared__ int sm[33];
    long base = (long)blockIdx.x * SCAN_TILE;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; k++) {
        long i = base + (long)k * SCAN_THREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    int tot;
    block_excl_scan(s, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int *in, int *out, long n,
                                                             const int *offsets, int *total) {
    __shared__ int sm[33];
    long base = (long)blockIdx.x * SCAN_TILE + (long)threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; k++) {
        long i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int tot;
    int run = block_excl_scan(s, sm, &tot);
    int off = offsets ? offsets[blockIdx.x] : 0;
    run += off;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; k++) {
        long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) total[0] = off + tot;
}

int scan_exclusive(const int *in, int *out, long n, int *total, cudaStream_t s) {
    if (n <= 0) {
        if (total) FL_CUDA(cudaMemsetAsync(total, 0, sizeof(int), s));
        return FL_SUCCESS;
    }
    long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        k_scan_apply<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr, total);
        FL_CUDA(cudaGetLastError());
        return FL_SUCCESS;
    }
    DevBuf<int> sums;
    FL_TRY(sums.alloc(nb, s));
    k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums.get());
    FL_CUDA(cudaGetLastError());
    FL_TRY(scan_exclusive(sums.get(), sums.get(), nb, nullptr, s));
    k_scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums.get(), total);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

__global__ void k_max(const int *in, long n, int *out) {
    int m = 0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        m = max(m, in[i]);
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

int max_reduce(const int *in, long n, int *out_dev, cudaStream_t s) {
    FL_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(int), s));
    if (n <= 0) return FL_SUCCESS;
    k_max<<<grid_for(n, 256), 256, 0, s>>>(in, n, out_dev);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

// ---------------------------------------------------------- radix sort ---
// Stable LSD radix sort, 8-bit digits.  Per pass: per-tile digit histograms
// (digit-major so one exclusive scan yields every tile's output base), then
// a scatter that ranks keys inside the tile in input order with
// __match_any_sync, which keeps equal digits in their original order.
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_IPT = 16;
constexpr int RS_TILE = RS_THREADS * RS_IPT;
constexpr int RS_BINS = 256;

__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const unsigned *keys, long n, int shift,
                                                           int *hist, int ntiles) {
    __shared__ int h[RS_BINS];
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    long base = (long)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int k = 0; k < RS_IPT; k++) {
        long i = base + (long)k * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) hist[(long)d * ntiles + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(const unsigned *kin, const unsigned *vin,
                                                              unsigned *kout, unsigned *vout, long n,
                                                              int shift, const int *offs, int ntiles) {
    __shared__ int base[RS_BINS];
    __shared__ int wcnt[RS_WARPS][RS_BINS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (int d = tid; d < RS_BINS; d += RS_THREADS) base[d] = offs[(long)d * ntiles + blockIdx.x];
    long tile0 = (long)blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_IPT; k++) {
        for (int i = tid; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
        __syncthreads();
        long i = tile0 + (long)k * RS_THREADS + tid;
        bool valid = i < n;
        unsigned key = valid ? kin[i] : 0u;
        unsigned val = valid ? vin[i] : 0u;
        int d = (int)((key >> shift) & 255u);
        unsigned peers = __match_any_sync(FULL, valid ? d : RS_BINS + lane);
        int rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int pos = base[d] + rank;
            for (int w = 0; w < warp; w++) pos += wcnt[w][d];
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        for (int dd = tid; dd < RS_BINS; dd += RS_THREADS) {
            int t = 0;
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) t += wcnt[w][dd];
            base[dd] += t;
        }
        __syncthreads();
    }
}

int radix_sort_pairs(unsigned *keys, unsigned *vals, long n, int bits, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return FL_SUCCESS;
    long ntiles = (n + RS_TILE - 1) / RS_TILE;
    DevBuf<unsigned> k2, v2;
    DevBuf<int> hist;
    FL_TRY(k2.alloc(n, s));
    FL_TRY(v2.alloc(n, s));
    FL_TRY(hist.alloc(ntiles * RS_BINS, s));
    unsigned *ki = keys, *vi = vals, *ko = k2.get(), *vo = v2.get();
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<(unsigned)ntiles, RS_THREADS, 0, s>>>(ki, n, shift, hist.get(), (int)ntiles);
        FL_CUDA(cudaGetLastError());
        FL_TRY(scan_exclusive(hist.get(), hist.get(), ntiles * RS_BINS, nullptr, s));
        k_radix_scatter<<<(unsigned)ntiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, hist.get(),
                                                                 (int)ntiles);
        FL_CUDA(cudaGetLastError());
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    if (ki != keys) {
        FL_CUDA(cudaMemcpyAsync(keys, ki, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
        FL_CUDA(cudaMemcpyAsync(vals, vi, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, s));
    }
    return FL_SUCCESS;
}

static int bits_for(unsigned long v) {
    int b = 0;
    while (v) { b++; v >>= 1; }
    return b;
}

// ------------------------------------------------------------- helpers ---
__global__ void k_iota(unsigned *a, long n) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        a[i] = (unsigned)i;
}

// Reads back a few device ints with one synchronisation.
static int read_back(cudaStream_t s, const int *dev, int *host, int count) {
    FL_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(int), cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

// ------------------------------------------------------------- CSR->CSC --
// err bits: 1 column index out of range, 2 rowptr decreasing, 4 rowptr ends.
__global__ void k_validate_csr(const int *rowptr, const int *colidx, int m, int n, int nnz, int *err) {
    long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, stride = (long)gridDim.x * blockDim.x;
    int e = 0;
    for (long p = tid; p < nnz; p += stride) {
        int c = colidx[p];
        if (c < 0 || c >= n) e |= 1;
    }
    for (long i = tid; i < m; i += stride)
        if (rowptr[i + 1] < rowptr[i]) e |= 2;
    if (tid == 0 && (rowptr[0] != 0 || rowptr[m] != nnz)) e |= 4;
    if (e) atomicOr(err, e);
}

__global__ void k_count_cols(const int *colidx, long nnz, int *cnt) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < nnz; p += (long)gridDim.x * blockDim.x)
        atomicAdd(cnt + colidx[p], 1);
}

__global__ void k_csc_gather(const unsigned *perm, long nnz, const int *rowptr, int m, const double *val,
                             int *cscrow, double *cscval) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nnz; q += (long)gridDim.x * blockDim.x) {
        int p = (int)perm[q];
        cscrow[q] = upper_index(rowptr, m, p);
        cscval[q] = val[p];
    }
}

int csr_to_csc_device(int m, int n, int nnz, const int *rowptr, const int *colidx, const double *val,
                      int *cscptr, int *cscrow, double *cscval, int *nnzpercol, cudaStream_t s) {
    if (m < 0 || n < 0 || nnz < 0) return fail(FL_ERR_ARG, "csr_to_csc: negative size (m=%d n=%d nnz=%d)", m, n, nnz);
    if (nnz > 0 && (m == 0 || n == 0)) return fail(FL_ERR_ARG, "csr_to_csc: nnz=%d with an empty dimension", nnz);
    DevBuf<int> scal;
    FL_TRY(scal.alloc(2, s));
    FL_CUDA(cudaMemsetAsync(scal.get(), 0, 2 * sizeof(int), s));
    if (m > 0) {
        k_validate_csr<<<grid_for(std::max(nnz, m), 256), 256, 0, s>>>(rowptr, colidx, m, n, nnz, scal.get());
        FL_CUDA(cudaGetLastError());
    }
    int h[2];
    FL_TRY(read_back(s, scal.get(), h, 2));
    if (h[0]) return fail(FL_ERR_ARG, "csr_to_csc: invalid CSR (flags 0x%x: 1=column index out of range, "
                                      "2=row_ptr decreasing, 4=row_ptr[0]!=0 or row_ptr[m]!=nnz)", h[0]);
    if (n > 0) FL_CUDA(cudaMemsetAsync(nnzpercol, 0, (size_t)n * sizeof(int), s));
    if (nnz > 0) {
        k_count_cols<<<grid_for(nnz, 256), 256, 0, s>>>(colidx, nnz, nnzpercol);
        FL_CUDA(cudaGetLastError());
    }
    FL_TRY(scan_exclusive(nnzpercol, cscptr, n, cscptr + n, s));
    if (nnz == 0) return FL_SUCCESS;
    DevBuf<unsigned> keys, perm;
    FL_TRY(keys.alloc(nnz, s));
    FL_TRY(perm.alloc(nnz, s));
    FL_CUDA(cudaMemcpyAsync(keys.get(), colidx, (size_t)nnz * sizeof(int), cudaMemcpyDeviceToDevice, s));
    k_iota<<<grid_for(nnz, 256), 256, 0, s>>>(perm.get(), nnz);
    FL_CUDA(cudaGetLastError());
    FL_TRY(radix_sort_pairs(keys.get(), perm.get(), nnz, bits_for((unsigned long)(n - 1)), s));
    k_csc_gather<<<grid_for(nnz, 256), 256, 0, s>>>(perm.get(), nnz, rowptr, m, val, cscrow, cscval);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

// ------------------------------------------------------------ col sort ---
// err bits: 1 negative count, 2 count disagrees with col_ptr, 4 col_ptr ends.
__global__ void k_validate_counts(const int *cnt, const int *cscptr, int n, int nnz, int *err) {
    long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, stride = (long)gridDim.x * blockDim.x;
    int e = 0;
    for (long c = tid; c < n; c += stride) {
        int k = cnt[c];
        if (k < 0) e |= 1;
        if (cscptr && cscptr[c + 1] - cscptr[c] != k) e |= 2;
    }
    if (tid == 0 && cscptr && (cscptr[0] != 0 || cscptr[n] != nnz)) e |= 4;
    if (e) atomicOr(err, e);
}

__global__ void k_gather_x(const unsigned *perm, int n, const double *x, double *xs) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        xs[i] = x[perm[i]];
}

__global__ void k_sorted_gather(const int *perm, const int *scolptr, int n, long nnz, const int *cscptr,
                                const int *cscrow, const double *cscval, int *srow, double *sval) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nnz; q += (long)gridDim.x * blockDim.x) {
        int i = upper_index(scolptr, n, (int)q);
        int src = cscptr[perm[i]] + ((int)q - scolptr[i]);
        srow[q] = cscrow[src];
        sval[q] = cscval[src];
    }
}

int col_sort_device(int n, int nnz, const int *nnzpercol, const int *cscptr, const int *cscrow,
                    const double *cscval, const double *x, int *perm, int *sortnnz, int *sortrowidx_tmp,
                    double *sortval_tmp, double *sortx, cudaStream_t s) {
    if (n < 0 || nnz < 0) return fail(FL_ERR_ARG, "col_sort: negative size (n=%d nnz=%d)", n, nnz);
    if (n == 0) {
        if (nnz != 0) return fail(FL_ERR_ARG, "col_sort: nnz=%d with no columns", nnz);
        return FL_SUCCESS;
    }
    DevBuf<int> scal;
    FL_TRY(scal.alloc(2, s));
    FL_CUDA(cudaMemsetAsync(scal.get(), 0, 2 * sizeof(int), s));
    k_validate_counts<<<grid_for(n, 256), 256, 0, s>>>(nnzpercol, cscptr, n, nnz, scal.get());
    FL_CUDA(cudaGetLastError());
    FL_TRY(max_reduce(nnzpercol, n, scal.get() + 1, s));
    int h[2];
    FL_TRY(read_back(s, scal.get(), h, 2));
    if (h[0]) return fail(FL_ERR_ARG, "col_sort: inconsistent input (flags 0x%x: 1=negative nnzPerCol, "
                                      "2=nnzPerCol disagrees with cscColPtr, 4=cscColPtr[0]!=0 or "
                                      "cscColPtr[colA]!=nnz)", h[0]);
    unsigned *keys = (unsigned *)sortnnz, *vals = (unsigned *)perm;
    FL_CUDA(cudaMemcpyAsync(keys, nnzpercol, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(vals, n);
    FL_CUDA(cudaGetLastError());
    FL_TRY(radix_sort_pairs(keys, vals, n, bits_for((unsigned long)h[1]), s));
    if (x && sortx) {
        k_gather_x<<<grid_for(n, 256), 256, 0, s>>>(vals, n, x, sortx);
        FL_CUDA(cudaGetLastError());
    }
    if (nnz > 0 && sortrowidx_tmp) {
        DevBuf<int> scolptr;
        FL_TRY(scolptr.alloc((size_t)n + 1, s));
        FL_TRY(scan_exclusive(sortnnz, scolptr.get(), n, scolptr.get() + n, s));
        k_sorted_gather<<<grid_for(nnz, 256), 256, 0, s>>>(perm, scolptr.get(), n, nnz, cscptr, cscrow, cscval,
                                                           sortrowidx_tmp, sortval_tmp);
        FL_CUDA(cudaGetLastError());
    }
    return FL_SUCCESS;
}

// --------------------------------------------------------- layout build --
// Steps of the staircase (formatTransform_GPU.h:8-57 SegmentReduce/prepare,
// coo2csc.h:153-186): sorted column k starts a step when its count exceeds
// the count of column k-1.  err bits: 1 negative, 2 not sorted.
__global__ void k_step_flags(const int *sortnnz, int n, int *flag, int *err) {
    int e = 0;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        int cur = sortnnz[k], prev = k ? sortnnz[k - 1] : 0;
        if (cur < 0) e |= 1;
        if (cur < prev) e |= 2;
        flag[k] = cur != prev;
    }
    if (e) atomicOr(err, e);
}

// Fills the step table; tiles per step = ceil((n-col)/32) * tall
// (countTileNum, formatTransform_GPU.h:85-98) and nonzeros per step =
// (n-col) * tall.  The 64-bit tile total guards the 32-bit index space.
__global__ void k_step_fill(const int *sortnnz, const int *flag, const int *stepidx, int n, int *col, int *base,
                            int *tall, int *tiles, int *nnzs, unsigned long long *tiles64) {
    unsigned long long local = 0;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        if (!flag[k]) continue;
        int s = stepidx[k];
        int prev = k ? sortnnz[k - 1] : 0;
        int t = sortnnz[k] - prev;
        long rem = n - k;
        long tl = ((rem + 31) / 32) * (long)t;
        col[s] = (int)k;
        base[s] = prev;
        tall[s] = t;
        tiles[s] = tl > 0x7fffffffL ? 0x7fffffff : (int)tl;
        long nz = rem * (long)t;
        nnzs[s] = nz > 0x7fffffffL ? 0x7fffffff : (int)nz;
        local += (unsigned long long)tl;
    }
    if (local) atomicAdd(tiles64, local);
}

// One warp per tile.  Tile t of step s is (chunk c, level l) with
// q = t - tile_off[s] = c * tall + l; its payload starts at
// nnz_off[s] + 32*tall*c + l*len because every chunk but the last is full
// (auxiliaryTrans + exclusive scan + dataTrans, formatTransform_GPU.h:113-171;
// coo2csc.h:229-296).  Lane i takes the level-th nonzero of sorted column
// colidx+i.  With reference arrays the warp also finds the runs of equal
// consecutive rows (Pre4CountRow .. Pre4tileclass, formatTransform_GPU.h:
// 188-285; coo2csc.h:314-448): run heads by a shuffle compare, lengths from
// the ballot of heads, tile_format 1/2 for full tiles, 0 for partial ones.
__global__ void __launch_bounds__(256) k_tile_build(StepView st, int n, int tilenum, const int *scolptr,
                                                    const int *srow_tmp, const double *sval_tmp, int *row,
                                                    double *val, int with_ref, int *tile_ptr, int *tile_len,
                                                    int *tile_colidx, int *tile_format, int *countrow,
                                                    int *sortrowindex) {
    const int lane = threadIdx.x & 31;
    long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long t = gw; t < tilenum; t += nw) {
        int s = upper_index(st.tile_off, st.steps, (int)t);
        int cs = __ldg(st.col + s), bs = __ldg(st.base + s), ts = __ldg(st.tall + s);
        int q = (int)t - __ldg(st.tile_off + s);
        int c = q / ts, l = q - c * ts;
        int rem = n - cs;
        int chunks = (rem + 31) >> 5;
        int len = (c == chunks - 1) ? rem - 32 * c : 32;
        int colidx = cs + 32 * c;
        int ptr = __ldg(st.nnz_off + s) + 32 * ts * c + l * len;
        int r = -1;
        if (lane < len) {
            int src = __ldg(scolptr + colidx + lane) + bs + l;
            r = __ldg(srow_tmp + src);
            row[ptr + lane] = r;
            val[ptr + lane] = __ldg(sval_tmp + src);
        }
        if (!with_ref) continue;
        int prev = __shfl_up_sync(FULL, r, 1);
        bool head = lane < len && (lane == 0 || r != prev);
        unsigned hm = __ballot_sync(FULL, head);
        if (lane < len) {
            unsigned after = hm & ~((2u << lane) - 1u);
            int runlen = (after ? __ffs(after) - 1 : len) - lane;
            sortrowindex[ptr + lane] = head ? runlen : 0;
        }
        if (lane == 0) {
            int runs = __popc(hm);
            tile_ptr[t] = ptr;
            tile_len[t] = len;
            tile_colidx[t] = colidx;
            countrow[t] = runs;
            tile_format[t] = len == 32 ? (runs == 1 ? 1 : 2) : 0;
        }
    }
}

// segmentoffset[r] = length of run r in global run order (coo2csc.h:391-417).
__global__ void __launch_bounds__(256) k_segoff(int tilenum, const int *tile_ptr, const int *tile_len,
                                                const int *row, const int *countrow, int *segoff) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long t = gw; t < tilenum; t += nw) {
        int ptr = __ldg(tile_ptr + t), len = __ldg(tile_len + t);
        int r = lane < len ? __ldg(row + ptr + lane) : -1;
        int prev = __shfl_up_sync(FULL, r, 1);
        bool head = lane < len && (lane == 0 || r != prev);
        unsigned hm = __ballot_sync(FULL, head);
        if (head) {
            unsigned after = hm & ~((2u << lane) - 1u);
            int runlen = (after ? __ffs(after) - 1 : len) - lane;
            segoff[__ldg(countrow + t) + __popc(hm & lt)] = runlen;
        }
    }
}

__global__ void k_fill_pad(int *row, double *val, long from, long to) {
    for (long i = from + blockIdx.x * (long)blockDim.x + threadIdx.x; i < to; i += (long)gridDim.x * blockDim.x) {
        row[i] = -1;
        val[i] = 0.0;
    }
}

__global__ void k_set_int(int *p, int v) { *p = v; }

int build_steps(Layout &L, int m, int n, int nnz, const int *sortnnz, cudaStream_t s) {
    if (m < 0 || n < 0 || nnz < 0) return fail(FL_ERR_ARG, "formatTransform: negative size");
    L.m = m;
    L.n = n;
    L.nnz = nnz;
    DevBuf<int> scal;  // 0 err, 1 steps, 2 tilenum, 3 nnz total, 4..5 tiles64
    FL_TRY(scal.alloc(8, s));
    FL_CUDA(cudaMemsetAsync(scal.get(), 0, 8 * sizeof(int), s));
    DevBuf<int> flag, stepidx;
    FL_TRY(flag.alloc((size_t)n + 1, s));
    FL_TRY(stepidx.alloc((size_t)n + 1, s));
    if (n > 0) {
        k_step_flags<<<grid_for(n, 256), 256, 0, s>>>(sortnnz, n, flag.get(), scal.get());
        FL_CUDA(cudaGetLastError());
    }
    FL_TRY(scan_exclusive(flag.get(), stepidx.get(), n, scal.get() + 1, s));
    int h[2];
    FL_TRY(read_back(s, scal.get(), h, 2));
    if (h[0]) return fail(FL_ERR_ARG, "formatTransform: sortnnz_tmp must be non-negative and sorted ascending "
                                      "(flags 0x%x)", h[0]);
    int steps = h[1];
    StepTable &st = L.st;
    st.steps = steps;
    DevBuf<int> tiles, nnzs;
    FL_TRY(st.col.alloc(steps + 1, s));
    FL_TRY(st.base.alloc(steps + 1, s));
    FL_TRY(st.tall.alloc(steps + 1, s));
    FL_TRY(st.tile_off.alloc(steps + 1, s));
    FL_TRY(st.nnz_off.alloc(steps + 1, s));
    FL_TRY(tiles.alloc(steps + 1, s));
    FL_TRY(nnzs.alloc(steps + 1, s));
    if (n > 0) {
        k_step_fill<<<grid_for(n, 256), 256, 0, s>>>(sortnnz, flag.get(), stepidx.get(), n, st.col.get(),
                                                      st.base.get(), st.tall.get(), tiles.get(), nnzs.get(),
                                                      (unsigned long long *)(scal.get() + 4));
        FL_CUDA(cudaGetLastError());
    }
    FL_TRY(scan_exclusive(tiles.get(), st.tile_off.get(), steps, st.tile_off.get() + steps, s));
    FL_TRY(scan_exclusive(nnzs.get(), st.nnz_off.get(), steps, st.nnz_off.get() + steps, s));
    FL_CUDA(cudaMemcpyAsync(scal.get() + 2, st.tile_off.get() + steps, sizeof(int), cudaMemcpyDeviceToDevice, s));
    FL_CUDA(cudaMemcpyAsync(scal.get() + 3, st.nnz_off.get() + steps, sizeof(int), cudaMemcpyDeviceToDevice, s));
    int h8[8];
    FL_TRY(read_back(s, scal.get(), h8, 8));
    unsigned long long tiles64;
    memcpy(&tiles64, h8 + 4, sizeof tiles64);
    if (tiles64 > 0x7fffffffULL) return fail(FL_ERR_OVERFLOW, "formatTransform: %llu tiles exceed 2^31-1", tiles64);
    if (h8[3] != nnz)
        return fail(FL_ERR_ARG, "formatTransform: sortnnz_tmp sums to %d, nnz is %d", h8[3], nnz);
    L.tilenum = h8[2];
    return build_regions(L, s);
}

int build_layout_device(Layout &L, int m, int n, int nnz, const int *sortnnz, const int *srow_tmp,
                        const double *sval_tmp, bool with_ref, cudaStream_t s, float *ms_tran, float *ms_class) {
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    for (auto &e : ev) FL_CUDA(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() { for (int i = 0; i < 3; i++) if (e[i]) cudaEventDestroy(e[i]); }
    } guard{ev};
    FL_CUDA(cudaEventRecord(ev[0], s));
    FL_TRY(build_steps(L, m, n, nnz, sortnnz, s));
    const int tilenum = L.tilenum;
    StepTable &st = L.st;
    DevBuf<int> scolptr;
    FL_TRY(scolptr.alloc((size_t)n + 1, s));
    FL_TRY(scan_exclusive(sortnnz, scolptr.get(), n, scolptr.get() + n, s));

    size_t np = padded(nnz);
    FL_TRY(L.row.alloc(np, s));
    FL_TRY(L.val.alloc(np, s));
    k_fill_pad<<<grid_for(np - nnz, 256), 256, 0, s>>>(L.row.get(), L.val.get(), nnz, (long)np);
    FL_CUDA(cudaGetLastError());
    if (with_ref) {
        FL_TRY(L.tile_ptr.alloc((size_t)tilenum + 1, s));
        FL_TRY(L.tile_len.alloc(std::max(tilenum, 1), s));
        FL_TRY(L.tile_colidx.alloc(std::max(tilenum, 1), s));
        FL_TRY(L.tile_format.alloc(std::max(tilenum, 1), s));
        FL_TRY(L.countrow.alloc((size_t)tilenum + 1, s));
        FL_TRY(L.sortrowindex.alloc(std::max(nnz, 1), s));
        k_set_int<<<1, 1, 0, s>>>(L.tile_ptr.get() + tilenum, nnz);
        FL_CUDA(cudaGetLastError());
    }
    StepView sv{st.col.get(), st.base.get(), st.tall.get(), st.tile_off.get(), st.nnz_off.get(), st.steps};
    if (tilenum > 0) {
        int blocks = grid_for((long)tilenum * 32, 256, 16);
        k_tile_build<<<blocks, 256, 0, s>>>(sv, n, tilenum, scolptr.get(), srow_tmp, sval_tmp, L.row.get(),
                                            L.val.get(), with_ref ? 1 : 0, L.tile_ptr.get(), L.tile_len.get(),
                                            L.tile_colidx.get(), L.tile_format.get(), L.countrow.get(),
                                            L.sortrowindex.get());
        FL_CUDA(cudaGetLastError());
    }
    FL_CUDA(cudaEventRecord(ev[1], s));
    if (with_ref) {
        FL_TRY(scan_exclusive(L.countrow.get(), L.countrow.get(), tilenum, L.countrow.get() + tilenum, s));
        int segsum = 0;
        FL_TRY(read_back(s, L.countrow.get() + tilenum, &segsum, 1));
        L.segsum = segsum;
        FL_TRY(L.segmentoffset.alloc((size_t)segsum + 1, s));
        k_set_int<<<1, 1, 0, s>>>(L.segmentoffset.get() + segsum, 0);
        FL_CUDA(cudaGetLastError());
        if (tilenum > 0) {
            int blocks = grid_for((long)tilenum * 32, 256, 16);
            k_segoff<<<blocks, 256, 0, s>>>(tilenum, L.tile_ptr.get(), L.tile_len.get(), L.row.get(),
                                            L.countrow.get(), L.segmentoffset.get());
            FL_CUDA(cudaGetLastError());
        }
    }
    FL_CUDA(cudaEventRecord(ev[2], s));
    FL_CUDA(cudaEventSynchronize(ev[2]));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    if (ms_tran) *ms_tran = a;
    if (ms_class) *ms_class = b;
    return FL_SUCCESS;
}

// Recomputes (ptr, len, colidx) of every tile from the step table and flags
// any tile whose host-provided arrays differ.
__global__ void k_tile_meta_check(StepView st, int n, int tilenum, const int *tile_ptr, const int *tile_len,
                                  const int *tile_colidx, int *err) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < tilenum; t += (long)gridDim.x * blockDim.x) {
        int s = upper_index(st.tile_off, st.steps, (int)t);
        int cs = st.col[s], ts = st.tall[s];
        int q = (int)t - st.tile_off[s];
        int c = q / ts, l = q - c * ts;
        int rem = n - cs, chunks = (rem + 31) >> 5;
        int len = (c == chunks - 1) ? rem - 32 * c : 32;
        int ptr = st.nnz_off[s] + 32 * ts * c + l * len;
        if (tile_ptr[t] != ptr || tile_len[t] != len || tile_colidx[t] != cs + 32 * c) atomicOr(err, 1);
    }
}

int check_tile_meta(const Layout &L, const int *tile_ptr, const int *tile_len, const int *tile_colidx,
                    cudaStream_t s) {
    if (L.tilenum == 0) return FL_SUCCESS;
    DevBuf<int> err;
    FL_TRY(err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), s));
    const StepTable &st = L.st;
    StepView sv{st.col.get(), st.base.get(), st.tall.get(), st.tile_off.get(), st.nnz_off.get(), st.steps};
    k_tile_meta_check<<<grid_for(L.tilenum, 256), 256, 0, s>>>(sv, L.n, L.tilenum, tile_ptr, tile_len,
                                                                 tile_colidx, err.get());
    FL_CUDA(cudaGetLastError());
    int h = 0;
    FL_TRY(read_back(s, err.get(), &h, 1));
    if (h) return fail(FL_ERR_ARG, "slide_matrix tile arrays do not follow the FastLoad staircase layout");
    return FL_SUCCESS;
}

__global__ void k_counts_from_ptr(const int *ptr, int n, int *cnt) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x)
        cnt[c] = ptr[c + 1] - ptr[c];
}

int counts_from_ptr(const int *ptr, int n, int *cnt, cudaStream_t s) {
    if (n <= 0) return FL_SUCCESS;
    k_counts_from_ptr<<<grid_for(n, 256), 256, 0, s>>>(ptr, n, cnt);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

__global__ void k_range(const int *idx, long count, int bound, int *err) {
    int e = 0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x) {
        int v = idx[i];
        if (v < 0 || v >= bound) e = 1;
    }
    if (e) atomicOr(err, 1);
}

int check_index_range(const int *idx, long count, int bound, const char *what, cudaStream_t s) {
    if (count <= 0) return FL_SUCCESS;
    DevBuf<int> err;
    FL_TRY(err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), s));
    k_range<<<grid_for(count, 256), 256, 0, s>>>(idx, count, bound, err.get());
    FL_CUDA(cudaGetLastError());
    int h = 0;
    FL_TRY(read_back(s, err.get(), &h, 1));
    if (h) return fail(FL_ERR_ARG, "%s: index out of range [0, %d)", what, bound);
    return FL_SUCCESS;
}

int permute_x(const int *perm, int n, const double *x, double *xs, cudaStream_t s) {
    if (n <= 0) return FL_SUCCESS;
    k_gather_x<<<grid_for(n, 256), 256, 0, s>>>((const unsigned *)perm, n, x, xs);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

// ------------------------------------------------------------- regions --
// Region 2s is the full-chunk part of step s, region 2s+1 its partial last
// chunk; items cut each region into pieces of at most `item` nonzeros with
// interior boundaries on multiples of four.
__global__ void k_region_fill(StepView st, int n, int item, RegionDesc *reg, int *pieces, int *ends) {
    for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < st.steps; s += (long)gridDim.x * blockDim.x) {
        int cs = st.col[s], ts = st.tall[s], off = st.nnz_off[s], off1 = st.nnz_off[s + 1];
        int rem = n - cs, nfull = rem >> 5, lenp = rem & 31;
        int mid = off + 32 * ts * nfull;
        RegionDesc a{off, cs, 32 * ts, 1};
        RegionDesc b{mid, cs + 32 * nfull, lenp ? lenp : 1, 0};
        reg[2 * s] = a;
        reg[2 * s + 1] = b;
        ends[2 * s] = mid;
        ends[2 * s + 1] = off1;
        int A0 = off & ~3, A1 = mid & ~3;
        pieces[2 * s] = mid > off ? (mid - A0 + item - 1) / item : 0;
        pieces[2 * s + 1] = off1 > mid ? (off1 - A1 + item - 1) / item : 0;
    }
}

__global__ void k_item_fill(const RegionDesc *reg, const int *ends, const int *poff, int nreg, int nitems,
                            int item, ItemDesc *items) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nitems; i += (long)gridDim.x * blockDim.x) {
        int r = upper_index(poff, nreg, (int)i);
        int rs = reg[r].start, re = ends[r];
        int A = rs & ~3;
        int j = (int)i - poff[r];
        int b = max(rs, A + j * item);
        int e = min(re, A + (j + 1) * item);
        items[i] = ItemDesc{b, e, r, 0};
    }
}

int item_nnz_for(long nnz) {
    // about two items per warp of the GPU, so a small matrix still spreads
    // over every SM; at most FL_ITEM, at least 128 (and a multiple of it)
    const long per = (nnz + 2L * num_sms() * 32 - 1) / (2L * num_sms() * 32);
    return (int)std::min<long>(FL_ITEM, std::max<long>(128, (per + 127) / 128 * 128));
}

int build_regions(Layout &L, cudaStream_t s) {
    return build_regions_sized(L, item_nnz_for(L.item_basis > 0 ? L.item_basis : L.nnz), L.regions, s);
}

int build_regions_sized(const Layout &L, int item, Regions &R, cudaStream_t s) {
    const StepTable &st = L.st;
    int nreg = 2 * st.steps;
    R.nregions = nreg;
    R.nitems = 0;
    if (nreg == 0) return FL_SUCCESS;
    DevBuf<int> pieces, ends, poff;
    FL_TRY(R.region.alloc(nreg, s));
    FL_TRY(pieces.alloc(nreg, s));
    FL_TRY(ends.alloc(nreg, s));
    FL_TRY(poff.alloc(nreg + 1, s));
    StepView sv{st.col.get(), st.base.get(), st.tall.get(), st.tile_off.get(), st.nnz_off.get(), st.steps};
    k_region_fill<<<grid_for(st.steps, 256), 256, 0, s>>>(sv, L.n, item, R.region.get(), pieces.get(), ends.get());
    FL_CUDA(cudaGetLastError());
    FL_TRY(scan_exclusive(pieces.get(), poff.get(), nreg, poff.get() + nreg, s));
    int nitems = 0;
    FL_TRY(read_back(s, poff.get() + nreg, &nitems, 1));
    R.nitems = nitems;
    if (nitems == 0) return FL_SUCCESS;
    FL_TRY(R.item.alloc(nitems, s));
    k_item_fill<<<grid_for(nitems, 256), 256, 0, s>>>(R.region.get(), ends.get(), poff.get(), nreg, nitems, item,
                                                      R.item.get());
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}


// ------------------------------------------------ allocation-free col sort --
// A variant of the column sort for callers that cannot allocate device
// memory at all -- for example a plugin inside a host application whose
// allocator pre-reserves the whole device and refuses further requests, or
// a latency-critical caller that cannot afford the synchronisation that
// cudaMalloc/cudaFree imply.  Its scratch (radix-sort ping-pong buffers,
// digit histograms, scan partial sums, the sorted column pointer and two
// status words) lives in the file-scope array below, sized for at most
// FL_NOALLOC_MAX_COLS columns; every GPU that loads this library holds it
// until the process exits.  Host code must not pass the array's name to a
// kernel (on the host it names a stand-in, not device memory): the first
// call on each device looks up its device address with
// cudaGetSymbolAddress while that device is current and caches it.
namespace {
constexpr long NA_COLS = FL_NOALLOC_MAX_COLS;
constexpr long NA_TILES = (NA_COLS + RS_TILE - 1) / RS_TILE;
constexpr long NA_HIST = RS_BINS * NA_TILES;
constexpr long NA_SUMS = 2048;  // scan partial sums, two levels deep
constexpr size_t NA_OFF_KEYS = 0;
constexpr size_t NA_OFF_VALS = NA_OFF_KEYS + NA_COLS * sizeof(unsigned);
constexpr size_t NA_OFF_HIST = NA_OFF_VALS + NA_COLS * sizeof(unsigned);
constexpr size_t NA_OFF_SUMS = NA_OFF_HIST + NA_HIST * sizeof(int);
constexpr size_t NA_OFF_COLPTR = NA_OFF_SUMS + NA_SUMS * sizeof(int);
constexpr size_t NA_OFF_STATUS = NA_OFF_COLPTR + ((NA_COLS + 1 + 63) / 64) * 64 * sizeof(int);
constexpr size_t NA_BYTES = NA_OFF_STATUS + 64;
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[256];

// Device address of the scratch array on the current device (set-up on the
// first call per device).
static int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    FL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(FL_ERR_INTERNAL, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(FL_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (unsigned char *)p;
    }
    *out = g_noalloc_ptr[dev];
    return FL_SUCCESS;
}

// Exclusive scan whose partial sums go to caller scratch (sums, cap ints).
static int scan_exclusive_into(const int *in, int *out, long n, int *total, int *sums, long cap, cudaStream_t s) {
    if (n <= 0) {
        if (total) FL_CUDA(cudaMemsetAsync(total, 0, sizeof(int), s));
        return FL_SUCCESS;
    }
    long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        k_scan_apply<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr, total);
        FL_CUDA(cudaGetLastError());
        return FL_SUCCESS;
    }
    if (nb > cap) return fail(FL_ERR_INTERNAL, "scan scratch too small (%ld > %ld)", nb, cap);
    k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums);
    FL_CUDA(cudaGetLastError());
    FL_TRY(scan_exclusive_into(sums, sums, nb, nullptr, sums + nb, cap - nb, s));
    k_scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums, total);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

}  // namespace fl

using namespace fl;

// At global scope: an extern "C" definition inside a namespace does not take
// the exported visibility of its declaration in fastload.h.
extern "C" int fl_col_sort_noalloc(int n, int nnz, const int *d_nnzpercol, const int *d_colptr,
                                   const int *d_rowidx, const double *d_val, const double *d_x, int *d_perm,
                                   int *d_sortnnz, int *d_sortrowidx_tmp, double *d_sortval_tmp, double *d_sortx,
                                   void *stream) {
    clear_error();
    cudaStream_t s = (cudaStream_t)stream;
    if (n < 0 || nnz < 0) return fail(FL_ERR_ARG, "col_sort_noalloc: negative size (n=%d nnz=%d)", n, nnz);
    if (n > FL_NOALLOC_MAX_COLS)
        return fail(FL_ERR_ARG, "col_sort_noalloc: n=%d exceeds FL_NOALLOC_MAX_COLS=%d (the scratch array size); "
                                "use fl_col_sort or a plan for larger matrices", n, FL_NOALLOC_MAX_COLS);
    if (n == 0) {
        if (nnz != 0) return fail(FL_ERR_ARG, "col_sort_noalloc: nnz=%d with no columns", nnz);
        return FL_SUCCESS;
    }
    if (!d_nnzpercol || !d_colptr || !d_perm || !d_sortnnz || (d_x && !d_sortx) ||
        (nnz && (!d_rowidx || !d_val || !d_sortrowidx_tmp || !d_sortval_tmp)))
        return fail(FL_ERR_ARG, "col_sort_noalloc: NULL array");
    unsigned char *base = nullptr;
    FL_TRY(noalloc_scratch(&base));
    unsigned *k2 = (unsigned *)(base + NA_OFF_KEYS), *v2 = (unsigned *)(base + NA_OFF_VALS);
    int *hist = (int *)(base + NA_OFF_HIST), *sums = (int *)(base + NA_OFF_SUMS);
    int *scolptr = (int *)(base + NA_OFF_COLPTR), *status = (int *)(base + NA_OFF_STATUS);
    // status words start at zero on every call (the array keeps the last
    // call's contents)
    FL_CUDA(cudaMemsetAsync(status, 0, 2 * sizeof(int), s));
    k_validate_counts<<<grid_for(n, 256), 256, 0, s>>>(d_nnzpercol, d_colptr, n, nnz, status);
    FL_CUDA(cudaGetLastError());
    k_max<<<grid_for(n, 256), 256, 0, s>>>(d_nnzpercol, n, status + 1);
    FL_CUDA(cudaGetLastError());
    int h[2] = {0, 0};
    FL_CUDA(cudaMemcpyAsync(h, status, sizeof h, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (h[0]) return fail(FL_ERR_ARG, "col_sort_noalloc: inconsistent input (flags 0x%x: 1=negative count, "
                                      "2=count disagrees with colptr, 4=colptr[0]!=0 or colptr[n]!=nnz)", h[0]);
    unsigned *ki = (unsigned *)d_sortnnz, *vi = (unsigned *)d_perm, *ko = k2, *vo = v2;
    FL_CUDA(cudaMemcpyAsync(ki, d_nnzpercol, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(vi, n);
    FL_CUDA(cudaGetLastError());
    const long ntiles = (n + RS_TILE - 1) / RS_TILE;
    for (int shift = 0; shift < bits_for((unsigned long)h[1]); shift += 8) {
        k_radix_hist<<<(unsigned)ntiles, RS_THREADS, 0, s>>>(ki, n, shift, hist, (int)ntiles);
        FL_CUDA(cudaGetLastError());
        FL_TRY(scan_exclusive_into(hist, hist, ntiles * RS_BINS, nullptr, sums, NA_SUMS, s));
        k_radix_scatter<<<(unsigned)ntiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, hist, (int)ntiles);
        FL_CUDA(cudaGetLastError());
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    if (ki != (unsigned *)d_sortnnz) {
        FL_CUDA(cudaMemcpyAsync(d_sortnnz, ki, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
        FL_CUDA(cudaMemcpyAsync(d_perm, vi, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    if (d_x) {
        k_gather_x<<<grid_for(n, 256), 256, 0, s>>>((const unsigned *)d_perm, n, d_x, d_sortx);
        FL_CUDA(cudaGetLastError());
    }
    if (nnz > 0) {
        FL_TRY(scan_exclusive_into(d_sortnnz, scolptr, n, scolptr + n, sums, NA_SUMS, s));
        k_sorted_gather<<<grid_for(nnz, 256), 256, 0, s>>>(d_perm, scolptr, n, nnz, d_colptr, d_rowidx, d_val,
                                                           d_sortrowidx_tmp, d_sortval_tmp);
        FL_CUDA(cudaGetLastError());
    }
    return FL_SUCCESS;
}

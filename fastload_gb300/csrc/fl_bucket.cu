// fl_bucket.cu -- bucketed FastLoad SpMV (FP64) for sm_103a.
//
// The column sort of FastLoad orders columns by nonzero count; a bucket
// threshold H0 splits that order in two:
//
//  * light columns [0, H0) keep the FastLoad layout (tiles of the staircase
//    restricted to those columns) and the streaming kernel's per-run atomics;
//  * the heavy band [H0, n) -- the densest columns, which on skewed matrices
//    hold most of the nonzeros -- is re-packed row-major into slices of 32
//    rows: lane l of a slice owns one row and walks its band nonzeros,
//    accumulating value * x with one FP64 FMA each, and adds the row's sum
//    to y with one atomic.  A band of at most 16,384 columns has its x
//    staged in shared memory by a TMA bulk copy at kernel start (overlapped
//    with the light work) and streams its values and columns through
//    per-warp cp.async rings; the automatic layout may also put every
//    column in the band (x read through the cache), and then each row is
//    owned by one lane and y is written without atomics.
//
// Work units are step ranges of the band (at least 256 entries, about four
// per resident warp; long slices are cut, their parts meeting in y by
// atomics) and light items of the tile stream, dealt to blocks round-robin.
//
// On GB300 scattered L2 atomics (about 221 G/s) and FP64 pipe slots (about
// 500 G/s) are the scarce resources of a CSC SpMV; the heavy band turns one
// atomic per nonzero into one per row and keeps exactly one FP64 operation
// per nonzero.  One persistent launch runs both parts.
#include "fl_forms.cuh"

#include <algorithm>
#include <vector>

namespace fl {

constexpr int BK_MAX_BAND = 24576;            // 192 KB of FP64 x in shared memory
constexpr int BK_AUTO_BAND_BYTES = 131072;    // automatic band: at most 128 KB of x in shared memory
constexpr int BK_AUTO_MIN_DEGREE = 32;        // densest columns worth a row slice

int bucket_max_band() { return BK_MAX_BAND; }

static int grid_cap(long n, int threads, int per_sm = 8) {
    long b = (n + threads - 1) / threads;
    long cap = (long)num_sms() * per_sm;
    return (int)std::max<long>(1, std::min(b, cap));
}

// ------------------------------------------------------------- build ----
__global__ void k_band_ptr(const int *scolptr, int H0, int nh, int *bandptr) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i <= nh; i += (long)gridDim.x * blockDim.x)
        bandptr[i] = scolptr[H0 + i] - scolptr[H0];
}

// key = maxlen - len (so an ascending stable sort lists rows longest first,
// ties in ascending row id); counts rows with band nonzeros.
__global__ void k_len_key(const int *rlen, int m, int maxlen, unsigned *key, unsigned *idx, int *nrows) {
    int c = 0;
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < m; r += (long)gridDim.x * blockDim.x) {
        int l = rlen[r];
        key[r] = (unsigned)(maxlen - l);
        idx[r] = (unsigned)r;
        c += l > 0;
    }
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULLM, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(nrows, c);
}

__global__ void k_slice_width(const unsigned *rows, const int *rlen, int nslices, int *width32) {
    for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < nslices; s += (long)gridDim.x * blockDim.x)
        width32[s] = 32 * rlen[rows[32 * s]];
}

// One warp per slice: lane l copies row rows[32s+l]'s band entries to
// slice_ptr[s] + 32 j + l; past the row's length value 0 and column pad
// (the band width nh: the zero the shared-memory x staging keeps at x[nh]).
__global__ void k_slice_fill(const unsigned *rows, const int *rlen, const int *rp, const int *hc,
                             const double *hv, int nrows, int nslices, const int *slice_ptr, double *val,
                             uint16_t *col, int *col32, int *srow, int *slen, int pad) {
    const int lane = threadIdx.x & 31;
    long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long s = gw; s < nslices; s += nw) {
        const long slot = 32 * s + lane;
        const int r = slot < nrows ? (int)rows[slot] : -1;
        const int len = r >= 0 ? rlen[r] : 0;
        srow[slot] = r;
        slen[slot] = len;
        const int base = slice_ptr[s], w = (slice_ptr[s + 1] - base) >> 5;
        const int src = r >= 0 ? rp[r] : 0;
        for (int j = 0; j < w; j++) {
            const long dst = base + 32L * j + lane;
            val[dst] = j < len ? hv[src + j] : 0.0;
            if (col) col[dst] = (uint16_t)(j < len ? hc[src + j] : pad);
            else col32[dst] = j < len ? hc[src + j] : pad;
        }
    }
}

static int read_ints(cudaStream_t s, const int *dev, int *host, int count) {
    FL_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(int), cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

static int bits_of(unsigned long v) {
    int b = 0;
    while (v) { b++; v >>= 1; }
    return b;
}

int auto_layout_band(const Layout &L, int x_bytes, bool *wide, cudaStream_t s) {
    int nh = bucket_auto_band(L.sortnnz.get(), L.n, L.nnz, s, x_bytes);
    if (nh < 0) return nh;
    *wide = nh > bucket_max_band();
    if (nh == 0 && L.nnz > 0) {
        // No dense columns.  Rows as slices (every column in the band, x
        // through the cache, one y update per row part) beat the FastLoad
        // stream's atomic per nonzero when x gathers have locality (banded,
        // block, stencil: mean |r/m - c/n| small), when rows are skewed (hot
        // rows make the stream's atomics collide; cut slices spread them
        // over units), and on large matrices of several nonzeros a column,
        // where the stream's random atomics bound it (1.5x at 5M+ uniformly
        // random nonzeros; below 1M the stream's lower fixed cost wins).
        float f[24];
        FL_TRY(plan_features(L, f, s));
        const bool big = L.nnz >= 1000000 && (long)L.nnz >= 4L * L.n;
        if (f[21] < 0.05f || f[22] > 2.0f || big) {
            nh = L.n;
            *wide = true;
        }
    }
    return nh;
}

bool make_units(const std::vector<int> &sp, long per_unit, std::vector<int> &unit_step,
                std::vector<int> &unit_slice) {
    unit_step.clear();
    unit_slice.clear();
    const int ns = (int)sp.size() - 1;
    // at least 8 steps a unit: below that a unit costs more to claim than to
    // run; small bands still spread over every SM
    per_unit = std::max(per_unit, 256L);
    bool split = false, open = false;
    long acc = 0;
    for (int q = 0; q < ns; q++) {
        const int a = sp[q] >> 5, b = sp[q + 1] >> 5;
        const long entries = (long)sp[q + 1] - sp[q];
        if (entries > 2 * per_unit) {
            // a long slice: pieces of about per_unit entries
            open = false;
            const long pieces = (entries + per_unit - 1) / per_unit;
            const int steps = (int)((b - a + pieces - 1) / pieces);
            for (int t = a; t < b; t += steps) {
                unit_step.push_back(t);
                unit_slice.push_back(q);
            }
            split = true;
            continue;
        }
        if (!open) {
            unit_step.push_back(a);
            unit_slice.push_back(q);
            open = true;
            acc = 0;
        }
        acc += entries;
        if (acc >= per_unit) open = false;
    }
    unit_step.push_back(ns > 0 ? sp[ns] >> 5 : 0);
    return split;
}

int bucket_auto_band(const int *sortnnz, int n, int nnz, cudaStream_t s, int x_bytes) {
    if (n <= 0 || nnz <= 0) return 0;
    // 16,384 columns of FP64 x, 32,768 of FP32 x: what fits 128 KB of shared
    // memory beside the per-warp rings.  (A 192 KB band of FP32 x, without
    // the rings, ran 64.1 against 50.8 us at the 2^20-column Zipf(1.8)
    // matrix with the matrix's streams cold in L2.)
    const int budget = BK_AUTO_BAND_BYTES;
    const int tail = std::min(n, budget / std::max(x_bytes, 1));
    std::vector<int> h(tail);
    FL_TRY(read_ints(s, sortnnz + (n - tail), h.data(), tail));
    int band = 0;
    long band_nnz = 0;
    for (int i = tail - 1; i >= 0 && h[i] >= BK_AUTO_MIN_DEGREE; i--) {
        band++;
        band_nnz += h[i];
    }
    band &= ~1;
    // a band worth its own pass holds a quarter of the matrix or more
    if (band < 64 || band_nnz * 4 < (long)nnz) return 0;
    return band;
}

int build_bucket(Bucket &B, int m, int n, int nnz, const int *sortnnz, const int *srow_tmp,
                 const double *sval_tmp, int nh, cudaStream_t s, bool wide, int unit_warps) {
    nh = std::max(0, std::min(nh, wide ? n : std::min(n, BK_MAX_BAND)));
    if (!wide || nh < n) nh &= ~1;
    const int H0 = n - nh;
    DevBuf<int> scolptr;
    FL_TRY(scolptr.alloc((size_t)n + 1, s));
    FL_TRY(scan_exclusive(sortnnz, scolptr.get(), n, scolptr.get() + n, s));
    int nnz_l = 0;
    FL_TRY(read_ints(s, scolptr.get() + H0, &nnz_l, 1));
    B.light.item_basis = nnz;  // light items sized for the whole matrix (a small light part of a large
                               // matrix keeps large items: fewer run-boundary atomics and claims)
    FL_TRY(build_layout_device(B.light, m, H0, nnz_l, sortnnz, srow_tmp, sval_tmp, false, s, nullptr, nullptr));
    HeavyBand &H = B.heavy;
    H.H0 = H0;
    H.nh = nh;
    H.nnz = (long)nnz - nnz_l;
    FL_TRY(B.err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(B.err.get(), 0, sizeof(int), s));
    if (nh == 0 || H.nnz == 0) {
        H.nh = 0;
        return FL_SUCCESS;
    }
    const int nnz_h = (int)H.nnz;
    // band as CSR over the matrix rows (local columns ascending in each row)
    DevBuf<int> bandptr, rp, hc, rlen, scal;
    DevBuf<double> hv;
    FL_TRY(bandptr.alloc((size_t)nh + 1, s));
    k_band_ptr<<<grid_cap(nh + 1, 256), 256, 0, s>>>(scolptr.get(), H0, nh, bandptr.get());
    FL_CUDA(cudaGetLastError());
    FL_TRY(rp.alloc((size_t)m + 1, s));
    FL_TRY(hc.alloc(nnz_h, s));
    FL_TRY(hv.alloc(nnz_h, s));
    FL_TRY(rlen.alloc(std::max(m, 1), s));
    FL_TRY(csr_to_csc_device(nh, m, nnz_h, bandptr.get(), srow_tmp + nnz_l, sval_tmp + nnz_l, rp.get(), hc.get(),
                             hv.get(), rlen.get(), s));
    // rows longest first
    FL_TRY(scal.alloc(2, s));
    FL_CUDA(cudaMemsetAsync(scal.get(), 0, 2 * sizeof(int), s));
    FL_TRY(max_reduce(rlen.get(), m, scal.get(), s));
    int h2[2];
    FL_TRY(read_ints(s, scal.get(), h2, 1));
    const int maxlen = h2[0];
    DevBuf<unsigned> keys, rows;
    FL_TRY(keys.alloc(m, s));
    FL_TRY(rows.alloc(m, s));
    k_len_key<<<grid_cap(m, 256), 256, 0, s>>>(rlen.get(), m, maxlen, keys.get(), rows.get(), scal.get() + 1);
    FL_CUDA(cudaGetLastError());
    FL_TRY(radix_sort_pairs(keys.get(), rows.get(), m, bits_of((unsigned long)maxlen), s));
    FL_TRY(read_ints(s, scal.get(), h2, 2));
    H.nrows = h2[1];
    H.nslices = (H.nrows + 31) / 32;
    FL_TRY(H.slice_ptr.alloc((size_t)H.nslices + 1, s));
    DevBuf<int> width32;
    FL_TRY(width32.alloc((size_t)H.nslices + 1, s));
    k_slice_width<<<grid_cap(H.nslices, 256), 256, 0, s>>>(rows.get(), rlen.get(), H.nslices, width32.get());
    FL_CUDA(cudaGetLastError());
    FL_TRY(scan_exclusive(width32.get(), H.slice_ptr.get(), H.nslices, H.slice_ptr.get() + H.nslices, s));
    int total = 0;
    FL_TRY(read_ints(s, H.slice_ptr.get() + H.nslices, &total, 1));
    H.padded = total;
    // one ring stage of zeros past the end (the ring kernels copy whole stages)
    FL_TRY(H.val.alloc((size_t)total + RING_PAD, s));
    FL_CUDA(cudaMemsetAsync(H.val.get() + total, 0, RING_PAD * sizeof(double), s));
    const bool narrow = nh <= 65535;
    if (narrow) {
        FL_TRY(H.col.alloc((size_t)total + RING_PAD, s));
        FL_CUDA(cudaMemsetAsync(H.col.get() + total, 0, RING_PAD * sizeof(uint16_t), s));
    } else {
        FL_TRY(H.col32.alloc((size_t)total + RING_PAD, s));
        FL_CUDA(cudaMemsetAsync(H.col32.get() + total, 0, RING_PAD * sizeof(int), s));
    }
    FL_TRY(H.row.alloc(32L * H.nslices, s));
    FL_TRY(H.len.alloc(32L * H.nslices, s));
    // work units: about four per resident warp (unit_warps), so that every
    // warp has work however the nonzeros fall into slices (short, fat
    // matrices have few slices of great width, and those are cut)
    {
        std::vector<int> sp(H.nslices + 1), ustep, uslice;
        FL_TRY(read_ints(s, H.slice_ptr.get(), sp.data(), H.nslices + 1));
        // a band of every column (no light part) takes two units a warp:
        // fewer unit starts, each a chain of dependent loads (7-point
        // Laplacian 128^3, FP32: 34.4 against 36.9 us; FP64 44.7 against
        // 46.4 us; the Zipf(1.8) matrix as row slices 47.7 against 50.3 us)
        const long uw = unit_warps > 0 ? unit_warps : (nh == n ? 2L : 4L);
        const long per_unit = (long)sp[H.nslices] / (uw * num_sms() * 32);
        H.split = make_units(sp, per_unit, ustep, uslice);
        H.nunits = (int)uslice.size();
        FL_TRY(H.unit_step.alloc(ustep.size(), s));
        FL_TRY(H.unit_slice.alloc(std::max<size_t>(uslice.size(), 1), s));
        FL_CUDA(cudaMemcpyAsync(H.unit_step.get(), ustep.data(), ustep.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        if (!uslice.empty())
            FL_CUDA(cudaMemcpyAsync(H.unit_slice.get(), uslice.data(), uslice.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, s));
        FL_CUDA(cudaStreamSynchronize(s));
    }
    k_slice_fill<<<grid_cap(32L * H.nslices, 256, 16), 256, 0, s>>>(
        rows.get(), rlen.get(), rp.get(), hc.get(), hv.get(), H.nrows, H.nslices, H.slice_ptr.get(), H.val.get(),
        narrow ? H.col.get() : nullptr, narrow ? nullptr : H.col32.get(), H.row.get(), H.len.get(), nh);
    FL_CUDA(cudaGetLastError());
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

// ------------------------------------------------------------ kernel ----
// The FP64 bucketed SpMV is the FP64, one right-hand-side instance of the
// generic form kernel (fl_forms.cuh): light items through the FastLoad stream,
// heavy units with x staged in shared memory by a TMA bulk copy.

bool bucket_overlap_ok(const Bucket &B) {
    const HeavyBand &H = B.heavy;
    // light and heavy parts, and the band's x staged in shared memory (the
    // kernels that take the light x late are those)
    return B.light.regions.nitems > 0 && H.nnz > 0 && H.nunits > 0 && H.H0 > 0 && H.nh > 0 &&
           (size_t)H.nh * sizeof(double) <= (size_t)FM_SMEM_MAX && H.nh <= 65535;
}

int spmv_bucket_f64(const Bucket &B, const double *xs, double *y, int accumulate, cudaStream_t s,
                    const XUpload *xu) {
    const HeavyBand &H = B.heavy;
    const Regions &R = B.light.regions;
    FormArgs<double, double> a;
    a.items = R.item.get();
    a.regions = R.region.get();
    a.row = B.light.row.get();
    a.val = B.light.val.get();
    a.nitems = R.nitems;
    a.H0 = H.H0;
    a.nh = H.nnz > 0 ? H.nh : 0;
    a.nslices = H.nnz > 0 ? H.nslices : 0;
    a.nunits = H.nnz > 0 ? H.nunits : 0;
    a.unit_slice = H.unit_slice.get();
    a.unit_step = H.unit_step.get();
    a.slice_ptr = H.slice_ptr.get();
    a.hrow = H.row.get();
    a.hlen = H.len.get();
    a.hval = H.val.get();
    a.hcol16 = H.col.get();
    a.hcol32 = H.col32.get();
    a.xs = xs;
    a.y = y;
    a.err = B.err.get();
    a.x_ready = nullptr;
    a.x_epoch = 0;
    a.err_host = nullptr;
    if (xu) {
        if (!bucket_overlap_ok(B)) return fail(FL_ERR_ARG, "spmv_bucket: overlapped upload does not apply");
        if (B.light_fine_built && B.light_fine.nitems > 0) {
            a.items = B.light_fine.item.get();
            a.regions = B.light_fine.region.get();
            a.nitems = B.light_fine.nitems;
        }
        a.x_ready = xu->flag;
        a.x_epoch = xu->epoch;
        a.err_host = xu->err_host;
    }
    // rows are owned by one lane when the band holds every column and no
    // slice is cut: y is then updated without atomics, and written without
    // zeroing first when every row has band nonzeros
    const int m = B.light.m;
    a.heavy_mode = (R.nitems > 0 || H.split) ? 0 : (!accumulate && H.nrows == m ? 2 : 1);
    a.after_zeroing = !accumulate && a.heavy_mode != 2;
    if (a.after_zeroing) FL_TRY(zero_device(y, (size_t)m * sizeof(double), s));
    const size_t bytes = (size_t)a.nh * sizeof(double);
    a.bulk = a.nh > 0 && ((uintptr_t)(xs + H.H0) % 16 == 0) && bytes % 16 == 0;
    if (a.nitems == 0 && a.nunits == 0) return FL_SUCCESS;
    return run_form_f64(a, 1, H.nh > 65535, s);
}

}  // namespace fl

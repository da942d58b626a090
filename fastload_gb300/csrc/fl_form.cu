// fl_form.cu -- building and running the storage / right-hand-side forms of
// a plan (FP32 values, BF16 hi+lo values, k right-hand sides, heavy bands up
// to every column).
//
// A form is built from the plan's FP64 FastLoad layout: the tile-ordered
// streams are scattered back into the column-sorted CSC (the inverse of the
// tile build), the bucketed split is rebuilt with the requested band, and
// the values are converted to the storage type (FP32: round to nearest;
// BF16 hi+lo: hi = bf16(v) and a 16-bit correction relative to hi, see
// bf16x2_encode in fl_stream.cuh).
#include "fl_forms.cuh"

#include <cuda_bf16.h>

namespace fl {

static int grid_n(long n, int threads, int per_sm = 8) {
    long b = (n + threads - 1) / threads;
    long cap = (long)num_sms() * per_sm;
    return (int)std::max<long>(1, std::min(b, cap));
}

// Inverse of k_tile_build: lane i of tile t goes back to position
// scolptr[colidx + i] + level of the column-sorted CSC.
__global__ void __launch_bounds__(256) k_untile(StepView st, int n, int tilenum, const int *scolptr,
                                                const int *row, const double *val, int *srow_tmp,
                                                double *sval_tmp) {
    const int lane = threadIdx.x & 31;
    long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long t = gw; t < tilenum; t += nw) {
        const int s = upper_index(st.tile_off, st.steps, (int)t);
        const int cs = __ldg(st.col + s), bs = __ldg(st.base + s), ts = __ldg(st.tall + s);
        const int q = (int)t - __ldg(st.tile_off + s);
        const int c = q / ts, l = q - c * ts;
        const int rem = n - cs;
        const int chunks = (rem + 31) >> 5;
        const int len = (c == chunks - 1) ? rem - 32 * c : 32;
        const int colidx = cs + 32 * c;
        const int ptr = __ldg(st.nnz_off + s) + 32 * ts * c + l * len;
        if (lane < len) {
            const int dst = __ldg(scolptr + colidx + lane) + bs + l;
            srow_tmp[dst] = row[ptr + lane];
            sval_tmp[dst] = val[ptr + lane];
        }
    }
}

int untile_layout(const Layout &L, DevBuf<int> &srow, DevBuf<double> &sval, cudaStream_t s) {
    const int n = L.n, nnz = L.nnz;
    DevBuf<int> scolptr;
    FL_TRY(scolptr.alloc((size_t)n + 1, s));
    FL_TRY(scan_exclusive(L.sortnnz.get(), scolptr.get(), n, scolptr.get() + n, s));
    FL_TRY(srow.alloc(std::max(nnz, 1), s));
    FL_TRY(sval.alloc(std::max(nnz, 1), s));
    if (L.tilenum > 0) {
        const StepTable &st = L.st;
        StepView sv{st.col.get(), st.base.get(), st.tall.get(), st.tile_off.get(), st.nnz_off.get(), st.steps};
        k_untile<<<grid_n((long)L.tilenum * 32, 256, 16), 256, 0, s>>>(sv, n, L.tilenum, scolptr.get(), L.row.get(),
                                                                       L.val.get(), srow.get(), sval.get());
        FL_CUDA(cudaGetLastError());
    }
    return FL_SUCCESS;
}

__global__ void k_to_f32(const double *in, float *out, long n) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void k_to_bf16x2(const double *in, uint32_t *out, long n) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = bf16x2_encode(in[i]);
}

static int convert(const DevBuf<double> &src, DevBuf<unsigned char> &dst, int vtype, cudaStream_t s) {
    const long n = (long)src.n;
    FL_TRY(dst.alloc((size_t)std::max<long>(n, 1) * 4, s));
    if (n == 0) return FL_SUCCESS;
    if (vtype == FL_VALUES_F32) k_to_f32<<<grid_n(n, 256), 256, 0, s>>>(src.get(), (float *)dst.get(), n);
    else k_to_bf16x2<<<grid_n(n, 256), 256, 0, s>>>(src.get(), (uint32_t *)dst.get(), n);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

// Values (converted, 4 bytes each) and columns of a slice-layout band to
// the packed layout of 4-byte bands; the band's column arrays are replaced.
int pack_band_p4(HeavyBand &H, const DevBuf<unsigned char> &vals, DevBuf<unsigned char> &out, cudaStream_t s) {
    const long steps = H.padded / 32, ne = p4_entries(steps);
    FL_TRY(out.alloc((size_t)ne * 4, s));
    k_to_p4<uint32_t><<<grid_n(ne, 256), 256, 0, s>>>((const uint32_t *)vals.get(), steps, (uint32_t *)out.get(), ne);
    FL_CUDA(cudaGetLastError());
    if (H.col.get()) {
        DevBuf<uint16_t> c;
        FL_TRY(c.alloc(ne, s));
        k_to_p4<uint16_t><<<grid_n(ne, 256), 256, 0, s>>>(H.col.get(), steps, c.get(), ne);
        FL_CUDA(cudaGetLastError());
        FL_CUDA(cudaStreamSynchronize(s));
        H.col = std::move(c);
    } else {
        DevBuf<int> c;
        FL_TRY(c.alloc(ne, s));
        k_to_p4<int><<<grid_n(ne, 256), 256, 0, s>>>(H.col32.get(), steps, c.get(), ne);
        FL_CUDA(cudaGetLastError());
        FL_CUDA(cudaStreamSynchronize(s));
        H.col32 = std::move(c);
    }
    return FL_SUCCESS;
}

int check_form_opts(const fl_form_opts &o) {
    if (o.value_type != FL_VALUES_F64 && o.value_type != FL_VALUES_F32 && o.value_type != FL_VALUES_BF16X2)
        return fail(FL_ERR_ARG, "add_form: unknown value type %d", o.value_type);
    if (o.y_f32 && o.value_type != FL_VALUES_F32) return fail(FL_ERR_ARG, "add_form: FP32 y needs FP32 values");
    if (o.heavy_band < FL_BAND_ALL) return fail(FL_ERR_ARG, "add_form: heavy band %d", o.heavy_band);
    if (o.light_item != 0 && (o.light_item < 128 || o.light_item > 8192 || o.light_item % 128))
        return fail(FL_ERR_ARG, "add_form: light item %d (0, or 128..8192 in steps of 128)", o.light_item);
    if (o.heavy_loop < FL_HEAVY_AUTO || o.heavy_loop > FL_HEAVY_REGS)
        return fail(FL_ERR_ARG, "add_form: heavy loop %d", o.heavy_loop);
    if (o.x_stage < FL_XSTAGE_AUTO || o.x_stage > FL_XSTAGE_GLOBAL)
        return fail(FL_ERR_ARG, "add_form: x staging %d", o.x_stage);
    if (o.unit_warps < 0 || o.unit_warps > 64) return fail(FL_ERR_ARG, "add_form: unit_warps %d (0..64)", o.unit_warps);
    if (o.reserved != 0) return fail(FL_ERR_ARG, "add_form: reserved field must be 0");
    return FL_SUCCESS;
}

int build_form(Form &F, const Layout &L, const fl_form_opts &o, cudaStream_t s) {
    FL_TRY(check_form_opts(o));
    const int vtype = o.value_type, band = o.heavy_band;
    F.vtype = vtype;
    F.yf32 = o.y_f32 != 0;
    F.band = band;
    F.opts = o;
    const int m = L.m, n = L.n, nnz = L.nnz;
    // the column-sorted CSC, recovered from the tile streams
    DevBuf<int> srow;
    DevBuf<double> sval;
    FL_TRY(untile_layout(L, srow, sval, s));
    int nh;
    bool wide = false;
    if (band == FL_BAND_NONE) {
        nh = 0;
    } else if (band == FL_BAND_ALL) {
        nh = n;
        wide = true;
    } else if (band == FL_BAND_AUTO) {
        nh = auto_layout_band(L, vtype == FL_VALUES_F64 ? 8 : 4, &wide, s);
        if (nh < 0) return nh;
    } else if (band > 0) {
        nh = std::min(band, n);
        wide = nh > bucket_max_band();
    } else {
        return fail(FL_ERR_ARG, "add_form: heavy band %d", band);
    }
    FL_TRY(build_bucket(F.B, m, n, nnz, L.sortnnz.get(), srow.get(), sval.get(), nh, s, wide, o.unit_warps));
    F.wide = F.B.heavy.nh > 65535;
    // light items: as asked, else for 4-byte values at most 1,024 nonzeros
    // (the light stream's items are serial chains on one warp; beside the
    // faster packed band, shorter chains end with it: 50.8 against 54.3 us
    // at the 2^20-column Zipf(1.8) matrix)
    const int auto_item = item_nnz_for(nnz);
    const int item = o.light_item > 0 ? o.light_item : (vtype == FL_VALUES_F64 ? auto_item : std::min(auto_item, 1024));
    if (F.B.light.nnz > 0 && item != auto_item) FL_TRY(build_regions_sized(F.B.light, item, F.B.light.regions, s));
    if (vtype != FL_VALUES_F64) {
        FL_TRY(convert(F.B.light.val, F.lval, vtype, s));
        HeavyBand &H = F.B.heavy;
        if (H.nnz > 0 && H.nh > 0) {
            // the band in lane-major packs of four steps (fl_forms.cuh)
            DevBuf<unsigned char> conv;
            FL_TRY(convert(H.val, conv, vtype, s));
            FL_TRY(pack_band_p4(H, conv, F.hval, s));
        }
        FL_CUDA(cudaStreamSynchronize(s));
        F.B.light.val.release();
        H.val.release();
    }
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

template <typename V, typename Y>
static FormArgs<V, Y> form_args(Form &F, const V *lval, const V *hval, const void *xs, void *y) {
    const Bucket &B = F.B;
    const HeavyBand &H = B.heavy;
    FormArgs<V, Y> a;
    a.items = B.light.regions.item.get();
    a.regions = B.light.regions.region.get();
    a.row = B.light.row.get();
    a.val = lval;
    a.nitems = B.light.regions.nitems;
    a.H0 = H.H0;
    a.nh = H.nnz > 0 ? H.nh : 0;
    a.nslices = H.nnz > 0 ? H.nslices : 0;
    a.nunits = H.nnz > 0 ? H.nunits : 0;
    a.unit_slice = H.unit_slice.get();
    a.unit_step = H.unit_step.get();
    a.slice_ptr = H.slice_ptr.get();
    a.hrow = H.row.get();
    a.hlen = H.len.get();
    a.hval = hval;
    a.hcol16 = H.col.get();
    a.hcol32 = H.col32.get();
    a.xs = (const typename VT<V>::X *)xs;
    a.y = (Y *)y;
    a.err = B.err.get();
    a.x_ready = nullptr;
    a.x_epoch = 0;
    a.err_host = nullptr;
    a.heavy_mode = 0;
    a.bulk = 0;
    a.heavy_loop = F.opts.heavy_loop;
    a.x_stage = F.opts.x_stage;
    return a;
}

int spmv_form(Form &F, int k, const void *xs, void *y, int accumulate, cudaStream_t s) {
    if (k != 1 && k != 8) return fail(FL_ERR_ARG, "spmv_form: k=%d (supported: 1, 8)", k);
    const Bucket &B = F.B;
    const int m = B.light.m;
    const size_t ysz = F.yf32 ? sizeof(float) : sizeof(double);
    const size_t xsz = F.vtype == FL_VALUES_F64 ? sizeof(double) : sizeof(float);
    if (k > 1 && (((uintptr_t)xs % 16) || ((uintptr_t)y % 16)))
        return fail(FL_ERR_ARG, "spmv_form: x and y must be 16-byte aligned for k > 1");
    // the heavy band owns whole rows when there is no light part and no
    // slice is cut across work units: then y is updated without atomics, and
    // written without zeroing first when every row has band nonzeros
    const bool light = B.light.regions.nitems > 0;
    const int mode = (light || B.heavy.split) ? 0 : (!accumulate && B.heavy.nrows == m ? 2 : 1);
    const bool zeroed = !accumulate && mode != 2;
    if (zeroed) FL_TRY(zero_device(y, (size_t)m * k * ysz, s));
    if (!light && B.heavy.nnz == 0) return FL_SUCCESS;
    const HeavyBand &H = B.heavy;
    const size_t band_bytes = (size_t)H.nh * k * xsz;
    const bool bulk = H.nh > 0 && ((uintptr_t)((const char *)xs + (size_t)H.H0 * k * xsz) % 16 == 0) &&
                      band_bytes % 16 == 0;
    if (F.vtype == FL_VALUES_F64) {
        auto a = form_args<double, double>(F, B.light.val.get(), B.heavy.val.get(), xs, y);
        a.bulk = bulk;
        a.heavy_mode = mode;
        a.after_zeroing = zeroed;
        return run_form_f64(a, k, F.wide, s);
    }
    if (F.vtype == FL_VALUES_F32) {
        if (F.yf32) {
            auto a = form_args<float, float>(F, (const float *)F.lval.get(), (const float *)F.hval.get(), xs, y);
            a.bulk = bulk;
            a.heavy_mode = mode;
            a.after_zeroing = zeroed;
            return run_form_f32_y32(a, k, F.wide, s);
        }
        auto a = form_args<float, double>(F, (const float *)F.lval.get(), (const float *)F.hval.get(), xs, y);
        a.bulk = bulk;
        a.heavy_mode = mode;
        a.after_zeroing = zeroed;
        return run_form_f32(a, k, F.wide, s);
    }
    auto a = form_args<bf16x2_t, double>(F, (const bf16x2_t *)F.lval.get(), (const bf16x2_t *)F.hval.get(), xs, y);
    a.bulk = bulk;
    a.heavy_mode = mode;
    a.after_zeroing = zeroed;
    return run_form_bf16(a, k, F.wide, s);
}

__global__ void k_permute_x_k(const int *perm, int n, int k, const double *x, double *xs64, float *xs32) {
    const long total = (long)n * k;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const long c = i / k, r = i - c * k;
        const double v = x[(long)perm[c] * k + r];
        if (xs32) xs32[i] = (float)v;
        else xs64[i] = v;
    }
}

int permute_x_k(const int *perm, int n, int k, const double *x, void *xs, int to_f32, cudaStream_t s) {
    if (n <= 0) return FL_SUCCESS;
    k_permute_x_k<<<grid_n((long)n * k, 256), 256, 0, s>>>(perm, n, k, x, to_f32 ? nullptr : (double *)xs,
                                                           to_f32 ? (float *)xs : nullptr);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

}  // namespace fl

using namespace fl;

extern "C" int fl_convert_values(int value_type, long n, const double *d_in, void *d_out, void *stream) {
    clear_error();
    if (value_type != FL_VALUES_F32 && value_type != FL_VALUES_BF16X2)
        return fail(FL_ERR_ARG, "convert_values: value type %d (FP32 or BF16 hi+lo)", value_type);
    if (n < 0 || (n && (!d_in || !d_out))) return fail(FL_ERR_ARG, "convert_values: bad arguments");
    if (n == 0) return FL_SUCCESS;
    const cudaStream_t s = (cudaStream_t)stream;
    if (value_type == FL_VALUES_F32) k_to_f32<<<grid_n(n, 256), 256, 0, s>>>(d_in, (float *)d_out, n);
    else k_to_bf16x2<<<grid_n(n, 256), 256, 0, s>>>(d_in, (uint32_t *)d_out, n);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

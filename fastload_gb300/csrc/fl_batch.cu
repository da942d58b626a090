// fl_batch.cu -- many matrices through one persistent launch.
//
// A batch stacks every matrix as row slices: each matrix's rows are put into
// the heavy-band layout with the band holding all of its columns (rows
// sorted by length, 32 rows per slice, one lane per row), the slices of all
// matrices are concatenated with rows shifted into the stacked y and columns
// into the stacked (sorted) x, and the stacked slices are cut into work
// units.  One launch of the form kernel then runs every matrix with each row
// owned by one lane: no atomics, y stored once per row (rows without
// nonzeros are zeroed first when there are any).  fl_batch_spmv_graph
// captures the launch into a CUDA graph once and replays it.
#include "fl_forms.cuh"

#include <cstring>
#include <vector>

using namespace fl;

struct fl_batch {
    int count = 0, vtype = FL_VALUES_F32, yf32 = 1;
    long M = 0, N = 0, NNZ = 0;
    std::vector<int> m_off, n_off;  // count+1 each
    // stacked row slices
    int nslices = 0, nunits = 0;
    bool all_rows = false;        // every row of the batch has a nonzero
    DevBuf<unsigned char> val;    // slice entries in the storage type
    DevBuf<int> col;              // stacked sorted column of each entry
    DevBuf<int> slice_ptr, srow, slen, unit_slice, unit_step;
    bool split = false;           // a slice is cut across units (y by atomics)
    DevBuf<int> perm;             // stacked sorted position -> stacked original column
    DevBuf<int> err;
    // captured graph and the pointers it was captured with
    cudaGraphExec_t exec = nullptr;
    const void *g_xs = nullptr;
    void *g_y = nullptr;
    cudaStream_t cap = nullptr;
    ~fl_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (cap) cudaStreamDestroy(cap);
    }
};

namespace {

int grid_b(long n, int threads) {
    long b = (n + threads - 1) / threads;
    long cap = (long)num_sms() * 8;
    return (int)std::max<long>(1, std::min(b, cap));
}

__global__ void k_stack_rows(const int *src, long n, int off, int *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int r = src[i];
        dst[i] = r < 0 ? -1 : r + off;
    }
}

__global__ void k_stack_cols(const uint16_t *c16, const int *c32, long n, int off, int *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = (c16 ? (int)c16[i] : c32[i]) + off;
}

__global__ void k_batch_vals(const double *src, long n, int vtype, unsigned char *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = src[i];
        if (vtype == FL_VALUES_F64) {
            ((double *)dst)[i] = v;
        } else if (vtype == FL_VALUES_F32) {
            ((float *)dst)[i] = (float)v;
        } else {
            ((uint32_t *)dst)[i] = bf16x2_encode(v);
        }
    }
}

__global__ void k_batch_permute(const int *perm, long n, const double *x, float *xs32, double *xs64) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = x[perm[i]];
        if (xs32) xs32[i] = (float)v;
        else xs64[i] = v;
    }
}

size_t vsize(int vtype) { return vtype == FL_VALUES_F64 ? 8 : 4; }

int launch(fl_batch *b, const void *xs, void *y, cudaStream_t s) {
    const size_t ysz = b->yf32 ? sizeof(float) : sizeof(double);
    if (!b->all_rows || b->split) FL_TRY(zero_device(y, (size_t)b->M * ysz, s));
    if (b->nunits == 0) return FL_SUCCESS;
    auto fill = [&](auto &a) {
        a.items = nullptr;
        a.regions = nullptr;
        a.row = nullptr;
        a.val = nullptr;
        a.nitems = 0;
        a.H0 = 0;
        a.nh = (int)std::max<long>(b->N, 1);
        a.nslices = b->nslices;
        a.nunits = b->nunits;
        a.bulk = 0;
        // every row with nonzeros is owned by one lane, unless its slice is
        // cut across units: then the parts meet in y by atomics
        a.heavy_mode = b->split ? 0 : 2;
        a.slice_ptr = b->slice_ptr.get();
        a.hrow = b->srow.get();
        a.hlen = b->slen.get();
        a.unit_slice = b->unit_slice.get();
        a.unit_step = b->unit_step.get();
        a.hcol16 = nullptr;
        a.hcol32 = b->col.get();
        a.err = b->err.get();
        a.x_ready = nullptr;
        a.x_epoch = 0;
        a.err_host = nullptr;
        a.contig = 1;  // a block's units from one matrix at a time: its x in the SM's L1
    };
    if (b->vtype == FL_VALUES_F64) {
        FormArgs<double, double> a;
        fill(a);
        a.hval = (const double *)b->val.get();
        a.xs = (const double *)xs;
        a.y = (double *)y;
        return run_form_f64(a, 1, true, s);
    }
    if (b->vtype == FL_VALUES_F32 && b->yf32) {
        FormArgs<float, float> a;
        fill(a);
        a.hval = (const float *)b->val.get();
        a.xs = (const float *)xs;
        a.y = (float *)y;
        return run_form_f32_y32(a, 1, true, s);
    }
    if (b->vtype == FL_VALUES_F32) {
        FormArgs<float, double> a;
        fill(a);
        a.hval = (const float *)b->val.get();
        a.xs = (const float *)xs;
        a.y = (double *)y;
        return run_form_f32(a, 1, true, s);
    }
    FormArgs<bf16x2_t, double> a;
    fill(a);
    a.hval = (const bf16x2_t *)b->val.get();
    a.xs = (const float *)xs;
    a.y = (double *)y;
    return run_form_bf16(a, 1, true, s);
}

}  // namespace

extern "C" {

int fl_batch_create(fl_batch_t *out, int count, const fl_plan_t *plans, int value_type, int y_f32) {
    clear_error();
    if (!out || count < 0 || (count && !plans)) return fail(FL_ERR_ARG, "batch_create: bad arguments");
    *out = nullptr;
    if (value_type != FL_VALUES_F64 && value_type != FL_VALUES_F32 && value_type != FL_VALUES_BF16X2)
        return fail(FL_ERR_ARG, "batch_create: unknown value type %d", value_type);
    if (y_f32 && value_type != FL_VALUES_F32) return fail(FL_ERR_ARG, "batch_create: FP32 y needs FP32 values");
    std::unique_ptr<fl_batch> b(new (std::nothrow) fl_batch());
    if (!b) return fail(FL_ERR_ALLOC, "batch_create: host allocation failed");
    b->count = count;
    b->vtype = value_type;
    b->yf32 = y_f32 != 0;
    b->m_off.assign(count + 1, 0);
    b->n_off.assign(count + 1, 0);
    for (int i = 0; i < count; i++) {
        if (!plans[i]) return fail(FL_ERR_ARG, "batch_create: plan %d is NULL", i);
        const Layout &L = plans[i]->L;
        const long mo = (long)b->m_off[i] + L.m, no = (long)b->n_off[i] + L.n;
        b->NNZ += L.nnz;
        if (mo > 0x7fffffffL || no > 0x7fffffffL || b->NNZ > 0x7fffffffL)
            return fail(FL_ERR_OVERFLOW, "batch_create: the stacked batch exceeds the 32-bit index space");
        b->m_off[i + 1] = (int)mo;
        b->n_off[i + 1] = (int)no;
    }
    b->M = b->m_off[count];
    b->N = b->n_off[count];
    const cudaStream_t s = 0;
    FL_CUDA(cudaDeviceSynchronize());
    // each matrix's rows as slices with every column in the band, built one
    // matrix at a time and appended to the stacked arrays
    std::vector<Bucket> parts(count);
    std::vector<long> e_off(count + 1, 0);
    std::vector<int> s_off(count + 1, 0);
    long rows_covered = 0;
    for (int i = 0; i < count; i++) {
        const Layout &L = plans[i]->L;
        if (L.nnz) {
            DevBuf<int> srow;
            DevBuf<double> sval;
            FL_TRY(untile_layout(L, srow, sval, s));
            FL_TRY(build_bucket(parts[i], L.m, L.n, L.nnz, L.sortnnz.get(), srow.get(), sval.get(), L.n, s, true));
        }
        const HeavyBand &H = parts[i].heavy;
        const int ns = L.nnz ? H.nslices : 0;
        e_off[i + 1] = e_off[i] + (L.nnz ? H.padded : 0);
        if ((long)s_off[i] + ns > 0x7fffffffL / 32 || e_off[i + 1] > 0x7fffffffL)
            return fail(FL_ERR_OVERFLOW, "batch_create: the stacked slices exceed the 32-bit index space");
        s_off[i + 1] = s_off[i] + ns;
        rows_covered += L.nnz ? H.nrows : 0;
        parts[i].light = Layout();  // band holds every column: no light part
    }
    b->nslices = s_off[count];
    b->all_rows = rows_covered == b->M;
    const long E = std::max<long>(e_off[count], 1);
    FL_TRY(b->val.alloc((size_t)E * vsize(value_type), s));
    FL_TRY(b->col.alloc(E, s));
    FL_TRY(b->slice_ptr.alloc((size_t)b->nslices + 1, s));
    FL_TRY(b->srow.alloc(std::max(32L * b->nslices, 1L), s));
    FL_TRY(b->slen.alloc(std::max(32L * b->nslices, 1L), s));
    std::vector<int> sp((size_t)b->nslices + 1, 0), perm(std::max<long>(b->N, 1));
    for (int i = 0; i < count; i++) {
        const Layout &L = plans[i]->L;
        const HeavyBand &H = parts[i].heavy;
        const int ns = s_off[i + 1] - s_off[i];
        if (ns) {
            const long ne = e_off[i + 1] - e_off[i];
            k_batch_vals<<<grid_b(ne, 256), 256, 0, s>>>(H.val.get(), ne, value_type,
                                                          b->val.get() + e_off[i] * vsize(value_type));
            FL_CUDA(cudaGetLastError());
            k_stack_cols<<<grid_b(ne, 256), 256, 0, s>>>(H.col.get(), H.col.get() ? nullptr : H.col32.get(), ne,
                                                          b->n_off[i], b->col.get() + e_off[i]);
            FL_CUDA(cudaGetLastError());
            k_stack_rows<<<grid_b(32L * ns, 256), 256, 0, s>>>(H.row.get(), 32L * ns, b->m_off[i],
                                                                b->srow.get() + 32L * s_off[i]);
            FL_CUDA(cudaGetLastError());
            FL_CUDA(cudaMemcpyAsync(b->slen.get() + 32L * s_off[i], H.len.get(), 32L * ns * sizeof(int),
                                    cudaMemcpyDeviceToDevice, s));
            FL_CUDA(cudaMemcpyAsync(sp.data() + s_off[i], H.slice_ptr.get(), (size_t)ns * sizeof(int),
                                    cudaMemcpyDeviceToHost, s));
        }
        if (L.n)
            FL_CUDA(cudaMemcpyAsync(perm.data() + b->n_off[i], L.perm.get(), L.n * sizeof(int), cudaMemcpyDeviceToHost,
                                    s));
        FL_CUDA(cudaStreamSynchronize(s));
        parts[i] = Bucket();  // release this matrix's band before the next
    }
    for (int i = 0; i < count; i++) {
        for (int q = s_off[i]; q < s_off[i + 1]; q++) sp[q] += (int)e_off[i];
        for (int c = b->n_off[i]; c < b->n_off[i + 1]; c++) perm[c] += b->n_off[i];
    }
    sp[b->nslices] = (int)e_off[count];
    if (vsize(value_type) == 4 && e_off[count] > 0) {
        // 4-byte values: the stacked band in lane-major packs of four steps
        // (fl_forms.cuh), values and columns alike
        const long steps = e_off[count] / 32, ne = p4_entries(steps);
        DevBuf<unsigned char> pv;
        DevBuf<int> pc;
        FL_TRY(pv.alloc((size_t)ne * 4, s));
        FL_TRY(pc.alloc(ne, s));
        k_to_p4<uint32_t><<<grid_b(ne, 256), 256, 0, s>>>((const uint32_t *)b->val.get(), steps,
                                                          (uint32_t *)pv.get(), ne);
        FL_CUDA(cudaGetLastError());
        k_to_p4<int><<<grid_b(ne, 256), 256, 0, s>>>(b->col.get(), steps, pc.get(), ne);
        FL_CUDA(cudaGetLastError());
        FL_CUDA(cudaStreamSynchronize(s));
        b->val = std::move(pv);
        b->col = std::move(pc);
    }
    // work units over the stacked slices, about sixteen per resident warp:
    // a block's contiguous range of units is claimed unit by unit, so
    // smaller units even out its warps' work (256 matrices of 186M
    // nonzeros: 0.82 / 0.67 / 0.64 / 0.62 / 0.60 ms at 1 / 2 / 4 / 8 / 16)
    std::vector<int> ustep, uslice;
    b->split = make_units(sp, e_off[count] / (16L * num_sms() * 32), ustep, uslice);
    b->nunits = (int)uslice.size();
    FL_TRY(b->unit_step.alloc(ustep.size(), s));
    FL_TRY(b->unit_slice.alloc(std::max<size_t>(uslice.size(), 1), s));
    FL_TRY(b->perm.alloc(perm.size(), s));
    FL_CUDA(cudaMemcpyAsync(b->slice_ptr.get(), sp.data(), sp.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    FL_CUDA(cudaMemcpyAsync(b->unit_step.get(), ustep.data(), ustep.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (!uslice.empty())
        FL_CUDA(cudaMemcpyAsync(b->unit_slice.get(), uslice.data(), uslice.size() * sizeof(int),
                                cudaMemcpyHostToDevice, s));
    FL_CUDA(cudaMemcpyAsync(b->perm.get(), perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    FL_TRY(b->err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(b->err.get(), 0, sizeof(int), s));
    FL_CUDA(cudaStreamSynchronize(s));
    *out = b.release();
    return FL_SUCCESS;
}

int fl_batch_info(fl_batch_t b, int *count, long *m_total, long *n_total, long *nnz_total, int *items) {
    clear_error();
    if (!b) return fail(FL_ERR_ARG, "batch_info: NULL batch");
    if (count) *count = b->count;
    if (m_total) *m_total = b->M;
    if (n_total) *n_total = b->N;
    if (nnz_total) *nnz_total = b->NNZ;
    if (items) *items = b->nunits;
    return FL_SUCCESS;
}

int fl_batch_offsets(fl_batch_t b, int *m_off, int *n_off) {
    clear_error();
    if (!b) return fail(FL_ERR_ARG, "batch_offsets: NULL batch");
    if (m_off) memcpy(m_off, b->m_off.data(), (b->count + 1) * sizeof(int));
    if (n_off) memcpy(n_off, b->n_off.data(), (b->count + 1) * sizeof(int));
    return FL_SUCCESS;
}

int fl_batch_permute_x(fl_batch_t b, const double *d_x, void *d_xs, void *stream) {
    clear_error();
    if (!b || (b->N && (!d_x || !d_xs))) return fail(FL_ERR_ARG, "batch_permute_x: NULL argument");
    if (!b->N) return FL_SUCCESS;
    const bool f32 = b->vtype != FL_VALUES_F64;
    k_batch_permute<<<grid_b(b->N, 256), 256, 0, (cudaStream_t)stream>>>(
        b->perm.get(), b->N, d_x, f32 ? (float *)d_xs : nullptr, f32 ? nullptr : (double *)d_xs);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

int fl_batch_spmv(fl_batch_t b, const void *d_xs, void *d_y, void *stream) {
    if (!b || (b->N && !d_xs) || (b->M && !d_y)) return fail(FL_ERR_ARG, "batch_spmv: NULL argument");
    return launch(b, d_xs, d_y, (cudaStream_t)stream);
}

int fl_batch_spmv_graph(fl_batch_t b, const void *d_xs, void *d_y, void *stream) {
    clear_error();
    if (!b || (b->N && !d_xs) || (b->M && !d_y)) return fail(FL_ERR_ARG, "batch_spmv_graph: NULL argument");
    if (!b->exec || b->g_xs != d_xs || b->g_y != d_y) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        if (!b->cap) FL_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        FL_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        const int rc = launch(b, d_xs, d_y, b->cap);
        cudaError_t e = cudaStreamEndCapture(b->cap, &g);
        if (rc != FL_SUCCESS) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(FL_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(FL_ERR_CUDA, "batch graph instantiate failed: %s", cudaGetErrorString(e));
        b->g_xs = d_xs;
        b->g_y = d_y;
    }
    FL_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return FL_SUCCESS;
}

int fl_batch_destroy(fl_batch_t b) {
    if (!b) return FL_SUCCESS;
    cudaDeviceSynchronize();
    delete b;
    return FL_SUCCESS;
}

}  // extern "C"

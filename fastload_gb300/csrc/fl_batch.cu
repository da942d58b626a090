// fl_batch.cu -- many matrices through one persistent FastLoad launch.
//
// A batch concatenates the FastLoad layouts of independent matrices: their
// tile-ordered streams (rows shifted by each matrix's offset in the stacked
// y, values converted to the storage type), their region tables (stream
// starts and first sorted columns shifted into the stacked x) and their work
// items.  One launch of the streaming form kernel then walks every matrix's
// work items with the dynamic work counter, so matrices of very different
// sizes share the GPU evenly.  fl_batch_spmv_graph captures the y zeroing,
// the counter reset and the launch into a CUDA graph once and replays it.
#include "fl_forms.cuh"

#include <cstring>
#include <vector>

namespace fl {

int run_form_f64(const FormArgs<double, double> &a, int k, bool wide, cudaStream_t s);
int run_form_f32(const FormArgs<float, double> &a, int k, bool wide, cudaStream_t s);
int run_form_f32_y32(const FormArgs<float, float> &a, int k, bool wide, cudaStream_t s);
int run_form_bf16(const FormArgs<bf16x2_t, double> &a, int k, bool wide, cudaStream_t s);

}  // namespace fl

using namespace fl;

struct fl_batch {
    int count = 0, vtype = FL_VALUES_F32, yf32 = 1;
    long M = 0, N = 0, NNZ = 0;
    std::vector<int> m_off, n_off;  // count+1 each
    DevBuf<int> row;
    DevBuf<unsigned char> val;
    DevBuf<RegionDesc> regions;
    DevBuf<ItemDesc> items;
    int nitems = 0;
    DevBuf<int> perm;  // stacked sorted position -> stacked original column
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

__global__ void k_batch_rows(const int *src, long n, int off, int *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i] + off;
}

__global__ void k_batch_vals(const double *src, long n, int vtype, unsigned char *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = src[i];
        if (vtype == FL_VALUES_F64) {
            ((double *)dst)[i] = v;
        } else if (vtype == FL_VALUES_F32) {
            ((float *)dst)[i] = (float)v;
        } else {
            const __nv_bfloat16 hi = __double2bfloat16(v);
            const __nv_bfloat16 lo = __double2bfloat16(v - (double)__bfloat162float(hi));
            ((uint32_t *)dst)[i] = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(lo) << 16);
        }
    }
}

__global__ void k_batch_fill(int *row, long from, long to) {
    for (long i = from + blockIdx.x * (long)blockDim.x + threadIdx.x; i < to; i += (long)gridDim.x * blockDim.x)
        row[i] = -1;
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
    if (b->M) FL_CUDA(cudaMemsetAsync(y, 0, (size_t)b->M * ysz, s));
    if (b->nitems == 0) return FL_SUCCESS;
    auto fill = [&](auto &a) {
        a.items = b->items.get();
        a.regions = b->regions.get();
        a.row = b->row.get();
        a.nitems = b->nitems;
        a.H0 = 0;
        a.nh = 0;
        a.nslices = 0;
        a.nunits = 0;
        a.bulk = 0;
        a.heavy_mode = 0;
        a.slice_ptr = a.hrow = a.hlen = a.unit_slice = nullptr;
        a.hval = nullptr;
        a.hcol16 = nullptr;
        a.hcol32 = nullptr;
        a.err = b->err.get();
    };
    if (b->vtype == FL_VALUES_F64) {
        FormArgs<double, double> a;
        fill(a);
        a.val = (const double *)b->val.get();
        a.xs = (const double *)xs;
        a.y = (double *)y;
        return run_form_f64(a, 1, false, s);
    }
    if (b->vtype == FL_VALUES_F32 && b->yf32) {
        FormArgs<float, float> a;
        fill(a);
        a.val = (const float *)b->val.get();
        a.xs = (const float *)xs;
        a.y = (float *)y;
        return run_form_f32_y32(a, 1, false, s);
    }
    if (b->vtype == FL_VALUES_F32) {
        FormArgs<float, double> a;
        fill(a);
        a.val = (const float *)b->val.get();
        a.xs = (const float *)xs;
        a.y = (double *)y;
        return run_form_f32(a, 1, false, s);
    }
    FormArgs<bf16x2_t, double> a;
    fill(a);
    a.val = (const bf16x2_t *)b->val.get();
    a.xs = (const float *)xs;
    a.y = (double *)y;
    return run_form_bf16(a, 1, false, s);
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
    std::vector<long> e_off(count + 1, 0);
    std::vector<int> r_off(count + 1, 0), i_off(count + 1, 0);
    for (int i = 0; i < count; i++) {
        if (!plans[i]) return fail(FL_ERR_ARG, "batch_create: plan %d is NULL", i);
        const Layout &L = plans[i]->L;
        b->m_off[i + 1] = b->m_off[i] + L.m;
        b->n_off[i + 1] = b->n_off[i] + L.n;
        e_off[i + 1] = e_off[i] + L.nnz;
        r_off[i + 1] = r_off[i] + L.regions.nregions;
        i_off[i + 1] = i_off[i] + L.regions.nitems;
        if ((long)b->m_off[i + 1] != (long)b->m_off[i] + L.m || e_off[i + 1] > 0x7fffffffL - 65536)
            return fail(FL_ERR_OVERFLOW, "batch_create: the stacked batch exceeds the 32-bit index space");
    }
    b->M = b->m_off[count];
    b->N = b->n_off[count];
    b->NNZ = e_off[count];
    b->nitems = i_off[count];
    cudaStream_t s = 0;
    FL_CUDA(cudaDeviceSynchronize());
    const size_t np = padded((size_t)b->NNZ);
    FL_TRY(b->row.alloc(np, s));
    FL_TRY(b->val.alloc(np * vsize(value_type), s));
    FL_CUDA(cudaMemsetAsync(b->val.get(), 0, np * vsize(value_type), s));
    k_batch_fill<<<grid_b(np - b->NNZ, 256), 256, 0, s>>>(b->row.get(), b->NNZ, (long)np);
    FL_CUDA(cudaGetLastError());
    std::vector<RegionDesc> reg(std::max(r_off[count], 1));
    std::vector<ItemDesc> itm(std::max(i_off[count], 1));
    std::vector<int> perm(std::max<long>(b->N, 1));
    for (int i = 0; i < count; i++) {
        const Layout &L = plans[i]->L;
        if (L.nnz) {
            k_batch_rows<<<grid_b(L.nnz, 256), 256, 0, s>>>(L.row.get(), L.nnz, b->m_off[i], b->row.get() + e_off[i]);
            FL_CUDA(cudaGetLastError());
            k_batch_vals<<<grid_b(L.nnz, 256), 256, 0, s>>>(L.val.get(), L.nnz, value_type,
                                                             b->val.get() + e_off[i] * vsize(value_type));
            FL_CUDA(cudaGetLastError());
        }
        if (L.regions.nregions)
            FL_CUDA(cudaMemcpyAsync(reg.data() + r_off[i], L.regions.region.get(),
                                    L.regions.nregions * sizeof(RegionDesc), cudaMemcpyDeviceToHost, s));
        if (L.regions.nitems)
            FL_CUDA(cudaMemcpyAsync(itm.data() + i_off[i], L.regions.item.get(), L.regions.nitems * sizeof(ItemDesc),
                                    cudaMemcpyDeviceToHost, s));
        if (L.n)
            FL_CUDA(cudaMemcpyAsync(perm.data() + b->n_off[i], L.perm.get(), L.n * sizeof(int), cudaMemcpyDeviceToHost,
                                    s));
    }
    FL_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < count; i++) {
        for (int r = r_off[i]; r < r_off[i + 1]; r++) {
            reg[r].start += (int)e_off[i];
            reg[r].col_base += b->n_off[i];
        }
        for (int t = i_off[i]; t < i_off[i + 1]; t++) {
            itm[t].begin += (int)e_off[i];
            itm[t].end += (int)e_off[i];
            itm[t].region += r_off[i];
        }
        for (int c = b->n_off[i]; c < b->n_off[i + 1]; c++) perm[c] += b->n_off[i];
    }
    FL_TRY(b->regions.alloc(reg.size(), s));
    FL_TRY(b->items.alloc(itm.size(), s));
    FL_TRY(b->perm.alloc(perm.size(), s));
    FL_CUDA(cudaMemcpyAsync(b->regions.get(), reg.data(), reg.size() * sizeof(RegionDesc), cudaMemcpyHostToDevice, s));
    FL_CUDA(cudaMemcpyAsync(b->items.get(), itm.data(), itm.size() * sizeof(ItemDesc), cudaMemcpyHostToDevice, s));
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
    if (items) *items = b->nitems;
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

// fl_cmp.cu -- comparators for reports: the reference's naive CSC kernel and
// cuSPARSE CSR SpMV, re-hosted on device buffers with stream-ordered launches
// so they can be timed with CUDA events next to the FastLoad kernels.  They
// are context lines, never a fallback of the FastLoad path.
//
// cuSPARSE is opened with dlopen on first use, so the library itself does
// not depend on it; without it the cuSPARSE calls return FL_ERR_UNAVAILABLE.
#include <dlfcn.h>
#include <cusparse.h>

#include <memory>
#include <mutex>

#include "fl_internal.cuh"

namespace fl {
namespace {

// One thread per column, one atomic per nonzero: the algorithm and launch
// shape (32 blocks of 64 threads per SM) of CSC_SpMV_kernel
// (src/CSCSpMV.h:4-27, launched at :68).
__global__ void k_csc_naive(int n, const int *__restrict__ colptr, const int *__restrict__ rowidx,
                            const double *__restrict__ val, const double *__restrict__ x, double *y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        const double xi = x[i];
        for (int j = colptr[i]; j < colptr[i + 1]; j++) atomicAdd(y + rowidx[j], val[j] * xi);
    }
}

struct CuSparseApi {
    void *so = nullptr;
    decltype(&cusparseCreate) create;
    decltype(&cusparseDestroy) destroy;
    decltype(&cusparseSetStream) set_stream;
    decltype(&cusparseCreateCsr) create_csr;
    decltype(&cusparseDestroySpMat) destroy_spmat;
    decltype(&cusparseCreateDnVec) create_dnvec;
    decltype(&cusparseDestroyDnVec) destroy_dnvec;
    decltype(&cusparseDnVecSetValues) dnvec_set;
    decltype(&cusparseSpMV_bufferSize) buffer_size;
    decltype(&cusparseSpMV_preprocess) preprocess;
    decltype(&cusparseSpMV) spmv;
    decltype(&cusparseGetErrorString) error_string;
};

std::mutex g_api_mu;
CuSparseApi g_api;
int g_api_state = 0;  // 0 not tried, 1 loaded, -1 unavailable

template <typename F>
bool sym(void *so, const char *name, F &f) {
    f = (F)dlsym(so, name);
    return f != nullptr;
}

int cusparse_api(const CuSparseApi **out) {
    std::lock_guard<std::mutex> lk(g_api_mu);
    if (g_api_state == 0) {
        void *so = dlopen("libcusparse.so.12", RTLD_NOW | RTLD_LOCAL);
        if (!so) so = dlopen("libcusparse.so", RTLD_NOW | RTLD_LOCAL);
        CuSparseApi a;
        a.so = so;
        const bool ok = so && sym(so, "cusparseCreate", a.create) && sym(so, "cusparseDestroy", a.destroy) &&
                        sym(so, "cusparseSetStream", a.set_stream) && sym(so, "cusparseCreateCsr", a.create_csr) &&
                        sym(so, "cusparseDestroySpMat", a.destroy_spmat) &&
                        sym(so, "cusparseCreateDnVec", a.create_dnvec) &&
                        sym(so, "cusparseDestroyDnVec", a.destroy_dnvec) &&
                        sym(so, "cusparseDnVecSetValues", a.dnvec_set) &&
                        sym(so, "cusparseSpMV_bufferSize", a.buffer_size) &&
                        sym(so, "cusparseSpMV_preprocess", a.preprocess) && sym(so, "cusparseSpMV", a.spmv) &&
                        sym(so, "cusparseGetErrorString", a.error_string);
        g_api_state = ok ? 1 : -1;
        if (ok) g_api = a;
    }
    if (g_api_state < 0) return fail(FL_ERR_UNAVAILABLE, "cuSPARSE comparator: libcusparse could not be loaded");
    *out = &g_api;
    return FL_SUCCESS;
}

}  // namespace
}  // namespace fl

using namespace fl;

struct fl_cusparse {
    const CuSparseApi *api = nullptr;
    cusparseHandle_t handle = nullptr;
    cusparseSpMatDescr_t A = nullptr;
    cusparseDnVecDescr_t x = nullptr, y = nullptr;
    cusparseSpMVAlg_t alg = CUSPARSE_SPMV_ALG_DEFAULT;
    DevBuf<unsigned char> buffer;
    DevBuf<double> xs, ys;  // vectors the descriptors are created and preprocessed with
    int m = 0, n = 0;
    ~fl_cusparse() {
        if (!api) return;
        if (x) api->destroy_dnvec(x);
        if (y) api->destroy_dnvec(y);
        if (A) api->destroy_spmat(A);
        if (handle) api->destroy(handle);
    }
};

#define FL_CUSPARSE(h, call)                                                                      \
    do {                                                                                          \
        cusparseStatus_t st_ = (call);                                                            \
        if (st_ != CUSPARSE_STATUS_SUCCESS)                                                       \
            return fail(FL_ERR_CUDA, "cuSPARSE: %s failed: %s", #call, (h)->api->error_string(st_)); \
    } while (0)

extern "C" int fl_csc_spmv_naive(int m, int n, int nnz, const int *d_colptr, const int *d_rowidx,
                                 const double *d_val, const double *d_x, double *d_y, int accumulate,
                                 void *stream) {
    if (m < 0 || n < 0 || nnz < 0) return fail(FL_ERR_ARG, "csc_spmv_naive: negative size");
    if ((n && (!d_colptr || !d_x)) || (nnz && (!d_rowidx || !d_val)) || (m && !d_y))
        return fail(FL_ERR_ARG, "csc_spmv_naive: NULL array");
    const cudaStream_t s = (cudaStream_t)stream;
    if (!accumulate && m) FL_CUDA(cudaMemsetAsync(d_y, 0, (size_t)m * sizeof(double), s));
    if (n == 0) return FL_SUCCESS;
    k_csc_naive<<<32 * num_sms(), 64, 0, s>>>(n, d_colptr, d_rowidx, d_val, d_x, d_y);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

extern "C" int fl_cusparse_create(fl_cusparse_t *out, int m, int n, int nnz, const int *d_rowptr,
                                  const int *d_colidx, const double *d_val, int alg, void *stream) {
    clear_error();
    if (!out) return fail(FL_ERR_ARG, "cusparse_create: NULL handle pointer");
    *out = nullptr;
    if (m < 1 || n < 1 || nnz < 0 || !d_rowptr || (nnz && (!d_colidx || !d_val)))
        return fail(FL_ERR_ARG, "cusparse_create: bad matrix (m=%d n=%d nnz=%d)", m, n, nnz);
    if (alg < 0 || alg > 2) return fail(FL_ERR_ARG, "cusparse_create: algorithm %d", alg);
    const cudaStream_t s = (cudaStream_t)stream;
    std::unique_ptr<fl_cusparse> h(new (std::nothrow) fl_cusparse());
    if (!h) return fail(FL_ERR_ALLOC, "cusparse_create: host allocation failed");
    FL_TRY(cusparse_api(&h->api));
    h->m = m;
    h->n = n;
    h->alg = alg == 1 ? CUSPARSE_SPMV_CSR_ALG1 : alg == 2 ? CUSPARSE_SPMV_CSR_ALG2 : CUSPARSE_SPMV_ALG_DEFAULT;
    FL_CUSPARSE(h, h->api->create(&h->handle));
    FL_CUSPARSE(h, h->api->set_stream(h->handle, s));
    FL_CUSPARSE(h, h->api->create_csr(&h->A, m, n, nnz, (void *)d_rowptr, (void *)d_colidx, (void *)d_val,
                                      CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_64F));
    FL_TRY(h->xs.alloc(n, s));
    FL_TRY(h->ys.alloc(m, s));
    FL_CUDA(cudaMemsetAsync(h->xs.get(), 0, (size_t)n * sizeof(double), s));
    FL_CUSPARSE(h, h->api->create_dnvec(&h->x, n, h->xs.get(), CUDA_R_64F));
    FL_CUSPARSE(h, h->api->create_dnvec(&h->y, m, h->ys.get(), CUDA_R_64F));
    const double one = 1.0, zero = 0.0;
    size_t bytes = 0;
    FL_CUSPARSE(h, h->api->buffer_size(h->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, h->A, h->x, &zero, h->y,
                                       CUDA_R_64F, h->alg, &bytes));
    FL_TRY(h->buffer.alloc(std::max<size_t>(bytes, 1), s));
    FL_CUSPARSE(h, h->api->preprocess(h->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, h->A, h->x, &zero, h->y,
                                      CUDA_R_64F, h->alg, h->buffer.get()));
    FL_CUDA(cudaStreamSynchronize(s));
    *out = h.release();
    return FL_SUCCESS;
}

extern "C" int fl_cusparse_spmv(fl_cusparse_t h, const double *d_x, double *d_y, void *stream) {
    if (!h || !d_x || !d_y) return fail(FL_ERR_ARG, "cusparse_spmv: NULL argument");
    const double one = 1.0, zero = 0.0;
    FL_CUSPARSE(h, h->api->set_stream(h->handle, (cudaStream_t)stream));
    FL_CUSPARSE(h, h->api->dnvec_set(h->x, (void *)d_x));
    FL_CUSPARSE(h, h->api->dnvec_set(h->y, d_y));
    FL_CUSPARSE(h, h->api->spmv(h->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, h->A, h->x, &zero, h->y, CUDA_R_64F,
                                h->alg, h->buffer.get()));
    return FL_SUCCESS;
}

extern "C" int fl_cusparse_destroy(fl_cusparse_t h) {
    delete h;
    return FL_SUCCESS;
}

namespace {

// Host-buffer helper: uploads, runs `launch` reps times between events, y back.
template <typename F>
int host_timed(int m, int n, int nnz, const int *ptr, int nptr, const int *idx, const double *val, const double *x,
               double *y, int reps, double *mean_ms, F launch) {
    if (m < 0 || n < 0 || nnz < 0 || reps < 1 || !ptr || !x || !y || !mean_ms || (nnz && (!idx || !val)))
        return fail(FL_ERR_ARG, "comparator: bad arguments (m=%d n=%d nnz=%d reps=%d)", m, n, nnz, reps);
    const cudaStream_t s = 0;
    SyncAtExit drain{s};
    DevBuf<int> dp, di;
    DevBuf<double> dv, dx, dy;
    FL_TRY(dp.alloc(nptr, s));
    FL_TRY(di.alloc(std::max(nnz, 1), s));
    FL_TRY(dv.alloc(std::max(nnz, 1), s));
    FL_TRY(dx.alloc(std::max(n, 1), s));
    FL_TRY(dy.alloc(std::max(m, 1), s));
    FL_CUDA(cudaMemcpyAsync(dp.get(), ptr, (size_t)nptr * sizeof(int), cudaMemcpyHostToDevice, s));
    if (nnz) {
        FL_CUDA(cudaMemcpyAsync(di.get(), idx, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice, s));
        FL_CUDA(cudaMemcpyAsync(dv.get(), val, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    if (n) FL_CUDA(cudaMemcpyAsync(dx.get(), x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
    struct Ev {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Ev() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    FL_CUDA(cudaEventCreate(&ev.a));
    FL_CUDA(cudaEventCreate(&ev.b));
    const cudaEvent_t a = ev.a, b = ev.b;
    FL_TRY(launch(dp.get(), di.get(), dv.get(), dx.get(), dy.get()));  // untimed: first-call set-up
    double total = 0;
    for (int r = 0; r < reps; r++) {
        if (m) FL_CUDA(cudaMemsetAsync(dy.get(), 0, (size_t)m * sizeof(double), s));
        FL_CUDA(cudaEventRecord(a, s));
        FL_TRY(launch(dp.get(), di.get(), dv.get(), dx.get(), dy.get()));
        FL_CUDA(cudaEventRecord(b, s));
        FL_CUDA(cudaEventSynchronize(b));
        float t = 0;
        FL_CUDA(cudaEventElapsedTime(&t, a, b));
        total += t;
    }
    if (m) FL_CUDA(cudaMemcpy(y, dy.get(), (size_t)m * sizeof(double), cudaMemcpyDeviceToHost));
    *mean_ms = total / reps;
    return FL_SUCCESS;
}

}  // namespace

extern "C" int fl_csc_spmv_naive_host(int m, int n, int nnz, const int *csc_ptr, const int *csc_rowidx,
                                      const double *csc_val, const double *x, double *y, int reps,
                                      double *mean_ms) {
    clear_error();
    return host_timed(m, n, nnz, csc_ptr, n + 1, csc_rowidx, csc_val, x, y, reps, mean_ms,
                      [&](const int *p, const int *i, const double *v, const double *dx, double *dy) {
                          return fl_csc_spmv_naive(m, n, nnz, p, i, v, dx, dy, 1, nullptr);
                      });
}

extern "C" int fl_cusparse_spmv_host(int m, int n, int nnz, const int *csr_rowptr, const int *csr_colidx,
                                     const double *csr_val, const double *x, double *y, int reps,
                                     double *mean_ms) {
    clear_error();
    fl_cusparse_t h = nullptr;
    std::unique_ptr<fl_cusparse> guard;
    return host_timed(m, n, nnz, csr_rowptr, m + 1, csr_colidx, csr_val, x, y, reps, mean_ms,
                      [&](const int *p, const int *i, const double *v, const double *dx, double *dy) {
                          if (!h) {
                              FL_TRY(fl_cusparse_create(&h, m, n, nnz, p, i, v, 0, nullptr));
                              guard.reset(h);
                          }
                          return fl_cusparse_spmv(h, dx, dy, nullptr);
                      });
}

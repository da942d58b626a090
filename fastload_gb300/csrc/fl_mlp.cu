// fl_mlp.cu -- the tuner's network: an MLP in -> h1 -> h2 -> out (ReLU
// hidden layers, linear output), trained and evaluated on the GPU by the
// kernels below (forward, mean-squared-error loss and gradient, backward
// through both layers' weights and inputs, Adam).  The layers are a few
// thousand weights, so plain SIMT kernels (one thread per output element)
// are the right tool; tensor cores would idle.
#include "fl_internal.cuh"

#include <cmath>
#include <cstring>
#include <vector>

using namespace fl;

namespace {

// Y[b,o] = act(sum_i X[b,i] W[i,o] + bias[o])
__global__ void k_dense_fwd(const float *X, const float *W, const float *bias, float *Y, int B, int I, int O,
                            int relu) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < (long)B * O; t += (long)gridDim.x * blockDim.x) {
        const int b = (int)(t / O), o = (int)(t % O);
        float s = bias[o];
        for (int i = 0; i < I; i++) s = fmaf(X[(long)b * I + i], W[(long)i * O + o], s);
        Y[t] = relu ? fmaxf(s, 0.0f) : s;
    }
}

// masked MSE: loss = sum M (Y - T)^2 / sum M;  dY = 2 M (Y - T) / sum M
__global__ void k_mse(const float *Y, const float *T, const float *M, long n, float inv_count, float *dY,
                      float *loss) {
    float acc = 0.0f;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const float d = (Y[t] - T[t]) * M[t];
        dY[t] = 2.0f * d * inv_count;
        acc += d * d * inv_count;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// dX[b,i] = (sum_o dY[b,o] W[i,o]) * [H[b,i] > 0]   (H = the ReLU output fed forward)
__global__ void k_dense_bwd_in(const float *dY, const float *W, const float *H, float *dX, int B, int I, int O) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < (long)B * I; t += (long)gridDim.x * blockDim.x) {
        const int b = (int)(t / I), i = (int)(t % I);
        float s = 0.0f;
        for (int o = 0; o < O; o++) s = fmaf(dY[(long)b * O + o], W[(long)i * O + o], s);
        dX[t] = H[t] > 0.0f ? s : 0.0f;
    }
}

// dW[i,o] = sum_b X[b,i] dY[b,o];  dbias[o] = sum_b dY[b,o]
__global__ void k_dense_bwd_w(const float *X, const float *dY, float *dW, float *db, int B, int I, int O) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < (long)(I + 1) * O;
         t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t / O), o = (int)(t % O);
        float s = 0.0f;
        if (i < I)
            for (int b = 0; b < B; b++) s = fmaf(X[(long)b * I + i], dY[(long)b * O + o], s);
        else
            for (int b = 0; b < B; b++) s += dY[(long)b * O + o];
        if (i < I) dW[t] = s;
        else db[o] = s;
    }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const float gt = g[t];
        m[t] = b1 * m[t] + (1 - b1) * gt;
        v[t] = b2 * v[t] + (1 - b2) * gt * gt;
        p[t] -= lr * (m[t] / c1) / (sqrtf(v[t] / c2) + eps);
    }
}

int gsz(long n) { return (int)std::min<long>(std::max<long>((n + 255) / 256, 1), 1024); }

}  // namespace

struct fl_mlp {
    int I = 0, H1 = 0, H2 = 0, O = 0;
    long np = 0;  // parameter count: W1 b1 W2 b2 W3 b3, contiguous
    DevBuf<float> p, g, m, v;
    int t = 0;
    long off[6];
    float *W(int k) { return p.get() + off[k]; }
    float *G(int k) { return g.get() + off[k]; }
};

namespace {

struct Work {
    DevBuf<float> X, T, M, h1, h2, y, dy, dh2, dh1, loss;
    int B = 0;
    int alloc(const fl_mlp &n, int B_, cudaStream_t s) {
        B = B_;
        FL_TRY(X.alloc((size_t)B * n.I, s));
        FL_TRY(T.alloc((size_t)B * n.O, s));
        FL_TRY(M.alloc((size_t)B * n.O, s));
        FL_TRY(h1.alloc((size_t)B * n.H1, s));
        FL_TRY(h2.alloc((size_t)B * n.H2, s));
        FL_TRY(y.alloc((size_t)B * n.O, s));
        FL_TRY(dy.alloc((size_t)B * n.O, s));
        FL_TRY(dh2.alloc((size_t)B * n.H2, s));
        FL_TRY(dh1.alloc((size_t)B * n.H1, s));
        FL_TRY(loss.alloc(1, s));
        return FL_SUCCESS;
    }
};

int forward(fl_mlp &n, Work &w, cudaStream_t s) {
    const int B = w.B;
    k_dense_fwd<<<gsz((long)B * n.H1), 256, 0, s>>>(w.X.get(), n.W(0), n.W(1), w.h1.get(), B, n.I, n.H1, 1);
    k_dense_fwd<<<gsz((long)B * n.H2), 256, 0, s>>>(w.h1.get(), n.W(2), n.W(3), w.h2.get(), B, n.H1, n.H2, 1);
    k_dense_fwd<<<gsz((long)B * n.O), 256, 0, s>>>(w.h2.get(), n.W(4), n.W(5), w.y.get(), B, n.H2, n.O, 0);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

int backward(fl_mlp &n, Work &w, float inv_count, cudaStream_t s) {
    const int B = w.B;
    FL_CUDA(cudaMemsetAsync(w.loss.get(), 0, sizeof(float), s));
    k_mse<<<gsz((long)B * n.O), 256, 0, s>>>(w.y.get(), w.T.get(), w.M.get(), (long)B * n.O, inv_count, w.dy.get(),
                                             w.loss.get());
    k_dense_bwd_w<<<gsz((long)(n.H2 + 1) * n.O), 256, 0, s>>>(w.h2.get(), w.dy.get(), n.G(4), n.G(5), B, n.H2, n.O);
    k_dense_bwd_in<<<gsz((long)B * n.H2), 256, 0, s>>>(w.dy.get(), n.W(4), w.h2.get(), w.dh2.get(), B, n.H2, n.O);
    k_dense_bwd_w<<<gsz((long)(n.H1 + 1) * n.H2), 256, 0, s>>>(w.h1.get(), w.dh2.get(), n.G(2), n.G(3), B, n.H1,
                                                               n.H2);
    k_dense_bwd_in<<<gsz((long)B * n.H1), 256, 0, s>>>(w.dh2.get(), n.W(2), w.h1.get(), w.dh1.get(), B, n.H1, n.H2);
    k_dense_bwd_w<<<gsz((long)(n.I + 1) * n.H1), 256, 0, s>>>(w.X.get(), w.dh1.get(), n.G(0), n.G(1), B, n.I, n.H1);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

int upload_batch(fl_mlp &n, Work &w, const float *X, const float *T, const float *M, int B, cudaStream_t s,
                 float *inv_count) {
    FL_TRY(w.alloc(n, B, s));
    FL_CUDA(cudaMemcpyAsync(w.X.get(), X, (size_t)B * n.I * 4, cudaMemcpyHostToDevice, s));
    if (T) {
        FL_CUDA(cudaMemcpyAsync(w.T.get(), T, (size_t)B * n.O * 4, cudaMemcpyHostToDevice, s));
        double cnt = 0;
        if (M) {
            FL_CUDA(cudaMemcpyAsync(w.M.get(), M, (size_t)B * n.O * 4, cudaMemcpyHostToDevice, s));
            for (long i = 0; i < (long)B * n.O; i++) cnt += M[i];
        } else {
            std::vector<float> ones((size_t)B * n.O, 1.0f);
            FL_CUDA(cudaMemcpyAsync(w.M.get(), ones.data(), ones.size() * 4, cudaMemcpyHostToDevice, s));
            FL_CUDA(cudaStreamSynchronize(s));
            cnt = (double)B * n.O;
        }
        *inv_count = cnt > 0 ? (float)(1.0 / cnt) : 0.0f;
    }
    return FL_SUCCESS;
}

}  // namespace

extern "C" {

int fl_mlp_create(fl_mlp_t *out, int in, int h1, int h2, int outn, unsigned long long seed) {
    clear_error();
    if (!out || in <= 0 || h1 <= 0 || h2 <= 0 || outn <= 0) return fail(FL_ERR_ARG, "mlp_create: bad sizes");
    *out = nullptr;
    std::unique_ptr<fl_mlp> n(new (std::nothrow) fl_mlp());
    if (!n) return fail(FL_ERR_ALLOC, "mlp_create: host allocation failed");
    n->I = in;
    n->H1 = h1;
    n->H2 = h2;
    n->O = outn;
    const long sizes[6] = {(long)in * h1, h1, (long)h1 * h2, h2, (long)h2 * outn, outn};
    long o = 0;
    for (int k = 0; k < 6; k++) {
        n->off[k] = o;
        o += sizes[k];
    }
    n->np = o;
    cudaStream_t s = 0;
    FL_TRY(n->p.alloc(o, s));
    FL_TRY(n->g.alloc(o, s));
    FL_TRY(n->m.alloc(o, s));
    FL_TRY(n->v.alloc(o, s));
    FL_CUDA(cudaMemsetAsync(n->m.get(), 0, o * 4, s));
    FL_CUDA(cudaMemsetAsync(n->v.get(), 0, o * 4, s));
    // He-uniform weights from a splitmix64 stream, zero biases
    std::vector<float> h((size_t)o, 0.0f);
    unsigned long long z = seed;
    auto next = [&]() {
        z += 0x9e3779b97f4a7c15ULL;
        unsigned long long x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        x ^= x >> 31;
        return (double)(x >> 11) / 9007199254740992.0;
    };
    const int fan[3] = {in, h1, h2};
    for (int l = 0; l < 3; l++) {
        const double lim = std::sqrt(6.0 / fan[l]);
        for (long i = 0; i < sizes[2 * l]; i++) h[n->off[2 * l] + i] = (float)((2 * next() - 1) * lim);
    }
    FL_CUDA(cudaMemcpyAsync(n->p.get(), h.data(), o * 4, cudaMemcpyHostToDevice, s));
    FL_CUDA(cudaStreamSynchronize(s));
    *out = n.release();
    return FL_SUCCESS;
}

long fl_mlp_num_params(fl_mlp_t n) { return n ? n->np : 0; }

int fl_mlp_get_params(fl_mlp_t n, float *out) {
    clear_error();
    if (!n || !out) return fail(FL_ERR_ARG, "mlp_get_params: NULL argument");
    FL_CUDA(cudaMemcpy(out, n->p.get(), n->np * 4, cudaMemcpyDeviceToHost));
    return FL_SUCCESS;
}

int fl_mlp_set_params(fl_mlp_t n, const float *in) {
    clear_error();
    if (!n || !in) return fail(FL_ERR_ARG, "mlp_set_params: NULL argument");
    FL_CUDA(cudaMemcpy(n->p.get(), in, n->np * 4, cudaMemcpyHostToDevice));
    return FL_SUCCESS;
}

int fl_mlp_forward(fl_mlp_t n, const float *X, int B, float *Y) {
    clear_error();
    if (!n || !X || !Y || B <= 0) return fail(FL_ERR_ARG, "mlp_forward: bad arguments");
    cudaStream_t s = 0;
    Work w;
    float ic = 0;
    FL_TRY(upload_batch(*n, w, X, nullptr, nullptr, B, s, &ic));
    FL_TRY(forward(*n, w, s));
    FL_CUDA(cudaMemcpyAsync(Y, w.y.get(), (size_t)B * n->O * 4, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

int fl_mlp_grad(fl_mlp_t n, const float *X, const float *T, const float *M, int B, float *loss, float *grad) {
    clear_error();
    if (!n || !X || !T || B <= 0) return fail(FL_ERR_ARG, "mlp_grad: bad arguments");
    cudaStream_t s = 0;
    Work w;
    float ic = 0;
    FL_TRY(upload_batch(*n, w, X, T, M, B, s, &ic));
    FL_TRY(forward(*n, w, s));
    FL_TRY(backward(*n, w, ic, s));
    if (loss) FL_CUDA(cudaMemcpyAsync(loss, w.loss.get(), 4, cudaMemcpyDeviceToHost, s));
    if (grad) FL_CUDA(cudaMemcpyAsync(grad, n->g.get(), n->np * 4, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

int fl_mlp_train(fl_mlp_t n, const float *X, const float *T, const float *M, int B, int epochs, float lr,
                 float *losses) {
    clear_error();
    if (!n || !X || !T || B <= 0 || epochs < 0) return fail(FL_ERR_ARG, "mlp_train: bad arguments");
    cudaStream_t s = 0;
    Work w;
    float ic = 0;
    FL_TRY(upload_batch(*n, w, X, T, M, B, s, &ic));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; e++) {
        FL_TRY(forward(*n, w, s));
        FL_TRY(backward(*n, w, ic, s));
        n->t++;
        const float c1 = 1.0f - std::pow(b1, (float)n->t), c2 = 1.0f - std::pow(b2, (float)n->t);
        k_adam<<<gsz(n->np), 256, 0, s>>>(n->p.get(), n->g.get(), n->m.get(), n->v.get(), n->np, lr, b1, b2, eps, c1,
                                          c2);
        FL_CUDA(cudaGetLastError());
        if (losses) FL_CUDA(cudaMemcpyAsync(losses + e, w.loss.get(), 4, cudaMemcpyDeviceToHost, s));
    }
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

int fl_mlp_destroy(fl_mlp_t n) {
    if (!n) return FL_SUCCESS;
    cudaDeviceSynchronize();
    delete n;
    return FL_SUCCESS;
}

}  // extern "C"

// fl_gen.cu -- synthetic CSC matrices generated on the GPU (the tuner's
// training families), and the per-matrix feature extractor.
//
// Generation: the caller fixes each column's degree (colptr); one warp per
// column draws that many rows inside the family's row window in ascending
// order -- ascending uniforms from normalised prefix sums of exponential
// spacings (the order statistics of uniforms), mapped through the family's
// monotone row map -- and a uniform value in [-1, 1).  A counter-based hash
// of (seed, column, index) makes every matrix reproducible.  Rows may repeat
// when a column's degree approaches its window; a repeated entry is a valid
// CSC entry (the SpMV adds both).
#include "fl_internal.cuh"

#include <algorithm>
#include <cmath>

namespace fl {

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// uniform in (0, 1]
__device__ __forceinline__ double u01(unsigned long long seed, unsigned long long a, unsigned long long b) {
    const unsigned long long h = mix64(seed ^ mix64(a * 0x100000001b3ULL + b));
    return ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

constexpr unsigned FM = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FM, v, o);
    return v;
}
__device__ __forceinline__ double warp_incl(double v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(FM, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// family: 0 uniform rows, 1 uniform rows (Zipf degrees set by the caller),
// 2 banded (window of width p centred on the diagonal), 3 block-diagonal
// (blocks of p rows/columns), 4 row-skewed (row = m * u^p).
__global__ void k_gen_fill(int family, int m, int n, const int *colptr, int *rowidx, double *val, double p,
                           unsigned long long seed) {
    const int lane = threadIdx.x & 31;
    const long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long c = gw; c < n; c += nw) {
        const int beg = colptr[c], d = colptr[c + 1] - beg;
        if (d <= 0) continue;
        long lo = 0, hi = m;
        if (family == 2) {
            const long centre = (long)((double)c * m / n);
            const long half = (long)(p / 2);
            lo = std::max(0L, centre - half);
            hi = std::min((long)m, centre + half + 1);
        } else if (family == 3) {
            const long b = (long)p;
            const long blk = (long)((double)c * m / n) / b;
            lo = blk * b;
            hi = std::min((long)m, lo + b);
        }
        if (hi <= lo) { lo = 0; hi = m; }
        const double W = (double)(hi - lo);
        // total of d+1 exponential spacings
        double s = 0;
        for (int k = lane; k <= d; k += 32) s += -log(u01(seed, (unsigned long long)c, (unsigned long long)k));
        const double S = warp_sum(s);
        double carry = 0;
        for (int k0 = 0; k0 < d; k0 += 32) {
            const int k = k0 + lane;
            const double e = k < d ? -log(u01(seed, (unsigned long long)c, (unsigned long long)k)) : 0.0;
            const double pre = carry + warp_incl(e, lane);  // spacings 0..k
            carry = __shfl_sync(FM, pre, 31);
            if (k < d) {
                double u = pre / S;  // ascending in (0, 1)
                if (family == 4) u = pow(u, p);
                long r = lo + (long)(u * W);
                if (r >= hi) r = hi - 1;
                rowidx[beg + k] = (int)r;
                val[beg + k] = 2.0 * u01(seed ^ 0xabcdefULL, (unsigned long long)c, (unsigned long long)k) - 1.0;
            }
        }
    }
}

int grid_g(long n, int threads) {
    long b = (n + threads - 1) / threads;
    long cap = (long)num_sms() * 16;
    return (int)std::max<long>(1, std::min(b, cap));
}

// ------------------------------------------------------------ features --
// Per-column degree statistics from the sorted counts, per-row counts and
// the normalised distance of each nonzero from the diagonal.
__global__ void k_feat_cols(const int *sortnnz, int n, double *acc, int *hist) {
    double s1 = 0, s2 = 0, s3 = 0;
    int mx = 0;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        const double d = sortnnz[c];
        s1 += d;
        s2 += d * d;
        s3 += d * d * d;
        mx = max(mx, sortnnz[c]);
        const int b = sortnnz[c] > 0 ? min(10, 31 - __clz(sortnnz[c])) : -1;
        if (b >= 0) atomicAdd(hist + b, 1);
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(FM, mx, o));
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc + 0, s1);
        atomicAdd(acc + 1, s2);
        atomicAdd(acc + 2, s3);
        atomicMax(hist + 11, mx);
    }
}

__global__ void k_feat_nnz(const int *row, long nnz, const RegionDesc *regions, const ItemDesc *items, int nitems,
                           int m, int n, const int *perm, int *rowcnt, double *acc) {
    // one warp per work item: the distance |row/m - col/n| of every nonzero
    const int lane = threadIdx.x & 31;
    const long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    double band = 0;
    for (long it = gw; it < nitems; it += nw) {
        const ItemDesc d = items[it];
        const RegionDesc rg = regions[d.region];
        for (int e = d.begin + lane; e < d.end; e += 32) {
            const int q = e - rg.start;
            const int col = rg.full ? rg.col_base + 32 * (q / rg.div) + (q & 31) : rg.col_base + q % rg.div;
            const int r = row[e];
            atomicAdd(rowcnt + r, 1);
            band += fabs((double)r / m - (double)perm[col] / n);
        }
    }
    band = warp_sum(band);
    if (lane == 0) atomicAdd(acc + 3, band);
}

__global__ void k_feat_rows(const int *rowcnt, int m, double *acc) {
    double s1 = 0, s2 = 0;
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < m; r += (long)gridDim.x * blockDim.x) {
        const double d = rowcnt[r];
        s1 += d;
        s2 += d * d;
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc + 4, s1);
        atomicAdd(acc + 5, s2);
    }
}

}  // namespace

int plan_features(const Layout &L, float *out, cudaStream_t s) {
    const int m = L.m, n = L.n;
    const long nnz = L.nnz;
    DevBuf<double> acc;
    DevBuf<int> hist, rowcnt, scol;
    FL_TRY(acc.alloc(8, s));
    FL_TRY(hist.alloc(12, s));
    FL_TRY(rowcnt.alloc(std::max(m, 1), s));
    FL_TRY(scol.alloc((size_t)n + 1, s));
    FL_CUDA(cudaMemsetAsync(acc.get(), 0, 8 * sizeof(double), s));
    FL_CUDA(cudaMemsetAsync(hist.get(), 0, 12 * sizeof(int), s));
    FL_CUDA(cudaMemsetAsync(rowcnt.get(), 0, std::max(m, 1) * sizeof(int), s));
    if (n) {
        k_feat_cols<<<grid_g(n, 256), 256, 0, s>>>(L.sortnnz.get(), n, acc.get(), hist.get());
        FL_CUDA(cudaGetLastError());
    }
    if (L.regions.nitems) {
        k_feat_nnz<<<grid_g((long)L.regions.nitems * 32, 256), 256, 0, s>>>(
            L.row.get(), nnz, L.regions.region.get(), L.regions.item.get(), L.regions.nitems, m, n, L.perm.get(),
            rowcnt.get(), acc.get());
        FL_CUDA(cudaGetLastError());
    }
    if (m) {
        k_feat_rows<<<grid_g(m, 256), 256, 0, s>>>(rowcnt.get(), m, acc.get());
        FL_CUDA(cudaGetLastError());
    }
    FL_TRY(scan_exclusive(L.sortnnz.get(), scol.get(), n, scol.get() + n, s));
    double a[8];
    int h[12];
    FL_CUDA(cudaMemcpyAsync(a, acc.get(), sizeof a, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaMemcpyAsync(h, hist.get(), sizeof h, cudaMemcpyDeviceToHost, s));
    const int bands[3] = {2048, 8192, 24576};
    int tops[3];
    for (int i = 0; i < 3; i++) {
        const int b = std::min(bands[i], n);
        FL_CUDA(cudaMemcpyAsync(tops + i, scol.get() + (n - b), sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    FL_CUDA(cudaStreamSynchronize(s));
    const double N = std::max(n, 1), M = std::max(m, 1), Z = std::max<double>(nnz, 1);
    const double mean = a[0] / N, var = std::max(0.0, a[1] / N - mean * mean), sd = std::sqrt(var);
    const double m3 = a[2] / N - 3 * mean * a[1] / N + 2 * mean * mean * mean;
    const double rmean = a[4] / M, rvar = std::max(0.0, a[5] / M - rmean * rmean);
    int f = 0;
    out[f++] = (float)std::log10(N);
    out[f++] = (float)std::log10(M);
    out[f++] = (float)std::log10(Z);
    out[f++] = (float)std::log10(mean + 1e-9 + 1.0);
    out[f++] = (float)(mean > 0 ? sd / mean : 0.0);                       // column-degree CV
    out[f++] = (float)(sd > 0 ? std::cbrt(m3) / sd : 0.0);                // column-degree skew (cube root scaled)
    out[f++] = (float)std::log10((double)h[11] + 1.0);                   // max column degree
    for (int b = 0; b < 11; b++) out[f++] = (float)(h[b] / N);           // log2 degree histogram
    for (int i = 0; i < 3; i++) out[f++] = (float)((double)(nnz - tops[i]) / Z);  // nnz share of densest columns
    out[f++] = (float)(a[3] / Z);                                        // mean |row/m - col/n|
    out[f++] = (float)(rmean > 0 ? std::sqrt(rvar) / rmean : 0.0);       // row-degree CV
    return FL_SUCCESS;  // f == 23 here; the caller adds the value-type flag
}

}  // namespace fl

using namespace fl;

extern "C" {

int fl_gen_fill(int family, int m, int n, const int *d_colptr, int *d_rowidx, double *d_val, double param,
                unsigned long long seed, void *stream) {
    clear_error();
    if (family < 0 || family > 4) return fail(FL_ERR_ARG, "gen_fill: family %d", family);
    if (m <= 0 || n < 0 || !d_colptr || (n && (!d_rowidx || !d_val))) return fail(FL_ERR_ARG, "gen_fill: bad arguments");
    if ((family == 2 || family == 3) && param < 1) return fail(FL_ERR_ARG, "gen_fill: window %g", param);
    if (n == 0) return FL_SUCCESS;
    k_gen_fill<<<grid_g((long)n * 32, 256), 256, 0, (cudaStream_t)stream>>>(family, m, n, d_colptr, d_rowidx, d_val,
                                                                            param, seed);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

int fl_plan_features(fl_plan_t plan, int value_type, float *out) {
    clear_error();
    if (!plan || !out) return fail(FL_ERR_ARG, "plan_features: NULL argument");
    FL_TRY(plan_features(plan->L, out, 0));
    out[23] = value_type == FL_VALUES_F64 ? 0.0f : 1.0f;
    return FL_SUCCESS;
}

}  // extern "C"

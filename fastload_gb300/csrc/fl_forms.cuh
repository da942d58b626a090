// fl_forms.cuh -- generic SpMV kernel for the storage / right-hand-side forms.
//
// One template covers every form beside the plain FP64 drop-in kernels:
//   V  value storage: double (FP64), float (FP32) or bf16x2_t (a BF16 hi+lo
//      split: v ~ float(hi) + float(lo), hi = bf16(v), lo = bf16(v - hi));
//   K  right-hand sides: x and y row-interleaved (x[col*K + r], y[row*K + r]);
//   XS x of the heavy band read from shared memory (staged by a TMA bulk copy)
//      or from global memory (bands wider than shared memory);
//   C16 heavy-band column indices stored as 16 bits (band <= 65535) or 32;
//   Y  y type (double, or float for the FP32-accumulating batched form).
// Products and per-row sums are computed in FP32 for the FP32/BF16 forms and
// in FP64 for the FP64 form; y is accumulated in Y.  The work is the bucketed
// split of fl_bucket.cu: light columns in the FastLoad tile stream with one
// atomic per run (K = 1) or per (nonzero, rhs) (K > 1), the heavy band in
// 32-row slices with one lane per row.  When the band holds every column
// (no light part) each row is owned by one lane and y is updated without
// atomics.
#pragma once

#include "fl_stream.cuh"

#include <algorithm>

namespace fl {

struct bf16x2_t {
    uint32_t u;
};

constexpr int FM_THREADS = 1024;
constexpr long FM_WAIT_LIMIT = 1L << 20;
constexpr int FM_SMEM_MAX = 196608;  // dynamic shared memory budget of the form kernels

__device__ __forceinline__ float bf16x2_decode(uint32_t u) {
    return __uint_as_float(u << 16) + __uint_as_float(u & 0xffff0000u);
}

template <typename V>
struct VT;

template <>
struct VT<double> {
    using X = double;
    using A = double;
    static __device__ __forceinline__ void load4(const double *p, A v[4]) {
        double2 a, b;
        asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(a.x), "=d"(a.y) : "l"(p));
        asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(b.x), "=d"(b.y) : "l"(p + 2));
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ A stream1(const double *p) {
        double r;
        asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ A cached1(const double *p) { return __ldg(p); }
};

template <>
struct VT<float> {
    using X = float;
    using A = float;
    static __device__ __forceinline__ void load4(const float *p, A v[4]) {
        asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
            : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]) : "l"(p));
    }
    static __device__ __forceinline__ A stream1(const float *p) {
        float r;
        asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(r) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ A cached1(const float *p) { return __ldg(p); }
};

template <>
struct VT<bf16x2_t> {
    using X = float;
    using A = float;
    static __device__ __forceinline__ void load4(const bf16x2_t *p, A v[4]) {
        uint32_t u[4];
        asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
            : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]) : "l"(p));
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = bf16x2_decode(u[k]);
    }
    static __device__ __forceinline__ A stream1(const bf16x2_t *p) {
        uint32_t u;
        asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(u) : "l"(p));
        return bf16x2_decode(u);
    }
    static __device__ __forceinline__ A cached1(const bf16x2_t *p) {
        return bf16x2_decode(__ldg((const unsigned *)p));
    }
};

template <typename V, typename Y>
struct FormArgs {
    using X = typename VT<V>::X;
    // light columns: FastLoad stream
    const ItemDesc *items;
    const RegionDesc *regions;
    const int *row;
    const V *val;
    int nitems;
    // heavy band
    int H0, nh, nslices, bulk, atomic_heavy;
    const int *slice_ptr, *hrow, *hlen;
    const V *hval;
    const uint16_t *hcol16;
    const int *hcol32;
    const X *xs;
    Y *y;
    int *err;
    int *next;
};

// Sorted column of nonzero e of a region (see fl_stream.cuh).
__device__ __forceinline__ int region_col(int e, const RegionDesc &rg) {
    const int q = e - rg.start;
    return rg.full ? rg.col_base + 32 * (q / rg.div) + (q & 31) : rg.col_base + q % rg.div;
}

// K = 1 light item: four nonzeros per lane, run merging as in process4_f64,
// products and run sums in A, one atomic per run into Y.
template <typename V, typename Y>
__device__ __forceinline__ void light_item_k1(const ItemDesc &d, const RegionDesc *__restrict__ regions,
                                              const int *__restrict__ row, const V *__restrict__ val,
                                              const typename VT<V>::X *__restrict__ xs, Y *__restrict__ y,
                                              int lane) {
    using A = typename VT<V>::A;
    const RegionDesc rg = regions[d.region];
    for (int e = d.begin & ~3; e < d.end; e += 128) {
        const int eb = e + 4 * lane;
        const int4 rr = ld_stream_i4(row + eb);
        A v[4];
        VT<V>::load4(val + eb, v);
        int r[4] = {rr.x, rr.y, rr.z, rr.w};
        A p[4];
        const int qa = eb - rg.start;
        const int qb = qa > 0 ? qa : 0;
        const int c0 = qb / rg.div;
        const int r0 = qb - c0 * rg.div;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int ek = eb + k;
            const bool valid = ek >= d.begin && ek < d.end;
            const int delta = qa + k - qb;
            int col;
            if (rg.full) {
                col = rg.col_base + 32 * (c0 + (r0 + delta >= rg.div ? 1 : 0)) + ((qa + k) & 31);
            } else {
                int t = r0 + delta;
#pragma unroll
                for (int w = 0; w < 3; w++)
                    if (t >= rg.div) t -= rg.div;
                col = rg.col_base + t;
            }
            if (valid) {
                p[k] = v[k] * (A)__ldg(xs + col);
            } else {
                p[k] = (A)0;
                r[k] = -1;
            }
        }
        const bool b1 = r[1] != r[0], b2 = r[2] != r[1], b3 = r[3] != r[2];
        const int prev_rl = __shfl_up_sync(FULLM, r[3], 1);
        const int next_rf = __shfl_down_sync(FULLM, r[0], 1);
        const bool cont = lane > 0 && r[0] >= 0 && prev_rl == r[0];
        const bool cont_next = lane < 31 && r[3] >= 0 && next_rf == r[3];
        const bool merge = (!b1 && r[0] >= 0) || (!b2 && r[1] >= 0) || (!b3 && r[2] >= 0) || cont;
        if (!__any_sync(FULLM, merge)) {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (r[k] >= 0) atomicAdd(y + r[k], (Y)p[k]);
            continue;
        }
        A T = p[3];
        if (!b3) {
            T += p[2];
            if (!b2) {
                T += p[1];
                if (!b1) T += p[0];
            }
        }
        const bool full_lane = !b1 && !b2 && !b3;
        A S = T;
        int h = (full_lane && cont) ? 0 : 1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const A Sn = __shfl_up_sync(FULLM, S, o);
            const int hn = __shfl_up_sync(FULLM, h, o);
            if (lane >= o && !h) {
                S += Sn;
                h = hn;
            }
        }
        const A Sp = __shfl_up_sync(FULLM, S, 1);
        const A C = cont ? Sp : (A)0;
        A acc = p[0];
        bool lead = true;
        const bool brk[4] = {false, b1, b2, b3};
#pragma unroll
        for (int k = 1; k < 4; k++) {
            if (brk[k]) {
                if (r[k - 1] >= 0) atomicAdd(y + r[k - 1], (Y)(lead ? acc + C : acc));
                acc = p[k];
                lead = false;
            } else {
                acc += p[k];
            }
        }
        if (!cont_next && r[3] >= 0) atomicAdd(y + r[3], (Y)S);
    }
}

// K > 1 light item: K lanes per nonzero, lane (g, r) adds the rhs-r product
// of nonzero e+g; a warp instruction's atomics cover 32/K rows x K
// consecutive y entries.
template <typename V, int K, typename Y>
__device__ __forceinline__ void light_item_kn(const ItemDesc &d, const RegionDesc *__restrict__ regions,
                                              const int *__restrict__ row, const V *__restrict__ val,
                                              const typename VT<V>::X *__restrict__ xs, Y *__restrict__ y,
                                              int lane) {
    using A = typename VT<V>::A;
    constexpr int EPR = 32 / K;
    const RegionDesc rg = regions[d.region];
    const int g = lane / K, rr = lane % K;
    for (int e = d.begin; e < d.end; e += EPR) {
        const int el = e + g;
        if (el < d.end) {
            const int col = region_col(el, rg);
            const A v = VT<V>::cached1(val + el);
            const int rw = __ldg(row + el);
            const A p = v * (A)__ldg(xs + (size_t)col * K + rr);
            atomicAdd(y + (size_t)rw * K + rr, (Y)p);
        }
    }
}

// K consecutive x values of one column: from shared memory (XS) or through
// the read-only cache; 16-byte vector loads when K*sizeof(X) allows.
template <typename X, int K, bool XS>
__device__ __forceinline__ void load_xk(const X *p, X out[K]) {
    if constexpr (K % 4 == 0 && sizeof(X) == 4) {
#pragma unroll
        for (int q = 0; q < K; q += 4) {
            float4 t;
            if constexpr (XS) t = *(const float4 *)(p + q);
            else t = __ldg((const float4 *)(p + q));
            out[q] = t.x; out[q + 1] = t.y; out[q + 2] = t.z; out[q + 3] = t.w;
        }
    } else if constexpr (K % 2 == 0 && sizeof(X) == 8) {
#pragma unroll
        for (int q = 0; q < K; q += 2) {
            double2 t;
            if constexpr (XS) t = *(const double2 *)(p + q);
            else t = __ldg((const double2 *)(p + q));
            out[q] = t.x; out[q + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int q = 0; q < K; q++) {
            if constexpr (XS) out[q] = p[q];
            else out[q] = __ldg(p + q);
        }
    }
}

// Heavy slice: lane owns one row, K sums in A.
template <typename V, int K, bool XS, bool C16, typename Y>
__device__ __forceinline__ void heavy_slice(const FormArgs<V, Y> &a, int sl, const typename VT<V>::X *xsrc, int lane) {
    using A = typename VT<V>::A;
    using X = typename VT<V>::X;
    const int base = __ldg(a.slice_ptr + sl);
    const int w = (__ldg(a.slice_ptr + sl + 1) - base) >> 5;
    const int r = __ldg(a.hrow + 32 * sl + lane), len = __ldg(a.hlen + 32 * sl + lane);
    A acc[K];
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = (A)0;
    const V *vp = a.hval + base + lane;
    constexpr int UNR = K == 1 ? 4 : 2;
    int j = 0;
    for (; j + UNR <= w; j += UNR) {
        A v[UNR];
        int c[UNR];
#pragma unroll
        for (int k = 0; k < UNR; k++) {
            if (j + k < len) {
                v[k] = VT<V>::stream1(vp + 32 * (j + k));
                if constexpr (C16) c[k] = (int)__ldg(a.hcol16 + base + 32 * (j + k) + lane);
                else c[k] = __ldg(a.hcol32 + base + 32 * (j + k) + lane);
            }
        }
#pragma unroll
        for (int k = 0; k < UNR; k++) {
            if (j + k < len) {
                X xv[K];
                load_xk<X, K, XS>(xsrc + (size_t)c[k] * K, xv);
#pragma unroll
                for (int q = 0; q < K; q++) acc[q] = fma(v[k], (A)xv[q], acc[q]);
            }
        }
    }
    for (; j < w; j++) {
        if (j < len) {
            const A v = VT<V>::stream1(vp + 32 * j);
            int c;
            if constexpr (C16) c = (int)__ldg(a.hcol16 + base + 32 * j + lane);
            else c = __ldg(a.hcol32 + base + 32 * j + lane);
            X xv[K];
            load_xk<X, K, XS>(xsrc + (size_t)c * K, xv);
#pragma unroll
            for (int q = 0; q < K; q++) acc[q] = fma(v, (A)xv[q], acc[q]);
        }
    }
    if (len > 0) {
        Y *yr = a.y + (size_t)r * K;
        if (a.atomic_heavy) {
#pragma unroll
            for (int q = 0; q < K; q++) atomicAdd(yr + q, (Y)acc[q]);
        } else {
#pragma unroll
            for (int q = 0; q < K; q++) yr[q] += (Y)acc[q];
        }
    }
}

template <typename V, int K, bool XS, bool C16, typename Y>
__global__ void __launch_bounds__(FM_THREADS, 1) k_spmv_form(const FormArgs<V, Y> a) {
    using X = typename VT<V>::X;
    extern __shared__ __align__(128) unsigned char fm_smem[];
    X *xh = (X *)fm_smem;
    __shared__ __align__(8) unsigned long long mbar;
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&mbar);
    const bool use_band = a.nh > 0 && a.nslices > 0;
    if (XS && use_band) {
        const uint32_t bytes = (uint32_t)a.nh * K * (uint32_t)sizeof(X);
        if (a.bulk) {
            if (tid == 0) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            }
            __syncthreads();
            if (tid == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                             : "memory");
                const char *src = (const char *)(a.xs + (size_t)a.H0 * K);
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(xh);
                for (uint32_t off = 0; off < bytes; off += 32768u) {
                    const uint32_t sz = min(32768u, bytes - off);
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                            "r"(dst + off),
                        "l"(src + off), "r"(sz), "r"(bar)
                        : "memory");
                }
            }
        } else {
            const int cnt = a.nh * K;
            for (int i = tid; i < cnt; i += blockDim.x) xh[i] = __ldg(a.xs + (size_t)a.H0 * K + i);
            __syncthreads();
        }
    }
    const X *xsrc = XS ? (const X *)xh : a.xs + (size_t)a.H0 * K;
    const int total = a.nitems + (use_band ? a.nslices : 0);
    bool staged = !(XS && use_band && a.bulk);
    for (;;) {
        int u = 0;
        if (lane == 0) u = atomicAdd(a.next, 1);
        u = __shfl_sync(FULLM, u, 0);
        if (u >= total) break;
        if (u < a.nitems) {
            if constexpr (K == 1) light_item_k1<V, Y>(a.items[u], a.regions, a.row, a.val, a.xs, a.y, lane);
            else light_item_kn<V, K, Y>(a.items[u], a.regions, a.row, a.val, a.xs, a.y, lane);
            continue;
        }
        if (!staged) {
            bool ok = false;
            for (long i = 0; i < FM_WAIT_LIMIT && !ok; i++) {
                uint32_t done;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(done)
                    : "r"(bar)
                    : "memory");
                ok = done != 0;
            }
            if (!ok) {
                if (lane == 0) atomicOr(a.err, 1);
                break;
            }
            staged = true;
        }
        heavy_slice<V, K, XS, C16, Y>(a, u - a.nitems, xsrc, lane);
    }
    if (XS && use_band && a.bulk && !staged) {
        bool ok = false;
        for (long i = 0; i < FM_WAIT_LIMIT && !ok; i++) {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(bar)
                : "memory");
            ok = done != 0;
        }
        if (!ok && lane == 0) atomicOr(a.err, 2);
    }
}

// Launch of one form kernel; xs/y typed per the form.
template <typename V, int K, bool XS, bool C16, typename Y>
int launch_form(const FormArgs<V, Y> &a, size_t smem, cudaStream_t s) {
    auto kern = k_spmv_form<V, K, XS, C16, Y>;
    if (smem > 0) FL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    FL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FM_THREADS, smem));
    if (per_sm <= 0) per_sm = 1;
    const long units = (long)a.nitems + a.nslices;
    const long grid = std::max<long>(1, std::min<long>((long)num_sms() * per_sm, (units + 31) / 32));
    kern<<<(int)grid, FM_THREADS, smem, s>>>(a);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

// Runs one form: picks the (K, x source, column width) instantiation.
template <typename V, typename Y>
int dispatch_form(const FormArgs<V, Y> &a, int k, bool wide_cols, cudaStream_t s) {
    using X = typename VT<V>::X;
    const size_t smem = (size_t)a.nh * k * sizeof(X);
    const bool xs_smem = a.nh > 0 && !wide_cols && smem <= (size_t)FM_SMEM_MAX;
    const size_t dyn = xs_smem ? smem : 0;
    if (k == 1) {
        if (xs_smem) return launch_form<V, 1, true, true, Y>(a, dyn, s);
        if (!wide_cols) return launch_form<V, 1, false, true, Y>(a, 0, s);
        return launch_form<V, 1, false, false, Y>(a, 0, s);
    }
    if (k == 8) {
        if (xs_smem) return launch_form<V, 8, true, true, Y>(a, dyn, s);
        if (!wide_cols) return launch_form<V, 8, false, true, Y>(a, 0, s);
        return launch_form<V, 8, false, false, Y>(a, 0, s);
    }
    return fail(FL_ERR_ARG, "spmv_form: k=%d (supported: 1, 8)", k);
}

}  // namespace fl

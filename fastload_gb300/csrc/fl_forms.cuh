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

constexpr int FM_THREADS = 1024;
constexpr long FM_WAIT_LIMIT = 1L << 20;
constexpr int FM_SMEM_MAX = 196608;  // dynamic shared memory budget of the form kernels

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
    int H0, nh, nslices, nunits, bulk;
    int heavy_mode;  // 0: atomic add, 1: y += (rows owned by one lane), 2: y = (every row owned, y not zeroed)
    const int *slice_ptr, *hrow, *hlen, *unit_slice, *unit_step;
    const V *hval;
    const uint16_t *hcol16;
    const int *hcol32;
    const X *xs;
    Y *y;
    int *err;
};

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

// Heavy unit: slices [ub, ue), lane l owns row l of each slice and keeps K
// sums in A.  Software-pipelined over (slice, group of G entries): the next
// group's value/column loads are issued before the current group's x gathers
// and FMAs, so each warp keeps two groups of loads in flight.
template <typename V, int G, bool C16, typename Y>
__device__ __forceinline__ void heavy_load_group(const FormArgs<V, Y> &a, int base, int j0, int len, int lane,
                                                 typename VT<V>::A v[G], int c[G]) {
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (j0 + g < len) {
            const int idx = base + 32 * (j0 + g) + lane;
            v[g] = VT<V>::stream1(a.hval + idx);
            if constexpr (C16) c[g] = (int)__ldg(a.hcol16 + idx);
            else c[g] = __ldg(a.hcol32 + idx);
        }
    }
}

// y[r] update of a finished row (atomic, read-modify-write or store).
template <typename A, int K, typename Y>
__device__ __forceinline__ void heavy_flush(int mode, Y *y, int r, const A acc[K]) {
    Y *yr = y + (size_t)r * K;
    if (mode == 0) {
#pragma unroll
        for (int q = 0; q < K; q++) atomicAdd(yr + q, (Y)acc[q]);
    } else if (mode == 1) {
#pragma unroll
        for (int q = 0; q < K; q++) yr[q] += (Y)acc[q];
    } else {
#pragma unroll
        for (int q = 0; q < K; q++) yr[q] = (Y)acc[q];
    }
}

// Heavy unit [T0, T1) (steps), starting in slice sl: lane l owns row l of
// each slice it reaches and keeps K sums in A.  Software-pipelined over
// (slice, group of G steps): the next group's value/column loads are issued
// before the current group's x gathers and FMAs, so each warp keeps two
// groups of loads in flight; the next slice's metadata is fetched one slice
// ahead.  A unit may begin or end inside a slice (long slices are cut into
// several units); each slice part is flushed to y on its own.
template <typename V, int K, bool XS, bool C16, typename Y>
__device__ __forceinline__ void heavy_unit(const FormArgs<V, Y> &a, int sl, int T0, int T1,
                                           const typename VT<V>::X *xsrc, int lane) {
    using A = typename VT<V>::A;
    using X = typename VT<V>::X;
    constexpr int G = K == 1 ? (sizeof(A) == 8 ? 4 : 8) : (sizeof(A) == 8 ? 1 : 2);
    if (T0 >= T1) return;
    int base = __ldg(a.slice_ptr + sl);
    int w = (__ldg(a.slice_ptr + sl + 1) - base) >> 5;
    int s0 = base >> 5;              // global step of the slice's first entry row
    int je = min(w, T1 - s0);        // end of this unit's part of the slice
    int r = __ldg(a.hrow + 32 * sl + lane), len = __ldg(a.hlen + 32 * sl + lane);
    int lim = min(len, je);
    int j0 = T0 - s0, jb = j0;       // current step, first step of the part
    // metadata of slice sl+1 when the unit reaches it
    int mb = 0, mw = 0, mr = 0, mlen = 0;
    if (s0 + w < T1) {
        mb = __ldg(a.slice_ptr + sl + 1);
        mw = (__ldg(a.slice_ptr + sl + 2) - mb) >> 5;
        mr = __ldg(a.hrow + 32 * (sl + 1) + lane);
        mlen = __ldg(a.hlen + 32 * (sl + 1) + lane);
    }
    A v[G];
    int c[G];
    heavy_load_group<V, G, C16, Y>(a, base, j0, lim, lane, v, c);
    A acc[K];
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = (A)0;
    for (;;) {
        int nsl = sl, nj0 = j0 + G, nbase = base, nw = w, ns0 = s0, nje = je, nr = r, nlen = len, nlim = lim;
        bool has_next = true;
        if (nj0 >= je) {
            has_next = s0 + w < T1;
            nsl = sl + 1;
            nj0 = 0;
            if (has_next) {
                nbase = mb;
                nw = mw;
                nr = mr;
                nlen = mlen;
                ns0 = nbase >> 5;
                nje = min(nw, T1 - ns0);
                nlim = min(nlen, nje);
                if (ns0 + nw < T1) {
                    mb = __ldg(a.slice_ptr + nsl + 1);
                    mw = (__ldg(a.slice_ptr + nsl + 2) - mb) >> 5;
                    mr = __ldg(a.hrow + 32 * (nsl + 1) + lane);
                    mlen = __ldg(a.hlen + 32 * (nsl + 1) + lane);
                }
            }
        }
        A nv[G];
        int nc[G];
        if (has_next) heavy_load_group<V, G, C16, Y>(a, nbase, nj0, nlim, lane, nv, nc);
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (j0 + g < lim) {
                X xv[K];
                load_xk<X, K, XS>(xsrc + (size_t)c[g] * K, xv);
#pragma unroll
                for (int q = 0; q < K; q++) acc[q] = fma(v[g], (A)xv[q], acc[q]);
            }
        }
        if (nsl != sl) {
            if (lim > jb) heavy_flush<A, K, Y>(a.heavy_mode, a.y, r, acc);
#pragma unroll
            for (int q = 0; q < K; q++) acc[q] = (A)0;
            jb = 0;
        }
        if (!has_next) break;
        sl = nsl;
        j0 = nj0;
        base = nbase;
        w = nw;
        s0 = ns0;
        je = nje;
        r = nr;
        len = nlen;
        lim = nlim;
#pragma unroll
        for (int g = 0; g < G; g++) {
            v[g] = nv[g];
            c[g] = nc[g];
        }
    }
}


// ---- heavy band through a shared-memory ring (K = 1, x and columns narrow) --
// A unit's slices are contiguous, so its values and 16-bit columns are one
// run of 32-entry steps.  Each warp streams that run through a ring of
// RING_STAGES stages of RING_STEPS steps in its own slice of shared memory
// with cp.async (16-byte copies, completion tracked per thread by
// cp.async.wait_group -- a hardware wait, no spin), so RING_STAGES-1 stages
// are in flight while one is consumed, without holding registers.
constexpr int RING_STEPS = 2;
constexpr int RING_STAGES = 4;
constexpr int SMEM_OPTIN = 232448;  // 227 KB: the largest dynamic shared memory of a block

template <typename V>
__host__ __device__ constexpr int ring_stage_bytes() {
    return RING_STEPS * (32 * (int)sizeof(V) + 32 * (int)sizeof(uint16_t));
}
template <typename V>
__host__ __device__ constexpr int ring_warp_bytes() {
    return RING_STAGES * ring_stage_bytes<V>();
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Stage k (steps RING_STEPS*k ...) of the unit starting at entry E0 with T
// steps into ring slot k % RING_STAGES; always commits a group (empty past
// the end) so the per-thread group count stays in step with k.
template <typename V>
__device__ __forceinline__ void ring_issue(unsigned char *ring, const V *hval, const uint16_t *hcol, int E0, int T,
                                           int k, int lane) {
    const int t0 = k * RING_STEPS;
    const int steps = min(RING_STEPS, T - t0);
    if (steps > 0) {
        unsigned char *slot = ring + (k % RING_STAGES) * ring_stage_bytes<V>();
        const int vbytes = steps * 32 * (int)sizeof(V), cbytes = steps * 64;
        const char *vsrc = (const char *)(hval + E0 + 32 * t0);
        const char *csrc = (const char *)(hcol + E0 + 32 * t0);
        for (int off = lane * 16; off < vbytes; off += 512) cp_async16(slot + off, vsrc + off);
        unsigned char *cdst = slot + RING_STEPS * 32 * sizeof(V);
        for (int off = lane * 16; off < cbytes; off += 512) cp_async16(cdst + off, csrc + off);
    }
    cp_async_commit();
}

template <typename V, typename Y>
__device__ __forceinline__ void heavy_unit_ring(const FormArgs<V, Y> &a, int sl, int T0, int T1,
                                                const typename VT<V>::X *xsrc, unsigned char *ring, int lane) {
    using A = typename VT<V>::A;
    if (T0 >= T1) return;
    const int E0 = 32 * T0;  // first entry of the unit
    const int T = T1 - T0;   // its steps
    const int nst = (T + RING_STEPS - 1) / RING_STEPS;
#pragma unroll
    for (int k = 0; k < RING_STAGES; k++) ring_issue<V>(ring, a.hval, a.hcol16, E0, T, k, lane);
    const int base = __ldg(a.slice_ptr + sl);
    int bnd = (__ldg(a.slice_ptr + sl + 1) >> 5) - T0;  // unit step where the slice ends
    int len = __ldg(a.hlen + 32 * sl + lane), r = __ldg(a.hrow + 32 * sl + lane);
    int j = T0 - (base >> 5), jb = j;                  // step within the slice, first of this part
    int nbnd = T, nlen = 0, nr = 0;                    // slice sl+1, when the unit reaches it
    if (bnd < T) {
        nbnd = (__ldg(a.slice_ptr + sl + 2) >> 5) - T0;
        nlen = __ldg(a.hlen + 32 * (sl + 1) + lane);
        nr = __ldg(a.hrow + 32 * (sl + 1) + lane);
    }
    A acc[1] = {(A)0};
    for (int k = 0; k < nst; k++) {
        cp_async_wait<RING_STAGES - 1>();
        __syncwarp();
        const unsigned char *slot = ring + (k % RING_STAGES) * ring_stage_bytes<V>();
        const V *sv = (const V *)slot;
        const uint16_t *sc = (const uint16_t *)(slot + RING_STEPS * 32 * sizeof(V));
#pragma unroll
        for (int q = 0; q < RING_STEPS; q++) {
            const int t = k * RING_STEPS + q;
            if (t < T) {
                if (j < len) {
                    const A v = VT<V>::plain1(sv + 32 * q + lane);  // shared memory
                    acc[0] = fma(v, (A)xsrc[sc[32 * q + lane]], acc[0]);
                }
                j++;
                const bool slice_end = t + 1 == bnd;
                if (slice_end || t + 1 == T) {
                    if (len > jb) heavy_flush<A, 1, Y>(a.heavy_mode, a.y, r, acc);
                    acc[0] = (A)0;
                    if (slice_end) {
                        sl++;
                        j = 0;
                        jb = 0;
                        len = nlen;
                        r = nr;
                        bnd = nbnd;
                        if (bnd < T) {
                            nbnd = (__ldg(a.slice_ptr + sl + 2) >> 5) - T0;
                            nlen = __ldg(a.hlen + 32 * (sl + 1) + lane);
                            nr = __ldg(a.hrow + 32 * (sl + 1) + lane);
                        }
                    }
                }
            }
        }
        __syncwarp();
        ring_issue<V>(ring, a.hval, a.hcol16, E0, T, k + RING_STAGES, lane);
    }
    cp_async_wait<0>();
    __syncwarp();
}

template <typename V, int K, bool XS, bool C16, typename Y, bool RING = false>
__global__ void __launch_bounds__(FM_THREADS, 1) k_spmv_form(const FormArgs<V, Y> a) {
    using X = typename VT<V>::X;
    extern __shared__ __align__(128) unsigned char fm_smem[];
    X *xh = (X *)fm_smem;
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ int claimed;  // units of this block handed out so far
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&mbar);
    if (tid == 0) claimed = 0;
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
    const int total = a.nitems + (use_band ? a.nunits : 0);
    bool staged = !(XS && use_band && a.bulk);
    // Work distribution: unit u (light items first, then heavy units) goes
    // to block u % gridDim.x, so every block gets an even share of both
    // kinds; inside the block warps claim the block's units through a
    // shared-memory counter.  No global atomics, no per-launch reset.
    __syncthreads();
    const int G = gridDim.x;
    const int mine = total > (int)blockIdx.x ? (total - 1 - (int)blockIdx.x) / G + 1 : 0;
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&claimed, 1);
        k = __shfl_sync(FULLM, k, 0);
        if (k >= mine) break;
        const int u = (int)blockIdx.x + G * k;
        if (u < a.nitems) {
            if constexpr (K == 1) stream_item<V, Y, 1>(a.items[u], a.regions, a.row, a.val, a.xs, a.y, lane);
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
        const int ui = u - a.nitems;
        const int sl = __ldg(a.unit_slice + ui), T0 = __ldg(a.unit_step + ui), T1 = __ldg(a.unit_step + ui + 1);
        if constexpr (RING) {
            const size_t xb = ((size_t)a.nh * K * sizeof(X) + 127) & ~(size_t)127;
            heavy_unit_ring<V, Y>(a, sl, T0, T1, xsrc, fm_smem + xb + (size_t)(tid >> 5) * ring_warp_bytes<V>(), lane);
        } else {
            heavy_unit<V, K, XS, C16, Y>(a, sl, T0, T1, xsrc, lane);
        }
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
template <typename V, int K, bool XS, bool C16, typename Y, bool RING = false>
int launch_form(const FormArgs<V, Y> &a, size_t smem, cudaStream_t s) {
    auto kern = k_spmv_form<V, K, XS, C16, Y, RING>;
    if (smem > 0) FL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    FL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FM_THREADS, smem));
    if (per_sm <= 0) per_sm = 1;
    const long units = (long)a.nitems + a.nunits;
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
        // the heavy band through per-warp shared-memory rings when x and the
        // rings fit beside each other
        const size_t xb = (smem + 127) & ~(size_t)127;
        const size_t ring = (size_t)(FM_THREADS / 32) * ring_warp_bytes<V>();
        if (xs_smem && a.nslices > 0 && xb + ring <= (size_t)SMEM_OPTIN)
            return launch_form<V, 1, true, true, Y, true>(a, xb + ring, s);
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

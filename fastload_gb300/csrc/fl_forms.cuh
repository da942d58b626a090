// fl_forms.cuh -- generic SpMV kernel for the storage / right-hand-side forms.
//
// One template covers every form beside the plain FP64 drop-in kernels:
//   V  value storage: double (FP64), float (FP32) or bf16x2_t (a BF16 hi+lo
//      split: hi = bf16(v) and a 16-bit correction relative to hi, 23
//      significant bits in all; fl_stream.cuh);
//   K  right-hand sides: x and y row-interleaved (x[col*K + r], y[row*K + r]);
//   XS x of the heavy band read from shared memory (staged by a TMA bulk copy)
//      or from global memory (bands wider than shared memory);
//   C16 heavy-band column indices stored as 16 bits (band <= 65535) or 32;
//   Y  y type (double, or float for the FP32-accumulating batched form);
//   RING the band's values and columns streamed through shared-memory rings
//      filled by cp.async (K = 1, x in shared memory) instead of the
//      register-pipelined loop: per warp for FP64 bands, per lane for the
//      4-byte bands kept in packs of four steps;
//   OVL the light columns' x still arriving when the kernel starts (the
//      overlapped host-buffer call): heavy units first, light items once a
//      flag says the x is in.
// Launched as a programmatic dependent of the kernel before it, the kernel
// waits for that kernel before touching memory -- or, behind the library's
// own y zeroing (FormArgs::after_zeroing, kernels with a staged band), before
// each thread's first y update, so the band's x staging and the light
// items' first loads overlap the zeroing -- and releases its own dependent
// when each block is done.
// Products and per-row sums are computed in FP32 for the FP32/BF16 forms and
// in FP64 for the FP64 form; y is accumulated in Y.  The work is the bucketed
// split of fl_bucket.cu: light columns in the FastLoad tile stream with one
// atomic per run (K = 1) or per (nonzero, rhs) (K > 1), the heavy band in
// 32-row slices with one lane per row.  When the band holds every column
// (no light part) each row is owned by one lane and y is updated without
// atomics.  Heavy units are dealt to blocks round-robin, or in contiguous
// ranges for batches (FormArgs::contig).
#pragma once

#include "fl_stream.cuh"

#include <algorithm>
#include <mutex>
#include <type_traits>

namespace fl {

constexpr int FM_THREADS = 1024;
constexpr long FM_WAIT_LIMIT = 1L << 20;
constexpr long FM_FLAG_LIMIT = 1L << 20;  // polls of x_ready (an L2 round trip and a short sleep each): about a second
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
    // x of the light columns still in flight (host call with overlapped
    // upload, kernels instantiated with OVL): it is in once *x_ready reaches
    // x_epoch.  nullptr: x complete at launch.
    const int *x_ready;
    int x_epoch;
    // host-mapped status word of a synchronous host call (nullptr: none):
    // an expired wait is also reported there, so the call needs no readback
    int *err_host;
    // launch options of the form (host side: they pick the instantiation)
    int heavy_loop = FL_HEAVY_AUTO;
    int x_stage = FL_XSTAGE_AUTO;
    // heavy units dealt to blocks in contiguous ranges (batches) rather
    // than round-robin
    int contig = 0;
    // the kernel launched just before this one is the library's y zeroing
    // (which releases its dependent only after its own wait for everything
    // before it): the band's x may be staged before waiting for it
    int after_zeroing = 0;
};

// An expired bounded wait: bits into the launch's status word (and the host
// call's mapped word).
template <typename V, typename Y>
__device__ __forceinline__ void form_fail(const FormArgs<V, Y> &a, int bits) {
    atomicOr(a.err, bits);
    if (a.err_host) *(volatile int *)a.err_host = bits;
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
            // columns streamed too (evict-first): allocated normally in L1
            // they evicted the x lines the gathers reuse (7-point Laplacian
            // 128^3, FP64 band of every column: 45.5 -> 41.4 us)
            if constexpr (C16) c[g] = (int)__ldcs(a.hcol16 + idx);
            else c[g] = __ldcs(a.hcol32 + idx);
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
// Entries of zero padding past the end of a band's value and column arrays:
// the ring copies whole stages.
constexpr int RING_PAD = RING_STEPS * 32;

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename V, typename Y>
__device__ __forceinline__ void heavy_unit_ring(const FormArgs<V, Y> &a, int sl, int T0, int T1,
                                                const typename VT<V>::X *xsrc, unsigned char *ring, int lane) {
    using A = typename VT<V>::A;
    if (T0 >= T1) return;
    constexpr int VB = RING_STEPS * 32 * (int)sizeof(V);  // value bytes of a stage
    constexpr int CB = RING_STEPS * 32 * (int)sizeof(uint16_t);  // column bytes of a stage
    constexpr int SB = ring_stage_bytes<V>();
    const int T = T1 - T0;  // the unit's steps
    const int nst = (T + RING_STEPS - 1) / RING_STEPS;
    // Stage k (steps RING_STEPS*k ...) goes to ring slot k % RING_STAGES,
    // always whole: a unit's last stage may run into the next unit's steps
    // or, for the band's last unit, the stage of zero padding the band
    // arrays carry past their end; the consumer stops at T.  Every call
    // commits a group (empty past the unit) so the per-thread group count
    // stays in step with k.  This lane's 16-byte pieces are fixed offsets.
    static_assert((RING_STAGES & (RING_STAGES - 1)) == 0, "ring slots are taken modulo a power of two");
    // this lane's pieces: source pointers advanced a stage per issue, slot
    // offsets fixed
    const char *vsrc = (const char *)(a.hval + 32 * (size_t)T0) + lane * 16;
    const char *csrc = (const char *)(a.hcol16 + 32 * (size_t)T0) + lane * 16;
    unsigned char *lring = ring + lane * 16;
    auto issue = [&](int k) {
        if (k < nst) {
            unsigned char *slot = lring + (k & (RING_STAGES - 1)) * SB;
#pragma unroll
            for (int off = 0; off < VB; off += 512)
                if (off + lane * 16 < VB) cp_async16(slot + off, vsrc + off);
            if (lane * 16 < CB) cp_async16(slot + VB, csrc);
            vsrc += VB;
            csrc += CB;
        }
        cp_async_commit();
    };
#pragma unroll
    for (int k = 0; k < RING_STAGES; k++) issue(k);
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
        const unsigned char *slot = ring + (k & (RING_STAGES - 1)) * SB;
        const V *sv = (const V *)slot;
        const uint16_t *sc = (const uint16_t *)(slot + VB);
        const int t0 = k * RING_STEPS;
        if (t0 + RING_STEPS < bnd && t0 + RING_STEPS < T) {
            // no slice end and no unit end inside this stage
#pragma unroll
            for (int q = 0; q < RING_STEPS; q++)
                if (j + q < len)
                    acc[0] = fma(VT<V>::plain1(sv + 32 * q + lane), (A)xsrc[sc[32 * q + lane]], acc[0]);
            j += RING_STEPS;
        } else {
#pragma unroll
            for (int q = 0; q < RING_STEPS; q++) {
                const int t = t0 + q;
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
        }
        __syncwarp();
        issue(k + RING_STAGES);
    }
    cp_async_wait<0>();
    __syncwarp();
}

// ---- heavy band of 4-byte values: lane-major packs of four steps ---------
// FP32 and BF16 hi+lo bands keep their entries in packs of four steps with
// each lane's four entries adjacent: entry (global step S, lane l) at
//     128 * (S / 4) + 4 * l + S % 4.
// A lane reads its four values of a pack with one 16-byte load and its four
// columns with one 8-byte (16-bit columns) or 16-byte (32-bit) load, and a
// warp's loads of one pack are contiguous.  Against one entry per load this
// cuts the instructions a nonzero costs by about four, which is what bounds
// a 4-byte band (its bytes per nonzero are half of FP64's).  Entries a row
// does not have (a lane past its row's length inside a slice) hold value 0
// and column nh, and the shared-memory staging of x keeps a zero at x[nh],
// so the ring loop needs no length test.
constexpr int P4_STAGES = 4;                // packs in a lane's ring (a power of two)
constexpr int P4_VB = 32 * 4 * 4;           // value bytes of a pack (512)
constexpr int P4_CB = 32 * 4 * 2;           // 16-bit column bytes of a pack (256)
constexpr int P4_SB = P4_VB + P4_CB;        // ring stage
constexpr int P4_RING_WARP = P4_STAGES * P4_SB;
static_assert((P4_STAGES & (P4_STAGES - 1)) == 0, "ring slots are taken modulo a power of two");

__host__ __device__ __forceinline__ long p4_index(long S, int l) { return 128 * (S >> 2) + 4 * l + (S & 3); }
// Entries of a packed band array of `steps` steps: whole packs, plus one
// pack of padding (the loops read whole packs).
inline long p4_entries(long steps) { return ((steps + 3) / 4 + 1) * 128; }

// Slice-layout array (entry j of step S, lane l at 32 S + l; `steps` steps)
// to packed layout; entries past the last step are zero.
template <typename T>
__global__ void k_to_p4(const T *__restrict__ in, long steps, T *__restrict__ out, long nout) {
    for (long d = blockIdx.x * (long)blockDim.x + threadIdx.x; d < nout; d += (long)gridDim.x * blockDim.x) {
        const long S = 4 * (d >> 7) + (d & 3);
        const int l = (int)((d >> 2) & 31);
        out[d] = S < steps ? in[32 * S + l] : (T)0;
    }
}

__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gsrc) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ uint4 ld_stream_v4(const void *p) {
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p));
    return r;
}
__device__ __forceinline__ uint2 ld_stream_v2(const void *p) {
    uint2 r;
    asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "l"(p));
    return r;
}

// A unit's walk over its slices in global steps: the current slice's first
// and end step, this lane's row and length in it, the first step of the
// unit's part of it, and the next slice's values, fetched one slice ahead.
struct SliceWalk {
    int s0, bnd, len, r, jb, sl;
    int nbnd, nlen, nr;
};

template <typename V, typename Y>
__device__ __forceinline__ void walk_fetch_next(SliceWalk &w, const FormArgs<V, Y> &a, int T1, int lane) {
    if (w.bnd < T1) {
        w.nbnd = __ldg(a.slice_ptr + w.sl + 2) >> 5;
        w.nlen = __ldg(a.hlen + 32 * (w.sl + 1) + lane);
        w.nr = __ldg(a.hrow + 32 * (w.sl + 1) + lane);
    }
}

template <typename V, typename Y>
__device__ __forceinline__ void walk_init(SliceWalk &w, const FormArgs<V, Y> &a, int sl, int T0, int T1, int lane) {
    w.sl = sl;
    w.s0 = __ldg(a.slice_ptr + sl) >> 5;
    w.bnd = __ldg(a.slice_ptr + sl + 1) >> 5;
    w.len = __ldg(a.hlen + 32 * sl + lane);
    w.r = __ldg(a.hrow + 32 * sl + lane);
    w.jb = T0 - w.s0;
    w.nbnd = w.nlen = w.nr = 0;
    walk_fetch_next(w, a, T1, lane);
}

// Step S, the last of a part (S + 1 ends the slice or the unit), is done:
// the part's sums go to y (when this lane's row has entries in the part)
// and the walk moves to the next slice when the slice ended.
template <typename V, int K, typename Y>
__device__ __forceinline__ void walk_end(SliceWalk &w, const FormArgs<V, Y> &a, float acc[K], int S, int T1,
                                         int lane) {
    if (w.len > w.jb) heavy_flush<float, K, Y>(a.heavy_mode, a.y, w.r, acc);
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = 0.f;
    if (S + 1 == w.bnd) {
        w.sl++;
        w.s0 = w.bnd;
        w.jb = 0;
        w.len = w.nlen;
        w.r = w.nr;
        w.bnd = w.nbnd;
        walk_fetch_next(w, a, T1, lane);
    }
}

// Heavy unit [T0, T1) of a packed 4-byte band through a per-lane ring in
// shared memory (K = 1, x and 16-bit columns staged): each lane copies its
// own 16 bytes of values and 8 bytes of columns of each pack with cp.async
// into its own slots, P4_STAGES packs deep, so no warp barrier is needed;
// cp.async.wait_group (a hardware wait) says when a pack is in.
template <typename V, typename Y>
__device__ __forceinline__ void heavy_unit_ring_p4(const FormArgs<V, Y> &a, int sl, int T0, int T1,
                                                   const float *xsrc, unsigned char *ring, int lane) {
    static_assert(sizeof(V) == 4, "packed bands hold 4-byte values");
    if (T0 >= T1) return;
    const int P0 = T0 >> 2, np = ((T1 + 3) >> 2) - P0;
    const char *vsrc = (const char *)(a.hval + 128L * P0) + 16 * lane;
    const char *csrc = (const char *)(a.hcol16 + 128L * P0) + 8 * lane;
    unsigned char *lv = ring + 16 * lane, *lc = ring + P4_VB + 8 * lane;
    auto issue = [&](int k) {
        if (k < np) {
            const int o = (k & (P4_STAGES - 1)) * P4_SB;
            cp_async16(lv + o, vsrc);
            cp_async8(lc + o, csrc);
            vsrc += P4_VB;
            csrc += P4_CB;
        }
        cp_async_commit();
    };
#pragma unroll
    for (int k = 0; k < P4_STAGES; k++) issue(k);
    SliceWalk w;
    walk_init(w, a, sl, T0, T1, lane);
    float acc[1] = {0.f};
    int S0 = P0 * 4;
    for (int k = 0; k < np; k++, S0 += 4) {
        cp_async_wait<P4_STAGES - 1>();
        const int o = (k & (P4_STAGES - 1)) * P4_SB;
        const uint4 v = *(const uint4 *)(lv + o);
        const uint2 c = *(const uint2 *)(lc + o);
        const float x0 = xsrc[c.x & 0xffffu], x1 = xsrc[c.x >> 16], x2 = xsrc[c.y & 0xffffu], x3 = xsrc[c.y >> 16];
        if (S0 >= T0 && S0 + 4 < w.bnd && S0 + 4 < T1) {
            // the pack lies inside the unit and inside one slice, not at its end
            acc[0] = fmaf(VT<V>::from_bits(v.x), x0, acc[0]);
            acc[0] = fmaf(VT<V>::from_bits(v.y), x1, acc[0]);
            acc[0] = fmaf(VT<V>::from_bits(v.z), x2, acc[0]);
            acc[0] = fmaf(VT<V>::from_bits(v.w), x3, acc[0]);
        } else {
            const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
            const float xx[4] = {x0, x1, x2, x3};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int S = S0 + q;
                if (S >= T0 && S < T1) {
                    acc[0] = fmaf(VT<V>::from_bits(vv[q]), xx[q], acc[0]);
                    if (S + 1 == w.bnd || S + 1 == T1) walk_end<V, 1, Y>(w, a, acc, S, T1, lane);
                }
            }
        }
        issue(k + P4_STAGES);
    }
    cp_async_wait<0>();
}

// Heavy unit [T0, T1) of a packed 4-byte band with loads held in registers:
// x in shared memory too wide for the ring beside it, x read through the
// cache, or K right-hand sides.  Groups of PG packs, the next group's loads
// issued before the current group is computed; entries past a row's length
// are skipped (x read from global memory has no zero slot).
template <typename V, int K, bool XS, bool C16, typename Y>
__device__ __forceinline__ void heavy_unit_p4(const FormArgs<V, Y> &a, int sl, int T0, int T1, const float *xsrc,
                                              int lane) {
    static_assert(sizeof(V) == 4, "packed bands hold 4-byte values");
    constexpr int PG = K == 1 ? 2 : 1;
    if (T0 >= T1) return;
    const int P0 = T0 >> 2, np = ((T1 + 3) >> 2) - P0;
    auto load = [&](int k, uint4 vv[PG], uint4 cc[PG]) {
#pragma unroll
        for (int g = 0; g < PG; g++) {
            if (k + g < np) {
                const long e = 128L * (P0 + k + g) + 4 * lane;
                vv[g] = ld_stream_v4(a.hval + e);
                if constexpr (C16) {
                    const uint2 t = ld_stream_v2(a.hcol16 + e);  // unpacked where used: two registers held
                    cc[g] = make_uint4(t.x, t.y, 0u, 0u);
                } else {
                    cc[g] = ld_stream_v4(a.hcol32 + e);
                }
            }
        }
    };
    SliceWalk w;
    walk_init(w, a, sl, T0, T1, lane);
    float acc[K];
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = 0.f;
    uint4 v[PG], c[PG];
    load(0, v, c);
    for (int k = 0; k < np; k += PG) {
        uint4 nv[PG], nc[PG];
        load(k + PG, nv, nc);
#pragma unroll
        for (int g = 0; g < PG; g++) {
            if (k + g < np) {
                const int S0 = 4 * (P0 + k + g);
                const uint32_t vv[4] = {v[g].x, v[g].y, v[g].z, v[g].w};
                uint32_t cc[4];
                if constexpr (C16) {
                    cc[0] = c[g].x & 0xffffu;
                    cc[1] = c[g].x >> 16;
                    cc[2] = c[g].y & 0xffffu;
                    cc[3] = c[g].y >> 16;
                } else {
                    cc[0] = c[g].x;
                    cc[1] = c[g].y;
                    cc[2] = c[g].z;
                    cc[3] = c[g].w;
                }
                if (S0 >= T0 && S0 + 4 < w.bnd && S0 + 4 < T1) {
                    const int j0 = S0 - w.s0;
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        if (j0 + q < w.len) {
                            float xv[K];
                            load_xk<float, K, XS>(xsrc + (size_t)cc[q] * K, xv);
                            const float f = VT<V>::from_bits(vv[q]);
#pragma unroll
                            for (int r = 0; r < K; r++) acc[r] = fmaf(f, xv[r], acc[r]);
                        }
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const int S = S0 + q;
                        if (S >= T0 && S < T1) {
                            if (S - w.s0 < w.len) {
                                float xv[K];
                                load_xk<float, K, XS>(xsrc + (size_t)cc[q] * K, xv);
                                const float f = VT<V>::from_bits(vv[q]);
#pragma unroll
                                for (int r = 0; r < K; r++) acc[r] = fmaf(f, xv[r], acc[r]);
                            }
                            if (S + 1 == w.bnd || S + 1 == T1) walk_end<V, K, Y>(w, a, acc, S, T1, lane);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int g = 0; g < PG; g++) {
            v[g] = nv[g];
            c[g] = nc[g];
        }
    }
}

// Whether the light columns' x is in (acquire: its bytes are visible to
// the reading thread afterwards).
template <typename V, typename Y>
__device__ __forceinline__ bool light_x_in(const FormArgs<V, Y> &a) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(a.x_ready) : "memory");
    return (int)((unsigned)v - (unsigned)a.x_epoch) >= 0;
}

// Block-shared word: some warp of the block has acquired the light x.
// Published with release, read with acquire, so a warp reading it inherits
// the acquiring warp's view of x.
__device__ __forceinline__ int shared_acquire(const int *w) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"((uint32_t)__cvta_generic_to_shared(w))
                 : "memory");
    return v;
}
__device__ __forceinline__ void shared_release(int *w, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(w)), "r"(v)
                 : "memory");
}

template <typename V, int K, bool XS, bool C16, typename Y, bool RING = false, bool OVL = false>
__global__ void __launch_bounds__(FM_THREADS, 1) k_spmv_form(const FormArgs<V, Y> a) {
    using X = typename VT<V>::X;
    extern __shared__ __align__(128) unsigned char fm_smem[];
    X *xh = (X *)fm_smem;
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ int claimed;    // units (OVL: light items) of this block handed out so far
    __shared__ int claimed_h;  // OVL: heavy units handed out
    __shared__ int x_in;       // OVL: some warp of the block has acquired the light x
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&mbar);
    if (tid == 0) claimed = claimed_h = x_in = 0;
    // Launched as a programmatic dependent of the kernel before it: the
    // block may be resident before that kernel ends, so it waits for it
    // before reading or writing anything -- except, when that kernel is the
    // library's y zeroing, for what does not touch y: the staging of the
    // band's x and the first loads of the light items then run beside the
    // zeroing (the zeroing kernel releases this one only after its own wait
    // for every kernel before it, so x is complete), and each thread waits
    // before its first y update (pdl_wait_once; heavy units wait once the
    // staged x is in) and, at the latest, before it exits.  Kernels without
    // a staged band wait at once (their register budget is spent on the
    // band loop).
    bool waited = !(XS && a.after_zeroing);
    if (waited) asm volatile("griddepcontrol.wait;" ::: "memory");
    const bool use_band = a.nh > 0 && a.nslices > 0;
    if (XS && use_band) {
        const uint32_t bytes = (uint32_t)a.nh * K * (uint32_t)sizeof(X);
        // x[nh] = 0 (16 bytes): the column of a packed band's padding entries
        if (tid < 4) ((uint32_t *)(fm_smem + bytes))[tid] = 0u;
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
    const int G = gridDim.x, b = (int)blockIdx.x;
    const int mine = total > b ? (total - 1 - b) / G + 1 : 0;
    // one heavy unit; the first waits (bounded) for the band's staged x
    auto heavy = [&](int ui) -> bool {
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
                if (lane == 0) form_fail(a, 1);
                return false;
            }
            staged = true;
        }
        if constexpr (XS) pdl_wait_once(&waited);
        const int sl = __ldg(a.unit_slice + ui), T0 = __ldg(a.unit_step + ui), T1 = __ldg(a.unit_step + ui + 1);
        // the rings start past x and its 16 bytes of zeros (x[nh])
        const size_t xb = ((size_t)a.nh * K * sizeof(X) + 16 + 127) & ~(size_t)127;
        if constexpr (sizeof(V) == 4) {
            if constexpr (RING)
                heavy_unit_ring_p4<V, Y>(a, sl, T0, T1, xsrc, fm_smem + xb + (size_t)(tid >> 5) * P4_RING_WARP, lane);
            else
                heavy_unit_p4<V, K, XS, C16, Y>(a, sl, T0, T1, xsrc, lane);
        } else if constexpr (RING) {
            heavy_unit_ring<V, Y>(a, sl, T0, T1, xsrc, fm_smem + xb + (size_t)(tid >> 5) * ring_warp_bytes<V>(), lane);
        } else {
            heavy_unit<V, K, XS, C16, Y>(a, sl, T0, T1, xsrc, lane);
        }
        return true;
    };
    auto light = [&](int u) {
        if constexpr (K == 1) {
            stream_item<V, Y, 1>(a.items[u], a.regions, a.row, a.val, a.xs, a.y, lane, XS ? &waited : nullptr);
        } else {
            if constexpr (XS) pdl_wait_once(&waited);
            light_item_kn<V, K, Y>(a.items[u], a.regions, a.row, a.val, a.xs, a.y, lane);
        }
    };
    if constexpr (!OVL) {
        // Work distribution: unit u (light items first, then heavy units)
        // goes to block u % gridDim.x, so every block gets an even share of
        // both kinds; inside the block warps claim the block's units through
        // a shared-memory counter.  No global atomics, no per-launch reset.
        // A batch (a.contig) deals its heavy units in one contiguous range
        // per block instead, so a block's warps work on the same matrix and
        // its x gathers share the SM's L1 (256 matrices of 186M nonzeros:
        // 0.73 -> 0.64 ms; for a single matrix the round-robin deal is
        // faster).
        const int ml = a.nitems > b ? (a.nitems - 1 - b) / G + 1 : 0;  // this block's light items
        const int hu = use_band ? a.nunits : 0;
        const int h0 = (int)((long)b * hu / G);
        const int nk = a.contig ? ml + (int)((long)(b + 1) * hu / G) - h0 : mine;
        for (;;) {
            int k = 0;
            if (lane == 0) k = atomicAdd(&claimed, 1);
            k = __shfl_sync(FULLM, k, 0);
            if (k >= nk) break;
            if (k < ml) {
                light(b + G * k);
                continue;
            }
            if (!heavy(a.contig ? h0 + k - ml : b + G * k - a.nitems)) break;
        }
    } else {
        // The light columns' x is still arriving.  The block's units are
        // dealt as above; a warp takes a heavy unit while the x is not in,
        // then the light items, and waits (bounded) for the x only when no
        // heavy unit is left.
        const int ml = a.nitems > b ? (a.nitems - 1 - b) / G + 1 : 0;  // this block's light items
        const int mh = mine - ml;                                        // and heavy units
        bool have = false;  // this warp has acquired the light x
        for (;;) {
            int kind = 0, k = 0;  // 0 none left, 1 light item k, 2 heavy unit k
            if (lane == 0) {
                for (;;) {
                    const int jl = *(volatile int *)&claimed, jh = *(volatile int *)&claimed_h;
                    const bool lav = jl < ml, hav = jh < mh;
                    if (!lav && !hav) break;
                    bool take_light = !hav;
                    if (lav && hav) {
                        take_light = have || *(volatile int *)&x_in;
                        if (!take_light && light_x_in(a)) {
                            shared_release(&x_in, 1);
                            take_light = true;
                        }
                    }
                    if (take_light) {
                        k = atomicAdd(&claimed, 1);
                        if (k < ml) {
                            kind = 1;
                            break;
                        }
                    } else {
                        k = atomicAdd(&claimed_h, 1);
                        if (k < mh) {
                            kind = 2;
                            break;
                        }
                    }
                }
            }
            kind = __shfl_sync(FULLM, kind, 0);
            k = __shfl_sync(FULLM, k, 0);
            if (kind == 0) break;
            if (kind == 2) {
                if (!heavy(b + G * (ml + k) - a.nitems)) break;
                continue;
            }
            if (!have) {
                // acquire the light x: through the block's word when another
                // warp already has, else from the flag (bounded wait)
                int ok = 0;
                if (lane == 0) {
                    for (long i = 0; i < FM_FLAG_LIMIT; i++) {
                        if (shared_acquire(&x_in)) {
                            ok = 1;
                            break;
                        }
                        if (light_x_in(a)) {
                            ok = 1;
                            shared_release(&x_in, 1);
                            break;
                        }
                        if (*(volatile int *)a.err & 4) break;  // another warp already gave up
                        __nanosleep(200);
                    }
                }
                ok = __shfl_sync(FULLM, ok, 0);
                __syncwarp();  // lane 0's acquire orders the warp's x loads
                if (!ok) {
                    if (lane == 0) form_fail(a, 4);
                    break;
                }
                have = true;
            }
            light(b + G * k);
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
        if (!ok && lane == 0) form_fail(a, 2);
    }
    // every thread has waited for the kernel before this one (a warp that
    // found no work has not yet), so this kernel never completes before it
    if constexpr (XS) pdl_wait_once(&waited);
    // this block is done: a dependent launch behind this kernel may start
    // (it waits for this kernel's completion before touching memory)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch of one form kernel; xs/y typed per the form.
template <typename V, int K, bool XS, bool C16, typename Y, bool RING = false, bool OVL = false>
int launch_form(const FormArgs<V, Y> &a, size_t smem, cudaStream_t s) {
    auto kern = k_spmv_form<V, K, XS, C16, Y, RING, OVL>;
    // the shared-memory opt-in and the occupancy query cost host time on
    // every launch: done once per (instantiation, shared-memory size)
    static std::mutex mu;
    static size_t smem_opted = 0, occ_smem = ~(size_t)0;
    static int occ_per_sm = 0;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (smem > smem_opted) {
            FL_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            smem_opted = smem;
        }
        if (smem != occ_smem) {
            FL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_per_sm, kern, FM_THREADS, smem));
            occ_smem = smem;
        }
        per_sm = occ_per_sm;
    }
    if (per_sm <= 0) per_sm = 1;
    const long units = (long)a.nitems + a.nunits;
    const long grid = std::max<long>(1, std::min<long>((long)num_sms() * per_sm, (units + 31) / 32));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(FM_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FL_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
    return FL_SUCCESS;
}

// Runs one form: picks the (K, x source, column width) instantiation.
template <typename V, typename Y>
int dispatch_form(const FormArgs<V, Y> &a, int k, bool wide_cols, cudaStream_t s) {
    using X = typename VT<V>::X;
    const size_t smem = (size_t)a.nh * k * sizeof(X);
    const bool xs_smem = a.x_stage != FL_XSTAGE_GLOBAL && a.nh > 0 && !wide_cols && smem <= (size_t)FM_SMEM_MAX;
    const size_t dyn = xs_smem ? smem + 16 : 0;  // x and 16 bytes of zeros (x[nh])
    if (k == 1) {
        // the heavy band through per-warp shared-memory rings when x and the
        // rings fit beside each other
        const size_t xb = (smem + 16 + 127) & ~(size_t)127;
        const size_t ring = (size_t)(FM_THREADS / 32) * (sizeof(V) == 4 ? (size_t)P4_RING_WARP : ring_warp_bytes<V>());
        const bool use_ring =
            a.heavy_loop != FL_HEAVY_REGS && xs_smem && a.nslices > 0 && xb + ring <= (size_t)SMEM_OPTIN;
        if (a.x_ready) {
            // x still arriving (FP64 host call): only the staged-band kernels
            if constexpr (std::is_same<V, double>::value && std::is_same<Y, double>::value) {
                if (use_ring) return launch_form<V, 1, true, true, Y, true, true>(a, xb + ring, s);
                if (xs_smem) return launch_form<V, 1, true, true, Y, false, true>(a, dyn, s);
            }
            return fail(FL_ERR_ARG, "spmv_form: overlapped upload needs the band's x in shared memory");
        }
        if (use_ring) return launch_form<V, 1, true, true, Y, true>(a, xb + ring, s);
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

// One instantiation set per value / y type, in its own translation unit
// (fl_form_f64.cu, fl_form_f32.cu, fl_form_bf16.cu).
int run_form_f64(const FormArgs<double, double> &a, int k, bool wide, cudaStream_t s);
int run_form_f32(const FormArgs<float, double> &a, int k, bool wide, cudaStream_t s);
int run_form_f32_y32(const FormArgs<float, float> &a, int k, bool wide, cudaStream_t s);
int run_form_bf16(const FormArgs<bf16x2_t, double> &a, int k, bool wide, cudaStream_t s);

}  // namespace fl

// fl_stream.cuh -- device side of the FastLoad streaming SpMV, shared by the
// plain streaming kernel (fl_spmv.cu), the light part of the bucketed kernel
// (fl_bucket.cu) and the storage forms (fl_forms.cuh).
//
// A warp walks a work item 32 nonzeros at a time: lane l takes nonzero
// e + 32k + l (k = 0..4U-1 per iteration), so every load of a 32-nonzero row
// is one coalesced 128-byte (rows) / 256-byte (FP64 values) request and, when
// a tile's rows are consecutive (banded matrices), every atomic instruction
// covers 8 sectors instead of 32.  The sorted column of each nonzero follows
// from the region descriptor with one division per lane per iteration:
// in a full region (32-wide chunks of `tall` levels) col = col_base +
// 32*(q / 32*tall) + q%32 and q%32 is the same for all of a lane's nonzeros;
// in a partial chunk col = col_base + q % len.  Runs of equal consecutive
// rows inside each 32-nonzero row are summed by a segmented shuffle scan
// (only when a ballot finds one) and added to y once per run -- the run
// semantics of the reference's tile formats 1/2 (FastLoad_GPU.h:192-270).
#pragma once

#include "fl_internal.cuh"

namespace fl {

constexpr unsigned FULLM = 0xffffffffu;

// BF16 hi+lo value storage, 4 bytes a value.  The high half is hi =
// bf16(v) (round to nearest even), a plain BF16 that a BF16 consumer can
// read on its own.  The low half is a signed 16-bit correction d relative to
// hi: v ~ hi * (1 + d * 2^-22), |d| <= 32767.  Since |v - hi| <= 2^-8 |hi|,
// d spans the residual with 15 bits, so hi and d together carry 23
// significant bits: the stored value is within 2^-23 |hi| of v, and the
// decoded FP32 value (one fma) within (2^-23 + 2^-24) |v|.  (A BF16 low
// half -- hi + bf16(v - hi) -- keeps 16 significant bits and leaves up to
// 2^-17 relative error per value, too coarse for a 1e-6 result.)  Values
// whose hi is zero, infinite, NaN or below 2^-100 in magnitude store d = 0.
struct bf16x2_t {
    uint32_t u;
};

constexpr int BF16X2_LO_SHIFT = 22;  // d is the residual in units of 2^-22 |hi|

__device__ __forceinline__ uint32_t bf16x2_encode(double v) {
    const __nv_bfloat16 h = __double2bfloat16(v);
    const double hf = (double)__bfloat162float(h);
    int d = 0;
    if (fabs(hf) >= 0x1p-100 && fabs(hf) <= 0x1.fep+127) {  // nonzero and finite
        // v - hf is exact (Sterbenz: hf and v are within a factor of two)
        const double t = rint((v - hf) / hf * (double)(1 << BF16X2_LO_SHIFT));
        d = (int)fmin(fmax(t, -32767.0), 32767.0);
    }
    return ((uint32_t)__bfloat16_as_ushort(h) << 16) | (uint32_t)(uint16_t)(int16_t)d;
}

__device__ __forceinline__ float bf16x2_decode(uint32_t u) {
    const float hi = __uint_as_float(u & 0xffff0000u);
    const float d = (float)(int16_t)(u & 0xffffu);
    return fmaf(hi * 0x1p-22f, d, hi);
}

__device__ __forceinline__ int ld_stream_i32(const int *p) {
    int r;
    asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}

// Value storage traits: X = x type, A = arithmetic type of products and sums.
template <typename V>
struct VT;

template <>
struct VT<double> {
    using X = double;
    using A = double;
    static __device__ __forceinline__ A stream1(const double *p) {
        double r;
        asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ A cached1(const double *p) { return __ldg(p); }
    static __device__ __forceinline__ A plain1(const double *p) { return *p; }  // any address space
};

template <>
struct VT<float> {
    using X = float;
    using A = float;
    static __device__ __forceinline__ A stream1(const float *p) {
        float r;
        asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(r) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ A cached1(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ A plain1(const float *p) { return *p; }  // any address space
    static __device__ __forceinline__ A from_bits(uint32_t u) { return __uint_as_float(u); }
};

template <>
struct VT<bf16x2_t> {
    using X = float;
    using A = float;
    static __device__ __forceinline__ A stream1(const bf16x2_t *p) {
        uint32_t u;
        asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(u) : "l"(p));
        return bf16x2_decode(u);
    }
    static __device__ __forceinline__ A cached1(const bf16x2_t *p) {
        return bf16x2_decode(__ldg((const unsigned *)p));
    }
    static __device__ __forceinline__ A plain1(const bf16x2_t *p) {  // any address space
        return bf16x2_decode(*(const unsigned *)p);
    }
    static __device__ __forceinline__ A from_bits(uint32_t u) { return bf16x2_decode(u); }
};

// Waits (once per thread) for the kernel this one is a programmatic
// dependent of, before the thread's first y update; *waited is the thread's
// flag, nullptr: nothing to wait for.
__device__ __forceinline__ void pdl_wait_once(bool *waited) {
    if (waited && !*waited) {
        asm volatile("griddepcontrol.wait;" ::: "memory");
        *waited = true;
    }
}

// y[r] += p for one 32-nonzero row of the stream (r = -1: no nonzero).
template <typename A, typename Y>
__device__ __forceinline__ void emit_row32(int r, A p, Y *__restrict__ y, int lane, bool *waited = nullptr) {
    pdl_wait_once(waited);
    const int prev = __shfl_up_sync(FULLM, r, 1);
    const bool join = lane > 0 && r >= 0 && prev == r;
    if (!__any_sync(FULLM, join)) {
        if (r >= 0) atomicAdd(y + r, (Y)p);
        return;
    }
    A S = p;
    int h = join ? 0 : 1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const A Sn = __shfl_up_sync(FULLM, S, o);
        const int hn = __shfl_up_sync(FULLM, h, o);
        if (lane >= o && !h) {
            S += Sn;
            h = hn;
        }
    }
    const int next = __shfl_down_sync(FULLM, r, 1);
    if ((lane == 31 || next != r) && r >= 0) atomicAdd(y + r, (Y)S);
}

// One work item; 4U rows of 32 nonzeros per warp iteration, all loads of an
// iteration issued before any is used.  An item is a serial chain of up to
// 16 iterations on one warp (a load of rows and values, then x gathers, then
// the y updates).
// waited: see pdl_wait_once (the first iteration's loads are issued before
// the wait).
template <typename V, typename Y, int U>
__device__ __forceinline__ void stream_item(const ItemDesc &d, const RegionDesc *__restrict__ regions,
                                            const int *__restrict__ row, const V *__restrict__ val,
                                            const typename VT<V>::X *__restrict__ xs, Y *__restrict__ y,
                                            int lane, bool *waited = nullptr) {
    using A = typename VT<V>::A;
    constexpr int R = 4 * U;
    const RegionDesc rg = regions[d.region];
    const int div = rg.div;
    const int s32 = rg.full ? 0 : 32 % div;  // partial chunk: column step per 32 nonzeros
    for (int e = d.begin & ~31; e < d.end; e += 32 * R) {
        const int el0 = e + lane;
        int rw[R];
        A v[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            rw[k] = ld_stream_i32(row + el0 + 32 * k);
            v[k] = VT<V>::stream1(val + el0 + 32 * k);
        }
        // columns of the lane's R nonzeros (they do not depend on the loads,
        // so every x gather is issued before any loaded value is used)
        const int q0 = el0 - rg.start;             // >= -31: items never start before their region
        const int k0 = q0 < 0 ? 1 : 0;
        const int qs = q0 + 32 * k0;
        int c = qs / div;
        int t = qs - c * div;
        const int lo = q0 & 31;
        // in a full region consecutive rows of a lane often share a column
        // (levels of one chunk): gather x only where the column changes
        typename VT<V>::X xv[R];
        bool fresh[R];
        int cprev = -1;
#pragma unroll
        for (int k = 0; k < R; k++) {
            if (k > k0) {  // advance the column state by 32 nonzeros
                if (rg.full) {
                    t += 32;
                    if (t >= div) { t -= div; c++; }
                } else {
                    t += s32;
                    if (t >= div) t -= div;
                }
            }
            const int el = el0 + 32 * k;
            const bool valid = el >= d.begin && el < d.end;
            const int col = rg.full ? rg.col_base + 32 * c + lo : rg.col_base + t;
            fresh[k] = valid && (!rg.full || c != cprev);
            if (fresh[k]) {
                xv[k] = __ldg(xs + col);
                cprev = c;
            }
        }
#pragma unroll
        for (int k = 0; k < R; k++) {
            const int el = el0 + 32 * k;
            const bool valid = el >= d.begin && el < d.end;
            if (k > 0 && !fresh[k]) xv[k] = xv[k - 1];
            emit_row32<A, Y>(valid ? rw[k] : -1, valid ? v[k] * (A)xv[k] : (A)0, y, lane, waited);
        }
    }
}

// Sorted column of nonzero e of a region.
__device__ __forceinline__ int region_col(int e, const RegionDesc &rg) {
    const int q = e - rg.start;
    return rg.full ? rg.col_base + 32 * (q / rg.div) + (q & 31) : rg.col_base + q % rg.div;
}

}  // namespace fl

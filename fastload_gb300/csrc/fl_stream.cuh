// fl_stream.cuh -- device side of the FastLoad streaming SpMV: 128-bit
// stream loads, per-nonzero column derivation from a region descriptor, and
// the run-merging warp reduction with one FP64 atomic per run.  Shared by the
// streaming kernel (fl_spmv.cu) and the light part of the bucketed kernel
// (fl_bucket.cu).
#pragma once

#include "fl_internal.cuh"

namespace fl {

constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ int4 ld_stream_i4(const int *p) {
    int4 r;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p));
    return r;
}
__device__ __forceinline__ double2 ld_stream_d2(const double *p) {
    double2 r;
    asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
    return r;
}

// Four consecutive nonzeros of one lane: products, run merging, atomics.
__device__ __forceinline__ void process4_f64(int eb, int4 rr, double2 va, double2 vb, const ItemDesc &d,
                                             const RegionDesc &rg, const double *__restrict__ xs,
                                             double *__restrict__ y, int lane) {
    int r[4] = {rr.x, rr.y, rr.z, rr.w};
    const double v[4] = {va.x, va.y, vb.x, vb.y};
    double p[4];
    // sorted column of each nonzero; one division per lane
    int qa = eb - rg.start;
    int qb = qa > 0 ? qa : 0;
    int c0 = qb / rg.div;
    int r0 = qb - c0 * rg.div;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int e = eb + k;
        bool valid = e >= d.begin && e < d.end;
        int delta = qa + k - qb;  // >= 0 whenever valid
        int col;
        if (rg.full) {
            int c = c0 + (r0 + delta >= rg.div ? 1 : 0);
            col = rg.col_base + 32 * c + ((qa + k) & 31);
        } else {
            int t = r0 + delta;
#pragma unroll
            for (int w = 0; w < 3; w++)
                if (t >= rg.div) t -= rg.div;
            col = rg.col_base + t;
        }
        if (valid) {
            p[k] = v[k] * __ldg(xs + col);
        } else {
            p[k] = 0.0;
            r[k] = -1;
        }
    }
    const bool b1 = r[1] != r[0], b2 = r[2] != r[1], b3 = r[3] != r[2];
    const int rf = r[0], rl = r[3];
    const int prev_rl = __shfl_up_sync(FULLM, rl, 1);
    const int next_rf = __shfl_down_sync(FULLM, rf, 1);
    const bool cont = lane > 0 && rf >= 0 && prev_rl == rf;
    const bool cont_next = lane < 31 && rl >= 0 && next_rf == rl;
    const bool merge = (!b1 && r[0] >= 0) || (!b2 && r[1] >= 0) || (!b3 && r[2] >= 0) || cont;
    if (!__any_sync(FULLM, merge)) {
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (r[k] >= 0) atomicAdd(y + r[k], p[k]);
        return;
    }
    // Trailing-run sum of the lane, then a segmented inclusive scan across
    // lanes: a lane continues the previous segment when all four of its
    // nonzeros are one run that started in an earlier lane.
    double T = p[3];
    if (!b3) {
        T += p[2];
        if (!b2) {
            T += p[1];
            if (!b1) T += p[0];
        }
    }
    const bool full_lane = !b1 && !b2 && !b3;
    double S = T;
    int h = (full_lane && cont) ? 0 : 1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double Sn = __shfl_up_sync(FULLM, S, o);
        int hn = __shfl_up_sync(FULLM, h, o);
        if (lane >= o && !h) {
            S += Sn;
            h = hn;
        }
    }
    const double Sp = __shfl_up_sync(FULLM, S, 1);
    const double C = cont ? Sp : 0.0;
    // runs ending inside the lane emit here; the lane's leading run adds the
    // carry from earlier lanes; the trailing run emits unless the next lane
    // continues it.
    double acc = p[0];
    bool lead = true;
    const bool brk[4] = {false, b1, b2, b3};
#pragma unroll
    for (int k = 1; k < 4; k++) {
        if (brk[k]) {
            if (r[k - 1] >= 0) atomicAdd(y + r[k - 1], lead ? acc + C : acc);
            acc = p[k];
            lead = false;
        } else {
            acc += p[k];
        }
    }
    if (!cont_next && r[3] >= 0) atomicAdd(y + r[3], S);
}

// One work item: 128*U nonzeros per warp iteration, loads of the U blocks
// issued before any of them is processed.
template <int U>
__device__ __forceinline__ void stream_item_f64(const ItemDesc &d, const RegionDesc *__restrict__ regions,
                                                const int *__restrict__ row, const double *__restrict__ val,
                                                const double *__restrict__ xs, double *__restrict__ y,
                                                int lane) {
    const RegionDesc rg = regions[d.region];
    for (int e = d.begin & ~3; e < d.end; e += 128 * U) {
        int4 rr[U];
        double2 va[U], vb[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int eb = e + 128 * u + 4 * lane;
            rr[u] = ld_stream_i4(row + eb);
            va[u] = ld_stream_d2(val + eb);
            vb[u] = ld_stream_d2(val + eb + 2);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int eb = e + 128 * u + 4 * lane;
            process4_f64(eb, rr[u], va[u], vb[u], d, rg, xs, y, lane);
        }
    }
}

}  // namespace fl

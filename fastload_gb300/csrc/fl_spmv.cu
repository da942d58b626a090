// fl_spmv.cu -- FP64 FastLoad SpMV kernels for sm_103a.
//
// Both kernels compute y += A xs over the FastLoad tile layout (the
// reference's FastLoad___kernel, src/FastLoad_GPU.h:146-273): xs is x in
// sorted column order, y in original row order, one FP64 atomic per run of
// equal consecutive rows.
//
//  * k_spmv_tile_f64: one warp per reference tile, reading the reference's
//    per-tile arrays (tile_ptr/len/colidx/format, sortrowindex) -- the
//    reference's kernel design, rebuilt for CUDA 13 with its defects fixed
//    (in-bounds loads, _sync shuffles, one product per lane).
//  * k_spmv_stream_f64: the streaming kernel.  It reads no per-tile metadata:
//    the tile-ordered value/row streams are cut into work items, each lane
//    takes four consecutive nonzeros with 128-bit loads, derives each one's
//    sorted column arithmetically from the step table (full 32-wide chunks:
//    col = col_base + 32*(q / (32*tall)) + q%32; partial chunk:
//    col = col_base + q % len) and gathers x through L1.  Runs of equal rows
//    are merged by a warp-wide segmented scan over the 128-nonzero block
//    (__shfl_sync), skipped when a ballot shows the block has none, so the
//    common case spends exactly one FP64 multiply per nonzero -- GB300's FP64
//    pipe is narrow and would otherwise bound the kernel.
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

template <int U>
__global__ void __launch_bounds__(256) k_spmv_stream_f64(const ItemDesc *__restrict__ items, int nitems,
                                                         const RegionDesc *__restrict__ regions,
                                                         const int *__restrict__ row,
                                                         const double *__restrict__ val,
                                                         const double *__restrict__ xs, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = gw; it < nitems; it += nw) {
        const ItemDesc d = items[it];
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
}

// One warp per reference tile (FastLoad_GPU.h:170-271): format 0 tiles add
// lane by lane; format 1/2 tiles sum each run (heads marked by sortrowindex)
// with a segmented scan and add once per run at the run's last lane.
__global__ void __launch_bounds__(256) k_spmv_tile_f64(int tilenum, const int *__restrict__ tile_ptr,
                                                       const int *__restrict__ tile_len,
                                                       const int *__restrict__ tile_colidx,
                                                       const int *__restrict__ tile_format,
                                                       const int *__restrict__ sortrowindex,
                                                       const int *__restrict__ row,
                                                       const double *__restrict__ val,
                                                       const double *__restrict__ xs, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    long gw = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long t = gw; t < tilenum; t += nw) {
        const int len = __ldg(tile_len + t), ptr = __ldg(tile_ptr + t);
        const int colidx = __ldg(tile_colidx + t), fmt = __ldg(tile_format + t);
        const bool act = lane < len;
        int r = -1;
        double v = 0.0;
        if (act) {
            r = __ldg(row + ptr + lane);
            v = __ldg(val + ptr + lane) * __ldg(xs + colidx + lane);
        }
        if (fmt == 0) {
            if (act) atomicAdd(y + r, v);
            continue;
        }
        const int head = __ldg(sortrowindex + ptr + lane) != 0;
        const int next_head = __shfl_down_sync(FULLM, head, 1);
        double S = v;
        int h = head;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double Sn = __shfl_up_sync(FULLM, S, o);
            int hn = __shfl_up_sync(FULLM, h, o);
            if (lane >= o && !h) {
                S += Sn;
                h = hn;
            }
        }
        if (lane == 31 || next_head) atomicAdd(y + r, S);
    }
}

static int occupancy_grid(const void *fn, int threads, long work_warps) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    if (per_sm <= 0) per_sm = 1;
    long g = (long)num_sms() * per_sm;
    long need = (work_warps * 32 + threads - 1) / threads;
    if (need < g) g = need;
    return (int)(g > 0 ? g : 1);
}

int spmv_stream_f64(const Layout &L, const double *xs, double *y, int variant, cudaStream_t s) {
    const Regions &R = L.regions;
    if (R.nitems == 0) return FL_SUCCESS;
    if (variant == FL_KERNEL_STREAM) {
        static int g = 0;
        int grid = occupancy_grid((const void *)k_spmv_stream_f64<1>, 256, R.nitems);
        (void)g;
        k_spmv_stream_f64<1><<<grid, 256, 0, s>>>(R.item.get(), R.nitems, R.region.get(), L.row.get(),
                                                  L.val.get(), xs, y);
    } else {
        int grid = occupancy_grid((const void *)k_spmv_stream_f64<2>, 256, R.nitems);
        k_spmv_stream_f64<2><<<grid, 256, 0, s>>>(R.item.get(), R.nitems, R.region.get(), L.row.get(),
                                                  L.val.get(), xs, y);
    }
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

int spmv_tile_f64(const Layout &L, const double *xs, double *y, cudaStream_t s) {
    if (L.tilenum == 0) return FL_SUCCESS;
    if (!L.tile_ptr.get()) return fail(FL_ERR_ARG, "tile kernel needs a plan built with reference arrays");
    int grid = occupancy_grid((const void *)k_spmv_tile_f64, 256, L.tilenum);
    k_spmv_tile_f64<<<grid, 256, 0, s>>>(L.tilenum, L.tile_ptr.get(), L.tile_len.get(), L.tile_colidx.get(),
                                         L.tile_format.get(), L.sortrowindex.get(), L.row.get(), L.val.get(),
                                         xs, y);
    FL_CUDA(cudaGetLastError());
    return FL_SUCCESS;
}

}  // namespace fl

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
//  * k_spmv_stream_f64: the streaming kernel (fl_stream.cuh).  It reads no
//    per-tile metadata: the tile-ordered value/row streams are cut into work
//    items walked 32 nonzeros per warp row, each nonzero's sorted column
//    derived arithmetically from the step table, x gathered through L1, runs
//    of equal rows merged by a segmented shuffle scan only when present -- so
//    the common case spends exactly one FP64 multiply per nonzero (GB300's
//    FP64 pipe is narrow and would otherwise bound the kernel).
#include "fl_stream.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

namespace fl {

template <int U>
__global__ void __launch_bounds__(256) k_spmv_stream_f64(const ItemDesc *__restrict__ items, int nitems,
                                                         const RegionDesc *__restrict__ regions,
                                                         const int *__restrict__ row,
                                                         const double *__restrict__ val,
                                                         const double *__restrict__ xs, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = gw; it < nitems; it += nw) stream_item<double, double, U>(items[it], regions, row, val, xs, y, lane);
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
    // resident blocks per SM of (kernel, block size): queried once, the query
    // costs host time on every call otherwise
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find({fn, threads});
        if (it != cache.end()) {
            per_sm = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess) {
                cudaGetLastError();
                per_sm = 0;
            }
            if (per_sm > 0) cache[{fn, threads}] = per_sm;
        }
    }
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
        int grid = occupancy_grid((const void *)k_spmv_stream_f64<1>, 256, R.nitems);
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

// y = 0 ahead of an accumulating SpMV kernel.  Launched as a programmatic
// dependent of the kernel before it (griddepcontrol): its blocks may be
// scheduled while that kernel drains, wait for it to finish, then release
// the SpMV kernel behind them before storing, so the two launches overlap
// their start-up.  words: 4-byte words; p16: p is 16-byte aligned.
__global__ void __launch_bounds__(512) k_zero_words(unsigned *p, long words, int p16) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x, T = (long)gridDim.x * blockDim.x;
    long head = 0;
    if (p16) {
        const long n4 = words >> 2;
        uint4 *q = reinterpret_cast<uint4 *>(p);
        for (long i = t; i < n4; i += T) q[i] = make_uint4(0u, 0u, 0u, 0u);
        head = n4 << 2;
    }
    for (long i = head + t; i < words; i += T) p[i] = 0u;
}

int zero_device(void *p, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return FL_SUCCESS;
    if (bytes % 4 || (uintptr_t)p % 4) return fail(FL_ERR_ARG, "zero_device: %zu bytes at %p", bytes, p);
    const long words = (long)(bytes / 4);
    const int p16 = (uintptr_t)p % 16 == 0;
    const long per_block = 512L * 16 * 4;  // 16 bytes per thread per pass, about four passes
    const long grid = std::max<long>(1, std::min<long>((long)num_sms() * 4, ((long)bytes + per_block - 1) / per_block));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(512);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FL_CUDA(cudaLaunchKernelEx(&cfg, k_zero_words, (unsigned *)p, words, p16));
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

// fl_cache.cu -- persistent plan files: the preprocessed FastLoad format of a
// plan written to disk and read back into a device plan.
//
// The reference rebuilds its format on every run and re-uploads it on every
// FastLoad_spmv call (src/FastLoad_GPU.h:318-327, called from
// src/main.cu:314).  A plan file keeps the format itself -- the column
// permutation, the nonzeros per sorted column and the tile-ordered row and
// value streams (the reference's sortrowidx / sortval) -- plus the plan's
// options: reference arrays on or off, the heavy band and the forms.
//
// File layout (little-endian; offsets in bytes):
//     0  char     magic[8]      "FLGBPLAN"
//     8  uint32   version       2 (1 is read too)
//    12  uint32   header_bytes  128
//    16  uint32   byte_order    0x01020304
//    20  int32    m, n, nnz
//    32  int32    tilenum, steps
//    40  int32    with_reference_arrays
//    44  int32    heavy         -1: no heavy band, else its requested width
//    48  int32    nforms
//    52  int32    reserved (0)
//    56  uint64   hash of perm, sortnnz, row, val, forms (5 words)
//    96  uint64   reserved (0) x 3
//   120  uint64   hash of bytes 0..119
//   128  int32    perm[n]       sorted position -> original column
//        int32    sortnnz[n]    nonzeros per sorted column (ascending)
//        int32    row[nnz]      tile-ordered row indices
//        float64  val[nnz]      tile-ordered values
//        int32    forms[8*nforms]  per form its fl_form_opts: value type,
//                                  heavy band, y_f32, light item, heavy
//                                  loop, x staging, units per warp, 0
//                                  (version 1: the first three only)
//
// Hash: 64-bit FNV-1a over little-endian 64-bit words (the tail zero-padded
// to a full word), then xor-ed with the byte count.  Loading checks the
// header, every hash and the file size, then validates the content the way
// fl_plan_create validates device input: perm is a permutation of [0, n),
// sortnnz is ascending and sums to nnz, rows lie in [0, m).  The layout is
// then rebuilt from the stored streams by the same deterministic device code
// fl_plan_create uses, so a loaded plan equals the saved one array for array.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "fl_internal.cuh"

namespace fl {
namespace {

constexpr char kMagic[8] = {'F', 'L', 'G', 'B', 'P', 'L', 'A', 'N'};
constexpr uint32_t kVersion = 2;
constexpr int kFormInts = 8;  // fl_form_opts, as int32 (version 1: 3)
constexpr uint32_t kHeaderBytes = 128;
constexpr uint32_t kByteOrder = 0x01020304u;
constexpr int kMaxForms = 1024;

struct FileHeader {
    char magic[8];
    uint32_t version, header_bytes, byte_order;
    int32_t m, n, nnz, tilenum, steps, with_ref, heavy, nforms, reserved0;
    uint64_t hash[5];
    uint64_t reserved[3];
    uint64_t header_hash;
};
static_assert(sizeof(FileHeader) == kHeaderBytes, "plan file header must be 128 bytes");

uint64_t hash_bytes(const void *data, size_t bytes) {
    const unsigned char *p = (const unsigned char *)data;
    uint64_t h = 0xcbf29ce484222325ull;
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t w;
        memcpy(&w, p + i, 8);
        h = (h ^ w) * 0x100000001b3ull;
    }
    if (i < bytes) {
        uint64_t w = 0;
        memcpy(&w, p + i, bytes - i);
        h = (h ^ w) * 0x100000001b3ull;
    }
    return h ^ (uint64_t)bytes;
}

struct File {
    FILE *f = nullptr;
    ~File() { if (f) fclose(f); }
};

int write_all(FILE *f, const void *p, size_t bytes, const char *path) {
    if (bytes && fwrite(p, 1, bytes, f) != bytes) return fail(FL_ERR_IO, "plan_save: write to %s failed", path);
    return FL_SUCCESS;
}

int read_all(FILE *f, void *p, size_t bytes, const char *path) {
    if (bytes && fread(p, 1, bytes, f) != bytes)
        return fail(FL_ERR_IO, "plan_load: %s is truncated", path);
    return FL_SUCCESS;
}

template <typename T>
int to_host(std::vector<T> &h, const T *d, size_t count, cudaStream_t s) {
    h.resize(count);
    if (count) FL_CUDA(cudaMemcpyAsync(h.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    return FL_SUCCESS;
}

// seen[v]++ for every value; err when a value is out of range or repeated.
__global__ void k_perm_count(const int *perm, int n, int *seen, int *err) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        int v = perm[i];
        if (v < 0 || v >= n) atomicOr(err, 1);
        else if (atomicAdd(seen + v, 1) != 0) atomicOr(err, 2);
    }
}

__global__ void k_fill_pad_stream(int *row, double *val, long from, long to) {
    for (long i = from + blockIdx.x * (long)blockDim.x + threadIdx.x; i < to; i += (long)gridDim.x * blockDim.x) {
        row[i] = -1;
        val[i] = 0.0;
    }
}

int grid(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, (long)num_sms() * 8)); }

int check_perm(const int *perm, int n, cudaStream_t s) {
    if (n == 0) return FL_SUCCESS;
    DevBuf<int> seen, err;
    FL_TRY(seen.alloc(n, s));
    FL_TRY(err.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(seen.get(), 0, (size_t)n * sizeof(int), s));
    FL_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), s));
    k_perm_count<<<grid(n), 256, 0, s>>>(perm, n, seen.get(), err.get());
    FL_CUDA(cudaGetLastError());
    int h = 0;
    FL_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (h) return fail(FL_ERR_ARG, "plan_load: the column permutation is not a permutation of [0, %d)", n);
    return FL_SUCCESS;
}

}  // namespace
}  // namespace fl

using namespace fl;

extern "C" int fl_plan_save(fl_plan_t p, const char *path) {
    clear_error();
    if (!p || !path) return fail(FL_ERR_ARG, "plan_save: NULL argument");
    const Layout &L = p->L;
    const cudaStream_t s = 0;
    FL_CUDA(cudaDeviceSynchronize());
    std::vector<int> perm, sortnnz, row, forms;
    std::vector<double> val;
    FL_TRY(to_host(perm, L.perm.get(), L.n, s));
    FL_TRY(to_host(sortnnz, L.sortnnz.get(), L.n, s));
    FL_TRY(to_host(row, L.row.get(), L.nnz, s));
    FL_TRY(to_host(val, L.val.get(), L.nnz, s));
    FL_CUDA(cudaStreamSynchronize(s));
    static_assert(sizeof(fl_form_opts) == kFormInts * sizeof(int32_t), "form options are 8 int32");
    for (const auto &F : p->forms) {
        const fl_form_opts &o = F->opts;
        const int v[kFormInts] = {o.value_type, o.heavy_band, o.y_f32, o.light_item,
                                  o.heavy_loop, o.x_stage,    o.unit_warps, 0};
        forms.insert(forms.end(), v, v + kFormInts);
    }
    FileHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = kHeaderBytes;
    h.byte_order = kByteOrder;
    h.m = L.m;
    h.n = L.n;
    h.nnz = L.nnz;
    h.tilenum = L.tilenum;
    h.steps = L.st.steps;
    h.with_ref = p->has_ref ? 1 : 0;
    h.heavy = p->bucket ? L.n - p->bucket->heavy.H0 : -1;
    h.nforms = (int)p->forms.size();
    h.hash[0] = hash_bytes(perm.data(), perm.size() * 4);
    h.hash[1] = hash_bytes(sortnnz.data(), sortnnz.size() * 4);
    h.hash[2] = hash_bytes(row.data(), row.size() * 4);
    h.hash[3] = hash_bytes(val.data(), val.size() * 8);
    h.hash[4] = hash_bytes(forms.data(), forms.size() * 4);
    h.header_hash = hash_bytes(&h, offsetof(FileHeader, header_hash));
    File f;
    f.f = fopen(path, "wb");
    if (!f.f) return fail(FL_ERR_IO, "plan_save: cannot open %s for writing", path);
    FL_TRY(write_all(f.f, &h, sizeof h, path));
    FL_TRY(write_all(f.f, perm.data(), perm.size() * 4, path));
    FL_TRY(write_all(f.f, sortnnz.data(), sortnnz.size() * 4, path));
    FL_TRY(write_all(f.f, row.data(), row.size() * 4, path));
    FL_TRY(write_all(f.f, val.data(), val.size() * 8, path));
    FL_TRY(write_all(f.f, forms.data(), forms.size() * 4, path));
    FILE *raw = f.f;
    f.f = nullptr;
    if (fclose(raw) != 0) return fail(FL_ERR_IO, "plan_save: closing %s failed", path);
    return FL_SUCCESS;
}

extern "C" int fl_plan_load(fl_plan_t *out, const char *path, void *stream) {
    clear_error();
    if (!out || !path) return fail(FL_ERR_ARG, "plan_load: NULL argument");
    *out = nullptr;
    const cudaStream_t s = (cudaStream_t)stream;
    File f;
    f.f = fopen(path, "rb");
    if (!f.f) return fail(FL_ERR_IO, "plan_load: cannot open %s", path);
    FileHeader h;
    if (fread(&h, 1, sizeof h, f.f) != sizeof h) return fail(FL_ERR_IO, "plan_load: %s is not a plan file", path);
    if (memcmp(h.magic, kMagic, 8) != 0) return fail(FL_ERR_IO, "plan_load: %s is not a plan file", path);
    if ((h.version != kVersion && h.version != 1) || h.header_bytes != kHeaderBytes || h.byte_order != kByteOrder)
        return fail(FL_ERR_IO, "plan_load: %s has version %u / header %u / byte order 0x%08x (expected %u or 1/%u/0x%08x)",
                    path, h.version, h.header_bytes, h.byte_order, kVersion, kHeaderBytes, kByteOrder);
    const int fi = h.version == 1 ? 3 : kFormInts;  // ints per form
    if (hash_bytes(&h, offsetof(FileHeader, header_hash)) != h.header_hash)
        return fail(FL_ERR_IO, "plan_load: %s: header checksum mismatch", path);
    if (h.m < 0 || h.n < 0 || h.nnz < 0 || h.nforms < 0 || h.nforms > kMaxForms || h.heavy < -1 || h.heavy > h.n)
        return fail(FL_ERR_IO, "plan_load: %s: header out of range (m=%d n=%d nnz=%d forms=%d heavy=%d)", path, h.m,
                    h.n, h.nnz, h.nforms, h.heavy);
    const int m = h.m, n = h.n, nnz = h.nnz;
    const long expect = (long)kHeaderBytes + 8L * n + 12L * nnz + 4L * fi * h.nforms;
    if (fseek(f.f, 0, SEEK_END) != 0) return fail(FL_ERR_IO, "plan_load: cannot seek in %s", path);
    const long size = ftell(f.f);
    if (size != expect)
        return fail(FL_ERR_IO, "plan_load: %s has %ld bytes, the header implies %ld", path, size, expect);
    if (fseek(f.f, kHeaderBytes, SEEK_SET) != 0) return fail(FL_ERR_IO, "plan_load: cannot seek in %s", path);
    std::vector<int> perm(n), sortnnz(n), row(nnz), forms((size_t)fi * h.nforms);
    std::vector<double> val(nnz);
    FL_TRY(read_all(f.f, perm.data(), perm.size() * 4, path));
    FL_TRY(read_all(f.f, sortnnz.data(), sortnnz.size() * 4, path));
    FL_TRY(read_all(f.f, row.data(), row.size() * 4, path));
    FL_TRY(read_all(f.f, val.data(), val.size() * 8, path));
    FL_TRY(read_all(f.f, forms.data(), forms.size() * 4, path));
    const uint64_t got[5] = {hash_bytes(perm.data(), perm.size() * 4), hash_bytes(sortnnz.data(), sortnnz.size() * 4),
                             hash_bytes(row.data(), row.size() * 4), hash_bytes(val.data(), val.size() * 8),
                             hash_bytes(forms.data(), forms.size() * 4)};
    static const char *names[5] = {"permutation", "column counts", "row stream", "value stream", "form list"};
    for (int i = 0; i < 5; i++)
        if (got[i] != h.hash[i]) return fail(FL_ERR_IO, "plan_load: %s: %s checksum mismatch", path, names[i]);

    std::unique_ptr<fl_plan> p(new (std::nothrow) fl_plan());
    if (!p) return fail(FL_ERR_ALLOC, "plan_load: host allocation failed");
    Layout &L = p->L;
    FL_TRY(L.perm.alloc(n, s));
    FL_TRY(L.sortnnz.alloc(n, s));
    if (n) {
        FL_CUDA(cudaMemcpyAsync(L.perm.get(), perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
        FL_CUDA(cudaMemcpyAsync(L.sortnnz.get(), sortnnz.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    }
    FL_TRY(check_perm(L.perm.get(), n, s));
    // the stored streams in a scratch layout: step table from the column
    // counts (which validates them), then back to the column-sorted CSC
    DevBuf<int> srow;
    DevBuf<double> sval;
    {
        Layout T;
        FL_TRY(build_steps(T, m, n, nnz, L.sortnnz.get(), s));
        if (T.tilenum != h.tilenum || T.st.steps != h.steps)
            return fail(FL_ERR_IO, "plan_load: %s: column counts imply %d tiles / %d steps, the header says %d / %d",
                        path, T.tilenum, T.st.steps, h.tilenum, h.steps);
        const size_t np = padded(nnz);
        FL_TRY(T.row.alloc(np, s));
        FL_TRY(T.val.alloc(np, s));
        FL_TRY(T.sortnnz.alloc(n, s));
        if (n) FL_CUDA(cudaMemcpyAsync(T.sortnnz.get(), L.sortnnz.get(), (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        if (nnz) {
            FL_CUDA(cudaMemcpyAsync(T.row.get(), row.data(), (size_t)nnz * 4, cudaMemcpyHostToDevice, s));
            FL_CUDA(cudaMemcpyAsync(T.val.get(), val.data(), (size_t)nnz * 8, cudaMemcpyHostToDevice, s));
        }
        k_fill_pad_stream<<<grid((long)(np - nnz)), 256, 0, s>>>(T.row.get(), T.val.get(), nnz, (long)np);
        FL_CUDA(cudaGetLastError());
        FL_TRY(check_index_range(T.row.get(), nnz, m, "plan_load: row index", s));
        FL_TRY(untile_layout(T, srow, sval, s));
        FL_CUDA(cudaStreamSynchronize(s));
    }
    FL_TRY(build_layout_device(L, m, n, nnz, L.sortnnz.get(), srow.get(), sval.get(), h.with_ref != 0, s, nullptr,
                               nullptr));
    p->has_ref = h.with_ref != 0;
    if (h.heavy >= 0) {
        p->bucket.reset(new (std::nothrow) Bucket());
        if (!p->bucket) return fail(FL_ERR_ALLOC, "plan_load: host allocation failed");
        // bands wider than shared memory hold x (every column, x through the
        // cache) are rebuilt the way they were built
        FL_TRY(build_bucket(*p->bucket, m, n, nnz, L.sortnnz.get(), srow.get(), sval.get(), h.heavy, s,
                            h.heavy > bucket_max_band()));
    }
    srow.release();
    sval.release();
    FL_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < h.nforms; i++) {
        std::unique_ptr<Form> F(new (std::nothrow) Form());
        if (!F) return fail(FL_ERR_ALLOC, "plan_load: host allocation failed");
        fl_form_opts o = {};
        const int *v = forms.data() + (size_t)fi * i;
        o.value_type = v[0];
        o.heavy_band = v[1];
        o.y_f32 = v[2] != 0;
        if (fi == kFormInts) {
            o.light_item = v[3];
            o.heavy_loop = v[4];
            o.x_stage = v[5];
            o.unit_warps = v[6];
            o.reserved = v[7];
        }
        FL_TRY(build_form(*F, L, o, s));
        p->forms.push_back(std::move(F));
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(FL_ERR_CUDA, "plan_load: %s", cudaGetErrorString(e));
    *out = p.release();
    return FL_SUCCESS;
}

// fl_tune.cu -- the learned tuner on the C ABI: the variant table the
// autotuner times and the network chooses among, and the tuned form.
//
// A variant is a complete set of form options (fl_form_opts): the heavy
// band (bucket threshold), the light columns' work-item size, the heavy
// band's loop (shared-memory ring or loads in registers), where the band
// reads x (staged in shared memory or through the cache), the heavy work
// units per warp, and the value storage (the caller's type, or BF16 hi+lo
// for callers asking for FP32 values).  The network (24 plan features ->
// 64 -> 64 -> one predicted log-time per variant) is trained by the
// project's own kernels (fl_mlp.cu) on the autotuner's timings; its file
// carries the variant table it was trained on, which must equal this one.
//
// Model file (little-endian):
//     0  char    magic[8]     "FLTUNER1"
//     8  int32   n_in, h1, h2, n_out, n_variants, 0, 0, 0
//    40  float   mu[n_in], sd[n_in]     feature scaling
//        float   params[...]            W1, b1, W2, b2, W3, b3 (fl_mlp order)
//        int32   variants[8 * n_variants]  the fl_form_opts of each output
#include <stdio.h>
#include <string.h>

#include <memory>
#include <vector>

#include "fl_internal.cuh"

namespace {

constexpr char kModelMagic[8] = {'F', 'L', 'T', 'U', 'N', 'E', 'R', '1'};
constexpr int kFeatures = 24;

// Built once: for each storage (the caller's type, then BF16 hi+lo) the
// library default, the tile stream alone with three item sizes, every
// column in the band with two unit sizes, and three band widths (8,192,
// 24,576 and 49,152 columns) crossed with three light item sizes and three
// heavy-band loops (ring, registers with x staged, registers with x read
// through the cache).
std::vector<fl_form_opts> make_table() {
    std::vector<fl_form_opts> t;
    auto add = [&](int vt, int band, int light, int heavy, int xs, int units) {
        fl_form_opts o = {};
        o.value_type = vt;
        o.heavy_band = band;
        o.light_item = light;
        o.heavy_loop = heavy;
        o.x_stage = xs;
        o.unit_warps = units;
        t.push_back(o);
    };
    const int lights[3] = {0, 512, 1024};
    for (int vt : {FL_TUNE_REQUESTED, FL_VALUES_BF16X2}) {
        add(vt, FL_BAND_AUTO, 0, FL_HEAVY_AUTO, FL_XSTAGE_AUTO, 0);
        for (int l : lights) add(vt, FL_BAND_NONE, l, FL_HEAVY_AUTO, FL_XSTAGE_AUTO, 0);
        for (int u : {0, 4}) add(vt, FL_BAND_ALL, 0, FL_HEAVY_AUTO, FL_XSTAGE_AUTO, u);
        for (int band : {8192, 24576, 49152})
            for (int l : lights) {
                add(vt, band, l, FL_HEAVY_RING, FL_XSTAGE_AUTO, 0);
                add(vt, band, l, FL_HEAVY_REGS, FL_XSTAGE_AUTO, 0);
                add(vt, band, l, FL_HEAVY_REGS, FL_XSTAGE_GLOBAL, 0);
            }
    }
    return t;
}

const std::vector<fl_form_opts> &table() {
    static const std::vector<fl_form_opts> t = make_table();
    return t;
}

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

int read_exact(FILE *f, void *dst, size_t bytes, const char *path) {
    if (fread(dst, 1, bytes, f) != bytes) return fl::fail(FL_ERR_IO, "tuned_form: %s is truncated", path);
    return FL_SUCCESS;
}

}  // namespace

using namespace fl;

extern "C" int fl_tuner_variants(fl_form_opts *out, int max) {
    clear_error();
    const auto &t = table();
    if (out)
        for (int i = 0; i < max && i < (int)t.size(); i++) out[i] = t[i];
    return (int)t.size();
}

extern "C" int fl_plan_add_tuned_form(fl_plan_t plan, const char *model_path, int value_type, int y_f32, int *form_id,
                                      int *variant) {
    clear_error();
    if (!plan || !model_path || !form_id) return fail(FL_ERR_ARG, "tuned_form: NULL argument");
    if (value_type != FL_VALUES_F64 && value_type != FL_VALUES_F32)
        return fail(FL_ERR_ARG, "tuned_form: value type %d (FP64 or FP32; FP32 callers may get BF16 hi+lo)",
                    value_type);
    if (y_f32 && value_type != FL_VALUES_F32) return fail(FL_ERR_ARG, "tuned_form: FP32 y needs FP32 values");
    const auto &t = table();
    // the model file
    File f;
    f.f = fopen(model_path, "rb");
    if (!f.f) return fail(FL_ERR_IO, "tuned_form: cannot open %s", model_path);
    char magic[8];
    int32_t hd[8];
    FL_TRY(read_exact(f.f, magic, 8, model_path));
    if (memcmp(magic, kModelMagic, 8) != 0) return fail(FL_ERR_IO, "tuned_form: %s is not a tuner model", model_path);
    FL_TRY(read_exact(f.f, hd, sizeof hd, model_path));
    const int n_in = hd[0], h1 = hd[1], h2 = hd[2], n_out = hd[3], nv = hd[4];
    if (n_in != kFeatures || h1 < 1 || h1 > 4096 || h2 < 1 || h2 > 4096 || n_out != nv || nv < 1 || nv > 4096)
        return fail(FL_ERR_IO, "tuned_form: %s: network %d -> %d -> %d -> %d with %d variants", model_path, n_in, h1,
                    h2, n_out, nv);
    if (nv != (int)t.size())
        return fail(FL_ERR_ARG, "tuned_form: %s was trained on %d variants, the library has %d", model_path, nv,
                    (int)t.size());
    const long np = (long)n_in * h1 + h1 + (long)h1 * h2 + h2 + (long)h2 * n_out + n_out;
    std::vector<float> mu(n_in), sd(n_in), params(np);
    std::vector<fl_form_opts> vars(nv);
    FL_TRY(read_exact(f.f, mu.data(), mu.size() * 4, model_path));
    FL_TRY(read_exact(f.f, sd.data(), sd.size() * 4, model_path));
    FL_TRY(read_exact(f.f, params.data(), params.size() * 4, model_path));
    FL_TRY(read_exact(f.f, vars.data(), vars.size() * sizeof(fl_form_opts), model_path));
    char extra;
    if (fread(&extra, 1, 1, f.f) != 0) return fail(FL_ERR_IO, "tuned_form: %s has trailing bytes", model_path);
    for (int i = 0; i < nv; i++)
        if (memcmp(&vars[i], &t[i], sizeof(fl_form_opts)) != 0)
            return fail(FL_ERR_ARG, "tuned_form: %s: variant %d differs from the library's table", model_path, i);
    for (int i = 0; i < n_in; i++)
        if (!(sd[i] > 0.0f)) return fail(FL_ERR_IO, "tuned_form: %s: feature scale %d is %g", model_path, i, sd[i]);
    // features -> network on the GPU
    float feat[kFeatures];
    FL_TRY(fl_plan_features(plan, value_type, feat));
    for (int i = 0; i < n_in; i++) feat[i] = (feat[i] - mu[i]) / sd[i];
    fl_mlp_t net = nullptr;
    FL_TRY(fl_mlp_create(&net, n_in, h1, h2, n_out, 0));
    std::unique_ptr<fl_mlp, int (*)(fl_mlp_t)> guard(net, fl_mlp_destroy);
    FL_TRY(fl_mlp_set_params(net, params.data()));
    std::vector<float> pred(n_out);
    FL_TRY(fl_mlp_forward(net, feat, 1, pred.data()));
    // the allowed variant with the lowest predicted time
    int best = -1;
    for (int i = 0; i < nv; i++) {
        const bool bf16 = t[i].value_type == FL_VALUES_BF16X2;
        if (bf16 && (value_type != FL_VALUES_F32 || y_f32)) continue;
        if (best < 0 || pred[i] < pred[best]) best = i;
    }
    if (best < 0) return fail(FL_ERR_INTERNAL, "tuned_form: no variant allowed");
    fl_form_opts o = t[best];
    if (o.value_type == FL_TUNE_REQUESTED) o.value_type = value_type;
    o.y_f32 = y_f32 != 0;
    FL_TRY(fl_plan_add_form_opts(plan, &o, form_id));
    if (variant) *variant = best;
    return FL_SUCCESS;
}

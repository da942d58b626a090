// fl_form_bf16.cu -- instantiations of the form kernels for BF16 hi+lo
// values (FP32 products, FP64 y).
#include "fl_forms.cuh"

namespace fl {
int run_form_bf16(const FormArgs<bf16x2_t, double> &a, int k, bool wide, cudaStream_t s) {
    return dispatch_form<bf16x2_t, double>(a, k, wide, s);
}
}  // namespace fl

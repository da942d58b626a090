// fl_form_f32.cu -- instantiations of the form kernels for FP32 values, with
// FP64 y and with FP32 y (the batched form's FP32 accumulation).
#include "fl_forms.cuh"

namespace fl {
int run_form_f32(const FormArgs<float, double> &a, int k, bool wide, cudaStream_t s) {
    return dispatch_form<float, double>(a, k, wide, s);
}
int run_form_f32_y32(const FormArgs<float, float> &a, int k, bool wide, cudaStream_t s) {
    return dispatch_form<float, float>(a, k, wide, s);
}
}  // namespace fl

// fl_form_f64.cu -- instantiations of the form kernels for FP64 values
// (one translation unit per storage type so they compile in parallel).
#include "fl_forms.cuh"

namespace fl {
int run_form_f64(const FormArgs<double, double> &a, int k, bool wide, cudaStream_t s) {
    return dispatch_form<double, double>(a, k, wide, s);
}
}  // namespace fl

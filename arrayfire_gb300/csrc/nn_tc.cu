// Tensor-core (tcgen05/TMEM) NN convolution kernels: BF16 and FP8-E4M3
// forms of af_convolve2_nn and its gradients.
#include "nn_conv.hpp"

namespace afgb {

bool tc_forward(const NNGeom &, const Array &, const Array &, Array &, afgb_precision,
                const Array *) {
    return false;
}
bool tc_data_grad(const NNGeom &, const Array &, const Array &, Array &) { return false; }
bool tc_filter_grad(const NNGeom &, const Array &, const Array &, Array &) { return false; }

}  // namespace afgb

// Mixed-precision (FP32 integrand) instantiation of the channel-task kernel.
#include "pffrg_flow.cuh"

namespace pffrg {

template <>
cudaError_t launch_pass<float>(const PassArgs<float>& a, cudaStream_t st) {
    return launch_pass_impl<float>(a, st);
}

}  // namespace pffrg

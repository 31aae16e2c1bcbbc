// Mixed-precision (FP32 integrand) instantiation of the channel-task kernel.
#include "pffrg_flow.cuh"

namespace pffrg {

template <>
cudaError_t launch_pass<float>(const PassArgs<float>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    if (a.L.C == 6) return launch_pass_u1dm<float>(a, Wsp, h_counters, st);
    return launch_pass_impl<float, 2>(a, Wsp, h_counters, st);
}

}  // namespace pffrg

// FP64 instantiation of the channel-task kernel.
#include "pffrg_flow.cuh"

namespace pffrg {

template <>
cudaError_t launch_pass<double>(const PassArgs<double>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    return launch_pass_impl<double>(a, Wsp, h_counters, st);
}

}  // namespace pffrg

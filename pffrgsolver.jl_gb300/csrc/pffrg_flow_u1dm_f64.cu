// FP64 instantiation of the channel-task kernel for U(1)-DM vertices (six components).
#include "pffrg_flow.cuh"

namespace pffrg {

template <>
cudaError_t launch_pass_u1dm<double>(const PassArgs<double>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    return launch_pass_impl<double, 6>(a, Wsp, h_counters, st);
}

}  // namespace pffrg

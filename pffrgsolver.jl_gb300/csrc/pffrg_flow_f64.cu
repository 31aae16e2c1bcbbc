// FP64 instantiation of the channel-task kernel.
#include "pffrg_flow.cuh"

namespace pffrg {

template <>
cudaError_t launch_pass<double>(const PassArgs<double>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    if (a.L.C == 6) return launch_pass_u1dm<double>(a, Wsp, h_counters, st);
    return launch_pass_impl<double, 2>(a, Wsp, h_counters, st);
}

}  // namespace pffrg

// Entry points of the channel-task passes: the team shape is chosen here, the kernels of every
// shape are instantiated in pffrg_shapes.cu.
#include "pffrg_flow.cuh"

namespace pffrg {

#define PFFRG_EXTERN(T, S)                                                                                       \
    extern template cudaError_t run_shape<double, 2, T, S>(const PassArgs<double>&, WaveSpace&, int*, cudaStream_t, \
                                                           int);                                                  \
    extern template cudaError_t run_shape<float, 2, T, S>(const PassArgs<float>&, WaveSpace&, int*, cudaStream_t,   \
                                                          int);                                                   \
    extern template cudaError_t run_shape<double, 6, T, S>(const PassArgs<double>&, WaveSpace&, int*, cudaStream_t, \
                                                           int);                                                  \
    extern template cudaError_t run_shape<float, 6, T, S>(const PassArgs<float>&, WaveSpace&, int*, cudaStream_t,   \
                                                          int);
PFFRG_TEAM_SHAPES(PFFRG_EXTERN)
#undef PFFRG_EXTERN

template <>
cudaError_t launch_pass<double>(const PassArgs<double>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    if (a.L.C == 6) return launch_pass_impl<double, 6>(a, Wsp, h_counters, st);
    return launch_pass_impl<double, 2>(a, Wsp, h_counters, st);
}

template <>
cudaError_t launch_pass<float>(const PassArgs<float>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    if (a.L.C == 6) return launch_pass_impl<float, 6>(a, Wsp, h_counters, st);
    return launch_pass_impl<float, 2>(a, Wsp, h_counters, st);
}

}  // namespace pffrg

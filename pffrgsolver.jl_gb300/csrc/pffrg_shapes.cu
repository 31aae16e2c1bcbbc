// Explicit instantiations of the pass kernels for one precision (PFFRG_R), component count
// (PFFRG_C: 2 for SU(2), 6 for U(1)-DM) and group of team shapes (PFFRG_GROUP); the build
// compiles this file once per combination, so the kernels compile in parallel.
#include "pffrg_flow.cuh"

namespace pffrg {

#define PFFRG_INST(T, S) \
    template cudaError_t run_shape<PFFRG_R, PFFRG_C, T, S>(const PassArgs<PFFRG_R>&, WaveSpace&, int*, cudaStream_t, int);
#if PFFRG_GROUP == 0
PFFRG_INST(8, 1)
PFFRG_INST(16, 1)
PFFRG_INST(32, 1)
#elif PFFRG_GROUP == 1
PFFRG_INST(16, 3)
PFFRG_INST(16, 4)
PFFRG_INST(32, 3)
#else
PFFRG_INST(32, 2)
PFFRG_INST(32, 4)
PFFRG_INST(32, 8)
#endif

}  // namespace pffrg

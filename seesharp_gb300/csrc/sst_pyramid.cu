// The shade kernel variants that also fill the technique pyramids (PathTracer.RenderTechniquePyramid,
// Integrators/PathTracer.cs:73-82, 204-266; Integrators/Bidir/TechPyramid.cs).  A translation unit
// of its own, so that these variants compile in parallel with the render and adjoint ones.
#include <cuda_runtime.h>

#include "sst_kernels.h"
#include "sst_shade.cuh"

namespace sst {

void launch_shade_pyramid(int ns, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee, int cap, float4* shRo,
                          float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples, DevStats* stats,
                          const PyrArgs& pyr, int maxItems, cudaStream_t s) {
    int grid = (maxItems + 127) / 128;
    if (grid == 0) return;
#define SST_PYR_CASE(N)                                                                                                                   \
    case N:                                                                                                                               \
        k_shade<N, false, true, true><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, nullptr, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, \
                                                           samples, stats, pyr);                                                          \
        break;
    switch (ns) {
        SST_PYR_CASE(1)
        SST_PYR_CASE(2)
        SST_PYR_CASE(3)
        default:
        SST_PYR_CASE(4)
    }
#undef SST_PYR_CASE
}

}  // namespace sst

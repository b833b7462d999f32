// The forward shade kernel with GenericMaterials (one shadow ray per technique) built for more
// resident blocks per SM than the default 8: 10, 12 and 14 blocks of 128 threads, that is 48, 40
// and 32 registers per thread.  More warps hide more of the kernel's memory and instruction-fetch
// latency, fewer registers spill more of its state to local memory; which wins depends on the
// scene, so the launch tuning picks the build (SstTuning.shadeBlocks).  A translation unit of its
// own, so that these instances compile in parallel with the others.
#include <cuda_runtime.h>

#include "sst_kernels.h"
#include "sst_shade.cuh"

namespace sst {

void launch_shade_generic_occ(int blocks, int grid, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee, int cap,
                              float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples,
                              DevStats* stats, cudaStream_t s) {
#define SST_OCC_CASE(N)                                                                                                                   \
    case N:                                                                                                                               \
        k_shade<1, false, true, false, N><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, nullptr, cap, shRo, shRd, shTgt, shJob, nIn, nOut,  \
                                                               nSh, samples, stats, PyrArgs{});                                           \
        break;
    switch (blocks) {
        SST_OCC_CASE(10)
        SST_OCC_CASE(12)
        default:
        SST_OCC_CASE(14)
    }
#undef SST_OCC_CASE
}

}  // namespace sst

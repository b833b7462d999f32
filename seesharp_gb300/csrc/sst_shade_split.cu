// The split form of the forward shade kernel: k_shade<..., SPLIT = true> (hit, emitter MIS, Russian
// roulette, next-event estimation) followed by k_shade_sample (BSDF sampling and the queue
// compaction), for GenericMaterials and one shadow ray per technique (with DiffuseMaterials only the
// fused kernel, which then needs no material dispatch, is faster).  Each half keeps less state live and holds less
// code than the fused kernel; the launch tuning (SstTuning.shadeSplit) picks the form.  A
// translation unit of its own, so that these instances compile in parallel with the others.
#include <cuda_runtime.h>

#include "sst_kernels.h"
#include "sst_shade.cuh"

namespace sst {

void launch_shade_split(int blocks, int grid, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee,
                        int cap, float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples,
                        DevStats* stats, cudaStream_t s) {
    if (blocks == SST_SHADE_GEN_DENSE_BLOCKS) {
        k_shade<1, false, true, false, SST_SHADE_GEN_DENSE_BLOCKS, true><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, nullptr, cap, shRo, shRd, shTgt,
                                                                                             shJob, nIn, nOut, nSh, samples, stats, PyrArgs{});
        k_shade_sample<true, SST_SHADE_GEN_DENSE_BLOCKS><<<grid, 128, 0, s>>>(jobs, A, B, cap, nIn, nOut, samples, stats);
    } else {
        k_shade<1, false, true, false, SST_SHADE_GEN_MIN_BLOCKS, true><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, nullptr, cap, shRo, shRd, shTgt,
                                                                                           shJob, nIn, nOut, nSh, samples, stats, PyrArgs{});
        k_shade_sample<true, SST_SHADE_GEN_MIN_BLOCKS><<<grid, 128, 0, s>>>(jobs, A, B, cap, nIn, nOut, samples, stats);
    }
}

}  // namespace sst

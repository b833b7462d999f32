// Launch wrappers of the kernels in sst_kernels.cu and sst_trace.cu (called by the host driver in sst_api.cu).
#pragma once
#include <cuda_runtime.h>

#include "sst_types.h"

namespace sst {

void launch_env_build(const float4* img, int w, int h, float* colCdf, float* rowMarg, int* hasCol, float* rowCdf, cudaStream_t s);
void launch_camera(const DevJob* jobs, const WaveChunk* chunks, const WaveDesc* waves, const int* curWave, const PathBuf& A, int* qCount,
                   int maxItems, cudaStream_t s);
void launch_light_start(const DevJob* jobs, const LightParams& P, const LightPathBuf& A, int* qCount, SstPathVertexDev* verts, int* lengths,
                        cudaStream_t s);
void launch_light_walk(const DevJob* jobs, const LightParams& P, const LightPathBuf& A, const LightPathBuf& B, const float4* hits, const int* nIn,
                       int* nOut, SstPathVertexDev* verts, int* lengths, int maxItems, cudaStream_t s);
// Outlier-rejecting RelMSE per iteration: `iterations` rows of P per-pixel errors -> out[row].
void launch_error_trim(const float* err, int P, int k, int iterations, double* out, cudaStream_t s);
void launch_variance_finish(const float* mean, const float* moment, int W, int H, float* out, double* sum, cudaStream_t s);
void launch_film_fold(const DevJob* jobs, const WaveChunk* chunks, const WaveDesc* waves, int* curWave, const float* samples, DevStats* st,
                      int maxFold, int advance, cudaStream_t s);
// Traversal launch configuration (sst_trace.cu): threads per block (64, 128 or 256), stack
// entries per thread kept in shared memory (16, 24 or 32), resident blocks per SM (0: as many as
// fit), BVH width (2, 4 or 8; a scene without a wide BVH misses every ray).
struct TraceTuning {
    int block = kTraceBlock;
    int smemStack = kSmemStack;
    int blocksPerSM = 0;
    int width = 4;  // BVH width: 2 (binary) or 4
    // 4- and 8-wide traversal: finished rays of a warp are replaced once this many of its 32 lanes are
    // idle (32: only when the whole warp is); the other lanes pause in place meanwhile
    int refillIdle = kTraceRefillIdle;
};
bool traceTuningValid(const TraceTuning& t);
int traceGrid(const TraceTuning& t);
int traceMaxBlocksPerSM(const TraceTuning& t);
void launch_trace_closest(const TraceTuning& t, const DevJob* jobs, const uint32_t* rayJob, const float4* ro, const float4* rd, const int* count,
                          int* work, float4* hits, DevStats* stats, cudaStream_t s);
void launch_trace_shadow(const TraceTuning& t, const DevJob* jobs, const uint32_t* rayJob, const float4* ro, const float4* rd, const int* tgt,
                         const int* count, int* work, float4* nee, DevStats* stats, cudaStream_t s);
void launch_trace_query(const TraceTuning& t, const DevJob* jobs, const float4* ro, const float4* rd, const int* count, int* work, float4* hits,
                        int* occl, DevStats* stats, bool anyHit, cudaStream_t s);
// shadeBlocks: the resident blocks per SM of the forward variant with GenericMaterials: the
// default build (8, 64 registers) or a denser one (10, 12 or 14: 48, 40 or 32 registers, more warps,
// more spilling); one shadow ray per technique has every build, more shadow rays the default one.
// The denser builds live in sst_shade_occ.cu.
// Writes the shade order of a bounce's queue (surface hits first) into order[0, *nIn).
void launch_wave_advance(int* wave, int by, cudaStream_t s);
void launch_partition(const uint32_t* depth, const float4* hits, const int* nIn, int* order, int* counts, int maxItems, cudaStream_t s);
bool shadeBlocksValid(int blocks);
// The split form (sst_shade_split.cu), forward, GenericMaterials, one shadow ray per technique: two
// kernels per bounce, A.rec must hold kShadeRec * cap float4.  blocks: 14 selects the dense build of
// both kernels, any other value the 8-block one.
void launch_shade_split(int blocks, int grid, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee,
                        int cap, float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples,
                        DevStats* stats, cudaStream_t s);
void launch_shade_generic_occ(int blocks, int grid, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee, int cap,
                              float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples,
                              DevStats* stats, cudaStream_t s);
void launch_shade(int ns, bool adj, bool generic, int shadeBlocks, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits,
                  float4* nee, float4* neeG, int cap, float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh,
                  float* samples, DevStats* stats, int maxItems, cudaStream_t s);
// k_shade with the technique pyramids (sst_pyramid.cu); the generic-material variant, no adjoint.
void launch_shade_pyramid(int ns, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits, float4* nee, int cap, float4* shRo,
                          float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh, float* samples, DevStats* stats,
                          const PyrArgs& pyr, int maxItems, cudaStream_t s);
// sst_trace's hit records: the compact traversal results expanded into SstHit (sst.h) layout.
void launch_hit_expand(const DevScene& sc, const float4* hits, int n, SstHitDev* out, cudaStream_t s);
void launch_debug_material_eval(const DevScene& sc, int mat, int n, const float* pts, const float* outs, const float* ins, float* vals, float* pdfs,
                                cudaStream_t s);
void launch_debug_material_sample(const DevScene& sc, int mat, int n, const float* pts, const float* outs, const float* us, float* dirs, float* pdfs,
                                  float* ws, cudaStream_t s);
void launch_debug_env(const DevScene& sc, int n, const float* us, float* dirs, float* pdfs, float* ws, const float* qd, float* rad, float* qpdf,
                      cudaStream_t s);
void launch_debug_rng(uint32_t base, uint32_t sample, int n, const uint32_t* pixels, int draws, uint32_t* out, cudaStream_t s);
void launch_debug_camera(const DevScene& sc, int n, const float* film, float* org, float* dir, cudaStream_t s);

}  // namespace sst

// GPU linear-BVH builder (sst_bvh.cu).
#pragma once
#include <cuda_runtime.h>

#include "sst_types.h"

namespace sst {

// Scratch bytes buildLbvh needs for n triangles.
size_t lbvhScratchBytes(int n);

// Builds the traversal BVH over n triangles (3 float4 per triangle, global order).  Writes at most
// n - 1 nodes (4 float4 each) to nodesOut and the leaf order (sorted position -> global triangle)
// to orderOut.  Returns 0 on success; the node count and the maximum inner-node depth are
// returned through the host pointers.
// method 0: the radix tree of the Morton codes (Karras 2012); 1: PLOC clustering (Meister and
// Bittner 2018) over the same sorted leaves.  Both finish with the SAH refit and leaf collapse.
int buildLbvh(const float4* tri, int n, float4* nodesOut, int* orderOut, void* scratch, size_t scratchBytes, int* hostNodeCount, int* hostMaxDepth,
              cudaStream_t st, int method);

// 4-wide BVH collapsed from the binary one (nNodes2 binary inner nodes in the layout above):
// at most nNodes2 nodes of 8 float4 each are written to nodes4.  Returns 0 on success with the
// node count and the number of levels through the host pointers.
size_t bvh4ScratchBytes(int nNodes2);
int buildBvh4(const float4* nodes2, int nNodes2, float4* nodes4, void* scratch, int* hostNodeCount, int* hostDepth, cudaStream_t st);

// 8-wide BVH over the same leaves, children in octant slots: at most nNodes2 nodes of 15 float4
// each are written to nodes8.  Returns 0 on success with the node count and the number of levels.
size_t bvh8ScratchBytes(int nNodes2);
int buildBvh8(const float4* nodes2, int nNodes2, float4* nodes8, void* scratch, int* hostNodeCount, int* hostDepth, cudaStream_t st);

// Gathers per-triangle records into leaf order: out[t] = in[order[t]] (triv also stamps the
// global id into v0.w).
void launch_leaf_gather(const int* order, int n, const float4* trivG, const float4* triNG, const int4* auxG, const int4* vtxG, float4* triv,
                        float4* triN, int4* aux, int4* vtx, cudaStream_t st);

}  // namespace sst

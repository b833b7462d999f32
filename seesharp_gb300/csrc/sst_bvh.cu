// GPU BVH construction (replaces the Embree build behind Raytracer.CommitScene, Scene.cs:108-113).
//
// Linear BVH after Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d
// Trees" (HPG 2012):
//   1. centroid bounds (atomic min/max on order-preserving integer images of the floats)
//   2. 63-bit Morton keys of the triangle centroids, radix-sorted with CUB
//   3. one thread per internal node finds its key range and split (longest common prefix, ties
//      broken by the sorted index)
//   4. bottom-up refit: the second child to arrive computes the parent's box, leaf count and the
//      surface-area cost C(n) = min(Ci N A(n) [N <= kMaxLeafSize], Ct A(n) + C(l) + C(r)), which
//      decides where subtrees collapse into multi-triangle leaves
//   5. kept inner nodes are numbered by a prefix sum and written in the traversal layout (both
//      child boxes in the parent, 64-byte nodes); a collapsed subtree becomes one leaf reference
//      to its contiguous range of sorted triangles.
#include <cub/cub.cuh>
#include <math_constants.h>
#include <algorithm>
#include <cstdlib>
#include <cuda_runtime.h>

#include "sst_bvh.h"
#include "sst_types.h"

namespace sst {

namespace {

// Traversal cost relative to one triangle test.  0.25 keeps most leaves at one triangle: on the
// 1M-triangle scene it traverses 3.4% faster than 1.0 (and 1.0 17% faster than 3.0).
constexpr float kCt = 0.25f;
constexpr float kCi = 1.0f;

__device__ __forceinline__ int floatOrd(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ordFloat(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__global__ void k_centroid_bounds(const float4* tri, int n, int* bounds /* 6: min xyz, max xyz (ordered ints) */) {
    __shared__ int smin[3], smax[3];
    if (threadIdx.x < 3) { smin[threadIdx.x] = 0x7FFFFFFF; smax[threadIdx.x] = (int)0x80000000; }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = tri[3 * (size_t)i], b = tri[3 * (size_t)i + 1], c = tri[3 * (size_t)i + 2];
        float cx = 0.5f * (fminf(a.x, fminf(b.x, c.x)) + fmaxf(a.x, fmaxf(b.x, c.x)));
        float cy = 0.5f * (fminf(a.y, fminf(b.y, c.y)) + fmaxf(a.y, fmaxf(b.y, c.y)));
        float cz = 0.5f * (fminf(a.z, fminf(b.z, c.z)) + fmaxf(a.z, fmaxf(b.z, c.z)));
        atomicMin(&smin[0], floatOrd(cx)); atomicMin(&smin[1], floatOrd(cy)); atomicMin(&smin[2], floatOrd(cz));
        atomicMax(&smax[0], floatOrd(cx)); atomicMax(&smax[1], floatOrd(cy)); atomicMax(&smax[2], floatOrd(cz));
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        atomicMin(&bounds[threadIdx.x], smin[threadIdx.x]);
        atomicMax(&bounds[3 + threadIdx.x], smax[threadIdx.x]);
    }
}

__device__ __forceinline__ unsigned long long spread21(unsigned int v) {
    unsigned long long x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* tri, int n, const int* bounds, unsigned long long* keys, int* vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3] = {ordFloat(bounds[0]), ordFloat(bounds[1]), ordFloat(bounds[2])};
    float hi[3] = {ordFloat(bounds[3]), ordFloat(bounds[4]), ordFloat(bounds[5])};
    float4 a = tri[3 * (size_t)i], b = tri[3 * (size_t)i + 1], c = tri[3 * (size_t)i + 2];
    float cc[3] = {0.5f * (fminf(a.x, fminf(b.x, c.x)) + fmaxf(a.x, fmaxf(b.x, c.x))),
                   0.5f * (fminf(a.y, fminf(b.y, c.y)) + fmaxf(a.y, fmaxf(b.y, c.y))),
                   0.5f * (fminf(a.z, fminf(b.z, c.z)) + fmaxf(a.z, fmaxf(b.z, c.z)))};
    unsigned int q[3];
    for (int k = 0; k < 3; ++k) {
        float ext = hi[k] - lo[k];
        float t = ext > 0.0f ? (cc[k] - lo[k]) / ext : 0.5f;
        q[k] = (unsigned int)fminf(fmaxf(t * 2097152.0f, 0.0f), 2097151.0f);
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = i;
}

// Longest common prefix of sorted keys i and j (-1 outside [0, n)); equal keys compare indices.
__device__ __forceinline__ int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll(a ^ b);
}

// Internal node i covers sorted leaves [first, last]; children encoded >= 0 internal, < 0 leaf ~idx.
__global__ void k_karras(const unsigned long long* k, int n, int2* range, int2* child, int* parentInner, int* parentLeaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(k, n, i, j);
    int s = 0;
    int div = 2;
    for (int t = (l + 1) / 2; ; t = (l + div - 1) / div) {
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
        div <<= 1;
    }
    int gamma = i + s * d + min(d, 0);
    int first = min(i, j), last = max(i, j);
    int left = (first == gamma) ? ~gamma : gamma;
    int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    range[i] = make_int2(first, last);
    child[i] = make_int2(left, right);
    if (left < 0) parentLeaf[~left] = i; else parentInner[left] = i;
    if (right < 0) parentLeaf[~right] = i; else parentInner[right] = i;
}

struct NodeFit {
    float lo[3], hi[3];
};

__device__ __forceinline__ float areaOf(const float* lo, const float* hi) {
    float dx = fmaxf(0.0f, hi[0] - lo[0]), dy = fmaxf(0.0f, hi[1] - lo[1]), dz = fmaxf(0.0f, hi[2] - lo[2]);
    return dx * dy + dy * dz + dz * dx;
}

// Bottom-up refit from every leaf.  boxes: 6 floats per inner node; cost: per inner node;
// collapse[i] = 1 when the subtree is cheaper as one leaf.
__global__ void k_refit(const float4* tri, const int* order, int n, const int2* range, const int2* child, const int* parentInner,
                        const int* parentLeaf, int* visits, float* boxes, float* cost, int* collapse, float ct, int maxLeaf) {
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int node = parentLeaf[li];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&visits[node], 1) == 0) return;  // the other child is not done yet
        __threadfence();
        int2 c = child[node];
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        float cs = 0.0f;
        for (int s = 0; s < 2; ++s) {
            int ch = s == 0 ? c.x : c.y;
            float clo[3], chi[3], ccost;
            if (ch < 0) {
                int t = order[~ch];
                float4 a = tri[3 * (size_t)t], b = tri[3 * (size_t)t + 1], d = tri[3 * (size_t)t + 2];
                clo[0] = fminf(a.x, fminf(b.x, d.x)); chi[0] = fmaxf(a.x, fmaxf(b.x, d.x));
                clo[1] = fminf(a.y, fminf(b.y, d.y)); chi[1] = fmaxf(a.y, fmaxf(b.y, d.y));
                clo[2] = fminf(a.z, fminf(b.z, d.z)); chi[2] = fmaxf(a.z, fmaxf(b.z, d.z));
                ccost = kCi * areaOf(clo, chi);
            } else {
                const volatile float* bx = boxes + 6 * (size_t)ch;
                for (int k = 0; k < 3; ++k) { clo[k] = bx[k]; chi[k] = bx[3 + k]; }
                ccost = ((const volatile float*)cost)[ch];
            }
            for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], clo[k]); hi[k] = fmaxf(hi[k], chi[k]); }
            cs += ccost;
        }
        float A = areaOf(lo, hi);
        int2 r = range[node];
        int cnt = r.y - r.x + 1;
        float split = ct * A + cs;
        float leaf = kCi * cnt * A;
        bool col = cnt <= maxLeaf && leaf <= split;
        float* bo = boxes + 6 * (size_t)node;
        for (int k = 0; k < 3; ++k) { bo[k] = lo[k]; bo[3 + k] = hi[k]; }
        cost[node] = col ? leaf : split;
        collapse[node] = col ? 1 : 0;
        node = parentInner[node];
    }
}

// kept[i] = 1 when inner node i is not inside a collapsed subtree (and is not collapsed itself);
// depth[i] = number of kept ancestors.  Walks to the root (depth bounded by the key length).
__global__ void k_kept(const int* parentInner, const int* collapse, int n, int* kept, int* maxDepth) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int k = (i == 0 || !collapse[i]) ? 1 : 0;
    int depth = 0;
    int p = parentInner[i];
    for (int guard = 0; p >= 0 && guard < 4096; ++guard) {
        if (collapse[p] && p != 0) k = 0;
        ++depth;
        p = parentInner[p];
    }
    kept[i] = k;
    if (k) atomicMax(maxDepth, depth);
}

// ---------------------------------------------------------------------------------------------
// PLOC topology (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
// Hierarchy Construction", 2018): the clusters start as the Morton-sorted leaves; in each round
// every cluster finds the cluster within a radius of positions whose union box has the smallest
// surface area, mutual nearest neighbours merge into a new inner node, and the cluster list is
// compacted in order.  The resulting tree is then given a depth-first leaf order so that every
// subtree covers a contiguous range, and the LBVH's refit / collapse / emit stages finish it.
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ float unionArea(const float* a, const float* b) {
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) { lo[k] = fminf(a[k], b[k]); hi[k] = fmaxf(a[3 + k], b[3 + k]); }
    return areaOf(lo, hi);
}

// clusters = sorted leaves ~i with their triangle boxes
__global__ void k_ploc_init(const float4* tri, const int* order, int n, int* clus, float* cbox) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t = order[i];
    float4 a = tri[3 * (size_t)t], b = tri[3 * (size_t)t + 1], d = tri[3 * (size_t)t + 2];
    float* o = cbox + 6 * (size_t)i;
    o[0] = fminf(a.x, fminf(b.x, d.x)); o[3] = fmaxf(a.x, fmaxf(b.x, d.x));
    o[1] = fminf(a.y, fminf(b.y, d.y)); o[4] = fmaxf(a.y, fmaxf(b.y, d.y));
    o[2] = fminf(a.z, fminf(b.z, d.z)); o[5] = fmaxf(a.z, fmaxf(b.z, d.z));
    clus[i] = ~i;
}

// nearest neighbour within `radius` positions (ties: the smaller index)
__global__ void k_ploc_nn(const float* cbox, const int* nc, int radius, int* nn) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = *nc;
    if (i >= n) return;
    float me[6];
    for (int k = 0; k < 6; ++k) me[k] = cbox[6 * (size_t)i + k];
    float best = CUDART_INF_F;
    int bj = -1;
    int j0 = max(0, i - radius), j1 = min(n - 1, i + radius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        float a = unionArea(me, cbox + 6 * (size_t)j);
        if (a < best) { best = a; bj = j; }
    }
    nn[i] = bj;
}

// flags: create[i] = i merges with its mutual neighbour (i the lower index); keep[i] = cluster i
// (possibly merged) stays in the list
__global__ void k_ploc_flags(const int* nn, const int* nc, int* create, int* keep) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = *nc;
    if (i >= n) return;
    int j = nn[i];
    bool mutual = j >= 0 && nn[j] == i;
    create[i] = (mutual && i < j) ? 1 : 0;
    keep[i] = (!mutual || i < j) ? 1 : 0;
}

// merged clusters become inner nodes numbered base + createIdx[i] in creation order
__global__ void k_ploc_compact(const int* clus, const float* cbox, const int* nn, const int* nc, const int* create, const int* createIdx,
                               const int* keep, const int* newPos, int base, int* clusOut, float* cboxOut, int2* child, float* ibox) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = *nc;
    if (i >= n || !keep[i]) return;
    int out = newPos[i];
    if (create[i]) {
        int j = nn[i];
        int id = base + createIdx[i];
        child[id] = make_int2(clus[i], clus[j]);
        float* b = cboxOut + 6 * (size_t)out;
        for (int k = 0; k < 3; ++k) {
            b[k] = fminf(cbox[6 * (size_t)i + k], cbox[6 * (size_t)j + k]);
            b[3 + k] = fmaxf(cbox[6 * (size_t)i + 3 + k], cbox[6 * (size_t)j + 3 + k]);
        }
        for (int k = 0; k < 6; ++k) ibox[6 * (size_t)id + k] = b[k];
        clusOut[out] = id;
    } else {
        clusOut[out] = clus[i];
        for (int k = 0; k < 6; ++k) cboxOut[6 * (size_t)out + k] = cbox[6 * (size_t)i + k];
    }
}

// creation ids -> final ids (root = 0: reversed creation order); parent pointers
__global__ void k_ploc_renumber(const int2* childC, int n, int2* child, int* parentInner, int* parentLeaf) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n - 1) return;
    int nid = (n - 2) - id;
    int2 c = childC[id];
    int a = c.x >= 0 ? (n - 2) - c.x : c.x;
    int b = c.y >= 0 ? (n - 2) - c.y : c.y;
    child[nid] = make_int2(a, b);
    if (a < 0) parentLeaf[~a] = nid; else parentInner[a] = nid;
    if (b < 0) parentLeaf[~b] = nid; else parentInner[b] = nid;
}

// subtree leaf counts, bottom-up from every leaf (the second child to arrive continues)
__global__ void k_ploc_sizes(const int2* child, const int* parentLeaf, const int* parentInner, int n, int* visits, int* size) {
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int node = parentLeaf[li];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&visits[node], 1) == 0) return;
        __threadfence();
        int2 c = child[node];
        int sa = c.x < 0 ? 1 : ((const volatile int*)size)[c.x];
        int sb = c.y < 0 ? 1 : ((const volatile int*)size)[c.y];
        size[node] = sa + sb;
        node = parentInner[node];
    }
}

// depth-first offsets: a node's first leaf is the number of leaves left of it, summed over the
// ancestors of which it lies in the right subtree.  Inner nodes get their leaf range; leaves their
// position in the new order.
__global__ void k_ploc_offsets(const int2* child, const int* parentInner, const int* parentLeaf, const int* size, int n, int2* range,
                               int* leafPos) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 2 * n - 1) return;
    bool leaf = x >= n - 1;
    int self = leaf ? ~(x - (n - 1)) : x;
    int p = leaf ? parentLeaf[x - (n - 1)] : parentInner[x];
    int off = 0, cur = self;
    for (int guard = 0; p >= 0 && guard < 1 << 20; ++guard) {
        int2 c = child[p];
        if (c.y == cur) off += c.x < 0 ? 1 : size[c.x];
        cur = p;
        p = parentInner[p];
    }
    if (leaf) leafPos[x - (n - 1)] = off;
    else range[x] = make_int2(off, off + size[x] - 1);
}

__global__ void k_ploc_leaf_parents(const int2* child, int n, int* parentLeaf) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n - 1) return;
    int2 c = child[x];
    if (c.x < 0) parentLeaf[~c.x] = x;
    if (c.y < 0) parentLeaf[~c.y] = x;
}

// leaves re-encoded by their depth-first position; the triangle order follows
__global__ void k_ploc_reorder(int2* child, const int* leafPos, const int* sortedOrder, int n, int* order) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) order[leafPos[x]] = sortedOrder[x];
    if (x < n - 1) {
        int2 c = child[x];
        if (c.x < 0) c.x = ~leafPos[~c.x];
        if (c.y < 0) c.y = ~leafPos[~c.y];
        child[x] = c;
    }
}

__device__ __forceinline__ uint32_t leafRef(int first, int count) {
    return kLeafFlag | ((uint32_t)(count - 1) << kLeafCountShift) | (uint32_t)first;
}

__global__ void k_emit(const float4* tri, const int* order, int n, const int2* range, const int2* child, const int* collapse, const int* kept,
                       const int* newIdx, const float* boxes, float4* nodes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1 || !kept[i]) return;
    int2 c = child[i];
    float4* out = nodes + 4 * (size_t)newIdx[i];
    float4 o0, o1, o2, o3;
    uint32_t refs[2];
    float b[2][6];
    for (int s = 0; s < 2; ++s) {
        int ch = s == 0 ? c.x : c.y;
        if (ch < 0) {
            int t = order[~ch];
            float4 a = tri[3 * (size_t)t], bb = tri[3 * (size_t)t + 1], d = tri[3 * (size_t)t + 2];
            b[s][0] = fminf(a.x, fminf(bb.x, d.x)); b[s][3] = fmaxf(a.x, fmaxf(bb.x, d.x));
            b[s][1] = fminf(a.y, fminf(bb.y, d.y)); b[s][4] = fmaxf(a.y, fmaxf(bb.y, d.y));
            b[s][2] = fminf(a.z, fminf(bb.z, d.z)); b[s][5] = fmaxf(a.z, fmaxf(bb.z, d.z));
            refs[s] = leafRef(~ch, 1);
        } else {
            for (int k = 0; k < 6; ++k) b[s][k] = boxes[6 * (size_t)ch + k];
            if (collapse[ch]) {
                int2 r = range[ch];
                refs[s] = leafRef(r.x, r.y - r.x + 1);
            } else {
                refs[s] = (uint32_t)newIdx[ch];
            }
        }
    }
    o0 = make_float4(b[0][0], b[0][3], b[0][1], b[0][4]);
    o1 = make_float4(b[1][0], b[1][3], b[1][1], b[1][4]);
    o2 = make_float4(b[0][2], b[0][5], b[1][2], b[1][5]);
    o3 = make_float4(__uint_as_float(refs[0]), __uint_as_float(refs[1]), 0.0f, 0.0f);
    out[0] = o0; out[1] = o1; out[2] = o2; out[3] = o3;
}

// Single-triangle scene: root with the same one-triangle leaf in both slots.
__global__ void k_emit_single(const float4* tri, float4* nodes) {
    float4 a = tri[0], b = tri[1], c = tri[2];
    float lo[3] = {fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z))};
    float hi[3] = {fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z))};
    uint32_t r = leafRef(0, 1);
    nodes[0] = make_float4(lo[0], hi[0], lo[1], hi[1]);
    nodes[1] = make_float4(lo[0], hi[0], lo[1], hi[1]);
    nodes[2] = make_float4(lo[2], hi[2], lo[2], hi[2]);
    nodes[3] = make_float4(__uint_as_float(r), __uint_as_float(r), 0.0f, 0.0f);
}

template <class T> T* carve(char*& p, size_t n) {
    size_t off = (reinterpret_cast<size_t>(p) + 255) & ~size_t(255);
    T* r = reinterpret_cast<T*>(off);
    p = reinterpret_cast<char*>(off + n * sizeof(T));
    return r;
}

}  // namespace

// CUB temporary storage shared by the radix sort and the prefix sum.
static size_t cubTempBytes(int n) {
    size_t sortBytes = 0, scanBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, (unsigned long long*)nullptr, (unsigned long long*)nullptr, (int*)nullptr, (int*)nullptr, n,
                                    0, 63);
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (int*)nullptr, (int*)nullptr, n > 1 ? n - 1 : 1);
    return std::max(sortBytes, scanBytes);
}

size_t lbvhScratchBytes(int n) {
    size_t tmp = cubTempBytes(n);
    size_t s = 0;
    s += 2 * sizeof(unsigned long long) * n + 2 * sizeof(int) * n;  // keys, values (double buffer)
    s += sizeof(int2) * n * 2;                                       // range, child
    s += sizeof(int) * n * 2;                                        // parents
    s += sizeof(int) * n * 4;                                        // visits, collapse, kept, newIdx
    s += sizeof(float) * n * 7;                                      // boxes, cost
    s += sizeof(int) * n * 11 + sizeof(float) * n * 18 + sizeof(int2) * n + 4096;  // PLOC clusters, boxes, flags, sizes
    s += tmp + 64 * 256 + 64;
    return s;
}

int buildLbvh(const float4* tri, int n, float4* nodesOut, int* orderOut, void* scratch, size_t scratchBytes, int* hostNodeCount, int* hostMaxDepth,
              cudaStream_t st, int method) {
    if (n <= 0) { *hostNodeCount = 0; *hostMaxDepth = 0; return 0; }
    if (n == 1) {
        k_emit_single<<<1, 1, 0, st>>>(tri, nodesOut);
        int zero = 0;
        cudaMemcpyAsync(orderOut, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
        *hostNodeCount = 1;
        *hostMaxDepth = 0;
        return cudaStreamSynchronize(st) == cudaSuccess ? 0 : -1;
    }
    char* p = static_cast<char*>(scratch);
    unsigned long long* keysA = carve<unsigned long long>(p, n);
    unsigned long long* keysB = carve<unsigned long long>(p, n);
    int* valsA = carve<int>(p, n);
    int* valsB = carve<int>(p, n);
    int2* range = carve<int2>(p, n);
    int2* child = carve<int2>(p, n);
    int* parentInner = carve<int>(p, n);
    int* parentLeaf = carve<int>(p, n);
    int* visits = carve<int>(p, n);
    int* collapse = carve<int>(p, n);
    int* kept = carve<int>(p, n);
    int* newIdx = carve<int>(p, n);
    float* boxes = carve<float>(p, 6 * size_t(n));
    float* cost = carve<float>(p, n);
    int* small = carve<int>(p, 16);  // 0..5 centroid bounds, 6 max depth, 7 kept total
    size_t tmpBytes = cubTempBytes(n);
    void* tmp = carve<char>(p, tmpBytes);
    if (size_t(p - static_cast<char*>(scratch)) > scratchBytes) return -2;

    int init[8] = {0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF, (int)0x80000000, (int)0x80000000, (int)0x80000000, 0, 0};
    cudaMemcpyAsync(small, init, sizeof(init), cudaMemcpyHostToDevice, st);
    int grid = (n + 255) / 256;
    k_centroid_bounds<<<std::min(grid, 1024), 256, 0, st>>>(tri, n, small);
    k_morton<<<grid, 256, 0, st>>>(tri, n, small, keysA, valsA);
    cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keysA, keysB, valsA, valsB, n, 0, 63, st);
    cudaMemsetAsync(parentInner, 0xFF, sizeof(int) * n, st);
    cudaMemsetAsync(visits, 0, sizeof(int) * n, st);
    const int* order = valsB;
    if (method == 1 && n > 2) {
        // PLOC topology in place of the radix tree
        const char* re = getenv("SST_PLOC_RADIUS");
        const int plocRadius = re ? std::max(1, std::min(256, atoi(re))) : 16;
        int* clus = carve<int>(p, n);
        int* clus2 = carve<int>(p, n);
        float* cbox = carve<float>(p, 6 * size_t(n));
        float* cbox2 = carve<float>(p, 6 * size_t(n));
        float* ibox = carve<float>(p, 6 * size_t(n));
        int* nn = carve<int>(p, n);
        int* create = carve<int>(p, n);
        int* keep = carve<int>(p, n);
        int* createIdx = carve<int>(p, n);
        int* newPos = carve<int>(p, n);
        int* nc = carve<int>(p, 4);
        int2* childC = carve<int2>(p, n);
        int* size = carve<int>(p, n);
        int* leafPos = carve<int>(p, n);
        int* order2 = carve<int>(p, n);
        if (size_t(p - static_cast<char*>(scratch)) > scratchBytes) return -2;
        k_ploc_init<<<grid, 256, 0, st>>>(tri, valsB, n, clus, cbox);
        int ncH = n, base = 0;
        cudaMemcpyAsync(nc, &ncH, sizeof(int), cudaMemcpyHostToDevice, st);
        size_t scanBytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, create, createIdx, n, st);
        if (scanBytes > tmpBytes) return -2;
        for (int round = 0; ncH > 1; ++round) {
            if (round > n) return -3;  // each round merges at least the globally closest pair
            int g = (ncH + 255) / 256;
            k_ploc_nn<<<g, 256, 0, st>>>(cbox, nc, plocRadius, nn);
            k_ploc_flags<<<g, 256, 0, st>>>(nn, nc, create, keep);
            cub::DeviceScan::ExclusiveSum(tmp, scanBytes, create, createIdx, ncH, st);
            cub::DeviceScan::ExclusiveSum(tmp, scanBytes, keep, newPos, ncH, st);
            k_ploc_compact<<<g, 256, 0, st>>>(clus, cbox, nn, nc, create, createIdx, keep, newPos, base, clus2, cbox2, childC, ibox);
            int h4[4];
            cudaMemcpyAsync(&h4[0], createIdx + (ncH - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&h4[1], create + (ncH - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&h4[2], newPos + (ncH - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&h4[3], keep + (ncH - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
            if (h4[0] + h4[1] == 0) return -3;  // no mutual pair: degenerate boxes
            base += h4[0] + h4[1];
            ncH = h4[2] + h4[3];
            cudaMemcpyAsync(nc, &ncH, sizeof(int), cudaMemcpyHostToDevice, st);
            std::swap(clus, clus2);
            std::swap(cbox, cbox2);
        }
        if (base != n - 1) return -4;
        k_ploc_renumber<<<grid, 256, 0, st>>>(childC, n, child, parentInner, parentLeaf);
        cudaMemsetAsync(size, 0, sizeof(int) * n, st);
        k_ploc_sizes<<<grid, 256, 0, st>>>(child, parentLeaf, parentInner, n, visits, size);
        cudaMemsetAsync(visits, 0, sizeof(int) * n, st);
        k_ploc_offsets<<<(2 * n - 1 + 255) / 256, 256, 0, st>>>(child, parentInner, parentLeaf, size, n, range, leafPos);
        k_ploc_reorder<<<grid, 256, 0, st>>>(child, leafPos, valsB, n, order2);
        // the leaves' parents in the new order
        cudaMemsetAsync(parentLeaf, 0xFF, sizeof(int) * n, st);
        k_ploc_leaf_parents<<<grid, 256, 0, st>>>(child, n, parentLeaf);
        order = order2;
    } else {
        k_karras<<<grid, 256, 0, st>>>(keysB, n, range, child, parentInner, parentLeaf);
    }
    // SAH constants: traversal cost relative to one triangle test and the largest leaf
    // (SST_BVH_CT / SST_BVH_LEAF override them for experiments)
    const char* ctEnv = getenv("SST_BVH_CT");
    const char* leafEnv = getenv("SST_BVH_LEAF");
    const float ct = ctEnv ? (float)atof(ctEnv) : kCt;
    const int maxLeaf = leafEnv ? std::max(1, std::min(kMaxLeafSize, atoi(leafEnv))) : kMaxLeafSize;
    k_refit<<<grid, 256, 0, st>>>(tri, order, n, range, child, parentInner, parentLeaf, visits, boxes, cost, collapse, ct, maxLeaf);
    k_kept<<<grid, 256, 0, st>>>(parentInner, collapse, n, kept, small + 6);
    size_t scanBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, kept, newIdx, n - 1, st);
    if (scanBytes > tmpBytes) return -2;
    cub::DeviceScan::ExclusiveSum(tmp, scanBytes, kept, newIdx, n - 1, st);
    int hs[2];
    cudaMemcpyAsync(&hs[0], newIdx + (n - 2), sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hs[1], kept + (n - 2), sizeof(int), cudaMemcpyDeviceToHost, st);
    int md = 0;
    cudaMemcpyAsync(&md, small + 6, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *hostNodeCount = hs[0] + hs[1];
    *hostMaxDepth = md;
    k_emit<<<grid, 256, 0, st>>>(tri, order, n, range, child, collapse, kept, newIdx, boxes, nodesOut);
    cudaMemcpyAsync(orderOut, order, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    return cudaStreamSynchronize(st) == cudaSuccess ? 0 : -1;
}

}  // namespace sst

namespace sst {
namespace {
__global__ void k_leaf_gather(const int* order, int n, const float4* trivG, const float4* triNG, const int4* auxG, const int4* vtxG, float4* triv,
                              float4* triN, int4* aux, int4* vtx) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int g = order[t];
    float4 a = trivG[3 * (size_t)g];
    a.w = __int_as_float(g);
    triv[3 * (size_t)t] = a;
    triv[3 * (size_t)t + 1] = trivG[3 * (size_t)g + 1];
    triv[3 * (size_t)t + 2] = trivG[3 * (size_t)g + 2];
    triN[t] = triNG[g];
    aux[t] = auxG[g];
    vtx[t] = vtxG[g];
}
}  // namespace

void launch_leaf_gather(const int* order, int n, const float4* trivG, const float4* triNG, const int4* auxG, const int4* vtxG, float4* triv,
                        float4* triN, int4* aux, int4* vtx, cudaStream_t st) {
    if (n <= 0) return;
    k_leaf_gather<<<(n + 255) / 256, 256, 0, st>>>(order, n, trivG, triNG, auxG, vtxG, triv, triN, aux, vtx);
}
}  // namespace sst

// =============================================================================================
// 4-wide BVH from the binary one.  Each 4-wide node is made from a binary inner node by opening
// its inner children with the largest surface area until it has four children (or only leaves
// remain); leaves are shared unchanged.  Level-synchronous: one launch per level of the 4-wide
// tree, the frontier holds (binary node, 4-wide slot) pairs.
// Node layout (8 float4, 128 bytes): lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4],
// child references[4] (a 4-wide node index or a leaf reference), (number of children, -, -, -).
// =============================================================================================
namespace sst {
namespace {
struct Child4 {
    uint32_t ref;
    float lo[3], hi[3];
};
__device__ float halfArea(const Child4& c) {
    float dx = c.hi[0] - c.lo[0], dy = c.hi[1] - c.lo[1], dz = c.hi[2] - c.lo[2];
    return dx * dy + dy * dz + dz * dx;
}
__device__ void readChildren(const float4* nodes2, uint32_t b, Child4& c0, Child4& c1) {
    const float4* nd = nodes2 + 4 * (size_t)b;
    float4 n0 = nd[0], n1 = nd[1], n2 = nd[2], n3 = nd[3];
    c0.lo[0] = n0.x; c0.hi[0] = n0.y; c0.lo[1] = n0.z; c0.hi[1] = n0.w; c0.lo[2] = n2.x; c0.hi[2] = n2.y;
    c1.lo[0] = n1.x; c1.hi[0] = n1.y; c1.lo[1] = n1.z; c1.hi[1] = n1.w; c1.lo[2] = n2.z; c1.hi[2] = n2.w;
    c0.ref = __float_as_uint(n3.x);
    c1.ref = __float_as_uint(n3.y);
}
__global__ void k_collapse4(const float4* nodes2, const int2* frontier, const int* nFront, float4* nodes4, int* nodeCounter, int2* next,
                            int* nNext) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nFront) return;
    int2 item = frontier[i];
    Child4 c[4];
    int cnt = 2;
    readChildren(nodes2, (uint32_t)item.x, c[0], c[1]);
    while (cnt < 4) {
        int best = -1;
        float bestA = -1.0f;
        for (int k = 0; k < cnt; ++k)
            if (!(c[k].ref & kLeafFlag)) {
                float a = halfArea(c[k]);
                if (a > bestA) { bestA = a; best = k; }
            }
        if (best < 0) break;
        Child4 a, b;
        readChildren(nodes2, c[best].ref, a, b);
        c[best] = a;
        c[cnt++] = b;
    }
    float4* out = nodes4 + 8 * (size_t)item.y;
    float v[6][4];
    uint32_t refs[4];
    for (int k = 0; k < 4; ++k) {
        if (k < cnt) {
            for (int a = 0; a < 3; ++a) { v[2 * a][k] = c[k].lo[a]; v[2 * a + 1][k] = c[k].hi[a]; }
            uint32_t r = c[k].ref;
            if (!(r & kLeafFlag)) {
                int slot = atomicAdd(nodeCounter, 1);
                next[atomicAdd(nNext, 1)] = make_int2((int)r, slot);
                r = (uint32_t)slot;
            }
            refs[k] = r;
        } else {
            for (int a = 0; a < 6; ++a) v[a][k] = 0.0f;
            refs[k] = 0u;
        }
    }
    for (int a = 0; a < 6; ++a) out[a] = make_float4(v[a][0], v[a][1], v[a][2], v[a][3]);
    out[6] = make_float4(__uint_as_float(refs[0]), __uint_as_float(refs[1]), __uint_as_float(refs[2]), __uint_as_float(refs[3]));
    out[7] = make_float4(__int_as_float(cnt), 0.0f, 0.0f, 0.0f);
}
__global__ void k_collapse_root(int2* frontier, int* nFront, int* nodeCounter) {
    frontier[0] = make_int2(0, 0);
    *nFront = 1;
    *nodeCounter = 1;
}
}  // namespace

size_t bvh4ScratchBytes(int nNodes2) { return 2 * sizeof(int2) * (size_t)std::max(1, nNodes2) + 1024; }

int buildBvh4(const float4* nodes2, int nNodes2, float4* nodes4, void* scratch, int* hostNodeCount, int* hostDepth, cudaStream_t st) {
    *hostNodeCount = 0;
    *hostDepth = 0;
    if (nNodes2 <= 0) return 0;
    char* p = static_cast<char*>(scratch);
    int* counters = reinterpret_cast<int*>(p);  // [0] node counter, [1], [2] frontier sizes
    int2* fr[2] = {reinterpret_cast<int2*>(p + 256), reinterpret_cast<int2*>(p + 256) + nNodes2};
    k_collapse_root<<<1, 1, 0, st>>>(fr[0], counters + 1, counters);
    int cur = 0, depth = 0, n = 1;
    int hostCnt = 0;
    while (n > 0) {
        if (++depth > 4 * kMaxBvhDepth) return -2;
        if (cudaMemsetAsync(counters + 2 - cur, 0, sizeof(int), st) != cudaSuccess) return -1;
        k_collapse4<<<(n + 127) / 128, 128, 0, st>>>(nodes2, fr[cur], counters + 1 + cur, nodes4, counters, fr[1 - cur], counters + 2 - cur);
        if (cudaMemcpyAsync(&n, counters + 2 - cur, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        cur = 1 - cur;
    }
    if (cudaMemcpyAsync(&hostCnt, counters, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *hostNodeCount = hostCnt;
    *hostDepth = depth;
    return 0;
}
}  // namespace sst

// =============================================================================================
// 8-wide BVH from the binary one, its children in octant slots.  Each node is made from a
// binary inner node by opening its inner children, largest surface area first, until it has eight
// children (or only leaves remain); leaves are the binary tree's leaves, unchanged.  The children
// are then placed in the eight slots by the octant of their box centre relative to the node's
// (slot bit 0: +x side, bit 1: +y, bit 2: +z), greedily, best-aligned (child, slot) pair first,
// as in the octant ordering of Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on
// GPUs Through Compressed Wide BVHs" (HPG 2017).  A ray whose direction has the sign bits o
// (bit set for a negative component) then visits the slots in the order s ^ o ascending, which
// puts the children that lie first along its direction first, without a per-node sort.
// Node layout (15 float4, 240 bytes): lo.x[8], hi.x[8], lo.y[8], hi.y[8], lo.z[8], hi.z[8] (two
// float4 each), child references[8] (an 8-wide node index or a leaf reference), and
// (valid-slot mask | inner-slot mask << 8, -, -, -).  Level-synchronous like the 4-wide build.
// =============================================================================================
namespace sst {
namespace {
__global__ void k_collapse8(const float4* nodes2, const int2* frontier, const int* nFront, float4* nodes8, int* nodeCounter, int2* next,
                            int* nNext) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nFront) return;
    int2 item = frontier[i];
    Child4 c[8];
    int cnt = 2;
    readChildren(nodes2, (uint32_t)item.x, c[0], c[1]);
    while (cnt < 8) {
        int best = -1;
        float bestA = -1.0f;
        for (int k = 0; k < cnt; ++k)
            if (!(c[k].ref & kLeafFlag)) {
                float a = halfArea(c[k]);
                if (a > bestA) { bestA = a; best = k; }
            }
        if (best < 0) break;
        Child4 a, b;
        readChildren(nodes2, c[best].ref, a, b);
        c[best] = a;
        c[cnt++] = b;
    }
    // node centre and the children's offsets from it
    float lo[3] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F}, hi[3] = {-CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F};
    for (int k = 0; k < cnt; ++k)
        for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], c[k].lo[a]); hi[a] = fmaxf(hi[a], c[k].hi[a]); }
    float off[8][3];
    for (int k = 0; k < cnt; ++k)
        for (int a = 0; a < 3; ++a) off[k][a] = 0.5f * (c[k].lo[a] + c[k].hi[a]) - 0.5f * (lo[a] + hi[a]);
    // greedy assignment: repeatedly the (child, slot) pair of largest alignment between the child's
    // offset and the slot's octant direction among the unassigned ones (ties: lower child, slot)
    int slotOf[8], childIn[8];
    for (int k = 0; k < 8; ++k) { slotOf[k] = -1; childIn[k] = -1; }
    for (int n = 0; n < cnt; ++n) {
        float bestV = -CUDART_INF_F;
        int bc = -1, bs = -1;
        for (int k = 0; k < cnt; ++k) {
            if (slotOf[k] >= 0) continue;
            for (int s = 0; s < 8; ++s) {
                if (childIn[s] >= 0) continue;
                float v = ((s & 1) ? off[k][0] : -off[k][0]) + ((s & 2) ? off[k][1] : -off[k][1]) + ((s & 4) ? off[k][2] : -off[k][2]);
                if (v > bestV) { bestV = v; bc = k; bs = s; }
            }
        }
        slotOf[bc] = bs;
        childIn[bs] = bc;
    }
    float v[6][8];
    uint32_t refs[8];
    uint32_t valid = 0, inner = 0;
    for (int s = 0; s < 8; ++s) {
        const int k = childIn[s];
        if (k >= 0) {
            for (int a = 0; a < 3; ++a) { v[2 * a][s] = c[k].lo[a]; v[2 * a + 1][s] = c[k].hi[a]; }
            uint32_t r = c[k].ref;
            valid |= 1u << s;
            if (!(r & kLeafFlag)) {
                int slot = atomicAdd(nodeCounter, 1);
                next[atomicAdd(nNext, 1)] = make_int2((int)r, slot);
                r = (uint32_t)slot;
                inner |= 1u << s;
            }
            refs[s] = r;
        } else {
            for (int a = 0; a < 6; ++a) v[a][s] = 0.0f;
            refs[s] = 0u;
        }
    }
    float4* out = nodes8 + 15 * (size_t)item.y;
    for (int a = 0; a < 6; ++a) {
        out[2 * a] = make_float4(v[a][0], v[a][1], v[a][2], v[a][3]);
        out[2 * a + 1] = make_float4(v[a][4], v[a][5], v[a][6], v[a][7]);
    }
    out[12] = make_float4(__uint_as_float(refs[0]), __uint_as_float(refs[1]), __uint_as_float(refs[2]), __uint_as_float(refs[3]));
    out[13] = make_float4(__uint_as_float(refs[4]), __uint_as_float(refs[5]), __uint_as_float(refs[6]), __uint_as_float(refs[7]));
    out[14] = make_float4(__uint_as_float(valid | (inner << 8)), 0.0f, 0.0f, 0.0f);
}
}  // namespace

size_t bvh8ScratchBytes(int nNodes2) { return 2 * sizeof(int2) * (size_t)std::max(1, nNodes2) + 1024; }

int buildBvh8(const float4* nodes2, int nNodes2, float4* nodes8, void* scratch, int* hostNodeCount, int* hostDepth, cudaStream_t st) {
    *hostNodeCount = 0;
    *hostDepth = 0;
    if (nNodes2 <= 0) return 0;
    char* p = static_cast<char*>(scratch);
    int* counters = reinterpret_cast<int*>(p);  // [0] node counter, [1], [2] frontier sizes
    int2* fr[2] = {reinterpret_cast<int2*>(p + 256), reinterpret_cast<int2*>(p + 256) + nNodes2};
    k_collapse_root<<<1, 1, 0, st>>>(fr[0], counters + 1, counters);
    int cur = 0, depth = 0, n = 1;
    int hostCnt = 0;
    while (n > 0) {
        if (++depth > 4 * kMaxBvhDepth) return -2;
        if (cudaMemsetAsync(counters + 2 - cur, 0, sizeof(int), st) != cudaSuccess) return -1;
        k_collapse8<<<(n + 127) / 128, 128, 0, st>>>(nodes2, fr[cur], counters + 1 + cur, nodes8, counters, fr[1 - cur], counters + 2 - cur);
        if (cudaMemcpyAsync(&n, counters + 2 - cur, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
        cur = 1 - cur;
    }
    if (cudaMemcpyAsync(&hostCnt, counters, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    *hostNodeCount = hostCnt;
    *hostDepth = depth;
    return 0;
}
}  // namespace sst

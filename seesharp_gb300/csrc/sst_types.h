// Device-side scene and wavefront layouts shared by the kernels and the host driver.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sst {

constexpr int kMaxShadowRays = 4;     // NumShadowRays supported per vertex
constexpr int kTraceBlock = 128;      // threads per block of the traversal kernels
constexpr int kSmemStack = 24;        // traversal stack entries kept in shared memory per thread
constexpr int kTraceRefillIdle = 20;  // idle lanes of a warp at which the 4-wide traversal takes new rays
constexpr int kMaxStack = 64;         // total stack entries (the BVH builder caps the depth below this)
constexpr int kMaxStack4 = 192;       // 4-wide traversal: at most 3 pending children per level of at most 60 levels
constexpr int kMaxBvhDepth = 60;
constexpr int kMaxLeafSize = 8;

// Node references: >= 0 inner node index; leaf = 0x80000000 | (count - 1) << 27 | first
constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr int kLeafCountShift = 27;
constexpr uint32_t kLeafFirstMask = (1u << kLeafCountShift) - 1u;

enum MaterialType : int { kDiffuse = 0, kGeneric = 1 };

struct DevMaterial {
    int type;
    int baseTex;   // texture index or -1
    int roughTex;  // texture index or -1
    int transmitter;
    float base[3];
    float rough;
    float metallic, specTint, aniso, specTrans, ior;
    int pad[1];
};

struct DevTexture {
    int w, h, channels, border;
    long long offset;  // float offset into the texel pool
};

// One emissive triangle with everything NEE needs (DiffuseEmitter / GlossyEmitter + Triangle)
struct DevEmitter {
    float4 v1, v2, v3;   // vertex positions (mesh order)
    float4 n1, n2, n3;   // vertex shading normals; n1.w = 1 when the mesh has them
    float4 faceN;        // face normal xyz, w = 1 / area
    float4 rad;          // radiance rgb, w = glossy exponent (< 0: diffuse)
    float norm;          // (exponent + 1) / (2 pi)
    int globalTri;
    int mesh, face;      // the emitter's mesh and face
};

struct DevEnv {
    int w, h;
    const float4* img;     // w*h texels (rgb, pad)
    const float* rowCdf;   // h
    const float* colCdf;   // h*w
    const int* hasCol;     // h
};

struct DevCamera {
    float v2c[16];  // viewToCamera (row-major, row-vector convention)
    float c2w[16];  // cameraToWorld
    int W, H;
};

struct DevScene {
    const float4* nodes;   // binary BVH: 4 float4 per node
    const float4* nodes4;  // 4-wide BVH over the same leaves: 8 float4 per node
    const float4* nodes8;  // 8-wide BVH over the same leaves, octant slots: 15 float4 per node
    const float4* triv;    // 3 float4 per leaf-ordered triangle: v1 (w = global tri id), v2, v3
    const float4* triN;    // per leaf-ordered triangle: face normal, w = emitter index (int bits, -1)
    const int4* triAux;    // (material, mesh, local face, attribute flags: 1 normals, 2 uvs)
    const int4* triVtx;    // global vertex indices of the three corners
    const float* vnrm;     // 3 floats per global vertex (0 when absent)
    const float* vuv;      // 2 floats per global vertex
    const DevMaterial* mats;
    const DevTexture* texs;
    const float* texData;
    const DevEmitter* emitters;
    int nEmitters;
    int nTri;
    int nNodes;
    int nNodes4;
    int nNodes8;
    int hasEnv;
    float3 sceneCenter;  // Scene.Center / Scene.Radius (Scene.cs:115-136)
    float sceneRadius;
    DevEnv env;
    DevCamera cam;
};

struct PTConfig {
    int W, H;
    int maxDepth, minDepth;
    uint32_t baseSeed;
    int numShadowRays;
    int enableBsdfDI;
    int ignoreNan;
    int shadingStats;  // count material calls (every next-event shadow ray is traced)
};

// Path-replay adjoint buffers of a job (all NULL for a plain render).
struct DevAdj {
    float* record;        // per (iteration, pixel) path radiance: written by the forward fold, read by the replay
    const float* dLdI;    // dLoss/dImage (W*H*3) for the replay
    float invSpp;         // 1 / totalSpp: dImage/dSample
    float* gTex;          // gradient of the texel pool (layout of DevScene.texData)
    float* gMatBase;      // 3 per material: constant base colour
    float* gMatRough;     // 1 per material: constant roughness
    float* gEmitter;      // 3 per emitter: radiance
};

// Light paths (sst_light.cu)
struct LightParams {
    int numPaths, maxDepth;
    uint32_t seed, iter;
};
struct LightPathBuf {  // structure of arrays of the light paths in flight
    uint32_t* path;    // path index
    uint32_t* rng;     // RNG state
    uint32_t* depth;   // depth | flags
    float4* prefix;    // prefix weight, w = pdf of the last sampled direction
    float4* approx;    // approximate throughput, w = reverse pdf for the next vertex
    float4* prevP;     // previous vertex position
    float4* prevN;     // previous vertex face normal
    float4* ro;        // ray origin, w = tmin
    float4* rd;        // ray direction, w = tmax
};
struct SstHitDev {  // the layout of SstHit
    float d, u, v;
    int prim, mesh;
    float eps;
    float p[3];
    float n[3];
};
struct SstPathVertexDev {  // the layout of SstPathVertex
    float p[16];
    int q[6];
};

// Frame-buffer layers of a job (all NULL unless requested).
struct DevLayers {
    float* varMean;     // per pixel: running mean of the iteration's pixel value (VarianceLayer meanImage)
    float* varMoment;   // per pixel: running mean of its square (VarianceLayer momentImage)
    const float* ref;   // W*H*3 reference image for the per-iteration error metrics
    double* errSum;     // 2 per iteration: sums of squared and of relative squared errors
    float* aovAlbedo;   // W*H*3 running mean of the primary hit's scatter strength
    float* aovNormal;   // W*H*3 running mean of the primary hit's shading normal
    float* aovSamples;  // 6 per wave item: this iteration's (albedo, normal), written by the first shade
    float* errPix;      // (iteration - errFirst) * W*H + pixel: the pixel's relative squared error after the
                        // iteration (mean over the channels), for the outlier-rejecting RelMSE
    int errFirst;       // first iteration of the call
    int nOut;           // OutlierReplayCache heap capacity per pixel (0: not tracked), at most kMaxOutliers
    float* outW;        // W*H*nOut heap priorities: the sample's channel average, 4-ary min-heap order
    int* outIt;         // W*H*nOut heap elements: the sample's 0-based iteration, -1 for an empty slot
    float* pyr;         // technique pyramids (raw, then MIS-weighted): 2 * 2*maxDepth layers of W*H*3;
                        // layer 2(d-1) is "{d}-hit", 2(d-1)+1 "{d}-next-event"
    int pyrSpp;         // TotalSpp: every registered sample is divided by it
};
constexpr int kMaxOutliers = 8;

// One render job: its scene and path-tracer settings (the kernels index this table by the job
// id every path carries).
struct DevJob {
    DevScene sc;
    PTConfig cfg;
    DevAdj adj;
    DevLayers lay;
};

// A chunk of a wave: nIter consecutive iterations of the pixel range [pixStart, pixStart +
// pixCount) of one job.  Wave items [itemOffset, itemOffset + nIter * pixCount) are its paths
// (iteration-major); fold threads [foldOffset, foldOffset + pixCount) fold them into the film.
struct WaveChunk {
    int job;
    int iterBase;
    int nIter;
    int pixStart;
    int pixCount;
    int itemOffset;
    int foldOffset;
    int pad;
    float* film;
};

// Technique-pyramid arguments of the shade kernel: the wave's chunk table (to map a wave item to
// its pixel) and the payload of each queued next-event sample (its contribution and MIS weight,
// added to the pyramid once the shadow ray has found it visible).
struct WaveDesc;
struct PyrArgs {
    const WaveChunk* chunks;
    const WaveDesc* waves;
    const int* curWave;
    float4* pyrG;  // one per NEE slot
};

// Per-wave parameters read by the kernels from device memory, so that the same kernel sequence
// (and one captured CUDA graph) serves every wave.
struct WaveDesc {
    int chunkBegin, chunkEnd;  // chunk index range
    int items;                 // paths in the wave
    int foldThreads;           // pixels to fold
};

// Device counters of one render (zeroed per render).
struct DevStats {
    unsigned long long rays;
    unsigned long long shadowRays;
    unsigned long long nanCount;
    // the four smallest keys (1-based iteration << 32 | pixel index) of the non-finite estimates,
    // stored complemented (~key) in descending order, 0 for an unused entry (see logNan)
    unsigned long long nanKey[4];
    unsigned long long matEvalPdf;  // ShadingStats: material evaluations (each comes with a pdf here)
    unsigned long long matSample;   // ShadingStats: material samples
    int errorFlags;  // bit 0: traversal stack overflow
    int pad[3];
};

// Structure-of-arrays path state for one buffer (double-buffered A/B).
struct PathBuf {
    uint32_t* job;     // render job of the path
    uint32_t* pix;
    uint32_t* rng;
    uint32_t* depth;   // bits 0-15 depth, 16-23 pending NEE slots, bit 31 done
    float4* pw;        // prefix weight rgb, previous pdf
    float4* rad;       // radiance estimate rgb
    float4* prev;      // previous hit position
    float4* ro;        // ray origin, tmin
    float4* rd;        // ray direction, tmax
    uint32_t* neeFrom; // the path's index in the previous queue: its pending next-event slots are at
                       // slot * cap + neeFrom (read only when the depth word has pending slots)
    float4* rec;       // split shade form only: per queued path, what the first kernel hands the second
                       // (kShadeRec float4 planes of the queue's capacity); NULL otherwise
    // adjoint replay only (NULL otherwise)
    float4* adjL;      // path radiance from the forward pass, w = base-colour target (int bits)
    float4* adjD;      // dLoss/dSample per channel, w = roughness target (int bits)
    float4* adjP;      // 3 float4 per path: d ln f_c / d(base r, g, b, roughness) of the pending BSDF factor
    // shade input only: the order in which the shade kernel's threads take the queued paths
    // (thread t shades path order[t]); NULL: thread t shades path t
    const int* order;
    // shade input only: the next-event slots of the queued paths, written by the previous bounce.
    // The shade kernel writes the next bounce's slots into the other buffer of the pair, so no
    // thread reads a slot that another thread of the same launch writes.
    const float4* neeIn;
    const float4* neeGIn;  // adjoint payloads of those slots
    const float4* pyrGIn;  // technique-pyramid payloads of those slots
};

constexpr uint32_t kDepthMask = 0xFFFFu;
constexpr int kShadeRec = 5;                  // float4 planes of PathBuf.rec (the split shade form)
constexpr uint32_t kRecSample = 0x80000000u;  // PathBuf.rec flag: the path goes on to BSDF sampling
constexpr int kNeeShift = 16;
constexpr uint32_t kDoneFlag = 0x80000000u;
constexpr uint32_t kAdjFactorFlag = 0x40000000u;  // adjoint: a BSDF-factor gradient is pending

struct WaveBuffers {
    PathBuf a, b;
    float4* hits;        // per path of the current queue: t, u, v, leaf triangle (int bits, -1 miss)
    float4* nee;         // [slot * cap + path]: pending NEE contribution, w = 1 until occluded
    float4* neeG;        // adjoint: 3 float4 per NEE slot, the gradient payload
    float4* shRo;        // shadow queue: origin, tmin
    float4* shRd;        // direction, tmax
    int* shTgt;          // nee slot index
    uint32_t* shJob;     // render job of the shadow ray
    int* counters;       // per bounce queue lengths and work counters
    int* order;          // shade order of the current queue (k_partition)
    int cap;             // paths per wave
    int shCap;           // shadow queue capacity
};

// Counter layout (ints): [0, 1024) queue length per depth; [1024, 2048) shadow-queue length per
// depth; [2048, 4096) work-fetch counters of the persistent traversal kernels (two per depth);
// [4096, 6144) append counters of the shade-order partition (two per depth).
constexpr int kMaxPathDepth = 1000;
constexpr int kCntQueue = 0;
constexpr int kCntShadow = 1024;
constexpr int kCntWork = 2048;
constexpr int kCntPart = 4096;
constexpr int kNumCounters = 6144;

}  // namespace sst

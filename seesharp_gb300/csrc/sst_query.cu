// Ray queries, the TinyEmbree Raytracer.Trace / IsOccluded drop-ins (Integrators/PathTracer.cs:319,467),
// their allocation-free form, and the light-path random walk (LightPathCache.TraceAllPaths).
#include "sst_host.h"

// A one-entry job table holding the scene (for the ray-query entry points).
const DevJob* jobTable(sst_scene* s) {
    DevJob j{};
    j.sc = s->dev;
    s->queryJob.ensure(sizeof(DevJob));
    CUDA_CHECK(cudaMemcpyAsync(s->queryJob.p, &j, sizeof(DevJob), cudaMemcpyHostToDevice, s->ctx->stream));
    return s->queryJob.as<DevJob>();
}

// Trace / IsOccluded over n rays.  The rays are split into origin and direction arrays and the
// results written by the device (sst_trace: the SstHit records are expanded on the device from the
// traversal's (t, u, v, triangle) records); host results come back in one copy.  The buffers are
// the context's and only grow, so repeated queries of the same size allocate nothing.
static void runQuery(sst_scene* s, const SstRay* rays, int n, SstHit* hits, int32_t* occl, int memory, bool anyHit) {
    static_assert(sizeof(SstHit) == sizeof(SstHitDev), "hit layout");
    if (!s || (n > 0 && !rays) || n < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid query");
    if (memory != SST_MEM_HOST && memory != SST_MEM_DEVICE) fail(SST_ERR_INVALID_ARGUMENT, "memory must be SST_MEM_HOST or SST_MEM_DEVICE");
    if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
    if (n == 0) return;
    sst_ctx* c = s->ctx;
    CUDA_CHECK(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const cudaMemcpyKind in = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind out = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    // separate origin / direction arrays (SstRay = org, tmin, dir, tmax = two float4)
    c->qRo.ensure(size_t(n) * 16);
    c->qRd.ensure(size_t(n) * 16);
    CUDA_CHECK(cudaMemcpy2DAsync(c->qRo.p, 16, rays, 32, 16, size_t(n), in, st));
    CUDA_CHECK(cudaMemcpy2DAsync(c->qRd.p, 16, reinterpret_cast<const char*>(rays) + 16, 32, 16, size_t(n), in, st));
    c->qCnt.ensure(sizeof(int) * 2);
    c->pinnedCount[0] = n;
    c->pinnedCount[1] = 0;
    CUDA_CHECK(cudaMemcpyAsync(c->qCnt.p, c->pinnedCount, sizeof(int) * 2, cudaMemcpyHostToDevice, st));
    c->stats.ensure(sizeof(DevStats));
    CUDA_CHECK(cudaMemsetAsync(c->stats.p, 0, sizeof(DevStats), st));
    int* cnt = c->qCnt.as<int>();
    if (anyHit) {
        int* dOcc = occl;
        if (memory != SST_MEM_DEVICE) {
            c->qOut.ensure(size_t(n) * 4);
            dOcc = c->qOut.as<int>();
        }
        const TraceTuning tt = traceForBuilding(c, &s, 1);
        launch_trace_query(tt, jobTable(s), c->qRo.as<float4>(), c->qRd.as<float4>(), cnt, cnt + 1, nullptr, dOcc, c->stats.as<DevStats>(), true, st);
        CUDA_CHECK(cudaGetLastError());
        if (memory != SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpyAsync(occl, dOcc, size_t(n) * 4, out, st));
    } else {
        c->qHits.ensure(size_t(n) * 16);
        const TraceTuning tt = traceForBuilding(c, &s, 1);
        launch_trace_query(tt, jobTable(s), c->qRo.as<float4>(), c->qRd.as<float4>(), cnt, cnt + 1, c->qHits.as<float4>(), nullptr, c->stats.as<DevStats>(),
                           false, st);
        SstHitDev* dHits = reinterpret_cast<SstHitDev*>(hits);
        if (memory != SST_MEM_DEVICE) {
            c->qOut.ensure(size_t(n) * sizeof(SstHitDev));
            dHits = c->qOut.as<SstHitDev>();
        }
        launch_hit_expand(s->dev, c->qHits.as<float4>(), n, dHits, st);
        CUDA_CHECK(cudaGetLastError());
        if (memory != SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpyAsync(hits, dHits, size_t(n) * sizeof(SstHitDev), out, st));
    }
    DevStats hs;
    CUDA_CHECK(cudaMemcpyAsync(&hs, c->stats.p, sizeof(DevStats), cudaMemcpyDeviceToHost, st));
    CUDA_CHECK(cudaStreamSynchronize(st));
    if (hs.errorFlags & 1) fail(SST_ERR_DEVICE_LIMIT, "BVH traversal stack overflow");
}

static LightPathBuf bindLight(DevBuf* b, size_t cap) {
    const size_t sz[9] = {4, 4, 4, 16, 16, 16, 16, 16, 16};
    for (int k = 0; k < 9; ++k) b[k].ensure(cap * sz[k]);
    LightPathBuf l;
    l.path = b[0].as<uint32_t>();
    l.rng = b[1].as<uint32_t>();
    l.depth = b[2].as<uint32_t>();
    l.prefix = b[3].as<float4>();
    l.approx = b[4].as<float4>();
    l.prevP = b[5].as<float4>();
    l.prevN = b[6].as<float4>();
    l.ro = b[7].as<float4>();
    l.rd = b[8].as<float4>();
    return l;
}

extern "C" {

int sst_trace(sst_scene* s, const SstRay* rays, int32_t n, SstHit* hits, int32_t memory) {
    return guarded([&] {
        if (!hits && n > 0) fail(SST_ERR_INVALID_ARGUMENT, "hits is NULL");
        runQuery(s, rays, n, hits, nullptr, memory, false);
    });
}

int sst_occluded(sst_scene* s, const SstRay* rays, int32_t n, int32_t* occluded, int32_t memory) {
    return guarded([&] {
        if (!occluded && n > 0) fail(SST_ERR_INVALID_ARGUMENT, "occluded is NULL");
        runQuery(s, rays, n, nullptr, occluded, memory, true);
    });
}


int sst_trace_light_paths(sst_scene* s, uint32_t seed, uint32_t iteration, int32_t numPaths, int32_t maxDepth, SstPathVertex* vertices,
                          int32_t* lengths, int32_t memory, SstRenderStats* stats) {
    static_assert(sizeof(SstPathVertex) == sizeof(SstPathVertexDev), "path vertex layout");
    return guarded([&] {
        if (!s || numPaths < 0 || numPaths > (1 << 24) || maxDepth < 1 || maxDepth > kMaxPathDepth || (numPaths > 0 && (!vertices || !lengths)))
            fail(SST_ERR_INVALID_ARGUMENT, "invalid light-path query");
        if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        SstRenderStats local = emptyStats();
        if (numPaths == 0) { if (stats) *stats = local; return; }
        sst_ctx* c = s->ctx;
        cudaStream_t st = c->stream;
        CUDA_CHECK(cudaSetDevice(c->device));
        const size_t n = size_t(numPaths), stride = size_t(maxDepth) + 1;
        LightPathBuf A = bindLight(c->lightA, n), B = bindLight(c->lightB, n);
        c->lightHits.ensure(n * 16);
        SstPathVertexDev* dv = reinterpret_cast<SstPathVertexDev*>(vertices);
        int* dl = lengths;
        if (memory != SST_MEM_DEVICE) {
            c->lightVerts.ensure(n * stride * sizeof(SstPathVertexDev));
            c->lightLengths.ensure(n * 4);
            dv = c->lightVerts.as<SstPathVertexDev>();
            dl = c->lightLengths.as<int>();
        }
        CUDA_CHECK(cudaMemsetAsync(dv, 0, n * stride * sizeof(SstPathVertexDev), st));
        c->lightCnt.ensure(sizeof(int) * 2 * (size_t(maxDepth) + 3));
        int* cnt = c->lightCnt.as<int>();
        CUDA_CHECK(cudaMemsetAsync(cnt, 0, sizeof(int) * 2 * (size_t(maxDepth) + 3), st));
        c->stats.ensure(sizeof(DevStats));
        CUDA_CHECK(cudaMemsetAsync(c->stats.p, 0, sizeof(DevStats), st));
        const TraceTuning tt = traceForBuilding(c, &s, 1);
        const DevJob* job = jobTable(s);
        LightParams P{numPaths, maxDepth, seed, iteration};
        CUDA_CHECK(cudaEventRecord(c->ev0, st));
        launch_light_start(job, P, A, cnt, dv, dl, st);
        CUDA_CHECK(cudaGetLastError());
        int items = 0;
        CUDA_CHECK(cudaMemcpyAsync(&items, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        // each step: closest hit, then one walk step (a path reaches at most maxDepth + 1 hits)
        for (int d = 0; d <= maxDepth && items > 0; ++d) {
            int* qIn = cnt + d;
            int* qOut = cnt + d + 1;
            int* work = cnt + (maxDepth + 2) + d;
            launch_trace_closest(tt, job, nullptr, A.ro, A.rd, qIn, work, c->lightHits.as<float4>(), c->stats.as<DevStats>(), st);
            launch_light_walk(job, P, A, B, c->lightHits.as<float4>(), qIn, qOut, dv, dl, items, st);
            CUDA_CHECK(cudaGetLastError());
            std::swap(A, B);
            CUDA_CHECK(cudaMemcpyAsync(&items, qOut, sizeof(int), cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
        }
        CUDA_CHECK(cudaEventRecord(c->ev1, st));
        if (memory != SST_MEM_DEVICE) {
            CUDA_CHECK(cudaMemcpyAsync(vertices, dv, n * stride * sizeof(SstPathVertexDev), cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaMemcpyAsync(lengths, dl, n * 4, cudaMemcpyDeviceToHost, st));
        }
        DevStats hs;
        CUDA_CHECK(cudaMemcpyAsync(&hs, c->stats.p, sizeof(DevStats), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (hs.errorFlags & 1) fail(SST_ERR_DEVICE_LIMIT, "BVH traversal stack overflow");
        float ms = 0.f;
        CUDA_CHECK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        local.renderTimeMs = ms;
        local.numRays = hs.rays;
        if (stats) *stats = local;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free occlusion query (sst_occluded_noalloc).  Its scratch is one array of fixed size
// in this library's device image, laid out as
//   [0, 256)      queue length and work counter of the traversal kernel
//   [256, 512)    DevStats (ray counts)
//   [512, 2048)   DevJob (the scene record the traversal kernel reads)
//   then          ray origins (float4 x max rays), ray directions (float4 x max rays),
//                 occlusion flags (int x max rays).
// ---------------------------------------------------------------------------------------------
namespace {
constexpr size_t kNaCounters = 0, kNaStats = 256, kNaJob = 512, kNaHeader = 2048;
constexpr size_t kNaMaxRays = SST_NOALLOC_MAX_RAYS;
constexpr size_t kNaBytes = kNaHeader + 2 * 16 * kNaMaxRays + 4 * kNaMaxRays;
static_assert(kNaBytes == 2361344, "the header states the scratch size");
static_assert(sizeof(DevStats) <= kNaJob - kNaStats && sizeof(DevJob) <= kNaHeader - kNaJob, "scratch header too small");
static_assert(alignof(DevJob) <= 256 && alignof(DevStats) <= 256, "scratch header alignment");
constexpr int kNaMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_noallocScratch[kNaBytes];
static std::mutex g_noallocLock;
static void* g_noallocAddr[kNaMaxDevices] = {};

// Device address of the scratch array on `device` (the current device).  Looked up on the first
// call for each device and kept; the caller holds g_noallocLock.
static unsigned char* noallocScratch(int device) {
    if (device < 0 || device >= kNaMaxDevices) fail(SST_ERR_INVALID_ARGUMENT, "device ordinal beyond the allocation-free query's table");
    if (!g_noallocAddr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noallocScratch);
        if (e != cudaSuccess || !ptr) fail(SST_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noallocAddr[device] = ptr;
    }
    return static_cast<unsigned char*>(g_noallocAddr[device]);
}

extern "C" int sst_occluded_noalloc(sst_scene* s, const SstRay* rays, int32_t n, int32_t* occluded, int32_t memory) {
    return guarded([&] {
        if (!s || n < 0 || (n > 0 && (!rays || !occluded))) fail(SST_ERR_INVALID_ARGUMENT, "invalid query");
        if (memory != SST_MEM_HOST && memory != SST_MEM_DEVICE) fail(SST_ERR_INVALID_ARGUMENT, "memory must be SST_MEM_HOST or SST_MEM_DEVICE");
        if (size_t(n) > kNaMaxRays)
            fail(SST_ERR_INVALID_ARGUMENT, "sst_occluded_noalloc: " + std::to_string(n) + " rays exceed the limit of " + std::to_string(kNaMaxRays) +
                                               " rays per call (SST_NOALLOC_MAX_RAYS)");
        if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (n == 0) return;
        std::lock_guard<std::mutex> lock(g_noallocLock);
        sst_ctx* c = s->ctx;
        CUDA_CHECK(cudaSetDevice(c->device));
        unsigned char* base = noallocScratch(c->device);
        cudaStream_t st = c->stream;
        int* cnt = reinterpret_cast<int*>(base + kNaCounters);
        DevStats* stats = reinterpret_cast<DevStats*>(base + kNaStats);
        DevJob* job = reinterpret_cast<DevJob*>(base + kNaJob);
        float4* ro = reinterpret_cast<float4*>(base + kNaHeader);
        float4* rd = ro + kNaMaxRays;
        int* occ = reinterpret_cast<int*>(rd + kNaMaxRays);
        const cudaMemcpyKind in = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        const cudaMemcpyKind out = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        // SstRay = {org, tmin, dir, tmax}: split into the origin and direction arrays
        CUDA_CHECK(cudaMemcpy2DAsync(ro, 16, rays, 32, 16, size_t(n), in, st));
        CUDA_CHECK(cudaMemcpy2DAsync(rd, 16, reinterpret_cast<const char*>(rays) + 16, 32, 16, size_t(n), in, st));
        // set every call: the queue length (n), the work counter and the statistics (zero), the job
        const int hostCnt[2] = {n, 0};
        CUDA_CHECK(cudaMemcpyAsync(cnt, hostCnt, sizeof(hostCnt), cudaMemcpyHostToDevice, st));
        CUDA_CHECK(cudaMemsetAsync(stats, 0, sizeof(DevStats), st));
        DevJob j{};
        j.sc = s->dev;
        CUDA_CHECK(cudaMemcpyAsync(job, &j, sizeof(DevJob), cudaMemcpyHostToDevice, st));
        launch_trace_query(traceFor(c, &s, 1), job, ro, rd, cnt, cnt + 1, nullptr, occ, stats, true, st);
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaMemcpyAsync(occluded, occ, size_t(n) * 4, out, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}


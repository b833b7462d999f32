// Private header of libsst's host driver (the C ABI of include/sst.h): error handling, device and
// pinned buffers, the context and scene records, and the functions the driver's translation
// units share.
//   sst_api.cu          context and scene construction, kernel timing, function-level entry points
//   sst_commit.cu       Scene.Prepare (sst_scene_commit): triangle tables, BVH build, emitter tables
//   sst_render.cu       the wavefront renderer (wave planning, renderJobs), sst_render*, tuning
//   sst_adjoint_api.cu  sst_forward / sst_backward and their batched forms
//   sst_query.cu        ray queries (sst_trace, sst_occluded, sst_occluded_noalloc), light paths
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sst.h"
#include "sst_bvh.h"
#include "sst_kernels.h"
#include "sst_types.h"

using namespace sst;

// ---------------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------------
extern thread_local std::string g_lastError;

struct SstException {
    int code;
    std::string msg;
};
[[noreturn]] inline void fail(int code, const std::string& msg) { throw SstException{code, msg}; }
#define CUDA_CHECK(x)                                                                                         \
    do {                                                                                                      \
        cudaError_t e_ = (x);                                                                                 \
        if (e_ != cudaSuccess) {                                                                              \
            fail(e_ == cudaErrorMemoryAllocation ? SST_ERR_OUT_OF_MEMORY : SST_ERR_CUDA,                      \
                 std::string(#x) + ": " + cudaGetErrorString(e_));                                            \
        }                                                                                                     \
    } while (0)

template <class F> int guarded(F&& f) {
    try {
        f();
        return SST_OK;
    } catch (const SstException& e) {
        g_lastError = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        g_lastError = "host out of memory";
        return SST_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_lastError = e.what();
        return SST_ERR_INVALID_ARGUMENT;
    }
}

// ---------------------------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t b) {
        if (b <= bytes) return;
        release();
        CUDA_CHECK(cudaMalloc(&p, b));
        bytes = b;
    }
    template <class T> void upload(const std::vector<T>& v, cudaStream_t s) {
        ensure(std::max<size_t>(1, v.size() * sizeof(T)));
        if (!v.empty()) CUDA_CHECK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    template <class T> void upload(const T* v, size_t n, cudaStream_t s) {
        ensure(std::max<size_t>(1, n * sizeof(T)));
        if (n) CUDA_CHECK(cudaMemcpyAsync(p, v, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Page-locked host memory that only grows (one per context): staging for large uploads, so that
// the copies run as asynchronous DMA and the pages stay resident from one scene commit to the next.
struct PinnedBuf {
    void* p = nullptr;
    size_t bytes = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t b) {
        if (b <= bytes) return;
        release();
        CUDA_CHECK(cudaHostAlloc(&p, b, cudaHostAllocDefault));
        bytes = b;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Runs fn(begin, end) over [0, n) in contiguous ranges on up to 16 host threads (one range per
// thread, at least minPerThread items each).  fn must not throw.
template <class F>
void parallelRanges(size_t n, size_t minPerThread, F fn) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), (n + minPerThread - 1) / std::max<size_t>(1, minPerThread));
    if (nt <= 1) {
        fn(size_t(0), n);
        return;
    }
    const size_t chunk = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) {
        size_t b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back(fn, b, e);
    }
    fn(size_t(0), std::min(n, chunk));
    for (auto& x : th) x.join();
}

// Faults in the pages of host output buffers on a helper thread while the GPU renders, so that the
// read-back afterwards runs at link speed.  A device-to-host copy into pages the process has not
// touched yet (a fresh numpy or malloc buffer) is bound by page faults: on the Grace host the 71 MB
// of film, denoiser layers and outlier cache of a 1024x1024 render took 10 ms that way, against
// 0.4 ms into touched pages.  Each page is read and the same byte written back, so the contents
// (the input of a resumed render) are unchanged.
class HostPrefault {
public:
    void add(void* p, size_t bytes) {
        if (p && bytes) bufs_.push_back({static_cast<char*>(p), bytes});
    }
    void start() {
        if (!bufs_.empty()) th_ = std::thread([this] { run(); });
    }
    void finish() {
        if (th_.joinable()) th_.join();
    }
    ~HostPrefault() { finish(); }

private:
    void run() {
        const size_t step = 4096;
        for (auto& b : bufs_) {
            volatile char* c = b.first;
            for (size_t off = 0; off < b.second; off += step) {
                const char v = c[off];
                c[off] = v;
            }
        }
    }
    std::vector<std::pair<char*, size_t>> bufs_;
    std::thread th_;
};

// ---------------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------------
// A job of the last sst_forward_batch (what sst_backward_batch must match).
struct BatchSig {
    sst_scene* scene;
    SstPathTracerParams params;
    bool hasCam;
    SstCamera cam;
};

// One set of wavefront buffers: path state (A and B), hits, next-event slots, shadow-ray queue,
// counters, shade order, per-item path estimates, the split shade form's record, the denoiser
// feature samples and the job table that points at them.  The context keeps kMaxWaveSets, so
// that that many waves can be in flight.
constexpr int kMaxWaveSets = 3;
struct WaveStore {
    DevBuf pathA[10], pathB[10];
    DevBuf hits, nee, shRo, shRd, shTgt, shJob, counters, order, samples, rec, aov, jobs;
    DevBuf adjA[3], adjB[3], neeG;  // the adjoint replay's per-path state and next-event payloads
    int cap = 0, neeSlots = 0;
    // its streams: the bounces (and, with one wave in flight, everything) run on `run`, a bounce's
    // shadow rays on `side` (evShade: the bounce's shade is done; evShadow: its shadow rays are;
    // evDone: the wave's bounces are done)
    cudaStream_t run = nullptr, side = nullptr;
    cudaEvent_t evShade = nullptr, evShadow = nullptr, evDone = nullptr, evFolded = nullptr;
};

struct sst_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int numSMs = 0;
    // scene commit: pinned staging of the packed triangle records and the BVH build's temporaries
    // (kept across commits: no allocation or device-wide free per Scene.Prepare once they fit)
    PinnedBuf commitStage;
    DevBuf commitTri[4], commitOrder, commitScratch, commitScratch4, commitScratch8;
    // wavefront buffers (store[1..] only while several waves are in flight)
    WaveStore store[kMaxWaveSets];
    DevBuf stats, film;
    DevBuf chunksBuf, wavesBuf, curWave;
    // ray queries (sst_trace, sst_occluded): split rays, queue counters, traversal records, results
    DevBuf qRo, qRd, qCnt, qHits, qOut;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evStart = nullptr;
    int* pinnedCount = nullptr;
    // light paths (sst_trace_light_paths)
    DevBuf lightA[9], lightB[9], lightHits, lightVerts, lightLengths, lightCnt;
    // frame-buffer layers (sst_render_layers)
    DevBuf layMean, layRef, layErr, layVar, laySum, layAlb, layNrm, layErrPix, layTrim, layOutW, layOutIt, layPyr, pyrG;
    // batched adjoint: the jobs of the last sst_forward_batch, their path radiance, dLoss/dImage
    std::vector<BatchSig> batchSig;
    std::vector<std::unique_ptr<DevBuf>> batchRecord, batchDLdI;
    // launch configuration (sst_set_tuning / sst_autotune)
    TraceTuning trace;
    int waveCapacity = 0;  // 0: the default
    int shadeBlocks = 8;   // resident blocks per SM of the forward shade kernel with GenericMaterials: 8, 10, 12 or 14
    int shadeOrder = 1;    // 1: each bounce's queue is shaded surface hits first (k_partition); 0: in queue order
    int shadeSplit = 1;    // 1: the forward shade kernel with GenericMaterials runs as two kernels per bounce (sst_shade_split.cu)
    // ShadingStats counting (sst_set_shading_stats)
    bool shadingStats = false;
    // kernel timing (sst_set_profiling)
    bool profiling = false;
    std::vector<cudaEvent_t> evPool;
    std::vector<std::pair<int, int>> evMarks;  // (class, event index of the start)
    double kMs[SST_KERNEL_CLASSES] = {};
    int64_t kLaunches[SST_KERNEL_CLASSES] = {};
    int64_t kItems[SST_KERNEL_CLASSES] = {};
};

// Kernel timing: an event pair around each launch, read back after the wave.
struct KTimer {
    sst_ctx* c;
    int cls;
    int start;
    KTimer(sst_ctx* ctx, int k) : c(ctx), cls(k), start(-1) {
        if (!c->profiling) return;
        start = int(c->evMarks.size()) * 2;
        while (int(c->evPool.size()) < start + 2) {
            cudaEvent_t e;
            CUDA_CHECK(cudaEventCreate(&e));
            c->evPool.push_back(e);
        }
        CUDA_CHECK(cudaEventRecord(c->evPool[start], c->stream));
    }
    ~KTimer() {
        if (start < 0) return;
        cudaEventRecord(c->evPool[start + 1], c->stream);
        c->evMarks.push_back({cls, start});
        c->kLaunches[cls]++;
    }
};
inline void flushTimers(sst_ctx* c) {
    if (!c->profiling || c->evMarks.empty()) return;
    CUDA_CHECK(cudaStreamSynchronize(c->stream));
    for (auto& m : c->evMarks) {
        float ms = 0;
        CUDA_CHECK(cudaEventElapsedTime(&ms, c->evPool[m.second], c->evPool[m.second + 1]));
        c->kMs[m.first] += ms;
    }
    c->evMarks.clear();
}

struct HostMesh {
    std::vector<float> V, N, UV;
    std::vector<int> I;
    int material = -1;
};

struct HostEmitter {
    int mesh, face;
    float rad[3];
    float exponent;
};
struct HostTexture {
    int w, h, ch, border;
    std::vector<float> data;
};

struct sst_scene {
    sst_ctx* ctx = nullptr;
    std::vector<HostTexture> textures;
    std::vector<DevMaterial> materials;
    std::vector<HostMesh> meshes;
    std::vector<HostEmitter> emitters;
    std::vector<float> envRgb;
    int envW = 0, envH = 0;
    float w2c[16] = {};
    float fovDeg = 0;
    bool cameraSet = false;
    bool committed = false;
    int W = 0, H = 0;
    // device
    DevBuf nodes, nodes4, nodes8, triv, triN, triAux, triVtx, vnrm, vuv, mats, texs, texData, ems, envImg, envRowCdf, envColCdf, envHasCol, envRowMarg, queryJob;
    DevScene dev{};
    int nTri = 0, nNodes = 0, bvhDepth = 0, nNodes4 = 0, bvh4Depth = 0, nNodes8 = 0, bvh8Depth = 0;
    bool bvh8Built = false;  // the 8-wide BVH of the committed geometry exists (ensureBvh8)
    // adjoint: per-path radiance of the last sst_forward and its settings
    DevBuf record, gTex, gMatBase, gMatRough, gEmitter, dLdI;
    bool recordValid = false;
    SstPathTracerParams recordParams{};
    std::vector<int> meshTriOffset;
};

struct Wave {
    WaveBuffers wb;
};

struct JobIn {
    sst_scene* s;
    SstPathTracerParams p;
    float* dFilm;
    int iterFirst, iterEnd;
    int done = 0;  // iterations rendered
    DevAdj adj{};  // adjoint buffers (forward record or replay)
    bool hasCam = false;  // a camera view that replaces the scene's camera for this job
    DevCamera cam{};
    DevLayers lay{};      // frame-buffer layers
};

// Copies n items of `bytes` each to the device (or uses device pointers directly).
template <class T> const T* toDevice(sst_ctx* c, DevBuf& buf, const T* p, size_t n, int memory) {
    if (memory == SST_MEM_DEVICE) return p;
    buf.ensure(std::max<size_t>(1, n * sizeof(T)));
    CUDA_CHECK(cudaMemcpyAsync(buf.p, p, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return buf.as<T>();
}

template <class T> T* devCopy(DevBuf& b, const T* h, size_t n, cudaStream_t st) {
    b.ensure(std::max<size_t>(1, n * sizeof(T)));
    if (h) CUDA_CHECK(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return b.as<T>();
}
template <class T> void hostCopy(T* h, const DevBuf& b, size_t n, cudaStream_t st) {
    CUDA_CHECK(cudaMemcpyAsync(h, b.p, n * sizeof(T), cudaMemcpyDeviceToHost, st));
}


// ---- shared functions ------------------------------------------------------------------------
// sst_commit.cu
bool invert4(const float* m, float* out);  // 4x4 inverse (row-major); false when singular
DevCamera makeCamera(const float w2c[16], float fovDeg, int W, int H);
void commitScene(sst_scene* s, int W, int H);
// sst_render.cu
int defaultWaveCapacity();
void ensureWave(sst_ctx* c, int cap, int ns, Wave& w, int set);
void checkParams(const sst_scene* s, const SstPathTracerParams* p);
void renderJobs(sst_ctx* c, std::vector<JobIn>& jobs, SstRenderStats* out, bool replay = false, const std::vector<WaveChunk>* paths = nullptr);
size_t texPoolFloats(const sst_scene* s);
void batchJobs(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, std::vector<JobIn>& in, std::vector<std::unique_ptr<DevBuf>>& staged,
               bool fromZero);
void batchFilmsOut(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, const std::vector<JobIn>& in);
SstRenderStats emptyStats();
// sst_query.cu
const DevJob* jobTable(sst_scene* s);
// sst_commit.cu: builds the scene's 8-wide BVH if it has not been built since the last commit.
void ensureBvh8(sst_scene* s);
// The context's traversal setting for rays of these scenes: a scene without an 8-wide BVH (not
// built yet, or with node indices that do not fit its stack entries) traverses 4-wide.
inline TraceTuning traceFor(const sst_ctx* c, const sst_scene* const* scenes, size_t n) {
    TraceTuning t = c->trace;
    if (t.width == 8)
        for (size_t k = 0; k < n; ++k)
            if (scenes[k]->nNodes > 0 && scenes[k]->nNodes8 == 0) t.width = 4;
    return t;
}
// The same, building the 8-wide BVHs first when the setting asks for them.  Call it before the
// scenes' DevScene records are copied into a job table.
inline TraceTuning traceForBuilding(sst_ctx* c, sst_scene* const* scenes, size_t n) {
    if (c->trace.width == 8)
        for (size_t k = 0; k < n; ++k) ensureBvh8(scenes[k]);
    return traceFor(c, scenes, n);
}


// libsst host driver: the C ABI of include/sst.h.
//
// Scene.Prepare (Scene.cs:103-164) becomes sst_scene_commit: the meshes are concatenated into
// one triangle table, a binned-SAH BVH is built, all per-triangle data are stored in BVH leaf
// order, and the environment-map sampling tables are built on the GPU.  PathTracerBase.Render
// (Integrators/PathTracer.cs:199-267) becomes sst_render: the (iteration, pixel) paths are cut
// into waves that fit the path-state buffers; each wave runs camera -> {closest hit, shade,
// shadow rays} x depth -> film fold on one CUDA stream.
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
static thread_local std::string g_lastError;

struct SstException {
    int code;
    std::string msg;
};
static void fail(int code, const std::string& msg) { throw SstException{code, msg}; }
#define CUDA_CHECK(x)                                                                                         \
    do {                                                                                                      \
        cudaError_t e_ = (x);                                                                                 \
        if (e_ != cudaSuccess) {                                                                              \
            fail(e_ == cudaErrorMemoryAllocation ? SST_ERR_OUT_OF_MEMORY : SST_ERR_CUDA,                      \
                 std::string(#x) + ": " + cudaGetErrorString(e_));                                            \
        }                                                                                                     \
    } while (0)

template <class F> static int guarded(F&& f) {
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
static void parallelRanges(size_t n, size_t minPerThread, F fn) {
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

struct sst_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int numSMs = 0;
    // scene commit: pinned staging of the packed triangle records and the BVH build's temporaries
    // (kept across commits: no allocation or device-wide free per Scene.Prepare once they fit)
    PinnedBuf commitStage;
    DevBuf commitTri[4], commitOrder, commitScratch, commitScratch4;
    // wavefront buffers
    DevBuf pathA[9], pathB[9];
    DevBuf hits, nee, shRo, shRd, shTgt, shJob, counters, samples, stats, film;
    DevBuf shadeOrderBuf;  // k_partition's shade order of the current queue (cap ints)
    DevBuf jobsBuf, chunksBuf, wavesBuf, curWave;
    DevBuf adjA[3], adjB[3], neeG;
    int cap = 0, shCap = 0, neeSlots = 0;
    size_t sampleCap = 0;
    DevBuf scratchIn, scratchOut, scratchOut2;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int* pinnedCount = nullptr;
    // light paths (sst_trace_light_paths)
    DevBuf lightA[9], lightB[9], lightHits, lightVerts, lightLengths, lightCnt;
    // frame-buffer layers (sst_render_layers)
    DevBuf layMean, layRef, layErr, layVar, laySum, layAlb, layNrm, aovSamples, layErrPix, layTrim, layOutW, layOutIt, layPyr, pyrG;
    // batched adjoint: the jobs of the last sst_forward_batch, their path radiance, dLoss/dImage
    std::vector<BatchSig> batchSig;
    std::vector<std::unique_ptr<DevBuf>> batchRecord, batchDLdI;
    // launch configuration (sst_set_tuning / sst_autotune)
    TraceTuning trace;
    int waveCapacity = 0;  // 0: the default
    int shadeBlocks = 8;   // resident blocks per SM of the forward shade kernel with GenericMaterials: 8 or 14
    int shadeOrder = 1;    // 1: each bounce's queue is shaded surface hits first (k_partition); 0: in queue order
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
static void flushTimers(sst_ctx* c) {
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
// Normalized cross(v2 - v1, v3 - v1) of a face (the geometric normal, Triangle.cs:22-36).  One
// out-of-line instance, so that the triangle records and the emitter table get the same bits.
__attribute__((noinline)) static void faceNormal(const float* V, const int* I, size_t f, float out[3]) {
    const float* a = &V[3 * size_t(I[3 * f])];
    const float* b = &V[3 * size_t(I[3 * f + 1])];
    const float* c = &V[3 * size_t(I[3 * f + 2])];
    float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) out[k] = n[k] / l;
}

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
    DevBuf nodes, nodes4, triv, triN, triAux, triVtx, vnrm, vuv, mats, texs, texData, ems, envImg, envRowCdf, envColCdf, envHasCol, envRowMarg, queryJob;
    DevScene dev{};
    int nTri = 0, nNodes = 0, bvhDepth = 0, nNodes4 = 0, bvh4Depth = 0;
    // adjoint: per-path radiance of the last sst_forward and its settings
    DevBuf record, gTex, gMatBase, gMatRough, gEmitter, dLdI;
    bool recordValid = false;
    SstPathTracerParams recordParams{};
    std::vector<int> meshTriOffset;
};

// ---------------------------------------------------------------------------------------------
// host math: 4x4 inverse (Laplace expansion over 2x2 minors), perspective matrix
// ---------------------------------------------------------------------------------------------
static bool invert4(const float* m, float* out) {
    float s0 = m[0] * m[5] - m[4] * m[1];
    float s1 = m[0] * m[6] - m[4] * m[2];
    float s2 = m[0] * m[7] - m[4] * m[3];
    float s3 = m[1] * m[6] - m[5] * m[2];
    float s4 = m[1] * m[7] - m[5] * m[3];
    float s5 = m[2] * m[7] - m[6] * m[3];
    float c5 = m[10] * m[15] - m[14] * m[11];
    float c4 = m[9] * m[15] - m[13] * m[11];
    float c3 = m[9] * m[14] - m[13] * m[10];
    float c2 = m[8] * m[15] - m[12] * m[11];
    float c1 = m[8] * m[14] - m[12] * m[10];
    float c0 = m[8] * m[13] - m[12] * m[9];
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (!(std::fabs(det) > 0.0f) || !std::isfinite(det)) return false;
    float id = 1.0f / det;
    out[0] = (m[5] * c5 - m[6] * c4 + m[7] * c3) * id;
    out[1] = (-m[1] * c5 + m[2] * c4 - m[3] * c3) * id;
    out[2] = (m[13] * s5 - m[14] * s4 + m[15] * s3) * id;
    out[3] = (-m[9] * s5 + m[10] * s4 - m[11] * s3) * id;
    out[4] = (-m[4] * c5 + m[6] * c2 - m[7] * c1) * id;
    out[5] = (m[0] * c5 - m[2] * c2 + m[3] * c1) * id;
    out[6] = (-m[12] * s5 + m[14] * s2 - m[15] * s1) * id;
    out[7] = (m[8] * s5 - m[10] * s2 + m[11] * s1) * id;
    out[8] = (m[4] * c4 - m[5] * c2 + m[7] * c0) * id;
    out[9] = (-m[0] * c4 + m[1] * c2 - m[3] * c0) * id;
    out[10] = (m[12] * s4 - m[13] * s2 + m[15] * s0) * id;
    out[11] = (-m[8] * s4 + m[9] * s2 - m[11] * s0) * id;
    out[12] = (-m[4] * c3 + m[5] * c1 - m[6] * c0) * id;
    out[13] = (m[0] * c3 - m[1] * c1 + m[2] * c0) * id;
    out[14] = (-m[12] * s3 + m[13] * s1 - m[14] * s0) * id;
    out[15] = (m[8] * s3 - m[9] * s1 + m[10] * s0) * id;
    return true;
}
// Matrix4x4.CreatePerspectiveFieldOfView (right-handed), PerspectiveCamera.cs:42-52
static void perspective(float fov, float aspect, float n, float f, float* m) {
    std::fill(m, m + 16, 0.0f);
    float y = 1.0f / std::tan(fov * 0.5f);
    float x = y / aspect;
    float nfr = f / (n - f);
    m[0] = x;
    m[5] = y;
    m[10] = nfr;
    m[11] = -1.0f;
    m[14] = n * nfr;
}

// ---------------------------------------------------------------------------------------------
// binned-SAH BVH (host build)
// ---------------------------------------------------------------------------------------------
struct Aabb {
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    void grow(const Aabb& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    float area() const {
        float dx = std::max(0.f, hi[0] - lo[0]), dy = std::max(0.f, hi[1] - lo[1]), dz = std::max(0.f, hi[2] - lo[2]);
        return dx * dy + dy * dz + dz * dx;
    }
};

struct BvhBuilder {
    std::vector<Aabb> box;
    std::vector<float> cen;  // 3 per prim
    std::vector<int> order;
    std::vector<float4> nodes;
    int maxDepth = 0;

    uint32_t leafRef(int first, int count) { return kLeafFlag | (uint32_t(count - 1) << kLeafCountShift) | uint32_t(first); }

    Aabb rangeBox(int first, int count, Aabb* cbox) {
        Aabb b, c;
        for (int i = first; i < first + count; ++i) {
            b.grow(box[order[i]]);
            c.grow(&cen[3 * size_t(order[i])]);
        }
        if (cbox) *cbox = c;
        return b;
    }

    void setChild(int node, int which, const Aabb& b, uint32_t ref) {
        float4* n = &nodes[4 * size_t(node)];
        if (which == 0) {
            n[0].x = b.lo[0]; n[0].y = b.hi[0]; n[0].z = b.lo[1]; n[0].w = b.hi[1];
            n[2].x = b.lo[2]; n[2].y = b.hi[2];
            n[3].x = __uint_as_float_host(ref);
        } else {
            n[1].x = b.lo[0]; n[1].y = b.hi[0]; n[1].z = b.lo[1]; n[1].w = b.hi[1];
            n[2].z = b.lo[2]; n[2].w = b.hi[2];
            n[3].y = __uint_as_float_host(ref);
        }
    }
    static float __uint_as_float_host(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

    // Chooses a split of [first, first+count); returns the split position or -1 for a leaf.
    int split(int first, int count, const Aabb& b, const Aabb& cb, int depth) {
        const int kBins = 16;
        if (count <= 1) return -1;
        float leafCost = float(count);
        int bestAxis = -1, bestBin = -1;
        float bestCost = 1e30f;
        float pa = b.area();
        bool forceMedian = depth >= 32;
        if (!forceMedian) {
            for (int ax = 0; ax < 3; ++ax) {
                float ext = cb.hi[ax] - cb.lo[ax];
                if (!(ext > 0.0f)) continue;
                Aabb bb[kBins];
                int bc[kBins] = {};
                float sc = kBins / ext;
                for (int i = first; i < first + count; ++i) {
                    int p = order[i];
                    int k = std::min(kBins - 1, int((cen[3 * size_t(p) + ax] - cb.lo[ax]) * sc));
                    bc[k]++;
                    bb[k].grow(box[p]);
                }
                float rArea[kBins];
                int rCnt[kBins];
                Aabb acc;
                int n = 0;
                for (int k = kBins - 1; k > 0; --k) {
                    acc.grow(bb[k]);
                    n += bc[k];
                    rArea[k] = acc.area();
                    rCnt[k] = n;
                }
                Aabb lacc;
                int ln = 0;
                for (int k = 0; k < kBins - 1; ++k) {
                    lacc.grow(bb[k]);
                    ln += bc[k];
                    if (ln == 0 || rCnt[k + 1] == 0) continue;
                    float cost = 1.0f + (lacc.area() * ln + rArea[k + 1] * rCnt[k + 1]) / std::max(pa, 1e-30f);
                    if (cost < bestCost) { bestCost = cost; bestAxis = ax; bestBin = k; }
                }
            }
        }
        if (bestAxis >= 0 && count <= kMaxLeafSize && leafCost <= bestCost) return -1;
        int mid;
        if (bestAxis >= 0) {
            float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
            float sc = kBins / ext;
            auto pred = [&](int p) { return std::min(kBins - 1, int((cen[3 * size_t(p) + bestAxis] - cb.lo[bestAxis]) * sc)) <= bestBin; };
            mid = int(std::partition(order.begin() + first, order.begin() + first + count, pred) - order.begin());
        } else {
            if (count <= kMaxLeafSize && !forceMedian) return -1;
            int ax = 0;
            float e = -1;
            for (int k = 0; k < 3; ++k)
                if (cb.hi[k] - cb.lo[k] > e) { e = cb.hi[k] - cb.lo[k]; ax = k; }
            mid = first + count / 2;
            std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count,
                             [&](int a, int c) { return cen[3 * size_t(a) + ax] < cen[3 * size_t(c) + ax]; });
        }
        if (mid <= first || mid >= first + count) mid = first + count / 2;
        return mid;
    }

    // Builds the subtree for [first, first+count) and returns its reference.
    uint32_t build(int first, int count, const Aabb& b, const Aabb& cb, int depth) {
        maxDepth = std::max(maxDepth, depth);
        int mid = split(first, count, b, cb, depth);
        if (mid < 0) {
            if (count > kMaxLeafSize) mid = first + count / 2;
            else return leafRef(first, count);
        }
        int node = int(nodes.size() / 4);
        nodes.resize(nodes.size() + 4, make_float4(0, 0, 0, 0));
        Aabb lcb, rcb;
        Aabb lb = rangeBox(first, mid - first, &lcb), rb = rangeBox(mid, first + count - mid, &rcb);
        uint32_t l = build(first, mid - first, lb, lcb, depth + 1);
        uint32_t r = build(mid, first + count - mid, rb, rcb, depth + 1);
        setChild(node, 0, lb, l);
        setChild(node, 1, rb, r);
        return uint32_t(node);
    }

    void run(int n) {
        order.resize(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        nodes.clear();
        if (n == 0) return;
        Aabb cb;
        Aabb b = rangeBox(0, n, &cb);
        // the root is always an inner node
        nodes.resize(4, make_float4(0, 0, 0, 0));
        int mid = split(0, n, b, cb, 0);
        if (mid < 0) {
            if (n == 1) {
                setChild(0, 0, b, leafRef(0, 1));
                setChild(0, 1, b, leafRef(0, 1));
                return;
            }
            mid = n / 2;
        }
        Aabb lcb, rcb;
        Aabb lb = rangeBox(0, mid, &lcb), rb = rangeBox(mid, n - mid, &rcb);
        uint32_t l = build(0, mid, lb, lcb, 1);
        uint32_t r = build(mid, n - mid, rb, rcb, 1);
        setChild(0, 0, lb, l);
        setChild(0, 1, rb, r);
    }
};

// ---------------------------------------------------------------------------------------------
// scene commit
// ---------------------------------------------------------------------------------------------
// Camera matrices of a perspective view (Camera.cs:34-42, PerspectiveCamera.cs:42-52).
static DevCamera makeCamera(const float w2c[16], float fovDeg, int W, int H) {
    DevCamera cam{};
    float c2v[16];
    if (!invert4(w2c, cam.c2w)) fail(SST_ERR_INVALID_ARGUMENT, "World to camera transform must be invertible.");
    perspective(fovDeg * 3.14159265f / 180.0f, float(W) / float(H), 0.001f, 1000.0f, c2v);
    if (!invert4(c2v, cam.v2c)) fail(SST_ERR_INVALID_ARGUMENT, "degenerate projection");
    cam.W = W;
    cam.H = H;
    return cam;
}

static void commitScene(sst_scene* s, int W, int H) {
    if (W <= 0 || H <= 0) fail(SST_ERR_INVALID_ARGUMENT, "frame buffer size must be positive");
    // Scene.IsValid (Scene.cs:170-197)
    if (s->meshes.empty()) fail(SST_ERR_INVALID_SCENE, "No meshes in the scene.");
    for (size_t i = 0; i < s->meshes.size(); ++i)
        if (s->meshes[i].material < 0) fail(SST_ERR_INVALID_SCENE, "Mesh[" + std::to_string(i) + "] does not have a material.");
    if (!s->cameraSet) fail(SST_ERR_INVALID_SCENE, "Camera not set.");
    if (s->emitters.empty() && s->envW == 0) fail(SST_ERR_INVALID_SCENE, "No emitters and no background in the scene.");
    cudaStream_t st = s->ctx->stream;
    CUDA_CHECK(cudaSetDevice(s->ctx->device));

    // global triangle table
    int nt = 0;
    s->meshTriOffset.clear();
    std::vector<int> vtxOffset;
    int nv = 0;
    bool anyNormals = false, anyUV = false;
    for (auto& m : s->meshes) {
        s->meshTriOffset.push_back(nt);
        vtxOffset.push_back(nv);
        nt += int(m.I.size() / 3);
        nv += int(m.V.size() / 3);
        anyNormals |= !m.N.empty();
        anyUV |= !m.UV.empty();
    }
    s->nTri = nt;
    std::vector<int> triEmitter(nt, -1);
    for (size_t e = 0; e < s->emitters.size(); ++e) {
        int g = s->meshTriOffset[s->emitters[e].mesh] + s->emitters[e].face;
        if (triEmitter[g] >= 0) fail(SST_ERR_INVALID_SCENE, "two emitters on the same triangle");
        triEmitter[g] = int(e);
    }
    // per-triangle records in global order, packed by several host threads over triangle ranges
    // (uninitialised arrays: every entry is written, and each thread touches its own pages first)
    sst_ctx* const cx = s->ctx;
    cx->commitStage.ensure(std::max<size_t>(1, 96 * size_t(nt)));
    float4* const trivG = cx->commitStage.as<float4>();
    float4* const triNG = trivG + 3 * size_t(nt);
    int4* const auxG = reinterpret_cast<int4*>(triNG + nt);
    int4* const vtxG = auxG + nt;
    parallelRanges(size_t(nt), 1 << 16, [&](size_t g0, size_t g1) {
        size_t mi = size_t(std::upper_bound(s->meshTriOffset.begin(), s->meshTriOffset.end(), int(g0)) - s->meshTriOffset.begin()) - 1;
        for (size_t g = g0; g < g1; ++g) {
            while (mi + 1 < s->meshes.size() && int(g) >= s->meshTriOffset[mi + 1]) ++mi;
            const HostMesh& m = s->meshes[mi];
            const size_t f = g - size_t(s->meshTriOffset[mi]);
            const int vo = vtxOffset[mi];
            const int flags = (m.N.empty() ? 0 : 1) | (m.UV.empty() ? 0 : 2);
            int i0 = m.I[3 * f], i1 = m.I[3 * f + 1], i2 = m.I[3 * f + 2];
            const float* a = &m.V[3 * size_t(i0)];
            const float* bb = &m.V[3 * size_t(i1)];
            const float* c = &m.V[3 * size_t(i2)];
            int gi = int(g);
            float gw;
            std::memcpy(&gw, &gi, 4);
            trivG[3 * g] = make_float4(a[0], a[1], a[2], gw);
            trivG[3 * g + 1] = make_float4(bb[0], bb[1], bb[2], 0.f);
            trivG[3 * g + 2] = make_float4(c[0], c[1], c[2], 0.f);
            float ew, fn[3];
            std::memcpy(&ew, &triEmitter[g], 4);
            faceNormal(m.V.data(), m.I.data(), f, fn);
            triNG[g] = make_float4(fn[0], fn[1], fn[2], ew);
            auxG[g] = make_int4(m.material, int(mi), int(f), flags);
            vtxG[g] = make_int4(vo + i0, vo + i1, vo + i2, 0);
        }
    });
    const char* bvhEnv = getenv("SST_BVH");
    bool hostBuild = bvhEnv && std::string(bvhEnv) == "sah";
    s->triv.ensure(std::max<size_t>(1, sizeof(float4) * 3 * size_t(nt)));
    s->triN.ensure(std::max<size_t>(1, sizeof(float4) * size_t(nt)));
    s->triAux.ensure(std::max<size_t>(1, sizeof(int4) * size_t(nt)));
    s->triVtx.ensure(std::max<size_t>(1, sizeof(int4) * size_t(nt)));
    if (!hostBuild && nt > 0) {
        // GPU linear BVH (sst_bvh.cu) and a leaf-order gather on the device
        DevBuf &gTriv = cx->commitTri[0], &gTriN = cx->commitTri[1], &gAux = cx->commitTri[2], &gVtx = cx->commitTri[3];
        DevBuf &order = cx->commitOrder, &scratch = cx->commitScratch;
        gTriv.upload(trivG, 3 * size_t(nt), st);
        gTriN.upload(triNG, size_t(nt), st);
        gAux.upload(auxG, size_t(nt), st);
        gVtx.upload(vtxG, size_t(nt), st);
        s->nodes.ensure(sizeof(float4) * 4 * size_t(std::max(1, nt - 1)));
        order.ensure(sizeof(int) * size_t(nt));
        size_t sb = lbvhScratchBytes(nt);
        scratch.ensure(sb);
        int nodeCount = 0, maxDepth = 0;
        // PLOC clustering by default (3.6% faster traversal than the radix tree on the 1M-triangle
        // scene, same build time); SST_BVH=lbvh selects the radix tree, SST_BVH=sah the host build
        int method = (bvhEnv && std::string(bvhEnv) == "lbvh") ? 0 : 1;
        int rc = buildLbvh(gTriv.as<float4>(), nt, s->nodes.as<float4>(), order.as<int>(), scratch.p, sb, &nodeCount, &maxDepth, st, method);
        if (rc != 0) fail(SST_ERR_CUDA, "GPU BVH build failed (" + std::to_string(rc) + "): " + cudaGetErrorString(cudaGetLastError()));
        if (maxDepth + 2 >= kMaxStack) {
            hostBuild = true;  // deeper than the traversal stack: use the host SAH build instead
        } else {
            launch_leaf_gather(order.as<int>(), nt, gTriv.as<float4>(), gTriN.as<float4>(), gAux.as<int4>(), gVtx.as<int4>(), s->triv.as<float4>(),
                               s->triN.as<float4>(), s->triAux.as<int4>(), s->triVtx.as<int4>(), st);
            CUDA_CHECK(cudaGetLastError());
            CUDA_CHECK(cudaStreamSynchronize(st));
            s->nNodes = nodeCount;
            s->bvhDepth = maxDepth;
        }
    }
    if (hostBuild || nt == 0) {
        BvhBuilder b;
        b.box.resize(nt);
        b.cen.resize(3 * size_t(nt));
        for (int g = 0; g < nt; ++g) {
            Aabb bb;
            for (int k = 0; k < 3; ++k) bb.grow(&trivG[3 * size_t(g) + k].x);
            b.box[g] = bb;
            for (int k = 0; k < 3; ++k) b.cen[3 * size_t(g) + k] = 0.5f * (bb.lo[k] + bb.hi[k]);
        }
        b.run(nt);
        if (b.maxDepth >= kMaxBvhDepth) fail(SST_ERR_DEVICE_LIMIT, "BVH deeper than the traversal stack");
        s->nNodes = int(b.nodes.size() / 4);
        s->bvhDepth = b.maxDepth;
        std::vector<float4> triv(3 * size_t(nt)), triN(nt);
        std::vector<int4> triAux(nt), triVtx(nt);
        for (int t = 0; t < nt; ++t) {
            int g = b.order[t];
            for (int k = 0; k < 3; ++k) triv[3 * size_t(t) + k] = trivG[3 * size_t(g) + k];
            triN[t] = triNG[g];
            triAux[t] = auxG[g];
            triVtx[t] = vtxG[g];
        }
        s->nodes.upload(b.nodes, st);
        s->triv.upload(triv, st);
        s->triN.upload(triN, st);
        s->triAux.upload(triAux, st);
        s->triVtx.upload(triVtx, st);
    }
    // 4-wide BVH over the same leaves (the traversal variant picked by the launch tuning)
    s->nNodes4 = 0;
    s->bvh4Depth = 0;
    if (s->nNodes > 0) {
        DevBuf& scratch4 = s->ctx->commitScratch4;
        s->nodes4.ensure(sizeof(float4) * 8 * size_t(s->nNodes));
        scratch4.ensure(bvh4ScratchBytes(s->nNodes));
        int rc = buildBvh4(s->nodes.as<float4>(), s->nNodes, s->nodes4.as<float4>(), scratch4.p, &s->nNodes4, &s->bvh4Depth, st);
        if (rc != 0) fail(SST_ERR_CUDA, "4-wide BVH build failed (" + std::to_string(rc) + "): " + cudaGetErrorString(cudaGetLastError()));
    }
    std::vector<float> vnrm, vuv;
    if (anyNormals) {
        vnrm.assign(3 * size_t(nv), 0.f);
        for (size_t mi = 0; mi < s->meshes.size(); ++mi)
            if (!s->meshes[mi].N.empty()) std::copy(s->meshes[mi].N.begin(), s->meshes[mi].N.end(), vnrm.begin() + 3 * size_t(vtxOffset[mi]));
    }
    if (anyUV) {
        vuv.assign(2 * size_t(nv), 0.f);
        for (size_t mi = 0; mi < s->meshes.size(); ++mi)
            if (!s->meshes[mi].UV.empty()) std::copy(s->meshes[mi].UV.begin(), s->meshes[mi].UV.end(), vuv.begin() + 2 * size_t(vtxOffset[mi]));
    }
    // emitters
    std::vector<DevEmitter> ems(s->emitters.size());
    for (size_t e = 0; e < s->emitters.size(); ++e) {
        const HostEmitter& he = s->emitters[e];
        const HostMesh& m = s->meshes[he.mesh];
        int f = he.face;
        DevEmitter& d = ems[e];
        const float* p[3];
        for (int k = 0; k < 3; ++k) p[k] = &m.V[3 * size_t(m.I[3 * f + k])];
        d.v1 = make_float4(p[0][0], p[0][1], p[0][2], 0.f);
        d.v2 = make_float4(p[1][0], p[1][1], p[1][2], 0.f);
        d.v3 = make_float4(p[2][0], p[2][1], p[2][2], 0.f);
        if (!m.N.empty()) {
            const float* q[3];
            for (int k = 0; k < 3; ++k) q[k] = &m.N[3 * size_t(m.I[3 * f + k])];
            d.n1 = make_float4(q[0][0], q[0][1], q[0][2], 1.f);
            d.n2 = make_float4(q[1][0], q[1][1], q[1][2], 0.f);
            d.n3 = make_float4(q[2][0], q[2][1], q[2][2], 0.f);
        } else {
            d.n1 = d.n2 = d.n3 = make_float4(0, 0, 0, 0);
        }
        // Triangle.cs:22-36: area = |cross(v2 - v1, v3 - v1)| * 0.5
        float e1[3], e2[3];
        for (int k = 0; k < 3; ++k) { e1[k] = p[1][k] - p[0][k]; e2[k] = p[2][k] - p[0][k]; }
        float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
        float area = std::sqrt(cx * cx + cy * cy + cz * cz) * 0.5f;
        float fn[3];
        faceNormal(m.V.data(), m.I.data(), size_t(f), fn);
        d.faceN = make_float4(fn[0], fn[1], fn[2], 1.0f / area);
        d.rad = make_float4(he.rad[0], he.rad[1], he.rad[2], he.exponent);
        d.norm = (he.exponent + 1.0f) / (2.0f * 3.14159265f);  // GlossyEmitter.cs:14
        d.globalTri = s->meshTriOffset[he.mesh] + f;
        d.mesh = he.mesh;
        d.face = f;
    }
    // textures
    std::vector<DevTexture> texs;
    std::vector<float> texPool;
    for (auto& t : s->textures) {
        DevTexture d{t.w, t.h, t.ch, t.border, (long long)texPool.size()};
        texs.push_back(d);
        texPool.insert(texPool.end(), t.data.begin(), t.data.end());
    }
    // upload
    s->vnrm.upload(vnrm, st);
    s->vuv.upload(vuv, st);
    s->mats.upload(s->materials, st);
    s->texs.upload(texs, st);
    s->texData.upload(texPool, st);
    s->ems.upload(ems, st);
    DevScene& d = s->dev;
    d = DevScene{};
    d.nodes = s->nodes.as<float4>();
    d.triv = s->triv.as<float4>();
    d.triN = s->triN.as<float4>();
    d.triAux = s->triAux.as<int4>();
    d.triVtx = s->triVtx.as<int4>();
    d.vnrm = anyNormals ? s->vnrm.as<float>() : nullptr;
    d.vuv = anyUV ? s->vuv.as<float>() : nullptr;
    d.mats = s->mats.as<DevMaterial>();
    d.texs = s->texs.as<DevTexture>();
    d.texData = s->texData.as<float>();
    d.emitters = s->ems.as<DevEmitter>();
    d.nEmitters = int(s->emitters.size());
    d.nTri = nt;
    d.nNodes = s->nNodes;
    d.nodes4 = s->nNodes4 > 0 ? s->nodes4.as<float4>() : nullptr;
    d.nNodes4 = s->nNodes4;
    {
        // Scene.Prepare (Scene.cs:115-136): the mean of all vertices and the distance to the
        // furthest one, summed in single precision in mesh and vertex order
        float cx = 0.f, cy = 0.f, cz = 0.f;
        unsigned long long total = 0;
        for (auto& m : s->meshes) {
            for (size_t v = 0; v + 2 < m.V.size(); v += 3) { cx += m.V[v]; cy += m.V[v + 1]; cz += m.V[v + 2]; }
            total += m.V.size() / 3;
        }
        float tf = float(std::max<unsigned long long>(total, 1));
        cx /= tf; cy /= tf; cz /= tf;
        float r2 = 0.f;
        for (auto& m : s->meshes)
            for (size_t v = 0; v + 2 < m.V.size(); v += 3) {
                float dx = m.V[v] - cx, dy = m.V[v + 1] - cy, dz = m.V[v + 2] - cz;
                r2 = std::max(dx * dx + dy * dy + dz * dz, r2);
            }
        d.sceneCenter = make_float3(cx, cy, cz);
        d.sceneRadius = std::sqrt(r2);
    }
    // environment map (EnvironmentMap.cs:139-156)
    d.hasEnv = s->envW > 0;
    if (d.hasEnv) {
        std::vector<float4> img(size_t(s->envW) * s->envH);
        for (size_t i = 0; i < img.size(); ++i) img[i] = make_float4(s->envRgb[3 * i], s->envRgb[3 * i + 1], s->envRgb[3 * i + 2], 0.f);
        s->envImg.upload(img, st);
        s->envColCdf.ensure(sizeof(float) * img.size());
        s->envRowCdf.ensure(sizeof(float) * s->envH);
        s->envRowMarg.ensure(sizeof(float) * s->envH);
        s->envHasCol.ensure(sizeof(int) * s->envH);
        launch_env_build(s->envImg.as<float4>(), s->envW, s->envH, s->envColCdf.as<float>(), s->envRowMarg.as<float>(), s->envHasCol.as<int>(),
                         s->envRowCdf.as<float>(), st);
        CUDA_CHECK(cudaGetLastError());
        d.env.w = s->envW;
        d.env.h = s->envH;
        d.env.img = s->envImg.as<float4>();
        d.env.rowCdf = s->envRowCdf.as<float>();
        d.env.colCdf = s->envColCdf.as<float>();
        d.env.hasCol = s->envHasCol.as<int>();
    }
    d.cam = makeCamera(s->w2c, s->fovDeg, W, H);
    CUDA_CHECK(cudaStreamSynchronize(st));
    s->W = W;
    s->H = H;
    s->committed = true;
}

// ---------------------------------------------------------------------------------------------
// wavefront buffers
// ---------------------------------------------------------------------------------------------
static void bindPath(DevBuf* bufs, PathBuf& p, int cap) {
    size_t c = size_t(cap);
    for (int k = 0; k < 4; ++k) bufs[k].ensure(c * 4);
    for (int k = 4; k < 9; ++k) bufs[k].ensure(c * 16);
    p.job = bufs[0].as<uint32_t>();
    p.pix = bufs[1].as<uint32_t>();
    p.rng = bufs[2].as<uint32_t>();
    p.depth = bufs[3].as<uint32_t>();
    p.pw = bufs[4].as<float4>();
    p.rad = bufs[5].as<float4>();
    p.prev = bufs[6].as<float4>();
    p.ro = bufs[7].as<float4>();
    p.rd = bufs[8].as<float4>();
    p.order = nullptr;
    p.neeIn = p.neeGIn = p.pyrGIn = nullptr;
}

static int defaultWaveCapacity() {
    const char* e = getenv("SST_WAVE_CAPACITY");
    if (e) return std::max(1024, atoi(e));
    return 1 << 21;
}

struct Wave {
    WaveBuffers wb;
};

static void ensureWave(sst_ctx* c, int cap, int ns, Wave& w) {
    if (cap > c->cap) {
        // grow all path buffers
        c->cap = cap;
        c->hits.ensure(size_t(cap) * 16);
    }
    bindPath(c->pathA, w.wb.a, c->cap);
    bindPath(c->pathB, w.wb.b, c->cap);
    c->neeSlots = std::max(c->neeSlots, 2 * ns);
    c->nee.ensure(2 * size_t(c->cap) * 16 * c->neeSlots);  // two buffers: read and written bounce by bounce
    size_t shCap = size_t(c->cap) * 2 * ns;
    c->shRo.ensure(shCap * 16);
    c->shRd.ensure(shCap * 16);
    c->shTgt.ensure(shCap * 4);
    c->shJob.ensure(shCap * 4);
    c->counters.ensure(sizeof(int) * kNumCounters);
    c->shadeOrderBuf.ensure(size_t(c->cap) * 4);
    c->stats.ensure(sizeof(DevStats));
    w.wb.hits = c->hits.as<float4>();
    w.wb.nee = c->nee.as<float4>();
    w.wb.shRo = c->shRo.as<float4>();
    w.wb.shRd = c->shRd.as<float4>();
    w.wb.shTgt = c->shTgt.as<int>();
    w.wb.shJob = c->shJob.as<uint32_t>();
    w.wb.counters = c->counters.as<int>();
    w.wb.order = c->shadeOrderBuf.as<int>();
    w.wb.cap = c->cap;
    w.wb.shCap = int(shCap);
}

// ---------------------------------------------------------------------------------------------
// render
// ---------------------------------------------------------------------------------------------
static void checkParams(const sst_scene* s, const SstPathTracerParams* p) {
    if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
    if (p->width != s->W || p->height != s->H) fail(SST_ERR_INVALID_ARGUMENT, "frame buffer size differs from the committed camera resolution");
    if (p->totalSpp < 0 || p->maxDepth < 1 || p->numShadowRays < 0 || p->numShadowRays > kMaxShadowRays || p->firstIteration < 0)
        fail(SST_ERR_INVALID_ARGUMENT, "invalid path tracer parameters");
    if (p->maxDepth > kMaxPathDepth) fail(SST_ERR_UNSUPPORTED, "MaxDepth above 1000 is not supported");
}

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

// Splits the (job, iteration, pixel) paths into waves of at most `cap` paths.  A job whose
// image fits a wave contributes chunks of whole iterations; a larger image is cut into pixel
// ranges of one iteration.  A pixel appears at most once per wave.
static void planWaves(std::vector<JobIn>& jobs, int cap, bool iterationPerWave, std::vector<WaveChunk>& chunks, std::vector<WaveDesc>& waves,
                      std::vector<std::vector<int>>& waveIterEnds) {
    WaveDesc cur{0, 0, 0, 0};
    auto closeWave = [&]() {
        if (cur.items == 0) return;
        cur.chunkEnd = int(chunks.size());
        waves.push_back(cur);
        cur = WaveDesc{int(chunks.size()), int(chunks.size()), 0, 0};
    };
    for (size_t j = 0; j < jobs.size(); ++j) {
        const JobIn& jb = jobs[j];
        int P = jb.p.width * jb.p.height;
        int it = jb.iterFirst;
        int pixCursor = 0;
        while (it < jb.iterEnd) {
            int space = cap - cur.items;
            WaveChunk ck{};
            ck.job = int(j);
            ck.film = jb.dFilm;
            ck.itemOffset = cur.items;
            ck.foldOffset = cur.foldThreads;
            if (P <= cap) {
                int k = std::min(jb.iterEnd - it, space / P);
                if (iterationPerWave) k = std::min(k, 1);
                if (k == 0) { closeWave(); continue; }
                ck.iterBase = it; ck.nIter = k; ck.pixStart = 0; ck.pixCount = P;
                it += k;
            } else {
                int cnt = std::min(space, P - pixCursor);
                if (cnt == 0) { closeWave(); continue; }
                ck.iterBase = it; ck.nIter = 1; ck.pixStart = pixCursor; ck.pixCount = cnt;
                pixCursor += cnt;
                if (pixCursor == P) { pixCursor = 0; ++it; }
            }
            chunks.push_back(ck);
            cur.items += ck.nIter * ck.pixCount;
            cur.foldThreads += ck.pixCount;
            if (iterationPerWave || cur.items == cap) closeWave();
        }
    }
    closeWave();
    (void)waveIterEnds;
}

// Renders the jobs' iterations [iterFirst, iterEnd) into their device films.
// paths: instead of the jobs' iteration ranges, render exactly these single-path chunks (one
// (pixel, iteration) each, at most one wave) without folding them into a film; each path's
// estimate is left in c->samples at its chunk's item offset.
static void renderJobs(sst_ctx* c, std::vector<JobIn>& jobs, SstRenderStats* out, bool replay = false,
                       const std::vector<WaveChunk>* paths = nullptr) {
    cudaStream_t st = c->stream;
    if (jobs.empty()) return;
    long long totalItems = 0;
    int ns = 1, maxDepth = 1;
    bool timeLimit = false;
    for (auto& j : jobs) {
        totalItems += (long long)j.p.width * j.p.height * std::max(0, j.iterEnd - j.iterFirst);
        ns = std::max(ns, j.p.numShadowRays);
        maxDepth = std::max(maxDepth, j.p.maxDepth);
        timeLimit |= j.p.maximumRenderTimeMs > 0;
    }
    if (paths) totalItems = (long long)paths->size();
    if (totalItems == 0) return;
    if (timeLimit && jobs.size() > 1) fail(SST_ERR_UNSUPPORTED, "MaximumRenderTimeMs is supported for single renders only");
    int cap = int(std::min<long long>(c->waveCapacity > 0 ? c->waveCapacity : defaultWaveCapacity(), totalItems));
    for (auto& j : jobs) cap = std::max(cap, 1);
    Wave w;
    ensureWave(c, cap, ns, w);
    c->samples.ensure(size_t(w.wb.cap) * 12);
    w.wb.a.adjL = w.wb.a.adjD = w.wb.a.adjP = nullptr;
    w.wb.b.adjL = w.wb.b.adjD = w.wb.b.adjP = nullptr;
    w.wb.neeG = nullptr;
    if (replay) {
        size_t cp = size_t(w.wb.cap);
        for (int k = 0; k < 2; ++k) { c->adjA[k].ensure(cp * 16); c->adjB[k].ensure(cp * 16); }
        c->adjA[2].ensure(cp * 48);
        c->adjB[2].ensure(cp * 48);
        c->neeG.ensure(2 * cp * 48 * 2 * ns);
        w.wb.a.adjL = c->adjA[0].as<float4>(); w.wb.a.adjD = c->adjA[1].as<float4>(); w.wb.a.adjP = c->adjA[2].as<float4>();
        w.wb.b.adjL = c->adjB[0].as<float4>(); w.wb.b.adjD = c->adjB[1].as<float4>(); w.wb.b.adjP = c->adjB[2].as<float4>();
        w.wb.neeG = c->neeG.as<float4>();
    }
    // any GenericMaterial in the wave's scenes (otherwise the shade kernel without generic code runs)
    bool generic = false;
    for (auto& j : jobs)
        for (auto& m : j.s->materials) generic |= m.type == kGeneric;
    // per-item samples of the denoiser feature layers (written by the first shade, read by the fold)
    bool anyAov = false, pyramid = false;
    for (auto& j : jobs) {
        anyAov |= j.lay.aovAlbedo != nullptr;
        pyramid |= j.lay.pyr != nullptr;
    }
    if (anyAov) c->aovSamples.ensure(size_t(w.wb.cap) * 24);
    if (pyramid && replay) fail(SST_ERR_UNSUPPORTED, "the technique pyramid is not available in the adjoint replay");
    // technique pyramid: the payload of every NEE slot
    if (pyramid) c->pyrG.ensure(2 * size_t(w.wb.cap) * 16 * 2 * ns);
    // job table
    std::vector<DevJob> hj(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) {
        const SstPathTracerParams* P = &jobs[k].p;
        hj[k].sc = jobs[k].s->dev;
        if (jobs[k].hasCam) hj[k].sc.cam = jobs[k].cam;
        hj[k].lay = jobs[k].lay;
        if (hj[k].lay.aovAlbedo) hj[k].lay.aovSamples = c->aovSamples.as<float>();
        hj[k].cfg = PTConfig{P->width, P->height, P->maxDepth, P->minDepth, P->baseSeed, P->numShadowRays, P->enableBsdfDI, P->ignoreNanAndInf};
        hj[k].adj = jobs[k].adj;
    }
    std::vector<WaveChunk> chunks;
    std::vector<WaveDesc> waves;
    std::vector<std::vector<int>> iterEnds;
    if (paths) {
        chunks = *paths;
        waves.push_back(WaveDesc{0, int(chunks.size()), int(chunks.size()), 0});
    } else {
        planWaves(jobs, w.wb.cap, timeLimit, chunks, waves, iterEnds);
    }
    c->jobsBuf.upload(hj, st);
    c->chunksBuf.upload(chunks, st);
    c->wavesBuf.upload(waves, st);
    c->curWave.ensure(sizeof(int) * 2);
    CUDA_CHECK(cudaMemsetAsync(c->curWave.p, 0, sizeof(int) * 2, st));
    const DevJob* dj = c->jobsBuf.as<DevJob>();
    const WaveChunk* dch = c->chunksBuf.as<WaveChunk>();
    const WaveDesc* dwv = c->wavesBuf.as<WaveDesc>();
    int* dcur = c->curWave.as<int>();
    DevStats* dstats = c->stats.as<DevStats>();
    CUDA_CHECK(cudaMemsetAsync(dstats, 0, sizeof(DevStats), st));
    int* cnt = w.wb.counters;
    int maxFold = 0;
    for (auto& wd : waves) maxFold = std::max(maxFold, wd.foldThreads);

    // One wave: camera, then per bounce closest hit / shade / shadow rays, then the film fold.
    long long launches = 0;  // kernels issued (in graph mode: the nodes of one wave)
    auto issueWave = [&](int items, bool allowEarlyExit) {
        launches += 2;  // camera and film fold
        CUDA_CHECK(cudaMemsetAsync(cnt, 0, sizeof(int) * kNumCounters, st));
        {
            KTimer kt(c, 0);
            launch_camera(dj, dch, dwv, dcur, w.wb.a, cnt + kCntQueue + 1, items, st);
        }
        PathBuf A = w.wb.a, B = w.wb.b;
        int maxItems = items;
        float4* curNee = w.wb.nee;  // the next-event slots the current bounce writes
        for (int d = 1; d <= maxDepth; ++d) {
            {
                KTimer kt(c, 1);
                launch_trace_closest(c->trace, dj, A.job, A.ro, A.rd, cnt + kCntQueue + d, cnt + kCntWork + 2 * d, w.wb.hits, dstats, st);
            }
            {
                KTimer kt(c, 2);
                PathBuf Ao = A;
                if (c->shadeOrder) {
                    launch_partition(A.depth, w.wb.hits, cnt + kCntQueue + d, w.wb.order, cnt + kCntPart + 2 * d, maxItems, st);
                    Ao.order = w.wb.order;
                }
                // next-event slots: read the buffer the previous bounce wrote, write the other
                const size_t neeHalf = size_t(w.wb.cap) * size_t(c->neeSlots);
                float4* neeOut = w.wb.nee + (d & 1) * neeHalf;
                Ao.neeIn = w.wb.nee + ((d + 1) & 1) * neeHalf;
                float4* neeGOut = nullptr;
                if (w.wb.neeG) {
                    const size_t gHalf = size_t(w.wb.cap) * 3 * 2 * size_t(ns);
                    neeGOut = w.wb.neeG + (d & 1) * gHalf;
                    Ao.neeGIn = w.wb.neeG + ((d + 1) & 1) * gHalf;
                }
                float4* pyrGOut = nullptr;
                if (pyramid) {
                    const size_t pHalf = size_t(w.wb.cap) * 2 * size_t(ns);
                    pyrGOut = c->pyrG.as<float4>() + (d & 1) * pHalf;
                    Ao.pyrGIn = c->pyrG.as<float4>() + ((d + 1) & 1) * pHalf;
                }
                curNee = neeOut;
                if (pyramid)
                    launch_shade_pyramid(ns, dj, Ao, B, w.wb.hits, neeOut, w.wb.cap, w.wb.shRo, w.wb.shRd, w.wb.shTgt, w.wb.shJob, cnt + kCntQueue + d,
                                         cnt + kCntQueue + d + 1, cnt + kCntShadow + d, c->samples.as<float>(), dstats,
                                         PyrArgs{dch, dwv, dcur, pyrGOut}, maxItems, st);
                else
                    launch_shade(ns, replay, generic, c->shadeBlocks, dj, Ao, B, w.wb.hits, neeOut, neeGOut, w.wb.cap, w.wb.shRo, w.wb.shRd, w.wb.shTgt, w.wb.shJob,
                                 cnt + kCntQueue + d, cnt + kCntQueue + d + 1, cnt + kCntShadow + d, c->samples.as<float>(), dstats, maxItems, st);
            }
            {
                KTimer kt(c, 3);
                launch_trace_shadow(c->trace, dj, w.wb.shJob, w.wb.shRo, w.wb.shRd, w.wb.shTgt, cnt + kCntShadow + d, cnt + kCntWork + 2 * d + 1, curNee,
                                    dstats, st);
            }
            launches += c->shadeOrder ? 4 : 3;  // closest hit, shade order, shade, shadow rays
            std::swap(A, B);
            if (allowEarlyExit && d >= 6 && d < maxDepth) {
                // stop early once the queue is empty (long MaxDepth with Russian roulette)
                CUDA_CHECK(cudaMemcpyAsync(c->pinnedCount, cnt + kCntQueue + d + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaStreamSynchronize(st));
                if (*c->pinnedCount == 0) break;
                maxItems = *c->pinnedCount;
            }
        }
        {
            KTimer kt(c, 4);
            launch_film_fold(dj, dch, dwv, dcur, (replay || paths) ? nullptr : c->samples.as<float>(), dstats, maxFold, 1, st);
        }
    };

    const char* ge = getenv("SST_GRAPH");
    bool useGraph = !c->profiling && !timeLimit && maxDepth <= 32 && !(ge && std::string(ge) == "0") && waves.size() > 1;
    CUDA_CHECK(cudaEventRecord(c->ev0, st));
    auto t0 = std::chrono::steady_clock::now();
    int wavesDone = 0;
    if (useGraph) {
        // capture one wave (fixed grid sizes; wave parameters are read from device memory)
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            issueWave(w.wb.cap, false);
        } catch (...) {
            cudaStreamEndCapture(st, &graph);
            throw;
        }
        CUDA_CHECK(cudaStreamEndCapture(st, &graph));
        CUDA_CHECK(cudaGraphInstantiate(&exec, graph, 0));
        for (size_t k = 0; k < waves.size(); ++k) CUDA_CHECK(cudaGraphLaunch(exec, st));
        launches *= (long long)waves.size();
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        wavesDone = int(waves.size());
    } else {
        for (size_t k = 0; k < waves.size(); ++k) {
            if (timeLimit && k > 0) {
                CUDA_CHECK(cudaStreamSynchronize(st));
                double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                double per = ms / double(k);
                if (ms + per > double(jobs[0].p.maximumRenderTimeMs)) break;  // PathTracer.cs:221-227
            }
            issueWave(waves[k].items, true);
            CUDA_CHECK(cudaGetLastError());
            if (c->profiling) {
                std::vector<int> hc(kNumCounters);
                CUDA_CHECK(cudaMemcpyAsync(hc.data(), cnt, sizeof(int) * kNumCounters, cudaMemcpyDeviceToHost, st));
                flushTimers(c);
                c->kItems[0] += waves[k].items;
                c->kItems[4] += waves[k].foldThreads;
                for (int d = 1; d <= maxDepth && d < 1024; ++d) {
                    c->kItems[1] += hc[kCntQueue + d];
                    c->kItems[2] += hc[kCntQueue + d];
                    c->kItems[3] += hc[kCntShadow + d];
                }
            }
            ++wavesDone;
        }
    }
    CUDA_CHECK(cudaEventRecord(c->ev1, st));
    CUDA_CHECK(cudaStreamSynchronize(st));
    float ms = 0;
    CUDA_CHECK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    DevStats hs;
    CUDA_CHECK(cudaMemcpy(&hs, dstats, sizeof(DevStats), cudaMemcpyDeviceToHost));
    if (hs.errorFlags & 1) fail(SST_ERR_DEVICE_LIMIT, "BVH traversal stack overflow");
    // iterations completed per job
    for (int k = 0; k < wavesDone; ++k)
        for (int ci = waves[k].chunkBegin; ci < waves[k].chunkEnd; ++ci) {
            const WaveChunk& ck = chunks[ci];
            JobIn& jb = jobs[ck.job];
            if (ck.pixStart + ck.pixCount == jb.p.width * jb.p.height) jb.done = std::max(jb.done, ck.iterBase + ck.nIter - jb.iterFirst);
        }
    if (out) {
        out->renderTimeMs += ms;
        out->numIterations += jobs.size() == 1 ? jobs[0].done : 0;
        out->numKernelLaunches += int(std::min<long long>(launches, 0x7FFFFFFF));
        out->numRays += hs.rays;
        out->numShadowRays += hs.shadowRays;
        uint64_t prev = out->numNanOrInf;
        for (uint64_t k = 0; k < std::min<uint64_t>(hs.nanCount, 4) && prev + k < 4; ++k) {
            out->nanPixel[prev + k] = hs.nanPixel[k];
            out->nanIteration[prev + k] = hs.nanIter[k];
        }
        out->numNanOrInf += hs.nanCount;
    }
}

// Copies n items of `bytes` each to the device (or uses device pointers directly).
template <class T> static const T* toDevice(sst_ctx* c, DevBuf& buf, const T* p, size_t n, int memory) {
    if (memory == SST_MEM_DEVICE) return p;
    buf.ensure(std::max<size_t>(1, n * sizeof(T)));
    CUDA_CHECK(cudaMemcpyAsync(buf.p, p, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return buf.as<T>();
}

template <class T> static T* devCopy(DevBuf& b, const T* h, size_t n, cudaStream_t st) {
    b.ensure(std::max<size_t>(1, n * sizeof(T)));
    if (h) CUDA_CHECK(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return b.as<T>();
}
template <class T> static void hostCopy(T* h, const DevBuf& b, size_t n, cudaStream_t st) {
    CUDA_CHECK(cudaMemcpyAsync(h, b.p, n * sizeof(T), cudaMemcpyDeviceToHost, st));
}

// A one-entry job table holding the scene (for the ray-query entry points).
static const DevJob* jobTable(sst_scene* s) {
    DevJob j{};
    j.sc = s->dev;
    s->queryJob.ensure(sizeof(DevJob));
    CUDA_CHECK(cudaMemcpyAsync(s->queryJob.p, &j, sizeof(DevJob), cudaMemcpyHostToDevice, s->ctx->stream));
    return s->queryJob.as<DevJob>();
}

static void runQuery(sst_scene* s, const SstRay* rays, int n, SstHit* hits, int32_t* occl, int memory, bool anyHit) {
    if (!s || (n > 0 && !rays) || n < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid query");
    if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
    if (n == 0) return;
    sst_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    const float4* dr = reinterpret_cast<const float4*>(toDevice(c, c->scratchIn, rays, n, memory));
    // separate origin / direction arrays (SstRay = org, tmin, dir, tmax = two float4)
    DevBuf ro, rd;
    ro.ensure(size_t(n) * 16);
    rd.ensure(size_t(n) * 16);
    CUDA_CHECK(cudaMemcpy2DAsync(ro.p, 16, dr, 32, 16, n, cudaMemcpyDeviceToDevice, st));
    CUDA_CHECK(cudaMemcpy2DAsync(rd.p, 16, reinterpret_cast<const char*>(dr) + 16, 32, 16, n, cudaMemcpyDeviceToDevice, st));
    DevBuf cnt, hitsBuf, occBuf;
    cnt.ensure(sizeof(int) * 2);
    int hostCnt[2] = {n, 0};
    CUDA_CHECK(cudaMemcpyAsync(cnt.p, hostCnt, sizeof(hostCnt), cudaMemcpyHostToDevice, st));
    c->stats.ensure(sizeof(DevStats));
    CUDA_CHECK(cudaMemsetAsync(c->stats.p, 0, sizeof(DevStats), st));
    if (anyHit) {
        occBuf.ensure(size_t(n) * 4);
        launch_trace_query(c->trace, jobTable(s), ro.as<float4>(), rd.as<float4>(), cnt.as<int>(), cnt.as<int>() + 1, nullptr, occBuf.as<int>(),
                           c->stats.as<DevStats>(), true, st);
        CUDA_CHECK(cudaMemcpyAsync(occl, occBuf.p, size_t(n) * 4, memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        return;
    }
    hitsBuf.ensure(size_t(n) * 16);
    launch_trace_query(c->trace, jobTable(s), ro.as<float4>(), rd.as<float4>(), cnt.as<int>(), cnt.as<int>() + 1, hitsBuf.as<float4>(), nullptr,
                       c->stats.as<DevStats>(), false, st);
    std::vector<float4> hh(n);
    CUDA_CHECK(cudaMemcpyAsync(hh.data(), hitsBuf.p, size_t(n) * 16, cudaMemcpyDeviceToHost, st));
    CUDA_CHECK(cudaStreamSynchronize(st));
    // expand into SstHit on the host (the device result is the compact (t, u, v, tri) record)
    std::vector<float4> tv(3), tn(1);
    std::vector<int4> aux(1);
    std::vector<SstHit> outHits(n);
    for (int i = 0; i < n; ++i) {
        SstHit& h = outHits[i];
        std::memset(&h, 0, sizeof(h));
        int ti;
        std::memcpy(&ti, &hh[i].w, 4);
        if (ti < 0) { h.meshId = -1; h.primId = -1; continue; }
        CUDA_CHECK(cudaMemcpy(tv.data(), s->triv.as<float4>() + 3 * size_t(ti), 48, cudaMemcpyDeviceToHost));
        CUDA_CHECK(cudaMemcpy(tn.data(), s->triN.as<float4>() + ti, 16, cudaMemcpyDeviceToHost));
        CUDA_CHECK(cudaMemcpy(aux.data(), s->triAux.as<int4>() + ti, 16, cudaMemcpyDeviceToHost));
        float u = hh[i].y, v = hh[i].z;
        h.distance = hh[i].x;
        h.u = u;
        h.v = v;
        h.meshId = aux[0].y;
        h.primId = aux[0].z;
        float w = 1.0f - u - v;
        const float* a = &tv[0].x;
        const float* b = &tv[1].x;
        const float* cc = &tv[2].x;
        float e[3];
        for (int k = 0; k < 3; ++k) {
            h.position[k] = u * b[k] + v * cc[k] + w * a[k];
            e[k] = std::fabs(u * b[k]) + std::fabs(v * cc[k]) + std::fabs(w * a[k]);
        }
        h.errorOffset = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * 32.0f * 1.19209e-07f;
        h.normal[0] = tn[0].x;
        h.normal[1] = tn[0].y;
        h.normal[2] = tn[0].z;
    }
    if (memory == SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpy(hits, outHits.data(), sizeof(SstHit) * n, cudaMemcpyHostToDevice));
    else std::memcpy(hits, outHits.data(), sizeof(SstHit) * n);
}

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

int sst_version(int32_t* major, int32_t* minor) {
    if (major) *major = 0;
    if (minor) *minor = 1;
    return SST_OK;
}

int sst_last_error(char* buffer, size_t size) {
    if (!buffer || size == 0) return SST_ERR_INVALID_ARGUMENT;
    std::strncpy(buffer, g_lastError.c_str(), size - 1);
    buffer[size - 1] = 0;
    return SST_OK;
}

int sst_create(int32_t device, sst_ctx** out) {
    return guarded([&] {
        if (!out) fail(SST_ERR_INVALID_ARGUMENT, "out is NULL");
        int n = 0;
        CUDA_CHECK(cudaGetDeviceCount(&n));
        if (device < 0 || device >= n) fail(SST_ERR_INVALID_ARGUMENT, "no such CUDA device");
        CUDA_CHECK(cudaSetDevice(device));
        auto c = std::make_unique<sst_ctx>();
        c->device = device;
        CUDA_CHECK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        CUDA_CHECK(cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device));
        CUDA_CHECK(cudaEventCreate(&c->ev0));
        CUDA_CHECK(cudaEventCreate(&c->ev1));
        CUDA_CHECK(cudaMallocHost(&c->pinnedCount, sizeof(int) * 4));
        *out = c.release();
    });
}

int sst_destroy(sst_ctx* ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->pinnedCount) cudaFreeHost(ctx->pinnedCount);
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
    });
}

int sst_scene_create(sst_ctx* ctx, sst_scene** out) {
    return guarded([&] {
        if (!ctx || !out) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        auto s = std::make_unique<sst_scene>();
        s->ctx = ctx;
        *out = s.release();
    });
}

int sst_scene_destroy(sst_scene* scene) {
    return guarded([&] {
        if (!scene) return;
        cudaSetDevice(scene->ctx->device);
        cudaStreamSynchronize(scene->ctx->stream);
        delete scene;
    });
}

int sst_scene_add_texture(sst_scene* s, const float* data, int32_t w, int32_t h, int32_t ch, int32_t border, int32_t* out) {
    return guarded([&] {
        if (!s || !data || !out || w <= 0 || h <= 0 || (ch != 1 && ch != 3) || (border != 0 && border != 1))
            fail(SST_ERR_INVALID_ARGUMENT, "invalid texture");
        HostTexture t{w, h, ch, border, std::vector<float>(data, data + size_t(w) * h * ch)};
        s->textures.push_back(std::move(t));
        s->committed = false;
        *out = int(s->textures.size()) - 1;
    });
}

static void checkTex(sst_scene* s, int tex, int wantCh) {
    if (tex >= int(s->textures.size())) fail(SST_ERR_INVALID_ARGUMENT, "texture index out of range");
    (void)wantCh;
}

int sst_scene_add_material_diffuse(sst_scene* s, const float base[3], int32_t tex, int32_t transmitter, int32_t* out) {
    return guarded([&] {
        if (!s || !base || !out) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkTex(s, tex, 3);
        DevMaterial m{};
        m.type = kDiffuse;
        m.baseTex = tex < 0 ? -1 : tex;
        m.roughTex = -1;
        m.transmitter = transmitter ? 1 : 0;
        for (int k = 0; k < 3; ++k) m.base[k] = base[k];
        m.rough = 1.0f;
        m.ior = 1.0f;
        s->materials.push_back(m);
        s->committed = false;
        *out = int(s->materials.size()) - 1;
    });
}

static DevMaterial genericFrom(sst_scene* s, const SstGenericMaterial* p) {
    checkTex(s, p->baseColorTexture, 3);
    checkTex(s, p->roughnessTexture, 1);
    DevMaterial m{};
    m.type = kGeneric;
    m.baseTex = p->baseColorTexture < 0 ? -1 : p->baseColorTexture;
    m.roughTex = p->roughnessTexture < 0 ? -1 : p->roughnessTexture;
    for (int k = 0; k < 3; ++k) m.base[k] = p->baseColor[k];
    m.rough = p->roughness;
    m.metallic = p->metallic;
    m.specTint = p->specularTintStrength;
    m.aniso = p->anisotropic;
    m.specTrans = p->specularTransmittance;
    m.ior = p->indexOfRefraction;
    return m;
}

int sst_scene_add_material_generic(sst_scene* s, const SstGenericMaterial* p, int32_t* out) {
    return guarded([&] {
        if (!s || !p || !out) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        s->materials.push_back(genericFrom(s, p));
        s->committed = false;
        *out = int(s->materials.size()) - 1;
    });
}

int sst_scene_update_material_generic(sst_scene* s, int32_t material, const SstGenericMaterial* p) {
    return guarded([&] {
        if (!s || !p || material < 0 || material >= int(s->materials.size()) || s->materials[material].type != kGeneric)
            fail(SST_ERR_INVALID_ARGUMENT, "invalid generic material");
        s->materials[material] = genericFrom(s, p);
        if (s->committed) {
            CUDA_CHECK(cudaMemcpyAsync(s->mats.as<DevMaterial>() + material, &s->materials[material], sizeof(DevMaterial), cudaMemcpyHostToDevice,
                                       s->ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
        }
    });
}

int sst_scene_add_mesh(sst_scene* s, const float* V, int32_t nV, const int32_t* I, int32_t nT, const float* N, const float* UV, int32_t material,
                       int32_t* out) {
    return guarded([&] {
        if (!s || !out || nV < 0 || nT < 0 || (nV > 0 && !V) || (nT > 0 && !I)) fail(SST_ERR_INVALID_ARGUMENT, "invalid mesh");
        if (material >= int(s->materials.size())) fail(SST_ERR_INVALID_ARGUMENT, "material index out of range");
        HostMesh m;
        m.V.assign(V, V + 3 * size_t(nV));
        m.I.assign(I, I + 3 * size_t(nT));
        if (N) m.N.assign(N, N + 3 * size_t(nV));
        if (UV) m.UV.assign(UV, UV + 2 * size_t(nV));
        m.material = material;
        std::mutex badLock;
        bool anyBad = false;
        parallelRanges(size_t(nT) * 3, 1 << 18, [&](size_t k0, size_t k1) {
            bool rangeBad = false;
            for (size_t k = k0; k < k1; ++k) rangeBad |= m.I[k] < 0 || m.I[k] >= nV;
            if (rangeBad) {
                std::lock_guard<std::mutex> g(badLock);
                anyBad = true;
            }
        });
        if (anyBad) fail(SST_ERR_INVALID_ARGUMENT, "vertex index out of range");
        s->meshes.push_back(std::move(m));
        s->committed = false;
        *out = int(s->meshes.size()) - 1;
    });
}

int sst_scene_add_emitters(sst_scene* s, int32_t mesh, const int32_t* faces, int32_t nFaces, const float rad[3], float exponent, int32_t* outFirst,
                           int32_t* outCount) {
    return guarded([&] {
        if (!s || !rad || mesh < 0 || mesh >= int(s->meshes.size())) fail(SST_ERR_INVALID_ARGUMENT, "invalid emitter mesh");
        const HostMesh& m = s->meshes[mesh];
        int nf = int(m.I.size() / 3);
        int first = int(s->emitters.size());
        int count = faces ? nFaces : nf;
        int added = 0;
        for (int k = 0; k < count; ++k) {
            int f = faces ? faces[k] : k;
            if (f < 0 || f >= nf) fail(SST_ERR_INVALID_ARGUMENT, "face index out of range");
            const float* a = &m.V[3 * size_t(m.I[3 * f])];
            const float* b = &m.V[3 * size_t(m.I[3 * f + 1])];
            const float* c = &m.V[3 * size_t(m.I[3 * f + 2])];
            float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            float area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) * 0.5f;
            if (area == 0.0f) {
                if (faces) fail(SST_ERR_INVALID_ARGUMENT, "Zero-area triangles cannot be emitters");
                continue;  // DiffuseEmitter.MakeFromMesh skips them (DiffuseEmitter.cs:24-28)
            }
            s->emitters.push_back(HostEmitter{mesh, f, {rad[0], rad[1], rad[2]}, exponent < 0 ? -1.0f : exponent});
            ++added;
        }
        s->committed = false;
        if (outFirst) *outFirst = first;
        if (outCount) *outCount = added;
    });
}

int sst_scene_set_emitter_radiance(sst_scene* s, int32_t first, int32_t count, const float* rgb) {
    return guarded([&] {
        if (!s || !rgb || first < 0 || count < 0 || first + count > int(s->emitters.size())) fail(SST_ERR_INVALID_ARGUMENT, "emitter range");
        for (int k = 0; k < count; ++k)
            for (int c = 0; c < 3; ++c) s->emitters[first + k].rad[c] = rgb[3 * k + c];
        if (s->committed) {
            // radiance lives in DevEmitter.rad: patch the device copies
            std::vector<DevEmitter> tmp(count);
            CUDA_CHECK(cudaMemcpy(tmp.data(), s->ems.as<DevEmitter>() + first, sizeof(DevEmitter) * count, cudaMemcpyDeviceToHost));
            for (int k = 0; k < count; ++k) tmp[k].rad = make_float4(rgb[3 * k], rgb[3 * k + 1], rgb[3 * k + 2], tmp[k].rad.w);
            CUDA_CHECK(cudaMemcpy(s->ems.as<DevEmitter>() + first, tmp.data(), sizeof(DevEmitter) * count, cudaMemcpyHostToDevice));
        }
    });
}

int sst_scene_set_envmap(sst_scene* s, const float* rgb, int32_t w, int32_t h) {
    return guarded([&] {
        if (!s || !rgb || w <= 0 || h <= 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid environment map");
        s->envRgb.assign(rgb, rgb + 3 * size_t(w) * h);
        s->envW = w;
        s->envH = h;
        s->committed = false;
    });
}

int sst_scene_set_camera(sst_scene* s, const float m[16], float fov) {
    return guarded([&] {
        if (!s || !m) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        float tmp[16];
        if (!invert4(m, tmp)) fail(SST_ERR_INVALID_ARGUMENT, "World to camera transform must be invertible.");
        if (!(fov > 0.0f && fov < 180.0f)) fail(SST_ERR_INVALID_ARGUMENT, "field of view out of range");
        std::memcpy(s->w2c, m, sizeof(float) * 16);
        s->fovDeg = fov;
        s->cameraSet = true;
        s->committed = false;
    });
}

int sst_scene_commit(sst_scene* s, int32_t w, int32_t h) {
    return guarded([&] {
        if (!s) fail(SST_ERR_INVALID_ARGUMENT, "NULL scene");
        commitScene(s, w, h);
    });
}

int sst_scene_info(sst_scene* s, int32_t* ne, int32_t* nt, int32_t* nn) {
    return guarded([&] {
        if (!s) fail(SST_ERR_INVALID_ARGUMENT, "NULL scene");
        if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (ne) *ne = int(s->emitters.size());
        if (nt) *nt = s->nTri;
        if (nn) *nn = s->nNodes;
    });
}

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

int sst_render(sst_scene* s, const SstPathTracerParams* p, float* film, int32_t memory, SstRenderStats* stats) {
    return guarded([&] {
        if (!s || !p || !film) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkParams(s, p);
        sst_ctx* c = s->ctx;
        CUDA_CHECK(cudaSetDevice(c->device));
        SstRenderStats local{};
        for (int k = 0; k < 4; ++k) { local.nanPixel[k] = -1; local.nanIteration[k] = -1; }
        size_t filmBytes = size_t(p->width) * p->height * 3 * sizeof(float);
        float* dFilm = film;
        auto tfb0 = std::chrono::steady_clock::now();
        if (memory != SST_MEM_DEVICE) {
            c->film.ensure(filmBytes);
            dFilm = c->film.as<float>();
            if (p->firstIteration > 0) CUDA_CHECK(cudaMemcpyAsync(dFilm, film, filmBytes, cudaMemcpyHostToDevice, c->stream));
            else CUDA_CHECK(cudaMemsetAsync(dFilm, 0, filmBytes, c->stream));
        } else if (p->firstIteration == 0) {
            CUDA_CHECK(cudaMemsetAsync(dFilm, 0, filmBytes, c->stream));
        }
        CUDA_CHECK(cudaStreamSynchronize(c->stream));
        double fbMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tfb0).count();
        HostPrefault prefault;
        if (memory != SST_MEM_DEVICE) prefault.add(film, filmBytes);
        prefault.start();
        if (p->firstIteration < p->totalSpp) {
            std::vector<JobIn> jobs(1);
            jobs[0].s = s;
            jobs[0].p = *p;
            jobs[0].dFilm = dFilm;
            jobs[0].iterFirst = p->firstIteration;
            jobs[0].iterEnd = p->totalSpp;
            renderJobs(c, jobs, &local);
        }
        prefault.finish();
        auto tfb1 = std::chrono::steady_clock::now();
        if (memory != SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpy(film, dFilm, filmBytes, cudaMemcpyDeviceToHost));
        fbMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tfb1).count();
        local.frameBufferTimeMs = fbMs;
        if (stats) *stats = local;
    });
}

int sst_render_paths(sst_scene* s, const SstPathTracerParams* p, const int32_t* pixels, const int32_t* iterations, int32_t n, float* rgb,
                     int32_t memory, SstRenderStats* stats) {
    return guarded([&] {
        if (!s || !p || n < 0 || (n > 0 && (!pixels || !iterations || !rgb))) fail(SST_ERR_INVALID_ARGUMENT, "invalid path list");
        checkParams(s, p);
        sst_ctx* c = s->ctx;
        CUDA_CHECK(cudaSetDevice(c->device));
        SstRenderStats local{};
        for (int k = 0; k < 4; ++k) { local.nanPixel[k] = -1; local.nanIteration[k] = -1; }
        std::vector<int32_t> px(pixels ? size_t(n) : 0), it(iterations ? size_t(n) : 0);
        if (n > 0) {
            const cudaMemcpyKind k = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
            CUDA_CHECK(cudaMemcpy(px.data(), pixels, size_t(n) * 4, k));
            CUDA_CHECK(cudaMemcpy(it.data(), iterations, size_t(n) * 4, k));
        }
        const long long P = (long long)p->width * p->height;
        for (int32_t k = 0; k < n; ++k)
            if (px[k] < 0 || px[k] >= P || it[k] < 0) fail(SST_ERR_INVALID_ARGUMENT, "pixel or iteration out of range");
        const int batch = c->waveCapacity > 0 ? c->waveCapacity : defaultWaveCapacity();
        std::vector<WaveChunk> chunks;
        for (int32_t b0 = 0; b0 < n; b0 += batch) {
            const int cnt = std::min(batch, n - b0);
            chunks.assign(size_t(cnt), WaveChunk{});
            for (int k = 0; k < cnt; ++k) {
                WaveChunk& ck = chunks[k];
                ck.job = 0;
                ck.iterBase = it[b0 + k];
                ck.nIter = 1;
                ck.pixStart = px[b0 + k];
                ck.pixCount = 1;
                ck.itemOffset = k;
                ck.film = nullptr;
            }
            std::vector<JobIn> jobs(1);
            jobs[0].s = s;
            jobs[0].p = *p;
            jobs[0].p.maximumRenderTimeMs = 0;
            jobs[0].iterFirst = 0;
            jobs[0].iterEnd = 1;
            renderJobs(c, jobs, &local, false, &chunks);
            const cudaMemcpyKind k = memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
            CUDA_CHECK(cudaMemcpyAsync(rgb + 3 * size_t(b0), c->samples.p, size_t(cnt) * 12, k, c->stream));
            CUDA_CHECK(cudaStreamSynchronize(c->stream));
        }
        local.numIterations = 0;
        if (stats) *stats = local;
    });
}

static TraceTuning toTrace(const SstTuning& t) { return TraceTuning{t.traceBlock, t.traceStackShared, t.traceBlocksPerSM, t.traceBvhWidth, t.traceRefillIdle}; }

static void checkTuning(const SstTuning& t) {
    if (!traceTuningValid(toTrace(t)))
        fail(SST_ERR_INVALID_ARGUMENT, "traceBlock must be 64, 128 or 256, traceStackShared 16, 24 or 32, traceBvhWidth 2 or 4, and traceRefillIdle in [1, 32]");
    if (t.waveCapacity != 0 && (t.waveCapacity < 1024 || t.waveCapacity > (1 << 24)))
        fail(SST_ERR_INVALID_ARGUMENT, "waveCapacity must be 0 or in [1024, 2^24]");
    if (t.traceBlocksPerSM < 0 || t.traceBlocksPerSM > 64) fail(SST_ERR_INVALID_ARGUMENT, "traceBlocksPerSM must be in [0, 64]");
    if (t.shadeOrder != 0 && t.shadeOrder != 1) fail(SST_ERR_INVALID_ARGUMENT, "shadeOrder must be 0 or 1");
    if (!shadeBlocksValid(t.shadeBlocks))
        fail(SST_ERR_INVALID_ARGUMENT, "shadeBlocks must be 8 or " + std::to_string(shadeDenseBlocks()));
}

static SstTuning currentTuning(const sst_ctx* c) {
    SstTuning t{};
    t.waveCapacity = c->waveCapacity;
    t.traceBlock = c->trace.block;
    t.traceStackShared = c->trace.smemStack;
    t.traceBlocksPerSM = c->trace.blocksPerSM;
    t.traceBvhWidth = c->trace.width;
    t.traceRefillIdle = c->trace.refillIdle;
    t.shadeBlocks = c->shadeBlocks;
    t.shadeOrder = c->shadeOrder;
    return t;
}

int sst_get_tuning(sst_ctx* c, SstTuning* out) {
    return guarded([&] {
        if (!c || !out) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        *out = currentTuning(c);
    });
}

int sst_set_tuning(sst_ctx* c, const SstTuning* t) {
    return guarded([&] {
        if (!c || !t) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkTuning(*t);
        c->trace = toTrace(*t);
        c->waveCapacity = t->waveCapacity;
        c->shadeBlocks = t->shadeBlocks;
        c->shadeOrder = t->shadeOrder;
    });
}

int sst_autotune(sst_scene* s, const SstPathTracerParams* p, int32_t trialIterations, SstTuning* chosen, double* bestTrialMs) {
    return guarded([&] {
        if (!s || !p || trialIterations < 1) fail(SST_ERR_INVALID_ARGUMENT, "invalid autotune arguments");
        SstPathTracerParams tp = *p;
        tp.firstIteration = 0;
        tp.totalSpp = trialIterations;
        tp.maximumRenderTimeMs = 0;
        checkParams(s, &tp);
        sst_ctx* c = s->ctx;
        CUDA_CHECK(cudaSetDevice(c->device));
        const SstTuning start = currentTuning(c);
        DevBuf film;
        film.ensure(size_t(tp.width) * tp.height * 3 * sizeof(float));
        const bool prof = c->profiling;
        c->profiling = false;
        // one candidate: the faster of two trial renders of `iters` iterations
        auto trial = [&](const SstTuning& t, int iters) {
            c->trace = toTrace(t);
            c->waveCapacity = t.waveCapacity;
            c->shadeBlocks = t.shadeBlocks;
            c->shadeOrder = t.shadeOrder;
            double best = 1e300;
            for (int r = 0; r < 2; ++r) {
                std::vector<JobIn> jobs(1);
                jobs[0].s = s;
                jobs[0].p = tp;
                jobs[0].p.totalSpp = iters;
                jobs[0].dFilm = film.as<float>();
                jobs[0].iterFirst = 0;
                jobs[0].iterEnd = iters;
                SstRenderStats st{};
                renderJobs(c, jobs, &st);
                best = std::min(best, st.renderTimeMs);
            }
            return best;
        };
        SstTuning best = start;
        double bestMs = 1e300;
        // the kernel stages time trials of at least one full default wave of paths: a trial of a
        // few small iterations lasts a fraction of a millisecond and its timing is mostly noise
        const long long tpix = (long long)tp.width * tp.height;
        const int kIters = (int)std::max<long long>(trialIterations, ((long long)defaultWaveCapacity() + tpix - 1) / tpix);
        try {
            // traversal variant
            for (int wdt : {2, 4})
                for (int b : {64, 128, 256})
                    for (int k : {16, 24, 32}) {
                        SstTuning t = best;
                        t.traceBvhWidth = wdt;
                        t.traceBlock = b;
                        t.traceStackShared = k;
                        t.traceBlocksPerSM = 0;
                        double ms = trial(t, kIters);
                        if (ms < bestMs) { bestMs = ms; best = t; }
                    }
            // refill threshold of the 4-wide traversal
            if (best.traceBvhWidth == 4)
                for (int ri : {32, 12, 24}) {
                    if (ri == best.traceRefillIdle) continue;
                    SstTuning t = best;
                    t.traceRefillIdle = ri;
                    double ms = trial(t, kIters);
                    if (ms < bestMs) { bestMs = ms; best = t; }
                }
            // occupancy build of the shade kernel with GenericMaterials
            {
                SstTuning t = best;
                t.shadeBlocks = best.shadeBlocks == 8 ? shadeDenseBlocks() : 8;
                double ms = trial(t, kIters);
                if (ms < bestMs) { bestMs = ms; best = t; }
            }
            // shade order: surface hits first, or queue order
            {
                SstTuning t = best;
                t.shadeOrder = 1 - best.shadeOrder;
                double ms = trial(t, kIters);
                if (ms < bestMs) { bestMs = ms; best = t; }
            }
            // resident traversal blocks per SM
            int m = traceMaxBlocksPerSM(toTrace(best));
            for (int bps : {m / 2, (3 * m) / 4}) {
                if (bps < 1 || bps >= m) continue;
                SstTuning t = best;
                t.traceBlocksPerSM = bps;
                double ms = trial(t, kIters);
                if (ms < bestMs) { bestMs = ms; best = t; }
            }
            // wave capacity: the trials hold about four waves of the largest candidate (within the
            // caller's spp), since a trial of one or two short waves favours small waves that
            // leave the GPU idle in their last bounces of a long render
            const long long pixels = (long long)tp.width * tp.height;
            const int wcIters = (int)std::max<long long>(trialIterations, std::min<long long>(p->totalSpp, (4LL << 22) / pixels + 1));
            const long long items = pixels * wcIters;
            SstTuning cur = best;
            double curMs = trial(cur, wcIters);
            for (int capLog = 19; capLog <= 22; ++capLog) {
                int cap = 1 << capLog;
                if (cap == (cur.waveCapacity > 0 ? cur.waveCapacity : defaultWaveCapacity())) continue;
                if ((long long)cap > 2 * items) break;
                SstTuning t = cur;
                t.waveCapacity = cap;
                double ms = trial(t, wcIters);
                if (ms < curMs) { curMs = ms; best = t; }
            }
            // the reported time is that of a trial of trialIterations iterations
            bestMs = wcIters == trialIterations ? curMs : trial(best, trialIterations);
        } catch (...) {
            c->trace = toTrace(start);
            c->waveCapacity = start.waveCapacity;
            c->shadeBlocks = start.shadeBlocks;
            c->shadeOrder = start.shadeOrder;
            c->profiling = prof;
            throw;
        }
        c->profiling = prof;
        c->trace = toTrace(best);
        c->waveCapacity = best.waveCapacity;
        c->shadeBlocks = best.shadeBlocks;
        c->shadeOrder = best.shadeOrder;
        if (chosen) *chosen = best;
        if (bestTrialMs) *bestTrialMs = bestMs;
    });
}

static size_t texPoolFloats(const sst_scene* s) {
    size_t n = 0;
    for (auto& t : s->textures) n += t.data.size();
    return n;
}

// Validates the jobs of a batch and fills the renderer's job list.  Films given in host memory
// are staged in device buffers (`staged`); with fromZero every film starts black.
static void batchJobs(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, std::vector<JobIn>& in, std::vector<std::unique_ptr<DevBuf>>& staged,
                      bool fromZero) {
    if (!ctx || (numJobs > 0 && !jobs) || numJobs < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid batch");
    in.assign(numJobs, JobIn{});
    staged.resize(numJobs);
    for (int j = 0; j < numJobs; ++j) {
        const SstRenderJob& J = jobs[j];
        if (!J.scene || !J.film) fail(SST_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": NULL scene or film");
        if (J.scene->ctx != ctx) fail(SST_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": scene belongs to another context");
        checkParams(J.scene, &J.params);
        if (fromZero && (J.params.firstIteration != 0 || J.params.maximumRenderTimeMs > 0))
            fail(SST_ERR_UNSUPPORTED, "job " + std::to_string(j) + ": the adjoint renders all iterations from zero");
        size_t filmBytes = size_t(J.params.width) * J.params.height * 3 * sizeof(float);
        float* dFilm = J.film;
        if (J.memory != SST_MEM_DEVICE) {
            staged[j].reset(new DevBuf());
            staged[j]->ensure(filmBytes);
            dFilm = staged[j]->as<float>();
            if (J.params.firstIteration > 0) CUDA_CHECK(cudaMemcpyAsync(dFilm, J.film, filmBytes, cudaMemcpyHostToDevice, ctx->stream));
            else CUDA_CHECK(cudaMemsetAsync(dFilm, 0, filmBytes, ctx->stream));
        } else if (J.params.firstIteration == 0) {
            CUDA_CHECK(cudaMemsetAsync(dFilm, 0, filmBytes, ctx->stream));
        }
        in[j].s = J.scene;
        in[j].p = J.params;
        in[j].dFilm = dFilm;
        in[j].iterFirst = J.params.firstIteration;
        in[j].iterEnd = std::max(J.params.firstIteration, J.params.totalSpp);
        if (J.camera) {
            in[j].hasCam = true;
            in[j].cam = makeCamera(J.camera->worldToCamera, J.camera->verticalFovDegrees, J.params.width, J.params.height);
        }
    }
}

// Copies the staged films of host-memory jobs back.
static void batchFilmsOut(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, const std::vector<JobIn>& in) {
    for (int j = 0; j < numJobs; ++j) {
        if (jobs[j].memory != SST_MEM_DEVICE) {
            size_t filmBytes = size_t(jobs[j].params.width) * jobs[j].params.height * 3 * sizeof(float);
            CUDA_CHECK(cudaMemcpyAsync(jobs[j].film, in[j].dFilm, filmBytes, cudaMemcpyDeviceToHost, ctx->stream));
        }
    }
    CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
}

static SstRenderStats emptyStats() {
    SstRenderStats t{};
    for (int k = 0; k < 4; ++k) { t.nanPixel[k] = -1; t.nanIteration[k] = -1; }
    return t;
}

int sst_render_layers(sst_scene* s, const SstPathTracerParams* p, float* film, int32_t memory, const SstFilmLayers* L, SstRenderStats* stats) {
    return guarded([&] {
        if (!s || !p || !film || !L) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkParams(s, p);
        const bool wantVar = L->variance || L->varianceAverage;
        if (wantVar && !L->varianceState) fail(SST_ERR_INVALID_ARGUMENT, "the variance layer needs its state array");
        if (L->errors && !L->reference) fail(SST_ERR_INVALID_ARGUMENT, "error metrics need a reference image");
        if ((L->albedo == nullptr) != (L->normal == nullptr)) fail(SST_ERR_INVALID_ARGUMENT, "albedo and normal layers come together");
        if (L->numOutliers < 0 || L->numOutliers > kMaxOutliers) fail(SST_ERR_INVALID_ARGUMENT, "numOutliers must be 0..8");
        if (L->numOutliers > 0 && (!L->outlierWeight || !L->outlierIteration))
            fail(SST_ERR_INVALID_ARGUMENT, "the outlier cache needs its weight and iteration arrays");
        sst_ctx* c = s->ctx;
        cudaStream_t st = c->stream;
        CUDA_CHECK(cudaSetDevice(c->device));
        const size_t P = size_t(p->width) * p->height;
        const int first = p->firstIteration, S = p->totalSpp;
        const bool resume = first > 0;
        const cudaMemcpyKind in = L->memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        const cudaMemcpyKind out = L->memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        SstRenderStats local = emptyStats();
        float* dFilm = film;
        if (memory != SST_MEM_DEVICE) {
            c->film.ensure(P * 12);
            dFilm = c->film.as<float>();
            if (resume) CUDA_CHECK(cudaMemcpyAsync(dFilm, film, P * 12, cudaMemcpyHostToDevice, st));
        }
        if (!resume) CUDA_CHECK(cudaMemsetAsync(dFilm, 0, P * 12, st));
        std::vector<JobIn> jobs(1);
        jobs[0].s = s;
        jobs[0].p = *p;
        jobs[0].dFilm = dFilm;
        jobs[0].iterFirst = first;
        jobs[0].iterEnd = std::max(first, S);
        DevLayers& lay = jobs[0].lay;
        // layer state: read back in when resuming, zero otherwise
        auto state = [&](DevBuf& b, size_t bytes, const float* src) {
            b.ensure(bytes);
            if (resume) CUDA_CHECK(cudaMemcpyAsync(b.p, src, bytes, in, st));
            else CUDA_CHECK(cudaMemsetAsync(b.p, 0, bytes, st));
            return b.as<float>();
        };
        if (wantVar) {
            lay.varMean = state(c->layMean, P * 8, L->varianceState);  // mean plane, then moment plane
            lay.varMoment = lay.varMean + P;
        }
        if (L->albedo) {
            lay.aovAlbedo = state(c->layAlb, P * 12, L->albedo);
            lay.aovNormal = state(c->layNrm, P * 12, L->normal);
        }
        if (L->reference) {
            lay.ref = toDevice(c, c->layRef, L->reference, P * 3, L->memory);
            c->layErr.ensure(std::max<size_t>(1, size_t(S) * 16));
            CUDA_CHECK(cudaMemsetAsync(c->layErr.p, 0, std::max<size_t>(1, size_t(S) * 16), st));
            lay.errSum = c->layErr.as<double>();
            if (L->errors && first < S) {
                // per-pixel errors of every iteration of this call, for the outlier-rejecting RelMSE
                c->layErrPix.ensure(size_t(S - first) * P * 4);
                lay.errPix = c->layErrPix.as<float>();
                lay.errFirst = first;
            }
        }
        if (L->techPyramid) {
            // technique pyramids of this call (the reference creates them anew in every Render)
            const size_t bytes = 2 * 2 * size_t(p->maxDepth) * P * 12;
            c->layPyr.ensure(bytes);
            CUDA_CHECK(cudaMemsetAsync(c->layPyr.p, 0, bytes, st));
            lay.pyr = c->layPyr.as<float>();
            lay.pyrSpp = p->totalSpp;
        }
        const int nOut = L->numOutliers;
        if (nOut > 0) {
            // OutlierReplayCache: created empty with the frame buffer's first iteration, kept after that
            const size_t n = P * size_t(nOut);
            c->layOutW.ensure(n * 4);
            c->layOutIt.ensure(n * 4);
            if (resume) {
                CUDA_CHECK(cudaMemcpyAsync(c->layOutW.p, L->outlierWeight, n * 4, in, st));
                CUDA_CHECK(cudaMemcpyAsync(c->layOutIt.p, L->outlierIteration, n * 4, in, st));
            } else {
                CUDA_CHECK(cudaMemsetAsync(c->layOutW.p, 0, n * 4, st));
                CUDA_CHECK(cudaMemsetAsync(c->layOutIt.p, 0xFF, n * 4, st));
            }
            lay.nOut = nOut;
            lay.outW = c->layOutW.as<float>();
            lay.outIt = c->layOutIt.as<int>();
        }
        HostPrefault prefault;
        if (memory != SST_MEM_DEVICE) prefault.add(film, P * 12);
        if (L->memory != SST_MEM_DEVICE) {
            if (L->techPyramid) prefault.add(L->techPyramid, 2 * 2 * size_t(p->maxDepth) * P * 12);
            if (nOut > 0) {
                prefault.add(L->outlierWeight, P * size_t(nOut) * 4);
                prefault.add(L->outlierIteration, P * size_t(nOut) * 4);
            }
            if (wantVar) prefault.add(L->varianceState, P * 8);
            if (L->variance) prefault.add(L->variance, P * 4);
            if (L->albedo) {
                prefault.add(L->albedo, P * 12);
                prefault.add(L->normal, P * 12);
            }
        }
        prefault.start();
        if (first < S) renderJobs(c, jobs, &local);
        prefault.finish();
        if (L->techPyramid) CUDA_CHECK(cudaMemcpyAsync(L->techPyramid, lay.pyr, 2 * 2 * size_t(p->maxDepth) * P * 12, out, st));
        if (nOut > 0) {
            const size_t n = P * size_t(nOut);
            CUDA_CHECK(cudaMemcpyAsync(L->outlierWeight, lay.outW, n * 4, out, st));
            CUDA_CHECK(cudaMemcpyAsync(L->outlierIteration, lay.outIt, n * 4, out, st));
        }
        std::vector<double> trim;
        if (lay.errPix) {
            const int nIt = S - first, done = std::min(nIt, std::max(0, local.numIterations));
            c->layTrim.ensure(size_t(nIt) * 8);
            CUDA_CHECK(cudaMemsetAsync(c->layTrim.p, 0, size_t(nIt) * 8, st));
            // the largest 0.1% of the pixels are dropped (SimpleImageIO's default percentage)
            launch_error_trim(lay.errPix, int(P), int(P / 1000), done, c->layTrim.as<double>(), st);
            CUDA_CHECK(cudaGetLastError());
            trim.resize(nIt);
            CUDA_CHECK(cudaMemcpyAsync(trim.data(), c->layTrim.p, size_t(nIt) * 8, cudaMemcpyDeviceToHost, st));
        }
        if (wantVar) {
            CUDA_CHECK(cudaMemcpyAsync(L->varianceState, lay.varMean, P * 8, out, st));
            c->layVar.ensure(P * 4);
            c->laySum.ensure(8);
            CUDA_CHECK(cudaMemsetAsync(c->laySum.p, 0, 8, st));
            launch_variance_finish(lay.varMean, lay.varMoment, p->width, p->height, c->layVar.as<float>(), c->laySum.as<double>(), st);
            CUDA_CHECK(cudaGetLastError());
            if (L->variance) CUDA_CHECK(cudaMemcpyAsync(L->variance, c->layVar.p, P * 4, out, st));
            if (L->varianceAverage) {
                double sum = 0.0;
                CUDA_CHECK(cudaMemcpyAsync(&sum, c->laySum.p, 8, cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaStreamSynchronize(st));
                float avg = float(sum / double(P));
                if (L->memory == SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpy(L->varianceAverage, &avg, 4, cudaMemcpyHostToDevice));
                else *L->varianceAverage = avg;
            }
        }
        if (L->albedo) {
            CUDA_CHECK(cudaMemcpyAsync(L->albedo, lay.aovAlbedo, P * 12, out, st));
            CUDA_CHECK(cudaMemcpyAsync(L->normal, lay.aovNormal, P * 12, out, st));
        }
        if (L->errors && first < S) {
            std::vector<double> e(2 * size_t(S));
            CUDA_CHECK(cudaMemcpyAsync(e.data(), c->layErr.p, e.size() * 8, cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
            const int nIt = S - first;
            std::vector<double> res(3 * size_t(nIt));
            for (int i = 0; i < nIt; ++i) {
                res[3 * i] = e[2 * size_t(first + i)] / double(3 * P);
                res[3 * i + 1] = e[2 * size_t(first + i) + 1] / double(3 * P);
                res[3 * i + 2] = trim[i];
            }
            if (L->memory == SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpy(L->errors, res.data(), res.size() * 8, cudaMemcpyHostToDevice));
            else std::copy(res.begin(), res.end(), L->errors);
        }
        if (memory != SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpyAsync(film, dFilm, P * 12, cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (stats) *stats = local;
    });
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
            launch_trace_closest(c->trace, job, nullptr, A.ro, A.rd, qIn, work, c->lightHits.as<float4>(), c->stats.as<DevStats>(), st);
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

int sst_render_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, SstRenderStats* stats) {
    return guarded([&] {
        if (!ctx) fail(SST_ERR_INVALID_ARGUMENT, "invalid batch");
        CUDA_CHECK(cudaSetDevice(ctx->device));
        SstRenderStats total = emptyStats();
        std::vector<JobIn> in;
        std::vector<std::unique_ptr<DevBuf>> staged;
        auto t0 = std::chrono::steady_clock::now();
        batchJobs(ctx, jobs, numJobs, in, staged, false);
        CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        double fbMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        HostPrefault prefault;
        for (int j = 0; j < numJobs; ++j)
            if (jobs[j].memory != SST_MEM_DEVICE) prefault.add(jobs[j].film, size_t(jobs[j].params.width) * jobs[j].params.height * 12);
        prefault.start();
        renderJobs(ctx, in, &total);
        prefault.finish();
        auto t1 = std::chrono::steady_clock::now();
        batchFilmsOut(ctx, jobs, numJobs, in);
        fbMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
        total.frameBufferTimeMs = fbMs;
        int it = 0;
        for (auto& j : in) it += j.done;
        total.numIterations = it;
        if (stats) *stats = total;
    });
}

static bool sameJob(const BatchSig& a, const SstRenderJob& J) {
    const SstPathTracerParams &r = a.params, *p = &J.params;
    if (a.scene != J.scene || r.width != p->width || r.height != p->height || r.totalSpp != p->totalSpp || r.maxDepth != p->maxDepth ||
        r.minDepth != p->minDepth || r.baseSeed != p->baseSeed || r.numShadowRays != p->numShadowRays || r.enableBsdfDI != p->enableBsdfDI)
        return false;
    if (a.hasCam != (J.camera != nullptr)) return false;
    return !a.hasCam || std::memcmp(&a.cam, J.camera, sizeof(SstCamera)) == 0;
}

int sst_forward_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, SstRenderStats* stats) {
    return guarded([&] {
        if (!ctx) fail(SST_ERR_INVALID_ARGUMENT, "invalid batch");
        CUDA_CHECK(cudaSetDevice(ctx->device));
        ctx->batchSig.clear();
        std::vector<JobIn> in;
        std::vector<std::unique_ptr<DevBuf>> staged;
        batchJobs(ctx, jobs, numJobs, in, staged, true);
        if ((int)ctx->batchRecord.size() < numJobs) ctx->batchRecord.resize(numJobs);
        for (int j = 0; j < numJobs; ++j) {
            size_t P = size_t(jobs[j].params.width) * jobs[j].params.height;
            if (!ctx->batchRecord[j]) ctx->batchRecord[j].reset(new DevBuf());
            ctx->batchRecord[j]->ensure(std::max<size_t>(1, P * size_t(jobs[j].params.totalSpp) * 12));
            in[j].adj.record = ctx->batchRecord[j]->as<float>();
        }
        SstRenderStats total = emptyStats();
        renderJobs(ctx, in, &total);
        batchFilmsOut(ctx, jobs, numJobs, in);
        for (int j = 0; j < numJobs; ++j) {
            BatchSig sig{};
            sig.scene = jobs[j].scene;
            sig.params = jobs[j].params;
            sig.hasCam = jobs[j].camera != nullptr;
            if (sig.hasCam) sig.cam = *jobs[j].camera;
            ctx->batchSig.push_back(sig);
        }
        int it = 0;
        for (auto& j : in) it += j.done;
        total.numIterations = it;
        if (stats) *stats = total;
    });
}

int sst_backward_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, const float* const* dLdI, int32_t memory, SstGradients* grads,
                       SstRenderStats* stats) {
    return guarded([&] {
        if (!ctx || !jobs || numJobs <= 0 || !dLdI || !grads) fail(SST_ERR_INVALID_ARGUMENT, "invalid batch");
        if ((int)ctx->batchSig.size() != numJobs) fail(SST_ERR_INVALID_ARGUMENT, "sst_backward_batch needs a preceding sst_forward_batch with the same jobs");
        for (int j = 0; j < numJobs; ++j)
            if (!sameJob(ctx->batchSig[j], jobs[j]) || !dLdI[j])
                fail(SST_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + " differs from the last sst_forward_batch (or has no dLoss/dImage)");
        CUDA_CHECK(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        std::vector<JobIn> in;
        std::vector<std::unique_ptr<DevBuf>> staged;
        batchJobs(ctx, jobs, numJobs, in, staged, true);
        if ((int)ctx->batchDLdI.size() < numJobs) ctx->batchDLdI.resize(numJobs);
        // gradient buffers of each distinct scene, zeroed once
        std::vector<sst_scene*> scenes;
        std::vector<int> firstJob;
        for (int j = 0; j < numJobs; ++j) {
            sst_scene* s = jobs[j].scene;
            if (std::find(scenes.begin(), scenes.end(), s) != scenes.end()) continue;
            scenes.push_back(s);
            firstJob.push_back(j);
            size_t nTex = texPoolFloats(s), nMat = s->materials.size(), nEm = s->emitters.size();
            s->gTex.ensure(std::max<size_t>(1, nTex * 4));
            s->gMatBase.ensure(std::max<size_t>(1, nMat * 12));
            s->gMatRough.ensure(std::max<size_t>(1, nMat * 4));
            s->gEmitter.ensure(std::max<size_t>(1, nEm * 12));
            CUDA_CHECK(cudaMemsetAsync(s->gTex.p, 0, std::max<size_t>(1, nTex * 4), st));
            CUDA_CHECK(cudaMemsetAsync(s->gMatBase.p, 0, std::max<size_t>(1, nMat * 12), st));
            CUDA_CHECK(cudaMemsetAsync(s->gMatRough.p, 0, std::max<size_t>(1, nMat * 4), st));
            CUDA_CHECK(cudaMemsetAsync(s->gEmitter.p, 0, std::max<size_t>(1, nEm * 12), st));
        }
        for (int j = 0; j < numJobs; ++j) {
            sst_scene* s = jobs[j].scene;
            size_t P = size_t(jobs[j].params.width) * jobs[j].params.height;
            if (!ctx->batchDLdI[j]) ctx->batchDLdI[j].reset(new DevBuf());
            in[j].dFilm = nullptr;
            DevAdj& a = in[j].adj;
            a.record = ctx->batchRecord[j]->as<float>();
            a.dLdI = toDevice(ctx, *ctx->batchDLdI[j], dLdI[j], P * 3, memory);
            a.invSpp = 1.0f / float(std::max(1, jobs[j].params.totalSpp));
            a.gTex = s->gTex.as<float>();
            a.gMatBase = s->gMatBase.as<float>();
            a.gMatRough = s->gMatRough.as<float>();
            a.gEmitter = s->gEmitter.as<float>();
        }
        SstRenderStats total = emptyStats();
        renderJobs(ctx, in, &total, true);
        for (size_t k = 0; k < scenes.size(); ++k) {
            sst_scene* s = scenes[k];
            SstGradients& g = grads[firstJob[k]];
            size_t nTex = texPoolFloats(s), nMat = s->materials.size(), nEm = s->emitters.size();
            auto out = [&](float* dst, const DevBuf& src, size_t n) {
                if (!dst || n == 0) return;
                CUDA_CHECK(cudaMemcpyAsync(dst, src.p, n * 4, g.memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
            };
            out(g.textures, s->gTex, nTex);
            out(g.materialBaseColor, s->gMatBase, nMat * 3);
            out(g.materialRoughness, s->gMatRough, nMat);
            out(g.emitterRadiance, s->gEmitter, nEm * 3);
        }
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (stats) *stats = total;
    });
}

int sst_scene_update_texture(sst_scene* s, int32_t texture, const float* data) {
    return guarded([&] {
        if (!s || !data || texture < 0 || texture >= int(s->textures.size())) fail(SST_ERR_INVALID_ARGUMENT, "invalid texture");
        HostTexture& t = s->textures[texture];
        std::copy(data, data + t.data.size(), t.data.begin());
        if (s->committed) {
            size_t off = 0;
            for (int k = 0; k < texture; ++k) off += s->textures[k].data.size();
            CUDA_CHECK(cudaMemcpyAsync(s->texData.as<float>() + off, t.data.data(), sizeof(float) * t.data.size(), cudaMemcpyHostToDevice,
                                       s->ctx->stream));
            CUDA_CHECK(cudaStreamSynchronize(s->ctx->stream));
        }
    });
}


int sst_forward(sst_scene* s, const SstPathTracerParams* p, float* film, int32_t memory, SstRenderStats* stats) {
    return guarded([&] {
        if (!s || !p || !film) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkParams(s, p);
        if (p->firstIteration != 0 || p->maximumRenderTimeMs > 0) fail(SST_ERR_UNSUPPORTED, "sst_forward renders all iterations from zero");
        sst_ctx* c = s->ctx;
        CUDA_CHECK(cudaSetDevice(c->device));
        size_t P = size_t(p->width) * p->height;
        s->record.ensure(std::max<size_t>(1, P * size_t(p->totalSpp) * 12));
        SstRenderStats local{};
        for (int k = 0; k < 4; ++k) { local.nanPixel[k] = -1; local.nanIteration[k] = -1; }
        size_t filmBytes = P * 3 * sizeof(float);
        float* dFilm = film;
        if (memory != SST_MEM_DEVICE) {
            c->film.ensure(filmBytes);
            dFilm = c->film.as<float>();
        }
        CUDA_CHECK(cudaMemsetAsync(dFilm, 0, filmBytes, c->stream));
        std::vector<JobIn> jobs(1);
        jobs[0].s = s;
        jobs[0].p = *p;
        jobs[0].dFilm = dFilm;
        jobs[0].iterFirst = 0;
        jobs[0].iterEnd = p->totalSpp;
        jobs[0].adj.record = s->record.as<float>();
        renderJobs(c, jobs, &local);
        if (memory != SST_MEM_DEVICE) CUDA_CHECK(cudaMemcpy(film, dFilm, filmBytes, cudaMemcpyDeviceToHost));
        s->recordValid = true;
        s->recordParams = *p;
        if (stats) *stats = local;
    });
}

int sst_backward(sst_scene* s, const SstPathTracerParams* p, const float* dLdI, int32_t memory, SstGradients* g, SstRenderStats* stats) {
    return guarded([&] {
        if (!s || !p || !dLdI || !g) fail(SST_ERR_INVALID_ARGUMENT, "NULL argument");
        checkParams(s, p);
        const SstPathTracerParams& r = s->recordParams;
        if (!s->recordValid || r.width != p->width || r.height != p->height || r.totalSpp != p->totalSpp || r.maxDepth != p->maxDepth ||
            r.minDepth != p->minDepth || r.baseSeed != p->baseSeed || r.numShadowRays != p->numShadowRays || r.enableBsdfDI != p->enableBsdfDI)
            fail(SST_ERR_INVALID_ARGUMENT, "sst_backward needs a preceding sst_forward with the same parameters");
        sst_ctx* c = s->ctx;
        cudaStream_t st = c->stream;
        CUDA_CHECK(cudaSetDevice(c->device));
        size_t P = size_t(p->width) * p->height;
        const float* dG = toDevice(c, s->dLdI, dLdI, P * 3, memory);
        size_t nTex = texPoolFloats(s), nMat = s->materials.size(), nEm = s->emitters.size();
        s->gTex.ensure(std::max<size_t>(1, nTex * 4));
        s->gMatBase.ensure(std::max<size_t>(1, nMat * 12));
        s->gMatRough.ensure(std::max<size_t>(1, nMat * 4));
        s->gEmitter.ensure(std::max<size_t>(1, nEm * 12));
        CUDA_CHECK(cudaMemsetAsync(s->gTex.p, 0, std::max<size_t>(1, nTex * 4), st));
        CUDA_CHECK(cudaMemsetAsync(s->gMatBase.p, 0, std::max<size_t>(1, nMat * 12), st));
        CUDA_CHECK(cudaMemsetAsync(s->gMatRough.p, 0, std::max<size_t>(1, nMat * 4), st));
        CUDA_CHECK(cudaMemsetAsync(s->gEmitter.p, 0, std::max<size_t>(1, nEm * 12), st));
        SstRenderStats local{};
        for (int k = 0; k < 4; ++k) { local.nanPixel[k] = -1; local.nanIteration[k] = -1; }
        std::vector<JobIn> jobs(1);
        jobs[0].s = s;
        jobs[0].p = *p;
        jobs[0].p.firstIteration = 0;
        jobs[0].dFilm = nullptr;
        jobs[0].iterFirst = 0;
        jobs[0].iterEnd = p->totalSpp;
        DevAdj& a = jobs[0].adj;
        a.record = s->record.as<float>();
        a.dLdI = dG;
        a.invSpp = 1.0f / float(std::max(1, p->totalSpp));
        a.gTex = s->gTex.as<float>();
        a.gMatBase = s->gMatBase.as<float>();
        a.gMatRough = s->gMatRough.as<float>();
        a.gEmitter = s->gEmitter.as<float>();
        renderJobs(c, jobs, &local, true);
        auto out = [&](float* dst, const DevBuf& src, size_t n) {
            if (!dst || n == 0) return;
            CUDA_CHECK(cudaMemcpyAsync(dst, src.p, n * 4, g->memory == SST_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        };
        out(g->textures, s->gTex, nTex);
        out(g->materialBaseColor, s->gMatBase, nMat * 3);
        out(g->materialRoughness, s->gMatRough, nMat);
        out(g->emitterRadiance, s->gEmitter, nEm * 3);
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (stats) *stats = local;
    });
}

int sst_set_profiling(sst_ctx* ctx, int32_t enable) {
    return guarded([&] {
        if (!ctx) fail(SST_ERR_INVALID_ARGUMENT, "NULL context");
        ctx->profiling = enable != 0;
        for (int k = 0; k < SST_KERNEL_CLASSES; ++k) { ctx->kMs[k] = 0; ctx->kLaunches[k] = 0; ctx->kItems[k] = 0; }
    });
}

int sst_get_kernel_times(sst_ctx* ctx, double* ms, int64_t* launches, int64_t* items, int32_t n) {
    return guarded([&] {
        if (!ctx || n < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid arguments");
        for (int k = 0; k < std::min(n, SST_KERNEL_CLASSES); ++k) {
            if (ms) ms[k] = ctx->kMs[k];
            if (launches) launches[k] = ctx->kLaunches[k];
            if (items) items[k] = ctx->kItems[k];
        }
    });
}

// ---- function-level entry points ----
int sst_debug_material_eval(sst_scene* s, int32_t mat, int32_t n, const float* pts, const float* outs, const float* ins, float* vals, float* pdfs) {
    return guarded([&] {
        if (!s || !s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (mat < 0 || mat >= int(s->materials.size()) || n < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid material query");
        if (n == 0) return;
        cudaStream_t st = s->ctx->stream;
        DevBuf a, b, c, d, e;
        float* dp = devCopy(a, pts, 11 * size_t(n), st);
        float* dout = devCopy(b, outs, 3 * size_t(n), st);
        float* din = devCopy(c, ins, 3 * size_t(n), st);
        float* dv = devCopy<float>(d, nullptr, 3 * size_t(n), st);
        float* dpdf = devCopy<float>(e, nullptr, 2 * size_t(n), st);
        launch_debug_material_eval(s->dev, mat, n, dp, dout, din, dv, dpdf, st);
        CUDA_CHECK(cudaGetLastError());
        hostCopy(vals, d, 3 * size_t(n), st);
        hostCopy(pdfs, e, 2 * size_t(n), st);
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int sst_debug_material_sample(sst_scene* s, int32_t mat, int32_t n, const float* pts, const float* outs, const float* us, float* dirs, float* pdfs,
                              float* ws) {
    return guarded([&] {
        if (!s || !s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (mat < 0 || mat >= int(s->materials.size()) || n < 0) fail(SST_ERR_INVALID_ARGUMENT, "invalid material query");
        if (n == 0) return;
        cudaStream_t st = s->ctx->stream;
        DevBuf a, b, c, d, e, f;
        float* dp = devCopy(a, pts, 11 * size_t(n), st);
        float* dout = devCopy(b, outs, 3 * size_t(n), st);
        float* du = devCopy(c, us, 3 * size_t(n), st);
        float* dd = devCopy<float>(d, nullptr, 3 * size_t(n), st);
        float* dpdf = devCopy<float>(e, nullptr, 2 * size_t(n), st);
        float* dw = devCopy<float>(f, nullptr, 3 * size_t(n), st);
        launch_debug_material_sample(s->dev, mat, n, dp, dout, du, dd, dpdf, dw, st);
        CUDA_CHECK(cudaGetLastError());
        hostCopy(dirs, d, 3 * size_t(n), st);
        hostCopy(pdfs, e, 2 * size_t(n), st);
        hostCopy(ws, f, 3 * size_t(n), st);
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int sst_debug_envmap(sst_scene* s, int32_t n, const float* us, float* dirs, float* pdfs, float* ws, const float* qd, float* rad, float* qpdf) {
    return guarded([&] {
        if (!s || !s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (!s->dev.hasEnv) fail(SST_ERR_INVALID_ARGUMENT, "scene has no environment map");
        if (n <= 0) return;
        cudaStream_t st = s->ctx->stream;
        DevBuf a, b, c, d, e, f, g;
        float* du = devCopy(a, us, 2 * size_t(n), st);
        float* dq = devCopy(b, qd, 3 * size_t(n), st);
        float* dd = devCopy<float>(c, nullptr, 3 * size_t(n), st);
        float* dp = devCopy<float>(d, nullptr, size_t(n), st);
        float* dw = devCopy<float>(e, nullptr, 3 * size_t(n), st);
        float* dr = devCopy<float>(f, nullptr, 3 * size_t(n), st);
        float* dqp = devCopy<float>(g, nullptr, size_t(n), st);
        launch_debug_env(s->dev, n, du, dd, dp, dw, dq, dr, dqp, st);
        CUDA_CHECK(cudaGetLastError());
        hostCopy(dirs, c, 3 * size_t(n), st);
        hostCopy(pdfs, d, size_t(n), st);
        hostCopy(ws, e, 3 * size_t(n), st);
        hostCopy(rad, f, 3 * size_t(n), st);
        hostCopy(qpdf, g, size_t(n), st);
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

int sst_debug_rng(uint32_t base, uint32_t sample, int32_t n, const uint32_t* pixels, int32_t draws, uint32_t* out) {
    return guarded([&] {
        if (n < 0 || draws < 0 || (n > 0 && (!pixels || !out))) fail(SST_ERR_INVALID_ARGUMENT, "invalid rng query");
        if (n == 0 || draws == 0) return;
        DevBuf a, b;
        uint32_t* dp = devCopy(a, pixels, size_t(n), 0);
        uint32_t* dout = devCopy<uint32_t>(b, nullptr, size_t(n) * draws, 0);
        launch_debug_rng(base, sample, n, dp, draws, dout, 0);
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaMemcpy(out, dout, sizeof(uint32_t) * size_t(n) * draws, cudaMemcpyDeviceToHost));
    });
}

int sst_debug_camera(sst_scene* s, int32_t n, const float* film, float* org, float* dir) {
    return guarded([&] {
        if (!s || !s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
        if (n <= 0) return;
        cudaStream_t st = s->ctx->stream;
        DevBuf a, b, c;
        float* df = devCopy(a, film, 2 * size_t(n), st);
        float* dor = devCopy<float>(b, nullptr, 3 * size_t(n), st);
        float* ddr = devCopy<float>(c, nullptr, 3 * size_t(n), st);
        launch_debug_camera(s->dev, n, df, dor, ddr, st);
        CUDA_CHECK(cudaGetLastError());
        hostCopy(org, b, 3 * size_t(n), st);
        hostCopy(dir, c, 3 * size_t(n), st);
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free occlusion query (sst_occluded_noalloc).  Its scratch is one array of fixed size
// in this library's device image, laid out as
//   [0, 256)      queue length and work counter of the traversal kernel
//   [256, 512)    DevStats (ray counts)
//   [512, 1024)   DevJob (the scene record the traversal kernel reads)
//   then          ray origins (float4 x max rays), ray directions (float4 x max rays),
//                 occlusion flags (int x max rays).
// ---------------------------------------------------------------------------------------------
namespace {
constexpr size_t kNaCounters = 0, kNaStats = 256, kNaJob = 512, kNaHeader = 1024;
constexpr size_t kNaMaxRays = SST_NOALLOC_MAX_RAYS;
constexpr size_t kNaBytes = kNaHeader + 2 * 16 * kNaMaxRays + 4 * kNaMaxRays;
static_assert(kNaBytes == 2360320, "the header states the scratch size");
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
        launch_trace_query(c->trace, job, ro, rd, cnt, cnt + 1, nullptr, occ, stats, true, st);
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaMemcpyAsync(occluded, occ, size_t(n) * 4, out, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

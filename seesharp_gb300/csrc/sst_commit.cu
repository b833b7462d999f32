// Scene.Prepare (Scene.cs:103-164) as sst_scene_commit: the meshes are concatenated into one
// triangle table, the BVH is built (on the GPU by default, a binned-SAH host build as the
// alternative), all per-triangle data are stored in BVH leaf order, and the emitter tables and the
// environment-map sampling tables are built.
#include "sst_host.h"

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

// ---------------------------------------------------------------------------------------------
// host math: 4x4 inverse (Laplace expansion over 2x2 minors), perspective matrix
// ---------------------------------------------------------------------------------------------
bool invert4(const float* m, float* out) {
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
DevCamera makeCamera(const float w2c[16], float fovDeg, int W, int H) {
    DevCamera cam{};
    float c2v[16];
    if (!invert4(w2c, cam.c2w)) fail(SST_ERR_INVALID_ARGUMENT, "World to camera transform must be invertible.");
    perspective(fovDeg * 3.14159265f / 180.0f, float(W) / float(H), 0.001f, 1000.0f, c2v);
    if (!invert4(c2v, cam.v2c)) fail(SST_ERR_INVALID_ARGUMENT, "degenerate projection");
    cam.W = W;
    cam.H = H;
    return cam;
}

void commitScene(sst_scene* s, int W, int H) {
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
    // the 8-wide BVH is built on first use (ensureBvh8)
    s->nNodes8 = 0;
    s->bvh8Depth = 0;
    s->bvh8Built = false;
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
    d.nodes8 = s->nNodes8 > 0 ? s->nodes8.as<float4>() : nullptr;
    d.nNodes8 = s->nNodes8;
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

// 8-wide BVH over the committed scene's leaves, children in octant slots, built when a traversal
// first asks for it (the launch tuning's traceBvhWidth = 8): the default 4-wide traversal never
// pays its build time or its memory.  Its traversal stack packs a node index into 24 bits; a scene
// with more 8-wide nodes is traversed 4-wide instead.
void ensureBvh8(sst_scene* s) {
    if (s->bvh8Built || !s->committed || s->nNodes == 0) return;
    cudaStream_t st = s->ctx->stream;
    DevBuf& scratch8 = s->ctx->commitScratch8;
    s->nodes8.ensure(sizeof(float4) * 15 * size_t(s->nNodes));
    scratch8.ensure(bvh8ScratchBytes(s->nNodes));
    int n8 = 0, depth8 = 0;
    int rc = buildBvh8(s->nodes.as<float4>(), s->nNodes, s->nodes8.as<float4>(), scratch8.p, &n8, &depth8, st);
    if (rc != 0) fail(SST_ERR_CUDA, "8-wide BVH build failed (" + std::to_string(rc) + "): " + cudaGetErrorString(cudaGetLastError()));
    s->bvh8Built = true;
    s->nNodes8 = n8 >= (1 << 24) ? 0 : n8;
    s->bvh8Depth = depth8;
    s->dev.nodes8 = s->nNodes8 > 0 ? s->nodes8.as<float4>() : nullptr;
    s->dev.nNodes8 = s->nNodes8;
}

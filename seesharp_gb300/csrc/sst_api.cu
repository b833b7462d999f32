// libsst host driver: the C ABI of include/sst.h.
//
// The context and scene-construction entry points and the function-level entry points of the
// parity tests.  The other entry points live in sst_commit.cu, sst_render.cu, sst_adjoint_api.cu
// and sst_query.cu (sst_host.h lists them).
#include "sst_host.h"

thread_local std::string g_lastError;

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
        CUDA_CHECK(cudaEventCreateWithFlags(&c->evStart, cudaEventDisableTiming));
        for (WaveStore& ws : c->store) {
            CUDA_CHECK(cudaStreamCreateWithFlags(&ws.run, cudaStreamNonBlocking));
            CUDA_CHECK(cudaStreamCreateWithFlags(&ws.side, cudaStreamNonBlocking));
            for (cudaEvent_t* e : {&ws.evShade, &ws.evShadow, &ws.evDone, &ws.evFolded}) CUDA_CHECK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        }
        CUDA_CHECK(cudaMallocHost(&c->pinnedCount, sizeof(int) * 4));
        *out = c.release();
    });
}

int sst_destroy(sst_ctx* ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (WaveStore& ws : ctx->store) {
            if (ws.run) cudaStreamSynchronize(ws.run);
            if (ws.side) cudaStreamSynchronize(ws.side);
        }
        if (ctx->pinnedCount) cudaFreeHost(ctx->pinnedCount);
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        if (ctx->evStart) cudaEventDestroy(ctx->evStart);
        for (WaveStore& ws : ctx->store) {
            for (cudaEvent_t e : {ws.evShade, ws.evShadow, ws.evDone, ws.evFolded})
                if (e) cudaEventDestroy(e);
            if (ws.side) cudaStreamDestroy(ws.side);
            if (ws.run) cudaStreamDestroy(ws.run);
        }
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

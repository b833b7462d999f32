// Path-replay adjoint entry points: sst_forward / sst_backward and the batched forms.  A path is a
// pure function of (BaseSeed, pixel, iteration) (PathTracerBase.ReplayPixel, PathTracer.cs:61-69),
// so the backward pass re-traces every path from its seed with the adjoint shade kernel.
#include "sst_host.h"

static bool sameJob(const BatchSig& a, const SstRenderJob& J) {
    const SstPathTracerParams &r = a.params, *p = &J.params;
    if (a.scene != J.scene || r.width != p->width || r.height != p->height || r.totalSpp != p->totalSpp || r.maxDepth != p->maxDepth ||
        r.minDepth != p->minDepth || r.baseSeed != p->baseSeed || r.numShadowRays != p->numShadowRays || r.enableBsdfDI != p->enableBsdfDI)
        return false;
    if (a.hasCam != (J.camera != nullptr)) return false;
    return !a.hasCam || std::memcmp(&a.cam, J.camera, sizeof(SstCamera)) == 0;
}

extern "C" {


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
}  // extern "C"

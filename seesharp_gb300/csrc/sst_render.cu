// PathTracerBase.Render (Integrators/PathTracer.cs:199-267) as the wavefront renderer: the
// (job, iteration, pixel) paths are cut into waves that fit the path-state buffers; each wave runs
// camera -> {closest hit, shade, shadow rays} x depth -> film fold on the context's stream, replayed
// as one CUDA graph per wave.  Also the launch tuning and autotuner, the frame-buffer layers and
// batched rendering.
#include "sst_host.h"

// ---------------------------------------------------------------------------------------------
// wavefront buffers
// ---------------------------------------------------------------------------------------------
static void bindPath(DevBuf* bufs, PathBuf& p, int cap) {
    size_t c = size_t(cap);
    for (int k = 0; k < 4; ++k) bufs[k].ensure(c * 4);
    for (int k = 4; k < 9; ++k) bufs[k].ensure(c * 16);
    bufs[9].ensure(c * 4);
    p.job = bufs[0].as<uint32_t>();
    p.pix = bufs[1].as<uint32_t>();
    p.rng = bufs[2].as<uint32_t>();
    p.depth = bufs[3].as<uint32_t>();
    p.pw = bufs[4].as<float4>();
    p.rad = bufs[5].as<float4>();
    p.prev = bufs[6].as<float4>();
    p.ro = bufs[7].as<float4>();
    p.rd = bufs[8].as<float4>();
    p.neeFrom = bufs[9].as<uint32_t>();
    p.rec = nullptr;
    p.order = nullptr;
    p.neeIn = p.neeGIn = p.pyrGIn = nullptr;
}

int defaultWaveCapacity() {
    const char* e = getenv("SST_WAVE_CAPACITY");
    if (e) return std::max(1024, atoi(e));
    return 1 << 21;
}

void ensureWave(sst_ctx* c, int cap, int ns, Wave& w, int set) {
    WaveStore& ws = c->store[set];
    if (cap > ws.cap) {
        // grow all path buffers
        ws.cap = cap;
        ws.hits.ensure(size_t(cap) * 16);
    }
    bindPath(ws.pathA, w.wb.a, ws.cap);
    bindPath(ws.pathB, w.wb.b, ws.cap);
    ws.neeSlots = std::max(ws.neeSlots, 2 * ns);
    ws.nee.ensure(2 * size_t(ws.cap) * 16 * ws.neeSlots);  // two buffers: read and written bounce by bounce
    size_t shCap = size_t(ws.cap) * 2 * ns;
    ws.shRo.ensure(shCap * 16);
    ws.shRd.ensure(shCap * 16);
    ws.shTgt.ensure(shCap * 4);
    ws.shJob.ensure(shCap * 4);
    ws.counters.ensure(sizeof(int) * kNumCounters);
    ws.order.ensure(size_t(ws.cap) * 4);
    c->stats.ensure(sizeof(DevStats));
    w.wb.hits = ws.hits.as<float4>();
    w.wb.nee = ws.nee.as<float4>();
    w.wb.shRo = ws.shRo.as<float4>();
    w.wb.shRd = ws.shRd.as<float4>();
    w.wb.shTgt = ws.shTgt.as<int>();
    w.wb.shJob = ws.shJob.as<uint32_t>();
    w.wb.counters = ws.counters.as<int>();
    w.wb.order = ws.order.as<int>();
    w.wb.cap = ws.cap;
    w.wb.shCap = int(shCap);
}

// ---------------------------------------------------------------------------------------------
// render
// ---------------------------------------------------------------------------------------------
void checkParams(const sst_scene* s, const SstPathTracerParams* p) {
    if (!s->committed) fail(SST_ERR_NOT_COMMITTED, "scene is not committed");
    if (p->width != s->W || p->height != s->H) fail(SST_ERR_INVALID_ARGUMENT, "frame buffer size differs from the committed camera resolution");
    if (p->totalSpp < 0 || p->maxDepth < 1 || p->numShadowRays < 0 || p->numShadowRays > kMaxShadowRays || p->firstIteration < 0)
        fail(SST_ERR_INVALID_ARGUMENT, "invalid path tracer parameters");
    if (p->maxDepth > kMaxPathDepth) fail(SST_ERR_UNSUPPORTED, "MaxDepth above 1000 is not supported");
}

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
// estimate is left in the first buffer set's samples at its chunk's item offset.
void renderJobs(sst_ctx* c, std::vector<JobIn>& jobs, SstRenderStats* out, bool replay, const std::vector<WaveChunk>* paths) {
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
    ensureWave(c, cap, ns, w, 0);
    WaveStore& s0 = c->store[0];
    s0.samples.ensure(size_t(w.wb.cap) * 12);
    w.wb.a.adjL = w.wb.a.adjD = w.wb.a.adjP = nullptr;
    w.wb.b.adjL = w.wb.b.adjD = w.wb.b.adjP = nullptr;
    w.wb.neeG = nullptr;
    // the adjoint replay's per-path state of a buffer set (sized by the set's capacity)
    auto bindAdj = [&](Wave& x, int set) {
        WaveStore& sk = c->store[set];
        const size_t cp = size_t(x.wb.cap);
        for (int k = 0; k < 2; ++k) { sk.adjA[k].ensure(cp * 16); sk.adjB[k].ensure(cp * 16); }
        sk.adjA[2].ensure(cp * 48);
        sk.adjB[2].ensure(cp * 48);
        sk.neeG.ensure(2 * cp * 48 * 2 * ns);
        x.wb.a.adjL = sk.adjA[0].as<float4>(); x.wb.a.adjD = sk.adjA[1].as<float4>(); x.wb.a.adjP = sk.adjA[2].as<float4>();
        x.wb.b.adjL = sk.adjB[0].as<float4>(); x.wb.b.adjD = sk.adjB[1].as<float4>(); x.wb.b.adjP = sk.adjB[2].as<float4>();
        x.wb.neeG = sk.neeG.as<float4>();
    };
    if (replay) bindAdj(w, 0);
    std::vector<sst_scene*> jobScenes;
    for (auto& j : jobs) jobScenes.push_back(j.s);
    const TraceTuning trace = traceForBuilding(c, jobScenes.data(), jobScenes.size());
    // any GenericMaterial in the wave's scenes (otherwise the shade kernel without generic code runs)
    bool generic = false;
    for (auto& j : jobs)
        for (auto& m : j.s->materials) generic |= m.type == kGeneric;
    // SST_SHADE_GENERIC=1 runs the generic build for every wave (the build a mixed batch uses)
    const char* sg = getenv("SST_SHADE_GENERIC");
    if (sg && std::string(sg) == "1") generic = true;
    // per-item samples of the denoiser feature layers (written by the first shade, read by the fold)
    bool anyAov = false, pyramid = false;
    for (auto& j : jobs) {
        anyAov |= j.lay.aovAlbedo != nullptr;
        pyramid |= j.lay.pyr != nullptr;
    }
    if (pyramid && replay) fail(SST_ERR_UNSUPPORTED, "the technique pyramid is not available in the adjoint replay");
    // technique pyramid: the payload of every NEE slot
    if (pyramid) c->pyrG.ensure(2 * size_t(w.wb.cap) * 16 * 2 * ns);
    // the split shade form: forward renders with one shadow ray per technique
    const bool split = c->shadeSplit && generic && !replay && !pyramid && ns == 1;
    // job table
    std::vector<DevJob> hj(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) {
        const SstPathTracerParams* P = &jobs[k].p;
        hj[k].sc = jobs[k].s->dev;
        if (jobs[k].hasCam) hj[k].sc.cam = jobs[k].cam;
        hj[k].lay = jobs[k].lay;
        hj[k].cfg = PTConfig{P->width, P->height, P->maxDepth, P->minDepth, P->baseSeed, P->numShadowRays, P->enableBsdfDI, P->ignoreNanAndInf,
                             (c->shadingStats && !replay) ? 1 : 0};
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
    const char* ge = getenv("SST_GRAPH");
    const bool useGraph = !c->profiling && !timeLimit && maxDepth <= 32 && !(ge && std::string(ge) == "0") && waves.size() > 1;
    // Several waves in flight: consecutive waves take turns over nSets buffer sets and their
    // streams, so that one wave's last bounces (few paths, latency-bound) run beside the next
    // wave's first ones; the film folds run in wave order on the context's stream.  Not for the
    // technique pyramid (single-set buffers) and without graphs.
    // SST_WAVES_IN_FLIGHT: 1 to kMaxWaveSets (default 2).
    const char* wf = getenv("SST_WAVES_IN_FLIGHT");
    const int wantSets = std::min(kMaxWaveSets, std::max(1, wf ? atoi(wf) : 2));
    const int nSets = (useGraph && !pyramid && !paths) ? int(std::min<size_t>(size_t(wantSets), waves.size())) : 1;
    const bool multiSets = nSets > 1;
    // the persistent traversal grids: with several waves in flight, three quarters of the resident
    // blocks unless the tuning fixes them, so that the traversal kernels of two waves run side by
    // side instead of one waiting for the other's last blocks (1M-triangle scene, 64-thread blocks:
    // 12 of 16 blocks 318.6 Msamples/s, 10 316.7, 14 315.7, 16 313.4)
    TraceTuning traceRun = trace;
    if (multiSets && traceRun.blocksPerSM == 0) traceRun.blocksPerSM = std::max(1, (3 * traceMaxBlocksPerSM(trace)) / 4);
    Wave ws[kMaxWaveSets];
    for (auto& x : ws) x = w;
    for (int k = 1; k < nSets; ++k) {
        ensureWave(c, w.wb.cap, ns, ws[k], k);
        ws[k].wb.a.adjL = ws[k].wb.a.adjD = ws[k].wb.a.adjP = nullptr;
        ws[k].wb.b.adjL = ws[k].wb.b.adjD = ws[k].wb.b.adjP = nullptr;
        ws[k].wb.neeG = nullptr;
        if (replay) bindAdj(ws[k], k);
        c->store[k].samples.ensure(size_t(ws[k].wb.cap) * 12);
    }
    for (int k = 0; k < nSets; ++k) {
        // sized by the set's own capacity (the sets grow separately), which indexes them
        WaveStore& sk = c->store[k];
        if (anyAov) sk.aov.ensure(size_t(ws[k].wb.cap) * 24);
        if (split) sk.rec.ensure(size_t(kShadeRec) * size_t(ws[k].wb.cap) * 16);
        // the set's job table (its own host copy, so that no upload depends on when the copy of the
        // host vector completes): the denoiser feature samples of its waves
        std::vector<DevJob> hs = hj;
        for (auto& j : hs)
            if (j.lay.aovAlbedo) j.lay.aovSamples = sk.aov.as<float>();
        sk.jobs.upload(hs, st);
        CUDA_CHECK(cudaStreamSynchronize(st));
    }
    c->chunksBuf.upload(chunks, st);
    c->wavesBuf.upload(waves, st);
    // wave indices: [0] the wave being folded, [1] the fold's finished-block count, [2 + 2s] the wave
    // whose bounces buffer set s runs (several waves in flight)
    c->curWave.ensure(sizeof(int) * (2 + 2 * kMaxWaveSets));
    {
        int init[2 + 2 * kMaxWaveSets] = {};
        for (int k = 0; k < kMaxWaveSets; ++k) init[2 + 2 * k] = k;
        CUDA_CHECK(cudaMemcpyAsync(c->curWave.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    }
    const WaveChunk* dch = c->chunksBuf.as<WaveChunk>();
    const WaveDesc* dwv = c->wavesBuf.as<WaveDesc>();
    int* dcur = c->curWave.as<int>();
    DevStats* dstats = c->stats.as<DevStats>();
    CUDA_CHECK(cudaMemsetAsync(dstats, 0, sizeof(DevStats), st));
    int maxFold = 0;
    for (auto& wd : waves) maxFold = std::max(maxFold, wd.foldThreads);

    // One wave of buffer set `set`: camera, then per bounce closest hit / shade / shadow rays on
    // stream `rs`, then (fold) the film fold.  A bounce's shadow rays only clear the next-event slots
    // that the next bounce's shade reads, so they are traced on the set's side stream beside the
    // next bounce's closest hits and shade order (each persistent traversal kernel's tail is filled
    // by the other's blocks), and the next shade waits for them.  Kernel timing (profiling) keeps
    // every launch on the one stream.  camWave: the wave index the camera (and the pyramid) read.
    const bool overlap = !c->profiling;
    long long launches = 0;  // kernels issued (in graph mode: the nodes of one wave)
    auto issueWave = [&](int set, cudaStream_t rs, int items, bool allowEarlyExit, bool fold, int* camWave) {
        const WaveBuffers& wb = ws[set].wb;
        WaveStore& sk = c->store[set];
        const DevJob* dj = sk.jobs.as<DevJob>();
        float* samples = sk.samples.as<float>();
        launches += fold ? 2 : 1;  // camera and film fold
        int* cnt = wb.counters;
        CUDA_CHECK(cudaMemsetAsync(cnt, 0, sizeof(int) * kNumCounters, rs));
        {
            KTimer kt(c, 0);
            launch_camera(dj, dch, dwv, camWave, wb.a, cnt + kCntQueue + 1, items, rs);
        }
        PathBuf A = wb.a, B = wb.b;
        int maxItems = items;
        float4* curNee = wb.nee;  // the next-event slots the current bounce writes
        for (int d = 1; d <= maxDepth; ++d) {
            {
                KTimer kt(c, 1);
                launch_trace_closest(traceRun, dj, A.job, A.ro, A.rd, cnt + kCntQueue + d, cnt + kCntWork + 2 * d, wb.hits, dstats, rs);
            }
            {
                KTimer kt(c, 2);
                PathBuf Ao = A;
                if (split) Ao.rec = sk.rec.as<float4>();
                if (c->shadeOrder) {
                    launch_partition(A.depth, wb.hits, cnt + kCntQueue + d, wb.order, cnt + kCntPart + 2 * d, maxItems, rs);
                    Ao.order = wb.order;
                }
                // next-event slots: read the buffer the previous bounce wrote, write the other
                const size_t neeHalf = size_t(wb.cap) * size_t(sk.neeSlots);
                float4* neeOut = wb.nee + (d & 1) * neeHalf;
                Ao.neeIn = wb.nee + ((d + 1) & 1) * neeHalf;
                float4* neeGOut = nullptr;
                if (wb.neeG) {
                    const size_t gHalf = size_t(wb.cap) * 3 * 2 * size_t(ns);
                    neeGOut = wb.neeG + (d & 1) * gHalf;
                    Ao.neeGIn = wb.neeG + ((d + 1) & 1) * gHalf;
                }
                float4* pyrGOut = nullptr;
                if (pyramid) {
                    const size_t pHalf = size_t(wb.cap) * 2 * size_t(ns);
                    pyrGOut = c->pyrG.as<float4>() + (d & 1) * pHalf;
                    Ao.pyrGIn = c->pyrG.as<float4>() + ((d + 1) & 1) * pHalf;
                }
                curNee = neeOut;
                // From the third bounce on the queue is a fraction of the wave, and a grid of the whole
                // wave capacity is mostly blocks that find nothing to do; the shade kernels loop over the
                // queue, so their grid is capped at 16 blocks per SM there (Cornell boxes 2.6% faster,
                // the 1M-triangle scene unchanged).
                const int shadeItems = d >= 3 ? std::min(maxItems, c->numSMs * 16 * 128) : maxItems;
                // the previous bounce's shadow rays have cleared the slots this shade reads
                if (overlap && d > 1) CUDA_CHECK(cudaStreamWaitEvent(rs, sk.evShadow, 0));
                if (pyramid)
                    launch_shade_pyramid(ns, dj, Ao, B, wb.hits, neeOut, wb.cap, wb.shRo, wb.shRd, wb.shTgt, wb.shJob, cnt + kCntQueue + d,
                                         cnt + kCntQueue + d + 1, cnt + kCntShadow + d, samples, dstats, PyrArgs{dch, dwv, camWave, pyrGOut}, maxItems, rs);
                else
                    launch_shade(ns, replay, generic, c->shadeBlocks, dj, Ao, B, wb.hits, neeOut, neeGOut, wb.cap, wb.shRo, wb.shRd, wb.shTgt, wb.shJob,
                                 cnt + kCntQueue + d, cnt + kCntQueue + d + 1, cnt + kCntShadow + d, samples, dstats, shadeItems, rs);
            }
            {
                KTimer kt(c, 3);
                cudaStream_t ss = rs;
                if (overlap) {
                    CUDA_CHECK(cudaEventRecord(sk.evShade, rs));
                    CUDA_CHECK(cudaStreamWaitEvent(sk.side, sk.evShade, 0));
                    ss = sk.side;
                }
                launch_trace_shadow(traceRun, dj, wb.shJob, wb.shRo, wb.shRd, wb.shTgt, cnt + kCntShadow + d, cnt + kCntWork + 2 * d + 1, curNee, dstats, ss);
                if (overlap) CUDA_CHECK(cudaEventRecord(sk.evShadow, sk.side));
            }
            launches += (c->shadeOrder ? 4 : 3) + (split ? 1 : 0);  // closest hit, shade order, shade (one or two), shadow rays
            std::swap(A, B);
            if (allowEarlyExit && d >= 6 && d < maxDepth) {
                // stop early once the queue is empty (long MaxDepth with Russian roulette)
                CUDA_CHECK(cudaMemcpyAsync(c->pinnedCount, cnt + kCntQueue + d + 1, sizeof(int), cudaMemcpyDeviceToHost, rs));
                CUDA_CHECK(cudaStreamSynchronize(rs));
                if (*c->pinnedCount == 0) break;
                maxItems = *c->pinnedCount;
            }
        }
        if (overlap) CUDA_CHECK(cudaStreamWaitEvent(rs, sk.evShadow, 0));  // the last bounce's shadow rays
        if (fold) {
            KTimer kt(c, 4);
            launch_film_fold(dj, dch, dwv, dcur, (replay || paths) ? nullptr : samples, dstats, maxFold, 1, rs);
        } else {
            launch_wave_advance(camWave, nSets, rs);  // this set's next wave
            ++launches;
        }
    };

    CUDA_CHECK(cudaEventRecord(c->ev0, st));
    auto t0 = std::chrono::steady_clock::now();
    int wavesDone = 0;
    if (multiSets) {
        // one graph per buffer set: camera, the bounces and the advance of the set's wave index; the
        // folds are plain launches on the context's stream, in wave order, each after its wave's
        // bounces (evDone) and before the set's next wave reuses the estimates (evFolded)
        // the graphs and their executables, released on every way out
        struct Graphs {
            cudaGraph_t g[kMaxWaveSets] = {};
            cudaGraphExec_t e[kMaxWaveSets] = {};
            ~Graphs() {
                for (int k = 0; k < kMaxWaveSets; ++k) {
                    if (e[k]) cudaGraphExecDestroy(e[k]);
                    if (g[k]) cudaGraphDestroy(g[k]);
                }
            }
        } gr;
        long long perWave = 0;
        for (int k = 0; k < nSets; ++k) {
            cudaStream_t rs = c->store[k].run;
            launches = 0;
            CUDA_CHECK(cudaStreamBeginCapture(rs, cudaStreamCaptureModeThreadLocal));
            try {
                issueWave(k, rs, w.wb.cap, false, false, dcur + 2 + 2 * k);
            } catch (...) {
                cudaStreamEndCapture(rs, &gr.g[k]);
                throw;
            }
            CUDA_CHECK(cudaStreamEndCapture(rs, &gr.g[k]));
            CUDA_CHECK(cudaGraphInstantiate(&gr.e[k], gr.g[k], 0));
            perWave = launches;
        }
        // the sets' streams start after the context stream's uploads and resets
        CUDA_CHECK(cudaEventRecord(c->evStart, st));
        for (int k = 0; k < nSets; ++k) CUDA_CHECK(cudaStreamWaitEvent(c->store[k].run, c->evStart, 0));
        for (size_t k = 0; k < waves.size(); ++k) {
            const int set = int(k % size_t(nSets));
            WaveStore& sk = c->store[set];
            if (k >= size_t(nSets)) CUDA_CHECK(cudaStreamWaitEvent(sk.run, sk.evFolded, 0));
            CUDA_CHECK(cudaGraphLaunch(gr.e[set], sk.run));
            CUDA_CHECK(cudaEventRecord(sk.evDone, sk.run));
            CUDA_CHECK(cudaStreamWaitEvent(st, sk.evDone, 0));
            launch_film_fold(sk.jobs.as<DevJob>(), dch, dwv, dcur, replay ? nullptr : sk.samples.as<float>(), dstats, maxFold, 1, st);
            CUDA_CHECK(cudaEventRecord(sk.evFolded, st));
        }
        launches = (perWave + 1) * (long long)waves.size();
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaStreamSynchronize(st));
        wavesDone = int(waves.size());
    } else if (useGraph) {
        // capture one wave (fixed grid sizes; wave parameters are read from device memory)
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            issueWave(0, st, w.wb.cap, false, true, dcur);
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
            issueWave(0, st, waves[k].items, true, true, dcur);
            CUDA_CHECK(cudaGetLastError());
            if (c->profiling) {
                std::vector<int> hc(kNumCounters);
                CUDA_CHECK(cudaMemcpyAsync(hc.data(), w.wb.counters, sizeof(int) * kNumCounters, cudaMemcpyDeviceToHost, st));
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
            const unsigned long long key = ~hs.nanKey[k];
            out->nanPixel[prev + k] = int(uint32_t(key & 0xFFFFFFFFull));
            out->nanIteration[prev + k] = int(uint32_t(key >> 32));
        }
        out->numNanOrInf += hs.nanCount;
        out->numMaterialEval += hs.matEvalPdf;
        out->numMaterialPdf += hs.matEvalPdf;
        out->numMaterialSample += hs.matSample;
    }
}


size_t texPoolFloats(const sst_scene* s) {
    size_t n = 0;
    for (auto& t : s->textures) n += t.data.size();
    return n;
}

// Validates the jobs of a batch and fills the renderer's job list.  Films given in host memory
// are staged in device buffers (`staged`); with fromZero every film starts black.
void batchJobs(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, std::vector<JobIn>& in, std::vector<std::unique_ptr<DevBuf>>& staged,
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
void batchFilmsOut(sst_ctx* ctx, const SstRenderJob* jobs, int numJobs, const std::vector<JobIn>& in) {
    for (int j = 0; j < numJobs; ++j) {
        if (jobs[j].memory != SST_MEM_DEVICE) {
            size_t filmBytes = size_t(jobs[j].params.width) * jobs[j].params.height * 3 * sizeof(float);
            CUDA_CHECK(cudaMemcpyAsync(jobs[j].film, in[j].dFilm, filmBytes, cudaMemcpyDeviceToHost, ctx->stream));
        }
    }
    CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
}

SstRenderStats emptyStats() {
    SstRenderStats t{};
    for (int k = 0; k < 4; ++k) { t.nanPixel[k] = -1; t.nanIteration[k] = -1; }
    return t;
}

static TraceTuning toTrace(const SstTuning& t) { return TraceTuning{t.traceBlock, t.traceStackShared, t.traceBlocksPerSM, t.traceBvhWidth, t.traceRefillIdle}; }

static void checkTuning(const SstTuning& t) {
    if (!traceTuningValid(toTrace(t)))
        fail(SST_ERR_INVALID_ARGUMENT, "traceBlock must be 64, 128 or 256, traceStackShared 16, 24 or 32, traceBvhWidth 2, 4 or 8, and traceRefillIdle in [1, 32]");
    if (t.waveCapacity != 0 && (t.waveCapacity < 1024 || t.waveCapacity > (1 << 24)))
        fail(SST_ERR_INVALID_ARGUMENT, "waveCapacity must be 0 or in [1024, 2^24]");
    if (t.traceBlocksPerSM < 0 || t.traceBlocksPerSM > 64) fail(SST_ERR_INVALID_ARGUMENT, "traceBlocksPerSM must be in [0, 64]");
    if (t.shadeOrder != 0 && t.shadeOrder != 1) fail(SST_ERR_INVALID_ARGUMENT, "shadeOrder must be 0 or 1");
    if (t.shadeSplit != 0 && t.shadeSplit != 1) fail(SST_ERR_INVALID_ARGUMENT, "shadeSplit must be 0 or 1");
    if (!shadeBlocksValid(t.shadeBlocks))
        fail(SST_ERR_INVALID_ARGUMENT, "shadeBlocks must be 8, 10, 12 or 14");
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
    t.shadeSplit = c->shadeSplit;
    return t;
}


extern "C" {

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
            CUDA_CHECK(cudaMemcpyAsync(rgb + 3 * size_t(b0), c->store[0].samples.p, size_t(cnt) * 12, k, c->stream));
            CUDA_CHECK(cudaStreamSynchronize(c->stream));
        }
        local.numIterations = 0;
        if (stats) *stats = local;
    });
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
        c->shadeSplit = t->shadeSplit;
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
        // one candidate: the fastest of three trial renders of `iters` iterations
        auto trial = [&](const SstTuning& t, int iters) {
            c->trace = toTrace(t);
            c->waveCapacity = t.waveCapacity;
            c->shadeBlocks = t.shadeBlocks;
            c->shadeOrder = t.shadeOrder;
            c->shadeSplit = t.shadeSplit;
            double best = 1e300;
            for (int r = 0; r < 3; ++r) {
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
        // after the traversal variant, a candidate replaces the setting so far only when its trial is
        // 2% faster: the trials vary by about that much from run to run, and the defaults are the
        // settings measured fastest on the benchmark scenes
        constexpr double kKeep = 0.98;
        try {
            // traversal variant
            for (int wdt : {2, 4, 8})
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
            // refill threshold of the wide traversals
            if (best.traceBvhWidth != 2)
                for (int ri : {32, 12, 24}) {
                    if (ri == best.traceRefillIdle) continue;
                    SstTuning t = best;
                    t.traceRefillIdle = ri;
                    double ms = trial(t, kIters);
                    if (ms < bestMs * kKeep) { bestMs = ms; best = t; }
                }
            // the shade kernel with GenericMaterials: fused, built for 8, 10, 12 or 14 blocks, or split
            // into two kernels, built for 8 or 14 (the split form's register budget changes which build
            // wins, so the two choices are tried together); a scene without one runs neither
            bool generic = false;
            for (auto& m : s->materials) generic |= m.type == kGeneric;
            if (generic) {
                const SstTuning base = best;
                for (int split : {0, 1})
                    for (int sb : {8, 10, 12, 14}) {
                        if (split && (sb == 10 || sb == 12)) continue;
                        if (sb == base.shadeBlocks && split == base.shadeSplit) continue;
                        SstTuning t = base;
                        t.shadeBlocks = sb;
                        t.shadeSplit = split;
                        double ms = trial(t, kIters);
                        if (ms < bestMs * kKeep) { bestMs = ms; best = t; }
                    }
            }
            // shade order: surface hits first, or queue order
            {
                SstTuning t = best;
                t.shadeOrder = 1 - best.shadeOrder;
                double ms = trial(t, kIters);
                if (ms < bestMs * kKeep) { bestMs = ms; best = t; }
            }

            // resident traversal blocks per SM
            int m = traceMaxBlocksPerSM(toTrace(best));
            for (int bps : {m / 2, (3 * m) / 4}) {
                if (bps < 1 || bps >= m) continue;
                SstTuning t = best;
                t.traceBlocksPerSM = bps;
                double ms = trial(t, kIters);
                if (ms < bestMs * kKeep) { bestMs = ms; best = t; }
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
                if (ms < curMs * kKeep) { curMs = ms; best = t; }
            }
            // the reported time is that of a trial of trialIterations iterations
            bestMs = wcIters == trialIterations ? curMs : trial(best, trialIterations);
        } catch (...) {
            c->trace = toTrace(start);
            c->waveCapacity = start.waveCapacity;
            c->shadeBlocks = start.shadeBlocks;
            c->shadeOrder = start.shadeOrder;
            c->shadeSplit = start.shadeSplit;
            c->profiling = prof;
            throw;
        }
        c->profiling = prof;
        c->trace = toTrace(best);
        c->waveCapacity = best.waveCapacity;
        c->shadeBlocks = best.shadeBlocks;
        c->shadeOrder = best.shadeOrder;
        c->shadeSplit = best.shadeSplit;
        if (chosen) *chosen = best;
        if (bestTrialMs) *bestTrialMs = bestMs;
    });
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

int sst_set_shading_stats(sst_ctx* ctx, int32_t enable) {
    return guarded([&] {
        if (!ctx) fail(SST_ERR_INVALID_ARGUMENT, "NULL context");
        ctx->shadingStats = enable != 0;
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

}  // extern "C"

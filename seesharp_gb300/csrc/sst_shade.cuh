// The shade kernel k_shade (one bounce of EstimateIncidentRadiance for every queued path, with
// queue compaction), shared by the translation units that instantiate its variants:
// sst_kernels.cu (render and adjoint) and sst_pyramid.cu (the technique pyramid).
#pragma once
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include "sst_adjoint.cuh"
#include "sst_device.cuh"

namespace cg = cooperative_groups;

// Minimum resident 128-thread blocks per SM the shade kernel is compiled for (its register
// budget).  The kernel is latency-bound: on GB300, 8 blocks (64 registers, some spilled to L1)
// shade 18% faster than the unconstrained 131-register build on the 1M-triangle scene and are
// the fastest cap on the Cornell box (the adjoint variant's cap is below).
// SST_SHADE_MIN_BLOCKS is the cap of the variant without GenericMaterials (8 is fastest there:
// 10, 12 and 16 blocks shade the Cornell box 15-42% slower).  The forward variant with
// GenericMaterials is compiled twice, and the launch tuning picks one per context: for
// SST_SHADE_GEN_MIN_BLOCKS (8, 64 registers; the default) and for SST_SHADE_GEN_DENSE_BLOCKS (14,
// 32 registers).  The dense build shades the 1M-triangle sphere field 6% faster; on the Cornell box
// with generic boxes it renders 19% slower, because its spills outgrow the caches.
#ifndef SST_SHADE_MIN_BLOCKS
#define SST_SHADE_MIN_BLOCKS 8
#endif
#ifndef SST_SHADE_GEN_MIN_BLOCKS
#define SST_SHADE_GEN_MIN_BLOCKS 8
#endif
#ifndef SST_SHADE_GEN_DENSE_BLOCKS
#define SST_SHADE_GEN_DENSE_BLOCKS 14
#endif
// The adjoint replay's shade kernel: 8 resident blocks (64 registers).  With the approximate
// division of the shading units it replays the differentiable Cornell box 13% and the large
// combined job 10% faster than the 16-block build (32 registers) that was faster before.
#ifndef SST_SHADE_ADJ_MIN_BLOCKS
#define SST_SHADE_ADJ_MIN_BLOCKS 8
#endif

namespace sst {

// =============================================================================================
// K5 + K7 + K8: one bounce of the estimator for every queued path.
// =============================================================================================
SST_D void splat(float* samples, uint32_t item, float3 v) {
    float* f = samples + 3 * (size_t)item;
    f[0] = v.x; f[1] = v.y; f[2] = v.z;
}

// PathTracerBase.RegisterSample (Integrators/PathTracer.cs:73-82) into the technique pyramids:
// the sample's contribution divided by TotalSpp is added to the image of its technique in the raw
// pyramid, and times its MIS weight in the weighted one (TechPyramid.Add, AtomicAdd per pixel).
SST_D void pyrAdd(const DevJob& jb, int pixel, int depth, bool nextEvent, float3 weight, float mis) {
    const DevLayers& lay = jb.lay;
    if (!lay.pyr) return;
    const float spp = (float)lay.pyrSpp;
    const float3 w = mk(weight.x / spp, weight.y / spp, weight.z / spp);
    const size_t P = (size_t)jb.cfg.W * jb.cfg.H;
    const int L = 2 * (depth - 1) + (nextEvent ? 1 : 0);
    float* a = lay.pyr + ((size_t)L * P + (size_t)pixel) * 3;
    float* b = lay.pyr + ((size_t)(2 * jb.cfg.maxDepth + L) * P + (size_t)pixel) * 3;
    atomicAdd(a, w.x);
    atomicAdd(a + 1, w.y);
    atomicAdd(a + 2, w.z);
    const float3 m = w * mis;
    atomicAdd(b, m.x);
    atomicAdd(b + 1, m.y);
    atomicAdd(b + 2, m.z);
}

// Queue `cnt` items per calling lane group and return this lane's slot.
SST_D int aggAppend(int* counter) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
    return g.shfl(base, 0) + (int)g.thread_rank();
}

// ADJ = true: path-replay adjoint.  The same decisions as the forward pass (same code, same
// RNG stream); in addition the pass accumulates parameter gradients with detached sampling:
//   - at an emitter hit: d/d radiance of prefix * mis * Le;
//   - at each NEE sample: d/d(material parameters) and d/d radiance of the contribution, applied
//     once the shadow ray has found the sample visible (payload in neeG);
//   - for the sampled BSDF factor f_k: d ln f_k / d(theta) times the radiance collected after it,
//     which is the forward pass's path radiance minus what has been collected up to vertex k
//     (applied at the next vertex, after that vertex has resolved vertex k's NEE).
// Every term is weighted by dLoss/dSample of the path's pixel.
// GEN = false: a wave without GenericMaterials (the generic code is not compiled in, which keeps
// the kernel's instruction footprint small).
// PYR = true: the technique pyramids (PathTracer.RenderTechniquePyramid) are filled as well.
// MINB: the resident blocks per SM the variant is compiled for.
// SPLIT = true (forward only): the first of two kernels.  It stops before BSDF sampling and leaves
// the shading point and the path's updated state in A.rec (kShadeRec float4 per queued path, see
// k_shade_sample); k_shade_sample then samples the direction and compacts the queue.  Each half holds
// less state and less code than the fused kernel.
template <int NS, bool ADJ, bool GEN, bool PYR = false,
          int MINB = (ADJ ? SST_SHADE_ADJ_MIN_BLOCKS : (GEN ? SST_SHADE_GEN_MIN_BLOCKS : SST_SHADE_MIN_BLOCKS)), bool SPLIT = false>
__global__ void __launch_bounds__(128, MINB) k_shade(const DevJob* __restrict__ jobs, PathBuf A, PathBuf B,
                                                                   const float4* __restrict__ hits, float4* nee, float4* neeG, int cap,
                                                                   float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn,
                                                                   int* nOut, int* nSh, float* samples, DevStats* stats, PyrArgs pyrA) {
    const int n = *nIn;
    // a grid-stride loop over whole blocks of the queue: a late bounce's launch caps its grid below
    // the wave capacity (every thread of a block takes the same turns, so the warp-wide ballots below
    // see whole warps)
    for (int blk = blockIdx.x * blockDim.x; blk < n; blk += gridDim.x * blockDim.x) {

    const int t = blk + threadIdx.x;
    const bool valid = t < n;
    const int i = (valid && A.order) ? A.order[t] : t;  // the queued path this thread shades

    bool cont = false;
    uint32_t job = 0;
    uint32_t outDepth = 0;
    float3 prefix = mk(1, 1, 1), radiance = mk(0, 0, 0);
    float prevPdfOut = 0.f;
    float3 hitPos = mk(0, 0, 0), nRo = mk(0, 0, 0), nRd = mk(0, 0, 0);
    float nTmax = CUDART_INF_F;
    uint32_t pix = 0;
    Rng rng{0};
    uint32_t pend = 0;  // next-event slots queued at this vertex (written at once, at this path's queue index)
    int queries = 0;
    int nEvalPdf = 0, nSample = 0;  // ShadingStats (counted only with cfg.shadingStats)
    bool sampled = false;           // SPLIT: the path goes on to k_shade_sample
    // adjoint state
    float3 adjLt = mk(0, 0, 0), adjDl = mk(0, 0, 0);
    int vBaseTgt = -1, vRoughTgt = -1;   // targets of this vertex (for the factor left pending)
    float4 fP[3] = {};                   // d ln f_c / d theta of this vertex's sampled BSDF factor
    bool factorPending = false;
    int pyrPixel = 0;

    if (valid) {
        job = A.job[i];
        const DevScene& sc = jobs[job].sc;
        const PTConfig& cfg = jobs[job].cfg;
        pix = A.pix[i];
        rng.s = A.rng[i];
        uint32_t dw = A.depth[i];
        float4 pw = A.pw[i];
        float4 rad4 = A.rad[i];
        prefix = f3(pw);
        float prevPdf = pw.w;
        radiance = f3(rad4);
        if (PYR) {
            // the wave item's pixel (as k_camera maps it)
            const WaveDesc wd = pyrA.waves[*pyrA.curWave];
            const WaveChunk& ck = pyrA.chunks[findChunk(pyrA.chunks, wd.chunkBegin, wd.chunkEnd, (int)pix)];
            pyrPixel = ck.pixStart + ((int)pix - ck.itemOffset) % ck.pixCount;
        }
        const DevAdj& adj = jobs[job].adj;
        // resolve the NEE of the previous bounce (PathTracer.cs:363) in slot order; the previous bounce
        // wrote them at the path's index in its own queue, which the compaction kept in neeFrom
        uint32_t pm = (dw >> kNeeShift) & 0xFFu;
        const size_t nf = pm ? (size_t)A.neeFrom[i] : 0;
        if (ADJ) {
            float4 l4 = A.adjL[i], d4 = A.adjD[i];
            adjLt = f3(l4);
            adjDl = f3(d4);
#pragma unroll
            for (int k = 0; k < 2 * NS; ++k) {
                if (!(pm & (1u << k))) continue;
                size_t slot = (size_t)k * cap + nf;
                float4 nv = A.neeIn[slot];
                if (nv.w == 0.0f) continue;  // occluded
                radiance = radiance + f3(nv);
                float4 g0 = A.neeGIn[3 * slot], g1 = A.neeGIn[3 * slot + 1], g2 = A.neeGIn[3 * slot + 2];
                addBaseGrad(adj, __float_as_int(g0.x), g0.y, g0.z, g0.w);
                addRoughGrad(adj, __float_as_int(g1.x), g1.y);
                addEmitterGrad(adj, __float_as_int(g1.z), f3(g2));
            }
            // the sampled-BSDF factor of the previous vertex: d ln f * radiance collected after it
            if (dw & kAdjFactorFlag) {
                float3 fut = adjLt - radiance;
                float3 w3 = adjDl * fut;
                float4 p0 = A.adjP[3 * (size_t)i], p1 = A.adjP[3 * (size_t)i + 1], p2 = A.adjP[3 * (size_t)i + 2];
                float gb0 = w3.x * p0.x + w3.y * p1.x + w3.z * p2.x;
                float gb1 = w3.x * p0.y + w3.y * p1.y + w3.z * p2.y;
                float gb2 = w3.x * p0.z + w3.y * p1.z + w3.z * p2.z;
                float gr = w3.x * p0.w + w3.y * p1.w + w3.z * p2.w;
                addBaseGrad(adj, __float_as_int(l4.w), gb0, gb1, gb2);
                addRoughGrad(adj, __float_as_int(d4.w), gr);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 2 * NS; ++k) {
                if (!(pm & (1u << k))) continue;
                const float4 nv = A.neeIn[(size_t)k * cap + nf];
                radiance = radiance + f3(nv);
                // a visible next-event sample: the reference evaluates the BSDF and its pdf
                if (cfg.shadingStats && nv.w != 0.0f) ++nEvalPdf;
                if (PYR && nv.w != 0.0f) {  // visible: the next-event sample of length `depth` counts
                    const float4 pg = A.pyrGIn[(size_t)k * cap + nf];
                    pyrAdd(jobs[job], pyrPixel, (int)(dw & kDepthMask), true, f3(pg), pg.w);
                }
            }
        }
        const uint32_t depth = dw & kDepthMask;
        bool terminate = false;
        if (dw & kDoneFlag) {
            terminate = true;
        } else {
            float4 rd4 = A.rd[i];
            float3 rdir = f3(rd4);
            float4 h = hits[i];
            int ti = __float_as_int(h.w);
            float* aov = (!ADJ && depth == 1) ? jobs[job].lay.aovSamples : nullptr;
            if (aov && ti < 0) {  // no primary hit: nothing is logged this iteration
                float* a6 = aov + 6 * (size_t)pix;
                a6[0] = a6[1] = a6[2] = a6[3] = a6[4] = a6[5] = 0.0f;
            }
            if (ti < 0) {
                // OnBackgroundHit (PathTracer.cs:384-400)
                if ((int)depth >= cfg.minDepth && sc.hasEnv && cfg.enableBsdfDI) {
                    float mis = 1.0f;
                    if (depth > 1) {
                        float pne = envPdf(sc.env, rdir) * (float)cfg.numShadowRays;
                        mis = 1.0f / (1.0f + pne / prevPdf);
                    }
                    const float3 le = envRadiance(sc.env, rdir);
                    radiance = radiance + prefix * mis * le;
                    if (PYR) pyrAdd(jobs[job], pyrPixel, (int)depth, false, le * prefix, mis);
                }
                terminate = true;
            } else {
                // SurfacePoint of the hit (Geometry/SurfacePoint.cs)
                float4 a4 = __ldg(&sc.triv[3 * (size_t)ti]), b4 = __ldg(&sc.triv[3 * (size_t)ti + 1]), c4 = __ldg(&sc.triv[3 * (size_t)ti + 2]);
                float4 fn = __ldg(&sc.triN[ti]);
                int4 aux = __ldg(&sc.triAux[ti]);
                float3 v1 = f3(a4), v2 = f3(b4), v3 = f3(c4);
                float u = h.y, v = h.z;
                Surf s;
                s.pos = baryPos(v1, v2, v3, u, v);
                s.n = f3(fn);
                s.eps = errorOffset(v1, v2, v3, u, v);
                s.mat = aux.x;
                int4 vi = make_int4(0, 0, 0, 0);
                if (aux.w) vi = __ldg(&sc.triVtx[ti]);
                if (aux.w & 1) {
                    float3 n1 = mk(sc.vnrm[3 * vi.x], sc.vnrm[3 * vi.x + 1], sc.vnrm[3 * vi.x + 2]);
                    float3 n2 = mk(sc.vnrm[3 * vi.y], sc.vnrm[3 * vi.y + 1], sc.vnrm[3 * vi.y + 2]);
                    float3 n3 = mk(sc.vnrm[3 * vi.z], sc.vnrm[3 * vi.z + 1], sc.vnrm[3 * vi.z + 2]);
                    s.sn = normalize(u * n2 + v * n3 + (1.0f - u - v) * n1);
                } else {
                    s.sn = s.n;
                }
                if (aux.w & 2) {
                    float w = 1.0f - u - v;
                    s.uv = make_float2(u * sc.vuv[2 * vi.y] + v * sc.vuv[2 * vi.z] + w * sc.vuv[2 * vi.x],
                                       u * sc.vuv[2 * vi.y + 1] + v * sc.vuv[2 * vi.z + 1] + w * sc.vuv[2 * vi.x + 1]);
                } else {
                    s.uv = make_float2(u, v);
                }
                hitPos = s.pos;
                if (aov) {
                    // DenoiseBuffers.LogPrimaryHit (PathTracer.cs:336-339): GetScatterStrength is the base
                    // colour at the hit for both materials (DiffuseMaterial.cs:37-38, GenericMaterial.cs:65)
                    const DevMaterial& mm = sc.mats[s.mat];
                    float3 alb = lookupRgb(sc, mm.baseTex, mm.base, s.uv);
                    float* a6 = aov + 6 * (size_t)pix;
                    a6[0] = alb.x; a6[1] = alb.y; a6[2] = alb.z;
                    a6[3] = s.sn.x; a6[4] = s.sn.y; a6[5] = s.sn.z;
                }
                // SurfaceShader / ShadingContext (PathTracer.cs:334)
                Ctx c;
                c.f.n = s.sn;
                basis(c.f.n, c.f.t, c.f.b);
                c.outW = -rdir;
                c.out = c.f.toLocal(c.outW);
                c.faceN = s.n;
                c.uv = s.uv;
                const DevMaterial& m = sc.mats[s.mat];
                Lp lp = {};
                float3 diffBase = mk(0, 0, 0);
                if (GEN && m.type == kGeneric) lp = localParams(sc, m, s.uv);
                else diffBase = lookupRgb(sc, m.baseTex, m.base, s.uv);

                // OnLightHit (PathTracer.cs:402-421)
                int emIdx = __float_as_int(fn.w);
                if (emIdx >= 0 && (int)depth >= cfg.minDepth) {
                    const DevEmitter& em = sc.emitters[emIdx];
                    float mis = 1.0f;
                    if (depth > 1) {
                        float3 prevPos = f3(A.prev[i]);
                        float jac = areaToSolidAngle(prevPos, s.pos, s.n);
                        float pne = em.faceN.w / (float)sc.nEmitters * (float)cfg.numShadowRays / jac;
                        mis = 1.0f / (pne / prevPdf + 1.0f);
                        if (!cfg.enableBsdfDI) mis = 0.0f;
                    }
                    const float3 le = emitted(em, s.sn, -rdir);
                    radiance = radiance + prefix * mis * le;
                    if (PYR) pyrAdd(jobs[job], pyrPixel, (int)depth, false, le * prefix, mis);
                    if (ADJ) addEmitterGrad(adj, emIdx, adjDl * prefix * (mis * emittedScale(em, s.sn, -rdir)));
                }
                // adjoint: parameter values and gradient targets of this shading point
                float3 baseV = mk(0, 0, 0);
                float roughV = 0.0f;
                if (ADJ) {
                    baseV = lookupRgb(sc, m.baseTex, m.base, s.uv);
                    roughV = m.type == kGeneric ? lookupMono(sc, m.roughTex, m.rough, s.uv) : 1.0f;
                    gradTargets(sc, s.mat, s.uv, vBaseTgt, vRoughTgt);
                }

                // Russian roulette (PathTracer.cs:277-282, :352-354)
                float surv = depth > 4 ? clampf(avg3(prefix), 0.05f, 0.95f) : 1.0f;
                if (rng.nextFloat() > surv || (int)depth == cfg.maxDepth) {
                    terminate = true;
                } else {
                    // Next event estimation (PathTracer.cs:357-364, :423-501)
                    float3 neeScale = prefix;  // contributions are stored as prefix * c / surv
                    if ((int)depth + 1 >= cfg.minDepth) {
#pragma unroll
                        for (int sIt = 0; sIt < NS; ++sIt) {
                            if (sIt >= cfg.numShadowRays) break;
                            if (sc.hasEnv) {
                                ++queries;
                                float e1 = rng.nextFloat(), e2 = rng.nextFloat();
                                float3 ed; float epdf; float3 ew;
                                envSample(sc.env, e1, e2, ed, epdf, ew);
                                float pb;
                                float3 bc = evalWithCos<GEN>(sc, m, lp, diffBase, c, ed, pb);
                                float3 val = mk(0, 0, 0);
                                bool use = false;
                                if (!(pb == 0.0f || epdf == 0.0f)) {
                                    float mis = cfg.enableBsdfDI ? 1.0f / (1.0f + pb / (epdf * (float)cfg.numShadowRays)) : 1.0f;
                                    float3 contrib = ew * bc / (float)cfg.numShadowRays;
                                    val = neeScale * (mis * contrib) / surv;
                                    if (!isBlack(val)) {
                                        use = true;
                                        const size_t sl = (size_t)(2 * sIt) * cap + i;
                                        if (ADJ) {
                                            // d val / d(material): prefix * mis * weight / ns / surv * |cos| * df
                                            float3 coef = adjDl * neeScale * (mis * ew / (float)cfg.numShadowRays) / surv * fabsf(c.f.toLocal(ed).z);
                                            Dl3 df = bsdfDeriv(m, baseV, roughV, c, ed);
                                            neeG[3 * sl] = make_float4(__int_as_float(vBaseTgt), coef.x * df.x.d[0] + coef.y * df.y.d[0] + coef.z * df.z.d[0],
                                                                       coef.x * df.x.d[1] + coef.y * df.y.d[1] + coef.z * df.z.d[1],
                                                                       coef.x * df.x.d[2] + coef.y * df.y.d[2] + coef.z * df.z.d[2]);
                                            neeG[3 * sl + 1] = make_float4(__int_as_float(vRoughTgt), coef.x * df.x.d[3] + coef.y * df.y.d[3] + coef.z * df.z.d[3],
                                                                           __int_as_float(-1), 0.f);
                                            neeG[3 * sl + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
                                        }
                                        if (PYR) {
                                            const float3 pc = contrib * neeScale;
                                            pyrA.pyrG[sl] = make_float4(pc.x, pc.y, pc.z, mis);
                                        }
                                    }
                                }
                                // LeavesScene (PathTracer.cs:428): traced for a contributing sample, and for
                                // every sample while shading statistics need its visibility (value zero)
                                if (use || (!ADJ && cfg.shadingStats)) {
                                    const int k = 2 * sIt;
                                    const size_t sl = (size_t)k * cap + i;
                                    if (PYR && !use) pyrA.pyrG[sl] = make_float4(0.f, 0.f, 0.f, 0.f);
                                    int q = aggAppend(nSh);
                                    shJob[q] = job;
                                    float3 o = offsetPoint(s.pos, s.n, s.eps, ed);
                                    shRo[q] = make_float4(o.x, o.y, o.z, 0.0f);
                                    shRd[q] = make_float4(ed.x, ed.y, ed.z, CUDART_INF_F);
                                    shTgt[q] = (int)sl;
                                    nee[sl] = make_float4(val.x, val.y, val.z, 1.f);
                                    pend |= 1u << k;
                                }
                            }
                            if (sc.nEmitters > 0) {
                                ++queries;
                                int idx = (int)rng.nextInt((uint32_t)sc.nEmitters);
                                const DevEmitter& em = sc.emitters[idx];
                                float selProb = 1.0f / (float)sc.nEmitters;
                                float l1 = rng.nextFloat(), l2 = rng.nextFloat();
                                float2 bar = toUniformTriangle(l1, l2);
                                float3 e1 = f3(em.v1), e2 = f3(em.v2), e3 = f3(em.v3);
                                float3 lpPos = baryPos(e1, e2, e3, bar.x, bar.y);
                                float3 lpN = f3(em.faceN);
                                float lpEps = errorOffset(e1, e2, e3, bar.x, bar.y);
                                float3 lpSn = lpN;
                                if (em.n1.w != 0.0f)
                                    lpSn = normalize(bar.x * f3(em.n2) + bar.y * f3(em.n3) + (1.0f - bar.x - bar.y) * f3(em.n1));
                                float3 l2s = normalize(s.pos - lpPos);
                                float3 emis = emitted(em, lpSn, l2s);
                                float jac = areaToSolidAngle(s.pos, lpPos, lpN);
                                float pb;
                                float3 bc = evalWithCos<GEN>(sc, m, lp, diffBase, c, -l2s, pb);
                                float lpPdf = em.faceN.w;
                                float pne = lpPdf * selProb * (float)cfg.numShadowRays;
                                float pbA = pb * jac;
                                float3 val = mk(0, 0, 0);
                                bool use = false;
                                if (jac != 0.0f) {
                                    float ratio = pbA / pne;
                                    float mis = cfg.enableBsdfDI ? 1.0f / (ratio + 1.0f) : 1.0f;
                                    float pdf = lpPdf / jac * selProb * (float)cfg.numShadowRays;
                                    float3 contrib = emis / pdf * bc;
                                    val = neeScale * (mis * contrib) / surv;
                                    if (!isBlack(val)) {
                                        use = true;
                                        const size_t sl = (size_t)(2 * sIt + 1) * cap + i;
                                        if (ADJ) {
                                            float3 coef = adjDl * neeScale * (mis * emis / pdf) / surv * fabsf(c.f.toLocal(-l2s).z);
                                            Dl3 df = bsdfDeriv(m, baseV, roughV, c, -l2s);
                                            float3 ge = adjDl * neeScale * (mis * emittedScale(em, lpSn, l2s) / pdf) * bc / surv;
                                            neeG[3 * sl] = make_float4(__int_as_float(vBaseTgt), coef.x * df.x.d[0] + coef.y * df.y.d[0] + coef.z * df.z.d[0],
                                                                       coef.x * df.x.d[1] + coef.y * df.y.d[1] + coef.z * df.z.d[1],
                                                                       coef.x * df.x.d[2] + coef.y * df.y.d[2] + coef.z * df.z.d[2]);
                                            neeG[3 * sl + 1] = make_float4(__int_as_float(vRoughTgt), coef.x * df.x.d[3] + coef.y * df.y.d[3] + coef.z * df.z.d[3],
                                                                           __int_as_float(idx), 0.f);
                                            neeG[3 * sl + 2] = make_float4(ge.x, ge.y, ge.z, 0.f);
                                        }
                                        if (PYR) {
                                            const float3 pc = contrib * neeScale;
                                            pyrA.pyrG[sl] = make_float4(pc.x, pc.y, pc.z, mis);
                                        }
                                    }
                                }
                                // IsOccluded (PathTracer.cs:467): traced for a contributing sample, and for every
                                // sample while shading statistics need its visibility (value zero)
                                if (use || (!ADJ && cfg.shadingStats)) {
                                    const int k = 2 * sIt + 1;
                                    const size_t sl = (size_t)k * cap + i;
                                    if (PYR && !use) pyrA.pyrG[sl] = make_float4(0.f, 0.f, 0.f, 0.f);
                                    int q = aggAppend(nSh);
                                    shJob[q] = job;
                                    float3 dd = lpPos - s.pos;
                                    float3 o = offsetPoint(s.pos, s.n, s.eps, dd);
                                    float3 e = offsetPoint(lpPos, lpN, lpEps, -dd);
                                    float3 sd = e - o;
                                    shRo[q] = make_float4(o.x, o.y, o.z, 0.0f);
                                    shRd[q] = make_float4(sd.x, sd.y, sd.z, 1.0f - 1e-5f);
                                    shTgt[q] = (int)sl;
                                    nee[sl] = make_float4(val.x, val.y, val.z, 1.f);
                                    pend |= 1u << k;
                                }
                            }
                        }
                    }
                    if constexpr (SPLIT) {
                        // hand the shading point and the path's state to k_shade_sample
                        const size_t cp = (size_t)cap;
                        A.rec[i] = make_float4(s.pos.x, s.pos.y, s.pos.z, s.eps);
                        A.rec[cp + i] = make_float4(s.n.x, s.n.y, s.n.z, __int_as_float(s.mat));
                        A.rec[2 * cp + i] = make_float4(s.sn.x, s.sn.y, s.sn.z, s.uv.x);
                        A.rec[3 * cp + i] = make_float4(s.uv.y, surv, __uint_as_float(rng.s), __uint_as_float(kRecSample | pend));
                        A.rec[4 * cp + i] = make_float4(radiance.x, radiance.y, radiance.z, 0.f);
                        sampled = true;
                    } else {
                    // SampleDirection (PathTracer.cs:526-530)
                    float uc = rng.nextFloat();
                    float u1 = rng.nextFloat(), u2 = rng.nextFloat();
                    float3 dirW; float bpdf = 0.f; float3 bw = mk(0, 0, 0);
                    bool ok = sampleMaterial<GEN>(sc, m, lp, diffBase, c, uc, u1, u2, dirW, bpdf, bw);
                    if (!ADJ && cfg.shadingStats) {
                        // Material.Sample; DiffuseMaterial.Sample also evaluates and computes the pdf
                        ++nSample;
                        if (!(GEN && m.type == kGeneric)) ++nEvalPdf;
                    }
                    if (!ok || bpdf == 0.0f || isBlack(bw)) {
                        // a finished path with queued NEE keeps its next length for the pyramid
                        if (pend) { cont = true; outDepth = kDoneFlag | (PYR ? depth + 1 : 0u); }
                        else terminate = true;
                    } else {
                        cont = true;
                        if (ADJ) {
                            Dl3 df = bsdfDeriv(m, baseV, roughV, c, dirW);
                            float ix = df.x.v != 0.0f ? 1.0f / df.x.v : 0.0f;
                            float iy = df.y.v != 0.0f ? 1.0f / df.y.v : 0.0f;
                            float iz = df.z.v != 0.0f ? 1.0f / df.z.v : 0.0f;
                            fP[0] = make_float4(df.x.d[0] * ix, df.x.d[1] * ix, df.x.d[2] * ix, df.x.d[3] * ix);
                            fP[1] = make_float4(df.y.d[0] * iy, df.y.d[1] * iy, df.y.d[2] * iy, df.y.d[3] * iy);
                            fP[2] = make_float4(df.z.d[0] * iz, df.z.d[1] * iz, df.z.d[2] * iz, df.z.d[3] * iz);
                            factorPending = true;
                        }
                        prefix = prefix * (bw / surv);  // PathTracer.cs:372-378
                        prevPdfOut = bpdf * surv;
                        outDepth = depth + 1;
                        nRo = offsetPoint(s.pos, s.n, s.eps, dirW);
                        nRd = dirW;
                    }
                    outDepth |= pend << kNeeShift;
                    }  // !SPLIT
                }
            }
        }
        if (terminate && !ADJ) splat(samples, pix, radiance);
        if (!cont) pend = 0;
        // the first kernel of the split form: a path that does not go on to sampling is finished
        // here (terminated, or a finished path whose queued next-event samples were resolved)
        if (SPLIT && !sampled) A.rec[3 * (size_t)cap + i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // shadow-query statistics (RayTracerStats.NumShadowRays semantics)
    int totq = __reduce_add_sync(0xffffffffu, queries);
    if ((threadIdx.x & 31) == 0 && totq) atomicAdd(&stats->shadowRays, (unsigned long long)totq);
    if (!ADJ) {
        const int te = __reduce_add_sync(0xffffffffu, nEvalPdf), ts = __reduce_add_sync(0xffffffffu, nSample);
        if ((threadIdx.x & 31) == 0 && te) atomicAdd(&stats->matEvalPdf, (unsigned long long)te);
        if ((threadIdx.x & 31) == 0 && ts) atomicAdd(&stats->matSample, (unsigned long long)ts);
    }
    if constexpr (SPLIT) continue;  // k_shade_sample compacts the queue

    // K7: warp ballot / popc compaction into the next queue
    unsigned m = __ballot_sync(0xffffffffu, cont);
    if (m == 0) continue;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(nOut, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!cont) continue;
    int j = base + __popc(m & ((1u << lane) - 1u));
    B.job[j] = job;
    B.pix[j] = pix;
    B.rng[j] = rng.s;
    B.depth[j] = outDepth;
    B.pw[j] = make_float4(prefix.x, prefix.y, prefix.z, prevPdfOut);
    B.rad[j] = make_float4(radiance.x, radiance.y, radiance.z, 0.f);
    B.prev[j] = make_float4(hitPos.x, hitPos.y, hitPos.z, 0.f);
    B.ro[j] = make_float4(nRo.x, nRo.y, nRo.z, 0.f);
    B.rd[j] = make_float4(nRd.x, nRd.y, nRd.z, (outDepth & kDoneFlag) ? -1.0f : nTmax);
    if (ADJ) {
        B.depth[j] = outDepth | (factorPending ? kAdjFactorFlag : 0u);
        B.adjL[j] = make_float4(adjLt.x, adjLt.y, adjLt.z, __int_as_float(vBaseTgt));
        B.adjD[j] = make_float4(adjDl.x, adjDl.y, adjDl.z, __int_as_float(vRoughTgt));
        B.adjP[3 * (size_t)j] = fP[0];
        B.adjP[3 * (size_t)j + 1] = fP[1];
        B.adjP[3 * (size_t)j + 2] = fP[2];
    }
    // the next-event slots of this vertex were written at this path's index in the current queue
    if (pend) B.neeFrom[j] = (uint32_t)i;
    }
}


// The second kernel of the split form (forward only): SampleDirection (PathTracer.cs:526-530) for the
// paths that k_shade<..., SPLIT = true> left in A.rec with kRecSample, then the queue compaction of
// the fused kernel.  The shading context, the GenericMaterial parameters and the RNG state are
// rebuilt from the record by the same arithmetic as in the fused kernel, so the path goes on
// exactly as there.
template <bool GEN, int MINB>
__global__ void __launch_bounds__(128, MINB) k_shade_sample(const DevJob* __restrict__ jobs, PathBuf A, PathBuf B, int cap, const int* nIn,
                                                           int* nOut, float* samples, DevStats* stats) {
    const int n = *nIn;
    // a grid-stride loop over whole blocks of the queue: a late bounce's launch caps its grid below
    // the wave capacity (every thread of a block takes the same turns, so the warp-wide ballots below
    // see whole warps)
    for (int blk = blockIdx.x * blockDim.x; blk < n; blk += gridDim.x * blockDim.x) {

    const int t = blk + threadIdx.x;
    const bool valid = t < n;
    const int i = (valid && A.order) ? A.order[t] : t;
    bool cont = false;
    uint32_t job = 0, pix = 0, outDepth = 0;
    float3 prefix = mk(1, 1, 1), radiance = mk(0, 0, 0), hitPos = mk(0, 0, 0), nRo = mk(0, 0, 0), nRd = mk(0, 0, 0);
    float prevPdfOut = 0.f;
    Rng rng{0};
    uint32_t pend = 0;
    int nEvalPdf = 0, nSample = 0;
    if (valid) {
        const size_t cp = (size_t)cap;
        const float4 r3 = A.rec[3 * cp + i];
        const uint32_t fl = __float_as_uint(r3.w);
        if (fl & kRecSample) {
            job = A.job[i];
            pix = A.pix[i];
            const DevScene& sc = jobs[job].sc;
            const PTConfig& cfg = jobs[job].cfg;
            const uint32_t depth = A.depth[i] & kDepthMask;
            prefix = f3(A.pw[i]);
            const float3 rdir = f3(A.rd[i]);
            const float4 r0 = A.rec[i], r1 = A.rec[cp + i], r2 = A.rec[2 * cp + i], r4 = A.rec[4 * cp + i];
            Surf s;
            s.pos = f3(r0);
            s.eps = r0.w;
            s.n = f3(r1);
            s.mat = __float_as_int(r1.w);
            s.sn = f3(r2);
            s.uv = make_float2(r2.w, r3.x);
            const float surv = r3.y;
            rng.s = __float_as_uint(r3.z);
            pend = fl & 0xFFu;
            radiance = f3(r4);
            hitPos = s.pos;
            Ctx c;
            c.f.n = s.sn;
            basis(c.f.n, c.f.t, c.f.b);
            c.outW = -rdir;
            c.out = c.f.toLocal(c.outW);
            c.faceN = s.n;
            c.uv = s.uv;
            const DevMaterial& m = sc.mats[s.mat];
            Lp lp = {};
            float3 diffBase = mk(0, 0, 0);
            if (GEN && m.type == kGeneric) lp = localParams(sc, m, s.uv);
            else diffBase = lookupRgb(sc, m.baseTex, m.base, s.uv);
            // SampleDirection (PathTracer.cs:526-530)
            float uc = rng.nextFloat();
            float u1 = rng.nextFloat(), u2 = rng.nextFloat();
            float3 dirW; float bpdf = 0.f; float3 bw = mk(0, 0, 0);
            bool ok = sampleMaterial<GEN>(sc, m, lp, diffBase, c, uc, u1, u2, dirW, bpdf, bw);
            if (cfg.shadingStats) {
                ++nSample;
                if (!(GEN && m.type == kGeneric)) ++nEvalPdf;
            }
            if (!ok || bpdf == 0.0f || isBlack(bw)) {
                if (pend) { cont = true; outDepth = kDoneFlag; }
                else splat(samples, pix, radiance);
            } else {
                cont = true;
                prefix = prefix * (bw / surv);  // PathTracer.cs:372-378
                prevPdfOut = bpdf * surv;
                outDepth = depth + 1;
                nRo = offsetPoint(s.pos, s.n, s.eps, dirW);
                nRd = dirW;
            }
            outDepth |= pend << kNeeShift;
        }
        if (!cont) pend = 0;
    }
    const int te = __reduce_add_sync(0xffffffffu, nEvalPdf), ts = __reduce_add_sync(0xffffffffu, nSample);
    if ((threadIdx.x & 31) == 0 && te) atomicAdd(&stats->matEvalPdf, (unsigned long long)te);
    if ((threadIdx.x & 31) == 0 && ts) atomicAdd(&stats->matSample, (unsigned long long)ts);
    // warp ballot / popc compaction into the next queue
    unsigned msk = __ballot_sync(0xffffffffu, cont);
    if (msk == 0) continue;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(nOut, __popc(msk));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!cont) continue;
    const int j = base + __popc(msk & ((1u << lane) - 1u));
    B.job[j] = job;
    B.pix[j] = pix;
    B.rng[j] = rng.s;
    B.depth[j] = outDepth;
    B.pw[j] = make_float4(prefix.x, prefix.y, prefix.z, prevPdfOut);
    B.rad[j] = make_float4(radiance.x, radiance.y, radiance.z, 0.f);
    B.prev[j] = make_float4(hitPos.x, hitPos.y, hitPos.z, 0.f);
    B.ro[j] = make_float4(nRo.x, nRo.y, nRo.z, 0.f);
    B.rd[j] = make_float4(nRd.x, nRd.y, nRd.z, (outDepth & kDoneFlag) ? -1.0f : CUDART_INF_F);
    if (pend) B.neeFrom[j] = (uint32_t)i;
    }
}

}  // namespace sst

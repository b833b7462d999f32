// Light paths on the device: LightPathCache.TraceAllPaths (Integrators/Bidir/LightPathCache.cs:
// 126-260) with the LightPathWalk modifier (:271-341) over RandomWalk (Integrators/Common/
// RandomWalk.cs:76-216).
//
// A wavefront like the camera paths': k_light_start selects the emitter or the background, samples
// the emitted ray and writes vertex 0; then per step the closest-hit traversal and k_light_walk,
// which writes the hit's vertex, applies Russian roulette, samples the BSDF on the light subpath
// (importance transport) and compacts the surviving paths.  Every path keeps its own RNG stream
// RNG(seed, path, iteration), so the vertices do not depend on the wave.  No next-event pdf
// callback is evaluated (PdfNextEventAncestor = 0), as with LightPathCache's null callback.
#include <cuda_runtime.h>

#include "sst_device.cuh"
#include "sst_kernels.h"

namespace sst {

namespace {

constexpr uint32_t kLpBgFirst = 0x40000000u;  // background path before its first hit
constexpr uint32_t kLpFromBg = 0x20000000u;   // the path started at the background
constexpr uint32_t kLpDepthMask = 0x00FFFFFFu;

// SampleWarp.ToCosineLobe (Sampling/SampleWarp.cs:171-182)
SST_D float3 toCosineLobe(float power, float u1, float u2, float& pdf) {
    float phi = kPi * 2.0f * u1;
    float cosTheta = powf(u2, 1.0f / (power + 1.0f));
    float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
    pdf = (power + 1.0f) * powf(cosTheta, power) * 1.0f / (2.0f * kPi);
    return mk(sinTheta * cosf(phi), sinTheta * sinf(phi), cosTheta);
}

// SampleWarp.ToConcentricDisc (Sampling/SampleWarp.cs:219-250), Shirley and Chiu's mapping
SST_D float2 toConcentricDisc(float u1, float u2) {
    float a = 2.0f * u1 - 1.0f, b = 2.0f * u2 - 1.0f;
    float r, phi;
    if (a > -b) {
        if (a > b) { r = a; phi = (kPi * 0.25f) * (b / a); }
        else { r = b; phi = (kPi * 0.25f) * (2.0f - (a / b)); }
    } else {
        if (a < b) { r = -a; phi = (kPi * 0.25f) * (4.0f + (b / a)); }
        else {
            r = -b;
            phi = (b != 0.0f) ? (kPi * 0.25f) * (6.0f - (a / b)) : 0.0f;
        }
    }
    return make_float2(r * cosf(phi), r * sinf(phi));
}

// The surface point of leaf-ordered triangle ti at barycentrics (u, v) (Geometry/SurfacePoint.cs),
// with its mesh and face.
SST_D void surfaceAt(const DevScene& sc, int ti, float u, float v, Surf& s, int& mesh, int& face) {
    float4 a4 = __ldg(&sc.triv[3 * (size_t)ti]), b4 = __ldg(&sc.triv[3 * (size_t)ti + 1]), c4 = __ldg(&sc.triv[3 * (size_t)ti + 2]);
    float4 fn = __ldg(&sc.triN[ti]);
    int4 aux = __ldg(&sc.triAux[ti]);
    float3 v1 = f3(a4), v2 = f3(b4), v3 = f3(c4);
    s.pos = baryPos(v1, v2, v3, u, v);
    s.n = f3(fn);
    s.eps = errorOffset(v1, v2, v3, u, v);
    s.mat = aux.x;
    mesh = aux.y;
    face = aux.z;
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
}

// GenericMaterial value with both pdfs and the light-subpath transmission factor
// (GenericMaterial.cs:152-338, :255).  The camera-path kernels use the leaner genericEval, which
// needs neither.
SST_D float3 genericEvalFull(const Ctx& c, const Lp& lp, float3 in, bool onLight, float& pdf, float& pdfRev) {
    Ggx ndf{lp.ax, lp.ay};
    const float3 o = c.out;
    float cO = fabsf(o.z), cI = fabsf(in.z);
    bool sameGeo = shouldReflect(c.faceN, c.outW, c.f.toWorld(in));
    bool sameH = sameHemi(o, in);
    float3 v = mk(0, 0, 0);
    float pf0 = 0.f, pf1 = 0.f, pf2 = 0.f, pr0 = 0.f, pr1 = 0.f, pr2 = 0.f;
    float fO = schlickWeight(cO), fI = schlickWeight(cI);
    if (sameH) {
        if (sameGeo) v = v + lp.diffuseRefl / kPi * (1.0f - fO * 0.5f) * (1.0f - fI * 0.5f);
        pf0 = cI / kPi;
        pr0 = cO / kPi;
    }
    float3 h = o + in;
    if (!isZero(h)) {
        h = normalize(h);
        float cIn = dot(in, h);
        float Rr = 2.0f * lp.rough * cIn * cIn;
        if (sameH && sameGeo) v = v + lp.retroRefl / kPi * Rr * (fO + fI + fO * fI * (Rr - 1.0f));
        if (cI != 0.0f && cO != 0.0f) {
            float cOut = dot(o, h);
            if (sameH && sameGeo && cIn * cOut > 0.0f) {
                float cHT = dot(in, (h.z < 0.0f) ? -h : h);
                float diel = fresnelDielectric(cHT, 1.0f, lp.ior);
                float3 sch = schlickFresnel(lp.r0, cHT);
                float3 fres = lerp3(lp.metallic, mk(diel, diel, diel), sch);
                v = v + lp.specTint * ndf.D(h) * ndf.G(o, in) * fres / (4.0f * cI * cO);
            }
            float jf = fabsf(4.0f * cOut), jr = fabsf(4.0f * cIn);
            if (jf != 0.0f && jr != 0.0f) {
                pf1 = ndf.pdf(o, h) / jf;
                pr1 = ndf.pdf(in, h) / jr;
            }
        }
    }
    float eta = o.z > 0.0f ? lp.ior : 1.0f / lp.ior;
    float3 ht = o + in * eta;
    if (cO != 0.0f && cI != 0.0f && !isZero(ht) && lp.specTransW > 0.0f) {
        ht = normalize(ht);
        ht = (ht.z < 0.0f) ? -ht : ht;
        float cOut = dot(o, ht), cIn = dot(in, ht);
        float sd = cOut + eta * cIn;
        if (!sameH && cOut * cIn < 0.0f) {
            float F = fresnelDielectric(cOut, 1.0f, lp.ior);
            float factor = onLight ? (1.0f / eta) : 1.0f;
            float3 wh = (!sameHemi(o, ht)) ? -ht : ht;
            float num = ndf.D(wh) * ndf.G(o, in);
            num *= eta * eta * fmaxf(0.0f, dot(in, -wh)) * fmaxf(0.0f, dot(o, wh));
            num *= factor * factor;
            float den = in.z * o.z * sd * sd;
            v = v + (mk(1, 1, 1) - mk(F, F, F)) * lp.specTrans * fabsf(num / den);
        }
        if (sd != 0.0f) {
            float3 wh = (!sameHemi(o, ht)) ? -ht : ht;
            float jac = eta * eta * fmaxf(0.0f, dot(in, -wh)) / (sd * sd);
            pf2 += ndf.pdf(o, wh) * jac;
        }
        float etaIn = in.z > 0.0f ? lp.ior : (1.0f / lp.ior);
        float3 hIn = normalize(o * etaIn + in);
        hIn = (hIn.z < 0.0f) ? -hIn : hIn;
        if (!isZero(hIn)) {
            float3 wh = (!sameHemi(in, hIn)) ? -hIn : hIn;
            float sdIn = dot(hIn, in) + etaIn * dot(o, hIn);
            if (sdIn != 0.0f) {
                float jac = etaIn * etaIn * fmaxf(0.0f, dot(o, -wh)) / (sdIn * sdIn);
                pr2 += ndf.pdf(in, wh) * jac;
            }
        }
    }
    float sF = avg3(schlickFresnel(lp.r0, fabsf(o.z)));
    float bias = fmaxf(1.0f - sF, 0.75f);
    float dw = bias * (1.0f - lp.metallic) * (1.0f - lp.specTransW);
    float fR = fresnelDielectric(dot(o, (h.z < 0.0f) ? -h : h), 1.0f, lp.ior);
    float selR = (1.0f - dw) * (1.0f - (1.0f - fR) * lp.specTransW);
    float fT = fresnelDielectric(dot(o, ht), 1.0f, lp.ior);
    float selT = (1.0f - dw) * (1.0f - fT) * lp.specTransW;
    pdf = pf0 * dw + pf1 * selR + pf2 * selT;
    pdfRev = pr0 * dw + pr1 * selR + pr2 * selT;  // the reverse selection reuses fT (GenericMaterial.cs:308-309)
    return v;
}

// Material.Sample with the forward and reverse pdfs (GenericMaterial.cs:92-150,
// DiffuseMaterial.cs:127-188).
SST_D bool sampleFull(const DevScene& sc, const DevMaterial& m, const Lp& lp, float3 diffBase, const Ctx& c, bool onLight, float u, float u1,
                      float u2, float3& dirW, float& pdf, float& pdfRev, float3& weight) {
    if (m.type == kGeneric) {
        if (c.out.z == 0.0f) return false;
        Ggx ndf{lp.ax, lp.ay};
        float eta = c.out.z > 0.0f ? (1.0f / lp.ior) : lp.ior;
        float sF = avg3(schlickFresnel(lp.r0, fabsf(c.out.z)));
        float bias = fmaxf(1.0f - sF, 0.75f);
        float dw = bias * (1.0f - lp.metallic) * (1.0f - lp.specTransW);
        float3 in;
        if (u <= dw) {
            float p;
            in = toCosHemisphere(u1, u2, p);
            if (c.out.z < 0.0f) in.z *= -1.0f;
        } else {
            float3 h = ndf.sample(c.out, u1, u2);
            float cOut = dot(c.out, (h.z < 0.0f) ? -h : h);
            float fr = fresnelDielectric(cOut, 1.0f, lp.ior);
            float selT = (1.0f - fr) * lp.specTransW;
            if ((u - dw) / (1.0f - dw) < selT) {
                if (dot(c.out, h) < 0.0f) return false;
                if (!refract(c.out, h, eta, in)) return false;
            } else {
                in = reflect(c.out, h);
            }
        }
        float3 v = genericEvalFull(c, lp, in, onLight, pdf, pdfRev);
        weight = v * fabsf(in.z) / pdf;
        dirW = c.f.toWorld(in);
        return true;
    }
    float p;
    float3 d = toCosHemisphere(u1, u2, p);
    if (m.transmitter && u < 0.5f) {
        if (c.out.z > 0.0f) d.z *= -1.0f;
    } else {
        if (c.out.z < 0.0f) d.z *= -1.0f;
    }
    float3 w = c.f.toWorld(d);
    float3 value = diffuseEval(c, diffBase, m.transmitter != 0, w, pdf);
    if (pdf == 0.0f) return false;
    // reverse pdf: the cosine at the outgoing direction (DiffuseMaterial.cs:167-188)
    float3 in = c.f.toLocal(w);
    bool sh = sameHemi(c.out, in);
    float rr = sh ? fabsf(c.out.z) / kPi : 0.0f;
    if (m.transmitter) {
        float tr = !sh ? fabsf(c.out.z) / kPi : 0.0f;
        pdfRev = (rr + tr) * 0.5f;
    } else {
        pdfRev = rr;
    }
    weight = value / pdf;
    dirW = w;
    return true;
}

SST_D void putVertex(SstPathVertexDev* out, const Surf& s, bool surface, int mesh, int face, float pdfFrom, float pdfRev, float3 weight,
                     float rough, int depth, int path, bool fromBg) {
    SstPathVertexDev v;
    v.p[0] = s.pos.x; v.p[1] = s.pos.y; v.p[2] = s.pos.z;
    v.p[3] = surface ? s.n.x : 0.0f; v.p[4] = surface ? s.n.y : 0.0f; v.p[5] = surface ? s.n.z : 0.0f;
    v.p[6] = surface ? s.sn.x : 0.0f; v.p[7] = surface ? s.sn.y : 0.0f; v.p[8] = surface ? s.sn.z : 0.0f;
    v.p[9] = pdfFrom; v.p[10] = pdfRev; v.p[11] = 0.0f;
    v.p[12] = weight.x; v.p[13] = weight.y; v.p[14] = weight.z;
    v.p[15] = rough;
    v.q[0] = surface ? mesh : -1; v.q[1] = surface ? face : -1; v.q[2] = depth; v.q[3] = path; v.q[4] = fromBg ? 1 : 0; v.q[5] = 0;
    *out = v;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// K10: light selection and the emitted ray (LightPathCache.TraceLightPath / TraceEmitterPath /
// TraceBackgroundPath, :151-241; DiffuseEmitter.SampleRay, GlossyEmitter.SampleRay,
// EnvironmentMap.SampleRay)
// ---------------------------------------------------------------------------------------------
__global__ void k_light_start(const DevJob* jobs, LightParams P, LightPathBuf A, int* qCount, SstPathVertexDev* verts, int* lengths) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= P.numPaths) return;
    const DevScene& sc = jobs[0].sc;
    Rng rng{hashSeed(P.seed, (uint32_t)idx, P.iter)};
    const int nEm = sc.nEmitters;
    const int stride = P.maxDepth + 1;
    SstPathVertexDev* out = verts + (size_t)idx * stride;
    float bgProb = sc.hasEnv ? 1.0f / (1.0f + (float)nEm) : 0.0f;
    bool background = false;
    float prob;
    int emIdx = -1;
    if (bgProb > 0.0f && rng.nextFloat() <= bgProb) {
        background = true;
        prob = bgProb;
    } else {
        emIdx = (int)rng.nextInt((uint32_t)nEm);
        prob = (1.0f - bgProb) / (float)nEm;
    }
    float3 ro, rd, prefix, prevPos = mk(0, 0, 0), prevN = mk(0, 0, 0);
    float pdfDir, tmin = 0.0f;
    uint32_t depthFlags;
    Surf s0;
    if (!background) {
        const DevEmitter& em = sc.emitters[emIdx];
        float p1 = rng.nextFloat(), p2 = rng.nextFloat();
        float d1 = rng.nextFloat(), d2 = rng.nextFloat();
        // Triangle.SampleUniformArea (Geometry/Triangle.cs:42-55)
        float2 bar = toUniformTriangle(p1, p2);
        float3 e1 = f3(em.v1), e2 = f3(em.v2), e3 = f3(em.v3);
        s0.pos = baryPos(e1, e2, e3, bar.x, bar.y);
        s0.n = f3(em.faceN);
        s0.sn = s0.n;
        if (em.n1.w != 0.0f) s0.sn = normalize(bar.x * f3(em.n2) + bar.y * f3(em.n3) + (1.0f - bar.x - bar.y) * f3(em.n1));
        s0.eps = errorOffset(e1, e2, e3, bar.x, bar.y);
        float posPdf = em.faceN.w;
        float3 t, b;
        basis(s0.sn, t, b);
        float3 local, weight;
        float lpdf;
        if (em.rad.w < 0.0f) {
            local = toCosHemisphere(d1, d2, lpdf);
            weight = f3(em.rad) / posPdf * kPi;
        } else {
            local = toCosineLobe(em.rad.w + 1.0f, d1, d2, lpdf);
            float3 w = f3(em.rad) * powf(local.z, em.rad.w + 1.0f) * em.norm;
            weight = w / posPdf / lpdf;
        }
        float3 dir = local.z * s0.sn + local.x * t + local.y * b;
        float pdf = lpdf * posPdf * prob;
        if (pdf == 0.0f || isBlack(weight)) { lengths[idx] = 0; return; }
        putVertex(out, s0, true, em.mesh, em.face, 0.0f, 0.0f, mk(0, 0, 0), 0.0f, 0, idx, false);
        lengths[idx] = 1;
        if (1 >= P.maxDepth) return;  // RandomWalk.ContinueWalk: while (depth < maxDepth)
        ro = offsetPoint(s0.pos, s0.n, s0.eps, dir);
        rd = dir;
        prefix = weight / prob;
        pdfDir = pdf;
        prevPos = s0.pos;
        prevN = s0.n;
        depthFlags = 1u;
    } else {
        float p1 = rng.nextFloat(), p2 = rng.nextFloat();
        float d1 = rng.nextFloat(), d2 = rng.nextFloat();
        float3 dsd, dsw;
        float dsp;
        envSample(sc.env, d1, d2, dsd, dsp, dsw);
        float2 disc = toConcentricDisc(p1, p2);
        float3 t, b;
        basis(dsd, t, b);
        float3 pos = sc.sceneCenter + sc.sceneRadius * (dsd + t * disc.x + b * disc.y);
        float posPdf = (1.0f / kPi) / (sc.sceneRadius * sc.sceneRadius);
        float3 weight = dsw / posPdf;
        float pdf = posPdf * dsp;
        pdf *= prob;
        weight = weight / prob;
        if (pdf == 0.0f || isBlack(weight)) { lengths[idx] = 0; return; }
        s0.pos = pos;
        putVertex(out, s0, false, -1, -1, 0.0f, 0.0f, mk(0, 0, 0), 0.0f, 0, idx, true);
        lengths[idx] = 1;
        ro = pos;
        rd = -dsd;
        prefix = weight;
        pdfDir = pdf;
        depthFlags = 1u | kLpBgFirst | kLpFromBg;
    }
    int q = atomicAdd(qCount, 1);
    A.path[q] = (uint32_t)idx;
    A.rng[q] = rng.s;
    A.depth[q] = depthFlags;
    A.prefix[q] = make_float4(prefix.x, prefix.y, prefix.z, pdfDir);
    A.approx[q] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    A.prevP[q] = make_float4(prevPos.x, prevPos.y, prevPos.z, 0.0f);
    A.prevN[q] = make_float4(prevN.x, prevN.y, prevN.z, 0.0f);
    A.ro[q] = make_float4(ro.x, ro.y, ro.z, tmin);
    A.rd[q] = make_float4(rd.x, rd.y, rd.z, CUDART_INF_F);
}

// ---------------------------------------------------------------------------------------------
// K11: one step of the light-path random walk (RandomWalk.StartFromBackground :86-124 for a
// background path's first hit, RandomWalk.ContinueWalk :145-216 otherwise)
// ---------------------------------------------------------------------------------------------
__global__ void k_light_walk(const DevJob* jobs, LightParams P, LightPathBuf A, LightPathBuf B, const float4* hits, const int* nIn, int* nOut,
                             SstPathVertexDev* verts, int* lengths) {
    const int n = *nIn;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ((int)(blockIdx.x * blockDim.x) >= n) return;
    bool cont = false;
    uint32_t path = 0, outDepth = 0;
    Rng rng{0};
    float3 prefix = mk(0, 0, 0), approx = mk(1, 1, 1), nro = mk(0, 0, 0), nrd = mk(0, 0, 0), hitPos = mk(0, 0, 0), hitN = mk(0, 0, 0);
    float pdfDir = 0.0f, nextRev = 0.0f;
    if (i < n) {
        const DevScene& sc = jobs[0].sc;
        path = A.path[i];
        rng.s = A.rng[i];
        uint32_t df = A.depth[i];
        const int depth = (int)(df & kLpDepthMask);
        const bool bgFirst = (df & kLpBgFirst) != 0, fromBg = (df & kLpFromBg) != 0;
        float4 pr4 = A.prefix[i], ap4 = A.approx[i];
        prefix = f3(pr4);
        pdfDir = pr4.w;
        approx = f3(ap4);
        nextRev = ap4.w;
        float3 prevPos = f3(A.prevP[i]), prevN = f3(A.prevN[i]);
        float4 h = hits[i];
        int ti = __float_as_int(h.w);
        const int stride = P.maxDepth + 1;
        SstPathVertexDev* out = verts + (size_t)path * stride;
        if (ti >= 0) {
            float3 rdir = f3(A.rd[i]);
            Surf s;
            int mesh, face;
            surfaceAt(sc, ti, h.y, h.z, s, mesh, face);
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
            if (m.type == kGeneric) lp = localParams(sc, m, s.uv);
            else diffBase = lookupRgb(sc, m.baseTex, m.base, s.uv);
            // LightPathWalk.OnHit (:323-337): MaximumRoughness takes the maximum with
            // Payload.maxRoughness, which stays 0
            float rough = fmaxf(m.type == kGeneric ? lp.rough : 1.0f, 0.0f);
            int len = lengths[path];
            if (bgFirst) {
                float uc = rng.nextFloat(), u1 = rng.nextFloat(), u2 = rng.nextFloat();
                float3 dirW, bw;
                float bp = 0.0f, bpr = 0.0f;
                bool ok = sampleFull(sc, m, lp, diffBase, c, true, uc, u1, u2, dirW, bp, bpr, bw);
                if (!ok) { bp = 0.0f; bpr = 0.0f; bw = mk(0, 0, 0); }
                approx = approx * bw;
                putVertex(out + len, s, true, mesh, face, pdfDir, nextRev, prefix, rough, 1, (int)path, fromBg);
                lengths[path] = len + 1;
                nextRev = bpr;
                if (P.maxDepth > 1 && bp != 0.0f && !isBlack(bw)) {
                    prefix = prefix * bw;
                    pdfDir = bp;
                    hitPos = s.pos;
                    hitN = s.n;
                    nro = offsetPoint(s.pos, s.n, s.eps, dirW);
                    nrd = dirW;
                    outDepth = 2u | kLpFromBg;
                    cont = 2 < P.maxDepth;  // ContinueWalk(..., 2): while (depth < maxDepth)
                }
            } else {
                float pdfFrom = pdfDir * areaToSolidAngle(prevPos, s.pos, s.n);
                if (pdfFrom != 0.0f) {
                    putVertex(out + len, s, true, mesh, face, pdfFrom, nextRev, prefix, rough, depth, (int)path, fromBg);
                    lengths[path] = len + 1;
                    if (depth + 1 < P.maxDepth) {
                        float surv = depth > 4 ? clampf(avg3(approx), 0.05f, 0.95f) : 1.0f;
                        if (!(rng.nextFloat() > surv)) {
                            float uc = rng.nextFloat(), u1 = rng.nextFloat(), u2 = rng.nextFloat();
                            float3 dirW, bw;
                            float bp = 0.0f, bpr = 0.0f;
                            bool ok = sampleFull(sc, m, lp, diffBase, c, true, uc, u1, u2, dirW, bp, bpr, bw);
                            if (!ok) { bp = 0.0f; bpr = 0.0f; bw = mk(0, 0, 0); }
                            approx = approx * (bw / surv);
                            nextRev = bpr * areaToSolidAngle(s.pos, prevPos, prevN);
                            if (bp != 0.0f && !isBlack(bw)) {
                                // the sampled weight carries the shading cosine; light transport needs the
                                // geometric one, and the incoming cosines cancel only for aligned normals
                                bw = bw * (fabsf(dot(s.n, dirW)) / fabsf(dot(s.sn, dirW)));
                                bw = bw * (fabsf(dot(s.sn, -rdir)) / fabsf(dot(s.n, -rdir)));
                                prefix = prefix * (bw / surv);
                                pdfDir = bp;
                                hitPos = s.pos;
                                hitN = s.n;
                                nro = offsetPoint(s.pos, s.n, s.eps, dirW);
                                nrd = dirW;
                                outDepth = (uint32_t)(depth + 1) | (fromBg ? kLpFromBg : 0u);
                                cont = depth + 1 < P.maxDepth;
                            }
                        }
                    }
                }
            }
        }
    }
    unsigned mk32 = __ballot_sync(0xffffffffu, cont);
    if (mk32 == 0) return;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(nOut, __popc(mk32));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!cont) return;
    int j = base + __popc(mk32 & ((1u << lane) - 1u));
    B.path[j] = path;
    B.rng[j] = rng.s;
    B.depth[j] = outDepth;
    B.prefix[j] = make_float4(prefix.x, prefix.y, prefix.z, pdfDir);
    B.approx[j] = make_float4(approx.x, approx.y, approx.z, nextRev);
    B.prevP[j] = make_float4(hitPos.x, hitPos.y, hitPos.z, 0.0f);
    B.prevN[j] = make_float4(hitN.x, hitN.y, hitN.z, 0.0f);
    B.ro[j] = make_float4(nro.x, nro.y, nro.z, 0.0f);
    B.rd[j] = make_float4(nrd.x, nrd.y, nrd.z, CUDART_INF_F);
}

void launch_light_start(const DevJob* jobs, const LightParams& P, const LightPathBuf& A, int* qCount, SstPathVertexDev* verts, int* lengths,
                        cudaStream_t s) {
    if (P.numPaths <= 0) return;
    k_light_start<<<(P.numPaths + 127) / 128, 128, 0, s>>>(jobs, P, A, qCount, verts, lengths);
}

void launch_light_walk(const DevJob* jobs, const LightParams& P, const LightPathBuf& A, const LightPathBuf& B, const float4* hits, const int* nIn,
                       int* nOut, SstPathVertexDev* verts, int* lengths, int maxItems, cudaStream_t s) {
    if (maxItems <= 0) return;
    k_light_walk<<<(maxItems + 127) / 128, 128, 0, s>>>(jobs, P, A, B, hits, nIn, nOut, verts, lengths);
}

}  // namespace sst

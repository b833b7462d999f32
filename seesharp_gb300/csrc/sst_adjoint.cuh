// Derivatives of the BSDF value with respect to the differentiable material parameters, for the
// path-replay adjoint.  Forward-mode dual numbers carry four partials: base colour r, g, b and
// roughness.  Directions do not depend on the parameters (no geometric derivatives), so only the
// parameter-dependent quantities of GenericMaterial.ComputeLocalParams /
// ComputeValueAndPdf (Shading/Materials/GenericMaterial.cs:152-381) are duals; the arithmetic
// follows sst_device.cuh's genericEval step by step.
#pragma once
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "sst_device.cuh"

namespace sst {

struct Dl {
    float v;
    float d[4];
};
SST_D Dl dconst(float v) { return Dl{v, {0.f, 0.f, 0.f, 0.f}}; }
SST_D Dl operator+(Dl a, Dl b) { Dl r; r.v = a.v + b.v; for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
SST_D Dl operator-(Dl a, Dl b) { Dl r; r.v = a.v - b.v; for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
SST_D Dl operator*(Dl a, Dl b) { Dl r; r.v = a.v * b.v; for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
SST_D Dl operator/(Dl a, Dl b) {
    Dl r;
    r.v = a.v / b.v;
    float ib = 1.0f / b.v;
    for (int k = 0; k < 4; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
SST_D Dl operator*(Dl a, float s) { Dl r; r.v = a.v * s; for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * s; return r; }
SST_D Dl operator*(float s, Dl a) { return a * s; }
SST_D Dl operator/(Dl a, float s) { Dl r; r.v = a.v / s; for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] / s; return r; }
SST_D Dl operator+(Dl a, float s) { a.v += s; return a; }
SST_D Dl operator+(float s, Dl a) { a.v += s; return a; }
SST_D Dl operator-(float s, Dl a) { Dl r; r.v = s - a.v; for (int k = 0; k < 4; ++k) r.d[k] = -a.d[k]; return r; }
SST_D Dl operator-(Dl a, float s) { a.v -= s; return a; }
SST_D Dl operator/(float s, Dl b) { return dconst(s) / b; }
SST_D Dl dsqrt(Dl a) {
    Dl r;
    r.v = sqrtf(a.v);
    float g = r.v > 0.0f ? 0.5f / r.v : 0.0f;
    for (int k = 0; k < 4; ++k) r.d[k] = a.d[k] * g;
    return r;
}
SST_D Dl dmax(Dl a, float b) { return a.v >= b ? a : dconst(b); }
SST_D Dl dabs(Dl a) { return a.v < 0.0f ? (-1.0f) * a : a; }

struct Dl3 {
    Dl x, y, z;
};
SST_D Dl3 d3(Dl a, Dl b, Dl c) { return Dl3{a, b, c}; }
SST_D Dl3 d3c(float3 a) { return Dl3{dconst(a.x), dconst(a.y), dconst(a.z)}; }
SST_D Dl3 operator+(Dl3 a, Dl3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
SST_D Dl3 operator*(Dl3 a, Dl s) { return d3(a.x * s, a.y * s, a.z * s); }
SST_D Dl3 operator*(Dl3 a, float s) { return d3(a.x * s, a.y * s, a.z * s); }
SST_D Dl3 operator*(float s, Dl3 a) { return a * s; }
SST_D Dl3 operator*(Dl3 a, Dl3 b) { return d3(a.x * b.x, a.y * b.y, a.z * b.z); }
SST_D Dl3 operator/(Dl3 a, Dl s) { return d3(a.x / s, a.y / s, a.z / s); }
SST_D Dl3 operator/(Dl3 a, float s) { return d3(a.x / s, a.y / s, a.z / s); }
// RgbColor.Lerp(w, from, to) = (1 - w) from + w to
SST_D Dl3 dlerp(float w, Dl3 from, Dl3 to) { return (1.0f - w) * from + w * to; }
SST_D Dl3 dlerp1(float w, float from, Dl3 to) { return d3((1.0f - w) * from + w * to.x, (1.0f - w) * from + w * to.y, (1.0f - w) * from + w * to.z); }

// GGX with dual alphas (TrowbridgeReitzDistribution.cs:22-63)
struct GgxD {
    Dl ax, ay;
    SST_D Dl D(float3 n) const {
        float tan2 = sin2(n) / cos2(n);
        if (isinf(tan2)) return dconst(0.0f);
        float c4 = cos2(n) * cos2(n);
        float cp = cosPhi(n), sp = sinPhi(n);
        Dl e = tan2 * (cp * cp / (ax * ax) + sp * sp / (ay * ay));
        Dl one = dconst(1.0f);
        return one / (kPi * ax * ay * c4 * (1.0f + e) * (1.0f + e));
    }
    SST_D Dl lambda(float3 o) const {
        float at = fabsf(sinT(o) / o.z);
        if (isinf(at)) return dconst(0.0f);
        float cp = cosPhi(o), sp = sinPhi(o);
        Dl a = dsqrt(cp * cp * ax * ax + sp * sp * ay * ay);
        Dl a2t2 = a * at * (a * at);
        return (-1.0f + dsqrt(1.0f + a2t2)) / 2.0f;
    }
    SST_D Dl G(float3 o, float3 i) const { return dconst(1.0f) / (1.0f + lambda(o) + lambda(i)); }
};

// Value of GenericMaterial at shading-space direction `in` with its partials with respect to
// (base r, g, b, roughness).  base/rough are the looked-up parameter values at the shading point.
SST_D Dl3 genericEvalDeriv(const Ctx& c, const DevMaterial& m, float3 baseV, float roughV, float3 in) {
    Dl3 base = d3(Dl{baseV.x, {1.f, 0.f, 0.f, 0.f}}, Dl{baseV.y, {0.f, 1.f, 0.f, 0.f}}, Dl{baseV.z, {0.f, 0.f, 1.f, 0.f}});
    Dl rough = Dl{roughV, {0.f, 0.f, 0.f, 1.f}};
    // ComputeLocalParams (GenericMaterial.cs:354-381)
    Dl lum = 0.2126f * base.x + 0.7152f * base.y + 0.0722f * base.z;
    Dl3 colorTint = lum.v > 0.0f ? base / lum : d3c(mk(1, 1, 1));
    Dl3 specTint = dlerp1(m.specTint, 1.0f, colorTint);
    float aspect = sqrtf(1.0f - m.aniso * .9f);
    GgxD ndf{dmax(rough * rough / aspect, .001f), dmax(rough * rough * aspect, .001f)};
    Dl3 r0 = dlerp(m.metallic, specTint * schlickR0(m.ior), base);
    float dwp = (1.0f - m.metallic) * (1.0f - m.specTrans);
    Dl3 diffuseRefl = base * dwp, retroRefl = base * dwp, specTransC = m.specTrans * base;

    const float3 o = c.out;
    float cO = fabsf(o.z), cI = fabsf(in.z);
    bool sameGeo = shouldReflect(c.faceN, c.outW, c.f.toWorld(in));
    bool sameH = sameHemi(o, in);
    Dl3 v = d3c(mk(0, 0, 0));
    float fO = schlickWeight(cO), fI = schlickWeight(cI);
    if (sameH && sameGeo) v = v + diffuseRefl / kPi * (1.0f - fO * 0.5f) * (1.0f - fI * 0.5f);
    float3 h = o + in;
    if (!isZero(h)) {
        h = normalize(h);
        float cIn = dot(in, h);
        Dl Rr = 2.0f * rough * cIn * cIn;
        if (sameH && sameGeo) v = v + retroRefl / kPi * Rr * (fO + fI + fO * fI * (Rr - 1.0f));
        if (cI != 0.0f && cO != 0.0f) {
            float cOut = dot(o, h);
            if (sameH && sameGeo && cIn * cOut > 0.0f) {
                float cHT = dot(in, (h.z < 0.0f) ? -h : h);
                float diel = fresnelDielectric(cHT, 1.0f, m.ior);
                float sw = schlickWeight(cHT);
                // SchlickFresnel: lerp(sw, R0, White) = (1 - sw) R0 + sw
                Dl3 sch = d3((1.0f - sw) * r0.x + sw, (1.0f - sw) * r0.y + sw, (1.0f - sw) * r0.z + sw);
                Dl3 fres = d3((1.0f - m.metallic) * diel + m.metallic * sch.x, (1.0f - m.metallic) * diel + m.metallic * sch.y,
                              (1.0f - m.metallic) * diel + m.metallic * sch.z);
                Dl dg = ndf.D(h) * ndf.G(o, in);
                v = v + specTint * dg * fres / (4.0f * cI * cO);
            }
        }
    }
    float eta = o.z > 0.0f ? m.ior : 1.0f / m.ior;
    float3 ht = o + in * eta;
    if (cO != 0.0f && cI != 0.0f && !isZero(ht) && m.specTrans > 0.0f) {
        ht = normalize(ht);
        ht = (ht.z < 0.0f) ? -ht : ht;
        float cOut = dot(o, ht), cIn = dot(in, ht);
        float sd = cOut + eta * cIn;
        if (!sameH && cOut * cIn < 0.0f) {
            float F = fresnelDielectric(cOut, 1.0f, m.ior);
            float3 wh = (!sameHemi(o, ht)) ? -ht : ht;
            Dl num = ndf.D(wh) * ndf.G(o, in);
            num = num * (eta * eta * fmaxf(0.0f, dot(in, -wh)) * fmaxf(0.0f, dot(o, wh)));
            float den = in.z * o.z * sd * sd;
            v = v + specTransC * (1.0f - F) * dabs(num / den);
        }
    }
    return v;
}

// BSDF value (no cosine) with partials for either material type at world direction inW.
SST_D Dl3 bsdfDeriv(const DevMaterial& m, float3 baseV, float roughV, const Ctx& c, float3 inW) {
    if (m.type == kGeneric) return genericEvalDeriv(c, m, baseV, roughV, c.f.toLocal(inW));
    // DiffuseMaterial.Evaluate (DiffuseMaterial.cs:109-122): f = base / pi or 0
    bool refl = shouldReflect(c.faceN, c.outW, inW);
    float3 in = c.f.toLocal(inW);
    bool sh = sameHemi(c.out, in);
    float K = 0.0f;
    if (m.transmitter && !refl) K = !sh ? 1.0f / kPi : 0.0f;
    else if (refl) K = sh ? 1.0f / kPi : 0.0f;
    return d3(Dl{baseV.x * K, {K, 0.f, 0.f, 0.f}}, Dl{baseV.y * K, {0.f, K, 0.f, 0.f}}, Dl{baseV.z * K, {0.f, 0.f, K, 0.f}});
}

// Gradient targets of a shading point: the base colour (a texel of a 3-channel texture:
// offset >= 0 into the texel pool; a constant: -(material + 2); -1: none) and the roughness
// (material index for a constant roughness of a GenericMaterial, else -1).
SST_D void gradTargets(const DevScene& sc, int matIdx, float2 uv, int& baseTgt, int& roughTgt) {
    const DevMaterial& m = sc.mats[matIdx];
    if (m.baseTex >= 0) {
        baseTgt = sc.texs[m.baseTex].channels == 3 ? (int)(texel(sc, m.baseTex, uv) - sc.texData) : -1;
    } else {
        baseTgt = -(matIdx + 2);
    }
    roughTgt = (m.type == kGeneric && m.roughTex < 0) ? matIdx : -1;
}
// Gradient accumulation.  Paths of one warp usually hit the same surface, so the lanes that add
// to the same target are summed first (labelled partition of the active lanes by target, shuffle
// reduction) and one lane per target issues the global atomics.
namespace adjcg = cooperative_groups;
SST_D void groupAdd(float* p, int label, float g0, float g1, float g2, int n) {
    adjcg::coalesced_group act = adjcg::coalesced_threads();
    adjcg::coalesced_group grp = adjcg::labeled_partition(act, label);
    if (grp.size() > 1) {
        g0 = adjcg::reduce(grp, g0, adjcg::plus<float>());
        if (n > 1) g1 = adjcg::reduce(grp, g1, adjcg::plus<float>());
        if (n > 2) g2 = adjcg::reduce(grp, g2, adjcg::plus<float>());
    }
    if (grp.thread_rank() != 0) return;
    if (g0 != 0.0f) atomicAdd(p, g0);
    if (n > 1 && g1 != 0.0f) atomicAdd(p + 1, g1);
    if (n > 2 && g2 != 0.0f) atomicAdd(p + 2, g2);
}
SST_D void addBaseGrad(const DevAdj& a, int tgt, float g0, float g1, float g2) {
    if (tgt >= 0) groupAdd(a.gTex + tgt, tgt, g0, g1, g2, 3);
    else if (tgt <= -2) groupAdd(a.gMatBase + 3 * (size_t)(-tgt - 2), tgt, g0, g1, g2, 3);
}
SST_D void addRoughGrad(const DevAdj& a, int tgt, float g) {
    if (tgt >= 0) groupAdd(a.gMatRough + tgt, tgt, g, 0.0f, 0.0f, 1);
}
SST_D void addEmitterGrad(const DevAdj& a, int idx, float3 g) {
    if (idx >= 0) groupAdd(a.gEmitter + 3 * (size_t)idx, idx, g.x, g.y, g.z, 3);
}
// d emitted / d radiance (per channel the same scalar): 1 or 0 for a diffuse emitter, the lobe
// factor for a glossy one (DiffuseEmitter.cs:33-37, GlossyEmitter.cs:36-40).
SST_D float emittedScale(const DevEmitter& em, float3 shadingN, float3 dir) {
    if (em.rad.w < 0.0f) return dot(shadingN, dir) < 0.0f ? 0.0f : 1.0f;
    float c = dot(shadingN, dir) / len(dir);
    if (c < 0.0f) return 0.0f;
    return powf(c, em.rad.w) * em.norm;
}

}  // namespace sst

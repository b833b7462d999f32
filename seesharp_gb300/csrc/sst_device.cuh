// Device functions of the path tracer: RNG, sample warps, shading frame, Fresnel, GGX, the two
// materials, environment map, emitters and camera.  Each function names the SeeSharp source it
// follows (paths relative to the SeeSharp project root).  All arithmetic is FP32.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include "sst_types.h"

namespace sst {

#define SST_D __device__ __forceinline__
#define SST_HD __host__ __device__ __forceinline__
// Large shading functions called from several places are compiled once (SST_DN) to keep the
// instruction footprint of the shade kernel small.
#ifdef SST_NOINLINE_MORE
#define SST_DN static __device__ __noinline__
#else
#define SST_DN __device__ __forceinline__
#endif

constexpr float kPi = 3.14159265f;  // MathF.PI

// ---------------------------------------------------------------------------------------------
// float3 helpers
// ---------------------------------------------------------------------------------------------
SST_HD float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
SST_HD float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
SST_HD float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
SST_HD float3 operator-(float3 a) { return mk(-a.x, -a.y, -a.z); }
SST_HD float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
SST_HD float3 operator*(float s, float3 a) { return mk(s * a.x, s * a.y, s * a.z); }
SST_HD float3 operator*(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
SST_HD float3 operator/(float3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
SST_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SST_HD float3 cross(float3 a, float3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
SST_D float len(float3 a) { return sqrtf(dot(a, a)); }
// Vector3.Normalize (NaN for a zero input), correctly rounded even where the unit divides and takes
// square roots with the approximate forms: a sharp microfacet lobe turns an ulp of a half vector or
// of a sampled direction into a relative 1e-3 of its density.
SST_D float3 normalize(float3 a) {
    const float l = __fsqrt_rn(dot(a, a));
    return mk(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
SST_HD float3 f3(float4 v) { return mk(v.x, v.y, v.z); }
SST_HD bool isZero(float3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
SST_HD bool isBlack(float3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
SST_D float avg3(float3 a) { return (a.x + a.y + a.z) / 3.0f; }  // RgbColor.Average
SST_D float3 fabs3(float3 a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
SST_D float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
// RgbColor.Lerp(w, from, to) = (1 - w) from + w to
SST_D float3 lerp3(float w, float3 from, float3 to) { return (1.0f - w) * from + w * to; }
// RgbColor.Luminance (Rec. 709 weights)
SST_D float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// ---------------------------------------------------------------------------------------------
// RNG (Sampling/RNG.cs:7-118)
// ---------------------------------------------------------------------------------------------
SST_HD uint32_t pcgHash(uint32_t in) {  // RNG.cs:107-111
    uint32_t s = in * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    return (w >> 22) ^ w;
}
SST_HD uint32_t fnvHash(uint32_t h, uint32_t d) {  // RNG.cs:99-105
    h = (h * 16777619u) ^ (d & 0xFFu);
    h = (h * 16777619u) ^ ((d >> 8) & 0xFFu);
    h = (h * 16777619u) ^ ((d >> 16) & 0xFFu);
    h = (h * 16777619u) ^ ((d >> 24) & 0xFFu);
    return h;
}
SST_HD uint32_t hashSeed(uint32_t base, uint32_t chain, uint32_t sample) {  // RNG.cs:113-118
    uint32_t h = fnvHash(2166136261u, pcgHash(base));
    h = fnvHash(h, pcgHash(chain));
    h = fnvHash(h, pcgHash(sample));
    return pcgHash(h);
}
struct Rng {
    uint32_t s;
    SST_D uint32_t next() {  // RNG.cs:90-94
        uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
        s = s * 747796405u + 2891336453u;
        return (w >> 22) ^ w;
    }
    // RNG.cs:43-45: [0, 1] inclusive.  Correctly rounded conversion and division.
    SST_D float nextFloat() { return __fdiv_rn(__uint2float_rn(next()), 4294967296.0f); }
    SST_D uint32_t nextInt(uint32_t max) {  // RNG.cs:56-70 (Lemire)
        uint32_t x = next();
        unsigned long long m = (unsigned long long)x * max;
        uint32_t l = (uint32_t)m;
        if (l < max) {
            uint32_t t = (0u - max) % max;
            // rejection probability per draw is below max / 2^32; the cap only bounds the loop
            for (int guard = 0; l < t && guard < 1024; ++guard) {
                x = next();
                m = (unsigned long long)x * max;
                l = (uint32_t)m;
            }
        }
        return (uint32_t)(m >> 32);
    }
};

// ---------------------------------------------------------------------------------------------
// Sample warps (Sampling/SampleWarp.cs)
// ---------------------------------------------------------------------------------------------
SST_D float3 sphericalToCartesian(float sinT, float cosT, float phi) {  // :89-96
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return mk(sinT * cp, sinT * sp, cosT);
}
SST_D float3 toCosHemisphere(float u1, float u2, float& pdf) {  // :130-137
    float3 d = sphericalToCartesian(sqrtf(1.0f - u2), sqrtf(u2), 2.0f * kPi * u1);
    pdf = d.z / kPi;
    return d;
}
SST_D float2 toUniformTriangle(float u1, float u2) {  // :9-14
    float s = sqrtf(u1);
    return make_float2(1.0f - s, u2 * s);
}

// ---------------------------------------------------------------------------------------------
// Shading space (Shading/ShadingSpace.cs)
// ---------------------------------------------------------------------------------------------
SST_D void basis(float3 n, float3& t, float3& b) {  // :14-23
    if (fabsf(n.x) > fabsf(n.y)) {
        float d = sqrtf(n.x * n.x + n.z * n.z);
        t = mk(-n.z, 0.0f, n.x) / d;
    } else {
        float d = sqrtf(n.y * n.y + n.z * n.z);
        t = mk(0.0f, n.z, -n.y) / d;
    }
    b = cross(n, t);
}
struct Frame {
    float3 n, t, b;
    SST_D float3 toLocal(float3 d) const { return mk(dot(t, d), dot(b, d), dot(n, d)); }  // :40-48
    SST_D float3 toWorld(float3 s) const { return s.z * n + s.x * t + s.y * b; }            // :64-71
};
SST_D bool sameHemi(float3 a, float3 b) { return a.z * b.z > 0.0f; }  // :140
SST_D float cos2(float3 d) { return d.z * d.z; }
SST_D float sin2(float3 d) { return fmaxf(0.0f, 1.0f - cos2(d)); }
SST_D float sinT(float3 d) { return sqrtf(sin2(d)); }
SST_D float cosPhi(float3 d) { float s = sinT(d); return s == 0.0f ? 1.0f : clampf(d.x / s, -1.0f, 1.0f); }  // :88-91
SST_D float sinPhi(float3 d) { float s = sinT(d); return s == 0.0f ? 0.0f : clampf(d.y / s, -1.0f, 1.0f); }  // :93-96
SST_D float3 reflect(float3 o, float3 n) { return -o + 2.0f * dot(o, n) * n; }  // :109-110
SST_D bool refract(float3 in, float3 n, float eta, float3& out) {  // :121-132
    float c = dot(n, in);
    float s2 = fmaxf(0.0f, 1.0f - c * c);
    float t2 = eta * eta * s2;
    if (t2 >= 1.0f) return false;
    float ct = sqrtf(1.0f - t2);
    out = eta * -in + (eta * c - ct) * n;
    return true;
}

// ---------------------------------------------------------------------------------------------
// Fresnel (Shading/Fresnel.cs)
// ---------------------------------------------------------------------------------------------
SST_D float fresnelDielectric(float cosI, float etaI, float etaT) {  // :4-25
    cosI = clampf(cosI, -1.0f, 1.0f);
    if (!(cosI > 0.0f)) {
        float tmp = etaI; etaI = etaT; etaT = tmp;
        cosI = fabsf(cosI);
    }
    float sinI = sqrtf(fmaxf(0.0f, 1.0f - cosI * cosI));
    float sinTT = etaI / etaT * sinI;
    if (sinTT >= 1.0f) return 1.0f;
    float cosTT = sqrtf(fmaxf(0.0f, 1.0f - sinTT * sinTT));
    float rpar = (etaT * cosI - etaI * cosTT) / (etaT * cosI + etaI * cosTT);
    float rper = (etaI * cosI - etaT * cosTT) / (etaI * cosI + etaT * cosTT);
    return (rpar * rpar + rper * rper) / 2.0f;
}
SST_D float schlickWeight(float c) {  // :34-37
    float m = clampf(1.0f - c, 0.0f, 1.0f);
    return (m * m) * (m * m) * m;
}
SST_D float3 schlickFresnel(float3 r0, float c) { return lerp3(schlickWeight(c), r0, mk(1, 1, 1)); }  // :39-41
SST_D float schlickR0(float eta) { float r = (eta - 1.0f) / (eta + 1.0f); return r * r; }           // :45-48

// ---------------------------------------------------------------------------------------------
// GGX (Shading/TrowbridgeReitzDistribution.cs)
// ---------------------------------------------------------------------------------------------
struct Ggx {
    float ax, ay;
    SST_D float D(float3 n) const {  // :22-34
        float tan2 = sin2(n) / cos2(n);
        if (isinf(tan2)) return 0.0f;
        float c4 = cos2(n) * cos2(n);
        float cp = cosPhi(n), sp = sinPhi(n);
        float e = tan2 * (cp * cp / (ax * ax) + sp * sp / (ay * ay));
        return 1.0f / (kPi * ax * ay * c4 * (1.0f + e) * (1.0f + e));
    }
    SST_D float lambda(float3 o) const {  // :107-113
        float at = fabsf(sinT(o) / o.z);
        if (isinf(at)) return 0.0f;
        float cp = cosPhi(o), sp = sinPhi(o);
        float a = sqrtf(cp * cp * ax * ax + sp * sp * ay * ay);
        float a2t2 = a * at * (a * at);
        return (-1.0f + sqrtf(1.0f + a2t2)) / 2.0f;
    }
    SST_D float G1(float3 o) const { return 1.0f / (1.0f + lambda(o)); }
    SST_D float G(float3 o, float3 i) const { return 1.0f / (1.0f + lambda(o) + lambda(i)); }
    SST_D float pdf(float3 o, float3 n) const {  // :59-63
        if (!sameHemi(o, n)) return 0.0f;
        return G1(o) * fmaxf(0.0f, dot(o, n)) * D(n) / fabsf(o.z);
    }
    // :70-100, Heitz 2018 visible normals; exact reciprocal square root where the reference
    // uses a platform-defined estimate.
    SST_D float3 sample(float3 o, float u1, float u2) const {
        bool flip = o.z < 0.0f;
        if (flip) o = -o;
        float3 vh = normalize(mk(ax * o.x, ay * o.y, o.z));
        float lsq = vh.x * vh.x + vh.y * vh.y;
        float3 t1 = lsq > 0.0f ? mk(-vh.y, vh.x, 0.0f) * (1.0f / sqrtf(lsq)) : mk(1.0f, 0.0f, 0.0f);
        float3 t2v = cross(vh, t1);
        float r = sqrtf(u1);
        float phi = 2.0f * kPi * u2;
        float sp, cp;
        sincosf(phi, &sp, &cp);
        float p1 = r * cp;
        float p2 = r * sp;
        float s = 0.5f * (1.0f + vh.z);
        p2 = (1.0f - s) * sqrtf(1.0f - p1 * p1) + s * p2;
        float3 nh = p1 * t1 + p2 * t2v + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
        float3 ne = normalize(mk(ax * nh.x, ay * nh.y, fmaxf(0.0f, nh.z)));
        return flip ? -ne : ne;
    }
};

// ---------------------------------------------------------------------------------------------
// Textures (Images/ImageTexture.cs:27-44, TextureRgb.cs:29-35, TextureMono.cs:32-38)
// ---------------------------------------------------------------------------------------------
SST_D const float* texel(const DevScene& sc, int ti, float2 uv) {
    const DevTexture& t = sc.texs[ti];
    int col = (int)(uv.x * (float)t.w);
    int row = (int)(uv.y * (float)t.h);
    if (t.border == 0) {
        row = (row % t.h + t.h) % t.h;
        col = (col % t.w + t.w) % t.w;
    } else {
        row = min(max(row, 0), t.h - 1);
        col = min(max(col, 0), t.w - 1);
    }
    return sc.texData + t.offset + ((long long)row * t.w + col) * t.channels;
}
SST_D float3 lookupRgb(const DevScene& sc, int tex, const float* c, float2 uv) {
    if (tex < 0) return mk(c[0], c[1], c[2]);
    const float* p = texel(sc, tex, uv);
    if (sc.texs[tex].channels == 1) return mk(p[0], p[0], p[0]);
    return mk(p[0], p[1], p[2]);
}
SST_D float lookupMono(const DevScene& sc, int tex, float c, float2 uv) {
    if (tex < 0) return c;
    return texel(sc, tex, uv)[0];
}

// ---------------------------------------------------------------------------------------------
// Surface point and shading context (Geometry/SurfacePoint.cs, ShadingContext.cs:3-27)
// ---------------------------------------------------------------------------------------------
struct Surf {
    float3 pos, n, sn;   // position, face normal, shading normal
    float2 uv;
    float eps;           // error offset (Geometry/Mesh.cs:50-60)
    int mat;
};
// Mesh.ComputeErrorOffset (Geometry/Mesh.cs:50-60) with (u, v) weighting the 2nd/3rd vertex
SST_D float errorOffset(float3 v1, float3 v2, float3 v3, float u, float v) {
    float3 e = fabs3(u * v2) + fabs3(v * v3) + fabs3((1.0f - u - v) * v1);
    return len(e) * 32.0f * 1.19209e-07f;
}
SST_D float3 baryPos(float3 v1, float3 v2, float3 v3, float u, float v) { return u * v2 + v * v3 + (1.0f - u - v) * v1; }

// Offset a point along its face normal to the side of dir (TinyEmbree Raytracer.SpawnRay).
SST_D float3 offsetPoint(float3 p, float3 n, float eps, float3 dir) {
    float sign = dot(dir, n) < 0.0f ? -1.0f : 1.0f;
    return p + (sign * eps) * n;
}

// ---------------------------------------------------------------------------------------------
// Materials
// ---------------------------------------------------------------------------------------------
struct Ctx {
    Frame f;
    float3 outW, out;  // outgoing direction: world, shading space
    float3 faceN;
    float2 uv;
};

// GenericMaterial.LocalParams (GenericMaterial.cs:343-381), plus the material's scalars.
struct Lp {
    float3 specTint, diffuseRefl, retroRefl, specTrans, r0;
    float rough, ax, ay;
    float metallic, specTransW, ior;
};
SST_DN Lp localParams(const DevScene& sc, const DevMaterial& m, float2 uv) {
    Lp r;
    float3 base = lookupRgb(sc, m.baseTex, m.base, uv);
    float lum = luminance(base);
    float3 colorTint = lum > 0.0f ? base / lum : mk(1, 1, 1);
    r.specTint = lerp3(m.specTint, mk(1, 1, 1), colorTint);
    r.rough = lookupMono(sc, m.roughTex, m.rough, uv);
    float aspect = sqrtf(1.0f - m.aniso * .9f);
    r.ax = fmaxf(.001f, r.rough * r.rough / aspect);
    r.ay = fmaxf(.001f, r.rough * r.rough * aspect);
    r.r0 = lerp3(m.metallic, schlickR0(m.ior) * r.specTint, base);
    float dw = (1.0f - m.metallic) * (1.0f - m.specTrans);
    r.diffuseRefl = base * dw;
    r.specTrans = m.specTrans * base;
    r.retroRefl = base * dw;
    r.metallic = m.metallic;
    r.specTransW = m.specTrans;
    r.ior = m.ior;
    return r;
}

// Material.cs:127-134 with the face normal
SST_D bool shouldReflect(float3 faceN, float3 outW, float3 inW) { return dot(outW, faceN) * dot(inW, faceN) >= 0.0f; }

// GenericMaterial.ComputeValueAndPdf (GenericMaterial.cs:152-338); returns the BSDF value and the
// forward pdf (the reverse pdf is not needed by the path tracer).
// Compiled once and called (not inlined) by default: the shade kernel evaluates it for three
// directions per bounce, and one copy of the code keeps the instruction cache warm.
#ifndef SST_EVAL_INLINE
static __device__ __noinline__
#else
SST_D
#endif
float3 genericEval(const Ctx& c, const Lp& lp, float3 in, float& pdf) {
    Ggx ndf{lp.ax, lp.ay};
    const float3 o = c.out;
    float cO = fabsf(o.z), cI = fabsf(in.z);
    bool sameGeo = shouldReflect(c.faceN, c.outW, c.f.toWorld(in));
    bool sameH = sameHemi(o, in);
    float3 v = mk(0, 0, 0);
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;
    float fO = schlickWeight(cO), fI = schlickWeight(cI);
    if (sameH) {
        if (sameGeo) v = v + lp.diffuseRefl / kPi * (1.0f - fO * 0.5f) * (1.0f - fI * 0.5f);
        p0 = cI / kPi;
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
            if (jf != 0.0f && jr != 0.0f) p1 = ndf.pdf(o, h) / jf;
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
            float3 wh = (!sameHemi(o, ht)) ? -ht : ht;
            float num = ndf.D(wh) * ndf.G(o, in);
            num *= eta * eta * fmaxf(0.0f, dot(in, -wh)) * fmaxf(0.0f, dot(o, wh));
            float den = in.z * o.z * sd * sd;
            v = v + (mk(1, 1, 1) - mk(F, F, F)) * lp.specTrans * fabsf(num / den);
        }
        if (sd != 0.0f) {
            float3 wh = (!sameHemi(o, ht)) ? -ht : ht;
            float jac = eta * eta * fmaxf(0.0f, dot(in, -wh)) / (sd * sd);
            p2 += ndf.pdf(o, wh) * jac;
        }
    }
    float sF = avg3(schlickFresnel(lp.r0, fabsf(o.z)));
    float bias = fmaxf(1.0f - sF, 0.75f);
    float dw = bias * (1.0f - lp.metallic) * (1.0f - lp.specTransW);
    float fR = fresnelDielectric(dot(o, (h.z < 0.0f) ? -h : h), 1.0f, lp.ior);
    float selR = (1.0f - dw) * (1.0f - (1.0f - fR) * lp.specTransW);
    float fT = fresnelDielectric(dot(o, ht), 1.0f, lp.ior);
    float selT = (1.0f - dw) * (1.0f - fT) * lp.specTransW;
    pdf = p0 * dw + p1 * selR + p2 * selT;
    return v;
}

// DiffuseMaterial.Evaluate + Pdf (DiffuseMaterial.cs:109-122, 167-188) for a world direction.
SST_DN float3 diffuseEval(const Ctx& c, float3 base, bool transmitter, float3 inW, float& pdf) {
    bool refl = shouldReflect(c.faceN, c.outW, inW);
    float3 in = c.f.toLocal(inW);
    bool sh = sameHemi(c.out, in);
    float3 f = mk(0, 0, 0);
    if (transmitter && !refl) {
        if (!sh) f = base / kPi;
    } else if (refl) {
        if (sh) f = base / kPi;
    }
    float rf = sh ? fabsf(in.z) / kPi : 0.0f;
    if (transmitter) {
        float tf = !sh ? fabsf(in.z) / kPi : 0.0f;
        pdf = (rf + tf) * 0.5f;
    } else {
        pdf = rf;
    }
    return f * fabsf(in.z);  // Material.EvaluateWithCosine (Material.cs:80-83)
}

// Material.EvaluateWithCosine and Material.Pdf for a world direction in one pass.
// GEN = false compiles the diffuse case only (for waves without GenericMaterials).
template <bool GEN = true>
SST_D float3 evalWithCos(const DevScene& sc, const DevMaterial& m, const Lp& lp, float3 diffBase, const Ctx& c, float3 inW, float& pdf) {
    if (GEN && m.type == kGeneric) {
        float3 in = c.f.toLocal(inW);
        float3 v = genericEval(c, lp, in, pdf);
        return v * fabsf(in.z);
    }
    return diffuseEval(c, diffBase, m.transmitter != 0, inW, pdf);
}

// Material.Sample: GenericMaterial.cs:92-150 / DiffuseMaterial.cs:127-164.  Returns false for an
// invalid sample (pdf 0).
template <bool GEN = true>
SST_DN bool sampleMaterial(const DevScene& sc, const DevMaterial& m, const Lp& lp, float3 diffBase, const Ctx& c, float u, float u1, float u2,
                          float3& dirW, float& pdf, float3& weight) {
    if (GEN && m.type == kGeneric) {
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
        float3 v = genericEval(c, lp, in, pdf);
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
    weight = value / pdf;
    dirW = w;
    return true;
}

// ---------------------------------------------------------------------------------------------
// Environment map (Shading/Background/EnvironmentMap.cs, Sampling/RegularGrid2d.cs,
// Sampling/PiecewiseConstant.cs)
// ---------------------------------------------------------------------------------------------
SST_D float4 envPixel(const DevEnv& e, int col, int row) {
    col = min(max(col, 0), e.w - 1);
    row = min(max(row, 0), e.h - 1);
    return __ldg(&e.img[(size_t)row * e.w + col]);
}
SST_D float2 worldToSpherical(float3 d) {  // :158-166
    d = normalize(d);
    float2 sp = make_float2(atan2f(d.z, d.x), atan2f(sqrtf(d.x * d.x + d.z * d.z), d.y));
    if (sp.x < 0.0f) sp.x += kPi * 2.0f;
    return sp;
}
SST_D float3 envRadiance(const DevEnv& e, float3 d) {  // :19-26
    float2 sp = worldToSpherical(d);
    float px = sp.x / (2.0f * kPi), py = sp.y / kPi;
    return f3(envPixel(e, (int)(px * (float)e.w), (int)(py * (float)e.h)));
}
// PiecewiseConstant.Sample (:37-50): first index with cdf >= u
SST_D int lowerBound(const float* cdf, int n, float u) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(&cdf[mid]) < u) lo = mid + 1; else hi = mid;
    }
    return min(lo, n - 1);
}
SST_D float cdfProb(const float* cdf, int i) { return i > 0 ? __ldg(&cdf[i]) - __ldg(&cdf[i - 1]) : __ldg(&cdf[i]); }
SST_D float gridPdf(const DevEnv& e, float x, float y) {  // RegularGrid2d.cs:40-47
    int row = min(max((int)(y * (float)e.h), 0), e.h - 1);
    int col = min(max((int)(x * (float)e.w), 0), e.w - 1);
    float p = cdfProb(e.rowCdf, row);
    if (p == 0.0f) return 0.0f;
    p *= cdfProb(e.colCdf + (size_t)row * e.w, col);
    return p * (float)(e.h * e.w);
}
SST_D float envPdf(const DevEnv& e, float3 d) {  // :81-85
    float2 sp = worldToSpherical(d);
    float px = sp.x / (2.0f * kPi), py = sp.y / kPi;
    return gridPdf(e, px, py) / (sinf(sp.y) * kPi * kPi * 2.0f);
}
// :40-73
SST_DN void envSample(const DevEnv& e, float u1, float u2, float3& dir, float& pdf, float3& weight) {
    int row = lowerBound(e.rowCdf, e.h, u2);
    float lo = row == 0 ? 0.0f : __ldg(&e.rowCdf[row - 1]);
    float relRow = (u2 - lo) / (__ldg(&e.rowCdf[row]) - lo);
    if (!__ldg(&e.hasCol[row])) {  // only reachable with u2 == 0 on an empty first row
        dir = mk(0, 1, 0); pdf = 0.0f; weight = mk(0, 0, 0);
        return;
    }
    const float* cc = e.colCdf + (size_t)row * e.w;
    int col = lowerBound(cc, e.w, u1);
    float clo = col == 0 ? 0.0f : __ldg(&cc[col - 1]);
    float relCol = (u1 - clo) / (__ldg(&cc[col]) - clo);
    float x = ((float)col + relCol) / (float)e.w;
    float y = ((float)row + relRow) / (float)e.h;
    float p = gridPdf(e, x, y);
    float phi = x * 2.0f * kPi, theta = y * kPi;
    float st = sinf(theta);
    dir = mk(st * cosf(phi), cosf(theta), st * sinf(phi));
    float jac = sinf(theta) * kPi * kPi * 2.0f;
    if (jac == 0.0f) { pdf = 0.0f; weight = mk(0, 0, 0); return; }
    p /= jac;
    weight = f3(envPixel(e, (int)(x * (float)e.w), (int)(y * (float)e.h))) / p;
    pdf = p;
}

// ---------------------------------------------------------------------------------------------
// Emitters (Shading/Emitters/DiffuseEmitter.cs:33-37, GlossyEmitter.cs:36-40)
// ---------------------------------------------------------------------------------------------
SST_D float3 emitted(const DevEmitter& em, float3 shadingN, float3 dir) {
    float3 rad = f3(em.rad);
    if (em.rad.w < 0.0f) {
        if (dot(shadingN, dir) < 0.0f) return mk(0, 0, 0);
        return rad;
    }
    float c = dot(shadingN, dir) / len(dir);
    if (c < 0.0f) return mk(0, 0, 0);
    return rad * powf(c, em.rad.w) * em.norm;
}
// SampleWarp.SurfaceAreaToSolidAngle (SampleWarp.cs:290-294)
SST_D float areaToSolidAngle(float3 from, float3 toPos, float3 toN) {
    float3 d = toPos - from;
    float dsq = dot(d, d);
    return fabsf(dot(toN, -d)) / (dsq * sqrtf(dsq));
}

// ---------------------------------------------------------------------------------------------
// Camera (Cameras/PerspectiveCamera.cs:64-102)
// ---------------------------------------------------------------------------------------------
SST_D void cameraRay(const DevCamera& c, float fx, float fy, float3& org, float3& dir) {
    float vx = 2.0f * fx / (float)c.W - 1.0f;
    float vy = 1.0f - 2.0f * fy / (float)c.H;
    const float* m = c.v2c;  // Vector3.Transform((vx, vy, 0), viewToCamera)
    float lx = vx * m[0] + vy * m[4] + 0.0f * m[8] + m[12];
    float ly = vx * m[1] + vy * m[5] + 0.0f * m[9] + m[13];
    float lz = vx * m[2] + vy * m[6] + 0.0f * m[10] + m[14];
    const float* w = c.c2w;  // Vector4.Transform((local, 0), cameraToWorld)
    float3 d = mk(lx * w[0] + ly * w[4] + lz * w[8], lx * w[1] + ly * w[5] + lz * w[9], lx * w[2] + ly * w[6] + lz * w[10]);
    org = mk(w[12], w[13], w[14]);
    dir = normalize(d);
}

// Last chunk of a wave with itemOffset <= item (the chunks are sorted by itemOffset).
__device__ __forceinline__ int findChunk(const WaveChunk* ch, int lo, int hi, int item) {
    // last chunk with itemOffset <= item (chunks are sorted by itemOffset)
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (ch[mid].itemOffset <= item) lo = mid; else hi = mid;
    }
    return lo;
}

}  // namespace sst

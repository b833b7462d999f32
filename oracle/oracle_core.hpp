// ORACLE -- test infrastructure only.
//
// CPU restatement of the arithmetic on SeeSharp's unidirectional PathTracer path, used as the
// checker for the CUDA implementation in seesharp_gb300/.  Nothing in the product links, imports
// or executes this code; only tests/, the smoke check and bench.py's CPU-baseline leg do.
//
// Every function names the reference file:line it restates (paths relative to the SeeSharp
// project root).  The code is templated on the scalar type T so that the same restatement runs
// in FP32 (the reference's own precision) and in FP64 (the high-precision replay used for
// gradient checks and intersection parity).
//
// Pinning: the functions here are checked against the known-answer tests in SeeSharp.Tests
// (camera rays, materials, microfacet distribution, environment map, warps, piecewise-constant
// distributions, mesh sampling, scene assembly).  Arithmetic that lives in the un-vendored
// TinyEmbree 1.2.0 / SimpleImageIO 1.8.3 packages (ray offsets, shading-normal interpolation,
// RgbColor.Luminance, RgbImage.GetPixel border handling) is restated from its published
// behaviour and marked "unpinned" where no reference test fixes it.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace ora {

// ------------------------------------------------------------------------------------------
// Vector / colour types (System.Numerics.Vector2/3 and SimpleImageIO.RgbColor semantics)
// ------------------------------------------------------------------------------------------
template <class T> struct V2 {
    T x = 0, y = 0;
    V2() = default;
    V2(T a, T b) : x(a), y(b) {}
};

template <class T> struct V3 {
    T x = 0, y = 0, z = 0;
    V3() = default;
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline bool operator==(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> inline bool operator!=(V3<T> a, V3<T> b) { return !(a == b); }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T lengthSq(V3<T> a) { return dot(a, a); }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
// Vector3.Normalize(v) == v / v.Length() (a zero vector yields NaNs, as in .NET)
template <class T> inline V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> inline V3<T> vabs(V3<T> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }

template <class T> struct Rgb {
    T r = 0, g = 0, b = 0;
    Rgb() = default;
    Rgb(T a, T b_, T c) : r(a), g(b_), b(c) {}
    explicit Rgb(T v) : r(v), g(v), b(v) {}
    static Rgb White() { return Rgb(T(1)); }
    static Rgb Black() { return Rgb(T(0)); }
    // SimpleImageIO RgbColor.Average: arithmetic mean of the channels.
    T Average() const { return (r + g + b) / T(3); }
    // SimpleImageIO RgbColor.Luminance (Rec. 709 weights).  Used by GenericMaterial.cs:360 and
    // EnvironmentMap.cs:144.  Unpinned: SimpleImageIO's source is not vendored.
    T Luminance() const { return T(0.2126f) * r + T(0.7152f) * g + T(0.0722f) * b; }
    bool IsBlack() const { return r == 0 && g == 0 && b == 0; }
};
template <class T> inline Rgb<T> operator+(Rgb<T> a, Rgb<T> b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
template <class T> inline Rgb<T> operator-(Rgb<T> a, Rgb<T> b) { return {a.r - b.r, a.g - b.g, a.b - b.b}; }
template <class T> inline Rgb<T> operator*(Rgb<T> a, Rgb<T> b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
template <class T> inline Rgb<T> operator*(Rgb<T> a, T s) { return {a.r * s, a.g * s, a.b * s}; }
template <class T> inline Rgb<T> operator*(T s, Rgb<T> a) { return {s * a.r, s * a.g, s * a.b}; }
template <class T> inline Rgb<T> operator/(Rgb<T> a, T s) { return {a.r / s, a.g / s, a.b / s}; }
template <class T> inline Rgb<T> operator/(Rgb<T> a, Rgb<T> b) { return {a.r / b.r, a.g / b.g, a.b / b.b}; }
// RgbColor.Lerp(w, from, to) = (1 - w) * from + w * to.  The argument order is pinned by the
// Schlick comment in Shading/Fresnel.cs:28-33 (R = R0 + (1 - R0) w).
template <class T> inline Rgb<T> lerp(T w, Rgb<T> from, Rgb<T> to) { return (T(1) - w) * from + w * to; }

template <class T> constexpr T kPi() { return T(3.14159265358979323846); }
// MathF.PI is the float nearest to pi; in FP32 both spellings agree.
template <class T> inline T PI() { return std::is_same<T, float>::value ? T(3.14159265f) : kPi<T>(); }

// ------------------------------------------------------------------------------------------
// RNG  (Sampling/RNG.cs:7-118)
// ------------------------------------------------------------------------------------------
struct Rng {
    uint32_t state;
    // RNG.cs:20
    explicit Rng(uint32_t seed = 0xAB20F90u) : state(seed) {}
    // RNG.cs:29-30
    Rng(uint32_t baseSeed, uint32_t chainIndex, uint32_t sampleIndex) : state(HashSeed(baseSeed, chainIndex, sampleIndex)) {}

    // RNG.cs:90-94: output word from the current state, then advance the LCG.
    uint32_t Next() {
        uint32_t word = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
        state = state * 747796405u + 2891336453u;
        return (word >> 22) ^ word;
    }
    // RNG.cs:43-45: [0,1] inclusive, u32 -> float then divide by (float)uint.MaxValue.
    float NextFloat() { return float(Next()) / float(4294967295u); }
    V2<float> NextFloat2D() {
        float a = NextFloat();
        float b = NextFloat();
        return {a, b};
    }
    // RNG.cs:56-70: Lemire's multiply-shift with rejection.
    uint32_t NextInt(uint32_t max) {
        uint32_t x = Next();
        uint64_t m = uint64_t(x) * uint64_t(max);
        uint32_t l = uint32_t(m);
        if (l < max) {
            uint32_t t = (0u - max) % max;
            while (l < t) {
                x = Next();
                m = uint64_t(x) * uint64_t(max);
                l = uint32_t(m);
            }
        }
        return uint32_t(m >> 32);
    }
    // RNG.cs:99-105
    static uint32_t FnvHash(uint32_t hash, uint32_t data) {
        const uint32_t prime = 16777619u;
        hash = (hash * prime) ^ (data & 0xFF);
        hash = (hash * prime) ^ ((data >> 8) & 0xFF);
        hash = (hash * prime) ^ ((data >> 16) & 0xFF);
        hash = (hash * prime) ^ ((data >> 24) & 0xFF);
        return hash;
    }
    // RNG.cs:107-111
    static uint32_t PcgHash(uint32_t input) {
        uint32_t s = input * 747796405u + 2891336453u;
        uint32_t word = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
        return (word >> 22) ^ word;
    }
    // RNG.cs:113-118
    static uint32_t HashSeed(uint32_t baseSeed, uint32_t chainIndex, uint32_t sampleIndex) {
        uint32_t h = FnvHash(2166136261u, PcgHash(baseSeed));
        h = FnvHash(h, PcgHash(chainIndex));
        h = FnvHash(h, PcgHash(sampleIndex));
        return PcgHash(h);
    }
};

// ------------------------------------------------------------------------------------------
// SampleWarp  (Sampling/SampleWarp.cs)
// ------------------------------------------------------------------------------------------
template <class T> struct DirectionSample { V3<T> Direction; T Pdf; };

// SampleWarp.cs:9-14
template <class T> inline V2<T> ToUniformTriangle(V2<T> p) {
    T s = std::sqrt(p.x);
    return {T(1) - s, p.y * s};
}
// SampleWarp.cs:16-22
template <class T> inline V2<T> FromUniformTriangle(V2<T> b) {
    if (b.x == T(1)) return {T(0), T(0)};
    return {(T(1) - b.x) * (T(1) - b.x), b.y / (T(1) - b.x)};
}
// SampleWarp.cs:89-96
template <class T> inline V3<T> SphericalToCartesian(T sintheta, T costheta, T phi) {
    T sp = std::sin(phi), cp = std::cos(phi);
    return {sintheta * cp, sintheta * sp, costheta};
}
// SampleWarp.cs:114-121
template <class T> inline V2<T> CartesianToSpherical(V3<T> d) {
    V2<T> sp(std::atan2(d.y, d.x), std::atan2(std::sqrt(d.x * d.x + d.y * d.y), d.z));
    if (sp.x < 0) sp.x += PI<T>() * T(2);
    return sp;
}
// SampleWarp.cs:130-137
template <class T> inline DirectionSample<T> ToCosHemisphere(V2<T> p) {
    V3<T> d = SphericalToCartesian<T>(std::sqrt(T(1) - p.y), std::sqrt(p.y), T(2) * PI<T>() * p.x);
    return {d, d.z / PI<T>()};
}
// SampleWarp.cs:139-145
template <class T> inline V2<T> FromCosHemisphere(V3<T> local) {
    V2<T> s = CartesianToSpherical(local);
    T x = s.x / (T(2) * PI<T>());
    T c = std::cos(s.y);
    return {x, c * c};
}
// SampleWarp.cs:171-182
template <class T> inline DirectionSample<T> ToCosineLobe(T power, V2<T> p) {
    T phi = PI<T>() * T(2) * p.x;
    T cosTheta = std::pow(p.y, T(1) / (power + T(1)));
    T sinTheta = std::sqrt(T(1) - cosTheta * cosTheta);
    V3<T> d = SphericalToCartesian(sinTheta, cosTheta, phi);
    return {d, (power + T(1)) * std::pow(cosTheta, power) * T(1) / (T(2) * PI<T>())};
}
// SampleWarp.cs:196-203
template <class T> inline DirectionSample<T> ToUniformSphere(V2<T> p) {
    T a = T(2) * PI<T>() * p.y;
    T b = T(2) * std::sqrt(p.x - p.x * p.x);
    return {SphericalToCartesian(b, T(1) - T(2) * p.x, a), T(1) / (T(4) * PI<T>())};
}
// SampleWarp.cs:205-212
template <class T> inline V2<T> FromUniformSphere(V3<T> dir) {
    V2<T> s = CartesianToSpherical(normalize(dir));
    return {(T(1) - std::cos(s.y)) / T(2), s.x / (T(2) * PI<T>())};
}
// SampleWarp.cs:219-247
template <class T> inline V2<T> ToConcentricDisc(V2<T> p) {
    T phi, r;
    T a = T(2) * p.x - T(1);
    T b = T(2) * p.y - T(1);
    if (a > -b) {
        if (a > b) { r = a; phi = (PI<T>() * T(0.25)) * (b / a); }
        else { r = b; phi = (PI<T>() * T(0.25)) * (T(2) - (a / b)); }
    } else {
        if (a < b) { r = -a; phi = (PI<T>() * T(0.25)) * (T(4) + (b / a)); }
        else {
            r = -b;
            if (b != 0) phi = (PI<T>() * T(0.25)) * (T(6) - (a / b));
            else phi = 0;
        }
    }
    return {r * std::cos(phi), r * std::sin(phi)};
}

// ------------------------------------------------------------------------------------------
// PiecewiseConstantPDF  (Sampling/PiecewiseConstant.cs:12-70)
// ------------------------------------------------------------------------------------------
template <class T> struct PiecewiseConstant {
    std::vector<T> cdf;
    PiecewiseConstant() = default;
    // PiecewiseConstant.cs:12-29
    explicit PiecewiseConstant(const T* w, int n) {
        cdf.resize(n);
        T sum = 0;
        for (int i = 0; i < n; ++i) { sum += w[i]; cdf[i] = sum; }
        T total = cdf[n - 1];
        for (int i = 0; i < n && total > T(0); ++i) cdf[i] /= total;
        cdf[n - 1] = T(1);
    }
    // PiecewiseConstant.cs:37-50.  List.BinarySearch followed by the walk down over equal
    // entries selects the first index whose cdf value is >= u (a lower bound).
    void Sample(T u, int& idx, T& rel) const {
        idx = int(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        if (idx >= int(cdf.size())) idx = int(cdf.size()) - 1;  // u > 1 cannot come from NextFloat
        T lo = idx == 0 ? T(0) : cdf[idx - 1];
        T delta = cdf[idx] - lo;
        rel = (u - lo) / delta;
    }
    // PiecewiseConstant.cs:58-62
    T SampleInverse(int idx, T rel) const {
        T lo = idx == 0 ? T(0) : cdf[idx - 1];
        return (cdf[idx] - lo) * rel + lo;
    }
    // PiecewiseConstant.cs:66-70
    T Probability(int idx) const { return idx > 0 ? cdf[idx] - cdf[idx - 1] : cdf[idx]; }
};

// ------------------------------------------------------------------------------------------
// RegularGrid2d  (Sampling/RegularGrid2d.cs)
// ------------------------------------------------------------------------------------------
template <class T> struct RegularGrid2d {
    int numCols = 0, numRows = 0;
    std::vector<T> density, rowMarginals;
    PiecewiseConstant<T> rowDistribution;
    std::vector<PiecewiseConstant<T>> colDistributions;
    std::vector<char> hasCol;

    void Init(int resX, int resY) {  // RegularGrid2d.cs:8-13
        numCols = resX; numRows = resY;
        density.assign(size_t(resX) * resY, T(0));
        rowMarginals.assign(resY, T(0));
    }
    void Splat(int col, int row, T value) {  // RegularGrid2d.cs:62-65
        density[size_t(row) * numCols + col] += value;
        rowMarginals[row] += value;
    }
    void Normalize() {  // RegularGrid2d.cs:67-81
        rowDistribution = PiecewiseConstant<T>(rowMarginals.data(), numRows);
        colDistributions.assign(numRows, PiecewiseConstant<T>());
        hasCol.assign(numRows, 0);
        for (int i = 0; i < numRows; ++i) {
            if (rowMarginals[i] == T(0)) continue;
            colDistributions[i] = PiecewiseConstant<T>(&density[size_t(i) * numCols], numCols);
            hasCol[i] = 1;
        }
    }
    // RegularGrid2d.cs:20-26.  A row without a column distribution can only be selected by
    // u == 0 exactly (where the reference dereferences null); the restatement reports `ok=false`.
    V2<T> Sample(V2<T> primary, bool& ok) const {
        int rowIdx, colIdx; T relRow, relCol;
        rowDistribution.Sample(primary.y, rowIdx, relRow);
        ok = hasCol[rowIdx] != 0;
        if (!ok) return {T(0), T(0)};
        colDistributions[rowIdx].Sample(primary.x, colIdx, relCol);
        return {(T(colIdx) + relCol) / T(numCols), (T(rowIdx) + relRow) / T(numRows)};
    }
    // RegularGrid2d.cs:40-47
    T Pdf(V2<T> pos) const {
        int row = std::min(std::max(int(pos.y * T(numRows)), 0), numRows - 1);
        int col = std::min(std::max(int(pos.x * T(numCols)), 0), numCols - 1);
        T p = rowDistribution.Probability(row);
        if (p == T(0)) return T(0);
        p *= colDistributions[row].Probability(col);
        return p * T(numRows * numCols);
    }
};

// ------------------------------------------------------------------------------------------
// ShadingSpace  (Shading/ShadingSpace.cs)
// ------------------------------------------------------------------------------------------
// ShadingSpace.cs:14-23
template <class T> inline void ComputeBasisVectors(V3<T> n, V3<T>& tangent, V3<T>& binormal) {
    if (std::fabs(n.x) > std::fabs(n.y)) {
        T denom = std::sqrt(n.x * n.x + n.z * n.z);
        tangent = V3<T>(-n.z, T(0), n.x) / denom;
    } else {
        T denom = std::sqrt(n.y * n.y + n.z * n.z);
        tangent = V3<T>(T(0), n.z, -n.y) / denom;
    }
    binormal = cross(n, tangent);
}
// ShadingSpace.cs:40-48
template <class T> inline V3<T> WorldToShading(V3<T> n, V3<T> t, V3<T> b, V3<T> d) {
    T z = dot(n, d), x = dot(t, d), y = dot(b, d);
    return {x, y, z};
}
template <class T> inline V3<T> WorldToShading(V3<T> n, V3<T> d) {  // ShadingSpace.cs:29-38
    V3<T> t, b; ComputeBasisVectors(n, t, b);
    return WorldToShading(n, t, b, d);
}
// ShadingSpace.cs:64-71
template <class T> inline V3<T> ShadingToWorld(V3<T> n, V3<T> t, V3<T> b, V3<T> s) {
    return s.z * n + s.x * t + s.y * b;
}
template <class T> inline V3<T> ShadingToWorld(V3<T> n, V3<T> s) {  // ShadingSpace.cs:54-62
    V3<T> t, b; ComputeBasisVectors(n, t, b);
    return ShadingToWorld(n, t, b, s);
}
template <class T> inline T CosThetaSqr(V3<T> d) { return d.z * d.z; }
template <class T> inline T SinThetaSqr(V3<T> d) { return std::max(T(0), T(1) - CosThetaSqr(d)); }
template <class T> inline T SinTheta(V3<T> d) { return std::sqrt(SinThetaSqr(d)); }
template <class T> inline T TanTheta(V3<T> d) { return SinTheta(d) / d.z; }
template <class T> inline T TanThetaSqr(V3<T> d) { return SinThetaSqr(d) / CosThetaSqr(d); }
template <class T> inline T CosPhi(V3<T> d) {  // ShadingSpace.cs:88-91
    T s = SinTheta(d);
    return s == T(0) ? T(1) : std::clamp(d.x / s, T(-1), T(1));
}
template <class T> inline T SinPhi(V3<T> d) {  // ShadingSpace.cs:93-96
    T s = SinTheta(d);
    return s == T(0) ? T(0) : std::clamp(d.y / s, T(-1), T(1));
}
// ShadingSpace.cs:109-110
template <class T> inline V3<T> Reflect(V3<T> o, V3<T> n) { return -o + T(2) * dot(o, n) * n; }
// ShadingSpace.cs:121-132
template <class T> inline bool Refract(V3<T> in, V3<T> n, T eta, V3<T>& out) {
    T cosThetaI = dot(n, in);
    T sin2ThetaI = std::max(T(0), T(1) - cosThetaI * cosThetaI);
    T sin2ThetaT = eta * eta * sin2ThetaI;
    if (sin2ThetaT >= T(1)) return false;
    T cosThetaT = std::sqrt(T(1) - sin2ThetaT);
    out = eta * -in + (eta * cosThetaI - cosThetaT) * n;
    return true;
}
// ShadingSpace.cs:140
template <class T> inline bool SameHemisphere(V3<T> a, V3<T> b) { return a.z * b.z > T(0); }

// ------------------------------------------------------------------------------------------
// Fresnel  (Shading/Fresnel.cs)
// ------------------------------------------------------------------------------------------
// Fresnel.cs:4-25
template <class T> inline T FresnelDielectric(T cosThetaI, T etaI, T etaT) {
    cosThetaI = std::clamp(cosThetaI, T(-1), T(1));
    bool entering = cosThetaI > T(0);
    if (!entering) { std::swap(etaI, etaT); cosThetaI = std::fabs(cosThetaI); }
    T sinThetaI = std::sqrt(std::max(T(0), T(1) - cosThetaI * cosThetaI));
    T sinThetaT = etaI / etaT * sinThetaI;
    if (sinThetaT >= T(1)) return T(1);
    T cosThetaT = std::sqrt(std::max(T(0), T(1) - sinThetaT * sinThetaT));
    T Rparl = (etaT * cosThetaI - etaI * cosThetaT) / (etaT * cosThetaI + etaI * cosThetaT);
    T Rperp = (etaI * cosThetaI - etaT * cosThetaT) / (etaI * cosThetaI + etaT * cosThetaT);
    return (Rparl * Rparl + Rperp * Rperp) / T(2);
}
// Fresnel.cs:34-37
template <class T> inline T SchlickWeight(T cosTheta) {
    T m = std::clamp(T(1) - cosTheta, T(0), T(1));
    return (m * m) * (m * m) * m;
}
// Fresnel.cs:39-41
template <class T> inline Rgb<T> SchlickFresnel(Rgb<T> R0, T cosTheta) { return lerp(SchlickWeight(cosTheta), R0, Rgb<T>::White()); }
// Fresnel.cs:45-48
template <class T> inline T SchlickR0FromEta(T eta) { T r = (eta - T(1)) / (eta + T(1)); return r * r; }

// ------------------------------------------------------------------------------------------
// TrowbridgeReitzDistribution  (Shading/TrowbridgeReitzDistribution.cs)
// ------------------------------------------------------------------------------------------
template <class T> struct GGX {
    T ax, ay;
    // TrowbridgeReitzDistribution.cs:22-34
    T D(V3<T> n) const {
        T tan2 = TanThetaSqr(n);
        if (std::isinf(tan2)) return T(0);
        T cos4 = CosThetaSqr(n) * CosThetaSqr(n);
        T cp = CosPhi(n), sp = SinPhi(n);
        T e = tan2 * (cp * cp / (ax * ax) + sp * sp / (ay * ay));
        return T(1) / (PI<T>() * ax * ay * cos4 * (T(1) + e) * (T(1) + e));
    }
    // TrowbridgeReitzDistribution.cs:107-113
    T Lambda(V3<T> o) const {
        T absTan = std::fabs(TanTheta(o));
        if (std::isinf(absTan)) return T(0);
        T cp = CosPhi(o), sp = SinPhi(o);
        T alpha = std::sqrt(cp * cp * ax * ax + sp * sp * ay * ay);
        T a2t2 = alpha * absTan * (alpha * absTan);
        return (T(-1) + std::sqrt(T(1) + a2t2)) / T(2);
    }
    T G1(V3<T> o) const { return T(1) / (T(1) + Lambda(o)); }                    // :44-46
    T G(V3<T> o, V3<T> i) const { return T(1) / (T(1) + Lambda(o) + Lambda(i)); }  // :48-50
    // TrowbridgeReitzDistribution.cs:59-63
    T Pdf(V3<T> o, V3<T> n) const {
        if (!SameHemisphere(o, n)) return T(0);
        return G1(o) * std::max(T(0), dot(o, n)) * D(n) / std::fabs(o.z);
    }
    // TrowbridgeReitzDistribution.cs:70-100 (Heitz 2018 visible-normal sampling).  The
    // reference's MathF.ReciprocalSqrtEstimate is a platform-defined approximation; the
    // restatement uses the exact reciprocal square root.
    V3<T> Sample(V3<T> o, V2<T> p) const {
        bool flip = false;
        if (o.z < T(0)) { flip = true; o = -o; }
        V3<T> Vh = normalize(V3<T>(ax * o.x, ay * o.y, o.z));
        T lensq = Vh.x * Vh.x + Vh.y * Vh.y;
        V3<T> T1 = lensq > T(0) ? V3<T>(-Vh.y, Vh.x, T(0)) * (T(1) / std::sqrt(lensq)) : V3<T>(T(1), T(0), T(0));
        V3<T> T2 = cross(Vh, T1);
        T r = std::sqrt(p.x);
        T phi = T(2) * PI<T>() * p.y;
        T t1 = r * std::cos(phi);
        T t2 = r * std::sin(phi);
        T s = T(0.5) * (T(1) + Vh.z);
        t2 = (T(1) - s) * std::sqrt(T(1) - t1 * t1) + s * t2;
        V3<T> Nh = t1 * T1 + t2 * T2 + std::sqrt(std::max(T(0), T(1) - t1 * t1 - t2 * t2)) * Vh;
        V3<T> Ne = normalize(V3<T>(ax * Nh.x, ay * Nh.y, std::max(T(0), Nh.z)));
        return flip ? -Ne : Ne;
    }
};

}  // namespace ora

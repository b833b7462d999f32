// ORACLE -- test infrastructure only (see oracle_core.hpp for the rules that apply here).
//
// Scene model, ray queries, materials, emitters, environment map, camera and the PathTracer
// estimator restated from SeeSharp.  Ray queries are answered by a CPU BVH with the watertight
// ray/triangle test of Woop, Benthin and Wald (JCGT 2013) in the template precision.
#pragma once
#include "oracle_core.hpp"

#include <functional>
#include <memory>
#include <stdexcept>
#include <string>

namespace ora {

// ------------------------------------------------------------------------------------------
// System.Numerics.Matrix4x4 (row-vector convention: v' = v * M)
// ------------------------------------------------------------------------------------------
template <class T> struct M44 {
    T m[4][4] = {};  // m[row][col], row 0 = M11..M14
    static M44 Identity() { M44 r; for (int i = 0; i < 4; ++i) r.m[i][i] = T(1); return r; }
};
// Vector3.Transform(v, M): xyz of (v, 1) * M (no perspective division)
template <class T> inline V3<T> TransformPoint(V3<T> v, const M44<T>& M) {
    return {v.x * M.m[0][0] + v.y * M.m[1][0] + v.z * M.m[2][0] + M.m[3][0],
            v.x * M.m[0][1] + v.y * M.m[1][1] + v.z * M.m[2][1] + M.m[3][1],
            v.x * M.m[0][2] + v.y * M.m[1][2] + v.z * M.m[2][2] + M.m[3][2]};
}
// Vector4.Transform((v, 0), M), xyz part
template <class T> inline V3<T> TransformDir(V3<T> v, const M44<T>& M) {
    return {v.x * M.m[0][0] + v.y * M.m[1][0] + v.z * M.m[2][0],
            v.x * M.m[0][1] + v.y * M.m[1][1] + v.z * M.m[2][1],
            v.x * M.m[0][2] + v.y * M.m[1][2] + v.z * M.m[2][2]};
}
// Matrix inverse by the adjugate (cofactor) formula.  Returns false for a singular matrix,
// which Camera.cs:34-42 turns into an ArgumentException.
template <class T> inline bool Invert(const M44<T>& A, M44<T>& R) {
    const T(&a)[4][4] = A.m;
    T inv[16];
    const T* s = &a[0][0];
    inv[0] = s[5] * s[10] * s[15] - s[5] * s[11] * s[14] - s[9] * s[6] * s[15] + s[9] * s[7] * s[14] + s[13] * s[6] * s[11] - s[13] * s[7] * s[10];
    inv[4] = -s[4] * s[10] * s[15] + s[4] * s[11] * s[14] + s[8] * s[6] * s[15] - s[8] * s[7] * s[14] - s[12] * s[6] * s[11] + s[12] * s[7] * s[10];
    inv[8] = s[4] * s[9] * s[15] - s[4] * s[11] * s[13] - s[8] * s[5] * s[15] + s[8] * s[7] * s[13] + s[12] * s[5] * s[11] - s[12] * s[7] * s[9];
    inv[12] = -s[4] * s[9] * s[14] + s[4] * s[10] * s[13] + s[8] * s[5] * s[14] - s[8] * s[6] * s[13] - s[12] * s[5] * s[10] + s[12] * s[6] * s[9];
    inv[1] = -s[1] * s[10] * s[15] + s[1] * s[11] * s[14] + s[9] * s[2] * s[15] - s[9] * s[3] * s[14] - s[13] * s[2] * s[11] + s[13] * s[3] * s[10];
    inv[5] = s[0] * s[10] * s[15] - s[0] * s[11] * s[14] - s[8] * s[2] * s[15] + s[8] * s[3] * s[14] + s[12] * s[2] * s[11] - s[12] * s[3] * s[10];
    inv[9] = -s[0] * s[9] * s[15] + s[0] * s[11] * s[13] + s[8] * s[1] * s[15] - s[8] * s[3] * s[13] - s[12] * s[1] * s[11] + s[12] * s[3] * s[9];
    inv[13] = s[0] * s[9] * s[14] - s[0] * s[10] * s[13] - s[8] * s[1] * s[14] + s[8] * s[2] * s[13] + s[12] * s[1] * s[10] - s[12] * s[2] * s[9];
    inv[2] = s[1] * s[6] * s[15] - s[1] * s[7] * s[14] - s[5] * s[2] * s[15] + s[5] * s[3] * s[14] + s[13] * s[2] * s[7] - s[13] * s[3] * s[6];
    inv[6] = -s[0] * s[6] * s[15] + s[0] * s[7] * s[14] + s[4] * s[2] * s[15] - s[4] * s[3] * s[14] - s[12] * s[2] * s[7] + s[12] * s[3] * s[6];
    inv[10] = s[0] * s[5] * s[15] - s[0] * s[7] * s[13] - s[4] * s[1] * s[15] + s[4] * s[3] * s[13] + s[12] * s[1] * s[7] - s[12] * s[3] * s[5];
    inv[14] = -s[0] * s[5] * s[14] + s[0] * s[6] * s[13] + s[4] * s[1] * s[14] - s[4] * s[2] * s[13] - s[12] * s[1] * s[6] + s[12] * s[2] * s[5];
    inv[3] = -s[1] * s[6] * s[11] + s[1] * s[7] * s[10] + s[5] * s[2] * s[11] - s[5] * s[3] * s[10] - s[9] * s[2] * s[7] + s[9] * s[3] * s[6];
    inv[7] = s[0] * s[6] * s[11] - s[0] * s[7] * s[10] - s[4] * s[2] * s[11] + s[4] * s[3] * s[10] + s[8] * s[2] * s[7] - s[8] * s[3] * s[6];
    inv[11] = -s[0] * s[5] * s[11] + s[0] * s[7] * s[9] + s[4] * s[1] * s[11] - s[4] * s[3] * s[9] - s[8] * s[1] * s[7] + s[8] * s[3] * s[5];
    inv[15] = s[0] * s[5] * s[10] - s[0] * s[6] * s[9] - s[4] * s[1] * s[10] + s[4] * s[2] * s[9] + s[8] * s[1] * s[6] - s[8] * s[2] * s[5];
    T det = s[0] * inv[0] + s[1] * inv[4] + s[2] * inv[8] + s[3] * inv[12];
    if (!(std::fabs(det) >= std::numeric_limits<float>::denorm_min())) return false;
    T invDet = T(1) / det;
    for (int i = 0; i < 16; ++i) (&R.m[0][0])[i] = inv[i] * invDet;
    return true;
}
// Matrix4x4.CreatePerspectiveFieldOfView (right-handed), restated from its documented formula.
template <class T> inline M44<T> PerspectiveFov(T fov, T aspect, T nearP, T farP) {
    M44<T> r;
    T yScale = T(1) / std::tan(fov * T(0.5));
    T xScale = yScale / aspect;
    r.m[0][0] = xScale;
    r.m[1][1] = yScale;
    T negFarRange = farP / (nearP - farP);
    r.m[2][2] = negFarRange;
    r.m[2][3] = T(-1);
    r.m[3][2] = nearP * negFarRange;
    return r;
}

// ------------------------------------------------------------------------------------------
// Scene data
// ------------------------------------------------------------------------------------------
// ImageTexture.cs: nearest texel, Repeat (default) or Clamp borders.  Image rows top to bottom.
template <class T> struct Texture {
    int w = 0, h = 0, channels = 1, border = 0;  // border: 0 = Repeat, 1 = Clamp
    std::vector<T> data;
    // ImageTexture.cs:27-37, 40-44
    void Texel(V2<T> uv, int& col, int& row) const {
        col = int(uv.x * T(w));
        row = int(uv.y * T(h));
        if (border == 0) {
            row = (row % h + h) % h;
            col = (col % w + w) % w;
        } else {
            row = std::clamp(row, 0, h - 1);
            col = std::clamp(col, 0, w - 1);
        }
    }
};
// A TextureRgb / TextureMono: constant value or image (TextureRgb.cs:29-35, TextureMono.cs:32-38)
template <class T> struct TexRef {
    Rgb<T> c;
    int tex = -1;
};

enum MaterialType { MAT_DIFFUSE = 0, MAT_GENERIC = 1 };
template <class T> struct Material {
    int type = MAT_DIFFUSE;
    TexRef<T> baseColor;      // Diffuse/GenericMaterial.Parameters.BaseColor
    TexRef<T> roughness;      // GenericMaterial.Parameters.Roughness (channel r)
    T metallic = 0, specularTint = 1, anisotropic = 0, specularTransmittance = 0, ior = T(1.45f);
    bool transmitter = false;  // DiffuseMaterial.Parameters.Transmitter
};

template <class T> struct Mesh {
    std::vector<V3<T>> V;
    std::vector<int> I;
    std::vector<V3<T>> N;   // optional per-vertex shading normals
    std::vector<V2<T>> UV;  // optional per-vertex texture coordinates
    int material = -1;
    std::vector<V3<T>> faceNormals;
    int numFaces() const { return int(I.size() / 3); }
    void Tri(int f, V3<T>& a, V3<T>& b, V3<T>& c) const { a = V[I[3 * f]]; b = V[I[3 * f + 1]]; c = V[I[3 * f + 2]]; }
    // Position from barycentrics: (u, v) weight the second and third vertex.  This is the
    // convention of Mesh.ComputeErrorOffset (Geometry/Mesh.cs:55-57) and Mesh.ComputePosition.
    V3<T> Position(int f, V2<T> b) const {
        V3<T> v1, v2, v3; Tri(f, v1, v2, v3);
        return b.x * v2 + b.y * v3 + (T(1) - b.x - b.y) * v1;
    }
    // Geometry/Mesh.cs:50-60
    T ErrorOffset(int f, V2<T> b) const {
        V3<T> v1, v2, v3; Tri(f, v1, v2, v3);
        V3<T> e = vabs(b.x * v2) + vabs(b.y * v3) + vabs((T(1) - b.x - b.y) * v1);
        return length(e) * T(32.0f) * T(1.19209e-07f);
    }
    // TinyEmbree Hit.ShadingNormal: barycentric interpolation of the vertex normals, normalized;
    // the face normal when the mesh has none.  (Unpinned: TinyEmbree is not vendored.)
    V3<T> ShadingNormal(int f, V2<T> b) const {
        if (N.empty()) return faceNormals[f];
        V3<T> n1 = N[I[3 * f]], n2 = N[I[3 * f + 1]], n3 = N[I[3 * f + 2]];
        return normalize(b.x * n2 + b.y * n3 + (T(1) - b.x - b.y) * n1);
    }
    // TinyEmbree Hit.TextureCoordinates: interpolated UVs; the barycentric coordinates when the
    // mesh has none.  (Unpinned.)
    V2<T> TexCoords(int f, V2<T> b) const {
        if (UV.empty()) return b;
        V2<T> t1 = UV[I[3 * f]], t2 = UV[I[3 * f + 1]], t3 = UV[I[3 * f + 2]];
        T w = T(1) - b.x - b.y;
        return {b.x * t2.x + b.y * t3.x + w * t1.x, b.x * t2.y + b.y * t3.y + w * t1.y};
    }
};

// Geometry/SurfacePoint.cs (wrapper around TinyEmbree.Hit)
template <class T> struct SurfacePoint {
    V3<T> position, normal, shadingNormal;
    V2<T> bary, uv;
    int mesh = -1;
    int prim = -1;
    T errorOffset = 0;
    T distance = 0;
    bool valid = false;
};

// Shading/Emitters: DiffuseEmitter (exponent < 0) or GlossyEmitter (exponent >= 0), one per
// triangle (DiffuseEmitter.cs:21-31, GlossyEmitter.cs:24-34).
template <class T> struct Emitter {
    int mesh = -1, face = -1;
    Rgb<T> radiance;
    T exponent = T(-1);
    T invArea = 0;          // Triangle.cs:132-138
    T normalization = 0;    // GlossyEmitter.cs:14
    bool glossy() const { return exponent >= T(0); }
    // DiffuseEmitter.cs:33-37, GlossyEmitter.cs:36-40
    Rgb<T> EmittedRadiance(const SurfacePoint<T>& p, V3<T> dir) const {
        if (!glossy()) {
            if (dot(p.shadingNormal, dir) < T(0)) return Rgb<T>::Black();
            return radiance;
        }
        T cosine = dot(p.shadingNormal, dir) / length(dir);
        if (cosine < T(0)) return Rgb<T>::Black();
        return radiance * std::pow(cosine, exponent) * normalization;
    }
};

template <class T> struct BackgroundSample { Rgb<T> Weight; V3<T> Direction; T Pdf; };

// Shading/Background/EnvironmentMap.cs
template <class T> struct EnvMap {
    int w = 0, h = 0;
    std::vector<Rgb<T>> img;
    RegularGrid2d<T> grid;
    // RgbImage.GetPixel; out-of-range coordinates are clamped (unpinned: SimpleImageIO).
    Rgb<T> GetPixel(int col, int row) const {
        col = std::clamp(col, 0, w - 1);
        row = std::clamp(row, 0, h - 1);
        return img[size_t(row) * w + col];
    }
    // EnvironmentMap.cs:139-156 (without MIS compensation)
    void Build() {
        grid.Init(w, h);
        for (int r = 0; r < h; ++r)
            for (int c = 0; c < w; ++c) grid.Splat(c, r, GetPixel(c, r).Luminance());
        grid.Normalize();
    }
    // EnvironmentMap.cs:158-166
    static V2<T> WorldToSpherical(V3<T> d) {
        d = normalize(d);
        V2<T> sp(std::atan2(d.z, d.x), std::atan2(std::sqrt(d.x * d.x + d.z * d.z), d.y));
        if (sp.x < T(0)) sp.x += PI<T>() * T(2);
        return sp;
    }
    // EnvironmentMap.cs:168-175
    static V3<T> SphericalToWorld(V2<T> s) {
        T st = std::sin(s.y);
        return {st * std::cos(s.x), std::cos(s.y), st * std::sin(s.x)};
    }
    static V2<T> SphericalToPixel(V2<T> s) { return {s.x / (T(2) * PI<T>()), s.y / PI<T>()}; }  // :177-178
    static V2<T> PixelToSpherical(V2<T> p) { return {p.x * T(2) * PI<T>(), p.y * PI<T>()}; }    // :180-181
    // EnvironmentMap.cs:19-26
    Rgb<T> EmittedRadiance(V3<T> dir) const {
        V2<T> px = SphericalToPixel(WorldToSpherical(dir));
        T col = px.x * T(w), row = px.y * T(h);
        return GetPixel(int(col), int(row));
    }
    // EnvironmentMap.cs:40-73
    BackgroundSample<T> SampleDirection(V2<T> primary) const {
        bool ok;
        V2<T> pp = grid.Sample(primary, ok);
        BackgroundSample<T> s;
        if (!ok) { s.Pdf = 0; s.Weight = Rgb<T>::Black(); s.Direction = V3<T>(0, 1, 0); return s; }
        T pdf = grid.Pdf(pp);
        V2<T> sph = PixelToSpherical(pp);
        V3<T> dir = SphericalToWorld(sph);
        T jac = std::sin(sph.y) * PI<T>() * PI<T>() * T(2);
        if (jac == T(0)) { s.Direction = dir; s.Pdf = 0; s.Weight = Rgb<T>::Black(); return s; }
        pdf /= jac;
        s.Weight = GetPixel(int(pp.x * T(w)), int(pp.y * T(h))) / pdf;
        s.Direction = dir;
        s.Pdf = pdf;
        return s;
    }
    // EnvironmentMap.cs:81-85
    T DirectionPdf(V3<T> dir) const {
        V2<T> sph = WorldToSpherical(dir);
        V2<T> px = SphericalToPixel(sph);
        return grid.Pdf(px) / (std::sin(sph.y) * PI<T>() * PI<T>() * T(2));
    }
};

// Cameras/PerspectiveCamera.cs (pinhole; lens radius is always zero in the reference)
template <class T> struct Camera {
    M44<T> worldToCamera, cameraToWorld, cameraToView, viewToCamera;
    T fovRadians = 0;
    int width = 0, height = 0;
    bool Set(const M44<T>& w2c, T fovDeg) {  // PerspectiveCamera.cs:32-37, Camera.cs:34-42
        worldToCamera = w2c;
        fovRadians = fovDeg * PI<T>() / T(180);
        return Invert(worldToCamera, cameraToWorld);
    }
    void UpdateResolution(int W, int H) {  // PerspectiveCamera.cs:42-52
        width = W; height = H;
        T aspect = T(W) / T(H);
        cameraToView = PerspectiveFov(fovRadians, aspect, T(0.001f), T(1000.0f));
        Invert(cameraToView, viewToCamera);
    }
    // PerspectiveCamera.cs:64-102 (returns origin and normalized direction)
    void GenerateRay(V2<T> film, V3<T>& org, V3<T>& dir) const {
        V3<T> view(T(2) * film.x / T(width) - T(1), T(1) - T(2) * film.y / T(height), T(0));
        V3<T> local = TransformPoint(view, viewToCamera);
        V3<T> d = TransformDir(local, cameraToWorld);
        org = TransformPoint(V3<T>(0, 0, 0), cameraToWorld);
        dir = normalize(d);
    }
};

// ------------------------------------------------------------------------------------------
// Ray queries (TinyEmbree Raytracer semantics; see the notes in the header comment)
// ------------------------------------------------------------------------------------------
template <class T> struct Ray { V3<T> org, dir; T tmin = 0, tmax = std::numeric_limits<T>::infinity(); };
template <class T> struct HitRec { T t; T u, v; int tri = -1; };

// Watertight ray/triangle intersection, Woop, Benthin and Wald, JCGT 2(1), 2013.  Returns true
// with (t, u, v) where u weights the second and v the third vertex.
template <class T> struct RayPre {
    int kx, ky, kz;
    T Sx, Sy, Sz;
    explicit RayPre(V3<T> d) {
        T ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
        kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
        kx = (kz + 1) % 3;
        ky = (kx + 1) % 3;
        if (d[kz] < T(0)) std::swap(kx, ky);
        Sx = d[kx] / d[kz];
        Sy = d[ky] / d[kz];
        Sz = T(1) / d[kz];
    }
};
template <class T> inline bool IntersectTri(const Ray<T>& r, const RayPre<T>& p, V3<T> v0, V3<T> v1, V3<T> v2, T tmax, T& t, T& u, T& v) {
    V3<T> A = v0 - r.org, B = v1 - r.org, C = v2 - r.org;
    T Ax = A[p.kx] - p.Sx * A[p.kz], Ay = A[p.ky] - p.Sy * A[p.kz];
    T Bx = B[p.kx] - p.Sx * B[p.kz], By = B[p.ky] - p.Sy * B[p.kz];
    T Cx = C[p.kx] - p.Sx * C[p.kz], Cy = C[p.ky] - p.Sy * C[p.kz];
    T U = Cx * By - Cy * Bx;
    T V = Ax * Cy - Ay * Cx;
    T W = Bx * Ay - By * Ax;
    if (std::is_same<T, float>::value && (U == T(0) || V == T(0) || W == T(0))) {
        double CxBy = double(Cx) * double(By), CyBx = double(Cy) * double(Bx);
        U = T(CxBy - CyBx);
        double AxCy = double(Ax) * double(Cy), AyCx = double(Ay) * double(Cx);
        V = T(AxCy - AyCx);
        double BxAy = double(Bx) * double(Ay), ByAx = double(By) * double(Ax);
        W = T(BxAy - ByAx);
    }
    if ((U < T(0) || V < T(0) || W < T(0)) && (U > T(0) || V > T(0) || W > T(0))) return false;
    T det = U + V + W;
    if (det == T(0)) return false;
    T Az = p.Sz * A[p.kz], Bz = p.Sz * B[p.kz], Cz = p.Sz * C[p.kz];
    T Tn = U * Az + V * Bz + W * Cz;
    T rcp = T(1) / det;
    T tt = Tn * rcp;
    if (!(tt > r.tmin) || !(tt < tmax)) return false;
    t = tt;
    u = V * rcp;
    v = W * rcp;
    return true;
}

struct BvhNode {
    float lo[3], hi[3];
    int left = -1, right = -1;  // inner node children
    int first = 0, count = 0;   // leaf range into the triangle order (count > 0 for leaves)
};

template <class T> struct Scene {
    std::vector<Texture<T>> textures;
    std::vector<Material<T>> materials;
    std::vector<Mesh<T>> meshes;
    std::vector<Emitter<T>> emitters;
    std::unique_ptr<EnvMap<T>> env;
    Camera<T> camera;
    bool cameraSet = false;
    // global triangle table (meshes concatenated)
    std::vector<int> triMesh, triFace;
    std::vector<int> meshTriOffset;
    std::vector<int> triEmitter;  // emitter index per global triangle, or -1 (Scene.cs:148-163)
    std::vector<BvhNode> nodes;
    std::vector<int> order;       // triangle ids in leaf order
    std::vector<V3<T>> tv0, tv1, tv2;  // per global triangle
    bool committed = false;
    int width = 0, height = 0;

    Rgb<T> TexLookupRgb(const TexRef<T>& r, V2<T> uv) const {
        if (r.tex < 0) return r.c;
        const Texture<T>& t = textures[r.tex];
        int col, row; t.Texel(uv, col, row);
        size_t i = (size_t(row) * t.w + col) * t.channels;
        if (t.channels == 1) return Rgb<T>(t.data[i]);
        return {t.data[i], t.data[i + 1], t.data[i + 2]};
    }
    T TexLookupMono(const TexRef<T>& r, V2<T> uv) const {
        if (r.tex < 0) return r.c.r;
        const Texture<T>& t = textures[r.tex];
        int col, row; t.Texel(uv, col, row);
        return t.data[(size_t(row) * t.w + col) * t.channels];
    }

    // Scene.Prepare (Scene.cs:103-164): validity, acceleration structure, camera resolution,
    // emitter lookup table.
    std::string Commit(int W, int H) {
        if (meshes.empty()) return "No meshes in the scene.";
        for (size_t i = 0; i < meshes.size(); ++i)
            if (meshes[i].material < 0) return "Mesh[" + std::to_string(i) + "] does not have a material.";
        if (!cameraSet) return "Camera not set.";
        if (emitters.empty() && !env) return "No emitters and no background in the scene.";
        width = W; height = H;
        triMesh.clear(); triFace.clear(); meshTriOffset.clear();
        for (size_t m = 0; m < meshes.size(); ++m) {
            meshTriOffset.push_back(int(triMesh.size()));
            for (int f = 0; f < meshes[m].numFaces(); ++f) { triMesh.push_back(int(m)); triFace.push_back(f); }
        }
        int nt = int(triMesh.size());
        triEmitter.assign(nt, -1);
        for (size_t e = 0; e < emitters.size(); ++e) triEmitter[meshTriOffset[emitters[e].mesh] + emitters[e].face] = int(e);
        tv0.resize(nt); tv1.resize(nt); tv2.resize(nt);
        for (int g = 0; g < nt; ++g) meshes[triMesh[g]].Tri(triFace[g], tv0[g], tv1[g], tv2[g]);
        BuildBvh();
        camera.UpdateResolution(W, H);
        committed = true;
        return "";
    }

    // Binned-SAH BVH over all triangles (CPU).
    void BuildBvh() {
        int nt = int(tv0.size());
        order.resize(nt);
        std::vector<float> clo(3 * size_t(nt)), chi(3 * size_t(nt)), cen(3 * size_t(nt));
        for (int g = 0; g < nt; ++g) {
            order[g] = g;
            for (int k = 0; k < 3; ++k) {
                float a = float(tv0[g][k]), b = float(tv1[g][k]), c = float(tv2[g][k]);
                clo[3 * size_t(g) + k] = std::min(a, std::min(b, c));
                chi[3 * size_t(g) + k] = std::max(a, std::max(b, c));
                cen[3 * size_t(g) + k] = 0.5f * (clo[3 * size_t(g) + k] + chi[3 * size_t(g) + k]);
            }
        }
        nodes.clear();
        nodes.reserve(2 * size_t(nt) + 1);
        struct Item { int node, first, count; };
        std::vector<Item> stack;
        nodes.push_back(BvhNode());
        stack.push_back({0, 0, nt});
        const int kBins = 16;
        while (!stack.empty()) {
            Item it = stack.back(); stack.pop_back();
            BvhNode& nd = nodes[it.node];
            float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
            float clo3[3] = {1e30f, 1e30f, 1e30f}, chi3[3] = {-1e30f, -1e30f, -1e30f};
            for (int i = it.first; i < it.first + it.count; ++i) {
                int g = order[i];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], clo[3 * size_t(g) + k]);
                    hi[k] = std::max(hi[k], chi[3 * size_t(g) + k]);
                    clo3[k] = std::min(clo3[k], cen[3 * size_t(g) + k]);
                    chi3[k] = std::max(chi3[k], cen[3 * size_t(g) + k]);
                }
            }
            for (int k = 0; k < 3; ++k) { nd.lo[k] = lo[k]; nd.hi[k] = hi[k]; }
            if (it.count <= 2) { nd.first = it.first; nd.count = it.count; continue; }
            // SAH over binned centroids
            float bestCost = 1e30f; int bestAxis = -1, bestSplit = -1;
            for (int ax = 0; ax < 3; ++ax) {
                float ext = chi3[ax] - clo3[ax];
                if (ext <= 0) continue;
                int cnt[kBins] = {};
                float blo[kBins][3], bhi[kBins][3];
                for (int b = 0; b < kBins; ++b) for (int k = 0; k < 3; ++k) { blo[b][k] = 1e30f; bhi[b][k] = -1e30f; }
                for (int i = it.first; i < it.first + it.count; ++i) {
                    int g = order[i];
                    int b = std::min(kBins - 1, int(kBins * (cen[3 * size_t(g) + ax] - clo3[ax]) / ext));
                    cnt[b]++;
                    for (int k = 0; k < 3; ++k) { blo[b][k] = std::min(blo[b][k], clo[3 * size_t(g) + k]); bhi[b][k] = std::max(bhi[b][k], chi[3 * size_t(g) + k]); }
                }
                float rA[kBins]; int rC[kBins];
                float alo[3] = {1e30f, 1e30f, 1e30f}, ahi[3] = {-1e30f, -1e30f, -1e30f}; int ac = 0;
                for (int b = kBins - 1; b > 0; --b) {
                    ac += cnt[b];
                    for (int k = 0; k < 3; ++k) { alo[k] = std::min(alo[k], blo[b][k]); ahi[k] = std::max(ahi[k], bhi[b][k]); }
                    float dx = std::max(0.f, ahi[0] - alo[0]), dy = std::max(0.f, ahi[1] - alo[1]), dz = std::max(0.f, ahi[2] - alo[2]);
                    rA[b] = dx * dy + dy * dz + dz * dx; rC[b] = ac;
                }
                float llo[3] = {1e30f, 1e30f, 1e30f}, lhi[3] = {-1e30f, -1e30f, -1e30f}; int lc = 0;
                for (int b = 0; b < kBins - 1; ++b) {
                    lc += cnt[b];
                    for (int k = 0; k < 3; ++k) { llo[k] = std::min(llo[k], blo[b][k]); lhi[k] = std::max(lhi[k], bhi[b][k]); }
                    if (lc == 0 || rC[b + 1] == 0) continue;
                    float dx = std::max(0.f, lhi[0] - llo[0]), dy = std::max(0.f, lhi[1] - llo[1]), dz = std::max(0.f, lhi[2] - llo[2]);
                    float cost = (dx * dy + dy * dz + dz * dx) * lc + rA[b + 1] * rC[b + 1];
                    if (cost < bestCost) { bestCost = cost; bestAxis = ax; bestSplit = b; }
                }
            }
            int mid;
            if (bestAxis < 0) {
                mid = it.first + it.count / 2;
            } else {
                float ext = chi3[bestAxis] - clo3[bestAxis];
                auto pred = [&](int g) {
                    int b = std::min(kBins - 1, int(kBins * (cen[3 * size_t(g) + bestAxis] - clo3[bestAxis]) / ext));
                    return b <= bestSplit;
                };
                mid = int(std::partition(order.begin() + it.first, order.begin() + it.first + it.count, pred) - order.begin());
                if (mid == it.first || mid == it.first + it.count) mid = it.first + it.count / 2;
            }
            int l = int(nodes.size()), r = l + 1;
            nodes.push_back(BvhNode()); nodes.push_back(BvhNode());
            nodes[it.node].left = l; nodes[it.node].right = r;
            stack.push_back({l, it.first, mid - it.first});
            stack.push_back({r, mid, it.first + it.count - mid});
        }
    }

    static bool BoxHit(const BvhNode& n, V3<T> org, V3<T> inv, T tmin, T tmax) {
        T t0 = tmin, t1 = tmax;
        for (int k = 0; k < 3; ++k) {
            T a = (T(n.lo[k]) - org[k]) * inv[k];
            T b = (T(n.hi[k]) - org[k]) * inv[k];
            if (a > b) std::swap(a, b);
            // NaN-safe (0 * inf) handling: a NaN bound never shrinks the interval
            if (a > t0) t0 = a;
            if (b < t1) t1 = b;
        }
        return t0 <= t1;
    }

    // Closest hit.  Ties in t resolve to the smaller global triangle id.
    HitRec<T> Intersect(const Ray<T>& r, bool anyHit) const {
        HitRec<T> best; best.t = r.tmax;
        RayPre<T> pre(r.dir);
        V3<T> inv(T(1) / r.dir.x, T(1) / r.dir.y, T(1) / r.dir.z);
        int stack[128]; int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const BvhNode& n = nodes[stack[--sp]];
            if (!BoxHit(n, r.org, inv, r.tmin, best.t)) continue;
            if (n.count > 0) {
                for (int i = n.first; i < n.first + n.count; ++i) {
                    int g = order[i];
                    T t, u, v;
                    // ">= best.t" must still accept an equal-t hit with a smaller id
                    if (IntersectTri(r, pre, tv0[g], tv1[g], tv2[g], std::nextafter(best.t, std::numeric_limits<T>::infinity()), t, u, v)) {
                        if (t < best.t || (t == best.t && (best.tri < 0 || g < best.tri))) {
                            best.t = t; best.u = u; best.v = v; best.tri = g;
                            if (anyHit) return best;
                        }
                    }
                }
            } else {
                if (sp + 2 > 128) throw std::runtime_error("bvh stack overflow");
                stack[sp++] = n.left;
                stack[sp++] = n.right;
            }
        }
        return best;
    }

    // FP64 brute force over all triangles (intersection parity reference)
    HitRec<double> IntersectBrute64(V3<double> org, V3<double> dir, double tmin) const {
        Ray<double> r; r.org = org; r.dir = dir; r.tmin = tmin;
        RayPre<double> pre(dir);
        HitRec<double> best; best.t = std::numeric_limits<double>::infinity();
        for (size_t g = 0; g < tv0.size(); ++g) {
            V3<double> a(tv0[g].x, tv0[g].y, tv0[g].z), b(tv1[g].x, tv1[g].y, tv1[g].z), c(tv2[g].x, tv2[g].y, tv2[g].z);
            double t, u, v;
            if (IntersectTri<double>(r, pre, a, b, c, best.t, t, u, v)) { best.t = t; best.u = u; best.v = v; best.tri = int(g); }
        }
        return best;
    }

    // FP64 closest hit over the BVH and the distance of the runner-up surface (the nearest hit of
    // any other triangle), for the intersection parity screening of near-ties.  Ties in t resolve
    // to the smaller global triangle id, as in Intersect.
    void IntersectTwo64(V3<double> org, V3<double> dir, double tmin, double tmax, HitRec<double>& best, double& second) const {
        Ray<double> r; r.org = org; r.dir = dir; r.tmin = tmin; r.tmax = tmax;
        RayPre<double> pre(dir);
        V3<double> inv(1.0 / dir.x, 1.0 / dir.y, 1.0 / dir.z);
        best = HitRec<double>(); best.t = tmax; best.tri = -1;
        second = tmax;
        if (nodes.empty()) return;
        int stack[128]; int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const BvhNode& n = nodes[stack[--sp]];
            if (!Scene<double>::BoxHit(n, org, inv, tmin, second)) continue;
            if (n.count > 0) {
                for (int i = n.first; i < n.first + n.count; ++i) {
                    int g = order[i];
                    V3<double> a(tv0[g].x, tv0[g].y, tv0[g].z), b(tv1[g].x, tv1[g].y, tv1[g].z), c(tv2[g].x, tv2[g].y, tv2[g].z);
                    double t, u, v;
                    if (!IntersectTri<double>(r, pre, a, b, c, std::nextafter(second, std::numeric_limits<double>::infinity()), t, u, v)) continue;
                    if (best.tri < 0 || t < best.t || (t == best.t && g < best.tri)) {
                        if (best.tri >= 0) second = best.t;
                        best.t = t; best.u = u; best.v = v; best.tri = g;
                    } else if (t < second) {
                        second = t;
                    }
                }
            } else {
                if (sp + 2 > 128) throw std::runtime_error("bvh stack overflow");
                stack[sp++] = n.left;
                stack[sp++] = n.right;
            }
        }
    }

    SurfacePoint<T> MakePoint(int g, V2<T> bary, T dist) const { return MakePointMF(triMesh[g], triFace[g], bary, dist); }
    SurfacePoint<T> MakePointMF(int mesh, int f, V2<T> bary, T dist) const {
        const Mesh<T>& m = meshes[mesh];
        SurfacePoint<T> p;
        p.valid = true;
        p.mesh = mesh;
        p.prim = f;
        p.bary = bary;
        p.position = m.Position(f, bary);
        p.normal = m.faceNormals[f];
        p.shadingNormal = m.ShadingNormal(f, bary);
        p.uv = m.TexCoords(f, bary);
        p.errorOffset = m.ErrorOffset(f, bary);
        p.distance = dist;
        return p;
    }

    // Raytracer.Trace (PathTracer.cs:319)
    SurfacePoint<T> Trace(const Ray<T>& r) const {
        HitRec<T> h = Intersect(r, false);
        if (h.tri < 0) return SurfacePoint<T>();
        return MakePoint(h.tri, V2<T>(h.u, h.v), h.t);
    }
    // Raytracer.SpawnRay (PathTracer.cs:528): offset along the face normal to the side of dir.
    static V3<T> OffsetPoint(const SurfacePoint<T>& p, V3<T> dir) {
        T sign = dot(dir, p.normal) < T(0) ? T(-1) : T(1);
        return p.position + (sign * p.errorOffset) * p.normal;
    }
    static Ray<T> SpawnRay(const SurfacePoint<T>& p, V3<T> dir) {
        Ray<T> r; r.org = OffsetPoint(p, dir); r.dir = dir; r.tmin = 0;
        return r;
    }
    // Raytracer.IsOccluded(from, to) (PathTracer.cs:467): segment between the two offset points,
    // shortened by a relative 1e-5 at the far end.
    bool IsOccluded(const SurfacePoint<T>& from, const SurfacePoint<T>& to) const {
        V3<T> d = to.position - from.position;
        V3<T> o = OffsetPoint(from, d);
        V3<T> e = OffsetPoint(to, -d);
        Ray<T> r; r.org = o; r.dir = e - o; r.tmin = 0; r.tmax = T(1) - T(1e-5f);
        return Intersect(r, true).tri >= 0;
    }
    // Raytracer.LeavesScene(from, dir) (PathTracer.cs:428)
    bool LeavesScene(const SurfacePoint<T>& from, V3<T> dir) const {
        Ray<T> r = SpawnRay(from, dir);
        return Intersect(r, true).tri < 0;
    }
};

// ------------------------------------------------------------------------------------------
// Shading context and materials
// ------------------------------------------------------------------------------------------
// Shading/Materials/ShadingContext.cs:3-27
template <class T> struct ShadingContext {
    SurfacePoint<T> point;
    V3<T> normal, tangent, binormal, outDir, outDirWorld;
    bool onLight = false;  // ShadingContext.IsOnLightSubpath
    ShadingContext(const SurfacePoint<T>& p, V3<T> outW, bool onLightSubpath = false) : point(p), onLight(onLightSubpath) {
        normal = p.shadingNormal;
        ComputeBasisVectors(normal, tangent, binormal);
        outDir = WorldToShading(normal, tangent, binormal, outW);
        outDirWorld = outW;
    }
    V3<T> ToShading(V3<T> d) const { return WorldToShading(normal, tangent, binormal, d); }
    V3<T> ToWorld(V3<T> d) const { return ShadingToWorld(normal, tangent, binormal, d); }
};

template <class T> struct BsdfSample { V3<T> Direction; T Pdf = 0, PdfReverse = 0; Rgb<T> Weight; };
template <class T> struct ComponentWeights { T pdfs[3] = {}, weights[3] = {}, pdfsRev[3] = {}, weightsRev[3] = {}; int n = 0; };

// Material.cs:127-134
template <class T> inline bool ShouldReflect(const SurfacePoint<T>& hit, V3<T> outDir, V3<T> inDir) {
    T a = dot(outDir, hit.normal), b = dot(inDir, hit.normal);
    return a * b >= T(0);
}

template <class T> struct MaterialEval {
    const Scene<T>& scene;
    const Material<T>& mat;
    // parameter overrides for derivative evaluation (NULL: look up the material)
    const Rgb<T>* baseOv = nullptr;
    const T* roughOv = nullptr;
    Rgb<T> Base(V2<T> uv) const { return baseOv ? *baseOv : scene.TexLookupRgb(mat.baseColor, uv); }
    T Rough(V2<T> uv) const { return roughOv ? *roughOv : scene.TexLookupMono(mat.roughness, uv); }

    struct Local {  // GenericMaterial.cs:343-352
        Rgb<T> colorTint, specularTint;
        T roughness, alphaX, alphaY;
        Rgb<T> diffuseReflectance, retroReflectance, specularTransmittance, specularReflectanceAtNormal;
    };
    // GenericMaterial.cs:354-381
    Local ComputeLocalParams(const ShadingContext<T>& c) const {
        Local r;
        Rgb<T> base = Base(c.point.uv);
        T lum = base.Luminance();
        r.colorTint = lum > T(0) ? (base / lum) : Rgb<T>::White();
        r.specularTint = lerp(mat.specularTint, Rgb<T>::White(), r.colorTint);
        r.roughness = Rough(c.point.uv);
        T aspect = std::sqrt(T(1) - mat.anisotropic * T(.9f));
        r.alphaX = std::max(T(.001f), r.roughness * r.roughness / aspect);
        r.alphaY = std::max(T(.001f), r.roughness * r.roughness * aspect);
        r.specularReflectanceAtNormal = lerp(mat.metallic, SchlickR0FromEta(mat.ior) * r.specularTint, base);
        T dw = (T(1) - mat.metallic) * (T(1) - mat.specularTransmittance);
        r.diffuseReflectance = base * dw;
        r.specularTransmittance = mat.specularTransmittance * base;
        r.retroReflectance = base * dw;
        return r;
    }

    // GenericMaterial.cs:152-338
    void GenericValueAndPdf(const ShadingContext<T>& c, V3<T> inDir, const Local& lp, Rgb<T>& value, T& pdf, T& pdfRev, ComponentWeights<T>* cw) const {
        GGX<T> ndf{lp.alphaX, lp.alphaY};
        const V3<T> o = c.outDir;
        T cosThetaO = std::fabs(o.z), cosThetaI = std::fabs(inDir.z);
        bool sameGeo = ShouldReflect(c.point, c.outDirWorld, c.ToWorld(inDir));
        Rgb<T> bsdf = Rgb<T>::Black();
        T pf[3] = {0, 0, 0}, pr[3] = {0, 0, 0};
        T fresnelOut = SchlickWeight(cosThetaO), fresnelIn = SchlickWeight(cosThetaI);
        if (SameHemisphere(o, inDir)) {
            if (sameGeo) bsdf = bsdf + lp.diffuseReflectance / PI<T>() * (T(1) - fresnelOut * T(0.5f)) * (T(1) - fresnelIn * T(0.5f));
            pf[0] = cosThetaI / PI<T>();
            pr[0] = cosThetaO / PI<T>();
        }
        V3<T> h = o + inDir;
        if (h != V3<T>(0, 0, 0)) {
            h = normalize(h);
            T cIn = dot(inDir, h);
            T Rr = T(2) * lp.roughness * cIn * cIn;
            if (SameHemisphere(o, inDir) && sameGeo)
                bsdf = bsdf + lp.retroReflectance / PI<T>() * Rr * (fresnelOut + fresnelIn + fresnelOut * fresnelIn * (Rr - T(1)));
            if (cosThetaI != T(0) && cosThetaO != T(0)) {
                T cOut = dot(o, h);
                if (SameHemisphere(o, inDir) && sameGeo && cIn * cOut > T(0)) {
                    T cosHT = dot(inDir, (h.z < T(0)) ? -h : h);
                    Rgb<T> diel(FresnelDielectric(cosHT, T(1), mat.ior));
                    Rgb<T> schlick = SchlickFresnel(lp.specularReflectanceAtNormal, cosHT);
                    Rgb<T> fres = lerp(mat.metallic, diel, schlick);
                    bsdf = bsdf + lp.specularTint * ndf.D(h) * ndf.G(o, inDir) * fres / (T(4) * cosThetaI * cosThetaO);
                }
                T jf = std::fabs(T(4) * cOut), jr = std::fabs(T(4) * cIn);
                if (jf != T(0) && jr != T(0)) {
                    pf[1] = ndf.Pdf(o, h) / jf;
                    pr[1] = ndf.Pdf(inDir, h) / jr;
                }
            }
        }
        T eta = o.z > T(0) ? mat.ior : (T(1) / mat.ior);
        V3<T> ht = o + inDir * eta;
        V3<T> htIn(0, 0, 0);
        if (cosThetaO != T(0) && cosThetaI != T(0) && ht != V3<T>(0, 0, 0) && mat.specularTransmittance > T(0)) {
            ht = normalize(ht);
            ht = (ht.z < T(0)) ? -ht : ht;
            T cOut = dot(o, ht), cIn = dot(inDir, ht);
            T sqrtDenom = cOut + eta * cIn;
            if (!SameHemisphere(o, inDir) && cOut * cIn < T(0)) {
                Rgb<T> F(FresnelDielectric(cOut, T(1), mat.ior));
                T factor = c.onLight ? T(1) / eta : T(1);  // GenericMaterial.cs:255
                V3<T> wh = (!SameHemisphere(o, ht)) ? -ht : ht;
                T num = ndf.D(wh) * ndf.G(o, inDir);
                num *= eta * eta * std::max(T(0), dot(inDir, -wh)) * std::max(T(0), dot(o, wh));
                num *= factor * factor;
                T den = inDir.z * o.z * sqrtDenom * sqrtDenom;
                bsdf = bsdf + (Rgb<T>::White() - F) * lp.specularTransmittance * std::fabs(num / den);
            }
            if (sqrtDenom != T(0)) {
                V3<T> wh = (!SameHemisphere(o, ht)) ? -ht : ht;
                T jac = eta * eta * std::max(T(0), dot(inDir, -wh)) / (sqrtDenom * sqrtDenom);
                pf[2] += ndf.Pdf(o, wh) * jac;
            }
            T etaIn = inDir.z > T(0) ? mat.ior : (T(1) / mat.ior);
            htIn = o * etaIn + inDir;
            htIn = normalize(htIn);
            htIn = (htIn.z < T(0)) ? -htIn : htIn;
            if (htIn != V3<T>(0, 0, 0)) {
                V3<T> wh = (!SameHemisphere(inDir, htIn)) ? -htIn : htIn;
                T sdIn = dot(htIn, inDir) + etaIn * dot(o, htIn);
                if (sdIn != T(0)) {
                    T jac = etaIn * etaIn * std::max(T(0), dot(o, -wh)) / (sdIn * sdIn);
                    pr[2] += ndf.Pdf(inDir, wh) * jac;
                }
            }
        }
        T schlickF = SchlickFresnel(lp.specularReflectanceAtNormal, std::fabs(o.z)).Average();
        T diffuseBias = std::max(T(1) - schlickF, T(0.75f));
        T dw = diffuseBias * (T(1) - mat.metallic) * (T(1) - mat.specularTransmittance);
        T fresnelR = FresnelDielectric(dot(o, (h.z < T(0)) ? -h : h), T(1), mat.ior);
        T selR = (T(1) - dw) * (T(1) - (T(1) - fresnelR) * mat.specularTransmittance);
        T fresnelT = FresnelDielectric(dot(o, ht), T(1), mat.ior);
        T selT = (T(1) - dw) * (T(1) - fresnelT) * mat.specularTransmittance;
        // GenericMaterial.cs:308-309: the reverse selection reuses fresnelT (reference quirk)
        T selTIn = (T(1) - dw) * (T(1) - fresnelT) * mat.specularTransmittance;
        pdf = pf[0] * dw + pf[1] * selR + pf[2] * selT;
        pdfRev = pr[0] * dw + pr[1] * selR + pr[2] * selTIn;
        value = bsdf;
        if (cw) {
            cw->n = 3;
            for (int k = 0; k < 3; ++k) { cw->pdfs[k] = pf[k]; cw->pdfsRev[k] = pr[k]; }
            cw->weights[0] = dw; cw->weights[1] = selR; cw->weights[2] = selT;
            cw->weightsRev[0] = dw; cw->weightsRev[1] = selR; cw->weightsRev[2] = selTIn;
        }
    }

    // ---- DiffuseMaterial (Shading/Materials/DiffuseMaterial.cs) ----
    // DiffuseMaterial.cs:109-122
    Rgb<T> DiffuseEvaluate(const ShadingContext<T>& c, V3<T> inW) const {
        bool refl = ShouldReflect(c.point, c.outDirWorld, inW);
        V3<T> in = c.ToShading(inW);
        Rgb<T> base = Base(c.point.uv);
        if (mat.transmitter && !refl) {
            if (SameHemisphere(c.outDir, in)) return Rgb<T>::Black();  // :79-84
            return base / PI<T>();
        } else if (refl) {
            if (!SameHemisphere(c.outDir, in)) return Rgb<T>::Black();  // :45-50
            return base / PI<T>();
        }
        return Rgb<T>::Black();
    }
    // DiffuseMaterial.cs:167-188
    void DiffusePdf(const ShadingContext<T>& c, V3<T> inW, T& fwd, T& rev, ComponentWeights<T>* cw) const {
        V3<T> in = c.ToShading(inW);
        T rf = 0, rr = 0;
        if (SameHemisphere(c.outDir, in)) { rf = std::fabs(in.z) / PI<T>(); rr = std::fabs(c.outDir.z) / PI<T>(); }
        if (mat.transmitter) {
            T tf = 0, tr = 0;
            if (!SameHemisphere(c.outDir, in)) { tf = std::fabs(in.z) / PI<T>(); tr = std::fabs(c.outDir.z) / PI<T>(); }
            fwd = (rf + tf) * T(0.5f);
            rev = (rr + tr) * T(0.5f);
            if (cw) { cw->n = 1; cw->pdfs[0] = fwd * T(2); cw->weights[0] = T(0.5f); cw->pdfsRev[0] = rev * T(2); cw->weightsRev[0] = T(0.5f); }
        } else {
            fwd = rf; rev = rr;
            if (cw) { cw->n = 1; cw->pdfs[0] = fwd; cw->weights[0] = T(1); cw->pdfsRev[0] = rev; cw->weightsRev[0] = T(1); }
        }
    }

    // ---- Public entry points (SurfaceShader.cs) ----
    // Material.EvaluateWithCosine (Material.cs:80-83; GenericMaterial.cs:77-82)
    Rgb<T> EvaluateWithCosine(const ShadingContext<T>& c, V3<T> inW) const {
        if (mat.type == MAT_GENERIC) {
            V3<T> in = c.ToShading(inW);
            Rgb<T> v; T p, pr;
            GenericValueAndPdf(c, in, ComputeLocalParams(c), v, p, pr, nullptr);
            return v * std::fabs(in.z);
        }
        Rgb<T> f = DiffuseEvaluate(c, inW);
        return f * std::fabs(c.ToShading(inW).z);
    }
    // Material.Pdf (GenericMaterial.cs:84-90; DiffuseMaterial.cs:167-188)
    void Pdf(const ShadingContext<T>& c, V3<T> inW, T& fwd, T& rev, ComponentWeights<T>* cw = nullptr) const {
        if (mat.type == MAT_GENERIC) {
            Rgb<T> v;
            GenericValueAndPdf(c, c.ToShading(inW), ComputeLocalParams(c), v, fwd, rev, cw);
            return;
        }
        DiffusePdf(c, inW, fwd, rev, cw);
    }
    // Material.Sample (GenericMaterial.cs:92-150; DiffuseMaterial.cs:127-164)
    BsdfSample<T> Sample(const ShadingContext<T>& c, T u, V2<T> p, ComponentWeights<T>* cw = nullptr) const {
        BsdfSample<T> s;
        if (mat.type == MAT_GENERIC) {
            if (c.outDir.z == T(0)) return s;  // invalid
            Local lp = ComputeLocalParams(c);
            GGX<T> ndf{lp.alphaX, lp.alphaY};
            T eta = c.outDir.z > T(0) ? (T(1) / mat.ior) : mat.ior;
            T schlickF = SchlickFresnel(lp.specularReflectanceAtNormal, std::fabs(c.outDir.z)).Average();
            T diffuseBias = std::max(T(1) - schlickF, T(0.75f));
            T dw = diffuseBias * (T(1) - mat.metallic) * (T(1) - mat.specularTransmittance);
            V3<T> in;
            if (u <= dw) {
                in = ToCosHemisphere(p).Direction;
                if (c.outDir.z < T(0)) in.z *= T(-1);
            } else {
                V3<T> h = ndf.Sample(c.outDir, p);
                T cOut = dot(c.outDir, (h.z < T(0)) ? -h : h);
                T fr = FresnelDielectric(cOut, T(1), mat.ior);
                T selT = (T(1) - fr) * mat.specularTransmittance;
                if ((u - dw) / (T(1) - dw) < selT) {
                    if (dot(c.outDir, h) < T(0)) return s;
                    if (!Refract(c.outDir, h, eta, in)) return s;
                } else {
                    in = Reflect(c.outDir, h);
                }
            }
            Rgb<T> v; T pdf, pdfRev;
            GenericValueAndPdf(c, in, lp, v, pdf, pdfRev, cw);
            s.Pdf = pdf;
            s.PdfReverse = pdfRev;
            s.Weight = v * std::fabs(in.z) / pdf;
            s.Direction = c.ToWorld(in);
            return s;
        }
        // DiffuseMaterial.Sample
        DirectionSample<T> local = ToCosHemisphere(p);
        V3<T> d = local.Direction;
        if (mat.transmitter && u < T(0.5f)) {
            if (c.outDir.z > T(0)) d.z *= T(-1);  // :86-95
        } else {
            if (c.outDir.z < T(0)) d.z *= T(-1);  // :52-61
        }
        V3<T> w = ShadingToWorld(c.normal, d);
        Rgb<T> value = EvaluateWithCosine(c, w);
        T fwd, rev;
        DiffusePdf(c, w, fwd, rev, cw);
        if (fwd == T(0)) return s;
        s.Pdf = fwd; s.PdfReverse = rev; s.Weight = value / fwd; s.Direction = w;
        return s;
    }
};

// ------------------------------------------------------------------------------------------
// PathTracer (Integrators/PathTracer.cs)
// ------------------------------------------------------------------------------------------
struct PTParams {
    int width, height, totalSpp, maxDepth, minDepth;
    uint32_t baseSeed;
    int numShadowRays, enableBsdfDI;
};

// RayTracerStats (rays, shadow rays) and ShadingStats (Shading/ShadingStats.cs:5-33): the material
// calls counted where the reference's Notify* calls sit (GenericMaterial.cs:71,78,86,93;
// DiffuseMaterial.cs:110,128,168 -- DiffuseMaterial.Sample also calls EvaluateWithCosine and Pdf).
struct PathStats {
    uint64_t rays = 0, shadowRays = 0;
    uint64_t matEval = 0, matSample = 0, matPdf = 0;
};

// Triangle.SampleUniformArea (Geometry/Triangle.cs:42-55)
template <class T> inline SurfacePoint<T> SampleEmitterArea(const Scene<T>& sc, const Emitter<T>& e, V2<T> primary) {
    V2<T> bary = ToUniformTriangle(primary);
    return sc.MakePointMF(e.mesh, e.face, bary, T(0));
}

// SampleWarp.SurfaceAreaToSolidAngle (SampleWarp.cs:290-294)
template <class T> inline T SurfaceAreaToSolidAngle(const SurfacePoint<T>& from, const SurfacePoint<T>& to) {
    V3<T> d = to.position - from.position;
    T dsq = lengthSq(d);
    return std::fabs(dot(to.normal, -d)) / (dsq * std::sqrt(dsq));
}

// PathTracerBase.RegisterSample (PathTracer.cs:73-82): called once per complete path sample with
// its length (edges), whether it is a next-event sample, its contribution (the reference's
// `contrib * state.PrefixWeight`; for next-event samples without the Russian-roulette division
// that the radiance estimate applies) and its MIS weight.  The technique pyramid is built from it.
template <class T> struct SampleLog {
    virtual void Register(int depth, bool nextEvent, const Rgb<T>& weight, T mis) = 0;
    virtual ~SampleLog() = default;
};

// PathTracerBase.RenderPixel + EstimateIncidentRadiance (PathTracer.cs:287-382) for one
// (pixel, sample).  Returns the radiance estimate that RenderPixel splats.
template <class T> Rgb<T> RenderPixel(const Scene<T>& sc, const PTParams& P, uint32_t row, uint32_t col, Rng& rng, PathStats* stats,
                                      SampleLog<T>* log = nullptr) {
    const int nEm = int(sc.emitters.size());
    const T nShadow = T(P.numShadowRays);
    V2<float> off = rng.NextFloat2D();  // :289
    V2<T> film(T(float(col) + off.x), T(float(row) + off.y));  // Vector2(col,row) + offset in float
    Ray<T> ray;
    sc.camera.GenerateRay(film, ray.org, ray.dir);  // :291
    ray.tmin = 0;

    Rgb<T> prefix = Rgb<T>::White(), approx = Rgb<T>::White();
    uint32_t depth = 1;
    SurfacePoint<T> prevHit;
    T prevPdf = 0;
    Rgb<T> radiance = Rgb<T>::Black();

    while (int(depth) <= P.maxDepth) {  // :318
        if (stats) stats->rays++;
        SurfacePoint<T> hit = sc.Trace(ray);
        if (!hit.valid) {  // :322-330
            if (int(depth) >= P.minDepth && sc.env && P.enableBsdfDI) {
                T mis = T(1);
                if (depth > 1) {  // :384-400
                    T pdfNE = sc.env->DirectionPdf(ray.dir) * nShadow;
                    mis = T(1) / (T(1) + pdfNE / prevPdf);
                }
                Rgb<T> em = sc.env->EmittedRadiance(ray.dir);
                if (log) log->Register(int(depth), false, em * prefix, mis);  // :397
                radiance = radiance + prefix * mis * em;
            }
            break;
        }
        ShadingContext<T> ctx(hit, -ray.dir);  // :334
        const Material<T>& mat = sc.materials[sc.meshes[hit.mesh].material];
        MaterialEval<T> me{sc, mat};

        int emIdx = sc.triEmitter[sc.meshTriOffset[hit.mesh] + hit.prim];
        if (emIdx >= 0 && int(depth) >= P.minDepth) {  // :342-346, OnLightHit :402-421
            const Emitter<T>& light = sc.emitters[emIdx];
            T mis = T(1);
            if (depth > 1) {
                T jac = SurfaceAreaToSolidAngle(prevHit, hit);
                T pdfNE = light.invArea / T(nEm) * nShadow / jac;
                T ratio = pdfNE / prevPdf;
                mis = T(1) / (ratio + T(1));
                if (!P.enableBsdfDI) mis = T(0);
            }
            Rgb<T> em = light.EmittedRadiance(hit, -ray.dir);
            if (log) log->Register(int(depth), false, em * prefix, mis);  // :418
            radiance = radiance + prefix * mis * em;
        }

        // Russian roulette (:352-354, ComputeSurvivalProbability :277-282)
        T surv = depth > 4 ? std::clamp(approx.Average(), T(0.05f), T(0.95f)) : T(1);
        if (T(rng.NextFloat()) > surv || int(depth) == P.maxDepth) break;

        // Next event estimation (:357-364)
        if (int(depth) + 1 >= P.minDepth) {
            Rgb<T> nee = Rgb<T>::Black();
            for (int i = 0; i < P.numShadowRays; ++i) {
                // PerformBackgroundNextEvent (:423-452)
                if (sc.env) {
                    V2<float> u2 = rng.NextFloat2D();
                    BackgroundSample<T> bs = sc.env->SampleDirection(V2<T>(T(u2.x), T(u2.y)));
                    if (stats) stats->shadowRays++;
                    if (sc.LeavesScene(hit, bs.Direction)) {
                        Rgb<T> bsdfCos = me.EvaluateWithCosine(ctx, bs.Direction);
                        T pdfBsdf, pr; me.Pdf(ctx, bs.Direction, pdfBsdf, pr);
                        if (stats) { stats->matEval++; stats->matPdf++; }
                        if (!(pdfBsdf == T(0) || bs.Pdf == T(0))) {
                            T mis = P.enableBsdfDI ? T(1) / (T(1) + pdfBsdf / (bs.Pdf * nShadow)) : T(1);
                            Rgb<T> contrib = bs.Weight * bsdfCos / nShadow;
                            if (log) log->Register(int(depth) + 1, true, contrib * prefix, mis);  // :443
                            nee = nee + mis * contrib;
                        }
                    }
                }
                // PerformNextEventEstimation (:454-501)
                if (nEm > 0) {
                    int idx = int(rng.NextInt(uint32_t(nEm)));
                    const Emitter<T>& light = sc.emitters[idx];
                    T selProb = T(1) / T(nEm);
                    V2<float> u2 = rng.NextFloat2D();
                    SurfacePoint<T> lp = SampleEmitterArea(sc, light, V2<T>(T(u2.x), T(u2.y)));
                    V3<T> l2s = normalize(hit.position - lp.position);
                    if (stats) stats->shadowRays++;
                    if (!sc.IsOccluded(hit, lp)) {
                        Rgb<T> em = light.EmittedRadiance(lp, l2s);
                        T jac = SurfaceAreaToSolidAngle(hit, lp);
                        Rgb<T> bsdfCos = me.EvaluateWithCosine(ctx, -l2s);
                        T pdfNE = light.invArea * selProb * nShadow;
                        T pdfBsdfSA, pr; me.Pdf(ctx, -l2s, pdfBsdfSA, pr);
                        if (stats) { stats->matEval++; stats->matPdf++; }
                        T pdfBsdf = pdfBsdfSA * jac;
                        if (jac != T(0)) {
                            T ratio = pdfBsdf / pdfNE;
                            T mis = P.enableBsdfDI ? T(1) / (ratio + T(1)) : T(1);
                            T pdf = light.invArea / jac * selProb * nShadow;
                            Rgb<T> contrib = em / pdf * bsdfCos;
                            if (log) log->Register(int(depth) + 1, true, contrib * prefix, mis);  // :492
                            nee = nee + mis * contrib;
                        }
                    }
                }
            }
            radiance = radiance + prefix * nee / surv;
        }

        // SampleDirection (:526-530)
        T uc = T(rng.NextFloat());
        V2<float> up = rng.NextFloat2D();
        BsdfSample<T> bs = me.Sample(ctx, uc, V2<T>(T(up.x), T(up.y)));
        if (stats) {
            stats->matSample++;
            if (mat.type != MAT_GENERIC) { stats->matEval++; stats->matPdf++; }
        }
        if (bs.Pdf == T(0) || bs.Weight.IsBlack()) break;
        ray = Scene<T>::SpawnRay(hit, bs.Direction);

        prefix = prefix * (bs.Weight / surv);  // :372-378
        approx = approx * (bs.Weight / surv);
        depth++;
        prevHit = hit;
        prevPdf = bs.Pdf * surv;
    }
    return radiance;
}

// ------------------------------------------------------------------------------------------
// Path-replay adjoint (reference gradient).  Replays the path of RenderPixel with the same RNG
// stream and accumulates dLoss/dtheta with detached sampling: emitter radiance at emitter hits
// and NEE samples, material parameters through the BSDF at NEE samples, and through each sampled
// BSDF factor times the radiance collected after it (the path's total radiance minus what was
// collected up to that vertex).  BSDF derivatives are central differences in the template
// precision (use T = double).
// ------------------------------------------------------------------------------------------
template <class T> struct Grads {
    std::vector<T> tex, matBase, matRough, emitter;
    std::vector<size_t> texOffset;  // float offset of each texture in the concatenated layout
};

template <class T> void GradTargets(const Scene<T>& sc, const Grads<T>& G, int matIdx, V2<T> uv, long long& baseTgt, int& roughTgt) {
    const Material<T>& m = sc.materials[matIdx];
    baseTgt = -1;
    if (m.baseColor.tex >= 0) {
        const Texture<T>& t = sc.textures[m.baseColor.tex];
        if (t.channels == 3) {
            int col, row; t.Texel(uv, col, row);
            baseTgt = (long long)(G.texOffset[m.baseColor.tex] + (size_t(row) * t.w + col) * 3);
        }
    } else {
        baseTgt = -(long long)(matIdx + 2);
    }
    roughTgt = (m.type == MAT_GENERIC && m.roughness.tex < 0) ? matIdx : -1;
}
template <class T> void AddBase(Grads<T>& G, long long tgt, Rgb<T> g) {
    if (tgt >= 0) { G.tex[tgt] += g.r; G.tex[tgt + 1] += g.g; G.tex[tgt + 2] += g.b; }
    else if (tgt <= -2) { size_t m = size_t(-tgt - 2); G.matBase[3 * m] += g.r; G.matBase[3 * m + 1] += g.g; G.matBase[3 * m + 2] += g.b; }
}

// BSDF value (no cosine) and its derivatives with respect to base r, g, b and roughness.
template <class T> void BsdfDeriv(const Scene<T>& sc, const Material<T>& mat, const ShadingContext<T>& ctx, V3<T> inW, Rgb<T>& f, Rgb<T> d[4]) {
    Rgb<T> base = sc.TexLookupRgb(mat.baseColor, ctx.point.uv);
    T rough = sc.TexLookupMono(mat.roughness, ctx.point.uv);
    auto eval = [&](Rgb<T> b, T r) {
        MaterialEval<T> me{sc, mat, &b, &r};
        if (mat.type == MAT_GENERIC) {
            Rgb<T> v; T p, pr;
            me.GenericValueAndPdf(ctx, ctx.ToShading(inW), me.ComputeLocalParams(ctx), v, p, pr, nullptr);
            return v;
        }
        return me.DiffuseEvaluate(ctx, inW);
    };
    f = eval(base, rough);
    const T h = T(1e-6);
    for (int k = 0; k < 3; ++k) {
        Rgb<T> bp = base, bm = base;
        (k == 0 ? bp.r : k == 1 ? bp.g : bp.b) += h;
        (k == 0 ? bm.r : k == 1 ? bm.g : bm.b) -= h;
        d[k] = (eval(bp, rough) - eval(bm, rough)) / (T(2) * h);
    }
    if (mat.type == MAT_GENERIC && mat.roughness.tex < 0) d[3] = (eval(base, rough + h) - eval(base, rough - h)) / (T(2) * h);
    else d[3] = Rgb<T>::Black();
}
template <class T> T dotc(Rgb<T> a, Rgb<T> b) { return a.r * b.r + a.g * b.g + a.b * b.b; }

template <class T> T EmittedScale(const Emitter<T>& e, const SurfacePoint<T>& p, V3<T> dir) {
    if (!e.glossy()) return dot(p.shadingNormal, dir) < T(0) ? T(0) : T(1);
    T c = dot(p.shadingNormal, dir) / length(dir);
    if (c < T(0)) return T(0);
    return std::pow(c, e.exponent) * e.normalization;
}

template <class T> void AdjointPixel(const Scene<T>& sc, const PTParams& P, uint32_t row, uint32_t col, Rng rng, Rgb<T> Ltot, Rgb<T> delta,
                                     Grads<T>& G) {
    const int nEm = int(sc.emitters.size());
    const T nShadow = T(P.numShadowRays);
    V2<float> off = rng.NextFloat2D();
    V2<T> film(T(float(col) + off.x), T(float(row) + off.y));
    Ray<T> ray;
    sc.camera.GenerateRay(film, ray.org, ray.dir);
    Rgb<T> prefix = Rgb<T>::White(), approx = Rgb<T>::White();
    uint32_t depth = 1;
    SurfacePoint<T> prevHit;
    T prevPdf = 0;
    Rgb<T> radiance = Rgb<T>::Black();
    bool havePending = false;
    Rgb<T> pendD[4];
    long long pendBase = -1;
    int pendRough = -1;
    auto applyPending = [&]() {
        if (!havePending) return;
        Rgb<T> w = delta * (Ltot - radiance);
        // pendD[k] holds d ln f_c / d theta_k over the colour channels c
        AddBase(G, pendBase, Rgb<T>(dotc(w, pendD[0]), dotc(w, pendD[1]), dotc(w, pendD[2])));
        if (pendRough >= 0) G.matRough[pendRough] += dotc(w, pendD[3]);
        havePending = false;
    };
    while (int(depth) <= P.maxDepth) {
        SurfacePoint<T> hit = sc.Trace(ray);
        // the previous vertex's sampled BSDF factor: everything not yet collected lies after it
        applyPending();
        if (!hit.valid) {
            if (int(depth) >= P.minDepth && sc.env && P.enableBsdfDI) {
                T mis = T(1);
                if (depth > 1) mis = T(1) / (T(1) + sc.env->DirectionPdf(ray.dir) * nShadow / prevPdf);
                radiance = radiance + prefix * mis * sc.env->EmittedRadiance(ray.dir);
            }
            break;
        }
        ShadingContext<T> ctx(hit, -ray.dir);
        const Material<T>& mat = sc.materials[sc.meshes[hit.mesh].material];
        MaterialEval<T> me{sc, mat};
        int emIdx = sc.triEmitter[sc.meshTriOffset[hit.mesh] + hit.prim];
        if (emIdx >= 0 && int(depth) >= P.minDepth) {
            const Emitter<T>& light = sc.emitters[emIdx];
            T mis = T(1);
            if (depth > 1) {
                T jac = SurfaceAreaToSolidAngle(prevHit, hit);
                T pdfNE = light.invArea / T(nEm) * nShadow / jac;
                mis = T(1) / (pdfNE / prevPdf + T(1));
                if (!P.enableBsdfDI) mis = T(0);
            }
            radiance = radiance + prefix * mis * light.EmittedRadiance(hit, -ray.dir);
            Rgb<T> ge = delta * prefix * (mis * EmittedScale(light, hit, -ray.dir));
            G.emitter[3 * emIdx] += ge.r; G.emitter[3 * emIdx + 1] += ge.g; G.emitter[3 * emIdx + 2] += ge.b;
        }
        long long baseTgt; int roughTgt;
        GradTargets(sc, G, sc.meshes[hit.mesh].material, hit.uv, baseTgt, roughTgt);
        T surv = depth > 4 ? std::clamp(approx.Average(), T(0.05f), T(0.95f)) : T(1);
        if (T(rng.NextFloat()) > surv || int(depth) == P.maxDepth) break;
        if (int(depth) + 1 >= P.minDepth) {
            for (int i = 0; i < P.numShadowRays; ++i) {
                if (sc.env) {
                    V2<float> u2 = rng.NextFloat2D();
                    BackgroundSample<T> bs = sc.env->SampleDirection(V2<T>(T(u2.x), T(u2.y)));
                    if (sc.LeavesScene(hit, bs.Direction)) {
                        Rgb<T> bsdfCos = me.EvaluateWithCosine(ctx, bs.Direction);
                        T pdfBsdf, pr; me.Pdf(ctx, bs.Direction, pdfBsdf, pr);
                        if (!(pdfBsdf == T(0) || bs.Pdf == T(0))) {
                            T mis = P.enableBsdfDI ? T(1) / (T(1) + pdfBsdf / (bs.Pdf * nShadow)) : T(1);
                            Rgb<T> val = prefix * (mis * (bs.Weight * bsdfCos / nShadow)) / surv;
                            radiance = radiance + val;
                            Rgb<T> f, d[4];
                            BsdfDeriv(sc, mat, ctx, bs.Direction, f, d);
                            Rgb<T> coef = delta * prefix * (mis * bs.Weight / nShadow) / surv * std::fabs(ctx.ToShading(bs.Direction).z);
                            AddBase(G, baseTgt, Rgb<T>(dotc(coef, d[0]), dotc(coef, d[1]), dotc(coef, d[2])));
                            if (roughTgt >= 0) G.matRough[roughTgt] += dotc(coef, d[3]);
                        }
                    }
                }
                if (nEm > 0) {
                    int idx = int(rng.NextInt(uint32_t(nEm)));
                    const Emitter<T>& light = sc.emitters[idx];
                    T selProb = T(1) / T(nEm);
                    V2<float> u2 = rng.NextFloat2D();
                    SurfacePoint<T> lp = SampleEmitterArea(sc, light, V2<T>(T(u2.x), T(u2.y)));
                    V3<T> l2s = normalize(hit.position - lp.position);
                    if (!sc.IsOccluded(hit, lp)) {
                        Rgb<T> em = light.EmittedRadiance(lp, l2s);
                        T jac = SurfaceAreaToSolidAngle(hit, lp);
                        Rgb<T> bsdfCos = me.EvaluateWithCosine(ctx, -l2s);
                        T pdfNE = light.invArea * selProb * nShadow;
                        T pdfBsdfSA, pr; me.Pdf(ctx, -l2s, pdfBsdfSA, pr);
                        if (jac != T(0)) {
                            T mis = P.enableBsdfDI ? T(1) / (pdfBsdfSA * jac / pdfNE + T(1)) : T(1);
                            T pdf = light.invArea / jac * selProb * nShadow;
                            Rgb<T> val = prefix * (mis * (em / pdf * bsdfCos)) / surv;
                            radiance = radiance + val;
                            Rgb<T> f, d[4];
                            BsdfDeriv(sc, mat, ctx, -l2s, f, d);
                            Rgb<T> coef = delta * prefix * (mis * em / pdf) / surv * std::fabs(ctx.ToShading(-l2s).z);
                            AddBase(G, baseTgt, Rgb<T>(dotc(coef, d[0]), dotc(coef, d[1]), dotc(coef, d[2])));
                            if (roughTgt >= 0) G.matRough[roughTgt] += dotc(coef, d[3]);
                            Rgb<T> ge = delta * prefix * (mis * EmittedScale(light, lp, l2s) / pdf) * bsdfCos / surv;
                            G.emitter[3 * idx] += ge.r; G.emitter[3 * idx + 1] += ge.g; G.emitter[3 * idx + 2] += ge.b;
                        }
                    }
                }
            }
        }
        T uc = T(rng.NextFloat());
        V2<float> up = rng.NextFloat2D();
        BsdfSample<T> bs = me.Sample(ctx, uc, V2<T>(T(up.x), T(up.y)));
        if (bs.Pdf == T(0) || bs.Weight.IsBlack()) break;
        {
            Rgb<T> f, d[4];
            BsdfDeriv(sc, mat, ctx, bs.Direction, f, d);
            Rgb<T> inv(f.r != T(0) ? T(1) / f.r : T(0), f.g != T(0) ? T(1) / f.g : T(0), f.b != T(0) ? T(1) / f.b : T(0));
            for (int k = 0; k < 4; ++k) pendD[k] = d[k] * inv;
            pendBase = baseTgt;
            pendRough = roughTgt;
            havePending = true;
        }
        ray = Scene<T>::SpawnRay(hit, bs.Direction);
        prefix = prefix * (bs.Weight / surv);
        approx = approx * (bs.Weight / surv);
        depth++;
        prevHit = hit;
        prevPdf = bs.Pdf * surv;
    }
    applyPending();
}

// ---------------------------------------------------------------------------------------------
// Light paths: LightPathCache.TraceAllPaths / TraceLightPath (Integrators/Bidir/LightPathCache.cs:
// 126-260) with the LightPathWalk modifier (:271-341) over RandomWalk (Integrators/Common/
// RandomWalk.cs:76-216).  No next-event pdf callback (PdfNextEventAncestor stays 0).
// ---------------------------------------------------------------------------------------------
template <class T> struct LightVertex {
    SurfacePoint<T> point;
    T pdfFromAncestor = 0, pdfReverseAncestor = 0, pdfNextEventAncestor = 0;
    Rgb<T> weight;
    int pathId = 0, depth = 0;
    T maxRoughness = 0;
    bool fromBackground = false;
};

// Scene.Prepare (Scene.cs:115-136): center = mean of all vertices, radius = distance to the
// furthest vertex
template <class T> void SceneBounds(const Scene<T>& sc, V3<T>& center, T& radius) {
    V3<T> c(0, 0, 0);
    double n = 0;
    for (const auto& m : sc.meshes)
        for (size_t v = 0; v < m.V.size(); ++v) { c = c + m.V[v]; n += 1; }
    center = c / T(n);
    T r = 0;
    for (const auto& m : sc.meshes)
        for (size_t v = 0; v < m.V.size(); ++v) r = std::max(r, lengthSq(m.V[v] - center));
    radius = std::sqrt(r);
}

template <class T> struct EmitterRaySample { SurfacePoint<T> point; V3<T> dir; T pdf = 0; Rgb<T> weight; };

// DiffuseEmitter.SampleRay (DiffuseEmitter.cs:44-64), GlossyEmitter.SampleRay (GlossyEmitter.cs:47-71)
template <class T> EmitterRaySample<T> EmitterSampleRay(const Scene<T>& sc, const Emitter<T>& e, V2<T> primaryPos, V2<T> primaryDir) {
    EmitterRaySample<T> r;
    r.point = SampleEmitterArea(sc, e, primaryPos);
    T posPdf = e.invArea;
    V3<T> n = r.point.shadingNormal, t, b;
    ComputeBasisVectors(n, t, b);
    if (!e.glossy()) {
        DirectionSample<T> local = ToCosHemisphere(primaryDir);
        r.dir = n * local.Direction.z + t * local.Direction.x + b * local.Direction.y;
        r.pdf = local.Pdf * posPdf;
        r.weight = e.radiance / posPdf * PI<T>();
    } else {
        DirectionSample<T> local = ToCosineLobe(e.exponent + T(1), primaryDir);
        r.dir = n * local.Direction.z + t * local.Direction.x + b * local.Direction.y;
        T cosine = local.Direction.z;
        Rgb<T> w = e.radiance * std::pow(cosine, e.exponent + T(1)) * e.normalization;
        r.pdf = local.Pdf * posPdf;
        r.weight = w / posPdf / local.Pdf;
    }
    return r;
}

template <class T> struct LightPathParams { uint32_t seed, iter; int maxDepth; };

// GetRoughness (DiffuseMaterial.cs:31, GenericMaterial.cs:64)
template <class T> T MaterialRoughness(const Scene<T>& sc, const SurfacePoint<T>& p) {
    const Material<T>& m = sc.materials[sc.meshes[p.mesh].material];
    return m.type == MAT_GENERIC ? sc.TexLookupMono(m.roughness, p.uv) : T(1);
}

template <class T> std::vector<LightVertex<T>> TraceLightPath(const Scene<T>& sc, const LightPathParams<T>& P, int idx, V3<T> center, T radius) {
    std::vector<LightVertex<T>> out;
    Rng rng(P.seed, uint32_t(idx), P.iter);
    const int nEm = int(sc.emitters.size());
    // SelectLight (:33-40)
    T bgProb = sc.env ? T(1) / (T(1) + T(nEm)) : T(0);
    bool background = false;
    const Emitter<T>* em = nullptr;
    T prob;
    if (bgProb > T(0) && T(rng.NextFloat()) <= bgProb) {
        background = true;
        prob = bgProb;
    } else {
        em = &sc.emitters[rng.NextInt(uint32_t(nEm))];
        prob = (T(1) - bgProb) / T(nEm);
    }
    Rgb<T> approx = Rgb<T>::White();
    T nextReversePdf = 0, maxRough = 0;
    Ray<T> ray;
    SurfacePoint<T> prev;
    T pdfDirection;
    Rgb<T> prefix;
    int depth;
    auto survival = [&](int d) { return d > 4 ? std::clamp(approx.Average(), T(0.05f), T(0.95f)) : T(1); };
    auto addVertex = [&](const SurfacePoint<T>& p, T pdfFrom, const Rgb<T>& w, int d) {
        LightVertex<T> v;
        v.point = p;
        v.pdfFromAncestor = pdfFrom;
        v.pdfReverseAncestor = nextReversePdf;
        v.pathId = idx;
        v.weight = w;
        v.depth = d;
        // LightPathWalk.OnHit takes the maximum with Payload.maxRoughness, which stays 0 (:323-337)
        v.maxRoughness = std::max(MaterialRoughness(sc, p), maxRough);
        v.fromBackground = background;
        out.push_back(v);
    };
    if (!background) {
        // TraceEmitterPath (:211-224)
        V2<float> pp = rng.NextFloat2D(), pd = rng.NextFloat2D();
        EmitterRaySample<T> es = EmitterSampleRay(sc, *em, V2<T>(T(pp.x), T(pp.y)), V2<T>(T(pd.x), T(pd.y)));
        es.pdf *= prob;
        if (es.pdf == T(0) || es.weight.IsBlack()) return out;
        LightVertex<T> v0;
        v0.point = es.point;
        v0.pathId = idx;
        out.push_back(v0);  // OnStartEmitter (:295-306)
        ray = Scene<T>::SpawnRay(es.point, es.dir);
        prev = es.point;
        pdfDirection = es.pdf;
        prefix = es.weight / prob;
        depth = 1;
    } else {
        // TraceBackgroundPath (:226-241), EnvironmentMap.SampleRay (EnvironmentMap.cs:87-111)
        V2<float> pp = rng.NextFloat2D(), pd = rng.NextFloat2D();
        BackgroundSample<T> ds = sc.env->SampleDirection(V2<T>(T(pd.x), T(pd.y)));
        V2<T> disc = ToConcentricDisc(V2<T>(T(pp.x), T(pp.y)));
        V3<T> t, b;
        ComputeBasisVectors(ds.Direction, t, b);
        V3<T> pos = center + (ds.Direction + t * disc.x + b * disc.y) * radius;
        T posPdf = (T(1) / PI<T>()) / (radius * radius);
        Rgb<T> weight = ds.Weight / posPdf;
        T pdf = posPdf * ds.Pdf;
        pdf *= prob;
        weight = weight / prob;
        if (pdf == T(0) || weight.IsBlack()) return out;
        LightVertex<T> v0;
        v0.point.position = pos;
        v0.pathId = idx;
        v0.fromBackground = true;
        out.push_back(v0);  // OnStartBackground (:308-319)
        // StartFromBackground (RandomWalk.cs:86-124)
        Ray<T> r0;
        r0.org = pos;
        r0.dir = -ds.Direction;
        r0.tmin = 0;
        SurfacePoint<T> hit = sc.Trace(r0);
        if (!hit.valid) return out;
        ShadingContext<T> ctx(hit, -r0.dir, true);
        MaterialEval<T> me{sc, sc.materials[sc.meshes[hit.mesh].material]};
        // SampleBsdf (RandomWalk.cs:126-135): Sample(rng.NextFloat(), rng.NextFloat2D())
        float uc = rng.NextFloat();
        V2<float> up = rng.NextFloat2D();
        BsdfSample<T> bs = me.Sample(ctx, T(uc), V2<T>(T(up.x), T(up.y)));
        approx = approx * bs.Weight;
        addVertex(hit, pdf, weight, 1);
        nextReversePdf = bs.PdfReverse;
        if (P.maxDepth <= 1) return out;
        if (bs.Pdf == T(0) || bs.Weight.IsBlack()) return out;
        ray = Scene<T>::SpawnRay(hit, bs.Direction);
        prev = hit;
        pdfDirection = bs.Pdf;
        prefix = weight * bs.Weight;
        depth = 2;
    }
    // ContinueWalk (RandomWalk.cs:145-216)
    while (depth < P.maxDepth) {
        SurfacePoint<T> hit = sc.Trace(ray);
        if (!hit.valid) break;
        ShadingContext<T> ctx(hit, -ray.dir, true);
        T pdfFromAncestor = pdfDirection * SurfaceAreaToSolidAngle(prev, hit);
        if (pdfFromAncestor == T(0)) break;
        addVertex(hit, pdfFromAncestor, prefix, depth);
        if (depth + 1 >= P.maxDepth) break;
        T surv = survival(depth);
        if (T(rng.NextFloat()) > surv) break;
        MaterialEval<T> me{sc, sc.materials[sc.meshes[hit.mesh].material]};
        float uc = rng.NextFloat();
        V2<float> up = rng.NextFloat2D();
        BsdfSample<T> bs = me.Sample(ctx, T(uc), V2<T>(T(up.x), T(up.y)));
        approx = approx * (bs.Weight / surv);
        T pdfToAncestor = bs.PdfReverse * SurfaceAreaToSolidAngle(hit, prev);
        nextReversePdf = pdfToAncestor;  // OnContinue
        if (bs.Pdf == T(0) || bs.Weight.IsBlack()) break;
        Rgb<T> w = bs.Weight;
        w = w * (std::fabs(dot(hit.normal, bs.Direction)) / std::fabs(dot(hit.shadingNormal, bs.Direction)));
        w = w * (std::fabs(dot(hit.shadingNormal, -ray.dir)) / std::fabs(dot(hit.normal, -ray.dir)));
        prefix = prefix * (w / surv);
        ++depth;
        pdfDirection = bs.Pdf;
        prev = hit;
        ray = Scene<T>::SpawnRay(hit, bs.Direction);
    }
    return out;
}

}  // namespace ora

// ORACLE -- test infrastructure only.
//
// C entry points over the restatement in oracle_core.hpp / oracle_pt.hpp, for the pytest suite
// (via ctypes) and for the CPU-baseline leg of bench.py.  The product never links this file.
#include "oracle_pt.hpp"

#include <atomic>
#include <thread>

using namespace ora;

namespace {
struct Handle {
    int fp64 = 0;
    Scene<float> s32;
    Scene<double> s64;
    std::string err;
};

template <class T> Scene<T>& S(Handle* h);
template <> Scene<float>& S<float>(Handle* h) { return h->s32; }
template <> Scene<double>& S<double>(Handle* h) { return h->s64; }

template <class T> void addTexture(Handle* h, const float* d, int w, int hh, int ch, int border) {
    Texture<T> t; t.w = w; t.h = hh; t.channels = ch; t.border = border;
    t.data.assign(d, d + size_t(w) * hh * ch);
    S<T>(h).textures.push_back(std::move(t));
}
template <class T> void addMaterial(Handle* h, int type, const float* bc, int bcTex, float rough, int roughTex, float metallic, float specTint,
                                    float aniso, float specTrans, float ior, int transmitter) {
    Material<T> m;
    m.type = type;
    m.baseColor.c = Rgb<T>(bc[0], bc[1], bc[2]);
    m.baseColor.tex = bcTex;
    m.roughness.c = Rgb<T>(rough);
    m.roughness.tex = roughTex;
    m.metallic = metallic; m.specularTint = specTint; m.anisotropic = aniso; m.specularTransmittance = specTrans; m.ior = ior;
    m.transmitter = transmitter != 0;
    S<T>(h).materials.push_back(m);
}
template <class T> void addMesh(Handle* h, const float* V, int nV, const int* I, int nT, const float* N, const float* UV, int mat) {
    Mesh<T> m;
    for (int i = 0; i < nV; ++i) m.V.push_back(V3<T>(V[3 * i], V[3 * i + 1], V[3 * i + 2]));
    m.I.assign(I, I + 3 * size_t(nT));
    if (N) for (int i = 0; i < nV; ++i) m.N.push_back(V3<T>(N[3 * i], N[3 * i + 1], N[3 * i + 2]));
    if (UV) for (int i = 0; i < nV; ++i) m.UV.push_back(V2<T>(UV[2 * i], UV[2 * i + 1]));
    m.material = mat;
    m.faceNormals.resize(nT);
    for (int f = 0; f < nT; ++f) {  // TinyEmbree face normal: normalized cross(v2 - v1, v3 - v1)
        V3<T> a, b, c; m.Tri(f, a, b, c);
        m.faceNormals[f] = normalize(cross(b - a, c - a));
    }
    S<T>(h).meshes.push_back(std::move(m));
}
// DiffuseEmitter/GlossyEmitter.MakeFromMesh: one emitter per triangle, zero-area triangles are
// skipped (DiffuseEmitter.cs:21-31, Triangle.cs:32-33).
template <class T> int addEmitters(Handle* h, int mesh, const int* faces, int nFaces, const float* rgb, float exponent) {
    Scene<T>& sc = S<T>(h);
    const Mesh<T>& m = sc.meshes[mesh];
    int count = faces ? nFaces : m.numFaces();
    int added = 0;
    for (int k = 0; k < count; ++k) {
        int f = faces ? faces[k] : k;
        V3<T> a, b, c; m.Tri(f, a, b, c);
        T area = length(cross(b - a, c - a)) * T(0.5f);
        if (area == T(0)) continue;
        Emitter<T> e;
        e.mesh = mesh; e.face = f;
        e.radiance = Rgb<T>(rgb[0], rgb[1], rgb[2]);
        e.exponent = exponent;
        e.invArea = T(1) / area;
        e.normalization = (T(exponent) + T(1)) / (T(2) * PI<T>());
        sc.emitters.push_back(e);
        ++added;
    }
    return added;
}
template <class T> void setEnv(Handle* h, const float* rgb, int w, int hh) {
    auto env = std::make_unique<EnvMap<T>>();
    env->w = w; env->h = hh;
    env->img.resize(size_t(w) * hh);
    for (size_t i = 0; i < env->img.size(); ++i) env->img[i] = Rgb<T>(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    env->Build();
    S<T>(h).env = std::move(env);
}
template <class T> int setCamera(Handle* h, const float* m16, float fov) {
    M44<T> m;
    for (int i = 0; i < 16; ++i) (&m.m[0][0])[i] = m16[i];
    S<T>(h).cameraSet = true;
    return S<T>(h).camera.Set(m, fov) ? 0 : -1;
}

template <class T> SurfacePoint<T> PointFrom(const float* pt) {
    SurfacePoint<T> p;
    p.valid = true;
    p.position = V3<T>(pt[0], pt[1], pt[2]);
    p.normal = V3<T>(pt[3], pt[4], pt[5]);
    p.shadingNormal = V3<T>(pt[6], pt[7], pt[8]);
    p.uv = V2<T>(pt[9], pt[10]);
    return p;
}

template <class T> void renderRows(Handle* h, const PTParams& P, uint32_t sampleIndex, float* film, int nthreads, uint64_t* stats, bool runningMean) {
    const Scene<T>& sc = S<T>(h);
    std::atomic<int> nextRow(0);
    std::atomic<uint64_t> rays(0), srays(0), mEval(0), mSample(0), mPdf(0);
    float k = float(sampleIndex + 1);
    auto worker = [&]() {
        PathStats st;
        for (;;) {
            int row = nextRow.fetch_add(1);
            if (row >= P.height) break;
            for (int col = 0; col < P.width; ++col) {
                uint32_t pix = uint32_t(row * P.width + col);
                Rng rng(P.baseSeed, pix, sampleIndex);
                Rgb<T> v = RenderPixel(sc, P, uint32_t(row), uint32_t(col), rng, &st);
                float* f = film + 3 * size_t(pix);
                if (runningMean) {
                    // FrameBuffer.StartIteration scale + Splat (FrameBuffer.cs:166-191, 232, 249)
                    if (sampleIndex > 0) {
                        float s = (k - 1.0f) / k;
                        f[0] *= s; f[1] *= s; f[2] *= s;
                    }
                    float avg = (float(v.r) + float(v.g) + float(v.b)) / 3.0f;
                    if (std::isfinite(avg)) {
                        f[0] += float(v.r) / k; f[1] += float(v.g) / k; f[2] += float(v.b) / k;
                    }
                } else {
                    f[0] = float(v.r); f[1] = float(v.g); f[2] = float(v.b);
                }
            }
        }
        rays += st.rays; srays += st.shadowRays;
        mEval += st.matEval; mSample += st.matSample; mPdf += st.matPdf;
    };
    int nt = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    if (stats) {
        stats[0] += rays.load(); stats[1] += srays.load();
        stats[2] += mEval.load(); stats[3] += mSample.load(); stats[4] += mPdf.load();
    }
}
template <class T> static void matEval(const Scene<T>& sc, int mat, const float* pt, const float* outDir, const float* inDir, float* value, float* pdf2,
                                       float* comp) {
    SurfacePoint<T> sp = PointFrom<T>(pt);
    ShadingContext<T> ctx(sp, V3<T>(outDir[0], outDir[1], outDir[2]));
    MaterialEval<T> me{sc, sc.materials[mat]};
    V3<T> in(inDir[0], inDir[1], inDir[2]);
    Rgb<T> v = me.EvaluateWithCosine(ctx, in);
    ComponentWeights<T> cw;
    T p0, p1;
    me.Pdf(ctx, in, p0, p1, &cw);
    pdf2[0] = float(p0); pdf2[1] = float(p1);
    value[0] = float(v.r); value[1] = float(v.g); value[2] = float(v.b);
    if (comp) {
        comp[0] = float(cw.n);
        for (int k = 0; k < 3; ++k) { comp[1 + k] = float(cw.pdfs[k]); comp[4 + k] = float(cw.weights[k]); comp[7 + k] = float(cw.pdfsRev[k]); comp[10 + k] = float(cw.weightsRev[k]); }
    }
}
template <class T> static void matSample(const Scene<T>& sc, int mat, const float* pt, const float* outDir, float u, float u1, float u2, float* dir,
                                         float* pdf2, float* weight, float* comp) {
    SurfacePoint<T> sp = PointFrom<T>(pt);
    ShadingContext<T> ctx(sp, V3<T>(outDir[0], outDir[1], outDir[2]));
    MaterialEval<T> me{sc, sc.materials[mat]};
    ComponentWeights<T> cw;
    BsdfSample<T> s = me.Sample(ctx, T(u), V2<T>(T(u1), T(u2)), &cw);
    dir[0] = float(s.Direction.x); dir[1] = float(s.Direction.y); dir[2] = float(s.Direction.z);
    pdf2[0] = float(s.Pdf); pdf2[1] = float(s.PdfReverse);
    weight[0] = float(s.Weight.r); weight[1] = float(s.Weight.g); weight[2] = float(s.Weight.b);
    if (comp) {
        comp[0] = float(cw.n);
        for (int k = 0; k < 3; ++k) { comp[1 + k] = float(cw.pdfs[k]); comp[4 + k] = float(cw.weights[k]); comp[7 + k] = float(cw.pdfsRev[k]); comp[10 + k] = float(cw.weightsRev[k]); }
    }
}
}  // namespace

// Monte Carlo integral over directions with a 99% confidence interval, restating the estimator of
// SeeSharp.Tests/Core/Shading/Material_SampleTransform.cs:40-69: 32 batches, batch i seeded
// RNG(18273912, i, 1313), per sample a 2D primary sample, then one more number for the component
// choice; zero-pdf samples are skipped; per-batch float sums of val / N and val^2 / N (added up in
// batch order here, under a lock in any order there); variance = E[v^2] - E[v]^2, interval
// mean +- 2.576 sqrt(variance / N).
template <class F>
static void mcInterval(int numSamples, F sampleFn, float* ci) {
    const int numBatches = 32;
    numSamples = (numSamples / numBatches) * numBatches;
    const float invNum = 1.0f / float(numSamples);
    float total = 0.0f, totalSquares = 0.0f;
    for (int b = 0; b < numBatches; ++b) {
        float result = 0.0f, squares = 0.0f;
        Rng rng(18273912u, uint32_t(b), 1313u);
        for (int j = 0; j < numSamples / numBatches; ++j) {
            V2<float> primary = rng.NextFloat2D();
            float u = rng.NextFloat();
            float val;
            if (!sampleFn(u, primary, val)) continue;
            result += val * invNum;
            squares += val * val * invNum;
        }
        total += result;
        totalSquares += squares;
    }
    const float variance = totalSquares - total * total;
    if (variance <= 0.0f) { ci[0] = ci[1] = total; return; }
    const float off = std::sqrt(variance) / std::sqrt(float(numSamples));
    ci[0] = total - 2.576f * off;
    ci[1] = total + 2.576f * off;
}

extern "C" {

void* ora_scene_create(int fp64) { auto* h = new Handle(); h->fp64 = fp64; return h; }
void ora_scene_destroy(void* p) { delete static_cast<Handle*>(p); }

int ora_add_texture(void* p, const float* d, int w, int h, int ch, int border) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) { addTexture<double>(H, d, w, h, ch, border); return int(H->s64.textures.size()) - 1; }
    addTexture<float>(H, d, w, h, ch, border); return int(H->s32.textures.size()) - 1;
}
int ora_add_material(void* p, int type, const float* bc, int bcTex, float rough, int roughTex, float metallic, float specTint, float aniso,
                     float specTrans, float ior, int transmitter) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) { addMaterial<double>(H, type, bc, bcTex, rough, roughTex, metallic, specTint, aniso, specTrans, ior, transmitter); return int(H->s64.materials.size()) - 1; }
    addMaterial<float>(H, type, bc, bcTex, rough, roughTex, metallic, specTint, aniso, specTrans, ior, transmitter);
    return int(H->s32.materials.size()) - 1;
}
int ora_add_mesh(void* p, const float* V, int nV, const int* I, int nT, const float* N, const float* UV, int mat) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) { addMesh<double>(H, V, nV, I, nT, N, UV, mat); return int(H->s64.meshes.size()) - 1; }
    addMesh<float>(H, V, nV, I, nT, N, UV, mat); return int(H->s32.meshes.size()) - 1;
}
int ora_add_emitters(void* p, int mesh, const int* faces, int nFaces, const float* rgb, float exponent) {
    Handle* H = static_cast<Handle*>(p);
    return H->fp64 ? addEmitters<double>(H, mesh, faces, nFaces, rgb, exponent) : addEmitters<float>(H, mesh, faces, nFaces, rgb, exponent);
}
int ora_set_envmap(void* p, const float* rgb, int w, int h) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) setEnv<double>(H, rgb, w, h); else setEnv<float>(H, rgb, w, h);
    return 0;
}
int ora_set_camera(void* p, const float* m16, float fov) {
    Handle* H = static_cast<Handle*>(p);
    return H->fp64 ? setCamera<double>(H, m16, fov) : setCamera<float>(H, m16, fov);
}
int ora_commit(void* p, int W, int Hh, char* err, int errlen) {
    Handle* H = static_cast<Handle*>(p);
    std::string e = H->fp64 ? H->s64.Commit(W, Hh) : H->s32.Commit(W, Hh);
    if (!e.empty()) {
        if (err && errlen > 0) { std::strncpy(err, e.c_str(), errlen - 1); err[errlen - 1] = 0; }
        return -2;
    }
    return 0;
}
int ora_num_emitters(void* p) {
    Handle* H = static_cast<Handle*>(p);
    return int(H->fp64 ? H->s64.emitters.size() : H->s32.emitters.size());
}
int ora_bvh_nodes(void* p) {
    Handle* H = static_cast<Handle*>(p);
    return int(H->fp64 ? H->s64.nodes.size() : H->s32.nodes.size());
}

// Progressive render of iterations [iterFirst, iterFirst + iterCount) into film (W*H*3, in/out)
// with the frame buffer's running mean.  stats[0] = traced rays, stats[1] = shadow rays, stats[2..4] =
// ShadingStats (material evaluations, samples, pdfs).
int ora_render(void* p, const PTParams* P, float* film, int nthreads, uint64_t* stats, int iterFirst, int iterCount) {
    Handle* H = static_cast<Handle*>(p);
    for (int it = iterFirst; it < iterFirst + iterCount; ++it) {
        if (H->fp64) renderRows<double>(H, *P, uint32_t(it), film, nthreads, stats, true);
        else renderRows<float>(H, *P, uint32_t(it), film, nthreads, stats, true);
    }
    return 0;
}

// The PathTracer's technique pyramids (RenderTechniquePyramid, PathTracer.cs:73-82, 204-266;
// Integrators/Bidir/TechPyramid.cs): every registered sample, divided by TotalSpp, is added to the
// image of its technique, "{d}-hit" (layer 2(d-1)) or "{d}-next-event" (layer 2(d-1)+1), in the
// raw pyramid (pyr) and, times its MIS weight, in the weighted one (pyr + 2*maxDepth layers).
// Iterations [iterFirst, iterFirst + iterCount), pixels in order, on one thread (the reference's
// per-pixel order of additions).  pyr: 2 * 2*maxDepth * W*H*3 floats, accumulated into.
namespace {
struct PyramidLog : SampleLog<float> {
    float* pyr;
    size_t P;
    int layers, pixel;
    float spp;
    void Register(int depth, bool nextEvent, const Rgb<float>& weight, float mis) override {
        Rgb<float> w(weight.r / spp, weight.g / spp, weight.b / spp);
        int L = 2 * (depth - 1) + (nextEvent ? 1 : 0);
        float* a = pyr + (size_t(L) * P + size_t(pixel)) * 3;
        float* b = pyr + (size_t(layers + L) * P + size_t(pixel)) * 3;
        a[0] += w.r; a[1] += w.g; a[2] += w.b;
        Rgb<float> m = w * mis;
        b[0] += m.r; b[1] += m.g; b[2] += m.b;
    }
};
}  // namespace

int ora_render_pyramid(void* p, const PTParams* P, int iterFirst, int iterCount, float* pyr) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) return -1;
    PyramidLog log;
    log.pyr = pyr;
    log.P = size_t(P->width) * P->height;
    log.layers = 2 * P->maxDepth;
    log.spp = float(P->totalSpp);
    for (int it = iterFirst; it < iterFirst + iterCount; ++it)
        for (uint32_t pix = 0; pix < uint32_t(log.P); ++pix) {
            log.pixel = int(pix);
            Rng rng(P->baseSeed, pix, uint32_t(it));
            RenderPixel(H->s32, *P, pix / uint32_t(P->width), pix % uint32_t(P->width), rng, nullptr, &log);
        }
    return 0;
}

// Radiance of individual paths: rgb[3*i] for pixel index pixels[i] and the given sample index.
int ora_render_paths(void* p, const PTParams* P, uint32_t sampleIndex, const int* pixels, int n, float* rgb, uint64_t* stats, int nthreads) {
    Handle* H = static_cast<Handle*>(p);
    std::atomic<int> next(0);
    std::atomic<uint64_t> rays(0), srays(0);
    auto worker = [&]() {
        PathStats st;
        for (;;) {
            int i0 = next.fetch_add(64);
            if (i0 >= n) break;
            for (int i = i0; i < std::min(n, i0 + 64); ++i) {
                uint32_t pix = uint32_t(pixels[i]);
                uint32_t row = pix / uint32_t(P->width), col = pix % uint32_t(P->width);
                Rng rng(P->baseSeed, pix, sampleIndex);
                if (H->fp64) {
                    Rgb<double> v = RenderPixel(H->s64, *P, row, col, rng, &st);
                    rgb[3 * i] = float(v.r); rgb[3 * i + 1] = float(v.g); rgb[3 * i + 2] = float(v.b);
                } else {
                    Rgb<float> v = RenderPixel(H->s32, *P, row, col, rng, &st);
                    rgb[3 * i] = v.r; rgb[3 * i + 1] = v.g; rgb[3 * i + 2] = v.b;
                }
            }
        }
        rays += st.rays; srays += st.shadowRays;
    };
    int nt = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    if (stats) { stats[0] += rays.load(); stats[1] += srays.load(); }
    return 0;
}

// rays: n * 8 floats (org xyz, tmin, dir xyz, tmax); hits: n * 4 floats (t, u, v, tri as float
// bits).  anyHit != 0 answers occlusion only (tri >= 0 when occluded).
int ora_trace(void* p, const float* rays, int n, float* hits, int anyHit) {
    Handle* H = static_cast<Handle*>(p);
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 8 * size_t(i);
        float* o = hits + 4 * size_t(i);
        int tri; float t = 0, u = 0, v = 0;
        if (H->fp64) {
            Ray<double> ray; ray.org = V3<double>(r[0], r[1], r[2]); ray.tmin = r[3]; ray.dir = V3<double>(r[4], r[5], r[6]); ray.tmax = r[7];
            HitRec<double> hr = H->s64.Intersect(ray, anyHit != 0);
            tri = hr.tri; t = float(hr.t); u = float(hr.u); v = float(hr.v);
        } else {
            Ray<float> ray; ray.org = V3<float>(r[0], r[1], r[2]); ray.tmin = r[3]; ray.dir = V3<float>(r[4], r[5], r[6]); ray.tmax = r[7];
            HitRec<float> hr = H->s32.Intersect(ray, anyHit != 0);
            tri = hr.tri; t = hr.t; u = hr.u; v = hr.v;
        }
        o[0] = t; o[1] = u; o[2] = v; std::memcpy(&o[3], &tri, 4);
    }
    return 0;
}

// FP64 brute-force closest hit.  rays: n * 7 doubles (org, dir, tmin); hits: n * 4 doubles
// (t, u, v, tri), plus per ray the runner-up distance in `second` (for degeneracy screening).
int ora_trace_brute64(void* p, const double* rays, int n, double* hits, double* second) {
    Handle* H = static_cast<Handle*>(p);
    auto run = [&](auto& sc) {
        for (int i = 0; i < n; ++i) {
            const double* r = rays + 7 * size_t(i);
            V3<double> org(r[0], r[1], r[2]), dir(r[3], r[4], r[5]);
            HitRec<double> hr = sc.IntersectBrute64(org, dir, r[6]);
            hits[4 * size_t(i)] = hr.t; hits[4 * size_t(i) + 1] = hr.u; hits[4 * size_t(i) + 2] = hr.v; hits[4 * size_t(i) + 3] = hr.tri;
            if (second) {
                // closest distance among the other triangles
                Ray<double> ray; ray.org = org; ray.dir = dir; ray.tmin = r[6];
                RayPre<double> pre(dir);
                double best = std::numeric_limits<double>::infinity();
                for (size_t g = 0; g < sc.tv0.size(); ++g) {
                    if (int(g) == hr.tri) continue;
                    V3<double> a(sc.tv0[g].x, sc.tv0[g].y, sc.tv0[g].z), b(sc.tv1[g].x, sc.tv1[g].y, sc.tv1[g].z), c(sc.tv2[g].x, sc.tv2[g].y, sc.tv2[g].z);
                    double t, u, v;
                    if (IntersectTri<double>(ray, pre, a, b, c, best, t, u, v)) best = t;
                }
                second[i] = best;
            }
        }
    };
    if (H->fp64) run(H->s64); else run(H->s32);
    return 0;
}

// FP64 closest hit over the BVH with the runner-up distance, on nthreads host threads.
// rays: n * 8 doubles (org xyz, tmin, dir xyz, tmax); hits: n * 4 doubles (t, u, v, tri); second: n.
int ora_trace_two64(void* p, const double* rays, int n, double* hits, double* second, int nthreads) {
    Handle* H = static_cast<Handle*>(p);
    std::atomic<int> next{0};
    auto worker = [&](auto& sc) {
        for (;;) {
            int i0 = next.fetch_add(64);
            if (i0 >= n) return;
            for (int i = i0; i < std::min(n, i0 + 64); ++i) {
                const double* r = rays + 8 * size_t(i);
                HitRec<double> hr; double sec;
                sc.IntersectTwo64(V3<double>(r[0], r[1], r[2]), V3<double>(r[4], r[5], r[6]), r[3], r[7], hr, sec);
                hits[4 * size_t(i)] = hr.t; hits[4 * size_t(i) + 1] = hr.u; hits[4 * size_t(i) + 2] = hr.v; hits[4 * size_t(i) + 3] = hr.tri;
                second[i] = sec;
            }
        }
    };
    auto run = [&](auto& sc) {
        std::vector<std::thread> th;
        for (int t = 1; t < std::max(1, nthreads); ++t) th.emplace_back([&] { worker(sc); });
        worker(sc);
        for (auto& t : th) t.join();
    };
    if (H->fp64) run(H->s64); else run(H->s32);
    return 0;
}

// Material_SampleTransform.cs:71-117 on the FP32 oracle: mode 0 integrates EvaluateWithCosine's
// channel average with uniform-sphere directions, mode 1 the same with the material's own Sample,
// mode 2 the material's pdf with uniform-sphere directions.  pt: the 11-float surface point.
int ora_material_integrate(void* p, int mat, const float* pt, const float* outDir, int mode, int numSamples, float* ci) {
    Handle* H = static_cast<Handle*>(p);
    const Scene<float>& sc = H->s32;
    if (mat < 0 || mat >= int(sc.materials.size()) || mode < 0 || mode > 2) return -1;
    SurfacePoint<float> sp = PointFrom<float>(pt);
    ShadingContext<float> ctx(sp, V3<float>(outDir[0], outDir[1], outDir[2]));
    MaterialEval<float> me{sc, sc.materials[mat]};
    mcInterval(numSamples, [&](float u, V2<float> primary, float& val) {
        V3<float> dir;
        float pdf;
        if (mode == 1) {
            BsdfSample<float> smp = me.Sample(ctx, u, primary);
            dir = smp.Direction;
            pdf = smp.Pdf;
        } else {
            DirectionSample<float> smp = ToUniformSphere(primary);
            dir = smp.Direction;
            pdf = smp.Pdf;
        }
        if (pdf == 0.0f) return false;
        float f;
        if (mode == 2) { float fwd, rev; me.Pdf(ctx, dir, fwd, rev); f = fwd; }
        else f = me.EvaluateWithCosine(ctx, dir).Average();
        val = f / pdf;
        return true;
    }, ci);
    return 0;
}

// Material_SampleTransform.cs:285-303: the visible-normal pdf TrowbridgeReitzDistribution.Pdf(outDir, dir)
// integrated over uniform-sphere directions.
void ora_ggx_pdf_integrate(float ax, float ay, const float* outDir, int numSamples, float* ci) {
    GGX<float> ndf{ax, ay};
    V3<float> o(outDir[0], outDir[1], outDir[2]);
    mcInterval(numSamples, [&](float, V2<float> primary, float& val) {
        DirectionSample<float> smp = ToUniformSphere(primary);
        if (smp.Pdf == 0.0f) return false;
        val = ndf.Pdf(o, smp.Direction) / smp.Pdf;
        return true;
    }, ci);
}

int ora_camera_ray(void* p, float fx, float fy, float* org, float* dir) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) {
        V3<double> o, d; H->s64.camera.GenerateRay(V2<double>(fx, fy), o, d);
        org[0] = float(o.x); org[1] = float(o.y); org[2] = float(o.z); dir[0] = float(d.x); dir[1] = float(d.y); dir[2] = float(d.z);
    } else {
        V3<float> o, d; H->s32.camera.GenerateRay(V2<float>(fx, fy), o, d);
        org[0] = o.x; org[1] = o.y; org[2] = o.z; dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
    }
    return 0;
}

// Material queries at an explicit surface point pt = (position 3, face normal 3, shading normal 3,
// uv 2).  comp (optional, 13 floats): n, pdfs[3], weights[3], pdfsRev[3], weightsRev[3].
// Runs in the scene's precision (FP64 scenes evaluate in double and round the outputs).
int ora_material_eval(void* p, int mat, const float* pt, const float* outDir, const float* inDir, float* value, float* pdf2, float* comp) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) matEval(H->s64, mat, pt, outDir, inDir, value, pdf2, comp);
    else matEval(H->s32, mat, pt, outDir, inDir, value, pdf2, comp);
    return 0;
}
int ora_material_sample(void* p, int mat, const float* pt, const float* outDir, float u, float u1, float u2, float* dir, float* pdf2, float* weight, float* comp) {
    Handle* H = static_cast<Handle*>(p);
    if (H->fp64) matSample(H->s64, mat, pt, outDir, u, u1, u2, dir, pdf2, weight, comp);
    else matSample(H->s32, mat, pt, outDir, u, u1, u2, dir, pdf2, weight, comp);
    return 0;
}

// Reference gradient by FP64 path replay (scene created with fp64 = 1).  dLdI: W*H*3 (float);
// outputs (double): gTex (all textures' texels concatenated), gMatBase (3 per material),
// gMatRough (1 per material), gEmitter (3 per emitter).  Each path's total radiance comes from an
// FP64 render of the same path; non-finite paths are skipped as the frame buffer skips them.
// Light paths of LightPathCache.TraceAllPaths for paths [0, n): per vertex 16 floats
// (position 3, normal 3, shading normal 3, pdfFromAncestor, pdfReverseAncestor, weight 3,
// maxRoughness, fromBackground) and 4 ints (mesh, prim, depth, pathId); stride = maxDepth + 1
// vertices per path; lengths[n].
int ora_light_paths(void* p, uint32_t seed, uint32_t iter, int maxDepth, int n, float* vf, int* vi, int* lengths) {
    Handle* H = static_cast<Handle*>(p);
    const int stride = maxDepth + 1;
    auto emit = [&](auto& sc) {
        using T = decltype(sc.emitters[0].invArea);
        V3<T> c; T r;
        SceneBounds(sc, c, r);
        LightPathParams<T> P{seed, iter, maxDepth};
        for (int i = 0; i < n; ++i) {
            std::vector<LightVertex<T>> path = TraceLightPath(sc, P, i, c, r);
            lengths[i] = int(path.size());
            for (int k = 0; k < int(path.size()) && k < stride; ++k) {
                const LightVertex<T>& v = path[k];
                float* f = vf + 16 * (size_t(i) * stride + k);
                int* q = vi + 4 * (size_t(i) * stride + k);
                const V3<T>* vs[3] = {&v.point.position, &v.point.normal, &v.point.shadingNormal};
                for (int a = 0; a < 3; ++a) { f[3 * a] = float(vs[a]->x); f[3 * a + 1] = float(vs[a]->y); f[3 * a + 2] = float(vs[a]->z); }
                f[9] = float(v.pdfFromAncestor); f[10] = float(v.pdfReverseAncestor);
                f[11] = float(v.weight.r); f[12] = float(v.weight.g); f[13] = float(v.weight.b);
                f[14] = float(v.maxRoughness); f[15] = v.fromBackground ? 1.0f : 0.0f;
                q[0] = v.point.mesh; q[1] = v.point.prim; q[2] = v.depth; q[3] = v.pathId;
            }
        }
    };
    if (H->fp64) emit(H->s64); else emit(H->s32);
    return 0;
}

int ora_adjoint(void* p, const PTParams* P, const float* dLdI, double* gTex, double* gMatBase, double* gMatRough, double* gEmitter, int nthreads) {
    Handle* H = static_cast<Handle*>(p);
    if (!H->fp64) return -1;
    const Scene<double>& sc = H->s64;
    size_t nTex = 0;
    std::vector<size_t> offs;
    for (auto& t : sc.textures) { offs.push_back(nTex); nTex += t.data.size(); }
    int nt = std::max(1, nthreads);
    std::vector<Grads<double>> G(nt);
    for (auto& g : G) {
        g.tex.assign(nTex, 0.0); g.matBase.assign(3 * sc.materials.size(), 0.0); g.matRough.assign(sc.materials.size(), 0.0);
        g.emitter.assign(3 * sc.emitters.size(), 0.0); g.texOffset = offs;
    }
    std::atomic<int> nextRow(0);
    auto worker = [&](int tid) {
        for (;;) {
            int row = nextRow.fetch_add(1);
            if (row >= P->height) break;
            for (int col = 0; col < P->width; ++col) {
                uint32_t pix = uint32_t(row * P->width + col);
                const float* d = dLdI + 3 * size_t(pix);
                if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) continue;  // every term is a multiple of dLoss/dPixel
                Rgb<double> delta(double(d[0]) / P->totalSpp, double(d[1]) / P->totalSpp, double(d[2]) / P->totalSpp);
                for (int s = 0; s < P->totalSpp; ++s) {
                    Rng rng(P->baseSeed, pix, uint32_t(s));
                    Rng rng2 = rng;
                    Rgb<double> L = RenderPixel(sc, *P, uint32_t(row), uint32_t(col), rng, nullptr);
                    if (!std::isfinite(L.Average())) continue;
                    AdjointPixel(sc, *P, uint32_t(row), uint32_t(col), rng2, L, delta, G[tid]);
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker, i);
    worker(0);
    for (auto& t : th) t.join();
    auto sum = [&](double* out, auto member) {
        if (!out) return;
        size_t n = (G[0].*member).size();
        for (size_t k = 0; k < n; ++k) { double s = 0; for (auto& g : G) s += (g.*member)[k]; out[k] = s; }
    };
    sum(gTex, &Grads<double>::tex);
    sum(gMatBase, &Grads<double>::matBase);
    sum(gMatRough, &Grads<double>::matRough);
    sum(gEmitter, &Grads<double>::emitter);
    return 0;
}

int ora_env_radiance(void* p, const float* dir, float* rgb) {
    Handle* H = static_cast<Handle*>(p);
    if (!H->s32.env) return -1;
    Rgb<float> c = H->s32.env->EmittedRadiance(V3<float>(dir[0], dir[1], dir[2]));
    rgb[0] = c.r; rgb[1] = c.g; rgb[2] = c.b;
    return 0;
}
int ora_env_sample(void* p, float u1, float u2, float* dir, float* pdf, float* weight) {
    Handle* H = static_cast<Handle*>(p);
    if (!H->s32.env) return -1;
    BackgroundSample<float> s = H->s32.env->SampleDirection(V2<float>(u1, u2));
    dir[0] = s.Direction.x; dir[1] = s.Direction.y; dir[2] = s.Direction.z;
    *pdf = s.Pdf;
    weight[0] = s.Weight.r; weight[1] = s.Weight.g; weight[2] = s.Weight.b;
    return 0;
}
float ora_env_pdf(void* p, const float* dir) {
    Handle* H = static_cast<Handle*>(p);
    return H->s32.env ? H->s32.env->DirectionPdf(V3<float>(dir[0], dir[1], dir[2])) : 0.0f;
}

// ---- stateless pieces for the known-answer tests ----
uint32_t ora_rng_hashseed(uint32_t b, uint32_t c, uint32_t s) { return Rng::HashSeed(b, c, s); }
void ora_rng_stream(uint32_t seed, int n, uint32_t* out) { Rng r(seed); for (int i = 0; i < n; ++i) out[i] = r.Next(); }
void ora_rng_floats(uint32_t seed, int n, float* out) { Rng r(seed); for (int i = 0; i < n; ++i) out[i] = r.NextFloat(); }
void ora_rng_ints(uint32_t seed, uint32_t max, int n, uint32_t* out, uint32_t* finalState) {
    Rng r(seed); for (int i = 0; i < n; ++i) out[i] = r.NextInt(max);
    if (finalState) *finalState = r.state;
}

float ora_ggx_D(float ax, float ay, const float* n) { return GGX<float>{ax, ay}.D(V3<float>(n[0], n[1], n[2])); }
float ora_ggx_pdf(float ax, float ay, const float* o, const float* n) { return GGX<float>{ax, ay}.Pdf(V3<float>(o[0], o[1], o[2]), V3<float>(n[0], n[1], n[2])); }
void ora_ggx_sample(float ax, float ay, const float* o, float u1, float u2, float* out) {
    V3<float> r = GGX<float>{ax, ay}.Sample(V3<float>(o[0], o[1], o[2]), V2<float>(u1, u2));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void ora_world_to_shading(const float* n, const float* d, float* out) {
    V3<float> r = WorldToShading(V3<float>(n[0], n[1], n[2]), V3<float>(d[0], d[1], d[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void ora_shading_to_world(const float* n, const float* d, float* out) {
    V3<float> r = ShadingToWorld(V3<float>(n[0], n[1], n[2]), V3<float>(d[0], d[1], d[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
// Piecewise-constant distribution: sample n values u[i] -> (idx, rel); prob[k] for all bins.
void ora_pwc(const float* w, int nw, const float* u, int n, int* idx, float* rel, float* prob) {
    PiecewiseConstant<float> d(w, nw);
    for (int i = 0; i < n; ++i) d.Sample(u[i], idx[i], rel[i]);
    if (prob) for (int k = 0; k < nw; ++k) prob[k] = d.Probability(k);
}
void ora_warp_triangle(float u1, float u2, float* bary, float* inv) {
    V2<float> b = ToUniformTriangle(V2<float>(u1, u2));
    V2<float> i = FromUniformTriangle(b);
    bary[0] = b.x; bary[1] = b.y; inv[0] = i.x; inv[1] = i.y;
}
void ora_warp_sphere(float u1, float u2, float* dir, float* inv) {
    DirectionSample<float> d = ToUniformSphere(V2<float>(u1, u2));
    V2<float> i = FromUniformSphere(d.Direction);
    dir[0] = d.Direction.x; dir[1] = d.Direction.y; dir[2] = d.Direction.z; inv[0] = i.x; inv[1] = i.y;
}
void ora_warp_coshemi(float u1, float u2, float* dir, float* pdf, float* inv) {
    DirectionSample<float> d = ToCosHemisphere(V2<float>(u1, u2));
    V2<float> i = FromCosHemisphere(d.Direction);
    dir[0] = d.Direction.x; dir[1] = d.Direction.y; dir[2] = d.Direction.z; *pdf = d.Pdf; inv[0] = i.x; inv[1] = i.y;
}
void ora_warp_disc(float u1, float u2, float* pos) {
    V2<float> r = ToConcentricDisc(V2<float>(u1, u2));
    pos[0] = r.x; pos[1] = r.y;
}
float ora_fresnel_dielectric(float c, float ei, float et) { return FresnelDielectric(c, ei, et); }

// Emitter/mesh sampling at the scene level: sample emitter e with primary (u1, u2); out = pos 3,
// normal 3, shading normal 3, pdf.
// Emitter.SampleRay followed by Emitter.SampleRayInverse (DiffuseEmitter.cs:44-79,
// GlossyEmitter.cs:47-86): the inverse maps the sampled point back through
// SampleWarp.FromUniformTriangle (:16-22) and the direction, in the shading frame of the point,
// through FromCosHemisphere (:139-145) or FromCosineLobe(exponent + 1) (:184-190).
// out: posPrimary (2), dirPrimary (2), point (3), direction (3), pdf, weight (3).
int ora_emitter_ray_roundtrip(void* p, int e, const float* primPos, const float* primDir, float* out) {
    Handle* H = static_cast<Handle*>(p);
    const Scene<float>& sc = H->s32;
    if (e < 0 || e >= int(sc.emitters.size())) return -1;
    const Emitter<float>& em = sc.emitters[e];
    EmitterRaySample<float> r = EmitterSampleRay(sc, em, V2<float>(primPos[0], primPos[1]), V2<float>(primDir[0], primDir[1]));
    V2<float> posP = FromUniformTriangle(r.point.bary);
    V3<float> n = r.point.shadingNormal, t, b;
    ComputeBasisVectors(n, t, b);
    V3<float> local(dot(t, r.dir), dot(b, r.dir), dot(n, r.dir));
    V2<float> dirP;
    if (!em.glossy()) {
        dirP = FromCosHemisphere(local);
    } else {
        V2<float> sph = CartesianToSpherical(local);
        float x = sph.x / (2.0f * PI<float>());
        float c = std::cos(sph.y);
        dirP = V2<float>(x, std::pow(c, (em.exponent + 1.0f) + 1.0f));
    }
    out[0] = posP.x; out[1] = posP.y; out[2] = dirP.x; out[3] = dirP.y;
    out[4] = r.point.position.x; out[5] = r.point.position.y; out[6] = r.point.position.z;
    out[7] = r.dir.x; out[8] = r.dir.y; out[9] = r.dir.z;
    out[10] = r.pdf; out[11] = r.weight.r; out[12] = r.weight.g; out[13] = r.weight.b;
    return 0;
}

// Mesh.ComputeShadingNormal (Geometry/Mesh.cs) of a face at barycentrics (u, v).
int ora_mesh_shading_normal(void* p, int mesh, int face, float u, float v, float* out) {
    Handle* H = static_cast<Handle*>(p);
    const Scene<float>& sc = H->s32;
    if (mesh < 0 || mesh >= int(sc.meshes.size()) || face < 0 || face >= sc.meshes[mesh].numFaces()) return -1;
    V3<float> n = sc.meshes[mesh].ShadingNormal(face, V2<float>(u, v));
    out[0] = n.x; out[1] = n.y; out[2] = n.z;
    return 0;
}

int ora_emitter_sample(void* p, int e, float u1, float u2, float* out) {
    Handle* H = static_cast<Handle*>(p);
    const Scene<float>& sc = H->s32;
    SurfacePoint<float> lp = SampleEmitterArea(sc, sc.emitters[e], V2<float>(u1, u2));
    out[0] = lp.position.x; out[1] = lp.position.y; out[2] = lp.position.z;
    out[3] = lp.normal.x; out[4] = lp.normal.y; out[5] = lp.normal.z;
    out[6] = lp.shadingNormal.x; out[7] = lp.shadingNormal.y; out[8] = lp.shadingNormal.z;
    out[9] = sc.emitters[e].invArea;
    return 0;
}
int ora_emitter_radiance(void* p, int e, const float* pt, const float* dir, float* rgb) {
    Handle* H = static_cast<Handle*>(p);
    SurfacePoint<float> sp = PointFrom<float>(pt);
    Rgb<float> c = H->s32.emitters[e].EmittedRadiance(sp, V3<float>(dir[0], dir[1], dir[2]));
    rgb[0] = c.r; rgb[1] = c.g; rgb[2] = c.b;
    return 0;
}
// Emitter index at a (mesh, face), or -1 (Scene.QueryEmitter, Scene.cs:204-210)
int ora_query_emitter(void* p, int mesh, int face) {
    Handle* H = static_cast<Handle*>(p);
    const Scene<float>& sc = H->s32;
    return sc.triEmitter[sc.meshTriOffset[mesh] + face];
}

}  // extern "C"

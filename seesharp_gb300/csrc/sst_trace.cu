// K3/K4: BVH traversal for sm_103a -- TinyEmbree Raytracer.Trace / IsOccluded / LeavesScene
// (Integrators/PathTracer.cs:319,428,467).
//
// Binary BVH with both child boxes stored in the parent (64-byte nodes read as four 128-bit
// loads), or the 4-wide (128-byte nodes) or 8-wide (240-byte nodes, children in octant slots) BVH
// over the same leaves, watertight ray/triangle test (Woop, Benthin, Wald 2013), a per-thread
// traversal stack in shared memory with a local-memory tail, and persistent warps: the binary
// kernel fetches 32 rays at a time, the wide ones replace finished rays once a set number of the
// warp's lanes are idle.
// The block size and the number of stack entries kept in shared memory are template parameters;
// the autotuner picks one of the instantiated variants per context (TraceTuning).  The result of
// a query does not depend on the variant: the traversal order is the same, and closest-hit ties
// resolve to the smaller global triangle id.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "sst_device.cuh"
#include "sst_kernels.h"

namespace sst {

struct RayPre {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
SST_D float comp(float3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
SST_D RayPre rayPre(float3 d) {
    RayPre p;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    p.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    p.kx = p.kz == 2 ? 0 : p.kz + 1;
    p.ky = p.kx == 2 ? 0 : p.kx + 1;
    float dz = comp(d, p.kz);
    if (dz < 0.0f) { int t = p.kx; p.kx = p.ky; p.ky = t; }
    p.Sx = comp(d, p.kx) / dz;
    p.Sy = comp(d, p.ky) / dz;
    p.Sz = 1.0f / dz;
    return p;
}
// Returns true with t, u (2nd vertex weight), v (3rd vertex weight) when tmin < t < tmax.
SST_D bool isectTri(float3 o, const RayPre& p, float3 v0, float3 v1, float3 v2, float tmin, float tmax, float& t, float& u, float& v) {
    float3 A = v0 - o, B = v1 - o, C = v2 - o;
    float Az_ = comp(A, p.kz), Bz_ = comp(B, p.kz), Cz_ = comp(C, p.kz);
    float Ax = comp(A, p.kx) - p.Sx * Az_, Ay = comp(A, p.ky) - p.Sy * Az_;
    float Bx = comp(B, p.kx) - p.Sx * Bz_, By = comp(B, p.ky) - p.Sy * Bz_;
    float Cx = comp(C, p.kx) - p.Sx * Cz_, Cy = comp(C, p.ky) - p.Sy * Cz_;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {  // edge case: exact evaluation in double
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * (p.Sz * Az_) + V * (p.Sz * Bz_) + W * (p.Sz * Cz_);
    float rcp = 1.0f / det;
    float tt = T * rcp;
    if (!(tt > tmin) || !(tt < tmax)) return false;
    t = tt;
    u = V * rcp;
    v = W * rcp;
    return true;
}

struct TraceResult {
    float t, u, v;
    int tri;  // leaf-ordered triangle, -1 for a miss
};

struct Bvh {
    const float4* nodes;
    const float4* triv;
    int nNodes;
};
SST_D Bvh bvhOf(const DevScene& sc) { return Bvh{sc.nodes, sc.triv, sc.nNodes}; }

// Closest hit (ANY = false; ties in t resolve to the smaller global triangle id) or any hit.
// sstack: this block's shared stack, SSTACK entries per thread, entry k of thread `tid` at
// k * BLOCK + tid (consecutive threads in consecutive banks).
template <bool ANY, int BLOCK, int SSTACK>
SST_D TraceResult traverse(const Bvh sc, float3 org, float3 dir, float tmin, float tmax, int* sstack, int* errFlags) {
    TraceResult r{tmax, 0.f, 0.f, -1};
    if (sc.nNodes == 0 || !(tmax > tmin)) return r;
    int bestGid = 0x7FFFFFFF;
    RayPre pre = rayPre(dir);
    float3 inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    float3 oi = mk(-org.x * inv.x, -org.y * inv.y, -org.z * inv.z);
    int lstack[kMaxStack - SSTACK];
    int sp = 0;
    uint32_t ref = 0;  // root inner node
    const int tid = threadIdx.x;
    for (;;) {
        if (!(ref & kLeafFlag)) {
            const float4* nd = sc.nodes + 4 * (size_t)ref;
            float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
            float hitT = r.t * 1.0000004f;  // conservative far bound (box/triangle rounding)
            // child 0
            float a0 = fmaf(n0.x, inv.x, oi.x), b0 = fmaf(n0.y, inv.x, oi.x);
            float c0 = fmaf(n0.z, inv.y, oi.y), d0 = fmaf(n0.w, inv.y, oi.y);
            float e0 = fmaf(n2.x, inv.z, oi.z), f0 = fmaf(n2.y, inv.z, oi.z);
            float tn0 = fmaxf(fmaxf(fminf(a0, b0), fminf(c0, d0)), fmaxf(fminf(e0, f0), tmin));
            float tf0 = fminf(fminf(fmaxf(a0, b0), fmaxf(c0, d0)), fminf(fmaxf(e0, f0), hitT));
            // child 1
            float a1 = fmaf(n1.x, inv.x, oi.x), b1 = fmaf(n1.y, inv.x, oi.x);
            float c1 = fmaf(n1.z, inv.y, oi.y), d1 = fmaf(n1.w, inv.y, oi.y);
            float e1 = fmaf(n2.z, inv.z, oi.z), f1 = fmaf(n2.w, inv.z, oi.z);
            float tn1 = fmaxf(fmaxf(fminf(a1, b1), fminf(c1, d1)), fmaxf(fminf(e1, f1), tmin));
            float tf1 = fminf(fminf(fmaxf(a1, b1), fmaxf(c1, d1)), fminf(fmaxf(e1, f1), hitT));
            bool h0 = tn0 <= tf0 * 1.0000004f, h1 = tn1 <= tf1 * 1.0000004f;
            uint32_t r0 = __float_as_uint(n3.x), r1 = __float_as_uint(n3.y);
            if (h0 && h1) {
                uint32_t nearR = r0, farR = r1;
                if (tn1 < tn0) { nearR = r1; farR = r0; }
                if (sp < SSTACK) sstack[sp * BLOCK + tid] = (int)farR;
                else if (sp < kMaxStack) lstack[sp - SSTACK] = (int)farR;
                else { atomicOr(errFlags, 1); return r; }
                ++sp;
                ref = nearR;
                continue;
            } else if (h0) { ref = r0; continue; }
            else if (h1) { ref = r1; continue; }
        } else {
            int first = (int)(ref & kLeafFirstMask);
            int cnt = (int)((ref >> kLeafCountShift) & 0xF) + 1;
            for (int k = 0; k < cnt; ++k) {
                int ti = first + k;
                float4 a = __ldg(&sc.triv[3 * (size_t)ti]), b = __ldg(&sc.triv[3 * (size_t)ti + 1]), c = __ldg(&sc.triv[3 * (size_t)ti + 2]);
                float t, u, v;
                // allow an equal distance so that ties can resolve to the smaller id
                float lim = ANY ? r.t : __uint_as_float(__float_as_uint(r.t) + (r.t < CUDART_INF_F ? 1u : 0u));
                if (isectTri(org, pre, f3(a), f3(b), f3(c), tmin, lim, t, u, v)) {
                    int gid = __float_as_int(a.w);
                    if (ANY) { r.t = t; r.u = u; r.v = v; r.tri = ti; return r; }
                    if (t < r.t || (t == r.t && gid < bestGid)) { r.t = t; r.u = u; r.v = v; r.tri = ti; bestGid = gid; }
                }
            }
        }
        if (sp == 0) break;
        --sp;
        ref = (uint32_t)(sp < SSTACK ? sstack[sp * BLOCK + tid] : lstack[sp - SSTACK]);
    }
    return r;
}

// 4-wide traversal over the same leaves.  Per node: the four slab tests, the hit children
// ordered by entry distance (a 5-comparator network), the nearest one visited next and the others
// pushed farthest first.  SSTACK entries per thread in shared memory, the rest in local memory
// (kMaxStack4 bounds three pending children per level).
struct Bvh4 {
    const float4* nodes4;
    const float4* triv;
    int nNodes4;
};
SST_D Bvh4 bvh4Of(const DevScene& sc) { return Bvh4{sc.nodes4, sc.triv, sc.nNodes4}; }

// Paired single precision (sm_100 and later): fma.rn.f32x2 rounds each half exactly as fmaf does,
// so the slab planes of two children cost one instruction instead of two.
SST_D float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\tmov.b64 pc, {%6, %7};\n\t"
        "fma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// Three-operand minimum and maximum (sm_100 and later): like two fminf / fmaxf, a NaN operand is
// ignored and the result is exact.
SST_D float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
SST_D float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// Entry and exit distances of four child boxes from their near- and far-plane rows (x, y, z each a
// float4 over the children): paired fused multiply-adds per plane row, then the three-operand
// max / min with the ray's interval.  Bitwise the scalar fmaf / fmaxf / fminf form.
SST_D void slab4(float4 nx, float4 fx, float4 ny, float4 fy, float4 nz, float4 fz, float3 inv, float3 oi, float tmin, float tmax,
                 float tn[4], float tf[4]) {
    const float2 ix = make_float2(inv.x, inv.x), iy = make_float2(inv.y, inv.y), iz = make_float2(inv.z, inv.z);
    const float2 ox = make_float2(oi.x, oi.x), oy = make_float2(oi.y, oi.y), oz = make_float2(oi.z, oi.z);
    const float2 nx0 = fma2(make_float2(nx.x, nx.y), ix, ox), nx1 = fma2(make_float2(nx.z, nx.w), ix, ox);
    const float2 ny0 = fma2(make_float2(ny.x, ny.y), iy, oy), ny1 = fma2(make_float2(ny.z, ny.w), iy, oy);
    const float2 nz0 = fma2(make_float2(nz.x, nz.y), iz, oz), nz1 = fma2(make_float2(nz.z, nz.w), iz, oz);
    const float2 fx0 = fma2(make_float2(fx.x, fx.y), ix, ox), fx1 = fma2(make_float2(fx.z, fx.w), ix, ox);
    const float2 fy0 = fma2(make_float2(fy.x, fy.y), iy, oy), fy1 = fma2(make_float2(fy.z, fy.w), iy, oy);
    const float2 fz0 = fma2(make_float2(fz.x, fz.y), iz, oz), fz1 = fma2(make_float2(fz.z, fz.w), iz, oz);
    tn[0] = max3f(nx0.x, ny0.x, fmaxf(nz0.x, tmin));
    tn[1] = max3f(nx0.y, ny0.y, fmaxf(nz0.y, tmin));
    tn[2] = max3f(nx1.x, ny1.x, fmaxf(nz1.x, tmin));
    tn[3] = max3f(nx1.y, ny1.y, fmaxf(nz1.y, tmin));
    tf[0] = min3f(fx0.x, fy0.x, fminf(fz0.x, tmax));
    tf[1] = min3f(fx0.y, fy0.y, fminf(fz0.y, tmax));
    tf[2] = min3f(fx1.x, fy1.x, fminf(fz1.x, tmax));
    tf[3] = min3f(fx1.y, fy1.y, fminf(fz1.y, tmax));
}

SST_D void cswap(float& ka, uint32_t& ra, float& kb, uint32_t& rb) {
    bool s = kb < ka;
    float k = s ? kb : ka;
    kb = s ? ka : kb;
    ka = k;
    uint32_t r = s ? rb : ra;
    rb = s ? ra : rb;
    ra = r;
}

// One lane's 4-wide traversal, resumable: the next node to visit, the stack depth and the closest
// hit so far stay in the structure when trav4Run pauses.
struct Trav4 {
    Bvh4 bvh;
    float3 org, inv, oi;
    RayPre pre;
    float tmin;
    TraceResult r;
    int bestGid;
    int sp;
    uint32_t ref;
    uint32_t oct;  // sign bits of the inverse direction: which plane of each slab is the near one
    bool done;
};

SST_D void trav4Begin(Trav4& s, const Bvh4 bvh, float3 org, float3 dir, float tmin, float tmax) {
    s.bvh = bvh;
    s.org = org;
    s.pre = rayPre(dir);
    s.inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    s.oi = mk(-org.x * s.inv.x, -org.y * s.inv.y, -org.z * s.inv.z);
    s.oct = (s.inv.x < 0.0f ? 1u : 0u) | (s.inv.y < 0.0f ? 2u : 0u) | (s.inv.z < 0.0f ? 4u : 0u);
    s.tmin = tmin;
    s.r = TraceResult{tmax, 0.f, 0.f, -1};
    s.bestGid = 0x7FFFFFFF;
    s.sp = 0;
    s.ref = 0;  // root
    s.done = bvh.nNodes4 == 0 || !(tmax > tmin);
}

// Traversal steps until the ray is finished (returns true, result in s.r) or, with pauseIdle > 0,
// until pauseIdle lanes of the warp are outside this loop (returns false after at least one
// step; a later call resumes).  The lanes are counted at the loop head, where every lane still
// traversing reconverges (__activemask counts the lanes converged at the instruction: counted
// after a stack pop instead, the lanes that had just descended were missing, warps paused after
// almost every step, and traversal was 45% slower).  lstack: this lane's local-memory stack tail.
template <bool ANY, int BLOCK, int SSTACK>
SST_D bool trav4Run(Trav4& s, int* sstack, int* lstack, int* errFlags, int pauseIdle) {
    const int tid = threadIdx.x;
    const Bvh4& sc = s.bvh;
    bool first = true;
    for (;;) {
        if (!first && pauseIdle > 0 && 32 - __popc(__activemask()) >= pauseIdle) return false;
        first = false;
        const uint32_t ref = s.ref;
        if (!(ref & kLeafFlag)) {
            const float4* nd = sc.nodes4 + 8 * (size_t)ref;
            // the near plane of each slab is lo for a positive direction component and hi for a
            // negative one; its t is then the smaller of the two (fma rounding is monotonic), so
            // reading the near and far planes directly gives the min / max of both without computing
            // them.  With an infinite inverse (a zero component) a NaN slab is ignored, which keeps
            // at least the boxes the min / max form keeps.
            const int ox = (int)(s.oct & 1u), oy = (int)((s.oct >> 1) & 1u), oz = (int)((s.oct >> 2) & 1u);
            const float4 nx = __ldg(nd + ox), fx = __ldg(nd + 1 - ox), ny = __ldg(nd + 2 + oy), fy = __ldg(nd + 3 - oy);
            const float4 nz = __ldg(nd + 4 + oz), fz = __ldg(nd + 5 - oz);
            const float4 rf = __ldg(nd + 6), meta = __ldg(nd + 7);
            const int cnt = __float_as_int(meta.x);
            const float hitT = s.r.t * 1.0000004f;  // conservative far bound (box/triangle rounding)
            float key[4];
            uint32_t cr[4];
            const float* RF = &rf.x;
            float tn[4], tf[4];
            slab4(nx, fx, ny, fy, nz, fz, s.inv, s.oi, s.tmin, hitT, tn, tf);
            int nh = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                bool hit = k < cnt && tn[k] <= tf[k] * 1.0000004f;
                key[k] = hit ? tn[k] : CUDART_INF_F;
                cr[k] = __float_as_uint(RF[k]);
                nh += hit ? 1 : 0;
            }
            if (nh > 0) {
                // ascending by entry distance; children that were not hit sort last (key = inf)
                cswap(key[0], cr[0], key[1], cr[1]);
                cswap(key[2], cr[2], key[3], cr[3]);
                cswap(key[0], cr[0], key[2], cr[2]);
                cswap(key[1], cr[1], key[3], cr[3]);
                cswap(key[1], cr[1], key[2], cr[2]);
                // push the farther hit children, farthest first
                for (int k = nh - 1; k >= 1; --k) {
                    uint32_t pr = k == 3 ? cr[3] : (k == 2 ? cr[2] : cr[1]);
                    if (s.sp < SSTACK) sstack[s.sp * BLOCK + tid] = (int)pr;
                    else if (s.sp < kMaxStack4) lstack[s.sp - SSTACK] = (int)pr;
                    else { atomicOr(errFlags, 1); return true; }
                    ++s.sp;
                }
                s.ref = cr[0];
                continue;
            }
        } else {
            int firstTri = (int)(ref & kLeafFirstMask);
            int cnt = (int)((ref >> kLeafCountShift) & 0xF) + 1;
            for (int k = 0; k < cnt; ++k) {
                int ti = firstTri + k;
                float4 a = __ldg(&sc.triv[3 * (size_t)ti]), b = __ldg(&sc.triv[3 * (size_t)ti + 1]), c = __ldg(&sc.triv[3 * (size_t)ti + 2]);
                float t, u, v;
                // allow an equal distance so that ties can resolve to the smaller id
                float lim = ANY ? s.r.t : __uint_as_float(__float_as_uint(s.r.t) + (s.r.t < CUDART_INF_F ? 1u : 0u));
                if (isectTri(s.org, s.pre, f3(a), f3(b), f3(c), s.tmin, lim, t, u, v)) {
                    int gid = __float_as_int(a.w);
                    if (ANY) { s.r.t = t; s.r.u = u; s.r.v = v; s.r.tri = ti; return true; }
                    if (t < s.r.t || (t == s.r.t && gid < s.bestGid)) { s.r.t = t; s.r.u = u; s.r.v = v; s.r.tri = ti; s.bestGid = gid; }
                }
            }
        }
        if (s.sp == 0) return true;
        --s.sp;
        s.ref = (uint32_t)(s.sp < SSTACK ? sstack[s.sp * BLOCK + tid] : lstack[s.sp - SSTACK]);
    }
}

// 8-wide traversal over the same leaves, children in octant slots (sst_bvh.cu).  A ray visits a
// node's hit children in the order slot ^ o ascending, o the sign bits of its direction, which
// approximates front to back without a sort.  A node visit tests the eight child boxes against the
// near and far planes the direction selects (the near-plane arrays are read directly, so every
// slab is one fused multiply-add).  It is the other widths' arithmetic: with a finite inverse
// direction the near plane's t is the smaller of the two, so a box passes here exactly when it
// passes there, and with an infinite one (a zero direction component) a NaN slab is ignored, which
// passes at least the boxes the other widths pass.  The hit children become a bit mask in visiting
// order.  The
// traversal keeps one (node, remaining mask) group in registers; moving to an inner child pushes
// the rest of the group as one stack entry (node << 8 | mask), and a leaf child is tested in
// place.  SSTACK entries per thread in shared memory, the rest in local memory (the depth of the
// tree bounds the stack).
struct Bvh8 {
    const float4* nodes8;
    const float4* triv;
    int nNodes8;
};
SST_D Bvh8 bvh8Of(const DevScene& sc) { return Bvh8{sc.nodes8, sc.triv, sc.nNodes8}; }

struct Trav8 {
    Bvh8 bvh;
    float3 org, inv, oi;
    RayPre pre;
    float tmin;
    TraceResult r;
    int bestGid;
    int sp;
    uint32_t node;  // the group in registers: an 8-wide node ...
    uint32_t mask;  // ... and its hit children not yet visited (bit j: slot j ^ oct)
    uint32_t oct;   // sign bits of the direction (bit a set when inv[a] < 0)
    bool done;
};

// Mask of the hit children of `node` in visiting order (bit j set: slot j ^ oct was hit).
SST_D uint32_t visit8(const Trav8& s, uint32_t node) {
    const float4* nd = s.bvh.nodes8 + 15 * (size_t)node;
    const int ox = (int)(s.oct & 1u), oy = (int)((s.oct >> 1) & 1u), oz = (int)((s.oct >> 2) & 1u);
    const uint32_t valid = __float_as_uint(__ldg(&nd[14].x)) & 0xFFu;
    const float hitT = s.r.t * 1.0000004f;  // conservative far bound (box/triangle rounding)
    uint32_t hm = 0;
    // two halves of four children (24 box floats live at a time); near planes: lo for a positive
    // direction component, hi for a negative one
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float4 nx = __ldg(nd + 2 * ox + h), fx = __ldg(nd + 2 - 2 * ox + h);
        const float4 ny = __ldg(nd + 4 + 2 * oy + h), fy = __ldg(nd + 6 - 2 * oy + h);
        const float4 nz = __ldg(nd + 8 + 2 * oz + h), fz = __ldg(nd + 10 - 2 * oz + h);
        float tn[4], tf[4];
        slab4(nx, fx, ny, fy, nz, fz, s.inv, s.oi, s.tmin, hitT, tn, tf);
#pragma unroll
        for (int k = 0; k < 4; ++k) hm |= (tn[k] <= tf[k] * 1.0000004f) ? (1u << (4 * h + k)) : 0u;
    }
    hm &= valid;
    // slot k -> bit k ^ oct
    if (s.oct & 1u) hm = ((hm & 0x55u) << 1) | ((hm >> 1) & 0x55u);
    if (s.oct & 2u) hm = ((hm & 0x33u) << 2) | ((hm >> 2) & 0x33u);
    if (s.oct & 4u) hm = ((hm & 0x0Fu) << 4) | ((hm >> 4) & 0x0Fu);
    return hm;
}

SST_D void trav8Begin(Trav8& s, const Bvh8 bvh, float3 org, float3 dir, float tmin, float tmax) {
    s.bvh = bvh;
    s.org = org;
    s.pre = rayPre(dir);
    s.inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    s.oi = mk(-org.x * s.inv.x, -org.y * s.inv.y, -org.z * s.inv.z);
    s.oct = (s.inv.x < 0.0f ? 1u : 0u) | (s.inv.y < 0.0f ? 2u : 0u) | (s.inv.z < 0.0f ? 4u : 0u);
    s.tmin = tmin;
    s.r = TraceResult{tmax, 0.f, 0.f, -1};
    s.bestGid = 0x7FFFFFFF;
    s.sp = 0;
    s.node = 0;
    s.done = bvh.nNodes8 == 0 || !(tmax > tmin);
    s.mask = s.done ? 0u : visit8(s, 0u);  // the root's hit children
    if (!s.done && s.mask == 0u) s.done = true;
}

// Traversal steps until the ray is finished (true, result in s.r) or, with pauseIdle > 0, until
// pauseIdle lanes of the warp are outside this loop (false after at least one step; a later call
// resumes).  lstack: this lane's local-memory stack tail.
template <bool ANY, int BLOCK, int SSTACK>
SST_D bool trav8Run(Trav8& s, int* sstack, int* lstack, int* errFlags, int pauseIdle) {
    const int tid = threadIdx.x;
    bool first = true;
    for (;;) {
        if (!first && pauseIdle > 0 && 32 - __popc(__activemask()) >= pauseIdle) return false;
        first = false;
        if (s.mask == 0u) {
            if (s.sp == 0) return true;
            --s.sp;
            const uint32_t e = (uint32_t)(s.sp < SSTACK ? sstack[s.sp * BLOCK + tid] : lstack[s.sp - SSTACK]);
            s.node = e >> 8;
            s.mask = e & 0xFFu;
        }
        const uint32_t j = (uint32_t)(__ffs((int)s.mask) - 1);
        s.mask &= s.mask - 1u;
        const uint32_t slot = j ^ s.oct;
        const uint32_t ref = __float_as_uint(__ldg(reinterpret_cast<const float*>(s.bvh.nodes8 + 15 * (size_t)s.node + 12) + slot));
        if (!(ref & kLeafFlag)) {
            if (s.mask) {
                const int e = (int)((s.node << 8) | s.mask);
                if (s.sp < SSTACK) sstack[s.sp * BLOCK + tid] = e;
                else if (s.sp < kMaxStack) lstack[s.sp - SSTACK] = e;
                else { atomicOr(errFlags, 1); return true; }
                ++s.sp;
            }
            s.node = ref;
            s.mask = visit8(s, ref);
        } else {
            const int firstTri = (int)(ref & kLeafFirstMask);
            const int cnt = (int)((ref >> kLeafCountShift) & 0xF) + 1;
            for (int k = 0; k < cnt; ++k) {
                const int ti = firstTri + k;
                const float4 a = __ldg(&s.bvh.triv[3 * (size_t)ti]), b = __ldg(&s.bvh.triv[3 * (size_t)ti + 1]), c = __ldg(&s.bvh.triv[3 * (size_t)ti + 2]);
                float t, u, v;
                // allow an equal distance so that ties can resolve to the smaller id
                const float lim = ANY ? s.r.t : __uint_as_float(__float_as_uint(s.r.t) + (s.r.t < CUDART_INF_F ? 1u : 0u));
                if (isectTri(s.org, s.pre, f3(a), f3(b), f3(c), s.tmin, lim, t, u, v)) {
                    const int gid = __float_as_int(a.w);
                    if (ANY) { s.r.t = t; s.r.u = u; s.r.v = v; s.r.tri = ti; return true; }
                    if (t < s.r.t || (t == s.r.t && gid < s.bestGid)) { s.r.t = t; s.r.u = u; s.r.v = v; s.r.tri = ti; s.bestGid = gid; }
                }
            }
        }
    }
}

// The resumable traversals (4- and 8-wide) behind one interface for the kernel's refill loop.
template <int W> struct WideTrav;
template <> struct WideTrav<4> {
    using State = Trav4;
    static constexpr int kStack = kMaxStack4;
    SST_D static void begin(State& s, const DevScene& sc, float3 o, float3 d, float tmin, float tmax) { trav4Begin(s, bvh4Of(sc), o, d, tmin, tmax); }
    template <bool ANY, int BLOCK, int SSTACK>
    SST_D static bool run(State& s, int* sstack, int* lstack, int* err, int pause) { return trav4Run<ANY, BLOCK, SSTACK>(s, sstack, lstack, err, pause); }
};
template <> struct WideTrav<8> {
    using State = Trav8;
    static constexpr int kStack = kMaxStack;
    SST_D static void begin(State& s, const DevScene& sc, float3 o, float3 d, float tmin, float tmax) { trav8Begin(s, bvh8Of(sc), o, d, tmin, tmax); }
    template <bool ANY, int BLOCK, int SSTACK>
    SST_D static bool run(State& s, int* sstack, int* lstack, int* err, int pause) { return trav8Run<ANY, BLOCK, SSTACK>(s, sstack, lstack, err, pause); }
};

// mode 0: closest hit -> hits[i]; mode 1: shadow rays, zero nee[tgt[i]] when occluded;
// mode 2: any hit -> occl[i] = 1/0.
// Resident threads per SM the traversal kernels are compiled for (register budget); 0: no bound.
// 1024 caps every block size at 64 registers: shadow rays 3% faster on the 1M-triangle scene than
// the unbounded build (66 registers for closest hit); 1280 (48 registers) is 10-30% slower.
#ifndef SST_TRACE_MIN_THREADS
#define SST_TRACE_MIN_THREADS 1024
#endif
// The 8-wide traversal keeps more per-ray state: at 64 registers it spills; 896 resident threads
// per SM give it 72.
#ifndef SST_TRACE8_MIN_THREADS
#define SST_TRACE8_MIN_THREADS 896
#endif
template <int MODE, int BLOCK, int SSTACK, int W>
__global__ void __launch_bounds__(BLOCK, (W == 8 ? SST_TRACE8_MIN_THREADS : SST_TRACE_MIN_THREADS) > 0
                                             ? (W == 8 ? SST_TRACE8_MIN_THREADS : SST_TRACE_MIN_THREADS) / BLOCK : 1) k_trace(const DevJob* __restrict__ jobs, const uint32_t* __restrict__ rayJob, const float4* ro,
                                                 const float4* rd, const int* count, int* work, float4* hits, const int* tgt, float4* nee,
                                                 int* occl, DevStats* stats, int countRays, int refillIdle) {
    __shared__ int sstack[SSTACK * BLOCK];
    const int n = *count;
    const int lane = threadIdx.x & 31;
    if (countRays && blockIdx.x == 0 && threadIdx.x == 0) {
        if (MODE == 0) atomicAdd(&stats->rays, (unsigned long long)n);
    }
    if constexpr (W != 2) {
        // Lanes whose ray is finished take new rays together once refillIdle of the warp's lanes
        // are idle (32: once the whole warp is); the others pause in place and resume after the
        // refill.  A scene without a wide BVH has no triangles: every ray misses.
        using T = WideTrav<W>;
        int lstack[T::kStack - SSTACK];
        typename T::State s;
        int i = -1;
        bool exhausted = false;
        const int thr = refillIdle > 0 && refillIdle < 32 ? refillIdle : 32;
        for (;;) {
            const unsigned idle = __ballot_sync(0xffffffffu, i < 0);
            if (!exhausted && __popc(idle) >= thr) {
                const int nIdle = __popc(idle);
                int base = 0;
                if (lane == 0) base = atomicAdd(work, nIdle);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base + nIdle >= n) exhausted = true;
                if (i < 0) {
                    const int j = base + __popc(idle & ((1u << lane) - 1u));
                    if (j < n) {
                        i = j;
                        const float4 o = ro[j], d = rd[j];
                        const uint32_t jb = rayJob ? rayJob[j] : 0u;
                        T::begin(s, jobs[jb].sc, f3(o), f3(d), o.w, d.w);
                    }
                }
            }
            if (__ballot_sync(0xffffffffu, i >= 0) == 0) break;  // every lane idle: the queue is drained
            if (i >= 0) {
                const bool fin = s.done || T::template run<MODE != 0, BLOCK, SSTACK>(s, sstack, lstack, &stats->errorFlags, exhausted ? 0 : thr);
                if (fin) {
                    const TraceResult& h = s.r;
                    if (MODE == 0) hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
                    else if (MODE == 1) { if (h.tri >= 0) nee[tgt[i]] = make_float4(0.f, 0.f, 0.f, 0.f); }
                    else occl[i] = h.tri >= 0 ? 1 : 0;
                    i = -1;
                }
            }
        }
    } else {
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        int i = base + lane;
        if (i < n) {
            float4 o = ro[i], d = rd[i];
            uint32_t jb = rayJob ? rayJob[i] : 0u;
            const DevScene& sc = jobs[jb].sc;
            TraceResult h = traverse<MODE != 0, BLOCK, SSTACK>(bvhOf(sc), f3(o), f3(d), o.w, d.w, sstack, &stats->errorFlags);
            if (MODE == 0) {
                hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
            } else if (MODE == 1) {
                if (h.tri >= 0) nee[tgt[i]] = make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                occl[i] = h.tri >= 0 ? 1 : 0;
            }
        }
    }
    }
}

// ---------------------------------------------------------------------------------------------
// Variant table: BVH width x block size x shared stack entries, for each of the three modes.
// ---------------------------------------------------------------------------------------------
using TraceKernel = void (*)(const DevJob*, const uint32_t*, const float4*, const float4*, const int*, int*, float4*, const int*, float4*, int*,
                             DevStats*, int, int);

template <int BLOCK, int SSTACK, int W>
struct TraceVariant {
    static constexpr TraceKernel k[3] = {k_trace<0, BLOCK, SSTACK, W>, k_trace<1, BLOCK, SSTACK, W>, k_trace<2, BLOCK, SSTACK, W>};
};

static const int kBlocks[3] = {64, 128, 256};
static const int kStacks[3] = {16, 24, 32};

static int indexOf(const int* a, int v) {
    for (int k = 0; k < 3; ++k)
        if (a[k] == v) return k;
    return -1;
}

// Variant index: (width 2, 4 or 8) x block x stack, 27 in all.
static int variantOf(const TraceTuning& t) {
    int bi = indexOf(kBlocks, t.block), si = indexOf(kStacks, t.smemStack);
    if (bi < 0 || si < 0 || (t.width != 2 && t.width != 4 && t.width != 8)) return -1;
    return (t.width == 8 ? 18 : (t.width == 4 ? 9 : 0)) + bi * 3 + si;
}

static TraceKernel traceKernel(int mode, int variant) {
#define SST_TV(B, S, W) TraceVariant<B, S, W>::k[mode]
    switch (variant) {
        case 0: return SST_TV(64, 16, 2);
        case 1: return SST_TV(64, 24, 2);
        case 2: return SST_TV(64, 32, 2);
        case 3: return SST_TV(128, 16, 2);
        case 4: return SST_TV(128, 24, 2);
        case 5: return SST_TV(128, 32, 2);
        case 6: return SST_TV(256, 16, 2);
        case 7: return SST_TV(256, 24, 2);
        case 8: return SST_TV(256, 32, 2);
        case 9: return SST_TV(64, 16, 4);
        case 10: return SST_TV(64, 24, 4);
        case 11: return SST_TV(64, 32, 4);
        case 12: return SST_TV(128, 16, 4);
        case 13: return SST_TV(128, 24, 4);
        case 14: return SST_TV(128, 32, 4);
        case 15: return SST_TV(256, 16, 4);
        case 16: return SST_TV(256, 24, 4);
        case 17: return SST_TV(256, 32, 4);
        case 18: return SST_TV(64, 16, 8);
        case 19: return SST_TV(64, 24, 8);
        case 20: return SST_TV(64, 32, 8);
        case 21: return SST_TV(128, 16, 8);
        case 22: return SST_TV(128, 24, 8);
        case 23: return SST_TV(128, 32, 8);
        case 24: return SST_TV(256, 16, 8);
        case 25: return SST_TV(256, 24, 8);
        default: return SST_TV(256, 32, 8);
    }
#undef SST_TV
}

bool traceTuningValid(const TraceTuning& t) { return variantOf(t) >= 0 && t.blocksPerSM >= 0 && t.refillIdle >= 1 && t.refillIdle <= 32; }

// Resident blocks per SM of a variant (occupancy) and the SM count, per device (the current one
// at the launch), computed on first use under a lock and kept.
constexpr int kTraceDevices = 64;
static std::mutex g_occLock;
static int g_occ[kTraceDevices][27];
static int g_sms[kTraceDevices];

static int currentDevice() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev >= 0 && dev < kTraceDevices ? dev : 0;
}

static int maxBlocksPerSM(int variant) {
    const int dev = currentDevice();
    std::lock_guard<std::mutex> lock(g_occLock);
    int& c = g_occ[dev][variant];
    if (c == 0) {
        int bps = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, traceKernel(0, variant), kBlocks[(variant % 9) / 3], 0);
        c = bps > 0 ? bps : 1;
    }
    return c;
}

static int numSMs() {
    const int dev = currentDevice();
    std::lock_guard<std::mutex> lock(g_occLock);
    int& sms = g_sms[dev];
    if (sms == 0) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

int traceGrid(const TraceTuning& t) {
    int v = variantOf(t);
    if (v < 0) v = 4;
    int m = maxBlocksPerSM(v);
    int b = t.blocksPerSM > 0 ? std::min(t.blocksPerSM, m) : m;
    return numSMs() * b;
}

int traceMaxBlocksPerSM(const TraceTuning& t) {
    int v = variantOf(t);
    return maxBlocksPerSM(v < 0 ? 4 : v);
}

static void launch(const TraceTuning& t, int mode, const DevJob* jobs, const uint32_t* rayJob, const float4* ro, const float4* rd, const int* count,
                   int* work, float4* hits, const int* tgt, float4* nee, int* occl, DevStats* stats, int countRays, cudaStream_t s) {
    int v = variantOf(t);
    if (v < 0) v = 4;  // 128 threads, 24 shared entries, binary
    traceKernel(mode, v)<<<traceGrid(t), kBlocks[(v % 9) / 3], 0, s>>>(jobs, rayJob, ro, rd, count, work, hits, tgt, nee, occl, stats, countRays,
                                                                        t.refillIdle);
}

void launch_trace_closest(const TraceTuning& t, const DevJob* jobs, const uint32_t* rayJob, const float4* ro, const float4* rd, const int* count,
                          int* work, float4* hits, DevStats* stats, cudaStream_t s) {
    launch(t, 0, jobs, rayJob, ro, rd, count, work, hits, nullptr, nullptr, nullptr, stats, 1, s);
}
void launch_trace_shadow(const TraceTuning& t, const DevJob* jobs, const uint32_t* rayJob, const float4* ro, const float4* rd, const int* tgt,
                         const int* count, int* work, float4* nee, DevStats* stats, cudaStream_t s) {
    launch(t, 1, jobs, rayJob, ro, rd, count, work, nullptr, tgt, nee, nullptr, stats, 0, s);
}
void launch_trace_query(const TraceTuning& t, const DevJob* jobs, const float4* ro, const float4* rd, const int* count, int* work, float4* hits,
                        int* occl, DevStats* stats, bool anyHit, cudaStream_t s) {
    if (anyHit) launch(t, 2, jobs, nullptr, ro, rd, count, work, nullptr, nullptr, nullptr, occl, stats, 0, s);
    else launch(t, 0, jobs, nullptr, ro, rd, count, work, hits, nullptr, nullptr, nullptr, stats, 0, s);
}

}  // namespace sst

// Wavefront path-tracing kernels for sm_103a.
//
//   k_env_build   -> EnvironmentMap.BuildSamplingGrid (Shading/Background/EnvironmentMap.cs:139-156)
//   k_camera      -> PathTracerBase.RenderPixel's camera ray (Integrators/PathTracer.cs:287-306)
//   k_trace       -> TinyEmbree Raytracer.Trace / IsOccluded / LeavesScene (PathTracer.cs:319,428,467)
//   k_shade       -> one bounce of EstimateIncidentRadiance (PathTracer.cs:318-378), with queue
//                    compaction and the FrameBuffer.Splat running mean (Images/FrameBuffer.cs:166-191)
#include <cuda_runtime.h>

#include "sst_kernels.h"
#include "sst_shade.cuh"


namespace sst {

// =============================================================================================
// K0: environment-map sampling tables.  One thread per row sums the row sequentially, exactly as
// RegularGrid2d.Splat/Normalize and the PiecewiseConstantPDF constructor do on the CPU
// (Sampling/RegularGrid2d.cs:62-81, Sampling/PiecewiseConstant.cs:12-29); the row distribution
// over the marginals is then built by a single thread.  Round-to-nearest intrinsics keep the
// additions uncontracted so the tables equal a scalar CPU build.
// =============================================================================================
__global__ void k_env_rows(const float4* img, int w, int h, float* colCdf, float* rowMarg, int* hasCol) {
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= h) return;
    float* cdf = colCdf + (size_t)row * w;
    float sum = 0.0f;
    for (int c = 0; c < w; ++c) {
        float4 p = img[(size_t)row * w + c];
        float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, p.x), __fmul_rn(0.7152f, p.y)), __fmul_rn(0.0722f, p.z));
        sum = __fadd_rn(sum, lum);
        cdf[c] = sum;
    }
    rowMarg[row] = sum;
    hasCol[row] = sum != 0.0f;
    if (sum > 0.0f)
        for (int c = 0; c < w; ++c) cdf[c] = __fdiv_rn(cdf[c], sum);
    cdf[w - 1] = 1.0f;
}
__global__ void k_env_marginal(const float* rowMarg, int h, float* rowCdf) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float sum = 0.0f;
    for (int r = 0; r < h; ++r) { sum = __fadd_rn(sum, rowMarg[r]); rowCdf[r] = sum; }
    if (sum > 0.0f)
        for (int r = 0; r < h; ++r) rowCdf[r] = __fdiv_rn(rowCdf[r], sum);
    rowCdf[h - 1] = 1.0f;
}

void launch_env_build(const float4* img, int w, int h, float* colCdf, float* rowMarg, int* hasCol, float* rowCdf, cudaStream_t s) {
    k_env_rows<<<(h + 127) / 128, 128, 0, s>>>(img, w, h, colCdf, rowMarg, hasCol);
    k_env_marginal<<<1, 32, 0, s>>>(rowMarg, h, rowCdf);
}

// =============================================================================================
// K2: camera rays.  Path p of the wave is pixel pixStart + p of iteration `iter`.
// =============================================================================================

__global__ void __launch_bounds__(256) k_camera(const DevJob* __restrict__ jobs, const WaveChunk* __restrict__ chunks, const WaveDesc* waves,
                                                const int* curWave, PathBuf A, int* qCount) {
    const WaveDesc wd = waves[*curWave];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *qCount = wd.items;
    if (i >= wd.items) return;
    int c = findChunk(chunks, wd.chunkBegin, wd.chunkEnd, i);
    const WaveChunk ck = chunks[c];
    const DevJob& jb = jobs[ck.job];
    int local = i - ck.itemOffset;
    int m = local / ck.pixCount;
    uint32_t pix = (uint32_t)(ck.pixStart + (local - m * ck.pixCount));
    uint32_t iter = (uint32_t)(ck.iterBase + m);
    uint32_t row = pix / (uint32_t)jb.cfg.W, col = pix - row * (uint32_t)jb.cfg.W;
    Rng rng{hashSeed(jb.cfg.baseSeed, pix, iter)};  // PathTracer.cs:236-237
    float ox = rng.nextFloat();                      // PathTracer.cs:289
    float oy = rng.nextFloat();
    float3 org, dir;
    cameraRay(jb.sc.cam, (float)col + ox, (float)row + oy, org, dir);
    A.job[i] = (uint32_t)ck.job;
    A.pix[i] = (uint32_t)i;  // wave item; the film fold maps it back to (iteration, pixel)
    A.rng[i] = rng.s;
    A.depth[i] = 1u;
    A.pw[i] = make_float4(1.f, 1.f, 1.f, 0.f);
    A.rad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    A.ro[i] = make_float4(org.x, org.y, org.z, 0.f);
    A.rd[i] = make_float4(dir.x, dir.y, dir.z, CUDART_INF_F);
    if (A.adjL) {
        // adjoint replay: the path's radiance from the forward pass and dLoss/dSample of its pixel
        const DevAdj& adj = jb.adj;
        size_t P = (size_t)jb.cfg.W * jb.cfg.H;
        const float* L = adj.record + 3 * ((size_t)iter * P + pix);
        float3 Lt = mk(L[0], L[1], L[2]);
        const float* g = adj.dLdI + 3 * (size_t)pix;
        float3 d = mk(g[0], g[1], g[2]) * adj.invSpp;
        if (!isfinite(avg3(Lt))) { Lt = mk(0, 0, 0); d = mk(0, 0, 0); }  // the film dropped this sample
        A.adjL[i] = make_float4(Lt.x, Lt.y, Lt.z, __int_as_float(-1));
        A.adjD[i] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    }
}

// OutlierReplayCache.Notify (Integrators/Util/OutlierReplayCache.cs:9-22): the pixel keeps the n
// samples of largest channel average in a .NET PriorityQueue, a 4-ary min-heap in an array.  While
// it holds fewer than n, Enqueue appends the sample and moves it up past every parent of strictly
// larger priority; after that EnqueueDequeue replaces the root only by a strictly larger sample and
// moves it down, each step to the first child of least priority, while that child is strictly
// smaller.  A sample that only ties the smallest kept one does not enter, and the array order is
// the reference's.
SST_D void outlierNotify(float* w, int* it, int& cnt, int n, float p, int iter) {
    int k;
    if (cnt < n) {
        k = cnt++;
        while (k > 0) {
            int par = (k - 1) >> 2;
            if (!(p < w[par])) break;
            w[k] = w[par];
            it[k] = it[par];
            k = par;
        }
    } else {
        if (cnt == 0 || !(p > w[0])) return;
        k = 0;
        for (;;) {
            int c = 4 * k + 1;
            if (c >= cnt) break;
            int m = c, e = min(c + 4, cnt);
            for (int j = c + 1; j < e; ++j)
                if (w[j] < w[m]) m = j;
            if (p <= w[m]) break;
            w[k] = w[m];
            it[k] = it[m];
            k = m;
        }
    }
    w[k] = p;
    it[k] = iter;
}

// =============================================================================================
// K8: fold the per-iteration path estimates of a wave into the film with the frame buffer's
// running mean: for iteration k (1-based) film = film * (k - 1) / k + v / k, non-finite
// estimates logged and skipped (FrameBuffer.Splat/Normalize, Images/FrameBuffer.cs:166-191, 232).
// =============================================================================================
// FrameBuffer.Splat's NaN / Inf log (Images/FrameBuffer.cs:166-179): counts every non-finite estimate
// and keeps the four smallest (iteration, pixel index) keys, the order in which a sequential render
// would log them.  An atomicMax cascade over the complemented keys: slot k keeps the largest
// complement that reaches it and passes the other value on, so slot k ends with the (k+1)-th smallest
// key of all values logged, whatever the order of the atomics.
__device__ __forceinline__ void logNan(DevStats* st, int iteration, int pixel) {
    atomicAdd(&st->nanCount, 1ull);
    unsigned long long v = ~(((unsigned long long)(unsigned)iteration << 32) | (unsigned)pixel);
    for (int k = 0; k < 4; ++k) {
        const unsigned long long old = atomicMax(&st->nanKey[k], v);
        if (old == 0ull) break;
        v = old < v ? old : v;
    }
}

SST_D float3 divRn(float3 a, float b) { return mk(__fdiv_rn(a.x, b), __fdiv_rn(a.y, b), __fdiv_rn(a.z, b)); }

__global__ void k_film_fold(const DevJob* __restrict__ jobs, const WaveChunk* __restrict__ chunks, const WaveDesc* waves, int* curWave,
                            const float* samples, DevStats* st, int advance) {
    const WaveDesc wd = waves[*curWave];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (samples && t < wd.foldThreads) {
        // chunk of this fold thread (sorted by foldOffset as well)
        int lo = wd.chunkBegin, hi = wd.chunkEnd;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (chunks[mid].foldOffset <= t) lo = mid; else hi = mid;
        }
        const WaveChunk ck = chunks[lo];
        const PTConfig& cfg = jobs[ck.job].cfg;
        int p = t - ck.foldOffset;
        size_t pix = (size_t)(ck.pixStart + p);
        float* f = ck.film + 3 * pix;
        float3 cur = mk(f[0], f[1], f[2]);
        const DevLayers& lay = jobs[ck.job].lay;
        float vMean = lay.varMean ? lay.varMean[pix] : 0.0f, vMoment = lay.varMoment ? lay.varMoment[pix] : 0.0f;
        float3 ref = lay.ref ? mk(lay.ref[3 * pix], lay.ref[3 * pix + 1], lay.ref[3 * pix + 2]) : mk(0, 0, 0);
        float3 alb = mk(0, 0, 0), nrm = mk(0, 0, 0);
        if (lay.aovAlbedo) {
            alb = mk(lay.aovAlbedo[3 * pix], lay.aovAlbedo[3 * pix + 1], lay.aovAlbedo[3 * pix + 2]);
            nrm = mk(lay.aovNormal[3 * pix], lay.aovNormal[3 * pix + 1], lay.aovNormal[3 * pix + 2]);
        }
        // the pixel's outlier heap (slots 0..cnt-1 are occupied, empty ones hold iteration -1)
        const int nOut = lay.nOut;
        float hw[kMaxOutliers];
        int hit[kMaxOutliers];
        int hcnt = 0;
        for (int j = 0; j < nOut; ++j) {
            hw[j] = lay.outW[pix * nOut + j];
            hit[j] = lay.outIt[pix * nOut + j];
            hcnt += hit[j] >= 0;
        }
        for (int m = 0; m < ck.nIter; ++m) {
            uint32_t iter = (uint32_t)(ck.iterBase + m);
            const float* s = samples + 3 * ((size_t)ck.itemOffset + (size_t)m * ck.pixCount + p);
            float3 v = mk(s[0], s[1], s[2]);
            float* rec = jobs[ck.job].adj.record;
            if (rec) {  // forward pass of the adjoint: keep every path's radiance
                float* r = rec + 3 * ((size_t)iter * cfg.W * cfg.H + pix);
                r[0] = v.x; r[1] = v.y; r[2] = v.z;
            }
            // the frame buffer's float arithmetic, correctly rounded whatever the unit's division flags
            const float kf = (float)(iter + 1);
            const float keep = __fdiv_rn(kf - 1.0f, kf);
            if (iter > 0) cur = cur * keep;
            float a = __fdiv_rn(v.x + v.y + v.z, 3.0f);  // RgbColor.Average
            bool finite = isfinite(a);
            if (!finite) logNan(st, (int)iter + 1, (int)pix);
            bool used = finite || !cfg.ignoreNan;
            if (used) cur = cur + divRn(v, kf);
            if (finite && nOut > 0) outlierNotify(hw, hit, hcnt, nOut, a, (int)iter);
            if (lay.aovAlbedo) {
                // RgbLayer running means (Images/Layer.cs:33-37, RgbLayer.cs:17-18)
                const float* a6 = lay.aovSamples + 6 * ((size_t)ck.itemOffset + (size_t)m * ck.pixCount + p);
                if (iter > 0) {
                    alb = alb * keep;
                    nrm = nrm * keep;
                }
                alb = alb + divRn(mk(a6[0], a6[1], a6[2]), kf);
                nrm = nrm + divRn(mk(a6[3], a6[4], a6[5]), kf);
            }
            if (lay.varMean) {
                // VarianceLayer (Images/VarianceLayer.cs:41-65): both images are running means of the
                // iteration's splatted value (the sample's channel average, 0 if it was skipped)
                float val = used ? a : 0.0f;
                if (iter > 0) {
                    vMoment = vMoment * keep;
                    vMean = vMean * keep;
                }
                vMoment = vMoment + __fdiv_rn(val * val, kf);
                vMean = vMean + __fdiv_rn(val, kf);
            }
            if (lay.ref) {
                // FrameBuffer error metrics after iteration iter + 1 (FrameBuffer.cs:276-277, 378-383)
                float3 d = cur - ref;
                double e1 = (double)d.x * d.x + (double)d.y * d.y + (double)d.z * d.z;
                double e2 = (double)d.x * d.x / ((double)ref.x * ref.x + 0.01) + (double)d.y * d.y / ((double)ref.y * ref.y + 0.01) +
                            (double)d.z * d.z / ((double)ref.z * ref.z + 0.01);
                if (lay.errPix) lay.errPix[(size_t)((int)iter - lay.errFirst) * cfg.W * cfg.H + pix] = (float)(e2 / 3.0);
                cg::coalesced_group act = cg::coalesced_threads();
                cg::coalesced_group grp = cg::labeled_partition(act, (int)iter);
                e1 = cg::reduce(grp, e1, cg::plus<double>());
                e2 = cg::reduce(grp, e2, cg::plus<double>());
                if (grp.thread_rank() == 0) {
                    atomicAdd(lay.errSum + 2 * (size_t)iter, e1);
                    atomicAdd(lay.errSum + 2 * (size_t)iter + 1, e2);
                }
            }
        }
        f[0] = cur.x; f[1] = cur.y; f[2] = cur.z;
        for (int j = 0; j < nOut; ++j) {
            lay.outW[pix * nOut + j] = hw[j];
            lay.outIt[pix * nOut + j] = hit[j];
        }
        if (lay.varMean) {
            lay.varMean[pix] = vMean;
            lay.varMoment[pix] = vMoment;
        }
        if (lay.aovAlbedo) {
            float* A = lay.aovAlbedo + 3 * pix;
            float* N = lay.aovNormal + 3 * pix;
            A[0] = alb.x; A[1] = alb.y; A[2] = alb.z;
            N[0] = nrm.x; N[1] = nrm.y; N[2] = nrm.z;
        }
    }
    // the last block to finish advances the wave counter (one CUDA graph serves every wave)
    if (advance) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            unsigned done = atomicAdd((unsigned*)(curWave + 1), 1u);
            if (done == gridDim.x - 1) {
                curWave[1] = 0;
                __threadfence();
                curWave[0] = curWave[0] + 1;
            }
        }
    }
}

// VarianceLayer.OnEndIteration (Images/VarianceLayer.cs:57-84): both images blurred by a 3x3 box
// (the mean of the window's pixels inside the image), variance = (moment - mean^2) / (mean^2 +
// 0.001), and the image average (summed in double).
__global__ void k_variance_finish(const float* mean, const float* moment, int W, int H, float* out, double* sum) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < W * H) {
        int x = i % W, y = i / W;
        float sm = 0.0f, so = 0.0f;
        int n = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = x + dx, yy = y + dy;
                if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
                sm += mean[yy * W + xx];
                so += moment[yy * W + xx];
                ++n;
            }
        float bm = sm / (float)n, bo = so / (float)n;
        float var = (bo - bm * bm) / (bm * bm + 0.001f);
        out[i] = var;
        v = var;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, v);
}

// FrameBuffer.ComputeErrorMetric's RelMSE_OutlierRejection (Images/FrameBuffer.cs:378-383, computed
// by SimpleImageIO's Metrics): the mean of the pixels' relative squared errors after the k largest
// are dropped.  One block per iteration.  The errors are non-negative, so their bit patterns order
// like their values (NaN above +inf); a most-significant-digit-first radix select over 8-bit digits
// finds the bits T of the k-th largest error and how many copies of T are among the k largest.  The
// kept errors (all below T, and the remaining copies of T) are then summed in double.
__global__ void __launch_bounds__(1024) k_error_trim(const float* err, int P, int k, double* out) {
    const uint32_t* e = reinterpret_cast<const uint32_t*>(err) + (size_t)blockIdx.x * P;
    __shared__ unsigned hist[256];
    __shared__ uint32_t sPrefix;
    __shared__ int sNeed;
    __shared__ double sSum[32];
    __shared__ unsigned sEq[32];
    const int tid = threadIdx.x, nt = blockDim.x;
    uint32_t prefix = 0xFFFFFFFFu, mask = 0;
    int need = 0;
    if (k > 0) {
        prefix = 0;
        need = k;
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int i = tid; i < 256; i += nt) hist[i] = 0;
            __syncthreads();
            for (int i = tid; i < P; i += nt) {
                uint32_t b = e[i];
                if ((b & mask) == prefix) atomicAdd(&hist[(b >> shift) & 255u], 1u);
            }
            __syncthreads();
            if (tid == 0) {
                // the digit d with fewer than `need` candidates above it and at least `need` from it up
                unsigned acc = 0;
                int d = 255;
                for (; d > 0; --d) {
                    if (acc + hist[d] >= (unsigned)need) break;
                    acc += hist[d];
                }
                sPrefix = prefix | ((uint32_t)d << shift);
                sNeed = need - (int)acc;
            }
            __syncthreads();
            prefix = sPrefix;
            need = sNeed;
            mask |= 255u << shift;
        }
    }
    double sum = 0.0;
    unsigned eq = 0;
    for (int i = tid; i < P; i += nt) {
        uint32_t b = e[i];
        if (b < prefix) sum += (double)__uint_as_float(b);
        else if (b == prefix) ++eq;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        eq += __shfl_xor_sync(0xffffffffu, eq, o);
    }
    if ((tid & 31) == 0) {
        sSum[tid >> 5] = sum;
        sEq[tid >> 5] = eq;
    }
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        unsigned q = 0;
        for (int w = 0; w < (nt + 31) / 32; ++w) {
            s += sSum[w];
            q += sEq[w];
        }
        if (q > (unsigned)need) s += (double)(q - (unsigned)need) * (double)__uint_as_float(prefix);
        out[blockIdx.x] = s / (double)(P - k);
    }
}

void launch_error_trim(const float* err, int P, int k, int iterations, double* out, cudaStream_t s) {
    if (iterations > 0 && P > k) k_error_trim<<<iterations, 1024, 0, s>>>(err, P, k, out);
}

void launch_variance_finish(const float* mean, const float* moment, int W, int H, float* out, double* sum, cudaStream_t s) {
    int n = W * H;
    k_variance_finish<<<(n + 255) / 256, 256, 0, s>>>(mean, moment, W, H, out, sum);
}

void launch_film_fold(const DevJob* jobs, const WaveChunk* chunks, const WaveDesc* waves, int* curWave, const float* samples, DevStats* st,
                      int maxFold, int advance, cudaStream_t s) {
    int grid = std::max(1, (maxFold + 255) / 256);
    k_film_fold<<<grid, 256, 0, s>>>(jobs, chunks, waves, curWave, samples, st, advance);
}

// Shade order of one bounce's queue: the paths that hit a surface first, then the misses and the
// finished paths, whose lanes only add the background or resolve pending next-event samples.  In
// queue order the expensive surface shading runs in every warp with the cheap lanes idle beside
// it; ordered, it runs in fewer, fuller warps.  Every path's result is the same in any order.
// counts[0], counts[1]: this bounce's append counters (zeroed with the wave's counters).
__global__ void __launch_bounds__(256) k_partition(const uint32_t* __restrict__ depth, const float4* __restrict__ hits, const int* nIn, int* order,
                                                    int* counts) {
    const int n = *nIn;
    if ((int)(blockIdx.x * blockDim.x) >= n) return;  // whole blocks: every warp below is complete
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const bool surf = valid && !(depth[i] & kDoneFlag) && __float_as_int(hits[i].w) >= 0;
    const unsigned ms = __ballot_sync(0xffffffffu, surf), mo = __ballot_sync(0xffffffffu, valid && !surf);
    const int lane = threadIdx.x & 31;
    int bs = 0, bo = 0;
    if (lane == 0) {
        if (ms) bs = atomicAdd(&counts[0], __popc(ms));
        if (mo) bo = atomicAdd(&counts[1], __popc(mo));
    }
    bs = __shfl_sync(0xffffffffu, bs, 0);
    bo = __shfl_sync(0xffffffffu, bo, 0);
    const unsigned below = (1u << lane) - 1u;
    if (surf) order[bs + __popc(ms & below)] = i;                   // from the front
    else if (valid) order[n - 1 - (bo + __popc(mo & below))] = i;   // from the back
}

void launch_partition(const uint32_t* depth, const float4* hits, const int* nIn, int* order, int* counts, int maxItems, cudaStream_t s) {
    const int grid = (maxItems + 255) / 256;
    if (grid == 0) return;
    k_partition<<<grid, 256, 0, s>>>(depth, hits, nIn, order, counts);
}

bool shadeBlocksValid(int b) { return b == SST_SHADE_GEN_MIN_BLOCKS || b == 10 || b == 12 || b == SST_SHADE_GEN_DENSE_BLOCKS; }

void launch_shade(int ns, bool adj, bool generic, int shadeBlocks, const DevJob* jobs, const PathBuf& A, const PathBuf& B, const float4* hits,
                  float4* nee, float4* neeG, int cap, float4* shRo, float4* shRd, int* shTgt, uint32_t* shJob, const int* nIn, int* nOut, int* nSh,
                  float* samples, DevStats* stats, int maxItems, cudaStream_t s) {
    int grid = (maxItems + 127) / 128;
    if (grid == 0) return;
    if (generic && !adj && ns == 1 && A.rec) {
        launch_shade_split(shadeBlocks, grid, jobs, A, B, hits, nee, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, samples, stats, s);
        return;
    }
    if (!generic && !adj && ns == 1) {
        k_shade<1, false, false><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, neeG, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, samples, stats, PyrArgs{});
        return;
    }
    if (generic && !adj && ns == 1 && shadeBlocks != SST_SHADE_GEN_MIN_BLOCKS) {
        launch_shade_generic_occ(shadeBlocks, grid, jobs, A, B, hits, nee, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, samples, stats, s);
        return;
    }
#define SST_SHADE_CASE(N)                                                                                                                    \
    case N:                                                                                                                                  \
        if (adj) k_shade<N, true, true><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, neeG, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, samples, stats, PyrArgs{}); \
        else k_shade<N, false, true><<<grid, 128, 0, s>>>(jobs, A, B, hits, nee, neeG, cap, shRo, shRd, shTgt, shJob, nIn, nOut, nSh, samples, stats, PyrArgs{}); \
        break;
    switch (ns) {
        SST_SHADE_CASE(1)
        SST_SHADE_CASE(2)
        SST_SHADE_CASE(3)
        default:
        SST_SHADE_CASE(4)
    }
#undef SST_SHADE_CASE
}

// Advances a buffer set's wave index by `by` (the last node of its wave graph, two waves in flight).
__global__ void k_wave_advance(int* wave, int by) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *wave += by;
}
void launch_wave_advance(int* wave, int by, cudaStream_t s) { k_wave_advance<<<1, 32, 0, s>>>(wave, by); }

void launch_camera(const DevJob* jobs, const WaveChunk* chunks, const WaveDesc* waves, const int* curWave, const PathBuf& A, int* qCount,
                   int maxItems, cudaStream_t s) {
    k_camera<<<std::max(1, (maxItems + 255) / 256), 256, 0, s>>>(jobs, chunks, waves, curWave, A, qCount);
}

// =============================================================================================
// Function-level kernels for the parity tests
// =============================================================================================
SST_D Ctx ctxFromPoint(const float* p, float3 outW) {
    Ctx c;
    c.faceN = mk(p[3], p[4], p[5]);
    c.f.n = mk(p[6], p[7], p[8]);
    basis(c.f.n, c.f.t, c.f.b);
    c.outW = outW;
    c.out = c.f.toLocal(outW);
    c.uv = make_float2(p[9], p[10]);
    return c;
}

// TinyEmbree Hit wrapped as SurfacePoint (Geometry/SurfacePoint.cs:7-77) for sst_trace: the compact
// traversal record (t, u, v, leaf triangle) expanded with the triangle's mesh, face, position, face
// normal and error offset (Geometry/Mesh.cs:50-60), one thread per ray.
__global__ void __launch_bounds__(256) k_hit_expand(DevScene sc, const float4* __restrict__ hits, int n, SstHitDev* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 h = hits[i];
    const int ti = __float_as_int(h.w);
    SstHitDev r;
    if (ti < 0) {
        r.d = 0.f; r.u = 0.f; r.v = 0.f;
        r.prim = -1; r.mesh = -1; r.eps = 0.f;
        r.p[0] = r.p[1] = r.p[2] = 0.f;
        r.n[0] = r.n[1] = r.n[2] = 0.f;
    } else {
        const float3 v1 = f3(__ldg(&sc.triv[3 * (size_t)ti])), v2 = f3(__ldg(&sc.triv[3 * (size_t)ti + 1])), v3 = f3(__ldg(&sc.triv[3 * (size_t)ti + 2]));
        const float4 fn = __ldg(&sc.triN[ti]);
        const int4 aux = __ldg(&sc.triAux[ti]);
        const float3 p = baryPos(v1, v2, v3, h.y, h.z);
        r.d = h.x; r.u = h.y; r.v = h.z;
        r.prim = aux.z; r.mesh = aux.y;
        r.eps = errorOffset(v1, v2, v3, h.y, h.z);
        r.p[0] = p.x; r.p[1] = p.y; r.p[2] = p.z;
        r.n[0] = fn.x; r.n[1] = fn.y; r.n[2] = fn.z;
    }
    out[i] = r;
}
void launch_hit_expand(const DevScene& sc, const float4* hits, int n, SstHitDev* out, cudaStream_t s) {
    if (n > 0) k_hit_expand<<<(n + 255) / 256, 256, 0, s>>>(sc, hits, n, out);
}

__global__ void k_debug_material_eval(DevScene sc, int mat, int n, const float* pts, const float* outs, const float* ins, float* vals, float* pdfs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pts + 11 * (size_t)i;
    Ctx c = ctxFromPoint(p, mk(outs[3 * i], outs[3 * i + 1], outs[3 * i + 2]));
    const DevMaterial& m = sc.mats[mat];
    Lp lp = {};
    float3 db = mk(0, 0, 0);
    if (m.type == kGeneric) lp = localParams(sc, m, c.uv);
    else db = lookupRgb(sc, m.baseTex, m.base, c.uv);
    float pdf;
    float3 v = evalWithCos(sc, m, lp, db, c, mk(ins[3 * i], ins[3 * i + 1], ins[3 * i + 2]), pdf);
    vals[3 * i] = v.x; vals[3 * i + 1] = v.y; vals[3 * i + 2] = v.z;
    pdfs[2 * i] = pdf;
    pdfs[2 * i + 1] = 0.0f;
}

__global__ void k_debug_material_sample(DevScene sc, int mat, int n, const float* pts, const float* outs, const float* us, float* dirs, float* pdfs,
                                        float* ws) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pts + 11 * (size_t)i;
    Ctx c = ctxFromPoint(p, mk(outs[3 * i], outs[3 * i + 1], outs[3 * i + 2]));
    const DevMaterial& m = sc.mats[mat];
    Lp lp = {};
    float3 db = mk(0, 0, 0);
    if (m.type == kGeneric) lp = localParams(sc, m, c.uv);
    else db = lookupRgb(sc, m.baseTex, m.base, c.uv);
    float3 d = mk(0, 0, 0), w = mk(0, 0, 0);
    float pdf = 0.0f;
    bool ok = sampleMaterial(sc, m, lp, db, c, us[3 * i], us[3 * i + 1], us[3 * i + 2], d, pdf, w);
    if (!ok) { d = mk(0, 0, 0); pdf = 0.0f; w = mk(0, 0, 0); }
    dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    pdfs[2 * i] = pdf;
    pdfs[2 * i + 1] = 0.0f;
    ws[3 * i] = w.x; ws[3 * i + 1] = w.y; ws[3 * i + 2] = w.z;
}

__global__ void k_debug_env(DevScene sc, int n, const float* us, float* dirs, float* pdfs, float* ws, const float* qd, float* rad, float* qpdf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 d, w;
    float pdf;
    envSample(sc.env, us[2 * i], us[2 * i + 1], d, pdf, w);
    dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    pdfs[i] = pdf;
    ws[3 * i] = w.x; ws[3 * i + 1] = w.y; ws[3 * i + 2] = w.z;
    float3 q = mk(qd[3 * i], qd[3 * i + 1], qd[3 * i + 2]);
    float3 r = envRadiance(sc.env, q);
    rad[3 * i] = r.x; rad[3 * i + 1] = r.y; rad[3 * i + 2] = r.z;
    qpdf[i] = envPdf(sc.env, q);
}

__global__ void k_debug_rng(uint32_t base, uint32_t sample, int n, const uint32_t* pixels, int draws, uint32_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng r{hashSeed(base, pixels[i], sample)};
    for (int k = 0; k < draws; ++k) out[(size_t)i * draws + k] = r.next();
}

__global__ void k_debug_camera(DevScene sc, int n, const float* film, float* org, float* dir) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 o, d;
    cameraRay(sc.cam, film[2 * i], film[2 * i + 1], o, d);
    org[3 * i] = o.x; org[3 * i + 1] = o.y; org[3 * i + 2] = o.z;
    dir[3 * i] = d.x; dir[3 * i + 1] = d.y; dir[3 * i + 2] = d.z;
}

void launch_debug_material_eval(const DevScene& sc, int mat, int n, const float* pts, const float* outs, const float* ins, float* vals, float* pdfs,
                                cudaStream_t s) {
    k_debug_material_eval<<<(n + 127) / 128, 128, 0, s>>>(sc, mat, n, pts, outs, ins, vals, pdfs);
}
void launch_debug_material_sample(const DevScene& sc, int mat, int n, const float* pts, const float* outs, const float* us, float* dirs, float* pdfs,
                                  float* ws, cudaStream_t s) {
    k_debug_material_sample<<<(n + 127) / 128, 128, 0, s>>>(sc, mat, n, pts, outs, us, dirs, pdfs, ws);
}
void launch_debug_env(const DevScene& sc, int n, const float* us, float* dirs, float* pdfs, float* ws, const float* qd, float* rad, float* qpdf,
                      cudaStream_t s) {
    k_debug_env<<<(n + 127) / 128, 128, 0, s>>>(sc, n, us, dirs, pdfs, ws, qd, rad, qpdf);
}
void launch_debug_rng(uint32_t base, uint32_t sample, int n, const uint32_t* pixels, int draws, uint32_t* out, cudaStream_t s) {
    k_debug_rng<<<(n + 127) / 128, 128, 0, s>>>(base, sample, n, pixels, draws, out);
}
void launch_debug_camera(const DevScene& sc, int n, const float* film, float* org, float* dir, cudaStream_t s) {
    k_debug_camera<<<(n + 127) / 128, 128, 0, s>>>(sc, n, film, org, dir);
}

}  // namespace sst

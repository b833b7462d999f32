/*
 * sst.h -- C ABI of libsst, the GB300 (sm_103a) wavefront path tracer that drops in for
 * SeeSharp's unidirectional PathTracer.
 *
 * Every entry point returns an int status: SST_OK (0) or a negative error class.  A message for
 * the last failure on the calling thread is available from sst_last_error().  No C++ exception
 * crosses this boundary.  Handles are opaque.  Caller-owned input arrays are copied; the scene
 * and context own their device memory.  Buffers passed with SST_MEM_DEVICE are CUDA device
 * pointers on the context's device; SST_MEM_HOST buffers are ordinary host memory.
 *
 * One host thread at a time per context.  Calls are synchronous: they return after the GPU work
 * they issued has finished.  Device arrays (SST_MEM_DEVICE) are read and written on the context's
 * own streams, which are not ordered with the caller's streams: the caller finishes its writes to
 * an input before the call (for example by synchronizing the stream that wrote it), and the outputs
 * are complete when the call returns.
 *
 * Each declaration names the SeeSharp interface it replaces (paths relative to the SeeSharp
 * project root).
 */
#ifndef SST_H
#define SST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SST_OK 0
#define SST_ERR_INVALID_ARGUMENT (-1) /* ArgumentException in SeeSharp */
#define SST_ERR_INVALID_SCENE (-2)    /* InvalidOperationException from Scene.Prepare */
#define SST_ERR_CUDA (-3)
#define SST_ERR_OUT_OF_MEMORY (-4)
#define SST_ERR_NOT_COMMITTED (-5)    /* scene used before sst_scene_commit */
#define SST_ERR_DEVICE_LIMIT (-6)     /* a device-side iteration or stack limit was reached */
#define SST_ERR_UNSUPPORTED (-7)

#define SST_MEM_HOST 0
#define SST_MEM_DEVICE 1

#define SST_BORDER_REPEAT 0 /* ImageTexture.BorderHandling.Repeat (Images/ImageTexture.cs:12-21) */
#define SST_BORDER_CLAMP 1  /* ImageTexture.BorderHandling.Clamp */

typedef struct sst_ctx sst_ctx;
typedef struct sst_scene sst_scene;

/* GenericMaterial.Parameters (Shading/Materials/GenericMaterial.cs:25-61).  A texture index < 0
 * selects the constant value. */
typedef struct SstGenericMaterial {
    float baseColor[3];
    int32_t baseColorTexture;
    float roughness;
    int32_t roughnessTexture;
    float metallic;
    float specularTintStrength;
    float anisotropic;
    float specularTransmittance;
    float indexOfRefraction;
} SstGenericMaterial;

/* TinyEmbree Ray: origin, MinDistance, direction, and the far end of the valid interval. */
typedef struct SstRay {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} SstRay;

/* TinyEmbree Hit (as wrapped by Geometry/SurfacePoint.cs:7-77).  meshId < 0 means no hit. */
typedef struct SstHit {
    float distance;
    float u, v; /* barycentrics: u weights the second, v the third vertex */
    int32_t primId;
    int32_t meshId;
    float errorOffset;
    float position[3];
    float normal[3];
} SstHit;

/* PathTracerBase public settings (Integrators/PathTracer.cs:16-49, Integrator.cs:10-16) plus the
 * frame buffer size and flags (Images/FrameBuffer.cs:101-133). */
typedef struct SstPathTracerParams {
    int32_t width, height;
    int32_t totalSpp;
    int32_t maxDepth;
    int32_t minDepth;
    uint32_t baseSeed;
    int32_t numShadowRays;
    int32_t enableBsdfDI;
    int32_t ignoreNanAndInf;    /* FrameBuffer.Flags.IgnoreNanAndInf */
    int32_t firstIteration;     /* iterations already averaged into `film` (resume); 0 = fresh */
    int64_t maximumRenderTimeMs; /* <= 0: no limit (PathTracer.cs:27, :221-227) */
} SstPathTracerParams;

/* FrameBuffer.MetaData entries written by PathTracer.Render (PathTracer.cs:254-257). */
typedef struct SstRenderStats {
    double renderTimeMs;      /* GPU time of the iterations, frame-buffer work excluded */
    double frameBufferTimeMs; /* film initialisation / copies */
    int32_t numIterations;
    int32_t numKernelLaunches; /* kernels this library launched for the render (graph replays counted per node) */
    uint64_t numRays;       /* RayTracerStats.NumRays */
    uint64_t numShadowRays; /* RayTracerStats.NumShadowRays */
    uint64_t numNanOrInf;   /* FrameBuffer.NaNWarnings count */
    int32_t nanPixel[4];    /* FrameBuffer.NaNWarnings: the first entries in (iteration, pixel index) order, -1 if unused */
    int32_t nanIteration[4]; /* their 1-based iteration (FrameBuffer.CurIteration) */
    /* ShadingStats (Shading/ShadingStats.cs:5-9, MetaData["ShadingStats"], PathTracer.cs:256): the material
     * Evaluate / Sample / Pdf calls the reference PathTracer makes for the rendered paths.  Counted only while
     * sst_set_shading_stats is on for the context (zero otherwise). */
    uint64_t numMaterialEval;
    uint64_t numMaterialSample;
    uint64_t numMaterialPdf;
} SstRenderStats;

/* ---- library / context --------------------------------------------------------------------- */
int sst_version(int32_t* major, int32_t* minor);
/* Copies the calling thread's last error message (NUL-terminated, truncated to size). */
int sst_last_error(char* buffer, size_t size);

/* Creates a context on a CUDA device: one stream, the device kernels, scratch pools. */
int sst_create(int32_t device, sst_ctx** out);
int sst_destroy(sst_ctx* ctx);

/* ---- scene (Scene.cs:26-58 members, Scene.Prepare :103-164) ---------------------------------- */
int sst_scene_create(sst_ctx* ctx, sst_scene** out);
int sst_scene_destroy(sst_scene* scene);

/* RgbImage / MonochromeImage used as TextureRgb / TextureMono (Images/TextureRgb.cs:16-21,
 * TextureMono.cs:47-58).  data: row-major, top row first, `channels` floats per texel (1 or 3). */
int sst_scene_add_texture(sst_scene* scene, const float* data, int32_t width, int32_t height, int32_t channels,
                          int32_t border, int32_t* outTexture);

/* new DiffuseMaterial(Parameters) (Shading/Materials/DiffuseMaterial.cs:10-28). */
int sst_scene_add_material_diffuse(sst_scene* scene, const float baseColor[3], int32_t baseColorTexture,
                                   int32_t transmitter, int32_t* outMaterial);
/* new GenericMaterial(Parameters) (Shading/Materials/GenericMaterial.cs:20). */
int sst_scene_add_material_generic(sst_scene* scene, const SstGenericMaterial* params, int32_t* outMaterial);
/* Replaces the parameters of an existing generic material (before or after commit). */
int sst_scene_update_material_generic(sst_scene* scene, int32_t material, const SstGenericMaterial* params);

/* new Mesh(vertices, indices, shadingNormals, textureCoordinates) + Mesh.Material
 * (Geometry/Mesh.cs:28-41).  vertices: numVertices*3 floats; indices: numTriangles*3;
 * shadingNormals (numVertices*3) and textureCoordinates (numVertices*2) may be NULL. */
int sst_scene_add_mesh(sst_scene* scene, const float* vertices, int32_t numVertices, const int32_t* indices,
                       int32_t numTriangles, const float* shadingNormals, const float* textureCoordinates,
                       int32_t material, int32_t* outMesh);

/* Scene.Emitters.AddRange(DiffuseEmitter.MakeFromMesh(mesh, radiance)) when glossyExponent < 0,
 * GlossyEmitter.MakeFromMesh(mesh, radiance, exponent) otherwise (Shading/Emitters/
 * DiffuseEmitter.cs:21-31, GlossyEmitter.cs:24-34).  faces == NULL: every face of the mesh,
 * zero-area faces skipped; otherwise exactly the listed faces, and a zero-area face is an error
 * (Geometry/Triangle.cs:32-33).  Emitters are appended in order; outFirst receives the index of
 * the first one, outCount how many were added. */
int sst_scene_add_emitters(sst_scene* scene, int32_t mesh, const int32_t* faces, int32_t numFaces,
                           const float radiance[3], float glossyExponent, int32_t* outFirst, int32_t* outCount);
/* Overwrites the radiance of emitters [first, first + count) (rgb: count*3 floats). */
int sst_scene_set_emitter_radiance(sst_scene* scene, int32_t first, int32_t count, const float* rgb);

/* Scene.Background = new EnvironmentMap(image) (Shading/Background/EnvironmentMap.cs:14-17).
 * rgb: width*height*3 floats, top row first. */
int sst_scene_set_envmap(sst_scene* scene, const float* rgb, int32_t width, int32_t height);

/* Scene.Camera = new PerspectiveCamera(worldToCamera, verticalFieldOfView)
 * (Cameras/PerspectiveCamera.cs:32-37).  worldToCamera: System.Numerics.Matrix4x4 in row-major
 * order M11..M44 (row-vector convention). */
int sst_scene_set_camera(sst_scene* scene, const float worldToCamera[16], float verticalFovDegrees);

/* Scene.Prepare() with FrameBuffer (width, height): validates, uploads, builds the BVH and the
 * environment-map sampling tables, and updates the camera resolution. */
int sst_scene_commit(sst_scene* scene, int32_t width, int32_t height);

/* Number of emitters / triangles / BVH nodes in a committed scene (any pointer may be NULL). */
int sst_scene_info(sst_scene* scene, int32_t* numEmitters, int32_t* numTriangles, int32_t* numBvhNodes);

/* ---- ray queries (TinyEmbree Raytracer.Trace / IsOccluded, PathTracer.cs:319,467) ----------- */
int sst_trace(sst_scene* scene, const SstRay* rays, int32_t n, SstHit* hits, int32_t memory);
int sst_occluded(sst_scene* scene, const SstRay* rays, int32_t n, int32_t* occluded, int32_t memory);

/* ---- launch configuration and autotuner (no counterpart in the reference) ---------------------
 * The wavefront's queue capacity, the traversal kernels' launch shape and the shade kernel's build.
 * None of them changes a result: films and query results are bitwise the same under every valid
 * setting, except shadeSplit, whose two kernels compile the shading arithmetic separately from the
 * fused kernel (and, with shadeSplit = 1, shadeBlocks 14 against the other values, which select a
 * separately compiled build of the split kernels), so the compiler may fuse a multiply-add
 * differently and move a path's estimate by an ulp (or, rarely, flip a decision that the ulp
 * decides). */
typedef struct SstTuning {
    int32_t waveCapacity;     /* paths in flight per wave; 0 = the default (2^21) */
    int32_t traceBlock;       /* threads per traversal block: 64, 128 (the default) or 256 */
    int32_t traceStackShared; /* traversal stack entries per thread kept in shared memory: 16, 24 (the default) or 32 */
    int32_t traceBlocksPerSM; /* resident traversal blocks per SM; 0 = as many as fit (three quarters of that while
                                 several waves are in flight) */
    int32_t traceBvhWidth;    /* BVH traversed: 2 (binary), 4 (4-wide, same leaves; the default) or 8 (8-wide, same leaves,
                                 children in octant slots; built for a scene by the first render or query that
                                 traverses it with this setting, and until then sst_occluded_noalloc, which
                                 allocates nothing, traverses the scene 4-wide) */
    int32_t traceRefillIdle;  /* 4- and 8-wide traversal: a warp's finished rays are replaced once this many of its
                                 32 lanes are idle (1..32; 32 = only when all are; the default is 20) */
    int32_t shadeBlocks;      /* resident 128-thread blocks per SM the forward shade kernel with GenericMaterials
                                 is built for: 8 (64 registers; the default), 10, 12 or 14 (48, 40 or 32
                                 registers: more warps, more spilling; one shadow ray per technique only) */
    int32_t shadeOrder;       /* 1 (the default): each bounce's paths are shaded surface hits first, misses and
                                 finished paths after them; 0: in queue order */
    int32_t shadeSplit;       /* 1 (the default): forward renders with GenericMaterials and one shadow ray per
                                 technique shade each bounce with two kernels (hit, emitter MIS, Russian roulette
                                 and next-event estimation; then BSDF sampling and the queue compaction), built for
                                 8 blocks, or for 14 when shadeBlocks is 14; 0: one fused kernel */
} SstTuning;
int sst_get_tuning(sst_ctx* ctx, SstTuning* out);
/* Invalid values return SST_ERR_INVALID_ARGUMENT and leave the setting unchanged. */
int sst_set_tuning(sst_ctx* ctx, const SstTuning* tuning);
/* Chooses the setting for this scene and these parameters by timing trial renders into a scratch
 * film (the caller's films are not touched), keeping the fastest of two runs per candidate:
 * first the traversal variant (BVH width x block size x shared stack entries), then the refill
 * threshold of the wide traversals, then the shade kernel's build (8, 10, 12 or 14 blocks), then the shade order, then
 * the resident blocks per SM, each with trials of at least trialIterations iterations and at least 2^21 paths; then the
 * wave capacity, with trials of about four waves of 2^22 paths (within the parameters' spp).  The
 * choice is applied to the scene's context and returned in `chosen`; bestTrialMs (may be NULL)
 * receives the time of a trialIterations-iteration render with it. */
int sst_autotune(sst_scene* scene, const SstPathTracerParams* params, int32_t trialIterations, SstTuning* chosen, double* bestTrialMs);

/* ---- allocation-free occlusion query: no counterpart in the reference --------------------------
 * The same any-hit queries as sst_occluded, with the same arguments and the same results, but the
 * call allocates no memory: no cudaMalloc or cudaFree, and no allocating CUDA library routine.
 * sst_occluded allocates its temporary device buffers on every call.  Some callers cannot do that:
 *  - a caller whose device memory is fully budgeted, e.g. one that shares the GPU with another
 *    process holding the rest of it, where a new allocation can fail in the middle of a frame;
 *  - a caller on a latency-bound loop (shadow or picking queries per frame): cudaFree waits for
 *    the whole device, and cudaMalloc may, which stalls every stream on the GPU, not just this one.
 * The scratch it uses (split ray arrays, queue counters, job record, ray statistics, result flags)
 * is one array of 2,361,344 bytes that is part of this library's device code.  Every GPU that
 * loads the library holds it until the process exits.
 * Limits and rules:
 *  - n <= SST_NOALLOC_MAX_RAYS; a larger n returns SST_ERR_INVALID_ARGUMENT and does nothing.
 *  - The first call on a device looks up the array's device address (cudaGetSymbolAddress).
 *    Make that first call before any CUDA stream capture begins.
 *  - All calls on a device share the array, so two calls whose GPU work overlapped would race.
 *    The function holds a process-wide lock for the whole call and returns only after its GPU
 *    work has finished, so its own calls in one process never overlap.
 *  - rays / occluded are host arrays (SST_MEM_HOST) or device arrays (SST_MEM_DEVICE).  Device arrays
 *    are accessed on the context's stream, with no ordering against the caller's streams: finish
 *    the writes to `rays` before the call; `occluded` is complete when the call returns. */
#define SST_NOALLOC_MAX_RAYS 65536
int sst_occluded_noalloc(sst_scene* scene, const SstRay* rays, int32_t n, int32_t* occluded, int32_t memory);

/* ---- rendering (PathTracerBase.Render, PathTracer.cs:199-267) -------------------------------- */
/* Renders iterations [firstIteration, totalSpp) into film (width*height*3 floats, row-major,
 * top row first) with the frame buffer's running mean.  When firstIteration > 0 the film must
 * hold the mean of the first `firstIteration` iterations.  stats may be NULL. */
int sst_render(sst_scene* scene, const SstPathTracerParams* params, float* film, int32_t memory,
               SstRenderStats* stats);

/* A camera view for one job of a batch (PerspectiveCamera(worldToCamera, fov), as
 * sst_scene_set_camera); the image size is the job's width and height. */
typedef struct SstCamera {
    float worldToCamera[16];
    float verticalFovDegrees;
    int32_t reserved;
} SstCamera;

/* ---- light paths: no counterpart in the reference's PathTracer -----------------------------------
 * LightPathCache.TraceAllPaths (Integrators/Bidir/LightPathCache.cs:126-260) for the bidirectional
 * integrators: numPaths random walks from the emitters and the background with the LightPathWalk
 * vertices (Integrators/Common/PathVertex.cs), path i seeded RNG(seed, i, iteration).  The next-
 * event pdf callback is not evaluated (pdfNextEventAncestor = 0). */
typedef struct SstPathVertex {
    float position[3];
    float normal[3];           /* face normal; 0 for the first vertex of a background path */
    float shadingNormal[3];
    float pdfFromAncestor;     /* surface-area pdf of this vertex from its ancestor */
    float pdfReverseAncestor;  /* surface-area pdf of the ancestor's ancestor from the ancestor */
    float pdfNextEventAncestor;
    float weight[3];           /* Monte Carlo weight of the subpath up to this vertex */
    float maximumRoughness;
    int32_t meshId;            /* -1 for the first vertex of a background path */
    int32_t primId;
    int32_t depth;             /* edges along the path */
    int32_t pathId;
    int32_t fromBackground;
    int32_t reserved;
} SstPathVertex;
/* vertices: numPaths * (maxDepth + 1) entries, path i at i * (maxDepth + 1); lengths: numPaths. */
int sst_trace_light_paths(sst_scene* scene, uint32_t seed, uint32_t iteration, int32_t numPaths, int32_t maxDepth, SstPathVertex* vertices,
                          int32_t* lengths, int32_t memory, SstRenderStats* stats);

/* ---- path replay (PathTracerBase.ReplayPixel, PathTracer.cs:60-68) ------------------------------
 * Renders the n paths (pixels[k], iterations[k]) exactly as sst_render renders them (a path is a
 * function of BaseSeed, its pixel index row*width+col and its 0-based iteration) and writes each
 * path's estimate, the value RenderPixel splats, to rgb[3k..3k+2].  Nothing is added to a film.
 * The path graph of the reference's ReplayPixel (a debugging aid) is not built.  memory applies to
 * pixels, iterations and rgb. */
int sst_render_paths(sst_scene* scene, const SstPathTracerParams* params, const int32_t* pixels, const int32_t* iterations, int32_t n,
                     float* rgb, int32_t memory, SstRenderStats* stats);

/* ---- frame-buffer layers ------------------------------------------------------------------------
 * Computed on the device while the film is folded:
 *  - the VarianceLayer (FrameBuffer.Flags.EstimatePixelVariance, Images/VarianceLayer.cs:10-84);
 *  - the per-iteration error metrics against FrameBuffer.ReferenceImage (FrameBuffer.cs:276-277,
 *    378-383): the mean over pixels and channels of (x - r)^2 and of (x - r)^2 / (r^2 + 0.01), and
 *    the outlier-rejecting RelMSE: each pixel's error is its mean over the channels of
 *    (x - r)^2 / (r^2 + 0.01), the largest floor(width*height / 1000) of them (0.1%) are dropped and
 *    the rest averaged.  It needs 4 bytes of device memory per pixel and iteration of the call;
 *  - the denoiser's feature layers (DenoiseBuffers.LogPrimaryHit, Integrators/Util/DenoiseBuffers.cs:20-23,
 *    logged at the primary hit as in PathTracer.cs:336-339): running means of the material's scatter
 *    strength and of the shading normal;
 *  - the OutlierReplayCache (Integrators/Util/OutlierReplayCache.cs:9-35, notified by
 *    FrameBuffer.Splat, FrameBuffer.cs:187-190): per pixel the numOutliers samples of largest channel
 *    average with their iteration, in the array order of .NET's 4-ary PriorityQueue min-heap;
 *  - the technique pyramids of PathTracer.RenderTechniquePyramid (PathTracer.cs:73-82, 204-266,
 *    Integrators/Bidir/TechPyramid.cs): every sample that RegisterSample would log (emitter and
 *    background hits of length d, visible next-event samples of length d), divided by TotalSpp, summed
 *    per technique image, raw and times its MIS weight.  48 * maxDepth bytes of device memory per
 *    pixel; not cumulative over calls.  A next-event sample whose MIS-weighted contribution is zero
 *    is not logged (the reference logs it with its raw contribution; this needs a zero MIS weight).
 * The running means and the heaps resume like the film: when firstIteration > 0 the state arrays
 * hold the layers after iteration firstIteration and are read, and they are always written back. */
typedef struct SstFilmLayers {
    float* variance;        /* out: width*height VarianceLayer image, or NULL */
    float* varianceAverage; /* out: 1 float, VarianceLayer.Average, or NULL */
    float* varianceState;   /* in/out: 2*width*height running means of the iteration's value and of its
                               square (required with variance or varianceAverage) */
    const float* reference; /* in: width*height*3 reference image, or NULL */
    double* errors;         /* out: 3 per iteration of this call (MSE, RelMSE, RelMSE_Outlier after it; zero for
                               iterations that a time limit skipped), or NULL */
    float* albedo;          /* in/out: width*height*3 "albedo" layer, or NULL */
    float* normal;          /* in/out: width*height*3 "normal" layer, or NULL */
    int32_t memory;         /* SST_MEM_HOST / SST_MEM_DEVICE for the arrays above */
    int32_t numOutliers;    /* OutlierReplayCache capacity per pixel, 0..8 (FrameBuffer.NumOutliersToTrack; 0: none) */
    float* outlierWeight;   /* in/out: width*height*numOutliers heap priorities (the sample's channel average) */
    int32_t* outlierIteration; /* in/out: width*height*numOutliers heap elements (0-based iteration, -1: empty) */
    float* techPyramid;     /* out: the technique pyramids of this call, or NULL: 2 * 2*maxDepth images of
                               width*height*3, the raw ones, then the MIS-weighted ones; image 2(d-1) is
                               "{d}-hit", image 2(d-1)+1 "{d}-next-event" (unused for d = 1) */
} SstFilmLayers;
/* sst_render that also fills the requested layers. */
int sst_render_layers(sst_scene* scene, const SstPathTracerParams* params, float* film, int32_t memory, const SstFilmLayers* layers,
                      SstRenderStats* stats);

/* One render job of a batch. */
typedef struct SstRenderJob {
    sst_scene* scene;
    SstPathTracerParams params;
    float* film;
    int32_t memory;
    int32_t reserved;
    const SstCamera* camera; /* NULL: the scene's camera; otherwise this view of the scene */
} SstRenderJob;
/* Renders many independent jobs (uneven resolutions, spp and depths) in one persistent
 * wavefront: all jobs' paths share the ray queues.  Films as in sst_render. */
int sst_render_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, SstRenderStats* stats);

/* ---- path-replay adjoint (differentiable rendering) ------------------------------------------
 * No counterpart in the reference's C# code beyond its replay semantics: a path is a pure
 * function of (BaseSeed, pixel, iteration) (PathTracerBase.ReplayPixel, PathTracer.cs:61-69), so
 * the backward pass re-traces every path from its seed instead of storing its vertices.
 * Gradients use detached sampling: pdfs, MIS weights and Russian roulette are constants; there
 * are no geometric or visibility derivatives.  The pair behaves like a torch.autograd.Function:
 * sst_forward(params) -> image, sst_backward(dLoss/dImage) -> dLoss/dparams. */
typedef struct SstGradients {
    float* textures;          /* every texture's texels, concatenated in the order they were added */
    float* materialBaseColor; /* 3 per material: constant base colour */
    float* materialRoughness; /* 1 per material: constant roughness (GenericMaterial) */
    float* emitterRadiance;   /* 3 per emitter */
    int32_t memory;           /* SST_MEM_HOST / SST_MEM_DEVICE for the arrays above */
    int32_t reserved;
} SstGradients;
/* Batched forms over many jobs (for example several camera views of one scene) in one shared
 * wavefront.  sst_forward_batch renders every job like sst_forward and keeps each job's path
 * radiance; sst_backward_batch takes one dLoss/dImage per job (the jobs must equal those of the
 * last sst_forward_batch on the context).  The gradients of a scene are summed over all of its
 * jobs and written to the SstGradients of the scene's first job in the list; the entries of its
 * other jobs are not used. */
int sst_forward_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, SstRenderStats* stats);
int sst_backward_batch(sst_ctx* ctx, const SstRenderJob* jobs, int32_t numJobs, const float* const* dLossDImage, int32_t memory,
                       SstGradients* grads, SstRenderStats* stats);
/* Overwrites the texels of a texture (same size and channels as when it was added). */
int sst_scene_update_texture(sst_scene* scene, int32_t texture, const float* data);
/* sst_render of iterations [0, totalSpp) that also keeps every path's radiance for the replay. */
int sst_forward(sst_scene* scene, const SstPathTracerParams* params, float* image, int32_t memory, SstRenderStats* stats);
/* Gradients of a scalar loss with respect to the scene parameters, given dLoss/dImage
 * (width*height*3) of the image that the last sst_forward with the same params produced.  The
 * gradient arrays are overwritten (any may be NULL). */
int sst_backward(sst_scene* scene, const SstPathTracerParams* params, const float* dLossDImage, int32_t memory,
                 SstGradients* gradients, SstRenderStats* stats);

/* ---- kernel timing ------------------------------------------------------------------------------
 * With profiling enabled, sst_render records CUDA events around every kernel launch on the
 * context's stream and accumulates, per kernel class (0 camera, 1 closest-hit traversal,
 * 2 shade, 3 shadow-ray traversal, 4 film fold), the GPU time in ms, the number of launches and
 * the number of items (rays or paths) processed.  Enabling it adds a device synchronisation per
 * wave; disabled by default. */
#define SST_KERNEL_CLASSES 5
int sst_set_profiling(sst_ctx* ctx, int32_t enable);
int sst_get_kernel_times(sst_ctx* ctx, double* ms, int64_t* launches, int64_t* items, int32_t numClasses);

/* ---- shading statistics (ShadingStatCounter, Shading/ShadingStats.cs:11-33) ---------------------
 * While enabled, renders on the context count the material calls that the reference PathTracer makes
 * for the same paths (SstRenderStats.numMaterial*): a BSDF sample per sampled direction (plus an
 * evaluation and a pdf for a DiffuseMaterial, whose Sample calls both), and an evaluation and a pdf
 * per next-event sample whose shadow ray finds the light visible (PathTracer.cs:428-430, 467-477).
 * The wavefront evaluates next-event BSDFs before their shadow rays are traced and traces only the
 * samples that contribute, so the counts need the visibility of the others as well: while enabled,
 * every next-event sample's shadow ray is traced.  Images are unchanged.  Disabled by default. */
int sst_set_shading_stats(sst_ctx* ctx, int32_t enable);

/* ---- function-level entry points used by the parity tests --------------------------------------
 * Each runs the device code of one reference function on a batch of inputs (host arrays). */
/* Material.EvaluateWithCosine + Material.Pdf (Material.cs:80-83).  points: n*11 floats
 * (position 3, face normal 3, shading normal 3, uv 2); out/in dirs: n*3; values n*3; pdfs n*2. */
int sst_debug_material_eval(sst_scene* scene, int32_t material, int32_t n, const float* points, const float* outDirs,
                            const float* inDirs, float* values, float* pdfs);
/* Material.Sample (GenericMaterial.cs:92-150, DiffuseMaterial.cs:127-164).  u: n*3 (component,
 * direction x, direction y); dirs n*3, pdfs n*2, weights n*3. */
int sst_debug_material_sample(sst_scene* scene, int32_t material, int32_t n, const float* points, const float* outDirs,
                              const float* u, float* dirs, float* pdfs, float* weights);
/* EnvironmentMap.SampleDirection / DirectionPdf / EmittedRadiance (EnvironmentMap.cs:19-85).
 * u: n*2 -> dirs n*3, pdfs n, weights n*3; queryDirs n*3 -> radiance n*3, queryPdfs n. */
int sst_debug_envmap(sst_scene* scene, int32_t n, const float* u, float* dirs, float* pdfs, float* weights,
                     const float* queryDirs, float* radiance, float* queryPdfs);
/* RNG(baseSeed, pixels[i], sampleIndex) followed by `draws` Next() calls (Sampling/RNG.cs). */
int sst_debug_rng(uint32_t baseSeed, uint32_t sampleIndex, int32_t n, const uint32_t* pixels, int32_t draws,
                  uint32_t* out);
/* PerspectiveCamera.GenerateRay for film positions (n*2) -> origins, directions (n*3 each). */
int sst_debug_camera(sst_scene* scene, int32_t n, const float* filmPos, float* origins, float* directions);

#ifdef __cplusplus
}
#endif
#endif /* SST_H */

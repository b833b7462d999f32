"""Benchmark: SeeSharp PathTracer throughput (Msamples/s) on the 1M-triangle sphere field.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 1]

A step is one full PathTracer render of the workload (all iterations).  The default workload is
the 1M-triangle configuration: 200 seeded displaced icospheres (5120 triangles each), 50 emissive
triangles, a 512x256 procedural HDR sky, 1024x1024 pixels, 64 spp, max depth 8; inputs are
synthetic and seeded.  `value` is device-timed (CUDA events on the renderer's stream) with the
scene resident in HBM; `e2e` is measured through the public API (Scene.Prepare + PathTracer.Render
with host buffers: geometry upload, BVH build, render, film read-back) per step.
`--impl reference` times the CPU restatement of the reference PathTracer (the oracle) on all
host cores over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    0: dict(name="cornell_box_36tri_256x256_16spp_depth5", builder="cornell", W=256, H=256, spp=16, depth=5),
    1: dict(name="sphere_field_1Mtri_1024x1024_64spp_depth8", builder="spheres", spheres=200, W=1024, H=1024, spp=64, depth=8),
    2: dict(name="batch_64jobs_10k-1Mtri_128-1024px_4-64spp_depth3-10", builder="batch", jobs=64, seed=2024),
    3: dict(name="cornell_adjoint_tex256_512x512_32spp_depth5", builder="adjoint", W=512, H=512, spp=32, depth=5, tex=256),
    4: dict(name="large_12.3Mtri_8views_1920x1080_256spp_depth10_adjoint_tex1024_rough2000", builder="large", W=1920, H=1080, spp=256, depth=10),
    5: dict(name="reference_scene_CornellBox.json_512x512_512spp_depth5", builder="scenefile", path="CornellBox/CornellBox.json", W=512, H=512,
            spp=512, depth=5, seed=571298512, recorded="CornellBox/References/MaxDepth5-Width512-Height512.json"),
}
CONFIGS[6] = dict(name="light_paths_sphere_field_1Mtri_262144paths_depth8", builder="lightpaths", spheres=200, W=1024, H=1024, paths=262144, depth=8)
CONFIGS[7] = dict(name="batch_256smalljobs_10k-200ktri_64-256px_1-16spp_depth3-10", builder="batch", jobs=256, seed=7, tris=(1e4, 2e5),
                  res=(64, 128, 256), spp=(1, 16), depth=(3, 10), scene_seed=5000)
SCENE_DIR = os.path.join(ROOT, "tests", "golden", "scenes")


def batch_jobs(cfg, seed_offset=0):
    """The batched configurations: jobs from the sphere-field generator with triangle counts
    log-uniform in cfg["tris"], square resolutions from cfg["res"], spp and max depth uniform over
    the integer ranges cfg["spp"] and cfg["depth"].  Configuration 2 (uneven jobs): 64 jobs, [10k,
    1M] triangles, 128..1024 pixels, 4..64 spp, depth 3..10.  Configuration 7 (serving-style small
    jobs, none of which fills the GPU alone): 256 jobs, [10k, 200k] triangles, 64..256 pixels,
    1..16 spp, depth 3..10."""
    from seesharp_gb300 import PathTracer, workloads
    rng = np.random.default_rng(cfg["seed"] + seed_offset)
    lo, hi = cfg.get("tris", (1e4, 1e6))
    res_choices = list(cfg.get("res", (128, 256, 512, 1024)))
    spp_lo, spp_hi = cfg.get("spp", (4, 64))
    d_lo, d_hi = cfg.get("depth", (3, 10))
    out = []
    for j in range(cfg["jobs"]):
        tris = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        res = int(rng.choice(res_choices))
        spp = int(rng.integers(spp_lo, spp_hi + 1))
        depth = int(rng.integers(d_lo, d_hi + 1))
        sc = workloads.sphere_field(max(2, int(round(tris / 5120))), res, res, seed=cfg.get("scene_seed", 1000) + j)
        out.append((sc, PathTracer(TotalSpp=spp, MaxDepth=depth)))
    return out


def run_batch(args, cfg):
    """Batched jobs in one shared wavefront vs the same jobs rendered one after another."""
    import torch
    from seesharp_gb300 import render_batch
    pairs = batch_jobs(cfg)
    for sc, _ in pairs:
        sc.Prepare()
    samples = sum(sc.FrameBuffer.Width * sc.FrameBuffer.Height * pt.TotalSpp for sc, pt in pairs)
    tris = [sum(m.NumFaces for m in sc.Meshes) for sc, _ in pairs]

    nlaunch = [0]

    def batched():
        for sc, _ in pairs:
            sc.FrameBuffer.Reset()
        st = render_batch(pairs)
        nlaunch[0] += st.numKernelLaunches
        return st.renderTimeMs

    def sequential():
        ms = 0.0
        for sc, pt in pairs:
            sc.FrameBuffer.Reset()
            pt.Render(sc)
            ms += pt.last_stats.renderTimeMs
        return ms

    for _ in range(args.warmup):
        batched()
        sequential()
    with ClockSampler(0) as clk:
        nlaunch[0] = 0
        w0 = time.perf_counter()
        tb = [batched() for _ in range(args.steps)]
        wall_b = (time.perf_counter() - w0) / args.steps
        batched_launches = nlaunch[0]
        w0 = time.perf_counter()
        ts = [sequential() for _ in range(args.steps)]
        wall_s = (time.perf_counter() - w0) / args.steps
    vb = samples / (np.mean(tb) / 1000) / 1e6
    vs = samples / (np.mean(ts) / 1000) / 1e6
    # e2e: wall clock through the public API with host films, averaged over `steps` batched calls
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batched()
    e2e_b = samples * args.steps / (time.perf_counter() - t0) / 1e6
    line = {"metric": "Msamples/s PathTracer (batched jobs)", "value": round(vb, 3), "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(float(np.mean(tb)), 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": cfg["name"], "jobs": len(pairs), "total_samples": int(samples), "triangles_min": min(tris), "triangles_max": max(tris),
                       "triangles_total": int(sum(tris))},
            "sequential": {"value": round(vs, 3), "ms_per_step": round(float(np.mean(ts)), 3)},
            "batched_over_sequential": round(vb / vs, 3),
            "wall_clock": {"batched_s": round(wall_b, 3), "sequential_s": round(wall_s, 3), "batched_over_sequential": round(wall_s / wall_b, 3),
                           "note": "host time per step through the public API, films read back to the host"},
            "gpu_launches": int(batched_launches),
            "e2e": {"value": round(e2e_b, 3), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(sum(sc.FrameBuffer.Image.data.nbytes for sc, _ in pairs))},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)



def run_adjoint(args, cfg):
    """Differentiation workload: forward (sst_forward) and path-replay backward (sst_backward) of
    an L2 image loss; the metric is backward time over forward time."""
    from seesharp_gb300 import PathTracer, workloads
    from seesharp_gb300.adjoint import DifferentiableRender, l2_loss
    W, H, spp = cfg["W"], cfg["H"], cfg["spp"]
    sc, tex, boxes, lights = workloads.cornell_box_differentiable(W, H, tex_res=cfg["tex"])
    sc.Prepare()
    dr = DifferentiableRender(sc, PathTracer(TotalSpp=spp, MaxDepth=cfg["depth"]), texture=tex, roughness_materials=boxes, emitters=[lights])
    rng = np.random.default_rng(11)
    tex0 = tex.Image.data.copy()
    dr.params.baseSeed = 0x5EED
    target = dr.forward(np.clip(tex0 * (1 + 0.3 * rng.standard_normal(tex0.shape)), 0.02, 0.98), [0.45, 0.4], [13.6, 13.2, 5.2])
    dr.params.baseSeed = 0xC030114
    img = dr.forward(tex0, [0.3, 0.6], [17, 12, 4])
    _, dldi = l2_loss(img, target)

    def step():
        im = dr.forward()
        loss, d = l2_loss(im, target)
        dr.backward(d)
        return dr.stats_forward.renderTimeMs, dr.stats_backward.renderTimeMs, dr.stats_forward.numKernelLaunches + dr.stats_backward.numKernelLaunches

    for _ in range(args.warmup):
        step()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        times = [step() for _ in range(args.steps)]
        wall = (time.perf_counter() - t0) / args.steps
    fwd = float(np.mean([t[0] for t in times]))
    bwd = float(np.mean([t[1] for t in times]))
    samples = W * H * spp
    line = {"metric": "adjoint/forward cost (PathTracer path-replay backward)", "value": round(bwd / fwd, 3), "unit": "x forward time", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(fwd + bwd, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded texture and scene)",
            "config": {"workload": cfg["name"], "texture": [cfg["tex"], cfg["tex"], 3], "roughness_params": len(boxes), "emitter_params": 3},
            "gpu_launches": int(sum(t[2] for t in times)),
            "forward": {"ms": round(fwd, 3), "Msamples_per_s": round(samples / fwd / 1e3, 3)},
            "backward": {"ms": round(bwd, 3), "Msamples_per_s": round(samples / bwd / 1e3, 3)},
            "e2e": {"value": round(wall * 1e3, 3), "unit": "ms per forward+loss+backward step", "h2d_bytes_per_step": int(dldi.nbytes),
                    "d2h_bytes_per_step": int(img.nbytes + 4 * (dr.n_tex + 4 * dr.n_mat + 3 * dr.n_em))},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_large(args, cfg):
    """The large combined job: 8 camera views of the 12.3M-triangle scene rendered in one batch
    with the path radiance kept (sst_forward_batch), an L2 loss against target views rendered
    with perturbed parameters, and the batched path-replay backward (sst_backward_batch) to the
    1024^2 x 3 terrain texture and the 2000 sphere roughness values."""
    from seesharp_gb300 import PathTracer, workloads
    from seesharp_gb300.adjoint import DifferentiableRender, l2_loss
    W, H, spp, depth = cfg["W"], cfg["H"], cfg["spp"], cfg["depth"]
    t0 = time.perf_counter()
    sc, tex, mats, views = workloads.large_combined(W, H)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sc.Prepare()
    prep_s = time.perf_counter() - t0
    info = sc.native.info()
    pt = PathTracer(TotalSpp=spp, MaxDepth=depth)
    tuning, tune_s = None, 0.0
    if not args.no_autotune:
        from seesharp_gb300 import _native
        t0 = time.perf_counter()
        tuning, _ = _native.autotune(sc.native, pt.params(sc), 1)
        tune_s = time.perf_counter() - t0
    dr = DifferentiableRender(sc, pt, texture=tex, roughness_materials=mats, views=views)
    rng = np.random.default_rng(5)
    tex0 = tex.Image.data.copy()
    r0 = np.array([m.MaterialParameters.Roughness.constColor for m in mats])
    dr.params.baseSeed = 0x5EED
    targets = dr.forward(np.clip(tex0 * (1 + 0.25 * rng.standard_normal(tex0.shape)), 0.02, 0.98), np.clip(r0 + 0.1 * rng.standard_normal(r0.shape), 0.05, 1.0))
    dr.params.baseSeed = 0xC030114
    dr.set_parameters(texture=tex0, roughness=r0)

    def step():
        imgs = dr.forward()
        losses = [l2_loss(i, t) for i, t in zip(imgs, targets)]
        g = dr.backward([d for _, d in losses])
        assert np.isfinite(g["texture"]).all() and np.isfinite(g["roughness"]).all()
        return dr.stats_forward.renderTimeMs, dr.stats_backward.renderTimeMs, dr.stats_forward.numKernelLaunches + dr.stats_backward.numKernelLaunches

    for _ in range(args.warmup):
        step()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        times = [step() for _ in range(args.steps)]
        wall = (time.perf_counter() - t0) / args.steps
    fwd = float(np.mean([t[0] for t in times]))
    bwd = float(np.mean([t[1] for t in times]))
    samples = len(views) * W * H * spp
    line = {"metric": "Msamples/s PathTracer, 8 views batched (forward) and adjoint/forward cost", "value": round(samples / fwd / 1e3, 3),
            "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(fwd + bwd, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": cfg["name"], "triangles": info["triangles"], "emitters": info["emitters"], "views": len(views), "width": W, "height": H,
                       "spp": spp, "max_depth": depth, "texture": list(tex0.shape), "roughness_params": len(mats)},
            "forward": {"ms": round(fwd, 3), "Msamples_per_s": round(samples / fwd / 1e3, 3)},
            "backward": {"ms": round(bwd, 3), "Msamples_per_s": round(samples / bwd / 1e3, 3)},
            "adjoint_over_forward": round(bwd / fwd, 3),
            "gpu_launches": int(sum(t[2] for t in times)),
            "e2e": {"value": round(samples / wall / 1e6, 3), "unit": "Msamples/s (forward samples per forward+loss+backward second)",
                    "h2d_bytes_per_step": int(len(views) * W * H * 12), "d2h_bytes_per_step": int(len(views) * W * H * 12 + 4 * (tex0.size + len(mats)))},
            "setup_s": {"generate": round(gen_s, 2), "prepare": round(prep_s, 2), "autotune": round(tune_s, 2)}, "tuning": tuning,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_lightpaths(args, cfg):
    """Light-path tracing for the bidirectional integrators (LightPathCache.TraceAllPaths) on the
    1M-triangle scene: Mpaths/s on the device (CUDA events), end to end with the vertices read
    back to the host, and the oracle's single-threaded restatement on a sample of the paths."""
    from oracle import pyoracle as O
    from seesharp_gb300 import workloads
    sc = workloads.sphere_field(cfg["spheres"], cfg["W"], cfg["H"])
    sc.Prepare()
    n, depth = cfg["paths"], cfg["depth"]
    for k in range(args.warmup):
        sc.native.trace_light_paths(99, k, n, depth)
    ms, verts = [], 0
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            _, _, lengths, st = sc.native.trace_light_paths(1234, k, n, depth)
            ms.append(st.renderTimeMs)
            verts += int(lengths.sum())
        wall = (time.perf_counter() - t0) / args.steps
    dev_ms = float(np.mean(ms))
    o = O.OracleScene.from_scene(sc)
    m = 4096
    t0 = time.perf_counter()
    o.light_paths(1234, 0, depth, m)
    cpu = m / (time.perf_counter() - t0) / 1e6
    stride_bytes = (depth + 1) * 88
    line = {"metric": "Mpaths/s light-path tracing (LightPathCache.TraceAllPaths)", "value": round(n / dev_ms / 1e3, 3), "unit": "Mpaths/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": cfg["name"], "paths": n, "max_depth": depth, "vertices_per_step": verts // max(args.steps, 1)},
            "e2e": {"value": round(n / wall / 1e6, 3), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": n * (stride_bytes + 4)},
            "cpu_baseline": {"value": round(cpu, 5), "unit": "Mpaths/s", "cores": 1, "kind": "port",
                             "sample": f"{m} paths of the same job, oracle restatement, one thread"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def make_scene(cfg):
    from seesharp_gb300 import FrameBuffer, workloads
    if cfg["builder"] == "cornell":
        return workloads.cornell_box(cfg["W"], cfg["H"])
    if cfg["builder"] == "scenefile":
        from seesharp_gb300 import sceneio
        sc = sceneio.load_json_scene(os.path.join(SCENE_DIR, cfg["path"]))
        sc.FrameBuffer = FrameBuffer(cfg["W"], cfg["H"])
        return sc
    return workloads.sphere_field(cfg["spheres"], cfg["W"], cfg["H"])


def scene_bytes(sc):
    """Bytes Scene.Prepare copies to the device: the packed triangle records (three float4
    vertices, a float4 face normal, an int4 material/mesh/face record and an int4 of vertex ids:
    96 bytes per triangle), the vertex normals and texture coordinates (for every vertex once any
    mesh has them), image textures and the environment map."""
    nt = sum(m.NumFaces for m in sc.Meshes)
    nv = sum(m.NumVertices for m in sc.Meshes)
    b = 96 * nt
    b += 12 * nv if any(m.ShadingNormals is not None for m in sc.Meshes) else 0
    b += 8 * nv if any(m.TextureCoordinates is not None for m in sc.Meshes) else 0
    seen = set()
    for m in sc.Meshes:
        for t in vars(getattr(m.Material, "MaterialParameters", object())).values() if m.Material is not None else ():
            img = getattr(t, "Image", None)
            if img is not None and id(img) not in seen:
                seen.add(id(img))
                b += img.data.nbytes
    if sc.Background is not None:
        b += sc.Background.Image.data.nbytes
    return int(b)


def film_readback_bytes(fb):
    """Bytes PathTracer.Render reads back into the frame buffer: the image, every layer and the
    outlier replay cache."""
    b = fb.Image.data.nbytes + sum(l.Image.data.nbytes for l in fb.layers.values() if l.Image is not None)
    if fb.OutlierCache is not None:
        b += fb.OutlierCache.weight.nbytes + fb.OutlierCache.iteration.nbytes
    return int(b)


def b_ray(ntri):
    """Algorithmic bytes of one ray query over N triangles: ray in (32) + hit out (16) + one
    root-to-leaf chain of 64-byte nodes + two leaf triangles (2 x 36)."""
    return 48 + 64 * math.ceil(math.log2(max(ntri, 2))) + 72


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def read_profile_traffic(kernel):
    """Per-ray DRAM traffic of a kernel from the committed ncu summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        parts = ln.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------------------------
def cpu_sample(cfg, seconds_target=15.0, min_paths=4096, nthreads=None, scene=None):
    """Times the oracle PathTracer on a bounded strided sample of the workload's paths.
    Returns (Msamples/s, description, threads)."""
    from oracle import pyoracle as O
    sc = scene if scene is not None else make_scene(cfg)
    o = O.OracleScene.from_scene(sc)
    p = o.params(cfg["W"], cfg["H"], cfg["spp"], cfg["depth"], baseSeed=cfg.get("seed", 0xC030114))
    nthreads = nthreads or os.cpu_count() or 1
    npix = cfg["W"] * cfg["H"]
    # calibrate on a small sample, then size the sample for ~seconds_target
    n = min_paths
    pix = np.linspace(0, npix - 1, n).astype(np.int32)
    t0 = time.perf_counter()
    o.render_paths(p, 0, pix, nthreads)
    dt = max(time.perf_counter() - t0, 1e-6)
    n = int(min(npix, max(min_paths, n * seconds_target / dt)))
    pix = np.linspace(0, npix - 1, n).astype(np.int32)
    t0 = time.perf_counter()
    o.render_paths(p, 1, pix, nthreads)
    dt = time.perf_counter() - t0
    return n / dt / 1e6, f"{n} strided paths of iteration 1 ({n / npix:.3f} of one spp)", nthreads, o, p, n


def run_reference_batch(args, cfg):
    """The batched workloads on the CPU restatement: the reference renders jobs one after another,
    so its throughput is the workload's samples over the sum of the jobs' times.  Bounded sample:
    8 jobs drawn with probability proportional to their sample counts (seeded), and the same
    number of strided paths of iteration 0 from each; the mean time per path of that sample
    estimates the workload's mean time per sample."""
    from oracle import pyoracle as O
    pairs = batch_jobs(cfg)
    sizes = np.array([sc.FrameBuffer.Width * sc.FrameBuffer.Height * pt.TotalSpp for sc, pt in pairs], np.float64)
    pick = np.random.default_rng(cfg["seed"] + 99).choice(len(pairs), size=8, replace=True, p=sizes / sizes.sum())
    nthreads = os.cpu_count() or 1
    jobs = []
    for j in pick:
        sc, pt = pairs[int(j)]
        o = O.OracleScene.from_scene(sc)
        W, H = sc.FrameBuffer.Width, sc.FrameBuffer.Height
        jobs.append((o, o.params(W, H, pt.TotalSpp, pt.MaxDepth), W * H))
    per_job = 2048
    o, p, npix = jobs[0]
    t0 = time.perf_counter()
    o.render_paths(p, 0, np.linspace(0, npix - 1, per_job).astype(np.int32), nthreads)
    dt = max(time.perf_counter() - t0, 1e-6)
    # size one step (all 8 jobs) for a few seconds of CPU work
    per_job = int(max(1024, per_job * max(2.0, 60.0 / max(1, args.steps + args.warmup)) / (8 * dt)))

    def step(it):
        # per_job paths of each job: strided pixels of as many iterations as that takes
        n = 0
        for o, p, npix in jobs:
            left, k = per_job, 0
            while left > 0:
                m = min(left, npix)
                o.render_paths(p, it + k, np.linspace(0, npix - 1, m).astype(np.int32), nthreads)
                left -= m
                n += m
                k += 1
        return n
    for w in range(args.warmup):
        step(1000 * (w + 1))
    t0 = time.perf_counter()
    n = sum(step(100000 + 1000 * k) for k in range(args.steps))
    dt = time.perf_counter() - t0
    val = n / dt / 1e6
    line = {
        "metric": "Msamples/s PathTracer (batched jobs)", "value": round(val, 4), "unit": "Msamples/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1000, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)", "impl": "reference",
        "config": {"workload": cfg["name"], "jobs": len(pairs)},
        "cpu_baseline": {"value": round(val, 4), "unit": "Msamples/s", "cores": nthreads, "kind": "port",
                         "sample": f"8 of the {len(pairs)} jobs drawn in proportion to their samples, {per_job} strided paths of each per step "
                                   f"(consecutive iterations), C++ restatement of the reference PathTracer on {nthreads} host threads"},
        "e2e": {"value": round(val, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, cfg):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    if cfg["builder"] == "batch":
        run_reference_batch(args, cfg)
        return
    from seesharp_gb300 import workloads  # noqa: F401  (scene generator only)
    sc = make_scene(cfg)
    nthreads = os.cpu_count() or 1
    # size one step for a few seconds of CPU work
    _, _, _, o, p, n = cpu_sample(cfg, seconds_target=max(2.0, 60.0 / max(1, args.steps + args.warmup)), nthreads=nthreads, scene=sc)
    pix = np.linspace(0, cfg["W"] * cfg["H"] - 1, n).astype(np.int32)
    for w in range(args.warmup):
        o.render_paths(p, 2 + w, pix, nthreads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        o.render_paths(p, 100 + k, pix, nthreads)
    dt = time.perf_counter() - t0
    val = n * args.steps / dt / 1e6
    line = {
        "metric": "Msamples/s PathTracer", "value": round(val, 4), "unit": "Msamples/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1000, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)", "impl": "reference",
        "config": {"workload": cfg["name"]},
        "cpu_baseline": {"value": round(val, 4), "unit": "Msamples/s", "cores": nthreads, "kind": "port",
                         "sample": f"{n} strided paths per step of the {cfg['W']}x{cfg['H']} image (one sample each), C++ restatement of the "
                                   f"reference PathTracer on {nthreads} host threads"},
        "e2e": {"value": round(val, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, cfg):
    import torch

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        # replicas: the only cross-rank traffic is the barrier and the max over ranks of the step time
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from seesharp_gb300 import PathTracer, _native

    sc = make_scene(cfg)
    sc.device = local
    t0 = time.perf_counter()
    sc.Prepare()
    prep_s = time.perf_counter() - t0
    ctx = _native.default_context(local)
    info = sc.native.info()
    W, H, spp, depth = cfg["W"], cfg["H"], cfg["spp"], cfg["depth"]
    samples = W * H * spp
    film = torch.zeros((H, W, 3), dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    params = _native.make_params(W, H, spp, depth, baseSeed=cfg.get("seed", 0xC030114))

    def step():
        return sc.native.render(params, film.data_ptr(), _native.SST_MEM_DEVICE)

    # launch configuration for this scene (sst_autotune: short trial renders, results unchanged)
    if args.tuning:
        _native.set_tuning(ctx, **json.loads(args.tuning))
    tuning, tune_s = _native.get_tuning(ctx), 0.0
    if not args.no_autotune and not args.tuning:
        t0 = time.perf_counter()
        tuning, _ = _native.autotune(sc.native, params, 2)
        tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        step()
    # timed region: K renders (the production path: one CUDA graph per wave), L2 flushed between
    # them, the renderer's CUDA-event time per render
    render_ms, rays, srays, launches = 0.0, 0, 0, 0
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize()
            st = step()
            render_ms += st.renderTimeMs
            rays += st.numRays
            srays += st.numShadowRays
            launches += st.numKernelLaunches
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    barrier(ws)
    # one more render with per-kernel CUDA events (kernel split and the roofline's kernel time)
    _native.set_profiling(ctx, True)
    flush.fill_(-1.0)
    torch.cuda.synchronize()
    step()
    ktimes = _native.kernel_times(ctx)
    _native.set_profiling(ctx, False)
    ms_per_step = max_over_ranks(ws, render_ms / args.steps)
    value = samples * ws / (ms_per_step / 1000.0) / 1e6

    # e2e through the public API with host buffers: Prepare (geometry H2D, BVH) + Render (film D2H)
    from seesharp_gb300 import FrameBuffer
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 3))
    h2d = scene_bytes(sc)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sc.FrameBuffer = FrameBuffer(W, H)
        sc.Prepare()
        PathTracer(TotalSpp=spp, MaxDepth=depth, BaseSeed=cfg.get("seed", 0xC030114)).Render(sc)
    e2e_s = max_over_ranks(ws, (time.perf_counter() - t0) / max(e2e_steps, 1))
    e2e_val = samples * ws / e2e_s / 1e6 if e2e_steps else None
    d2h = film_readback_bytes(sc.FrameBuffer) if e2e_steps else W * H * 12
    if e2e_steps:
        assert np.isfinite(sc.FrameBuffer.Image.data).all()

    # roofline of the dominant traversal kernel
    peak, peak_kind = measured_peaks()
    tc = ktimes["trace_closest"]
    bpr = b_ray(info["triangles"])
    per_launch_bytes = tc["items"] * bpr / max(tc["launches"], 1)
    avg_ms = tc["ms"] / max(tc["launches"], 1)
    achieved = per_launch_bytes / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
    tpr = read_profile_traffic("trace_closest")
    roofline = {"kernel": "k_trace<0> (closest-hit BVH traversal)", "bound": "hbm", "achieved": round(achieved, 2), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": None if tpr is None else round(tpr * tc["items"] / max(tc["launches"], 1)),
                "algorithmic_bytes_per_ray": bpr, "rays_per_launch": round(tc["items"] / max(tc["launches"], 1)),
                "avg_launch_ms": round(avg_ms, 4)}
    # algorithmic bytes per sample (B_sample) from the traced ray counts
    steps = args.steps
    ext, sh = rays / steps / samples, srays / steps / samples
    b_sample = ext * (bpr + 172) + sh * (bpr - 12) + 12

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        val, desc, thr, _, _, _ = cpu_sample(cfg, seconds_target=args.cpu_seconds, scene=sc)
        cpu = {"value": round(val, 4), "unit": "Msamples/s", "cores": thr, "kind": "port",
               "sample": desc + f"; C++ restatement of the reference PathTracer, {thr} threads"}
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": "Msamples/s PathTracer", "value": round(value, 3), "unit": "Msamples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32",
            "data": "the reference's own scene file (tests/golden/scenes)" if cfg["builder"] == "scenefile" else "synthetic (seeded scene generator)",
            "config": {"workload": cfg["name"], "triangles": info["triangles"], "emitters": info["emitters"], "bvh_nodes": info["bvh_nodes"],
                       "width": W, "height": H, "spp": spp, "max_depth": depth, "l2": "256 MB buffer written between timed steps",
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": None if e2e_val is None else round(e2e_val, 3), "unit": "Msamples/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "s_per_step": round(e2e_s, 4), "includes": "Scene.Prepare (upload + BVH build) + PathTracer.Render (film, layers and outlier cache read back)"},
            "roofline": roofline,
            "bytes_per_sample": round(b_sample, 1), "rays_per_sample": round(ext, 4), "shadow_rays_per_sample": round(sh, 4),
            "gpu_launches": launches,
            "kernel_ms": {k: round(v["ms"], 3) for k, v in ktimes.items()},
            "kernel_ms_note": "one extra render with per-kernel CUDA events after the timed region",
            "tuning": tuning, "autotune_s": round(tune_s, 3),
            "prepare_s": round(prep_s, 3), "bvh": os.environ.get("SST_BVH", "ploc"),
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        if cfg.get("recorded"):
            with open(os.path.join(SCENE_DIR, cfg["recorded"])) as f:
                rec_ms = float(json.load(f)["RenderTime"])
            line["reference_recorded"] = {"render_time_ms": rec_ms, "Msamples_per_s": round(samples / rec_ms / 1e3, 4),
                                          "source": "the reference's stored reference-image metadata for this scene and configuration "
                                                    "(Data/Scenes/" + cfg["recorded"] + "), measured by its authors on their CPU"}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=sorted(CONFIGS))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default=None, help="pin the launch configuration (JSON of SstTuning fields; implies --no-autotune)")
    ap.add_argument("--width", type=int, default=None, help="override (profiling cases)")
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--spp", type=int, default=None)
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    for k, a in (("W", args.width), ("H", args.height), ("spp", args.spp)):
        if a is not None:
            cfg[k] = a
            cfg["name"] = cfg["name"] + f"_{k}{a}"
    os.environ.setdefault("SST_BVH", "ploc")
    if args.impl == "reference" and cfg["builder"] in ("adjoint", "large", "lightpaths"):
        if dist_info()[1] == 0:
            print(json.dumps({"impl": "reference", "unavailable": "this workload has no counterpart in the reference PathTracer's CPU path"}))
    elif args.impl == "reference":
        run_reference(args, cfg)
    elif cfg["builder"] == "batch":
        run_batch(args, cfg)
    elif cfg["builder"] == "adjoint":
        run_adjoint(args, cfg)
    elif cfg["builder"] == "large":
        run_large(args, cfg)
    elif cfg["builder"] == "lightpaths":
        run_lightpaths(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()

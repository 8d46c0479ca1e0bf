"""Benchmark: incoherent closest-hit traversal on the 1M-triangle scene (the headline Mrays/s metric).

Workload: a seeded mesh of 1 000 000 triangles (icosphere of frequency 200 displaced by 3-octave value noise,
plus 200 000 random small triangles in [-2, 2]^3) and 4 194 304 incoherent rays (area-uniform surface origins,
cosine-distributed directions). One step = one lgb_trace_closest over all rays.

  value  rays / device time of the trace kernel (CUDA events on the launching stream), L2 flushed with a
         256 MB write before every step so each step starts cold
  e2e    the same query on host buffers through lgb_trace_closest_host: the kernel loads every ray from pinned
         host memory and stores every hit there (each crosses the CPU-GPU link once), inside the timed region
  cpu_baseline  the CPU oracle (binary SAH BVH, same watertight test) on a bounded sample of the rays,
         all host threads

--impl reference times the CPU oracle (the reference path restated on the CPU; Lumen itself needs a
Vulkan ray-tracing device) on the same workload. N > 1 GPUs run independent replicas (the path shards by
ray with no exchange step), one rank per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_INCOHERENT = 4 * 1024 * 1024
METRIC = "Mrays/s incoherent closest-hit"
WORKLOAD = "traversal: 1M-triangle displaced icosphere + random triangles, 4M incoherent closest-hit rays"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(cache=True):
    from lumen_gb300 import procedural
    path = os.path.join("/tmp", "lgb_bench_traversal_v1.npz")
    if cache and os.path.exists(path):
        z = np.load(path, allow_pickle=True)
        arrays = procedural.traversal_scene(sphere_freq=1, n_random=0)  # shell with the right meshes/materials
        for k in ("positions", "normals", "uvs", "indices", "meshes"):
            setattr(arrays, k, z[k])
        return arrays, z["rays"]
    arrays = procedural.traversal_scene()
    rays = procedural.incoherent_rays(arrays, N_INCOHERENT, seed=3)
    if cache:
        try:
            np.savez(path, positions=arrays.positions, normals=arrays.normals, uvs=arrays.uvs, indices=arrays.indices,
                     meshes=arrays.meshes, rays=rays)
        except OSError:
            pass
    return arrays, rays


TRAVERSAL_SOURCES = ("lumen_gb300/csrc/traverse.cuh", "lumen_gb300/csrc/traverse.cu", "lumen_gb300/csrc/lgb_internal.cuh")


def measured_traffic(rays: int) -> dict:
    """DRAM and L2 bytes of one launch of the closest-hit kernel from the committed ncu record
    (profiles/trace_closest_incoherent_1M.ncu.json), scaled to `rays`, when the record was taken of the traversal
    sources being run (same SHA-256 over TRAVERSAL_SOURCES); otherwise nulls and the reason."""
    import hashlib
    none = {"dram_bytes": None, "l2_bytes": None, "l2_bytes_per_ray": None, "dram_bytes_per_ray": None}
    path = os.path.join(ROOT, "profiles", "trace_closest_incoherent_1M.ncu.json")
    if not os.path.exists(path):
        return {**none, "source": "no ncu record"}
    with open(path) as f:
        rec = json.load(f)
    h = hashlib.sha256()
    for name in TRAVERSAL_SOURCES:
        with open(os.path.join(ROOT, name), "rb") as f:
            h.update(f.read())
    if rec.get("source_sha256") != h.hexdigest():
        return {**none, "source": "ncu record is of other traversal sources (stale): not used"}
    per_ray_dram = rec["dram_bytes_per_ray"]
    return {"dram_bytes": per_ray_dram * rays, "l2_bytes": rec["l2_bytes_per_ray"] * rays,
            "l2_bytes_per_ray": rec["l2_bytes_per_ray"], "dram_bytes_per_ray": per_ray_dram,
            "source": "ncu record of this kernel version (profiles/trace_closest_incoherent_1M.ncu.json): "
                      + rec["command"]}


def measure_l2_peak(device: int) -> float:
    """Read bandwidth of a 32 MB L2-resident buffer streamed 64 times by every SM (lgb_measure_l2_read_gbs)."""
    import ctypes as C
    from lumen_gb300 import abi
    out = C.c_double(0.0)
    st = abi.load().lgb_measure_l2_read_gbs(device, 32 << 20, 64, C.byref(out))
    return out.value if st == abi.LGB_OK else float("nan")


CPU_WINDOW = 100_000  # rays per timed step of the CPU oracle


def cpu_oracle_steps(arrays, rays, steps, warmup, threads=None):
    """The CPU oracle (binary SAH BVH, same watertight test) on all host threads: each step traces one window of
    CPU_WINDOW contiguous rays at a seeded random offset of the 4M incoherent set; returns (Mrays/s per timed step,
    threads). Both the cpu_baseline of the GPU line and --impl reference time it this way."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    ora = oracle_lib.Oracle()
    threads = threads or (os.cpu_count() or 1)
    bvh = ora.bvh(arrays.tri_verts())
    rng = np.random.default_rng(11)
    vals = []
    for step in range(warmup + steps):
        idx = int(rng.integers(0, len(rays) - CPU_WINDOW))
        t0 = time.perf_counter()
        bvh.closest(rays[idx:idx + CPU_WINDOW], threads)
        dt = time.perf_counter() - t0
        if step >= warmup:
            vals.append(CPU_WINDOW / dt / 1e6)
    return vals, threads


def cpu_integrator_rate(kind, arrays, w, h, frames, depth, **kw):
    """The CPU oracle's integrator `kind` ("vcm", "sppm", "restir_di", "bdpt") on `frames` frames at w x h, all
    host cores: the cpu_baseline entry of a secondary line (pixels per second as Msamples/s)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    from lumen_gb300.scene import camera_forward, camera_lookat, scene_radius, vcm_params, vcm_radius
    ora = oracle_lib.Oracle()
    osc = ora.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    threads = os.cpu_count() or 1
    nl, ltc, spot = len(arrays.lights), arrays.light_triangle_count, kw.get("spot_angle", 0.0)
    if kind == "vcm":
        st = osc.vcm_state(w, h, depth)
        R = scene_radius(arrays)
    elif kind == "sppm":
        st = oracle_lib.sppm_state(w, h, depth)
    elif kind == "restir_di":
        st = oracle_lib.restir_state(w, h)
    else:
        st = oracle_lib.bdpt_state(w, h)
    t0 = time.perf_counter()
    for f in range(frames):
        if kind == "vcm":
            g = vcm_params(arrays, depth, vcm_radius(R, 1.0, f, 0.75), 1000 + f, 5000 + f, f, spot_angle=spot)
            p = oracle_lib.VcmParams()
            for name in ("max_depth", "num_lights", "light_triangle_count", "radius", "use_vm", "use_vc",
                         "light_seed", "eye_seed", "frame_num", "flags", "spot_angle"):
                setattr(p, name, getattr(g, name))
            p.scene_min[:] = list(g.scene_min)
            p.scene_max[:] = list(g.scene_max)
            osc.vcm_iteration(cam, view, proj, p, st, threads)
        elif kind == "sppm":
            p = oracle_lib.SppmParams()
            p.max_depth, p.num_lights, p.light_triangle_count, p.base_radius = depth, nl, ltc, kw.get("base_radius", 0.03)
            p.seed, p.frame_num, p.spot_angle = 77, f, spot
            oracle_lib.sppm_iteration(osc, cam, p, st, threads)
        elif kind == "restir_di":
            p = oracle_lib.RestirParams()
            p.num_lights, p.light_triangle_count, p.seed, p.frame_num = nl, ltc, 91, f
            p.do_spatiotemporal, p.enable_accumulation, p.spot_angle, p.flags = 1 if f else 0, 1, spot, kw.get("flags", 0)
            oracle_lib.restir_iteration(osc, cam, view, proj, p, st, threads)
        else:
            p = oracle_lib.BdptParams()
            p.max_depth, p.num_lights, p.light_triangle_count, p.seed, p.frame_num, p.spot_angle = depth, nl, ltc, 53, f, spot
            oracle_lib.bdpt_iteration(osc, cam, view, proj, p, st, threads)
    dt = time.perf_counter() - t0
    return {"value": w * h * frames / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{frames} frames of the same scene at {w}x{h} on the CPU oracle"}


def cornell_secondary(torch, ctx_cls, scene_cls, local, cpu_leg: bool):
    """The Cornell-box path tracer (256^2, 16 spp, depth 8): GPU Msamples/s through lgb_render_path, L2 not
    flushed (the scene is 36 triangles), and the CPU oracle on a bounded sample of the same frames."""
    from lumen_gb300 import procedural
    from lumen_gb300.scene import camera_lookat, path_params
    cb = procedural.cornell_box()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, cb)
    sc.build()
    w = h = 256
    spp = 16
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    params = path_params(cb, 8)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        sc.render_path(cam, params, 0, spp, film, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    times = []
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        sc.render_path(cam, params, 0, spp, film, stream=stream.cuda_stream)
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e))
    sc.sync(stream.cuda_stream)
    ms = float(np.median(times))
    out = {"workload": "Cornell box 36 triangles, 256x256, 16 spp, max depth 8, FP32", "ms": ms,
           "msamples_per_s": w * h * spp / (ms * 1e-3) / 1e6, "mean_radiance": float(film[:, :3].mean()),
           "graph": "bounce loop captured once as a CUDA graph and replayed"}
    out["rmse_vs_fp64"] = {"value": reference_rmse(torch, ctx, film, "cornell_256_fp64_ref.npy"),
                           "render": "this 16-spp film, 256x256",
                           "reference": "FP64 CPU oracle, 2048 spp (tests/golden/cornell_256_fp64_ref.npy)"}
    if cpu_leg:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib
        ora = oracle_lib.Oracle()
        osc = ora.scene(cb)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        osc.film(cam, 8, w, h, 0, 2, threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": w * h * 2 / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
                               "sample": "frames 0-1 of the same render"}
    return out


def reference_rmse(torch, ctx, film, name):
    """RMSE (lgb_film_rmse, RGB) of an (N, 4) CUDA film against a committed converged render in tests/golden, or
    None when the file is absent."""
    from lumen_gb300.scene import film_rmse
    path = os.path.join(ROOT, "tests", "golden", name)
    if not os.path.exists(path):
        return None
    ref = np.load(path).reshape(-1, 3)
    ref4 = torch.from_numpy(np.concatenate([ref, np.ones((len(ref), 1), np.float32)], 1)).cuda()
    return film_rmse(ctx, film, ref4, 0)


def adjoint_secondary(torch, ctx_cls, scene_cls, local):
    """Differentiable rendering (512^2, 32 spp, max depth 6, textured back wall + two GGX conductor boxes):
    time of the primal (lgb_diff_render keeping the per-sample radiance) and of the adjoint replay
    (lgb_adjoint_path from those samples) for gradients of an L2 image loss wrt 64x64 texels, roughness and
    emission; the ratio (primal + adjoint) / primal is the cost of one gradient step."""
    from lumen_gb300 import procedural
    from lumen_gb300.scene import camera_lookat, path_params
    arrays = procedural.cornell_diff()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, arrays)
    sc.build()
    w = h = 512
    spp = 32
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    params = path_params(arrays, 6)
    tex = torch.from_numpy(np.ascontiguousarray(arrays.textures[0])).cuda()
    rough = torch.from_numpy(arrays.materials["roughness"].astype(np.float32)).cuda()
    emis = torch.from_numpy(arrays.materials["emissive_factor"].astype(np.float32)).cuda()
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    samples = torch.empty((spp * w * h, 4), dtype=torch.float32, device="cuda")
    target = torch.from_numpy(np.random.default_rng(7).uniform(0.0, 1.0, (w * h, 4)).astype(np.float32)).cuda()
    gt, gr, ge = torch.zeros_like(tex), torch.zeros_like(rough), torch.zeros_like(emis)
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream

    def primal():
        sc.diff_render(cam, params, 0, spp, film, 0, tex, rough, emis, samples=samples, stream=cs)

    def backward():
        dimage = (film - target) * (2.0 / film.numel())
        sc.adjoint_path(cam, params, 0, spp, dimage, 0, tex, rough, emis, gt, gr, ge, samples=samples, stream=cs)

    for _ in range(2):
        primal()
        backward()
    torch.cuda.synchronize()
    tp, ta = [], []
    for _ in range(5):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        primal()
        e[1].record(stream)
        backward()
        e[2].record(stream)
        e[2].synchronize()
        tp.append(e[0].elapsed_time(e[1]))
        ta.append(e[1].elapsed_time(e[2]))
    sc.sync(cs)
    mp, ma = float(np.median(tp)), float(np.median(ta))
    rmse = reference_rmse(torch, ctx, film, "diff_512_fp64_ref.npy")
    grad_norms = {"texels": float(gt.norm()), "roughness": float(gr.norm()), "emission": float(ge.norm())}
    adam = adam_recovery(torch, sc, arrays, cam, params, w, h, spp, cs)
    return {"workload": "differentiable Cornell box, 512x512, 32 spp, max depth 6, 64x64 RGB texels + per-material "
                        "roughness + emission, L2 image loss", "primal_ms": mp, "adjoint_ms": ma,
            "primal_plus_adjoint_over_primal": (mp + ma) / mp,
            "primal_msamples_per_s": w * h * spp / (mp * 1e-3) / 1e6,
            "rmse_vs_fp64": {"value": rmse, "render": "the primal image, 32 spp, 512x512",
                             "reference": "FP64 CPU oracle, 512 spp (tests/golden/diff_512_fp64_ref.npy)"},
            "grad_norms": grad_norms, "adam_200_steps": adam}


def adam_recovery(torch, sc, arrays, cam, params, w, h, spp, cs, steps=200):
    """200 Adam steps at the configuration's size (512^2, 32 spp per step) from the scene's parameters towards a
    target rendered (256 spp) with another seeded texture (seed 6), box roughnesses 0.2 / 0.3 and emission
    (14, 12.5, 11). Each step renders fresh frames with lgb_diff_render (sampling with the current values) and
    replays independent frames with lgb_adjoint_path for d (mean squared image error) / d parameter. Reports the
    parameter RMSE against the target before and after (texels: those the camera sees directly), the image loss
    and the time per step. The replay frames get their own primal with stored samples, so the adjoint runs as the
    wavefront replay of stored samples (three wavefront passes per step)."""
    from lumen_gb300 import abi, procedural
    emitter, short, tall = 3, 5, 6
    tex_t = torch.from_numpy(procedural.albedo_texture(6)).cuda()
    rough_t = torch.from_numpy(arrays.materials["roughness"].astype(np.float32)).cuda()
    rough_t[short], rough_t[tall] = 0.2, 0.3
    emis_t = torch.from_numpy(arrays.materials["emissive_factor"].astype(np.float32)).cuda()
    emis_t[emitter] = torch.tensor([14.0, 12.5, 11.0])
    npix = w * h
    target = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    sc.diff_render(cam, params, 1 << 20, 256, target, 0, tex_t, rough_t, emis_t, stream=cs)
    tex = torch.from_numpy(np.ascontiguousarray(arrays.textures[0])).cuda()
    rough = torch.from_numpy(arrays.materials["roughness"].astype(np.float32)).cuda()
    emis = torch.from_numpy(arrays.materials["emissive_factor"].astype(np.float32)).cuda()
    # texels the camera sees directly: the texel gradient of the image sum at path length 2
    vis = torch.zeros_like(tex)
    ones = torch.ones((npix, 4), dtype=torch.float32, device="cuda")
    p2 = abi.PathParams.from_buffer_copy(params)
    p2.max_depth = 2
    sc.adjoint_path(cam, p2, 0, 4, ones, 0, tex, rough, emis, vis, torch.zeros_like(rough), torch.zeros_like(emis),
                    stream=cs)
    torch.cuda.synchronize()
    vis = vis[..., :3].abs().sum(-1)
    mask = vis > torch.quantile(vis[vis > 0], 0.5)

    def rmse():
        return {"texels_seen": float((tex - tex_t)[..., :3][mask].pow(2).mean().sqrt()),
                "roughness": float((rough - rough_t)[[short, tall]].pow(2).mean().sqrt()),
                "emission": float((emis - emis_t)[emitter].pow(2).mean().sqrt())}

    film = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    replay = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    samples = torch.empty((spp * npix, 4), dtype=torch.float32, device="cuda")

    def image_loss():
        sc.diff_render(cam, params, 1 << 22, 64, film, 0, tex, rough, emis, stream=cs)
        return float(((film[:, :3] - target[:, :3]) ** 2).mean())

    before, loss0 = rmse(), image_loss()
    state = [(p, torch.zeros_like(p), torch.zeros_like(p), lr) for p, lr in ((tex, 0.05), (rough, 0.01), (emis, 0.2))]
    g = [torch.zeros_like(tex), torch.zeros_like(rough), torch.zeros_like(emis)]
    b1, b2, eps = 0.9, 0.999, 1e-8
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for step in range(steps):
        sc.diff_render(cam, params, step * spp, spp, film, 0, tex, rough, emis, flags=abi.DIFF_SAMPLE_PARAMS,
                       stream=cs)
        dimage = (film - target) * (2.0 / (3 * npix))
        dimage[:, 3] = 0.0
        for x in g:
            x.zero_()
        sc.diff_render(cam, params, (1 << 24) + step * spp, spp, replay, 0, tex, rough, emis, samples=samples,
                       flags=abi.DIFF_SAMPLE_PARAMS, stream=cs)
        sc.adjoint_path(cam, params, (1 << 24) + step * spp, spp, dimage, 0, tex, rough, emis, g[0], g[1], g[2],
                        samples=samples, flags=abi.DIFF_SAMPLE_PARAMS, stream=cs)
        t = step + 1
        for (p, m, v, lr), gr in zip(state, g):
            m.mul_(b1).add_(gr, alpha=1 - b1)
            v.mul_(b2).addcmul_(gr, gr, value=1 - b2)
            p.sub_(lr * (m / (1 - b1 ** t)) / ((v / (1 - b2 ** t)).sqrt() + eps))
        tex.clamp_(0.01, 1.0)
        rough.clamp_(0.1, 1.0)
        emis.clamp_(min=0.0)
    e1.record(stream)
    e1.synchronize()
    after, loss1 = rmse(), image_loss()
    return {"steps": steps, "spp_per_step": spp, "ms_per_step": e0.elapsed_time(e1) / steps,
            "parameter_rmse_before": before, "parameter_rmse_after": after,
            "image_loss_64spp_before": loss0, "image_loss_64spp_after": loss1}


def batch_secondary(torch, ctx_cls, scene_cls, local):
    """Batched rendering: the 32-scene configuration (10k-2M triangles, 128^2-1024^2, 8-64 spp, depth 12,
    principled / dielectric materials) rendered (a) scene after scene through lgb_render_path and (b) as one
    tuned lgb_batch_render. Both give the same per-path computation, so the films are compared for equality
    (equal RMSE against any reference) and the Msamples/s of the two are reported."""
    import multiprocessing as mp
    from lumen_gb300 import procedural
    from lumen_gb300.scene import Batch, camera_lookat, path_params
    cfg = procedural.batch_config()
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        arrays = pool.starmap(procedural.batch_scene, [(seed, tris) for seed, tris, _, _, _ in cfg])
    gen_s = time.perf_counter() - t0
    ctx = ctx_cls(local)
    scenes = []
    for a in arrays:
        sc = scene_cls(ctx, a)
        sc.build()
        scenes.append(sc)
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream
    jobs, films_a, films_b = [], [], []
    for i, (a, (_, _, w, h, spp)) in enumerate(zip(arrays, cfg)):
        cam = camera_lookat(a.camera_pos, a.camera_dir, a.fov, w, h)
        films_a.append(torch.zeros((w * h, 4), dtype=torch.float32, device="cuda"))
        films_b.append(torch.zeros((w * h, 4), dtype=torch.float32, device="cuda"))
        jobs.append((i, cam, path_params(a, 12), spp))
    samples = sum(w * h * spp for _, _, w, h, spp in cfg)

    def alone():
        for i, cam, params, spp in jobs:
            scenes[i].render_path(cam, params, 0, spp, films_a[i], stream=cs)

    batch = Batch(ctx, scenes)
    bjobs = [Batch.job(i, cam, params, 0, spp, films_b[i]) for i, cam, params, spp in jobs]
    t0 = time.perf_counter()
    best = batch.tune(bjobs, stream=cs)
    tune_s = time.perf_counter() - t0

    def batched():
        batch.render(bjobs, stream=cs)

    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        out = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return min(out)

    ms_alone = timed(alone)
    ms_batch = timed(batched)
    batch.sync(cs)
    max_diff = max(float((fa - fb).abs().max()) for fa, fb in zip(films_a, films_b))
    # convergence: three of the scenes at 128^2 with their own spp, batched and scene by scene, against the
    # committed FP64 oracle references (2048 spp, independent frames)
    rmse = []
    for idx in (1, 13, 21):
        a = arrays[idx]
        spp = cfg[idx][4]
        cam = camera_lookat(a.camera_pos, a.camera_dir, a.fov, 128, 128)
        fa = torch.zeros((128 * 128, 4), dtype=torch.float32, device="cuda")
        fb = torch.zeros((128 * 128, 4), dtype=torch.float32, device="cuda")
        scenes[idx].render_path(cam, path_params(a, 12), 0, spp, fa, stream=cs)
        batch.render([Batch.job(idx, cam, path_params(a, 12), 0, spp, fb)], stream=cs)
        batch.sync(cs)
        ref = f"batch_scene{idx}_128_fp64_ref.npy"
        rmse.append({"scene": idx, "triangles": cfg[idx][1], "spp": spp,
                     "per_scene": reference_rmse(torch, ctx, fa, ref), "batched": reference_rmse(torch, ctx, fb, ref)})
    res = {"workload": "32 scenes, 10k-2M triangles (log-uniform, 14.3M total), 128^2-1024^2, 8-64 spp, depth 12, "
                       "principled (80 %) and dielectric (20 %) materials, 1-8 quad lights",
           "samples": samples, "per_scene_ms": ms_alone, "batched_ms": ms_batch,
           "per_scene_msamples_per_s": samples / (ms_alone * 1e-3) / 1e6,
           "batched_msamples_per_s": samples / (ms_batch * 1e-3) / 1e6,
           "speedup": ms_alone / ms_batch, "films_max_abs_diff": max_diff,
           "rmse_vs_fp64": {"scenes": rmse, "render": "128x128 at the scene's own spp",
                            "reference": "FP64 CPU oracle, 2048 spp (tests/golden/batch_scene*_128_fp64_ref.npy)"},
           "tuned": {"path_capacity": best.path_capacity, "work_blocks_per_sm": best.work_blocks_per_sm,
                     "stack": "shared" if best.stack_placement == 1 else "local",
                     "path_regeneration": best.chunk_paths != 1,
                     "traversal": {0: "by size", 1: "coherent", 2: "incoherent"}.get(best.traversal, "?")},
           "tune_s": tune_s, "scene_generation_s": gen_s}
    batch.close()
    for sc in scenes:
        sc.close()
    return res


def traversal_secondary(torch, sc, rays, flush, stream, reps=10, warmup=3):
    """The other two traversal figures of the 1M-triangle configuration, on the same BVH: 1M coherent primary
    rays (1024^2 pinhole at (0, 0, -4) looking at the origin, fov 45 degrees, pixel centres) closest-hit, and
    any-hit for the 4M incoherent origins with tmax = 0.5. Median of `reps` launches, L2 flushed before each."""
    from lumen_gb300 import procedural
    sptr = stream.cuda_stream
    prim = torch.from_numpy(procedural.primary_rays(1024, 1024)).cuda()
    hits = torch.empty((prim.shape[0], 4), dtype=torch.int32, device="cuda")
    short = torch.from_numpy(rays).cuda()
    short[:, 7] = 0.5
    bits = torch.zeros((len(rays) + 31) // 32, dtype=torch.int32, device="cuda")

    def timed(fn, prep):
        for _ in range(warmup):
            prep()
            fn()
        ts = []
        for _ in range(reps):
            prep()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            ts.append(s.elapsed_time(e))
        return statistics.median(ts)

    def prep_bits():
        flush.fill_(1.0)
        bits.zero_()

    t_c = timed(lambda: sc.trace_closest(prim, hits, stream=sptr), lambda: flush.fill_(1.0))
    t_a = timed(lambda: sc.trace_any(short, bits, stream=sptr), prep_bits)
    counters = torch.zeros(2, dtype=torch.int64, device="cuda")
    sc.trace_closest_counted(prim, hits, counters, stream=sptr)
    sc.sync(sptr)
    n_nodes, n_tris = (counters.cpu().numpy() / prim.shape[0]).tolist()
    return {"coherent_closest_mrays_per_s": prim.shape[0] / (t_c * 1e-3) / 1e6,
            "coherent_rays": int(prim.shape[0]), "coherent_nodes_per_ray": n_nodes, "coherent_tris_per_ray": n_tris,
            "coherent_hit_fraction": float((hits[:, 0] != -1).float().mean()),
            "incoherent_any_tmax_0.5_mrays_per_s": len(rays) / (t_a * 1e-3) / 1e6,
            "any_occluded_fraction": float(np.unpackbits(bits.cpu().numpy().view(np.uint8)).sum()) / len(rays),
            "l2": "flushed with a 256 MB write before every launch"}


def vcm_secondary(torch, ctx_cls, scene_cls, local, cpu_leg=False, iters=63):
    """VCM caustics configuration: dielectric torus (200k triangles) on a diffuse plane, spot light (cone
    half-angle 20 degrees, falloff from 25/30 of it), 1024^2, one light subpath and one eye subpath per pixel per
    iteration (1M each), max depth 10, merge radius 0.01 x scene radius shrinking with alpha = 0.75, 64
    iterations: the first is the warm-up, the other 63 are timed (device time per lgb_vcm_iteration)."""
    from lumen_gb300 import procedural
    from lumen_gb300.scene import camera_lookat, scene_radius, vcm_params, vcm_radius
    arrays = procedural.vcm_scene()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, arrays)
    sc.build()
    w = h = 1024
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    R = scene_radius(arrays)
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream

    def it(i):
        sc.vcm_iteration(cam, vcm_params(arrays, 10, vcm_radius(R, 1.0, i, 0.75), 1000 + i, 5000 + i, i,
                                         spot_angle=20.0), film, stream=cs)

    it(0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(1, iters + 1):
        it(i)
    e1.record(stream)
    e1.synchronize()
    sc.sync(cs)
    ms = e0.elapsed_time(e1) / iters
    # convergence: the same 64 iterations at 256^2 against the committed 2048-iteration FP64 oracle render
    w2 = h2 = 256
    cam2 = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w2, h2)
    film2 = torch.zeros((w2 * h2, 4), dtype=torch.float32, device="cuda")
    for i in range(64):
        sc.vcm_iteration(cam2, vcm_params(arrays, 10, vcm_radius(R, 1.0, i, 0.75), 1000 + i, 5000 + i, i,
                                          spot_angle=20.0), film2, stream=cs)
    sc.sync(cs)
    rmse = reference_rmse(torch, ctx, film2, "vcm_torus_256_fp64_ref.npy")
    out = {"workload": "VCM: dielectric torus (200k triangles, IOR 1.5) on a diffuse plane, spot light L = 100 "
                       "with a 20 degree cone, 1024x1024, 1M light subpaths per iteration, max depth 10, radius "
                       "0.01 x scene radius, alpha 0.75, 64 iterations",
           "ms_per_iteration": ms, "msamples_per_s": w * h / (ms * 1e-3) / 1e6,
           "light_plus_eye_paths_per_s": 2 * w * h / (ms * 1e-3),
           "mean_radiance": float(film[:, :3].mean()), "iterations_timed": iters,
           "rmse_vs_fp64": {"value": rmse, "render": "64 iterations at 256x256 (same seeds and radii)",
                            "reference": "FP64 CPU oracle, 2048 iterations at 256x256 "
                                         "(tests/golden/vcm_torus_256_fp64_ref.npy)"}}
    sc.close()
    if cpu_leg:
        out["cpu_baseline"] = cpu_integrator_rate("vcm", arrays, 256, 256, 8, 10, spot_angle=20.0)
    return out


def sppm_secondary(torch, ctx_cls, scene_cls, local, cpu_leg=False, frames=64):
    """SPPM on the Cornell box (256^2, max depth 6, base radius 0.03 as the shipped cornell_box_sppm.json):
    device time per lgb_sppm_iteration over `frames` frames after one warm-up frame (one eye path and one light
    path per pixel per frame)."""
    from lumen_gb300 import procedural
    from lumen_gb300.scene import camera_lookat, sppm_params
    cb = procedural.cornell_box()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, cb)
    sc.build()
    w = h = 256
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream
    sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 77, 0), film, stream=cs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for f in range(1, frames + 1):
        sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 77, f), film, stream=cs)
    e1.record(stream)
    e1.synchronize()
    sc.sync(cs)
    ms = e0.elapsed_time(e1) / frames
    out = {"workload": "SPPM: Cornell box 36 triangles, 256x256, max depth 6, base radius 0.03, one eye and one "
                       "light path per pixel per frame", "ms_per_frame": ms,
           "msamples_per_s": w * h / (ms * 1e-3) / 1e6, "frames_timed": frames,
           "mean_radiance": float(film[:, :3].mean())}
    sc.close()
    if cpu_leg:
        out["cpu_baseline"] = cpu_integrator_rate("sppm", cb, w, h, 16, 6, base_radius=0.03)
    return out


def bdpt_secondary(torch, ctx_cls, scene_cls, local, cpu_leg=False, frames=64):
    """BDPT on the Cornell box (256^2, path length 6 as the shipped cornell_box_bdpt.json): device time per
    lgb_bdpt_iteration over `frames` frames after one warm-up frame (per pixel one light and one camera subpath of
    up to 7 vertices and 26 connection strategies)."""
    from lumen_gb300 import procedural
    from lumen_gb300.scene import bdpt_params, camera_lookat
    cb = procedural.cornell_box()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, cb)
    sc.build()
    w = h = 256
    depth = 6
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream
    sc.bdpt_iteration(cam, bdpt_params(cb, depth, 53, 0), film, stream=cs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for f in range(1, frames + 1):
        sc.bdpt_iteration(cam, bdpt_params(cb, depth, 53, f), film, stream=cs)
    e1.record(stream)
    e1.synchronize()
    sc.sync(cs)
    ms = e0.elapsed_time(e1) / frames
    strategies = (depth - 1) + depth * (depth + 1) // 2
    out = {"workload": "BDPT: Cornell box 36 triangles, 256x256, path length 6, one light and one camera subpath "
                       "per pixel per frame, 26 connection strategies per pixel", "ms_per_frame": ms,
           "msamples_per_s": w * h / (ms * 1e-3) / 1e6,
           "strategies_per_s": w * h * strategies / (ms * 1e-3), "frames_timed": frames,
           "mean_radiance": float(film[:, :3].mean())}
    sc.close()
    if cpu_leg:
        out["cpu_baseline"] = cpu_integrator_rate("bdpt", cb, w, h, 16, depth)
    return out


def restir_secondary(torch, ctx_cls, scene_cls, local, cpu_leg=False, frames=64):
    """ReSTIR DI on the Cornell box (256^2: 2 light candidates per pixel, temporal and 5-neighbour spatial reuse,
    with the spatial sample count fixed): device time per lgb_restir_di_iteration over `frames` frames after one
    warm-up frame."""
    from lumen_gb300 import abi, procedural
    from lumen_gb300.scene import camera_lookat, restir_params
    cb = procedural.cornell_box()
    ctx = ctx_cls(local)
    sc = scene_cls(ctx, cb)
    sc.build()
    w = h = 256
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    cs = stream.cuda_stream
    fix = abi.RESTIR_SPATIAL_COUNT_FIX
    sc.restir_di_iteration(cam, restir_params(cb, 91, 0, 0, flags=fix), film, stream=cs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for f in range(1, frames + 1):
        sc.restir_di_iteration(cam, restir_params(cb, 91, f, 1, flags=fix), film, stream=cs)
    e1.record(stream)
    e1.synchronize()
    sc.sync(cs)
    ms = e0.elapsed_time(e1) / frames
    out = {"workload": "ReSTIR DI: Cornell box 36 triangles, 256x256, light candidates min(light triangles, 32) = 2, "
                       "temporal + 5-neighbour spatial reuse, spatial sample count fixed", "ms_per_frame": ms,
           "msamples_per_s": w * h / (ms * 1e-3) / 1e6, "frames_timed": frames,
           "mean_radiance": float(film[:, :3].mean())}
    sc.close()
    if cpu_leg:
        out["cpu_baseline"] = cpu_integrator_rate("restir_di", cb, w, h, 64, 6, flags=fix)
    return out


def replica_throughput(step_ms, e2e_ms, units_per_rank, world, device="cuda"):
    """Replicas only: every rank processes its own copy of the workload; the job's step time is the maximum
    over ranks (all_reduce MAX on `device`: NCCL on GPUs, gloo on CPU), and the whole-job throughput is
    world * units_per_rank per step. Returns (step_ms, e2e_ms, value, e2e) with value and e2e in M units/s."""
    import torch
    if world > 1:
        t = torch.tensor([step_ms, e2e_ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms, e2e_ms = t.tolist()
    value = world * units_per_rank / (step_ms * 1e-3) / 1e6
    e2e = world * units_per_rank / (e2e_ms * 1e-3) / 1e6
    return step_ms, e2e_ms, value, e2e


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    arrays, rays = make_workload()
    vals, threads = cpu_oracle_steps(arrays, rays, args.steps, args.warmup)
    sample = CPU_WINDOW
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sample / (value * 1e6) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rays_per_step": sample,
                   "sample": f"one window of {sample} contiguous rays of the 4M incoherent set per step"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} rays per step of the 4M incoherent set"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference path (Lumen runs only through Vulkan ray tracing, "
                "unavailable on this box); binary SAH BVH, watertight FP32 test",
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from lumen_gb300 import abi
    from lumen_gb300.scene import Context, GpuScene
    arrays, rays = make_workload()
    ctx = Context(local)
    sc = GpuScene(ctx, arrays)
    stats = sc.build()
    n = len(rays)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    # bytes/ray accounting from the counting variant (untimed)
    counters = torch.zeros(2, dtype=torch.int64, device="cuda")
    sc.trace_closest_counted(d_rays, d_hits, counters, stream=sptr)
    sc.sync(sptr)
    n_nodes, n_tris = (counters.cpu().numpy() / n).tolist()
    bytes_per_ray = 32 + 16 + 80 * n_nodes + 48 * n_tris

    for _ in range(args.warmup):
        flush.fill_(1.0)
        sc.trace_closest(d_rays, d_hits, stream=sptr)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for s, e in ev:
        flush.fill_(1.0)
        s.record(stream)
        sc.trace_closest(d_rays, d_hits, stream=sptr)
        e.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    ms = [s.elapsed_time(e) for s, e in ev]
    # end-to-end through the C ABI with host buffers: lgb_trace_closest_host reads the pinned host rays and writes
    # the hits to pinned host memory from the trace kernel itself, all inside the timed region
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((n, 4), dtype=torch.int32).pin_memory()
    e2e_ms = []
    for step in range(args.warmup + args.steps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(1.0)
        h_hits.fill_(0)
        s.record(stream)
        sc.trace_closest_host(h_rays, h_hits, stream=sptr)
        e.record(stream)
        e.synchronize()
        if step >= args.warmup:
            e2e_ms.append(s.elapsed_time(e))
    e2e_check = np.array_equal(h_hits.numpy(), d_hits.cpu().numpy())
    clk = clocks.stop()
    sc.sync(sptr)
    step_ms, e2e_step, value, e2e = replica_throughput(float(np.mean(ms)), float(np.mean(e2e_ms)), n, world)
    if rank != 0:
        return
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            hbm_peak = float(json.load(f).get("hbm_gbs", hbm_peak))
        peak_src = "measured"
    l2_peak = measure_l2_peak(local)
    achieved = bytes_per_ray * n / (step_ms * 1e-3) / 1e9
    prof = measured_traffic(n)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        vals, threads = cpu_oracle_steps(arrays, rays, 20, 3)
        cpu = {"value": float(np.median(vals)), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": f"median of 20 windows of {CPU_WINDOW} contiguous rays of the 4M incoherent set (3 warm-up), "
                         "oracle binary SAH BVH, build untimed; the same method as --impl reference"}
    secondary = {}
    if not args.no_secondary:
        secondary["traversal"] = traversal_secondary(torch, sc, rays, flush, stream)
        secondary["path_tracer"] = cornell_secondary(torch, Context, GpuScene, local, world == 1 and not args.no_cpu_baseline)
        secondary["adjoint"] = adjoint_secondary(torch, Context, GpuScene, local)
        secondary["batched"] = batch_secondary(torch, Context, GpuScene, local)
        cpu_legs = world == 1 and not args.no_cpu_baseline
        secondary["vcm"] = vcm_secondary(torch, Context, GpuScene, local, cpu_legs)
        secondary["sppm"] = sppm_secondary(torch, Context, GpuScene, local, cpu_legs)
        secondary["restir_di"] = restir_secondary(torch, Context, GpuScene, local, cpu_legs)
        secondary["bdpt"] = bdpt_secondary(torch, Context, GpuScene, local, cpu_legs)
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rays_per_step": n, "triangles": stats.num_tris,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed with a 256 MB write before every step", "bvh_nodes": stats.num_nodes,
                   "bvh_depth": stats.max_depth, "bvh_build_ms": stats.build_ms, "sah_cost": stats.sah_cost,
                   "wall_s_timed_region": wall},
        "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": int(rays.nbytes),
                "d2h_bytes_per_step": int(n * 16), "api": "lgb_trace_closest_host (pinned host buffers: the trace "
                "kernel loads the rays from and stores the hits to host memory over NVLink-C2C)", "hits_equal_device_query": bool(e2e_check)},
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                     "frac": achieved / l2_peak, "traffic": prof["dram_bytes"],
                     "peak_source": "measured in this run: lgb_measure_l2_read_gbs, a 32 MB L2-resident buffer "
                                    "read by every SM",
                     "bytes_per_ray": bytes_per_ray, "nodes_per_ray": n_nodes, "tris_per_ray": n_tris,
                     "l2_bytes_measured": prof["l2_bytes"], "l2_bytes_per_ray_measured": prof["l2_bytes_per_ray"],
                     "dram_bytes_per_ray_measured": prof["dram_bytes_per_ray"], "traffic_source": prof["source"],
                     "hbm_peak": hbm_peak, "hbm_peak_source": peak_src, "frac_of_hbm_peak": achieved / hbm_peak,
                     "note": "achieved counts ray + hit + 80 B per node and 48 B per triangle fetched (algorithmic "
                             "bytes); the node and triangle working set is L2-resident, so the L2 read peak bounds "
                             "the kernel; traffic is the DRAM bytes of one ncu capture of this kernel version"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": args.steps,
        "secondary": secondary,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


LEGS = ("path_tracer", "adjoint", "batched", "vcm", "sppm", "restir_di", "bdpt")


def run_leg(name):
    import torch
    from lumen_gb300.scene import Context, GpuScene
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if name == "path_tracer":
        out = cornell_secondary(torch, Context, GpuScene, local, False)
    elif name == "adjoint":
        out = adjoint_secondary(torch, Context, GpuScene, local)
    elif name == "batched":
        out = batch_secondary(torch, Context, GpuScene, local)
    elif name == "sppm":
        out = sppm_secondary(torch, Context, GpuScene, local)
    elif name == "restir_di":
        out = restir_secondary(torch, Context, GpuScene, local)
    elif name == "bdpt":
        out = bdpt_secondary(torch, Context, GpuScene, local)
    else:
        out = vcm_secondary(torch, Context, GpuScene, local)
    print(json.dumps({"leg": name, **out}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the secondary measurements (other traversal figures, path tracer, adjoint, batched, VCM)")
    ap.add_argument("--leg", choices=sorted(LEGS),
                    help="run one secondary measurement alone and print its JSON (for profiling that workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.leg:
        run_leg(args.leg)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Headline benchmark: closest-hit Mrays/s on the LBVH microbenchmark.

Workload (one GPU): icosphere subdivided 8 times (1,310,720 triangles)
displaced by 3-octave value noise; 4,194,304 coherent primary rays (one per
pixel centre of a 2048x2048 pinhole camera) plus 4,194,304 incoherent rays
(area-weighted surface points, cosine directions). A step is one
closest-hit traversal of all 8,388,608 rays (runCollisionSystem, through
wpbr_collide_device on resident buffers). Inputs (268 MB of rays) exceed the
129 MB L2, so no flush is needed between steps.

Also reported: `e2e` through wpbr_collide with pinned host buffers
(host->device rays and device->host hits inside the timed region), the GPU
LBVH build rate, the any-hit rate, the roofline of the traversal kernel and
the oracle's CPU baseline (the reference's prune-free traversal restated in
C++, all host threads, bounded sample).

Every other reported rate carries a roofline of its own from the byte
models below (`roofline` beside each render and build entry).

`--impl reference` times that CPU implementation alone (the reference cannot
be built here: its ECS, math and allocator libraries are not vendored) on all
8,388,608 rays of the same set in the same order, with inputs from the oracle
library's own copy of the scene generator (the product library is not
loaded).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RES = 2048
LEVEL = 8
METRIC = "Mrays/s closest-hit"
WORKLOAD = "LBVH microbench: icosphere L8 (1,310,720 tris, 3-octave noise), 4M coherent + 4M incoherent rays"

# Algorithmic bytes of one sample of the direct-lighting pass (RGB): camera
# sample 44, primary hit 40, surface interaction 140, light sample 52, shadow
# ray 32, BSDF eval 104, MIS 56, BSDF sample 112, shadow ray 32, MIS 56, film
# splat 16 px x 16 B = 256; an environment light adds its Li lookup (96) for
# 1,020 B, a sphere light needs none (964 B). Traversal fetches come on top:
# 32 B per box test and 36 B per primitive test of the camera ray and the
# shadow rays. The 64-bin spectral pass moves the same per-sample data except
# the film: its splat touches 16 pixels of 64 bins + weight (16 x 260 B =
# 4,160 B instead of 256 B); its other spectra are made from RGB inputs in
# registers and never stored.
SAMPLE_BYTES_SPHERE = 964.0
SAMPLE_BYTES_ENV = 1020.0
SAMPLE_BYTES_SAMPLED64 = SAMPLE_BYTES_ENV - 256.0 + 16 * (64 * 4 + 4)
# LBVH build per primitive: bounds and Morton codes 56 B (3 indices + 3
# vertices in, 8 B out), radix sort 64 B (16 B per pass, 4 passes), emit and
# refit 120 B (codes 12, node 12, leaf bounds 24, child bounds 48, write 24).
BUILD_BYTES_PER_PRIM = 56.0 + 64.0 + 120.0
# kernels of one fused sample pass: camera traversal, spawn, shadow traversal,
# finish, film; films of 2^17 pixels and more add the two kernels that order
# the pixels by material category
SORT_MIN_PIXELS = 1 << 17


def pass_launches(pixels):
    return 5 + (2 if pixels >= SORT_MIN_PIXELS else 0)


STAGES = ["CAMERA_RAYS", "COLLIDE_PRIMARY", "EMITTED_LIGHT", "BSDF_SETUP", "SAMPLE_LIGHT", "SHADOW_LIGHT",
          "BSDF_COMPUTE", "INTEGRATE_LIGHT", "SAMPLE_BSDF", "SHADOW_BSDF", "LIGHT_COMPUTE", "INTEGRATE_BSDF"]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-render", action="store_true")
    p.add_argument("--profile", action="store_true",
                   help="small case for ncu: 1,310,720 triangles, 1024x1024 + 1M incoherent rays, 5 launches")
    p.add_argument("--profile-render", action="store_true",
                   help="small render cases for ncu: full frame 640x360 x 2 spp, adjoint 256x256 x 2 spp "
                        "forward + backward, 8 batched scenes x 2 spp")
    p.add_argument("--profile-spectral", type=int, nargs=2, metavar=("W", "H"),
                   help="Sampled64 case for ncu: config 2 (level 8) at W x H, one 2-spp frame")
    p.add_argument("--profile-build", action="store_true",
                   help="LBVH build case for ncu: 8 builds of the 1,310,720-triangle mesh (3 warm-up, 5 timed)")
    p.add_argument("--profile-collide", action="store_true",
                   help="collide case for ncu: one build of the microbenchmark mesh (38 launches), then three "
                        "closest-hit collides of all 8,388,608 rays on resident buffers (13 launches each)")
    p.add_argument("--profile-frame", action="store_true",
                   help="render case for ncu: config 2 (level 8) at 1920x1080, two 8-spp frames")
    return p.parse_args()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_ray():
    """DRAM bytes per ray of the traversal kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "trace_c1_traffic.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("dram_bytes_per_ray")
    return None


def ncu_l2():
    """L2 throughput and L1/L2 hit rates of the traversal kernel from the
    committed ncu summary (the kernel's working set is L2-resident)."""
    path = os.path.join(ROOT, "profiles", "trace_c1_traffic.json")
    if os.path.exists(path):
        return json.load(open(path)).get("l2")
    return None


def roofline(nbytes, seconds, model, what):
    """Roofline entry of a rate: algorithmic bytes over the measured time,
    against the measured HBM copy bandwidth."""
    peak, kind = measured_peaks()
    achieved = nbytes / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": kind, "bytes_model": model, "timed": what}


def pass_traversal_terms(W, ctx, res, spp, shadow_any):
    """Traversal bytes per sample of a direct-lighting pass: the staged jobs
    of pass 0 run over the whole film, and the camera rays and the shadow rays
    they trace (light branch o = p + 0.1 wi, BSDF branch o = p + 0.01 wi) are
    counted by wpbr_collide_stats over the reference's leaves (a subsample of
    at most 2^18 rays per kind): 32 B per box test + 36 B per primitive test,
    times the rays of that kind per sample."""
    import numpy as np

    Wd, Hd = res
    n = Wd * Hd
    ctx.render_setup(spp, seed=0)
    for s in STAGES:
        ctx.job(s, 0)
    rec = ctx.record(0, 0, Wd, Hd, fields=["ray_o", "ray_d", "si_p", "l_wi", "l_flags", "b_wi", "b_flags"])

    def rays_of(o, d):
        r = np.zeros((len(o), 8), np.float32)
        r[:, :3] = o
        r[:, 4:7] = d
        r[:, 7] = np.inf
        return r

    untouched = np.uint32(0xFFFFFFFF)
    lm = (rec["l_flags"] != untouched) & ((rec["l_flags"] & 1) != 0)
    bm = (rec["b_flags"] != untouched) & ((rec["b_flags"] & 2) != 0)
    kinds = [("camera", rays_of(rec["ray_o"], rec["ray_d"]), W.TRACE_CLOSEST),
             ("light_shadow", rays_of(rec["si_p"][lm] + np.float32(0.1) * rec["l_wi"][lm], rec["l_wi"][lm]),
              W.TRACE_ANY if shadow_any else W.TRACE_CLOSEST),
             ("bsdf_shadow", rays_of(rec["si_p"][bm] + np.float32(0.01) * rec["b_wi"][bm], rec["b_wi"][bm]),
              W.TRACE_ANY if shadow_any else W.TRACE_CLOSEST)]
    total, out = 0.0, {}
    for name, rays, mode in kinds:
        if len(rays) == 0:
            continue
        sub = rays[:: max(1, len(rays) // 262144)]
        _, st = ctx.collide(sub, mode=mode, stats=True)
        V, P = float(st[:, 0].mean()), float(st[:, 1].mean())
        per_sample = len(rays) / n
        total += per_sample * (32.0 * V + 36.0 * P)
        out[name] = {"rays_per_sample": per_sample, "box_tests": V, "prim_tests": P}
    ctx.check_device_errors()
    return total, out


def cpu_trace_rate(desc, rays, seconds, threads=None):
    """Oracle (the reference's prune-free candidate traversal) on host cores."""
    import numpy as np
    from oracle import binding as O

    L = O.lib()
    if threads:
        L.orc_set_threads(threads)
    cores = L.orc_num_threads()
    o = O.OracleScene(desc)
    n = rays.shape[0]
    probe = rays[np.linspace(0, n - 1, 50000).astype(np.int64)]
    t = time.perf_counter()
    o.trace(probe, mode=0)
    rate = probe.shape[0] / max(time.perf_counter() - t, 1e-6)
    # a contiguous slice of each half (coherent, incoherent) sized for ~`seconds`
    m = int(min(n, max(20000, rate * seconds))) // 2
    sample = np.concatenate([rays[: m], rays[n // 2: n // 2 + m]])
    t = time.perf_counter()
    o.trace(sample, mode=0)
    dt = time.perf_counter() - t
    return dict(value=2 * m / dt / 1e6, unit="Mrays/s", cores=cores, kind="port",
                sample="%d rays (the first %d coherent and first %d incoherent of the set), prune-free "
                       "candidate traversal + min-t reduce as in JobProcessRayCasts/Results, %.1f s"
                       % (2 * m, m, m, dt)), o


def render_rate(W, torch, config, res, spp, level=0, frames=1, spectrum=None, profile=None):
    """Msamples/s of whole frames through the fused, graph-captured pass
    (config 0: 64 spheres + quad + sphere light; config 2: the 1.31 M-triangle
    mesh + 256 spheres + 1024x512 environment light; config 5: config 0 with
    textured metal). spectrum=W.SPECTRUM_SAMPLED64 times the 64-bin pass.
    The roofline divides the per-sample byte model (static part by light
    kind and spectral representation, plus the traversal terms of the
    frame's own rays) by the frame time."""
    g = W.SceneGen(config, 0, res, level=level)
    d = g.desc.contents
    env = bool(d.envmap)
    env_only = env and all(d.lights[i].type == W.LIGHT_ENV for i in range(d.n_lights))
    ctx = W.Context(torch.cuda.current_device())
    stream = torch.cuda.Stream()  # a capturable (non-default) stream for the pass graph
    ctx.set_stream(stream.cuda_stream)
    if spectrum is not None:
        ctx.set_spectrum(spectrum)
    ctx.upload(g.desc)
    ctx.build()
    ctx.render_setup(spp, seed=0)
    ctx.render()  # warm-up frame (captures the pass graph)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(frames):
        ctx.render_setup(spp, seed=0)
        ctx.render()
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.check_device_errors()
    ms = e0.elapsed_time(e1) / frames
    samples = res[0] * res[1] * spp
    # byte model: static part + traversal terms of pass 0's rays (staged jobs, RGB)
    ctx.set_spectrum(W.SPECTRUM_RGB)
    trav, terms = pass_traversal_terms(W, ctx, res, spp, env_only)
    ctx.close()
    static = SAMPLE_BYTES_SAMPLED64 if spectrum == W.SPECTRUM_SAMPLED64 else (
        SAMPLE_BYTES_ENV if env else SAMPLE_BYTES_SPHERE)
    per_sample = static + trav
    out = {"msamples_per_s": samples / ms / 1e3, "ms_per_frame": ms, "film": "%dx%d" % res, "spp": spp,
           "kernel_launches_per_pass": pass_launches(res[0] * res[1]),
           "roofline": roofline(per_sample * samples, ms / 1e3,
                                "%.0f B/sample static + %.0f B/sample traversal (32 B per box test, 36 B per "
                                "primitive test of the camera and shadow rays)%s"
                                % (static, trav, "; texture fetches not counted" if d.n_textures else ""),
                                "whole frame, CUDA events on the pass stream"),
           "traversal_terms": terms}
    if profile:
        out["roofline"]["profile"] = profile
    return out


def cpu_render_rate(W, config, res, spp, spectral=False, level=0, min_seconds=1.0):
    """The oracle's render (the per-sample job list restated on the CPU, all
    host threads) of the same scene and film: whole passes (pass 0, 1, ...
    of an spp-pass frame) until about min_seconds have passed, Msamples/s
    beside the GPU's. Scene generation and the oracle's BVH build are not
    timed."""
    from oracle import binding as O

    g = O.SceneGen(config, 0, res, level=level)
    o = O.OracleScene(g.desc)  # builds the oracle's BVH
    passes = 0
    t = time.perf_counter()
    while True:
        if spectral:
            o.render_spectral(res[0], res[1], 1)
        else:
            o.render_passes(res[0], res[1], spp, [passes % spp])
        passes += 1
        dt = time.perf_counter() - t
        if dt > min_seconds:
            break
    return {"value": res[0] * res[1] * passes / dt / 1e6, "unit": "Msamples/s", "cores": O.lib().orc_num_threads(),
            "kind": "port",
            "sample": "%dx%d film, %d whole pass%s%s, %.2f s" % (res[0], res[1], passes, "es" if passes > 1 else "",
                                                                 " (Sampled64)" if spectral else "", dt)}


def cpu_batch_rate(n_scenes=32, film_scale=1024, max_count=2000000):
    """The oracle's render of pass 0 of every scene of the batched set, one
    scene after another on all host threads (oracle BVH builds not timed)."""
    from oracle import binding as O

    samples, dt = 0, 0.0
    for k in range(n_scenes):
        g = O.SceneGen(3, seed=3, res=(film_scale, max_count), level=k)
        cam = g.desc.contents.camera
        o = O.OracleScene(g.desc)
        t = time.perf_counter()
        o.render_passes(cam.res_x, cam.res_y, 16, [0], 0, k)
        dt += time.perf_counter() - t
        samples += cam.res_x * cam.res_y
        o.close()
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": O.lib().orc_num_threads(), "kind": "port",
            "sample": "pass 0 of all %d scenes (%d samples), %.2f s" % (n_scenes, samples, dt)}


def batch_rate(W, torch, n_scenes=32, spp=16, film_scale=1024, max_count=2000000):
    """Aggregate Msamples/s of the batched-scenes set (32 scenes, triangle
    counts log-uniform on [10k, 2M], films from {256..1024}^2, 16 spp): all
    scenes through one wpbr_batch (pooled arena, one graph launch per pass,
    autotuned traversal queue depth) against the same scenes rendered one
    at a time through wpbr_ctx on the same stream."""
    gens = [W.SceneGen(3, seed=3, res=(film_scale, max_count), level=k) for k in range(n_scenes)]
    stream = torch.cuda.Stream()
    dev = torch.cuda.current_device()
    pixels = sum(g.desc.contents.camera.res_x * g.desc.contents.camera.res_y for g in gens)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    b = W.Batch(dev)
    b.set_stream(stream.cuda_stream)
    for g in gens:
        b.add(g.desc)
    t = time.perf_counter()
    b.build()
    build_s = time.perf_counter() - t
    b.render_setup(spp, seed=0)
    info = b.autotune(use_cache=True)
    b.render()  # warm-up frame
    b.render_setup(spp, seed=0)  # clear the films (and recapture) before the timed frame
    b.synchronize()
    e0.record(stream)
    b.render()
    e1.record(stream)
    torch.cuda.synchronize()
    b.check_device_errors()
    ms_batch = e0.elapsed_time(e1)
    L0, w0 = b.film(0)
    b.close()

    ctxs = []
    for g in gens:
        c = W.Context(dev)
        c.set_stream(stream.cuda_stream)
        c.upload(g.desc)
        c.build()
        c.render_setup(spp, seed=0)
        c.render()  # warm-up frame (captures the scene's pass graph)
        ctxs.append(c)
    torch.cuda.synchronize()
    e0.record(stream)
    for c in ctxs:
        c.render_setup(spp, seed=0)
        c.render()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1)
    cam = gens[0].desc.contents.camera
    L1, w1 = ctxs[0].film(cam.res_x, cam.res_y)
    for c in ctxs:
        c.check_device_errors()
        c.close()
    same = bool((L0.view("u4") == L1.view("u4")).all() and (w0 == w1).all())
    samples = pixels * spp
    model = ("%.0f B/sample (the static per-sample bytes with an environment light); traversal terms not "
             "counted, so the fraction is a lower bound" % SAMPLE_BYTES_ENV)
    return {"roofline": roofline(SAMPLE_BYTES_ENV * samples, ms_batch / 1e3, model,
                                 "one batched frame (all scenes), CUDA events on the batch stream"),
            "roofline_sequential": roofline(SAMPLE_BYTES_ENV * samples, ms_seq / 1e3, model,
                                            "the same scenes one at a time"),
            "scenes": n_scenes, "spp": spp, "total_pixels": pixels, "total_prims": info["total_prims"],
            "arena_bytes": info["arena_bytes"], "rays_per_block": info["rays_per_block"],
            "autotune_source": ["default", "measured", "cache", "caller"][info["autotune_source"]],
            "msamples_per_s_batched": samples / ms_batch / 1e3, "ms_per_frame_batched": ms_batch,
            "msamples_per_s_sequential": samples / ms_seq / 1e3, "ms_per_frame_sequential": ms_seq,
            "speedup": ms_seq / ms_batch, "build_ms_all_scenes": build_s * 1e3,
            "scene0_film_identical": same,
            "graph_launches_per_frame": spp,
            "kernel_launches_per_frame": spp * sum(pass_launches(g.desc.contents.camera.res_x *
                                                                g.desc.contents.camera.res_y) for g in gens)}


def _c4_params(desc):
    import numpy as np

    d = desc.contents
    mats = [d.materials[i] for i in range(d.n_materials)]
    mat = np.array([[m.alpha_x, *m.R, *m.eta_t, *m.k] for m in mats], np.float32).reshape(-1)
    e = d.envmap.contents
    env = np.ctypeslib.as_array(e.rgb, shape=(e.width * e.height * 3,)).astype(np.float32)
    return mat, env


def adjoint_rate(W, torch, res=(512, 512), spp=16, n_fd=64, n_fp64=64, fp64=True):
    """Differentiable estimator on the config-4 scene (512x512, 16 spp, 64
    materials x 10 parameters + a 256x128 RGB environment = 98,944
    parameters): forward + backward time, gradient parameters/s, the rate of
    central differences (h = 1e-3) through the same forward, their agreement,
    and on the 64 parameters of those differences the FP64 oracle's
    dual-number gradient and FP64 central differences (h = 1e-3) of the same
    frozen estimator. Roofline: the forward pass's per-sample bytes (static
    part + the traversal terms of its rays), the backward pass twice that."""
    import numpy as np

    g0 = W.SceneGen(4, 0, res, level=0)
    g1 = W.SceneGen(4, 0, res, level=1)
    dev = torch.cuda.current_device()
    stream = torch.cuda.Stream()
    ctx = W.Context(dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(g0.desc)
    ctx.build()
    nm, ne = ctx.adjoint_setup(spp, seed=0, stream=0)
    m0, e0 = _c4_params(g0.desc)
    mh, eh = _c4_params(g1.desc)
    ctx.adjoint_set_params(mh, eh)
    ctx.adjoint_freeze()
    target, _ = ctx.adjoint_forward(*res)
    ctx.adjoint_set_params(m0, e0)
    ctx.adjoint_freeze()
    n = res[0] * res[1]
    with torch.cuda.stream(stream):
        d_target = torch.from_numpy(target.reshape(-1).copy()).to("cuda")
        d_gm = torch.zeros(nm, device="cuda")
        d_ge = torch.zeros(ne, device="cuda")
    torch.cuda.synchronize()
    e0_ = torch.cuda.Event(enable_timing=True)
    e1_ = torch.cuda.Event(enable_timing=True)
    e2_ = torch.cuda.Event(enable_timing=True)
    for _ in range(2):  # warm-up
        ctx.adjoint_forward_device(d_target.data_ptr())
        ctx.adjoint_backward_device(d_gm.data_ptr(), d_ge.data_ptr())
    reps = 3
    fwd_ms = bwd_ms = 0.0
    for _ in range(reps):
        e0_.record(stream)
        loss = ctx.adjoint_forward_device(d_target.data_ptr())
        e1_.record(stream)
        ctx.adjoint_backward_device(d_gm.data_ptr(), d_ge.data_ptr())
        e2_.record(stream)
        torch.cuda.synchronize()
        fwd_ms += e0_.elapsed_time(e1_) / reps
        bwd_ms += e1_.elapsed_time(e2_) / reps
    grad = np.concatenate([d_gm.cpu().numpy(), d_ge.cpu().numpy()])
    # end to end through the host-buffer entry points
    t = time.perf_counter()
    img, _ = ctx.adjoint_forward(*res, target)
    gm_h, ge_h = ctx.adjoint_backward()
    e2e_s = time.perf_counter() - t
    # central differences through the same forward
    rng = np.random.default_rng(4)
    sel = np.concatenate([rng.choice(nm, n_fd // 2, replace=False),
                          nm + rng.choice(np.nonzero(grad[nm:])[0], n_fd // 2, replace=False)])
    h = 1e-3
    fd = np.zeros(n_fd)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for k, i in enumerate(sel):
        vals = []
        for s in (+1, -1):
            m, e = m0.copy(), e0.copy()
            if i < nm:
                m[i] += s * h
            else:
                e[i - nm] += s * h
            ctx.adjoint_set_params(m, e)
            vals.append(ctx.adjoint_forward_device(d_target.data_ptr()))
        fd[k] = (vals[0] - vals[1]) / (2 * h)
    fd_s = time.perf_counter() - t
    ctx.adjoint_set_params(m0, e0)
    ctx.check_device_errors()
    trav, terms = pass_traversal_terms(W, ctx, res, spp, False)
    ctx.close()
    g_sel = grad[sel]
    fwd_bytes = (SAMPLE_BYTES_ENV + trav) * n * spp
    out = {"film": "%dx%d" % res, "spp": spp, "params": int(nm + ne), "loss": loss,
           "forward_ms": fwd_ms, "backward_ms": bwd_ms,
           "gradient_params_per_s": (nm + ne) / ((fwd_ms + bwd_ms) / 1e3),
           "fd_params_per_s": n_fd / fd_s, "fd_h": h,
           "speedup_vs_fd": ((nm + ne) / ((fwd_ms + bwd_ms) / 1e3)) / (n_fd / fd_s),
           "rel_err_vs_fd32_norm": float(np.linalg.norm(g_sel - fd) / np.linalg.norm(fd)),
           "e2e_forward_backward_s": e2e_s, "msamples_per_s_forward": n * spp / fwd_ms / 1e3,
           "kernel_launches": {"forward_per_pass": 5, "backward_per_pass": 4},
           "roofline": roofline(3 * fwd_bytes, (fwd_ms + bwd_ms) / 1e3,
                                "forward %.0f B/sample (%.0f static + %.0f traversal), backward twice the "
                                "forward bytes" % (SAMPLE_BYTES_ENV + trav, SAMPLE_BYTES_ENV, trav),
                                "forward + backward, CUDA events on the context stream"),
           "roofline_forward": roofline(fwd_bytes, fwd_ms / 1e3, "forward bytes as above", "forward only"),
           "traversal_terms": terms}
    if fp64:
        from oracle import binding as O

        o = O.OracleScene(g0.desc)
        sub = np.concatenate([sel[: n_fp64 // 2], sel[n_fd // 2: n_fd // 2 + n_fp64 // 2]])
        t = time.perf_counter()
        _, _, g64 = o.adjoint_eval(res[0], res[1], spp, 0, 0, m0.astype(np.float64), e0.astype(np.float64),
                                   target, sub)
        dual_s = time.perf_counter() - t
        t = time.perf_counter()
        fd64 = o.adjoint_fd(spp, 0, 0, m0.astype(np.float64), e0.astype(np.float64), target, sub, h=h)
        fd64_s = time.perf_counter() - t
        gs = grad[sub].astype(np.float64)

        def errs(ref):
            # per parameter |g - ref| / |ref|, unfloored; and with the
            # denominator floored at 1 % of the largest |ref| of the set, which
            # keeps parameters whose gradient is near zero (a texel few
            # samples see) from dividing FP32 accumulation noise by ~0
            a = np.abs(gs - ref)
            nz = np.abs(ref) > 0
            return {"rel_err_max": float(np.max(a / np.maximum(np.abs(ref), 1e-2 * np.abs(ref).max()))),
                    "rel_err_max_unfloored": float(np.max(a[nz] / np.abs(ref[nz]))) if nz.any() else 0.0,
                    "rel_err_median_unfloored": float(np.median(a[nz] / np.abs(ref[nz]))) if nz.any() else 0.0,
                    "rel_err_norm": float(np.linalg.norm(gs - ref) / np.linalg.norm(ref))}

        out["fp64"] = dict(params=int(len(sub)), seconds=dual_s, cores=O.lib().orc_num_threads(), **errs(g64))
        out["fp64_central_differences"] = dict(params=int(len(sub)), h=h, seconds=fd64_s,
                                               cores=O.lib().orc_num_threads(), **errs(fd64))
    return out


def workload_config(n, sizes, hit_frac, world):
    """The `config` object of both arms' lines (the same workload)."""
    return {"workload": WORKLOAD, "rays_per_step": n, "triangles": sizes["n_prims"], "bvh_nodes": sizes["n_nodes"],
            "treelets": sizes["n_treelets"], "bvh_depth": sizes["max_depth"], "hit_fraction": hit_frac,
            "l2": "inputs larger than L2 (268 MB of rays), no flush",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle's prune-free
    candidate traversal + min-t reduce, JobProcessRayCasts/Results restated)
    on every host thread: each step traces all 8,388,608 rays of the set, in
    the GPU arm's order. Inputs come from the oracle library's copy of the
    scene generator; the product library is never loaded."""
    import numpy as np

    from oracle import binding as O
    from oracle.build import build_oracle

    build_oracle()
    g = O.SceneGen(1, 0, (RES, RES), level=LEVEL, rays=True)
    rays = g.rays()
    n = rays.shape[0]
    o = O.OracleScene(g.desc)
    cores = O.lib().orc_num_threads()
    times = []
    hits = None
    for s in range(args.warmup + args.steps):
        t = time.perf_counter()
        hits = o.trace(rays, mode=0)
        dt = time.perf_counter() - t
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    v = n * args.steps / tot / 1e6
    hit_frac = float(np.mean(hits[:, 1].view(np.uint32) != 0xFFFFFFFF))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; the reference publishes no dataset)",
        "config": workload_config(n, o.sizes(), hit_frac, 1),
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": "all %d rays of the set per step, in the GPU arm's order; prune-free candidate "
                                   "traversal + min-t reduce as in JobProcessRayCasts/Results" % n},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_profile_case():
    """Small case sized for an ncu capture: the full mesh, 2,097,152 rays
    (64 MB of rays + ~100 MB of BVH and triangles, above the 129 MB L2),
    2 warm-up + 3 timed closest-hit launches."""
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(1, 0, (1024, 1024), level=LEVEL, rays=True)
    rays = g.rays()
    n = rays.shape[0]
    ctx = W.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(g.desc)
    ctx.build()
    d_rays = torch.from_numpy(rays).to("cuda")
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    for _ in range(2):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.check_device_errors()
    ms = e0.elapsed_time(e1) / 3
    print(json.dumps({"profile_case": "C1 mesh, %d rays" % n, "ms_per_launch": ms,
                      "mrays_per_s": n / ms / 1e3}))
    ctx.close()


def run_render_profile_case():
    """Small render cases sized for ncu captures of the render, adjoint and
    batched kernels (each a few hundred MB on the device at most)."""
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    out = {"full_frame": render_rate(W, torch, 2, (640, 360), 2, level=LEVEL),
           "adjoint": adjoint_rate(W, torch, res=(256, 256), spp=2, n_fd=4, fp64=False),
           "batched": batch_rate(W, torch, n_scenes=8, spp=2, film_scale=512, max_count=200000)}
    print(json.dumps(out))


def run_spectral_profile_case(res):
    """One 2-spp frame of the full-frame scene in Sampled64 mode (render
    setup, two graph-captured passes, the frame's toRGB)."""
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(2, 0, tuple(res), level=LEVEL)
    ctx = W.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    ctx.upload(g.desc)
    ctx.build()
    ctx.render_setup(2, seed=0)
    ctx.render()
    torch.cuda.synchronize()
    ctx.check_device_errors()
    ctx.close()
    print(json.dumps({"profile_case": "Sampled64 config 2, %dx%d, 2 spp" % tuple(res)}))


def run_collide_profile_case():
    """One build of the microbenchmark mesh, then three closest-hit collides
    of the whole ray set through wpbr_collide_device (each: ray keys, the
    ray-order sort, the traversal)."""
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(1, 0, (RES, RES), level=LEVEL, rays=True)
    rays = g.rays()
    n = rays.shape[0]
    ctx = W.Context(0)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    ctx.upload(g.desc)
    ctx.build()
    d_rays = torch.from_numpy(rays).to("cuda")
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    for _ in range(3):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    torch.cuda.synchronize()
    ctx.check_device_errors()
    ctx.close()
    print(json.dumps({"profile_case": "closest hit, %d rays, 3 collides after one build" % n}))


def run_frame_profile_case():
    """Two 8-spp frames of the full-frame scene (config 2, level 8) at
    1920x1080 through the graph-captured RGB pass."""
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(2, 0, (1920, 1080), level=LEVEL)
    ctx = W.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(g.desc)
    ctx.build()
    for _ in range(2):
        ctx.render_setup(8, seed=0)
        ctx.render()
    torch.cuda.synchronize()
    ctx.check_device_errors()
    ctx.close()
    print(json.dumps({"profile_case": "config 2, 1920x1080, two 8-spp frames"}))


def run_build_profile_case():
    """Eight LBVH builds of the 1,310,720-triangle microbenchmark mesh (three
    warm-up builds, then five timed back to back on the context's stream)."""
    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(1, 0, (64, 64), level=LEVEL)
    ctx = W.Context(0)
    ctx.upload(g.desc)
    for _ in range(3):
        ctx.build()
    ctx.synchronize()
    t = time.perf_counter()
    for _ in range(5):
        ctx.build()
    ctx.synchronize()
    ms = (time.perf_counter() - t) / 5 * 1e3
    ctx.check_device_errors()
    info = ctx.bvh_info()
    ctx.close()
    print(json.dumps({"profile_case": "LBVH build, %d triangles" % info["n_prims"], "ms_per_build": ms,
                      "mprims_per_s": info["n_prims"] / ms / 1e3}))


def main():
    args = parse()
    if args.profile_build:
        run_build_profile_case()
        return
    if args.profile_collide:
        run_collide_profile_case()
        return
    if args.profile_frame:
        run_frame_profile_case()
        return
    if args.profile_spectral:
        run_spectral_profile_case(args.profile_spectral)
        return
    if args.profile_render:
        run_render_profile_case()
        return
    if args.profile:
        run_profile_case()
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args)
        return
    import numpy as np
    import torch

    from __graft_entry__ import build

    build()
    import woodenpbrengine_gb300 as W

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world)
    stream = torch.cuda.current_stream()
    g = W.SceneGen(1, 0, (RES, RES), level=LEVEL, rays=True)
    rays = g.rays()
    n = rays.shape[0]
    ctx = W.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(g.desc)

    # --- LBVH build rate (reported beside the headline) ---
    # wpbr_bvh_build returns once the tree is built (it reads a few sizes back
    # while it runs): wall time per build, and CUDA events on the context's
    # stream from before its first kernel to after its last
    for _ in range(2):
        ctx.build()
    torch.cuda.synchronize()
    nb = 5
    eb0 = torch.cuda.Event(enable_timing=True)
    eb1 = torch.cuda.Event(enable_timing=True)
    build_dev_ms = 0.0
    t = time.perf_counter()
    for _ in range(nb):
        eb0.record(stream)
        ctx.build()
        eb1.record(stream)
        eb1.synchronize()
        build_dev_ms += eb0.elapsed_time(eb1) / nb
    build_s = (time.perf_counter() - t) / nb
    info = ctx.bvh_info()

    # --- headline: closest-hit traversal over resident rays ---
    d_rays = torch.from_numpy(rays).to("cuda")
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1)
    ctx.check_device_errors()
    if dist:
        t_ = torch.tensor([ms], device="cuda")
        dist.all_reduce(t_, op=dist.ReduceOp.MAX)
        ms = float(t_.item())
        dist.barrier()
    ms_step = ms / args.steps
    value = world * n * args.steps / (ms / 1e3) / 1e6
    hits = d_hits.cpu().numpy()
    hit_frac = float(np.mean(hits[:, 1].view(np.uint32) != 0xFFFFFFFF))

    # the dominant kernel alone: CUDA events around each traversal launch,
    # on the context's stream (the step also runs the ray-order sort)
    ctx.set_kernel_timing(True)
    for _ in range(args.steps):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_CLOSEST)
    trav_total_ms, trav_launches = ctx.kernel_timing()
    ctx.set_kernel_timing(False)
    trav_ms = trav_total_ms / max(trav_launches, 1)

    # any-hit
    ea = torch.cuda.Event(enable_timing=True)
    eb = torch.cuda.Event(enable_timing=True)
    ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_ANY)
    ea.record(stream)
    for _ in range(5):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), W.TRACE_ANY)
    eb.record(stream)
    torch.cuda.synchronize()
    any_rate = n * 5 / (ea.elapsed_time(eb) / 1e3) / 1e6

    # byte model: 48 B/ray + 32 B per box test + 36 B per triangle test
    sample = rays[::64]
    _, st = ctx.collide(sample, stats=True)
    V = float(st[:, 0].mean())
    P = float(st[:, 1].mean())
    bytes_per_ray = 48.0 + 32.0 * V + 36.0 * P
    achieved = bytes_per_ray * n / (trav_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    tpr = ncu_traffic_per_ray()
    build_bytes = BUILD_BYTES_PER_PRIM * info["n_prims"]

    # --- e2e through the public host-buffer API (pinned) ---
    h_rays = torch.from_numpy(rays).pin_memory().numpy()
    h_hits = torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()
    import ctypes as C

    lib = W.lib()
    fp = C.POINTER(C.c_float)
    rp, hp = h_rays.ctypes.data_as(fp), h_hits.ctypes.data_as(fp)
    lib.wpbr_collide(ctx.handle, rp, n, hp, 0)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        st_ = lib.wpbr_collide(ctx.handle, rp, n, hp, 0)
        assert st_ == 0
    e2e_s = (time.perf_counter() - t) / e2e_steps
    e2e = world * n / e2e_s / 1e6

    render = None
    if rank == 0 and not args.no_render:
        prof = "profiles/render_passes_profile_case.md"
        render = {
            "c0_plain_256x256_4spp": render_rate(W, torch, 0, (256, 256), 4, frames=3, profile=prof),
            "c2_fullframe_1080p_64spp": render_rate(W, torch, 2, (1920, 1080), 64, level=LEVEL, profile=prof),
            "c2_fullframe_1080p_16spp_sampled64": render_rate(W, torch, 2, (1920, 1080), 16, level=LEVEL,
                                                              spectrum=W.SPECTRUM_SAMPLED64,
                                                              profile="profiles/sampled64_pass_c2.md"),
            "c5_textured_metal_1080p_16spp": render_rate(W, torch, 5, (1920, 1080), 16, profile=prof),
            "c3_batched_32_scenes_16spp": batch_rate(W, torch),
            "c4_adjoint_512x512_16spp": adjoint_rate(W, torch, fp64=not args.no_cpu)}
        render["c3_batched_32_scenes_16spp"]["roofline"]["profile"] = prof
        render["c4_adjoint_512x512_16spp"]["roofline"]["profile"] = prof
        if not args.no_cpu:
            # the oracle's CPU render of the same frames on the host threads, beside each GPU rate
            r = render
            r["c0_plain_256x256_4spp"]["cpu_baseline"] = cpu_render_rate(W, 0, (256, 256), 4)
            r["c0_plain_256x256_4spp"]["cpu_baseline_sampled64"] = cpu_render_rate(W, 0, (256, 256), 4,
                                                                                   spectral=True)
            r["c2_fullframe_1080p_64spp"]["cpu_baseline"] = cpu_render_rate(W, 2, (1920, 1080), 64, level=LEVEL)
            r["c2_fullframe_1080p_16spp_sampled64"]["cpu_baseline"] = cpu_render_rate(
                W, 2, (1920, 1080), 16, spectral=True, level=LEVEL)
            r["c5_textured_metal_1080p_16spp"]["cpu_baseline"] = cpu_render_rate(W, 5, (1920, 1080), 16)
            r["c3_batched_32_scenes_16spp"]["cpu_baseline"] = cpu_batch_rate()
            r["c4_adjoint_512x512_16spp"]["cpu_baseline_forward"] = cpu_render_rate(W, 4, (512, 512), 16)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, _ = cpu_trace_rate(g.desc, rays, args.cpu_seconds)
        # the same restatement on one core (a smaller contiguous sample)
        cores = cpu["cores"]
        one, _ = cpu_trace_rate(g.desc, rays, args.cpu_seconds / 4, threads=1)
        from oracle import binding as _O

        _O.lib().orc_set_threads(cores)
        cpu["single_core"] = {"value": one["value"], "unit": "Mrays/s", "sample": one["sample"]}

    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; the reference publishes no dataset)",
        "config": workload_config(n, info, hit_frac, world),
        "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 16 * n},
        "gpu_launches": args.steps * ctx.collide_launches(n),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "kernel": "k_trace_persistent (closest hit)",
                     "kernel_ms_per_launch": trav_ms, "timed_launches": trav_launches,
                     "step_frac": bytes_per_ray * n / (ms_step / 1e3) / 1e9 / peak,
                     "traffic": (tpr * n) if tpr else None,
                     # DRAM bytes actually moved (ncu, scaled by rays) over the launch time: most of the
                     # byte model's node and primitive fetches are served from L2
                     "traffic_frac": ((tpr * n) / (trav_ms / 1e3) / 1e9 / peak) if tpr else None,
                     "l2": ncu_l2(),
                     "bytes_model": "48 + 32*V + 36*P per ray, V=%.2f box tests, P=%.2f triangle tests" % (V, P)},
        "clocks": ck,
        "build": {"mprims_per_s": info["n_prims"] / build_s / 1e6, "ms": build_s * 1e3,
                  "mprims_per_s_device": info["n_prims"] / build_dev_ms / 1e3, "ms_device": build_dev_ms,
                  "timing": "ms: wall time per build (host returns after the last kernel); ms_device: CUDA events "
                            "around each build on the context's stream",
                  "roofline": roofline(build_bytes, build_dev_ms / 1e3,
                                       "240 B per primitive (bounds + Morton 56, radix sort 64, emit + refit 120)",
                                       "CUDA events around one build")},
        "anyhit_mrays_per_s": any_rate,
        "render": render,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

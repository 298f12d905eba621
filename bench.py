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

`--impl reference` times that CPU implementation alone (the reference cannot
be built here: its ECS, math and allocator libraries are not vendored).
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


def render_rate(W, torch, config, res, spp, level=0, frames=1, spectrum=None):
    """Msamples/s of whole frames through the fused, graph-captured pass
    (config 0: 64 spheres + quad + sphere light; config 2: the 1.31 M-triangle
    mesh + 256 spheres + 1024x512 environment light; config 5: config 0 with
    textured metal). spectrum=W.SPECTRUM_SAMPLED64 times the 64-bin pass."""
    g = W.SceneGen(config, 0, res, level=level)
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
    ctx.close()
    return {"msamples_per_s": samples / ms / 1e3, "ms_per_frame": ms, "film": "%dx%d" % res, "spp": spp,
            "kernel_launches_per_pass": 5}


def cpu_render_rate(W, config, res, spp, spectral=False):
    """The oracle's render (the per-sample job list restated on the CPU, all
    host cores) of the same frame: Msamples/s beside the GPU's."""
    from oracle import binding as O

    g = W.SceneGen(config, 0, res)
    o = O.OracleScene(g.desc)  # builds the oracle's BVH
    frames = 0
    t = time.perf_counter()
    while True:  # whole frames until about a second has passed
        if spectral:
            o.render_spectral(res[0], res[1], spp)
        else:
            o.render(res[0], res[1], spp)
        frames += 1
        dt = time.perf_counter() - t
        if dt > 1.0:
            break
    return {"msamples_per_s": res[0] * res[1] * spp * frames / dt / 1e6, "cores": O.lib().orc_num_threads(),
            "kind": "port", "sample": "%dx%d x %d spp, %d frames, %.2f s" % (res[0], res[1], spp, frames, dt)}


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
    return {"scenes": n_scenes, "spp": spp, "total_pixels": pixels, "total_prims": info["total_prims"],
            "arena_bytes": info["arena_bytes"], "rays_per_block": info["rays_per_block"],
            "autotune_source": ["default", "measured", "cache", "caller"][info["autotune_source"]],
            "msamples_per_s_batched": samples / ms_batch / 1e3, "ms_per_frame_batched": ms_batch,
            "msamples_per_s_sequential": samples / ms_seq / 1e3, "ms_per_frame_sequential": ms_seq,
            "speedup": ms_seq / ms_batch, "build_ms_all_scenes": build_s * 1e3,
            "scene0_film_identical": same,
            "graph_launches_per_frame": spp, "kernel_launches_per_frame": 5 * n_scenes * spp}


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
    and the FP64 oracle's dual-number gradient on a subset."""
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
    ctx.close()
    g_sel = grad[sel]
    out = {"film": "%dx%d" % res, "spp": spp, "params": int(nm + ne), "loss": loss,
           "forward_ms": fwd_ms, "backward_ms": bwd_ms,
           "gradient_params_per_s": (nm + ne) / ((fwd_ms + bwd_ms) / 1e3),
           "fd_params_per_s": n_fd / fd_s, "fd_h": h,
           "speedup_vs_fd": ((nm + ne) / ((fwd_ms + bwd_ms) / 1e3)) / (n_fd / fd_s),
           "rel_err_vs_fd32_norm": float(np.linalg.norm(g_sel - fd) / np.linalg.norm(fd)),
           "e2e_forward_backward_s": e2e_s, "msamples_per_s_forward": n * spp / fwd_ms / 1e3,
           "kernel_launches": {"forward_per_pass": 5, "backward_per_pass": 4}}
    if fp64:
        from oracle import binding as O

        o = O.OracleScene(g0.desc)
        sub = np.concatenate([sel[: n_fp64 // 2], sel[n_fd // 2: n_fd // 2 + n_fp64 // 2]])
        t = time.perf_counter()
        _, _, g64 = o.adjoint_eval(res[0], res[1], spp, 0, 0, m0.astype(np.float64), e0.astype(np.float64),
                                   target, sub)
        gs = grad[sub]
        floor = 1e-2 * np.abs(g64).max()
        out["fp64"] = {"params": int(len(sub)), "seconds": time.perf_counter() - t,
                       "rel_err_max": float(np.max(np.abs(gs - g64) / np.maximum(np.abs(g64), floor))),
                       "rel_err_norm": float(np.linalg.norm(gs - g64) / np.linalg.norm(g64)),
                       "cores": O.lib().orc_num_threads()}
    return out


def run_reference(args):
    import numpy as np
    import woodenpbrengine_gb300 as W

    g = W.SceneGen(1, 0, (RES, RES), level=LEVEL, rays=True)
    rays = g.rays()
    from oracle import binding as O

    o = O.OracleScene(g.desc)
    cores = O.lib().orc_num_threads()
    n = rays.shape[0]
    step_rays = []
    times = []
    rng = np.random.default_rng(3)
    per_step = 4000
    probe = rays[rng.choice(n, 2000, replace=False)]
    t = time.perf_counter()
    o.trace(probe, mode=0)
    rate = probe.shape[0] / max(time.perf_counter() - t, 1e-6)
    per_step = int(max(2000, rate * 2.0))
    for s in range(args.warmup + args.steps):
        sel = rng.choice(n, per_step, replace=False)
        t = time.perf_counter()
        o.trace(rays[sel], mode=0)
        dt = time.perf_counter() - t
        if s >= args.warmup:
            times.append(dt)
            step_rays.append(per_step)
    tot = sum(times)
    v = sum(step_rays) / tot / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_rays_per_step": per_step},
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": "%d random rays of the set per step, prune-free candidate traversal" % per_step},
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
        from __graft_entry__ import build

        build()
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
    for _ in range(2):
        ctx.build()
    torch.cuda.synchronize()
    t = time.perf_counter()
    nb = 5
    for _ in range(nb):
        ctx.build()
    torch.cuda.synchronize()
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
        c0 = render_rate(W, torch, 0, (256, 256), 4, frames=3)
        if not args.no_cpu:
            c0["cpu_baseline"] = cpu_render_rate(W, 0, (256, 256), 4)
            c0["cpu_baseline_sampled64"] = cpu_render_rate(W, 0, (256, 256), 4, spectral=True)
        render = {"c0_plain_256x256_4spp": c0,
                  "c2_fullframe_1080p_64spp": render_rate(W, torch, 2, (1920, 1080), 64, level=LEVEL),
                  "c2_fullframe_1080p_16spp_sampled64": render_rate(W, torch, 2, (1920, 1080), 16, level=LEVEL,
                                                                    spectrum=W.SPECTRUM_SAMPLED64),
                  "c5_textured_metal_1080p_16spp": render_rate(W, torch, 5, (1920, 1080), 16),
                  "c3_batched_32_scenes_16spp": batch_rate(W, torch),
                  "c4_adjoint_512x512_16spp": adjoint_rate(W, torch, fp64=not args.no_cpu)}

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
        "config": {"workload": WORKLOAD, "rays_per_step": n, "triangles": info["n_prims"],
                   "bvh_nodes": info["n_nodes"], "treelets": info["n_treelets"], "bvh_depth": info["max_depth"],
                   "hit_fraction": hit_frac, "l2": "inputs larger than L2 (268 MB of rays), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 16 * n},
        "gpu_launches": args.steps * ctx.collide_launches(n),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "kernel": "k_trace_persistent (closest hit)",
                     "kernel_ms_per_launch": trav_ms, "timed_launches": trav_launches,
                     "step_frac": bytes_per_ray * n / (ms_step / 1e3) / 1e9 / peak,
                     "traffic": (tpr * n) if tpr else None,
                     "bytes_model": "48 + 32*V + 36*P per ray, V=%.2f box tests, P=%.2f triangle tests" % (V, P)},
        "clocks": ck,
        "build": {"mprims_per_s": info["n_prims"] / build_s / 1e6, "ms": build_s * 1e3},
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

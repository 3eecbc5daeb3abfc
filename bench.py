#!/usr/bin/env python
"""Benchmark: Msamples/s of the GB300 wavefront path tracer at 1080p, depth 8.

Workload (default, one "step" = one full frame): the procedural studio scene,
1920x1080, 64 spp, max depth 8, min RR depth 3, thin lens (aperture radius
0.05, focus 4.0), 8 moving instances, 64 displaced spheres x 32,768 triangles
(+ ground quad), 2048x1024 procedural HDRI, alias-table environment sampling.
Seeded synthetic inputs; no datasets or external assets.

  value  = samples / device time of the timed steps (scene resident in HBM,
           film written to device buffers; CUDA events on the library's stream)
  e2e    = the same through the public C ABI with a host film: every step
           sends the camera/params and reads back the four film channels
  roofline = the extend (closest-hit) stage: algorithmic bytes per launch
           (32 B ray in + 20 B hit out per ray, plus the scene's triangle and
           node arrays once per launch) / its average launch time
  cpu_baseline = the CPU oracle (C++ restatement of the reference's CPU path)
           on a bounded row sample of the same frame, all host cores

--impl reference times that CPU restatement alone (the reference itself is
Rust and cannot be built on this image; no Rust toolchain, crates not
vendored).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s @1080p depth 8"
UNIT = "Msamples/s"
W, H, SPP, DEPTH, RR = 1920, 1080, 64, 8, 3
# CPU sample: every third image row at full spp (about 10-15 s on 16 cores)
CPU_ROWS = 360


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=0, help="rows in the CPU sample (0 = auto)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--graph", type=int, default=0, help="replay waves through a CUDA graph")
    ap.add_argument("--bvh-width", type=int, default=0, help="instance BVH width 2, 4 or 8 (0 = 2)")
    ap.add_argument("--sort", type=int, default=1,
                    help="shade queue order (sort_by_material): 1 = sorted by material within tiles of 4096 "
                         "entries (the fastest on this frame), 0 = the library default (unsorted), 2 = unsorted, "
                         "3 = the whole queue sorted")
    ap.add_argument("--wave-paths", type=int, default=0, help="paths in flight per wave (0 = library default)")
    ap.add_argument("--block", type=int, default=0, help="threads per block of the stage kernels (0 = default)")
    ap.add_argument("--refill", type=int, default=0,
                    help="traversal: idle lanes of a warp that trigger a ray refetch (0 = library default)")
    ap.add_argument("--workload", default="studio", choices=["studio", "batch", "adjoint"],
                    help="studio: the 1080p headline frame; batch: 256 Cornell-variant jobs in one batched launch")
    ap.add_argument("--jobs", type=int, default=256, help="batch workload: number of jobs")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the microbenchmark, adjoint and batch entries of the studio line")
    return ap.parse_args()


def run_adjoint(args):
    """Differentiable render: the studio at 512x512 (64 sphere materials + ground, 512x256 HDRI), L2 loss
    against a target rendered from perturbed parameters; a step = 32-spp forward + 32-spp path-replay adjoint."""
    import torch

    from pyre_gb300 import CudaIntegrator, PathIntegrator
    from pyre_gb300 import presets as P
    torch.cuda.set_device(0)
    w = h = 512
    spp = 32
    sc, tgt, cam = P.adjoint_problem(w, h)
    ctx = CudaIntegrator(0)
    ds, dt = ctx.upload(sc), ctx.upload(tgt)
    it = PathIntegrator(8, 3)
    target = ctx.render(dt, cam, it, w, h, 256, spp_begin=1 << 20).radiance.astype(np.float64)

    def step(s0):
        img = ctx.forward(ds, cam, it, w, h, spp, spp_begin=s0).radiance
        f_ms = ctx.stats().ms_total
        dl = (2.0 * (img - target) / img.size).astype(np.float32)
        gm, ge = ctx.backward(ds, cam, it, w, h, spp, dl, spp_begin=s0)
        return f_ms, ctx.stats().ms_total, float(np.mean((img - target) ** 2)), gm, ge

    for k in range(args.warmup):
        step(k * spp)
    fwd, adj = [], []
    for k in range(args.steps):
        f_ms, a_ms, _, _, _ = step((args.warmup + k) * spp)
        fwd.append(f_ms)
        adj.append(a_ms)
    # a few gradient-descent steps on materials and env texels (loss must fall)
    mats = list(sc.materials)
    env = sc.env.pixels.copy()
    losses = []
    lr_m, lr_e = 0.02, 0.5
    for k in range(6):
        _, _, l, gm, ge = step(10_000 + k * spp)
        losses.append(l)
        new = []
        for m, g in zip(mats, gm):
            from pyre_gb300.scene import DisneyBsdf, Lambertian
            gn = g / (np.abs(g).max() + 1e-12)
            if isinstance(m, DisneyBsdf):
                new.append(DisneyBsdf(np.clip(m.base_color - lr_m * gn[:3], 0, 1),
                                      float(np.clip(m.metallic - lr_m * gn[3], 0, 1)),
                                      float(np.clip(m.roughness - lr_m * gn[4], 0.05, 1)),
                                      float(np.clip(m.specular - lr_m * gn[5], 0, 1))))
            else:
                new.append(Lambertian(np.clip(m.albedo - lr_m * gn[:3], 0, 1)))
        mats = new
        env = np.maximum(env - lr_e * ge / (np.abs(ge).max() + 1e-12) * env, 0).astype(np.float32)
        ctx.set_materials(ds, mats)
        ctx.set_env(ds, env, sc.env.intensity)
    f = float(np.median(fwd))
    a = float(np.median(adj))
    line = {"metric": "adjoint/forward time (512x512, 32 spp, depth 8)", "value": (f + a) / f, "unit": "x",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": f + a, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 gradient sums)",
            "data": "synthetic (seeded procedural studio, perturbed target)",
            "config": {"workload": "studio 512x512, 65 materials, 512x256 HDRI, 32 spp forward + 32 spp adjoint",
                       "parameters": len(sc.materials) * 6 + sc.env.width * sc.env.height * 3},
            "forward_ms": f, "adjoint_ms": a, "loss_trace": losses}
    print(json.dumps(line), flush=True)
    ds.close()
    dt.close()
    ctx.close()
    return 0


def run_batch(args):
    """256 jobs (Cornell variants with 10..200k-triangle inserts, 128^2..1024^2, 4/16/64 spp, depth 4-12):
    the autotuned batched launch against one plain pyre_render per job."""
    import torch

    from pyre_gb300 import CudaIntegrator
    from pyre_gb300 import autotune
    from pyre_gb300 import presets as P
    torch.cuda.set_device(0)
    t0 = time.time()
    jobs = P.batch_jobs(args.jobs, seed=11)
    gen_s = time.time() - t0
    ctx = CudaIntegrator(0)
    # scene upload with the instance BVHs built on the host threads, then on the GPU
    t0 = time.perf_counter()
    ctx.upload_batch([j["scene"] for j in jobs]).close()
    upload_host_s = time.perf_counter() - t0
    ctx.set_bvh_builder("device")
    ctx.upload_batch([j["scene"] for j in jobs]).close()  # warm-up of the build kernels
    t0 = time.perf_counter()
    ds = ctx.upload_batch([j["scene"] for j in jobs])
    upload_device_s = time.perf_counter() - t0
    ctx.set_bvh_builder("host")
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    samples = sum(j["width"] * j["height"] * j["spp"] for j in jobs)
    best, trials = autotune.tune_batch(ctx, ds, spec)
    knobs = dict(wave_paths=best["wave_paths"], use_graph=best["use_graph"], block_size=best["block_size"],
                 sort_by_material=best.get("sort_by_material", 0), refill_lanes=best.get("refill_lanes", 0),
                 bvh_width=best.get("bvh_width", 0))
    for _ in range(args.warmup):
        ctx.render_batch(ds, spec, **knobs)
    batch_ms = []
    launches = 0
    with Clocks(0) as clk:
        for _ in range(args.steps):
            ctx.render_batch(ds, spec, **knobs)
            s = ctx.stats()
            batch_ms.append(s.ms_total)
            launches += s.kernel_launches
    # per-view plain launches: one scene and one pyre_render per job, default knobs
    singles = [ctx.upload(j["scene"]) for j in jobs]
    for ds1, j in zip(singles, jobs):  # warm-up pass
        ctx.render(ds1, j["camera"], j["integrator"], j["width"], j["height"], j["spp"])
    view_ms = []
    for _ in range(args.steps):
        tot = 0.0
        for ds1, j in zip(singles, jobs):
            ctx.render(ds1, j["camera"], j["integrator"], j["width"], j["height"], j["spp"])
            tot += ctx.stats().ms_total
        view_ms.append(tot)
    b = float(np.median(batch_ms)) / 1e3
    v = float(np.median(view_ms)) / 1e3
    line = {"metric": "Msamples/s batched (256 Cornell-variant jobs)", "value": samples / b / 1e6,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": b * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Cornell variants)",
            "config": {"workload": f"{args.jobs} jobs, 128^2-1024^2, spp 4/16/64, depth 4-12, inserts 10-200k "
                                   "triangles", "samples": samples, "scene_gen_s": round(gen_s, 1),
                       "l2": "inputs larger than L2",
                       "scene_upload_s": {"host_bvh_build": round(upload_host_s, 3),
                                          "device_bvh_build": round(upload_device_s, 3)}},
            "per_view_value": samples / v / 1e6, "per_view_ms": v * 1e3, "batched_over_per_view": v / b,
            "autotune": {"best": best, "trials": len(trials)}, "gpu_launches": int(launches),
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    for s1 in singles:
        s1.close()
    ds.close()
    ctx.close()
    return 0


def extra_microbench(reps: int = 3) -> dict:
    """The ray-intersection microbenchmark: level-8 displaced icosphere (1,310,720 triangles), 16,777,216 rays
    from seed 1, closest hit and any hit. Device rate: rays and hits resident in HBM, the query kernel's CUDA-event
    time. End to end: the same call with host rays and host results (copies inside the timed region)."""
    import ctypes as C

    import torch

    from pyre_gb300 import CudaIntegrator
    from pyre_gb300 import native as N
    from pyre_gb300 import presets as P
    sc = P.microbench_scene(level=8)
    mesh = sc.primitives[0].instance.mesh
    n = 1 << 24
    org, d, tmin, tmax = P.random_rays(mesh, n, seed=1)
    ctx = CudaIntegrator(0)
    ctx.set_bvh_builder("device")  # the same BVH as the host build, built in ~30 ms
    ds = ctx.upload(sc)
    dev = {k: torch.from_numpy(v).cuda() for k, v in (("o", org), ("d", d), ("tmin", tmin), ("tmax", tmax))}
    rays = N.Rays(N.dptr(dev["o"]), N.dptr(dev["d"]), N.dptr(dev["tmin"]), N.dptr(dev["tmax"]), None)
    out = {k: torch.empty(n, dtype=torch.int32, device="cuda") for k in ("kind", "inst", "tri")}
    out.update({k: torch.empty(n, dtype=torch.float32, device="cuda") for k in ("t", "u", "v")})
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    hits = N.Hits(N.dptr(out["kind"], C.c_int32), N.dptr(out["inst"], C.c_int32), N.dptr(out["tri"], C.c_int32),
                  N.dptr(out["t"]), N.dptr(out["u"]), N.dptr(out["v"]))
    # the same rays and results in pinned host memory, for the end-to-end calls
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in (("o", org), ("d", d), ("tmin", tmin), ("tmax", tmax))}
    hrays = N.Rays(N.dptr(pin["o"]), N.dptr(pin["d"]), N.dptr(pin["tmin"]), N.dptr(pin["tmax"]), None)
    hout = {k: torch.empty(n, dtype=torch.int32, pin_memory=True) for k in ("kind", "inst", "tri")}
    hout.update({k: torch.empty(n, dtype=torch.float32, pin_memory=True) for k in ("t", "u", "v")})
    hocc = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    hhits = N.Hits(N.dptr(hout["kind"], C.c_int32), N.dptr(hout["inst"], C.c_int32), N.dptr(hout["tri"], C.c_int32),
                   N.dptr(hout["t"]), N.dptr(hout["u"]), N.dptr(hout["v"]))
    res = {"workload": "displaced icosphere level 8 (1,310,720 triangles), 16,777,216 rays from seed 1, "
                       "t_min 1e-4, t_max inf", "rays": n, "triangles": int(mesh.triangle_count()),
           "e2e": "rays in and results out through the C ABI from / to pinned host memory, copies in the timed call"}
    for q in ("closest", "any"):
        def call():
            if q == "closest":
                ctx.check(ctx.lib.pyre_intersect_closest(ctx.handle, ds.handle, C.byref(rays), n, C.byref(hits),
                                                         N.PYRE_MEM_DEVICE))
            else:
                ctx.check(ctx.lib.pyre_intersect_any(ctx.handle, ds.handle, C.byref(rays), n,
                                                     N.dptr(occ, C.c_uint8), N.PYRE_MEM_DEVICE))
            return ctx.stats().ms_total
        call()
        ms = sorted(call() for _ in range(reps))[reps // 2]
        res[f"{q}_grays_per_s"] = n / ms / 1e6
        res[f"{q}_ms"] = ms
        # end to end through the C ABI: rays from pinned host memory in, results to pinned host memory out
        def host_call():
            if q == "closest":
                ctx.check(ctx.lib.pyre_intersect_closest(ctx.handle, ds.handle, C.byref(hrays), n, C.byref(hhits),
                                                         N.PYRE_MEM_HOST))
            else:
                ctx.check(ctx.lib.pyre_intersect_any(ctx.handle, ds.handle, C.byref(hrays), n,
                                                     N.dptr(hocc, C.c_uint8), N.PYRE_MEM_HOST))
        host_call()
        wall = []
        for _ in range(reps):
            t0 = time.perf_counter()
            host_call()
            wall.append(time.perf_counter() - t0)
        res[f"{q}_e2e_grays_per_s"] = n / sorted(wall)[reps // 2] / 1e9
    res["gpu_launches"] = 2 * reps
    ds.close()
    ctx.close()
    return res


def extra_adjoint(reps: int = 3) -> dict:
    """The differentiable render: the studio at 512x512 (64 sphere materials + ground, 512x256 HDRI), 32 spp
    forward (pyre_forward) + 32 spp path-replay adjoint (pyre_backward) of an L2 loss against a target rendered
    from perturbed parameters. Device times from the library's CUDA events."""
    from pyre_gb300 import CudaIntegrator, PathIntegrator
    from pyre_gb300 import presets as P
    w = h = 512
    spp = 32
    sc, tgt, cam = P.adjoint_problem(w, h)
    ctx = CudaIntegrator(0)
    ds, dt = ctx.upload(sc), ctx.upload(tgt)
    it = PathIntegrator(8, 3)
    target = ctx.render(dt, cam, it, w, h, 64, spp_begin=1 << 20).radiance.astype(np.float64)
    fwd, adj, wall = [], [], []
    for k in range(reps + 1):
        t0 = time.perf_counter()
        img = ctx.forward(ds, cam, it, w, h, spp, spp_begin=k * spp).radiance
        f_ms = ctx.stats().ms_total
        dl = (2.0 * (img - target) / img.size).astype(np.float32)
        ctx.backward(ds, cam, it, w, h, spp, dl, spp_begin=k * spp)
        if k:
            fwd.append(f_ms)
            adj.append(ctx.stats().ms_total)
            wall.append(time.perf_counter() - t0)
    f, a = float(np.median(fwd)), float(np.median(adj))
    ds.close()
    dt.close()
    ctx.close()
    return {"workload": "studio 512x512, 65 materials, 512x256 HDRI, 32 spp forward + 32 spp adjoint, depth 8",
            "parameters": len(sc.materials) * 6 + sc.env.width * sc.env.height * 3,
            "forward_ms": f, "adjoint_ms": a, "forward_plus_adjoint_over_forward": (f + a) / f,
            "e2e_step_ms": 1e3 * float(np.median(wall))}


def extra_batch(reps: int = 3) -> dict:
    """256 batched jobs (Cornell variants with 10..200k-triangle inserts, 128^2..1024^2, 4/16/64 spp, depth
    4-12) against one pyre_render per job. Both arms write the same caller-owned host films and are timed on the
    wall clock (e2e: every launch, host gap, film copy and synchronisation) and by the library's CUDA events
    (device)."""
    from pyre_gb300 import CudaIntegrator
    from pyre_gb300 import presets as P
    jobs = P.batch_jobs(256, seed=11)
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    samples = sum(j["width"] * j["height"] * j["spp"] for j in jobs)
    ctx = CudaIntegrator(0)
    ctx.set_bvh_builder("device")
    ds = ctx.upload_batch([j["scene"] for j in jobs])
    singles = [ctx.upload(j["scene"]) for j in jobs]
    # the caller's host films, allocated (and their pages touched) once and reused by every call of both arms,
    # as a renderer reuses its frame buffers
    from pyre_gb300 import native as N
    from pyre_gb300.scene import Film
    films = [Film(j["width"], j["height"]) for j in jobs]
    for f in films:
        for a in (f.radiance, f.albedo, f.normal, f.depth):
            a.fill(0.0)
    cfilms = [N.Film(N.fptr(f.radiance), N.fptr(f.albedo), N.fptr(f.normal), N.fptr(f.depth), N.PYRE_MEM_HOST)
              for f in films]
    params = [CudaIntegrator.params(j["width"], j["height"], 0, j["spp"], j["integrator"]) for j in jobs]

    def batched():
        t0 = time.perf_counter()
        ctx.render_batch(ds, spec, use_graph=1, films=films)
        return time.perf_counter() - t0, ctx.stats().ms_total / 1e3

    per_job = {}

    def per_view(small_only=False):
        wall = dev = 0.0
        n = 0
        for k, (ds1, j) in enumerate(zip(singles, jobs)):
            if small_only and j["width"] > 256:
                continue
            t0 = time.perf_counter()
            ctx.render_into(ds1, j["camera"], params[k], cfilms[k])
            w1 = time.perf_counter() - t0
            d1 = ctx.stats().ms_total / 1e3
            wall += w1
            dev += d1
            n += j["width"] * j["height"] * j["spp"]
            per_job[k] = (w1, d1)
        return wall, dev, n

    batched()
    with Clocks(0) as clk_b:
        b = sorted(batched() for _ in range(reps))[reps // 2]
    per_view()
    with Clocks(0) as clk_v:
        v = sorted(per_view()[:2] for _ in range(reps))[reps // 2]
    # per-view cost by image size: where the samples and the time are
    by_size = {}
    for k, j in enumerate(jobs):
        e = by_size.setdefault(f"{j['width']}^2", {"jobs": 0, "samples": 0, "per_view_e2e_ms": 0.0,
                                                   "per_view_device_ms": 0.0})
        e["jobs"] += 1
        e["samples"] += j["width"] * j["height"] * j["spp"]
        e["per_view_e2e_ms"] += 1e3 * per_job[k][0]
        e["per_view_device_ms"] += 1e3 * per_job[k][1]
    for e in by_size.values():
        e["per_view_device_msamples_per_s"] = e["samples"] / e["per_view_device_ms"] / 1e3
        e["per_view_e2e_msamples_per_s"] = e["samples"] / e["per_view_e2e_ms"] / 1e3
    # the small views alone (128^2 and 256^2), where launch and host gaps weigh most
    small_idx = [k for k, j in enumerate(jobs) if j["width"] <= 256]
    sub = CudaIntegrator(0)
    sub.set_bvh_builder("device")
    dsub = sub.upload_batch([jobs[k]["scene"] for k in small_idx])
    sspec = [dict(spec[k], part=i) for i, k in enumerate(small_idx)]
    sfilms = [films[k] for k in small_idx]
    sub.render_batch(dsub, sspec, use_graph=1, films=sfilms)

    def small_batched():
        t0 = time.perf_counter()
        sub.render_batch(dsub, sspec, use_graph=1, films=sfilms)
        return time.perf_counter() - t0, sub.stats().ms_total / 1e3

    sb_wall, sb_dev = sorted(small_batched() for _ in range(reps))[reps // 2]
    sv_wall, sv_dev, s_samples = sorted(per_view(small_only=True) for _ in range(reps))[reps // 2]
    dsub.close()
    sub.close()
    for s1 in singles:
        s1.close()
    ds.close()
    ctx.close()
    return {"workload": "256 jobs: Cornell variants + 10..200k-triangle displaced spheres, 128^2..1024^2, spp "
                        "4/16/64, depth 4-12, Disney materials; host films", "samples": samples,
            "batched_e2e_msamples_per_s": samples / b[0] / 1e6, "batched_device_msamples_per_s": samples / b[1] / 1e6,
            "per_view_e2e_msamples_per_s": samples / v[0] / 1e6, "per_view_device_msamples_per_s": samples / v[1] / 1e6,
            "batched_over_per_view_e2e": v[0] / b[0], "batched_over_per_view_device": v[1] / b[1],
            "per_view_by_size": dict(sorted(by_size.items(), key=lambda kv: int(kv[0].split("^")[0]))),
            "clocks": {"batched": clk_b.summary(), "per_view": clk_v.summary()},
            "small_jobs": {"jobs": len(small_idx), "samples": s_samples,
                           "batched_over_per_view_e2e": sv_wall / sb_wall,
                           "batched_over_per_view_device": sv_dev / sb_dev}}


def adjoint_cosine_check() -> dict:
    """Gradient check beside the CPU baseline: pyre_backward on the small gradient-check scene (48x48, 4 spp,
    depth 6, 4 materials, 16x8 HDRI) against the oracle's forward-mode dual-number gradient (same seeds, same
    detached convention)."""
    from oracle import oracle as O
    from pyre_gb300 import CudaIntegrator, PathIntegrator
    from pyre_gb300 import native as N
    from pyre_gb300 import presets as P
    sc, cam = P.adjoint_check_scene()
    w = h = 48
    it = PathIntegrator(6, 3)
    dl = np.random.default_rng(9).normal(size=(h, w, 3)).astype(np.float32)
    ctx = CudaIntegrator(0)
    ds = ctx.upload(sc)
    g_mat, g_env = ctx.backward(ds, cam, it, w, h, 4, dl, env_sampling=N.PYRE_ENV_CDF)
    ds.close()
    ctx.close()
    o_mat, o_env = O.OracleScene(sc).render_grad(cam, w, h, 4, dl, len(sc.materials), (8, 16), max_depth=6,
                                                  min_rr_depth=3)

    def cos(a, b):
        a, b = np.ravel(a).astype(np.float64), np.ravel(b).astype(np.float64)
        return float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-300))
    return {"scene": "48x48, 4 spp, depth 6, 4 materials, 16x8 HDRI", "cos_materials": cos(g_mat, o_mat),
            "cos_env": cos(g_env, o_env)}


class Clocks:
    """Samples nvidia-smi every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k] == "Active":
                    reasons.add(nm)
        pw = [float(r[3]) for r in self.rows if len(r) > 3 and r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows),
                "power_w": statistics.median(pw) if pw else None}


def make_workload():
    from pyre_gb300 import presets as P
    t0 = time.time()
    scene = P.studio_procedural()
    cam = P.studio_procedural_camera(W, H, 0.05, 4.0)
    return scene, cam, time.time() - t0


def cpu_model() -> str:
    """CPU model name of this host (lscpu, else /proc/cpuinfo, else the platform string)."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def cpu_sample(scene, cam, rows: int, threads: int):
    """Oracle render of `rows` image rows spread over the frame at full spp, with the oracle built for this CPU
    (-mcpu=native / -march=native, no FMA contraction: the same bits as the portable build)."""
    from oracle import oracle as O
    osc = O.OracleScene(scene, nthreads=threads, build="native")
    ys = np.linspace(0, H - 1, rows).round().astype(int)
    t0 = time.time()
    for y in ys:
        osc.render(cam, W, H, SPP, crop=(0, int(y), W, int(y) + 1))
    dt = time.time() - t0
    samples = rows * W * SPP
    return samples / dt / 1e6, dt, samples


def cpu_build_info(scene, cam, threads: int) -> dict:
    """Flags and CPU of the timed oracle build, and whether it renders the portable build's bits (a 64x2 crop)."""
    from oracle import oracle as O
    crop = (W // 2 - 32, H // 2 - 1, W // 2 + 32, H // 2 + 1)
    a = O.OracleScene(scene, nthreads=threads).render(cam, W, H, 4, crop=crop)["radiance"]
    b = O.OracleScene(scene, nthreads=threads, build="native").render(cam, W, H, 4, crop=crop)["radiance"]
    return {"flags": O.native_flags(), "cpu_model": cpu_model(),
            "bit_identical_to_portable_build": bool(np.array_equal(a.view(np.uint32), b.view(np.uint32)))}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.lib("native")
    scene, cam, _ = make_workload()
    threads = os.cpu_count() or 1
    rows = args.cpu_rows or CPU_ROWS
    binfo = cpu_build_info(scene, cam, threads)
    for _ in range(args.warmup):
        cpu_sample(scene, cam, max(1, rows // 4), threads)
    vals, times = [], []
    for _ in range(args.steps):
        v, dt, n = cpu_sample(scene, cam, rows, threads)
        vals.append(v)
        times.append(dt)
    value = float(np.median(vals))
    sample = f"{rows} rows of 1920 px spread over the frame at 64 spp ({rows * W * SPP} samples) per step"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "procedural studio 1920x1080, 64 spp, depth 8, thin lens, motion blur, "
                                   "2.1M triangles, 2048x1024 HDRI", "global_batch": 1, "seq_len": None,
                       "parallelism": "cpu threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample + "; C++ restatement of the reference's CPU path (the Rust "
                                       "reference cannot be built here)", **binfo},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from pyre_gb300 import CudaIntegrator, PathIntegrator
    from pyre_gb300 import native as N

    scene, cam, gen_s = make_workload()
    ctx = CudaIntegrator(local)
    t0 = time.time()
    ds = ctx.upload(scene)
    upload_s = time.time() - t0
    info = ds.info()
    integ = PathIntegrator(DEPTH, RR)
    # Weak scaling: rank r renders samples [r*64, (r+1)*64) of the frame.
    s0 = rank * SPP
    params = CudaIntegrator.params(W, H, s0, s0 + SPP, integ, env_sampling=N.PYRE_ENV_ALIAS, use_graph=args.graph,
                                    refill_lanes=args.refill, bvh_width=args.bvh_width,
                                    wave_paths=args.wave_paths, block_size=args.block)
    params.sort_by_material = args.sort
    npix = W * H
    dev = {k: torch.empty(npix * c, dtype=torch.float32, device="cuda") for k, c in
           (("radiance", 3), ("albedo", 3), ("normal", 3), ("depth", 1))}
    dfilm = N.Film(N.dptr(dev["radiance"]), N.dptr(dev["albedo"]), N.dptr(dev["normal"]), N.dptr(dev["depth"]),
                   N.PYRE_MEM_DEVICE)

    for _ in range(args.warmup):
        ctx.render_into(ds, cam, params, dfilm)
    ctx.set_stage_timing(True)
    dev_ms, ext_ms, shade_ms, shadow_ms, other_ms = [], [], [], [], []
    ext_rays = shadow_rays = samples = launches = waves = 0
    barrier()
    with Clocks(local) as clk:
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.render_into(ds, cam, params, dfilm)
            s = ctx.stats()
            dev_ms.append(s.ms_total)
            ext_ms.append(s.ms_extend); shade_ms.append(s.ms_shade); shadow_ms.append(s.ms_shadow)
            other_ms.append(s.ms_other)
            ext_rays += s.extend_rays; shadow_rays += s.shadow_rays; samples += s.samples
            launches += s.kernel_launches; waves += s.waves
        barrier()
        wall = time.perf_counter() - wall0
    ctx.set_stage_timing(False)
    dev_s = sum(dev_ms) / 1e3
    t_local = torch.tensor([dev_s], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(t_local, op=dist.ReduceOp.MAX)
    t_max = float(t_local.item())
    value = samples * world / t_max / 1e6

    # ---- end to end through the public API with a host film
    host = {k: np.zeros(npix * c, np.float32) for k, c in (("radiance", 3), ("albedo", 3), ("normal", 3),
                                                            ("depth", 1))}
    try:  # pinned host memory for the film read-back
        pins = {k: torch.empty(npix * c, dtype=torch.float32, pin_memory=True) for k, c in
                (("radiance", 3), ("albedo", 3), ("normal", 3), ("depth", 1))}
        hptr = {k: N.dptr(v) for k, v in pins.items()}
    except RuntimeError:
        hptr = {k: N.fptr(v) for k, v in host.items()}
    hfilm = N.Film(hptr["radiance"], hptr["albedo"], hptr["normal"], hptr["depth"], N.PYRE_MEM_HOST)
    ctx.render_into(ds, cam, params, hfilm)
    barrier()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.render_into(ds, cam, params, hfilm)
    barrier()
    e2e_s = time.perf_counter() - e0
    e2e_t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
    e2e_value = samples * world / float(e2e_t.item()) / 1e6

    # ---- roofline of the extend stage (dominant kernel)
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak, peak_src = 6800.0, "fallback"
    if peaks_path.exists():
        peak, peak_src = float(json.loads(peaks_path.read_text())["hbm_gbs"]), "measured"
    ext_launches = waves * DEPTH
    scene_bytes = info.triangle_bytes + info.node_bytes
    alg_bytes = ext_rays * 52 + ext_launches * scene_bytes
    ext_s = sum(ext_ms) / 1e3
    achieved = alg_bytes / ext_s / 1e9 if ext_s > 0 else None
    stage_total = sum(ext_ms) + sum(shade_ms) + sum(shadow_ms) + sum(other_ms)
    roofline = {"bound": "hbm", "kernel": "k_extend (closest-hit traversal)",
                "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": None,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else
                "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": alg_bytes / max(ext_launches, 1),
                "avg_launch_ms": sum(ext_ms) / max(ext_launches, 1),
                "stage_share": {"extend": sum(ext_ms) / stage_total, "shade": sum(shade_ms) / stage_total,
                                "shadow": sum(shadow_ms) / stage_total, "other": sum(other_ms) / stage_total}}
    traffic_file = ROOT / "profiles" / "extend_traffic.json"
    if traffic_file.exists():
        tj = json.loads(traffic_file.read_text())
        roofline["traffic"] = tj.get("bytes_per_launch")
        roofline["traffic_note"] = tj.get("note")
    counters_file = ROOT / "profiles" / "k_extend_counters.json"
    if counters_file.exists():  # the kernel is issue-bound: these counters say more than the HBM fraction
        roofline["ncu_counters_bounces_0_1_2"] = json.loads(counters_file.read_text())

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": "procedural studio 1920x1080, 64 spp, depth 8, RR from 3, thin lens 0.05/4.0, "
                                   "8 moving instances, 64x32768-triangle displaced spheres + ground quad, "
                                   "2048x1024 HDRI (alias sampling)",
                       "global_batch": world, "seq_len": None, "parallelism": f"replicas x{world} (spp ranges)",
                       "l2": "inputs larger than L2 (scene %.0f MB + path state)" % (info.device_bytes / 1e6),
                       "triangles": int(info.n_triangles), "scene_gen_s": round(gen_s, 2),
                       "scene_upload_s": round(upload_s, 2), "use_graph": args.graph,
                       "refill_lanes": args.refill, "bvh_width": args.bvh_width, "sort_by_material": args.sort,
                       "wave_paths": args.wave_paths, "block_size": args.block},
            "mrays_per_s": (ext_rays + shadow_rays) * world / t_max / 1e6,
            "rays": {"extend": ext_rays // args.steps, "shadow": shadow_rays // args.steps},
            "wall_s_timed": wall,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step":
                    C_sizeof_params(), "d2h_bytes_per_step": npix * 10 * 4},
            "gpu_launches": int(launches),
            "roofline": roofline}
    if rank == 0 and world == 1 and not args.no_extras:
        line["microbench"] = extra_microbench()
        line["adjoint"] = extra_adjoint()
        line["batch"] = extra_batch()
    if rank == 0 and world == 1 and not args.no_cpu:
        if "adjoint" in line:
            line["adjoint"]["gradient_check"] = adjoint_cosine_check()
        threads = os.cpu_count() or 1
        rows = args.cpu_rows or CPU_ROWS
        binfo = cpu_build_info(scene, cam, threads)
        v, dt, n = cpu_sample(scene, cam, rows, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{rows} rows x 1920 px at 64 spp ({n} samples, {dt:.1f} s); C++ "
                                          "restatement of the reference's CPU path (Rust reference not buildable "
                                          "here)", **binfo}
    line["clocks"] = clk.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)
    ds.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def C_sizeof_params() -> int:
    from pyre_gb300 import native as N
    import ctypes
    return ctypes.sizeof(N.CameraDesc) + ctypes.sizeof(N.RenderParams)


if __name__ == "__main__":
    sys.exit(main())

"""Command-line renderer on the GB300 backend (the GPU counterpart of the
reference CLI's offline path, crates/pyre-cli/src/main.rs:17-95,106-303).

  python -m pyre_gb300.cli --preset cornell --width 800 --height 600 --spp 16
  python -m pyre_gb300.cli --preset studio-procedural --width 960 --height 540 --spp 4 --repeat 2
  python -m pyre_gb300.cli --preset microbench --rays 16777216 --query closest

Prints one JSON log line per render (elapsed_ms, Msamples/s, rays) like the
reference's `render complete` line; `--output x.npy` saves the radiance.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def parse(argv=None):
    ap = argparse.ArgumentParser(prog="pyre_gb300.cli")
    ap.add_argument("--preset", default="cornell",
                    choices=["cornell", "cornell-box", "studio", "studio-procedural", "microbench", "adjoint"])
    ap.add_argument("--width", type=int, default=800)
    ap.add_argument("--height", type=int, default=600)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--max-depth", type=int, default=8)
    ap.add_argument("--aperture", type=float, default=0.0)
    ap.add_argument("--focus-distance", type=float, default=None)
    ap.add_argument("--motion-blur", action="store_true")
    ap.add_argument("--env-sampling", default="alias", choices=["alias", "cdf"])
    ap.add_argument("--graph", action="store_true", help="replay each wave through a CUDA graph")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--output", default=None, help="save radiance as .npy")
    ap.add_argument("--rays", type=int, default=1 << 24, help="microbench: number of rays")
    ap.add_argument("--query", default="closest", choices=["closest", "any", "both"])
    ap.add_argument("--level", type=int, default=8, help="microbench: icosphere subdivision level")
    ap.add_argument("--bvh-width", type=int, default=2, choices=[2, 4, 8], help="instance BVH width")
    return ap.parse_args(argv)


def _scene(args):
    from . import presets as P
    if args.preset == "cornell":
        return P.cornell_ref(args.motion_blur), P.cornell_ref_camera(args.width, args.height)
    if args.preset == "cornell-box":
        return P.cornell_box(), P.cornell_box_camera(args.width, args.height)
    if args.preset == "studio":
        return P.studio_ref(args.motion_blur), P.studio_ref_camera(args.width, args.height, args.aperture)
    ap = args.aperture if args.aperture > 0 else 0.05
    fd = args.focus_distance if args.focus_distance is not None else 4.0
    return P.studio_procedural(), P.studio_procedural_camera(args.width, args.height, ap, fd)


def microbench(args, ctx) -> int:
    import torch

    from . import native as N
    from . import presets as P
    import ctypes as C
    sc = P.microbench_scene(args.level)
    mesh = sc.primitives[0].instance.mesh
    org, d, tmin, tmax = P.random_rays(mesh, args.rays, seed=1)
    ds = ctx.upload(sc)
    ds.set_bvh_width(args.bvh_width)
    dev = {k: torch.from_numpy(v).cuda() for k, v in (("o", org), ("d", d), ("tmin", tmin), ("tmax", tmax))}
    rays = N.Rays(N.dptr(dev["o"]), N.dptr(dev["d"]), N.dptr(dev["tmin"]), N.dptr(dev["tmax"]), None)
    n = args.rays
    out = {k: torch.empty(n, dtype=torch.int32, device="cuda") for k in ("kind", "inst", "tri")}
    out.update({k: torch.empty(n, dtype=torch.float32, device="cuda") for k in ("t", "u", "v")})
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    hits = N.Hits(N.dptr(out["kind"], C.c_int32), N.dptr(out["inst"], C.c_int32), N.dptr(out["tri"], C.c_int32),
                  N.dptr(out["t"]), N.dptr(out["u"]), N.dptr(out["v"]))
    queries = ["closest", "any"] if args.query == "both" else [args.query]
    for q in queries:
        for rep in range(args.repeat):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if q == "closest":
                ctx.check(ctx.lib.pyre_intersect_closest(ctx.handle, ds.handle, C.byref(rays), n, C.byref(hits),
                                                         N.PYRE_MEM_DEVICE))
            else:
                ctx.check(ctx.lib.pyre_intersect_any(ctx.handle, ds.handle, C.byref(rays), n,
                                                     N.dptr(occ, C.c_uint8), N.PYRE_MEM_DEVICE))
            dt = time.perf_counter() - t0
            print(json.dumps({"query": q, "rays": n, "triangles": mesh.triangle_count(), "bvh_width": args.bvh_width,
                              "elapsed_ms": dt * 1e3, "mrays_per_s": n / dt / 1e6}), flush=True)
    ds.close()
    return 0


def adjoint(args, ctx) -> int:
    """One forward render and one path-replay adjoint of the differentiable-render problem."""
    from . import presets as P
    from .scene import PathIntegrator
    sc, tgt, cam = P.adjoint_problem(args.width, args.height, env_size=(512, 256))
    ds, dt = ctx.upload(sc), ctx.upload(tgt)
    it = PathIntegrator(args.max_depth, 3)
    target = ctx.render(dt, cam, it, args.width, args.height, args.spp, spp_begin=1 << 20).radiance
    for _ in range(args.repeat):
        img = ctx.forward(ds, cam, it, args.width, args.height, args.spp).radiance
        f_ms = ctx.stats().ms_total
        dl = (2.0 * (img - target) / img.size).astype(np.float32)
        gm, ge = ctx.backward(ds, cam, it, args.width, args.height, args.spp, dl)
        print(json.dumps({"preset": "adjoint", "forward_ms": f_ms, "adjoint_ms": ctx.stats().ms_total,
                          "loss": float(np.mean((img - target) ** 2)), "grad_norm_materials": float(np.linalg.norm(gm)),
                          "grad_norm_env": float(np.linalg.norm(ge))}), flush=True)
    ds.close()
    dt.close()
    return 0


def main(argv=None) -> int:
    args = parse(argv)
    from .native import PYRE_ENV_ALIAS, PYRE_ENV_CDF
    from .scene import CudaIntegrator, PathIntegrator
    ctx = CudaIntegrator(0)
    if args.preset == "microbench":
        return microbench(args, ctx)
    if args.preset == "adjoint":
        return adjoint(args, ctx)
    scene, cam = _scene(args)
    ds = ctx.upload(scene)
    ds.set_bvh_width(args.bvh_width)
    integ = PathIntegrator(args.max_depth, 3)
    env = PYRE_ENV_CDF if args.env_sampling == "cdf" else PYRE_ENV_ALIAS
    film = None
    for _ in range(args.repeat):
        t0 = time.perf_counter()
        film = ctx.render(ds, cam, integ, args.width, args.height, args.spp, env_sampling=env,
                          use_graph=1 if args.graph else 0)
        dt = time.perf_counter() - t0
        s = ctx.stats()
        print(json.dumps({"preset": args.preset, "elapsed_ms": dt * 1e3, "device_ms": s.ms_total,
                          "triangles": scene.triangle_count(), "spp": args.spp,
                          "pixels": args.width * args.height, "msamples_per_s": s.samples / (s.ms_total / 1e3) / 1e6,
                          "extend_rays": s.extend_rays, "shadow_rays": s.shadow_rays, "waves": s.waves}), flush=True)
    if args.output:
        np.save(args.output, film.radiance)
    ds.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

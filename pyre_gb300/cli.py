"""Command-line renderer on the GB300 backend (the GPU counterpart of the
reference CLI's offline path, crates/pyre-cli/src/main.rs:17-95,106-303).

  python -m pyre_gb300.cli --preset cornell --width 800 --height 600 --spp 16
  python -m pyre_gb300.cli --preset studio-procedural --width 960 --height 540 --spp 4 --repeat 2
  python -m pyre_gb300.cli --preset microbench --rays 16777216 --query closest
  python -m pyre_gb300.cli --scene room.pbrt --env sky.hdr --output frame.exr --aovs all --save-aov-pngs
  python -m pyre_gb300.cli --preset cornell --spp 64 --progressive --output frame.png

Prints one JSON log line per render (elapsed_ms, Msamples/s, rays) like the
reference's `render complete` line. `--output` writes a PNG (gamma 2.2) or
an EXR (linear, with the `--aovs` channels) like the reference CLI
(main.rs:288-330); `.npy` saves the raw radiance. `--scene` loads .pbrt,
.gltf or .glb (main.rs:114-150); `--env` a Radiance .hdr. `--progressive`
is the viewer's loop without a window (viewer.rs:114-185): one-sample passes
merged into a running mean, saved to `--output` when the passes are done.
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
    ap.add_argument("--output", "-o", default=None, help="write .png / .exr (film sinks) or .npy (radiance)")
    ap.add_argument("--scene", "-s", default=None, help="load a .pbrt, .gltf or .glb scene")
    ap.add_argument("--env", default=None, help="Radiance .hdr environment map")
    ap.add_argument("--env-intensity", type=float, default=1.0)
    ap.add_argument("--aovs", default="", help="EXR channels besides beauty: albedo,normal,depth or all")
    ap.add_argument("--save-aov-pngs", action="store_true", help="also write <stem>.albedo/normal/depth.png")
    ap.add_argument("--progressive", action="store_true",
                    help="one-sample passes merged into a running mean (the viewer's loop, no window)")
    ap.add_argument("--pass-chunk", type=int, default=8, help="progressive: passes per library call")
    ap.add_argument("--rays", type=int, default=1 << 24, help="microbench: number of rays")
    ap.add_argument("--query", default="closest", choices=["closest", "any", "both"])
    ap.add_argument("--level", type=int, default=8, help="microbench: icosphere subdivision level")
    ap.add_argument("--bvh-width", type=int, default=2, choices=[2, 4, 8], help="instance BVH width")
    ap.add_argument("--sort", type=int, default=0, choices=[0, 1, 2, 3],
                    help="shade queue order (sort_by_material): 0 = the library default, 1 = sorted by material "
                         "within tiles, 2 = unsorted, 3 = the whole queue sorted")
    return ap.parse_args(argv)


def scene_bounds(scene):
    """Scene::bounds (scene.rs:146-152): union of the instances' world bounds."""
    lo, hi = np.full(3, np.inf, np.float32), np.full(3, -np.inf, np.float32)
    for prim in scene.primitives:
        mesh = prim.instance.mesh
        if mesh.triangle_count() == 0:
            continue
        v = mesh.positions[np.unique(mesh.indices)]
        blo, bhi = v.min(axis=0), v.max(axis=0)
        m = prim.instance.motion
        if m is not None:
            blo = np.minimum(blo + m.offset_t0, blo + m.offset_t1)
            bhi = np.maximum(bhi + m.offset_t0, bhi + m.offset_t1)
        lo, hi = np.minimum(lo, blo), np.maximum(hi, bhi)
    return lo.astype(np.float32), hi.astype(np.float32)


def auto_frame(lo, hi, vfov_deg: float, aspect: float):
    """auto_frame_params (main.rs:336-350): look at the bounds' centre from
    +z and a little above, far enough that the bounding sphere fits."""
    F = np.float32
    center = ((lo + hi) * F(0.5)).astype(F)
    radius = max(F(np.linalg.norm(hi - lo)) * F(0.5), F(1e-3))
    half_v = F(np.radians(F(vfov_deg))) * F(0.5)
    half_h = F(np.arctan(F(aspect) * F(np.tan(half_v))))
    dist = max(radius / F(np.sin(half_v)), radius / F(np.sin(half_h))) * F(1.15)
    d = np.array([0.0, 0.3, 1.0], F)
    d = (d / np.linalg.norm(d)).astype(F)
    return (center + dist * d).astype(F), center


def _loaded_scene(args):
    """main.rs:114-150: a PBRT file (with its camera when it has one) or glTF
    meshes with one white Lambertian material."""
    from pathlib import Path

    from .scene import Lambertian, MeshInstance, Primitive, Scene
    ext = Path(args.scene).suffix.lower()
    if ext == ".pbrt":
        from .io import load_pbrt
        ld = load_pbrt(args.scene)
        c = ld.camera
        return ld.scene, ((c.origin, c.target, c.up, c.vfov_deg) if c is not None else None)
    if ext in (".gltf", ".glb"):
        from .io import load_gltf
        sc = Scene()
        sc.materials.append(Lambertian([0.73, 0.73, 0.73]))
        for mesh in load_gltf(args.scene):
            sc.primitives.append(Primitive(MeshInstance.build(mesh), 0))
        return sc, None
    raise SystemExit(f"unsupported scene extension {ext!r}: expected .pbrt, .gltf or .glb")


def _camera(args, origin, target, up, vfov):
    from .scene import PinholeCamera, ThinLensCamera
    aspect = np.float32(args.width) / np.float32(args.height)
    if args.aperture > 0:
        fd = args.focus_distance if args.focus_distance is not None else float(
            np.linalg.norm(np.asarray(target, np.float32) - np.asarray(origin, np.float32)))
        return ThinLensCamera.look_at(origin, target, up, vfov, aspect, args.aperture, fd)
    return PinholeCamera.look_at(origin, target, up, vfov, aspect)


def _scene(args):
    from . import presets as P
    if args.scene:
        scene, cam = _loaded_scene(args)
        if cam is None:
            lo, hi = scene_bounds(scene)
            diag = float(np.linalg.norm(hi - lo))
            if np.isfinite(diag) and diag > 0:
                o, t = auto_frame(lo, hi, 45.0, np.float32(args.width) / np.float32(args.height))
                cam = (o, t, (0, 1, 0), 45.0)
            else:
                cam = ((0, 0, 3), (0, 0, 0), (0, 1, 0), 45.0)
        return scene, _camera(args, *cam)
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
    if args.env:
        from .io import load_hdri
        scene.env = load_hdri(args.env, args.env_intensity)
    ds = ctx.upload(scene)
    ds.set_bvh_width(args.bvh_width)
    integ = PathIntegrator(args.max_depth, 3)
    env = PYRE_ENV_CDF if args.env_sampling == "cdf" else PYRE_ENV_ALIAS
    if args.progressive:
        return progressive(args, ctx, ds, scene, cam, integ, env)
    film = None
    for _ in range(args.repeat):
        t0 = time.perf_counter()
        film = ctx.render(ds, cam, integ, args.width, args.height, args.spp, env_sampling=env,
                          use_graph=1 if args.graph else 0, sort_by_material=args.sort)
        dt = time.perf_counter() - t0
        s = ctx.stats()
        print(json.dumps({"preset": args.preset, "elapsed_ms": dt * 1e3, "device_ms": s.ms_total,
                          "triangles": scene.triangle_count(), "spp": args.spp,
                          "pixels": args.width * args.height, "msamples_per_s": s.samples / (s.ms_total / 1e3) / 1e6,
                          "extend_rays": s.extend_rays, "shadow_rays": s.shadow_rays, "waves": s.waves}), flush=True)
    if args.output:
        save_output(args, film)
    ds.close()
    ctx.close()
    return 0


def save_output(args, film) -> None:
    """save_film (main.rs:318-334) and the AOV sidecar PNGs (film.rs:117-186)."""
    from pathlib import Path

    from . import sinks
    ext = Path(args.output).suffix.lower()
    aovs = {a.strip().lower() for a in args.aovs.split(",") if a.strip()}
    bad = aovs - {"all", "albedo", "normal", "n", "depth", "z"}
    if bad:
        raise SystemExit(f"unknown AOV {sorted(bad)[0]!r} (expected albedo, normal, depth or all)")
    on = {"albedo": "albedo" in aovs or "all" in aovs, "normal": bool(aovs & {"normal", "n", "all"}),
          "depth": bool(aovs & {"depth", "z", "all"})}
    if ext == ".npy":
        np.save(args.output, film.radiance)
    elif ext == ".exr":
        sinks.save_exr(film, args.output, **on)
    elif ext in (".png", ""):
        sinks.save_png(film, args.output)
    else:
        raise SystemExit(f"unsupported output extension {ext!r} (expected .png or .exr)")
    if args.save_aov_pngs:
        sinks.save_aov_pngs(film, args.output, **on)


def progressive(args, ctx, ds, scene, cam, integ, env) -> int:
    """The viewer's render loop without a window: passes 0 .. spp-1 of one
    sample per pixel, each merged into the running mean in pass order."""
    from .scene import Film
    mean = np.zeros((args.height, args.width, 3), np.float32)
    done = 0
    t0 = time.perf_counter()
    while done < args.spp:
        k = min(args.pass_chunk, args.spp - done)
        ctx.render_progressive(ds, cam, integ, args.width, args.height, k, mean=mean, pass_begin=done,
                               env_sampling=env)
        done += k
        print(json.dumps({"progressive_passes": done, "elapsed_ms": (time.perf_counter() - t0) * 1e3}),
              flush=True)
    if args.output:
        film = Film(args.width, args.height)
        film.radiance[:] = mean.reshape(film.radiance.shape)
        save_output(args, film)
    ds.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

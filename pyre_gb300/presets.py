"""Scene presets and seeded synthetic workloads.

* ``cornell_ref`` / ``studio_ref``: the Pyre CLI's built-in presets
  (crates/pyre-cli/src/main.rs:365-563, make_uv_sphere :565-599).
* ``cornell_box``: the 256x256 Lambertian Cornell box of the benchmark plan
  (5 wall quads, a 0.25x0.25 ceiling light of radiance (17,12,4), two rotated
  boxes). Box sizes are not given by the plan; they are fixed here:
  tall box 0.6 x 1.2 x 0.6 rotated +17 deg at (-0.33, -1, -0.28), short box
  0.6 x 0.6 x 0.6 rotated -18 deg at (0.35, -1, 0.3), faces with explicit
  outward normals.
* ``icosphere_displaced`` + ``random_rays``: the ray-query microbenchmark
  (level-8 icosphere, 1,310,720 triangles, radial value-noise displacement of
  amplitude 0.1; rays with origins uniform in the 1.5x-scaled mesh AABB and
  directions uniform on the sphere).
* ``studio_procedural``: 64 seeded displaced spheres of 32,768 triangles on a
  ground quad, 8 of them moving, seeded Disney materials and a procedural
  2048x1024 HDRI (sky gradient plus a log-normal sun lobe of peak 5e4).

All geometry is generated in float32 with the reference's operation order
where a reference formula exists; trigonometric values are computed in float64
and rounded to float32. No external assets or datasets are used.
"""
from __future__ import annotations

import math

import numpy as np

from .scene import (DiffuseAreaQuadLight, DisneyBsdf, HdriEnvironmentLight, InstanceMotion, Lambertian,
                    MeshInstance, PathIntegrator, PinholeCamera, Primitive, Scene, ThinLensCamera, TriangleMesh)

F32 = np.float32
PI32 = F32(math.pi)
TAU32 = F32(2 * math.pi)


def _sin32(x):
    return np.sin(np.asarray(x, np.float64)).astype(F32)


def _cos32(x):
    return np.cos(np.asarray(x, np.float64)).astype(F32)


def quad_mesh(corners, normal) -> TriangleMesh:
    """main.rs:353-360."""
    c = np.asarray(corners, F32).reshape(4, 3)
    return TriangleMesh(c, np.array([0, 1, 2, 0, 2, 3], np.uint32), np.tile(np.asarray(normal, F32), (4, 1)))


def make_uv_sphere(center, radius, u_segments: int, v_segments: int) -> TriangleMesh:
    """main.rs:565-599 in float32."""
    center = np.asarray(center, F32)
    radius = F32(radius)
    v = np.arange(v_segments + 1, dtype=F32)
    u = np.arange(u_segments + 1, dtype=F32)
    phi = PI32 * v / F32(v_segments)
    theta = TAU32 * u / F32(u_segments)
    sp, cp = _sin32(phi)[:, None], _cos32(phi)[:, None]
    st, ct = _sin32(theta)[None, :], _cos32(theta)[None, :]
    n = np.stack([sp * ct, np.broadcast_to(cp, (v_segments + 1, u_segments + 1)), sp * st], axis=-1).astype(F32)
    n = n.reshape(-1, 3)
    pos = (center[None, :] + radius * n).astype(F32)
    row = u_segments + 1
    vv, uu = np.meshgrid(np.arange(v_segments, dtype=np.uint32), np.arange(u_segments, dtype=np.uint32), indexing="ij")
    i00 = vv * row + uu
    i01 = i00 + 1
    i10 = (vv + 1) * row + uu
    i11 = i10 + 1
    idx = np.stack([i00, i10, i11, i00, i11, i01], axis=-1).reshape(-1).astype(np.uint32)
    return TriangleMesh(pos, idx, n)


def _defaults_camera(preset: str, width: int, height: int, aperture: float = 0.0, focus: float | None = None):
    aspect = F32(width) / F32(height)
    if preset == "studio":
        o, t, fov = (1.6, 0.5, 2.6), (0.0, 0.05, 0.0), 38.0
    else:
        o, t, fov = (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0
    if aperture > 0:
        fd = focus if focus is not None else float(np.linalg.norm(np.subtract(t, o).astype(F32)))
        return ThinLensCamera.look_at(o, t, (0, 1, 0), fov, aspect, aperture, fd)
    return PinholeCamera.look_at(o, t, (0, 1, 0), fov, aspect)


def cornell_ref(motion_blur: bool = False) -> Scene:
    """The reference's default preset, cornell_box (main.rs:365-496)."""
    sc = Scene()
    sc.materials += [Lambertian([0.73] * 3), Lambertian([0.65, 0.05, 0.05]), Lambertian([0.12, 0.45, 0.15])]
    white, red, green = 0, 1, 2
    s = 1.0
    walls = [
        (quad_mesh([(-s, -s, -s), (s, -s, -s), (s, -s, s), (-s, -s, s)], (0, 1, 0)), white),
        (quad_mesh([(-s, s, -s), (s, s, -s), (s, s, s), (-s, s, s)], (0, -1, 0)), white),
        (quad_mesh([(-s, -s, -s), (s, -s, -s), (s, s, -s), (-s, s, -s)], (0, 0, 1)), white),
        (quad_mesh([(-s, -s, -s), (-s, -s, s), (-s, s, s), (-s, s, -s)], (1, 0, 0)), red),
        (quad_mesh([(s, -s, -s), (s, s, -s), (s, s, s), (s, -s, s)], (-1, 0, 0)), green),
    ]
    for mesh, mat in walls:
        sc.primitives.append(Primitive(MeshInstance.build(mesh), mat))
    sc.materials.append(DisneyBsdf([1.0, 0.766, 0.336], 1.0, 0.1, 0.5))
    gold = make_uv_sphere((0.35, -0.65, 0.25), 0.35, 48, 24)
    inst = (MeshInstance.build_animated(gold, InstanceMotion((0, 0, 0), (0, 0.25, 0))) if motion_blur
            else MeshInstance.build(gold))
    sc.primitives.append(Primitive(inst, 3))
    sc.materials.append(DisneyBsdf([0.72] * 3, 0.0, 0.18, 0.5))
    sc.primitives.append(Primitive(MeshInstance.build(make_uv_sphere((-0.35, -0.65, -0.3), 0.35, 48, 24)), 4))
    sc.lights.append(DiffuseAreaQuadLight((-0.3, 0.999, -0.3), (0.6, 0, 0), (0, 0, 0.6), (15.0, 15.0, 15.0)))
    return sc


def cornell_ref_camera(width: int = 800, height: int = 600):
    return _defaults_camera("cornell", width, height)


def studio_ref(motion_blur: bool = False, env_intensity: float = 1.0) -> Scene:
    """studio_scene (main.rs:502-563) with the procedural gradient sky the CLI adds (main.rs:167-175)."""
    sc = Scene()
    sc.materials.append(Lambertian([0.55] * 3))
    s = 50.0
    sc.primitives.append(Primitive(MeshInstance.build(
        quad_mesh([(-s, 0, -s), (s, 0, -s), (s, 0, s), (-s, 0, s)], (0, 1, 0))), 0))
    sc.materials.append(DisneyBsdf([1.0, 0.766, 0.336], 1.0, 0.1, 0.5))
    gold = make_uv_sphere((0.4, 0.35, 0.0), 0.35, 64, 32)
    inst = (MeshInstance.build_animated(gold, InstanceMotion((-0.15, 0, 0), (0.15, 0, 0))) if motion_blur
            else MeshInstance.build(gold))
    sc.primitives.append(Primitive(inst, 1))
    sc.materials.append(DisneyBsdf([0.72] * 3, 0.0, 0.2, 0.5))
    sc.primitives.append(Primitive(MeshInstance.build(make_uv_sphere((-0.4, 0.35, 0.0), 0.35, 64, 32)), 2))
    sc.env = HdriEnvironmentLight.gradient((0.20, 0.35, 0.65), (0.95, 0.85, 0.70), env_intensity)
    return sc


def studio_ref_camera(width: int = 800, height: int = 600, aperture: float = 0.0):
    return _defaults_camera("studio", width, height, aperture)


# --------------------------------------------------------- Cornell (plan) --
def _box(center_xz, size, rot_deg, y0=-1.0) -> TriangleMesh:
    sx, sy, sz = size
    c, s = math.cos(math.radians(rot_deg)), math.sin(math.radians(rot_deg))

    def xf(p):
        x, y, z = p
        return (center_xz[0] + c * x + s * z, y0 + y, center_xz[1] - s * x + c * z)

    def nrm(n):
        x, y, z = n
        return (c * x + s * z, y, -s * x + c * z)

    hx, hz = sx / 2, sz / 2
    faces = [  # corners (counter-clockwise seen from outside) and outward normal
        ([(-hx, sy, -hz), (-hx, sy, hz), (hx, sy, hz), (hx, sy, -hz)], (0, 1, 0)),
        ([(-hx, 0, -hz), (hx, 0, -hz), (hx, 0, hz), (-hx, 0, hz)], (0, -1, 0)),
        ([(-hx, 0, hz), (hx, 0, hz), (hx, sy, hz), (-hx, sy, hz)], (0, 0, 1)),
        ([(hx, 0, -hz), (-hx, 0, -hz), (-hx, sy, -hz), (hx, sy, -hz)], (0, 0, -1)),
        ([(hx, 0, hz), (hx, 0, -hz), (hx, sy, -hz), (hx, sy, hz)], (1, 0, 0)),
        ([(-hx, 0, -hz), (-hx, 0, hz), (-hx, sy, hz), (-hx, sy, -hz)], (-1, 0, 0)),
    ]
    pos, nor, idx = [], [], []
    for corners, n in faces:
        b = len(pos)
        pos += [xf(p) for p in corners]
        nor += [nrm(n)] * 4
        idx += [b, b + 1, b + 2, b, b + 2, b + 3]
    return TriangleMesh(np.asarray(pos, F32), np.asarray(idx, np.uint32), np.asarray(nor, F32))


def cornell_box() -> Scene:
    """Lambertian Cornell box of the benchmark plan (256x256, 16 spp, depth 8)."""
    sc = Scene()
    sc.materials += [Lambertian([0.725, 0.71, 0.68]), Lambertian([0.63, 0.065, 0.05]), Lambertian([0.14, 0.45, 0.09])]
    white, red, green = 0, 1, 2
    s = 1.0
    walls = [
        (quad_mesh([(-s, -s, -s), (s, -s, -s), (s, -s, s), (-s, -s, s)], (0, 1, 0)), white),
        (quad_mesh([(-s, s, -s), (s, s, -s), (s, s, s), (-s, s, s)], (0, -1, 0)), white),
        (quad_mesh([(-s, -s, -s), (s, -s, -s), (s, s, -s), (-s, s, -s)], (0, 0, 1)), white),
        (quad_mesh([(-s, -s, -s), (-s, -s, s), (-s, s, s), (-s, s, -s)], (1, 0, 0)), red),
        (quad_mesh([(s, -s, -s), (s, s, -s), (s, s, s), (s, -s, s)], (-1, 0, 0)), green),
    ]
    for mesh, mat in walls:
        sc.primitives.append(Primitive(MeshInstance.build(mesh), mat))
    sc.primitives.append(Primitive(MeshInstance.build(_box((-0.33, -0.28), (0.6, 1.2, 0.6), 17.0)), white))
    sc.primitives.append(Primitive(MeshInstance.build(_box((0.35, 0.3), (0.6, 0.6, 0.6), -18.0)), white))
    sc.lights.append(DiffuseAreaQuadLight((-0.125, 0.999, -0.125), (0.25, 0, 0), (0, 0, 0.25), (17.0, 12.0, 4.0)))
    return sc


def cornell_box_camera(width: int = 256, height: int = 256):
    return PinholeCamera.look_at((0, 0, 3), (0, 0, 0), (0, 1, 0), 45.0, F32(width) / F32(height))


# ------------------------------------------------------------ value noise --
def _hash3(ix, iy, iz, seed: int):
    """Integer lattice hash -> [0,1) (xorshift-multiply mixing on uint32)."""
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) \
        ^ (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B9 & 0xFFFFFFFF)
    h = h ^ (h >> np.uint32(16))
    h = h * np.uint32(0x7FEB352D)
    h = h ^ (h >> np.uint32(15))
    h = h * np.uint32(0x846CA68B)
    h = h ^ (h >> np.uint32(16))
    return (h >> np.uint32(8)).astype(np.float64) * (1.0 / 16777216.0)


def value_noise(p: np.ndarray, seed: int, octaves: int = 3, freq: float = 3.0) -> np.ndarray:
    """Fractal trilinear value noise in [0,1) with smoothstep weights (float64)."""
    total = np.zeros(p.shape[0])
    norm = 0.0
    amp = 1.0
    with np.errstate(over="ignore"):
        for o in range(octaves):
            q = p * (freq * (2.0 ** o)) + 17.0 * o
            i0 = np.floor(q)
            f = q - i0
            w = f * f * (3.0 - 2.0 * f)
            i0 = i0.astype(np.int64)
            acc = np.zeros(p.shape[0])
            for dx in (0, 1):
                for dy in (0, 1):
                    for dz in (0, 1):
                        val = _hash3(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed + 101 * o)
                        wx = w[:, 0] if dx else 1.0 - w[:, 0]
                        wy = w[:, 1] if dy else 1.0 - w[:, 1]
                        wz = w[:, 2] if dz else 1.0 - w[:, 2]
                        acc += wx * wy * wz * val
            total += amp * acc
            norm += amp
            amp *= 0.5
    return total / norm


def smooth_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    tri = idx.reshape(-1, 3)
    p = pos.astype(np.float64)
    fn = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]])
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, tri[:, k], fn)
    ln = np.linalg.norm(vn, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (vn / ln).astype(F32)


# ------------------------------------------------------------- icosphere --
def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        a, b = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
        key = a * nv + b
        uniq, inv = np.unique(key, return_inverse=True)
        ua, ub = uniq // nv, uniq % nv
        mid = v[ua] + v[ub]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        nf = f.shape[0]
        m01, m12, m20 = inv[:nf] + nv, inv[nf:2 * nf] + nv, inv[2 * nf:] + nv
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def icosphere_displaced(level: int = 8, amplitude: float = 0.1, seed: int = 7) -> TriangleMesh:
    v, f = icosphere(level)
    r = 1.0 + amplitude * (2.0 * value_noise(v, seed) - 1.0)
    pos = (v * r[:, None]).astype(F32)
    return TriangleMesh(pos, f.reshape(-1).astype(np.uint32), None)


def random_rays(mesh: TriangleMesh, n: int, seed: int = 1):
    """Origins uniform in the mesh AABB scaled 1.5x about its centre; directions uniform on S^2."""
    rng = np.random.default_rng(seed)
    lo, hi = mesh.positions.min(0).astype(np.float64), mesh.positions.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.5
    org = (c + (rng.random((n, 3)) * 2 - 1) * h).astype(F32)
    z = rng.random(n) * 2 - 1
    phi = rng.random(n) * 2 * math.pi
    s = np.sqrt(np.maximum(0.0, 1 - z * z))
    d = np.stack([s * np.cos(phi), s * np.sin(phi), z], 1).astype(F32)
    tmin = np.full(n, 1e-4, F32)
    tmax = np.full(n, np.inf, F32)
    return org, d, tmin, tmax


def microbench_scene(level: int = 8, seed: int = 7) -> Scene:
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    sc.primitives.append(Primitive(MeshInstance.build(icosphere_displaced(level, 0.1, seed)), 0))
    return sc


# ------------------------------------------------------ procedural studio --
def procedural_hdri(width: int = 2048, height: int = 1024, sun_peak: float = 5e4,
                    sun_dir=(0.45, 0.55, -0.70), sun_a0: float = 0.004, sun_sigma: float = 0.35) -> np.ndarray:
    """Equirect (row 0 = zenith) sky gradient plus a log-normal sun lobe.

    sky(d)  = lerp(horizon, zenith, d.y) above the horizon, horizon*max(1+d.y/2, 0)*0.5 below
    sun(a)  = sun_peak * exp(-(ln(1 + a/a0))^2 / (2 sigma^2)), a = angle to sun_dir (radians)
    """
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = u * 2 * math.pi - math.pi
    theta = v * math.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    d = np.stack([st * np.cos(phi)[None, :], np.broadcast_to(ct, (height, width)), st * np.sin(phi)[None, :]], -1)
    zen = np.array([0.20, 0.35, 0.65])
    hor = np.array([0.95, 0.85, 0.70])
    y = d[..., 1:2]
    sky = np.where(y >= 0, hor * (1 - y) + zen * y, hor * np.maximum(1 + 0.5 * y, 0) * 0.5)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    a = np.arccos(np.clip((d * s).sum(-1), -1, 1))
    sun = sun_peak * np.exp(-np.log1p(a / sun_a0) ** 2 / (2 * sun_sigma ** 2))
    img = sky + sun[..., None] * np.array([1.0, 0.95, 0.85])
    return img.astype(F32)


def displaced_sphere(center, radius: float, segments: int, seed: int, amplitude: float = 0.08) -> TriangleMesh:
    base = make_uv_sphere((0, 0, 0), 1.0, segments, segments)
    p = base.positions.astype(np.float64)
    r = 1.0 + amplitude * (2.0 * value_noise(p, seed, octaves=3, freq=2.5) - 1.0)
    pos = (np.asarray(center, np.float64) + radius * p * r[:, None]).astype(F32)
    nrm = smooth_normals(pos, base.indices)
    # make_uv_sphere winds its triangles clockwise seen from outside: orient outward
    if np.sum(nrm.astype(np.float64) * p) < 0:
        nrm = -nrm
    return TriangleMesh(pos, base.indices, nrm)


def studio_procedural(n_side: int = 8, segments: int = 128, n_moving: int = 8, seed: int = 3,
                      hdri_size=(2048, 1024)) -> Scene:
    """64 displaced spheres (2 x 128 x 128 = 32,768 triangles each) on a ground quad, HDRI lit."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    sc.materials.append(Lambertian([0.55] * 3))
    s = 50.0
    sc.primitives.append(Primitive(MeshInstance.build(
        quad_mesh([(-s, 0, -s), (s, 0, -s), (s, 0, s), (-s, 0, s)], (0, 1, 0))), 0))
    n = n_side * n_side
    moving = set(rng.choice(n, size=min(n_moving, n), replace=False).tolist())
    for k in range(n):
        i, j = k % n_side, k // n_side
        radius = 0.35
        center = ((i - (n_side - 1) / 2) * 1.0, radius, (j - (n_side - 1) / 2) * 1.0)
        mesh = displaced_sphere(center, radius, segments, seed=1000 + k)
        base = rng.random(3)
        rough = 0.05 + 0.95 * rng.random()
        metal = 1.0 if rng.random() < 0.3 else 0.0
        sc.materials.append(DisneyBsdf(base, metal, rough, 0.5))
        if k in moving:
            dv = rng.normal(size=3)
            dv[1] = abs(dv[1]) * 0.3
            dv = 0.2 * dv / np.linalg.norm(dv)
            inst = MeshInstance.build_animated(mesh, InstanceMotion((0, 0, 0), dv))
        else:
            inst = MeshInstance.build(mesh)
        sc.primitives.append(Primitive(inst, len(sc.materials) - 1))
    w, h = hdri_size
    sc.env = HdriEnvironmentLight(w, h, procedural_hdri(w, h), 1.0)
    return sc


def studio_procedural_camera(width: int = 1920, height: int = 1080, aperture: float = 0.05, focus: float = 4.0):
    aspect = F32(width) / F32(height)
    return ThinLensCamera.look_at((0.0, 3.4, 7.2), (0.0, 0.0, 0.6), (0, 1, 0), 45.0, aspect, aperture, focus)


DEFAULT_INTEGRATOR = PathIntegrator(8, 3)


# ------------------------------------------------------------ batch jobs --
def batch_jobs(n_jobs: int = 256, seed: int = 11, resolutions=(128, 256, 512, 1024), spps=(4, 16, 64),
               depth_range=(4, 12), tri_range=(10, 200_000)):
    """Batched-rendering workload: Cornell-box variants, each with a seeded
    displaced-sphere insert of log-uniform triangle count, a seeded Disney
    material on it, a random square resolution, spp and max depth.

    Returns a list of dicts: scene, camera, width, height, spp, integrator.
    """
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        sc = cornell_box()
        n_tri = float(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        seg = max(3, int(round((n_tri / 2.0) ** 0.5)))  # a seg x seg UV grid has 2*seg^2 triangles
        center = (rng.uniform(-0.4, 0.4), -0.55, rng.uniform(-0.3, 0.5))
        mesh = displaced_sphere(center, 0.3, seg, seed=5000 + j, amplitude=0.08)
        sc.materials.append(DisneyBsdf(rng.random(3), 1.0 if rng.random() < 0.3 else 0.0,
                                       0.05 + 0.95 * rng.random(), 0.5))
        sc.primitives.append(Primitive(MeshInstance.build(mesh), len(sc.materials) - 1))
        res = int(rng.choice(resolutions))
        jobs.append({"scene": sc, "camera": cornell_box_camera(res, res), "width": res, "height": res,
                     "spp": int(rng.choice(spps)),
                     "integrator": PathIntegrator(int(rng.integers(depth_range[0], depth_range[1] + 1)), 3)})
    return jobs


# ----------------------------------------------------- differentiable render --
def adjoint_problem(width: int = 512, height: int = 512, env_size=(512, 256), seed: int = 21, n_side: int = 8,
                    segments: int = 128):
    """The differentiable-render workload: the procedural studio at width x height
    with its 64 sphere materials (+ ground) and an env_size FP32 HDRI. Returns
    (scene, target_scene, camera): the target's parameters are seeded
    perturbations of the scene's (+-20 % on base color, roughness, metallic,
    specular, clamped to their ranges; env texels x U[0.5, 2])."""
    sc = studio_procedural(n_side=n_side, segments=segments, hdri_size=env_size)
    rng = np.random.default_rng(seed)
    tgt = Scene(list(sc.primitives), [], list(sc.lights), None)
    for m in sc.materials:
        if isinstance(m, DisneyBsdf):
            f = 1.0 + rng.uniform(-0.2, 0.2, size=6)
            tgt.materials.append(DisneyBsdf(np.clip(m.base_color * f[:3], 0, 1), float(np.clip(m.metallic * f[3], 0, 1)),
                                            float(np.clip(m.roughness * f[4], 0.05, 1)),
                                            float(np.clip(m.specular * f[5], 0, 1))))
        else:
            tgt.materials.append(Lambertian(np.clip(m.albedo * (1.0 + rng.uniform(-0.2, 0.2, size=3)), 0, 1)))
    px = sc.env.pixels * rng.uniform(0.5, 2.0, size=sc.env.pixels.shape).astype(F32)
    tgt.env = HdriEnvironmentLight(sc.env.width, sc.env.height, px.astype(F32), sc.env.intensity)
    cam = studio_procedural_camera(width, height)
    return sc, tgt, cam


def adjoint_check_scene():
    """A small scene for gradient checks against the CPU dual-number gradient: a Lambertian ground quad, three
    Disney spheres (one metallic) and a 16x8 HDRI with one bright texel; 48x48 camera. Returns (scene, camera)."""
    sc = Scene()
    sc.materials.append(Lambertian([0.55, 0.5, 0.45]))
    s = 20.0
    sc.primitives.append(Primitive(MeshInstance.build(
        quad_mesh([(-s, 0, -s), (s, 0, -s), (s, 0, s), (-s, 0, s)], (0, 1, 0))), 0))
    rng = np.random.default_rng(4)
    for k, (x, z) in enumerate([(-0.5, 0.0), (0.4, 0.1), (0.0, -0.6)]):
        sc.materials.append(DisneyBsdf(rng.random(3), float(k == 1), 0.2 + 0.3 * k, 0.5))
        sc.primitives.append(Primitive(MeshInstance.build(make_uv_sphere((x, 0.3, z), 0.3, 24, 12)), k + 1))
    px = (0.3 + rng.random((8, 16, 3))).astype(F32)
    px[2, 5] = [20.0, 18.0, 14.0]  # a bright texel
    sc.env = HdriEnvironmentLight(16, 8, px, 1.0)
    return sc, studio_ref_camera(48, 48)


def fd_check_scene():
    """A scene for finite-difference gradient checks: a Lambertian ground quad, a Disney sphere with metallic
    0.4 (between dielectric and conductor) and roughness 0.35, a dielectric Disney sphere with roughness 0.6,
    a 16x8 HDRI with one bright (sun) texel and dim sky texels, and a quad light above; 64x64 pinhole camera.
    Returns (scene, camera)."""
    sc = Scene()
    sc.materials.append(Lambertian([0.6, 0.58, 0.55]))
    s = 20.0
    sc.primitives.append(Primitive(MeshInstance.build(
        quad_mesh([(-s, 0, -s), (s, 0, -s), (s, 0, s), (-s, 0, s)], (0, 1, 0))), 0))
    sc.materials.append(DisneyBsdf([0.75, 0.45, 0.25], 0.4, 0.35, 0.5))
    sc.primitives.append(Primitive(MeshInstance.build(make_uv_sphere((-0.35, 0.35, 0.0), 0.35, 32, 16)), 1))
    sc.materials.append(DisneyBsdf([0.2, 0.5, 0.75], 0.0, 0.6, 0.5))
    sc.primitives.append(Primitive(MeshInstance.build(make_uv_sphere((0.4, 0.3, -0.1), 0.3, 32, 16)), 2))
    rng = np.random.default_rng(5)
    px = (0.2 + 0.3 * rng.random((8, 16, 3))).astype(F32)
    px[2, 5] = [30.0, 27.0, 21.0]  # the sun texel
    sc.env = HdriEnvironmentLight(16, 8, px, 1.0)
    sc.lights.append(DiffuseAreaQuadLight((-0.5, 2.0, -0.5), (1.0, 0, 0), (0, 0, 1.0), (4.0, 4.0, 4.0)))
    cam = PinholeCamera.look_at((0, 0.9, 2.2), (0, 0.3, 0), (0, 1, 0), 40.0, 1.0)
    return sc, cam

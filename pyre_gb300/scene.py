"""Host-side mirror of the Pyre renderer's scene API, backed by the CUDA library.

Class and field names follow the reference (crates/pyre/src): ``TriangleMesh``
(geometry/mesh.rs:5-11), ``InstanceMotion`` (mesh.rs:46-60), ``MeshInstance``
(mesh.rs:70-88), ``Primitive`` / ``Scene`` (scene.rs:19-34), ``Lambertian`` /
``DisneyBsdf`` (material.rs:42-94), ``DiffuseAreaQuadLight`` (light.rs:46-76),
``HdriEnvironmentLight`` (light.rs:205-272), ``PinholeCamera`` /
``ThinLensCamera`` (camera.rs:28-122), ``PathIntegrator`` (integrator.rs:36-48)
and ``Film`` (film.rs:15-20). ``CudaIntegrator.render`` is the GPU drop-in for
the CLI render loop (crates/pyre-cli/src/main.rs:248-286).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native as N

F32 = np.float32


def _v3(v) -> np.ndarray:
    a = np.asarray(v, dtype=F32).reshape(3)
    return a


def pixel_seed(x: int, y: int, sample: int) -> int:
    """sampler.rs:41-49 (SplitMix64-style hash), in Python integers."""
    m = (1 << 64) - 1
    h = ((x << 32) | y) & m
    h ^= (sample * 0x9E3779B97F4A7C15) & m
    h ^= h >> 30
    h = (h * 0xBF58476D1CE4E5B9) & m
    h ^= h >> 27
    h = (h * 0x94D049BB133111EB) & m
    return h ^ (h >> 31)


@dataclass
class TriangleMesh:
    positions: np.ndarray            # (n_vertices, 3) float32
    indices: np.ndarray              # (n_triangles*3,) uint32
    normals: np.ndarray | None = None  # (n_vertices, 3) float32
    uvs: np.ndarray | None = None

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, dtype=F32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.uint32).reshape(-1)
        if self.normals is not None:
            self.normals = np.ascontiguousarray(self.normals, dtype=F32).reshape(-1, 3)
        if self.indices.size % 3:
            raise ValueError("indices must hold 3 entries per triangle")

    def triangle_count(self) -> int:
        return self.indices.size // 3


@dataclass
class InstanceMotion:
    offset_t0: np.ndarray
    offset_t1: np.ndarray

    def __post_init__(self):
        self.offset_t0 = _v3(self.offset_t0)
        self.offset_t1 = _v3(self.offset_t1)


@dataclass
class MeshInstance:
    mesh: TriangleMesh
    motion: InstanceMotion | None = None
    bvh_nodes: np.ndarray | None = None   # BVH2_DTYPE records, as Bvh::nodes()
    bvh_prim: np.ndarray | None = None    # uint32, as Bvh::primitive_indices()

    @staticmethod
    def build(mesh: TriangleMesh) -> "MeshInstance":
        return MeshInstance(mesh)

    @staticmethod
    def build_animated(mesh: TriangleMesh, motion: InstanceMotion) -> "MeshInstance":
        return MeshInstance(mesh, motion)


@dataclass
class Primitive:
    instance: MeshInstance
    material_id: int


@dataclass
class Lambertian:
    albedo: np.ndarray

    def __post_init__(self):
        self.albedo = _v3(self.albedo)


@dataclass
class DisneyBsdf:
    base_color: np.ndarray
    metallic: float
    roughness: float
    specular: float = 0.5

    def __post_init__(self):
        self.base_color = _v3(self.base_color)


@dataclass
class DiffuseAreaQuadLight:
    p0: np.ndarray
    edge_u: np.ndarray
    edge_v: np.ndarray
    emission: np.ndarray

    def __post_init__(self):
        self.p0, self.edge_u, self.edge_v, self.emission = map(_v3, (self.p0, self.edge_u, self.edge_v, self.emission))


@dataclass
class HdriEnvironmentLight:
    width: int
    height: int
    pixels: np.ndarray   # (height, width, 3) float32, row 0 = zenith
    intensity: float = 1.0

    def __post_init__(self):
        self.pixels = np.ascontiguousarray(self.pixels, dtype=F32).reshape(self.height, self.width, 3)

    @staticmethod
    def constant(color, intensity: float) -> "HdriEnvironmentLight":
        return HdriEnvironmentLight(1, 1, _v3(color).reshape(1, 1, 3), intensity)

    @staticmethod
    def gradient(zenith, horizon, intensity: float) -> "HdriEnvironmentLight":
        """light.rs:252-272: 128x64 two-tone sky, darkened below the horizon."""
        h, w = 64, 128
        zen, hor = _v3(zenith), _v3(horizon)
        px = np.empty((h, w, 3), dtype=F32)
        for y in range(h):
            v = (F32(y) + F32(0.5)) / F32(h)
            cos_t = F32(1.0) - F32(2.0) * v
            if cos_t >= 0:
                color = hor * (F32(1.0) - cos_t) + zen * cos_t
            else:
                color = hor * max(F32(1.0) + cos_t * F32(0.5), F32(0.0))
            px[y, :, :] = color.astype(F32)
        return HdriEnvironmentLight(w, h, px, intensity)


@dataclass
class Scene:
    primitives: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    lights: list = field(default_factory=list)
    env: HdriEnvironmentLight | None = None

    def triangle_count(self) -> int:
        return sum(p.instance.mesh.triangle_count() for p in self.primitives)


@dataclass
class CameraSpec:
    kind: int
    origin: np.ndarray
    target: np.ndarray
    up: np.ndarray
    vfov_deg: float
    aspect: float
    aperture_radius: float = 0.0
    focus_distance: float = 0.0

    def to_desc(self) -> N.CameraDesc:
        d = N.CameraDesc()
        d.kind = self.kind
        d.origin[:] = [float(x) for x in _v3(self.origin)]
        d.target[:] = [float(x) for x in _v3(self.target)]
        d.up[:] = [float(x) for x in _v3(self.up)]
        d.vfov_deg, d.aspect = float(self.vfov_deg), float(self.aspect)
        d.aperture_radius, d.focus_distance = float(self.aperture_radius), float(self.focus_distance)
        return d

    def as_array(self) -> np.ndarray:
        """[thin, origin, target, up, vfov, aspect, aperture, focus] for the oracle."""
        return np.concatenate([[F32(self.kind)], _v3(self.origin), _v3(self.target), _v3(self.up),
                               [F32(self.vfov_deg), F32(self.aspect), F32(self.aperture_radius),
                                F32(self.focus_distance)]]).astype(F32)


class PinholeCamera:
    @staticmethod
    def look_at(origin, target, world_up, vfov_deg, aspect) -> CameraSpec:
        return CameraSpec(N.PYRE_CAMERA_PINHOLE, _v3(origin), _v3(target), _v3(world_up), float(vfov_deg),
                          float(np.float32(aspect)))


class ThinLensCamera:
    @staticmethod
    def look_at(origin, target, world_up, vfov_deg, aspect, aperture_radius, focus_distance) -> CameraSpec:
        return CameraSpec(N.PYRE_CAMERA_THIN_LENS, _v3(origin), _v3(target), _v3(world_up), float(vfov_deg),
                          float(np.float32(aspect)), float(aperture_radius), float(focus_distance))


@dataclass
class PathIntegrator:
    max_depth: int = 8
    min_rr_depth: int = 3


class Film:
    """Per-pixel means (PixelSample fields) of a render, row-major, top-left origin."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.radiance = np.zeros((height, width, 3), F32)
        self.albedo = np.zeros((height, width, 3), F32)
        self.normal = np.zeros((height, width, 3), F32)
        self.depth = np.zeros((height, width), F32)


# ---------------------------------------------------------------- flatten --
def _material_desc(m) -> N.MaterialDesc:
    md = N.MaterialDesc()
    if isinstance(m, Lambertian):
        md.kind = N.PYRE_MAT_LAMBERTIAN
        md.base_color[:] = [float(x) for x in m.albedo]
    elif isinstance(m, DisneyBsdf):
        md.kind = N.PYRE_MAT_DISNEY
        md.base_color[:] = [float(x) for x in m.base_color]
        md.metallic, md.roughness, md.specular = float(m.metallic), float(m.roughness), float(m.specular)
    else:
        raise TypeError(f"unsupported material {type(m).__name__}")
    return md


class _Flat:
    """A SceneDesc plus the numpy arrays it points into (kept alive)."""

    def __init__(self, scene: Scene):
        keep = []
        mesh_ids: dict[int, int] = {}
        meshes = []
        insts = []
        for prim in scene.primitives:
            inst = prim.instance
            key = id(inst.mesh) if inst.bvh_nodes is None else id(inst)
            if key not in mesh_ids:
                m = inst.mesh
                md = N.MeshDesc()
                md.positions = N.fptr(m.positions)
                md.n_vertices = m.positions.shape[0]
                md.indices = N.u32ptr(m.indices)
                md.n_triangles = m.triangle_count()
                md.normals = N.fptr(m.normals) if m.normals is not None else None
                keep += [m.positions, m.indices, m.normals]
                if inst.bvh_nodes is not None:
                    nodes = np.ascontiguousarray(inst.bvh_nodes, dtype=N.BVH2_DTYPE)
                    prim_idx = np.ascontiguousarray(inst.bvh_prim, dtype=np.uint32)
                    keep += [nodes, prim_idx]
                    md.bvh_nodes = nodes.ctypes.data_as(C.POINTER(N.Bvh2Node))
                    md.n_bvh_nodes = nodes.shape[0]
                    md.bvh_prim_indices = N.u32ptr(prim_idx)
                mesh_ids[key] = len(meshes)
                meshes.append(md)
            idd = N.InstanceDesc()
            idd.mesh = mesh_ids[key]
            idd.material = int(prim.material_id)
            if inst.motion is not None:
                idd.has_motion = 1
                idd.offset_t0[:] = [float(x) for x in inst.motion.offset_t0]
                idd.offset_t1[:] = [float(x) for x in inst.motion.offset_t1]
            insts.append(idd)
        mats = [_material_desc(m) for m in scene.materials]
        lights = []
        for l in scene.lights:
            ld = N.QuadLightDesc()
            ld.p0[:] = [float(x) for x in l.p0]
            ld.edge_u[:] = [float(x) for x in l.edge_u]
            ld.edge_v[:] = [float(x) for x in l.edge_v]
            ld.emission[:] = [float(x) for x in l.emission]
            lights.append(ld)
        self.meshes = (N.MeshDesc * max(1, len(meshes)))(*meshes)
        self.insts = (N.InstanceDesc * max(1, len(insts)))(*insts)
        self.mats = (N.MaterialDesc * max(1, len(mats)))(*mats)
        self.lights = (N.QuadLightDesc * max(1, len(lights)))(*lights)
        self.env = None
        d = N.SceneDesc()
        d.meshes, d.n_meshes = self.meshes, len(meshes)
        d.instances, d.n_instances = self.insts, len(insts)
        d.materials, d.n_materials = self.mats, len(mats)
        d.lights, d.n_lights = self.lights, len(lights)
        if scene.env is not None:
            e = N.EnvDesc()
            px = np.ascontiguousarray(scene.env.pixels, dtype=F32)
            keep.append(px)
            e.width, e.height, e.rgb, e.intensity = scene.env.width, scene.env.height, N.fptr(px), float(scene.env.intensity)
            self.env = e
            d.env = C.pointer(self.env)
        self.desc = d
        self.keep = keep


def build_bvh(mesh: TriangleMesh) -> tuple[np.ndarray, np.ndarray]:
    """Bvh::build over the mesh's triangles (bvh.rs:45-64) -> (nodes, primitive indices)."""
    lib = N.load()
    n = mesh.triangle_count()
    nodes = np.zeros(max(2 * n, 1), dtype=N.BVH2_DTYPE)
    prim = np.zeros(max(n, 1), dtype=np.uint32)
    count = C.c_uint32(0)
    N.check(lib.pyre_bvh_build(N.fptr(mesh.positions), mesh.positions.shape[0], N.u32ptr(mesh.indices), n,
                               nodes.ctypes.data_as(C.POINTER(N.Bvh2Node)), N.u32ptr(prim), C.byref(count)))
    return nodes[: count.value].copy(), prim[:n].copy()


class DeviceScene:
    def __init__(self, ctx: "CudaIntegrator", handle: C.c_void_p, scene: Scene):
        self.ctx, self.handle, self.scene = ctx, handle, scene

    def info(self) -> N.SceneInfo:
        s = N.SceneInfo()
        N.check(N.load().pyre_scene_get_info(self.handle, C.byref(s)))
        return s

    def set_bvh_width(self, width: int) -> None:
        """pyre_scene_set_bvh_width: default instance-BVH width (2, 4 or 8)."""
        self.ctx.check(N.load().pyre_scene_set_bvh_width(self.ctx.handle, self.handle, width))

    def close(self):
        if self.handle:
            N.load().pyre_scene_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CudaIntegrator:
    """Owns a context (one CUDA stream) on one device."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        h = C.c_void_p()
        N.check(self.lib.pyre_ctx_create(device, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.pyre_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int):
        N.check(rc, self.handle)

    def upload(self, scene: Scene) -> DeviceScene:
        flat = _Flat(scene)
        h = C.c_void_p()
        self.check(self.lib.pyre_scene_upload(self.handle, C.byref(flat.desc), C.byref(h)))
        return DeviceScene(self, h, scene)

    @staticmethod
    def params(width, height, spp_begin, spp_end, integrator: PathIntegrator, crop=None, env_sampling=0,
               wave_paths=0, use_graph=0, block_size=0, refill_lanes=0, bvh_width=0,
               sort_by_material=0) -> N.RenderParams:
        p = N.RenderParams()
        p.width, p.height, p.spp_begin, p.spp_end = width, height, spp_begin, spp_end
        p.max_depth, p.min_rr_depth = integrator.max_depth, integrator.min_rr_depth
        if crop is not None:
            p.crop[:] = list(crop)
        p.env_sampling, p.wave_paths, p.use_graph, p.block_size = env_sampling, wave_paths, use_graph, block_size
        p.refill_lanes, p.bvh_width, p.sort_by_material = refill_lanes, bvh_width, sort_by_material
        return p

    def render(self, dscene: DeviceScene, camera: CameraSpec, integrator: PathIntegrator, width: int, height: int,
               spp: int, spp_begin: int = 0, crop=None, env_sampling: int = 0, wave_paths: int = 0,
               use_graph: int = 0, refill_lanes: int = 0, bvh_width: int = 0, sort_by_material: int = 0) -> Film:
        """Renders samples [spp_begin, spp_begin+spp) into a (crop-sized) host Film."""
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, width, height)
        film = Film(x1 - x0, y1 - y0)
        f = N.Film(N.fptr(film.radiance), N.fptr(film.albedo), N.fptr(film.normal), N.fptr(film.depth), N.PYRE_MEM_HOST)
        cam = camera.to_desc()
        p = self.params(width, height, spp_begin, spp_begin + spp, integrator, crop, env_sampling, wave_paths, use_graph,
                        refill_lanes=refill_lanes, bvh_width=bvh_width, sort_by_material=sort_by_material)
        self.check(self.lib.pyre_render(self.handle, dscene.handle, C.byref(cam), C.byref(p), C.byref(f)))
        return film

    def upload_batch(self, scenes: list) -> DeviceScene:
        """pyre_scene_upload_batch: one device scene with one part per scene."""
        flats = [_Flat(s) for s in scenes]
        arr = (N.SceneDesc * len(flats))(*[f.desc for f in flats])
        h = C.c_void_p()
        self.check(self.lib.pyre_scene_upload_batch(self.handle, arr, len(flats), C.byref(h)))
        return DeviceScene(self, h, scenes)

    def render_batch(self, dscene: DeviceScene, jobs: list, wave_paths: int = 0, use_graph: int = 0,
                     block_size: int = 0, sort_by_material: int = 0, refill_lanes: int = 0,
                     bvh_width: int = 0, films: list | None = None) -> list:
        """jobs: dicts with part, camera, width, height, spp, spp_begin (0), integrator -> list of Films.
        `films` (one Film per job, of its size) are filled in place instead of new ones."""
        cjobs = []
        if films is None:
            films = [Film(jb["width"], jb["height"]) for jb in jobs]
        if len(films) != len(jobs):
            raise ValueError("one film per job")
        for jb, film in zip(jobs, films):
            w, h = jb["width"], jb["height"]
            if film.radiance.shape != (h, w, 3):
                raise ValueError("film size differs from the job's image size")
            it = jb.get("integrator", PathIntegrator())
            b = N.BatchJob()
            b.part = jb["part"]
            b.camera = jb["camera"].to_desc()
            b.width, b.height = w, h
            b.spp_begin = jb.get("spp_begin", 0)
            b.spp_end = b.spp_begin + jb["spp"]
            b.max_depth, b.min_rr_depth = it.max_depth, it.min_rr_depth
            b.film = N.Film(N.fptr(film.radiance), N.fptr(film.albedo), N.fptr(film.normal), N.fptr(film.depth),
                            N.PYRE_MEM_HOST)
            cjobs.append(b)
        arr = (N.BatchJob * len(cjobs))(*cjobs)
        p = N.RenderParams()
        p.wave_paths, p.use_graph, p.block_size = wave_paths, use_graph, block_size
        p.sort_by_material, p.refill_lanes, p.bvh_width = sort_by_material, refill_lanes, bvh_width
        self.check(self.lib.pyre_render_batch(self.handle, dscene.handle, arr, len(cjobs), C.byref(p)))
        return films

    def set_bvh_builder(self, builder: str) -> None:
        """pyre_set_bvh_builder: "host" (threads) or "device" (one GPU pass over
        all meshes) for the BVHs that uploads build."""
        code = {"host": N.PYRE_BVH_BUILDER_HOST, "device": N.PYRE_BVH_BUILDER_DEVICE}[builder]
        self.check(self.lib.pyre_set_bvh_builder(self.handle, code))

    def bvh_build(self, mesh: TriangleMesh) -> tuple[np.ndarray, np.ndarray]:
        """pyre_bvh_build_device: the reference BVH of `mesh` built on the GPU
        (nodes in the Bvh::nodes layout, primitive indices)."""
        n = mesh.triangle_count()
        nodes = np.zeros(max(2 * n, 1), N.BVH2_DTYPE)
        prim = np.zeros(max(n, 1), np.uint32)
        cnt = C.c_uint32()
        self.check(self.lib.pyre_bvh_build_device(self.handle, N.fptr(mesh.positions), mesh.positions.shape[0],
                                                  N.u32ptr(mesh.indices), n,
                                                  nodes.ctypes.data_as(C.POINTER(N.Bvh2Node)), N.u32ptr(prim),
                                                  C.byref(cnt)))
        return nodes[:cnt.value].copy(), prim[:n].copy()

    def render_progressive(self, dscene: DeviceScene, camera: CameraSpec, integrator: PathIntegrator, width: int,
                           height: int, passes: int, mean: np.ndarray | None = None, pass_begin: int = 0,
                           crop=None, env_sampling: int = 0, **knobs) -> np.ndarray:
        """pyre_render_progressive: merges passes [pass_begin, pass_begin + passes)
        (one sample per pixel each) into the running radiance mean (crop h x w x 3
        float32, updated in place and returned; zeros when None)."""
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, width, height)
        if mean is None:
            mean = np.zeros((y1 - y0, x1 - x0, 3), np.float32)
        if mean.dtype != np.float32 or not mean.flags.c_contiguous or mean.size != (y1 - y0) * (x1 - x0) * 3:
            raise ValueError("mean must be a C-contiguous float32 array of crop height x width x 3")
        cam = camera.to_desc()
        p = self.params(width, height, pass_begin, pass_begin + passes, integrator, crop, env_sampling, **knobs)
        self.check(self.lib.pyre_render_progressive(self.handle, dscene.handle, C.byref(cam), C.byref(p),
                                                    mean.ctypes.data_as(C.c_void_p), N.PYRE_MEM_HOST))
        return mean

    def render_into(self, dscene: DeviceScene, camera: CameraSpec, params: N.RenderParams, film: N.Film) -> None:
        """pyre_render into caller-provided film buffers (host or device pointers)."""
        cam = camera.to_desc()
        self.check(self.lib.pyre_render(self.handle, dscene.handle, C.byref(cam), C.byref(params), C.byref(film)))

    def set_stage_timing(self, enabled: bool) -> None:
        self.check(self.lib.pyre_set_stage_timing(self.handle, 1 if enabled else 0))

    def forward(self, dscene: DeviceScene, camera: CameraSpec, integrator: PathIntegrator, width: int, height: int,
                spp: int, spp_begin: int = 0, crop=None, env_sampling: int = 0) -> Film:
        """pyre_forward: render() that also keeps per-path radiance for backward()."""
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, width, height)
        film = Film(x1 - x0, y1 - y0)
        f = N.Film(N.fptr(film.radiance), N.fptr(film.albedo), N.fptr(film.normal), N.fptr(film.depth), N.PYRE_MEM_HOST)
        cam = camera.to_desc()
        p = self.params(width, height, spp_begin, spp_begin + spp, integrator, crop, env_sampling)
        self.check(self.lib.pyre_forward(self.handle, dscene.handle, C.byref(cam), C.byref(p), C.byref(f)))
        return film

    def backward(self, dscene: DeviceScene, camera: CameraSpec, integrator: PathIntegrator, width: int, height: int,
                 spp: int, dl_di: np.ndarray, spp_begin: int = 0, crop=None, env_sampling: int = 0,
                 env_grad: bool = True):
        """pyre_backward: gradients of a loss with d loss / d film = dl_di (crop h, w, 3).

        Returns (material gradients (n_materials, 6) float64, env gradients (h, w, 3) or None)."""
        sc = dscene.scene
        p = self.params(width, height, spp_begin, spp_begin + spp, integrator, crop, env_sampling)
        mat = np.zeros((len(sc.materials), 6), np.float64)
        env = np.zeros((sc.env.height, sc.env.width, 3), F32) if (sc.env is not None and env_grad) else None
        g = N.Gradients(mat.ctypes.data_as(C.POINTER(C.c_double)), N.fptr(env) if env is not None else None,
                        N.PYRE_MEM_HOST)
        d = np.ascontiguousarray(dl_di, F32)
        cam = camera.to_desc()
        self.check(self.lib.pyre_backward(self.handle, dscene.handle, C.byref(cam), C.byref(p), N.fptr(d),
                                          N.PYRE_MEM_HOST, C.byref(g)))
        return mat, env

    def set_materials(self, dscene: DeviceScene, materials: list) -> None:
        arr = (N.MaterialDesc * max(1, len(materials)))(*[_material_desc(m) for m in materials])
        self.check(self.lib.pyre_scene_set_materials(self.handle, dscene.handle, arr, len(materials)))
        dscene.scene.materials = list(materials)

    def set_env(self, dscene: DeviceScene, pixels: np.ndarray, intensity: float = 1.0) -> None:
        px = np.ascontiguousarray(pixels, F32)
        self.check(self.lib.pyre_scene_set_env(self.handle, dscene.handle, N.fptr(px), float(intensity)))
        env = dscene.scene.env
        dscene.scene.env = HdriEnvironmentLight(env.width, env.height, px, intensity)

    def stats(self) -> N.RenderStats:
        s = N.RenderStats()
        self.check(self.lib.pyre_get_render_stats(self.handle, C.byref(s)))
        return s

    def intersect(self, dscene: DeviceScene, org, dirs, tmin, tmax, time=None, any_hit=False):
        """Host-array ray queries; returns dict of numpy arrays (closest) or uint8 mask (any)."""
        org = np.ascontiguousarray(org, F32)
        dirs = np.ascontiguousarray(dirs, F32)
        tmin = np.ascontiguousarray(tmin, F32)
        tmax = np.ascontiguousarray(tmax, F32)
        n = tmin.shape[0]
        rays = N.Rays(N.fptr(org), N.fptr(dirs), N.fptr(tmin), N.fptr(tmax),
                      N.fptr(np.ascontiguousarray(time, F32)) if time is not None else None)
        if any_hit:
            occ = np.zeros(n, np.uint8)
            self.check(self.lib.pyre_intersect_any(self.handle, dscene.handle, C.byref(rays), n,
                                                   occ.ctypes.data_as(N.P_u8), N.PYRE_MEM_HOST))
            return occ
        out = {k: np.zeros(n, np.int32) for k in ("kind", "instance", "triangle")}
        out.update({k: np.zeros(n, F32) for k in ("t", "u", "v")})
        hits = N.Hits(N.i32ptr(out["kind"]), N.i32ptr(out["instance"]), N.i32ptr(out["triangle"]), N.fptr(out["t"]),
                      N.fptr(out["u"]), N.fptr(out["v"]))
        self.check(self.lib.pyre_intersect_closest(self.handle, dscene.handle, C.byref(rays), n, C.byref(hits),
                                                   N.PYRE_MEM_HOST))
        return out

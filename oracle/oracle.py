"""ctypes wrapper of the CPU oracle (oracle/pyre_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product path. The oracle restates
the Pyre renderer's CPU path (crates/pyre) in C++; see the header of
pyre_oracle.cpp for what is pinned by the reference's own tests and what is
not.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libpyre_oracle.so"
# the same source built for the CPU it runs on (-mcpu=native / -march=native):
# the timed CPU baseline of bench.py; results are bit-identical to LIB's
LIB_NATIVE = HERE / "_build" / "libpyre_oracle_native.so"
F32 = np.float32

P_f = C.POINTER(C.c_float)
P_d = C.POINTER(C.c_double)
P_u32 = C.POINTER(C.c_uint32)
P_i32 = C.POINTER(C.c_int32)
P_u8 = C.POINTER(C.c_uint8)
P_u64 = C.POINTER(C.c_uint64)

_SIG = {
    "orc_pixel_seed": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_uint32]),
    "orc_rng_stream": (None, [C.c_uint64, C.c_uint32, P_f, P_u64]),
    "orc_rng_u64_stream": (None, [C.c_uint64, C.c_uint32, P_u64]),
    "orc_dist1d_sample": (None, [P_f, C.c_uint32, P_f, C.c_uint32, P_f, P_f, P_u32]),
    "orc_dist2d_pdf": (None, [P_f, C.c_uint32, C.c_uint32, P_f, C.c_uint32, P_f]),
    "orc_dist2d_sample": (None, [P_f, C.c_uint32, C.c_uint32, P_f, C.c_uint32, P_f, P_f]),
    "orc_bsdf_eval": (None, [P_f, P_f, P_f, C.c_uint32, P_f, P_f]),
    "orc_bsdf_sample": (None, [P_f, P_f, P_f, C.c_uint32, P_u8, P_f, P_f, P_f]),
    "orc_disney_consistency": (C.c_int, [P_f, C.c_uint64, C.c_uint32, P_f, P_f, P_f, P_f]),
    "orc_disney_draws": (None, [C.c_uint64, C.c_uint32, P_f, P_f]),
    "orc_bvh_build": (C.c_uint32, [P_f, P_u32, C.c_uint32, C.c_void_p, P_u32]),
    "orc_scene_new": (C.c_void_p, []),
    "orc_scene_free": (None, [C.c_void_p]),
    "orc_scene_add_lambertian": (C.c_int, [C.c_void_p, P_f]),
    "orc_scene_add_disney": (C.c_int, [C.c_void_p, P_f, C.c_float, C.c_float, C.c_float]),
    "orc_scene_set_material": (None, [C.c_void_p, C.c_uint32, P_f]),
    "orc_scene_add_meshes": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(P_f), P_u32, C.POINTER(P_u32), P_u32,
                                       C.POINTER(P_f), P_u32, C.POINTER(P_f), C.c_int]),
    "orc_scene_add_quad_light": (C.c_int, [C.c_void_p, P_f, P_f, P_f, P_f]),
    "orc_scene_set_env": (None, [C.c_void_p, C.c_uint32, C.c_uint32, P_f, C.c_float]),
    "orc_env_query": (None, [C.c_void_p, P_f, C.c_uint32, P_f, P_f, P_f, P_f, P_f]),
    "orc_scene_bvh_nodes": (C.c_uint32, [C.c_void_p, C.c_uint32, C.c_void_p, P_u32]),
    "orc_intersect": (None, [C.c_void_p, P_f, P_f, P_f, P_f, P_f, C.c_uint64, C.c_int, C.c_int, P_i32, P_i32, P_i32,
                             P_f, P_f, P_f, P_f]),
    "orc_occluded": (None, [C.c_void_p, P_f, P_f, P_f, P_f, P_f, C.c_uint64, C.c_int, P_u8]),
    "orc_camera_rays": (None, [P_f, C.c_uint32, C.c_uint32, P_u32, C.c_uint32, P_f, P_f, P_f]),
    "orc_render": (C.c_uint64, [C.c_void_p, P_f, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, P_f, P_f, P_f,
                                P_f, P_d]),
    "orc_render_one": (None, [C.c_void_p, P_f, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                              C.c_uint32, C.c_uint32, P_f]),
    "orc_num_threads": (C.c_int, []),
    "orc_render_grad": (None, [C.c_void_p, P_f, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P_f, P_d, C.c_int]),
}

_libs: dict = {}


def build() -> Path:
    """Compiles both builds of the oracle with its Makefile (g++, -ffp-contract=off)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def native_flags() -> str:
    """The compiler command line of the CPU-tuned build."""
    f = HERE / "_build" / "native_flags.txt"
    return f.read_text().strip() if f.exists() else ""


def lib(kind: str = "portable") -> C.CDLL:
    """The portable build (the checker) or the CPU-tuned one ("native", for timing)."""
    if kind not in _libs:
        path = {"portable": LIB, "native": LIB_NATIVE}[kind]
        if not path.exists() or path.stat().st_mtime < (HERE / "pyre_oracle.cpp").stat().st_mtime:
            build()
        L = C.CDLL(str(path))
        for k, (res, args) in _SIG.items():
            fn = getattr(L, k)
            fn.restype, fn.argtypes = res, args
        _libs[kind] = L
    return _libs[kind]


def _f(a):
    return None if a is None else a.ctypes.data_as(P_f)


def _c(a, dt=F32):
    return np.ascontiguousarray(a, dtype=dt)


def pixel_seed(x, y, s) -> int:
    return lib().orc_pixel_seed(x, y, s)


def rng_stream(seed: int, n: int):
    out = np.zeros(n, F32)
    st = np.zeros(4, np.uint64)
    lib().orc_rng_stream(seed, n, _f(out), st.ctypes.data_as(P_u64))
    return out, st


def rng_u64_stream(seed: int, n: int):
    out = np.zeros(n, np.uint64)
    lib().orc_rng_u64_stream(seed, n, out.ctypes.data_as(P_u64))
    return out


def dist1d_sample(weights, us):
    w, u = _c(weights), _c(us)
    t, pdf, b = np.zeros(u.size, F32), np.zeros(u.size, F32), np.zeros(u.size, np.uint32)
    lib().orc_dist1d_sample(_f(w), w.size, _f(u), u.size, _f(t), _f(pdf), b.ctypes.data_as(P_u32))
    return t, pdf, b


def dist2d_pdf(weights, width, height, uv):
    w, q = _c(weights), _c(uv).reshape(-1, 2)
    out = np.zeros(q.shape[0], F32)
    lib().orc_dist2d_pdf(_f(w), width, height, _f(q), q.shape[0], _f(out))
    return out


def dist2d_sample(weights, width, height, u):
    w, q = _c(weights), _c(u).reshape(-1, 2)
    uv, pdf = np.zeros_like(q), np.zeros(q.shape[0], F32)
    lib().orc_dist2d_sample(_f(w), width, height, _f(q), q.shape[0], _f(uv), _f(pdf))
    return uv, pdf


def material_params(m) -> np.ndarray:
    from pyre_gb300.scene import DisneyBsdf, Lambertian
    if isinstance(m, Lambertian):
        return np.array([0, *m.albedo, 0, 0, 0], F32)
    if isinstance(m, DisneyBsdf):
        return np.array([1, *m.base_color, m.metallic, m.roughness, m.specular], F32)
    raise TypeError(type(m))


def bsdf_eval(mat, wo, wi):
    p, a, b = material_params(mat), _c(wo).reshape(-1, 3), _c(wi).reshape(-1, 3)
    f, pdf = np.zeros_like(a), np.zeros(a.shape[0], F32)
    lib().orc_bsdf_eval(_f(p), _f(a), _f(b), a.shape[0], _f(f), _f(pdf))
    return f, pdf


def bsdf_sample(mat, wo, u):
    p, a, q = material_params(mat), _c(wo).reshape(-1, 3), _c(u).reshape(-1, 2)
    n = a.shape[0]
    ok, wi, f, pdf = np.zeros(n, np.uint8), np.zeros((n, 3), F32), np.zeros((n, 3), F32), np.zeros(n, F32)
    lib().orc_bsdf_sample(_f(p), _f(a), _f(q), n, ok.ctypes.data_as(P_u8), _f(wi), _f(f), _f(pdf))
    return ok.astype(bool), wi, f, pdf


def disney_consistency(mats, seed: int, iters: int):
    p = np.concatenate([material_params(m) for m in mats]).astype(F32)
    vals = [C.c_float() for _ in range(4)]
    n = lib().orc_disney_consistency(_f(p), seed, iters, *[C.byref(v) for v in vals])
    return n, [v.value for v in vals]


def disney_draws(seed: int, iters: int):
    """The (wo, u) inputs of the reference's Disney consistency test, 3 * iters each."""
    wo, u = np.zeros((3 * iters, 3), F32), np.zeros((3 * iters, 2), F32)
    lib().orc_disney_draws(seed, iters, _f(wo), _f(u))
    return wo, u


def bvh_build(mesh):
    from pyre_gb300.native import BVH2_DTYPE
    n = mesh.triangle_count()
    nodes = np.zeros(max(2 * n, 1), BVH2_DTYPE)
    prim = np.zeros(max(n, 1), np.uint32)
    cnt = lib().orc_bvh_build(_f(mesh.positions), mesh.indices.ctypes.data_as(P_u32), n,
                              nodes.ctypes.data_as(C.c_void_p), prim.ctypes.data_as(P_u32))
    return nodes[:cnt].copy(), prim[:n].copy()


class OracleScene:
    """The reference's Scene (scene.rs:24-34) built from a pyre_gb300.scene.Scene."""

    def __init__(self, scene, nthreads: int = 0, build: str = "portable"):
        from pyre_gb300.scene import DisneyBsdf, Lambertian
        L = self.L = lib(build)
        self.h = C.c_void_p(L.orc_scene_new())
        self.nthreads = nthreads
        for m in scene.materials:
            if isinstance(m, Lambertian):
                L.orc_scene_add_lambertian(self.h, _f(_c(m.albedo)))
            elif isinstance(m, DisneyBsdf):
                L.orc_scene_add_disney(self.h, _f(_c(m.base_color)), m.metallic, m.roughness, m.specular)
        keep = []
        n = len(scene.primitives)
        pos = (P_f * max(n, 1))()
        idx = (P_u32 * max(n, 1))()
        nor = (P_f * max(n, 1))()
        mot = (P_f * max(n, 1))()
        nv = np.zeros(max(n, 1), np.uint32)
        nt = np.zeros(max(n, 1), np.uint32)
        mid = np.zeros(max(n, 1), np.uint32)
        for k, prim in enumerate(scene.primitives):
            m = prim.instance.mesh
            keep += [m.positions, m.indices]
            pos[k] = _f(m.positions)
            idx[k] = m.indices.ctypes.data_as(P_u32)
            nv[k], nt[k], mid[k] = m.positions.shape[0], m.triangle_count(), prim.material_id
            if m.normals is not None:
                keep.append(m.normals)
                nor[k] = _f(m.normals)
            if prim.instance.motion is not None:
                mv = np.concatenate([prim.instance.motion.offset_t0, prim.instance.motion.offset_t1]).astype(F32)
                keep.append(mv)
                mot[k] = _f(mv)
        if n:
            L.orc_scene_add_meshes(self.h, n, pos, nv.ctypes.data_as(P_u32), idx, nt.ctypes.data_as(P_u32), nor,
                                   mid.ctypes.data_as(P_u32), mot, nthreads)
        for l in scene.lights:
            L.orc_scene_add_quad_light(self.h, _f(_c(l.p0)), _f(_c(l.edge_u)), _f(_c(l.edge_v)), _f(_c(l.emission)))
        if scene.env is not None:
            px = _c(scene.env.pixels)
            L.orc_scene_set_env(self.h, scene.env.width, scene.env.height, _f(px), scene.env.intensity)

    def __del__(self):
        try:
            self.L.orc_scene_free(self.h)
        except Exception:
            pass

    def bvh(self, prim: int):
        from pyre_gb300.native import BVH2_DTYPE
        n = self.L.orc_scene_bvh_nodes(self.h, prim, None, None)
        nodes = np.zeros(n, BVH2_DTYPE)
        self.L.orc_scene_bvh_nodes(self.h, prim, nodes.ctypes.data_as(C.c_void_p), None)
        return nodes

    def intersect(self, org, dirs, tmin, tmax, time=None, canonical=True, normals=False):
        org, dirs, tmin, tmax = _c(org), _c(dirs), _c(tmin), _c(tmax)
        n = tmin.size
        t_ = _c(time) if time is not None else None
        out = {k: np.zeros(n, np.int32) for k in ("kind", "instance", "triangle")}
        out.update({k: np.zeros(n, F32) for k in ("t", "u", "v")})
        if normals:
            out["normal"] = np.zeros((n, 3), F32)
        self.L.orc_intersect(self.h, _f(org), _f(dirs), _f(tmin), _f(tmax), _f(t_), n, 1 if canonical else 0,
                            self.nthreads, out["kind"].ctypes.data_as(P_i32), out["instance"].ctypes.data_as(P_i32),
                            out["triangle"].ctypes.data_as(P_i32), _f(out["t"]), _f(out["u"]), _f(out["v"]),
                            _f(out.get("normal")))
        return out

    def occluded(self, org, dirs, tmin, tmax, time=None):
        org, dirs, tmin, tmax = _c(org), _c(dirs), _c(tmin), _c(tmax)
        n = tmin.size
        t_ = _c(time) if time is not None else None
        occ = np.zeros(n, np.uint8)
        self.L.orc_occluded(self.h, _f(org), _f(dirs), _f(tmin), _f(tmax), _f(t_), n, self.nthreads,
                           occ.ctypes.data_as(P_u8))
        return occ

    def env_query(self, u):
        q = _c(u).reshape(-1, 2)
        n = q.shape[0]
        wi, li, pdf = np.zeros((n, 3), F32), np.zeros((n, 3), F32), np.zeros(n, F32)
        pdf_back, le_back = np.zeros(n, F32), np.zeros((n, 3), F32)
        self.L.orc_env_query(self.h, _f(q), n, _f(wi), _f(li), _f(pdf), _f(pdf_back), _f(le_back))
        return wi, li, pdf, pdf_back, le_back

    def render(self, camera, width, height, spp, spp_begin=0, crop=None, max_depth=8, min_rr_depth=3,
               accum64=False):
        """main.rs:253-286 over a crop; returns per-pixel means (and FP64 radiance sums)."""
        cam = camera.as_array()
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, width, height)
        cw, ch = x1 - x0, y1 - y0
        rgb, alb, nor, dep = (np.zeros((ch, cw, 3), F32), np.zeros((ch, cw, 3), F32), np.zeros((ch, cw, 3), F32),
                              np.zeros((ch, cw), F32))
        acc = np.zeros((ch, cw, 3), np.float64) if accum64 else None
        b = self.L.orc_render(self.h, _f(cam), width, height, spp_begin, spp_begin + spp, max_depth, min_rr_depth,
                             x0, y0, x1, y1, self.nthreads, _f(rgb), _f(alb), _f(nor), _f(dep),
                             acc.ctypes.data_as(P_d) if acc is not None else None)
        return {"radiance": rgb, "albedo": alb, "normal": nor, "depth": dep, "bounces": int(b), "accum64": acc}

    def render_grad(self, camera, width, height, spp, dl_di, n_materials, env_shape=None, spp_begin=0, crop=None,
                    max_depth=8, min_rr_depth=3):
        """Forward-mode (dual-number) gradient of a loss with d loss / d film = dl_di (crop h, w, 3).
        Returns (material grads (n_materials, 6), env grads (h, w, 3) or None)."""
        x0, y0, x1, y1 = crop if crop is not None else (0, 0, width, height)
        d = _c(dl_di).reshape(-1)
        n_env = 0 if env_shape is None else env_shape[0] * env_shape[1] * 3
        out = np.zeros(n_materials * 6 + n_env, np.float64)
        self.L.orc_render_grad(self.h, _f(camera.as_array()), width, height, spp_begin, spp_begin + spp, max_depth,
                              min_rr_depth, x0, y0, x1, y1, _f(d), out.ctypes.data_as(P_d), self.nthreads)
        mat = out[: n_materials * 6].reshape(n_materials, 6)
        env = out[n_materials * 6:].reshape(env_shape[0], env_shape[1], 3) if env_shape is not None else None
        return mat, env

    def render_one(self, camera, width, height, x, y, s, max_depth=8, min_rr_depth=3):
        out = np.zeros(10, F32)
        self.L.orc_render_one(self.h, _f(camera.as_array()), width, height, x, y, s, max_depth, min_rr_depth, _f(out))
        return out


def camera_rays(camera, width, height, xys):
    q = np.ascontiguousarray(xys, np.uint32).reshape(-1, 3)
    n = q.shape[0]
    o, d, t = np.zeros((n, 3), F32), np.zeros((n, 3), F32), np.zeros(n, F32)
    lib().orc_camera_rays(_f(camera.as_array()), width, height, q.ctypes.data_as(P_u32), n, _f(o), _f(d), _f(t))
    return o, d, t


def num_threads() -> int:
    return lib().orc_num_threads()


if os.environ.get("PYRE_ORACLE_THREADS"):
    os.environ.setdefault("OMP_NUM_THREADS", os.environ["PYRE_ORACLE_THREADS"])

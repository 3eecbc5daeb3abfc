"""The GPU BVH build (pyre_bvh_build_device) against the reference build on
the host (pyre_bvh_build, node-for-node equal to the oracle's restatement of
Bvh::build): the same tree, leaf ranges, split axes and primitive order, and
the same bounds (compared as floats: a min over -0.0 and +0.0 may keep either
zero)."""
import time

import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.scene import TriangleMesh, build_bvh

pytestmark = pytest.mark.gpu
F32 = np.float32


def _meshes():
    rng = np.random.default_rng(0)
    yield "icosphere L3", P.icosphere_displaced(level=3)
    yield "uv sphere", P.make_uv_sphere((0, 0, 0), 1.0, 48, 24)
    pos = rng.random((300, 3)).astype(F32)
    yield "soup", TriangleMesh(pos, rng.integers(0, 300, 900).astype(np.uint32))
    yield "coincident", TriangleMesh(np.zeros((60, 3), F32), np.arange(60, dtype=np.uint32))
    yield "clusters", TriangleMesh(np.repeat(rng.random((5, 3)).astype(F32), 12, axis=0),
                                   np.arange(60, dtype=np.uint32))
    yield "one triangle", TriangleMesh(rng.random((3, 3)).astype(F32), np.arange(3, dtype=np.uint32))
    yield "quad", P.quad_mesh([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)], (0, 0, 1))
    yield "studio sphere 32k", P.displaced_sphere((0, 0, 0), 0.5, 128, seed=3)
    yield "icosphere L8 1.3M", P.icosphere_displaced(level=8)


def _same(a, b):
    assert a.shape == b.shape, (a.shape, b.shape)
    for f in ("offset", "n_primitives", "axis"):
        assert np.array_equal(a[f], b[f]), f
    assert np.array_equal(a["bounds_min"], b["bounds_min"]) and np.array_equal(a["bounds_max"], b["bounds_max"])


@pytest.mark.parametrize("name,mesh", list(_meshes()), ids=[n for n, _ in _meshes()])
def test_device_build_matches_host_build(gpu_ctx, name, mesh):
    gpu_ctx.bvh_build(mesh)  # warm-up
    t0 = time.perf_counter()
    dn, dp = gpu_ctx.bvh_build(mesh)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    hn, hp = build_bvh(mesh)
    t_host = time.perf_counter() - t0
    print({"mesh": name, "triangles": mesh.triangle_count(), "nodes": int(dn.shape[0]),
           "device_ms": round(t_dev * 1e3, 2), "host_ms": round(t_host * 1e3, 2)})
    _same(dn, hn)
    assert np.array_equal(dp, hp)


def test_device_built_scene_gives_the_same_hits_and_films(gpu_ctx, oracle_mod):
    """pyre_scene_upload with the device builder: every mesh BVH, node and
    triangle record comes from the GPU build; hits and films are bit-identical
    to the host-built scene and hits match the oracle."""
    from pyre_gb300.scene import PathIntegrator
    sc = P.studio_procedural(n_side=3, segments=24, n_moving=2, hdri_size=(256, 128))
    cam = P.studio_procedural_camera(64, 48)
    try:
        gpu_ctx.set_bvh_builder("device")
        dev = gpu_ctx.upload(sc)
    finally:
        gpu_ctx.set_bvh_builder("host")
    host = gpu_ctx.upload(sc)
    assert dev.info().n_nodes == host.info().n_nodes
    rng = np.random.default_rng(7)
    org = (rng.random((50_000, 3)) * 4 - 2).astype(F32)
    d = rng.normal(size=(50_000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    tmin, tmax = np.full(50_000, 1e-4, F32), np.full(50_000, np.inf, F32)
    a, b = gpu_ctx.intersect(dev, org, d, tmin, tmax), gpu_ctx.intersect(host, org, d, tmin, tmax)
    for k in ("kind", "instance", "triangle", "t", "u", "v"):
        assert np.array_equal(a[k], b[k]), k
    r = oracle_mod.OracleScene(sc).intersect(org, d, tmin, tmax)
    assert np.array_equal(a["triangle"], r["triangle"]) and np.array_equal(a["instance"], r["instance"])
    it = PathIntegrator(8, 3)
    fa, fb = gpu_ctx.render(dev, cam, it, 64, 48, 4), gpu_ctx.render(host, cam, it, 64, 48, 4)
    assert np.array_equal(fa.radiance, fb.radiance) and np.array_equal(fa.depth, fb.depth)
    dev.close()
    host.close()


def test_device_built_batch_scene(gpu_ctx):
    jobs = P.batch_jobs(n_jobs=6, seed=5, resolutions=(32, 48), spps=(1, 2), tri_range=(10, 3000))
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    try:
        gpu_ctx.set_bvh_builder("device")
        dev = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    finally:
        gpu_ctx.set_bvh_builder("host")
    host = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    for fa, fb in zip(gpu_ctx.render_batch(dev, spec), gpu_ctx.render_batch(host, spec)):
        assert np.array_equal(fa.radiance, fb.radiance)
    dev.close()
    host.close()

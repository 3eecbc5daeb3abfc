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

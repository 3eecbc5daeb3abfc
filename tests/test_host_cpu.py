"""CPU-only checks of the product library and host logic (no GPU calls).

* libpyre_cuda.so loads without a GPU and exports every function that
  include/pyre_cuda.h declares;
* the library's host BVH builder (pyre_bvh_build) equals the oracle's
  restatement of Bvh::build node for node;
* the Python mirror of pixel_seed equals the oracle's.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from pyre_gb300 import native as N
from pyre_gb300 import presets as P
from pyre_gb300.scene import TriangleMesh, build_bvh, pixel_seed

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from pyre_gb300 import build as B
    B.build()
    return N.load()


def header_functions():
    text = (ROOT / "include" / "pyre_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pyre_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    names = header_functions()
    assert "pyre_render" in names and "pyre_scene_upload" in names
    for name in names:
        assert hasattr(lib, name), f"{name} declared in pyre_cuda.h but not exported"
        assert name in N.SIGNATURES, f"{name} missing from the ctypes signature table"
    assert lib.pyre_version() == 1


def test_ctx_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.pyre_ctx_create(0, C.byref(h))
    assert rc != N.PYRE_OK and not h.value
    assert lib.pyre_last_error(None)


def test_node_layout():
    assert C.sizeof(N.Bvh2Node) == 32
    assert C.sizeof(N.RenderParams) == 4 * 19


@pytest.mark.parametrize("mesh_fn", [
    lambda: P.icosphere_displaced(level=4),
    lambda: P.make_uv_sphere((0.1, 0.2, 0.3), 0.5, 48, 24),
    lambda: P.displaced_sphere((0, 0, 0), 1.0, 32, seed=5),
    lambda: TriangleMesh(np.array([[-1, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.arange(3, dtype=np.uint32)),
    # coincident centroids: one leaf of many primitives (bvh.rs:205-208)
    lambda: TriangleMesh(np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (20, 1)),
                         np.arange(60, dtype=np.uint32)),
    # two stacked triangles (mesh.rs:213-234)
    lambda: TriangleMesh(np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [-1, -1, -1], [1, -1, -1], [0, 1, -1]],
                                  np.float32), np.arange(6, dtype=np.uint32)),
], ids=["icosphere4", "uvsphere", "displaced", "single", "coincident", "two"])
def test_bvh_builder_matches_oracle(lib, oracle_mod, mesh_fn):
    mesh = mesh_fn()
    nodes, prim = build_bvh(mesh)
    onodes, oprim = oracle_mod.bvh_build(mesh)
    assert nodes.shape == onodes.shape
    assert np.array_equal(nodes.view(np.uint8), onodes.view(np.uint8)), "node arrays differ"
    assert np.array_equal(prim, oprim)


def test_bvh_build_rejects_bad_indices(lib):
    pos = np.zeros((3, 3), np.float32)
    idx = np.array([0, 1, 7], np.uint32)
    nodes = np.zeros(2, N.BVH2_DTYPE)
    prim = np.zeros(1, np.uint32)
    cnt = C.c_uint32()
    rc = lib.pyre_bvh_build(N.fptr(pos), 3, N.u32ptr(idx), 1, nodes.ctypes.data_as(C.POINTER(N.Bvh2Node)),
                            N.u32ptr(prim), C.byref(cnt))
    assert rc == N.PYRE_ERR_INVALID


def test_pixel_seed_python_matches_oracle(oracle_mod):
    rng = np.random.default_rng(0)
    for x, y, s in rng.integers(0, 1 << 16, size=(200, 3)):
        assert pixel_seed(int(x), int(y), int(s)) == oracle_mod.pixel_seed(int(x), int(y), int(s))
    assert pixel_seed(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF) == oracle_mod.pixel_seed(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF)

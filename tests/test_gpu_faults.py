"""Error paths without faulting the GPU: injected allocation failures (host
side, pyre_inject_alloc_failure) and a traversal that runs out of stack on a
valid but degenerate caller BVH. Each failing call returns its status and
the context keeps working."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.native import BVH2_DTYPE, PYRE_ERR_OOM, PYRE_ERR_OVERFLOW, PyreError
from pyre_gb300.scene import Lambertian, MeshInstance, PathIntegrator, Primitive, Scene, TriangleMesh

pytestmark = pytest.mark.gpu


def test_injected_allocation_failures(gpu_ctx):
    # a context of its own: how large the shared context's workspace has grown depends on the tests before
    from pyre_gb300.scene import CudaIntegrator
    ctx = CudaIntegrator(0)
    try:
        sc, it = P.cornell_ref(), PathIntegrator(8, 3)
        ds = ctx.upload(sc)
        small = ctx.render(ds, P.cornell_ref_camera(32, 24), it, 32, 24, 2)
        # a larger render needs a larger workspace: its allocation fails
        ctx.lib.pyre_inject_alloc_failure(ctx.handle, 0)
        with pytest.raises(PyreError) as e:
            ctx.render(ds, P.cornell_ref_camera(640, 480), it, 640, 480, 4)
        assert e.value.code == PYRE_ERR_OOM
        again = ctx.render(ds, P.cornell_ref_camera(32, 24), it, 32, 24, 2)
        np.testing.assert_array_equal(again.radiance, small.radiance)
        # a scene upload that fails part-way frees what it had allocated
        for after in (0, 2, 5):
            ctx.lib.pyre_inject_alloc_failure(ctx.handle, after)
            with pytest.raises(PyreError) as e:
                ctx.upload(sc)
            assert e.value.code == PYRE_ERR_OOM
        ctx.lib.pyre_inject_alloc_failure(ctx.handle, -1)
        ds2 = ctx.upload(sc)
        np.testing.assert_array_equal(ctx.render(ds2, P.cornell_ref_camera(32, 24), it, 32, 24, 2).radiance,
                                      small.radiance)
        ds.close()
        ds2.close()
    finally:
        ctx.lib.pyre_inject_alloc_failure(ctx.handle, -1)
        ctx.close()


def _deep_bvh(levels: int):
    """A valid reference-layout BVH whose every level has two interior
    children with the same box: a nearest-first traversal continues down the
    left chain and pushes the right child at each level."""
    nodes, prims = [], [0]
    box = ([-1.0, -1.0, -1.0], [1.0, 1.0, 1.0])

    def add(offset, count):
        nodes.append((box[0], box[1], offset, count, 0, 0))
        return len(nodes) - 1

    def leaf():
        i = add(prims[0], 1)
        prims[0] += 1
        return i

    def small():
        i = add(0, 0)
        leaf()
        r = leaf()
        nodes[i] = (box[0], box[1], r, 0, 0, 0)
        return i

    def chain(level):
        i = add(0, 0)
        if level == levels:
            nodes[i] = (box[0], box[1], prims[0], 1, 0, 0)
            prims[0] += 1
            return i
        chain(level + 1)
        r = small()
        nodes[i] = (box[0], box[1], r, 0, 0, 0)
        return i

    chain(0)
    arr = np.zeros(len(nodes), BVH2_DTYPE)
    for k, (lo, hi, off, cnt, axis, pad) in enumerate(nodes):
        arr[k] = (lo, hi, off, cnt, axis, pad)
    return arr, prims[0]


def test_traversal_stack_overflow_is_reported(gpu_ctx):
    nodes, n = _deep_bvh(80)
    rng = np.random.default_rng(0)
    pos = (rng.random((3 * n, 3)) * 0.2 + 0.7).astype(np.float32)  # small triangles near (0.8, 0.8, 0.8)
    mesh = TriangleMesh(pos, np.arange(3 * n, dtype=np.uint32))
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    sc.primitives.append(Primitive(MeshInstance(mesh, None, nodes, np.arange(n, dtype=np.uint32)), 0))
    ds = gpu_ctx.upload(sc)
    org = np.zeros((64, 3), np.float32)
    d = np.tile(np.float32([1.0, 0.0, 0.0]), (64, 1))
    tmin, tmax = np.full(64, 1e-4, np.float32), np.full(64, np.inf, np.float32)
    with pytest.raises(PyreError) as e:
        gpu_ctx.intersect(ds, org, d, tmin, tmax)
    assert e.value.code == PYRE_ERR_OVERFLOW
    # the flag is cleared: a scene of ordinary depth works on the same context
    ok = gpu_ctx.upload(P.cornell_box())
    out = gpu_ctx.intersect(ok, org, d, tmin, tmax)
    assert (out["kind"] > 0).all()
    ds.close()
    ok.close()

"""GPU ray queries vs the CPU oracle: hit identity bit-exact, t/u/v bit-exact.

The oracle uses the canonical tie rule (min t, then lowest instance, then
lowest triangle), which the kernels implement; the reference's own traversal
order only differs on exact ties in t.
"""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.scene import DisneyBsdf, InstanceMotion, Lambertian, MeshInstance, Primitive, Scene

pytestmark = pytest.mark.gpu


def _compare(gpu, ref, label):
    assert np.array_equal(gpu["kind"], ref["kind"]), f"{label}: hit/miss/light kind differs"
    assert np.array_equal(gpu["instance"], ref["instance"]), f"{label}: instance ids differ"
    assert np.array_equal(gpu["triangle"], ref["triangle"]), f"{label}: triangle ids differ"
    hit = ref["kind"] > 0
    for k in ("t", "u", "v"):
        a, b = gpu[k][hit], ref[k][hit]
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), \
            f"{label}: {k} not bit-exact, max rel {np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30))}"


@pytest.mark.parametrize("width", [2, 4, 8])
def test_icosphere_closest_and_any(gpu_ctx, oracle_mod, width):
    sc = P.microbench_scene(level=6)
    org, d, tmin, tmax = P.random_rays(sc.primitives[0].instance.mesh, 300_000, seed=1)
    ds = gpu_ctx.upload(sc)
    ds.set_bvh_width(width)
    g = gpu_ctx.intersect(ds, org, d, tmin, tmax)
    osc = oracle_mod.OracleScene(sc)
    r = osc.intersect(org, d, tmin, tmax, canonical=True)
    assert (r["kind"] > 0).mean() > 0.2
    _compare(g, r, "icosphere L6")
    occ = gpu_ctx.intersect(ds, org, d, tmin, tmax, any_hit=True)
    assert np.array_equal(occ, osc.occluded(org, d, tmin, tmax))


def test_reference_tie_rule_agrees(oracle_mod):
    """The reference's visit-order rule and the canonical rule pick the same hits here."""
    sc = P.microbench_scene(level=5)
    org, d, tmin, tmax = P.random_rays(sc.primitives[0].instance.mesh, 100_000, seed=3)
    osc = oracle_mod.OracleScene(sc)
    a = osc.intersect(org, d, tmin, tmax, canonical=True)
    b = osc.intersect(org, d, tmin, tmax, canonical=False)
    assert (a["triangle"] != b["triangle"]).mean() < 1e-4


def _rays_in_box(n, lo, hi, seed, tmax=np.inf):
    rng = np.random.default_rng(seed)
    org = (lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return org, d, np.full(n, 1e-4, np.float32), np.full(n, tmax, np.float32)


@pytest.mark.parametrize("width", [2, 4, 8])
@pytest.mark.parametrize("name", ["cornell_box", "cornell_ref"])
def test_cornell_scenes(gpu_ctx, oracle_mod, name, width):
    sc = getattr(P, name)()
    org, d, tmin, tmax = _rays_in_box(200_000, np.float32(-0.99), np.float32(0.99), seed=5)
    ds = gpu_ctx.upload(sc)
    ds.set_bvh_width(width)
    g = gpu_ctx.intersect(ds, org, d, tmin, tmax)
    osc = oracle_mod.OracleScene(sc)
    r = osc.intersect(org, d, tmin, tmax)
    assert (r["kind"] == 2).sum() > 0, "some rays should reach the quad light"
    _compare(g, r, name)
    # finite t_max, as shadow rays use
    tm = np.full(org.shape[0], 0.7, np.float32)
    assert np.array_equal(gpu_ctx.intersect(ds, org, d, np.full_like(tm, 1e-3), tm, any_hit=True),
                          osc.occluded(org, d, np.full_like(tm, 1e-3), tm))


def _axis_rays():
    """Origins on a grid whose values include the Cornell box's node planes (the walls at +-1), and directions
    with zero components of either sign, so that 1/d is +inf or -inf and (plane - origin) * (1/d) is 0 * inf."""
    vals = np.array([-1.0, -0.999, -0.5, -0.125, -0.0, 0.0, 0.125, 0.3, 0.999, 1.0], np.float32)
    org = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    dirs = []
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        for s in (1.0, -1.0):
            for zb in (0.0, -0.0):
                for zc in (0.0, -0.0):
                    d = [0.0] * 3
                    d[a], d[b], d[c] = s, zb, zc
                    dirs.append(d)
        for sa in (0.6, -0.6):
            for sb in (0.8, -0.8):
                for zc in (0.0, -0.0):
                    d = [0.0] * 3
                    d[a], d[b], d[c] = sa, sb, zc
                    dirs.append(d)
    dirs = np.array(dirs, np.float32)
    o = np.repeat(org, len(dirs), axis=0)
    d = np.tile(dirs, (len(org), 1))
    return np.ascontiguousarray(o), np.ascontiguousarray(d)


@pytest.mark.parametrize("width", [2, 4, 8])
def test_axis_aligned_rays_on_node_planes(gpu_ctx, oracle_mod, width):
    """Rays that make the slab test (bvh.rs:146-153) multiply 0 by an infinity: its min / max reductions then
    see NaN operands, which Rust's f32::min / f32::max (and the kernels' min / max) ignore. Hits, t/u/v and
    occlusion answers must be the oracle's, closest hit and any hit."""
    sc = P.cornell_box()
    org, d = _axis_rays()
    assert np.signbit(d).any() and (d == 0).any()
    n = org.shape[0]
    tmin, tmax = np.full(n, 1e-4, np.float32), np.full(n, np.inf, np.float32)
    ds = gpu_ctx.upload(sc)
    ds.set_bvh_width(width)
    osc = oracle_mod.OracleScene(sc)
    r = osc.intersect(org, d, tmin, tmax)
    assert (r["kind"] > 0).mean() > 0.5
    _compare(gpu_ctx.intersect(ds, org, d, tmin, tmax), r, "axis-aligned")
    for t_hi in (0.5, 1.0, np.inf):
        tm = np.full(n, t_hi, np.float32)
        assert np.array_equal(gpu_ctx.intersect(ds, org, d, tmin, tm, any_hit=True), osc.occluded(org, d, tmin, tm))


@pytest.mark.parametrize("width", [2, 4, 8])
def test_motion_blur_instances(gpu_ctx, oracle_mod, width):
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    for k in range(6):
        m = P.make_uv_sphere((k * 0.5 - 1.25, 0.0, 0.0), 0.3, 24, 12)
        mot = InstanceMotion((0, 0, 0), (0.0, 0.4 * (k % 3) - 0.4, 0.2)) if k % 2 == 0 else None
        sc.primitives.append(Primitive(MeshInstance(m, mot), 0))
    org, d, tmin, tmax = _rays_in_box(200_000, np.array([-2, -1, -1], np.float32), np.array([2, 1, 1], np.float32), 9)
    time = np.random.default_rng(2).random(org.shape[0]).astype(np.float32)
    ds = gpu_ctx.upload(sc)
    ds.set_bvh_width(width)
    g = gpu_ctx.intersect(ds, org, d, tmin, tmax, time=time)
    r = oracle_mod.OracleScene(sc).intersect(org, d, tmin, tmax, time=time)
    _compare(g, r, "motion")


def test_caller_supplied_bvh_matches(gpu_ctx, oracle_mod):
    """A BVH handed over by the host (Bvh::nodes layout) gives the same hits."""
    mesh = P.icosphere_displaced(level=4)
    nodes, prim = oracle_mod.bvh_build(mesh)
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    sc.primitives.append(Primitive(MeshInstance(mesh, None, nodes, prim), 0))
    org, d, tmin, tmax = P.random_rays(mesh, 50_000, seed=4)
    g = gpu_ctx.intersect(gpu_ctx.upload(sc), org, d, tmin, tmax)
    r = oracle_mod.OracleScene(sc).intersect(org, d, tmin, tmax)
    _compare(g, r, "caller BVH")


@pytest.mark.parametrize("width", [2, 4, 8])
def test_empty_and_degenerate(gpu_ctx, oracle_mod, width):
    sc = Scene()
    sc.materials.append(DisneyBsdf([0.5] * 3, 0.0, 0.5))
    # degenerate (zero-area) triangles and coincident centroids
    pos = np.zeros((30, 3), np.float32)
    pos[:, 0] = np.repeat(np.arange(10, dtype=np.float32), 3) * 0.0
    from pyre_gb300.scene import TriangleMesh
    sc.primitives.append(Primitive(MeshInstance(TriangleMesh(pos, np.arange(30, dtype=np.uint32))), 0))
    sc.primitives.append(Primitive(MeshInstance(P.make_uv_sphere((0, 0, 0), 0.5, 8, 4)), 0))
    org, d, tmin, tmax = _rays_in_box(20_000, np.float32(-1), np.float32(1), 11)
    ds = gpu_ctx.upload(sc)
    ds.set_bvh_width(width)
    _compare(gpu_ctx.intersect(ds, org, d, tmin, tmax), oracle_mod.OracleScene(sc).intersect(org, d, tmin, tmax),
             "degenerate")
    # zero rays
    z = np.zeros((0, 3), np.float32)
    out = gpu_ctx.intersect(ds, z, z, np.zeros(0, np.float32), np.zeros(0, np.float32))
    assert out["kind"].size == 0


def test_bvh_width_rejects_bad_values(gpu_ctx):
    ds = gpu_ctx.upload(P.cornell_box())
    from pyre_gb300.native import PyreError
    for w in (0, 3, 16):
        with pytest.raises(PyreError):
            ds.set_bvh_width(w)


def test_microbenchmark_full_size_bit_exact(gpu_ctx, oracle_mod):
    """The ray-intersection microbenchmark at its own size: the level-8 displaced icosphere (1,310,720
    triangles, radial value noise of amplitude 0.1) and 16,777,216 rays from seed 1 (origins uniform in the
    mesh box scaled 1.5x, directions uniform on the sphere). Closest hit: kind, instance, triangle and the bits
    of t, u and v equal the oracle's (mesh.rs:153-178 on the BVH of bvh.rs:86-153, canonical tie rule); any
    hit equals Scene::occluded (scene.rs:120-140) for every ray."""
    sc = P.microbench_scene(level=8)
    mesh = sc.primitives[0].instance.mesh
    assert mesh.triangle_count() == 1_310_720
    org, d, tmin, tmax = P.random_rays(mesh, 16_777_216, seed=1)
    ds = gpu_ctx.upload(sc)
    g = gpu_ctx.intersect(ds, org, d, tmin, tmax)
    osc = oracle_mod.OracleScene(sc)
    r = osc.intersect(org, d, tmin, tmax, canonical=True)
    assert 0.2 < (r["kind"] > 0).mean() < 0.5
    _compare(g, r, "microbenchmark 1.31M triangles x 16.8M rays")
    del g, r
    occ = gpu_ctx.intersect(ds, org, d, tmin, tmax, any_hit=True)
    assert np.array_equal(occ, osc.occluded(org, d, tmin, tmax))
    ds.close()

"""Edge cases of the render path against the oracle: shallow depths, scenes
with only an environment or no light at all, large sample indices, one-pixel
images and crops, and parameters the library must reject."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.native import PYRE_ENV_CDF, PyreError
from pyre_gb300.scene import HdriEnvironmentLight, Lambertian, MeshInstance, PathIntegrator, Primitive, Scene

pytestmark = pytest.mark.gpu


def relmse(x, r):
    return float(np.mean(np.sum((x - r) ** 2 / (r ** 2 + 1e-2), axis=-1)))


@pytest.mark.parametrize("max_depth", [1, 2, 3])
def test_shallow_depths(gpu_ctx, oracle_mod, max_depth):
    sc, cam = P.studio_ref(), P.studio_ref_camera(48, 32)
    ds = gpu_ctx.upload(sc)
    film = gpu_ctx.render(ds, cam, PathIntegrator(max_depth, 3), 48, 32, 8, env_sampling=PYRE_ENV_CDF)
    ref = oracle_mod.OracleScene(sc).render(cam, 48, 32, 8, max_depth=max_depth)
    assert relmse(film.radiance, ref["radiance"]) < 1e-2
    np.testing.assert_allclose(film.depth, ref["depth"], rtol=1e-3, atol=1e-3)


def test_zero_depth_is_all_zeros(gpu_ctx):
    """max_depth 0 runs no bounce (integrator.rs:75): every channel of every
    sample is zero, also for a job of that depth inside a batch."""
    sc, cam = P.studio_ref(), P.studio_ref_camera(40, 24)
    ds = gpu_ctx.upload(sc)
    film = gpu_ctx.render(ds, cam, PathIntegrator(0, 3), 40, 24, 4)
    for ch in (film.radiance, film.albedo, film.normal, film.depth):
        assert not np.any(ch)
    ds.close()
    jobs = P.batch_jobs(n_jobs=3, seed=9, resolutions=(32,), spps=(2,), tri_range=(10, 500))
    jobs[1]["integrator"] = PathIntegrator(0, 3)
    db = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    films = gpu_ctx.render_batch(db, spec)
    for ch in (films[1].radiance, films[1].albedo, films[1].normal, films[1].depth):
        assert not np.any(ch)
    assert np.any(films[0].radiance) and np.any(films[2].radiance)
    db.close()


def test_environment_only_scene(gpu_ctx, oracle_mod):
    sc = Scene()
    sc.env = HdriEnvironmentLight.gradient((0.2, 0.35, 0.65), (0.95, 0.85, 0.7), 1.5)
    cam = P.studio_ref_camera(40, 30)
    ds = gpu_ctx.upload(sc)
    film = gpu_ctx.render(ds, cam, PathIntegrator(8, 3), 40, 30, 4, env_sampling=PYRE_ENV_CDF)
    ref = oracle_mod.OracleScene(sc).render(cam, 40, 30, 4)
    np.testing.assert_allclose(film.radiance, ref["radiance"], rtol=1e-5, atol=1e-6)
    assert np.all(film.depth == 0) and np.all(film.albedo == 0)


def test_scene_without_light_is_black(gpu_ctx, oracle_mod):
    sc = Scene()
    sc.materials.append(Lambertian([0.5, 0.5, 0.5]))
    sc.primitives.append(Primitive(MeshInstance.build(P.make_uv_sphere((0, 0, 0), 0.6, 24, 12)), 0))
    cam = P.cornell_box_camera(32, 32)
    ds = gpu_ctx.upload(sc)
    film = gpu_ctx.render(ds, cam, PathIntegrator(8, 3), 32, 32, 2)
    ref = oracle_mod.OracleScene(sc).render(cam, 32, 32, 2)
    assert np.all(film.radiance == 0) and np.all(ref["radiance"] == 0)
    np.testing.assert_allclose(film.depth, ref["depth"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(film.albedo, ref["albedo"], atol=1e-6)


def test_large_sample_index_and_one_pixel(gpu_ctx, oracle_mod):
    sc, cam = P.cornell_ref(), P.cornell_ref_camera(1, 1)
    ds = gpu_ctx.upload(sc)
    osc = oracle_mod.OracleScene(sc)
    a = gpu_ctx.render(ds, cam, PathIntegrator(8, 3), 1, 1, 64, spp_begin=(1 << 31) - 64)
    b = osc.render(cam, 1, 1, 64, spp_begin=(1 << 31) - 64)
    assert relmse(a.radiance, b["radiance"]) < 1e-2
    cam2 = P.cornell_ref_camera(37, 23)
    whole = gpu_ctx.render(ds, cam2, PathIntegrator(8, 3), 37, 23, 3)
    corner = gpu_ctx.render(ds, cam2, PathIntegrator(8, 3), 37, 23, 3, crop=(36, 22, 37, 23))
    np.testing.assert_array_equal(corner.radiance[0, 0], whole.radiance[22, 36])


@pytest.mark.parametrize("kw,match", [
    ({"width": 0}, "size"),
    ({"spp": 0}, "sample range"),
    ({"crop": (0, 0, 40, 10)}, "crop"),
    ({"crop": (5, 5, 5, 8)}, "crop"),
    ({"integrator": PathIntegrator(65, 3)}, "max_depth"),
])
def test_invalid_parameters_are_rejected(gpu_ctx, kw, match):
    sc, cam = P.cornell_ref(), P.cornell_ref_camera(32, 16)
    ds = gpu_ctx.upload(sc)
    args = dict(width=32, height=16, spp=1, integrator=PathIntegrator(8, 3), crop=None)
    args.update(kw)
    with pytest.raises(PyreError, match=match):
        gpu_ctx.render(ds, cam, args["integrator"], args["width"], args["height"], args["spp"], crop=args["crop"])


def test_crop_area_above_2_31_is_rejected_before_any_work(gpu_ctx):
    """A 65536 x 65536 crop has 2^32 pixels, which wraps a 32-bit product to 0: every entry point must reject
    it from the 64-bit pixel count with PYRE_ERR_INVALID (the buffers passed are tiny: nothing may be written)."""
    import ctypes as C

    from pyre_gb300 import native as N
    from pyre_gb300.scene import CudaIntegrator
    sc, cam = P.cornell_box(), P.cornell_box_camera(65536, 65536)
    ds = gpu_ctx.upload(sc)
    lib, h = gpu_ctx.lib, gpu_ctx.handle
    desc = cam.to_desc()
    params = CudaIntegrator.params(65536, 65536, 0, 1, PathIntegrator(8, 3))
    buf = np.zeros(16, np.float32)
    hfilm = N.Film(N.fptr(buf), None, None, None, N.PYRE_MEM_HOST)
    calls = {
        "pyre_render": lambda: lib.pyre_render(h, ds.handle, C.byref(desc), C.byref(params), C.byref(hfilm)),
        "pyre_forward": lambda: lib.pyre_forward(h, ds.handle, C.byref(desc), C.byref(params), C.byref(hfilm)),
        "pyre_render_progressive": lambda: lib.pyre_render_progressive(h, ds.handle, C.byref(desc), C.byref(params),
                                                                       N.fptr(buf), N.PYRE_MEM_HOST),
        "pyre_backward": lambda: lib.pyre_backward(
            h, ds.handle, C.byref(desc), C.byref(params), N.fptr(buf), N.PYRE_MEM_HOST,
            C.byref(N.Gradients(None, None, N.PYRE_MEM_HOST))),
    }
    import torch
    dbuf = torch.zeros(16, dtype=torch.float32, device="cuda")
    dfilm = N.Film(N.dptr(dbuf), None, None, None, N.PYRE_MEM_DEVICE)
    calls["pyre_render_noalloc"] = lambda: lib.pyre_render_noalloc(h, ds.handle, C.byref(desc), C.byref(params),
                                                                   C.byref(dfilm))
    for name, call in calls.items():
        assert call() == N.PYRE_ERR_INVALID, name
        assert b"2^31" in lib.pyre_last_error(h), (name, lib.pyre_last_error(h))
    # the same crop as a batch job
    db = gpu_ctx.upload_batch([sc])
    job = N.BatchJob()
    job.part, job.camera, job.width, job.height = 0, desc, 65536, 65536
    job.spp_begin, job.spp_end, job.max_depth, job.min_rr_depth = 0, 1, 8, 3
    job.film = hfilm
    assert lib.pyre_render_batch(h, db.handle, C.byref(job), 1, C.byref(params)) == N.PYRE_ERR_INVALID
    assert b"2^31" in lib.pyre_last_error(h)
    # the context is still usable
    film = gpu_ctx.render(ds, P.cornell_box_camera(8, 8), PathIntegrator(8, 3), 8, 8, 1)
    assert np.isfinite(film.radiance).all()
    db.close()
    ds.close()


def test_unknown_sort_kind_is_rejected(gpu_ctx):
    """sort_by_material takes 0 (the call's default), 1 (within tiles), 2 (off) and 3 (the whole queue)."""
    from pyre_gb300 import native as N
    from pyre_gb300.scene import Film
    sc, cam = P.cornell_ref(), P.cornell_ref_camera(32, 16)
    ds = gpu_ctx.upload(sc)
    film = Film(32, 16)
    f = N.Film(N.fptr(film.radiance), N.fptr(film.albedo), N.fptr(film.normal), N.fptr(film.depth), N.PYRE_MEM_HOST)
    p = gpu_ctx.params(32, 16, 0, 1, PathIntegrator(8, 3))
    p.sort_by_material = 4
    with pytest.raises(PyreError, match="sort_by_material"):
        gpu_ctx.render_into(ds, cam, p, f)
    ds.close()

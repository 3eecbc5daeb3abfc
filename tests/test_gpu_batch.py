"""Batched rendering: every job's film equals rendering that job alone.

The batch packs all jobs' (pixel, sample) paths into shared waves; each job's
samples still reach its film in sample order, so films are bit-identical to
single renders, with or without CUDA-graph replay.
"""
import numpy as np
import pytest

from pyre_gb300 import presets as P

pytestmark = pytest.mark.gpu


def _jobs():
    return P.batch_jobs(n_jobs=7, seed=5, resolutions=(32, 48, 64), spps=(1, 3, 4), tri_range=(10, 3000))


# sort: 0 = the default (unsorted), 1 = sorted by material within tiles, 2 = unsorted, 3 = the whole queue sorted
@pytest.mark.parametrize("use_graph,sort,width", [(0, 0, 2), (1, 2, 2), (0, 1, 2), (1, 3, 4), (0, 0, 8)])
@pytest.mark.parametrize("wave_paths", [0, 9000])
def test_batch_matches_single_renders(gpu_ctx, use_graph, sort, width, wave_paths):
    jobs = _jobs()
    ds = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    films = gpu_ctx.render_batch(ds, spec, wave_paths=wave_paths, use_graph=use_graph, sort_by_material=sort,
                                 bvh_width=width)
    st = gpu_ctx.stats()
    assert st.samples == sum(j["width"] * j["height"] * j["spp"] for j in jobs)
    if wave_paths:
        assert st.waves > 1
    for j, film in zip(jobs, films):
        single_scene = gpu_ctx.upload(j["scene"])
        ref = gpu_ctx.render(single_scene, j["camera"], j["integrator"], j["width"], j["height"], j["spp"])
        np.testing.assert_array_equal(film.radiance, ref.radiance)
        np.testing.assert_array_equal(film.albedo, ref.albedo)
        np.testing.assert_array_equal(film.depth, ref.depth)
        single_scene.close()
    ds.close()


def test_batch_matches_oracle(gpu_ctx, oracle_mod):
    jobs = _jobs()[:3]
    ds = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    films = gpu_ctx.render_batch(ds, spec)
    for j, film in zip(jobs, films):
        it = j["integrator"]
        ref = oracle_mod.OracleScene(j["scene"]).render(j["camera"], j["width"], j["height"], j["spp"],
                                                        max_depth=it.max_depth, min_rr_depth=it.min_rr_depth)
        e = float(np.mean(np.sum((film.radiance - ref["radiance"]) ** 2 / (ref["radiance"] ** 2 + 1e-2), -1)))
        assert e < 1e-2
    ds.close()


def test_batch_rejects_bad_part(gpu_ctx):
    jobs = _jobs()[:2]
    ds = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    spec = [{"part": 5, "camera": jobs[0]["camera"], "width": 8, "height": 8, "spp": 1}]
    from pyre_gb300.native import PyreError
    with pytest.raises(PyreError):
        gpu_ctx.render_batch(ds, spec)
    ds.close()


@pytest.mark.parametrize("use_graph", [0, 1])
def test_batch_device_films_and_missing_channels(gpu_ctx, use_graph):
    """Films in device memory (copied on the library's second stream while later waves render) and films with
    some channels left NULL get the same bits as host films, over several waves."""
    import ctypes as C

    import torch

    from pyre_gb300 import native as N
    jobs = _jobs()
    ds = gpu_ctx.upload_batch([j["scene"] for j in jobs])
    spec = [{"part": k, "camera": j["camera"], "width": j["width"], "height": j["height"], "spp": j["spp"],
             "integrator": j["integrator"]} for k, j in enumerate(jobs)]
    ref = gpu_ctx.render_batch(ds, spec, wave_paths=9000)
    dev, cjobs = [], []
    for k, j in enumerate(jobs):
        npix = j["width"] * j["height"]
        t = {c: torch.full((npix * n,), -1.0, dtype=torch.float32, device="cuda")
             for c, n in (("radiance", 3), ("albedo", 3), ("normal", 3), ("depth", 1))}
        dev.append(t)
        b = N.BatchJob()
        b.part, b.camera = k, j["camera"].to_desc()
        b.width, b.height, b.spp_begin, b.spp_end = j["width"], j["height"], 0, j["spp"]
        b.max_depth, b.min_rr_depth = j["integrator"].max_depth, j["integrator"].min_rr_depth
        # odd jobs leave albedo and normal out
        skip = k % 2 == 1
        b.film = N.Film(N.dptr(t["radiance"]), None if skip else N.dptr(t["albedo"]),
                        None if skip else N.dptr(t["normal"]), N.dptr(t["depth"]), N.PYRE_MEM_DEVICE)
        cjobs.append(b)
    arr = (N.BatchJob * len(cjobs))(*cjobs)
    p = N.RenderParams()
    p.wave_paths, p.use_graph = 9000, use_graph
    gpu_ctx.check(gpu_ctx.lib.pyre_render_batch(gpu_ctx.handle, ds.handle, arr, len(cjobs), C.byref(p)))
    assert gpu_ctx.stats().waves > 1
    for k, (t, f) in enumerate(zip(dev, ref)):
        np.testing.assert_array_equal(t["radiance"].cpu().numpy().reshape(f.radiance.shape), f.radiance)
        np.testing.assert_array_equal(t["depth"].cpu().numpy().reshape(f.depth.shape), f.depth)
        if k % 2 == 1:
            assert bool((t["albedo"] == -1.0).all()) and bool((t["normal"] == -1.0).all())
        else:
            np.testing.assert_array_equal(t["albedo"].cpu().numpy().reshape(f.albedo.shape), f.albedo)
            np.testing.assert_array_equal(t["normal"].cpu().numpy().reshape(f.normal.shape), f.normal)
    ds.close()

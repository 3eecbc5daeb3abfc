"""pyre_render_noalloc: rendering for callers that cannot call cudaMalloc.

Some hosts own all GPU memory through their own allocator, or run a frame
loop that must not stall the device, so they cannot let the renderer allocate
while it renders. pyre_render_noalloc keeps its path state in a static device
array instead and writes into the caller's device film. These tests call it
through the C ABI twice in a row and compare each result with pyre_render on
the same crop and samples (same tolerance as the other render tests:
relMSE < 1e-2; the kernels are the same, so the films agree exactly).

This file is collected last so that a failure here cannot stop the rest of the
GPU suite from running first.
"""
import ctypes as C

import numpy as np
import pytest

from pyre_gb300 import native as N
from pyre_gb300 import presets as P
from pyre_gb300.scene import CudaIntegrator, PathIntegrator

pytestmark = pytest.mark.gpu


def _relmse(x, r):
    return float(np.mean(np.sum((x - r) ** 2 / (r ** 2 + 1e-2), axis=-1)))


def _noalloc(ctx, ds, cam, params, npix):
    import torch
    dev = {k: torch.full((npix * c,), -1.0, dtype=torch.float32, device="cuda")
           for k, c in (("radiance", 3), ("albedo", 3), ("normal", 3), ("depth", 1))}
    film = N.Film(N.dptr(dev["radiance"]), N.dptr(dev["albedo"]), N.dptr(dev["normal"]), N.dptr(dev["depth"]),
                  N.PYRE_MEM_DEVICE)
    desc = cam.to_desc()
    rc = ctx.lib.pyre_render_noalloc(ctx.handle, ds.handle, C.byref(desc), C.byref(params), C.byref(film))
    ctx.check(rc)
    return {k: v.cpu().numpy() for k, v in dev.items()}


@pytest.mark.parametrize("name", ["cornell_box", "studio_ref"])
def test_noalloc_matches_render_twice(gpu_ctx, name):
    if name == "cornell_box":
        sc, cam, w, h = P.cornell_box(), P.cornell_box_camera(128, 128), 128, 128
    else:
        sc, cam, w, h = P.studio_ref(motion_blur=True), P.studio_ref_camera(160, 120, aperture=0.05), 160, 120
    ds = gpu_ctx.upload(sc)
    it = PathIntegrator(8, 3)
    crop = (8, 4, w - 8, h - 4)
    npix = (crop[2] - crop[0]) * (crop[3] - crop[1])
    ref = gpu_ctx.render(ds, cam, it, w, h, 8, crop=crop)
    params = CudaIntegrator.params(w, h, 0, 8, it, crop=crop)
    for _ in range(2):  # the static array keeps the previous call's contents
        out = _noalloc(gpu_ctx, ds, cam, params, npix)
        rad = out["radiance"].reshape(ref.radiance.shape)
        assert _relmse(rad, ref.radiance) < 1e-2
        np.testing.assert_allclose(rad, ref.radiance, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(out["albedo"].reshape(ref.albedo.shape), ref.albedo, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(out["normal"].reshape(ref.normal.shape), ref.normal, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(out["depth"].reshape(ref.depth.shape), ref.depth, rtol=1e-6, atol=1e-7)
    ds.close()


def test_noalloc_on_fresh_context_allocates_nothing(gpu_ctx):
    """A context that has never rendered: every allocation it would try from now on fails (injected
    out-of-memory), yet pyre_render_noalloc succeeds, twice, with the same film as pyre_render."""
    sc, cam, w, h = P.cornell_box(), P.cornell_box_camera(96, 96), 96, 96
    it = PathIntegrator(8, 3)
    ref = gpu_ctx.render(gpu_ctx.upload(sc), cam, it, w, h, 4)
    fresh = CudaIntegrator(0)
    try:
        ds = fresh.upload(sc)
        params = CudaIntegrator.params(w, h, 0, 4, it)
        fresh.check(fresh.lib.pyre_inject_alloc_failure(fresh.handle, 0))
        try:
            for _ in range(2):
                out = _noalloc(fresh, ds, cam, params, w * h)
                np.testing.assert_allclose(out["radiance"].reshape(ref.radiance.shape), ref.radiance,
                                           rtol=1e-6, atol=1e-7)
                np.testing.assert_allclose(out["normal"].reshape(ref.normal.shape), ref.normal, rtol=1e-6, atol=1e-7)
        finally:
            fresh.check(fresh.lib.pyre_inject_alloc_failure(fresh.handle, -1))
        ds.close()
    finally:
        fresh.close()


def test_noalloc_rejects_oversized_crop(gpu_ctx):
    sc, cam = P.cornell_box(), P.cornell_box_camera(1024, 1024)
    ds = gpu_ctx.upload(sc)
    params = CudaIntegrator.params(1024, 1024, 0, 1, PathIntegrator(8, 3))
    import torch
    buf = torch.zeros(1024 * 1024 * 3, dtype=torch.float32, device="cuda")
    film = N.Film(N.dptr(buf), None, None, None, N.PYRE_MEM_DEVICE)
    desc = cam.to_desc()
    rc = gpu_ctx.lib.pyre_render_noalloc(gpu_ctx.handle, ds.handle, C.byref(desc), C.byref(params), C.byref(film))
    assert rc == N.PYRE_ERR_INVALID
    assert b"exceeds" in gpu_ctx.lib.pyre_last_error(gpu_ctx.handle)
    # host films are refused: the caller must own device memory
    hfilm = N.Film(N.fptr(np.zeros(3, np.float32)), None, None, None, N.PYRE_MEM_HOST)
    small = CudaIntegrator.params(1024, 1024, 0, 1, PathIntegrator(8, 3), crop=(0, 0, 1, 1))
    rc = gpu_ctx.lib.pyre_render_noalloc(gpu_ctx.handle, ds.handle, C.byref(desc), C.byref(small), C.byref(hfilm))
    assert rc == N.PYRE_ERR_INVALID
    ds.close()

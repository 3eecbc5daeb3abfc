"""Progressive accumulation (pyre_render_progressive) against the viewer's
loop (crates/pyre/src/viewer.rs:114-185): pass s renders one sample per pixel
with sample index s and merges as mean += (L_s - mean) / (s + 1) in float32."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.native import PYRE_ENV_CDF
from pyre_gb300.scene import PathIntegrator

pytestmark = pytest.mark.gpu
F32 = np.float32


def welford(passes):
    m = np.zeros_like(passes[0], dtype=F32)
    for s, L in enumerate(passes):
        m = (m + (L.astype(F32) - m) / F32(s + 1)).astype(F32)
    return m


def _scene():
    sc = P.studio_procedural(n_side=3, segments=24, n_moving=2, hdri_size=(256, 128))
    return sc, P.studio_procedural_camera(48, 32)


def test_progressive_matches_viewer_merge(gpu_ctx, oracle_mod):
    sc, cam = _scene()
    ds = gpu_ctx.upload(sc)
    it = PathIntegrator(8, 3)
    n = 6
    # CDF environment sampling follows the reference's sample paths (alias tables agree only statistically)
    single = [gpu_ctx.render(ds, cam, it, 48, 32, 1, spp_begin=s, env_sampling=PYRE_ENV_CDF).radiance.reshape(32, 48, 3)
              for s in range(n)]
    mean = gpu_ctx.render_progressive(ds, cam, it, 48, 32, n, env_sampling=PYRE_ENV_CDF)
    np.testing.assert_array_equal(mean, welford(single))
    osc = oracle_mod.OracleScene(sc)
    ref = welford([osc.render(cam, 48, 32, 1, spp_begin=s)["radiance"].reshape(32, 48, 3) for s in range(n)])
    rel = float(np.mean(np.sum((mean - ref) ** 2 / (ref ** 2 + 1e-2), axis=-1)))
    assert rel < 1e-2, rel
    ds.close()


def test_progressive_chaining_and_waves(gpu_ctx):
    sc, cam = _scene()
    ds = gpu_ctx.upload(sc)
    it = PathIntegrator(8, 3)
    whole = gpu_ctx.render_progressive(ds, cam, it, 48, 32, 7)
    m = gpu_ctx.render_progressive(ds, cam, it, 48, 32, 3)
    m = gpu_ctx.render_progressive(ds, cam, it, 48, 32, 4, mean=m, pass_begin=3)
    np.testing.assert_array_equal(m, whole)
    # one pass per wave (wave capacity = one sample of every pixel)
    small = gpu_ctx.render_progressive(ds, cam, it, 48, 32, 7, wave_paths=48 * 32)
    np.testing.assert_array_equal(small, whole)
    # a crop merges exactly the crop's pixels
    crop = gpu_ctx.render_progressive(ds, cam, it, 48, 32, 7, crop=(8, 4, 40, 20))
    np.testing.assert_array_equal(crop, whole[4:20, 8:40])
    ds.close()

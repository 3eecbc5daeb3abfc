"""Path-replay adjoint vs (1) the oracle's forward-mode dual-number gradient
(same seeds, same detached convention: cosine >= 0.999) and (2) central
finite differences with common random numbers."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.native import PYRE_ENV_CDF
from pyre_gb300.scene import (DisneyBsdf, HdriEnvironmentLight, Lambertian, MeshInstance, PathIntegrator, Primitive,
                              Scene)

pytestmark = pytest.mark.gpu


def cosine(a, b):
    a, b = np.ravel(a).astype(np.float64), np.ravel(b).astype(np.float64)
    return float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-300))


def small_env_scene():
    return P.adjoint_check_scene()


def test_adjoint_matches_dual_number_oracle(gpu_ctx, oracle_mod):
    sc, cam = small_env_scene()
    w = h = 48
    it = PathIntegrator(6, 3)
    dl = np.random.default_rng(9).normal(size=(h, w, 3)).astype(np.float32)
    ds = gpu_ctx.upload(sc)
    g_mat, g_env = gpu_ctx.backward(ds, cam, it, w, h, 4, dl, env_sampling=PYRE_ENV_CDF)
    o_mat, o_env = oracle_mod.OracleScene(sc).render_grad(cam, w, h, 4, dl, len(sc.materials), (8, 16),
                                                          max_depth=6, min_rr_depth=3)
    cm, ce = cosine(g_mat, o_mat), cosine(g_env, o_env)
    rel_m = float(np.linalg.norm(g_mat - o_mat) / np.linalg.norm(o_mat))
    rel_e = float(np.linalg.norm(g_env - o_env) / np.linalg.norm(o_env))
    print({"cos_materials": cm, "cos_env": ce, "rel_l2_materials": rel_m, "rel_l2_env": rel_e})
    assert cm >= 0.999 and ce >= 0.999, (cm, ce)
    assert rel_m < 0.02 and rel_e < 0.02
    ds.close()


def test_adjoint_matches_finite_differences(gpu_ctx):
    """Lambertian Cornell box, RR off: d loss / d albedo by central differences (common random numbers)."""
    sc, cam = P.cornell_box(), P.cornell_box_camera(64, 64)
    w = h = 64
    it = PathIntegrator(5, 99)  # min_rr_depth beyond max_depth: no Russian roulette
    spp = 64
    ds = gpu_ctx.upload(sc)
    target = gpu_ctx.render(ds, cam, it, w, h, 256, spp_begin=5000).radiance * 0.8

    def loss(img):
        return float(np.mean((img.astype(np.float64) - target) ** 2))

    img = gpu_ctx.render(ds, cam, it, w, h, spp).radiance
    dl = (2.0 * (img - target) / img.size).astype(np.float32)
    g_mat, _ = gpu_ctx.backward(ds, cam, it, w, h, spp, dl)
    base = list(sc.materials)
    eps = 1e-3
    checked = 0
    for m in range(3):
        for c in range(3):
            plus = [Lambertian(x.albedo.copy()) for x in base]
            minus = [Lambertian(x.albedo.copy()) for x in base]
            plus[m].albedo[c] += eps
            minus[m].albedo[c] -= eps
            gpu_ctx.set_materials(ds, plus)
            lp = loss(gpu_ctx.render(ds, cam, it, w, h, spp).radiance)
            gpu_ctx.set_materials(ds, minus)
            lm = loss(gpu_ctx.render(ds, cam, it, w, h, spp).radiance)
            fd = (lp - lm) / (2 * eps)
            ad = g_mat[m, c]
            assert abs(ad - fd) <= 0.03 * abs(fd) + 1e-7, (m, c, ad, fd)
            checked += 1
    gpu_ctx.set_materials(ds, base)
    assert checked == 9
    ds.close()


def test_backward_uses_forward_tape(gpu_ctx):
    """backward() after forward() (kept radiance) equals backward() that re-renders it."""
    sc, cam = small_env_scene()
    it = PathIntegrator(6, 3)
    dl = np.random.default_rng(2).normal(size=(48, 48, 3)).astype(np.float32)
    ds = gpu_ctx.upload(sc)
    a_m, a_e = gpu_ctx.backward(ds, cam, it, 48, 48, 4, dl, env_sampling=PYRE_ENV_CDF, spp_begin=7)
    film = gpu_ctx.forward(ds, cam, it, 48, 48, 4, env_sampling=PYRE_ENV_CDF, spp_begin=7)
    ref = gpu_ctx.render(ds, cam, it, 48, 48, 4, env_sampling=PYRE_ENV_CDF, spp_begin=7)
    np.testing.assert_array_equal(film.radiance, ref.radiance)
    b_m, b_e = gpu_ctx.backward(ds, cam, it, 48, 48, 4, dl, env_sampling=PYRE_ENV_CDF, spp_begin=7)
    np.testing.assert_allclose(a_m, b_m, rtol=1e-9, atol=1e-12)
    # Texel gradients sum by FP32 atomics whose order varies run to run.
    np.testing.assert_allclose(a_e, b_e, rtol=0, atol=1e-5 * float(np.abs(b_e).max()))
    ds.close()

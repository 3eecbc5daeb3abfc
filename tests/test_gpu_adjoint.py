"""Path-replay adjoint vs (1) the oracle's forward-mode dual-number gradient
(same seeds, same detached convention: cosine >= 0.999) and (2) central
finite differences with common random numbers."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.native import PYRE_ENV_CDF
from pyre_gb300.scene import (DisneyBsdf, HdriEnvironmentLight, Lambertian, MeshInstance, PathIntegrator, Primitive,
                              Scene)  # noqa: F401

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
    # Material terms are summed per warp in FP32 before the FP64 sums, and
    # which paths share a warp follows the material-sorted queue, whose order
    # within a material varies run to run (differences of a few 1e-9 of the
    # largest gradient, seen on entries that cancel); texel gradients sum by
    # FP32 atomics whose order varies as well.
    np.testing.assert_allclose(a_m, b_m, rtol=1e-5, atol=1e-7 * float(np.abs(b_m).max()))
    np.testing.assert_allclose(a_e, b_e, rtol=0, atol=1e-5 * float(np.abs(b_e).max()))
    ds.close()


def _with_param(sc, param, d):
    """A copy of the scene with one parameter moved by d: ("mat", m, k) is parameter k (base r, g, b, metallic,
    roughness, specular) of material m; ("env", y, x, c) is channel c of texel (y, x)."""
    from pyre_gb300.scene import Scene
    if param[0] == "env":
        px = sc.env.pixels.copy()
        px[param[1], param[2], param[3]] += d
        return Scene(sc.primitives, sc.materials, sc.lights,
                     HdriEnvironmentLight(sc.env.width, sc.env.height, px, sc.env.intensity))
    mats = []
    for j, x in enumerate(sc.materials):
        if isinstance(x, Lambertian):
            a = x.albedo.copy()
            if j == param[1]:
                a[param[2]] += d
            mats.append(Lambertian(a))
        else:
            p = [*map(float, x.base_color), x.metallic, x.roughness, x.specular]
            if j == param[1]:
                p[param[2]] += d
            mats.append(DisneyBsdf(p[:3], p[3], p[4], p[5]))
    return Scene(sc.primitives, mats, sc.lights, sc.env)


@pytest.mark.parametrize("rr", [False, True], ids=["rr_off", "rr_on"])
def test_adjoint_matches_finite_differences_disney_and_env(gpu_ctx, rr):
    """d loss / d (all six Disney parameters of a half-metallic and of a dielectric sphere, a bright sun texel
    and a dim sky texel) by the path-replay adjoint against central finite differences (eps 1e-3, common random
    numbers), with Russian roulette off and on.

    Finite differences with common random numbers move each sample with the parameters. Where a parameter
    changes the sampling (the lobe choice u.x < pd of the Disney BSDF, material.rs:205-214, or a path crossing
    a silhouette), a few samples jump to another path; those jumps carry a share of the derivative that only
    shows with many samples at eps 1e-3 (with 2.4 M samples the lobe-switch share of d/d base blue, about 3 %,
    was missed). So both sides use 16 blocks of 64x64 pixels x 16,384 spp (1.07 G samples), the loss is linear
    in the image (d loss / d image fixed, from an L2 loss at an independent render), and each parameter passes
    when the mean of the 16 paired differences (adjoint - finite difference) is within 4.5 standard errors, or
    within 3 % of the finite difference."""
    from pyre_gb300.native import PYRE_ENV_CDF
    sc, cam = P.fd_check_scene()
    # the device scene keeps `sc` and set_materials / set_env replace its fields: perturb copies of the base
    base = Scene(list(sc.primitives), list(sc.materials), list(sc.lights), sc.env)
    w = h = 64
    it = PathIntegrator(5, 2 if rr else 99)
    spp, blocks, eps = 16384, 16, 1e-3
    ds = gpu_ctx.upload(sc)
    ref = gpu_ctx.render(ds, cam, it, w, h, 1024, spp_begin=1 << 28, env_sampling=PYRE_ENV_CDF).radiance
    tmats = [m if isinstance(m, Lambertian) else
             DisneyBsdf(np.clip(m.base_color * 0.8, 0, 1), m.metallic * 0.7, min(1.0, m.roughness * 1.3), m.specular)
             for m in sc.materials]
    gpu_ctx.set_materials(ds, tmats)
    tgt = gpu_ctx.render(ds, cam, it, w, h, 1024, spp_begin=1 << 29, env_sampling=PYRE_ENV_CDF).radiance
    gpu_ctx.set_materials(ds, base.materials)
    dl = (2.0 * (ref.astype(np.float64) - tgt) / ref.size).astype(np.float32)
    params = [("mat", m, k) for m in (1, 2) for k in range(6)] + [("env", 2, 5, 0), ("env", 6, 3, 1)]
    if rr:  # the half-metallic sphere and the sun texel
        params = [p for p in params if p[0] == "env" and p[1] == 2 or p[0] == "mat" and p[1] == 1]
    AD = np.zeros((blocks, len(params)))
    for b in range(blocks):
        gm, ge = gpu_ctx.backward(ds, cam, it, w, h, spp, dl, spp_begin=b * spp, env_sampling=PYRE_ENV_CDF)
        for j, p in enumerate(params):
            AD[b, j] = gm[p[1], p[2]] if p[0] == "mat" else ge[p[1], p[2], p[3]]
    FD = np.zeros((blocks, len(params)))
    d64 = dl.astype(np.float64)
    for j, p in enumerate(params):
        imgs = {}
        for sign in (1, -1):
            s2 = _with_param(base, p, sign * eps)
            if p[0] == "mat":
                gpu_ctx.set_materials(ds, s2.materials)
            else:
                gpu_ctx.set_env(ds, s2.env.pixels, s2.env.intensity)
            imgs[sign] = [gpu_ctx.render(ds, cam, it, w, h, spp, spp_begin=b * spp, env_sampling=PYRE_ENV_CDF)
                          .radiance.astype(np.float64) for b in range(blocks)]
        gpu_ctx.set_materials(ds, base.materials)
        gpu_ctx.set_env(ds, base.env.pixels, base.env.intensity)
        for b in range(blocks):
            FD[b, j] = float(np.sum(d64 * (imgs[1][b] - imgs[-1][b]))) / (2 * eps)
    D = AD - FD
    rows = []
    for j, p in enumerate(params):
        md, se = float(D[:, j].mean()), float(D[:, j].std(ddof=1) / np.sqrt(blocks))
        fd, ad = float(FD[:, j].mean()), float(AD[:, j].mean())
        se_fd = float(FD[:, j].std(ddof=1) / np.sqrt(blocks))
        rows.append({"param": p, "adjoint": ad, "finite_difference": fd, "se_fd": se_fd,
                     "diff_over_se": md / se if se > 0 else 0.0, "rel": md / abs(fd) if fd else 0.0,
                     "pass": abs(md) <= max(4.5 * se, 0.03 * abs(fd))})
    for r in rows:
        print(r)
    assert all(r["pass"] for r in rows), [r for r in rows if not r["pass"]]
    # the check has teeth: most parameters carry a gradient far above the finite differences' noise
    assert sum(abs(r["finite_difference"]) > 10 * r["se_fd"] for r in rows) >= len(rows) // 2, rows
    ds.close()


@pytest.mark.parametrize("crop", [(224, 224, 256, 256), (96, 352, 128, 384)], ids=["centre", "lower_left"])
def test_adjoint_matches_dual_numbers_on_the_differentiable_render_problem(gpu_ctx, oracle_mod, crop):
    """The differentiable-render workload itself (the procedural studio at 512x512: 64 sphere materials and the
    ground, a 512x256 HDRI; depth 8, Russian roulette from depth 3) on 32x32 crops at 16 spp: the adjoint's
    gradients of all 390 material parameters and all 393,216 texel channels against the oracle's forward-mode
    dual-number gradient with the same samples and convention: cosine >= 0.999."""
    from pyre_gb300.native import PYRE_ENV_CDF
    sc, _, cam = P.adjoint_problem(512, 512)
    it = PathIntegrator(8, 3)
    x0, y0, x1, y1 = crop
    dl = np.random.default_rng(x0 + y0).normal(size=(y1 - y0, x1 - x0, 3)).astype(np.float32)
    ds = gpu_ctx.upload(sc)
    g_mat, g_env = gpu_ctx.backward(ds, cam, it, 512, 512, 16, dl, crop=crop, env_sampling=PYRE_ENV_CDF)
    o_mat, o_env = oracle_mod.OracleScene(sc).render_grad(cam, 512, 512, 16, dl, len(sc.materials),
                                                          (sc.env.height, sc.env.width), crop=crop)
    cm, ce = cosine(g_mat, o_mat), cosine(g_env, o_env)
    print({"crop": crop, "cos_materials": cm, "cos_env": ce, "materials_touched": int((o_mat != 0).any(1).sum()),
           "texels_touched": int((o_env != 0).any(-1).sum())})
    assert (o_mat != 0).any(1).sum() >= 2 and (o_env != 0).any()
    assert cm >= 0.999 and ce >= 0.999, (cm, ce)
    ds.close()

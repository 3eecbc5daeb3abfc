"""The reference's own unit tests that pin this path, run against the device
code (tests/golden/reference_kats.json; the same cases run against the
oracle in test_oracle_kats.py): Möller–Trumbore hits and misses
(mesh.rs:197-234), Distribution1D/2D (distribution.rs:178-220) through the
environment light's sampling code, and the Disney sample/eval/pdf
consistency test (material.rs:332-387) on the reference's seeded draws."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from pyre_gb300 import native as N
from pyre_gb300.scene import DisneyBsdf, Lambertian, MeshInstance, Primitive, Scene, TriangleMesh, _material_desc

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
F32 = np.float32


def dist_query(ctx, weights, w, h, mode, u, uv=None):
    wts = np.ascontiguousarray(weights, F32)
    u = np.ascontiguousarray(u, F32).reshape(-1, 2)
    uv = np.zeros((0, 2), F32) if uv is None else np.ascontiguousarray(uv, F32).reshape(-1, 2)
    out, pdf = np.zeros((u.shape[0], 5), F32), np.zeros(uv.shape[0], F32)
    ctx.check(ctx.lib.pyre_distribution2d_query(ctx.handle, N.fptr(wts), w, h, mode, u.shape[0], N.fptr(u),
                                                N.fptr(out), uv.shape[0], N.fptr(uv), N.fptr(pdf)))
    return out, pdf


@pytest.mark.parametrize("case", KATS["mesh"], ids=lambda c: c["name"])
def test_mesh_kats_on_device(gpu_ctx, case):
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    mesh = TriangleMesh(np.asarray(case["positions"], F32), np.asarray(case["indices"], np.uint32))
    sc.primitives.append(Primitive(MeshInstance.build(mesh), 0))
    d = np.asarray(case["direction"], F32)
    d = (d / np.linalg.norm(d)).astype(F32)
    r = gpu_ctx.intersect(gpu_ctx.upload(sc), np.asarray([case["origin"]], F32), d[None], np.float32([1e-4]),
                          np.float32([np.inf]))
    assert bool(r["kind"][0] == 1) == case["expect_hit"]
    if case["expect_hit"]:
        assert abs(float(r["t"][0]) - case["t"]) < case["t_tol"]


@pytest.mark.parametrize("case", KATS["distribution1d"], ids=lambda c: c["name"])
def test_distribution1d_kats_on_device(gpu_ctx, case):
    w = len(case["weights"])
    u = [(c["u"], 0.5) for c in case["cases"]]
    out, _ = dist_query(gpu_ctx, case["weights"], w, 1, N.PYRE_ENV_CDF, u)
    for k, c in enumerate(case["cases"]):
        t, pdf, b = out[k, 0], out[k, 2], int(out[k, 3])
        assert b == c["bin"]
        assert abs(float(pdf) - c["pdf"]) < c["pdf_tol"]
        if "t" in c:
            assert abs(float(t) - c["t"]) < c["t_tol"]
        else:
            lo, hi = c["t_range"]
            assert lo <= float(t) < hi


@pytest.mark.parametrize("mode", [N.PYRE_ENV_CDF, N.PYRE_ENV_ALIAS])
def test_distribution2d_normalizes_on_device(gpu_ctx, mode):
    case = KATS["distribution2d"][0]
    n = case["grid"]
    g = (np.arange(n, dtype=F32) + F32(0.5)) / F32(n)
    uv = np.stack(np.meshgrid(g, g, indexing="xy"), -1).reshape(-1, 2)
    _, pdf = dist_query(gpu_ctx, case["weights"], case["width"], case["height"], mode, np.zeros((0, 2)), uv)
    total = float(pdf.sum(dtype=np.float32)) / (n * n)
    assert abs(total - case["integral"]) < case["tol"]
    # both samplers draw bins with the distribution's probabilities, and report their pdf
    rng = np.random.default_rng(3)
    out, _ = dist_query(gpu_ctx, case["weights"], case["width"], case["height"], mode, rng.random((200_000, 2)))
    w = np.asarray(case["weights"], np.float64)
    freq = np.bincount((out[:, 4] * case["width"] + out[:, 3]).astype(int), minlength=w.size) / out.shape[0]
    np.testing.assert_allclose(freq, w / w.sum(), atol=3e-3)
    np.testing.assert_allclose(out[:, 2], (w / w.sum() * w.size)[(out[:, 4] * case["width"] + out[:, 3]).astype(int)],
                               rtol=1e-5)


def test_disney_consistency_on_device(gpu_ctx, oracle_mod):
    kat = KATS["disney_consistency"]
    wo, u = oracle_mod.disney_draws(kat["seed"], kat["iters"])
    sampled = 0
    for b, params in enumerate(kat["bsdfs"]):
        mat = DisneyBsdf(params["base_color"], params["metallic"], params["roughness"], params["specular"])
        sl = slice(b * kat["iters"], (b + 1) * kat["iters"])
        out = np.zeros((kat["iters"], 13), F32)
        desc = _material_desc(mat)
        gpu_ctx.check(gpu_ctx.lib.pyre_bsdf_query(gpu_ctx.handle, C.byref(desc), kat["iters"],
                                                  N.fptr(np.ascontiguousarray(wo[sl])),
                                                  N.fptr(np.ascontiguousarray(u[sl])), N.fptr(out)))
        ok = out[:, 0] > 0
        sampled += int(ok.sum())
        f, pdf, fe, pe, wi = out[ok, 4:7], out[ok, 7], out[ok, 8:11], out[ok, 11], out[ok, 1:4]
        # material.rs:332-387: the sample's f and pdf are eval and pdf of the sampled direction
        assert np.linalg.norm(fe - f, axis=1).max() < kat["tol"]
        assert np.abs(pe - pdf).max() < kat["tol"]
        # the sample's f and pdf come from the fused evaluation shade uses;
        # it must equal the separate eval and pdf to the bit
        assert np.array_equal(f.view(np.uint32), fe.view(np.uint32))
        assert np.array_equal(pdf.view(np.uint32), pe.view(np.uint32))
        assert pdf.min() > 0.0 and wi[:, 2].min() > 0.0
        # and the device agrees with the oracle draw by draw: the same sampled
        # directions (to the ulps of CUDA's and glibc's sin/cos), and the same
        # f and pdf at the device's direction (comparing the two samples' own
        # pdfs instead would amplify those ulps by the peak of the GGX lobe)
        ook, owi, _, _ = oracle_mod.bsdf_sample(mat, wo[sl], u[sl])
        assert (ook == ok).mean() > 0.999
        both = ok & ook
        np.testing.assert_allclose(out[both, 1:4], owi[both], atol=2e-5)
        of, opdf = oracle_mod.bsdf_eval(mat, wo[sl][ok], out[ok, 1:4])
        np.testing.assert_allclose(pdf, opdf, rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(f, of, rtol=2e-5, atol=1e-7)
    assert sampled > 0.9 * 3 * kat["iters"]

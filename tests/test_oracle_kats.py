"""The oracle against the reference's own unit tests (tests/golden/reference_kats.json)."""
import json
from pathlib import Path

import numpy as np
import pytest

from pyre_gb300.scene import DisneyBsdf, Lambertian, MeshInstance, Primitive, Scene, TriangleMesh

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.mark.parametrize("case", KATS["mesh"], ids=lambda c: c["name"])
def test_mesh_kats(oracle_mod, case):
    sc = Scene()
    sc.materials.append(Lambertian([0.5] * 3))
    mesh = TriangleMesh(np.asarray(case["positions"], np.float32), np.asarray(case["indices"], np.uint32))
    sc.primitives.append(Primitive(MeshInstance.build(mesh), 0))
    d = np.asarray(case["direction"], np.float32)
    d = (d / np.linalg.norm(d)).astype(np.float32)  # Ray::new normalizes (math.rs:16-24)
    r = oracle_mod.OracleScene(sc).intersect(np.asarray([case["origin"]], np.float32), d[None], [1e-4], [np.inf],
                                             normals=True)
    assert bool(r["kind"][0] == 1) == case["expect_hit"]
    if case["expect_hit"]:
        assert abs(float(r["t"][0]) - case["t"]) < case["t_tol"]
        if "normal_dot_z_min" in case:
            assert float(r["normal"][0, 2]) > case["normal_dot_z_min"]


@pytest.mark.parametrize("case", KATS["distribution1d"], ids=lambda c: c["name"])
def test_distribution1d_kats(oracle_mod, case):
    us = [c["u"] for c in case["cases"]]
    t, pdf, b = oracle_mod.dist1d_sample(case["weights"], us)
    for k, c in enumerate(case["cases"]):
        assert int(b[k]) == c["bin"]
        assert abs(float(pdf[k]) - c["pdf"]) < c["pdf_tol"]
        if "t" in c:
            assert abs(float(t[k]) - c["t"]) < c["t_tol"]
        else:
            lo, hi = c["t_range"]
            assert lo <= float(t[k]) < hi


def test_distribution2d_normalizes(oracle_mod):
    case = KATS["distribution2d"][0]
    n = case["grid"]
    g = (np.arange(n, dtype=np.float32) + 0.5) / n
    uv = np.stack(np.meshgrid(g, g, indexing="xy"), -1).reshape(-1, 2)
    pdf = oracle_mod.dist2d_pdf(case["weights"], case["width"], case["height"], uv)
    total = float(pdf.astype(np.float32).sum(dtype=np.float32)) / (n * n)
    assert abs(total - case["integral"]) < case["tol"]


def test_disney_sample_eval_pdf_consistency(oracle_mod):
    kat = KATS["disney_consistency"]
    mats = [DisneyBsdf(b["base_color"], b["metallic"], b["roughness"], b["specular"]) for b in kat["bsdfs"]]
    n, (max_df, max_dp, min_pdf, min_wiz) = oracle_mod.disney_consistency(mats, kat["seed"], kat["iters"])
    assert n > 0.9 * 3 * kat["iters"]
    assert max_df < kat["tol"] and max_dp < kat["tol"]
    assert min_pdf > 0.0 and min_wiz > 0.0

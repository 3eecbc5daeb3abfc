"""Scenes ingested from files render through the GPU path exactly like the
same scenes built in code (PBRT text -> Scene -> pyre_scene_upload)."""
import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.io import load_pbrt
from pyre_gb300.scene import PathIntegrator, PinholeCamera
from test_io_cpu import scene_to_pbrt

pytestmark = pytest.mark.gpu


def test_pbrt_cornell_renders_like_the_preset(gpu_ctx, oracle_mod, tmp_path):
    sc = P.cornell_box()
    f = tmp_path / "cornell.pbrt"
    f.write_text(scene_to_pbrt(sc, (0, 0, 3), (0, 0, 0), (0, 1, 0), 45, 64, 64))
    ld = load_pbrt(f)
    c = ld.camera
    cam = PinholeCamera.look_at(c.origin, c.target, c.up, c.vfov_deg, np.float32(ld.film.width) / ld.film.height)
    it = PathIntegrator(8, 3)
    ds_file, ds_code = gpu_ctx.upload(ld.scene), gpu_ctx.upload(sc)
    a = gpu_ctx.render(ds_file, cam, it, 64, 64, 8)
    b = gpu_ctx.render(ds_code, P.cornell_box_camera(64, 64), it, 64, 64, 8)
    # the loader re-normalizes "normal N" like the reference's builder, which can
    # move the last bit of the rotated boxes' normals: equal up to that rounding
    for ch in ("radiance", "albedo", "normal", "depth"):
        np.testing.assert_allclose(getattr(a, ch), getattr(b, ch), rtol=1e-5, atol=1e-7)
    ref = oracle_mod.OracleScene(ld.scene).render(cam, 64, 64, 8)["radiance"]
    rel = float(np.mean(np.sum((a.radiance - ref) ** 2 / (ref ** 2 + 1e-2), axis=-1)))
    assert rel < 1e-2, rel
    ds_file.close()
    ds_code.close()


def test_cli_scene_file_to_exr_and_progressive_png(tmp_path):
    """python -m pyre_gb300.cli --scene x.pbrt --output y.exr --aovs all --save-aov-pngs, and --progressive."""
    from pyre_gb300 import cli, sinks
    sc = P.cornell_box()
    f = tmp_path / "cornell.pbrt"
    f.write_text(scene_to_pbrt(sc, (0, 0, 3), (0, 0, 0), (0, 1, 0), 45, 64, 48))
    out = tmp_path / "frame.exr"
    assert cli.main(["--scene", str(f), "--width", "64", "--height", "48", "--spp", "4", "--output", str(out),
                     "--aovs", "all", "--save-aov-pngs"]) == 0
    planes = sinks.read_exr(out)
    assert planes["R"].shape == (48, 64) and "N.Z" in planes and "Z" in planes
    assert planes["R"].max() > 0
    for name in ("frame.albedo.png", "frame.normal.png", "frame.depth.png"):
        assert (tmp_path / name).exists()
    png = tmp_path / "prog.png"
    assert cli.main(["--scene", str(f), "--width", "64", "--height", "48", "--spp", "5", "--pass-chunk", "2",
                     "--progressive", "--output", str(png)]) == 0
    img = sinks.read_png(png)
    assert img.shape == (48, 64, 3) and img.max() > 0

"""CLI helpers on CPU: auto-framing (main.rs:336-350), scene bounds, output
dispatch and AOV parsing."""
import numpy as np
import pytest

from pyre_gb300 import cli, presets as P
from pyre_gb300.scene import Film


def test_auto_frame_fits_the_bounding_sphere():
    lo, hi = np.float32([-1, -2, -3]), np.float32([1, 2, 3])
    o, t = cli.auto_frame(lo, hi, 45.0, np.float32(4) / np.float32(3))
    np.testing.assert_allclose(t, [0, 0, 0])
    r = np.linalg.norm(hi - lo) / 2
    d = np.linalg.norm(o - t)
    assert abs(d - 1.15 * r / np.sin(np.radians(22.5))) < 1e-4 * d  # vertical fov is the tighter one
    np.testing.assert_allclose((o - t) / d, np.array([0, 0.3, 1]) / np.linalg.norm([0, 0.3, 1]), atol=1e-6)


def test_scene_bounds_include_motion():
    sc = P.studio_ref(motion_blur=True)
    lo, hi = cli.scene_bounds(sc)
    assert np.all(lo < hi)
    still = P.studio_ref(motion_blur=False)
    slo, shi = cli.scene_bounds(still)
    assert np.all(lo <= slo) and np.all(hi >= shi)


def test_output_dispatch(tmp_path):
    from pyre_gb300 import sinks
    f = Film(5, 4)
    f.radiance[:] = 0.5
    f.depth[:] = 2.0
    args = cli.parse(["--output", str(tmp_path / "a.exr"), "--aovs", "albedo,z", "--save-aov-pngs"])
    cli.save_output(args, f)
    assert sorted(sinks.read_exr(tmp_path / "a.exr")) == ["B", "G", "R", "Z", "albedo.B", "albedo.G", "albedo.R"]
    assert (tmp_path / "a.albedo.png").exists() and (tmp_path / "a.depth.png").exists()
    assert not (tmp_path / "a.normal.png").exists()
    args = cli.parse(["--output", str(tmp_path / "b.png")])
    cli.save_output(args, f)
    assert sinks.read_png(tmp_path / "b.png").shape == (4, 5, 3)
    for bad in (["--output", str(tmp_path / "c.tga")], ["--output", str(tmp_path / "c.exr"), "--aovs", "spec"]):
        with pytest.raises(SystemExit):
            cli.save_output(cli.parse(bad), f)

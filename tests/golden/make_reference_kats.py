"""Writes reference_kats.json: the known-answer cases of the Pyre renderer's own
unit tests that touch the hot path, transcribed with their tolerances.

Sources (paths relative to the Pyre repository root):
  crates/pyre/src/geometry/mesh.rs:197-234   hits/misses/closest-of-two
  crates/pyre/src/distribution.rs:178-220    Distribution1D/2D
  crates/pyre/src/material.rs:332-387        Disney sample/eval/pdf consistency

Run:  python tests/golden/make_reference_kats.py
"""
import json
from pathlib import Path

KATS = {
    "mesh": [
        {"name": "hits_triangle_along_minus_z", "source": "crates/pyre/src/geometry/mesh.rs:197-204",
         "positions": [[-1, 0, 0], [1, 0, 0], [0, 1, 0]], "indices": [0, 1, 2],
         "origin": [0, 0.3, 1], "direction": [0, 0, -1], "expect_hit": True, "t": 1.0, "t_tol": 1e-4,
         "normal_dot_z_min": 0.99},
        {"name": "misses_triangle_below", "source": "crates/pyre/src/geometry/mesh.rs:206-211",
         "positions": [[-1, 0, 0], [1, 0, 0], [0, 1, 0]], "indices": [0, 1, 2],
         "origin": [0, -1, 1], "direction": [0, 0, -1], "expect_hit": False},
        {"name": "bvh_finds_closest_of_two", "source": "crates/pyre/src/geometry/mesh.rs:213-234",
         "positions": [[-1, -1, 0], [1, -1, 0], [0, 1, 0], [-1, -1, -1], [1, -1, -1], [0, 1, -1]],
         "indices": [0, 1, 2, 3, 4, 5], "origin": [0, 0, 2], "direction": [0, 0, -1], "expect_hit": True,
         "t": 2.0, "t_tol": 1e-4},
    ],
    "distribution1d": [
        {"name": "distribution1d_uniform_samples_uniformly", "source": "crates/pyre/src/distribution.rs:178-190",
         "weights": [1.0, 1.0, 1.0, 1.0],
         "cases": [{"u": 0.0, "t": 0.0, "t_tol": 1e-6, "pdf": 1.0, "pdf_tol": 1e-6, "bin": 0},
                   {"u": 0.999999, "t_range": [0.75, 1.0], "pdf": 1.0, "pdf_tol": 1e-3, "bin": 3}]},
        {"name": "distribution1d_concentrates_mass", "source": "crates/pyre/src/distribution.rs:192-201",
         "weights": [0.05, 0.9, 0.05],
         "cases": [{"u": 0.5, "t_range": [1.0 / 3.0, 2.0 / 3.0], "pdf": 2.7, "pdf_tol": 1e-3, "bin": 1}]},
    ],
    "distribution2d": [
        {"name": "distribution2d_pdf_normalizes", "source": "crates/pyre/src/distribution.rs:203-220",
         "weights": [float(i) + 1.0 for i in range(16)], "width": 4, "height": 4, "grid": 32,
         "integral": 1.0, "tol": 1e-2},
    ],
    "disney_consistency": {
        "source": "crates/pyre/src/material.rs:332-387", "seed": 0xDEADBEEF, "iters": 500, "tol": 1e-5,
        "bsdfs": [
            {"base_color": [0.7, 0.3, 0.2], "metallic": 0.0, "roughness": 0.4, "specular": 0.5},
            {"base_color": [1.0, 0.766, 0.336], "metallic": 1.0, "roughness": 0.1, "specular": 0.5},
            {"base_color": [0.5, 0.5, 0.5], "metallic": 0.5, "roughness": 0.7, "specular": 0.5},
        ],
    },
}

if __name__ == "__main__":
    out = Path(__file__).with_name("reference_kats.json")
    out.write_text(json.dumps(KATS, indent=1) + "\n")
    print(out)

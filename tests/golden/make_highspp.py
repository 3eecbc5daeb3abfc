"""Writes highspp_refs.npz: 65,536-spp, FP64-accumulated oracle renders of
small crops, the reference images for parity check (d).

Each crop is rendered by the CPU oracle (C++ restatement of the reference's
CPU path) with per-sample radiance summed in float64, samples [0, 65536) of
the reference's per-pixel seeds. Scenes: the plan's Cornell box (256x256),
the reference's own Cornell preset (800x600, crates/pyre-cli/src/main.rs:365-496)
and the procedural studio (1920x1080, thin lens, motion blur, HDRI).

Run:  python tests/golden/make_highspp.py   (a few minutes on 8 cores)
"""
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from pyre_gb300 import presets as P  # noqa: E402

SPP = 65536
CASES = [
    ("cornell_box", 256, 256, [(120, 20, 136, 36), (40, 150, 56, 166), (150, 180, 166, 196)]),
    ("cornell_ref", 800, 600, [(392, 380, 408, 396), (150, 250, 166, 266)]),
    ("studio_procedural", 1920, 1080, [(900, 700, 912, 712), (300, 200, 312, 212)]),
]


def scene_and_camera(name, w, h):
    if name == "cornell_box":
        return P.cornell_box(), P.cornell_box_camera(w, h)
    if name == "cornell_ref":
        return P.cornell_ref(), P.cornell_ref_camera(w, h)
    return P.studio_procedural(), P.studio_procedural_camera(w, h)


def main():
    out = {}
    for name, w, h, crops in CASES:
        sc, cam = scene_and_camera(name, w, h)
        osc = O.OracleScene(sc)
        for k, crop in enumerate(crops):
            t0 = time.time()
            r = osc.render(cam, w, h, SPP, crop=crop, accum64=True)
            mean = r["accum64"] / SPP
            out[f"{name}/{k}"] = mean
            out[f"{name}/{k}/crop"] = np.asarray(crop, np.int32)
            print(f"{name} crop {crop}: {time.time() - t0:.1f} s, mean {mean.mean(axis=(0, 1))}", flush=True)
    np.savez_compressed(Path(__file__).with_name("highspp_refs.npz"), **out)


if __name__ == "__main__":
    main()

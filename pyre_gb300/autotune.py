"""Autotuner for the wavefront's launch knobs.

Knobs (pyre_render_params): wave_paths (queue capacity = paths in flight per
wave), block_size (threads per block of the stage kernels, capped at 224 for
the forward shade and 128 for the traversals; 0 = the library's defaults
256 / 224 / 128), use_graph (CUDA-graph replay),
sort_by_material (shade visits the live paths sorted by material) and
refill_lanes (a warp refetches rays once this many of its lanes are idle) and
bvh_width (instance BVHs traversed as binary, 4-wide or 8-wide nodes).

Search: coordinate descent from the defaults (each knob swept with the others
fixed, best kept), timed with the library's CUDA events. Results are cached in
a JSON file keyed by a workload signature and the GPU name, so repeated runs
reuse the tuned values.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

KNOBS = {
    "wave_paths": [0, 8 << 20, 32 << 20, 128 << 20],  # 0: the library's memory-based choice
    "block_size": [0, 128],  # 0: the library's defaults
    "use_graph": [0, 1],
    "bvh_width": [2, 4, 8],
    "sort_by_material": [0, 1, 3],  # 0: the library's default (off), 1: within tiles, 3: the whole queue
    "refill_lanes": [0, 4, 8, 16, 32],  # 0: the library's defaults (12 closest hit, 8 any hit)
}
DEFAULT = {"wave_paths": 0, "block_size": 0, "use_graph": 0, "bvh_width": 2, "sort_by_material": 0,
           "refill_lanes": 0}


def cache_path() -> Path:
    p = os.environ.get("PYRE_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "pyre_gb300" / "autotune.json"


def signature(kind: str, parts: list) -> str:
    h = hashlib.sha256(kind.encode())
    for x in parts:
        h.update(repr(x).encode())
    try:
        import torch
        h.update(torch.cuda.get_device_name(0).encode())
    except Exception:
        pass
    return h.hexdigest()[:24]


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, entry: dict) -> None:
    data = _load()
    data[key] = entry
    path = cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text(json.dumps(data, indent=1))


def tune(run, key: str, reps: int = 1, use_cache: bool = True) -> tuple[dict, list]:
    """run(knobs) -> device milliseconds. Returns (best knobs, trial log)."""
    if use_cache:
        hit = _load().get(key)
        if hit:
            return hit["best"], hit.get("trials", [])
    trials = []
    cache = {}

    def measure(knobs):
        k = json.dumps(knobs, sort_keys=True)
        if k not in cache:
            cache[k] = min(run(knobs) for _ in range(reps))
            trials.append({"knobs": dict(knobs), "ms": cache[k]})
        return cache[k]

    best = dict(DEFAULT)
    best_ms = measure(best)
    for name, values in KNOBS.items():
        for v in values:
            cand = dict(best)
            cand[name] = v
            ms = measure(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    _store(key, {"best": best, "best_ms": best_ms, "trials": trials})
    return best, trials


def tune_batch(ctx, dscene, spec: list, reps: int = 1, use_cache: bool = True):
    key = signature("batch", [(j["part"], j["width"], j["height"], j["spp"], j["integrator"].max_depth)
                              for j in spec])

    def run(knobs):
        ctx.render_batch(dscene, spec, wave_paths=knobs["wave_paths"], use_graph=knobs["use_graph"],
                         block_size=knobs["block_size"], sort_by_material=knobs["sort_by_material"],
                         refill_lanes=knobs["refill_lanes"], bvh_width=knobs["bvh_width"])
        return ctx.stats().ms_total

    return tune(run, key, reps, use_cache)


def tune_render(ctx, dscene, camera, integrator, width: int, height: int, spp: int, env_sampling: int = 0,
                reps: int = 1, use_cache: bool = True):
    import numpy as np

    from . import native as N
    from .scene import CudaIntegrator
    key = signature("render", [dscene.info().n_triangles, width, height, spp, integrator.max_depth, env_sampling])
    out = np.zeros(width * height * 3, np.float32)

    def run(knobs):
        p = CudaIntegrator.params(width, height, 0, spp, integrator, env_sampling=env_sampling,
                                  wave_paths=knobs["wave_paths"], use_graph=knobs["use_graph"],
                                  block_size=knobs["block_size"], refill_lanes=knobs["refill_lanes"],
                                  bvh_width=knobs["bvh_width"])
        p.sort_by_material = knobs["sort_by_material"]
        ctx.render_into(dscene, camera, p, N.Film(N.fptr(out), None, None, None, N.PYRE_MEM_HOST))
        return ctx.stats().ms_total

    return tune(run, key, reps, use_cache)

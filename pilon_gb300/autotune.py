"""Autotuner for the pileup walk: tile width (positions per CTA), warps per CTA
and the shared-counter variant, chosen by timing the walk kernel (CUDA events
on the engine stream) on the caller's own regions.  Results are cached per
(device name, workload key) in pilon_gb300/_build/autotune.json."""
import json
import os

from .build import BUILD

CACHE = os.path.join(BUILD, "autotune.json")
TILES = (256, 512, 1024, 2048, 4096)
WARPS = (8, 16)
VARIANTS = (0, 1, 2, 3)   # lanes per simple read: 32, 16, 8, 4


def _load():
    try:
        return json.load(open(CACHE))
    except Exception:
        return {}


def tune(engine, regions, params, key, repeats=3, batched=True, force=False):
    """Times every configuration; sets and returns the fastest as
    (tile_width, warps, variant, walk_ms) plus the full table."""
    cache = _load()
    if key in cache and not force:
        t, w, v, ms = cache[key]["best"]
        engine.set_tuning(t, w, v)
        return (t, w, v, ms), cache[key]["table"]
    table = []
    for t in TILES:
        for w in WARPS:
            for v in VARIANTS:
                engine.set_tuning(t, w, v)
                engine.pileup_regions(regions, params, batched=batched)  # warm-up
                best = None
                for _ in range(repeats):
                    engine.pileup_regions(regions, params, batched=batched)
                    walk, total, _ = engine.last_kernel_ms()
                    best = walk if best is None else min(best, walk)
                table.append((t, w, v, best))
    t, w, v, ms = min(table, key=lambda x: x[3])
    engine.set_tuning(t, w, v)
    cache[key] = {"best": [t, w, v, ms], "table": table}
    try:
        os.makedirs(BUILD, exist_ok=True)
        json.dump(cache, open(CACHE, "w"), indent=1)
    except OSError:
        pass
    return (t, w, v, ms), table

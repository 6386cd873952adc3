"""Launch-shape autotuner for the pair kernel and the neighbour list.

Picks threads per atom (4, 8, 16, 32), threads per block (128, 256), the pair-kernel
tile (list entries a lane takes per iteration: 1, or 2 packed in FP32x2 lanes) and the
neighbour skin (1.0, 1.5, 2.0 A) by timing short device-resident NVE runs of a representative
system as production runs them (steps replayed as CUDA graphs; CUDA events on the
engine's stream around the run).  Timing kernels one by one instead adds a launch gap
per kernel, which ranks the shapes of small systems wrongly (7,200 atoms: host-driven
timing picked 8 threads per atom, the graph replay is fastest at 32).  The score of a
candidate is the device time of one step plus the amortised cost of a list rebuild
(rebuild time / expected steps between rebuilds, estimated from the largest
displacement seen during the probe).  Forces do not depend on any of these knobs: the
cutoff test is exact and the skin only sets how many candidates the list carries.

Results are cached in a JSON file keyed by (GPU name, precision, size bucket,
element count), so a production run tunes once per machine and workload class.
"""
from __future__ import annotations

import json
import math
import os
import time
from typing import Dict, Iterable, Optional, Tuple

import numpy as np

from . import capi

CACHE = os.environ.get("LMFF_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "lmff_gb300_tune.json"))


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:  # noqa: BLE001 - name is only a cache key
        return "unknown"


def _bucket(n: int) -> int:
    return int(round(math.log2(max(n, 1))))


def _key(precision: int, n: int, nelem: int) -> str:
    return f"{_gpu_name()}|p{precision}|n2^{_bucket(n)}|e{nelem}"


def load_cache() -> Dict:
    try:
        return json.load(open(CACHE))
    except (OSError, ValueError):
        return {}


def save_cache(c: Dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + f".tmp{os.getpid()}"
        json.dump(c, open(tmp, "w"), indent=1)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def tune(system, tersoff_file: str, ilp_file: str, elements=("C", "B", "N"), precision: int = capi.MIXED,
         device: int = 0, tpas: Iterable[int] = (8, 16, 32), blocks: Iterable[int] = (128, 256),
         skins: Iterable[float] = (1.0, 1.5, 2.0), steps: Optional[int] = None, use_cache: bool = True,
         n_full: Optional[int] = None, tiles: Iterable[int] = (2, 1)) -> Dict:
    """Time the candidates on `system` and return the best {"tpa", "block", "skin", ...}.
    `n_full` (the production system size) selects the cache bucket when `system` is a
    smaller stand-in with the same density.  `steps` (timed steps per candidate) defaults
    to about 2 M atom-steps, 4 to 200 steps."""
    key = _key(precision, n_full or system.n, len(elements))
    if steps is None:
        steps = max(4, min(200, 2_000_000 // max(system.n, 1)))
    cache = load_cache() if use_cache else {}
    if key in cache:
        out = dict(cache[key])
        out["cached"] = True
        return out
    results = []
    for skin in skins:
        for tpa in tpas:
            for block in blocks:
                for tile in (tiles if precision == capi.MIXED else (2,)):
                    eng = capi.Engine(tersoff_file, ilp_file, elements=elements, precision=precision, skin=skin,
                                      device=device)
                    eng.set_option("tpa", tpa)
                    eng.set_option("block", block)
                    eng.set_option("pair_tile", tile)
                    eng.upload(system)
                    eng.run_nve(2, 0.001)   # captures the step graph
                    x0, _, _ = eng.download()
                    eng.run_nve(steps, 0.001)
                    x1, _, _ = eng.download()
                    st = eng.stats()
                    step_ms = st["ms_last_run"] / steps
                    # amortised rebuild: steps until the fastest atom moves skin/2 at the probe's rate
                    L = system.box_hi - system.box_lo
                    d = x1 - x0
                    for c in range(3):
                        if system.periodic[c]:
                            d[:, c] -= L[c] * np.rint(d[:, c] / L[c])
                    vmax = float(np.sqrt((d * d).sum(1)).max()) / steps
                    steps_between = (0.5 * skin / vmax) if vmax > 0 else 1e9
                    build_ms = st["ms_last_build"]
                    score = step_ms + build_ms / max(steps_between, 1.0)
                    results.append({"tpa": tpa, "block": block, "skin": skin, "tile": tile, "step_ms": step_ms,
                                    "build_ms": build_ms,
                                    "steps_between_rebuilds": steps_between, "score_ms": score})
                    eng.close()
    best = min(results, key=lambda r: r["score_ms"])
    out = {"tpa": best["tpa"], "block": best["block"], "skin": best["skin"], "tile": best["tile"],
           "score_ms": best["score_ms"],
           "probe_atoms": system.n, "steps": steps, "key": key, "candidates": results, "when": time.time()}
    if use_cache:
        cache[key] = {k: v for k, v in out.items() if k != "candidates"}
        save_cache(cache)
    out["cached"] = False
    return out

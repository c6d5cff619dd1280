"""Launch-configuration tuner for the batched march.

The persistent march kernel has four knobs that change speed but never
results: the ray-block shape of its work items (128 consecutive rays, or
2 x 64, 4 x 32, 8 x 16, 16 x 8 rectangles of rays: the footprint of a block's 8-corner
neighbourhoods in a tilted march), the march variant for Lerp/Slerp
(warp-cooperative with the interpolating steps compacted across the warp, or
one thread per ray; both give the same bits), work items taken per queue grab,
and resident CTAs per SM.  ``tune(batch)`` times them on the batch itself
(CUDA events, after a warm-up run) by coordinate descent — shape, then
variant, then grab, then CTAs, each with the best of the knobs before — and
keeps the fastest; the best shape and variant depend on the tissue (sparse
tiles favour the cooperative march, dense ones the per-thread march).
Choices are cached in a JSON file keyed by device, interpolation mode and a
coarse shape bucket (pairs, mean steps per ray), so a later batch of the
same kind skips the search.  Cache path: ``$FPGB_AUTOTUNE_CACHE`` or
``fastpli_gb300/_lib/autotune.json``.
"""

import json
import math
import os
import threading

_LOCK = threading.Lock()
_DEFAULT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")
CTAS = (0, 4, 2)        # 0 = as many as fit
GRABS = (1, 2, 4)
COOP = (1, 0)
SHAPES = (0, 1, 2, 3, 4)   # TileBatch.SHAPES
START = (0, 2, 1, 0)    # (ctas_per_sm, items_per_grab, coop, shape)


def cache_path():
    return os.environ.get("FPGB_AUTOTUNE_CACHE", _DEFAULT)


_MEMO = {}


def _load():
    """The cache file's contents, parsed again only when the file changed
    (the server reads it for every batch it launches)."""
    p = cache_path()
    try:
        st = os.stat(p)
    except OSError:
        return {}
    stamp = (p, st.st_mtime_ns, st.st_size)
    if _MEMO.get("stamp") != stamp:
        try:
            with open(p) as f:
                data = json.load(f)
        except Exception:
            data = {}
        _MEMO.update(stamp=stamp, data=data)
    return dict(_MEMO["data"])


def _store(d):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def key(batch):
    import torch
    name = torch.cuda.get_device_name()
    interp = batch._setup.struct.interpolate
    pairs = int(batch.info.n_pairs)
    steps_per_ray = batch.steps / max(1, sum(
        int(t.dim[0]) * int(t.dim[1]) * len(batch.pairs_of(i)) for i, t in enumerate(batch.tiles)))
    return (f"{name}|interp{interp}|pairs2^{int(math.log2(max(1, pairs)))}"
            f"|z2^{int(math.log2(max(1, steps_per_ray)))}|v5")


def time_config(batch, ctas, grab, coop=1, shape=0, reps=3):
    import torch
    batch.run(ctas, grab, coop, shape=shape)  # warm
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        batch.run(ctas, grab, coop, shape=shape)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(batch, force=False, reps=3):
    """Pick (ctas_per_sm, items_per_grab, coop, shape) for ``batch`` (already
    allocated); sets ``batch.config`` and returns (config, ms, table)."""
    k = key(batch)
    with _LOCK:
        cache = _load()
    if not force and k in cache and len(cache[k]["config"]) == 4:
        batch.config = tuple(cache[k]["config"])
        return batch.config, cache[k]["ms"], None
    table = {}
    best = START
    for dim, values in ((3, SHAPES), (2, COOP), (1, GRABS), (0, CTAS)):
        for v in values:
            cand = tuple(v if i == dim else c for i, c in enumerate(best))
            if cand not in table:
                table[cand] = time_config(batch, *cand, reps=reps)
        best = min((c for c in table if all(c[i] == best[i] for i in range(4) if i != dim)),
                   key=table.get)
    batch.config = best
    with _LOCK:
        cache = _load()
        cache[k] = {"config": list(best), "ms": table[best]}
        _store(cache)
    return best, table[best], table

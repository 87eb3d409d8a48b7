"""Autotuner for the draw path's execution choices: the screen-tile side of ordered (blending) passes and
the launch schedule of a command buffer (batched phases or one persistent kernel).

`tune(time_config, ...)` measures every candidate with a caller-supplied timing function and returns the
fastest; `Tuner` wraps it with a JSON cache keyed by a workload signature (GPU name, raster classes,
bucketed draw count, triangle count and resolution), so a workload seen before is not re-measured.
`scene_timer` is the timing function for a recorded scene on this driver: it re-records only the
command buffer (vkEndCommandBuffer lowers it with the current options) over the same resident buffers
and times submissions with CUDA events on the queue stream."""
import json
import math
import os
from dataclasses import dataclass

MODES = ("batched", "persistent")
TILES = (8, 16, 32, 64)


@dataclass(frozen=True)
class Config:
    mode: str
    tile: int


def candidates(modes=MODES, tiles=TILES, ordered=True):
    """every (mode, tile) pair; the tile side only matters to ordered passes, so opaque-only workloads
    try one tile"""
    ts = tiles if ordered else (16,)
    return [Config(m, t) for m in modes for t in ts]


def tune(time_config, configs, repeats=1):
    """time each config (`time_config(cfg)` -> ms, best of `repeats`); returns (best, {config: ms})"""
    table = {}
    for cfg in configs:
        table[cfg] = min(time_config(cfg) for _ in range(max(1, repeats)))
    best = min(table, key=lambda c: (table[c], c.mode != "batched", c.tile))
    return best, table


def _bucket(x):
    return 0 if x <= 0 else int(round(math.log2(x)))


def signature(gpu, ordered, draws, triangles, width, height):
    """workloads that share a signature share a tuning result"""
    return "%s|%s|d%d|t%d|p%d" % (gpu, "ordered" if ordered else "opaque", _bucket(draws), _bucket(triangles),
                                   _bucket(width * height))


class Tuner:
    def __init__(self, path=None):
        self.path = path or os.path.join(os.path.expanduser("~"), ".cache", "kazan_gb300", "tune.json")
        self.cache = {}
        if os.path.exists(self.path):
            try:
                with open(self.path, encoding="utf-8") as f:
                    self.cache = json.load(f)
            except (OSError, ValueError):
                self.cache = {}

    def lookup(self, sig):
        e = self.cache.get(sig)
        return Config(e["mode"], int(e["tile"])) if e else None

    def choose(self, sig, time_config, configs, repeats=1):
        """the cached choice for `sig`, or measure `configs` and remember the best; returns (config, table or
        None when cached)"""
        hit = self.lookup(sig)
        if hit is not None:
            return hit, None
        best, table = tune(time_config, configs, repeats)
        self.cache[sig] = {"mode": best.mode, "tile": best.tile,
                           "ms": {"%s/%d" % (c.mode, c.tile): round(v, 4) for c, v in table.items()}}
        self.save()
        return best, table

    def save(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w", encoding="utf-8") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def scene_timer(run, steps=5, warmup=2):
    """timing function for a recorded SceneRun: re-record its command buffer with `cfg` and return the
    mean ms per submission measured with CUDA events on the queue stream"""
    import torch

    def time_config(cfg):
        d = run.r.drv
        d.set_option("mode", cfg.mode)
        d.set_option("tile", cfg.tile)
        old = run.cb
        run.cb = run.record()
        run.r.free_command_buffer(old)
        stream = torch.cuda.ExternalStream(run.r.stream())
        for _ in range(warmup):
            run.submit()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            run.submit(wait=False)
        e1.record(stream)
        e1.synchronize()
        run.r.drv.vkQueueWaitIdle(run.r.queue)
        return e0.elapsed_time(e1) / steps

    return time_config

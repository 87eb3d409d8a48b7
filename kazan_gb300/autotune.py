"""Autotuner for the draw path's execution choices: the launch schedule of a command buffer (batched phases
or one persistent kernel), the screen-tile side of ordered (blending) passes, and for opaque passes the
visibility path's knobs: the largest triangle box a geometry warp rasterises (`warp_px`; larger triangles
become jobs), the 8x8 blocks per large-triangle job (`job_blocks`) and the geometry kernel's blocks per SM
(`geo_blocks`, 0 = all resident).

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
WARP_PX = (96, 128, 256, 384)
JOB_BLOCKS = (8, 32)
GEO_BLOCKS = (2, 3)
DEFAULTS = {"warp_px": 192, "job_blocks": 16, "geo_blocks": 0}


@dataclass(frozen=True)
class Config:
    mode: str
    tile: int
    warp_px: int = DEFAULTS["warp_px"]
    job_blocks: int = DEFAULTS["job_blocks"]
    geo_blocks: int = DEFAULTS["geo_blocks"]

    def label(self):
        """'mode/tile', followed by the knobs that differ from their defaults"""
        extra = "".join("/%s%d" % (k, getattr(self, k)) for k in ("warp_px", "job_blocks", "geo_blocks")
                        if getattr(self, k) != DEFAULTS[k])
        return "%s/%d%s" % (self.mode, self.tile, extra)

    def options(self):
        """the driver options that select this configuration"""
        return {"mode": self.mode, "tile": self.tile, "warp_px": self.warp_px, "job_blocks": self.job_blocks,
                "geo_blocks": self.geo_blocks}


def candidates(modes=MODES, tiles=TILES, ordered=True, knobs=True):
    """ordered workloads: every (mode, tile) pair.  Opaque workloads (the tile side does not matter to
    them): each mode at the default knobs, then, in the batched schedule, each knob varied alone"""
    if ordered:
        return [Config(m, t) for m in modes for t in tiles]
    out = [Config(m, 16) for m in modes]
    if knobs and "batched" in modes:
        out += [Config("batched", 16, warp_px=w) for w in WARP_PX]
        out += [Config("batched", 16, job_blocks=j) for j in JOB_BLOCKS]
        out += [Config("batched", 16, geo_blocks=g) for g in GEO_BLOCKS]
    return out


def tune(time_config, configs, repeats=1):
    """time each config (`time_config(cfg)` -> ms, best of `repeats`); returns (best, {config: ms})"""
    table = {}
    for cfg in configs:
        table[cfg] = min(time_config(cfg) for _ in range(max(1, repeats)))
    best = min(table, key=lambda c: (table[c], c.mode != "batched", c.tile, c.label()))
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
        if not e:
            return None
        return Config(e["mode"], int(e["tile"]), *(int(e.get(k, DEFAULTS[k])) for k in
                                                   ("warp_px", "job_blocks", "geo_blocks")))

    def choose(self, sig, time_config, configs, repeats=1):
        """the cached choice for `sig`, or measure `configs` and remember the best; returns (config, table or
        None when cached)"""
        hit = self.lookup(sig)
        if hit is not None:
            return hit, None
        best, table = tune(time_config, configs, repeats)
        self.cache[sig] = dict(best.options(), ms={c.label(): round(v, 4) for c, v in table.items()})
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
        for k, v in cfg.options().items():
            d.set_option(k, v)
        old = run.cb
        try:
            run.cb = run.record()
        finally:
            for k, v in DEFAULTS.items():
                d.set_option(k, v)
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

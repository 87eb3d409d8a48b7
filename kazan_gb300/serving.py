"""Serving loop for the draw path: render requests from many clients arrive over time and are submitted to
one Vulkan queue in batches.

Workload (the serving configuration): 64 clients; aggregate Poisson arrivals at rate lambda; each client owns
a resident scene (a sphere mesh from the single-draw generator with a log-uniform triangle count in
[1,000, 500,000], one resolution drawn from {256x256, 512x512, 1024x1024, 1920x1080}, Lambert shading) and a
few recorded camera views; a request renders one view of its client's scene.

- Residency and admission: vertex/index buffers, attachments and the driver's per-command-buffer scratch
  stay on the device.  Clients are admitted in order while their device bytes fit the HBM budget;
  requests of clients that were not admitted are rejected (counted, not served).
- Batching: the dispatcher submits every request that has arrived (up to `max_batch`) with one
  vkQueueSubmit and one fence, keeping at most `max_inflight` submissions in flight.
- Latency: arrival time -> the host sees the submission's fence signalled.
- The one-request-at-a-time baseline serves the same request stream with max_batch = max_inflight = 1.

The scheduler (`serve`) drives any backend with submit / poll, so the policy is tested on the CPU with a
simulated queue (tests/test_serving.py)."""
import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]


@dataclass
class ClientSpec:
    index: int
    triangles: int
    width: int
    height: int
    seed: int


@dataclass
class Request:
    client: int
    view: int
    arrival: float                 # seconds from the start of the run
    start: Optional[float] = None  # submitted
    done: Optional[float] = None   # fence seen signalled
    rejected: bool = False


def client_specs(n_clients=64, seed=5, tmin=1000, tmax=500_000):
    """the clients' scenes: triangle count log-uniform in [tmin, tmax], resolution uniform over RESOLUTIONS"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_clients):
        t = int(math.exp(rng.uniform(math.log(tmin), math.log(tmax))))
        w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
        out.append(ClientSpec(i, t, w, h, seed ^ (i + 1)))
    return out


def poisson_requests(rate, n_requests, n_clients, n_views, seed=5):
    """`n_requests` arrivals of a Poisson process of aggregate rate `rate` (per second); each request names
    a uniformly drawn client and view"""
    rng = np.random.default_rng(seed * 7919 + int(rate))
    gaps = rng.exponential(1.0 / rate, n_requests)
    t = np.cumsum(gaps)
    clients = rng.integers(0, n_clients, n_requests)
    views = rng.integers(0, n_views, n_requests)
    return [Request(int(c), int(v), float(a)) for a, c, v in zip(t, clients, views)]


def admit(sizes, budget):
    """clients admitted in order while the running total of their device bytes stays within `budget`"""
    admitted, total = [], 0
    for i, s in enumerate(sizes):
        if total + s <= budget:
            admitted.append(i)
            total += s
    return admitted, total


def percentile(values, q):
    """the q-th percentile (0..100) by linear interpolation between closest ranks"""
    if not values:
        return None
    v = sorted(values)
    if len(v) == 1:
        return v[0]
    pos = (len(v) - 1) * q / 100.0
    lo = int(math.floor(pos))
    hi = min(lo + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (pos - lo)


class Backend:
    """what the scheduler needs from the GPU side"""

    def submit(self, requests):  # -> handle
        raise NotImplementedError

    def poll(self, handle):  # -> True when the submission has completed
        raise NotImplementedError

    def wait(self, handle):
        while not self.poll(handle):
            time.sleep(0)

    def triangles(self, request):
        raise NotImplementedError


@dataclass
class ServeResult:
    rate: float
    served: int
    rejected: int
    wall_s: float
    p50_ms: Optional[float]
    p99_ms: Optional[float]
    mean_batch: float
    mtris_per_s: float
    latencies_ms: List[float] = field(default_factory=list, repr=False)

    def as_dict(self):
        return {"rate_req_per_s": self.rate, "served": self.served, "rejected": self.rejected,
                "wall_s": round(self.wall_s, 4), "p50_ms": _r(self.p50_ms), "p99_ms": _r(self.p99_ms),
                "mean_batch": round(self.mean_batch, 2), "mtris_per_s": round(self.mtris_per_s, 2),
                "achieved_req_per_s": round(self.served / self.wall_s, 1) if self.wall_s > 0 else None}


def _r(x):
    return None if x is None else round(x, 4)


def serve(backend, requests, admitted, max_batch=64, max_inflight=4, clock=time.perf_counter, sleep=time.sleep):
    """Serve `requests` (sorted by arrival) in real time on `backend`; requests of clients not in
    `admitted` are rejected.  Returns a ServeResult."""
    admitted = set(admitted)
    pending = []          # arrived, not yet submitted
    inflight = []         # (handle, [requests])
    batches = []
    served = []
    i, n = 0, len(requests)
    t0 = clock()
    while i < n or pending or inflight:
        now = clock() - t0
        while i < n and requests[i].arrival <= now:
            r = requests[i]
            if r.client in admitted:
                pending.append(r)
            else:
                r.rejected = True
            i += 1
        # retire completed submissions in order
        while inflight and backend.poll(inflight[0][0]):
            h, reqs = inflight.pop(0)
            t = clock() - t0
            for r in reqs:
                r.done = t
            served.extend(reqs)
        if pending and len(inflight) < max_inflight:
            batch, pending = pending[:max_batch], pending[max_batch:]
            t = clock() - t0
            for r in batch:
                r.start = t
            inflight.append((backend.submit(batch), batch))
            batches.append(len(batch))
            continue
        if not pending and not inflight and i < n:
            wait = requests[i].arrival - (clock() - t0)
            if wait > 0:
                sleep(min(wait, 0.001))
        elif inflight:
            sleep(0)
    wall = clock() - t0
    lat = [(r.done - r.arrival) * 1e3 for r in served]
    tris = sum(backend.triangles(r) for r in served)
    rate = n / requests[-1].arrival if n and requests[-1].arrival > 0 else 0.0
    return ServeResult(rate=rate, served=len(served), rejected=sum(r.rejected for r in requests), wall_s=wall,
                       p50_ms=percentile(lat, 50), p99_ms=percentile(lat, 99),
                       mean_batch=(sum(batches) / len(batches)) if batches else 0.0,
                       mtris_per_s=tris / wall / 1e6 if wall > 0 else 0.0, latencies_ms=lat)


class VulkanBackend(Backend):
    """the clients' resident scenes on one Vulkan device of this driver; one recorded command buffer per
    (client, view); a submission is one vkQueueSubmit of its requests' command buffers with one fence"""

    def __init__(self, renderer, specs, n_views=4, mode="batched"):
        from ctypes import byref, c_uint32, c_void_p
        from . import render, scenes, vk
        self.r, self.vk = renderer, vk
        self.specs = specs
        self.n_views = n_views
        self.cbs = []         # per client: one recorded command buffer per view
        self.sizes = []       # per client: device bytes (buffers, attachments, driver scratch per view)
        for sp in specs:
            v, idx = scenes.sphere_mesh(sp.seed, sp.triangles)
            mvps = []
            for k in range(n_views):
                m = np.empty(16, dtype=np.float32)
                scenes.lib().kz_mvp_batched(sp.seed, k, sp.width, sp.height, scenes._fp(m))
                mvps.append(m)
            sc = scenes.Scene("serve", sp.width, sp.height, "lambert", v, idx,
                              [scenes.Draw(0, sp.triangles, 0, mvps[0])], cull=2)
            run = render.SceneRun(renderer, sc, host_visible=False, mode=mode)
            views = [run.cb]
            for m in mvps[1:]:
                sc.draws[0].mvp = m
                views.append(run.record())
            self.cbs.append(views)
            st = renderer.drv.stats(run.cb)
            per_view_scratch = st.rec_cap * 64 + st.pair_cap * 4 + sp.width * sp.height * 8 + 4096
            self.sizes.append(v.nbytes + idx.nbytes + sp.width * sp.height * 8 + n_views * per_view_scratch)
        self._fences = []
        self._c_void_p, self._byref, self._c_uint32 = c_void_p, byref, c_uint32

    def _fence(self):
        if self._fences:
            return self._fences.pop()
        vk = self.vk
        f = self._c_void_p()
        fci = vk.VkFenceCreateInfo(vk.ST_FENCE_CREATE_INFO, None, 0)
        vk.check("vkCreateFence", self.r.drv.vkCreateFence(self.r.device, self._byref(fci), None, self._byref(f)))
        return f

    def submit(self, requests):
        vk = self.vk
        cbs = (self._c_void_p * len(requests))(*[self.cbs[q.client][q.view].value for q in requests])
        si = vk.VkSubmitInfo(vk.ST_SUBMIT_INFO, None, 0, None, None, len(requests), cbs, 0, None)
        f = self._fence()
        vk.check("vkQueueSubmit", self.r.drv.vkQueueSubmit(self.r.queue, 1, self._byref(si), f))
        return f

    def poll(self, f):
        rc = self.r.drv.vkGetFenceStatus(self.r.device, f)
        if rc == self.vk.VK_SUCCESS:
            arr = (self._c_void_p * 1)(f)
            self.r.drv.vkResetFences(self.r.device, 1, arr)
            self._fences.append(f)
            return True
        if rc != self.vk.VK_NOT_READY:
            raise self.vk.VkError("vkGetFenceStatus", rc)
        return False

    def triangles(self, request):
        return self.specs[request.client].triangles

    def close(self):
        for f in self._fences:
            self.r.drv.vkDestroyFence(self.r.device, f, None)
        self._fences = []


def sweep(backend, admitted, rates, n_requests, n_views, seed=5, max_batch=64, max_inflight=4):
    """serve the same-rate request streams batched and one at a time; returns (batched, one_at_a_time)"""
    batched, single = [], []
    for rate in rates:
        reqs = poisson_requests(rate, n_requests, len(backend.specs), n_views, seed)
        batched.append(serve(backend, reqs, admitted, max_batch=max_batch, max_inflight=max_inflight))
        reqs = poisson_requests(rate, n_requests, len(backend.specs), n_views, seed)
        single.append(serve(backend, reqs, admitted, max_batch=1, max_inflight=1))
    return batched, single

"""Serving loop for the draw path: render requests from many clients arrive over time and are submitted to
one Vulkan queue in batches.

Workload (the serving configuration): 64 clients; aggregate Poisson arrivals at rate lambda.  Every request
carries its own data: a resolution drawn uniformly from {256x256, 512x512, 1024x1024, 1920x1080}, a triangle
count log-uniform in [1,000, 500,000] and a random model-view-projection matrix (a uniform random rotation
and a translation in [-5, 5]^3, as the batched draws).  Each client keeps resident a sphere mesh of 500,000
triangles from the single-draw generator; a request draws the first `triangles` of them.

- Residency and admission: the clients' meshes, one colour + depth framebuffer per client and resolution,
  and one recorded command buffer per client and resolution (with the driver's scratch) stay on the device.
  Clients are admitted in order while their device bytes fit the HBM budget; requests of clients that were
  not admitted are rejected (counted, not served).
- Per-request data: the command buffers draw through vkCmdDrawIndexedIndirect with the matrix in a uniform
  buffer; before a request is submitted the host writes its matrix (64 bytes) and its indirect command
  (20 bytes) into that command buffer's host-visible parameter buffers, which the driver uploads with the
  submission.  Two requests that need the same command buffer are never in flight together: the dispatcher
  holds the later one back.
- Batching: the dispatcher submits every request that has arrived (up to `max_batch`) with one
  vkQueueSubmit and one fence, keeping at most `max_inflight` submissions in flight.
- Latency: arrival time -> the host sees the submission's fence signalled.
- The one-request-at-a-time baseline serves the same request stream with max_batch = max_inflight = 1.

The scheduler (`serve`) drives any backend with submit / poll, so the policy is tested on the CPU with a
simulated queue (tests/test_serving.py)."""
import ctypes
import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080)]
TMIN, TMAX = 1000, 500_000


@dataclass
class ClientSpec:
    index: int
    triangles: int   # triangles of the client's resident mesh (requests draw a prefix of them)
    seed: int


@dataclass
class Request:
    client: int
    view: int                      # the request's camera: stream index of its random MVP (kz_mvp_batched)
    arrival: float                 # seconds from the start of the run
    res: int = 0                   # index into RESOLUTIONS
    triangles: int = TMIN          # triangles drawn (a prefix of the client's mesh)
    start: Optional[float] = None  # submitted
    done: Optional[float] = None   # fence seen signalled
    rejected: bool = False


def client_specs(n_clients=64, seed=5, tmax=TMAX):
    """the clients' resident meshes: `tmax` triangles each, their own seeds"""
    return [ClientSpec(i, tmax, seed ^ (i + 1)) for i in range(n_clients)]


def poisson_requests(rate, n_requests, n_clients, seed=5, tmin=TMIN, tmax=TMAX):
    """`n_requests` arrivals of a Poisson process of aggregate rate `rate` (per second); each request names a
    uniformly drawn client and resolution, a triangle count log-uniform in [tmin, tmax] and its own camera"""
    rng = np.random.default_rng(seed * 7919 + int(rate))
    gaps = rng.exponential(1.0 / rate, n_requests)
    t = np.cumsum(gaps)
    clients = rng.integers(0, n_clients, n_requests)
    res = rng.integers(0, len(RESOLUTIONS), n_requests)
    tris = np.exp(rng.uniform(math.log(tmin), math.log(tmax), n_requests)).astype(np.int64)
    tris = np.clip(tris, tmin, tmax)
    return [Request(int(c), k, float(a), int(rz), int(n)) for k, (a, c, rz, n) in enumerate(zip(t, clients, res, tris))]


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

    def slot(self, request):
        """what a request occupies while it is in flight (two requests with the same slot are never in flight
        together); None: nothing"""
        return None


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
    busy = set()          # slots of the requests in flight
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
                busy.discard(backend.slot(r))
            served.extend(reqs)
        if pending and len(inflight) < max_inflight:
            batch, held = [], []
            for r in pending:
                sl = backend.slot(r)
                if len(batch) < max_batch and (sl is None or sl not in busy):
                    batch.append(r)
                    if sl is not None:
                        busy.add(sl)
                else:
                    held.append(r)
            if batch:
                pending = held
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
    """the clients' resident meshes, framebuffers and command buffers on one Vulkan device of this driver; a
    submission is one vkQueueSubmit of its requests' command buffers with one fence"""

    def __init__(self, renderer, specs, mode="batched"):
        from ctypes import byref, c_uint32, c_void_p
        from . import render, scenes, vk
        self.r, self.vk, self.render, self.scenes = renderer, vk, render, scenes
        self.specs = specs
        self.meshes = []      # per client: (vertices, indices) on the host (for checks)
        self.runs = []        # per client: one SceneRun per resolution (indirect draw, matrix in a uniform buffer)
        self.params = []      # per client and resolution: (mapped uniform buffer, mapped indirect command)
        self.sizes = []       # per client: device bytes (mesh, framebuffers, command buffers' scratch)
        for sp in specs:
            v, idx = scenes.sphere_mesh(sp.seed, sp.triangles)
            self.meshes.append((v, idx))
            vb = renderer.create_buffer(v.nbytes, vk.BUFFER_USAGE_VERTEX, False)
            renderer.write_buffer(vb, v)
            ib = renderer.create_buffer(idx.nbytes, vk.BUFFER_USAGE_INDEX, False)
            renderer.write_buffer(ib, idx)
            size = v.nbytes + idx.nbytes
            runs, params = [], []
            for w, h in RESOLUTIONS:
                sc = scenes.Scene("serve", w, h, "lambert", v, idx, [scenes.Draw(0, sp.triangles, 0, self.mvp(sp, 0, w, h))],
                                  cull=2, ubo=True)
                run = render.SceneRun(renderer, sc, host_visible=False, mode=mode, indirect="host",
                                      ubo_host_visible=True, buffers=(vb, ib))
                runs.append(run)
                params.append((renderer.map(run.ubo_buf), renderer.map(run.cmds)))
                st = renderer.drv.stats(run.cb)
                size += w * h * 8 + st.rec_cap * 64 + st.pair_cap * 4 + w * h * 8 + 65536
            self.runs.append(runs)
            self.params.append(params)
            self.sizes.append(size)
        self._fences = []
        self._c_void_p, self._byref, self._c_uint32 = c_void_p, byref, c_uint32

    def mvp(self, spec, view, width, height):
        """the column-major matrix of camera `view` of a client (random rotation, translation in [-5, 5]^3)"""
        m = np.empty(16, dtype=np.float32)
        self.scenes.lib().kz_mvp_batched(spec.seed, view, width, height, self.scenes._fp(m))
        return m

    def request_scene(self, q):
        """what request q renders, as a scene (for the oracle)"""
        v, idx = self.meshes[q.client]
        w, h = RESOLUTIONS[q.res]
        sp = self.specs[q.client]
        return self.scenes.Scene("serve", w, h, "lambert", v, idx,
                                 [self.scenes.Draw(0, q.triangles, 0, self.mvp(sp, q.view, w, h))], cull=2, ubo=True)

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
        for q in requests:
            sp = self.specs[q.client]
            w, h = RESOLUTIONS[q.res]
            ubo, cmd = self.params[q.client][q.res]
            m = self.mvp(sp, q.view, w, h)
            ctypes.memmove(ubo, m.ctypes.data, 64)
            c = np.array([3 * min(q.triangles, sp.triangles), 1, 0, 0, 0], dtype=np.uint32)
            ctypes.memmove(cmd, c.ctypes.data, c.nbytes)
        cbs = (self._c_void_p * len(requests))(*[self.runs[q.client][q.res].cb.value for q in requests])
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
        return min(request.triangles, self.specs[request.client].triangles)

    def slot(self, request):
        return (request.client, request.res)

    def image(self, request):
        """the colour image of request's framebuffer (read after the request completed)"""
        return self.runs[request.client][request.res].read()[0]

    def close(self):
        for f in self._fences:
            self.r.drv.vkDestroyFence(self.r.device, f, None)
        self._fences = []


def sweep(backend, admitted, rates, n_requests, seed=5, max_batch=64, max_inflight=4, tmin=TMIN, tmax=TMAX):
    """serve the same-rate request streams batched and one at a time; returns (batched, one_at_a_time)"""
    batched, single = [], []
    for rate in rates:
        reqs = poisson_requests(rate, n_requests, len(backend.specs), seed, tmin, tmax)
        batched.append(serve(backend, reqs, admitted, max_batch=max_batch, max_inflight=max_inflight))
        reqs = poisson_requests(rate, n_requests, len(backend.specs), seed, tmin, tmax)
        single.append(serve(backend, reqs, admitted, max_batch=1, max_inflight=1))
    return batched, single

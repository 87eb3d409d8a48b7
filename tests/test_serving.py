"""The serving loop's host logic on the CPU: request generation, HBM-budget admission, percentiles, and
the batching scheduler against a simulated queue (a FIFO device with a per-request service time)."""
import numpy as np
import pytest

from kazan_gb300 import serving


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 2e-6)


class SimQueue(serving.Backend):
    """a device that runs submissions in order; a request costs `base + per_tri * triangles` seconds and a
    submission adds `launch` seconds; the host spends `host` seconds per submit.  With `slots`, a request
    occupies its (client, resolution) slot while in flight, and the queue records any overlap."""

    def __init__(self, clock, base=20e-6, per_tri=2e-10, launch=5e-6, host=10e-6, slots=False):
        self.clock = clock
        self.base, self.per_tri, self.launch, self.host = base, per_tri, launch, host
        self.free_at = 0.0
        self.submissions = 0
        self.slots = slots
        self.inflight = {}   # slot -> completion time
        self.overlaps = 0

    def submit(self, requests):
        self.clock.t += self.host
        start = max(self.clock.t, self.free_at)
        cost = self.launch + sum(self.base + self.per_tri * r.triangles for r in requests)
        self.free_at = start + cost
        self.submissions += 1
        if self.slots:
            for r in requests:
                sl = self.slot(r)
                if self.inflight.get(sl, -1.0) > self.clock.t:
                    self.overlaps += 1
                self.inflight[sl] = self.free_at
        return self.free_at

    def poll(self, handle):
        return self.clock.t >= handle

    def triangles(self, request):
        return request.triangles

    def slot(self, request):
        return (request.client, request.res) if self.slots else None


def test_client_specs_and_requests_are_seeded():
    a, b = serving.client_specs(), serving.client_specs()
    assert a == b and len(a) == 64 and all(s.triangles == 500_000 for s in a)
    r1 = serving.poisson_requests(1000, 4000, 64)
    r2 = serving.poisson_requests(1000, 4000, 64)
    assert [(r.client, r.view, r.arrival, r.res, r.triangles) for r in r1] == \
        [(r.client, r.view, r.arrival, r.res, r.triangles) for r in r2]
    rate = len(r1) / r1[-1].arrival
    assert 900 < rate < 1100
    # every request its own camera; resolutions uniform; triangle counts log-uniform in [1000, 500000]
    assert len({r.view for r in r1}) == len(r1)
    counts = np.bincount([r.res for r in r1], minlength=4)
    assert counts.min() > 0.2 * len(r1)
    t = np.array([r.triangles for r in r1])
    assert t.min() >= 1000 and t.max() <= 500_000
    assert abs(np.mean(np.log(t)) - 0.5 * (np.log(1000) + np.log(500_000))) < 0.15


def test_admission_respects_budget():
    admitted, total = serving.admit([10, 20, 30, 5, 40], 50)
    assert admitted == [0, 1, 3] and total == 35
    assert serving.admit([], 10) == ([], 0)


def test_percentile_matches_numpy():
    v = list(np.random.default_rng(1).exponential(3.0, 1001))
    for q in (0, 50, 90, 99, 100):
        assert serving.percentile(v, q) == pytest.approx(np.percentile(v, q))
    assert serving.percentile([], 50) is None


def _run(rate, max_batch, max_inflight, admitted=None, n=2000, slots=False):
    clock = FakeClock()
    specs = serving.client_specs()
    q = SimQueue(clock, slots=slots)
    reqs = serving.poisson_requests(rate, n, len(specs))
    adm = list(range(len(specs))) if admitted is None else admitted
    res = serving.serve(q, reqs, adm, max_batch=max_batch, max_inflight=max_inflight, clock=clock,
                        sleep=clock.sleep)
    return res, reqs, q


def test_every_admitted_request_is_served_once_and_in_time_order():
    res, reqs, q = _run(2000, 64, 4)
    assert res.served == len(reqs) and res.rejected == 0
    for r in reqs:
        assert r.arrival <= r.start <= r.done
    assert res.p50_ms <= res.p99_ms


def test_rejected_clients_are_not_served():
    res, reqs, q = _run(2000, 64, 4, admitted=list(range(32)))
    assert res.rejected == sum(1 for r in reqs if r.client >= 32) > 0
    assert res.served == len(reqs) - res.rejected


def test_batching_beats_one_at_a_time_under_load():
    """near the simulated device's capacity batching cuts queueing latency; above it, batching also
    raises throughput (fewer submissions, no per-request submit cost on the critical path)"""
    batched, _, qb = _run(20000, 64, 4)
    single, _, qs = _run(20000, 1, 1)
    assert single.mean_batch == 1.0 and batched.mean_batch > 1.0
    assert batched.p99_ms < single.p99_ms
    batched, _, qb = _run(50000, 64, 4)
    single, _, qs = _run(50000, 1, 1)
    assert batched.mean_batch > 1.5 and qb.submissions < qs.submissions
    assert batched.p99_ms < single.p99_ms
    assert batched.mtris_per_s > single.mtris_per_s


def test_requests_sharing_a_slot_are_never_in_flight_together():
    """requests of one client and resolution use one command buffer and its parameter buffers: the
    dispatcher holds a request back while another with the same slot is in flight"""
    res, reqs, q = _run(50000, 64, 4, slots=True)
    assert res.served == len(reqs) and q.overlaps == 0
    for r in reqs:
        assert r.arrival <= r.start <= r.done

"""GPU checks at the workloads' full sizes: every configuration rendered through the Vulkan entry points
equals the CPU oracle bit for bit (colour bytes, depth bits, fragment count); the launch schedules and
tile sides agree with each other; allocation failures injected on the host come back as Vulkan errors and
leave the driver usable; and the serving loop serves a short request stream."""
import ctypes
import os

import numpy as np
import pytest

from kazan_gb300 import render, scenes, serving, vk
from oracle import kz_oracle

THREADS = os.cpu_count() or 4

WORKLOADS = {
    "plain_2048_tris_256sq": lambda: scenes.small_soup(),
    "single_1M_tris_1080p": lambda: scenes.single_large(),
    "batched_4096_draws_2048sq": lambda: scenes.batched(),
    "blend_200K_tris_1080p": lambda: scenes.ordered_blend(),
}


@pytest.fixture(scope="module")
def workloads():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = WORKLOADS[name]()
        return cache[name]
    return get


def _render(renderer, scene, mode="batched", tile=16):
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    run.submit()
    color, depth = run.read()
    st = run.stats()
    renderer.free_command_buffer(run.cb)
    return color, depth, st


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_fullsize_parity_with_oracle(renderer, workloads, name):
    scene = workloads(name)
    color, depth, st = _render(renderer, scene)
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=THREADS)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "%s: colour differs at %d pixels, first %s" % (name, len(mism), mism[:1])
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32)), name
    assert st.status == 0
    assert st.fragments == ost["fragments"] % (1 << 32)


@pytest.mark.gpu
def test_fullsize_schedules_agree(renderer, workloads):
    scene = workloads("batched_4096_draws_2048sq")
    c1, d1, _ = _render(renderer, scene, mode="batched")
    c2, d2, _ = _render(renderer, scene, mode="persistent")
    assert np.array_equal(c1, c2) and np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [8, 32])
def test_fullsize_blend_tiles_agree(renderer, workloads, tile):
    scene = workloads("blend_200K_tris_1080p")
    c1, d1, _ = _render(renderer, scene, tile=16)
    c2, d2, st = _render(renderer, scene, tile=tile)
    assert st.status == 0
    assert np.array_equal(c1, c2) and np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


@pytest.mark.gpu
def test_injected_allocation_failures(driver, renderer):
    """KZ_FAULT-style injection on the host: the next device allocation fails"""
    try:
        driver.set_option("fault_alloc", 1)
        with pytest.raises(vk.VkError) as e:
            renderer.create_buffer(1 << 20, vk.BUFFER_USAGE_VERTEX, host_visible=False)
        assert e.value.code == vk.VK_ERROR_OUT_OF_DEVICE_MEMORY
        # lowering needs device scratch: the failure surfaces at vkEndCommandBuffer
        scene = scenes.small_soup(n=64, width=64, height=64)
        driver.set_option("fault_alloc", -1)
        run = render.SceneRun(renderer, scene)
        driver.set_option("fault_alloc", 1)
        cb = renderer.begin()
        rbi_clear = (vk.VkClearValue * 2)()
        rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                       vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(64, 64)), 2, rbi_clear)
        driver.vkCmdBeginRenderPass(cb, ctypes.byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
        driver.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
        bufs = (ctypes.c_void_p * 1)(run.vb.handle.value)
        offs = (ctypes.c_uint64 * 1)(0)
        driver.vkCmdBindVertexBuffers(cb, 0, 1, bufs, offs)
        driver.vkCmdDraw(cb, 3 * 64, 1, 0, 0)
        driver.vkCmdEndRenderPass(cb)
        assert driver.vkEndCommandBuffer(cb) == vk.VK_ERROR_OUT_OF_DEVICE_MEMORY
        renderer.free_command_buffer(cb)
    finally:
        driver.set_option("fault_alloc", -1)
    # the driver stays usable: the same scene renders and matches the oracle
    run.submit()
    color, depth = run.read()
    ref_c, ref_d, _ = kz_oracle.render(scene)
    assert np.array_equal(color, ref_c) and np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))


@pytest.mark.gpu
def test_serving_loop_serves_a_request_stream(renderer):
    specs = serving.client_specs(n_clients=4, tmax=20_000)
    backend = serving.VulkanBackend(renderer, specs)
    admitted, resident = serving.admit(backend.sizes, 40e9)
    assert admitted == [0, 1, 2, 3] and resident > 0
    reqs = serving.poisson_requests(2000, 300, len(specs), tmin=1000, tmax=20_000)
    res = serving.serve(backend, reqs, admitted, max_batch=16, max_inflight=2)
    assert res.served == 300 and res.rejected == 0
    assert 0 < res.p50_ms <= res.p99_ms
    # a budget below one client's bytes admits nobody, and every request is rejected
    none, _ = serving.admit(backend.sizes, min(backend.sizes) - 1)
    res = serving.serve(backend, serving.poisson_requests(2000, 50, len(specs)), none)
    assert res.served == 0 and res.rejected == 50
    backend.close()


class _CheckingBackend(serving.VulkanBackend):
    """reads each request's image back as soon as its fence signals (one request in flight at a time)"""

    def submit(self, requests):
        self.last = list(requests)
        return super().submit(requests)

    def poll(self, handle):
        done = super().poll(handle)
        if done:
            for q in self.last:
                self.images.append((q, self.image(q)))
        return done


@pytest.mark.gpu
def test_served_images_match_the_oracle(renderer):
    """a seeded sample of requests, each with its own resolution, triangle count and camera, served one at a
    time; every image equals the oracle's render of that request"""
    specs = serving.client_specs(n_clients=3, tmax=20_000)
    backend = _CheckingBackend(renderer, specs)
    backend.images = []
    reqs = serving.poisson_requests(500, 12, len(specs), seed=11, tmin=1000, tmax=20_000)
    res = serving.serve(backend, reqs, [0, 1, 2], max_batch=1, max_inflight=1)
    assert res.served == 12 and len(backend.images) == 12
    assert len({q.res for q in reqs}) >= 3 and len({q.triangles for q in reqs}) == 12
    lit = 0
    for q, img in backend.images:
        ref_c, _, st = kz_oracle.render(backend.request_scene(q), threads=8)
        mism = np.argwhere(np.any(img != ref_c, axis=-1))
        assert mism.size == 0, "request %d: colour differs at %d pixels" % (q.view, len(mism))
        lit += st["fragments"] > 0
    assert lit >= 6
    backend.close()

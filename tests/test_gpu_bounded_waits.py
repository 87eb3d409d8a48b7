"""Bounded waits, tested without faulting or hanging the GPU.

- A persistent kernel's grid barrier gives up after a limit (the "barrier_ns" driver option): the test sets
  the limit to 0, so the first block that has to wait gives up at once.  The kernel flags
  KZ_STATUS_BARRIER_TIMEOUT and every block returns; the submission completes with VK_ERROR_DEVICE_LOST and
  that device stays lost, while the CUDA context stays usable: the next device renders bit-exact images.
  Both persistent kernels are covered (an opaque pass runs kz_k_persistent_vis, a blended one
  kz_k_persistent).
- vkGetFenceStatus and vkWaitForFences with short timeouts on work still in flight return VK_NOT_READY and
  VK_TIMEOUT (vulkan-driver/src/api_impl.rs:3689 vkWaitForFences, :3414 vkQueueSubmit), and an unbounded
  wait then returns VK_SUCCESS with the finished image."""
import ctypes
from ctypes import c_void_p

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from scene_cases import small_cases

KZ_STATUS_BARRIER_TIMEOUT = 4
DEFAULT_BARRIER_NS = 4_000_000_000
CASES = small_cases()


def _check(scene, run):
    color, depth = run.read()
    ref_c, ref_d, st = kz_oracle.render(scene, threads=8)
    assert np.array_equal(color, ref_c)
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert run.stats().status == 0
    assert run.stats().fragments == st["fragments"] % (1 << 32)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["batched", "blend"])
def test_persistent_barrier_timeout_loses_the_device_not_the_gpu(driver, renderer, case):
    scene = CASES[case]
    lost = render.Renderer(driver)
    try:
        driver.set_option("barrier_ns", 0)
        try:
            run = render.SceneRun(lost, scene, mode="persistent", tile=16)
        finally:
            driver.set_option("barrier_ns", DEFAULT_BARRIER_NS)
        lost.submit(run.cb, lost.fence)
        fences = (c_void_p * 1)(lost.fence)
        assert driver.vkWaitForFences(lost.device, 1, fences, 1, 30_000_000_000) == vk.VK_ERROR_DEVICE_LOST
        assert run.stats().status & KZ_STATUS_BARRIER_TIMEOUT
        # the device stays lost
        arr = (c_void_p * 1)(run.cb)
        si = vk.VkSubmitInfo(vk.ST_SUBMIT_INFO, None, 0, None, None, 1, arr, 0, None)
        assert driver.vkQueueSubmit(lost.queue, 1, ctypes.byref(si), None) == vk.VK_ERROR_DEVICE_LOST
    finally:
        lost.close()
    # the GPU and the CUDA context are fine: a command buffer recorded with the default limit renders exactly
    run = render.SceneRun(renderer, scene, mode="persistent", tile=16)
    run.submit()
    _check(scene, run)


@pytest.mark.gpu
def test_fence_waits_time_out_on_work_in_flight(driver, renderer):
    scene = scenes.batched(ndraws=256, width=1024, height=1024, lo=16, hi=65536)
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    run.submit()  # warm: the kernel image is linked and loaded
    for _ in range(100):
        renderer.submit(run.cb)
    renderer.submit(run.cb, renderer.fence)
    fences = (c_void_p * 1)(renderer.fence)
    # about 100 submissions of 2M triangles each are queued: none of these waits can see the last one finish
    assert driver.vkGetFenceStatus(renderer.device, renderer.fence) == vk.VK_NOT_READY
    assert driver.vkWaitForFences(renderer.device, 1, fences, 1, 0) == vk.VK_TIMEOUT
    assert driver.vkWaitForFences(renderer.device, 1, fences, 1, 1000) == vk.VK_TIMEOUT
    assert driver.vkWaitForFences(renderer.device, 1, fences, 1, 0xFFFFFFFFFFFFFFFF) == vk.VK_SUCCESS
    assert driver.vkGetFenceStatus(renderer.device, renderer.fence) == vk.VK_SUCCESS
    vk.check("vkResetFences", driver.vkResetFences(renderer.device, 1, fences))
    _check(scene, run)

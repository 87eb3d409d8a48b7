"""kzRasterTrianglesNoAlloc: the entry point for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc at the moment they render: programs that give all device memory to their
own pool allocator up front, and serving loops that must not take the device-wide synchronisation an
allocation or free can cause.  This entry point keeps its scratch in a fixed array inside the library instead.
These tests check that it draws exactly what the Vulkan path (the library's existing entry point) and the CPU
oracle draw for the same triangles, on calls in a row (no call may see what an earlier one left in the shared
scratch, including one whose scratch overflowed), that free device memory does not change across a call, and
that it refuses sizes beyond its fixed limits.

This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

from kazan_gb300 import render, scenes
from oracle import kz_oracle

MAX_PIXELS = 1024 * 1024
MAX_TRIANGLES = 65536


def _bind(driver):
    f = driver.lib.kzRasterTrianglesNoAlloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_void_p]
    return f


def _clear(scene):
    return (ctypes.c_float * 4)(*scene.clear_color)


def test_sizes_beyond_the_limits_are_refused(driver):
    """over-limit calls fail before touching the GPU (the pointers are never used)"""
    f = _bind(driver)
    fake = ctypes.c_void_p(256)
    clear = (ctypes.c_float * 4)(0, 0, 0, 1)
    assert f(fake, 1, 2048, 1024, fake, fake, clear, 1.0, None) == -1       # 2 Mi pixels
    assert f(fake, MAX_TRIANGLES + 1, 64, 64, fake, fake, clear, 1.0, None) == -1
    assert f(fake, 1, 0, 64, fake, fake, clear, 1.0, None) == -1
    assert f(None, 1, 64, 64, fake, fake, clear, 1.0, None) == -1


def _vulkan_image(renderer, scene):
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    run.submit()
    return run.read()


def _cases():
    """scenes within the limits: the 2,048-triangle draw twice (different seeds), no triangles, an odd-sized
    1000x333 image, and 96 triangles spanning much of a 1024x1024 image (large-triangle records and jobs)"""
    soup5 = scenes.small_soup(seed=5)
    soup1 = scenes.small_soup(seed=1)
    empty = scenes.small_soup(seed=2, n=0, width=64, height=48)
    empty.clear_color = (0.2, 0.4, 0.6, 0.8)
    empty.clear_depth = 0.75
    odd = scenes.small_soup(seed=3, n=3000, width=1000, height=333)
    big = scenes.small_soup(seed=4, n=96, width=1024, height=1024)
    return [("soup5", soup5), ("soup1", soup1), ("empty", empty), ("odd", odd), ("big", big)]


def _call(f, torch, scene):
    dev = torch.device("cuda:0")
    verts = torch.from_numpy(np.ascontiguousarray(scene.vertices.reshape(-1, 8) if scene.triangles else
                                                  np.zeros((3, 8), np.float32))).to(dev)
    color = torch.full((scene.height, scene.width), 0x5A5A5A5A, dtype=torch.int32, device=dev)
    depth = torch.full((scene.height, scene.width), -7.0, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    rc = f(verts.data_ptr(), scene.triangles, scene.width, scene.height, color.data_ptr(), depth.data_ptr(),
           _clear(scene), scene.clear_depth, None)
    after = torch.cuda.mem_get_info()[0]
    got_c = color.cpu().numpy().view(np.uint8).reshape(scene.height, scene.width, 4)
    got_d = depth.cpu().numpy()
    return rc, got_c, got_d, before, after


def _same(name, got_c, got_d, ref_c, ref_d, what):
    # the tolerance of every image test here: colour bytes and depth bits equal
    mism = np.argwhere(np.any(got_c != ref_c, axis=-1))
    assert mism.size == 0, "%s: colour differs from %s at %d pixels, first %s" % (name, what, len(mism), mism[0])
    assert np.array_equal(got_d.view(np.uint32), ref_d.view(np.uint32)), "%s: depth differs from %s" % (name, what)


@pytest.mark.gpu
def test_no_alloc_matches_the_vulkan_path_and_the_oracle(driver, renderer):
    torch = pytest.importorskip("torch")
    f = _bind(driver)
    cases = _cases()
    for name, scene in cases:
        assert scene.triangles <= MAX_TRIANGLES and scene.width * scene.height <= MAX_PIXELS
    expected = {}
    for name, scene in cases:
        ref_c, ref_d, _ = kz_oracle.render(scene, threads=8)
        expected[name] = (ref_c, ref_d)
        if scene.triangles:
            vk_c, vk_d = _vulkan_image(renderer, scene)
            _same(name, vk_c, vk_d, ref_c, ref_d, "the oracle (Vulkan path)")
            expected[name] = (vk_c, vk_d)
    # the first call on the device loads the library's scratch; after it, calls allocate nothing
    first = True
    for name, scene in cases:
        rc, got_c, got_d, before, after = _call(f, torch, scene)
        assert rc == 0, (name, rc)
        ref_c, ref_d = expected[name]
        _same(name, got_c, got_d, ref_c, ref_d, "the Vulkan path")
        _same(name, got_c, got_d, *kz_oracle.render(scene, threads=8)[:2], "the oracle")
        if not first:
            assert after == before, "%s: free device memory changed by %d bytes" % (name, before - after)
        first = False


@pytest.mark.gpu
def test_no_alloc_reports_job_overflow_and_recovers(driver):
    """2,000 triangles that each span a 1024x1024 image need about 2M 8x8-block jobs, beyond the 2^20 the
    scratch holds: the call returns -3; the next call renders correctly from the same scratch"""
    torch = pytest.importorskip("torch")
    f = _bind(driver)
    n = 2000
    rng = np.random.default_rng(9)
    v = np.zeros((3 * n, 8), np.float32)
    corners = np.array([[-1.2, -1.2], [3.5, -1.2], [-1.2, 3.5]], np.float32)
    for t in range(n):
        flip = t % 2
        for j in range(3):
            x, y = corners[j]
            v[3 * t + j] = [-x if flip else x, -y if flip else y, rng.uniform(0.1, 0.9), 1.0] + list(rng.uniform(0, 1, 4))
    big = scenes.triangles_from(v, 1024, 1024)
    assert big.triangles == n
    rc, _, _, _, _ = _call(f, torch, big)
    assert rc == -3
    name, scene = _cases()[0]
    rc, got_c, got_d, before, after = _call(f, torch, scene)
    assert rc == 0 and after == before
    _same(name, got_c, got_d, *kz_oracle.render(scene, threads=8)[:2], "the oracle")

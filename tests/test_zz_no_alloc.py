"""kzRasterTrianglesNoAlloc: the entry point for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc at the moment they render: code running while a stream is being
captured into a CUDA graph (an allocation there breaks the capture), serving loops that must not take the
device-wide synchronisation an allocation or free can cause, and programs that give all device memory to
their own pool.  This entry point keeps its scratch in a fixed array inside the library instead.  These
tests check that it draws exactly what the Vulkan path draws for the same triangles, on two calls in a row
(the second call must not see anything the first one left in the shared scratch), and that it refuses
sizes beyond its fixed limits.

This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

from kazan_gb300 import render, scenes

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


def _driver_image(renderer, scene):
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    run.submit()
    color, depth = run.read()
    return color, depth


@pytest.mark.gpu
def test_no_alloc_matches_the_vulkan_path_twice(driver, renderer):
    torch = pytest.importorskip("torch")
    f = _bind(driver)
    first = scenes.small_soup(seed=5)
    second = scenes.small_soup(seed=1)
    expected = [_driver_image(renderer, s) for s in (first, second)]

    dev = torch.device("cuda:0")
    for scene, (ref_c, ref_d) in zip((first, second), expected):
        assert scene.triangles <= MAX_TRIANGLES and scene.width * scene.height <= MAX_PIXELS
        verts = torch.from_numpy(np.ascontiguousarray(scene.vertices)).to(dev)
        color = torch.full((scene.height, scene.width), 0x5A5A5A5A, dtype=torch.int32, device=dev)
        depth = torch.full((scene.height, scene.width), -7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        rc = f(verts.data_ptr(), scene.triangles, scene.width, scene.height, color.data_ptr(), depth.data_ptr(),
               _clear(scene), scene.clear_depth, None)
        assert rc == 0
        got_c = color.cpu().numpy().view(np.uint8).reshape(scene.height, scene.width, 4)
        got_d = depth.cpu().numpy()
        # the tolerance of every image test here: colour bytes and depth bits equal
        mism = np.argwhere(np.any(got_c != ref_c, axis=-1))
        assert mism.size == 0, "colour differs at %d pixels, first %s" % (len(mism), mism[0])
        assert np.array_equal(got_d.view(np.uint32), ref_d.view(np.uint32)), "depth differs"

"""The drop-in boundary on the CPU: libkazan_driver.so loads without a GPU, exports every function the
public headers declare, and answers the loader-facing calls the way the reference's ICD does
(vulkan-driver/src/lib.rs:38-130)."""
import ctypes
import os
import re

import pytest

from kazan_gb300 import vk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _declared_symbols():
    names = set()
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        with open(os.path.join(INCLUDE, h), encoding="utf-8") as f:
            text = f.read()
        # KZ_API <return type> <name>(
        names.update(re.findall(r"KZ_API\s+[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(driver):
    names = _declared_symbols()
    assert {"vk_icdGetInstanceProcAddr", "vk_icdNegotiateLoaderICDInterfaceVersion",
            "vk_icdGetPhysicalDeviceProcAddr", "kzDriverSetOption", "kzGetKernelTimes", "kzShaderCompile",
            "kzShaderLink", "kzRasterTrianglesNoAlloc"} <= names
    missing = [n for n in sorted(names) if not hasattr(driver.lib, n)]
    assert not missing, "declared in include/ but not exported: %s" % missing


def test_negotiate_clamps_to_version_5(driver):
    """lib.rs:51-63: the loader proposes a version, the ICD answers min(proposed, 5)"""
    for proposed, expected in [(7, 5), (5, 5), (3, 3)]:
        v = ctypes.c_uint32(proposed)
        assert driver.lib.vk_icdNegotiateLoaderICDInterfaceVersion(ctypes.byref(v)) == vk.VK_SUCCESS
        assert v.value == expected


def test_draw_path_entry_points_resolve(driver):
    for name in vk.DRAW_PATH_ENTRY_POINTS:
        assert driver.lib.vk_icdGetInstanceProcAddr(None, name.encode()), name
    assert not driver.lib.vk_icdGetInstanceProcAddr(None, b"vkNoSuchFunction")
    # physical-device-level names go through vk_icdGetPhysicalDeviceProcAddr too
    assert driver.lib.vk_icdGetPhysicalDeviceProcAddr(None, b"vkGetPhysicalDeviceProperties")
    assert not driver.lib.vk_icdGetPhysicalDeviceProcAddr(None, b"vkCmdDraw")


def test_instance_without_gpu_has_no_physical_device(driver):
    info = vk.VkInstanceCreateInfo(vk.ST_INSTANCE_CREATE_INFO, None, 0, None, 0, None, 0, None)
    inst = ctypes.c_void_p()
    assert driver.vkCreateInstance(ctypes.byref(info), None, ctypes.byref(inst)) == vk.VK_SUCCESS
    try:
        # the dispatchable handle starts with the loader's magic word (handle.rs:23-37)
        assert ctypes.c_uint64.from_address(inst.value).value == 0x01CDC0DE
        n = ctypes.c_uint32(99)
        assert driver.vkEnumeratePhysicalDevices(inst, ctypes.byref(n), None) == vk.VK_SUCCESS
        import torch
        if not torch.cuda.is_available():
            assert n.value == 0
    finally:
        driver.vkDestroyInstance(inst, None)


@pytest.mark.parametrize("key,value,ok", [("mode", "persistent", True), ("mode", "batched", True),
                                          ("mode", "perdraw", True), ("mode", "fast", False),
                                          ("tile", "16", True), ("tile", "12", False),
                                          ("kernel_timing", "1", True), ("kernel_timing", "2", False),
                                          ("trace", "0", True), ("no_such_option", "1", False),
                                          ("pdl", "0", True), ("pdl", "yes", False),
                                          ("tma", "0", True), ("tma", "2", False),
                                          ("vector_fetch", "0", True), ("vector_fetch", "", False),
                                          ("barrier_ns", "0", True), ("barrier_ns", "4294967296", False),
                                          ("barrier_ns", "-1", False),
                                          ("warp_px", "1", True), ("warp_px", "4096", True),
                                          ("warp_px", "0", False), ("warp_px", "4097", False),
                                          ("warp_px", "12a", False),
                                          ("job_blocks", "1", True), ("job_blocks", "32", True),
                                          ("job_blocks", "0", False), ("job_blocks", "33", False),
                                          ("geo_blocks", "0", True), ("geo_blocks", "64", True),
                                          ("geo_blocks", "65", False), ("geo_blocks", "", False)])
def test_driver_options(driver, key, value, ok):
    rc = driver.lib.kzDriverSetOption(key.encode(), value.encode())
    assert (rc == 0) == ok
    for k, v in ((b"mode", b"persistent"), (b"tile", b"16"), (b"kernel_timing", b"0"), (b"pdl", b"1"),
                 (b"tma", b"1"), (b"vector_fetch", b"1"), (b"barrier_ns", b"4000000000"), (b"warp_px", b"192"),
                 (b"job_blocks", b"16"), (b"geo_blocks", b"0")):
        driver.lib.kzDriverSetOption(k, v)

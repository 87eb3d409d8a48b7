"""GPU parity of the 8-bit sRGB colour attachments (R8G8B8A8_SRGB, B8G8R8A8_SRGB): opaque passes (the
visibility path's resolve encodes), blended passes (the ordered tile raster decodes the destination, blends
in linear and encodes), render-pass clears and vkCmdClearColorImage, each bit for bit against the oracle."""
import dataclasses
from ctypes import byref

import numpy as np
import pytest

from kazan_gb300 import render, vk
from oracle import kz_oracle

from scene_cases import small_cases

CLEAR = (0.25, 0.5, 0.75, 0.6)


def _scene(case, fmt):
    return dataclasses.replace(small_cases()[case], color_format=fmt, clear_color=CLEAR)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["rgba8_srgb", "bgra8_srgb"])
@pytest.mark.parametrize("case", ["batched", "blend", "sphere", "ties"])
@pytest.mark.parametrize("mode", ["batched", "persistent"])
def test_srgb_attachment_matches_oracle(renderer, case, fmt, mode):
    scene = _scene(case, fmt)
    run = render.SceneRun(renderer, scene, mode=mode, tile=16)
    run.submit()
    color, depth = run.read()
    st = run.stats()
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s: gpu %s oracle %s" % (
        len(mism), mism[0], color[tuple(mism[0])], ref_c[tuple(mism[0])])
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == ost["fragments"] % (1 << 32)
    # the encoding is not the UNORM one: the same scene stored as UNORM differs
    unorm_c, _, _ = kz_oracle.render(dataclasses.replace(scene, color_format="rgba8"), threads=8)
    assert not np.array_equal(color, unorm_c)
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["rgba8_srgb", "bgra8_srgb"])
def test_clear_color_image_srgb(renderer, fmt):
    img = renderer.create_image(37, 9, vk.COLOR_FORMATS[fmt], vk.IMAGE_USAGE_COLOR_ATTACHMENT, True)
    cb = renderer.begin()
    cc = vk.VkClearColorValue()
    cc.float32[:] = [0.5, 0.2140, 0.0031308, 0.6]
    renderer.drv.vkCmdClearColorImage(cb, img.handle, vk.IMAGE_LAYOUT_GENERAL, byref(cc), 1,
                                      byref(vk.VkImageSubresourceRange(vk.IMAGE_ASPECT_COLOR, 0, 1, 0, 1)))
    renderer.end_submit_wait(cb)
    renderer.free_command_buffer(cb)
    got = renderer.read_image(img)
    L = kz_oracle.lib()
    rgba = [L.kzo_srgb8(0.5), L.kzo_srgb8(0.2140), L.kzo_srgb8(0.0031308), kz_oracle.unorm8(0.6)]
    want = rgba if fmt == "rgba8_srgb" else [rgba[2], rgba[1], rgba[0], rgba[3]]
    assert rgba[:2] == [188, 127]
    assert np.all(got == np.array(want, dtype=np.uint8))


@pytest.mark.gpu
def test_srgb_image_is_not_a_texture(renderer):
    """sampling does not decode sRGB, so sRGB images are attachment-only: the device reports no sampled
    feature for them"""
    props = vk.VkFormatProperties()
    renderer.drv.vkGetPhysicalDeviceFormatProperties(renderer.physical, vk.FORMAT_R8G8B8A8_SRGB, byref(props))
    assert props.optimalTilingFeatures & vk.FORMAT_FEATURE_COLOR_ATTACHMENT
    assert not props.optimalTilingFeatures & vk.FORMAT_FEATURE_SAMPLED_IMAGE

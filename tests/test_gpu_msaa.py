"""GPU parity of 4x multisampling: coverage, depth test, depth write and colour per sample at the standard
sample positions, the fragment shader once per pixel at its centre, and the resolve (per byte, the rounded
mean of the four samples) equal the CPU oracle bit for bit: every colour sample, every depth sample, the
resolved image and the fragment count, in both launch schedules and every tile side; vkCmdResolveImage
resolves a sub-rectangle."""
import dataclasses
from ctypes import byref

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from scene_cases import equal_depth_ties, guard_band_and_near, small_cases, top_left_square


def _cases():
    c = small_cases()
    return {
        "soup": c["soup"],
        "sphere": c["sphere"],
        "blend": c["blend"],
        "tess": c["tess"],
        "topleft": top_left_square(),
        "clip": guard_band_and_near(),
        "ties": equal_depth_ties(),
        "textured": scenes.textured(seed=9, n=600, width=160, height=120, linear=True),
    }


CASES = _cases()


def _run(renderer, scene, mode, tile):
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    run.submit()
    resolved, depth4 = run.read()
    color4 = renderer.read_image(run.samples)
    return run, resolved, depth4, color4


@pytest.mark.gpu
@pytest.mark.parametrize("mode,tile", [("batched", 16), ("persistent", 16), ("batched", 8), ("batched", 32)])
@pytest.mark.parametrize("case", sorted(CASES))
def test_msaa_matches_oracle(renderer, case, mode, tile):
    scene = dataclasses.replace(CASES[case], samples=4)
    run, resolved, depth4, color4 = _run(renderer, scene, mode, tile)
    ref_c4, ref_d4, ref_r, ost = kz_oracle.render_ms(scene, threads=8)
    mism = np.argwhere(np.any(color4 != ref_c4, axis=-1))
    assert mism.size == 0, "colour samples differ at %d, first %s" % (len(mism), mism[:1])
    assert np.array_equal(depth4.view(np.uint32), ref_d4.view(np.uint32)), "depth samples differ"
    assert np.array_equal(resolved, ref_r), "resolved colour differs"
    st = run.stats()
    assert st.status == 0
    assert st.fragments == ost["fragments"] % (1 << 32)
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_msaa_edges_are_antialiased(renderer):
    """the resolved image of the random soup has pixels whose four samples differ (partly covered edges)
    and a single-sample render of the same scene equals neither everywhere"""
    scene = dataclasses.replace(CASES["soup"], samples=4)
    run, resolved, _, color4 = _run(renderer, scene, "batched", 16)
    mixed = np.any(color4 != color4[:, :, :1, :], axis=(2, 3))
    assert mixed.mean() > 0.05
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_resolve_image_region(renderer):
    """vkCmdResolveImage of a sub-rectangle into an offset destination"""
    r, d = renderer, renderer.drv
    scene = dataclasses.replace(CASES["soup"], samples=4)
    run, _, _, color4 = _run(r, scene, "batched", 16)
    dst = r.create_image(100, 80, vk.FORMAT_R8G8B8A8_UNORM, vk.IMAGE_USAGE_COLOR_ATTACHMENT, True)
    cb = r.begin()
    sub = vk.VkImageSubresourceLayers(vk.IMAGE_ASPECT_COLOR, 0, 0, 1)
    reg = vk.VkImageResolve(sub, vk.VkOffset3D(37, 21, 0), sub, vk.VkOffset3D(5, 9, 0), vk.VkExtent3D(61, 44, 1))
    d.vkCmdResolveImage(cb, run.samples.handle, vk.IMAGE_LAYOUT_GENERAL, dst.handle, vk.IMAGE_LAYOUT_GENERAL, 1,
                        byref(reg))
    r.end_submit_wait(cb)
    r.free_command_buffer(cb)
    got = r.read_image(dst)[9:9 + 44, 5:5 + 61]
    want = ((color4[21:21 + 44, 37:37 + 61].astype(np.uint32).sum(axis=2) + 2) // 4).astype(np.uint8)
    assert np.array_equal(got, want)
    r.free_command_buffer(run.cb)

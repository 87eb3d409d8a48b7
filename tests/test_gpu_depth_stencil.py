"""GPU parity of the D16_UNORM and D24_UNORM_S8_UINT depth attachments and of the stencil test: every scene
family renders into them bit for bit what the CPU oracle renders (colour and the packed depth/stencil
texels), stencil ops and compare functions (per face, under compare and write masks, from a cleared
stencil value) follow API order, and vkCmdClearDepthStencilImage writes the converted clear value."""
import ctypes
import dataclasses
from ctypes import byref

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from scene_cases import equal_depth_ties, guard_band_and_near, small_cases

S = scenes.StencilOp
# VkStencilOp: KEEP 0, ZERO 1, REPLACE 2, INCREMENT_AND_CLAMP 3, DECREMENT_AND_CLAMP 4, INVERT 5,
# INCREMENT_AND_WRAP 6, DECREMENT_AND_WRAP 7; VkCompareOp: NEVER 0 .. ALWAYS 7
STENCILS = {
    "count_overdraw": (dict(front=S(pass_=6), back=S(pass_=6)), dict(depth_test=False, depth_write=False), 0),
    "first_wins": (dict(front=S(fail=0, pass_=3, depth_fail=7, compare=2, reference=0),
                        back=S(fail=0, pass_=3, depth_fail=7, compare=2, reference=0)), {}, 0),
    "faces_masks": (dict(front=S(fail=1, pass_=6, depth_fail=4, compare=5, compare_mask=0x03, write_mask=0x0F,
                             reference=2),
                         back=S(fail=2, pass_=5, depth_fail=3, compare=6, compare_mask=0xF0, write_mask=0xF3,
                                reference=0x35)), {}, 0x5A),
    "replace_greater": (dict(front=S(fail=7, pass_=2, depth_fail=1, compare=4, reference=6),
                             back=S(fail=3, pass_=2, depth_fail=0, compare=3, reference=6)),
                        dict(depth_compare=3), 5),
}


def _check(scene, color, depth, st):
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s" % (len(mism), mism[:1])
    dm = np.argwhere(depth != ref_d)
    assert dm.size == 0, "depth/stencil differs at %d pixels, first %s: gpu %s oracle %s" % (
        len(dm), dm[:1], depth[tuple(dm[0])] if len(dm) else None, ref_d[tuple(dm[0])] if len(dm) else None)
    assert st.status == 0
    assert st.fragments == ost["fragments"] % (1 << 32)


def _render(renderer, scene, mode="batched", tile=16):
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    run.submit()
    color, depth = run.read()
    out = color, depth, run.stats()
    renderer.free_command_buffer(run.cb)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched"])
@pytest.mark.parametrize("fmt", ["d16", "d24s8"])
@pytest.mark.parametrize("case", ["sphere", "batched", "blend", "ties", "clip", "soup"])
def test_depth_formats_match_oracle(renderer, case, fmt, mode):
    base = {"ties": equal_depth_ties, "clip": guard_band_and_near}.get(case)
    scene = base() if base else small_cases()[case]
    scene = dataclasses.replace(scene, depth_format=fmt, clear_depth=0.875 if case == "soup" else scene.clear_depth)
    _check(scene, *_render(renderer, scene, mode))


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("name", sorted(STENCILS))
def test_stencil_matches_oracle(renderer, name, tile):
    faces, state, clear = STENCILS[name]
    scene = dataclasses.replace(small_cases()["soup"], depth_format="d24s8", stencil=faces, clear_stencil=clear,
                                **state)
    out = _render(renderer, scene, "batched", tile)
    _check(scene, *out)
    # the stencil ops did something: the stencil byte differs from the clear value somewhere, and counting
    # overdraw reaches several values
    values = np.unique(out[1] >> 24)
    assert len(values) >= (3 if name == "count_overdraw" else 2)


@pytest.mark.gpu
def test_stencil_on_the_blend_workload(renderer):
    """blending with a stencil that lets each pixel blend at most three times"""
    faces = dict(front=S(pass_=3, compare=4, reference=3), back=S(pass_=3, compare=4, reference=3))
    scene = dataclasses.replace(small_cases()["blend"], depth_format="d24s8", stencil=faces)
    _check(scene, *_render(renderer, scene, "persistent"))


@pytest.mark.gpu
@pytest.mark.parametrize("fmt,width", [("d16", 37), ("d24s8", 20), ("d32", 9)])
def test_clear_depth_stencil_image(renderer, fmt, width):
    r, d = renderer, renderer.drv
    img = r.create_image(width, 5, vk.DEPTH_FORMATS[fmt], vk.IMAGE_USAGE_DEPTH_STENCIL_ATTACHMENT, True)
    cb = r.begin()
    v = vk.VkClearDepthStencilValue(0.3, 0xAB)
    rng = vk.VkImageSubresourceRange(render._aspect(img.format), 0, 1, 0, 1)
    d.vkCmdClearDepthStencilImage(cb, img.handle, vk.IMAGE_LAYOUT_GENERAL, byref(v), 1, byref(rng))
    r.end_submit_wait(cb)
    r.free_command_buffer(cb)
    got = r.read_image(img)
    if fmt == "d16":
        want = np.full((5, width), int(np.rint(np.float32(0.3) * np.float32(65535.0))), dtype=np.uint16)
    elif fmt == "d24s8":
        q = int(np.rint(np.float32(0.3) * np.float32(16777215.0)))
        want = np.full((5, width), q | (0xAB << 24), dtype=np.uint32)
    else:
        want = np.full((5, width), np.float32(0.3), dtype=np.float32)
    assert np.array_equal(got, want)
    assert kz_oracle.lib().kzo_depth_value(ctypes.c_float(0.3), kz_oracle.DEPTH_FORMAT[fmt]) == (
        float(want.flat[0] & 0xFFFFFF) if fmt == "d24s8" else float(want.flat[0]))

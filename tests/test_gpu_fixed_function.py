"""GPU parity of the fixed-function state space of the depth test and the colour blend against the CPU oracle,
bit for bit (colour bytes, depth bits, fragment counts):
  - every VkCompareOp on a single-sample D32 attachment, with and without depth writes.  With writes, LESS,
    LESS_OR_EQUAL, GREATER and GREATER_OR_EQUAL render through the visibility path (each with its own key and
    tie order); the other ops, and every op without writes, through the ordered tile path;
  - every single-source blend factor in each of the four factor slots, every blend op in both op slots, blend
    constants inside and outside [0, 1] (clamped for the normalized attachment), partial write masks, on UNORM
    and sRGB attachments;
  - colour write masks without blending (visibility path);
  - blend constants set by vkCmdSetBlendConstants between draws.
The oracle's own handling of these states is pinned against an exact rational restatement on the CPU
(tests/test_oracle.py, tests/py_raster.py)."""
import ctypes
import dataclasses
from ctypes import byref

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from fixed_function_cases import BLEND_CONSTS, CLEAR_DEPTH, COMPARE_OPS, WRITE_MASKS, blend_states
from scene_cases import equal_depth_ties, small_cases


def _mixed(seed=7, n=600, size=128):
    """triangles with colours reaching outside [0, 1] and varied alpha; every other one coplanar at depth 0.25
    (ties for EQUAL, LESS_OR_EQUAL, GREATER_OR_EQUAL), the rest at random depths"""
    rng = np.random.default_rng(seed)
    rows = []
    for t in range(n):
        c = rng.uniform(0, size, 2)
        r = np.exp(rng.uniform(np.log(2.0), np.log(size / 3), 1))[0]
        z = [0.25] * 3 if t % 2 else list(rng.uniform(0.05, 0.95, 3))
        col = rng.uniform(-0.25, 1.25, (3, 4))
        for j in range(3):
            x, y = c + rng.normal(0, r, 2)
            rows.append([2.0 * x / size - 1.0, 2.0 * y / size - 1.0, z[j], 1.0] + list(col[j]))
    return scenes.triangles_from(np.array(rows, dtype=np.float32), size, size, clear_color=(0.3, 0.6, 0.9, 0.45))


SCENES = {"ties": equal_depth_ties(), "mixed": _mixed(), "batched": small_cases()["batched"]}


def _render(renderer, scene, mode, tile=16):
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    run.submit()
    color, depth = run.read()
    return color, depth, run.stats()


def _check(scene, color, depth, stats, ref=None):
    ref_c, ref_d, st = ref if ref is not None else kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s: gpu %s oracle %s" % (
        len(mism), mism[0], color[tuple(mism[0])], ref_c[tuple(mism[0])])
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32)), "depth differs"
    assert stats.status == 0
    assert stats.fragments == st["fragments"] % (1 << 32), (stats.fragments, st["fragments"])


def _modes(depth_write):
    return ["batched", "persistent", "perdraw"] if depth_write else ["batched", "persistent"]


CMP_CASES = [(s, op, w, m) for s in sorted(SCENES) for op in sorted(COMPARE_OPS) for w in (True, False)
             for m in _modes(w)]


@pytest.mark.gpu
@pytest.mark.parametrize("scene_name,op,depth_write,mode", CMP_CASES,
                         ids=["%s-%s-%s-%s" % (s, COMPARE_OPS[op], "write" if w else "nowrite", m)
                              for s, op, w, m in CMP_CASES])
def test_depth_compare_ops(renderer, scene_name, op, depth_write, mode):
    scene = dataclasses.replace(SCENES[scene_name], depth_compare=op, depth_write=depth_write,
                                clear_depth=CLEAR_DEPTH[op])
    color, depth, stats = _render(renderer, scene, mode)
    _check(scene, color, depth, stats)


def _blend_scene(i, color_format="rgba8"):
    return dataclasses.replace(SCENES["mixed"], blend=True, blend_state=blend_states()[i],
                               blend_const=BLEND_CONSTS[i % len(BLEND_CONSTS)],
                               write_mask=WRITE_MASKS[i % len(WRITE_MASKS)], depth_compare=3, depth_write=False,
                               color_format=color_format)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent"])
@pytest.mark.parametrize("i", range(15))
def test_blend_factors_ops_constants_masks(renderer, i, mode):
    scene = _blend_scene(i)
    color, depth, stats = _render(renderer, scene, mode)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("i", [0, 2, 4, 6, 8, 10, 14])
def test_blend_states_on_srgb(renderer, i):
    """destination decoded from sRGB before blending, result encoded after (red, green, blue)"""
    scene = _blend_scene(i, "bgra8_srgb" if i % 4 else "rgba8_srgb")
    color, depth, stats = _render(renderer, scene, "batched", tile=32)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
@pytest.mark.parametrize("mask", [0x0, 0x1, 0x6, 0xB, 0xE])
def test_write_masks_without_blending(renderer, mask, mode):
    """opaque passes (visibility path) store only the channels the mask selects; the rest keep the clear"""
    scene = dataclasses.replace(SCENES["mixed"], write_mask=mask)
    color, depth, stats = _render(renderer, scene, mode)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent"])
def test_dynamic_blend_constants_between_draws(renderer, mode):
    """a pipeline with dynamic blend constants: each draw blends with the constants set before it"""
    base = SCENES["mixed"]
    scene = dataclasses.replace(base, blend=True, blend_state=(10, 11, 0, 12, 13, 0), depth_compare=7,
                                depth_write=False, draws=[scenes.Draw(0, 200), scenes.Draw(600, 200),
                                                          scenes.Draw(1200, 200)])
    consts = [(0.2, 0.4, 0.6, 0.8), (1.0, 0.0, 0.5, 0.25), (1.7, -0.5, 0.33, 0.66)]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16)
    vs, fs = scene.shaders()
    run.pipe = renderer.pipeline(scene, run.rp, run.layout, vs, fs, dynamic=(vk.DYNAMIC_STATE_BLEND_CONSTANTS,))
    cb = renderer.begin()
    d = renderer.drv
    clears = (vk.VkClearValue * 2)()
    clears[0].color.float32[:] = list(scene.clear_color)
    clears[1].depthStencil.depth = scene.clear_depth
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                   vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(scene.width, scene.height)), 2,
                                   clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
    d.vkCmdBindVertexBuffers(cb, 0, 1, (ctypes.c_void_p * 1)(run.vb.handle.value), (ctypes.c_uint64 * 1)(0))
    for dr, k in zip(scene.draws, consts):
        d.vkCmdSetBlendConstants(cb, (ctypes.c_float * 4)(*k))
        d.vkCmdDraw(cb, 3 * dr.count, 1, dr.first, 0)
    d.vkCmdEndRenderPass(cb)
    vk.check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
    renderer.submit_wait(cb)
    color, depth = run.read()
    stats = renderer.drv.stats(cb)
    renderer.free_command_buffer(cb)
    # the oracle: the same draws, each with its constants
    col, dep = kz_oracle.clear_images(scene)
    arr, n = kz_oracle.make_draws(scene)
    for i, k in enumerate(consts):
        arr[i].blend_const[:] = list(k)
    ost = kz_oracle.KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, scene.width, scene.height)
    kz_oracle.lib().kzo_render_ds(scene.width, scene.height, col.ctypes.data, dep.ctypes.data, None, 0, area, n, arr,
                                  8, byref(ost))
    _check(scene, color, depth, stats, ref=(col, dep, ost.as_dict()))
    # the three constants gave three different results: the same draws under the first constants differ
    only_first = dataclasses.replace(scene, blend_const=consts[0])
    c1, _, _ = kz_oracle.render(only_first, threads=8)
    assert not np.array_equal(c1, col)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
@pytest.mark.parametrize("compare", [1, 3])
def test_opaque_and_blended_draws_in_one_pass(renderer, mode, compare):
    """one render pass whose pipelines alternate between an opaque one (depth writes on: the visibility path)
    and a blended one (depth writes off: the ordered tile path) over the same vertex buffer: each segment
    starts from the attachments the previous one left, as the oracle draws them in API order"""
    base = SCENES["mixed"]
    opaque = dataclasses.replace(base, depth_compare=compare)
    blended = dataclasses.replace(base, blend=True, depth_compare=compare, depth_write=False)
    order = [(opaque, scenes.Draw(0, 150)), (blended, scenes.Draw(450, 150)), (opaque, scenes.Draw(900, 150)),
             (blended, scenes.Draw(1350, 150))]
    run = render.SceneRun(renderer, opaque, mode=mode, tile=16)
    vs, fs = opaque.shaders()
    pipes = {id(opaque): run.pipe,
             id(blended): renderer.pipeline(blended, run.rp, run.layout, vs, fs)}
    d = renderer.drv
    d.set_option("mode", mode)
    cb = renderer.begin()
    clears = (vk.VkClearValue * 2)()
    clears[0].color.float32[:] = list(base.clear_color)
    clears[1].depthStencil.depth = base.clear_depth
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                   vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(base.width, base.height)), 2,
                                   clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindVertexBuffers(cb, 0, 1, (ctypes.c_void_p * 1)(run.vb.handle.value), (ctypes.c_uint64 * 1)(0))
    for sc, dr in order:
        d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, pipes[id(sc)])
        d.vkCmdDraw(cb, 3 * dr.count, 1, dr.first, 0)
    d.vkCmdEndRenderPass(cb)
    vk.check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
    renderer.submit_wait(cb)
    color, depth = run.read()
    stats = d.stats(cb)
    renderer.free_command_buffer(cb)
    col, dep = kz_oracle.clear_images(base)
    arr = (kz_oracle.KzoDraw * len(order))()
    for i, (sc, dr) in enumerate(order):
        one, _ = kz_oracle.make_draws(sc, [dr])
        arr[i] = one[0]
    ost = kz_oracle.KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, base.width, base.height)
    kz_oracle.lib().kzo_render_ds(base.width, base.height, col.ctypes.data, dep.ctypes.data, None, 0, area,
                                  len(order), arr, 8, byref(ost))
    _check(base, color, depth, stats, ref=(col, dep, ost.as_dict()))
    assert stats.segments == len(order)


@pytest.mark.gpu
@pytest.mark.parametrize("front_ccw", [True, False])
@pytest.mark.parametrize("cull", [0, 1, 2, 3])
@pytest.mark.parametrize("path", ["opaque", "blended"])
def test_cull_modes_and_front_faces(renderer, path, cull, front_ccw):
    """VkCullModeFlags NONE / FRONT / BACK / FRONT_AND_BACK under both front-face windings, on the visibility
    path (opaque) and the tile path (blended), over triangles of both windings"""
    scene = dataclasses.replace(SCENES["mixed"], cull=cull, front_ccw=front_ccw)
    if path == "blended":
        scene = dataclasses.replace(scene, blend=True, depth_write=False)
    color, depth, stats = _render(renderer, scene, "batched")
    _check(scene, color, depth, stats)
    if cull == 3:
        assert stats.fragments == 0

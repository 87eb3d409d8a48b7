"""GPU parity of indirect draws (vkCmdDrawIndirect / vkCmdDrawIndexedIndirect): the counts of each draw come
from a buffer at execution, so a scene drawn through indirect commands must equal the CPU oracle's image of
the same draws bit for bit, whether the commands were written by the host or by a vkCmdCopyBuffer earlier in
the same command buffer, in every launch schedule; rewriting the commands between submissions changes the
image accordingly; and a command that reaches past its bound buffers is skipped with a status bit instead of
being read."""
import ctypes
import dataclasses

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from scene_cases import guard_band_and_near, equal_depth_ties, small_cases

STATUS_INDIRECT_RANGE = 16


def _split(scene, bounds):
    """the scene's single draw split into draws [a, b) of triangles, listed in the given order"""
    return dataclasses.replace(scene, draws=[scenes.Draw(a, b - a) for a, b in bounds])


def _cases():
    c = small_cases()
    return {
        "soup_split": _split(c["soup"], [(0, 500), (1500, 2048), (500, 1500)]),
        "sphere": c["sphere"],
        "batched": c["batched"],
        "blend_split": _split(c["blend"], [(0, 1000), (1000, 1001), (1001, 4000)]),
        "clip": guard_band_and_near(),
        "ties": equal_depth_ties(),
    }


CASES = _cases()


def _check(scene, color, depth, st, status=0):
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s" % (len(mism), mism[:1])
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32)), "depth differs"
    assert st.status == status
    assert st.fragments == ost["fragments"] % (1 << 32)


def _submit(run):
    run.submit()
    color, depth = run.read()
    return color, depth, run.stats()


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("mode", ["persistent", "batched", "perdraw"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_indirect_matches_oracle(renderer, case, mode, where):
    scene = CASES[case]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, indirect=where)
    _check(scene, *_submit(run))
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched"])
def test_indirect_commands_rewritten_between_submissions(renderer, mode):
    """one recorded command buffer, three sets of commands: every other draw with instanceCount 0, every
    draw with instanceCount 2 (instance-major order: the same as each draw recorded twice), and the
    original commands"""
    scene = CASES["batched"]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, indirect="host")
    base = render.indirect_commands(scene)

    half = base.copy()
    half[1::2, 1] = 0
    renderer.write_buffer(run.cmds, half)
    kept = dataclasses.replace(scene, draws=scene.draws[0::2])
    _check(kept, *_submit(run))

    renderer.write_buffer(run.cmds, render.indirect_commands(scene, instances=2))
    twice = dataclasses.replace(scene, draws=[d for d in scene.draws for _ in range(2)])
    _check(twice, *_submit(run))

    renderer.write_buffer(run.cmds, base)
    _check(scene, *_submit(run))
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("case,field,value", [
    ("soup_split", 2, 1 << 30),        # firstVertex past the vertex buffer
    ("soup_split", 3, 0xFFFFFFFF),     # firstInstance + instanceCount past 2^32 - 1
    ("batched", 2, 1 << 30),           # firstIndex past the index buffer
])
def test_indirect_out_of_range_command_is_skipped(renderer, case, field, value):
    scene = CASES[case]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16, indirect="host")
    cmds = render.indirect_commands(scene)
    cmds[1, field] = value
    renderer.write_buffer(run.cmds, cmds)
    rest = dataclasses.replace(scene, draws=[d for i, d in enumerate(scene.draws) if i != 1])
    _check(rest, *_submit(run), status=STATUS_INDIRECT_RANGE)
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["single", "batched"])
def test_indirect_full_size_equals_direct(renderer, name):
    """the 1M-triangle draw (4096 chunks of one draw) and the 4096-draw scene: indirect commands written by a
    copy give the direct draws' image, depth and fragment count"""
    scene = scenes.single_large() if name == "single" else scenes.batched()
    outs = []
    for indirect in (None, "device"):
        run = render.SceneRun(renderer, scene, mode="batched", tile=16, indirect=indirect)
        outs.append(_submit(run))
        renderer.free_command_buffer(run.cb)
    (c0, d0, s0), (c1, d1, s1) = outs
    assert s0.status == 0 and s1.status == 0
    assert np.array_equal(c0, c1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))
    assert s0.fragments == s1.fragments


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched"])
def test_indirect_beyond_table_room(renderer, mode):
    """instanceCount 8 on the 60K-triangle sphere: 480K triangles outgrow the chunk table and draw lookup
    sized at recording from the bound index buffer, so chunks and primitives find their draw by searching;
    the image equals the draw recorded eight times"""
    scene = CASES["sphere"]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, indirect="host")
    renderer.write_buffer(run.cmds, render.indirect_commands(scene, instances=8))
    eight = dataclasses.replace(scene, draws=[scene.draws[0]] * 8)
    _check(eight, *_submit(run))
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched"])
def test_indirect_count_from_buffer(renderer, mode):
    """vkCmdDraw*IndirectCountKHR: the draw count is read from a buffer at execution and capped by
    maxDrawCount; one call of three non-indexed draws, then 48 indexed calls of at most one draw each"""
    scene = CASES["soup_split"]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, indirect="host", counts=[2])
    _check(dataclasses.replace(scene, draws=scene.draws[:2]), *_submit(run))
    for count, keep in ((0, 0), (7, 3), (3, 3), (1, 1)):
        renderer.write_buffer(run.count_buf, np.array([count], dtype=np.uint32))
        _check(dataclasses.replace(scene, draws=scene.draws[:keep]), *_submit(run))
    renderer.free_command_buffer(run.cb)

    scene = CASES["batched"]
    counts = np.arange(len(scene.draws), dtype=np.uint32) % 2 == 0
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, indirect="device", counts=counts.astype(np.uint32))
    _check(dataclasses.replace(scene, draws=scene.draws[0::2]), *_submit(run))
    renderer.write_buffer(run.count_buf, np.full(len(scene.draws), 5, dtype=np.uint32))
    _check(scene, *_submit(run))
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_device_advertises_indirect_draws(renderer):
    """VK_KHR_draw_indirect_count is listed (count query, then fill), and multiDrawIndirect and
    drawIndirectFirstInstance are reported as features"""
    d = renderer.drv
    n = ctypes.c_uint32(0)
    assert d.vkEnumerateDeviceExtensionProperties(renderer.physical, None, ctypes.byref(n), None) == vk.VK_SUCCESS
    props = (vk.VkExtensionProperties * n.value)()
    assert d.vkEnumerateDeviceExtensionProperties(renderer.physical, None, ctypes.byref(n), props) == vk.VK_SUCCESS
    assert b"VK_KHR_draw_indirect_count" in [p.extensionName for p in props]
    feats = (ctypes.c_uint32 * 55)()
    d.vkGetPhysicalDeviceFeatures(renderer.physical, feats)
    assert feats[1] == 1 and feats[9] == 1 and feats[10] == 1

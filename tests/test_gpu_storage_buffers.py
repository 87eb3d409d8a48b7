"""GPU checks of read-only storage buffers: a fragment shader reads element uint(a.x) of a runtime-sized
array (and a fixed member) of a storage block; indices past the bound range are limited to its last whole
element, so each cell's bits equal the numpy restatement, for two bound ranges and a descriptor offset."""
import dataclasses

import numpy as np
import pytest

from kazan_gb300 import render, vk

import shader_ops as so


def _record_dynamic(run, dset, dyn_offset):
    """the run's draw with its set bound at a dynamic offset"""
    from ctypes import byref, c_uint32, c_uint64, c_void_p
    r, s, d = run.r, run.scene, run.r.drv
    cb = r.begin()
    clears = (vk.VkClearValue * 2)()
    clears[0].color.float32[:] = list(s.clear_color)
    clears[1].depthStencil.depth = s.clear_depth
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                   vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(s.width, s.height)), 2, clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
    d.vkCmdBindVertexBuffers(cb, 0, 1, (c_void_p * 1)(run.vb.handle.value), (c_uint64 * 1)(0))
    d.vkCmdBindDescriptorSets(cb, vk.BIND_POINT_GRAPHICS, run.layout, 0, 1, (c_void_p * 1)(dset.value), 1,
                              (c_uint32 * 1)(dyn_offset))
    d.vkCmdDraw(cb, 3 * s.draws[0].count, 1, s.draws[0].first, 0)
    d.vkCmdEndRenderPass(cb)
    vk.check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
    return cb


@pytest.mark.gpu
@pytest.mark.parametrize("dynamic", [False, True])
@pytest.mark.parametrize("n, extra", [(100, 0), (37, 4)])
def test_runtime_array_read_and_clamped(renderer, n, extra, dynamic):
    r = renderer
    idx = np.concatenate([np.arange(0, 120), np.arange(120, 1000, 7)[:100],
                          [1e4, 65535, 3e6, 4e9, 0.5, 36.9, 37.0, 99.0]]).astype(np.float32)[:so.GRID * so.GRID]
    inputs = np.zeros((len(idx), 4), dtype=np.float32)
    inputs[:, 0] = idx
    scene = so.cell_scene(inputs, so.storage_fs())
    rng = np.random.default_rng(n)
    words = rng.integers(0, 2 ** 32, 16 + (so.SSBO_BASE + so.SSBO_STRIDE * (n + 8)) // 4, dtype=np.uint64)
    words = words.astype(np.uint32)
    offset = 64  # the block starts 64 bytes into the buffer (beyond it: unrelated words)
    buf = r.create_buffer(words.nbytes, vk.BUFFER_USAGE_STORAGE, True)
    r.write_buffer(buf, words)
    rng_bytes = so.SSBO_BASE + so.SSBO_STRIDE * n + extra

    # the run's own pipeline with the plain colour shader, then the storage-buffer pipeline in its place
    run = render.SceneRun(r, dataclasses.replace(scene, fs_words=None), mode="batched", tile=16)
    dtype = vk.DESCRIPTOR_STORAGE_BUFFER_DYNAMIC if dynamic else vk.DESCRIPTOR_STORAGE_BUFFER
    lay = r.set_layout([(0, dtype, 1)])
    dset = r.descriptor_sets(lay)[0]
    # dynamic: the descriptor at offset 0, the block's 64 bytes given as the dynamic offset at binding
    r.write_buffer_descriptor(dset, 0, buf, 0 if dynamic else offset, rng_bytes, dtype=dtype)
    run.layout = r.pipeline_layout(0, [lay])
    vs, _ = scene.shaders()
    run.pipe = r.pipeline(scene, run.rp, run.layout, vs, scene.fs_words)
    run.dsets = [dset]
    r.free_command_buffer(run.cb)
    run.cb = _record_dynamic(run, dset, offset) if dynamic else run.record()
    run.submit()
    color, _ = run.read()
    got = so.read_bits(color, len(idx))

    blk = words[offset // 4:]
    bias = blk[0]
    vals = blk[so.SSBO_BASE // 4:].reshape(-1, 2)
    e = np.minimum(idx.astype(np.float64).astype(np.uint64), n - 1)
    want = (vals[e, 1] ^ bias).astype(np.uint32)
    assert np.array_equal(got, want), np.argwhere(got != want)[:5]
    r.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_range_smaller_than_the_block_is_a_recording_error(renderer):
    r = renderer
    scene = so.cell_scene(np.zeros((4, 4), dtype=np.float32), so.storage_fs())
    buf = r.create_buffer(256, vk.BUFFER_USAGE_STORAGE, True)
    # the run's own pipeline with the plain colour shader, then the storage-buffer pipeline in its place
    run = render.SceneRun(r, dataclasses.replace(scene, fs_words=None), mode="batched", tile=16)
    lay = r.set_layout([(0, vk.DESCRIPTOR_STORAGE_BUFFER, 1)])
    dset = r.descriptor_sets(lay)[0]
    r.write_buffer_descriptor(dset, 0, buf, 0, so.SSBO_BASE + so.SSBO_STRIDE - 4, dtype=vk.DESCRIPTOR_STORAGE_BUFFER)
    run.layout = r.pipeline_layout(0, [lay])
    vs, _ = scene.shaders()
    run.pipe = r.pipeline(scene, run.rp, run.layout, vs, scene.fs_words)
    run.dsets = [dset]
    r.free_command_buffer(run.cb)
    with pytest.raises(vk.VkError):
        run.cb = run.record()

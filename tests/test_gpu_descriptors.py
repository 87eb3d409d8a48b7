"""GPU parity of descriptor sets: combined image samplers read by the fragment shader (every filter, address
mode, border colour and texel byte order, normalized and unnormalized coordinates) and uniform buffers read
by the vertex shader (one buffer, a dynamic offset per draw) render bit for bit what the CPU oracle
renders; descriptors the shaders need but the draw lacks are errors at recording, not reads of unset
memory."""
import ctypes
import dataclasses
from ctypes import byref, c_uint32, c_void_p

import numpy as np
import pytest

from kazan_gb300 import render, scenes, spirv_asm, vk
from oracle import kz_oracle

from scene_cases import small_cases

SAMPLERS = {
    "nearest_repeat": dict(),
    "nearest_mirror_clamp": dict(address_u=1, address_v=2),
    "nearest_border_white_bgra": dict(address_u=3, address_v=3, border=2, bgra=True),
    "linear_repeat": dict(linear=True),
    "linear_mirror": dict(linear=True, address_u=1, address_v=1),
    "linear_edge_border": dict(linear=True, address_u=2, address_v=3, border=1),
    "linear_mirror_clamp_edge": dict(linear=True, address_u=4, address_v=4),
    "linear_border_black_transparent": dict(linear=True, address_u=3, address_v=0, border=0),
    "nearest_unnormalized": dict(unnormalized=True, address_u=2, address_v=2),
    "linear_unnormalized_bgra": dict(linear=True, unnormalized=True, address_u=3, address_v=3, border=2, bgra=True),
}


def _scene(name):
    kw = dict(SAMPLERS[name])
    unnorm = kw.get("unnormalized", False)
    return scenes.textured(seed=6 + len(name), uv_lo=-7.0 if unnorm else -1.5, uv_hi=68.0 if unnorm else 2.5, **kw)


def _check(scene, color, depth, st):
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s: gpu %s oracle %s" % (
        len(mism), mism[:1], color[tuple(mism[0])] if len(mism) else None, ref_c[tuple(mism[0])] if len(mism) else None)
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.status == 0
    assert st.fragments == ost["fragments"] % (1 << 32)


def _render(renderer, scene, mode="batched", **kw):
    run = render.SceneRun(renderer, scene, mode=mode, tile=16, **kw)
    run.submit()
    color, depth = run.read()
    out = color, depth, run.stats()
    renderer.free_command_buffer(run.cb)
    return run, out


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent"])
@pytest.mark.parametrize("name", sorted(SAMPLERS))
def test_textured_matches_oracle(renderer, name, mode):
    scene = _scene(name)
    _, out = _render(renderer, scene, mode)
    _check(scene, *out)


@pytest.mark.gpu
def test_explicit_lod_samples_the_same(renderer):
    """OpImageSampleExplicitLod with Lod 0 on a one-level image is the implicit-LOD sample"""
    scene = _scene("linear_mirror")
    scene.fs_words = spirv_asm.textured_fs(explicit_lod=True)
    _, out = _render(renderer, scene)
    _check(scene, *out)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
def test_uniform_buffer_matrices_match_oracle(renderer, mode):
    """the 48-draw Lambert scene with each draw's matrix read from a uniform buffer at a dynamic offset
    renders what the push-constant form (and the oracle) renders"""
    scene = dataclasses.replace(small_cases()["batched"], ubo=True)
    _, out = _render(renderer, scene, mode)
    _check(scene, *out)


@pytest.mark.gpu
def test_uniform_buffer_with_indirect_draws(renderer):
    scene = dataclasses.replace(small_cases()["batched"], ubo=True)
    _, out = _render(renderer, scene, indirect="device")
    _check(scene, *out)


@pytest.mark.gpu
def test_rewritten_descriptor_takes_effect_at_recording(renderer):
    """a command buffer recorded after vkUpdateDescriptorSets points the set at another image samples that
    image"""
    scene = _scene("linear_repeat")
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    other = np.ascontiguousarray(scene.texture.texels[::-1, ::-1])
    img = renderer.create_image(other.shape[1], other.shape[0], vk.FORMAT_R8G8B8A8_UNORM, vk.IMAGE_USAGE_SAMPLED, True)
    renderer.write_image(img, other)
    renderer.write_image_descriptor(run.dsets[0], 0, 0, renderer.sampler(scene.texture), img)
    renderer.free_command_buffer(run.cb)
    run.cb = run.record()
    run.submit()
    color, depth = run.read()
    _check(dataclasses.replace(scene, texture=dataclasses.replace(scene.texture, texels=other)), color, depth,
           run.stats())
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_array_of_samplers_with_run_time_index(renderer):
    """texture(tex[u < 0.5 ? 0 : 1], uv): every pixel equals the render with tex[0] alone or with tex[1]
    alone (each checked against the oracle), and both occur"""
    base = _scene("nearest_repeat")
    other = scenes.Texture(np.ascontiguousarray(base.texture.texels[:, ::-1]))
    ref0 = _render(renderer, base)[1]
    alt = dataclasses.replace(base, texture=other)
    ref1 = _render(renderer, alt)[1]
    _check(base, *ref0)
    _check(alt, *ref1)
    r = renderer
    run = render.SceneRun(r, base, mode="batched", tile=16)
    lay = r.set_layout([(0, vk.DESCRIPTOR_COMBINED_IMAGE_SAMPLER, 2)])
    dset = r.descriptor_sets(lay)[0]
    img1 = r.create_image(other.texels.shape[1], other.texels.shape[0], vk.FORMAT_R8G8B8A8_UNORM,
                          vk.IMAGE_USAGE_SAMPLED, True)
    r.write_image(img1, other.texels)
    smp = r.sampler(base.texture)
    r.write_image_descriptor(dset, 0, 0, smp, run.tex_image)
    r.write_image_descriptor(dset, 0, 1, smp, img1)
    run.layout = r.pipeline_layout(0, [lay])
    vs, _ = base.shaders()
    run.pipe = r.pipeline(base, run.rp, run.layout, vs, spirv_asm.textured_array_fs(2))
    run.dsets = [dset]
    r.free_command_buffer(run.cb)
    run.cb = run.record()
    run.submit()
    color, _ = run.read()
    is0 = np.all(color == ref0[0], axis=-1)
    is1 = np.all(color == ref1[0], axis=-1)
    assert np.all(is0 | is1)
    assert np.any(is0 & ~is1) and np.any(is1 & ~is0)
    r.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_missing_descriptors_are_recording_errors(renderer):
    """a pipeline whose layout lacks the shader's binding fails to create; a draw with the set unbound, or
    bound but never written, fails at vkEndCommandBuffer; a sampler with different min and mag filters is
    refused"""
    r, d = renderer, renderer.drv
    scene = _scene("nearest_repeat")
    run = render.SceneRun(r, scene, mode="batched", tile=16)
    vs, fs = scene.shaders()
    with pytest.raises(vk.VkError):
        r.pipeline(scene, run.rp, r.pipeline_layout(0), vs, fs)

    def record(bind, dset):
        cb = r.begin()
        clears = (vk.VkClearValue * 2)()
        rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                       vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(scene.width, scene.height)), 2,
                                       clears)
        d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
        d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
        if bind:
            sets = (c_void_p * 1)(dset.value)
            d.vkCmdBindDescriptorSets(cb, vk.BIND_POINT_GRAPHICS, run.layout, 0, 1, sets, 0, None)
        bufs = (c_void_p * 1)(run.vb.handle.value)
        d.vkCmdBindVertexBuffers(cb, 0, 1, bufs, (ctypes.c_uint64 * 1)(0))
        d.vkCmdDraw(cb, 3 * scene.triangles, 1, 0, 0)
        d.vkCmdEndRenderPass(cb)
        rc = d.vkEndCommandBuffer(cb)
        r.free_command_buffer(cb)
        return rc

    assert record(True, run.dsets[0]) == vk.VK_SUCCESS
    assert record(False, None) == vk.VK_ERROR_INITIALIZATION_FAILED
    empty = r.descriptor_sets(run.set_layouts[0])[0]
    assert record(True, empty) == vk.VK_ERROR_INITIALIZATION_FAILED
    ci = vk.VkSamplerCreateInfo(vk.ST_SAMPLER_CREATE_INFO, None, 0, vk.FILTER_LINEAR, vk.FILTER_NEAREST, 0, 0, 0, 0,
                                0.0, 0, 1.0, 0, 0, 0.0, 0.0, 0, 0)
    h = c_void_p()
    assert d.vkCreateSampler(r.device, byref(ci), None, byref(h)) == vk.VK_ERROR_FEATURE_NOT_PRESENT
    r.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["nearest_repeat", "linear_edge_border", "linear_unnormalized_bgra"])
def test_separate_image_and_sampler(renderer, name):
    """texture(sampler2D(tex, smp), uv) with a sampled image at binding 0 and a sampler at binding 1 (the
    sampler's state replaces the image descriptor's in a local copy): the same pixels as the combined image
    sampler, checked against the oracle"""
    scene = _scene(name)
    r = renderer
    run = render.SceneRun(r, scene, mode="batched", tile=16)
    lay = r.set_layout([(0, vk.DESCRIPTOR_SAMPLED_IMAGE, 1), (1, vk.DESCRIPTOR_SAMPLER, 1)])
    dset = r.descriptor_sets(lay)[0]
    r.write_image_descriptor(dset, 0, 0, None, run.tex_image, vk.DESCRIPTOR_SAMPLED_IMAGE)
    r.write_image_descriptor(dset, 1, 0, r.sampler(scene.texture), None, vk.DESCRIPTOR_SAMPLER)
    run.layout = r.pipeline_layout(0, [lay])
    vs, _ = scene.shaders()
    run.pipe = r.pipeline(scene, run.rp, run.layout, vs, spirv_asm.textured_separate_fs())
    run.dsets = [dset]
    r.free_command_buffer(run.cb)
    run.cb = run.record()
    run.submit()
    color, depth = run.read()
    _check(scene, color, depth, run.stats())
    r.free_command_buffer(run.cb)

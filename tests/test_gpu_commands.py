"""GPU checks of the transfer and state commands around the draw path: vkCmdUpdateBuffer (vertex data written by
the command buffer itself), vkCmdCopyImage, vkCmdClearAttachments between draws of one render pass, and
dynamic stencil reference / masks, each against the CPU oracle or a numpy restatement."""
import ctypes
import dataclasses
from ctypes import byref, c_uint32, c_uint64, c_void_p

import numpy as np
import pytest

from kazan_gb300 import render, scenes, vk
from oracle import kz_oracle

from scene_cases import small_cases


def _record(run, body, before=None):
    """a command buffer: `before(d, cb)` outside the pass, then the pass with the run's pipeline and vertex
    buffer bound and `body(d, cb)` recording the draws"""
    r, s, d = run.r, run.scene, run.r.drv
    cb = r.begin()
    if before:
        before(d, cb)
    clears = (vk.VkClearValue * 2)()
    clears[0].color.float32[:] = list(s.clear_color)
    clears[1].depthStencil.depth = s.clear_depth
    clears[1].depthStencil.stencil = s.clear_stencil
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                   vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(s.width, s.height)), 2, clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
    bufs = (c_void_p * 1)(run.vb.handle.value)
    d.vkCmdBindVertexBuffers(cb, 0, 1, bufs, (c_uint64 * 1)(0))
    if run.ib is not None:
        d.vkCmdBindIndexBuffer(cb, run.ib.handle, 0, vk.INDEX_TYPE_UINT32)
    body(d, cb)
    d.vkCmdEndRenderPass(cb)
    vk.check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
    return cb


def _submit(run, cb):
    run.r.submit_wait(cb)
    color, depth = run.read()
    st = run.r.drv.stats(cb)
    run.r.free_command_buffer(cb)
    return color, depth, st


def _draw(d, cb, run, dr):
    if dr.mvp is not None:
        m = np.ascontiguousarray(dr.mvp, dtype=np.float32)
        d.vkCmdPushConstants(cb, run.layout, vk.SHADER_STAGE_VERTEX, 0, 64, m.ctypes.data)
    if run.scene.indexed:
        d.vkCmdDrawIndexed(cb, 3 * dr.count, 1, dr.first, dr.vertex_offset, 0)
    else:
        d.vkCmdDraw(cb, 3 * dr.count, 1, dr.first, 0)


@pytest.mark.gpu
def test_update_buffer_writes_vertex_data(renderer):
    """the soup's vertices reach a device-local buffer only through vkCmdUpdateBuffer (64 KB pieces) in the
    command buffer that draws them"""
    scene = small_cases()["soup"]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    vb2 = renderer.create_buffer(scene.vertices.nbytes, vk.BUFFER_USAGE_VERTEX, False)
    raw = np.ascontiguousarray(scene.vertices).view(np.uint8).ravel()

    def before(d, cb):
        for off in range(0, raw.size, 65536):
            piece = np.ascontiguousarray(raw[off:off + 65536])
            d.vkCmdUpdateBuffer(cb, vb2.handle, off, piece.size, piece.ctypes.data)

    run.vb = vb2
    cb = _record(run, lambda d, cb: _draw(d, cb, run, scene.draws[0]), before)
    color, depth, st = _submit(run, cb)
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    assert np.array_equal(color, ref_c) and np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == ost["fragments"]


@pytest.mark.gpu
def test_copy_image_region(renderer):
    scene = small_cases()["soup"]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    run.submit()
    color, _ = run.read()
    dst = renderer.create_image(90, 70, vk.FORMAT_R8G8B8A8_UNORM, vk.IMAGE_USAGE_COLOR_ATTACHMENT, True)
    cb = renderer.begin()
    sub = vk.VkImageSubresourceLayers(vk.IMAGE_ASPECT_COLOR, 0, 0, 1)
    reg = vk.VkImageCopy(sub, vk.VkOffset3D(100, 33, 0), sub, vk.VkOffset3D(7, 3, 0), vk.VkExtent3D(80, 60, 1))
    renderer.drv.vkCmdCopyImage(cb, run.color.handle, vk.IMAGE_LAYOUT_GENERAL, dst.handle, vk.IMAGE_LAYOUT_GENERAL, 1,
                                byref(reg))
    renderer.end_submit_wait(cb)
    renderer.free_command_buffer(cb)
    got = renderer.read_image(dst)
    assert np.array_equal(got[3:63, 7:87], color[33:93, 100:180])
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent"])
def test_clear_attachments_between_draws(renderer, mode):
    """half of the 48 draws, a clear of two colour rectangles and one depth rectangle, then the other half:
    the oracle renders the first half, applies the clears to its images and renders the rest into them"""
    scene = small_cases()["batched"]
    run = render.SceneRun(renderer, scene, mode=mode, tile=16)
    half = len(scene.draws) // 2
    crects = [(20, 30, 200, 100), (300, 250, 120, 220)]
    drect = (150, 150, 256, 256)
    ccol = (0.25, 0.5, 1.0, 0.75)

    def body(d, cb):
        for dr in scene.draws[:half]:
            _draw(d, cb, run, dr)
        atts = (vk.VkClearAttachment * 2)()
        atts[0].aspectMask = vk.IMAGE_ASPECT_COLOR
        atts[0].colorAttachment = 0
        atts[0].clearValue.color.float32[:] = list(ccol)
        atts[1].aspectMask = vk.IMAGE_ASPECT_DEPTH
        atts[1].clearValue.depthStencil.depth = 0.0
        rc = (vk.VkClearRect * 2)(*[vk.VkClearRect(vk.VkRect2D(vk.VkOffset2D(x, y), vk.VkExtent2D(w, h)), 0, 1)
                                    for x, y, w, h in crects])
        d.vkCmdClearAttachments(cb, 1, ctypes.cast(atts, c_void_p), 2, ctypes.cast(rc, c_void_p))
        rd = vk.VkClearRect(vk.VkRect2D(vk.VkOffset2D(drect[0], drect[1]), vk.VkExtent2D(drect[2], drect[3])), 0, 1)
        d.vkCmdClearAttachments(cb, 1, ctypes.cast(byref(atts[1]), c_void_p), 1, ctypes.cast(byref(rd), c_void_p))
        for dr in scene.draws[half:]:
            _draw(d, cb, run, dr)

    color, depth, st = _submit(run, _record(run, body))
    ref_c, ref_d, s0 = kz_oracle.render(scene, threads=8, draws=scene.draws[:half])
    px = [kz_oracle.unorm8(v) for v in ccol]
    for x, y, w, h in crects:
        ref_c[y:y + h, x:x + w] = px
    ref_d[drect[1]:drect[1] + drect[3], drect[0]:drect[0] + drect[2]] = 0.0
    ref_c, ref_d, s1 = kz_oracle.render(scene, threads=8, draws=scene.draws[half:], color=ref_c, depth=ref_d)
    assert np.array_equal(color, ref_c)
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == s0["fragments"] + s1["fragments"]
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_dynamic_stencil_reference_and_masks(renderer):
    """REPLACE with a dynamic reference: 3 for the first draw, then 7 for front faces only with a dynamic write
    mask of 0x0F; the oracle renders the same two draws with those static states"""
    S = scenes.StencilOp
    base = small_cases()["soup"]
    scene = dataclasses.replace(base, draws=[scenes.Draw(0, 1024), scenes.Draw(1024, 1024)], depth_format="d24s8",
                                stencil=dict(front=S(pass_=2, depth_fail=2, write_mask=0xFF),
                                             back=S(pass_=2, depth_fail=2, write_mask=0xFF)), clear_stencil=0x50)
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    vs, fs = scene.shaders()
    run.pipe = renderer.pipeline(scene, run.rp, run.layout, vs, fs,
                                 dynamic=(vk.DYNAMIC_STATE_STENCIL_WRITE_MASK, vk.DYNAMIC_STATE_STENCIL_REFERENCE))

    def body(d, cb):
        d.vkCmdSetStencilWriteMask(cb, 3, 0xFF)
        d.vkCmdSetStencilReference(cb, 3, 3)
        _draw(d, cb, run, scene.draws[0])
        d.vkCmdSetStencilReference(cb, 1, 7)
        d.vkCmdSetStencilWriteMask(cb, 1, 0x0F)
        _draw(d, cb, run, scene.draws[1])

    color, depth, st = _submit(run, _record(run, body))
    # the oracle: the same draws, each with its stencil state written out
    col, dep = kz_oracle.clear_images(scene)
    sten = np.full((scene.height, scene.width), 0x50, dtype=np.uint8)
    arr, n = kz_oracle.make_draws(scene)
    for face in ("front", "back"):
        getattr(arr[0], face).reference = 3
        getattr(arr[1], face).reference = 7 if face == "front" else 3
    arr[1].front.write_mask = 0x0F
    ost = kz_oracle.KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, scene.width, scene.height)
    kz_oracle.lib().kzo_render_ds(scene.width, scene.height, col.ctypes.data, dep.ctypes.data, sten.ctypes.data,
                                  kz_oracle.DEPTH_FORMAT["d24s8"], area, n, arr, 8, byref(ost))
    assert np.array_equal(color, col)
    assert np.array_equal(depth, kz_oracle.packed_depth(dep, sten, "d24s8"))
    assert len(np.unique(depth >> 24)) >= 3


def _region(buf_off, row_len, x, y, w, h):
    return vk.VkBufferImageCopy(buf_off, row_len, 0, vk.VkImageSubresourceLayers(vk.IMAGE_ASPECT_COLOR, 0, 0, 1),
                                vk.VkOffset3D(x, y, 0), vk.VkExtent3D(w, h, 1))


@pytest.mark.gpu
def test_fill_and_buffer_image_copies(renderer):
    """vkCmdFillBuffer at an unaligned word offset, vkCmdCopyBufferToImage with and without bufferRowLength and
    vkCmdCopyImageToBuffer at a buffer offset, in one command buffer, against the same steps in numpy"""
    W, H = 64, 48
    rng = np.random.default_rng(11)
    raw = rng.integers(0, 256, W * H * 4 + 4096, dtype=np.uint8)
    src = renderer.create_buffer(raw.size, 0, True)
    renderer.write_buffer(src, raw)
    img = renderer.create_image(W, H, vk.FORMAT_R8G8B8A8_UNORM, vk.IMAGE_USAGE_TRANSFER_DST, False)
    out_w, out_h, out_off = W - 6, H - 9, 64
    dst = renderer.create_buffer(out_off + out_w * out_h * 4, 0, True)
    fill_off, word = W * H * 4 + 4, 0xA5C30F11
    d = renderer.drv
    cb = renderer.begin()
    d.vkCmdFillBuffer(cb, src.handle, fill_off, 16 * 16 * 4, word)
    regions = [_region(0, 0, 0, 0, W, H),                 # the whole image, tight rows
               _region(fill_off, 16, 5, 7, 16, 16),       # the filled words
               _region(12, 50, 30, 20, 20, 10)]           # rows 50 texels apart in the buffer
    for reg in regions:
        d.vkCmdCopyBufferToImage(cb, src.handle, img.handle, vk.IMAGE_LAYOUT_GENERAL, 1, byref(reg))
    back = _region(out_off, 0, 2, 3, out_w, out_h)
    d.vkCmdCopyImageToBuffer(cb, img.handle, vk.IMAGE_LAYOUT_GENERAL, dst.handle, 1, byref(back))
    renderer.end_submit_wait(cb)
    renderer.free_command_buffer(cb)

    model = raw[:W * H * 4].reshape(H, W, 4).copy()
    model[7:23, 5:21] = np.frombuffer(np.full(256, word, dtype="<u4").tobytes(), np.uint8).reshape(16, 16, 4)
    rows = raw[12:12 + 50 * 4 * 10].reshape(10, 200)[:, :80]
    model[20:30, 30:50] = rows.reshape(10, 20, 4)
    p = renderer.map(dst)
    got = np.ctypeslib.as_array((ctypes.c_uint8 * (out_w * out_h * 4)).from_address(p + out_off)).copy()
    renderer.unmap(dst)
    assert np.array_equal(got.reshape(out_h, out_w, 4), model[3:3 + out_h, 2:2 + out_w])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["copy_past_end", "fill_past_end", "fill_unaligned", "image_region_outside",
                                  "buffer_too_small", "row_length_short"])
def test_transfer_regions_outside_their_objects_are_recording_errors(renderer, case):
    """a region that leaves its buffer or image fails vkEndCommandBuffer; nothing of it reaches the device"""
    a = renderer.create_buffer(4096, 0, True)
    b = renderer.create_buffer(1024, 0, True)
    img = renderer.create_image(32, 16, vk.FORMAT_R8G8B8A8_UNORM, vk.IMAGE_USAGE_TRANSFER_DST, False)
    d = renderer.drv
    cb = renderer.begin()
    if case == "copy_past_end":
        reg = vk.VkBufferCopy(0, 512, 1024)
        d.vkCmdCopyBuffer(cb, a.handle, b.handle, 1, byref(reg))
    elif case == "fill_past_end":
        d.vkCmdFillBuffer(cb, b.handle, 1020, 8, 0)
    elif case == "fill_unaligned":
        d.vkCmdFillBuffer(cb, b.handle, 2, 8, 0)
    elif case == "image_region_outside":
        reg = _region(0, 0, 20, 0, 16, 4)
        d.vkCmdCopyBufferToImage(cb, a.handle, img.handle, vk.IMAGE_LAYOUT_GENERAL, 1, byref(reg))
    elif case == "buffer_too_small":
        reg = _region(0, 0, 0, 0, 32, 16)
        d.vkCmdCopyImageToBuffer(cb, img.handle, vk.IMAGE_LAYOUT_GENERAL, b.handle, 1, byref(reg))
    else:
        reg = _region(0, 8, 0, 0, 16, 4)
        d.vkCmdCopyBufferToImage(cb, a.handle, img.handle, vk.IMAGE_LAYOUT_GENERAL, 1, byref(reg))
    assert d.vkEndCommandBuffer(cb) == vk.VK_ERROR_INITIALIZATION_FAILED
    renderer.free_command_buffer(cb)


# (x, y, width, height, minDepth, maxDepth): the whole framebuffer; a fractional offset with a narrowed
# depth range; a viewport reaching past the left edge with an inverted depth range; a y-flipped viewport
_VIEWPORTS = [None, (37.5, 20.25, 300.0, 260.0, 0.2, 0.9), (-100.0, 64.0, 700.0, 380.0, 1.0, 0.0),
              (20.0, 460.0, 420.0, -400.0, 0.0, 1.0)]
_SCISSORS = [None, (0, 0, 256, 512), (100, 37, 333, 250), (60, 0, 1000, 1000)]


def _split_draws(scene, parts):
    """the same triangles as `parts` consecutive non-indexed draws"""
    n = scene.draws[0].count
    step = (n + parts - 1) // parts
    draws = [scenes.Draw(3 * k, min(step, n - k)) for k in range(0, n, step)]
    return dataclasses.replace(scene, draws=draws)


@pytest.mark.gpu
@pytest.mark.parametrize("case,tile", [("batched", 16), ("blend", 16), ("blend8", 16), ("blend8", 32)])
def test_viewports_scissors_and_render_area(renderer, case, tile):
    """dynamic viewport and scissor changed between draws, inside a render area smaller than the framebuffer
    whose loadOp CLEAR clears only that area: the attachments were filled beforehand by vkCmdClearColorImage
    and vkCmdClearDepthStencilImage, and the oracle gets the same per-draw rectangles.  blend8: the blended
    scene as 8 draws, so that every viewport and scissor reaches the ordered (tile) path, in its common kernel
    (tile 16) and its general one (tile 32)"""
    scene = _split_draws(small_cases()["blend"], 8) if case == "blend8" else small_cases()[case]
    W, H = scene.width, scene.height
    area = (16, 24, W - 52, H - 40)                      # x, y, width, height
    run = render.SceneRun(renderer, scene, mode="batched", tile=tile)
    vs, fs = scene.shaders()
    run.pipe = renderer.pipeline(scene, run.rp, run.layout, vs, fs,
                                 dynamic=(vk.DYNAMIC_STATE_VIEWPORT, vk.DYNAMIC_STATE_SCISSOR))
    pre_color, pre_depth = (0.9, 0.1, 0.4, 0.6), 0.8

    def viewport(i):
        v = _VIEWPORTS[i % len(_VIEWPORTS)] or (0.0, 0.0, float(W), float(H), 0.0, 1.0)
        return vk.VkViewport(*v), list(v)

    def scissor(i):
        s = _SCISSORS[(i // 2) % len(_SCISSORS)] or (0, 0, W, H)
        return vk.VkRect2D(vk.VkOffset2D(s[0], s[1]), vk.VkExtent2D(s[2], s[3])), list(s)

    r, d = renderer, renderer.drv
    cb = r.begin()
    cc = vk.VkClearColorValue()
    cc.float32[:] = list(pre_color)
    d.vkCmdClearColorImage(cb, run.color.handle, vk.IMAGE_LAYOUT_GENERAL, byref(cc), 1,
                           byref(vk.VkImageSubresourceRange(vk.IMAGE_ASPECT_COLOR, 0, 1, 0, 1)))
    d.vkCmdClearDepthStencilImage(cb, run.depth.handle, vk.IMAGE_LAYOUT_GENERAL,
                                  byref(vk.VkClearDepthStencilValue(pre_depth, 0)), 1,
                                  byref(vk.VkImageSubresourceRange(render._aspect(run.depth.format), 0, 1, 0, 1)))
    clears = (vk.VkClearValue * 2)()
    clears[0].color.float32[:] = list(scene.clear_color)
    clears[1].depthStencil.depth = scene.clear_depth
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, run.fb,
                                   vk.VkRect2D(vk.VkOffset2D(area[0], area[1]), vk.VkExtent2D(area[2], area[3])),
                                   2, clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
    d.vkCmdBindVertexBuffers(cb, 0, 1, (c_void_p * 1)(run.vb.handle.value), (c_uint64 * 1)(0))
    if run.ib is not None:
        d.vkCmdBindIndexBuffer(cb, run.ib.handle, 0, vk.INDEX_TYPE_UINT32)
    for i, dr in enumerate(scene.draws):
        vp, _ = viewport(i)
        sc, _ = scissor(i)
        d.vkCmdSetViewport(cb, 0, 1, byref(vp))
        d.vkCmdSetScissor(cb, 0, 1, byref(sc))
        _draw(d, cb, run, dr)
    d.vkCmdEndRenderPass(cb)
    vk.check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
    color, depth, st = _submit(run, cb)

    col = np.empty((H, W, 4), dtype=np.uint8)
    col[:] = [kz_oracle.unorm8(v) for v in pre_color]
    dep = np.full((H, W), np.float32(pre_depth), dtype=np.float32)
    x0, y0, x1, y1 = area[0], area[1], area[0] + area[2], area[1] + area[3]
    col[y0:y1, x0:x1] = [kz_oracle.unorm8(v) for v in scene.clear_color]
    dep[y0:y1, x0:x1] = np.float32(scene.clear_depth)
    arr, n = kz_oracle.make_draws(scene)
    for i in range(n):
        arr[i].viewport[:] = viewport(i)[1]
        arr[i].scissor[:] = scissor(i)[1]
    ost = kz_oracle.KzoStats()
    rect = (ctypes.c_int32 * 4)(x0, y0, x1, y1)
    rc = kz_oracle.lib().kzo_render_ds(W, H, col.ctypes.data, dep.ctypes.data, None, kz_oracle.DEPTH_FORMAT["d32"],
                                       rect, n, arr, 8, byref(ost))
    assert rc == 0
    assert np.array_equal(color, col)
    assert np.array_equal(depth.view(np.uint32), dep.view(np.uint32))
    assert st.fragments == ost.as_dict()["fragments"]
    assert 0 < st.fragments
    r.free_command_buffer(run.cb)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["soup", "batched"])
def test_empty_and_ragged_draws(renderer, case):
    """draws with no vertices, with no instances, and with 1 or 2 vertices past the last whole triangle
    (ignored) among the scene's draws, and one draw reaching past the end of its buffer (skipped): the image
    is the scene's own"""
    scene = small_cases()[case]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)

    def body(d, cb):
        for k, dr in enumerate(scene.draws):
            if dr.mvp is not None:
                m = np.ascontiguousarray(dr.mvp, dtype=np.float32)
                d.vkCmdPushConstants(cb, run.layout, vk.SHADER_STAGE_VERTEX, 0, 64, m.ctypes.data)
            extra = 1 + k % 2
            if scene.indexed:
                d.vkCmdDrawIndexed(cb, 0, 1, dr.first, dr.vertex_offset, 0)
                d.vkCmdDrawIndexed(cb, 3 * dr.count, 0, dr.first, dr.vertex_offset, 0)
                d.vkCmdDrawIndexed(cb, 3 * dr.count + extra, 1, dr.first, dr.vertex_offset, 0)
            else:
                d.vkCmdDraw(cb, 0, 1, dr.first, 0)
                d.vkCmdDraw(cb, 3 * dr.count, 0, dr.first, 0)
                d.vkCmdDraw(cb, 3 * dr.count + extra, 1, dr.first, 0)
        # past the end of the bound index or vertex buffer: skipped at recording
        if scene.indexed:
            d.vkCmdDrawIndexed(cb, 6, 1, len(scene.indices) - 3, 0, 0)
        else:
            d.vkCmdDraw(cb, 6, 1, len(scene.vertices) - 3, 0)

    color, depth, st = _submit(run, _record(run, body))
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    assert np.array_equal(color, ref_c)
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == ost["fragments"]
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_pass_without_draws_only_clears(renderer):
    scene = small_cases()["batched"]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    color, depth, st = _submit(run, _record(run, lambda d, cb: None))
    ref_c, ref_d = kz_oracle.clear_images(scene)
    assert np.array_equal(color, ref_c) and np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == 0
    renderer.free_command_buffer(run.cb)


def _instanced_vs():
    """gl_Position = in0 + in2 (in2 read per instance); out0 = in1 + (gl_InstanceIndex * 0.125, 0, 0, 0)"""
    from kazan_gb300 import spirv_asm as sa
    m = sa.Module()
    m.capability(sa.CapShader)
    f32, i32 = m.f32(), m.i32(1)
    v4 = m.vec(f32, 4)
    pv = sa._per_vertex(m)
    in_pos, in_col = sa._io(m, sa.SCInput, v4, 0), sa._io(m, sa.SCInput, v4, 1)
    in_off = sa._io(m, sa.SCInput, v4, 2)
    inst = m.variable(sa.SCInput, m.ptr(sa.SCInput, i32))
    m.decorate(inst, sa.DecBuiltIn, sa.BuiltInInstanceIndex)
    out_col = sa._io(m, sa.SCOutput, v4, 0)
    fn = sa._begin_main(m)
    p = m.res(sa.OpFAdd, v4, m.res(sa.OpLoad, v4, in_pos), m.res(sa.OpLoad, v4, in_off))
    m.op(sa.OpStore, m.res(sa.OpAccessChain, m.ptr(sa.SCOutput, v4), pv, m.ci(0)), p)
    c = m.res(sa.OpLoad, v4, in_col)
    k = m.res(sa.OpFMul, f32, m.res(sa.OpConvertSToF, f32, m.res(sa.OpLoad, i32, inst)), m.cf(0.125))
    comps = [m.res(sa.OpCompositeExtract, f32, c, j) for j in range(4)]
    comps[0] = m.res(sa.OpFAdd, f32, comps[0], k)
    m.op(sa.OpStore, out_col, m.res(sa.OpCompositeConstruct, v4, *comps))
    sa._end_main(m)
    m.entry(sa.ExecVertex, fn, "main", [pv, in_pos, in_col, in_off, inst, out_col])
    return m.to_words()


@pytest.mark.gpu
@pytest.mark.parametrize("indirect", [False, True])
def test_instanced_draw_with_per_instance_attribute(renderer, indirect):
    """3 instances from firstInstance 1 of the 2,048-triangle soup: each instance moved by its own offset
    (a per-instance vertex attribute) and tinted by gl_InstanceIndex; the oracle draws the instances one
    after another (instance-major primitive order) with the same arithmetic done in float32"""
    base = small_cases()["soup"]
    offs = np.array([[9, 9, 9, 0], [0.05, -0.1, 0.02, 0.0], [-0.125, 0.0625, -0.05, 0.0], [0.2, 0.15, 0.1, 0.0]],
                    dtype=np.float32)
    first, count = 1, 3
    run = render.SceneRun(renderer, base, mode="batched", tile=16)
    _, fs = base.shaders()
    run.pipe = renderer.pipeline(base, run.rp, run.layout, _instanced_vs(), fs,
                                 instance_attr=(2, vk.FORMAT_R32G32B32A32_SFLOAT, 16))
    ibuf = renderer.create_buffer(offs.nbytes, vk.BUFFER_USAGE_VERTEX, True)
    renderer.write_buffer(ibuf, offs)
    cmd = renderer.create_buffer(16, vk.BUFFER_USAGE_INDIRECT, True)
    renderer.write_buffer(cmd, np.array([3 * base.draws[0].count, count, 0, first], dtype=np.uint32))

    def body(d, cb):
        d.vkCmdBindVertexBuffers(cb, 1, 1, (c_void_p * 1)(ibuf.handle.value), (c_uint64 * 1)(0))
        if indirect:
            d.vkCmdDrawIndirect(cb, cmd.handle, 0, 1, 16)
        else:
            d.vkCmdDraw(cb, 3 * base.draws[0].count, count, 0, first)
        # one instance past the instance buffer's 4 entries: skipped
        d.vkCmdDraw(cb, 3, 1, 0, 4)

    color, depth, st = _submit(run, _record(run, body))
    verts = []
    for i in range(first, first + count):
        v = base.vertices.copy()
        v[:, 0:4] = v[:, 0:4] + offs[i]
        v[:, 4] = v[:, 4] + np.float32(i * 0.125)
        verts.append(v)
    nt = base.draws[0].count
    scene = dataclasses.replace(base, vertices=np.concatenate(verts),
                                draws=[scenes.Draw(3 * nt * k, nt) for k in range(count)])
    ref_c, ref_d, ost = kz_oracle.render(scene, threads=8)
    assert np.array_equal(color, ref_c)
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
    assert st.fragments == ost["fragments"]
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_framebuffer_larger_than_its_attachments_is_a_recording_error(renderer):
    scene = small_cases()["soup"]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    fb = renderer.framebuffer(run.rp, [run.color.view, run.depth.view], scene.width + 16, scene.height)
    d = renderer.drv
    cb = renderer.begin()
    clears = (vk.VkClearValue * 2)()
    rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, run.rp, fb,
                                   vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(scene.width + 16, scene.height)),
                                   2, clears)
    d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
    d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, run.pipe)
    d.vkCmdDraw(cb, 3, 1, 0, 0)
    d.vkCmdEndRenderPass(cb)
    assert d.vkEndCommandBuffer(cb) == vk.VK_ERROR_INITIALIZATION_FAILED
    renderer.free_command_buffer(cb)
    renderer.free_command_buffer(run.cb)


@pytest.mark.gpu
def test_buffers_without_memory(renderer):
    """a vertex buffer with no memory bound fetches nothing (its draw is skipped: the pass only clears), and
    a fill of such a buffer is a recording error"""
    scene = small_cases()["soup"]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    d = renderer.drv
    bci = vk.VkBufferCreateInfo(vk.ST_BUFFER_CREATE_INFO, None, 0, scene.vertices.nbytes,
                                vk.BUFFER_USAGE_VERTEX | vk.BUFFER_USAGE_TRANSFER_DST, 0, 0, None)
    h = c_void_p()
    vk.check("vkCreateBuffer", d.vkCreateBuffer(renderer.device, byref(bci), None, byref(h)))
    try:
        unbound = render.Buffer(h, None, scene.vertices.nbytes, False)
        run.vb = unbound
        color, depth, st = _submit(run, _record(run, lambda d, cb: _draw(d, cb, run, scene.draws[0])))
        ref_c, ref_d = kz_oracle.clear_images(scene)
        assert np.array_equal(color, ref_c) and np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))
        assert st.fragments == 0
        cb = renderer.begin()
        d.vkCmdFillBuffer(cb, h, 0, 64, 0)
        assert d.vkEndCommandBuffer(cb) == vk.VK_ERROR_INITIALIZATION_FAILED
        renderer.free_command_buffer(cb)
    finally:
        d.vkDestroyBuffer(renderer.device, h, None)
    renderer.free_command_buffer(run.cb)

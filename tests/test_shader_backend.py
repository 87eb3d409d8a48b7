"""Shader path on the CPU: SPIR-V decoding against the reference's golden dumps, translation of the
workload shaders (interface masks), PTX emission and nvJitLink linking with the pipeline kernels."""
import os

import numpy as np
import pytest

from kazan_gb300 import shader, spirv_asm

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "spirv")


@pytest.mark.parametrize("name", ["test", "test2", "test3"])
def test_disassembly_matches_reference_golden(built, name):
    """spirv-parser/src/lib.rs parse_test / parse_test2 / parse_test3: byte-identical dump text"""
    words = np.fromfile(os.path.join(GOLDEN, name + ".spv"), dtype="<u4")
    with open(os.path.join(GOLDEN, name + ".dis"), encoding="utf-8") as f:
        expected = f.read()
    assert shader.disassemble(words) == expected


def test_invalid_module_is_rejected(built):
    with pytest.raises(shader.ShaderError):
        shader.disassemble(np.array([0xDEADBEEF, 0, 0, 0, 0], dtype=np.uint32))
    with pytest.raises(shader.ShaderError):
        shader.Shader(np.array([0x07230203, 0x10000, 0, 1, 0], dtype=np.uint32), shader.VERTEX)


def test_reference_vertex_fixture_translates(built):
    """test.spv is the reference's vertex shader fixture (gl_Position = vec4(in.xyz, 1) with an OpSwitch);
    the reference translator cannot load it (its simple_test is #[ignore]d)"""
    words = np.fromfile(os.path.join(GOLDEN, "test.spv"), dtype="<u4")
    info = shader.Shader(words, shader.VERTEX).info()
    assert info["writes_position"] == 1
    assert info["input_locations"] == 1 and info["pos_input_locations"] == 1


def test_workload_shader_interfaces(built):
    cvs = shader.Shader(spirv_asm.color_vs(), shader.VERTEX).info()
    assert cvs["input_locations"] == 0b11 and cvs["pos_input_locations"] == 0b1
    assert cvs["output_slots"] == 0xF and cvs["writes_position"]
    cfs = shader.Shader(spirv_asm.color_fs(), shader.FRAGMENT).info()
    assert cfs["input_slots"] == 0xF and cfs["writes_color"] and not cfs["discards"]
    lvs = shader.Shader(spirv_asm.lambert_vs(), shader.VERTEX).info()
    assert lvs["input_locations"] == 0b11 and lvs["pos_input_locations"] == 0b1
    assert lvs["output_slots"] == 0x7 and lvs["push_bytes"] == 64
    lfs = shader.Shader(spirv_asm.lambert_fs(), shader.FRAGMENT).info()
    assert lfs["input_slots"] == 0x7 and lfs["writes_color"]
    tfs = shader.Shader(spirv_asm.threshold_fs(), shader.FRAGMENT).info()
    assert tfs["discards"] == 1
    # only the colour shader is a pure copy of varyings 0..3 to the colour (the kernels skip its call)
    assert cfs["color_passthrough"] == 1
    assert lfs["color_passthrough"] == 0 and tfs["color_passthrough"] == 0 and cvs["color_passthrough"] == 0


def test_wrong_stage_entry_point_is_rejected(built):
    with pytest.raises(shader.ShaderError, match="entry point"):
        shader.Shader(spirv_asm.color_fs(), shader.VERTEX)


def _layouts():
    color = shader.layout([(0, 0, 4, 0), (1, 0, 4, 16)], [32])
    lam = shader.layout([(0, 0, 3, 0), (1, 0, 3, 12)], [24])
    return color, lam


def test_ptx_rounding_is_explicit(built):
    vs = shader.Shader(spirv_asm.lambert_vs(), shader.VERTEX)
    fs = shader.Shader(spirv_asm.lambert_fs(), shader.FRAGMENT)
    ptx = shader.emit_ptx([(vs, fs)], [_layouts()[1]])
    assert ".visible .func" in ptx and "kz_vs_pos" in ptx and "kz_fs" in ptx
    # every float op carries its rounding mode, so ptxas cannot contract or approximate them
    for op in ("add.f32", "mul.f32", "fma.f32", "div.f32", "sqrt.f32", "div.approx", "sqrt.approx"):
        assert op not in ptx
    assert "fma.rn.f32" in ptx and "sqrt.rn.f32" in ptx and "div.rn.f32" in ptx


def test_link_pipeline_set(built):
    """two pipelines in one set: PTX assembles and links with the relocatable kernel object"""
    cvs, cfs = shader.Shader(spirv_asm.color_vs(), 0), shader.Shader(spirv_asm.color_fs(), 4)
    lvs, lfs = shader.Shader(spirv_asm.lambert_vs(), 0), shader.Shader(spirv_asm.lambert_fs(), 4)
    tfs = shader.Shader(spirv_asm.threshold_fs(), 4)
    ptx = shader.emit_ptx([(cvs, cfs), (lvs, lfs), (cvs, tfs), (cvs, None)], list(_layouts()) + list(_layouts()))
    img = shader.link(ptx)
    assert len(img) > 100_000 and img[:4] == b"\x7fELF"


def _heavy_vs():
    """a vertex shader with many live values: two push-constant matrices and a chain of products"""
    from kazan_gb300.spirv_asm import (Module, CapShader, DecOffset, DecColMajor, DecMatrixStride, DecBlock,
                                       SCPushConstant, SCInput, SCOutput, OpAccessChain, OpLoad, OpStore,
                                       OpMatrixTimesVector, OpFAdd, OpFMul, ExecVertex, _per_vertex, _io,
                                       _begin_main, _end_main)
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v4 = m.vec(f32, 4)
    m4 = m.mat(v4, 4)
    blk = m.struct(m4, m4)
    for i in range(2):
        m.member_decorate(blk, i, DecOffset, 64 * i)
        m.member_decorate(blk, i, DecColMajor)
        m.member_decorate(blk, i, DecMatrixStride, 16)
    m.decorate(blk, DecBlock)
    pc = m.variable(SCPushConstant, m.ptr(SCPushConstant, blk))
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v4, 0)
    in_col = _io(m, SCInput, v4, 1)
    out_col = _io(m, SCOutput, v4, 0)
    fn = _begin_main(m)
    a = m.res(OpLoad, m4, m.res(OpAccessChain, m.ptr(SCPushConstant, m4), pc, m.ci(0)))
    b = m.res(OpLoad, m4, m.res(OpAccessChain, m.ptr(SCPushConstant, m4), pc, m.ci(1)))
    p = m.res(OpLoad, v4, in_pos)
    q = [m.res(OpMatrixTimesVector, v4, a, p), m.res(OpMatrixTimesVector, v4, b, p)]
    for i in range(6):
        q.append(m.res(OpMatrixTimesVector, v4, a if i % 2 else b, m.res(OpFAdd, v4, q[-1], q[-2])))
    acc = q[0]
    for v in q[1:]:
        acc = m.res(OpFMul, v4, acc, v)
    m.op(OpStore, m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0)), acc)
    m.op(OpStore, out_col, m.res(OpLoad, v4, in_col))
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [pc, pv, in_pos, in_col, out_col])
    return m.to_words()


def test_register_heavy_shader_links(built):
    """shader functions are compiled within the kernels' 64-register limit, so a heavy vertex shader (whose
    three-vertex function would need more) still links, spilling instead of failing"""
    vs = shader.Shader(_heavy_vs(), shader.VERTEX)
    fs = shader.Shader(spirv_asm.color_fs(), shader.FRAGMENT)
    img = shader.link(shader.emit_ptx([(vs, fs)], [_layouts()[0]]))
    assert img[:4] == b"\x7fELF"


def test_function_calls_are_inlined(built):
    """helper functions (value and pointer parameters, returns from two branches, four call sites of the same
    function) translate, keep the interfaces of the call-free shaders and link"""
    import call_shaders
    fs = shader.Shader(call_shaders.color_fs_calls(), shader.FRAGMENT)
    vs = shader.Shader(call_shaders.lambert_vs_calls(), shader.VERTEX)
    fi, vi = fs.info(), vs.info()
    assert fi["input_slots"] == 0xF and fi["writes_color"] and not fi["discards"]
    assert vi["input_locations"] == 0b11 and vi["pos_input_locations"] == 0b1 and vi["push_bytes"] == 64
    img = shader.link(shader.emit_ptx([(vs, fs)], [_layouts()[1]]))
    assert img[:4] == b"\x7fELF"


def test_run_time_indices_translate(built):
    """loops with run-time indices into a local array and into vectors translate and link"""
    import call_shaders
    fs = shader.Shader(call_shaders.color_fs_loops(), shader.FRAGMENT)
    assert fs.info()["input_slots"] == 0xF and fs.info()["writes_color"]
    vs = shader.Shader(spirv_asm.color_vs(), shader.VERTEX)
    img = shader.link(shader.emit_ptx([(vs, fs)], [_layouts()[0]]))
    assert img[:4] == b"\x7fELF"


def test_descriptor_bindings_translate_and_link(built):
    """a uniform block in the vertex shader and combined image samplers in the fragment shader: the stages
    report their bindings, the PTX reads the block through the draw's descriptor slot and calls the
    sampling function of the pipeline-kernel object, and the set links"""
    uvs = shader.Shader(spirv_asm.lambert_ubo_vs(0, 0), shader.VERTEX)
    assert uvs.bindings() == [(0, 0, 0, 1, 64)]
    tvs = shader.Shader(spirv_asm.textured_vs(), shader.VERTEX)
    tfs = shader.Shader(spirv_asm.textured_fs(1, 3), shader.FRAGMENT)
    assert tfs.bindings() == [(1, 3, 1, 1, 0)]
    afs = shader.Shader(spirv_asm.textured_array_fs(2, 0, 2), shader.FRAGMENT)
    assert afs.bindings() == [(0, 2, 1, 2, 0)]
    efs = shader.Shader(spirv_asm.textured_fs(explicit_lod=True), shader.FRAGMENT)
    lam = shader.layout([(0, 0, 3, 0), (1, 0, 3, 12)], [24])
    tex = shader.layout([(0, 0, 4, 0), (1, 0, 2, 16)], [24])
    slots = [{(0, 0): 0}, {(1, 3): 5}, {(0, 2): 1}, {(0, 0): 0}]
    ptx = shader.emit_ptx([(uvs, shader.Shader(spirv_asm.lambert_fs(), 4)), (tvs, tfs), (tvs, afs), (tvs, efs)],
                          [lam, tex, tex, tex], slots)
    # the block's address from slot 0 (byte 128 of the snapshot), texture descriptor 5 at 128 + 32 * 5
    assert "[%kzpush+128]" in ptx
    assert "add.s64 %kzd, %kzpg, 288;" in ptx
    assert "call (kzt_r), kz_tex2d" in ptx and ".extern .func" in ptx
    # the run-time array index scales by the descriptor size
    assert "mul.wide.u32 %kzoff" in ptx
    img = shader.link(ptx)
    assert img[:4] == b"\x7fELF"


def test_storage_buffer_translates_read_only(built):
    """a storage block with a runtime-sized array: binding kind 2 whose range must cover the block with one
    element (16 + 8 bytes); the PTX limits the index by the descriptor's range (byte 8 of its slot); a
    store into the block is refused"""
    import shader_ops
    fs = shader.Shader(shader_ops.storage_fs(), shader.FRAGMENT)
    assert fs.bindings() == [(0, 0, 2, 1, 24)]
    ptx = shader.emit_ptx([(shader.Shader(spirv_asm.color_vs(), shader.VERTEX), fs)],
                          [shader.layout([(0, 0, 4, 0), (1, 0, 4, 16)], [32])], [{(0, 0): 3}])
    assert "[%kzpush+232]" in ptx  # 128 + 32 * 3 + 8: the range of descriptor slot 3
    assert "div.u32" in ptx
    shader.link(ptx)
    with pytest.raises(shader.ShaderError, match="storage buffers"):
        shader.Shader(shader_ops.storage_fs(store=True), shader.FRAGMENT)


def test_separate_image_and_sampler_translate(built):
    """a texture2D and a sampler combined by OpSampledImage: bindings of kind 3 (sampled image) and 4
    (sampler); the PTX copies the image descriptor to local memory with the sampler's state word (byte 28 of
    the sampler's slot) and samples through the copy"""
    fs = shader.Shader(spirv_asm.textured_separate_fs(0, 2, 5), shader.FRAGMENT)
    assert sorted(fs.bindings()) == [(0, 2, 3, 1, 0), (0, 5, 4, 1, 0)]
    tex = shader.layout([(0, 0, 4, 0), (1, 0, 2, 16)], [24])
    ptx = shader.emit_ptx([(shader.Shader(spirv_asm.textured_vs(), shader.VERTEX), fs)], [tex],
                          [{(0, 2): 0, (0, 5): 1}])
    assert "[%kzpush+188]" in ptx  # 128 + 32 * 1 + 28
    assert "st.local.v4.u32 [kzsd+16]" in ptx and "cvta.local.u64 %kzd" in ptx
    shader.link(ptx)


def test_unsupported_descriptor_forms_are_rejected(built):
    """unsupported image forms are reported, not mistranslated"""
    from kazan_gb300.spirv_asm import (Module, CapShader, SCUniformConstant, OpTypeImage, ExecFragment,
                                       ModeOriginUpperLeft, DecDescriptorSet, DecBinding, _begin_main, _end_main,
                                       _io, SCOutput)
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    img = m._type(("image3d",), OpTypeImage, f32, 2, 0, 0, 0, 1, 0)  # Dim 3D
    var = m.variable(SCUniformConstant, m.ptr(SCUniformConstant, img))
    m.decorate(var, DecDescriptorSet, 0)
    m.decorate(var, DecBinding, 0)
    o = _io(m, SCOutput, m.vec(f32, 4), 0)
    fn = _begin_main(m)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [var, o])
    m.mode(fn, ModeOriginUpperLeft)
    with pytest.raises(shader.ShaderError, match="only 2D images"):
        shader.Shader(m.to_words(), shader.FRAGMENT)

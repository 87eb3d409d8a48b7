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

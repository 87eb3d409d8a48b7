"""Test fragment shaders that evaluate one SPIR-V operation on a flat vec4 input `a` (location 0) and write the
32-bit result's bytes as the colour (byte k / 255 in component k, which the UNORM8 store turns back into byte k),
so a render returns the exact result bits of every pixel; and the cell-grid scene that feeds each 8x8 cell
its own input vector."""
import struct
from fractions import Fraction

import numpy as np

from kazan_gb300 import scenes, spirv_asm as sa

# opcodes and GLSL.std.450 numbers (SPIR-V specification) beyond those spirv_asm names
OpConvertUToF = 112
OpShiftRightLogical = 194
OpSMod, OpFRem, OpFMod = 139, 140, 141
OpAny, OpAll, OpIsInf = 154, 155, 157
OpBitFieldInsert, OpBitFieldSExtract, OpBitFieldUExtract, OpBitReverse, OpBitCount = 201, 202, 203, 204, 205
G = dict(SAbs=5, FSign=6, SSign=7, Radians=11, Degrees=12, Tan=15, Asin=16, Acos=17, Atan=18, Sinh=19, Cosh=20,
         Tanh=21, Asinh=22, Acosh=23, Atanh=24, Atan2=25, Exp=27, Log=28, Determinant=33, MatrixInverse=34,
         UClamp=44, SClamp=45, SmoothStep=49, Ldexp=53, PackSnorm4x8=54, PackUnorm4x8=55, PackHalf2x16=58,
         UnpackHalf2x16=62, UnpackSnorm4x8=63, UnpackUnorm4x8=64, FaceForward=70, Reflect=71, Refract=72,
         FindILsb=73, FindSMsb=74, FindUMsb=75)

CELL, GRID = 8, 16  # 8x8-pixel cells, 16x16 of them: 256 inputs per render


class Ctx:
    """ids of the common types and of the input components while a shader body is being built"""

    def __init__(self, m, glsl, a):
        self.m, self.glsl, self.a = m, glsl, a
        self.f32, self.u32, self.i32 = m.f32(), m.i32(0), m.i32(1)
        self.v2, self.v4 = m.vec(self.f32, 2), m.vec(self.f32, 4)
        self.x, self.y, self.z, self.w = [m.res(sa.OpCompositeExtract, self.f32, a, k) for k in range(4)]

    def ext(self, rt, name, *args):
        return self.m.res(sa.OpExtInst, rt, self.glsl, G[name], *args)

    def bits(self, f):
        """float -> uint bits"""
        return self.m.res(sa.OpBitcast, self.u32, f)

    def to_int(self, f):
        return self.m.res(sa.OpConvertFToS, self.i32, f)

    def vec2(self, p, q):
        return self.m.res(sa.OpCompositeConstruct, self.v2, p, q)


def op_fs(body):
    """fragment shader: r = body(ctx) -> (id, "f32" | "i32" | "u32"); colour = the bytes of r's 32 bits"""
    m = sa.Module()
    m.capability(sa.CapShader)
    glsl = m.ext_import("GLSL.std.450")
    f32 = m.f32()
    v4 = m.vec(f32, 4)
    u32 = m.i32(0)
    v_a = sa._io(m, sa.SCInput, v4, 0, flat=True)
    o = sa._io(m, sa.SCOutput, v4, 0)
    c255 = m.cf(255.0)
    fn = sa._begin_main(m)
    a = m.res(sa.OpLoad, v4, v_a)
    ctx = Ctx(m, glsl, a)
    r, kind = body(ctx)
    u = r if kind == "u32" else m.res(sa.OpBitcast, u32, r)
    comps = []
    for k in range(4):
        b = m.res(OpShiftRightLogical, u32, u, m.ci(8 * k, 0))
        b = m.res(sa.OpBitwiseAnd, u32, b, m.ci(0xFF, 0))
        comps.append(m.res(sa.OpFDiv, f32, m.res(OpConvertUToF, f32, b), c255))
    m.op(sa.OpStore, o, m.res(sa.OpCompositeConstruct, v4, *comps))
    sa._end_main(m)
    m.entry(sa.ExecFragment, fn, "main", [v_a, o])
    m.mode(fn, sa.ModeOriginUpperLeft)
    return m.to_words()


def cell_scene(inputs, fs_words):
    """GRID x GRID cells of CELL x CELL pixels, cell i drawn as two triangles whose colour attribute (the flat
    input of the fragment shader) is inputs[i] (float32 [n <= 256, 4])"""
    size = CELL * GRID
    rows = []
    for i, v in enumerate(np.asarray(inputs, dtype=np.float32)):
        cx, cy = i % GRID, i // GRID
        x0, y0 = 2.0 * cx * CELL / size - 1.0, 2.0 * cy * CELL / size - 1.0
        x1, y1 = x0 + 2.0 * CELL / size, y0 + 2.0 * CELL / size
        for (px, py) in ((x0, y0), (x1, y0), (x0, y1), (x1, y0), (x1, y1), (x0, y1)):
            rows.append([px, py, 0.5, 1.0] + list(v))
    s = scenes.Scene("ops", size, size, "color", np.array(rows, dtype=np.float32), None,
                     [scenes.Draw(0, len(rows) // 3)], cull=0)
    s.fs_words = fs_words
    return s


def read_bits(color, n):
    """the 32-bit result of each of the first n cells, from the pixel at the cell's centre"""
    out = np.empty(n, dtype=np.uint32)
    for i in range(n):
        cx, cy = i % GRID, i // GRID
        px = color[cy * CELL + CELL // 2, cx * CELL + CELL // 2].astype(np.uint32)
        out[i] = px[0] | (px[1] << 8) | (px[2] << 16) | (px[3] << 24)
    return out


# ---- exact float32 restatements ----

def f32(x):
    return np.float32(x)


def bits(x):
    return struct.unpack("<I", struct.pack("<f", float(np.float32(x))))[0]


def round_f32(q):
    """the float32 nearest to the exact rational q (ties to even)"""
    c = np.float32(float(q))
    cands = [c, np.nextafter(c, np.float32(np.inf)), np.nextafter(c, np.float32(-np.inf))]
    best = min(cands, key=lambda v: (abs(Fraction(float(v)) - q), bits(v) & 1))
    return np.float32(best)


def fma(a, b, c):
    """fused multiply-add in float32, rounded once"""
    a, b, c = f32(a), f32(b), f32(c)
    if not (np.isfinite(a) and np.isfinite(b) and np.isfinite(c)):
        return f32(np.float64(a) * np.float64(b) + np.float64(c))
    return round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


# ---- a read-only storage buffer (set 0, binding 0) with a runtime-sized array ----
OpConvertFToU, OpBitwiseXor, OpTypeRuntimeArray = 109, 198, 29
DecBufferBlock, DecArrayStride = 3, 6
SSBO_BASE, SSBO_STRIDE = 16, 8  # block { uint bias; uint pad[3]; uvec2 vals[]; } in std430


def storage_fs(store=False):
    """fragment shader reading b.vals[uint(a.x)].y ^ b.bias from the storage block
    `layout(set = 0, binding = 0) buffer B { uint bias; uint pad[3]; uvec2 vals[]; } b` (Uniform storage
    class with BufferBlock); `store`: also writes b.bias (which translation must refuse)"""

    def body(c):
        m = c.m
        uv2 = m.vec(c.u32, 2)
        rt = m._type(("rtarr", uv2), OpTypeRuntimeArray, uv2)
        m.decorate(rt, DecArrayStride, SSBO_STRIDE)
        pad = m.array(c.u32, 3)
        m.decorate(pad, DecArrayStride, 4)
        blk = m.struct(c.u32, pad, rt)
        for k, off in enumerate((0, 4, SSBO_BASE)):
            m.member_decorate(blk, k, sa.DecOffset, off)
        m.decorate(blk, DecBufferBlock)
        var = m.variable(sa.SCUniform, m.ptr(sa.SCUniform, blk))
        m.decorate(var, sa.DecDescriptorSet, 0)
        m.decorate(var, sa.DecBinding, 0)
        pu = m.ptr(sa.SCUniform, c.u32)
        idx = m.res(OpConvertFToU, c.u32, c.x)
        v = m.res(sa.OpLoad, c.u32, m.res(sa.OpAccessChain, pu, var, m.ci(2), idx, m.ci(1)))
        bias_p = m.res(sa.OpAccessChain, pu, var, m.ci(0))
        if store:
            m.op(sa.OpStore, bias_p, v)
        return m.res(OpBitwiseXor, c.u32, v, m.res(sa.OpLoad, c.u32, bias_p)), "u32"

    return op_fs(body)

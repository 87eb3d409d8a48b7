"""SPIR-V binary encoder and the shaders of the draw-path workloads.

No glslang or SPIRV-Tools exist in this environment, so shaders are assembled directly from the
SPIR-V specification's binary form (header, then instructions whose first word is
word_count << 16 | opcode).  The reference's own SPIR-V fixtures are hand-checked binaries too
(spirv-parser/test_inputs/*.spv).

The workload shaders:
  * color_vs / color_fs    pass-through: gl_Position = in0 (vec4), out0 = in1 (vec4); fragment
                           colour = interpolated out0
  * lambert_vs / lambert_fs  gl_Position = mvp * vec4(in0.xyz, 1) with mvp a column-major mat4 push
                           constant; out0 = in1.xyz (normal); fragment colour
                           = vec4(ALBEDO * max(dot(normalize(n), LIGHT), 0), 1)
  * lambert_ubo_vs         the same with mvp in a uniform buffer (set 0, binding 0)
  * textured_vs / textured_fs  gl_Position = in0 (vec4), out0 = in1 (vec2 uv); fragment colour
                           = texture(sampler2D at set 0 binding 0, uv)
"""
import struct

import numpy as np

# opcodes (SPIR-V specification, "Instructions")
OpExtInstImport = 11
OpExtInst = 12
OpMemoryModel = 14
OpEntryPoint = 15
OpExecutionMode = 16
OpCapability = 17
OpTypeVoid = 19
OpTypeBool = 20
OpTypeInt = 21
OpTypeFloat = 22
OpTypeVector = 23
OpTypeMatrix = 24
OpTypeImage = 25
OpTypeSampler = 26
OpTypeSampledImage = 27
OpTypeArray = 28
OpTypeStruct = 30
OpTypePointer = 32
OpTypeFunction = 33
OpConstantTrue = 41
OpConstantFalse = 42
OpConstant = 43
OpConstantComposite = 44
OpSpecConstant = 50
OpFunction = 54
OpFunctionEnd = 56
OpFunctionParameter = 55
OpFunctionCall = 57
OpVariable = 59
OpLoad = 61
OpStore = 62
OpAccessChain = 65
OpDecorate = 71
OpMemberDecorate = 72
OpImageSampleImplicitLod = 87
OpImageSampleExplicitLod = 88
OpImageSampleProjImplicitLod = 91
OpImageFetch = 95
OpImage = 100
OpSampledImage = 86
OpVectorExtractDynamic = 77
OpVectorInsertDynamic = 78
OpVectorShuffle = 79
OpCompositeConstruct = 80
OpCompositeExtract = 81
OpConvertFToS = 110
OpConvertSToF = 111
OpBitcast = 124
OpFNegate = 127
OpIAdd = 128
OpFAdd = 129
OpISub = 130
OpFSub = 131
OpIMul = 132
OpFMul = 133
OpFDiv = 136
OpVectorTimesScalar = 142
OpMatrixTimesVector = 145
OpDot = 148
OpSelect = 169
OpIEqual = 170
OpFOrdLessThan = 184
OpFOrdGreaterThan = 186
OpBitwiseAnd = 199
OpPhi = 245
OpSLessThan = 177
OpLoopMerge = 246
OpSelectionMerge = 247
OpLabel = 248
OpBranch = 249
OpBranchConditional = 250
OpKill = 252
OpReturn = 253
OpReturnValue = 254

# enumerants
CapShader = 1
AddressingLogical = 0
MemoryGLSL450 = 1
ExecVertex = 0
ExecFragment = 4
ModeOriginUpperLeft = 7
SCUniformConstant = 0
SCInput = 1
SCUniform = 2
SCOutput = 3
SCPushConstant = 9
SCFunction = 7
DecSpecId = 1
DecBlock = 2
DecColMajor = 5
DecMatrixStride = 7
DecBuiltIn = 11
DecNoPerspective = 13
DecFlat = 14
DecLocation = 30
DecBinding = 33
DecDescriptorSet = 34
ImageOperandsLod = 0x2
DecOffset = 35
BuiltInPosition = 0
BuiltInFragCoord = 15
BuiltInFrontFacing = 17
BuiltInVertexIndex = 42
BuiltInInstanceIndex = 43
GLSLNormalize = 69
GLSLFMax = 40
GLSLFMin = 37
GLSLFloor = 8
GLSLSqrt = 31

# fragment-shader constants of the Lambert workload (float32 values used verbatim by the oracle)
ALBEDO = np.array([0.8, 0.7, 0.6], dtype=np.float32)
_l = np.array([0.3, 0.5, 0.8], dtype=np.float64)
LIGHT = (_l / np.linalg.norm(_l)).astype(np.float32)


def _string_words(s):
    b = s.encode("utf-8") + b"\0"
    b += b"\0" * ((4 - len(b) % 4) % 4)
    return list(struct.unpack("<%dI" % (len(b) // 4), b))


def f32_bits(v):
    return struct.unpack("<I", struct.pack("<f", float(np.float32(v))))[0]


class Module:
    """Builds one SPIR-V module.  Results are ids; operands are ints (ids or literals) or strings."""

    def __init__(self):
        self.bound = 1
        self.caps, self.exts, self.memmodel, self.entries, self.modes = [], [], [], [], []
        self.names, self.annotations, self.globals, self.functions = [], [], [], []
        self._types = {}
        self._consts = {}

    def new_id(self):
        i = self.bound
        self.bound += 1
        return i

    @staticmethod
    def _ins(section, opcode, operands):
        words = []
        for o in operands:
            if isinstance(o, str):
                words += _string_words(o)
            else:
                words.append(int(o) & 0xFFFFFFFF)
        section.append([(len(words) + 1) << 16 | opcode] + words)

    def op(self, opcode, *operands):
        """function-body instruction"""
        self._ins(self.functions, opcode, operands)

    def res(self, opcode, type_id, *operands):
        """function-body instruction with a result; returns the result id"""
        r = self.new_id()
        self._ins(self.functions, opcode, (type_id, r) + operands)
        return r

    # ---- types (deduplicated) ----
    def _type(self, key, opcode, *operands):
        if key not in self._types:
            r = self.new_id()
            self._ins(self.globals, opcode, (r,) + operands)
            self._types[key] = r
        return self._types[key]

    def void(self):
        return self._type(("void",), OpTypeVoid)

    def bool(self):
        return self._type(("bool",), OpTypeBool)

    def f32(self):
        return self._type(("f32",), OpTypeFloat, 32)

    def i32(self, signed=1):
        return self._type(("i32", signed), OpTypeInt, 32, signed)

    def vec(self, comp, n):
        return self._type(("vec", comp, n), OpTypeVector, comp, n)

    def mat(self, col, n):
        return self._type(("mat", col, n), OpTypeMatrix, col, n)

    def ptr(self, storage, t):
        return self._type(("ptr", storage, t), OpTypePointer, storage, t)

    def fn_type(self, ret, *params):
        return self._type(("fn", ret) + params, OpTypeFunction, ret, *params)

    def array(self, elem, length):
        return self._type(("array", elem, length), OpTypeArray, elem, self.ci(length, 0))

    def struct(self, *members):
        r = self.new_id()
        self._ins(self.globals, OpTypeStruct, (r,) + members)
        return r

    # ---- constants ----
    def cf(self, v):
        bits = f32_bits(v)
        key = ("f", bits)
        if key not in self._consts:
            r = self.new_id()
            self._ins(self.globals, OpConstant, (self.f32(), r, bits))
            self._consts[key] = r
        return self._consts[key]

    def ci(self, v, signed=1):
        key = ("i", signed, int(v) & 0xFFFFFFFF)
        if key not in self._consts:
            r = self.new_id()
            self._ins(self.globals, OpConstant, (self.i32(signed), r, int(v) & 0xFFFFFFFF))
            self._consts[key] = r
        return self._consts[key]

    def cvec(self, values):
        comps = [self.cf(v) for v in values]
        r = self.new_id()
        self._ins(self.globals, OpConstantComposite, (self.vec(self.f32(), len(values)), r) + tuple(comps))
        return r

    def spec_f(self, spec_id, default):
        r = self.new_id()
        self._ins(self.globals, OpSpecConstant, (self.f32(), r, f32_bits(default)))
        self.decorate(r, DecSpecId, spec_id)
        return r

    # ---- module-level ----
    def capability(self, c):
        self._ins(self.caps, OpCapability, (c,))

    def ext_import(self, name):
        r = self.new_id()
        self._ins(self.exts, OpExtInstImport, (r, name))
        return r

    def decorate(self, target, dec, *lits):
        self._ins(self.annotations, OpDecorate, (target, dec) + lits)

    def member_decorate(self, target, member, dec, *lits):
        self._ins(self.annotations, OpMemberDecorate, (target, member, dec) + lits)

    def variable(self, storage, ptr_type):
        r = self.new_id()
        self._ins(self.globals, OpVariable, (ptr_type, r, storage))
        return r

    def entry(self, model, fn, name, interface):
        self._ins(self.entries, OpEntryPoint, (model, fn, name) + tuple(interface))

    def mode(self, fn, mode, *lits):
        self._ins(self.modes, OpExecutionMode, (fn, mode) + lits)

    def to_words(self):
        self._ins(self.memmodel, OpMemoryModel, (AddressingLogical, MemoryGLSL450))
        words = [0x07230203, 0x00010000, 0, self.bound, 0]
        for section in (self.caps, self.exts, self.memmodel, self.entries, self.modes, self.names,
                        self.annotations, self.globals, self.functions):
            for ins in section:
                words += ins
        return np.array(words, dtype=np.uint32)


def _begin_main(m):
    void = m.void()
    fn = m.new_id()
    m._ins(m.functions, OpFunction, (void, fn, 0, m.fn_type(void)))
    m.op(OpLabel, m.new_id())
    return fn


def _end_main(m):
    m.op(OpReturn)
    m._ins(m.functions, OpFunctionEnd, ())


def begin_function(m, ret_type, param_types):
    """a helper function: returns (function id, parameter ids); its first block is open"""
    fn = m.new_id()
    m._ins(m.functions, OpFunction, (ret_type, fn, 0, m.fn_type(ret_type, *param_types)))
    params = []
    for t in param_types:
        pid = m.new_id()
        m._ins(m.functions, OpFunctionParameter, (t, pid))
        params.append(pid)
    m.op(OpLabel, m.new_id())
    return fn, params


def end_function(m):
    m._ins(m.functions, OpFunctionEnd, ())


def _per_vertex(m):
    v4 = m.vec(m.f32(), 4)
    block = m.struct(v4)
    m.member_decorate(block, 0, DecBuiltIn, BuiltInPosition)
    m.decorate(block, DecBlock)
    var = m.variable(SCOutput, m.ptr(SCOutput, block))
    return var


def _io(m, storage, t, location, flat=False, noperspective=False):
    var = m.variable(storage, m.ptr(storage, t))
    m.decorate(var, DecLocation, location)
    if flat:
        m.decorate(var, DecFlat)
    if noperspective:
        m.decorate(var, DecNoPerspective)
    return var


def color_vs():
    """gl_Position = in0; out0 = in1 (both vec4)"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v4 = m.vec(f32, 4)
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v4, 0)
    in_col = _io(m, SCInput, v4, 1)
    out_col = _io(m, SCOutput, v4, 0)
    fn = _begin_main(m)
    p = m.res(OpLoad, v4, in_pos)
    dst = m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0))
    m.op(OpStore, dst, p)
    c = m.res(OpLoad, v4, in_col)
    m.op(OpStore, out_col, c)
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [pv, in_pos, in_col, out_col])
    return m.to_words()


def color_fs():
    """colour = interpolated in0"""
    m = Module()
    m.capability(CapShader)
    v4 = m.vec(m.f32(), 4)
    v_col = _io(m, SCInput, v4, 0)
    o = _io(m, SCOutput, v4, 0)
    fn = _begin_main(m)
    c = m.res(OpLoad, v4, v_col)
    m.op(OpStore, o, c)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [v_col, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def lambert_vs():
    """gl_Position = mvp * vec4(in0, 1); out0 = in1 (vec3 normal); mvp: push constant mat4 at offset 0"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v3, v4 = m.vec(f32, 3), m.vec(f32, 4)
    m4 = m.mat(v4, 4)
    pc_block = m.struct(m4)
    m.member_decorate(pc_block, 0, DecOffset, 0)
    m.member_decorate(pc_block, 0, DecColMajor)
    m.member_decorate(pc_block, 0, DecMatrixStride, 16)
    m.decorate(pc_block, DecBlock)
    pc = m.variable(SCPushConstant, m.ptr(SCPushConstant, pc_block))
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v3, 0)
    in_nrm = _io(m, SCInput, v3, 1)
    out_nrm = _io(m, SCOutput, v3, 0)
    one = m.cf(1.0)
    fn = _begin_main(m)
    mp = m.res(OpAccessChain, m.ptr(SCPushConstant, m4), pc, m.ci(0))
    mvp = m.res(OpLoad, m4, mp)
    p = m.res(OpLoad, v3, in_pos)
    x = m.res(OpCompositeExtract, f32, p, 0)
    y = m.res(OpCompositeExtract, f32, p, 1)
    z = m.res(OpCompositeExtract, f32, p, 2)
    p4 = m.res(OpCompositeConstruct, v4, x, y, z, one)
    clip = m.res(OpMatrixTimesVector, v4, mvp, p4)
    dst = m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0))
    m.op(OpStore, dst, clip)
    n = m.res(OpLoad, v3, in_nrm)
    m.op(OpStore, out_nrm, n)
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [pc, pv, in_pos, in_nrm, out_nrm])
    return m.to_words()


def lambert_ubo_vs(set_=0, binding=0):
    """lambert_vs with mvp read from a uniform block { mat4 mvp; } at (set_, binding)"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v3, v4 = m.vec(f32, 3), m.vec(f32, 4)
    m4 = m.mat(v4, 4)
    blk = m.struct(m4)
    m.member_decorate(blk, 0, DecOffset, 0)
    m.member_decorate(blk, 0, DecColMajor)
    m.member_decorate(blk, 0, DecMatrixStride, 16)
    m.decorate(blk, DecBlock)
    ubo = m.variable(SCUniform, m.ptr(SCUniform, blk))
    m.decorate(ubo, DecDescriptorSet, set_)
    m.decorate(ubo, DecBinding, binding)
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v3, 0)
    in_nrm = _io(m, SCInput, v3, 1)
    out_nrm = _io(m, SCOutput, v3, 0)
    one = m.cf(1.0)
    fn = _begin_main(m)
    mp = m.res(OpAccessChain, m.ptr(SCUniform, m4), ubo, m.ci(0))
    mvp = m.res(OpLoad, m4, mp)
    p = m.res(OpLoad, v3, in_pos)
    x = m.res(OpCompositeExtract, f32, p, 0)
    y = m.res(OpCompositeExtract, f32, p, 1)
    z = m.res(OpCompositeExtract, f32, p, 2)
    p4 = m.res(OpCompositeConstruct, v4, x, y, z, one)
    clip = m.res(OpMatrixTimesVector, v4, mvp, p4)
    dst = m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0))
    m.op(OpStore, dst, clip)
    n = m.res(OpLoad, v3, in_nrm)
    m.op(OpStore, out_nrm, n)
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [ubo, pv, in_pos, in_nrm, out_nrm])
    return m.to_words()


def textured_vs():
    """gl_Position = in0 (vec4); out0 = in1 (vec2 texture coordinates)"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v2, v4 = m.vec(f32, 2), m.vec(f32, 4)
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v4, 0)
    in_uv = _io(m, SCInput, v2, 1)
    out_uv = _io(m, SCOutput, v2, 0)
    fn = _begin_main(m)
    p = m.res(OpLoad, v4, in_pos)
    dst = m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0))
    m.op(OpStore, dst, p)
    uv = m.res(OpLoad, v2, in_uv)
    m.op(OpStore, out_uv, uv)
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [pv, in_pos, in_uv, out_uv])
    return m.to_words()


def _sampler2d(m, set_, binding, count=None):
    """a UniformConstant sampler2D variable (an array of `count` when given); returns (var, sampled image type)"""
    f32 = m.f32()
    img = m._type(("image2d",), OpTypeImage, f32, 1, 0, 0, 0, 1, 0)   # Dim 2D, sampled, Unknown format
    simg = m._type(("sampledimage", img), OpTypeSampledImage, img)
    t = simg if count is None else m.array(simg, count)
    var = m.variable(SCUniformConstant, m.ptr(SCUniformConstant, t))
    m.decorate(var, DecDescriptorSet, set_)
    m.decorate(var, DecBinding, binding)
    return var, simg


def textured_fs(set_=0, binding=0, explicit_lod=False):
    """colour = texture(tex, uv) (OpImageSampleImplicitLod; OpImageSampleExplicitLod with Lod 0 when
    `explicit_lod`)"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v2, v4 = m.vec(f32, 2), m.vec(f32, 4)
    tex, simg = _sampler2d(m, set_, binding)
    v_uv = _io(m, SCInput, v2, 0)
    o = _io(m, SCOutput, v4, 0)
    zero = m.cf(0.0)
    fn = _begin_main(m)
    si = m.res(OpLoad, simg, tex)
    uv = m.res(OpLoad, v2, v_uv)
    if explicit_lod:
        c = m.res(OpImageSampleExplicitLod, v4, si, uv, ImageOperandsLod, zero)
    else:
        c = m.res(OpImageSampleImplicitLod, v4, si, uv)
    m.op(OpStore, o, c)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [tex, v_uv, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def textured_separate_fs(set_=0, image_binding=0, sampler_binding=1):
    """colour = texture(sampler2D(tex, smp), uv): a separate texture2D and sampler (set `set_`, bindings
    `image_binding` and `sampler_binding`) combined by OpSampledImage"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v2, v4 = m.vec(f32, 2), m.vec(f32, 4)
    img = m._type(("image2d",), OpTypeImage, f32, 1, 0, 0, 0, 1, 0)
    smp_t = m._type(("sampler",), OpTypeSampler)
    simg = m._type(("sampledimage", img), OpTypeSampledImage, img)
    tex = m.variable(SCUniformConstant, m.ptr(SCUniformConstant, img))
    m.decorate(tex, DecDescriptorSet, set_)
    m.decorate(tex, DecBinding, image_binding)
    smp = m.variable(SCUniformConstant, m.ptr(SCUniformConstant, smp_t))
    m.decorate(smp, DecDescriptorSet, set_)
    m.decorate(smp, DecBinding, sampler_binding)
    v_uv = _io(m, SCInput, v2, 0)
    o = _io(m, SCOutput, v4, 0)
    fn = _begin_main(m)
    si = m.res(OpSampledImage, simg, m.res(OpLoad, img, tex), m.res(OpLoad, smp_t, smp))
    c = m.res(OpImageSampleImplicitLod, v4, si, m.res(OpLoad, v2, v_uv))
    m.op(OpStore, o, c)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [tex, smp, v_uv, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def textured_array_fs(count=2, set_=0, binding=0):
    """colour = texture(tex[i], uv) with i = 1 where uv.x >= 0.5, else 0: a run-time index into an array of
    combined image samplers"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    i32 = m.i32()
    v2, v4 = m.vec(f32, 2), m.vec(f32, 4)
    tex, simg = _sampler2d(m, set_, binding, count)
    v_uv = _io(m, SCInput, v2, 0)
    o = _io(m, SCOutput, v4, 0)
    half = m.cf(0.5)
    fn = _begin_main(m)
    uv = m.res(OpLoad, v2, v_uv)
    u = m.res(OpCompositeExtract, f32, uv, 0)
    lt = m.res(OpFOrdLessThan, m.bool(), u, half)
    idx = m.res(OpSelect, i32, lt, m.ci(0), m.ci(1))
    ptr = m.res(OpAccessChain, m.ptr(SCUniformConstant, simg), tex, idx)
    si = m.res(OpLoad, simg, ptr)
    c = m.res(OpImageSampleImplicitLod, v4, si, uv)
    m.op(OpStore, o, c)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [tex, v_uv, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def lambert_fs(albedo=ALBEDO, light=LIGHT):
    """colour = vec4(albedo * max(dot(normalize(n), light), 0), 1)"""
    m = Module()
    m.capability(CapShader)
    glsl = m.ext_import("GLSL.std.450")
    f32 = m.f32()
    v3, v4 = m.vec(f32, 3), m.vec(f32, 4)
    v_n = _io(m, SCInput, v3, 0)
    o = _io(m, SCOutput, v4, 0)
    c_albedo = m.cvec(albedo)
    c_light = m.cvec(light)
    zero, one = m.cf(0.0), m.cf(1.0)
    fn = _begin_main(m)
    n = m.res(OpLoad, v3, v_n)
    nn = m.res(OpExtInst, v3, glsl, GLSLNormalize, n)
    d = m.res(OpDot, f32, nn, c_light)
    d = m.res(OpExtInst, f32, glsl, GLSLFMax, d, zero)
    c = m.res(OpVectorTimesScalar, v3, c_albedo, d)
    r = m.res(OpCompositeExtract, f32, c, 0)
    g = m.res(OpCompositeExtract, f32, c, 1)
    b = m.res(OpCompositeExtract, f32, c, 2)
    out = m.res(OpCompositeConstruct, v4, r, g, b, one)
    m.op(OpStore, o, out)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [v_n, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def threshold_fs(threshold=0.5):
    """colour = in0 unless in0.r < threshold, in which case the fragment is discarded (OpKill);
    exercises control flow and discard"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v4 = m.vec(f32, 4)
    v_col = _io(m, SCInput, v4, 0)
    o = _io(m, SCOutput, v4, 0)
    thr = m.cf(threshold)
    fn = _begin_main(m)
    c = m.res(OpLoad, v4, v_col)
    r = m.res(OpCompositeExtract, f32, c, 0)
    cond = m.res(OpFOrdLessThan, m.bool(), r, thr)
    kill_l, keep_l = m.new_id(), m.new_id()
    m.op(OpSelectionMerge, keep_l, 0)
    m.op(OpBranchConditional, cond, kill_l, keep_l)
    m.op(OpLabel, kill_l)
    m.op(OpKill)
    m.op(OpLabel, keep_l)
    m.op(OpStore, o, c)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [v_col, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()

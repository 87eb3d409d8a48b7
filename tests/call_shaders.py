"""Shaders with function calls, built with kazan_gb300.spirv_asm, each computing exactly what one of the
workload shaders computes (so the GPU images must still equal the oracle's)."""
from kazan_gb300.spirv_asm import (Module, CapShader, DecOffset, DecColMajor, DecMatrixStride, DecBlock, SCInput,
                                   SCOutput, SCPushConstant, SCFunction, OpAccessChain, OpLoad, OpStore,
                                   OpVariable, OpMatrixTimesVector, OpVectorTimesScalar, OpCompositeExtract,
                                   OpCompositeConstruct, OpFOrdLessThan, OpSelectionMerge, OpBranchConditional,
                                   OpLabel, OpReturn, OpReturnValue, OpFunctionCall, ExecVertex, ExecFragment,
                                   ModeOriginUpperLeft, _per_vertex, _io, _begin_main, _end_main, begin_function,
                                   end_function)


def color_fs_calls():
    """colour = interpolated in0, routed through `vec4 ident(vec4)`, `void scale(inout vec4, float)` with
    factor 1.0, and a branchy `float sat(float)` called from four call sites"""
    m = Module()
    m.capability(CapShader)
    f32 = m.f32()
    v4 = m.vec(f32, 4)
    pv4 = m.ptr(SCFunction, v4)
    v_col = _io(m, SCInput, v4, 0)
    o = _io(m, SCOutput, v4, 0)
    # vec4 ident(vec4 c) { return c; }
    f_ident, (pc,) = begin_function(m, v4, [v4])
    m.op(OpReturnValue, pc)
    end_function(m)
    # void scale(inout vec4 v, float k) { v = v * k; }
    f_scale, (pv, pk) = begin_function(m, m.void(), [pv4, f32])
    t = m.res(OpLoad, v4, pv)
    m.op(OpStore, pv, m.res(OpVectorTimesScalar, v4, t, pk))
    m.op(OpReturn)
    end_function(m)
    # float sat(float x) { if (x < 0) return 0; return x; }   (inputs are in [0, 1]: the identity)
    f_sat, (px,) = begin_function(m, f32, [f32])
    neg = m.res(OpFOrdLessThan, m.bool(), px, m.cf(0.0))
    l_neg, l_pos = m.new_id(), m.new_id()
    m.op(OpSelectionMerge, l_pos, 0)
    m.op(OpBranchConditional, neg, l_neg, l_pos)
    m.op(OpLabel, l_neg)
    m.op(OpReturnValue, m.cf(0.0))
    m.op(OpLabel, l_pos)
    m.op(OpReturnValue, px)
    end_function(m)
    fn = _begin_main(m)
    local = m.res(OpVariable, pv4, SCFunction)
    c = m.res(OpLoad, v4, v_col)
    m.op(OpStore, local, m.res(OpFunctionCall, v4, f_ident, c))
    m.res(OpFunctionCall, m.void(), f_scale, local, m.cf(1.0))
    r = m.res(OpLoad, v4, local)
    comps = [m.res(OpFunctionCall, f32, f_sat, m.res(OpCompositeExtract, f32, r, k)) for k in range(4)]
    m.op(OpStore, o, m.res(OpCompositeConstruct, v4, *comps))
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [v_col, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()


def lambert_vs_calls():
    """gl_Position = transform(mvp, vec4(in0, 1)) with `vec4 transform(mat4, vec4)`; out0 = in1"""
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
    pc = m.variable(SCPushConstant, m.ptr(SCPushConstant, blk))
    pv = _per_vertex(m)
    in_pos = _io(m, SCInput, v3, 0)
    in_nrm = _io(m, SCInput, v3, 1)
    out_nrm = _io(m, SCOutput, v3, 0)
    f_xf, (pm, pp) = begin_function(m, v4, [m4, v4])
    m.op(OpReturnValue, m.res(OpMatrixTimesVector, v4, pm, pp))
    end_function(m)
    fn = _begin_main(m)
    mvp = m.res(OpLoad, m4, m.res(OpAccessChain, m.ptr(SCPushConstant, m4), pc, m.ci(0)))
    p = m.res(OpLoad, v3, in_pos)
    p4 = m.res(OpCompositeConstruct, v4, *[m.res(OpCompositeExtract, f32, p, k) for k in range(3)], m.cf(1.0))
    clip = m.res(OpFunctionCall, v4, f_xf, mvp, p4)
    m.op(OpStore, m.res(OpAccessChain, m.ptr(SCOutput, v4), pv, m.ci(0)), clip)
    m.op(OpStore, out_nrm, m.res(OpLoad, v3, in_nrm))
    _end_main(m)
    m.entry(ExecVertex, fn, "main", [pc, pv, in_pos, in_nrm, out_nrm])
    return m.to_words()


def color_fs_loops():
    """colour = interpolated in0, copied component by component into a local float[4] in a loop (run-time
    index into the array, OpVectorExtractDynamic), then read back in a second loop (run-time index loads,
    OpVectorInsertDynamic into a vec4 phi)"""
    from kazan_gb300.spirv_asm import (OpPhi, OpLoopMerge, OpBranch, OpSLessThan, OpIAdd,
                                       OpVectorExtractDynamic, OpVectorInsertDynamic)
    m = Module()
    m.capability(CapShader)
    f32, i32 = m.f32(), m.i32()
    v4 = m.vec(f32, 4)
    arr = m.array(f32, 4)
    v_col = _io(m, SCInput, v4, 0)
    o = _io(m, SCOutput, v4, 0)
    fn = _begin_main(m)
    local = m.res(OpVariable, m.ptr(SCFunction, arr), SCFunction)   # variables live in the first block
    entry_l = m.new_id()
    m.op(OpBranch, entry_l)
    m.op(OpLabel, entry_l)
    c = m.res(OpLoad, v4, v_col)
    zero, one, four = m.ci(0), m.ci(1), m.ci(4)
    # loop 1: for (i = 0; i < 4; i++) local[i] = c[i];
    h1, b1, k1, e1 = m.new_id(), m.new_id(), m.new_id(), m.new_id()
    m.op(OpBranch, h1)
    m.op(OpLabel, h1)
    i = m.new_id()
    i_next = m.new_id()
    m._ins(m.functions, OpPhi, (i32, i, zero, entry_l, i_next, k1))
    m.op(OpLoopMerge, e1, k1, 0)
    m.op(OpBranchConditional, m.res(OpSLessThan, m.bool(), i, four), b1, e1)
    m.op(OpLabel, b1)
    comp = m.res(OpVectorExtractDynamic, f32, c, i)
    m.op(OpStore, m.res(OpAccessChain, m.ptr(SCFunction, f32), local, i), comp)
    m.op(OpBranch, k1)
    m.op(OpLabel, k1)
    m._ins(m.functions, OpIAdd, (i32, i_next, i, one))
    m.op(OpBranch, h1)
    m.op(OpLabel, e1)
    # loop 2: r = vec4(0); for (j = 0; j < 4; j++) r[j] = local[j];
    h2, b2, k2, e2 = m.new_id(), m.new_id(), m.new_id(), m.new_id()
    zero4 = m.res(OpCompositeConstruct, v4, m.cf(0.0), m.cf(0.0), m.cf(0.0), m.cf(0.0))
    m.op(OpBranch, h2)
    m.op(OpLabel, h2)
    j, j_next, r, r_next = m.new_id(), m.new_id(), m.new_id(), m.new_id()
    m._ins(m.functions, OpPhi, (i32, j, zero, e1, j_next, k2))
    m._ins(m.functions, OpPhi, (v4, r, zero4, e1, r_next, k2))
    m.op(OpLoopMerge, e2, k2, 0)
    m.op(OpBranchConditional, m.res(OpSLessThan, m.bool(), j, four), b2, e2)
    m.op(OpLabel, b2)
    x = m.res(OpLoad, f32, m.res(OpAccessChain, m.ptr(SCFunction, f32), local, j))
    m._ins(m.functions, OpVectorInsertDynamic, (v4, r_next, r, x, j))
    m.op(OpBranch, k2)
    m.op(OpLabel, k2)
    m._ins(m.functions, OpIAdd, (i32, j_next, j, one))
    m.op(OpBranch, h2)
    m.op(OpLabel, e2)
    m.op(OpStore, o, r)
    _end_main(m)
    m.entry(ExecFragment, fn, "main", [v_col, o])
    m.mode(fn, ModeOriginUpperLeft)
    return m.to_words()

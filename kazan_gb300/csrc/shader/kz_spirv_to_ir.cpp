/*
 * kz_spirv_to_ir.cpp - SPIR-V vertex/fragment entry point -> scalar register IR.
 *
 * Role of the reference's shader-compiler-translate-spirv-to-ir (TranslatedSPIRVShader::new,
 * shader-compiler-translate-spirv-to-ir/src/lib.rs:191-214), which today translates only an empty
 * main (OpLoad/OpStore/OpAccessChain are `todo!()` at parse/memory_instructions.rs:99,124,141 and the
 * arithmetic opcodes are unimplemented, parse/unimplemented_instructions.rs).  This translator covers
 * the opcodes vertex and fragment shaders of the draw path use: typed constants and specialisation
 * constants, interface variables (Location, Component, BuiltIn, Flat, NoPerspective), push-constant
 * blocks (Offset, MatrixStride, ArrayStride, RowMajor), function/private variables, composites,
 * float/int/bool arithmetic, matrix products, GLSL.std.450, and unstructured control flow with OpPhi.
 * Interface variables are laid out in 16-byte locations as the reference's io_layout does
 * (shader-compiler-translate-spirv-to-ir/src/io_layout.rs:6-13).
 *
 * Fixed evaluation order (the CPU oracle restates the same):
 *   OpDot(a, b)               t = a0*b0; t = fma(ak, bk, t) for k = 1..n-1
 *   OpMatrixTimesVector(M, v) r_i = M[0][i]*v0, then fma(M[c][i], vc, r_i) for c = 1..C-1
 *   Normalize(x)              x * (1 / sqrt(dot(x, x)))   (sqrt and divide correctly rounded)
 *   Length(x)                 sqrt(dot(x, x))
 *   FMix(x, y, a)             fma(a, y - x, x)
 *   FMod / FRem(x, y)         fma(-y, floor / trunc(x / y), x)
 *   Reflect(I, N)             fma(-(2 dot(N, I)), N, I)
 *   Determinant / Inverse     2x2 minors a d - b c as fma(a, d, -(b c)); cofactor expansion along row 0
 *   Exp, Log                  exp2(x log2 e), log2(x) ln 2 (hardware approximations)
 *   Atan                      |x| reduced to [0, tan(pi/12)] (reciprocal, then the addition formula for
 *                             pi/6), Taylor series to t^13; Asin / Acos / Atan2 through it
 * Derivatives (dFdx, dFdy, fwidth) are refused: fragments are shaded one at a time, not in quads.
 */
#include <cstring>
#include <map>
#include <unordered_map>

#include "kz_ir.h"
#include "kz_spirv.h"

namespace kz {
namespace ir {

using namespace spv;

namespace {

struct TypeInfo {
  enum Kind {
    Void, Bool, Int, Float, Vector, Matrix, Array, RuntimeArray, Struct, Pointer, Function, Image, SampledImage,
    Sampler, Other
  } kind = Other;
  uint32_t width = 32;
  bool is_signed = false;
  uint32_t elem = 0;
  uint32_t count = 0;
  uint32_t storage = 0;
  std::vector<uint32_t> members;
};

struct DecSet {
  std::vector<std::pair<uint32_t, std::vector<uint32_t>>> list;
  bool has(uint32_t d) const {
    for (auto& e : list)
      if (e.first == d) return true;
    return false;
  }
  bool get(uint32_t d, uint32_t& v) const {
    for (auto& e : list)
      if (e.first == d) {
        v = e.second.empty() ? 0 : e.second[0];
        return true;
      }
    return false;
  }
};

/* per-scalar address of a variable; a combined image sampler is one Tex slot per array element */
enum class Space : uint8_t { None, In, Out, Push, Reg, Ubo, Tex };
struct Slot {
  Space space = Space::None;
  uint32_t offset = 0;  /* byte offset for In/Out/Push/Ubo; array element for Tex */
  int32_t reg = -1;     /* shadow register for Out/Reg */
  bool is_bool_in = false;
  uint32_t key = 0;     /* Ubo/Tex: descriptor binding, set << 16 | binding */
};

struct Var {
  uint32_t storage = 0;
  uint32_t type = 0; /* pointee type */
  std::vector<Slot> slots;
  /* a storage block ending in a runtime-sized array: the array's byte offset in the block, its element
   * stride, and the bytes of an element the shader can read (its slots hold element 0) */
  bool has_rt = false;
  uint32_t rt_base = 0, rt_stride = 0, rt_end = 0;
};

struct Place {
  uint32_t var = 0;
  uint32_t type = 0;
  uint32_t first = 0;
  uint32_t push_byte = 0; /* unused: push slots carry their own offsets */
  /* one index known only at run time: element dyn of dyn_count, each dyn_stride slots, starts at slot
   * first + dyn * dyn_stride (constant indices after it are already in `first`) */
  int32_t dyn = -1;
  uint32_t dyn_stride = 0, dyn_count = 0;
  bool rt = false; /* dyn indexes the variable's runtime-sized array: its length comes from the descriptor */
};

struct Val {
  uint32_t type = 0;
  std::vector<int32_t> regs;
  /* a combined image sampler (or its image) of binding tex_key: array element tex_elem, or, when
   * tex_dyn, the element in regs[0] */
  bool is_tex = false, tex_dyn = false;
  uint32_t tex_key = 0, tex_elem = 0;
  /* OpSampledImage of a separate image and sampler: the sampler's binding and array element */
  bool has_smp = false;
  uint32_t smp_key = 0, smp_elem = 0;
};

struct PhiInfo {
  uint32_t result;
  uint32_t type;
  std::vector<std::pair<uint32_t, uint32_t>> incoming; /* (value id, parent label) */
};

class Translator {
 public:
  Translator(const Module& m, Stage stage, const char* entry, const std::vector<std::pair<uint32_t, uint32_t>>& spec,
             Shader& out)
      : m_(m), stage_(stage), entry_name_(entry), spec_(spec), out_(out), fn_(out.fn) {}

  std::string run();

 private:
  const Module& m_;
  Stage stage_;
  std::string entry_name_;
  const std::vector<std::pair<uint32_t, uint32_t>>& spec_;
  Shader& out_;
  Function& fn_;
  std::string err_;

  std::unordered_map<uint32_t, TypeInfo> types_;
  std::unordered_map<uint32_t, DecSet> decs_;
  std::map<std::pair<uint32_t, uint32_t>, DecSet> member_decs_;
  std::unordered_map<uint32_t, std::pair<uint32_t, std::vector<uint32_t>>> consts_; /* id -> (type, bits) */
  std::unordered_map<uint32_t, Var> vars_;
  std::unordered_map<uint32_t, Place> places_;
  std::unordered_map<uint32_t, Val> vals_;
  std::unordered_map<uint32_t, std::string> ext_sets_;
  std::unordered_map<uint32_t, uint32_t> labels_; /* SPIR-V label id -> IR label */
  std::unordered_map<uint32_t, std::vector<PhiInfo>> phis_;
  uint32_t entry_id_ = 0;
  std::vector<uint32_t> interface_ids_;
  uint32_t cur_block_ = 0;
  /* function calls are inlined: each function's body [begin, end) in m_.insns, and the frames of the
   * calls being translated (where the callee returns to, and the registers of its result) */
  std::unordered_map<uint32_t, std::pair<size_t, size_t>> fn_ranges_;
  struct Frame {
    uint32_t ret_label = 0;
    Val result;
    bool has_result = false;
  };
  std::vector<Frame> frames_;

  bool fail(const std::string& s) {
    if (err_.empty()) err_ = s;
    return false;
  }

  /* ---- types ---- */
  const TypeInfo& ty(uint32_t id) {
    static TypeInfo none;
    auto it = types_.find(id);
    return it == types_.end() ? none : it->second;
  }
  uint32_t scalars(uint32_t t) {
    const TypeInfo& ti = ty(t);
    switch (ti.kind) {
      case TypeInfo::Bool:
      case TypeInfo::Int:
      case TypeInfo::Float: return 1;
      case TypeInfo::Vector: return ti.count;
      case TypeInfo::Matrix: return ti.count * scalars(ti.elem);
      case TypeInfo::Array: return ti.count * scalars(ti.elem);
      case TypeInfo::Image:
      case TypeInfo::SampledImage:
      case TypeInfo::Sampler: return 1; /* one Tex slot */
      case TypeInfo::Struct: {
        uint32_t n = 0;
        for (uint32_t mbr : ti.members) n += scalars(mbr);
        return n;
      }
      default: return 0;
    }
  }
  void flat_types(uint32_t t, std::vector<Ty>& outv) {
    const TypeInfo& ti = ty(t);
    switch (ti.kind) {
      case TypeInfo::Bool: outv.push_back(Ty::Pred); break;
      case TypeInfo::Int: outv.push_back(Ty::B32); break;
      case TypeInfo::Float: outv.push_back(Ty::F32); break;
      case TypeInfo::Vector:
      case TypeInfo::Matrix:
      case TypeInfo::Array:
        for (uint32_t i = 0; i < ti.count; i++) flat_types(ti.elem, outv);
        break;
      case TypeInfo::Struct:
        for (uint32_t mbr : ti.members) flat_types(mbr, outv);
        break;
      default: break;
    }
  }
  /* scalar offset and type of member `idx` inside composite type t */
  bool member(uint32_t t, uint32_t idx, uint32_t& off, uint32_t& mt) {
    const TypeInfo& ti = ty(t);
    switch (ti.kind) {
      case TypeInfo::Vector:
      case TypeInfo::Matrix:
      case TypeInfo::Array:
        if (ti.count && idx >= ti.count) return fail("composite index out of range");
        mt = ti.elem;
        off = idx * scalars(ti.elem);
        return true;
      case TypeInfo::Struct: {
        if (idx >= ti.members.size()) return fail("struct member index out of range");
        off = 0;
        for (uint32_t i = 0; i < idx; i++) off += scalars(ti.members[i]);
        mt = ti.members[idx];
        return true;
      }
      default: return fail("index into a non-composite type");
    }
  }
  bool is_float(uint32_t t) {
    const TypeInfo& ti = ty(t);
    if (ti.kind == TypeInfo::Float) return true;
    if (ti.kind == TypeInfo::Vector || ti.kind == TypeInfo::Matrix) return is_float(ti.elem);
    return false;
  }
  bool is_signed_int(uint32_t t) {
    const TypeInfo& ti = ty(t);
    if (ti.kind == TypeInfo::Int) return ti.is_signed;
    if (ti.kind == TypeInfo::Vector) return is_signed_int(ti.elem);
    return false;
  }

  /* ---- emission helpers ---- */
  int32_t konst(Ty t, uint32_t bits) {
    int32_t r = fn_.reg(t);
    Inst i;
    i.op = Op::Const;
    i.ty = t;
    i.dst = r;
    i.imm = bits;
    fn_.emit(i);
    return r;
  }
  int32_t op1(Op op, Ty t, int32_t a) {
    int32_t r = fn_.reg(t);
    Inst i;
    i.op = op;
    i.ty = t;
    i.dst = r;
    i.a = a;
    fn_.emit(i);
    return r;
  }
  int32_t op2(Op op, Ty t, int32_t a, int32_t b, uint32_t imm = 0) {
    int32_t r = fn_.reg(t);
    Inst i;
    i.op = op;
    i.ty = t;
    i.dst = r;
    i.a = a;
    i.b = b;
    i.imm = imm;
    fn_.emit(i);
    return r;
  }
  int32_t op3(Op op, Ty t, int32_t a, int32_t b, int32_t c) {
    int32_t r = fn_.reg(t);
    Inst i;
    i.op = op;
    i.ty = t;
    i.dst = r;
    i.a = a;
    i.b = b;
    i.c = c;
    fn_.emit(i);
    return r;
  }
  void mov(Ty t, int32_t dst, int32_t a) {
    Inst i;
    i.op = Op::Mov;
    i.ty = t;
    i.dst = dst;
    i.a = a;
    fn_.emit(i);
  }
  void label(uint32_t l) {
    Inst i;
    i.op = Op::Label;
    i.imm = l;
    fn_.emit(i);
  }
  void bra(uint32_t l) {
    Inst i;
    i.op = Op::Bra;
    i.imm = l;
    fn_.emit(i);
  }
  void bra_if(int32_t p, uint32_t l) {
    Inst i;
    i.op = Op::BraIf;
    i.ty = Ty::Pred;
    i.a = p;
    i.imm = l;
    fn_.emit(i);
  }
  Ty reg_ty(int32_t r) { return fn_.regs[(size_t)r]; }

  Val* val(uint32_t id) {
    auto it = vals_.find(id);
    if (it == vals_.end()) {
      fail("use of an undefined value %" + std::to_string(id));
      return nullptr;
    }
    return &it->second;
  }
  uint32_t label_of(uint32_t id) {
    auto it = labels_.find(id);
    if (it != labels_.end()) return it->second;
    uint32_t l = fn_.label();
    labels_[id] = l;
    return l;
  }

  /* ---- module scan ---- */
  bool scan_module();
  bool eval_spec_op(const Insn& in);
  bool layout_interface(uint32_t var_id, Var& v);
  void assign_io(uint32_t t, const DecSet* d, uint32_t struct_type, uint32_t member_idx, uint32_t& location,
                 std::vector<Slot>& slots, bool is_input);
  void assign_push(uint32_t t, uint32_t byte, std::vector<Slot>& slots, uint32_t stride_hint, bool row_major);
  bool layout_descriptor(uint32_t var_id, Var& v);
  bool image_sample(const Insn& in);
  Space block_space_ = Space::Push; /* what assign_push lays out: push constants or a uniform block */
  uint32_t block_key_ = 0;
  uint32_t block_bytes_ = 0;
  bool block_storage_ = false; /* laying out a storage block: a last runtime-sized array member is allowed */
  bool block_rt_ = false;
  uint32_t block_rt_base_ = 0, block_rt_stride_ = 0, block_rt_end_ = 0;

  /* ---- function body ---- */
  bool translate_entry();
  void prescan_phis(size_t begin, size_t end);
  bool inline_call(const Insn& in);
  bool do_insn(const Insn& in);
  bool branch_to(uint32_t target);
  bool load(const Place& p, Val& v);
  bool store(const Place& p, const Val& v);
  bool ext_inst(const Insn& in);
  void finish_outputs();
  int32_t dot(const std::vector<int32_t>& a, const std::vector<int32_t>& b, size_t n);
};

bool Translator::scan_module() {
  for (const Insn& in : m_.insns) {
    const auto& o = in.ops;
    switch (in.opcode) {
      case OpCapability: {
        uint32_t c = o.empty() ? 0 : o[0];
        if (c != 0 && c != 1 && c != 11 && c != 32 && c != 33) {
          /* Matrix, Shader, Int64 (decode only), ClipDistance, CullDistance */
        }
        break;
      }
      case OpExtInstImport: {
        size_t i = 1;
        ext_sets_[o[0]] = read_string(o, i);
        break;
      }
      case OpEntryPoint: {
        size_t i = 2;
        std::string name = read_string(o, i);
        uint32_t model = o[0];
        bool want = (stage_ == Stage::Vertex && model == EMVertex) || (stage_ == Stage::Fragment && model == EMFragment);
        if (want && name == entry_name_) {
          entry_id_ = o[1];
          interface_ids_.assign(o.begin() + (long)i, o.end());
        }
        break;
      }
      case OpExecutionMode:
        if (o.size() >= 2 && o[1] == ModeOriginLowerLeft && stage_ == Stage::Fragment && o[0] == entry_id_)
          return fail("OriginLowerLeft is not supported (Vulkan requires OriginUpperLeft)");
        if (o.size() >= 2 && o[1] == ModeDepthReplacing && o[0] == entry_id_)
          return fail("fragment depth output is not supported");
        break;
      case OpDecorate: {
        std::vector<uint32_t> rest(o.begin() + 2, o.end());
        decs_[o[0]].list.push_back({o[1], rest});
        break;
      }
      case OpMemberDecorate: {
        std::vector<uint32_t> rest(o.begin() + 3, o.end());
        member_decs_[{o[0], o[1]}].list.push_back({o[2], rest});
        break;
      }
      case OpTypeVoid: types_[o[0]].kind = TypeInfo::Void; break;
      case OpTypeBool: types_[o[0]].kind = TypeInfo::Bool; break;
      case OpTypeInt: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Int;
        t.width = o[1];
        t.is_signed = o[2] != 0;
        break;
      }
      case OpTypeFloat: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Float;
        t.width = o[1];
        break;
      }
      case OpTypeVector:
      case OpTypeMatrix: {
        TypeInfo& t = types_[o[0]];
        t.kind = in.opcode == OpTypeVector ? TypeInfo::Vector : TypeInfo::Matrix;
        t.elem = o[1];
        t.count = o[2];
        break;
      }
      case OpTypeArray: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Array;
        t.elem = o[1];
        auto c = consts_.find(o[2]);
        t.count = c == consts_.end() || c->second.second.empty() ? 0 : c->second.second[0];
        break;
      }
      case OpTypeRuntimeArray: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::RuntimeArray;
        t.elem = o[1];
        break;
      }
      case OpTypeStruct: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Struct;
        t.members.assign(o.begin() + 1, o.end());
        break;
      }
      case OpTypePointer: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Pointer;
        t.storage = o[1];
        t.elem = o[2];
        break;
      }
      case OpTypeFunction: types_[o[0]].kind = TypeInfo::Function; break;
      case OpTypeImage: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::Image;
        t.count = o.size() > 2 ? o[2] : 0; /* Dim */
        break;
      }
      case OpTypeSampler: types_[o[0]].kind = TypeInfo::Sampler; break;
      case OpTypeSampledImage: {
        TypeInfo& t = types_[o[0]];
        t.kind = TypeInfo::SampledImage;
        t.elem = o[1];
        break;
      }
      case OpTypeOpaque: types_[o[0]].kind = TypeInfo::Other; break;
      case OpConstantTrue:
      case OpConstantFalse:
        consts_[o[1]] = {o[0], {in.opcode == OpConstantTrue ? 1u : 0u}};
        break;
      case OpSpecConstantTrue:
      case OpSpecConstantFalse: {
        uint32_t v = in.opcode == OpSpecConstantTrue ? 1u : 0u, sid;
        if (decs_[o[1]].get(DecSpecId, sid))
          for (auto& s : spec_)
            if (s.first == sid) v = s.second != 0;
        consts_[o[1]] = {o[0], {v}};
        break;
      }
      case OpConstant:
      case OpSpecConstant: {
        if (o.size() < 3) return fail("constant without a value");
        if (ty(o[0]).width != 32) {
          consts_[o[1]] = {o[0], {o[2]}}; /* 64-bit constants keep their low word (decode-only support) */
          break;
        }
        uint32_t v = o[2], sid;
        if (in.opcode == OpSpecConstant && decs_[o[1]].get(DecSpecId, sid))
          for (auto& s : spec_)
            if (s.first == sid) v = s.second;
        consts_[o[1]] = {o[0], {v}};
        break;
      }
      case OpConstantComposite:
      case OpSpecConstantComposite: {
        std::vector<uint32_t> bits;
        for (size_t i = 2; i < o.size(); i++) {
          auto c = consts_.find(o[i]);
          if (c == consts_.end()) return fail("composite constant of a non-constant");
          bits.insert(bits.end(), c->second.second.begin(), c->second.second.end());
        }
        consts_[o[1]] = {o[0], bits};
        break;
      }
      case OpConstantNull:
        consts_[o[1]] = {o[0], std::vector<uint32_t>(scalars(o[0]), 0u)};
        break;
      case OpSpecConstantOp:
        if (!eval_spec_op(in)) return false;
        break;
      case OpVariable: {
        if (o[2] == SCFunction) break; /* handled inside the function */
        Var v;
        v.storage = o[2];
        v.type = ty(o[0]).elem;
        vars_[o[1]] = v;
        break;
      }
      default: break;
    }
  }
  if (!entry_id_) return fail("entry point \"" + entry_name_ + "\" not found for this stage");
  return err_.empty();
}

bool Translator::eval_spec_op(const Insn& in) {
  const auto& o = in.ops;
  uint32_t opc = o[2];
  auto arg = [&](size_t i, uint32_t& v) -> bool {
    auto c = consts_.find(o[i]);
    if (c == consts_.end() || c->second.second.empty()) return fail("OpSpecConstantOp operand is not constant");
    v = c->second.second[0];
    return true;
  };
  uint32_t a = 0, b = 0, r = 0;
  if (!arg(3, a)) return false;
  if (o.size() > 4 && !arg(4, b)) return false;
  switch (opc) {
    case OpIAdd: r = a + b; break;
    case OpISub: r = a - b; break;
    case OpIMul: r = a * b; break;
    case OpUDiv: r = b ? a / b : 0; break;
    case OpSDiv: r = b ? (uint32_t)((int32_t)a / (int32_t)b) : 0; break;
    case OpUMod: r = b ? a % b : 0; break;
    case OpSRem: r = b ? (uint32_t)((int32_t)a % (int32_t)b) : 0; break;
    case OpBitwiseAnd: r = a & b; break;
    case OpBitwiseOr: r = a | b; break;
    case OpBitwiseXor: r = a ^ b; break;
    case OpShiftLeftLogical: r = a << (b & 31); break;
    case OpShiftRightLogical: r = a >> (b & 31); break;
    case OpShiftRightArithmetic: r = (uint32_t)((int32_t)a >> (b & 31)); break;
    case OpNot: r = ~a; break;
    case OpSNegate: r = (uint32_t)(-(int32_t)a); break;
    case OpIEqual: r = a == b; break;
    case OpINotEqual: r = a != b; break;
    case OpLogicalAnd: r = a && b; break;
    case OpLogicalOr: r = a || b; break;
    case OpLogicalNot: r = !a; break;
    default: return fail("unsupported OpSpecConstantOp opcode " + std::to_string(opc));
  }
  consts_[o[1]] = {o[0], {r}};
  return true;
}

/* interface layout: each location is 16 bytes (four 32-bit components) */
void Translator::assign_io(uint32_t t, const DecSet* d, uint32_t struct_type, uint32_t member_idx, uint32_t& location,
                           std::vector<Slot>& slots, bool is_input) {
  uint32_t loc, comp = 0, bi;
  DecSet empty;
  const DecSet& ds = d ? *d : empty;
  if (ds.get(DecLocation, loc)) location = loc;
  ds.get(DecComponent, comp);
  bool flat = ds.has(DecFlat), noper = ds.has(DecNoPerspective);
  const TypeInfo& ti = ty(t);
  if (ds.get(DecBuiltIn, bi)) {
    uint32_t n = scalars(t);
    for (uint32_t k = 0; k < n; k++) {
      Slot s;
      if (is_input) {
        s.space = Space::In;
        if (stage_ == Stage::Vertex && (bi == BuiltInVertexIndex || bi == BuiltInVertexId)) s.offset = 128;
        else if (stage_ == Stage::Vertex && (bi == BuiltInInstanceIndex || bi == BuiltInInstanceId)) s.offset = 132;
        else if (stage_ == Stage::Fragment && bi == BuiltInFragCoord) s.offset = 64 + 4 * k;
        else if (stage_ == Stage::Fragment && bi == BuiltInFrontFacing) {
          s.offset = 80;
          s.is_bool_in = true;
        } else {
          fail("unsupported input built-in " + std::to_string(bi));
          s.space = Space::None;
        }
      } else {
        s.space = Space::Out;
        if (stage_ == Stage::Vertex && bi == BuiltInPosition && k < 4) {
          s.offset = 4 * k;
          out_.iface.writes_position = true;
        } else if (stage_ == Stage::Fragment && bi == BuiltInFragDepth) {
          fail("fragment depth output is not supported");
        } else {
          s.space = Space::None; /* PointSize, ClipDistance, CullDistance: accepted and ignored */
        }
      }
      slots.push_back(s);
    }
    return;
  }
  (void)struct_type;
  (void)member_idx;
  switch (ti.kind) {
    case TypeInfo::Bool:
    case TypeInfo::Int:
    case TypeInfo::Float:
    case TypeInfo::Vector: {
      uint32_t n = scalars(t);
      for (uint32_t k = 0; k < n; k++) {
        Slot s;
        uint32_t c = comp + k;
        uint32_t slot = location * 4 + c;
        if (is_input) {
          s.space = Space::In;
          s.offset = location * 16 + c * 4;
          if (stage_ == Stage::Vertex) {
            if (location >= 8) fail("vertex input location beyond 7");
            out_.iface.input_locations |= 1u << location;
          } else {
            if (slot >= 16) fail("fragment input beyond 16 scalar varyings");
            out_.iface.input_slots |= 1u << slot;
            out_.iface.input_locations |= 1u << location;
            if (flat) out_.iface.flat_slots |= 1u << slot;
            if (noper) out_.iface.noperspective_slots |= 1u << slot;
          }
        } else {
          s.space = Space::Out;
          if (stage_ == Stage::Vertex) {
            if (slot >= 16) fail("vertex output beyond 16 scalar varyings");
            s.offset = 16 + slot * 4;
            out_.iface.output_slots |= 1u << slot;
            if (flat) out_.iface.flat_slots |= 1u << slot;
            if (noper) out_.iface.noperspective_slots |= 1u << slot;
          } else {
            if (location == 0) {
              s.offset = c * 4;
              out_.iface.writes_color = true;
            } else {
              s.space = Space::None; /* only one colour attachment */
            }
          }
        }
        slots.push_back(s);
      }
      location++;
      break;
    }
    case TypeInfo::Matrix:
    case TypeInfo::Array:
      for (uint32_t i = 0; i < ti.count; i++) assign_io(ti.elem, nullptr, 0, 0, location, slots, is_input);
      break;
    case TypeInfo::Struct:
      for (uint32_t i = 0; i < ti.members.size(); i++) {
        auto it = member_decs_.find({t, i});
        const DecSet* md = it == member_decs_.end() ? nullptr : &it->second;
        uint32_t mloc;
        if (md && md->get(DecLocation, mloc)) location = mloc;
        DecSet merged;
        if (md) merged = *md;
        if (flat && !merged.has(DecFlat)) merged.list.push_back({DecFlat, {}});
        if (noper && !merged.has(DecNoPerspective)) merged.list.push_back({DecNoPerspective, {}});
        assign_io(ti.members[i], &merged, t, i, location, slots, is_input);
      }
      break;
    default: fail("unsupported interface variable type"); break;
  }
}

void Translator::assign_push(uint32_t t, uint32_t byte, std::vector<Slot>& slots, uint32_t stride_hint,
                             bool row_major) {
  const TypeInfo& ti = ty(t);
  switch (ti.kind) {
    case TypeInfo::Bool:
    case TypeInfo::Int:
    case TypeInfo::Float: {
      Slot s;
      s.space = block_space_;
      s.offset = byte;
      s.key = block_key_;
      slots.push_back(s);
      if (block_space_ == Space::Push && byte + 4 > out_.iface.push_bytes) out_.iface.push_bytes = byte + 4;
      if (block_space_ == Space::Ubo && byte + 4 > block_bytes_) block_bytes_ = byte + 4;
      break;
    }
    case TypeInfo::Vector:
      for (uint32_t i = 0; i < ti.count; i++) assign_push(ti.elem, byte + 4 * i, slots, 0, false);
      break;
    case TypeInfo::Matrix: {
      uint32_t rows = ty(ti.elem).count;
      uint32_t stride = stride_hint ? stride_hint : 16;
      for (uint32_t c = 0; c < ti.count; c++)
        for (uint32_t r = 0; r < rows; r++) {
          uint32_t off = row_major ? byte + r * stride + 4 * c : byte + c * stride + 4 * r;
          assign_push(ty(ti.elem).elem, off, slots, 0, false);
        }
      break;
    }
    case TypeInfo::Array: {
      uint32_t stride = 0;
      decs_[t].get(DecArrayStride, stride);
      if (!stride) stride = 4 * scalars(ti.elem);
      for (uint32_t i = 0; i < ti.count; i++) assign_push(ti.elem, byte + i * stride, slots, stride_hint, row_major);
      break;
    }
    case TypeInfo::Struct:
      for (uint32_t i = 0; i < ti.members.size(); i++) {
        auto it = member_decs_.find({t, i});
        uint32_t off = 0, ms = 0;
        bool rm = false;
        if (it != member_decs_.end()) {
          it->second.get(DecOffset, off);
          it->second.get(DecMatrixStride, ms);
          rm = it->second.has(DecRowMajor);
        }
        assign_push(ti.members[i], byte + off, slots, ms, rm);
      }
      break;
    case TypeInfo::RuntimeArray: {
      /* the last member of a storage block: element 0 is laid out; other elements are addressed at run
       * time from the array's stride, and the bound range limits the index */
      if (block_space_ != Space::Ubo || !block_storage_ || block_rt_) {
        fail("a runtime-sized array is supported only as the last member of a storage buffer");
        break;
      }
      uint32_t stride = 0;
      decs_[t].get(DecArrayStride, stride);
      if (!stride) stride = 4 * scalars(ti.elem);
      size_t first = slots.size();
      assign_push(ti.elem, byte, slots, stride_hint, row_major);
      uint32_t end = 0;
      for (size_t k = first; k < slots.size(); k++) end = std::max(end, slots[k].offset + 4 - byte);
      if (end > stride) {
        fail("runtime-sized array elements wider than their stride");
        break;
      }
      block_rt_ = true;
      block_rt_base_ = byte;
      block_rt_stride_ = stride;
      block_rt_end_ = end;
      break;
    }
    default: fail("unsupported push-constant member type"); break;
  }
}

bool Translator::layout_interface(uint32_t var_id, Var& v) {
  v.slots.clear();
  if (v.storage == SCInput || v.storage == SCOutput) {
    uint32_t location = 0;
    auto it = decs_.find(var_id);
    assign_io(v.type, it == decs_.end() ? nullptr : &it->second, 0, 0, location, v.slots, v.storage == SCInput);
  } else if (v.storage == SCPushConstant) {
    block_space_ = Space::Push;
    assign_push(v.type, 0, v.slots, 0, false);
  } else if (v.storage == SCUniform || v.storage == SCUniformConstant || v.storage == SCStorageBuffer) {
    if (!layout_descriptor(var_id, v)) return false;
  } else if (v.storage == SCPrivate || v.storage == SCFunction) {
    std::vector<Ty> tys;
    flat_types(v.type, tys);
    for (Ty t : tys) {
      Slot s;
      s.space = Space::Reg;
      s.reg = fn_.reg(t);
      v.slots.push_back(s);
    }
  } else {
    return fail("unsupported variable storage class " + std::to_string(v.storage));
  }
  if (v.storage == SCOutput) {
    std::vector<Ty> tys;
    flat_types(v.type, tys);
    for (size_t k = 0; k < v.slots.size() && k < tys.size(); k++) v.slots[k].reg = fn_.reg(tys[k]);
  }
  return err_.empty();
}

/* OpImageSample[Proj]{Implicit,Explicit}Lod and OpImageFetch on a combined image sampler of one mip
 * level: level-of-detail operands (Bias, Lod, Grad, MinLod) select nothing; Proj divides s and t by the
 * last coordinate component */
bool Translator::image_sample(const Insn& in) {
  const auto& o = in.ops;
  if (o.size() < 4) return fail("image instruction with too few operands");
  Val* img = val(o[2]);
  Val* coord = val(o[3]);
  if (!img || !coord) return false;
  if (!img->is_tex) return fail("image operand is not a combined image sampler variable");
  const bool fetch = in.opcode == OpImageFetch;
  const bool proj = in.opcode == OpImageSampleProjImplicitLod || in.opcode == OpImageSampleProjExplicitLod;
  if (o.size() > 4) {
    const uint32_t allowed = fetch ? 0x2u : (0x1u | 0x2u | 0x4u | 0x80u);
    if (o[4] & ~allowed) return fail("image operands other than Bias, Lod, Grad and MinLod are not supported");
  }
  if (coord->regs.size() < 2) return fail("image coordinate with fewer than two components");
  const TypeInfo& rt = ty(o[0]);
  if (rt.kind != TypeInfo::Vector || rt.count != 4 || ty(rt.elem).kind != TypeInfo::Float)
    return fail("image results other than vec4 are not supported (UNORM images)");
  int32_t s = coord->regs[0], t = coord->regs[1];
  if (proj) {
    int32_t q = coord->regs.back();
    s = op2(Op::FDiv, Ty::F32, s, q);
    t = op2(Op::FDiv, Ty::F32, t, q);
  }
  Inst i;
  i.op = fetch ? Op::TexFetch : Op::Tex;
  i.ty = Ty::F32;
  i.dst = fn_.reg(Ty::F32);
  for (int k = 1; k < 4; k++) fn_.reg(Ty::F32);
  i.a = s;
  i.b = t;
  i.c = img->tex_dyn ? img->regs[0] : -1;
  i.imm = img->tex_dyn ? 0u : img->tex_elem;
  i.imm2 = img->tex_key;
  if (img->has_smp) {
    i.smp = img->smp_key;
    i.smp_elem = img->smp_elem;
  }
  fn_.emit(i);
  Val r;
  r.type = o[0];
  for (int k = 0; k < 4; k++) r.regs.push_back(i.dst + k);
  vals_[o[1]] = r;
  return true;
}

bool Translator::layout_descriptor(uint32_t var_id, Var& v) {
  uint32_t set = 0, binding = 0;
  auto it = decs_.find(var_id);
  if (it != decs_.end()) {
    it->second.get(DecDescriptorSet, set);
    it->second.get(DecBinding, binding);
  }
  if (set >= KZ_IR_MAX_SETS || binding >= KZ_IR_MAX_BINDINGS)
    return fail("descriptor set " + std::to_string(set) + " binding " + std::to_string(binding) +
                " is beyond the driver's limits (sets 0..3, bindings 0..15)");
  Interface::Binding b;
  b.set = set;
  b.binding = binding;
  const uint32_t key = set << 16 | binding;
  uint32_t t = v.type, count = 1;
  if (ty(t).kind == TypeInfo::Array) {
    count = ty(t).count;
    t = ty(t).elem;
  }
  const TypeInfo& ti = ty(t);
  if (v.storage == SCUniformConstant) {
    /* combined image samplers, and separate sampled images and samplers (combined by OpSampledImage) */
    if (!count || (ti.kind != TypeInfo::SampledImage && ti.kind != TypeInfo::Image && ti.kind != TypeInfo::Sampler))
      return fail("unsupported UniformConstant variable");
    if ((ti.kind == TypeInfo::SampledImage && ty(ti.elem).count != 1) || (ti.kind == TypeInfo::Image && ti.count != 1))
      return fail("only 2D images are supported");
    b.kind = ti.kind == TypeInfo::SampledImage ? 1 : ti.kind == TypeInfo::Image ? 3 : 4;
    b.count = count;
    for (uint32_t k = 0; k < count; k++) {
      Slot s;
      s.space = Space::Tex;
      s.offset = k;
      s.key = key;
      v.slots.push_back(s);
    }
  } else {
    /* uniform blocks, and storage blocks (StorageBuffer storage class, or Uniform with BufferBlock), which
     * shaders read only: stores to them are refused */
    const bool storage = v.storage == SCStorageBuffer || decs_[t].has(DecBufferBlock);
    if (t != v.type) return fail("arrays of uniform or storage blocks are not supported");
    if (ti.kind != TypeInfo::Struct) return fail("a Uniform variable that is not a block");
    block_space_ = Space::Ubo;
    block_key_ = key;
    block_bytes_ = 0;
    block_storage_ = storage;
    block_rt_ = false;
    assign_push(t, 0, v.slots, 0, false);
    block_space_ = Space::Push;
    block_storage_ = false;
    if (block_rt_) {
      v.has_rt = true;
      v.rt_base = block_rt_base_;
      v.rt_stride = block_rt_stride_;
      v.rt_end = block_rt_end_;
    }
    b.kind = storage ? 2 : 0;
    b.bytes = block_bytes_;
  }
  out_.iface.bindings.push_back(b);
  return err_.empty();
}

bool Translator::load(const Place& p, Val& v) {
  if (p.dyn >= 0 && !vars_[p.var].slots.empty() && p.first < vars_[p.var].slots.size() &&
      (vars_[p.var].slots[p.first].space == Space::Ubo || vars_[p.var].slots[p.first].space == Space::Tex)) {
    /* run-time index into a uniform block's array or an array of combined image samplers: clamped to the
     * array, then addressed directly */
    const Var& var = vars_[p.var];
    const Slot& s0 = var.slots[p.first];
    int32_t lim;
    if (p.rt) {
      /* the last element the bound range holds: (range - base - element bytes) / stride (recording checks
       * that the range covers the block with one element) */
      Inst r;
      r.op = Op::LdDescRange;
      r.ty = Ty::B32;
      r.dst = fn_.reg(Ty::B32);
      r.imm2 = s0.key;
      fn_.emit(r);
      int32_t avail = op2(Op::ISub, Ty::B32, r.dst, konst(Ty::B32, var.rt_base + var.rt_end));
      lim = op2(Op::UDiv, Ty::B32, avail, konst(Ty::B32, var.rt_stride));
    } else {
      lim = konst(Ty::B32, p.dyn_count - 1);
    }
    int32_t idx = op3(Op::Selp, Ty::B32, lim, p.dyn, op2(Op::SetpU, Ty::Pred, p.dyn, lim, CmpGt));
    v.type = p.type;
    v.regs.clear();
    if (s0.space == Space::Tex) {
      v.is_tex = v.tex_dyn = true;
      v.tex_key = s0.key;
      v.regs.push_back(op2(Op::IAdd, Ty::B32, idx, konst(Ty::B32, s0.offset)));
      return true;
    }
    uint32_t stride = p.rt ? var.rt_stride
                  : p.dyn_count > 1 && p.first + p.dyn_stride < var.slots.size()
                          ? var.slots[p.first + p.dyn_stride].offset - s0.offset
                          : 0;
    int32_t boff = op2(Op::IMul, Ty::B32, idx, konst(Ty::B32, stride));
    std::vector<Ty> tys;
    flat_types(p.type, tys);
    for (size_t k = 0; k < tys.size(); k++) {
      if (p.first + k >= var.slots.size()) return fail("load outside a variable");
      const Slot& s = var.slots[p.first + k];
      Ty t = tys[k] == Ty::Pred ? Ty::B32 : tys[k];
      Inst i;
      i.op = Op::LdUbo;
      i.ty = t;
      i.dst = fn_.reg(t);
      i.a = boff;
      i.imm = s.offset;
      i.imm2 = s.key;
      fn_.emit(i);
      v.regs.push_back(tys[k] == Ty::Pred ? op1(Op::B32ToP, Ty::Pred, i.dst) : i.dst);
    }
    return true;
  }
  if (p.dyn >= 0) {
    /* run-time index: load every candidate element and select the one the index names (an index out of
     * range reads element 0) */
    Place e = p;
    e.dyn = -1;
    Val acc;
    if (!load(e, acc)) return false;
    for (uint32_t k = 1; k < p.dyn_count; k++) {
      e.first = p.first + k * p.dyn_stride;
      Val cand;
      if (!load(e, cand)) return false;
      int32_t hit = op2(Op::SetpU, Ty::Pred, p.dyn, konst(Ty::B32, k), CmpEq);
      for (size_t c = 0; c < acc.regs.size(); c++) {
        Ty t = reg_ty(acc.regs[c]);
        if (t == Ty::Pred) {
          acc.regs[c] = op2(Op::POr, Ty::Pred, op2(Op::PAnd, Ty::Pred, hit, cand.regs[c]),
                            op2(Op::PAnd, Ty::Pred, op1(Op::PNot, Ty::Pred, hit), acc.regs[c]));
        } else {
          acc.regs[c] = op3(Op::Selp, t, cand.regs[c], acc.regs[c], hit);
        }
      }
    }
    v = acc;
    v.type = p.type;
    return true;
  }
  Var& var = vars_[p.var];
  std::vector<Ty> tys;
  flat_types(p.type, tys);
  v.type = p.type;
  v.regs.clear();
  if (p.first < var.slots.size() && var.slots[p.first].space == Space::Tex) {
    const TypeInfo& ti = ty(p.type);
    if (ti.kind != TypeInfo::SampledImage && ti.kind != TypeInfo::Image && ti.kind != TypeInfo::Sampler)
      return fail("load of a whole array of images or samplers");
    v.is_tex = true;
    v.tex_key = var.slots[p.first].key;
    v.tex_elem = var.slots[p.first].offset;
    return true;
  }
  for (size_t k = 0; k < tys.size(); k++) {
    if (p.first + k >= var.slots.size()) return fail("load outside a variable");
    const Slot& s = var.slots[p.first + k];
    switch (s.space) {
      case Space::In: {
        if (s.is_bool_in) {
          int32_t r = fn_.reg(Ty::B32);
          Inst i;
          i.op = Op::LdIn;
          i.ty = Ty::B32;
          i.dst = r;
          i.imm = s.offset;
          fn_.emit(i);
          v.regs.push_back(op1(Op::B32ToP, Ty::Pred, r));
        } else {
          int32_t r = fn_.reg(tys[k]);
          Inst i;
          i.op = Op::LdIn;
          i.ty = tys[k];
          i.dst = r;
          i.imm = s.offset;
          fn_.emit(i);
          v.regs.push_back(r);
        }
        break;
      }
      case Space::Push:
      case Space::Ubo: {
        Ty t = tys[k] == Ty::Pred ? Ty::B32 : tys[k];
        int32_t r = fn_.reg(t);
        Inst i;
        i.op = s.space == Space::Push ? Op::LdPush : Op::LdUbo;
        i.ty = t;
        i.dst = r;
        i.imm = s.offset;
        i.imm2 = s.key;
        fn_.emit(i);
        v.regs.push_back(tys[k] == Ty::Pred ? op1(Op::B32ToP, Ty::Pred, r) : r);
        break;
      }
      case Space::Out:
      case Space::Reg: {
        int32_t r = fn_.reg(tys[k]);
        mov(tys[k], r, s.reg);
        v.regs.push_back(r);
        break;
      }
      default: v.regs.push_back(konst(tys[k], 0)); break;
    }
  }
  return true;
}

bool Translator::store(const Place& p, const Val& v) {
  Var& var = vars_[p.var];
  if (p.rt || var.storage == SCUniform || var.storage == SCStorageBuffer)
    return fail("writes to uniform and storage buffers are not supported (shaders only read them)");
  if (p.dyn >= 0) {
    /* run-time index: every candidate element keeps its value unless the index names it */
    for (uint32_t e = 0; e < p.dyn_count; e++) {
      int32_t hit = op2(Op::SetpU, Ty::Pred, p.dyn, konst(Ty::B32, e), CmpEq);
      for (size_t k = 0; k < v.regs.size(); k++) {
        size_t idx = p.first + e * p.dyn_stride + k;
        if (idx >= var.slots.size()) return fail("store outside a variable");
        const Slot& s = var.slots[idx];
        if (!(s.space == Space::Out || s.space == Space::Reg)) {
          if (s.space == Space::None && var.storage == SCOutput) continue;
          return fail("store to a read-only variable");
        }
        Ty t = reg_ty(s.reg);
        int32_t nv;
        if (t == Ty::Pred)
          nv = op2(Op::POr, Ty::Pred, op2(Op::PAnd, Ty::Pred, hit, v.regs[k]),
                   op2(Op::PAnd, Ty::Pred, op1(Op::PNot, Ty::Pred, hit), s.reg));
        else
          nv = op3(Op::Selp, t, v.regs[k], s.reg, hit);
        mov(t, s.reg, nv);
      }
    }
    return true;
  }
  for (size_t k = 0; k < v.regs.size(); k++) {
    if (p.first + k >= var.slots.size()) return fail("store outside a variable");
    const Slot& s = var.slots[p.first + k];
    if (s.space == Space::Out || s.space == Space::Reg) mov(reg_ty(v.regs[k]), s.reg, v.regs[k]);
    else if (s.space == Space::None && var.storage == SCOutput) continue;
    else return fail("store to a read-only variable");
  }
  return true;
}

void Translator::finish_outputs() {
  for (auto& kv : vars_) {
    Var& v = kv.second;
    if (v.storage != SCOutput) continue;
    for (const Slot& s : v.slots) {
      if (s.space != Space::Out || s.reg < 0) continue;
      Inst i;
      i.op = Op::StOut;
      i.ty = reg_ty(s.reg);
      i.a = s.reg;
      i.imm = s.offset;
      fn_.emit(i);
    }
  }
}

int32_t Translator::dot(const std::vector<int32_t>& a, const std::vector<int32_t>& b, size_t n) {
  int32_t t = op2(Op::FMul, Ty::F32, a[0], b[0]);
  for (size_t k = 1; k < n; k++) t = op3(Op::FFma, Ty::F32, a[k], b[k], t);
  return t;
}

bool Translator::branch_to(uint32_t target) {
  auto it = phis_.find(target);
  if (it != phis_.end()) {
    std::vector<std::pair<int32_t, int32_t>> moves; /* (phi reg, temp) */
    for (const PhiInfo& ph : it->second) {
      const Val& dst = vals_[ph.result];
      for (auto& inc : ph.incoming) {
        if (inc.second != cur_block_) continue;
        Val* src = nullptr;
        auto c = vals_.find(inc.first);
        if (c != vals_.end()) src = &c->second;
        if (!src) return fail("OpPhi operand %" + std::to_string(inc.first) + " not available");
        for (size_t k = 0; k < dst.regs.size() && k < src->regs.size(); k++) {
          int32_t tmp = fn_.reg(reg_ty(dst.regs[k]));
          mov(reg_ty(dst.regs[k]), tmp, src->regs[k]);
          moves.push_back({dst.regs[k], tmp});
        }
      }
    }
    for (auto& mv : moves) mov(reg_ty(mv.first), mv.first, mv.second);
  }
  bra(label_of(target));
  return true;
}

bool Translator::ext_inst(const Insn& in) {
  const auto& o = in.ops;
  uint32_t rt = o[0], res = o[1], set = o[2], num = o[3];
  if (ext_sets_[set] != "GLSL.std.450") return fail("unsupported extended instruction set");
  std::vector<Val*> args;
  for (size_t i = 4; i < o.size(); i++) {
    Val* v = val(o[i]);
    if (!v) return false;
    args.push_back(v);
  }
  Val out;
  out.type = rt;
  uint32_t n = scalars(rt);
  auto need = [&](size_t k) { return args.size() >= k || fail("extended instruction with too few operands"); };
  auto per = [&](Op op) {
    for (uint32_t k = 0; k < n; k++) out.regs.push_back(op1(op, Ty::F32, args[0]->regs[k]));
  };
  auto per2 = [&](Op op, Ty t) {
    for (uint32_t k = 0; k < n; k++) out.regs.push_back(op2(op, t, args[0]->regs[k], args[1]->regs[k]));
  };
  /* scalar building blocks (each a separately rounded single operation) */
  auto F = [&](float v) {
    uint32_t b;
    std::memcpy(&b, &v, 4);
    return konst(Ty::F32, b);
  };
  auto I = [&](uint32_t v) { return konst(Ty::B32, v); };
  auto add = [&](int32_t a, int32_t b) { return op2(Op::FAdd, Ty::F32, a, b); };
  auto sub = [&](int32_t a, int32_t b) { return op2(Op::FSub, Ty::F32, a, b); };
  auto mul = [&](int32_t a, int32_t b) { return op2(Op::FMul, Ty::F32, a, b); };
  auto div = [&](int32_t a, int32_t b) { return op2(Op::FDiv, Ty::F32, a, b); };
  auto fma = [&](int32_t a, int32_t b, int32_t c) { return op3(Op::FFma, Ty::F32, a, b, c); };
  auto sel = [&](Ty t, int32_t p, int32_t a, int32_t b) { return op3(Op::Selp, t, a, b, p); };
  auto fcmp = [&](int32_t a, int32_t b, uint32_t c) { return op2(Op::SetpF, Ty::Pred, a, b, c); };
  auto scmp = [&](int32_t a, int32_t b, uint32_t c) { return op2(Op::SetpS, Ty::Pred, a, b, c); };
  /* e^x = 2^(x log2 e) and ln x = log2 x ln 2, with the hardware exp2 / log2 approximations */
  auto fexp = [&](int32_t x) { return op1(Op::FEx2, Ty::F32, mul(x, F(1.44269504f))); };
  auto flog = [&](int32_t x) { return mul(op1(Op::FLg2, Ty::F32, x), F(0.693147181f)); };
  /* arctangent: |x| reduced to [0, 1] by atan x = pi/2 - atan(1/x), then to [0, tan(pi/12)] by the addition
   * formula atan a = pi/6 + atan((a sqrt3 - 1) / (a + sqrt3)); there the Taylor series
   * t - t^3/3 + ... + t^13/13 (truncation below 3e-10 for t <= 0.268) in Horner form; the sign restored */
  auto fatan = [&](int32_t x) {
    int32_t a = op1(Op::FAbs, Ty::F32, x);
    int32_t big = fcmp(a, F(1.0f), CmpGt);
    a = sel(Ty::F32, big, div(F(1.0f), a), a);
    int32_t red = fcmp(a, F(0.267949192f), CmpGt);
    int32_t ar = div(sub(mul(a, F(1.73205081f)), F(1.0f)), add(a, F(1.73205081f)));
    int32_t t = sel(Ty::F32, red, ar, a);
    int32_t t2 = mul(t, t);
    int32_t p = F(1.0f / 13.0f);
    const float c[] = {-1.0f / 11.0f, 1.0f / 9.0f, -1.0f / 7.0f, 1.0f / 5.0f, -1.0f / 3.0f};
    for (float ck : c) p = fma(p, t2, F(ck));
    int32_t r = fma(mul(p, t2), t, t);
    r = sel(Ty::F32, red, add(r, F(0.523598776f)), r);
    r = sel(Ty::F32, big, sub(F(1.57079633f), r), r);
    return sel(Ty::F32, fcmp(x, F(0.0f), CmpLt), op1(Op::FNeg, Ty::F32, r), r);
  };
  /* atan2(y, x): atan(y / x) moved to the quadrant of (x, y) */
  auto fatan2 = [&](int32_t y, int32_t x) {
    int32_t r = fatan(div(y, x));
    int32_t neg_x = fcmp(x, F(0.0f), CmpLt);
    int32_t pi = sel(Ty::F32, fcmp(y, F(0.0f), CmpLt), F(-3.14159265f), F(3.14159265f));
    r = sel(Ty::F32, neg_x, add(r, pi), r);
    int32_t zx = fcmp(x, F(0.0f), CmpEq);
    int32_t half = sel(Ty::F32, fcmp(y, F(0.0f), CmpLt), F(-1.57079633f), F(1.57079633f));
    return sel(Ty::F32, zx, sel(Ty::F32, fcmp(y, F(0.0f), CmpEq), F(0.0f), half), r);
  };
  auto det2 = [&](int32_t a, int32_t b, int32_t c, int32_t d) { /* a d - b c */
    return fma(a, d, op1(Op::FNeg, Ty::F32, mul(b, c)));
  };
  switch (num) {
    case GFAbs: if (!need(1)) return false; per(Op::FAbs); break;
    case GFloor: if (!need(1)) return false; per(Op::FFloor); break;
    case GCeil: if (!need(1)) return false; per(Op::FCeil); break;
    case GTrunc: if (!need(1)) return false; per(Op::FTrunc); break;
    case GRoundEven:
    case GRound: if (!need(1)) return false; per(Op::FRoundEven); break;
    case GSqrt: if (!need(1)) return false; per(Op::FSqrt); break;
    case GSin: if (!need(1)) return false; per(Op::FSin); break;
    case GCos: if (!need(1)) return false; per(Op::FCos); break;
    case GExp2: if (!need(1)) return false; per(Op::FEx2); break;
    case GLog2: if (!need(1)) return false; per(Op::FLg2); break;
    case GInverseSqrt:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op2(Op::FDiv, Ty::F32, konst(Ty::F32, 0x3F800000u), op1(Op::FSqrt, Ty::F32, args[0]->regs[k])));
      break;
    case GFract:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op2(Op::FSub, Ty::F32, args[0]->regs[k], op1(Op::FFloor, Ty::F32, args[0]->regs[k])));
      break;
    case GFMin: if (!need(2)) return false; per2(Op::FMin, Ty::F32); break;
    case GFMax: if (!need(2)) return false; per2(Op::FMax, Ty::F32); break;
    case GFClamp:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op2(Op::FMin, Ty::F32, op2(Op::FMax, Ty::F32, args[0]->regs[k], args[1]->regs[k]),
                               args[2]->regs[k]));
      break;
    case GFMix:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op3(Op::FFma, Ty::F32, args[2]->regs[k],
                               op2(Op::FSub, Ty::F32, args[1]->regs[k], args[0]->regs[k]), args[0]->regs[k]));
      break;
    case GFma:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op3(Op::FFma, Ty::F32, args[0]->regs[k], args[1]->regs[k], args[2]->regs[k]));
      break;
    case GStep:
      if (!need(2)) return false;
      /* step(edge, x) = x < edge ? 0 : 1 */
      for (uint32_t k = 0; k < n; k++) {
        int32_t p = op2(Op::SetpF, Ty::Pred, args[1]->regs[k], args[0]->regs[k], CmpLt);
        out.regs.push_back(op3(Op::Selp, Ty::F32, konst(Ty::F32, 0), konst(Ty::F32, 0x3F800000u), p));
      }
      break;
    case GSMin: if (!need(2)) return false; for (uint32_t k = 0; k < n; k++) { int32_t p = op2(Op::SetpS, Ty::Pred, args[0]->regs[k], args[1]->regs[k], CmpLt); out.regs.push_back(op3(Op::Selp, Ty::B32, args[0]->regs[k], args[1]->regs[k], p)); } break;
    case GSMax: if (!need(2)) return false; for (uint32_t k = 0; k < n; k++) { int32_t p = op2(Op::SetpS, Ty::Pred, args[0]->regs[k], args[1]->regs[k], CmpGt); out.regs.push_back(op3(Op::Selp, Ty::B32, args[0]->regs[k], args[1]->regs[k], p)); } break;
    case GUMin: if (!need(2)) return false; for (uint32_t k = 0; k < n; k++) { int32_t p = op2(Op::SetpU, Ty::Pred, args[0]->regs[k], args[1]->regs[k], CmpLt); out.regs.push_back(op3(Op::Selp, Ty::B32, args[0]->regs[k], args[1]->regs[k], p)); } break;
    case GUMax: if (!need(2)) return false; for (uint32_t k = 0; k < n; k++) { int32_t p = op2(Op::SetpU, Ty::Pred, args[0]->regs[k], args[1]->regs[k], CmpGt); out.regs.push_back(op3(Op::Selp, Ty::B32, args[0]->regs[k], args[1]->regs[k], p)); } break;
    case GLength: {
      if (!need(1)) return false;
      size_t m = args[0]->regs.size();
      out.regs.push_back(op1(Op::FSqrt, Ty::F32, dot(args[0]->regs, args[0]->regs, m)));
      break;
    }
    case GDistance: {
      if (!need(2)) return false;
      size_t m = args[0]->regs.size();
      std::vector<int32_t> d;
      for (size_t k = 0; k < m; k++) d.push_back(op2(Op::FSub, Ty::F32, args[0]->regs[k], args[1]->regs[k]));
      out.regs.push_back(op1(Op::FSqrt, Ty::F32, dot(d, d, m)));
      break;
    }
    case GNormalize: {
      if (!need(1)) return false;
      size_t m = args[0]->regs.size();
      int32_t len = op1(Op::FSqrt, Ty::F32, dot(args[0]->regs, args[0]->regs, m));
      int32_t inv = op2(Op::FDiv, Ty::F32, konst(Ty::F32, 0x3F800000u), len);
      for (size_t k = 0; k < m; k++) out.regs.push_back(op2(Op::FMul, Ty::F32, args[0]->regs[k], inv));
      break;
    }
    case GCross: {
      if (!need(2)) return false;
      const auto& a = args[0]->regs;
      const auto& b = args[1]->regs;
      /* cross = a.yzx * b.zxy - a.zxy * b.yzx, each component as fma(a1, b2, -(a2 * b1)) */
      int idx[3][4] = {{1, 2, 2, 1}, {2, 0, 0, 2}, {0, 1, 1, 0}};
      for (int k = 0; k < 3; k++) {
        int32_t t = op1(Op::FNeg, Ty::F32, op2(Op::FMul, Ty::F32, a[idx[k][2]], b[idx[k][3]]));
        out.regs.push_back(op3(Op::FFma, Ty::F32, a[idx[k][0]], b[idx[k][1]], t));
      }
      break;
    }
    case GPow: {
      if (!need(2)) return false;
      /* pow(x, y) = exp2(y * log2(x)) with the hardware approximations */
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op1(Op::FEx2, Ty::F32, op2(Op::FMul, Ty::F32, args[1]->regs[k], op1(Op::FLg2, Ty::F32, args[0]->regs[k]))));
      break;
    }
    case GSAbs:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) {
        int32_t x = args[0]->regs[k];
        out.regs.push_back(sel(Ty::B32, scmp(x, I(0), CmpLt), op1(Op::INeg, Ty::B32, x), x));
      }
      break;
    case GFSign:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) {
        int32_t x = args[0]->regs[k];
        out.regs.push_back(sel(Ty::F32, fcmp(x, F(0.0f), CmpGt), F(1.0f),
                               sel(Ty::F32, fcmp(x, F(0.0f), CmpLt), F(-1.0f), F(0.0f))));
      }
      break;
    case GSSign:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) {
        int32_t x = args[0]->regs[k];
        out.regs.push_back(sel(Ty::B32, scmp(x, I(0), CmpGt), I(1), sel(Ty::B32, scmp(x, I(0), CmpLt), I(~0u), I(0))));
      }
      break;
    case GRadians:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(mul(args[0]->regs[k], F(0.0174532925f)));
      break;
    case GDegrees:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(mul(args[0]->regs[k], F(57.2957795f)));
      break;
    case GTan:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(div(op1(Op::FSin, Ty::F32, args[0]->regs[k]), op1(Op::FCos, Ty::F32, args[0]->regs[k])));
      break;
    case GExp:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(fexp(args[0]->regs[k]));
      break;
    case GLog:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(flog(args[0]->regs[k]));
      break;
    case GSinh:
    case GCosh:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) {
        int32_t e = fexp(args[0]->regs[k]), ei = div(F(1.0f), e);
        out.regs.push_back(mul(num == GSinh ? sub(e, ei) : add(e, ei), F(0.5f)));
      }
      break;
    case GTanh:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) { /* (e^2x - 1) / (e^2x + 1), |x| clamped to 10 (tanh 10 rounds to 1) */
        int32_t x = op2(Op::FMin, Ty::F32, op2(Op::FMax, Ty::F32, args[0]->regs[k], F(-10.0f)), F(10.0f));
        int32_t e = fexp(add(x, x));
        out.regs.push_back(div(sub(e, F(1.0f)), add(e, F(1.0f))));
      }
      break;
    case GAsinh:
    case GAcosh:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) {
        int32_t x = args[0]->regs[k];
        if (num == GAsinh) { /* sign(x) ln(|x| + sqrt(x^2 + 1)) */
          int32_t a = op1(Op::FAbs, Ty::F32, x);
          int32_t r = flog(add(a, op1(Op::FSqrt, Ty::F32, fma(a, a, F(1.0f)))));
          out.regs.push_back(sel(Ty::F32, fcmp(x, F(0.0f), CmpLt), op1(Op::FNeg, Ty::F32, r), r));
        } else { /* ln(x + sqrt(x^2 - 1)) */
          out.regs.push_back(flog(add(x, op1(Op::FSqrt, Ty::F32, fma(x, x, F(-1.0f))))));
        }
      }
      break;
    case GAtanh:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) { /* ln((1 + x) / (1 - x)) / 2 */
        int32_t x = args[0]->regs[k];
        out.regs.push_back(mul(flog(div(add(F(1.0f), x), sub(F(1.0f), x))), F(0.5f)));
      }
      break;
    case GAtan:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(fatan(args[0]->regs[k]));
      break;
    case GAtan2:
      if (!need(2)) return false;
      for (uint32_t k = 0; k < n; k++) out.regs.push_back(fatan2(args[0]->regs[k], args[1]->regs[k]));
      break;
    case GAsin:
    case GAcos:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) { /* asin x = atan2(x, sqrt(1 - x^2)), acos x = atan2(sqrt(1 - x^2), x) */
        int32_t x = args[0]->regs[k];
        int32_t c = op1(Op::FSqrt, Ty::F32, fma(op1(Op::FNeg, Ty::F32, x), x, F(1.0f)));
        out.regs.push_back(num == GAsin ? fatan2(x, c) : fatan2(c, x));
      }
      break;
    case GSClamp:
    case GUClamp:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++) {
        Op cmp = num == GSClamp ? Op::SetpS : Op::SetpU;
        int32_t x = args[0]->regs[k], lo = args[1]->regs[k], hi = args[2]->regs[k];
        int32_t m = sel(Ty::B32, op2(cmp, Ty::Pred, x, lo, CmpLt), lo, x);
        out.regs.push_back(sel(Ty::B32, op2(cmp, Ty::Pred, m, hi, CmpGt), hi, m));
      }
      break;
    case GNMin: if (!need(2)) return false; per2(Op::FMin, Ty::F32); break;
    case GNMax: if (!need(2)) return false; per2(Op::FMax, Ty::F32); break;
    case GNClamp:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++)
        out.regs.push_back(op2(Op::FMin, Ty::F32, op2(Op::FMax, Ty::F32, args[0]->regs[k], args[1]->regs[k]),
                               args[2]->regs[k]));
      break;
    case GSmoothStep:
      if (!need(3)) return false;
      for (uint32_t k = 0; k < n; k++) { /* t = clamp((x - e0) / (e1 - e0), 0, 1); t t (3 - 2 t) */
        int32_t e0 = args[0]->regs[k], e1 = args[1]->regs[k], x = args[2]->regs[k];
        int32_t t = div(sub(x, e0), sub(e1, e0));
        t = op2(Op::FMin, Ty::F32, op2(Op::FMax, Ty::F32, t, F(0.0f)), F(1.0f));
        out.regs.push_back(mul(mul(t, t), fma(F(-2.0f), t, F(3.0f))));
      }
      break;
    case GFaceForward: {
      if (!need(3)) return false; /* dot(Nref, I) < 0 ? N : -N */
      size_t m = args[0]->regs.size();
      int32_t p = fcmp(dot(args[2]->regs, args[1]->regs, m), F(0.0f), CmpLt);
      for (size_t k = 0; k < m; k++)
        out.regs.push_back(sel(Ty::F32, p, args[0]->regs[k], op1(Op::FNeg, Ty::F32, args[0]->regs[k])));
      break;
    }
    case GReflect: {
      if (!need(2)) return false; /* I - 2 dot(N, I) N */
      size_t m = args[0]->regs.size();
      int32_t d2 = mul(F(2.0f), dot(args[1]->regs, args[0]->regs, m));
      for (size_t k = 0; k < m; k++)
        out.regs.push_back(fma(op1(Op::FNeg, Ty::F32, d2), args[1]->regs[k], args[0]->regs[k]));
      break;
    }
    case GRefract: {
      if (!need(3)) return false; /* k = 1 - eta^2 (1 - dot(N, I)^2); k < 0 ? 0 : eta I - (eta dot(N, I) + sqrt k) N */
      size_t m = args[0]->regs.size();
      int32_t eta = args[2]->regs[0];
      int32_t d = dot(args[1]->regs, args[0]->regs, m);
      int32_t kk = sub(F(1.0f), mul(mul(eta, eta), fma(op1(Op::FNeg, Ty::F32, d), d, F(1.0f))));
      int32_t neg = fcmp(kk, F(0.0f), CmpLt);
      int32_t f = fma(eta, d, op1(Op::FSqrt, Ty::F32, kk));
      for (size_t k = 0; k < m; k++) {
        int32_t r = fma(eta, args[0]->regs[k], op1(Op::FNeg, Ty::F32, mul(f, args[1]->regs[k])));
        out.regs.push_back(sel(Ty::F32, neg, F(0.0f), r));
      }
      break;
    }
    case GLdexp:
      if (!need(2)) return false;
      for (uint32_t k = 0; k < n; k++) { /* x 2^e as two exact power-of-two products, e clamped to [-252, 254] */
        int32_t e = args[1]->regs[k];
        e = sel(Ty::B32, scmp(e, I((uint32_t)-252), CmpLt), I((uint32_t)-252), e);
        e = sel(Ty::B32, scmp(e, I(254), CmpGt), I(254), e);
        int32_t e1 = op2(Op::Sar, Ty::B32, e, I(1)), e2 = op2(Op::ISub, Ty::B32, e, e1);
        int32_t p1 = op2(Op::Shl, Ty::B32, op2(Op::IAdd, Ty::B32, e1, I(127)), I(23));
        int32_t p2 = op2(Op::Shl, Ty::B32, op2(Op::IAdd, Ty::B32, e2, I(127)), I(23));
        out.regs.push_back(mul(mul(args[0]->regs[k], p1), p2));
      }
      break;
    case GFindILsb:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) { /* x == 0 ? -1 : popc((x & -x) - 1) */
        int32_t x = args[0]->regs[k];
        int32_t low = op2(Op::And, Ty::B32, x, op1(Op::INeg, Ty::B32, x));
        int32_t r = op1(Op::Popc, Ty::B32, op2(Op::ISub, Ty::B32, low, I(1)));
        out.regs.push_back(sel(Ty::B32, op2(Op::SetpU, Ty::Pred, x, I(0), CmpEq), I(~0u), r));
      }
      break;
    case GFindUMsb:
    case GFindSMsb:
      if (!need(1)) return false;
      for (uint32_t k = 0; k < n; k++) { /* 31 - clz(x) (for signed: of ~x when x < 0); -1 when no bit */
        int32_t x = args[0]->regs[k];
        if (num == GFindSMsb) x = sel(Ty::B32, scmp(x, I(0), CmpLt), op1(Op::Not, Ty::B32, x), x);
        out.regs.push_back(op2(Op::ISub, Ty::B32, I(31), op1(Op::Clz, Ty::B32, x)));
      }
      break;
    case GPackUnorm4x8:
    case GPackSnorm4x8: {
      if (!need(1)) return false; /* rint(clamp(c) * 255 or 127), bytes from component 0 up */
      bool sn = num == GPackSnorm4x8;
      int32_t acc = I(0);
      for (int k = 0; k < 4; k++) {
        int32_t c = op2(Op::FMin, Ty::F32, op2(Op::FMax, Ty::F32, args[0]->regs[k], F(sn ? -1.0f : 0.0f)), F(1.0f));
        int32_t q = op1(Op::CvtF2S, Ty::B32, op1(Op::FRoundEven, Ty::F32, mul(c, F(sn ? 127.0f : 255.0f))));
        acc = op2(Op::Or, Ty::B32, acc, op2(Op::Shl, Ty::B32, op2(Op::And, Ty::B32, q, I(0xFF)), I(8 * k)));
      }
      out.regs.push_back(acc);
      break;
    }
    case GUnpackUnorm4x8:
    case GUnpackSnorm4x8: {
      if (!need(1)) return false; /* byte / 255, or clamp(signed byte / 127, -1, 1) */
      bool sn = num == GUnpackSnorm4x8;
      for (int k = 0; k < 4; k++) {
        Inst b;
        b.op = Op::Bfe;
        b.ty = Ty::B32;
        b.dst = fn_.reg(Ty::B32);
        b.a = args[0]->regs[0];
        b.b = I(8 * k);
        b.c = I(8);
        b.imm = sn ? 1 : 0;
        fn_.emit(b);
        int32_t f = op1(sn ? Op::CvtS2F : Op::CvtU2F, Ty::F32, b.dst);
        f = div(f, F(sn ? 127.0f : 255.0f));
        if (sn) f = op2(Op::FMax, Ty::F32, f, F(-1.0f));
        out.regs.push_back(f);
      }
      break;
    }
    case GPackHalf2x16:
      if (!need(1)) return false;
      out.regs.push_back(op2(Op::Or, Ty::B32, op1(Op::F2H, Ty::B32, args[0]->regs[0]),
                             op2(Op::Shl, Ty::B32, op1(Op::F2H, Ty::B32, args[0]->regs[1]), I(16))));
      break;
    case GUnpackHalf2x16:
      if (!need(1)) return false;
      out.regs.push_back(op1(Op::H2F, Ty::F32, op2(Op::And, Ty::B32, args[0]->regs[0], I(0xFFFF))));
      out.regs.push_back(op1(Op::H2F, Ty::F32, op2(Op::Shr, Ty::B32, args[0]->regs[0], I(16))));
      break;
    case GModfStruct:
      if (!need(1)) return false; /* { x - trunc(x), trunc(x) } */
      for (uint32_t k = 0; k < args[0]->regs.size(); k++)
        out.regs.push_back(sub(args[0]->regs[k], op1(Op::FTrunc, Ty::F32, args[0]->regs[k])));
      for (uint32_t k = 0; k < args[0]->regs.size(); k++) out.regs.push_back(op1(Op::FTrunc, Ty::F32, args[0]->regs[k]));
      break;
    case GDeterminant: {
      if (!need(1)) return false;
      const auto& a = args[0]->regs; /* column-major: element (row r, column c) at c * N + r */
      size_t N = a.size() == 4 ? 2 : a.size() == 9 ? 3 : 4;
      auto at = [&](size_t r, size_t c) { return a[c * N + r]; };
      if (N == 2) {
        out.regs.push_back(det2(at(0, 0), at(0, 1), at(1, 0), at(1, 1)));
      } else if (N == 3) { /* expansion along row 0 */
        int32_t c0 = det2(at(1, 1), at(1, 2), at(2, 1), at(2, 2));
        int32_t c1 = det2(at(1, 0), at(1, 2), at(2, 0), at(2, 2));
        int32_t c2 = det2(at(1, 0), at(1, 1), at(2, 0), at(2, 1));
        out.regs.push_back(fma(at(0, 2), c2, fma(op1(Op::FNeg, Ty::F32, at(0, 1)), c1, mul(at(0, 0), c0))));
      } else { /* Laplace expansion by the 2x2 minors of rows 0-1 and 2-3 */
        int32_t s[6], c[6];
        const int pr[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
        for (int k = 0; k < 6; k++) {
          s[k] = det2(at(0, pr[k][0]), at(0, pr[k][1]), at(1, pr[k][0]), at(1, pr[k][1]));
          c[k] = det2(at(2, pr[k][0]), at(2, pr[k][1]), at(3, pr[k][0]), at(3, pr[k][1]));
        }
        int32_t d = mul(s[0], c[5]);
        d = fma(op1(Op::FNeg, Ty::F32, s[1]), c[4], d);
        d = fma(s[2], c[3], d);
        d = fma(s[3], c[2], d);
        d = fma(op1(Op::FNeg, Ty::F32, s[4]), c[1], d);
        d = fma(s[5], c[0], d);
        out.regs.push_back(d);
      }
      break;
    }
    case GMatrixInverse: {
      if (!need(1)) return false;
      const auto& a = args[0]->regs;
      size_t N = a.size() == 4 ? 2 : a.size() == 9 ? 3 : 4;
      auto at = [&](size_t r, size_t c) { return a[c * N + r]; };
      /* the adjugate divided by the determinant: cofactor C(r, c) = (-1)^(r+c) minor(r, c); inverse(c, r) = C / det */
      auto minor = [&](size_t r, size_t c) -> int32_t {
        std::vector<size_t> rs, cs;
        for (size_t i = 0; i < N; i++) {
          if (i != r) rs.push_back(i);
          if (i != c) cs.push_back(i);
        }
        if (N == 2) return at(rs[0], cs[0]);
        if (N == 3) return det2(at(rs[0], cs[0]), at(rs[0], cs[1]), at(rs[1], cs[0]), at(rs[1], cs[1]));
        int32_t c0 = det2(at(rs[1], cs[1]), at(rs[1], cs[2]), at(rs[2], cs[1]), at(rs[2], cs[2]));
        int32_t c1 = det2(at(rs[1], cs[0]), at(rs[1], cs[2]), at(rs[2], cs[0]), at(rs[2], cs[2]));
        int32_t c2 = det2(at(rs[1], cs[0]), at(rs[1], cs[1]), at(rs[2], cs[0]), at(rs[2], cs[1]));
        return fma(at(rs[0], cs[2]), c2, fma(op1(Op::FNeg, Ty::F32, at(rs[0], cs[1])), c1, mul(at(rs[0], cs[0]), c0)));
      };
      std::vector<int32_t> cof(N * N);
      for (size_t r = 0; r < N; r++)
        for (size_t c = 0; c < N; c++) {
          int32_t m = minor(r, c);
          cof[r * N + c] = ((r + c) & 1) ? op1(Op::FNeg, Ty::F32, m) : m;
        }
      int32_t det = mul(at(0, 0), cof[0]);
      for (size_t c = 1; c < N; c++) det = fma(at(0, c), cof[c], det);
      int32_t inv = div(F(1.0f), det);
      out.regs.assign(N * N, -1);
      for (size_t r = 0; r < N; r++)
        for (size_t c = 0; c < N; c++) out.regs[r * N + c] = mul(cof[r * N + c], inv); /* inverse(c, r), column r */
      break;
    }
    default: return fail("unsupported GLSL.std.450 instruction " + std::to_string(num));
  }
  vals_[res] = out;
  return true;
}

bool Translator::do_insn(const Insn& in) {
  const auto& o = in.ops;
  auto unary_f = [&](Op op) {
    Val* a = val(o[2]);
    if (!a) return false;
    Val r;
    r.type = o[0];
    for (int32_t x : a->regs) r.regs.push_back(op1(op, Ty::F32, x));
    vals_[o[1]] = r;
    return true;
  };
  auto binary = [&](Op op, Ty t) {
    Val* a = val(o[2]);
    Val* b = val(o[3]);
    if (!a || !b) return false;
    Val r;
    r.type = o[0];
    for (size_t k = 0; k < a->regs.size() && k < b->regs.size(); k++) r.regs.push_back(op2(op, t, a->regs[k], b->regs[k]));
    vals_[o[1]] = r;
    return true;
  };
  auto compare = [&](Op op, uint32_t cmp) {
    Val* a = val(o[2]);
    Val* b = val(o[3]);
    if (!a || !b) return false;
    Val r;
    r.type = o[0];
    for (size_t k = 0; k < a->regs.size() && k < b->regs.size(); k++)
      r.regs.push_back(op2(op, Ty::Pred, a->regs[k], b->regs[k], cmp));
    vals_[o[1]] = r;
    return true;
  };
  switch (in.opcode) {
    case OpLine:
    case OpNop:
    case OpSelectionMerge:
    case OpLoopMerge:
    case OpName:
    case OpMemberName:
    case OpPhi: /* registers allocated in the pre-scan; moves emitted on the incoming edges */
      return true;
    case OpLabel:
      cur_block_ = o[0];
      label(label_of(o[0]));
      return true;
    case OpVariable: {
      Var v;
      v.storage = SCFunction;
      v.type = ty(o[0]).elem;
      if (!layout_interface(o[1], v)) return false;
      if (o.size() > 3) {
        Val* init = val(o[3]);
        if (!init) return false;
        for (size_t k = 0; k < v.slots.size() && k < init->regs.size(); k++) mov(reg_ty(v.slots[k].reg), v.slots[k].reg, init->regs[k]);
      }
      vars_[o[1]] = v;
      Place p;
      p.var = o[1];
      p.type = v.type;
      places_[o[1]] = p;
      return true;
    }
    case OpAccessChain:
    case OpInBoundsAccessChain: {
      auto it = places_.find(o[2]);
      if (it == places_.end()) return fail("access chain on something that is not a variable");
      Place p = it->second;
      for (size_t i = 3; i < o.size(); i++) {
        if (ty(p.type).kind == TypeInfo::RuntimeArray) {
          /* an element of a storage block's runtime-sized array: a run-time index (a constant one too),
           * limited by the bound range when it is loaded */
          if (!vars_[p.var].has_rt || p.dyn >= 0) return fail("unsupported access to a runtime-sized array");
          auto ci = consts_.find(o[i]);
          int32_t reg;
          if (ci != consts_.end() && !ci->second.second.empty()) {
            reg = konst(Ty::B32, ci->second.second[0]);
          } else {
            Val* iv = val(o[i]);
            if (!iv || iv->regs.empty() || reg_ty(iv->regs[0]) != Ty::B32) return fail("bad run-time index");
            reg = iv->regs[0];
          }
          p.dyn = reg;
          p.dyn_stride = scalars(ty(p.type).elem);
          p.dyn_count = 0;
          p.rt = true;
          p.type = ty(p.type).elem;
          continue;
        }
        auto c = consts_.find(o[i]);
        if (c == consts_.end() || c->second.second.empty()) {
          /* an index known at run time: into an array, matrix or vector (one such index per chain) */
          const TypeInfo& ti = ty(p.type);
          if (ti.kind != TypeInfo::Array && ti.kind != TypeInfo::Matrix && ti.kind != TypeInfo::Vector)
            return fail("run-time index into a struct");
          if (!ti.count) return fail("run-time index into a runtime-sized array");
          if (p.dyn >= 0) return fail("more than one run-time index in an access chain");
          Val* iv = val(o[i]);
          if (!iv || iv->regs.empty() || reg_ty(iv->regs[0]) != Ty::B32) return fail("bad run-time index");
          p.dyn = iv->regs[0];
          p.dyn_stride = scalars(ti.elem);
          p.dyn_count = ti.count;
          p.type = ti.elem;
          continue;
        }
        uint32_t off, mt;
        if (!member(p.type, c->second.second[0], off, mt)) return false;
        p.first += off;
        p.type = mt;
      }
      places_[o[1]] = p;
      return true;
    }
    case OpLoad: {
      auto it = places_.find(o[2]);
      if (it == places_.end()) return fail("load through an unknown pointer");
      Val v;
      if (!load(it->second, v)) return false;
      v.type = o[0];
      vals_[o[1]] = v;
      return true;
    }
    case OpStore: {
      auto it = places_.find(o[0]);
      if (it == places_.end()) return fail("store through an unknown pointer");
      Val* v = val(o[1]);
      if (!v) return false;
      return store(it->second, *v);
    }
    case OpVectorExtractDynamic: { /* component `index` of a vector (out of range: component 0) */
      Val* vec = val(o[2]);
      Val* ix = val(o[3]);
      if (!vec || !ix || vec->regs.empty() || ix->regs.empty()) return false;
      int32_t acc = vec->regs[0];
      for (uint32_t k = 1; k < vec->regs.size(); k++) {
        int32_t hit = op2(Op::SetpU, Ty::Pred, ix->regs[0], konst(Ty::B32, k), CmpEq);
        acc = op3(Op::Selp, reg_ty(acc), vec->regs[k], acc, hit);
      }
      Val r;
      r.type = o[0];
      r.regs.push_back(acc);
      vals_[o[1]] = r;
      return true;
    }
    case OpVectorInsertDynamic: { /* the vector with component `index` replaced */
      Val* vec = val(o[2]);
      Val* comp = val(o[3]);
      Val* ix = val(o[4]);
      if (!vec || !comp || !ix || comp->regs.empty() || ix->regs.empty()) return false;
      Val r;
      r.type = o[0];
      for (uint32_t k = 0; k < vec->regs.size(); k++) {
        int32_t hit = op2(Op::SetpU, Ty::Pred, ix->regs[0], konst(Ty::B32, k), CmpEq);
        r.regs.push_back(op3(Op::Selp, reg_ty(vec->regs[k]), comp->regs[0], vec->regs[k], hit));
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpCopyObject:
    case OpImage: { /* the image of a combined image sampler: the same binding and element */
      Val* a = val(o[2]);
      if (!a) return false;
      vals_[o[1]] = *a;
      vals_[o[1]].type = o[0];
      return true;
    }
    case OpSampledImage: { /* a separate image and sampler combined: the image's binding, the sampler's state */
      Val* img = val(o[2]);
      Val* smp = val(o[3]);
      if (!img || !smp || !img->is_tex || !smp->is_tex) return fail("OpSampledImage of something that is not a descriptor");
      if (smp->tex_dyn) return fail("run-time indices into arrays of samplers are not supported");
      Val r = *img;
      r.type = o[0];
      r.has_smp = true;
      r.smp_key = smp->tex_key;
      r.smp_elem = smp->tex_elem;
      vals_[o[1]] = r;
      return true;
    }
    case OpImageSampleImplicitLod:
    case OpImageSampleExplicitLod:
    case OpImageSampleProjImplicitLod:
    case OpImageSampleProjExplicitLod:
    case OpImageFetch:
      return image_sample(in);
    case OpUndef: {
      std::vector<Ty> tys;
      flat_types(o[0], tys);
      Val r;
      r.type = o[0];
      for (Ty t : tys) r.regs.push_back(konst(t, 0));
      vals_[o[1]] = r;
      return true;
    }
    case OpCompositeConstruct: {
      Val r;
      r.type = o[0];
      for (size_t i = 2; i < o.size(); i++) {
        Val* a = val(o[i]);
        if (!a) return false;
        r.regs.insert(r.regs.end(), a->regs.begin(), a->regs.end());
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpCompositeExtract: {
      Val* a = val(o[2]);
      if (!a) return false;
      uint32_t t = a->type, first = 0;
      for (size_t i = 3; i < o.size(); i++) {
        uint32_t off, mt;
        if (!member(t, o[i], off, mt)) return false;
        first += off;
        t = mt;
      }
      Val r;
      r.type = o[0];
      uint32_t n = scalars(t);
      for (uint32_t k = 0; k < n; k++) r.regs.push_back(a->regs[first + k]);
      vals_[o[1]] = r;
      return true;
    }
    case OpCompositeInsert: {
      Val* obj = val(o[2]);
      Val* comp = val(o[3]);
      if (!obj || !comp) return false;
      uint32_t t = comp->type, first = 0;
      for (size_t i = 4; i < o.size(); i++) {
        uint32_t off, mt;
        if (!member(t, o[i], off, mt)) return false;
        first += off;
        t = mt;
      }
      Val r = *comp;
      r.type = o[0];
      for (size_t k = 0; k < obj->regs.size(); k++) r.regs[first + k] = obj->regs[k];
      vals_[o[1]] = r;
      return true;
    }
    case OpVectorShuffle: {
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      Val r;
      r.type = o[0];
      for (size_t i = 4; i < o.size(); i++) {
        uint32_t s = o[i];
        if (s == 0xFFFFFFFFu) r.regs.push_back(konst(Ty::F32, 0));
        else if (s < a->regs.size()) r.regs.push_back(a->regs[s]);
        else r.regs.push_back(b->regs[s - a->regs.size()]);
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpFAdd: return binary(Op::FAdd, Ty::F32);
    case OpFSub: return binary(Op::FSub, Ty::F32);
    case OpFMul: return binary(Op::FMul, Ty::F32);
    case OpFDiv: return binary(Op::FDiv, Ty::F32);
    case OpFNegate: return unary_f(Op::FNeg);
    case OpIAdd: return binary(Op::IAdd, Ty::B32);
    case OpISub: return binary(Op::ISub, Ty::B32);
    case OpIMul: return binary(Op::IMul, Ty::B32);
    case OpUDiv: return binary(Op::UDiv, Ty::B32);
    case OpSDiv: return binary(Op::SDiv, Ty::B32);
    case OpUMod: return binary(Op::URem, Ty::B32);
    case OpSRem: return binary(Op::SRem, Ty::B32);
    case OpBitwiseAnd: return binary(Op::And, Ty::B32);
    case OpBitwiseOr: return binary(Op::Or, Ty::B32);
    case OpBitwiseXor: return binary(Op::Xor, Ty::B32);
    case OpShiftLeftLogical: return binary(Op::Shl, Ty::B32);
    case OpShiftRightLogical: return binary(Op::Shr, Ty::B32);
    case OpShiftRightArithmetic: return binary(Op::Sar, Ty::B32);
    case OpNot:
    case OpSNegate: {
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) r.regs.push_back(op1(in.opcode == OpNot ? Op::Not : Op::INeg, Ty::B32, x));
      vals_[o[1]] = r;
      return true;
    }
    case OpLogicalAnd: return binary(Op::PAnd, Ty::Pred);
    case OpLogicalOr: return binary(Op::POr, Ty::Pred);
    case OpLogicalNotEqual: return binary(Op::PXor, Ty::Pred);
    case OpLogicalEqual: {
      if (!binary(Op::PXor, Ty::Pred)) return false;
      for (int32_t& x : vals_[o[1]].regs) x = op1(Op::PNot, Ty::Pred, x);
      return true;
    }
    case OpLogicalNot: {
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) r.regs.push_back(op1(Op::PNot, Ty::Pred, x));
      vals_[o[1]] = r;
      return true;
    }
    case OpSelect: {
      Val* c = val(o[2]);
      Val* a = val(o[3]);
      Val* b = val(o[4]);
      if (!c || !a || !b) return false;
      Val r;
      r.type = o[0];
      for (size_t k = 0; k < a->regs.size(); k++) {
        int32_t p = c->regs.size() == 1 ? c->regs[0] : c->regs[k];
        Ty t = reg_ty(a->regs[k]);
        if (t == Ty::Pred) {
          int32_t x = op2(Op::PAnd, Ty::Pred, p, a->regs[k]);
          int32_t y = op2(Op::PAnd, Ty::Pred, op1(Op::PNot, Ty::Pred, p), b->regs[k]);
          r.regs.push_back(op2(Op::POr, Ty::Pred, x, y));
        } else {
          r.regs.push_back(op3(Op::Selp, t, a->regs[k], b->regs[k], p));
        }
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpIEqual: return compare(Op::SetpU, CmpEq);
    case OpINotEqual: return compare(Op::SetpU, CmpNe);
    case OpUGreaterThan: return compare(Op::SetpU, CmpGt);
    case OpSGreaterThan: return compare(Op::SetpS, CmpGt);
    case OpUGreaterThanEqual: return compare(Op::SetpU, CmpGe);
    case OpSGreaterThanEqual: return compare(Op::SetpS, CmpGe);
    case OpULessThan: return compare(Op::SetpU, CmpLt);
    case OpSLessThan: return compare(Op::SetpS, CmpLt);
    case OpULessThanEqual: return compare(Op::SetpU, CmpLe);
    case OpSLessThanEqual: return compare(Op::SetpS, CmpLe);
    case OpFOrdEqual: return compare(Op::SetpF, CmpEq);
    case OpFUnordEqual: return compare(Op::SetpF, CmpEq | CmpUnordered);
    case OpFOrdNotEqual: return compare(Op::SetpF, CmpNe);
    case OpFUnordNotEqual: return compare(Op::SetpF, CmpNe | CmpUnordered);
    case OpFOrdLessThan: return compare(Op::SetpF, CmpLt);
    case OpFUnordLessThan: return compare(Op::SetpF, CmpLt | CmpUnordered);
    case OpFOrdGreaterThan: return compare(Op::SetpF, CmpGt);
    case OpFUnordGreaterThan: return compare(Op::SetpF, CmpGt | CmpUnordered);
    case OpFOrdLessThanEqual: return compare(Op::SetpF, CmpLe);
    case OpFUnordLessThanEqual: return compare(Op::SetpF, CmpLe | CmpUnordered);
    case OpFOrdGreaterThanEqual: return compare(Op::SetpF, CmpGe);
    case OpFUnordGreaterThanEqual: return compare(Op::SetpF, CmpGe | CmpUnordered);
    case OpIsNan: {
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) r.regs.push_back(op2(Op::SetpF, Ty::Pred, x, x, CmpNe | CmpUnordered));
      vals_[o[1]] = r;
      return true;
    }
    case OpIsInf: { /* |x| == +inf */
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs)
        r.regs.push_back(op2(Op::SetpF, Ty::Pred, op1(Op::FAbs, Ty::F32, x), konst(Ty::F32, 0x7F800000u), CmpEq));
      vals_[o[1]] = r;
      return true;
    }
    case OpAny:
    case OpAll: { /* OR / AND of a boolean vector */
      Val* a = val(o[2]);
      if (!a || a->regs.empty()) return false;
      int32_t acc = a->regs[0];
      for (size_t k = 1; k < a->regs.size(); k++)
        acc = op2(in.opcode == OpAny ? Op::POr : Op::PAnd, Ty::Pred, acc, a->regs[k]);
      Val r;
      r.type = o[0];
      r.regs.push_back(acc);
      vals_[o[1]] = r;
      return true;
    }
    case OpFMod:
    case OpFRem: { /* x - y floor(x / y) (sign of y), or x - y trunc(x / y) (sign of x) */
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      Val r;
      r.type = o[0];
      for (size_t k = 0; k < a->regs.size() && k < b->regs.size(); k++) {
        int32_t q = op2(Op::FDiv, Ty::F32, a->regs[k], b->regs[k]);
        q = op1(in.opcode == OpFMod ? Op::FFloor : Op::FTrunc, Ty::F32, q);
        r.regs.push_back(op3(Op::FFma, Ty::F32, op1(Op::FNeg, Ty::F32, b->regs[k]), q, a->regs[k]));
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpSMod: { /* remainder with the sign of the divisor: srem, plus the divisor when the signs differ */
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      Val r;
      r.type = o[0];
      for (size_t k = 0; k < a->regs.size() && k < b->regs.size(); k++) {
        int32_t rem = op2(Op::SRem, Ty::B32, a->regs[k], b->regs[k]);
        int32_t nz = op2(Op::SetpS, Ty::Pred, rem, konst(Ty::B32, 0), CmpNe);
        int32_t diff = op2(Op::SetpS, Ty::Pred, op2(Op::Xor, Ty::B32, rem, b->regs[k]), konst(Ty::B32, 0), CmpLt);
        int32_t fix = op2(Op::PAnd, Ty::Pred, nz, diff);
        r.regs.push_back(op3(Op::Selp, Ty::B32, op2(Op::IAdd, Ty::B32, rem, b->regs[k]), rem, fix));
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpBitCount:
    case OpBitReverse: {
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) r.regs.push_back(op1(in.opcode == OpBitCount ? Op::Popc : Op::Brev, Ty::B32, x));
      vals_[o[1]] = r;
      return true;
    }
    case OpBitFieldSExtract:
    case OpBitFieldUExtract: { /* bits [offset, offset + count) of each component */
      Val* a = val(o[2]);
      Val* off = val(o[3]);
      Val* cnt = val(o[4]);
      if (!a || !off || !cnt) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) {
        Inst i;
        i.op = Op::Bfe;
        i.ty = Ty::B32;
        i.dst = fn_.reg(Ty::B32);
        i.a = x;
        i.b = off->regs[0];
        i.c = cnt->regs[0];
        i.imm = in.opcode == OpBitFieldSExtract ? 1u : 0u;
        fn_.emit(i);
        r.regs.push_back(i.dst);
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpBitFieldInsert: { /* mask = ((1 << count) - 1) << offset; (base & ~mask) | ((insert << offset) & mask) */
      Val* base = val(o[2]);
      Val* ins = val(o[3]);
      Val* off = val(o[4]);
      Val* cnt = val(o[5]);
      if (!base || !ins || !off || !cnt) return false;
      int32_t ones = op2(Op::Shl, Ty::B32, konst(Ty::B32, 1), cnt->regs[0]); /* count 32: the shift gives 0 */
      int32_t mask = op2(Op::Shl, Ty::B32, op2(Op::ISub, Ty::B32, ones, konst(Ty::B32, 1)), off->regs[0]);
      Val r;
      r.type = o[0];
      for (size_t k = 0; k < base->regs.size() && k < ins->regs.size(); k++) {
        int32_t keep = op2(Op::And, Ty::B32, base->regs[k], op1(Op::Not, Ty::B32, mask));
        int32_t put = op2(Op::And, Ty::B32, op2(Op::Shl, Ty::B32, ins->regs[k], off->regs[0]), mask);
        r.regs.push_back(op2(Op::Or, Ty::B32, keep, put));
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpDPdx:
    case OpDPdy:
    case OpFwidth:
      return fail("derivatives (dFdx, dFdy, fwidth) are not supported: fragments are shaded one at a time");
    case OpImageQuerySize:
    case OpImageQuerySizeLod: { /* textureSize: (width, height) of the image */
      Val* img = val(o[2]);
      if (!img || !img->is_tex) return fail("textureSize of something that is not a combined image sampler");
      Inst i;
      i.op = Op::TexSize;
      i.ty = Ty::B32;
      i.dst = fn_.reg(Ty::B32);
      fn_.reg(Ty::B32);
      i.c = img->tex_dyn ? img->regs[0] : -1;
      i.imm = img->tex_dyn ? 0u : img->tex_elem;
      i.imm2 = img->tex_key;
      fn_.emit(i);
      Val r;
      r.type = o[0];
      r.regs = {i.dst, i.dst + 1};
      vals_[o[1]] = r;
      return true;
    }
    case OpConvertFToS:
    case OpConvertFToU:
    case OpConvertSToF:
    case OpConvertUToF:
    case OpBitcast:
    case OpUConvert:
    case OpSConvert:
    case OpFConvert: {
      Val* a = val(o[2]);
      if (!a) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) {
        switch (in.opcode) {
          case OpConvertFToS: r.regs.push_back(op1(Op::CvtF2S, Ty::B32, x)); break;
          case OpConvertFToU: r.regs.push_back(op1(Op::CvtF2U, Ty::B32, x)); break;
          case OpConvertSToF: r.regs.push_back(op1(Op::CvtS2F, Ty::F32, x)); break;
          case OpConvertUToF: r.regs.push_back(op1(Op::CvtU2F, Ty::F32, x)); break;
          case OpBitcast: {
            Ty t = is_float(o[0]) ? Ty::F32 : Ty::B32;
            int32_t d = fn_.reg(t);
            Inst i;
            i.op = Op::Mov;
            i.ty = t;
            i.dst = d;
            i.a = x;
            fn_.emit(i);
            r.regs.push_back(d);
            break;
          }
          default: r.regs.push_back(x); break; /* 32-bit only: width conversions are identities */
        }
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpVectorTimesScalar:
    case OpMatrixTimesScalar: {
      Val* a = val(o[2]);
      Val* s = val(o[3]);
      if (!a || !s) return false;
      Val r;
      r.type = o[0];
      for (int32_t x : a->regs) r.regs.push_back(op2(Op::FMul, Ty::F32, x, s->regs[0]));
      vals_[o[1]] = r;
      return true;
    }
    case OpDot: {
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      Val r;
      r.type = o[0];
      r.regs.push_back(dot(a->regs, b->regs, a->regs.size()));
      vals_[o[1]] = r;
      return true;
    }
    case OpMatrixTimesVector: {
      Val* mtx = val(o[2]);
      Val* v = val(o[3]);
      if (!mtx || !v) return false;
      const TypeInfo& mt = ty(mtx->type);
      uint32_t cols = mt.count, rows = ty(mt.elem).count;
      Val r;
      r.type = o[0];
      for (uint32_t i = 0; i < rows; i++) {
        int32_t t = op2(Op::FMul, Ty::F32, mtx->regs[i], v->regs[0]);
        for (uint32_t c = 1; c < cols; c++) t = op3(Op::FFma, Ty::F32, mtx->regs[c * rows + i], v->regs[c], t);
        r.regs.push_back(t);
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpVectorTimesMatrix: {
      Val* v = val(o[2]);
      Val* mtx = val(o[3]);
      if (!v || !mtx) return false;
      const TypeInfo& mt = ty(mtx->type);
      uint32_t cols = mt.count, rows = ty(mt.elem).count;
      Val r;
      r.type = o[0];
      for (uint32_t c = 0; c < cols; c++) {
        std::vector<int32_t> col(mtx->regs.begin() + c * rows, mtx->regs.begin() + (c + 1) * rows);
        r.regs.push_back(dot(v->regs, col, rows));
      }
      vals_[o[1]] = r;
      return true;
    }
    case OpMatrixTimesMatrix: {
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      const TypeInfo& at = ty(a->type);
      const TypeInfo& bt = ty(b->type);
      uint32_t k_dim = at.count, rows = ty(at.elem).count, cols = bt.count;
      Val r;
      r.type = o[0];
      for (uint32_t c = 0; c < cols; c++)
        for (uint32_t i = 0; i < rows; i++) {
          int32_t t = op2(Op::FMul, Ty::F32, a->regs[i], b->regs[c * k_dim]);
          for (uint32_t k = 1; k < k_dim; k++) t = op3(Op::FFma, Ty::F32, a->regs[k * rows + i], b->regs[c * k_dim + k], t);
          r.regs.push_back(t);
        }
      vals_[o[1]] = r;
      return true;
    }
    case OpOuterProduct: {
      Val* a = val(o[2]);
      Val* b = val(o[3]);
      if (!a || !b) return false;
      Val r;
      r.type = o[0];
      for (int32_t y : b->regs)
        for (int32_t x : a->regs) r.regs.push_back(op2(Op::FMul, Ty::F32, x, y));
      vals_[o[1]] = r;
      return true;
    }
    case OpTranspose: {
      Val* a = val(o[2]);
      if (!a) return false;
      const TypeInfo& at = ty(a->type);
      uint32_t cols = at.count, rows = ty(at.elem).count;
      Val r;
      r.type = o[0];
      for (uint32_t i = 0; i < rows; i++)
        for (uint32_t c = 0; c < cols; c++) r.regs.push_back(a->regs[c * rows + i]);
      vals_[o[1]] = r;
      return true;
    }
    case OpExtInst: return ext_inst(in);
    case OpBranch: return branch_to(o[0]);
    case OpBranchConditional: {
      Val* c = val(o[0]);
      if (!c) return false;
      uint32_t t_l = fn_.label();
      bra_if(c->regs[0], t_l);
      if (!branch_to(o[2])) return false;
      label(t_l);
      return branch_to(o[1]);
    }
    case OpSwitch: {
      Val* sel = val(o[0]);
      if (!sel) return false;
      std::vector<std::pair<uint32_t, uint32_t>> cases; /* (IR label of the trampoline, target) */
      /* literals are as wide as the selector; 64-bit selectors are carried in 32 bits, so a case
       * matches on its low word only when its high word is zero */
      size_t lw = ty(sel->type).width > 32 ? 2 : 1;
      for (size_t i = 2; i + lw < o.size(); i += lw + 1) {
        if (lw == 2 && o[i + 1] != 0) continue;
        int32_t k = konst(Ty::B32, o[i]);
        int32_t p = op2(Op::SetpU, Ty::Pred, sel->regs[0], k, CmpEq);
        uint32_t l = fn_.label();
        bra_if(p, l);
        cases.push_back({l, o[i + lw]});
      }
      if (!branch_to(o[1])) return false;
      for (auto& cs : cases) {
        label(cs.first);
        if (!branch_to(cs.second)) return false;
      }
      return true;
    }
    case OpReturn: {
      if (!frames_.empty()) { /* end of an inlined call */
        bra(frames_.back().ret_label);
        return true;
      }
      finish_outputs();
      Inst i;
      i.op = Op::Ret;
      fn_.emit(i);
      return true;
    }
    case OpReturnValue: {
      if (frames_.empty()) return fail("OpReturnValue in the entry point");
      Frame& f = frames_.back();
      Val* v = val(o[0]);
      if (!v) return false;
      for (size_t k = 0; k < f.result.regs.size() && k < v->regs.size(); k++)
        mov(reg_ty(f.result.regs[k]), f.result.regs[k], v->regs[k]);
      bra(f.ret_label);
      return true;
    }
    case OpKill: {
      out_.iface.discards = true;
      Inst i;
      i.op = Op::Kill;
      fn_.emit(i);
      return true;
    }
    case OpUnreachable: {
      if (!frames_.empty()) {
        bra(frames_.back().ret_label);
        return true;
      }
      Inst i;
      i.op = Op::Ret;
      fn_.emit(i);
      return true;
    }
    case OpFunctionCall: return inline_call(in);
    default: return fail(std::string("unsupported instruction ") + opcode_name(in.opcode));
  }
}

/* phis of the blocks in [begin, end): result registers up front, incoming edges recorded per block */
void Translator::prescan_phis(size_t begin, size_t end) {
  uint32_t block = 0;
  for (size_t i = begin; i < end; i++) {
    const Insn& in = m_.insns[i];
    if (in.opcode == OpLabel) {
      block = in.ops[0];
      phis_.erase(block);
    }
    if (in.opcode == OpPhi) {
      PhiInfo ph;
      ph.type = in.ops[0];
      ph.result = in.ops[1];
      for (size_t k = 2; k + 1 < in.ops.size(); k += 2) ph.incoming.push_back({in.ops[k], in.ops[k + 1]});
      std::vector<Ty> tys;
      flat_types(ph.type, tys);
      Val v;
      v.type = ph.type;
      for (Ty t : tys) v.regs.push_back(fn_.reg(t));
      vals_[ph.result] = v;
      phis_[block].push_back(ph);
    }
  }
}

/* OpFunctionCall: the callee's body is translated in place.  Its parameters name the arguments (pointer
 * arguments name the same variable), its labels and phi registers are fresh for this call, and its returns
 * become moves into the call's result registers and a branch past the body.  Shaders cannot recurse. */
bool Translator::inline_call(const Insn& in) {
  const auto& o = in.ops;
  if (o.size() < 3) return fail("malformed OpFunctionCall");
  auto fr = fn_ranges_.find(o[2]);
  if (fr == fn_ranges_.end()) return fail("call of an unknown function %" + std::to_string(o[2]));
  if (frames_.size() >= 32) return fail("function calls nested deeper than 32 (recursion is not allowed)");
  const size_t begin = fr->second.first, end = fr->second.second;
  Frame f;
  f.ret_label = fn_.label();
  if (ty(o[0]).kind != TypeInfo::Void) {
    std::vector<Ty> tys;
    flat_types(o[0], tys);
    f.result.type = o[0];
    for (Ty t : tys) f.result.regs.push_back(fn_.reg(t));
    f.has_result = true;
  }
  size_t arg = 3;
  for (size_t i = begin; i < end; i++) {
    const Insn& p = m_.insns[i];
    if (p.opcode == OpLabel) labels_.erase(p.ops[0]);
    if (p.opcode != OpFunctionParameter) continue;
    if (arg >= o.size()) return fail("OpFunctionCall with too few arguments");
    uint32_t a = o[arg++];
    auto pl = places_.find(a);
    if (pl != places_.end()) {
      places_[p.ops[1]] = pl->second;
    } else {
      Val* v = val(a);
      if (!v) return false;
      vals_[p.ops[1]] = *v;
    }
  }
  prescan_phis(begin, end);
  const uint32_t caller_block = cur_block_;
  frames_.push_back(f);
  for (size_t i = begin; i < end; i++) {
    const Insn& b = m_.insns[i];
    if (b.opcode == OpFunctionParameter) continue;
    if (!do_insn(b)) return false;
  }
  Frame done = frames_.back();
  frames_.pop_back();
  label(done.ret_label);
  cur_block_ = caller_block;
  if (done.has_result) vals_[o[1]] = done.result;
  return true;
}

bool Translator::translate_entry() {
  /* locate the entry function */
  size_t begin = 0, end = 0;
  for (size_t i = 0; i < m_.insns.size(); i++) {
    const Insn& in = m_.insns[i];
    if (in.opcode == OpFunction && in.ops.size() > 1 && in.ops[1] == entry_id_) begin = i + 1;
    if (begin && in.opcode == OpFunctionEnd && i >= begin) {
      end = i;
      break;
    }
  }
  if (!begin || !end) return fail("entry function body not found");
  /* constants: materialised once at the top of the function */
  for (auto& kv : consts_) {
    std::vector<Ty> tys;
    flat_types(kv.second.first, tys);
    Val v;
    v.type = kv.second.first;
    for (size_t k = 0; k < tys.size() && k < kv.second.second.size(); k++) v.regs.push_back(konst(tys[k], kv.second.second[k]));
    vals_[kv.first] = v;
  }
  /* module-scope variables */
  for (auto& kv : vars_) {
    if (!layout_interface(kv.first, kv.second)) return false;
    Place p;
    p.var = kv.first;
    p.type = kv.second.type;
    places_[kv.first] = p;
    for (const Slot& s : kv.second.slots)
      if (s.reg >= 0) mov(reg_ty(s.reg), s.reg, konst(reg_ty(s.reg), 0));
  }
  /* every function's body, for inlining calls */
  for (size_t i = 0; i < m_.insns.size(); i++) {
    const Insn& in = m_.insns[i];
    if (in.opcode != OpFunction || in.ops.size() < 2) continue;
    size_t j = i + 1;
    while (j < m_.insns.size() && m_.insns[j].opcode != OpFunctionEnd) j++;
    fn_ranges_[in.ops[1]] = {i + 1, j};
  }
  prescan_phis(begin, end);
  for (size_t i = begin; i < end; i++) {
    const Insn& in = m_.insns[i];
    if (in.opcode == OpFunctionParameter) return fail("entry point with parameters");
    if (!do_insn(in)) return false;
  }
  return err_.empty();
}

std::string Translator::run() {
  out_.iface.stage = stage_;
  out_.entry = entry_name_;
  if (!scan_module()) return err_;
  if (!translate_entry()) return err_;
  /* positions-only liveness: which vertex inputs feed gl_Position */
  if (stage_ == Stage::Vertex) {
    for (uint32_t off : live_inputs(fn_, 0, 16))
      if (off < 128) out_.iface.pos_input_locations |= 1u << (off / 16);
  }
  return "";
}

}  // namespace

std::string translate_spirv(const uint32_t* words, size_t count, Stage stage, const char* entry,
                            const std::vector<std::pair<uint32_t, uint32_t>>& spec, Shader& out) {
  Module m;
  std::string e = decode(words, count, m);
  if (!e.empty()) return e;
  out = Shader();
  Translator t(m, stage, entry ? entry : "main", spec, out);
  return t.run();
}

std::vector<uint32_t> live_inputs(const Function& fn, uint32_t out_lo, uint32_t out_hi) {
  std::vector<char> live(fn.regs.size(), 0);
  bool changed = true;
  auto mark = [&](int32_t r) {
    if (r >= 0 && !live[(size_t)r]) {
      live[(size_t)r] = 1;
      changed = true;
    }
  };
  while (changed) {
    changed = false;
    for (const Inst& i : fn.code) {
      bool root = false;
      switch (i.op) {
        case Op::StOut: root = i.imm >= out_lo && i.imm < out_hi; break;
        case Op::BraIf:
        case Op::Kill: root = true; break;
        default: break;
      }
      bool live_dst = i.dst >= 0 && live[(size_t)i.dst];
      if ((i.op == Op::Tex || i.op == Op::TexFetch) && i.dst >= 0)
        for (int k = 1; k < 4; k++) live_dst |= live[(size_t)i.dst + k] != 0;
      if (i.op == Op::TexSize && i.dst >= 0) live_dst |= live[(size_t)i.dst + 1] != 0;
      if (root || live_dst) {
        mark(i.a);
        mark(i.b);
        mark(i.c);
      }
    }
  }
  std::vector<uint32_t> offs;
  for (const Inst& i : fn.code)
    if (i.op == Op::LdIn && i.dst >= 0 && live[(size_t)i.dst]) offs.push_back(i.imm);
  return offs;
}

/* the pipeline kernels write the interpolated varyings directly for such a shader, with the same values
 * the call would return */
bool color_passthrough(const Function& fn) {
  /* straight-line code only (labels but no branches): follow each register to the input word it holds */
  std::vector<int64_t> held(fn.regs.size(), -1);
  uint32_t stored = 0;
  for (const Inst& i : fn.code) {
    switch (i.op) {
      case Op::LdIn:
        if (i.dst < 0) return false;
        held[(size_t)i.dst] = (i.ty == Ty::F32 && i.imm < 16 && i.imm % 4 == 0) ? (int64_t)i.imm : -1;
        break;
      case Op::Mov:
        if (i.dst < 0 || i.a < 0) return false;
        held[(size_t)i.dst] = (i.ty == Ty::F32 && fn.regs[(size_t)i.a] == Ty::F32) ? held[(size_t)i.a] : -1;
        break;
      case Op::Const:
        if (i.dst < 0) return false;
        held[(size_t)i.dst] = -1;
        break;
      case Op::StOut:
        if (i.imm >= 16 || i.imm % 4 != 0 || i.a < 0 || held[(size_t)i.a] != (int64_t)i.imm) return false;
        stored |= 1u << (i.imm / 4);
        break;
      case Op::Label:
        break;
      case Op::Ret: /* what follows is unreachable */
        return stored == 0xFu;
      default:
        return false;
    }
  }
  return stored == 0xFu;
}

}  // namespace ir
}  // namespace kz

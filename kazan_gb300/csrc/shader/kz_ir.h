/*
 * kz_ir.h - the shader IR the PTX backend lowers.
 *
 * Role of the reference's shader-compiler-ir (shader-compiler-ir/src/module.rs:128-149,
 * instructions_impl.rs:395-430): the form a shader takes between the SPIR-V front end and a code
 * generator.  The reference IR is a structured SSA IR with only `add` and `load`; this one is a flat,
 * scalarised register IR (vectors and matrices are split into scalar registers, blocks are labels,
 * mutable variables are plain registers) with the f32/i32/bool arithmetic, interface loads/stores and
 * control flow that vertex and fragment shaders need.  Each operation's rounding is fixed (see
 * kz_ptx_backend.cpp), which is what makes shader results reproducible bit for bit.
 */
#ifndef KZ_IR_H
#define KZ_IR_H

#include <cstdint>
#include <string>
#include <vector>

#include "../kz_raster_abi.h"

#define KZ_IR_MAX_SETS KZ_MAX_DESC_SETS
#define KZ_IR_MAX_BINDINGS KZ_MAX_DESC_BINDINGS

namespace kz {
namespace ir {

enum class Ty : uint8_t { F32, B32, Pred };

enum class Op : uint8_t {
  Const,   /* dst = imm (bit pattern; Pred: imm != 0) */
  Mov,     /* dst = a */
  LdIn,    /* dst = 32-bit load from the stage input block at byte offset imm */
  LdPush,  /* dst = 32-bit load from the push-constant block at byte offset imm */
  StOut,   /* 32-bit store of a to the stage output block at byte offset imm */
  LdUbo,   /* dst = 32-bit load from the uniform buffer of binding imm2 (set << 16 | binding) at byte offset
              imm, plus the byte offset in register a when a >= 0 */
  LdDescRange, /* dst = bytes of the buffer range bound to binding imm2 (its descriptor's range) */
  Tex,     /* dst..dst+3 (f32 registers allocated in a row) = the combined image sampler of binding imm2,
              array element imm (plus register c when c >= 0), sampled at (a, b) */
  TexFetch,/* dst..dst+3 = texel (a, b) (integers; outside the image: 0) of binding imm2, element imm (+ c) */
  TexSize, /* dst, dst+1 (b32) = width, height of the image of binding imm2, element imm (+ c) */
  Popc,    /* dst = number of set bits of a */
  Brev,    /* dst = a with its 32 bits reversed */
  Clz,     /* dst = leading zero bits of a (32 for 0) */
  Bfe,     /* dst = bits [b, b + c) of a, sign-extended when imm != 0 (PTX bfe) */
  F2H,     /* dst (b32) = a rounded to binary16 (nearest even), in the low 16 bits */
  H2F,     /* dst (f32) = the binary16 value in the low 16 bits of a */
  FAdd, FSub, FMul, FDiv, FFma, FMin, FMax, FNeg, FAbs, FSqrt, FFloor, FCeil, FTrunc, FRoundEven,
  FSin, FCos, FEx2, FLg2,
  IAdd, ISub, IMul, UDiv, SDiv, URem, SRem, And, Or, Xor, Not, Shl, Shr, Sar, INeg,
  CvtF2S, CvtF2U, CvtS2F, CvtU2F,
  SetpF,   /* dst(pred) = compare a, b as f32; imm = Cmp */
  SetpS,   /* signed 32-bit compare */
  SetpU,   /* unsigned 32-bit compare */
  Selp,    /* dst = c ? a : b (c is a Pred register) */
  PAnd, POr, PXor, PNot,
  PToB32,  /* dst(b32) = a ? 1 : 0 */
  B32ToP,  /* dst(pred) = a != 0 */
  Label,   /* imm = label */
  Bra,     /* goto imm */
  BraIf,   /* if a goto imm */
  Ret,     /* leave the function (outputs already stored) */
  Kill     /* fragment discarded */
};

enum Cmp : uint32_t { CmpEq = 0, CmpNe, CmpLt, CmpLe, CmpGt, CmpGe, CmpUnordered = 8 };

struct Inst {
  Op op;
  Ty ty = Ty::F32;  /* type of dst (or of the operands for stores/compares) */
  int32_t dst = -1, a = -1, b = -1, c = -1;
  uint32_t imm = 0;
  uint32_t imm2 = 0;
  /* Tex through OpSampledImage of a separate sampler: the sampler's binding (set << 16 | binding) and
   * array element; ~0u for a combined image sampler */
  uint32_t smp = ~0u, smp_elem = 0;
};

struct Function {
  std::vector<Ty> regs;
  std::vector<Inst> code;
  uint32_t num_labels = 0;

  int32_t reg(Ty t) {
    regs.push_back(t);
    return (int32_t)regs.size() - 1;
  }
  uint32_t label() { return num_labels++; }
  void emit(const Inst& i) { code.push_back(i); }
};

enum class Stage : uint8_t { Vertex = 0, Fragment = 4 };

/* what a compiled stage reads and writes, in the kernels' ABI (kz_raster_abi.h KzVsIn/KzVsOut/KzFsIn) */
struct Interface {
  Stage stage = Stage::Vertex;
  uint32_t input_locations = 0;  /* vertex: attribute locations read; fragment: varying locations read */
  uint32_t pos_input_locations = 0; /* vertex: locations that feed gl_Position */
  uint32_t output_slots = 0;     /* vertex: scalar varying slots written (bit = location*4 + component) */
  uint32_t input_slots = 0;      /* fragment: scalar varying slots read */
  uint32_t flat_slots = 0;       /* slots decorated Flat */
  uint32_t noperspective_slots = 0;
  bool writes_position = false;
  bool writes_color = false;     /* fragment: location 0 written */
  bool discards = false;
  uint32_t push_bytes = 0;       /* highest push-constant byte read */
  /* descriptor bindings the stage declares (every module-scope Uniform / UniformConstant variable) */
  struct Binding {
    uint32_t set = 0, binding = 0;
    uint32_t kind = 0;   /* 0 uniform buffer, 1 combined image sampler, 2 storage buffer, 3 sampled image,
                          4 sampler */
    uint32_t count = 1;  /* array elements */
    uint32_t bytes = 0;  /* uniform or storage buffer: bytes the bound range must cover (the block; with a
                            runtime-sized array, the block with one element) */
  };
  std::vector<Binding> bindings;
};

struct Shader {
  Function fn;
  Interface iface;
  std::string entry;
};

/* translate the named entry point of a SPIR-V module; spec constants: (id, 32-bit value) pairs */
std::string translate_spirv(const uint32_t* words, size_t count, Stage stage, const char* entry,
                            const std::vector<std::pair<uint32_t, uint32_t>>& spec, Shader& out);

/* flow-insensitive liveness from the output stores at byte offsets [lo, hi) (and kills/branches);
 * returns the input byte offsets (LdIn imm) that are live */
std::vector<uint32_t> live_inputs(const Function& fn, uint32_t out_lo, uint32_t out_hi);

/* a fragment shader whose only effect is colour component k = input varying k for k = 0..3 (no other
 * instruction than loads of those inputs, the four stores and the return) */
bool color_passthrough(const Function& fn);

}  // namespace ir
}  // namespace kz

#endif

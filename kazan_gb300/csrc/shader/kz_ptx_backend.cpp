/*
 * kz_ptx_backend.cpp - shader-compiler-backend-ptx: IR -> PTX device functions -> JIT link.
 *
 * Takes the place of the reference's LLVM 7 backend (shader-compiler-backend-llvm-7, LLVM7Compiler::run
 * at backend.rs:553-690), which JIT-compiles for the host CPU.  Here a pipeline set (the pipelines one
 * command buffer uses) becomes one PTX module that defines the three functions the pipeline kernels
 * call (kz_raster_abi.h):
 *
 *   .func kz_vs(pipe, KzDraw* draw, vid, iid, push, KzVsOut* out)        full vertex shader
 *   .func (.b8[16] pos) kz_vs_pos(pipe, KzDraw* draw, vid, iid, push)  only gl_Position, returned by value
 *                                                                       (dead outputs dropped, ptxas removes
 *                                                                       their math)
 *   .func (.b8[48] pos) kz_vs_pos3(pipe, draw, vid0, vid1, vid2, iid, push)  gl_Position of a triangle's three
 *                                                                       vertices: push constants loaded once,
 *                                                                       three straight copies of the body
 *   .func (.b32 discard) kz_fs(pipe, KzFsIn* in, push, float* color)   fragment shader
 *   .func (.b8[32] colour, discard) kz_fs_r8(pipe, push, v0..v7, fc0..fc3, front)  the same for
 *                                                                       interfaces of at most 8 varyings,
 *                                                                       inputs and outputs in registers
 *
 * The vertex functions fetch their own attributes: the pipeline's vertex input state (binding, format,
 * offset, stride, input rate) is compiled into direct loads from the draw's vertex buffers, so no
 * attribute block passes through local memory.
 *
 * Each function branches on `pipe` to the inlined body of that pipeline.  nvJitLink then links the
 * module with the relocatable sm_103a object holding the kernels (kz_pipeline.cu) into one cubin; the
 * result plays the role of the reference's `CompiledCode` (shader-compiler-backend/src/lib.rs:200-205),
 * with kernels looked up by name instead of host function pointers.
 *
 * Rounding is explicit in every instruction (add.rn, mul.rn, fma.rn, div.rn, sqrt.rn, cvt.rn...), so
 * ptxas never contracts or approximates the IEEE operations the CPU oracle restates.  Only the GLSL
 * transcendental functions (sin, cos, exp2, log2, pow) use the approximate hardware instructions.
 */
#include <nvJitLink.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "kz_ir.h"
#include "kz_raster_abi.h"
#include "kz_shader_backend_impl.h"

namespace kz {
namespace ptx {

using ir::Function;
using ir::Inst;
using ir::Op;
using ir::Ty;

namespace {

struct RegMap {
  std::vector<std::string> names;
};

const char* cmp_name(uint32_t c) {
  static const char* ord[] = {"eq", "ne", "lt", "le", "gt", "ge"};
  static const char* unord[] = {"equ", "neu", "ltu", "leu", "gtu", "geu"};
  uint32_t k = c & 7u;
  if (k > 5) k = 0;
  return (c & ir::CmpUnordered) ? unord[k] : ord[k];
}

enum class Kind { VertexFull, VertexPos, VertexPos3, Fragment, FragmentRegs };

class Emitter {
 public:
  std::string out;
  uint32_t nf = 0, nr = 0, np = 0, nk = 0;
  std::map<uint32_t, std::string> push_regs; /* push-constant word (byte offset) -> register loaded up front */
  std::map<uint32_t, std::string> ubo_regs;  /* uniform-buffer binding -> register holding its address */
  uint32_t nu = 0;                            /* %kzu registers */
  bool uses_tex = false, uses_fetch = false;  /* calls kz_tex2d / kz_tex_fetch */
  bool uses_sep = false;                      /* samples through a separate sampler (a local descriptor) */
  uint32_t copy = 0;                          /* VertexPos3: which vertex the body computes */

  static uint32_t slot_of(const VertexLayout* lay, uint32_t key) {
    uint32_t set = key >> 16, binding = key & 0xFFFFu;
    if (!lay || set >= KZ_MAX_DESC_SETS || binding >= KZ_MAX_DESC_BINDINGS) return ~0u;
    return lay->desc_slot[set][binding];
  }

  /* the address of every uniform buffer `fn` reads, loaded once from the draw's descriptor slots */
  void preload_ubo(const Function& fn, const VertexLayout* lay) {
    ubo_regs.clear();
    char buf[200];
    for (const Inst& i : fn.code) {
      if (i.op != Op::LdUbo || ubo_regs.count(i.imm2)) continue;
      uint32_t slot = slot_of(lay, i.imm2);
      std::string r = "%kzu" + std::to_string(nu++);
      ubo_regs[i.imm2] = r;
      if (slot == ~0u) { /* not in the layout (pipeline creation rejects this): reads as address 0 */
        line("mov.b64 " + r + ", 0;");
        continue;
      }
      std::snprintf(buf, sizeof buf, "ld.global.nc.u64 %s, [%%kzpush+%u];\n  cvta.to.global.u64 %s, %s;", r.c_str(),
                    KZ_DESC_OFFSET + 32u * slot, r.c_str(), r.c_str());
      line(buf);
    }
  }

  /* load every push-constant word `fn` reads once, as 16-byte vectors where an aligned group is used twice
   * or more (the push block is 16-byte aligned and KZ_PUSH_BYTES long) */
  void preload_push(const Function& fn) {
    push_regs.clear();
    std::map<uint32_t, uint32_t> groups; /* 16-byte group -> mask of words read */
    for (const Inst& i : fn.code)
      if (i.op == Op::LdPush && i.imm % 4 == 0) groups[i.imm / 16] |= 1u << ((i.imm % 16) / 4);
    char buf[200];
    for (const auto& g : groups) {
      uint32_t base = g.first * 16;
      if (__builtin_popcount(g.second) >= 2 && base + 16 <= KZ_PUSH_BYTES) {
        uint32_t r0 = nk;
        nk += 4;
        std::snprintf(buf, sizeof buf, "ld.global.nc.v4.b32 {%%kp%u, %%kp%u, %%kp%u, %%kp%u}, [%%kzpush+%u];", r0,
                      r0 + 1, r0 + 2, r0 + 3, base);
        line(buf);
        for (uint32_t w = 0; w < 4; w++) push_regs[base + 4 * w] = "%kp" + std::to_string(r0 + w);
      } else {
        for (uint32_t w = 0; w < 4; w++) {
          if (!(g.second & (1u << w))) continue;
          std::string r = "%kp" + std::to_string(nk++);
          std::snprintf(buf, sizeof buf, "ld.global.nc.b32 %s, [%%kzpush+%u];", r.c_str(), base + 4 * w);
          line(buf);
          push_regs[base + 4 * w] = r;
        }
      }
    }
  }

  void line(const std::string& s) { out += "  " + s + "\n"; }

  /* vertex inputs loaded in the prologue (vector fetch): bit 4a + c set when component c of attribute a is in
   * register %kza<4a + c> */
  uint32_t preloaded = 0;

  /* attribute index of a location in the layout, or -1 */
  static int attr_of(const VertexLayout* lay, uint32_t loc) {
    int a = -1;
    for (uint32_t i = 0; lay && i < lay->num_attrs; i++)
      if (lay->location[i] == loc) a = (int)i;
    return a;
  }

  /* The vector fetch: with 16-byte aligned binding bases, the components the function reads of each 32-bit
   * attribute are loaded once at the start, with ld.global.nc.v4 where a run of four starts 16-byte aligned
   * (attribute offset and binding stride), v2 where a run of two starts 8-byte aligned, single words
   * otherwise; only the attribute's own bytes are read.  The loads then become register moves. */
  void vertex_preload(const Function& fn, const VertexLayout* lay) {
    preloaded = 0;
    if (!lay || lay->base_align < 16) return;
    uint32_t comps[8] = {};  /* per attribute: components read (bit c) */
    for (const Inst& i : fn.code) {
      if (i.op != Op::LdIn || i.imm >= 128) continue;
      int a = attr_of(lay, i.imm / 16);
      if (a < 0) continue;
      uint32_t fmt = lay->format[a];
      uint32_t ncomp = (fmt >= 1 && fmt <= 4) ? fmt : (fmt >= 6 && fmt <= 9) ? fmt - 5 : 0u;
      uint32_t c = (i.imm % 16) / 4;
      if (c < ncomp) comps[a] |= 1u << c;
    }
    char buf[200];
    for (uint32_t a = 0; a < lay->num_attrs && a < 8; a++) {
      if (!comps[a]) continue;
      uint32_t k = 32 - __builtin_clz(comps[a]); /* components 0..k-1 are loaded */
      uint32_t b = lay->binding[a], stride = lay->stride[b];
      for (uint32_t j = 0; j < k;) {
        uint32_t o = lay->offset[a] + 4 * j, r = 4 * a + j;
        if (k - j >= 4 && o % 16 == 0 && stride % 16 == 0) {
          std::snprintf(buf, sizeof buf, "ld.global.nc.v4.b32 {%%kza%u, %%kza%u, %%kza%u, %%kza%u}, [%%kzvb%u+%u];", r,
                        r + 1, r + 2, r + 3, b, o);
          j += 4;
        } else if (k - j >= 2 && o % 8 == 0 && stride % 8 == 0) {
          std::snprintf(buf, sizeof buf, "ld.global.nc.v2.b32 {%%kza%u, %%kza%u}, [%%kzvb%u+%u];", r, r + 1, b, o);
          j += 2;
        } else {
          std::snprintf(buf, sizeof buf, "ld.global.nc.b32 %%kza%u, [%%kzvb%u+%u];", r, b, o);
          j += 1;
        }
        line(buf);
      }
      preloaded |= ((1u << k) - 1u) << (4 * a);
    }
  }

  /* load of vertex input (location, component) for the generated fetch */
  void vertex_load(const VertexLayout* lay, uint32_t off, Ty ty, const std::string& dst) {
    char buf[160];
    if (off == 128 || off == 132) {
      line("mov.b32 " + dst + ", " + (off == 128 ? "%kzvid" : "%kziid") + ";");
      return;
    }
    {
      int a = attr_of(lay, off / 16);
      uint32_t c = (off % 16) / 4;
      if (a >= 0 && a < 8 && ((preloaded >> (4 * a + c)) & 1u)) {
        std::snprintf(buf, sizeof buf, "mov.b32 %s, %%kza%u;", dst.c_str(), 4 * (uint32_t)a + c);
        line(buf);
        return;
      }
    }
    uint32_t loc = off / 16, comp = (off % 16) / 4;
    int a = -1;
    for (uint32_t i = 0; lay && i < lay->num_attrs; i++)
      if (lay->location[i] == loc) a = (int)i;
    uint32_t fmt = a >= 0 ? lay->format[a] : 0;
    uint32_t ncomp = (fmt >= 1 && fmt <= 4) ? fmt : (fmt == 5 ? 4u : (fmt >= 6 && fmt <= 9) ? fmt - 5 : 0u);
    if (a < 0 || comp >= ncomp) {
      uint32_t bits = comp == 3 ? (ty == Ty::F32 ? 0x3F800000u : 1u) : 0u;
      std::snprintf(buf, sizeof buf, ty == Ty::F32 ? "mov.f32 %s, 0f%08X;" : "mov.b32 %s, %u;", dst.c_str(), bits);
      line(buf);
      return;
    }
    uint32_t b = lay->binding[a];
    if (fmt == 5) { /* R8G8B8A8_UNORM: byte / 255, correctly rounded */
      std::snprintf(buf, sizeof buf, "ld.global.nc.u32 %%kzt, [%%kzvb%u+%u];", b, lay->offset[a]);
      line(buf);
      std::snprintf(buf, sizeof buf, "bfe.u32 %%kzt, %%kzt, %u, 8;", 8 * comp);
      line(buf);
      if (ty == Ty::F32) {
        line("cvt.rn.f32.u32 " + dst + ", %kzt;");
        line("div.rn.f32 " + dst + ", " + dst + ", 0f437F0000;");
      } else {
        line("mov.b32 " + dst + ", %kzt;");
      }
      return;
    }
    std::snprintf(buf, sizeof buf, "ld.global.nc.%s %s, [%%kzvb%u+%u];", ty == Ty::F32 ? "f32" : "u32", dst.c_str(), b,
                  lay->offset[a] + 4 * comp);
    line(buf);
  }

  /* per-vertex base address of each binding the layout uses */
  void vertex_prologue(const VertexLayout* lay) {
    if (!lay) return;
    uint32_t used = 0;
    for (uint32_t i = 0; i < lay->num_attrs; i++) used |= 1u << lay->binding[i];
    char buf[200];
    for (uint32_t b = 0; b < 8; b++) {
      if (!(used & (1u << b))) continue;
      std::snprintf(buf, sizeof buf,
                    "ld.global.nc.u64 %%kzvb%u, [%%kzdraw+%u];\n  mul.wide.u32 %%kzoff, %s, %u;\n"
                    "  add.s64 %%kzvb%u, %%kzvb%u, %%kzoff;\n  cvta.to.global.u64 %%kzvb%u, %%kzvb%u;",
                    b, 8 * b, ((lay->instanced >> b) & 1u) ? "%kziid" : "%kzvid", lay->stride[b], b, b, b, b);
      line(buf);
    }
  }

  /* body of one pipeline stage; registers numbered from the running counters */
  void body(const Function& fn, const std::string& pfx, Kind kind, const VertexLayout* lay = nullptr) {
    std::vector<std::string> name(fn.regs.size());
    for (size_t i = 0; i < fn.regs.size(); i++) {
      switch (fn.regs[i]) {
        case Ty::F32: name[i] = "%f" + std::to_string(nf++); break;
        case Ty::B32: name[i] = "%r" + std::to_string(nr++); break;
        case Ty::Pred: name[i] = "%p" + std::to_string(np++); break;
      }
    }
    auto R = [&](int32_t r) { return name[(size_t)r]; };
    auto L = [&](uint32_t l) { return "$" + pfx + "_L" + std::to_string(l); };
    char buf[160];
    bool vertex = kind != Kind::Fragment && kind != Kind::FragmentRegs;
    if (vertex) {
      vertex_prologue(lay);
      vertex_preload(fn, lay);
    }
    for (const Inst& i : fn.code) {
      switch (i.op) {
        case Op::Const:
          if (i.ty == Ty::F32) {
            std::snprintf(buf, sizeof buf, "mov.f32 %s, 0f%08X;", R(i.dst).c_str(), i.imm);
            line(buf);
          } else if (i.ty == Ty::B32) {
            std::snprintf(buf, sizeof buf, "mov.b32 %s, %u;", R(i.dst).c_str(), i.imm);
            line(buf);
          } else {
            std::snprintf(buf, sizeof buf, "mov.b32 %%kzt, %u;", i.imm ? 1u : 0u);
            line(buf);
            line("setp.ne.u32 " + R(i.dst) + ", %kzt, 0;");
          }
          break;
        case Op::Mov: {
          Ty st = fn.regs[(size_t)i.a];
          if (i.ty == Ty::Pred && st == Ty::Pred) line("mov.pred " + R(i.dst) + ", " + R(i.a) + ";");
          else if (i.ty == Ty::F32 && st == Ty::F32) line("mov.f32 " + R(i.dst) + ", " + R(i.a) + ";");
          else if (i.ty == Ty::Pred) line("setp.ne.u32 " + R(i.dst) + ", " + R(i.a) + ", 0;");
          else if (st == Ty::Pred) line("selp.u32 " + R(i.dst) + ", 1, 0, " + R(i.a) + ";");
          else line("mov.b32 " + R(i.dst) + ", " + R(i.a) + ";");
          break;
        }
        case Op::LdIn:
          if (vertex) {
            vertex_load(lay, i.imm, i.ty, R(i.dst));
            break;
          }
          if (kind == Kind::FragmentRegs) {
            /* inputs arrive as scalar parameters: varyings 0..7, FragCoord, FrontFacing */
            const char* t = i.ty == Ty::F32 ? "f32" : "b32";
            if (i.imm < 32 && i.imm % 4 == 0)
              std::snprintf(buf, sizeof buf, "ld.param.%s %s, [kz_fs_r8_v%u];", t, R(i.dst).c_str(), i.imm / 4);
            else if (i.imm >= 64 && i.imm < 80 && i.imm % 4 == 0)
              std::snprintf(buf, sizeof buf, "ld.param.%s %s, [kz_fs_r8_fc%u];", t, R(i.dst).c_str(), (i.imm - 64) / 4);
            else if (i.imm == 80)
              std::snprintf(buf, sizeof buf, "ld.param.%s %s, [kz_fs_r8_front];", t, R(i.dst).c_str());
            else
              std::snprintf(buf, sizeof buf, "mov.b32 %s, 0;", R(i.dst).c_str());
            line(buf);
            break;
          }
          std::snprintf(buf, sizeof buf, "ld.%s %s, [%%kzin+%u];", i.ty == Ty::F32 ? "f32" : "u32", R(i.dst).c_str(),
                        i.imm);
          line(buf);
          break;
        case Op::LdPush: {
          auto pr = push_regs.find(i.imm);
          if (pr != push_regs.end()) {
            line("mov.b32 " + R(i.dst) + ", " + pr->second + ";");
            break;
          }
          std::snprintf(buf, sizeof buf, "ld.global.nc.%s %s, [%%kzpush+%u];", i.ty == Ty::F32 ? "f32" : "u32",
                        R(i.dst).c_str(), i.imm);
          line(buf);
          break;
        }
        case Op::LdUbo: {
          auto ur = ubo_regs.find(i.imm2);
          std::string base = ur != ubo_regs.end() ? ur->second : std::string("%kzub");
          if (ur == ubo_regs.end()) line("mov.b64 %kzub, 0;");
          if (i.a >= 0) {
            line("cvt.u64.u32 %kzoff, " + R(i.a) + ";");
            line("add.s64 %kzub, " + base + ", %kzoff;");
            base = "%kzub";
          }
          std::snprintf(buf, sizeof buf, "ld.global.nc.%s %s, [%s+%u];", i.ty == Ty::F32 ? "f32" : "u32",
                        R(i.dst).c_str(), base.c_str(), i.imm);
          line(buf);
          break;
        }
        case Op::LdDescRange: { /* KzDescriptor::range of the binding's slot in the draw's snapshot */
          uint32_t slot = slot_of(lay, i.imm2);
          if (slot == ~0u) { /* not in the layout (pipeline creation rejects this) */
            line("mov.b32 " + R(i.dst) + ", 0;");
            break;
          }
          std::snprintf(buf, sizeof buf, "ld.global.nc.u32 %s, [%%kzpush+%u];", R(i.dst).c_str(),
                        KZ_DESC_OFFSET + 32u * slot + 8u);
          line(buf);
          break;
        }
        case Op::Tex:
        case Op::TexFetch: {
          /* descriptor address (generic): push + KZ_DESC_OFFSET + 32 * (slot + element) */
          uint32_t slot = slot_of(lay, i.imm2);
          if (slot == ~0u) { /* not in the layout (pipeline creation rejects this) */
            for (int k = 0; k < 4; k++) line("mov.f32 " + R(i.dst + k) + ", 0f00000000;");
            break;
          }
          std::snprintf(buf, sizeof buf, "add.s64 %%kzd, %%kzpg, %u;", KZ_DESC_OFFSET + 32u * (slot + i.imm));
          line(buf);
          if (i.c >= 0) {
            line("mul.wide.u32 %kzoff, " + R(i.c) + ", 32;");
            line("add.s64 %kzd, %kzd, %kzoff;");
          }
          const uint32_t sslot = i.smp == ~0u ? ~0u : slot_of(lay, i.smp);
          if (i.op == Op::Tex && sslot != ~0u) {
            /* a separate sampler: a local copy of the image's descriptor with the sampler's state word
             * (KzDescriptor::sampler, byte 28) in place of its own */
            line("ld.v4.u32 {%kzs0, %kzs1, %kzs2, %kzs3}, [%kzd];");
            line("ld.v4.u32 {%kzs4, %kzs5, %kzs6, %kzs7}, [%kzd+16];");
            std::snprintf(buf, sizeof buf, "ld.global.nc.u32 %%kzs7, [%%kzpush+%u];",
                          KZ_DESC_OFFSET + 32u * (sslot + i.smp_elem) + 28u);
            line(buf);
            line("st.local.v4.u32 [kzsd], {%kzs0, %kzs1, %kzs2, %kzs3};");
            line("st.local.v4.u32 [kzsd+16], {%kzs4, %kzs5, %kzs6, %kzs7};");
            line("mov.u64 %kzd, kzsd;");
            line("cvta.local.u64 %kzd, %kzd;");
            uses_sep = true;
          }
          const char* fnn = i.op == Op::Tex ? "kz_tex2d" : "kz_tex_fetch";
          const char* at = i.op == Op::Tex ? "f32" : "b32";
          line("{");
          line(".param .b64 kzt_p0;");
          line(std::string(".param .b32 kzt_p1;\n  .param .b32 kzt_p2;\n  .param .align 16 .b8 kzt_r[16];"));
          line("st.param.b64 [kzt_p0], %kzd;");
          line(std::string("st.param.") + at + " [kzt_p1], " + R(i.a) + ";");
          line(std::string("st.param.") + at + " [kzt_p2], " + R(i.b) + ";");
          line(std::string("call (kzt_r), ") + fnn + ", (kzt_p0, kzt_p1, kzt_p2);");
          for (int k = 0; k < 4; k++) line("ld.param.f32 " + R(i.dst + k) + ", [kzt_r+" + std::to_string(4 * k) + "];");
          line("}");
          uses_tex |= i.op == Op::Tex;
          uses_fetch |= i.op == Op::TexFetch;
          break;
        }
        case Op::TexSize: {
          uint32_t slot = slot_of(lay, i.imm2);
          if (slot == ~0u) {
            line("mov.b32 " + R(i.dst) + ", 0;");
            line("mov.b32 " + R(i.dst + 1) + ", 0;");
            break;
          }
          std::snprintf(buf, sizeof buf, "add.s64 %%kzd, %%kzpush, %u;", KZ_DESC_OFFSET + 32u * (slot + i.imm));
          line(buf);
          if (i.c >= 0) {
            line("mul.wide.u32 %kzoff, " + R(i.c) + ", 32;");
            line("add.s64 %kzd, %kzd, %kzoff;");
          }
          line("ld.global.nc.u32 " + R(i.dst) + ", [%kzd+12];");
          line("ld.global.nc.u32 " + R(i.dst + 1) + ", [%kzd+16];");
          break;
        }
        case Op::Popc: line("popc.b32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::Brev: line("brev.b32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::Clz: line("clz.b32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::Bfe:
          line(std::string(i.imm ? "bfe.s32 " : "bfe.u32 ") + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ", " + R(i.c) +
               ";");
          break;
        case Op::F2H:
          line("{ .reg .b16 %kzh; cvt.rn.f16.f32 %kzh, " + R(i.a) + "; cvt.u32.u16 " + R(i.dst) + ", %kzh; }");
          break;
        case Op::H2F:
          line("{ .reg .b16 %kzh; cvt.u16.u32 %kzh, " + R(i.a) + "; cvt.f32.f16 " + R(i.dst) + ", %kzh; }");
          break;
        case Op::StOut: {
          if ((kind == Kind::VertexPos || kind == Kind::VertexPos3) && i.imm >= 16) break;
          if (kind == Kind::VertexPos3) {
            std::string v3 = R(i.a);
            if (fn.regs[(size_t)i.a] == Ty::Pred) {
              line("selp.u32 %kzt, 1, 0, " + v3 + ";");
              v3 = "%kzt";
            }
            std::snprintf(buf, sizeof buf, "st.param.%s [func_retval0+%u], %s;",
                          fn.regs[(size_t)i.a] == Ty::F32 ? "f32" : "b32", 16 * copy + i.imm, v3.c_str());
            line(buf);
            break;
          }
          std::string v = R(i.a);
          if (fn.regs[(size_t)i.a] == Ty::Pred) {
            line("selp.u32 %kzt, 1, 0, " + v + ";");
            v = "%kzt";
          }
          if (kind == Kind::FragmentRegs) {
            if (i.imm >= 16) break;
            std::snprintf(buf, sizeof buf, "st.param.%s [func_retval0+%u], %s;",
                          fn.regs[(size_t)i.a] == Ty::F32 ? "f32" : "b32", i.imm, v.c_str());
            line(buf);
            break;
          }
          if (kind == Kind::VertexPos)
            std::snprintf(buf, sizeof buf, "st.param.%s [func_retval0+%u], %s;",
                          fn.regs[(size_t)i.a] == Ty::F32 ? "f32" : "b32", i.imm, v.c_str());
          else
            std::snprintf(buf, sizeof buf, "st.%s [%%kzout+%u], %s;",
                          fn.regs[(size_t)i.a] == Ty::F32 ? "f32" : "u32", i.imm, v.c_str());
          line(buf);
          break;
        }
        case Op::FAdd: line("add.rn.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FSub: line("sub.rn.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FMul: line("mul.rn.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FDiv: line("div.rn.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FFma: line("fma.rn.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ", " + R(i.c) + ";"); break;
        case Op::FMin: line("min.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FMax: line("max.f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::FNeg: line("neg.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FAbs: line("abs.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FSqrt: line("sqrt.rn.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FFloor: line("cvt.rmi.f32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FCeil: line("cvt.rpi.f32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FTrunc: line("cvt.rzi.f32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FRoundEven: line("cvt.rni.f32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FSin: line("sin.approx.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FCos: line("cos.approx.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FEx2: line("ex2.approx.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::FLg2: line("lg2.approx.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::IAdd: line("add.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::ISub: line("sub.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::IMul: line("mul.lo.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::UDiv: line("div.u32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::SDiv: line("div.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::URem: line("rem.u32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::SRem: line("rem.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::And: line("and.b32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::Or: line("or.b32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::Xor: line("xor.b32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::Not: line("not.b32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::Shl: line("shl.b32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::Shr: line("shr.u32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::Sar: line("shr.s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::INeg: line("neg.s32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::CvtF2S: line("cvt.rzi.s32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::CvtF2U: line("cvt.rzi.u32.f32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::CvtS2F: line("cvt.rn.f32.s32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::CvtU2F: line("cvt.rn.f32.u32 " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::SetpF:
          line(std::string("setp.") + cmp_name(i.imm) + ".f32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";");
          break;
        case Op::SetpS:
          line(std::string("setp.") + cmp_name(i.imm & 7u) + ".s32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";");
          break;
        case Op::SetpU:
          line(std::string("setp.") + cmp_name(i.imm & 7u) + ".u32 " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";");
          break;
        case Op::Selp:
          line(std::string(i.ty == Ty::F32 ? "selp.f32 " : "selp.b32 ") + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) +
               ", " + R(i.c) + ";");
          break;
        case Op::PAnd: line("and.pred " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::POr: line("or.pred " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::PXor: line("xor.pred " + R(i.dst) + ", " + R(i.a) + ", " + R(i.b) + ";"); break;
        case Op::PNot: line("not.pred " + R(i.dst) + ", " + R(i.a) + ";"); break;
        case Op::PToB32: line("selp.u32 " + R(i.dst) + ", 1, 0, " + R(i.a) + ";"); break;
        case Op::B32ToP: line("setp.ne.u32 " + R(i.dst) + ", " + R(i.a) + ", 0;"); break;
        case Op::Label: out += L(i.imm) + ":\n"; break;
        case Op::Bra: line("bra " + L(i.imm) + ";"); break;
        case Op::BraIf: line("@" + R(i.a) + " bra " + L(i.imm) + ";"); break;
        case Op::Ret:
          if (kind == Kind::VertexPos3) {
            line("bra $" + pfx + "_end;");
            break;
          }
          if (kind == Kind::Fragment) {
            line("mov.b32 %kzt, 0;");
            line("st.param.b32 [func_retval0], %kzt;");
          }
          if (kind == Kind::FragmentRegs) {
            line("mov.b32 %kzt, 0;");
            line("st.param.b32 [func_retval0+16], %kzt;");
          }
          line("ret;");
          break;
        case Op::Kill:
          if (kind == Kind::Fragment) {
            line("mov.b32 %kzt, 1;");
            line("st.param.b32 [func_retval0], %kzt;");
          }
          if (kind == Kind::FragmentRegs) {
            line("mov.b32 %kzt, 1;");
            line("st.param.b32 [func_retval0+16], %kzt;");
          }
          line("ret;");
          break;
      }
    }
    if (kind == Kind::VertexPos3) { /* the next vertex's copy follows */
      out += "$" + pfx + "_end:\n";
      return;
    }
    /* a body always ends in Ret; keep a fallback for malformed input */
    if (kind == Kind::Fragment) {
      line("mov.b32 %kzt, 0;");
      line("st.param.b32 [func_retval0], %kzt;");
    }
    if (kind == Kind::FragmentRegs) {
      line("mov.b32 %kzt, 0;");
      line("st.param.b32 [func_retval0+16], %kzt;");
    }
    line("ret;");
  }
};

std::string function_text(const char* fname, Kind kind, const std::vector<const ir::Shader*>& stages,
                          const std::vector<VertexLayout>& layouts, bool& uses_tex, bool& uses_fetch) {
  Emitter e;
  std::string bodies;
  for (size_t p = 0; p < stages.size(); p++) {
    e.out.clear();
    std::string pfx = std::string(fname) + "_p" + std::to_string(p);
    e.out += "$" + pfx + ":\n";
    if (stages[p]) e.preload_ubo(stages[p]->fn, p < layouts.size() ? &layouts[p] : nullptr);
    if (stages[p] && kind == Kind::VertexPos3) {
      e.preload_push(stages[p]->fn);
      for (uint32_t k = 0; k < 3; k++) {
        e.copy = k;
        e.line("mov.b32 %kzvid, %kzv" + std::to_string(k) + ";");
        e.body(stages[p]->fn, pfx + "_v" + std::to_string(k), kind, p < layouts.size() ? &layouts[p] : nullptr);
      }
      e.push_regs.clear();
      e.line("ret;");
    } else if (stages[p]) {
      if (kind == Kind::FragmentRegs) /* colour components the shader does not write read as 0 */
        for (uint32_t k = 0; k < 4; k++) e.line("st.param.b32 [func_retval0+" + std::to_string(4 * k) + "], 0;");
      e.body(stages[p]->fn, pfx, kind, p < layouts.size() ? &layouts[p] : nullptr);
    } else {
      if (kind == Kind::Fragment) {
        e.line("mov.b32 %kzt, 0;");
        e.line("st.param.b32 [func_retval0], %kzt;");
      }
      if (kind == Kind::FragmentRegs) {
        for (uint32_t k = 0; k < 4; k++) e.line("st.param.b32 [func_retval0+" + std::to_string(4 * k) + "], 0;");
        e.line("st.param.b32 [func_retval0+16], 0;");
      }
      e.line("ret;");
    }
    bodies += e.out;
  }
  std::string s;
  char buf[512];
  if (kind == Kind::Fragment) {
    std::snprintf(buf, sizeof buf,
                  ".visible .func (.param .b32 func_retval0) %s(\n  .param .b32 %s_pipe,\n  .param .b64 %s_in,\n"
                  "  .param .b64 %s_push,\n  .param .b64 %s_out\n)\n{\n",
                  fname, fname, fname, fname, fname);
  } else if (kind == Kind::FragmentRegs) {
    std::string h = ".visible .func (.param .align 16 .b8 func_retval0[32]) " + std::string(fname) + "(\n  .param .b32 " +
                    fname + "_pipe,\n  .param .b64 " + fname + "_push";
    for (int k = 0; k < 8; k++) h += ",\n  .param .b32 " + std::string(fname) + "_v" + std::to_string(k);
    for (int k = 0; k < 4; k++) h += ",\n  .param .b32 " + std::string(fname) + "_fc" + std::to_string(k);
    h += ",\n  .param .b32 " + std::string(fname) + "_front\n)\n{\n";
    std::snprintf(buf, sizeof buf, "%s", h.c_str());
  } else if (kind == Kind::VertexPos3) {
    std::snprintf(buf, sizeof buf,
                  ".visible .func (.param .align 16 .b8 func_retval0[48]) %s(\n  .param .b32 %s_pipe,\n"
                  "  .param .b64 %s_draw,\n  .param .b32 %s_vid0,\n  .param .b32 %s_vid1,\n  .param .b32 %s_vid2,\n"
                  "  .param .b32 %s_iid,\n  .param .b64 %s_push\n)\n{\n",
                  fname, fname, fname, fname, fname, fname, fname, fname);
  } else if (kind == Kind::VertexPos) {
    std::snprintf(buf, sizeof buf,
                  ".visible .func (.param .align 16 .b8 func_retval0[16]) %s(\n  .param .b32 %s_pipe,\n"
                  "  .param .b64 %s_draw,\n  .param .b32 %s_vid,\n  .param .b32 %s_iid,\n  .param .b64 %s_push\n)\n{\n",
                  fname, fname, fname, fname, fname, fname);
  } else {
    std::snprintf(buf, sizeof buf,
                  ".visible .func %s(\n  .param .b32 %s_pipe,\n  .param .b64 %s_draw,\n  .param .b32 %s_vid,\n"
                  "  .param .b32 %s_iid,\n  .param .b64 %s_push,\n  .param .b64 %s_out\n)\n{\n",
                  fname, fname, fname, fname, fname, fname, fname);
  }
  s += buf;
  s += "  .reg .b32 %kzsel, %kzt, %kzvid, %kziid, %kzv0, %kzv1, %kzv2;\n"
       "  .reg .b64 %kzin, %kzpush, %kzout, %kzdraw, %kzoff, %kzpg, %kzub, %kzd;\n  .reg .b64 %kzvb<8>;\n"
       "  .reg .b32 %kza<32>;\n"
       "  .reg .pred %kzp;\n";
  if (e.nu) s += "  .reg .b64 %kzu<" + std::to_string(e.nu) + ">;\n";
  if (e.uses_sep) s += "  .reg .b32 %kzs<8>;\n  .local .align 16 .b8 kzsd[32];\n";
  uses_tex |= e.uses_tex;
  uses_fetch |= e.uses_fetch;
  if (e.nk) s += "  .reg .b32 %kp<" + std::to_string(e.nk) + ">;\n";
  if (e.nf) s += "  .reg .f32 %f<" + std::to_string(e.nf) + ">;\n";
  if (e.nr) s += "  .reg .b32 %r<" + std::to_string(e.nr) + ">;\n";
  if (e.np) s += "  .reg .pred %p<" + std::to_string(e.np) + ">;\n";
  std::snprintf(buf, sizeof buf, "  ld.param.u32 %%kzsel, [%s_pipe];\n  ld.param.u64 %%kzpush, [%s_push];\n"
                                 "  mov.b64 %%kzpg, %%kzpush;\n  cvta.to.global.u64 %%kzpush, %%kzpush;\n", fname, fname);
  s += buf;
  if (kind == Kind::Fragment) {
    std::snprintf(buf, sizeof buf, "  ld.param.u64 %%kzin, [%s_in];\n  ld.param.u64 %%kzout, [%s_out];\n", fname, fname);
  } else if (kind == Kind::FragmentRegs) {
    buf[0] = 0;
  } else if (kind == Kind::VertexPos3) {
    std::snprintf(buf, sizeof buf,
                  "  ld.param.u64 %%kzdraw, [%s_draw];\n  cvta.to.global.u64 %%kzdraw, %%kzdraw;\n"
                  "  ld.param.u32 %%kzv0, [%s_vid0];\n  ld.param.u32 %%kzv1, [%s_vid1];\n"
                  "  ld.param.u32 %%kzv2, [%s_vid2];\n  ld.param.u32 %%kziid, [%s_iid];\n",
                  fname, fname, fname, fname, fname);
    s += buf;
    buf[0] = 0;
  } else {
    std::snprintf(buf, sizeof buf,
                  "  ld.param.u64 %%kzdraw, [%s_draw];\n  cvta.to.global.u64 %%kzdraw, %%kzdraw;\n"
                  "  ld.param.u32 %%kzvid, [%s_vid];\n  ld.param.u32 %%kziid, [%s_iid];\n",
                  fname, fname, fname);
    s += buf;
    if (kind == Kind::VertexFull) std::snprintf(buf, sizeof buf, "  ld.param.u64 %%kzout, [%s_out];\n", fname);
    else buf[0] = 0;
  }
  s += buf;
  for (size_t p = 0; p + 1 < stages.size(); p++) {
    std::snprintf(buf, sizeof buf, "  setp.eq.u32 %%kzp, %%kzsel, %zu;\n  @%%kzp bra $%s_p%zu;\n", p, fname, p);
    s += buf;
  }
  std::snprintf(buf, sizeof buf, "  bra $%s_p%zu;\n", fname, stages.empty() ? (size_t)0 : stages.size() - 1);
  s += buf;
  if (stages.empty()) {
    s += "$" + std::string(fname) + "_p0:\n";
    if (kind == Kind::Fragment) s += "  mov.b32 %kzt, 0;\n  st.param.b32 [func_retval0], %kzt;\n";
    if (kind == Kind::FragmentRegs) s += "  st.param.b32 [func_retval0+16], 0;\n";
    s += "  ret;\n";
  }
  s += bodies;
  s += "}\n\n";
  return s;
}

}  // namespace

std::string module_text(const std::vector<const ir::Shader*>& vs, const std::vector<const ir::Shader*>& fs,
                        const std::vector<VertexLayout>& layouts) {
  bool tex = false, fetch = false;
  std::string body;
  body += function_text("kz_vs", Kind::VertexFull, vs, layouts, tex, fetch);
  body += function_text("kz_vs_pos", Kind::VertexPos, vs, layouts, tex, fetch);
  body += function_text("kz_vs_pos3", Kind::VertexPos3, vs, layouts, tex, fetch);
  body += function_text("kz_fs", Kind::Fragment, fs, layouts, tex, fetch);
  body += function_text("kz_fs_r8", Kind::FragmentRegs, fs, layouts, tex, fetch);
  std::string s = ".version 9.0\n.target sm_103a\n.address_size 64\n\n";
  /* sampling functions defined in the pipeline-kernel object (kz_pipeline.cu) */
  if (tex)
    s += ".extern .func (.param .align 16 .b8 func_retval0[16]) kz_tex2d(.param .b64 kz_tex2d_param_0, "
         ".param .b32 kz_tex2d_param_1, .param .b32 kz_tex2d_param_2);\n\n";
  if (fetch)
    s += ".extern .func (.param .align 16 .b8 func_retval0[16]) kz_tex_fetch(.param .b64 kz_tex_fetch_param_0, "
         ".param .b32 kz_tex_fetch_param_1, .param .b32 kz_tex_fetch_param_2);\n\n";
  return s + body;
}

std::string link(const std::string& ptx, const void* object, size_t object_size, std::vector<char>& cubin,
                 const void* tex_object, size_t tex_size) {
  nvJitLinkHandle h = nullptr;
  /* shader functions are called from kernels launched with at most 64 registers per thread (the geometry
   * kernel runs 4 blocks of 256 per SM); the linker rejects a callee that needs more than its caller's
   * limit, so the shader PTX is compiled within 64 registers (a heavy shader spills instead) */
  const char* opts[] = {"-arch=sm_103a", "-O3", "-maxrregcount=64"};
  std::string err;
  if (nvJitLinkCreate(&h, 3, opts) != NVJITLINK_SUCCESS) return "nvJitLinkCreate failed";
  auto log = [&](const char* what) {
    size_t n = 0;
    nvJitLinkGetErrorLogSize(h, &n);
    std::string l(n + 1, '\0');
    if (n) nvJitLinkGetErrorLog(h, &l[0]);
    return std::string(what) + ": " + l.c_str();
  };
  if (nvJitLinkAddData(h, NVJITLINK_INPUT_CUBIN, object, object_size, "kz_pipeline") != NVJITLINK_SUCCESS) {
    err = log("adding the pipeline kernels");
  } else if (tex_object && tex_size &&
             nvJitLinkAddData(h, NVJITLINK_INPUT_CUBIN, tex_object, tex_size, "kz_tex") != NVJITLINK_SUCCESS) {
    err = log("adding the texture functions");
  } else if (nvJitLinkAddData(h, NVJITLINK_INPUT_PTX, ptx.c_str(), ptx.size() + 1, "kz_shaders") != NVJITLINK_SUCCESS) {
    err = log("adding the shader PTX");
  } else if (nvJitLinkComplete(h) != NVJITLINK_SUCCESS) {
    err = log("linking");
  } else {
    size_t n = 0;
    nvJitLinkGetLinkedCubinSize(h, &n);
    cubin.resize(n);
    if (nvJitLinkGetLinkedCubin(h, cubin.data()) != NVJITLINK_SUCCESS) err = "fetching the linked cubin failed";
  }
  nvJitLinkDestroy(&h);
  return err;
}

}  // namespace ptx
}  // namespace kz

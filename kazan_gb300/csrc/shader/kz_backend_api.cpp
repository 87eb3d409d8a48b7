/*
 * kz_backend_api.cpp - C ABI of the PTX shader backend (declared in include/kz_shader_backend.h).
 */
#include <cstring>
#include <string>
#include <vector>

#include "kz_ir.h"
#include "kz_shader_backend.h"
#include "kz_shader_backend_impl.h"
#include "kz_spirv.h"

namespace kz {
const std::vector<char>& pipeline_object();
const std::vector<char>& texture_object();
}

namespace {

void set_err(char* err, size_t n, const std::string& s) {
  if (err && n) {
    std::strncpy(err, s.c_str(), n - 1);
    err[n - 1] = 0;
  }
}

struct CompiledCode {
  std::vector<char> cubin;
};

}  // namespace

extern "C" KZ_API int kzShaderCompile(const uint32_t* code, size_t word_count, uint32_t stage, const char* entry,
                                      const uint32_t* spec_ids, const uint32_t* spec_values, uint32_t spec_count,
                                      void** out_shader, char* err, size_t err_size) {
  *out_shader = nullptr;
  if (stage != 0 && stage != 4) {
    set_err(err, err_size, "only vertex (0) and fragment (4) stages are supported");
    return -1;
  }
  std::vector<std::pair<uint32_t, uint32_t>> spec;
  for (uint32_t i = 0; i < spec_count; i++) spec.push_back({spec_ids[i], spec_values[i]});
  kz::ir::Shader* s = new kz::ir::Shader();
  std::string e = kz::ir::translate_spirv(code, word_count, stage == 0 ? kz::ir::Stage::Vertex : kz::ir::Stage::Fragment,
                                          entry, spec, *s);
  if (!e.empty()) {
    set_err(err, err_size, e);
    delete s;
    return -1;
  }
  *out_shader = s;
  return 0;
}

extern "C" KZ_API void kzShaderInfo(const void* shader, KzShaderInfo* out) {
  const kz::ir::Shader* s = static_cast<const kz::ir::Shader*>(shader);
  std::memset(out, 0, sizeof(*out));
  const kz::ir::Interface& i = s->iface;
  out->stage = (uint32_t)i.stage;
  out->input_locations = i.input_locations;
  out->pos_input_locations = i.pos_input_locations;
  out->output_slots = i.output_slots;
  out->input_slots = i.input_slots;
  out->flat_slots = i.flat_slots;
  out->noperspective_slots = i.noperspective_slots;
  out->writes_position = i.writes_position;
  out->writes_color = i.writes_color;
  out->discards = i.discards;
  out->push_bytes = i.push_bytes;
  out->ir_instructions = (uint32_t)s->fn.code.size();
  out->color_passthrough = i.stage == kz::ir::Stage::Fragment && kz::ir::color_passthrough(s->fn) ? 1u : 0u;
  out->ir_registers = (uint32_t)s->fn.regs.size();
}

extern "C" KZ_API void kzShaderDestroy(void* shader) { delete static_cast<kz::ir::Shader*>(shader); }

extern "C" KZ_API uint32_t kzShaderBindings(const void* shader, KzShaderBinding* out, uint32_t max) {
  const kz::ir::Shader* s = static_cast<const kz::ir::Shader*>(shader);
  const auto& b = s->iface.bindings;
  for (uint32_t i = 0; out && i < max && i < b.size(); i++) {
    out[i].set = b[i].set;
    out[i].binding = b[i].binding;
    out[i].kind = b[i].kind;
    out[i].count = b[i].count;
    out[i].bytes = b[i].bytes;
  }
  return (uint32_t)b.size();
}

extern "C" KZ_API size_t kzShaderEmitPtx(const void* const* vs, const void* const* fs,
                                         const KzVertexInputLayout* layouts, uint32_t count, char* buf, size_t size) {
  return kzShaderEmitPtxDescriptors(vs, fs, layouts, nullptr, count, buf, size);
}

extern "C" KZ_API size_t kzShaderEmitPtxDescriptors(const void* const* vs, const void* const* fs,
                                                    const KzVertexInputLayout* layouts, const KzDescriptorSlots* slots,
                                                    uint32_t count, char* buf, size_t size) {
  std::vector<const kz::ir::Shader*> v, f;
  std::vector<kz::ptx::VertexLayout> lay;
  for (uint32_t i = 0; i < count; i++) {
    v.push_back(static_cast<const kz::ir::Shader*>(vs[i]));
    f.push_back(fs ? static_cast<const kz::ir::Shader*>(fs[i]) : nullptr);
    kz::ptx::VertexLayout l;
    if (layouts) {
      const KzVertexInputLayout& src = layouts[i];
      l.num_attrs = src.num_attrs < 8 ? src.num_attrs : 8;
      for (uint32_t k = 0; k < 8; k++) {
        l.location[k] = src.location[k];
        l.binding[k] = src.binding[k] & 7u;
        l.format[k] = src.format[k];
        l.offset[k] = src.offset[k];
        l.stride[k] = src.stride[k];
      }
      l.instanced = src.instanced;
    }
    if (slots)
      for (uint32_t s = 0; s < 4; s++)
        for (uint32_t b = 0; b < 16; b++) l.desc_slot[s][b] = slots[i].slot[s][b];
    lay.push_back(l);
  }
  std::string ptx = kz::ptx::module_text(v, f, lay);
  if (buf && size) {
    size_t n = ptx.size() + 1 < size ? ptx.size() + 1 : size;
    std::memcpy(buf, ptx.c_str(), n - 1);
    buf[n - 1] = 0;
  }
  return ptx.size() + 1;
}

extern "C" KZ_API int kzShaderLink(const char* ptx, const void* object, size_t object_size, void** out_code, char* err,
                                   size_t err_size) {
  *out_code = nullptr;
  if (!object) {
    const std::vector<char>& o = kz::pipeline_object();
    if (o.empty()) {
      set_err(err, err_size, "pipeline kernel object not found");
      return -1;
    }
    object = o.data();
    object_size = o.size();
  }
  CompiledCode* c = new CompiledCode();
  const std::vector<char>& tex = kz::texture_object();
  std::string e = kz::ptx::link(ptx, object, object_size, c->cubin, tex.data(), tex.size());
  if (!e.empty()) {
    set_err(err, err_size, e);
    delete c;
    return -1;
  }
  *out_code = c;
  return 0;
}

extern "C" KZ_API const void* kzCompiledCodeImage(const void* code, size_t* size) {
  const CompiledCode* c = static_cast<const CompiledCode*>(code);
  *size = c->cubin.size();
  return c->cubin.data();
}

extern "C" KZ_API void kzCompiledCodeDestroy(void* code) { delete static_cast<CompiledCode*>(code); }

extern "C" KZ_API size_t kzSpirvDisassemble(const uint32_t* code, size_t word_count, char* buf, size_t size) {
  kz::spv::Module m;
  if (!kz::spv::decode(code, word_count, m).empty()) return 0;
  std::string t = kz::spv::disassemble(m);
  if (buf && size) {
    size_t n = t.size() + 1 < size ? t.size() + 1 : size;
    std::memcpy(buf, t.c_str(), n - 1);
    buf[n - 1] = 0;
  }
  return t.size() + 1;
}

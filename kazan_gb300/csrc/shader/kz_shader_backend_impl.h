/*
 * kz_shader_backend_impl.h - internal C++ interface of the PTX shader backend (see kz_ptx_backend.cpp).
 */
#ifndef KZ_SHADER_BACKEND_IMPL_H
#define KZ_SHADER_BACKEND_IMPL_H

#include <string>
#include <vector>

#include "kz_ir.h"

namespace kz {
namespace ptx {

/* vertex input state of a pipeline, as the generated vertex-shader code fetches it */
struct VertexLayout {
  uint32_t num_attrs = 0;
  uint32_t location[8] = {}, binding[8] = {}, format[8] = {}, offset[8] = {}; /* format: KzAttrFormat */
  uint32_t stride[8] = {};
  uint32_t instanced = 0; /* bit b: binding b advances per instance */
  /* byte alignment every binding's base address (buffer + bind offset) has in the draws that use this entry:
   * 4 (what Vulkan requires of 32-bit components), or 16; with 16, attribute components are fetched with
   * 8- and 16-byte vector loads where their offsets and the binding stride allow */
  uint32_t base_align = 4;
  /* descriptor slot of the first array element of (set, binding) in the pipeline layout (KZ_DESC_OFFSET +
   * 32 * slot bytes into a draw's push snapshot); ~0u for bindings the layout does not have */
  uint32_t desc_slot[KZ_MAX_DESC_SETS][KZ_MAX_DESC_BINDINGS];
  VertexLayout() {
    for (auto& s : desc_slot)
      for (auto& b : s) b = ~0u;
  }
};

/* PTX module defining kz_vs / kz_vs_pos / kz_fs for a pipeline set (entry p = pipeline index p;
 * a null fragment stage yields a fragment function that writes nothing) */
std::string module_text(const std::vector<const ir::Shader*>& vs, const std::vector<const ir::Shader*>& fs,
                        const std::vector<VertexLayout>& layouts);

/* nvJitLink the shader PTX with the relocatable kernel object and, when given, the texture-sampling object;
 * returns "" on success */
std::string link(const std::string& ptx, const void* object, size_t object_size, std::vector<char>& cubin,
                 const void* tex_object = nullptr, size_t tex_size = 0);

}  // namespace ptx
}  // namespace kz

#endif

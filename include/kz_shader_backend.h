/*
 * kz_shader_backend.h - C ABI of shader-compiler-backend-ptx, part of libkazan_driver.so.
 *
 * Counterpart of the reference's backend contract (shader-compiler-backend/src/lib.rs):
 *   kzShaderCompile       front end of Compiler::run (lib.rs:245-257) for one stage: SPIR-V entry point ->
 *                         shader IR (role of TranslatedSPIRVShader::new,
 *                         shader-compiler-translate-spirv-to-ir/src/lib.rs:191-214)
 *   kzShaderEmitPtx       code generation for a pipeline set: PTX device functions kz_vs, kz_vs_pos,
 *                         kz_vs_pos3, kz_fs
 *   kzShaderLink          JIT link with the pipeline kernels -> CompiledCode (lib.rs:200-205)
 *   kzCompiledCodeImage   the linked sm_103a image; kernels are looked up by name (CompiledCode::get)
 *   kzSpirvDisassemble    text dump of a module in the reference decoder's format
 *                         (spirv-parser/src/lib.rs:28-43 parse_and_dump)
 * Strings and buffers are caller-owned; functions return 0 on success unless stated otherwise.
 */
#ifndef KZ_SHADER_BACKEND_H
#define KZ_SHADER_BACKEND_H

#include <stddef.h>
#include <stdint.h>

#ifndef KZ_API
#define KZ_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct KzShaderInfo {
  uint32_t stage;               /* 0 vertex, 4 fragment (SPIR-V execution model numbers) */
  uint32_t input_locations;     /* bit L: input location L is read */
  uint32_t pos_input_locations; /* vertex: locations that feed gl_Position */
  uint32_t output_slots;        /* vertex: bit location*4+component of each varying written */
  uint32_t input_slots;         /* fragment: bit location*4+component of each varying read */
  uint32_t flat_slots, noperspective_slots;
  uint32_t writes_position, writes_color, discards;
  uint32_t push_bytes;          /* bytes of the push-constant block read */
  uint32_t ir_instructions, ir_registers;
  uint32_t color_passthrough;   /* fragment: colour component k = input varying k (k = 0..3), nothing else */
} KzShaderInfo;

/* Translate one entry point.  stage: 0 vertex or 4 fragment.  spec_ids/spec_values: specialisation
 * constants (32-bit).  On failure returns -1 and writes a message into err. */
KZ_API int kzShaderCompile(const uint32_t* code, size_t word_count, uint32_t stage, const char* entry,
                           const uint32_t* spec_ids, const uint32_t* spec_values, uint32_t spec_count,
                           void** out_shader, char* err, size_t err_size);
KZ_API void kzShaderInfo(const void* shader, KzShaderInfo* out);
KZ_API void kzShaderDestroy(void* shader);

/* Vertex input state of one pipeline (VkPipelineVertexInputStateCreateInfo in the form the generated
 * vertex fetch uses).  format: 1..4 = R32..R32G32B32A32_SFLOAT, 5 = R8G8B8A8_UNORM, 6..9 = 1..4 x 32-bit
 * integers. */
typedef struct KzVertexInputLayout {
  uint32_t num_attrs;
  uint32_t location[8], binding[8], format[8], offset[8];
  uint32_t stride[8];
  uint32_t instanced; /* bit b: binding b advances per instance */
} KzVertexInputLayout;

/* PTX module for a pipeline set (fs[i] may be NULL; layouts may be NULL, then vertex inputs read as 0).
 * Returns the size needed including the terminating NUL; writes at most `size` bytes into buf when buf
 * is not NULL. */
KZ_API size_t kzShaderEmitPtx(const void* const* vs, const void* const* fs, const KzVertexInputLayout* layouts,
                              uint32_t count, char* buf, size_t size);

/* Descriptor bindings a compiled stage declares (module-scope Uniform / UniformConstant variables). */
typedef struct KzShaderBinding {
  uint32_t set, binding;
  uint32_t kind;   /* 0 uniform buffer, 1 combined image sampler, 2 storage buffer, 3 sampled image, 4 sampler */
  uint32_t count;  /* array elements */
  uint32_t bytes;  /* uniform or storage buffer: bytes the bound range must cover (the block; for a storage
                      block ending in a runtime-sized array, the block with one element) */
} KzShaderBinding;
/* Writes at most `max` bindings into out (may be NULL) and returns how many the stage declares. */
KZ_API uint32_t kzShaderBindings(const void* shader, KzShaderBinding* out, uint32_t max);

/* Descriptor slots of one pipeline layout: slot[set][binding] is the slot of the binding's first array
 * element in a draw's snapshot (byte KZ_DESC_OFFSET + 32 * slot after the push constants, one 32-byte
 * KzDescriptor per slot, kz_raster_abi.h), ~0u where the layout has no such binding. */
typedef struct KzDescriptorSlots {
  uint32_t slot[4][16];
} KzDescriptorSlots;
/* kzShaderEmitPtx for stages that read descriptors: slots[i] belongs to pipeline i (slots may be NULL). */
KZ_API size_t kzShaderEmitPtxDescriptors(const void* const* vs, const void* const* fs,
                                         const KzVertexInputLayout* layouts, const KzDescriptorSlots* slots,
                                         uint32_t count, char* buf, size_t size);

/* Link PTX with the relocatable pipeline-kernel object (NULL: the object built next to the library). */
KZ_API int kzShaderLink(const char* ptx, const void* object, size_t object_size, void** out_code, char* err,
                        size_t err_size);
KZ_API const void* kzCompiledCodeImage(const void* code, size_t* size);
KZ_API void kzCompiledCodeDestroy(void* code);

/* Text dump of a SPIR-V module; returns the size needed including the NUL (0 if the module is invalid). */
KZ_API size_t kzSpirvDisassemble(const uint32_t* code, size_t word_count, char* buf, size_t size);

#ifdef __cplusplus
}
#endif

#endif /* KZ_SHADER_BACKEND_H */

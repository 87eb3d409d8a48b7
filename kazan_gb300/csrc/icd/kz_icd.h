/*
 * kz_icd.h - objects of the kazan GB300 Vulkan driver (internal).
 *
 * Mirrors the reference driver's object model (vulkan-driver/src/handle.rs, api_impl.rs): dispatchable
 * handles (instance, physical device, device, queue, command buffer) start with the loader dispatch
 * word initialised to ICD_LOADER_MAGIC (handle.rs:23-37); every other handle is a pointer to a heap
 * object owned by the application between vkCreate* and vkDestroy* (handle.rs:121-209).
 *
 * Where the reference keeps memory in host RAM (device_memory.rs:206-217) and has no command
 * execution at all (api_impl.rs:3414, 4436-4970 are `unimplemented!()`), this driver keeps memory in
 * HBM and executes recorded command buffers with the sm_103a pipeline kernels.
 */
#ifndef KZ_ICD_H
#define KZ_ICD_H

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../kz_raster_abi.h"
#include "../shader/kz_ir.h"
#include "kz_vk_abi.h"

namespace kz {

struct Instance;
struct PhysicalDevice;
struct Device;
struct Queue;
struct CommandBuffer;

struct Dispatchable {
  uintptr_t loader_magic = ICD_LOADER_MAGIC;
};

struct PhysicalDevice : Dispatchable {
  Instance* instance = nullptr;
  int cuda_device = 0;
  int sm_count = 0;
  size_t hbm_bytes = 0;
  std::string name;
};

struct Instance : Dispatchable {
  PhysicalDevice* pd = nullptr;
  uint32_t api_version = VK_API_VERSION_1_1;
};

/* memory types: 0 = DEVICE_LOCAL|HOST_VISIBLE|HOST_COHERENT|HOST_CACHED (the reference's single
 * "Main" type, device_memory.rs:30-38), 1 = DEVICE_LOCAL only */
struct DeviceMemory {
  Device* dev = nullptr;
  VkDeviceSize size = 0;
  uint32_t type = 0;
  char* dptr = nullptr;        /* HBM */
  char* host = nullptr;        /* pinned host shadow behind vkMapMemory (type 0 only) */
  bool mapped = false;
  bool device_newer = false;   /* the GPU wrote it since the host shadow was last refreshed */
  cudaEvent_t last_use = nullptr; /* recorded on the queue stream after the last submission that used it */
};

struct Buffer {
  VkDeviceSize size = 0;
  VkBufferUsageFlags usage = 0;
  DeviceMemory* mem = nullptr;
  VkDeviceSize offset = 0;
  char* ptr() const { return mem ? mem->dptr + offset : nullptr; }
};

struct Image {
  VkFormat format = VK_FORMAT_UNDEFINED;
  uint32_t width = 0, height = 0;
  uint32_t samples = 1; /* 4: KZ_MS_SAMPLES consecutive samples per pixel */
  VkImageTiling tiling = VK_IMAGE_TILING_OPTIMAL;
  VkImageUsageFlags usage = 0;
  uint32_t bpp = 4;
  uint32_t pitch = 0;
  VkDeviceSize size = 0;
  DeviceMemory* mem = nullptr;
  VkDeviceSize offset = 0;
  char* ptr() const { return mem ? mem->dptr + offset : nullptr; }
};

struct ImageView {
  Image* image = nullptr;
  VkFormat format = VK_FORMAT_UNDEFINED;
};

struct ShaderModule {
  std::vector<uint32_t> code;
};

/* ---- descriptor sets (vulkan-driver/src/descriptor_set.rs, sampler.rs) ---- */

struct Sampler {
  uint32_t bits = 0; /* KzSamplerBits */
};

/* one binding of a descriptor set layout */
struct SetBinding {
  uint32_t binding = 0;
  VkDescriptorType type = VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER;
  uint32_t count = 0;
  uint32_t first = 0;              /* index of its first descriptor within a set */
  std::vector<uint32_t> immutable; /* KzSamplerBits of its immutable samplers (empty: none) */
};

struct SetLayoutInfo {
  std::vector<SetBinding> bindings; /* sorted by binding number */
  uint32_t descriptors = 0;
  uint32_t dynamic = 0;             /* UNIFORM_BUFFER_DYNAMIC descriptors (dynamic offsets a bind consumes) */
  const SetBinding* find(uint32_t binding) const {
    for (const SetBinding& b : bindings)
      if (b.binding == binding) return &b;
    return nullptr;
  }
};

struct DescriptorSetLayout {
  std::shared_ptr<SetLayoutInfo> info;
};

/* a descriptor as written; device addresses are resolved when a draw is recorded */
struct DescriptorEntry {
  bool written = false;
  Buffer* buffer = nullptr;
  VkDeviceSize offset = 0, range = 0;
  ImageView* view = nullptr;
  uint32_t sampler = 0; /* KzSamplerBits */
};

struct DescriptorPool;
struct DescriptorSet {
  std::shared_ptr<SetLayoutInfo> layout;
  std::vector<DescriptorEntry> entries;
  DescriptorPool* pool = nullptr;
};

struct DescriptorPool {
  uint32_t max_sets = 0;
  std::vector<DescriptorSet*> sets;
};

/* the descriptor slots of a pipeline layout: set s's descriptor k is slot slot_base[s] + k */
struct PipelineLayoutInfo {
  std::vector<std::shared_ptr<SetLayoutInfo>> sets;
  uint32_t slot_base[KZ_MAX_DESC_SETS] = {};
  uint32_t slots = 0;
};

struct PipelineLayout {
  uint32_t push_size = 0;
  std::shared_ptr<PipelineLayoutInfo> info;
};

struct RenderPass {
  std::vector<VkAttachmentDescription> atts;
  int color_att = -1;
  int depth_att = -1;
  int resolve_att = -1; /* single-sample image the colour attachment resolves into at the end of the pass */
};

struct Framebuffer {
  RenderPass* rp = nullptr;
  std::vector<ImageView*> views;
  uint32_t width = 0, height = 0;
};

struct Pipeline {
  uint64_t uid = 0;
  KzPipe pipe{};
  std::shared_ptr<ir::Shader> vs, fs;
  VkViewport viewport{};
  VkRect2D scissor{};
  bool dyn_viewport = false, dyn_scissor = false, dyn_blend = false;
  uint32_t dyn_stencil = 0; /* bit 0 compare mask, bit 1 write mask, bit 2 reference are dynamic state */
  bool rasterizer_discard = false;
  int vis_key = -1; /* KzVisKey when the pipeline can be resolved order-independently, else -1 */
  std::shared_ptr<PipelineLayoutInfo> layout;   /* descriptor slots (null: no descriptor sets) */
  std::vector<ir::Interface::Binding> bindings; /* what the stages declare (checked at each draw) */
};

struct Fence {
  cudaEvent_t ev = nullptr;
  bool signaled = false;
  bool pending = false;
  VkResult error = VK_SUCCESS;
};

struct Semaphore {};

/* kinds of kernel launch, as reported by kzGetKernelTimes */
enum KernelKind {
  KK_PERSISTENT = 0,
  KK_VIS_INIT,
  KK_VIS_GEOMETRY,
  KK_VIS_LARGE,
  KK_VIS_RESOLVE,
  KK_GEOMETRY,
  KK_SCAN,
  KK_BIN,
  KK_RASTER,
  KK_CLEAR,
  KK_INDIRECT,
  KK_INDIRECT_TABLES,
  KK_RESOLVE,
  KK_PERSISTENT_VIS,
  KK_RASTER_DIRECT,
  KK_RASTER_DS,
  KK_RASTER_MS,
  KK_COUNT
};

/* one timed kernel launch: events recorded right before and right after it on the queue stream */
struct TimedLaunch {
  int kind = 0;
  cudaEvent_t before = nullptr, after = nullptr;
};
struct PipelineCache {};

/* a linked pipeline-kernel module for one pipeline set */
struct KernelSet {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t geometry = nullptr, scan = nullptr, bin = nullptr, raster = nullptr, persistent = nullptr,
               persistent_vis = nullptr, raster_direct = nullptr, raster_ds = nullptr, raster_ms = nullptr,
               clear = nullptr, vis_init = nullptr,
               vis_geometry = nullptr,
               vis_large = nullptr, vis_resolve = nullptr, indirect = nullptr, indirect_tables = nullptr,
               resolve = nullptr;
  int persistent_blocks = 0;
  int persistent_vis_blocks = 0; /* resident blocks of kz_k_persistent_vis (opaque passes) */
  int geometry_blocks = 0; /* resident blocks of kz_k_vis_geometry on the whole GPU */
};

/* ---- recording ---- */

struct DrawRec {
  Pipeline* pipe = nullptr;
  KzDraw d{};
  uint8_t push[KZ_PUSH_BYTES];
  uint64_t triangles = 0;  /* direct draws; indirect draws count theirs on the device */
  bool indirect = false;
  DeviceMemory* reads[KZ_MAX_BINDINGS + 3] = {};
  std::vector<KzDescriptor> desc;          /* the pipeline layout's descriptor slots, resolved */
  std::vector<DeviceMemory*> desc_reads;   /* memory behind them */
};

struct PassRec {
  Framebuffer* fb = nullptr;
  RenderPass* rp = nullptr;
  bool cont = false; /* continues the render pass instance before a vkCmdClearAttachments: attachments load */
  int32_t area[4] = {0, 0, 0, 0};
  VkClearValue clear_color{}, clear_depth{};
  std::vector<DrawRec> draws;
};

enum class OpKind { Pass, Clear, Copy, Copy2D, Fill, Resolve };

struct RecOp {
  OpKind kind = OpKind::Pass;
  size_t pass = 0;                       /* index into passes for Pass */
  /* Clear / Fill: rows [y0,y1) x [x0,x1) of a 4-byte-per-pixel surface */
  char* base = nullptr;
  uint32_t pitch = 0;
  int32_t rect[4] = {0, 0, 0, 0};
  uint32_t value = 0;
  /* Copy / Copy2D / Resolve (Resolve: src/spitch the multisampled image at rect x0, y0; dst/dpitch the
   * single-sample image at dst_x, dst_y; rect[2], rect[3] the extent) */
  int32_t dst_x = 0, dst_y = 0;
  char* dst = nullptr;
  const char* src = nullptr;
  size_t bytes = 0, width_bytes = 0, rows = 0, dpitch = 0, spitch = 0;
  DeviceMemory* wmem = nullptr;          /* memory the op writes */
  DeviceMemory* rmem = nullptr;          /* memory the op reads */
  std::vector<uint8_t> data;             /* vkCmdUpdateBuffer: the bytes, copied from device memory at execution */
};

/* lowered command buffer */
struct Lowered {
  uint32_t launches = 0;                   /* kernels one submission of the whole command buffer launches */
  std::vector<KzDraw> draws;
  std::vector<KzPipe> pipes;
  std::vector<Pipeline*> pipe_objs;
  std::vector<uint32_t> pipe_align;        /* per pipeline entry: alignment of its draws' vertex-buffer bases */
  std::vector<KzChunk> chunks;
  std::vector<KzSegment> segments;
  std::vector<uint64_t> prims_guess;       /* per segment: triangles the scratch is first sized for */
  std::vector<uint64_t> table_guess;       /* per indirect segment: triangles its device tables have room for */
  std::vector<uint8_t> push;
  std::vector<uint32_t> draw_lut;          /* all segments' draw lookup tables, back to back */
  std::vector<std::pair<uint32_t, uint32_t>> draw_chunks; /* per draw: its chunks [begin, end) within its segment
                                                             (direct draws; the per-draw launch form) */
  std::vector<size_t> draw_lut_offset;     /* per segment: first entry in draw_lut */
  struct LOp {
    OpKind kind;
    uint32_t seg_begin = 0, seg_end = 0;  /* Pass: segments [begin, end); others: segments before it */
    RecOp op;
  };
  std::vector<LOp> ops;
  std::vector<DeviceMemory*> reads, writes;
  uint64_t triangles = 0;
  uint32_t max_tiles = 0;
  /* device memory */
  char* d_tables = nullptr;
  size_t tables_bytes = 0;
  std::vector<uint8_t> tmaps;              /* per segment: the colour and depth tensor maps (128 bytes each) */
  size_t o_tmaps = 0;                      /* their offset in d_tables */
  KzFrame frame{};
  char* d_records = nullptr;
  char* d_bins = nullptr;
  uint32_t* d_tiles = nullptr;
  char* d_vis = nullptr;
  char* d_shades = nullptr;   /* ordered segments: per-record shading setup (KzSegment::shades) */
  char* d_inline = nullptr;   /* vkCmdUpdateBuffer data of the command buffer */
  uint32_t shade_stride = 0;
  KzSegCounters* d_counters = nullptr;
  KzStatus* d_status = nullptr;
  KzStatus* h_status = nullptr;
  uint32_t rec_cap = 0, pair_cap = 0;
  KernelSet* ks = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  int mode = 0; /* 0 persistent, 1 batched, 2 per-draw (geometry launched per draw, the pass-wide phases once
                   per segment; launched at submit, not captured) */
  uint32_t tile = 16;
  bool timed = false; /* kernel timing: launched at submit with an event pair around each kernel */
  uint32_t geo_blocks = 0; /* blocks per SM of the batched geometry launches (0: all resident) */
};

struct CommandPool {
  Device* dev = nullptr;
  std::vector<CommandBuffer*> buffers;
};

struct CommandBuffer : Dispatchable {
  Device* dev = nullptr;
  CommandPool* pool = nullptr;
  bool recording = false;
  /* recording state */
  Pipeline* pipe = nullptr;
  VkViewport viewport{};
  VkRect2D scissor{};
  bool have_viewport = false, have_scissor = false;
  float blend_const[4] = {0, 0, 0, 0};
  bool have_blend_const = false;
  Buffer* vb[KZ_MAX_BINDINGS] = {};
  VkDeviceSize vb_off[KZ_MAX_BINDINGS] = {};
  Buffer* ib = nullptr;
  VkDeviceSize ib_off = 0;
  VkIndexType ib_type = VK_INDEX_TYPE_UINT32;
  uint8_t push[KZ_PUSH_BYTES] = {};
  DescriptorSet* sets[KZ_MAX_DESC_SETS] = {};
  uint32_t stencil_dyn[3][2] = {}; /* vkCmdSetStencil{CompareMask,WriteMask,Reference}: [state][front, back] */
  std::vector<uint32_t> dyn_offsets[KZ_MAX_DESC_SETS]; /* per bound set, its dynamic offsets */
  int cur_pass = -1;
  std::vector<PassRec> passes;
  std::vector<RecOp> ops;
  VkResult record_error = VK_SUCCESS;
  std::unique_ptr<Lowered> low;
  /* statistics of the last completed execution */
  KzStatus last_status{};
  float last_ms = 0.0f;
  /* kernel timing: device time and launches per KernelKind, summed over completed submissions */
  double kernel_ms[KK_COUNT] = {};
  uint32_t kernel_launches[KK_COUNT] = {};
  std::vector<TimedLaunch> timing; /* launches of the submission being enqueued */
};

struct Submission {
  CommandBuffer* cb = nullptr;
  cudaEvent_t done = nullptr;
  Fence* fence = nullptr;
  std::vector<TimedLaunch> timing;
};

struct Queue : Dispatchable {
  Device* dev = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<Submission> inflight;
  VkResult lost = VK_SUCCESS;
};

struct Device : Dispatchable {
  PhysicalDevice* pd = nullptr;
  Queue queue;
  cudaStream_t capture_stream = nullptr;
  cudaStream_t copy_stream = nullptr;   /* uploads of host-visible memory (a copy engine beside the queue) */
  std::recursive_mutex mu;
  std::map<std::vector<uint64_t>, KernelSet*> kernel_sets;        /* by pipeline ids (not owning) */
  std::unordered_map<std::string, KernelSet*> kernel_sets_by_ptx; /* by generated PTX (owning) */
  std::vector<cudaEvent_t> event_pool;
  std::vector<cudaEvent_t> timing_pool; /* events with timing enabled */
};

/* global options (kzDriverSetOption / KZ_* environment variables) */
struct Options {
  int mode = 0;       /* KZ_MODE: persistent (0), batched (1), perdraw (2) */
  uint32_t tile = 16; /* KZ_TILE */
  double rec_slack = 1.25;
  int trace = 0;      /* KZ_TRACE */
  long fault_alloc = -1; /* KZ_FAULT=alloc:N: the Nth device allocation fails */
  int kernel_timing = 0; /* KZ_KERNEL_TIMING */
  int pdl = 1;        /* KZ_PDL: a kernel that follows another kernel in a submission is launched with
                         programmatic stream serialization (its launch overlaps the predecessor's completion) */
  uint32_t barrier_ns = 4000000000u; /* a persistent kernel's grid barrier gives up after waiting this long */
  int tma = 1;        /* KZ_TMA: kz_k_raster_direct stages each tile's colour and depth through tensor copies */
  int vector_fetch = 1; /* KZ_VECTOR_FETCH: draws whose vertex buffers start 16-byte aligned fetch attributes with
                           vector loads */
  uint32_t warp_px = KZ_WARP_PX_DEFAULT;       /* visibility path: largest box (pixels) a geometry warp rasterises */
  uint32_t job_blocks = KZ_JOB_BLOCKS_DEFAULT; /* visibility path: 8x8 blocks per large-triangle job */
  uint32_t geo_blocks = 0; /* blocks per SM of the batched geometry launches (0: as many as are resident) */
};
Options& options();

/* internal helpers shared by the translation units */
VkResult device_alloc(size_t bytes, void** out);
void device_free(void* p);
const std::vector<char>& pipeline_object();
const std::vector<char>& texture_object();
/* the linked kernel image for the pipeline entries of a command buffer; base_align[i]: the alignment of the
 * vertex-buffer base addresses of the draws that use entry i (4 or 16) */
KernelSet* kernel_set_for(Device* dev, const std::vector<Pipeline*>& pipes, const std::vector<uint32_t>& base_align,
                          std::string& err);
void log_error(const char* fmt, ...);

/* command buffer / queue entry points implemented in kz_cmd.cpp */
VkResult lower_command_buffer(CommandBuffer* cb);
void free_lowered(Lowered* low);
VkResult queue_submit(Queue* q, uint32_t count, const VkSubmitInfo* submits, Fence* fence);
VkResult queue_wait_idle(Queue* q);
VkResult fence_status(Device* dev, Fence* f);
VkResult wait_fences(Device* dev, uint32_t n, const VkFence* fences, VkBool32 all, uint64_t timeout);

}  // namespace kz

#endif

/*
 * kz_cmd.cpp - command pools and buffers, recording, lowering, submission and fences.
 *
 * The reference declares these entry points and implements none of them
 * (vulkan-driver/src/api_impl.rs:4436-4970 vkCmd*, :3414 vkQueueSubmit, :3653-3700 fences;
 * CommandBuffer/Fence are empty structs, handle.rs:315,327).
 *
 * Recording resolves all state at the vkCmdDraw* call (device addresses, viewport transform, pixel
 * rectangle, push-constant snapshot).  vkEndCommandBuffer lowers the recording into device tables
 * (kz_raster_abi.h: KzDraw / KzPipe / KzChunk / KzSegment), links the pipeline set's shaders into the
 * pipeline kernels, sizes the scratch (triangle records, tile bins) and, for the persistent and batched
 * modes, captures the launch sequence as a CUDA graph.  vkQueueSubmit replays that graph on the queue's
 * stream, bracketed by the host<->device copies that keep HOST_COHERENT memory coherent.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "kazan_driver.h"
#include "kz_icd.h"
#include "../kz_srgb_table.h"

namespace kz {

template <class T>
static T* H(const void* h) {
  return reinterpret_cast<T*>(const_cast<void*>(h));
}

static uint8_t unorm8(float v) {
  float c = std::fmin(std::fmax(v, 0.0f), 1.0f);
  return (uint8_t)(int)std::rint(c * 255.0f);
}

static const float kz_srgb_thr[255] = KZ_SRGB_THRESHOLDS;

/* the 8-bit sRGB code of linear v (the kernels' srgb8, over the same table) */
static uint8_t srgb8(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 1.0f) return 255;
  uint32_t n = 0;
  for (uint32_t step = 128; step > 0; step >>= 1)
    if (n + step <= 255u && kz_srgb_thr[n + step - 1] <= v) n += step;
  return (uint8_t)n;
}

/* a clear colour as the attachment's texel: UNORM8 channels, or sRGB codes for red, green and blue */
static uint32_t pack_color(VkFormat f, const float* c) {
  const bool srgb = f == VK_FORMAT_R8G8B8A8_SRGB || f == VK_FORMAT_B8G8R8A8_SRGB;
  uint8_t r = srgb ? srgb8(c[0]) : unorm8(c[0]), g = srgb ? srgb8(c[1]) : unorm8(c[1]);
  uint8_t b = srgb ? srgb8(c[2]) : unorm8(c[2]), a = unorm8(c[3]);
  if (f == VK_FORMAT_B8G8R8A8_UNORM || f == VK_FORMAT_B8G8R8A8_SRGB)
    return (uint32_t)b | ((uint32_t)g << 8) | ((uint32_t)r << 16) | ((uint32_t)a << 24);
  return (uint32_t)r | ((uint32_t)g << 8) | ((uint32_t)b << 16) | ((uint32_t)a << 24);
}

static uint32_t float_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

/* ------------------------------------------------------------------------------------------------ */
/* recording                                                                                        */

static void draw_rect(const Framebuffer* fb, const int32_t area[4], const VkRect2D& sc, const VkViewport& vp,
                      int32_t out[4]) {
  /* framebuffer & render area & scissor & viewport; pixel x is inside the viewport iff x + 0.5 lies in
   * [x, x + width) (the oracle's kzo_draw_rect uses the same formula) */
  int32_t x0 = 0, y0 = 0, x1 = (int32_t)fb->width, y1 = (int32_t)fb->height;
  x0 = std::max(x0, area[0]);
  y0 = std::max(y0, area[1]);
  x1 = std::min(x1, area[2]);
  y1 = std::min(y1, area[3]);
  x0 = std::max(x0, sc.offset.x);
  y0 = std::max(y0, sc.offset.y);
  x1 = std::min(x1, sc.offset.x + (int32_t)sc.extent.width);
  y1 = std::min(y1, sc.offset.y + (int32_t)sc.extent.height);
  float ylo = vp.height >= 0.0f ? vp.y : vp.y + vp.height, yhi = vp.height >= 0.0f ? vp.y + vp.height : vp.y;
  int32_t px0 = (int32_t)std::ceil(vp.x - 0.5f), px1 = (int32_t)std::ceil(vp.x + vp.width - 0.5f);
  int32_t py0 = (int32_t)std::ceil(ylo - 0.5f), py1 = (int32_t)std::ceil(yhi - 0.5f);
  out[0] = std::max(x0, px0);
  out[1] = std::max(y0, py0);
  out[2] = std::min(x1, px1);
  out[3] = std::min(y1, py1);
}

/* a draw needs a render pass and a bound pipeline (else a recording error) */
static bool draw_state_ok(CommandBuffer* cb) {
  if (cb->cur_pass < 0 || !cb->pipe) {
    log_error("draw outside a render pass or without a bound pipeline");
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return false;
  }
  return true;
}

static uint32_t color_format(VkFormat f);

/* the pipeline layout's descriptor slots from the bound sets, resolved to device addresses (dynamic offsets
 * applied to dynamic uniform buffers, in binding order); every descriptor the shaders declare must be
 * written: a combined image sampler with an RGBA8/BGRA8 image, a uniform buffer with a range that covers
 * the block.  Otherwise a recording error, so that no kernel reads through an unset descriptor. */
static bool snapshot_descriptors(CommandBuffer* cb, const Pipeline* p, DrawRec& dr) {
  const PipelineLayoutInfo& L = *p->layout;
  dr.desc.assign(L.slots, KzDescriptor{});
  for (uint32_t s = 0; s < L.sets.size(); s++) {
    const DescriptorSet* ds = cb->sets[s];
    if (!ds) continue;
    uint32_t dyn = 0;
    for (const SetBinding& lb : L.sets[s]->bindings) {
      const SetBinding* sb = ds->layout->find(lb.binding);
      for (uint32_t e = 0; e < lb.count; e++) {
        if (!sb || e >= sb->count) continue;
        const DescriptorEntry& de = ds->entries[sb->first + e];
        uint32_t dyn_off = 0;
        if (sb->type == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC || sb->type == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC) {
          const std::vector<uint32_t>& offs = cb->dyn_offsets[s];
          dyn_off = dyn < offs.size() ? offs[dyn] : 0;
          dyn++;
        }
        if (!de.written) continue;
        KzDescriptor& d = dr.desc[L.slot_base[s] + lb.first + e];
        if (sb->type == VK_DESCRIPTOR_TYPE_SAMPLER) {
          d.sampler = de.sampler;
          d.range = 1; /* written */
        } else if (sb->type == VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER || sb->type == VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE) {
          if (!de.view || !de.view->image || !de.view->image->mem) continue;
          const Image* img = de.view->image;
          d.addr = (uint64_t)(uintptr_t)img->ptr();
          d.width = img->width;
          d.height = img->height;
          d.pitch = img->pitch;
          d.format = color_format(img->format);
          d.sampler = sb->type == VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER ? de.sampler : 0u;
          dr.desc_reads.push_back(img->mem);
        } else {
          if (!de.buffer || !de.buffer->mem) continue;
          VkDeviceSize off = de.offset + dyn_off;
          VkDeviceSize range = de.range == VK_WHOLE_SIZE ? (off < de.buffer->size ? de.buffer->size - off : 0) : de.range;
          if (off + range > de.buffer->size) continue;
          d.addr = (uint64_t)(uintptr_t)(de.buffer->ptr() + off);
          d.range = (uint32_t)std::min<VkDeviceSize>(range, 0xFFFFFFFFu);
          dr.desc_reads.push_back(de.buffer->mem);
        }
      }
    }
  }
  for (const ir::Interface::Binding& b : p->bindings) {
    const SetBinding* lb = b.set < L.sets.size() ? L.sets[b.set]->find(b.binding) : nullptr;
    for (uint32_t e = 0; lb && e < b.count; e++) {
      const KzDescriptor& d = dr.desc[L.slot_base[b.set] + lb->first + e];
      const bool image = b.kind == 1 || b.kind == 3;
      bool ok = image         ? d.addr && d.width && d.height && d.format != KZ_CF_NONE
                : b.kind == 4 ? d.range != 0
                              : d.addr && d.range >= b.bytes;
      if (!ok) {
        log_error("draw: set %u binding %u element %u is not bound or not written with a %s", b.set, b.binding, e,
                  image ? "RGBA8/BGRA8 image" : b.kind == 4 ? "sampler" : "buffer range covering the block");
        cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
        return false;
      }
    }
  }
  return true;
}

/* the state every draw resolves at recording: vertex buffers, index buffer, viewport transform, pixel
 * rectangle and push-constant snapshot.  False (and a recording error) for an indexed draw without an
 * index buffer. */
static bool begin_draw(CommandBuffer* cb, bool indexed, DrawRec& dr, int& nreads) {
  if (indexed && !cb->ib) {
    log_error("indexed draw without an index buffer");
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return false;
  }
  Pipeline* p = cb->pipe;
  PassRec& pass = cb->passes[(size_t)cb->cur_pass];
  std::memset(&dr.d, 0, sizeof dr.d);
  dr.pipe = p;
  KzDraw& d = dr.d;
  nreads = 0;
  for (int b = 0; b < KZ_MAX_BINDINGS; b++) {
    if (cb->vb[b]) {
      d.vb[b] = (uint64_t)(uintptr_t)(cb->vb[b]->ptr() + cb->vb_off[b]);
      dr.reads[nreads++] = cb->vb[b]->mem;
    }
  }
  if (indexed) {
    d.indexed = cb->ib_type == VK_INDEX_TYPE_UINT16 ? 2 : 1;
    d.ib_base = (uint64_t)(uintptr_t)(cb->ib->ptr() + cb->ib_off);
    d.ib = d.ib_base;
    dr.reads[nreads++] = cb->ib->mem;
  }
  VkViewport vp = p->dyn_viewport ? cb->viewport : p->viewport;
  VkRect2D sc = p->dyn_scissor ? cb->scissor : p->scissor;
  d.hx = 0.5f * vp.width;
  d.ox = vp.x + d.hx;
  d.hy = 0.5f * vp.height;
  d.oy = vp.y + d.hy;
  d.pz = vp.maxDepth - vp.minDepth;
  d.oz = vp.minDepth;
  d.zmin = std::fmin(vp.minDepth, vp.maxDepth);
  d.zmax = std::fmax(vp.minDepth, vp.maxDepth);
  draw_rect(pass.fb, pass.area, sc, vp, d.rect);
  std::memcpy(dr.push, cb->push, KZ_PUSH_BYTES);
  /* blend constants in effect at this draw.  The colour attachments are unsigned normalized, so the
   * constants are clamped to [0, 1] before they act as blend factors, as source and destination are. */
  const float* bc = p->dyn_blend && cb->have_blend_const ? cb->blend_const : p->pipe.blend_const;
  for (int k = 0; k < 4; k++) d.blend_const[k] = std::fmin(std::fmax(bc[k], 0.0f), 1.0f);
  /* stencil words of the draw: the pipeline's, with the dynamic compare mask / write mask / reference */
  for (int f = 0; f < 2; f++) {
    uint32_t w1 = p->pipe.stencil[2 * f + 1];
    if (p->dyn_stencil & 1u) w1 = (w1 & ~0xFFu) | (cb->stencil_dyn[0][f] & 0xFFu);
    if (p->dyn_stencil & 2u) w1 = (w1 & ~0xFF00u) | ((cb->stencil_dyn[1][f] & 0xFFu) << 8);
    if (p->dyn_stencil & 4u) w1 = (w1 & ~0xFF0000u) | ((cb->stencil_dyn[2][f] & 0xFFu) << 16);
    d.stencil[2 * f] = p->pipe.stencil[2 * f];
    d.stencil[2 * f + 1] = w1;
  }
  if (p->layout && !snapshot_descriptors(cb, p, dr)) return false;
  return true;
}

static uint32_t fetch_limit(const CommandBuffer* cb, const KzPipe& kp, bool per_instance);

static void record_draw(CommandBuffer* cb, uint32_t tri_count, uint32_t instances, uint32_t first_instance, bool indexed,
                        uint32_t first_index, int32_t vertex_offset) {
  if (!draw_state_ok(cb) || cb->pipe->rasterizer_discard || tri_count == 0 || instances == 0) return;
  DrawRec dr;
  int nreads = 0;
  if (!begin_draw(cb, indexed, dr, nreads)) return;
  KzDraw& d = dr.d;
  /* the draw's elements and instances must lie in the bound buffers, as kz_k_indirect checks for indirect
   * commands; a draw outside them is skipped, so no fetch leaves a buffer */
  const KzPipe& kp = cb->pipe->pipe;
  uint64_t elems = indexed ? (cb->ib->mem && cb->ib_off < cb->ib->size
                                  ? (cb->ib->size - cb->ib_off) / (d.indexed == 1 ? 4u : 2u) : 0)
                           : fetch_limit(cb, kp, false);
  uint64_t first_elem = indexed ? first_index : (uint64_t)(uint32_t)vertex_offset;
  if (first_elem + 3ull * tri_count > elems || (uint64_t)first_instance + instances > fetch_limit(cb, kp, true)) {
    log_error("draw skipped: elements [%llu, %llu) or instances [%u, %llu) outside the bound buffers",
              (unsigned long long)first_elem, (unsigned long long)(first_elem + 3ull * tri_count), first_instance,
              (unsigned long long)first_instance + instances);
    return;
  }
  if (indexed) d.ib = d.ib_base + (uint64_t)first_index * (d.indexed == 1 ? 4u : 2u);
  d.vertex_offset = vertex_offset;
  d.first_instance = first_instance;
  d.instance_count = instances;
  d.tri_count = tri_count;
  dr.triangles = (uint64_t)tri_count * instances;
  cb->passes[(size_t)cb->cur_pass].draws.push_back(dr);
}

static uint32_t attr_bytes(uint32_t fmt) {
  switch (fmt) {
    case KZ_FMT_F32x1: case KZ_FMT_U32x1: case KZ_FMT_U8x4_UNORM: return 4;
    case KZ_FMT_F32x2: case KZ_FMT_U32x2: return 8;
    case KZ_FMT_F32x3: case KZ_FMT_U32x3: return 12;
    default: return 16;
  }
}

/* how many vertices (per_instance false) or instances (true) every attribute the shaders read can fetch
 * from its bound vertex buffer; UINT32_MAX when no such attribute */
static uint32_t fetch_limit(const CommandBuffer* cb, const KzPipe& kp, bool per_instance) {
  uint64_t lim = 0xFFFFFFFFull;
  uint32_t used = kp.pos_input_mask | kp.full_input_mask;
  for (uint32_t i = 0; i < kp.num_attrs && i < KZ_MAX_VS_INPUTS; i++) {
    const KzAttr& a = kp.attrs[i];
    if (!((used >> a.location) & 1u) || (((kp.binding_instanced >> a.binding) & 1u) != 0) != per_instance) continue;
    const Buffer* b = cb->vb[a.binding];
    uint64_t avail = b && b->mem && cb->vb_off[a.binding] < b->size ? b->size - cb->vb_off[a.binding] : 0;
    uint64_t need = (uint64_t)a.offset + attr_bytes(a.format), stride = kp.binding_stride[a.binding];
    uint64_t n = avail < need ? 0 : stride == 0 ? 0xFFFFFFFFull : (avail - need) / stride + 1;
    lim = std::min(lim, n);
  }
  return (uint32_t)lim;
}

/* vkCmdDrawIndirect / vkCmdDrawIndexedIndirect: one KzDraw per command, whose counts kz_k_indirect reads
 * from the buffer when the command buffer executes (so the buffer may be written by earlier commands or by
 * the host between submissions) */
static void record_indirect(CommandBuffer* cb, VkBuffer buffer, VkDeviceSize offset, uint32_t draw_count,
                            uint32_t stride, bool indexed, VkBuffer count_buffer = nullptr,
                            VkDeviceSize count_offset = 0) {
  if (!draw_state_ok(cb) || cb->pipe->rasterizer_discard || draw_count == 0) return;
  const Buffer* buf = H<Buffer>(buffer);
  const Buffer* cbuf = H<Buffer>(count_buffer);
  if (count_buffer && (!cbuf || !cbuf->mem || (count_offset & 3) || count_offset + 4 > cbuf->size)) {
    log_error("indirect draw count: offset %llu does not fit the count buffer", (unsigned long long)count_offset);
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  uint32_t cmd_bytes = indexed ? 20u : 16u;
  if (draw_count == 1) stride = cmd_bytes;
  if (!buf || !buf->mem || (offset & 3) || (stride & 3) || stride < cmd_bytes ||
      offset + (VkDeviceSize)(draw_count - 1) * stride + cmd_bytes > buf->size) {
    log_error("indirect draw: offset %llu, stride %u, %u commands do not fit the buffer",
              (unsigned long long)offset, stride, draw_count);
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  DrawRec dr;
  int nreads = 0;
  if (!begin_draw(cb, indexed, dr, nreads)) return;
  dr.reads[nreads++] = buf->mem;
  if (cbuf) dr.reads[nreads++] = cbuf->mem;
  KzDraw& d = dr.d;
  if (cbuf) d.count_addr = (uint64_t)(uintptr_t)(cbuf->ptr() + count_offset);
  const KzPipe& kp = cb->pipe->pipe;
  if (indexed) {
    uint32_t isz = d.indexed == 1 ? 4u : 2u;
    d.elem_limit = (uint32_t)std::min<uint64_t>(
        cb->ib->mem && cb->ib_off < cb->ib->size ? (cb->ib->size - cb->ib_off) / isz : 0, 0xFFFFFFFFull);
  } else {
    d.elem_limit = fetch_limit(cb, kp, false);
  }
  d.instance_limit = fetch_limit(cb, kp, true);
  dr.triangles = 0;
  dr.indirect = true;
  PassRec& pass = cb->passes[(size_t)cb->cur_pass];
  for (uint32_t i = 0; i < draw_count; i++) {
    d.indirect = (uint64_t)(uintptr_t)(buf->ptr() + offset + (VkDeviceSize)i * stride);
    d.call_index = i;
    pass.draws.push_back(dr);
  }
}

}  // namespace kz

using namespace kz;

extern "C" {

VkResult VKAPI_CALL kzCreateCommandPool(VkDevice device, const VkCommandPoolCreateInfo* ci, const VkAllocationCallbacks*,
                                        VkCommandPool* out) {
  /* api_impl.rs:4436 vkCreateCommandPool */
  if (!ci || ci->queueFamilyIndex != 0) return VK_ERROR_INITIALIZATION_FAILED;
  CommandPool* pool = new CommandPool();
  pool->dev = H<Device>(device);
  *out = reinterpret_cast<VkCommandPool>(pool);
  return VK_SUCCESS;
}

namespace kz {
static void process_completions(Queue* q, bool block_all);
}

/* finish and retire every submission on the device's queue, so that none refers to a command buffer that
 * is about to be freed or re-recorded */
static void drain_queue(Device* dev) {
  std::lock_guard<std::recursive_mutex> lock(dev->mu);
  cudaSetDevice(dev->pd->cuda_device);
  process_completions(&dev->queue, true);
  cudaStreamSynchronize(dev->queue.stream);
}

static void destroy_cb(CommandBuffer* cb) {
  if (cb->low) {
    drain_queue(cb->dev);
    free_lowered(cb->low.get());
  }
  delete cb;
}

void VKAPI_CALL kzDestroyCommandPool(VkDevice, VkCommandPool pool_h, const VkAllocationCallbacks*) {
  CommandPool* pool = H<CommandPool>(pool_h);
  if (!pool) return;
  for (CommandBuffer* cb : pool->buffers) destroy_cb(cb);
  delete pool;
}

static void reset_cb(CommandBuffer* cb) {
  if (cb->low) {
    drain_queue(cb->dev);
    free_lowered(cb->low.get());
    cb->low.reset();
  }
  cb->recording = false;
  cb->pipe = nullptr;
  cb->have_viewport = cb->have_scissor = cb->have_blend_const = false;
  std::memset(cb->vb, 0, sizeof cb->vb);
  std::memset(cb->vb_off, 0, sizeof cb->vb_off);
  cb->ib = nullptr;
  cb->ib_off = 0;
  std::memset(cb->push, 0, sizeof cb->push);
  for (int s = 0; s < KZ_MAX_DESC_SETS; s++) {
    cb->sets[s] = nullptr;
    cb->dyn_offsets[s].clear();
  }
  std::memset(cb->stencil_dyn, 0, sizeof cb->stencil_dyn);
  cb->cur_pass = -1;
  cb->passes.clear();
  cb->ops.clear();
  cb->record_error = VK_SUCCESS;
}

VkResult VKAPI_CALL kzResetCommandPool(VkDevice, VkCommandPool pool_h, VkCommandPoolResetFlags) {
  CommandPool* pool = H<CommandPool>(pool_h);
  for (CommandBuffer* cb : pool->buffers) reset_cb(cb);
  return VK_SUCCESS;
}

VkResult VKAPI_CALL kzAllocateCommandBuffers(VkDevice device, const VkCommandBufferAllocateInfo* ai,
                                             VkCommandBuffer* out) {
  /* api_impl.rs:4464 vkAllocateCommandBuffers (secondary command buffers are not supported) */
  if (!ai || ai->level != VK_COMMAND_BUFFER_LEVEL_PRIMARY) return VK_ERROR_FEATURE_NOT_PRESENT;
  CommandPool* pool = H<CommandPool>(ai->commandPool);
  for (uint32_t i = 0; i < ai->commandBufferCount; i++) {
    CommandBuffer* cb = new CommandBuffer();
    cb->dev = H<Device>(device);
    cb->pool = pool;
    pool->buffers.push_back(cb);
    out[i] = reinterpret_cast<VkCommandBuffer>(cb);
  }
  return VK_SUCCESS;
}

void VKAPI_CALL kzFreeCommandBuffers(VkDevice, VkCommandPool pool_h, uint32_t n, const VkCommandBuffer* cbs) {
  CommandPool* pool = H<CommandPool>(pool_h);
  for (uint32_t i = 0; i < n; i++) {
    CommandBuffer* cb = H<CommandBuffer>(cbs[i]);
    if (!cb) continue;
    for (size_t k = 0; k < pool->buffers.size(); k++)
      if (pool->buffers[k] == cb) {
        pool->buffers.erase(pool->buffers.begin() + (long)k);
        break;
      }
    destroy_cb(cb);
  }
}

VkResult VKAPI_CALL kzBeginCommandBuffer(VkCommandBuffer cbh, const VkCommandBufferBeginInfo*) {
  /* api_impl.rs:4483 vkBeginCommandBuffer (implicit reset) */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  reset_cb(cb);
  cb->recording = true;
  return VK_SUCCESS;
}

VkResult VKAPI_CALL kzEndCommandBuffer(VkCommandBuffer cbh) {
  /* api_impl.rs:4491 vkEndCommandBuffer: lower and capture */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (!cb->recording) return VK_ERROR_INITIALIZATION_FAILED;
  cb->recording = false;
  if (cb->record_error != VK_SUCCESS) return cb->record_error;
  return lower_command_buffer(cb);
}

VkResult VKAPI_CALL kzResetCommandBuffer(VkCommandBuffer cbh, VkCommandBufferResetFlags) {
  reset_cb(H<CommandBuffer>(cbh));
  return VK_SUCCESS;
}

void VKAPI_CALL kzCmdBindPipeline(VkCommandBuffer cbh, VkPipelineBindPoint bp, VkPipeline p) {
  /* api_impl.rs:4506 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (bp != VK_PIPELINE_BIND_POINT_GRAPHICS) {
    cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
    return;
  }
  cb->pipe = H<Pipeline>(p);
}

void VKAPI_CALL kzCmdSetViewport(VkCommandBuffer cbh, uint32_t first, uint32_t n, const VkViewport* vps) {
  /* api_impl.rs:4515 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (first == 0 && n >= 1) {
    cb->viewport = vps[0];
    cb->have_viewport = true;
  }
}

void VKAPI_CALL kzCmdSetScissor(VkCommandBuffer cbh, uint32_t first, uint32_t n, const VkRect2D* sc) {
  /* api_impl.rs:4525 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (first == 0 && n >= 1) {
    cb->scissor = sc[0];
    cb->have_scissor = true;
  }
}

void VKAPI_CALL kzCmdSetBlendConstants(VkCommandBuffer cbh, const float c[4]) {
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  std::memcpy(cb->blend_const, c, sizeof cb->blend_const);
  cb->have_blend_const = true;
}

void VKAPI_CALL kzCmdBindVertexBuffers(VkCommandBuffer cbh, uint32_t first, uint32_t n, const VkBuffer* bufs,
                                       const VkDeviceSize* offs) {
  /* api_impl.rs:4621 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  for (uint32_t i = 0; i < n && first + i < KZ_MAX_BINDINGS; i++) {
    cb->vb[first + i] = H<Buffer>(bufs[i]);
    cb->vb_off[first + i] = offs[i];
  }
}

void VKAPI_CALL kzCmdBindIndexBuffer(VkCommandBuffer cbh, VkBuffer buf, VkDeviceSize off, VkIndexType type) {
  /* api_impl.rs:4611 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  cb->ib = H<Buffer>(buf);
  cb->ib_off = off;
  cb->ib_type = type;
}

void VKAPI_CALL kzCmdPushConstants(VkCommandBuffer cbh, VkPipelineLayout, VkShaderStageFlags, uint32_t offset,
                                   uint32_t size, const void* data) {
  /* api_impl.rs:4932 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (offset + size > KZ_PUSH_BYTES) {
    cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
    return;
  }
  std::memcpy(cb->push + offset, data, size);
}

void VKAPI_CALL kzCmdDraw(VkCommandBuffer cbh, uint32_t vertexCount, uint32_t instanceCount, uint32_t firstVertex,
                          uint32_t firstInstance) {
  /* api_impl.rs:4632 vkCmdDraw: triangle list over vertices firstVertex + k */
  record_draw(H<CommandBuffer>(cbh), vertexCount / 3, instanceCount, firstInstance, false, 0, (int32_t)firstVertex);
}

void VKAPI_CALL kzCmdDrawIndexed(VkCommandBuffer cbh, uint32_t indexCount, uint32_t instanceCount, uint32_t firstIndex,
                                 int32_t vertexOffset, uint32_t firstInstance) {
  /* api_impl.rs:4643 vkCmdDrawIndexed: vertex = index[firstIndex + k] + vertexOffset */
  record_draw(H<CommandBuffer>(cbh), indexCount / 3, instanceCount, firstInstance, true, firstIndex, vertexOffset);
}

void VKAPI_CALL kzCmdBindDescriptorSets(VkCommandBuffer cbh, VkPipelineBindPoint bp, VkPipelineLayout,
                                        uint32_t firstSet, uint32_t count, const VkDescriptorSet* sets,
                                        uint32_t dynCount, const uint32_t* dynOffsets) {
  /* api_impl.rs:4597 vkCmdBindDescriptorSets: each set consumes as many dynamic offsets as it has dynamic
   * uniform buffers, in order */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (bp != VK_PIPELINE_BIND_POINT_GRAPHICS || firstSet + count > KZ_MAX_DESC_SETS) {
    cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
    return;
  }
  uint32_t used = 0;
  for (uint32_t i = 0; i < count; i++) {
    DescriptorSet* s = H<DescriptorSet>(sets[i]);
    cb->sets[firstSet + i] = s;
    std::vector<uint32_t>& offs = cb->dyn_offsets[firstSet + i];
    offs.clear();
    for (uint32_t k = 0; s && k < s->layout->dynamic && used < dynCount; k++) offs.push_back(dynOffsets[used++]);
  }
}

void VKAPI_CALL kzCmdDrawIndirect(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize offset, uint32_t drawCount,
                                  uint32_t stride) {
  /* api_impl.rs:4655 vkCmdDrawIndirect: drawCount VkDrawIndirectCommand structs, `stride` bytes apart */
  record_indirect(H<CommandBuffer>(cbh), buffer, offset, drawCount, stride, false);
}

void VKAPI_CALL kzCmdDrawIndexedIndirect(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize offset,
                                         uint32_t drawCount, uint32_t stride) {
  /* api_impl.rs:4666 vkCmdDrawIndexedIndirect: drawCount VkDrawIndexedIndirectCommand structs */
  record_indirect(H<CommandBuffer>(cbh), buffer, offset, drawCount, stride, true);
}

void VKAPI_CALL kzCmdDrawIndirectCount(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize offset, VkBuffer countBuffer,
                                       VkDeviceSize countBufferOffset, uint32_t maxDrawCount, uint32_t stride) {
  /* api_impl.rs:6025 vkCmdDrawIndirectCountKHR: min(count, maxDrawCount) commands, the count read from
   * countBuffer when the command buffer executes */
  record_indirect(H<CommandBuffer>(cbh), buffer, offset, maxDrawCount, stride, false, countBuffer, countBufferOffset);
}

void VKAPI_CALL kzCmdDrawIndexedIndirectCount(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize offset,
                                              VkBuffer countBuffer, VkDeviceSize countBufferOffset,
                                              uint32_t maxDrawCount, uint32_t stride) {
  /* api_impl.rs:6039 vkCmdDrawIndexedIndirectCountKHR */
  record_indirect(H<CommandBuffer>(cbh), buffer, offset, maxDrawCount, stride, true, countBuffer, countBufferOffset);
}

/* every attachment of the pass is an image with memory bound and at least the framebuffer's size, so no
 * kernel of the pass addresses memory outside an attachment */
static bool pass_targets_ok(const Framebuffer* fb, const RenderPass* rp) {
  if (!fb || !rp) return false;
  for (int a : {rp->color_att, rp->depth_att, rp->resolve_att}) {
    if (a < 0) continue;
    if ((size_t)a >= fb->views.size() || !fb->views[(size_t)a] || !fb->views[(size_t)a]->image) return false;
    const Image* im = fb->views[(size_t)a]->image;
    if (!im->mem || im->width < fb->width || im->height < fb->height) return false;
  }
  return true;
}

void VKAPI_CALL kzCmdBeginRenderPass(VkCommandBuffer cbh, const VkRenderPassBeginInfo* bi, VkSubpassContents) {
  /* api_impl.rs:4944 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (!bi || !pass_targets_ok(H<Framebuffer>(bi->framebuffer), H<RenderPass>(bi->renderPass))) {
    log_error("render pass begun with a missing attachment, one without memory, or one smaller than the framebuffer");
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  PassRec pr;
  pr.fb = H<Framebuffer>(bi->framebuffer);
  pr.rp = H<RenderPass>(bi->renderPass);
  pr.area[0] = bi->renderArea.offset.x;
  pr.area[1] = bi->renderArea.offset.y;
  pr.area[2] = bi->renderArea.offset.x + (int32_t)bi->renderArea.extent.width;
  pr.area[3] = bi->renderArea.offset.y + (int32_t)bi->renderArea.extent.height;
  if (pr.rp->color_att >= 0 && (uint32_t)pr.rp->color_att < bi->clearValueCount)
    pr.clear_color = bi->pClearValues[pr.rp->color_att];
  if (pr.rp->depth_att >= 0 && (uint32_t)pr.rp->depth_att < bi->clearValueCount)
    pr.clear_depth = bi->pClearValues[pr.rp->depth_att];
  cb->passes.push_back(pr);
  cb->cur_pass = (int)cb->passes.size() - 1;
  RecOp op;
  op.kind = OpKind::Pass;
  op.pass = cb->passes.size() - 1;
  cb->ops.push_back(op);
}

static void clear_image(CommandBuffer* cb, Image* img, uint32_t value);

static void record_resolve(CommandBuffer* cb, Image* src, Image* dst, int32_t sx, int32_t sy, int32_t dx, int32_t dy,
                           int32_t w, int32_t h) {
  RecOp op;
  op.kind = OpKind::Resolve;
  op.src = src->ptr();
  op.spitch = src->pitch;
  op.dst = dst->ptr();
  op.dpitch = dst->pitch;
  op.rect[0] = sx;
  op.rect[1] = sy;
  op.rect[2] = w;
  op.rect[3] = h;
  op.dst_x = dx;
  op.dst_y = dy;
  op.rmem = src->mem;
  op.wmem = dst->mem;
  cb->ops.push_back(op);
}

void VKAPI_CALL kzCmdEndRenderPass(VkCommandBuffer cbh) {
  /* api_impl.rs:4961; a subpass resolve attachment receives the average of the colour attachment's samples
   * over the render area */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (cb->cur_pass >= 0) {
    const PassRec& pr = cb->passes[(size_t)cb->cur_pass];
    const RenderPass* rp = pr.rp;
    if (rp->resolve_att >= 0 && rp->color_att >= 0 && (size_t)rp->resolve_att < pr.fb->views.size() &&
        (size_t)rp->color_att < pr.fb->views.size()) {
      Image* src = pr.fb->views[(size_t)rp->color_att]->image;
      Image* dst = pr.fb->views[(size_t)rp->resolve_att]->image;
      int32_t x0 = std::max(0, pr.area[0]), y0 = std::max(0, pr.area[1]);
      int32_t x1 = std::min({pr.area[2], (int32_t)src->width, (int32_t)dst->width});
      int32_t y1 = std::min({pr.area[3], (int32_t)src->height, (int32_t)dst->height});
      if (src->samples > 1 && dst->samples == 1 && x1 > x0 && y1 > y0)
        record_resolve(cb, src, dst, x0, y0, x0, y0, x1 - x0, y1 - y0);
    }
  }
  cb->cur_pass = -1;
}

void VKAPI_CALL kzCmdClearAttachments(VkCommandBuffer cbh, uint32_t n, const VkClearAttachment* atts, uint32_t nr,
                                      const VkClearRect* rects) {
  /* vkCmdClearAttachments inside a render pass: the draws recorded so far and the ones after the clears
   * become two passes over the same framebuffer (the second loads its attachments), with the clears, rects
   * clipped to the framebuffer and render area, in between */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (cb->cur_pass < 0) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  const PassRec cur = cb->passes[(size_t)cb->cur_pass];
  const RenderPass* rp = cur.rp;
  for (uint32_t i = 0; i < n; i++) {
    const VkClearAttachment& a = atts[i];
    int att = (a.aspectMask & VK_IMAGE_ASPECT_COLOR_BIT) ? (a.colorAttachment == 0 ? rp->color_att : -1) : rp->depth_att;
    if (att < 0 || (size_t)att >= cur.fb->views.size()) continue;
    Image* img = cur.fb->views[(size_t)att]->image;
    uint32_t value;
    if (a.aspectMask & VK_IMAGE_ASPECT_COLOR_BIT) {
      value = pack_color(img->format, a.clearValue.color.float32);
    } else if (img->format == VK_FORMAT_D32_SFLOAT) {
      value = float_bits(a.clearValue.depthStencil.depth);
    } else if (img->format == VK_FORMAT_D24_UNORM_S8_UINT &&
               (a.aspectMask & (VK_IMAGE_ASPECT_DEPTH_BIT | VK_IMAGE_ASPECT_STENCIL_BIT)) ==
                   (VK_IMAGE_ASPECT_DEPTH_BIT | VK_IMAGE_ASPECT_STENCIL_BIT)) {
      value = (uint32_t)std::rint(a.clearValue.depthStencil.depth * 16777215.0f) |
              ((a.clearValue.depthStencil.stencil & 0xFFu) << 24);
    } else {
      log_error("vkCmdClearAttachments: D16 images and single aspects of D24S8 are not cleared by rectangle");
      cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
      return;
    }
    for (uint32_t k = 0; k < nr; k++) {
      const VkRect2D& r = rects[k].rect;
      int32_t x0 = std::max({r.offset.x, cur.area[0], 0}), y0 = std::max({r.offset.y, cur.area[1], 0});
      int32_t x1 = std::min({r.offset.x + (int32_t)r.extent.width, cur.area[2], (int32_t)img->width});
      int32_t y1 = std::min({r.offset.y + (int32_t)r.extent.height, cur.area[3], (int32_t)img->height});
      if (x1 <= x0 || y1 <= y0) continue;
      clear_image(cb, img, value);
      RecOp& op = cb->ops.back();
      const int32_t spp = (int32_t)img->samples; /* 32-bit words per pixel */
      op.rect[0] = x0 * spp;
      op.rect[1] = y0;
      op.rect[2] = x1 * spp;
      op.rect[3] = y1;
    }
  }
  PassRec next;
  next.fb = cur.fb;
  next.rp = cur.rp;
  std::memcpy(next.area, cur.area, sizeof next.area);
  next.clear_color = cur.clear_color;
  next.clear_depth = cur.clear_depth;
  next.cont = true;
  cb->passes.push_back(next);
  cb->cur_pass = (int)cb->passes.size() - 1;
  RecOp op;
  op.kind = OpKind::Pass;
  op.pass = cb->passes.size() - 1;
  cb->ops.push_back(op);
}

void VKAPI_CALL kzCmdResolveImage(VkCommandBuffer cbh, VkImage srcImage, VkImageLayout, VkImage dstImage,
                                  VkImageLayout, uint32_t n, const VkImageResolve* regions) {
  /* vkCmdResolveImage: each region's samples averaged into the single-sample image, clipped to both images */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Image* src = H<Image>(srcImage);
  Image* dst = H<Image>(dstImage);
  if (!src || !dst || !src->mem || !dst->mem) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  if (src->samples <= 1 || dst->samples != 1) {
    cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
    return;
  }
  for (uint32_t i = 0; i < n; i++) {
    const VkImageResolve& r = regions[i];
    int32_t w = (int32_t)r.extent.width, h = (int32_t)r.extent.height;
    w = std::min({w, (int32_t)src->width - r.srcOffset.x, (int32_t)dst->width - r.dstOffset.x});
    h = std::min({h, (int32_t)src->height - r.srcOffset.y, (int32_t)dst->height - r.dstOffset.y});
    if (w <= 0 || h <= 0 || r.srcOffset.x < 0 || r.srcOffset.y < 0 || r.dstOffset.x < 0 || r.dstOffset.y < 0) continue;
    record_resolve(cb, src, dst, r.srcOffset.x, r.srcOffset.y, r.dstOffset.x, r.dstOffset.y, w, h);
  }
}

static void clear_image(CommandBuffer* cb, Image* img, uint32_t value) {
  if (!img || !img->mem) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  RecOp op;
  op.kind = OpKind::Clear;
  op.base = img->ptr();
  op.pitch = img->pitch;
  op.rect[0] = 0;
  op.rect[1] = 0;
  op.rect[2] = (int32_t)img->width;
  op.rect[3] = (int32_t)img->height;
  op.value = value;
  op.wmem = img->mem;
  cb->ops.push_back(op);
}

void VKAPI_CALL kzCmdClearColorImage(VkCommandBuffer cbh, VkImage image, VkImageLayout, const VkClearColorValue* c,
                                     uint32_t, const VkImageSubresourceRange*) {
  /* api_impl.rs:4780 vkCmdClearColorImage: the clear colour converted to the image format (UNORM8, round
   * to nearest even) fills the single mip level / layer */
  Image* img = H<Image>(image);
  clear_image(H<CommandBuffer>(cbh), img, pack_color(img->format, c->float32));
}

void VKAPI_CALL kzCmdClearDepthStencilImage(VkCommandBuffer cbh, VkImage image, VkImageLayout,
                                            const VkClearDepthStencilValue* v, uint32_t n,
                                            const VkImageSubresourceRange* ranges) {
  /* api_impl.rs:4792: the clear value in the image's format (D16 / D24: rint(depth * (2^bits - 1)), as the
   * kernels convert fragment depths); a D24S8 image is cleared in both aspects at once */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Image* img = H<Image>(image);
  if (img->format == VK_FORMAT_D16_UNORM) {
    uint32_t q = (uint32_t)std::rint(v->depth * 65535.0f);
    clear_image(cb, img, q | (q << 16));
    cb->ops.back().rect[2] = (int32_t)((img->width + 1) / 2); /* two texels per 32-bit word */
  } else if (img->format == VK_FORMAT_D24_UNORM_S8_UINT) {
    VkImageAspectFlags aspects = 0;
    for (uint32_t i = 0; i < n; i++) aspects |= ranges[i].aspectMask;
    if ((aspects & (VK_IMAGE_ASPECT_DEPTH_BIT | VK_IMAGE_ASPECT_STENCIL_BIT)) !=
        (VK_IMAGE_ASPECT_DEPTH_BIT | VK_IMAGE_ASPECT_STENCIL_BIT)) {
      log_error("vkCmdClearDepthStencilImage: a D24S8 image is cleared in both aspects together");
      cb->record_error = VK_ERROR_FEATURE_NOT_PRESENT;
      return;
    }
    clear_image(cb, img, (uint32_t)std::rint(v->depth * 16777215.0f) | ((v->stencil & 0xFFu) << 24));
  } else {
    clear_image(cb, img, float_bits(v->depth));
  }
}

void VKAPI_CALL kzCmdPipelineBarrier(VkCommandBuffer, VkPipelineStageFlags, VkPipelineStageFlags, VkDependencyFlags,
                                     uint32_t, const VkMemoryBarrier*, uint32_t, const VkBufferMemoryBarrier*,
                                     uint32_t, const VkImageMemoryBarrier*) {
  /* api_impl.rs:4863: every command executes in order on one stream, so barriers order nothing new */
}

/* A transfer region must lie inside memory the object has bound; a region that does not is a recording
   error (the command buffer's vkEndCommandBuffer fails), so no copy or fill ever leaves its object. */
static bool buffer_range_ok(const Buffer* b, VkDeviceSize off, VkDeviceSize size) {
  return b && b->mem && off <= b->size && size <= b->size - off;
}

static bool image_rect_ok(const Image* img, int32_t x, int32_t y, uint32_t w, uint32_t h) {
  return img && img->mem && x >= 0 && y >= 0 && (uint64_t)x + w <= img->width && (uint64_t)y + h <= img->height;
}

void VKAPI_CALL kzCmdCopyBuffer(VkCommandBuffer cbh, VkBuffer src, VkBuffer dst, uint32_t n, const VkBufferCopy* r) {
  /* api_impl.rs:4696 */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Buffer* s = H<Buffer>(src);
  Buffer* d = H<Buffer>(dst);
  for (uint32_t i = 0; i < n; i++) {
    if (!buffer_range_ok(s, r[i].srcOffset, r[i].size) || !buffer_range_ok(d, r[i].dstOffset, r[i].size)) {
      cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
      return;
    }
    RecOp op;
    op.kind = OpKind::Copy;
    op.src = s->ptr() + r[i].srcOffset;
    op.dst = d->ptr() + r[i].dstOffset;
    op.bytes = (size_t)r[i].size;
    op.rmem = s->mem;
    op.wmem = d->mem;
    cb->ops.push_back(op);
  }
}

static void image_buffer_copy(CommandBuffer* cb, Image* img, Buffer* buf, const VkBufferImageCopy& r, bool to_buffer) {
  /* one-sample images only; the buffer's rows are bufferRowLength texels apart (the extent's width if 0) */
  uint32_t row_len = r.bufferRowLength ? r.bufferRowLength : r.imageExtent.width;
  if (!img || img->samples != 1 || row_len < r.imageExtent.width ||
      !image_rect_ok(img, r.imageOffset.x, r.imageOffset.y, r.imageExtent.width, r.imageExtent.height)) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  size_t bpitch = (size_t)row_len * img->bpp;
  VkDeviceSize span = r.imageExtent.height == 0 || r.imageExtent.width == 0
                          ? 0
                          : (VkDeviceSize)bpitch * (r.imageExtent.height - 1) + (VkDeviceSize)r.imageExtent.width * img->bpp;
  if (!buffer_range_ok(buf, r.bufferOffset, span)) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  if (span == 0) return;
  RecOp op;
  op.kind = OpKind::Copy2D;
  char* ip = img->ptr() + (size_t)r.imageOffset.y * img->pitch + (size_t)r.imageOffset.x * img->bpp;
  char* bp = buf->ptr() + r.bufferOffset;
  op.width_bytes = (size_t)r.imageExtent.width * img->bpp;
  op.rows = r.imageExtent.height;
  if (to_buffer) {
    op.dst = bp;
    op.dpitch = bpitch;
    op.src = ip;
    op.spitch = img->pitch;
    op.rmem = img->mem;
    op.wmem = buf->mem;
  } else {
    op.dst = ip;
    op.dpitch = img->pitch;
    op.src = bp;
    op.spitch = bpitch;
    op.rmem = buf->mem;
    op.wmem = img->mem;
  }
  cb->ops.push_back(op);
}

void VKAPI_CALL kzCmdCopyImageToBuffer(VkCommandBuffer cbh, VkImage image, VkImageLayout, VkBuffer buffer, uint32_t n,
                                       const VkBufferImageCopy* r) {
  /* api_impl.rs:4746 */
  for (uint32_t i = 0; i < n; i++) image_buffer_copy(H<CommandBuffer>(cbh), H<Image>(image), H<Buffer>(buffer), r[i], true);
}

void VKAPI_CALL kzCmdCopyBufferToImage(VkCommandBuffer cbh, VkBuffer buffer, VkImage image, VkImageLayout, uint32_t n,
                                       const VkBufferImageCopy* r) {
  for (uint32_t i = 0; i < n; i++) image_buffer_copy(H<CommandBuffer>(cbh), H<Image>(image), H<Buffer>(buffer), r[i], false);
}

static void set_stencil_state(VkCommandBuffer cbh, int which, VkFlags faces, uint32_t v) {
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  if (faces & 1u) cb->stencil_dyn[which][0] = v; /* VK_STENCIL_FACE_FRONT_BIT */
  if (faces & 2u) cb->stencil_dyn[which][1] = v; /* VK_STENCIL_FACE_BACK_BIT */
}

void VKAPI_CALL kzCmdSetStencilCompareMask(VkCommandBuffer cbh, VkFlags faces, uint32_t v) {
  set_stencil_state(cbh, 0, faces, v);
}
void VKAPI_CALL kzCmdSetStencilWriteMask(VkCommandBuffer cbh, VkFlags faces, uint32_t v) {
  set_stencil_state(cbh, 1, faces, v);
}
void VKAPI_CALL kzCmdSetStencilReference(VkCommandBuffer cbh, VkFlags faces, uint32_t v) {
  set_stencil_state(cbh, 2, faces, v);
}

void VKAPI_CALL kzCmdUpdateBuffer(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize off, VkDeviceSize size,
                                  const void* data) {
  /* vkCmdUpdateBuffer: the bytes are copied at recording and written at execution, in command order */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Buffer* b = H<Buffer>(buffer);
  if (!b || (off & 3) || (size & 3) || size > 65536 || off + size > b->size) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  RecOp op;
  op.kind = OpKind::Copy;
  op.dst = b->ptr() + off;
  op.bytes = (size_t)size;
  op.data.assign(static_cast<const uint8_t*>(data), static_cast<const uint8_t*>(data) + size);
  op.wmem = b->mem;
  cb->ops.push_back(op);
}

void VKAPI_CALL kzCmdCopyImage(VkCommandBuffer cbh, VkImage srcImage, VkImageLayout, VkImage dstImage, VkImageLayout,
                               uint32_t n, const VkImageCopy* regions) {
  /* vkCmdCopyImage between images of the same texel size and sample count, clipped to both */
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Image* s = H<Image>(srcImage);
  Image* d = H<Image>(dstImage);
  if (!s || !d || !s->mem || !d->mem) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  if (s->bpp != d->bpp || s->samples != d->samples) {
    cb->record_error = VK_ERROR_FORMAT_NOT_SUPPORTED;
    return;
  }
  const size_t tb = (size_t)s->bpp * s->samples;
  for (uint32_t i = 0; i < n; i++) {
    const VkImageCopy& r = regions[i];
    if (r.srcOffset.x < 0 || r.srcOffset.y < 0 || r.dstOffset.x < 0 || r.dstOffset.y < 0) continue;
    int32_t w = std::min({(int32_t)r.extent.width, (int32_t)s->width - r.srcOffset.x, (int32_t)d->width - r.dstOffset.x});
    int32_t h = std::min({(int32_t)r.extent.height, (int32_t)s->height - r.srcOffset.y,
                          (int32_t)d->height - r.dstOffset.y});
    if (w <= 0 || h <= 0) continue;
    RecOp op;
    op.kind = OpKind::Copy2D;
    op.src = s->ptr() + (size_t)r.srcOffset.y * s->pitch + (size_t)r.srcOffset.x * tb;
    op.spitch = s->pitch;
    op.dst = d->ptr() + (size_t)r.dstOffset.y * d->pitch + (size_t)r.dstOffset.x * tb;
    op.dpitch = d->pitch;
    op.width_bytes = (size_t)w * tb;
    op.rows = (size_t)h;
    op.rmem = s->mem;
    op.wmem = d->mem;
    cb->ops.push_back(op);
  }
}

void VKAPI_CALL kzCmdFillBuffer(VkCommandBuffer cbh, VkBuffer buffer, VkDeviceSize off, VkDeviceSize size,
                                uint32_t data) {
  CommandBuffer* cb = H<CommandBuffer>(cbh);
  Buffer* b = H<Buffer>(buffer);
  if (b && off <= b->size && size == VK_WHOLE_SIZE) size = (b->size - off) & ~(VkDeviceSize)3;
  if (!buffer_range_ok(b, off, size) || (off & 3) || (size & 3) || size / 4 > (VkDeviceSize)INT32_MAX) {
    cb->record_error = VK_ERROR_INITIALIZATION_FAILED;
    return;
  }
  if (size == 0) return;
  RecOp op;
  op.kind = OpKind::Fill;
  op.base = b->ptr() + off;
  op.pitch = (uint32_t)size;
  op.rect[0] = 0;
  op.rect[1] = 0;
  op.rect[2] = (int32_t)(size / 4);
  op.rect[3] = 1;
  op.value = data;
  op.wmem = b->mem;
  cb->ops.push_back(op);
}

}  // extern "C"

namespace kz {

/* ------------------------------------------------------------------------------------------------ */
/* lowering                                                                                         */

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

void free_lowered(Lowered* low) {
  if (!low) return;
  if (low->exec) cudaGraphExecDestroy(low->exec);
  if (low->graph) cudaGraphDestroy(low->graph);
  if (low->ev_begin) cudaEventDestroy(low->ev_begin);
  if (low->ev_end) cudaEventDestroy(low->ev_end);
  device_free(low->d_tables);
  device_free(low->d_records);
  device_free(low->d_bins);
  device_free(low->d_shades);
  low->d_shades = nullptr;
  device_free(low->d_tiles);
  device_free(low->d_inline);
  low->d_inline = nullptr;
  device_free(low->d_vis);
  low->d_vis = nullptr;
  if (low->h_status) cudaFreeHost(low->h_status);
  low->exec = nullptr;
  low->graph = nullptr;
  low->d_tables = low->d_records = low->d_bins = nullptr;
  low->d_tiles = nullptr;
  low->h_status = nullptr;
}

static void add_unique(std::vector<DeviceMemory*>& v, DeviceMemory* m) {
  if (!m) return;
  for (DeviceMemory* x : v)
    if (x == m) return;
  v.push_back(m);
}

static uint32_t color_format(VkFormat f) {
  /* texture images: UNORM only (sampling does not decode sRGB) */
  if (f == VK_FORMAT_R8G8B8A8_UNORM) return KZ_CF_RGBA8;
  if (f == VK_FORMAT_B8G8R8A8_UNORM) return KZ_CF_BGRA8;
  return KZ_CF_NONE;
}

static uint32_t attachment_format(VkFormat f) {
  if (f == VK_FORMAT_R8G8B8A8_SRGB) return KZ_CF_RGBA8_SRGB;
  if (f == VK_FORMAT_B8G8R8A8_SRGB) return KZ_CF_BGRA8_SRGB;
  return color_format(f);
}

/* fill the framebuffer part of a segment from a render pass instance */
static void segment_target(const PassRec& pr, KzSegment& s, uint32_t tile, bool first, Lowered& low) {
  const RenderPass* rp = pr.rp;
  const Framebuffer* fb = pr.fb;
  s.width = fb->width;
  s.height = fb->height;
  s.tile = tile;
  s.tiles_x = (s.width + tile - 1) / tile;
  s.tiles_y = (s.height + tile - 1) / tile;
  s.area[0] = std::max(0, pr.area[0]);
  s.area[1] = std::max(0, pr.area[1]);
  s.area[2] = std::min((int32_t)fb->width, pr.area[2]);
  s.area[3] = std::min((int32_t)fb->height, pr.area[3]);
  s.color_load = s.depth_load = KZ_LOAD_LOAD;
  s.color_store = s.depth_store = 1;
  s.samples = 1;
  /* multisampled passes render through tiles of at most 16 x 16 (the ordered raster keeps a pixel's four
   * samples in registers) */
  int ca = rp->color_att >= 0 && (size_t)rp->color_att < fb->views.size() ? rp->color_att : rp->depth_att;
  if (ca >= 0 && (size_t)ca < fb->views.size() && fb->views[(size_t)ca]->image->samples > 1) {
    s.samples = fb->views[(size_t)ca]->image->samples;
    if (tile > 16) tile = 16;
    s.tile = tile;
  }
  if (rp->color_att >= 0 && (size_t)rp->color_att < fb->views.size()) {
    Image* img = fb->views[(size_t)rp->color_att]->image;
    s.color = (uint64_t)(uintptr_t)img->ptr();
    s.color_pitch = img->pitch;
    s.color_format = attachment_format(img->format);
    s.width = std::min(s.width, img->width);
    s.height = std::min(s.height, img->height);
    const VkAttachmentDescription& a = rp->atts[(size_t)rp->color_att];
    if (first && a.loadOp == VK_ATTACHMENT_LOAD_OP_CLEAR) s.color_load = KZ_LOAD_CLEAR;
    s.clear_color = pack_color(img->format, pr.clear_color.color.float32);
    add_unique(low.writes, img->mem);
    if (s.color_load == KZ_LOAD_LOAD) add_unique(low.reads, img->mem);
  }
  if (rp->depth_att >= 0 && (size_t)rp->depth_att < fb->views.size()) {
    Image* img = fb->views[(size_t)rp->depth_att]->image;
    s.depth = (uint64_t)(uintptr_t)img->ptr();
    s.depth_pitch = img->pitch;
    s.width = std::min(s.width, img->width);
    s.height = std::min(s.height, img->height);
    const VkAttachmentDescription& a = rp->atts[(size_t)rp->depth_att];
    if (first && a.loadOp == VK_ATTACHMENT_LOAD_OP_CLEAR) s.depth_load = KZ_LOAD_CLEAR;
    s.clear_depth = pr.clear_depth.depthStencil.depth;
    s.stencil_load = KZ_LOAD_LOAD;
    if (img->format == VK_FORMAT_D16_UNORM) {
      s.depth_format = KZ_DF_D16;
      s.clear_depth = std::rint(s.clear_depth * 65535.0f);
    } else if (img->format == VK_FORMAT_D24_UNORM_S8_UINT) {
      s.depth_format = KZ_DF_D24S8;
      s.clear_depth = std::rint(s.clear_depth * 16777215.0f);
      s.clear_stencil = pr.clear_depth.depthStencil.stencil & 0xFFu;
      if (first && a.stencilLoadOp == VK_ATTACHMENT_LOAD_OP_CLEAR) s.stencil_load = KZ_LOAD_CLEAR;
    }
    add_unique(low.writes, img->mem);
    if (s.depth_load == KZ_LOAD_LOAD) add_unique(low.reads, img->mem);
  }
  /* colour and depth of a multisampled pass must have the same sample count (else the depth texels would
   * be addressed with the wrong width): a mismatched depth attachment is left out */
  if (s.depth && rp->depth_att >= 0 && fb->views[(size_t)rp->depth_att]->image->samples != s.samples) {
    log_error("render pass: depth attachment sample count differs from the colour attachment's; depth ignored");
    s.depth = 0;
  }
  s.tiles_x = (s.width + tile - 1) / tile;
  s.tiles_y = (s.height + tile - 1) / tile;
  s.area[2] = std::min((int32_t)s.width, s.area[2]);
  s.area[3] = std::min((int32_t)s.height, s.area[3]);
}

/* a vertex fetch with vector loads can merge some of the pipeline's attribute loads: an attribute the shaders
 * read with at least two 32-bit components, in a binding whose stride is a multiple of 8 bytes */
static bool fetch_vectorizable(const KzPipe& kp) {
  uint32_t used = kp.pos_input_mask | kp.full_input_mask;
  for (uint32_t i = 0; i < kp.num_attrs && i < KZ_MAX_VS_INPUTS; i++) {
    const KzAttr& a = kp.attrs[i];
    bool wide = (a.format >= KZ_FMT_F32x2 && a.format <= KZ_FMT_F32x4) || (a.format >= KZ_FMT_U32x2 && a.format <= KZ_FMT_U32x4);
    if (((used >> a.location) & 1u) && wide && kp.binding_stride[a.binding] % 8 == 0) return true;
  }
  return false;
}

/* every binding the shaders read starts 16-byte aligned in this draw */
static bool bases_aligned16(const KzDraw& d, const KzPipe& kp) {
  uint32_t used = kp.pos_input_mask | kp.full_input_mask;
  for (uint32_t i = 0; i < kp.num_attrs && i < KZ_MAX_VS_INPUTS; i++) {
    const KzAttr& a = kp.attrs[i];
    if (((used >> a.location) & 1u) && (d.vb[a.binding] & 15u)) return false;
  }
  return true;
}

static int raster_class(const DrawRec& d, bool vis_ok) {
  /* draws that share a class can share one segment: visibility mode with the same key and write mask,
   * or ordered mode; indirect draws never share a segment with direct ones.  Passes whose depth
   * attachment is not D32 render in ordered mode only. */
  int k = vis_ok && d.pipe->vis_key >= 0 ? 1 + d.pipe->vis_key + 16 * (int)d.pipe->pipe.write_mask : 0;
  return d.indirect ? k + 1024 : k;
}

static VkResult size_scratch(Device* dev, Lowered& low, uint32_t rec_cap, uint32_t pair_cap) {
  cudaSetDevice(dev->pd->cuda_device);
  device_free(low.d_records);
  device_free(low.d_bins);
  device_free(low.d_shades);
  low.d_records = low.d_bins = low.d_shades = nullptr;
  void* p = nullptr;
  VkResult r = device_alloc((size_t)rec_cap * sizeof(KzTriRecord), &p);
  if (r != VK_SUCCESS) return r;
  low.d_records = static_cast<char*>(p);
  r = device_alloc((size_t)pair_cap * 4, &p);
  if (r != VK_SUCCESS) return r;
  low.d_bins = static_cast<char*>(p);
  /* ordered segments keep each unclipped record's shading setup beside it: 1/w of the three vertices
   * (16 bytes) then three vertices' varyings */
  bool ordered = false;
  for (const KzSegment& s : low.segments) ordered |= s.mode == KZ_MODE_ORDERED && (s.num_chunks > 0 || s.indirect);
  if (ordered) {
    uint32_t nv = 0;
    for (const KzPipe& kp : low.pipes) nv = std::max(nv, kp.num_varyings);
    low.shade_stride = (uint32_t)align_up(16 + 12 * (size_t)nv, 16);
    r = device_alloc((size_t)rec_cap * low.shade_stride, &p);
    if (r != VK_SUCCESS) return r;
    low.d_shades = static_cast<char*>(p);
  }
  low.rec_cap = rec_cap;
  low.pair_cap = pair_cap;
  for (KzSegment& s : low.segments) {
    s.records = (uint64_t)(uintptr_t)low.d_records;
    s.bins = (uint64_t)(uintptr_t)low.d_bins;
    s.shades = (uint64_t)(uintptr_t)low.d_shades;
    s.shade_stride = low.shade_stride;
    s.rec_cap = rec_cap;
    s.pair_cap = pair_cap;
  }
  return VK_SUCCESS;
}

/* cuTensorMapEncodeTiled, reached through the runtime (the library links no libcuda) */
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

/* The tensor map of a tile's block of a 4-byte-per-texel attachment: 32-bit texels, width x height, rows
 * `pitch` bytes apart, box tile x tile.  Needs a 16-byte aligned base and pitch (the tensor copies' rule);
 * false (plain loads and stores) otherwise. */
static bool encode_tile_map(CUtensorMap* m, uint64_t base, uint32_t width, uint32_t height, uint32_t pitch,
                            uint32_t tile) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || !base || (base & 15u) || (pitch & 15u) || tile > 16 || width == 0 || height == 0) return false;
  cuuint64_t dims[2] = {width, height};
  cuuint64_t strides[1] = {pitch};
  cuuint32_t box[2] = {tile, tile};
  cuuint32_t elem[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, reinterpret_cast<void*>(base), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static void upload_tables(Lowered& low) {
  size_t o_draws = 0;
  size_t o_pipes = align_up(o_draws + low.draws.size() * sizeof(KzDraw), 256);
  size_t o_chunks = align_up(o_pipes + low.pipes.size() * sizeof(KzPipe), 256);
  size_t o_segs = align_up(o_chunks + low.chunks.size() * sizeof(KzChunk), 256);
  size_t o_push = align_up(o_segs + low.segments.size() * sizeof(KzSegment), 256);
  size_t o_lut = align_up(o_push + low.push.size(), 256);
  std::vector<char> host(low.tables_bytes, 0);
  if (!low.draw_lut.empty())
    std::memcpy(host.data() + o_lut, low.draw_lut.data(), low.draw_lut.size() * sizeof(uint32_t));
  if (!low.draws.empty()) std::memcpy(host.data() + o_draws, low.draws.data(), low.draws.size() * sizeof(KzDraw));
  if (!low.pipes.empty()) std::memcpy(host.data() + o_pipes, low.pipes.data(), low.pipes.size() * sizeof(KzPipe));
  if (!low.chunks.empty()) std::memcpy(host.data() + o_chunks, low.chunks.data(), low.chunks.size() * sizeof(KzChunk));
  if (!low.segments.empty())
    std::memcpy(host.data() + o_segs, low.segments.data(), low.segments.size() * sizeof(KzSegment));
  if (!low.push.empty()) std::memcpy(host.data() + o_push, low.push.data(), low.push.size());
  cudaMemcpy(low.d_tables, host.data(), o_lut + low.draw_lut.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (!low.tmaps.empty()) cudaMemcpy(low.d_tables + low.o_tmaps, low.tmaps.data(), low.tmaps.size(), cudaMemcpyHostToDevice);
}

static uint32_t grid_cap(Device* dev) { return (uint32_t)std::max(1, dev->pd->sm_count) * 8u; }

static cudaEvent_t timing_event(Device* dev) {
  if (!dev->timing_pool.empty()) {
    cudaEvent_t e = dev->timing_pool.back();
    dev->timing_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

/* one kernel launch; with `timing` set, bracketed by a pair of timing events on the same stream */
/* `chain`: the previous operation on the stream was one of the pipeline kernels.  Such a kernel is then
 * launched with programmatic stream serialization, so its launch overlaps the previous kernel's
 * completion; each kernel waits at entry (griddepcontrol.wait) until its predecessor has completed.
 * Timed launches (an event between the kernels) and cooperative launches are not chained. */
static void launch(Device* dev, std::vector<TimedLaunch>* timing, int kind, const cudaLaunchConfig_t& cfg,
                   cudaKernel_t fn, void** args, bool& chain) {
  TimedLaunch t;
  if (timing) {
    t.kind = kind;
    t.before = timing_event(dev);
    t.after = timing_event(dev);
    cudaEventRecord(t.before, cfg.stream);
  }
  cudaLaunchAttribute at[1];
  cudaLaunchConfig_t c = cfg;
  if (chain && !timing && options().pdl && cfg.numAttrs == 0) {
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = 1;
  }
  cudaLaunchKernelExC(&c, (const void*)fn, args);
  if (timing) {
    cudaEventRecord(t.after, cfg.stream);
    timing->push_back(t);
  }
  chain = true;
}

/* an ordered segment that kz_k_raster_direct serves: one sample per pixel, D32 depth, tiles of at most
 * 16x16, and no draw whose fragment shader is a function call (only none, or the colour pass-through) */
static bool raster_direct(const Lowered& low, const KzSegment& seg) {
  if (seg.samples > 1 || seg.depth_format != KZ_DF_D32 || seg.tile > 16) return false;
  for (uint32_t i = seg.first_draw; i < seg.first_draw + seg.num_draws; i++) {
    const KzPipe& p = low.pipes[low.draws[i].pipe];
    if (p.has_fs && !p.fs_passthrough) return false;
  }
  return true;
}

/* enqueue the lowered command buffer from segment `start` on */
static uint32_t launch_ops(CommandBuffer* cb, cudaStream_t st, uint32_t start, bool capture,
                           std::vector<TimedLaunch>* timing = nullptr) {
  Lowered& low = *cb->low;
  Device* dev = cb->dev;
  uint32_t launches = 0;
  uint32_t nseg = (uint32_t)low.segments.size();
  cudaMemsetAsync(low.d_status, 0, sizeof(KzStatus), st);
  if (nseg > start) cudaMemsetAsync(low.d_counters + start, 0, (nseg - start) * sizeof(KzSegCounters), st);
  if (low.max_tiles) cudaMemsetAsync(low.d_tiles, 0, (size_t)low.max_tiles * 4, st);
  if (capture) cudaEventRecordWithFlags(low.ev_begin, st, cudaEventRecordExternal);
  else cudaEventRecord(low.ev_begin, st);
  KernelSet* ks = low.ks;
  bool chain = false;
  for (const Lowered::LOp& lop : low.ops) {
    if (lop.kind == OpKind::Pass) {
      if (lop.seg_end <= start) continue;
      uint32_t s0 = std::max(lop.seg_begin, start);
      /* indirect segments first read their commands: nothing inside a render pass writes the buffers */
      for (uint32_t s = s0; s < lop.seg_end; s++) {
        if (!low.segments[s].indirect) continue;
        KzFrame f = low.frame;
        void* args[] = {&f, &s};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(1);
        cfg.blockDim = dim3(1024);
        cfg.stream = st;
        launch(dev, timing, KK_INDIRECT, cfg, ks->indirect, args, chain);
        const KzSegment& sg = low.segments[s];
        cfg.gridDim = dim3(std::min(grid_cap(dev), std::max(1u, (std::max(sg.chunk_cap, sg.lut_cap) + 255) / 256)));
        cfg.blockDim = dim3(256);
        launch(dev, timing, KK_INDIRECT_TABLES, cfg, ks->indirect_tables, args, chain);
        launches += 2;
      }
      if (low.mode == 0) {
        KzFrame f = low.frame;
        f.first_segment = s0;
        f.num_segments = lop.seg_end;
        void* args[] = {&f};
        /* passes whose segments are all opaque run the kernel with only the visibility phases */
        bool all_vis = true;
        for (uint32_t s = s0; s < lop.seg_end; s++) all_vis &= low.segments[s].mode == KZ_MODE_VISIBILITY;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(all_vis ? ks->persistent_vis_blocks : ks->persistent_blocks));
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = all_vis ? 0 : KZ_DYN_SMEM;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (all_vis) launch(dev, timing, KK_PERSISTENT_VIS, cfg, ks->persistent_vis, args, chain);
        else launch(dev, timing, KK_PERSISTENT, cfg, ks->persistent, args, chain);
        launches++;
      } else {
        for (uint32_t s = s0; s < lop.seg_end; s++) {
          const KzSegment& seg = low.segments[s];
          KzFrame f = low.frame;
          void* args[] = {&f, &s};
          cudaLaunchConfig_t cfg = {};
          cfg.blockDim = dim3(256);
          cfg.stream = st;
          /* the per-draw launch form: each direct draw's geometry is a launch of its own (with, for opaque
           * segments, the large-triangle jobs it made); the pass-wide phases run once per segment */
          const bool per_draw = low.mode == 2 && !seg.indirect;
          uint32_t gb = (uint32_t)std::max(1, ks->geometry_blocks);
          if (low.geo_blocks) gb = std::min(gb, low.geo_blocks * (uint32_t)dev->pd->sm_count);
          if (seg.mode == KZ_MODE_VISIBILITY) {
            cfg.gridDim = dim3(std::min(grid_cap(dev), std::max(1u, (seg.width * seg.height + 255) / 256)));
            launch(dev, timing, KK_VIS_INIT, cfg, ks->vis_init, args, chain);
            if (per_draw) {
              for (uint32_t di = seg.first_draw; di < seg.first_draw + seg.num_draws; di++) {
                const std::pair<uint32_t, uint32_t> dc = low.draw_chunks[di];
                if (dc.first == dc.second) continue;
                KzFrame fd = f;
                fd.chunk_begin = dc.first;
                fd.chunk_end = dc.second;
                fd.jobs_incremental = 1;
                void* dargs[] = {&fd, &s};
                cfg.gridDim = dim3(std::min<uint32_t>(dc.second - dc.first, gb));
                launch(dev, timing, KK_VIS_GEOMETRY, cfg, ks->vis_geometry, dargs, chain);
                cfg.gridDim = dim3(grid_cap(dev));
                launch(dev, timing, KK_VIS_LARGE, cfg, ks->vis_large, dargs, chain);
                launches += 2;
              }
            } else if (seg.num_chunks || seg.indirect) {
              cfg.gridDim = dim3(seg.indirect ? gb : std::min<uint32_t>(seg.num_chunks, gb));
              launch(dev, timing, KK_VIS_GEOMETRY, cfg, ks->vis_geometry, args, chain);
              cfg.gridDim = dim3(grid_cap(dev));
              launch(dev, timing, KK_VIS_LARGE, cfg, ks->vis_large, args, chain);
              launches += 2;
            }
            cfg.gridDim = dim3(grid_cap(dev));
            launch(dev, timing, KK_VIS_RESOLVE, cfg, ks->vis_resolve, args, chain);
            launches += 2;
            continue;
          }
          if (per_draw) {
            for (uint32_t di = seg.first_draw; di < seg.first_draw + seg.num_draws; di++) {
              const std::pair<uint32_t, uint32_t> dc = low.draw_chunks[di];
              if (dc.first == dc.second) continue;
              KzFrame fd = f;
              fd.chunk_begin = dc.first;
              fd.chunk_end = dc.second;
              void* dargs[] = {&fd, &s};
              cfg.gridDim = dim3(dc.second - dc.first);
              launch(dev, timing, KK_GEOMETRY, cfg, ks->geometry, dargs, chain);
              launches++;
            }
          } else if (seg.num_chunks || seg.indirect) {
            cfg.gridDim = dim3(seg.indirect ? grid_cap(dev) : seg.num_chunks);
            launch(dev, timing, KK_GEOMETRY, cfg, ks->geometry, args, chain);
            launches++;
          }
          cfg.gridDim = dim3(1);
          launch(dev, timing, KK_SCAN, cfg, ks->scan, args, chain);
          cfg.gridDim = dim3(std::min(grid_cap(dev), std::max(1u, (seg.rec_cap + 255) / 256)));
          launch(dev, timing, KK_BIN, cfg, ks->bin, args, chain);
          cfg.gridDim = dim3(std::min(grid_cap(dev), std::max(1u, seg.tiles_x * seg.tiles_y)));
          cfg.dynamicSmemBytes = KZ_DYN_SMEM;
          if (raster_direct(low, seg)) launch(dev, timing, KK_RASTER_DIRECT, cfg, ks->raster_direct, args, chain);
          else if (seg.samples > 1) launch(dev, timing, KK_RASTER_MS, cfg, ks->raster_ms, args, chain);
          else if (seg.depth_format != KZ_DF_D32 && seg.tile <= 16)
            launch(dev, timing, KK_RASTER_DS, cfg, ks->raster_ds, args, chain);
          else launch(dev, timing, KK_RASTER, cfg, ks->raster, args, chain);
          launches += 3;
        }
      }
    } else {
      if (lop.seg_begin < start) continue;
      const RecOp& op = lop.op;
      if (op.kind == OpKind::Clear || op.kind == OpKind::Fill) {
        uint64_t base = (uint64_t)(uintptr_t)op.base;
        uint32_t pitch = op.pitch;
        int32_t x0 = op.rect[0], y0 = op.rect[1], x1 = op.rect[2], y1 = op.rect[3];
        uint32_t value = op.value;
        void* args[] = {&base, &pitch, &x0, &y0, &x1, &y1, &value};
        cudaLaunchConfig_t cfg = {};
        cfg.blockDim = dim3(256);
        long long work = (long long)(x1 - x0) * (y1 - y0) / 4 + 1;
        cfg.gridDim = dim3((unsigned)std::min<long long>(grid_cap(dev), (work + 255) / 256));
        cfg.stream = st;
        launch(dev, timing, KK_CLEAR, cfg, ks->clear, args, chain);
        launches++;
      } else if (op.kind == OpKind::Copy) {
        cudaMemcpyAsync(op.dst, op.src, op.bytes, cudaMemcpyDeviceToDevice, st);
        chain = false;
      } else if (op.kind == OpKind::Copy2D) {
        cudaMemcpy2DAsync(op.dst, op.dpitch, op.src, op.spitch, op.width_bytes, op.rows, cudaMemcpyDeviceToDevice, st);
        chain = false;
      } else if (op.kind == OpKind::Resolve) {
        uint64_t src = (uint64_t)(uintptr_t)op.src, dst = (uint64_t)(uintptr_t)op.dst;
        uint32_t spitch = (uint32_t)op.spitch, dpitch = (uint32_t)op.dpitch;
        int32_t sx = op.rect[0], sy = op.rect[1], w = op.rect[2], h = op.rect[3], dx = op.dst_x, dy = op.dst_y;
        void* args[] = {&src, &spitch, &sx, &sy, &dst, &dpitch, &dx, &dy, &w, &h};
        cudaLaunchConfig_t cfg = {};
        cfg.blockDim = dim3(256);
        cfg.gridDim = dim3((unsigned)std::min<long long>(grid_cap(dev), ((long long)w * h + 255) / 256));
        cfg.stream = st;
        launch(dev, timing, KK_RESOLVE, cfg, ks->resolve, args, chain);
        launches++;
      }
    }
  }
  if (capture) cudaEventRecordWithFlags(low.ev_end, st, cudaEventRecordExternal);
  else cudaEventRecord(low.ev_end, st);
  cudaMemcpyAsync(low.h_status, low.d_status, sizeof(KzStatus), cudaMemcpyDeviceToHost, st);
  if (start == 0) low.launches = launches;
  return launches;
}

VkResult lower_command_buffer(CommandBuffer* cb) {
  Device* dev = cb->dev;
  std::lock_guard<std::recursive_mutex> lock(dev->mu);
  cudaSetDevice(dev->pd->cuda_device);
  cb->low.reset(new Lowered());
  Lowered& low = *cb->low;
  low.mode = options().mode;
  low.tile = options().tile;
  low.timed = options().kernel_timing != 0;
  low.geo_blocks = options().geo_blocks;
  /* one pipeline entry per pipeline and vertex-buffer alignment class: draws whose bound vertex buffers all
   * start 16-byte aligned use an entry whose vertex fetch uses vector loads */
  std::map<std::pair<Pipeline*, uint32_t>, uint32_t> pipe_index;
  auto pipe_of = [&](Pipeline* p, const KzDraw& d) -> uint32_t {
    uint32_t align = options().vector_fetch && fetch_vectorizable(p->pipe) && bases_aligned16(d, p->pipe) ? 16u : 4u;
    auto key = std::make_pair(p, align);
    auto it = pipe_index.find(key);
    if (it != pipe_index.end()) return it->second;
    KzPipe kp = p->pipe;
    uint32_t idx = (uint32_t)low.pipes.size();
    low.pipes.push_back(kp);
    low.pipe_objs.push_back(p);
    low.pipe_align.push_back(align);
    pipe_index[key] = idx;
    return idx;
  };
  /* vkCmdUpdateBuffer data: one device block, uploaded now, that the copies read at execution */
  size_t inline_bytes = 0, inline_off = 0;
  for (const RecOp& op : cb->ops) inline_bytes += align_up(op.data.size(), 16);
  if (inline_bytes) {
    void* ip = nullptr;
    VkResult ir = device_alloc(inline_bytes, &ip);
    if (ir != VK_SUCCESS) return ir;
    low.d_inline = static_cast<char*>(ip);
    std::vector<uint8_t> staged(inline_bytes, 0);
    size_t o = 0;
    for (const RecOp& op : cb->ops) {
      if (op.data.empty()) continue;
      std::memcpy(staged.data() + o, op.data.data(), op.data.size());
      o += align_up(op.data.size(), 16);
    }
    cudaMemcpy(low.d_inline, staged.data(), inline_bytes, cudaMemcpyHostToDevice);
  }
  for (const RecOp& op : cb->ops) {
    Lowered::LOp lop;
    lop.kind = op.kind;
    lop.op = op;
    if (!op.data.empty()) {
      lop.op.src = low.d_inline + inline_off;
      lop.op.data.clear();
      inline_off += align_up(op.data.size(), 16);
    }
    lop.seg_begin = (uint32_t)low.segments.size();
    if (op.kind != OpKind::Pass) {
      add_unique(low.writes, op.wmem);
      add_unique(low.reads, op.rmem);
      lop.seg_end = lop.seg_begin;
      low.ops.push_back(lop);
      continue;
    }
    const PassRec& pr = cb->passes[op.pass];
    bool vis_ok = true;
    if (pr.rp->depth_att >= 0 && (size_t)pr.rp->depth_att < pr.fb->views.size()) {
      const Image* di = pr.fb->views[(size_t)pr.rp->depth_att]->image;
      vis_ok = di->format == VK_FORMAT_D32_SFLOAT && di->samples == 1;
    }
    if (pr.rp->color_att >= 0 && (size_t)pr.rp->color_att < pr.fb->views.size() &&
        pr.fb->views[(size_t)pr.rp->color_att]->image->samples > 1)
      vis_ok = false;
    /* split the pass into segments */
    std::vector<std::pair<size_t, size_t>> runs; /* [begin, end) draw indices */
    {
      size_t b = 0;
      for (size_t i = 1; i <= pr.draws.size(); i++)
        if (i == pr.draws.size() || raster_class(pr.draws[i], vis_ok) != raster_class(pr.draws[b], vis_ok)) {
          runs.push_back({b, i});
          b = i;
        }
    }
    bool needs_clear = false; /* a continuation after vkCmdClearAttachments loads its attachments */
    if (pr.rp->color_att >= 0 && pr.rp->atts[(size_t)pr.rp->color_att].loadOp == VK_ATTACHMENT_LOAD_OP_CLEAR)
      needs_clear = true;
    if (pr.rp->depth_att >= 0 && pr.rp->atts[(size_t)pr.rp->depth_att].loadOp == VK_ATTACHMENT_LOAD_OP_CLEAR)
      needs_clear = true;
    if (pr.cont) needs_clear = false;
    if (runs.empty() && needs_clear) runs.push_back({0, 0});
    for (size_t r = 0; r < runs.size(); r++) {
      KzSegment s;
      std::memset(&s, 0, sizeof s);
      segment_target(pr, s, low.tile, r == 0 && !pr.cont, low);
      s.segment_index = (uint32_t)low.segments.size();
      s.first_draw = (uint32_t)low.draws.size();
      s.first_chunk = (uint32_t)low.chunks.size();
      s.mode = KZ_MODE_ORDERED;
      s.vis_key = 0;
      uint64_t prims = 0, guess = 0;
      for (size_t i = runs[r].first; i < runs[r].second; i++) {
        const DrawRec& dr = pr.draws[i];
        if (dr.indirect) {
          /* sizing guess: the draws together cover their bound buffers about once; an overflow grows the
           * scratch and replays */
          s.indirect = 1;
          guess = std::max<uint64_t>(guess, dr.d.elem_limit / 3);
        }
        if (i == runs[r].first && vis_ok && dr.pipe->vis_key >= 0) {
          s.mode = KZ_MODE_VISIBILITY;
          s.vis_key = (uint32_t)dr.pipe->vis_key;
        }
        KzDraw d = dr.d;
        d.samples = s.samples;
        d.rect[2] = std::min(d.rect[2], (int32_t)s.width);
        d.rect[3] = std::min(d.rect[3], (int32_t)s.height);
        d.pipe = pipe_of(dr.pipe, d);
        d.prim_base = (uint32_t)prims;
        /* the draw's snapshot: push constants, then its descriptors, padded to whole KZ_PUSH_BYTES units */
        d.push_index = (uint32_t)(low.push.size() / KZ_PUSH_BYTES);
        low.push.insert(low.push.end(), dr.push, dr.push + KZ_PUSH_BYTES);
        if (!dr.desc.empty()) {
          const uint8_t* db = reinterpret_cast<const uint8_t*>(dr.desc.data());
          low.push.insert(low.push.end(), db, db + dr.desc.size() * sizeof(KzDescriptor));
          low.push.resize(align_up(low.push.size(), KZ_PUSH_BYTES), 0);
        }
        for (DeviceMemory* m : dr.desc_reads) add_unique(low.reads, m);
        uint32_t di = (uint32_t)low.draws.size();
        const uint32_t chunk0 = (uint32_t)(low.chunks.size() - s.first_chunk);
        for (uint64_t c = 0; !dr.indirect && c < dr.triangles; c += KZ_CHUNK) {
          KzChunk ch;
          ch.draw = di;
          ch.first = (uint32_t)c;
          ch.count = (uint32_t)std::min<uint64_t>(KZ_CHUNK, dr.triangles - c);
          ch.pad = 0;
          low.chunks.push_back(ch);
        }
        low.draws.push_back(d);
        low.draw_chunks.push_back({chunk0, (uint32_t)(low.chunks.size() - s.first_chunk)});
        for (DeviceMemory* m : dr.reads) add_unique(low.reads, m);
        prims += dr.triangles;
      }
      if (prims >= 0xFFFFFFF0ull) {
        log_error("a render pass of %llu triangles exceeds the 2^32 primitive limit", (unsigned long long)prims);
        return VK_ERROR_OUT_OF_DEVICE_MEMORY;
      }
      s.num_draws = (uint32_t)(low.draws.size() - s.first_draw);
      s.num_chunks = (uint32_t)(low.chunks.size() - s.first_chunk);
      s.num_prims = (uint32_t)prims;
      low.triangles += prims;
      low.max_tiles = std::max(low.max_tiles, s.tiles_x * s.tiles_y);
      low.segments.push_back(s);
      /* scratch records for at most 4M guessed triangles (an overflow grows them); the chunk table and draw
       * lookup, 4 bytes per 256 triangles, take the whole guess */
      low.prims_guess.push_back(s.indirect ? std::min<uint64_t>(guess, 1u << 22) : prims);
      low.table_guess.push_back(s.indirect ? guess : 0);
    }
    lop.seg_end = (uint32_t)low.segments.size();
    low.ops.push_back(lop);
  }
  /* scratch sizing: records for every triangle plus clipping headroom; bins for a few tiles per record */
  uint64_t max_prims = 0, max_tiles = 0;
  for (size_t i = 0; i < low.segments.size(); i++) {
    const KzSegment& s = low.segments[i];
    max_prims = std::max<uint64_t>(max_prims, low.prims_guess[i]);
    max_tiles = std::max<uint64_t>(max_tiles, (uint64_t)s.tiles_x * s.tiles_y);
  }
  uint64_t rec_cap = (uint64_t)((double)max_prims * options().rec_slack) + 4096;
  uint64_t pair_cap = rec_cap * 4 + max_tiles * 16 + (1u << 18);
  rec_cap = std::min<uint64_t>(rec_cap, 0xFFFFFFF0ull);
  pair_cap = std::min<uint64_t>(pair_cap, 0xFFFFFFF0ull);
  /* per segment, the draw holding every 256th primitive (shading finds a primitive's draw from it) */
  low.draw_lut.clear();
  low.draw_lut_offset.assign(low.segments.size(), 0);
  for (size_t i = 0; i < low.segments.size(); i++) {
    const KzSegment& sg = low.segments[i];
    low.draw_lut_offset[i] = low.draw_lut.size();
    uint32_t d = sg.first_draw;
    for (uint64_t g = 0; g < sg.num_prims; g += 256) {
      while (d + 1 < sg.first_draw + sg.num_draws && low.draws[d + 1].prim_base <= g) d++;
      low.draw_lut.push_back(d);
    }
  }
  /* indirect segments: room for the chunk table and the draw lookup that kz_k_indirect_tables fills, sized
   * from the guess (a segment that outgrows them searches the draws instead) */
  std::vector<size_t> ind_off(low.segments.size(), 0);
  size_t ind_words = 0;
  for (size_t i = 0; i < low.segments.size(); i++) {
    KzSegment& sg = low.segments[i];
    if (!sg.indirect) continue;
    uint64_t g = low.table_guess[i] / KZ_CHUNK;
    sg.chunk_cap = (uint32_t)std::min<uint64_t>(g + sg.num_draws + 1024, 1u << 24);
    sg.lut_cap = (uint32_t)std::min<uint64_t>(g + 1024, 1u << 24);
    ind_off[i] = ind_words;
    ind_words += (size_t)sg.chunk_cap * (sizeof(KzChunk) / 4) + sg.lut_cap;
  }
  /* device tables: draws | pipes | chunks | segments | push | draw lookup | indirect tables, then counters
   * and status */
  size_t o_pipes = align_up(low.draws.size() * sizeof(KzDraw), 256);
  size_t o_chunks = align_up(o_pipes + low.pipes.size() * sizeof(KzPipe), 256);
  size_t o_segs = align_up(o_chunks + low.chunks.size() * sizeof(KzChunk), 256);
  size_t o_push = align_up(o_segs + low.segments.size() * sizeof(KzSegment), 256);
  size_t o_lut = align_up(o_push + low.push.size(), 256);
  size_t o_ind = align_up(o_lut + low.draw_lut.size() * sizeof(uint32_t), 256);
  size_t o_tmaps = align_up(o_ind + ind_words * sizeof(uint32_t), 256);
  size_t o_counters = align_up(o_tmaps + low.segments.size() * 2 * sizeof(CUtensorMap), 256);
  size_t o_status = align_up(o_counters + low.segments.size() * sizeof(KzSegCounters), 256);
  low.tables_bytes = o_status + sizeof(KzStatus);
  void* p = nullptr;
  VkResult r = device_alloc(low.tables_bytes, &p);
  if (r != VK_SUCCESS) return r;
  low.d_tables = static_cast<char*>(p);
  low.d_counters = reinterpret_cast<KzSegCounters*>(low.d_tables + o_counters);
  low.d_status = reinterpret_cast<KzStatus*>(low.d_tables + o_status);
  r = device_alloc(std::max<size_t>(4, (size_t)(low.max_tiles + 1) * 4 * 4), &p);
  if (r != VK_SUCCESS) return r;
  low.d_tiles = static_cast<uint32_t*>(p);
  size_t vis_px = 0;
  for (const KzSegment& sg : low.segments)
    if (sg.mode == KZ_MODE_VISIBILITY) vis_px = std::max(vis_px, (size_t)sg.width * sg.height);
  if (vis_px) {
    r = device_alloc(vis_px * 8, &p);
    if (r != VK_SUCCESS) return r;
    low.d_vis = static_cast<char*>(p);
  }
  for (size_t i = 0; i < low.segments.size(); i++) {
    KzSegment& s = low.segments[i];
    s.tile_count = (uint64_t)(uintptr_t)low.d_tiles;
    s.tile_offset = (uint64_t)(uintptr_t)(low.d_tiles + low.max_tiles);
    s.tile_cursor = (uint64_t)(uintptr_t)(low.d_tiles + 2 * (size_t)low.max_tiles + 1);
    s.tile_order = (uint64_t)(uintptr_t)(low.d_tiles + 3 * (size_t)low.max_tiles + 1);
    s.counters = (uint64_t)(uintptr_t)(low.d_counters + i);
    s.draw_lut = s.num_prims ? (uint64_t)(uintptr_t)(low.d_tables + o_lut + low.draw_lut_offset[i] * sizeof(uint32_t))
                             : 0;
    s.vis = s.mode == KZ_MODE_VISIBILITY ? (uint64_t)(uintptr_t)low.d_vis : 0;
    if (s.indirect) {
      s.chunk_table = (uint64_t)(uintptr_t)(low.d_tables + o_ind + ind_off[i] * sizeof(uint32_t));
      s.lut_table = s.chunk_table + (uint64_t)s.chunk_cap * sizeof(KzChunk);
    }
  }
  /* ordered segments that kz_k_raster_direct serves stage each tile's colour and depth through tensor copies */
  static_assert(sizeof(CUtensorMap) == 128, "tensor map size");
  low.o_tmaps = o_tmaps;
  low.tmaps.assign(low.segments.size() * 2 * sizeof(CUtensorMap), 0);
  for (size_t i = 0; i < low.segments.size() && options().tma; i++) {
    KzSegment& s = low.segments[i];
    if (s.mode != KZ_MODE_ORDERED || !raster_direct(low, s)) continue;
    CUtensorMap* m = reinterpret_cast<CUtensorMap*>(low.tmaps.data()) + 2 * i;
    const uint64_t at = (uint64_t)(uintptr_t)(low.d_tables + o_tmaps + 2 * i * sizeof(CUtensorMap));
    if (encode_tile_map(m, s.color, s.width, s.height, s.color_pitch, s.tile)) s.tmap_color = at;
    if (encode_tile_map(m + 1, s.depth, s.width, s.height, s.depth_pitch, s.tile)) s.tmap_depth = at + sizeof(CUtensorMap);
  }
  r = size_scratch(dev, low, (uint32_t)rec_cap, (uint32_t)pair_cap);
  if (r != VK_SUCCESS) return r;
  low.frame.draws = (uint64_t)(uintptr_t)low.d_tables;
  low.frame.pipes = (uint64_t)(uintptr_t)(low.d_tables + o_pipes);
  low.frame.chunks = (uint64_t)(uintptr_t)(low.d_tables + o_chunks);
  low.frame.segments = (uint64_t)(uintptr_t)(low.d_tables + o_segs);
  low.frame.push = (uint64_t)(uintptr_t)(low.d_tables + o_push);
  low.frame.status = (uint64_t)(uintptr_t)low.d_status;
  low.frame.num_segments = (uint32_t)low.segments.size();
  low.frame.first_segment = 0;
  low.frame.chunk_begin = 0;
  low.frame.chunk_end = 0xFFFFFFFFu;
  low.frame.jobs_incremental = 0;
  low.frame.barrier_ns = options().barrier_ns;
  low.frame.warp_px = options().warp_px;
  low.frame.job_blocks = options().job_blocks;
  upload_tables(low);
  if (cudaMallocHost((void**)&low.h_status, sizeof(KzStatus)) != cudaSuccess) return VK_ERROR_OUT_OF_HOST_MEMORY;
  std::memset(low.h_status, 0, sizeof(KzStatus));
  cudaEventCreate(&low.ev_begin);
  cudaEventCreate(&low.ev_end);
  std::string err;
  low.ks = kernel_set_for(dev, low.pipe_objs, low.pipe_align, err);
  if (!low.ks) {
    log_error("pipeline link failed: %s", err.c_str());
    return VK_ERROR_INITIALIZATION_FAILED;
  }
  if (low.mode != 2 && !low.timed) {
    cudaStream_t cs = dev->capture_stream;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      log_error("stream capture failed to start: %s", cudaGetErrorString(cudaGetLastError()));
      return VK_ERROR_INITIALIZATION_FAILED;
    }
    launch_ops(cb, cs, 0, true);
    cudaError_t e = cudaStreamEndCapture(cs, &low.graph);
    if (e != cudaSuccess || cudaGraphInstantiate(&low.exec, low.graph, 0) != cudaSuccess) {
      log_error("graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : cudaGetLastError()));
      return VK_ERROR_INITIALIZATION_FAILED;
    }
  }
  if (options().trace)
    log_error("lowered: %zu draws, %zu segments, %llu triangles, mode %d, tile %u, records %u, pairs %u",
              low.draws.size(), low.segments.size(), (unsigned long long)low.triangles, low.mode, low.tile,
              low.rec_cap, low.pair_cap);
  return VK_SUCCESS;
}

/* ------------------------------------------------------------------------------------------------ */
/* submission and completion                                                                        */

static cudaEvent_t pool_event(Device* dev) {
  if (!dev->event_pool.empty()) {
    cudaEvent_t e = dev->event_pool.back();
    dev->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  return e;
}

/* Host-visible memory the command buffer reads is uploaded from its pinned shadow on the device's copy
 * stream, after the queue's last use of that memory; the queue waits for the uploads before it launches.
 * So the upload of one submission overlaps the kernels of the submissions before it whenever they use
 * other memory (double-buffered inputs), and never overwrites memory they still read or write. */
static void enqueue(CommandBuffer* cb, cudaStream_t st) {
  Lowered& low = *cb->low;
  Device* dev = cb->dev;
  bool uploaded = false;
  for (DeviceMemory* m : low.reads) {
    if (!(m->host && m->mapped)) continue;
    if (m->last_use) cudaStreamWaitEvent(dev->copy_stream, m->last_use, 0);
    cudaMemcpyAsync(m->dptr, m->host, (size_t)m->size, cudaMemcpyHostToDevice, dev->copy_stream);
    uploaded = true;
  }
  if (uploaded) {
    cudaEvent_t ev = pool_event(dev);
    cudaEventRecord(ev, dev->copy_stream);
    cudaStreamWaitEvent(st, ev, 0);
    dev->event_pool.push_back(ev); /* a recorded event can be re-recorded once the wait is enqueued */
  }
  if (low.exec) cudaGraphLaunch(low.exec, st);
  else launch_ops(cb, st, 0, false, low.timed ? &cb->timing : nullptr);
  for (DeviceMemory* m : low.writes) {
    if (m->host && m->mapped) cudaMemcpyAsync(m->host, m->dptr, (size_t)m->size, cudaMemcpyDeviceToHost, st);
    else m->device_newer = true;
  }
  auto mark = [&](DeviceMemory* m) {
    if (!m) return;
    if (!m->last_use) cudaEventCreateWithFlags(&m->last_use, cudaEventDisableTiming);
    cudaEventRecord(m->last_use, st);
  };
  for (DeviceMemory* m : low.reads) mark(m);
  for (DeviceMemory* m : low.writes) mark(m);
}

/* grow the scratch after an overflow and run the command buffer again from the failing segment;
 * called only when nothing was enqueued after it */
static bool replay(CommandBuffer* cb, Queue* q) {
  Lowered& low = *cb->low;
  for (int attempt = 0; attempt < 4; attempt++) {
    KzStatus st = *low.h_status;
    if (!(st.flags & (KZ_STATUS_RECORD_OVERFLOW | KZ_STATUS_PAIR_OVERFLOW))) return true; /* others: complete() */
    uint64_t rec = std::max<uint64_t>(low.rec_cap, (uint64_t)((double)st.need_records * 1.25) + 4096);
    uint64_t pair = std::max<uint64_t>(low.pair_cap, (uint64_t)((double)st.need_pairs * 1.25) + 65536);
    if (options().trace) log_error("scratch overflow in segment %u: growing to %llu records, %llu pairs",
                                   st.failed_segment, (unsigned long long)rec, (unsigned long long)pair);
    if (rec > 0xFFFFFFF0ull || pair > 0xFFFFFFF0ull) return false;
    if (size_scratch(cb->dev, low, (uint32_t)rec, (uint32_t)pair) != VK_SUCCESS) return false;
    upload_tables(low);
    launch_ops(cb, q->stream, st.failed_segment, false);
    for (DeviceMemory* m : low.writes)
      if (m->host && m->mapped) cudaMemcpyAsync(m->host, m->dptr, (size_t)m->size, cudaMemcpyDeviceToHost, q->stream);
    cudaStreamSynchronize(q->stream);
  }
  return false;
}

static void complete(Queue* q, Submission& s) {
  Device* dev = q->dev;
  VkResult err = VK_SUCCESS;
  if (s.cb && s.cb->low) {
    CommandBuffer* cb = s.cb;
    Lowered& low = *cb->low;
    KzStatus st = *low.h_status;
    if (st.flags & (KZ_STATUS_RECORD_OVERFLOW | KZ_STATUS_PAIR_OVERFLOW)) {
      bool last = &s == &q->inflight.back();
      if (!last || !replay(cb, q)) {
        log_error("triangle-record or tile-bin capacity exceeded and the submission could not be replayed");
        err = VK_ERROR_DEVICE_LOST;
      }
      st = *low.h_status;
    }
    if (st.flags & KZ_STATUS_BARRIER_TIMEOUT) {
      log_error("persistent kernel barrier timed out");
      err = VK_ERROR_DEVICE_LOST;
    }
    if (st.flags & KZ_STATUS_BIN_TOO_LARGE) {
      log_error("a tile's bin exceeds the ordered-mode sort capacity; use a smaller tile");
      err = VK_ERROR_DEVICE_LOST;
    }
    /* out-of-range indirect commands are skipped, as robust buffer access would leave them without
     * effect; the status word keeps the bit for the application */
    if (st.flags & KZ_STATUS_INDIRECT_RANGE) log_error("an indirect command reads past its bound buffers: skipped");
    if (st.flags & KZ_STATUS_INDIRECT_LIMIT) {
      log_error("an indirect segment reaches 2^32 triangles: skipped");
      err = VK_ERROR_DEVICE_LOST;
    }
    cb->last_status = st;
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, low.ev_begin, low.ev_end) == cudaSuccess) cb->last_ms = ms;
    else cudaGetLastError();
    for (const TimedLaunch& t : s.timing) {
      float kms = 0.0f;
      if (cudaEventElapsedTime(&kms, t.before, t.after) == cudaSuccess) {
        cb->kernel_ms[t.kind] += kms;
        cb->kernel_launches[t.kind]++;
      } else {
        cudaGetLastError();
      }
    }
  }
  for (const TimedLaunch& t : s.timing) {
    dev->timing_pool.push_back(t.before);
    dev->timing_pool.push_back(t.after);
  }
  s.timing.clear();
  if (err != VK_SUCCESS) q->lost = err;
  if (s.fence) {
    s.fence->signaled = true;
    s.fence->pending = false;
    s.fence->error = err;
  }
  dev->event_pool.push_back(s.done);
}

static void process_completions(Queue* q, bool block_all) {
  while (!q->inflight.empty()) {
    Submission& s = q->inflight.front();
    cudaError_t e = block_all ? cudaEventSynchronize(s.done) : cudaEventQuery(s.done);
    if (e == cudaErrorNotReady) return;
    if (e != cudaSuccess) {
      log_error("device error: %s", cudaGetErrorString(e));
      q->lost = VK_ERROR_DEVICE_LOST;
    }
    complete(q, s);
    q->inflight.erase(q->inflight.begin());
  }
}

VkResult queue_submit(Queue* q, uint32_t count, const VkSubmitInfo* submits, Fence* fence) {
  Device* dev = q->dev;
  std::lock_guard<std::recursive_mutex> lock(dev->mu);
  cudaSetDevice(dev->pd->cuda_device);
  if (q->lost != VK_SUCCESS) return q->lost;
  process_completions(q, false);
  for (uint32_t i = 0; i < count; i++)
    for (uint32_t k = 0; k < submits[i].commandBufferCount; k++) {
      CommandBuffer* cb = H<CommandBuffer>(submits[i].pCommandBuffers[k]);
      if (!cb->low) return VK_ERROR_INITIALIZATION_FAILED;
    }
  for (uint32_t i = 0; i < count; i++)
    for (uint32_t k = 0; k < submits[i].commandBufferCount; k++) {
      CommandBuffer* cb = H<CommandBuffer>(submits[i].pCommandBuffers[k]);
      enqueue(cb, q->stream);
      Submission s;
      s.cb = cb;
      s.timing.swap(cb->timing);
      s.done = pool_event(dev);
      cudaEventRecord(s.done, q->stream);
      q->inflight.push_back(s);
    }
  if (fence) {
    if (q->inflight.empty()) {
      Submission s;
      s.done = pool_event(dev);
      cudaEventRecord(s.done, q->stream);
      q->inflight.push_back(s);
    }
    cudaEventRecord(fence->ev, q->stream);
    fence->pending = true;
    fence->signaled = false;
    fence->error = VK_SUCCESS;
    q->inflight.back().fence = fence;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    log_error("submission failed: %s", cudaGetErrorString(e));
    return VK_ERROR_DEVICE_LOST;
  }
  return VK_SUCCESS;
}

VkResult queue_wait_idle(Queue* q) {
  Device* dev = q->dev;
  std::lock_guard<std::recursive_mutex> lock(dev->mu);
  cudaSetDevice(dev->pd->cuda_device);
  process_completions(q, true);
  cudaStreamSynchronize(q->stream);
  return q->lost;
}

VkResult fence_status(Device* dev, Fence* f) {
  std::lock_guard<std::recursive_mutex> lock(dev->mu);
  cudaSetDevice(dev->pd->cuda_device);
  process_completions(&dev->queue, false);
  if (f->signaled) return f->error;
  return VK_NOT_READY;
}

VkResult wait_fences(Device* dev, uint32_t n, const VkFence* fences, VkBool32 all, uint64_t timeout) {
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    {
      std::lock_guard<std::recursive_mutex> lock(dev->mu);
      cudaSetDevice(dev->pd->cuda_device);
      process_completions(&dev->queue, false);
      uint32_t done = 0;
      VkResult err = VK_SUCCESS;
      for (uint32_t i = 0; i < n; i++) {
        Fence* f = H<Fence>(fences[i]);
        if (f->signaled) {
          done++;
          if (f->error != VK_SUCCESS) err = f->error;
        }
      }
      if (err != VK_SUCCESS) return err;
      if ((all && done == n) || (!all && done > 0)) return VK_SUCCESS;
      if (timeout == 0) return VK_TIMEOUT;
      /* block on the oldest submission when waiting without a deadline */
      if (timeout == UINT64_MAX && !dev->queue.inflight.empty()) {
        cudaEventSynchronize(dev->queue.inflight.front().done);
        continue;
      }
    }
    auto el = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    if ((uint64_t)el >= timeout) return VK_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace kz

extern "C" KZ_API void* kzGetQueueStream(VkQueue queue) {
  return (void*)kz::H<kz::Queue>(queue)->stream;
}

extern "C" KZ_API int kzGetKernelTimes(VkCommandBuffer cbh, double* total_ms, uint32_t* launches, uint32_t count,
                                       int reset) {
  kz::CommandBuffer* cb = kz::H<kz::CommandBuffer>(cbh);
  if (!cb) return -1;
  std::lock_guard<std::recursive_mutex> lock(cb->dev->mu);
  for (uint32_t k = 0; k < count && k < (uint32_t)kz::KK_COUNT; k++) {
    if (total_ms) total_ms[k] = cb->kernel_ms[k];
    if (launches) launches[k] = cb->kernel_launches[k];
  }
  if (reset) {
    for (int k = 0; k < kz::KK_COUNT; k++) {
      cb->kernel_ms[k] = 0.0;
      cb->kernel_launches[k] = 0;
    }
  }
  return (int)kz::KK_COUNT;
}

extern "C" KZ_API int kzGetCommandBufferStats(VkCommandBuffer cbh, KzCommandBufferStats* out) {
  kz::CommandBuffer* cb = kz::H<kz::CommandBuffer>(cbh);
  if (!cb || !out) return -1;
  std::memset(out, 0, sizeof(*out));
  if (!cb->low) return -1;
  const kz::Lowered& low = *cb->low;
  out->triangles = low.triangles;
  out->draws = (uint32_t)low.draws.size();
  out->segments = (uint32_t)low.segments.size();
  out->mode = (uint32_t)low.mode;
  out->tile = low.tile;
  out->status = cb->last_status.flags;
  out->records = cb->last_status.need_records;
  out->pairs = cb->last_status.need_pairs;
  out->fragments = cb->last_status.fragments_lo;
  out->rec_cap = low.rec_cap;
  out->pair_cap = low.pair_cap;
  out->gpu_ms = cb->last_ms;
  out->launches = low.launches; /* counted by the launch sequence itself when it was captured or last ran */
  return 0;
}

/*
 * kazan_driver.h - C ABI of libkazan_driver.so, the GB300 drop-in for the kazan Vulkan driver's draw path.
 *
 * Loader-facing exports (same names, signatures and semantics as the reference):
 *   vk_icdGetInstanceProcAddr                 replaces vulkan-driver/src/lib.rs:38-43
 *   vk_icdNegotiateLoaderICDInterfaceVersion  replaces vulkan-driver/src/lib.rs:51-63 (clamps to 5)
 *   vk_icdGetPhysicalDeviceProcAddr           replaces vulkan-driver/src/lib.rs:68-130
 * Every vk* entry point is reached through vk_icdGetInstanceProcAddr, as in the reference's
 * get_proc_address (vulkan-driver/src/api_impl.rs:432-860).  The draw path's entry points replace:
 *   vkCmdDraw api_impl.rs:4632, vkCmdDrawIndexed :4643, vkCmdClearColorImage :4780,
 *   vkCmdClearDepthStencilImage :4792, vkCmdBindVertexBuffers :4621, vkCmdBindIndexBuffer :4611,
 *   vkCmdPushConstants :4932, vkCmdBindPipeline :4506, vkCmdSetViewport :4515, vkCmdSetScissor :4525,
 *   vkCmdBeginRenderPass :4944, vkCmdEndRenderPass :4961, vkCreateFramebuffer :4383,
 *   vkCreateRenderPass :4402, vkCreateCommandPool :4436, vkAllocateCommandBuffers :4464,
 *   vkBeginCommandBuffer :4483, vkEndCommandBuffer :4491, vkQueueSubmit :3414, vkQueueWaitIdle :3424,
 *   vkCreateFence :3653, vkWaitForFences :3689, vkCreateGraphicsPipelines :4018,
 *   vkCreatePipelineLayout :4061, vkCreateShaderModule :3946, vkAllocateMemory :3434, vkMapMemory :3488,
 *   vkCreateBuffer :3795, vkCreateImage :3851, vkBindBufferMemory2 :4975, vkBindImageMemory2 :5013,
 *   vkCmdDrawIndirect :4655, vkCmdDrawIndexedIndirect :4666, vkCmdDrawIndirectCountKHR :6025,
 *   vkCmdDrawIndexedIndirectCountKHR :6039 (also under the core names vkCmdDraw*IndirectCount), and
 *   vkEnumerateDeviceExtensionProperties, which lists VK_KHR_draw_indirect_count.
 *
 * The kz* functions below have no counterpart in the reference: they expose the driver's execution
 * options and statistics to the benchmark and tests without a Vulkan extension.
 */
#ifndef KAZAN_DRIVER_H
#define KAZAN_DRIVER_H

#include <stdint.h>

#include "kz_vk_abi.h"

#define KZ_API __attribute__((visibility("default")))

#ifdef __cplusplus
extern "C" {
#endif

KZ_API PFN_vkVoidFunction vk_icdGetInstanceProcAddr(VkInstance instance, const char* pName);
KZ_API VkResult vk_icdNegotiateLoaderICDInterfaceVersion(uint32_t* pSupportedVersion);
KZ_API PFN_vkVoidFunction vk_icdGetPhysicalDeviceProcAddr(VkInstance instance, const char* pName);

/* Execution options, read at vkEndCommandBuffer.  Keys and values:
 *   "mode"  "persistent" (default: one cooperative kernel per run of render passes, captured in a CUDA
 *           graph), "batched" (one launch per pipeline phase per render pass, captured in a CUDA graph),
 *           "perdraw" (one launch per phase per draw, launched at submit: the plain baseline)
 *   "tile"  screen-tile side in pixels: "8", "16", "32" or "64"
 *   "trace" "0" / "1": log lowering and linking decisions to stderr
 *   "fault_alloc" "N": the Nth device allocation from now fails with VK_ERROR_OUT_OF_DEVICE_MEMORY
 *   "kernel_timing" "0" / "1": command buffers ended while it is on launch their kernels at each submit
 *           (no graph capture) with a pair of timing events around every launch; see kzGetKernelTimes
 *   "pdl"   "1" (default) / "0": command buffers ended while it is on launch each kernel that follows
 *           another with programmatic stream serialization (its launch overlaps the predecessor's end)
 *   "tma"   "1" (default) / "0": command buffers ended while it is on stage the colour and depth of each
 *           tile of kz_k_raster_direct through TMA tensor copies (where the attachment's base address and
 *           row pitch are multiples of 16 bytes); with "0" the tiles are read and written with plain loads
 *   "warp_px" "N" (1..4096, default 192): in opaque passes of command buffers ended while it is set, unclipped
 *           triangles whose boxes hold at most N pixels are rasterised by their geometry warp, larger ones are
 *           split into jobs of 8x8-pixel blocks
 *   "job_blocks" "N" (1..32, default 16): 8x8-pixel blocks per large-triangle job
 *   "geo_blocks" "N" (0..64, default 0): blocks per SM of the batched geometry launches (0: as many as
 *           are resident)
 *   "vector_fetch" "1" (default) / "0": command buffers ended while it is on fetch vertex attributes with
 *           8- and 16-byte vector loads in draws whose bound vertex buffers start 16-byte aligned
 *   "barrier_ns" "N": command buffers ended while it is set give their persistent kernels' grid barriers
 *           up after waiting N nanoseconds (default 4000000000; 0 gives up at the first check).  A barrier
 *           that gives up sets KZ_STATUS_BARRIER_TIMEOUT and the submission completes with
 *           VK_ERROR_DEVICE_LOST; the kernel returns and the CUDA context stays usable
 * Returns 0, or -1 for an unknown key or value.  The KZ_MODE, KZ_TILE, KZ_TRACE, KZ_KERNEL_TIMING, KZ_PDL,
 * KZ_TMA, KZ_VECTOR_FETCH and KZ_FAULT=alloc:N environment variables set the initial values. */
KZ_API int kzDriverSetOption(const char* key, const char* value);

/* The CUDA stream (cudaStream_t) a queue executes on, for callers that time submissions with CUDA
 * events on that stream. */
KZ_API void* kzGetQueueStream(VkQueue queue);

typedef struct KzCommandBufferStats {
  uint64_t triangles;     /* triangles submitted (all draws, all instances) */
  uint32_t draws;
  uint32_t segments;      /* raster segments after lowering */
  uint32_t mode;          /* 0 persistent, 1 batched, 2 per-draw */
  uint32_t tile;          /* tile side in pixels */
  uint32_t status;        /* KzStatusBits of the last completed execution */
  uint32_t records;       /* largest number of triangle records any segment produced */
  uint32_t pairs;         /* largest number of (tile, record) pairs any segment produced */
  uint32_t fragments;     /* covered fragments of the last execution (low 32 bits) */
  uint32_t rec_cap, pair_cap;
  float gpu_ms;           /* device time of the last execution (CUDA events around the kernels) */
  uint32_t launches;      /* kernel launches per execution */
} KzCommandBufferStats;

/* Statistics of a command buffer's lowering and last completed execution (0 = success). */
KZ_API int kzGetCommandBufferStats(VkCommandBuffer commandBuffer, KzCommandBufferStats* out);

/* Kernel kinds of kzGetKernelTimes, in array order. */
#define KZ_KERNEL_KIND_NAMES                                                                          \
  {"kz_k_persistent", "kz_k_vis_init", "kz_k_vis_geometry", "kz_k_vis_large", "kz_k_vis_resolve",      \
   "kz_k_geometry",   "kz_k_scan",     "kz_k_bin",          "kz_k_raster",    "kz_k_clear",         \
   "kz_k_indirect",   "kz_k_indirect_tables", "kz_k_resolve", "kz_k_persistent_vis", "kz_k_raster_direct",  \
   "kz_k_raster_ds",  "kz_k_raster_ms"}
#define KZ_KERNEL_KINDS 17

/* Device time of a command buffer recorded with "kernel_timing" on: for each kernel kind, the summed
 * durations (CUDA events on the queue stream around each launch) and the number of launches over all
 * submissions completed since the last reset.  Fills the first `count` entries of either array (either
 * may be NULL), resets the sums when `reset` is non-zero, and returns KZ_KERNEL_KINDS (-1 for a bad
 * handle).  Submissions complete at vkQueueWaitIdle, vkWaitForFences and vkGetFenceStatus. */
KZ_API int kzGetKernelTimes(VkCommandBuffer commandBuffer, double* totalMs, uint32_t* launches, uint32_t count,
                            int reset);

/* No counterpart in the reference.  Renders without allocating device memory, for callers that cannot call
 * cudaMalloc when they draw: programs that hand all device memory to their own pool allocator up front, and
 * latency-bound serving loops that must not take the device-wide synchronisation an allocation or free
 * may cause.  The Vulkan path allocates its scratch at vkEndCommandBuffer; this call uses one fixed scratch
 * array inside the library instead (about 24 MiB, held on every GPU that loads the library until the
 * process exits).
 *
 * Draws `triangleCount` triangles (non-indexed list, 8 floats per vertex: clip-space x, y, z, w, then
 * colour r, g, b, a) into a width x height RGBA8 image and D32 depth image (tight rows), both cleared
 * first: full viewport, depth range [0, 1], depth test LESS with writes, no culling, no blending -- the
 * same pixels the Vulkan path gives for that pipeline.  Pointers are device pointers owned by the caller;
 * `stream` is a cudaStream_t (NULL: legacy default stream); the call synchronises that stream and returns
 * once the work has finished.
 * Limits: width * height <= 1048576 and triangleCount <= 65536 (else -1, before any GPU work); at most
 * 131072 large-triangle records (one per triangle whose box exceeds 192 pixels, and per clipped
 * sub-triangle whose box exceeds 32) and 2^20 8x8-block jobs of those records (else -3: the scratch
 * overflowed and the image is incomplete).  Returns 0 on success and -2 for a CUDA error.  Allocates
 * nothing: no cudaMalloc, cudaFree or allocating library call.
 *
 * The first call on a device, and the first after its context changed, looks up the scratch array's device
 * address.  All calls share the scratch, which keeps the last call's contents; each call clears what must
 * start at zero, but calls whose work overlaps on the GPU (other streams, other threads) race. */
KZ_API int kzRasterTrianglesNoAlloc(const float* vertices, uint32_t triangleCount, uint32_t width, uint32_t height,
                                    uint32_t* color, float* depth, const float clearColor[4], float clearDepth,
                                    void* stream);

#ifdef __cplusplus
}
#endif

#endif /* KAZAN_DRIVER_H */

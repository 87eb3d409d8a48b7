/*
 * kz_noalloc.cu - an entry point that renders without allocating any device memory.
 *
 * Some callers of this library cannot call cudaMalloc when they draw: programs that hand all device memory
 * to their own pool allocator up front (so a cudaMalloc of the driver's scratch would fail or fragment
 * their pool), and latency-bound serving loops that must not take the implicit device-wide
 * synchronisation cudaMalloc and cudaFree can cause.  The Vulkan path allocates its scratch (visibility
 * keys, triangle records, work lists) at vkEndCommandBuffer; kzRasterTrianglesNoAlloc instead keeps that
 * scratch in one file-scope __device__ array of fixed size, which every GPU that loads this library holds
 * until the process exits (KZ_NOALLOC_SCRATCH_BYTES, about 24 MiB).
 *
 * It runs the same visibility-buffer kernels as the Vulkan path (this file compiles kz_pipeline.cu
 * together with the pass-through colour stage: gl_Position = attribute 0, colour = attribute 1), so the
 * image equals what the driver renders for the same triangles.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "kazan_driver.h"
#include "kz_pipeline.cu"

/* limits of the fixed scratch */
#define KZ_NOALLOC_MAX_PIXELS (1024u * 1024u)
#define KZ_NOALLOC_MAX_TRIS 65536u
#define KZ_NOALLOC_MAX_RECORDS (2u * KZ_NOALLOC_MAX_TRIS)
#define KZ_NOALLOC_MAX_JOBS (1u << 20)

/* layout of the scratch array (byte offsets, each 256-byte aligned) */
#define KZ_NA_VIS 0u
#define KZ_NA_RECORDS (KZ_NA_VIS + KZ_NOALLOC_MAX_PIXELS * 8u)
#define KZ_NA_JOBS (KZ_NA_RECORDS + KZ_NOALLOC_MAX_RECORDS * (uint32_t)sizeof(KzTriRecord))
#define KZ_NA_CHUNKS (KZ_NA_JOBS + KZ_NOALLOC_MAX_JOBS * 8u)
#define KZ_NA_TABLES (KZ_NA_CHUNKS + (KZ_NOALLOC_MAX_TRIS / KZ_CHUNK) * (uint32_t)sizeof(KzChunk))
#define KZ_NA_DRAW (KZ_NA_TABLES)
#define KZ_NA_PIPE (KZ_NA_DRAW + 256u)
#define KZ_NA_SEG (KZ_NA_PIPE + 512u)
#define KZ_NA_PUSH (KZ_NA_SEG + 512u)
#define KZ_NA_COUNTERS (KZ_NA_PUSH + 256u)
#define KZ_NA_STATUS (KZ_NA_COUNTERS + 256u)
#define KZ_NOALLOC_SCRATCH_BYTES (KZ_NA_STATUS + 256u)

static_assert(sizeof(KzDraw) <= 256 && sizeof(KzPipe) <= 512 && sizeof(KzSegment) <= 512, "table slots");
static_assert(KZ_NA_RECORDS % 256 == 0 && KZ_NA_JOBS % 256 == 0 && KZ_NA_CHUNKS % 256 == 0 && KZ_NA_TABLES % 256 == 0,
              "scratch regions stay aligned");

/* the scratch: shared by every call on a device; calls that overlap on the GPU race on it */
static __device__ __align__(256) unsigned char kz_noalloc_scratch[KZ_NOALLOC_SCRATCH_BYTES];

/* pass-through colour stage (the same results as the SPIR-V pass-through shaders compiled by the backend:
 * no arithmetic, attribute words copied) */
extern "C" __device__ float4 kz_vs_pos(uint32_t, const KzDraw* d, uint32_t vid, uint32_t, const uint8_t*) {
  const float* v = reinterpret_cast<const float*>(d->vb[0]) + (size_t)vid * 8;
  return make_float4(v[0], v[1], v[2], v[3]);
}

extern "C" __device__ KzPos3 kz_vs_pos3(uint32_t pipe, const KzDraw* d, uint32_t v0, uint32_t v1, uint32_t v2,
                                        uint32_t iid, const uint8_t* push) {
  KzPos3 r;
  r.p[0] = kz_vs_pos(pipe, d, v0, iid, push);
  r.p[1] = kz_vs_pos(pipe, d, v1, iid, push);
  r.p[2] = kz_vs_pos(pipe, d, v2, iid, push);
  return r;
}

extern "C" __device__ void kz_vs(uint32_t, const KzDraw* d, uint32_t vid, uint32_t, const uint8_t*, KzVsOut* out) {
  const float* v = reinterpret_cast<const float*>(d->vb[0]) + (size_t)vid * 8;
  for (int k = 0; k < 4; k++) out->pos[k] = v[k];
  for (int k = 0; k < 4; k++) out->var[k] = v[4 + k];
}

extern "C" __device__ uint32_t kz_fs(uint32_t, const KzFsIn* in, const uint8_t*, float* color) {
  for (int k = 0; k < 4; k++) color[k] = in->var[k];
  return 0;
}

extern "C" __device__ KzFsResult kz_fs_r8(uint32_t, const uint8_t*, uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3,
                                          uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t,
                                          uint32_t) {
  KzFsResult r;
  r.c[0] = __uint_as_float(v0);
  r.c[1] = __uint_as_float(v1);
  r.c[2] = __uint_as_float(v2);
  r.c[3] = __uint_as_float(v3);
  r.discard = 0;
  r.pad[0] = r.pad[1] = r.pad[2] = 0;
  return r;
}

/* writes the tables of one draw into the scratch and zeroes the counters (one block) */
extern "C" __global__ void kz_k_noalloc_setup(KzDraw draw, KzPipe pipe, KzSegment seg, unsigned char* base,
                                              uint32_t tri_count) {
  if (threadIdx.x == 0) {
    *reinterpret_cast<KzDraw*>(base + KZ_NA_DRAW) = draw;
    *reinterpret_cast<KzPipe*>(base + KZ_NA_PIPE) = pipe;
    *reinterpret_cast<KzSegment*>(base + KZ_NA_SEG) = seg;
  }
  KzChunk* chunks = reinterpret_cast<KzChunk*>(base + KZ_NA_CHUNKS);
  uint32_t nchunks = (tri_count + KZ_CHUNK - 1) / KZ_CHUNK;
  for (uint32_t i = threadIdx.x; i < nchunks; i += blockDim.x) {
    KzChunk ch;
    ch.draw = 0;
    ch.first = i * KZ_CHUNK;
    ch.count = min((uint32_t)KZ_CHUNK, tri_count - i * KZ_CHUNK);
    ch.pad = 0;
    chunks[i] = ch;
  }
  uint32_t* zero = reinterpret_cast<uint32_t*>(base + KZ_NA_PUSH);
  for (uint32_t i = threadIdx.x; i < (KZ_NOALLOC_SCRATCH_BYTES - KZ_NA_PUSH) / 4; i += blockDim.x) zero[i] = 0;
}

namespace {

/* the driver API's cuCtxGetCurrent, reached through the runtime (the library links no libcuda) */
typedef int (*CtxGetCurrentFn)(void** ctx);

std::mutex g_mu;
struct ScratchAddr {
  void* ctx = nullptr;   /* the context the address belongs to */
  void* base = nullptr;  /* device address of kz_noalloc_scratch in it */
};
ScratchAddr g_base[64];
CtxGetCurrentFn g_ctx_get = nullptr;

/* Set-up, with the device current: the device address of the scratch array, looked up with
 * cudaGetSymbolAddress the first time a device is used, and again whenever the device's current context
 * is not the one the address was taken in (after cudaDeviceReset the module is loaded anew, at another
 * address).  The array's name in host code is only a host-side stand-in for the symbol; kernels must be
 * given this address. */
cudaError_t scratch_base(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ctx_get) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return e != cudaSuccess ? e : cudaErrorUnknown;
    g_ctx_get = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  void* ctx = nullptr;
  if (g_ctx_get(&ctx) != 0) return cudaErrorDeviceUninitialized;
  ScratchAddr& a = g_base[dev];
  if (!ctx || !a.base || a.ctx != ctx) {
    /* the lookup also makes the device's primary context current when no context is */
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, kz_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (g_ctx_get(&ctx) != 0 || !ctx) return cudaErrorDeviceUninitialized;
    a.base = p;
    a.ctx = ctx;
  }
  *out = a.base;
  return cudaSuccess;
}

uint8_t host_unorm8(float v) {
  float c = std::fmin(std::fmax(v, 0.0f), 1.0f);
  return (uint8_t)(int)std::rint(c * 255.0f);
}

}  // namespace

/* Render `triangle_count` triangles (non-indexed list; 8 floats per vertex: clip-space position x, y, z,
 * w then colour r, g, b, a) into a width x height RGBA8 colour image and D32 depth image (tightly packed
 * rows), both cleared first: depth test LESS with writes, no culling, no blending.  All pointers are
 * device pointers owned by the caller; `stream` is a cudaStream_t (NULL for the legacy default stream).
 * The call synchronises `stream` and returns after the rendering finished.
 *
 * Limits: width * height <= 1048576 pixels (KZ_NOALLOC_MAX_PIXELS), triangle_count <= 65536, at most
 * 131072 large-triangle records (one per triangle whose box exceeds 192 pixels, and per clipped
 * sub-triangle whose box exceeds 32), and at most 2^20 8x8-block warp jobs of those records.  Returns 0 on
 * success, -1 for arguments beyond the first two limits (before any GPU work), -2 for a CUDA error, -3
 * when the records or the jobs overflow their scratch (the image is then incomplete).
 *
 * Allocates nothing: no cudaMalloc, cudaFree or allocating library call.  The first call on a device (and
 * the first after the device's context changed) looks up the scratch array's device address.  Every call
 * shares the scratch array, which keeps the last call's contents; each call clears what must start at
 * zero (counters and status) and initialises the visibility keys, but calls whose work overlaps on the GPU
 * (other streams, other threads) race on it. */
extern "C" KZ_API int kzRasterTrianglesNoAlloc(const float* vertices, uint32_t triangle_count, uint32_t width,
                                                      uint32_t height, uint32_t* color, float* depth,
                                                      const float clear_color[4], float clear_depth, void* stream) {
  if (!vertices || !color || !depth || !clear_color || width == 0 || height == 0 || width > 8192 ||
      height > 8192 || (uint64_t)width * height > KZ_NOALLOC_MAX_PIXELS || triangle_count > KZ_NOALLOC_MAX_TRIS)
    return -1;
  void* basep = nullptr;
  if (scratch_base(&basep) != cudaSuccess) return -2;
  unsigned char* base = static_cast<unsigned char*>(basep);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  KzDraw d;
  std::memset(&d, 0, sizeof d);
  d.vb[0] = (uint64_t)(uintptr_t)vertices;
  d.indexed = 0;
  d.vertex_offset = 0;
  d.first_instance = 0;
  d.instance_count = 1;
  d.tri_count = triangle_count;
  d.pipe = 0;
  d.prim_base = 0;
  d.push_index = 0;
  float vw = (float)width, vh = (float)height;
  d.hx = 0.5f * vw;
  d.ox = 0.0f + d.hx;
  d.hy = 0.5f * vh;
  d.oy = 0.0f + d.hy;
  d.pz = 1.0f - 0.0f;
  d.oz = 0.0f;
  d.zmin = 0.0f;
  d.zmax = 1.0f;
  d.rect[0] = 0;
  d.rect[1] = 0;
  d.rect[2] = (int32_t)width;
  d.rect[3] = (int32_t)height;

  KzPipe p;
  std::memset(&p, 0, sizeof p);
  p.num_attrs = 2;
  p.attrs[0].location = 0;
  p.attrs[0].format = KZ_FMT_F32x4;
  p.attrs[1].location = 1;
  p.attrs[1].format = KZ_FMT_F32x4;
  p.attrs[1].offset = 16;
  p.pos_input_mask = 1;
  p.full_input_mask = 3;
  p.num_varyings = 4;
  p.binding_stride[0] = 32;
  p.cull_mode = 0;
  p.front_ccw = 1;
  p.depth_test = 1;
  p.depth_write = 1;
  p.depth_compare = 1; /* VK_COMPARE_OP_LESS */
  p.write_mask = 0xF;
  p.has_fs = 1;

  KzSegment s;
  std::memset(&s, 0, sizeof s);
  s.first_draw = 0;
  s.num_draws = 1;
  s.first_chunk = 0;
  s.num_chunks = (triangle_count + KZ_CHUNK - 1) / KZ_CHUNK;
  s.num_prims = triangle_count;
  s.mode = KZ_MODE_VISIBILITY;
  s.vis_key = KZ_VIS_LESS;
  s.tile = 16;
  s.tiles_x = (width + 15) / 16;
  s.tiles_y = (height + 15) / 16;
  s.color = (uint64_t)(uintptr_t)color;
  s.depth = (uint64_t)(uintptr_t)depth;
  s.width = width;
  s.height = height;
  s.color_pitch = width * 4;
  s.depth_pitch = width * 4;
  s.color_format = KZ_CF_RGBA8;
  s.color_load = KZ_LOAD_CLEAR;
  s.depth_load = KZ_LOAD_CLEAR;
  s.color_store = s.depth_store = 1;
  s.clear_color = (uint32_t)host_unorm8(clear_color[0]) | ((uint32_t)host_unorm8(clear_color[1]) << 8) |
                  ((uint32_t)host_unorm8(clear_color[2]) << 16) | ((uint32_t)host_unorm8(clear_color[3]) << 24);
  s.clear_depth = clear_depth;
  s.area[0] = 0;
  s.area[1] = 0;
  s.area[2] = (int32_t)width;
  s.area[3] = (int32_t)height;
  s.records = (uint64_t)(uintptr_t)(base + KZ_NA_RECORDS);
  s.bins = (uint64_t)(uintptr_t)(base + KZ_NA_JOBS);
  s.counters = (uint64_t)(uintptr_t)(base + KZ_NA_COUNTERS);
  s.vis = (uint64_t)(uintptr_t)(base + KZ_NA_VIS);
  s.rec_cap = KZ_NOALLOC_MAX_RECORDS;
  s.pair_cap = 2 * KZ_NOALLOC_MAX_JOBS; /* jobs take two words each */

  KzFrame f;
  std::memset(&f, 0, sizeof f);
  f.draws = (uint64_t)(uintptr_t)(base + KZ_NA_DRAW);
  f.pipes = (uint64_t)(uintptr_t)(base + KZ_NA_PIPE);
  f.chunks = (uint64_t)(uintptr_t)(base + KZ_NA_CHUNKS);
  f.segments = (uint64_t)(uintptr_t)(base + KZ_NA_SEG);
  f.push = (uint64_t)(uintptr_t)(base + KZ_NA_PUSH);
  f.status = (uint64_t)(uintptr_t)(base + KZ_NA_STATUS);
  f.num_segments = 1;
  f.first_segment = 0;
  f.chunk_begin = 0;
  f.chunk_end = 0xFFFFFFFFu;
  f.jobs_incremental = 0;
  f.barrier_ns = 0; /* no persistent kernel runs here */
  f.warp_px = KZ_WARP_PX_DEFAULT;
  f.job_blocks = KZ_JOB_BLOCKS_DEFAULT;

  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  uint32_t cap = (uint32_t)(sms > 0 ? sms : 1) * 8u;
  uint32_t seg_index = 0;
  kz_k_noalloc_setup<<<1, 256, 0, st>>>(d, p, s, base, triangle_count);
  kz_k_vis_init<<<std::min(cap, (width * height + 255) / 256), 256, 0, st>>>(f, seg_index);
  if (s.num_chunks) {
    kz_k_vis_geometry<<<s.num_chunks, 256, 0, st>>>(f, seg_index);
    kz_k_vis_large<<<cap, 256, 0, st>>>(f, seg_index);
  }
  kz_k_vis_resolve<<<cap, 256, 0, st>>>(f, seg_index);
  if (cudaGetLastError() != cudaSuccess) return -2;
  KzStatus status;
  if (cudaMemcpyAsync(&status, base + KZ_NA_STATUS, sizeof status, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return -2;
  if (status.flags & (KZ_STATUS_RECORD_OVERFLOW | KZ_STATUS_PAIR_OVERFLOW)) return -3;
  return status.flags ? -2 : 0;
}

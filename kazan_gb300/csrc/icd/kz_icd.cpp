/*
 * kz_icd.cpp - loader interface, dispatch, and the device/resource/pipeline objects of the kazan GB300
 * Vulkan driver.
 *
 * Entry points keep the reference driver's names, signatures and error conventions
 * (vulkan-driver/src/lib.rs:38-130, api_impl.rs); each function cites the reference function it replaces.
 * Invalid usage that the reference answers with a panic is answered here with a VkResult error and a
 * message on stderr, never with an abort of the host process.
 */
#include <algorithm>
#include "kz_icd.h"

#include <dlfcn.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>

#include "../shader/kz_shader_backend_impl.h"
#include "kazan_driver.h"

namespace kz {

/* ------------------------------------------------------------------------------------------------ */
/* options, logging, allocation                                                                     */

Options& options() {
  static Options o = [] {
    Options r;
    const char* m = std::getenv("KZ_MODE");
    if (m) {
      if (!std::strcmp(m, "batched")) r.mode = 1;
      else if (!std::strcmp(m, "perdraw")) r.mode = 2;
    }
    const char* t = std::getenv("KZ_TILE");
    if (t) r.tile = (uint32_t)std::atoi(t);
    const char* tr = std::getenv("KZ_TRACE");
    if (tr) r.trace = std::atoi(tr);
    const char* f = std::getenv("KZ_FAULT");
    if (f && !std::strncmp(f, "alloc:", 6)) r.fault_alloc = std::atol(f + 6);
    const char* kt = std::getenv("KZ_KERNEL_TIMING");
    if (kt) r.kernel_timing = std::atoi(kt);
    const char* tm = std::getenv("KZ_TMA");
    if (tm) r.tma = std::atoi(tm) != 0;
    const char* vf = std::getenv("KZ_VECTOR_FETCH");
    if (vf) r.vector_fetch = std::atoi(vf) != 0;
    const char* pd = std::getenv("KZ_PDL");
    if (pd) r.pdl = std::atoi(pd) != 0;
    return r;
  }();
  return o;
}

void log_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::fprintf(stderr, "kazan: ");
  std::vfprintf(stderr, fmt, ap);
  std::fprintf(stderr, "\n");
  va_end(ap);
}

static long g_alloc_count = 0;

VkResult device_alloc(size_t bytes, void** out) {
  *out = nullptr;
  long n = __atomic_add_fetch(&g_alloc_count, 1, __ATOMIC_RELAXED);
  if (options().fault_alloc >= 0 && n == options().fault_alloc) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(out, bytes) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  }
  return VK_SUCCESS;
}

void device_free(void* p) {
  if (p) cudaFree(p);
}

/* a relocatable object built next to this library (`env` overrides its path) */
static std::vector<char> load_object(const char* env, const char* name) {
  std::vector<char> v;
  std::string path;
  const char* e = std::getenv(env);
  if (e) {
    path = e;
  } else {
    Dl_info info;
    if (dladdr((void*)&load_object, &info) && info.dli_fname) {
      path = info.dli_fname;
      size_t slash = path.rfind('/');
      path = (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/" + name;
    }
  }
  std::ifstream f(path, std::ios::binary);
  if (f) v.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  else log_error("object not found at %s", path.c_str());
  return v;
}

/* the relocatable pipeline-kernel object */
const std::vector<char>& pipeline_object() {
  static std::vector<char> obj = load_object("KZ_PIPELINE_OBJECT", "kz_pipeline.cubin");
  return obj;
}

/* the relocatable texture-sampling object the shaders call into */
const std::vector<char>& texture_object() {
  static std::vector<char> obj = load_object("KZ_TEXTURE_OBJECT", "kz_tex.cubin");
  return obj;
}

KernelSet* kernel_set_for(Device* dev, const std::vector<Pipeline*>& pipes, const std::vector<uint32_t>& base_align,
                          std::string& err) {
  std::vector<uint64_t> key;
  for (size_t i = 0; i < pipes.size(); i++) key.push_back((pipes[i]->uid << 5) | (base_align[i] & 31u));
  auto it = dev->kernel_sets.find(key);
  if (it != dev->kernel_sets.end()) return it->second;
  const std::vector<char>& obj = pipeline_object();
  if (obj.empty()) {
    err = "the pipeline kernel object is missing (run the package build)";
    return nullptr;
  }
  std::vector<const ir::Shader*> vs, fs;
  std::vector<ptx::VertexLayout> layouts;
  for (size_t i = 0; i < pipes.size(); i++) {
    Pipeline* p = pipes[i];
    vs.push_back(p->vs.get());
    fs.push_back(p->fs.get());
    ptx::VertexLayout l;
    l.base_align = base_align[i];
    l.num_attrs = p->pipe.num_attrs;
    for (uint32_t k = 0; k < p->pipe.num_attrs; k++) {
      l.location[k] = p->pipe.attrs[k].location;
      l.binding[k] = p->pipe.attrs[k].binding;
      l.format[k] = p->pipe.attrs[k].format;
      l.offset[k] = p->pipe.attrs[k].offset;
    }
    for (uint32_t b = 0; b < KZ_MAX_BINDINGS; b++) l.stride[b] = p->pipe.binding_stride[b];
    l.instanced = p->pipe.binding_instanced;
    if (p->layout)
      for (size_t s = 0; s < p->layout->sets.size(); s++)
        for (const SetBinding& b : p->layout->sets[s]->bindings)
          l.desc_slot[s][b.binding] = p->layout->slot_base[s] + b.first;
    layouts.push_back(l);
  }
  std::string ptx = ptx::module_text(vs, fs, layouts);
  /* pipelines that differ only in fixed-function state (viewport, depth, blend: data in KzPipe) give the
   * same PTX and share one linked image */
  auto same = dev->kernel_sets_by_ptx.find(ptx);
  if (same != dev->kernel_sets_by_ptx.end()) {
    dev->kernel_sets[key] = same->second;
    return same->second;
  }
  std::vector<char> cubin;
  const std::vector<char>& tex = texture_object();
  err = ptx::link(ptx, obj.data(), obj.size(), cubin, tex.data(), tex.size());
  if (!err.empty()) return nullptr;
  KernelSet* ks = new KernelSet();
  cudaSetDevice(dev->pd->cuda_device);
  if (cudaLibraryLoadData(&ks->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
    err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(cudaGetLastError());
    delete ks;
    return nullptr;
  }
  struct {
    const char* name;
    cudaKernel_t* k;
  } names[] = {{"kz_k_geometry", &ks->geometry}, {"kz_k_scan", &ks->scan},
               {"kz_k_bin", &ks->bin},           {"kz_k_raster", &ks->raster},
               {"kz_k_persistent", &ks->persistent}, {"kz_k_persistent_vis", &ks->persistent_vis},
               {"kz_k_raster_direct", &ks->raster_direct}, {"kz_k_raster_ds", &ks->raster_ds},
               {"kz_k_raster_ms", &ks->raster_ms},
               {"kz_k_clear", &ks->clear},
               {"kz_k_vis_init", &ks->vis_init}, {"kz_k_vis_geometry", &ks->vis_geometry},
               {"kz_k_vis_large", &ks->vis_large}, {"kz_k_vis_resolve", &ks->vis_resolve},
               {"kz_k_indirect", &ks->indirect}, {"kz_k_indirect_tables", &ks->indirect_tables},
               {"kz_k_resolve", &ks->resolve}};
  for (auto& n : names) {
    if (cudaLibraryGetKernel(n.k, ks->lib, n.name) != cudaSuccess) {
      err = std::string("kernel ") + n.name + " missing from the linked module";
      cudaGetLastError();
      delete ks;
      return nullptr;
    }
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)ks->persistent, 256, KZ_DYN_SMEM) !=
          cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  ks->persistent_blocks = per_sm * dev->pd->sm_count;
  int vis_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&vis_sm, (const void*)ks->persistent_vis, 256, 0) != cudaSuccess ||
      vis_sm < 1) {
    cudaGetLastError();
    vis_sm = 1;
  }
  ks->persistent_vis_blocks = vis_sm * dev->pd->sm_count;
  int geo_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&geo_sm, (const void*)ks->vis_geometry, 256, 0) != cudaSuccess ||
      geo_sm < 1) {
    cudaGetLastError();
    geo_sm = 1;
  }
  ks->geometry_blocks = geo_sm * dev->pd->sm_count;
  if (options().trace) log_error("kernel set linked: %zu pipelines, persistent grid %d", pipes.size(), ks->persistent_blocks);
  dev->kernel_sets[key] = ks;
  dev->kernel_sets_by_ptx[ptx] = ks;
  return ks;
}

/* ------------------------------------------------------------------------------------------------ */
/* helpers                                                                                          */

template <class T>
static T* from_handle(const void* h) {
  return reinterpret_cast<T*>(const_cast<void*>(h));
}

template <class H, class T>
static H to_handle(T* p) {
  return reinterpret_cast<H>(p);
}

static VkResult copy_props(uint32_t* count, void* out, const void* src, size_t n, size_t elem) {
  if (!out) {
    *count = (uint32_t)n;
    return VK_SUCCESS;
  }
  size_t k = *count < n ? *count : n;
  std::memcpy(out, src, k * elem);
  *count = (uint32_t)k;
  return k < n ? VK_INCOMPLETE : VK_SUCCESS;
}

static uint32_t format_bpp(VkFormat f) {
  switch (f) {
    case VK_FORMAT_R8G8B8A8_UNORM:
    case VK_FORMAT_B8G8R8A8_UNORM:
    case VK_FORMAT_R8G8B8A8_SRGB:
    case VK_FORMAT_B8G8R8A8_SRGB:
    case VK_FORMAT_D32_SFLOAT:
    case VK_FORMAT_D24_UNORM_S8_UINT: return 4;
    case VK_FORMAT_D16_UNORM: return 2;
    default: return 0;
  }
}

static uint32_t attr_format(VkFormat f) {
  switch (f) {
    case VK_FORMAT_R32_SFLOAT: return KZ_FMT_F32x1;
    case VK_FORMAT_R32G32_SFLOAT: return KZ_FMT_F32x2;
    case VK_FORMAT_R32G32B32_SFLOAT: return KZ_FMT_F32x3;
    case VK_FORMAT_R32G32B32A32_SFLOAT: return KZ_FMT_F32x4;
    case VK_FORMAT_R8G8B8A8_UNORM: return KZ_FMT_U8x4_UNORM;
    case VK_FORMAT_R32_UINT:
    case VK_FORMAT_R32_SINT: return KZ_FMT_U32x1;
    case VK_FORMAT_R32G32_UINT:
    case VK_FORMAT_R32G32_SINT: return KZ_FMT_U32x2;
    case VK_FORMAT_R32G32B32_UINT:
    case VK_FORMAT_R32G32B32_SINT: return KZ_FMT_U32x3;
    case VK_FORMAT_R32G32B32A32_UINT:
    case VK_FORMAT_R32G32B32A32_SINT: return KZ_FMT_U32x4;
    default: return KZ_FMT_NONE;
  }
}

/* ------------------------------------------------------------------------------------------------ */
/* instance and physical device (api_impl.rs:862-3400)                                              */

static PFN_vkVoidFunction lookup(const char* name);

static VkResult VKAPI_CALL kzCreateInstance(const VkInstanceCreateInfo* ci, const VkAllocationCallbacks*,
                                            VkInstance* out) {
  /* api_impl.rs:3155 vkCreateInstance / :2941 Instance::new; no instance extensions or layers */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_INSTANCE_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  if (ci->enabledLayerCount) return VK_ERROR_LAYER_NOT_PRESENT;
  if (ci->enabledExtensionCount) return VK_ERROR_EXTENSION_NOT_PRESENT;
  Instance* inst = new Instance();
  if (ci->pApplicationInfo && ci->pApplicationInfo->apiVersion) inst->api_version = ci->pApplicationInfo->apiVersion;
  int n = 0;
  if (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) {
    PhysicalDevice* pd = new PhysicalDevice();
    pd->instance = inst;
    pd->cuda_device = 0;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) {
      pd->sm_count = prop.multiProcessorCount;
      pd->hbm_bytes = prop.totalGlobalMem;
      pd->name = std::string("Kazan GB300 Renderer (") + prop.name + ")";
    }
    inst->pd = pd;
  } else {
    cudaGetLastError();
  }
  *out = to_handle<VkInstance>(inst);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyInstance(VkInstance instance, const VkAllocationCallbacks*) {
  Instance* inst = from_handle<Instance>(instance);
  if (!inst) return;
  delete inst->pd;
  delete inst;
}

static VkResult VKAPI_CALL kzEnumerateInstanceVersion(uint32_t* v) {
  *v = VK_MAKE_VERSION(1, 1, 0);
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzEnumerateInstanceExtensionProperties(const char* layer, uint32_t* count,
                                                                  VkExtensionProperties*) {
  if (layer) return VK_ERROR_LAYER_NOT_PRESENT;
  *count = 0;
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzEnumerateInstanceLayerProperties(uint32_t* count, VkLayerProperties*) {
  *count = 0;
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzEnumeratePhysicalDevices(VkInstance instance, uint32_t* count, VkPhysicalDevice* out) {
  /* api_impl.rs:3179; one physical device per instance when a GPU is present */
  Instance* inst = from_handle<Instance>(instance);
  uint32_t n = inst->pd ? 1u : 0u;
  if (!out) {
    *count = n;
    return VK_SUCCESS;
  }
  if (*count < n) {
    *count = 0;
    return VK_INCOMPLETE;
  }
  if (n) out[0] = to_handle<VkPhysicalDevice>(inst->pd);
  *count = n;
  return VK_SUCCESS;
}

static void VKAPI_CALL kzGetPhysicalDeviceProperties(VkPhysicalDevice physicalDevice, VkPhysicalDeviceProperties* p) {
  /* api_impl.rs:1512-1599 (limits); 16.8 fixed point is advertised as 8 sub-pixel bits */
  PhysicalDevice* pd = from_handle<PhysicalDevice>(physicalDevice);
  std::memset(p, 0, sizeof(*p));
  p->apiVersion = VK_MAKE_VERSION(1, 1, 0);
  p->driverVersion = VK_MAKE_VERSION(0, 1, 0);
  p->vendorID = 0;
  p->deviceID = 0;
  p->deviceType = VK_PHYSICAL_DEVICE_TYPE_DISCRETE_GPU;
  std::snprintf(p->deviceName, sizeof p->deviceName, "%s", pd->name.c_str());
  VkPhysicalDeviceLimits& l = p->limits;
  l.maxImageDimension1D = 8192;
  l.maxImageDimension2D = 8192;
  l.maxImageDimension3D = 1;
  l.maxImageDimensionCube = 1;
  l.maxImageArrayLayers = 1;
  l.maxTexelBufferElements = 0;
  l.maxUniformBufferRange = 65536;
  l.maxStorageBufferRange = 0xFFFFFFFFu; /* read-only storage buffers: the descriptor's range is 32-bit */
  l.maxPushConstantsSize = KZ_PUSH_BYTES;
  l.maxMemoryAllocationCount = 1u << 20;
  l.maxSamplerAllocationCount = 1u << 16;
  l.bufferImageGranularity = 1;
  l.maxBoundDescriptorSets = KZ_MAX_DESC_SETS;
  l.maxPerStageDescriptorSamplers = l.maxPerStageDescriptorSampledImages = KZ_MAX_DESC_SLOTS;
  l.maxPerStageDescriptorUniformBuffers = KZ_MAX_DESC_SLOTS;
  l.maxPerStageResources = KZ_MAX_DESC_SLOTS;
  l.maxDescriptorSetSamplers = l.maxDescriptorSetSampledImages = KZ_MAX_DESC_SLOTS;
  l.maxDescriptorSetUniformBuffers = KZ_MAX_DESC_SLOTS;
  l.maxDescriptorSetUniformBuffersDynamic = KZ_MAX_DESC_SLOTS;
  l.maxPerStageDescriptorStorageBuffers = KZ_MAX_DESC_SLOTS;
  l.maxDescriptorSetStorageBuffers = KZ_MAX_DESC_SLOTS;
  l.maxDescriptorSetStorageBuffersDynamic = KZ_MAX_DESC_SLOTS;
  l.maxVertexInputAttributes = KZ_MAX_VS_INPUTS;
  l.maxVertexInputBindings = KZ_MAX_BINDINGS;
  l.maxVertexInputAttributeOffset = 2047;
  l.maxVertexInputBindingStride = 2048;
  l.maxVertexOutputComponents = KZ_MAX_VARYINGS + 4;
  l.maxFragmentInputComponents = KZ_MAX_VARYINGS;
  l.maxFragmentOutputAttachments = 1;
  l.maxFragmentCombinedOutputResources = 1;
  l.subPixelPrecisionBits = KZ_SUBPIXEL_BITS;
  l.subTexelPrecisionBits = 0;
  l.mipmapPrecisionBits = 0;
  l.maxDrawIndexedIndexValue = 0xFFFFFFFFu;
  l.maxDrawIndirectCount = 0xFFFFFFFFu;
  l.maxViewports = 1;
  l.maxViewportDimensions[0] = l.maxViewportDimensions[1] = 8192;
  l.viewportBoundsRange[0] = -16384.0f;
  l.viewportBoundsRange[1] = 16383.0f;
  l.viewportSubPixelBits = 0;
  l.minMemoryMapAlignment = 128;
  l.minTexelBufferOffsetAlignment = 64;
  l.minUniformBufferOffsetAlignment = 16;
  l.minStorageBufferOffsetAlignment = 64;
  l.maxFramebufferWidth = 8192;
  l.maxFramebufferHeight = 8192;
  l.maxFramebufferLayers = 1;
  l.framebufferColorSampleCounts = VK_SAMPLE_COUNT_1_BIT | VK_SAMPLE_COUNT_4_BIT;
  l.framebufferDepthSampleCounts = VK_SAMPLE_COUNT_1_BIT | VK_SAMPLE_COUNT_4_BIT;
  l.framebufferStencilSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.framebufferNoAttachmentsSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.maxColorAttachments = 1;
  l.sampledImageColorSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.sampledImageIntegerSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.sampledImageDepthSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.sampledImageStencilSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.storageImageSampleCounts = VK_SAMPLE_COUNT_1_BIT;
  l.maxSampleMaskWords = 1;
  l.timestampComputeAndGraphics = VK_FALSE;
  l.timestampPeriod = 0.0f;
  l.discreteQueuePriorities = 2;
  l.pointSizeRange[0] = l.pointSizeRange[1] = 1.0f;
  l.lineWidthRange[0] = l.lineWidthRange[1] = 1.0f;
  l.strictLines = VK_FALSE;
  l.standardSampleLocations = VK_TRUE;
  l.optimalBufferCopyOffsetAlignment = 16;
  l.optimalBufferCopyRowPitchAlignment = 16;
  l.nonCoherentAtomSize = 1;
}

static void VKAPI_CALL kzGetPhysicalDeviceFeatures(VkPhysicalDevice, VkPhysicalDeviceFeatures* f) {
  std::memset(f, 0, sizeof(*f));
  f->fullDrawIndexUint32 = VK_TRUE;
  f->multiDrawIndirect = VK_TRUE;
  f->drawIndirectFirstInstance = VK_TRUE;
}

static void VKAPI_CALL kzGetPhysicalDeviceQueueFamilyProperties(VkPhysicalDevice, uint32_t* count,
                                                                 VkQueueFamilyProperties* out) {
  /* one family with one queue, as the reference (lib.rs:30-32) */
  VkQueueFamilyProperties q{};
  q.queueFlags = VK_QUEUE_GRAPHICS_BIT | VK_QUEUE_COMPUTE_BIT | VK_QUEUE_TRANSFER_BIT;
  q.queueCount = 1;
  q.minImageTransferGranularity = {1, 1, 1};
  copy_props(count, out, &q, 1, sizeof q);
}

static void VKAPI_CALL kzGetPhysicalDeviceMemoryProperties(VkPhysicalDevice physicalDevice,
                                                            VkPhysicalDeviceMemoryProperties* m) {
  PhysicalDevice* pd = from_handle<PhysicalDevice>(physicalDevice);
  std::memset(m, 0, sizeof(*m));
  m->memoryTypeCount = 2;
  m->memoryTypes[0].propertyFlags = VK_MEMORY_PROPERTY_DEVICE_LOCAL_BIT | VK_MEMORY_PROPERTY_HOST_VISIBLE_BIT |
                                    VK_MEMORY_PROPERTY_HOST_COHERENT_BIT | VK_MEMORY_PROPERTY_HOST_CACHED_BIT;
  m->memoryTypes[0].heapIndex = 0;
  m->memoryTypes[1].propertyFlags = VK_MEMORY_PROPERTY_DEVICE_LOCAL_BIT;
  m->memoryTypes[1].heapIndex = 0;
  m->memoryHeapCount = 1;
  m->memoryHeaps[0].size = pd->hbm_bytes;
  m->memoryHeaps[0].flags = VK_MEMORY_HEAP_DEVICE_LOCAL_BIT;
}

static void VKAPI_CALL kzGetPhysicalDeviceFormatProperties(VkPhysicalDevice, VkFormat format, VkFormatProperties* p) {
  /* api_impl.rs:1616 get_format_properties (every entry is a FIXME zero there) */
  std::memset(p, 0, sizeof(*p));
  const VkFormatFeatureFlags xfer = VK_FORMAT_FEATURE_TRANSFER_SRC_BIT | VK_FORMAT_FEATURE_TRANSFER_DST_BIT;
  switch (format) {
    case VK_FORMAT_R8G8B8A8_UNORM:
      p->bufferFeatures = VK_FORMAT_FEATURE_VERTEX_BUFFER_BIT;
      /* fall through */
    case VK_FORMAT_B8G8R8A8_UNORM:
      p->optimalTilingFeatures = p->linearTilingFeatures =
          VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BIT | VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT | xfer |
          VK_FORMAT_FEATURE_SAMPLED_IMAGE_BIT | VK_FORMAT_FEATURE_SAMPLED_IMAGE_FILTER_LINEAR_BIT;
      break;
    case VK_FORMAT_R8G8B8A8_SRGB:
    case VK_FORMAT_B8G8R8A8_SRGB: /* colour attachments (encoded at store, decoded for blending); not sampled */
      p->optimalTilingFeatures = p->linearTilingFeatures =
          VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BIT | VK_FORMAT_FEATURE_COLOR_ATTACHMENT_BLEND_BIT | xfer;
      break;
    case VK_FORMAT_D32_SFLOAT:
    case VK_FORMAT_D16_UNORM:
    case VK_FORMAT_D24_UNORM_S8_UINT:
      p->optimalTilingFeatures = p->linearTilingFeatures = VK_FORMAT_FEATURE_DEPTH_STENCIL_ATTACHMENT_BIT | xfer;
      break;
    default:
      if (attr_format(format) != KZ_FMT_NONE) p->bufferFeatures = VK_FORMAT_FEATURE_VERTEX_BUFFER_BIT;
      break;
  }
}

static VkResult VKAPI_CALL kzGetPhysicalDeviceImageFormatProperties(VkPhysicalDevice, VkFormat format, VkImageType type,
                                                                   VkImageTiling, VkImageUsageFlags, VkImageCreateFlags,
                                                                   VkImageFormatProperties* p) {
  std::memset(p, 0, sizeof(*p));
  if (type != VK_IMAGE_TYPE_2D || format_bpp(format) == 0) return VK_ERROR_FORMAT_NOT_SUPPORTED;
  p->maxExtent = {8192, 8192, 1};
  p->maxMipLevels = 1;
  p->maxArrayLayers = 1;
  p->sampleCounts = VK_SAMPLE_COUNT_1_BIT;
  if (format == VK_FORMAT_R8G8B8A8_UNORM || format == VK_FORMAT_B8G8R8A8_UNORM || format == VK_FORMAT_D32_SFLOAT)
    p->sampleCounts |= VK_SAMPLE_COUNT_4_BIT; /* attachments of multisampled passes */
  p->maxResourceSize = (VkDeviceSize)8192 * 8192 * 4;
  return VK_SUCCESS;
}

/* the one device extension: VK_KHR_draw_indirect_count (vkCmdDraw*IndirectCountKHR) */
static const char* const kDeviceExtensions[] = {"VK_KHR_draw_indirect_count"};

static VkResult VKAPI_CALL kzEnumerateDeviceExtensionProperties(VkPhysicalDevice, const char* layer, uint32_t* count,
                                                                VkExtensionProperties* out) {
  if (layer) return VK_ERROR_LAYER_NOT_PRESENT;
  const uint32_t n = (uint32_t)(sizeof kDeviceExtensions / sizeof kDeviceExtensions[0]);
  if (!out) {
    *count = n;
    return VK_SUCCESS;
  }
  uint32_t k = std::min(*count, n);
  for (uint32_t i = 0; i < k; i++) {
    std::memset(&out[i], 0, sizeof out[i]);
    std::strncpy(out[i].extensionName, kDeviceExtensions[i], VK_MAX_EXTENSION_NAME_SIZE - 1);
    out[i].specVersion = 1;
  }
  *count = k;
  return k < n ? VK_INCOMPLETE : VK_SUCCESS;
}

static VkResult VKAPI_CALL kzEnumerateDeviceLayerProperties(VkPhysicalDevice, uint32_t* count, VkLayerProperties*) {
  *count = 0;
  return VK_SUCCESS;
}

/* ------------------------------------------------------------------------------------------------ */
/* device and queue (api_impl.rs:1322-1472, 3320, 5415)                                             */

static VkResult VKAPI_CALL kzCreateDevice(VkPhysicalDevice physicalDevice, const VkDeviceCreateInfo* ci,
                                          const VkAllocationCallbacks*, VkDevice* out) {
  PhysicalDevice* pd = from_handle<PhysicalDevice>(physicalDevice);
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_DEVICE_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  for (uint32_t i = 0; i < ci->enabledExtensionCount; i++) {
    bool known = false;
    for (const char* e : kDeviceExtensions) known |= std::strcmp(ci->ppEnabledExtensionNames[i], e) == 0;
    if (!known) return VK_ERROR_EXTENSION_NOT_PRESENT;
  }
  if (ci->pEnabledFeatures) {
    const VkBool32* f = reinterpret_cast<const VkBool32*>(ci->pEnabledFeatures);
    for (size_t i = 0; i < sizeof(VkPhysicalDeviceFeatures) / sizeof(VkBool32); i++)
      if (f[i] && i != 1 && i != 9 && i != 10)
        return VK_ERROR_FEATURE_NOT_PRESENT; /* fullDrawIndexUint32, multiDrawIndirect, drawIndirectFirstInstance */
  }
  for (uint32_t i = 0; i < ci->queueCreateInfoCount; i++) {
    const VkDeviceQueueCreateInfo& q = ci->pQueueCreateInfos[i];
    if (q.queueFamilyIndex != 0 || q.queueCount != 1) return VK_ERROR_INITIALIZATION_FAILED;
  }
  if (cudaSetDevice(pd->cuda_device) != cudaSuccess) return VK_ERROR_INITIALIZATION_FAILED;
  Device* dev = new Device();
  dev->pd = pd;
  dev->queue.dev = dev;
  if (cudaStreamCreateWithFlags(&dev->queue.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&dev->capture_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&dev->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete dev;
    return VK_ERROR_INITIALIZATION_FAILED;
  }
  *out = to_handle<VkDevice>(dev);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyDevice(VkDevice device, const VkAllocationCallbacks*) {
  Device* dev = from_handle<Device>(device);
  if (!dev) return;
  cudaSetDevice(dev->pd->cuda_device);
  cudaStreamSynchronize(dev->queue.stream);
  for (auto& kv : dev->kernel_sets_by_ptx) {
    if (kv.second->lib) cudaLibraryUnload(kv.second->lib);
    delete kv.second;
  }
  dev->kernel_sets.clear();
  dev->kernel_sets_by_ptx.clear();
  for (cudaEvent_t e : dev->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : dev->timing_pool) cudaEventDestroy(e);
  cudaStreamDestroy(dev->queue.stream);
  cudaStreamDestroy(dev->capture_stream);
  cudaStreamDestroy(dev->copy_stream);
  delete dev;
}

static void VKAPI_CALL kzGetDeviceQueue(VkDevice device, uint32_t family, uint32_t index, VkQueue* out) {
  Device* dev = from_handle<Device>(device);
  *out = (family == 0 && index == 0) ? to_handle<VkQueue>(&dev->queue) : nullptr;
}

static VkResult VKAPI_CALL kzDeviceWaitIdle(VkDevice device) {
  Device* dev = from_handle<Device>(device);
  return queue_wait_idle(&dev->queue);
}

static VkResult VKAPI_CALL kzQueueSubmit(VkQueue queue, uint32_t count, const VkSubmitInfo* submits, VkFence fence) {
  /* api_impl.rs:3414 vkQueueSubmit */
  Queue* q = from_handle<Queue>(queue);
  return queue_submit(q, count, submits, from_handle<Fence>(fence));
}

static VkResult VKAPI_CALL kzQueueWaitIdle(VkQueue queue) {
  /* api_impl.rs:3424 vkQueueWaitIdle */
  return queue_wait_idle(from_handle<Queue>(queue));
}

/* ------------------------------------------------------------------------------------------------ */
/* memory (api_impl.rs:3434-3520, device_memory.rs)                                                 */

static VkResult VKAPI_CALL kzAllocateMemory(VkDevice device, const VkMemoryAllocateInfo* ai, const VkAllocationCallbacks*,
                                            VkDeviceMemory* out) {
  /* api_impl.rs:3434 vkAllocateMemory: size/alloc failure -> VK_ERROR_OUT_OF_DEVICE_MEMORY (:3456-3470) */
  Device* dev = from_handle<Device>(device);
  if (!ai || ai->memoryTypeIndex > 1) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  cudaSetDevice(dev->pd->cuda_device);
  DeviceMemory* m = new DeviceMemory();
  m->dev = dev;
  m->size = ai->allocationSize;
  m->type = ai->memoryTypeIndex;
  void* p = nullptr;
  VkResult r = device_alloc((size_t)ai->allocationSize, &p);
  if (r != VK_SUCCESS) {
    delete m;
    return r;
  }
  m->dptr = static_cast<char*>(p);
  *out = to_handle<VkDeviceMemory>(m);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzFreeMemory(VkDevice device, VkDeviceMemory memory, const VkAllocationCallbacks*) {
  DeviceMemory* m = from_handle<DeviceMemory>(memory);
  if (!m) return;
  Device* dev = from_handle<Device>(device);
  cudaSetDevice(dev->pd->cuda_device);
  cudaStreamSynchronize(dev->copy_stream);
  cudaStreamSynchronize(dev->queue.stream);
  device_free(m->dptr);
  if (m->host) cudaFreeHost(m->host);
  if (m->last_use) cudaEventDestroy(m->last_use);
  delete m;
}

static VkResult VKAPI_CALL kzMapMemory(VkDevice device, VkDeviceMemory memory, VkDeviceSize offset, VkDeviceSize,
                                       VkMemoryMapFlags, void** out) {
  /* api_impl.rs:3488 vkMapMemory returns the host pointer; here the pointer is a pinned host shadow of
   * the HBM allocation, kept coherent by the queue (uploaded before and downloaded after each
   * submission that uses the memory) */
  Device* dev = from_handle<Device>(device);
  DeviceMemory* m = from_handle<DeviceMemory>(memory);
  if (m->type != 0) return VK_ERROR_MEMORY_MAP_FAILED;
  cudaSetDevice(dev->pd->cuda_device);
  if (!m->host) {
    if (cudaMallocHost((void**)&m->host, (size_t)(m->size ? m->size : 16)) != cudaSuccess) {
      cudaGetLastError();
      m->host = nullptr;
      return VK_ERROR_MEMORY_MAP_FAILED;
    }
    m->device_newer = true;
  }
  if (m->device_newer) {
    cudaStreamSynchronize(dev->queue.stream);
    cudaMemcpy(m->host, m->dptr, (size_t)m->size, cudaMemcpyDeviceToHost);
    m->device_newer = false;
  }
  m->mapped = true;
  *out = m->host + offset;
  return VK_SUCCESS;
}

static void VKAPI_CALL kzUnmapMemory(VkDevice device, VkDeviceMemory memory) {
  Device* dev = from_handle<Device>(device);
  DeviceMemory* m = from_handle<DeviceMemory>(memory);
  if (!m || !m->mapped) return;
  cudaSetDevice(dev->pd->cuda_device);
  cudaMemcpyAsync(m->dptr, m->host, (size_t)m->size, cudaMemcpyHostToDevice, dev->queue.stream);
  cudaStreamSynchronize(dev->queue.stream);
  m->mapped = false;
}

static VkResult VKAPI_CALL kzFlushMappedMemoryRanges(VkDevice device, uint32_t n, const VkMappedMemoryRange* r) {
  Device* dev = from_handle<Device>(device);
  cudaSetDevice(dev->pd->cuda_device);
  for (uint32_t i = 0; i < n; i++) {
    DeviceMemory* m = from_handle<DeviceMemory>(r[i].memory);
    if (!m || !m->host) continue;
    VkDeviceSize size = r[i].size == VK_WHOLE_SIZE ? m->size - r[i].offset : r[i].size;
    cudaMemcpyAsync(m->dptr + r[i].offset, m->host + r[i].offset, (size_t)size, cudaMemcpyHostToDevice,
                    dev->queue.stream);
  }
  cudaStreamSynchronize(dev->queue.stream);
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzInvalidateMappedMemoryRanges(VkDevice device, uint32_t n, const VkMappedMemoryRange* r) {
  Device* dev = from_handle<Device>(device);
  cudaSetDevice(dev->pd->cuda_device);
  cudaStreamSynchronize(dev->queue.stream);
  for (uint32_t i = 0; i < n; i++) {
    DeviceMemory* m = from_handle<DeviceMemory>(r[i].memory);
    if (!m || !m->host) continue;
    VkDeviceSize size = r[i].size == VK_WHOLE_SIZE ? m->size - r[i].offset : r[i].size;
    cudaMemcpy(m->host + r[i].offset, m->dptr + r[i].offset, (size_t)size, cudaMemcpyDeviceToHost);
  }
  return VK_SUCCESS;
}

/* ------------------------------------------------------------------------------------------------ */
/* buffers and images (api_impl.rs:3795-3945, 4975-5190; buffer.rs; image.rs)                       */

static VkResult VKAPI_CALL kzCreateBuffer(VkDevice, const VkBufferCreateInfo* ci, const VkAllocationCallbacks*,
                                          VkBuffer* out) {
  /* api_impl.rs:3795 vkCreateBuffer */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_BUFFER_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  Buffer* b = new Buffer();
  b->size = ci->size;
  b->usage = ci->usage;
  *out = to_handle<VkBuffer>(b);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyBuffer(VkDevice, VkBuffer buffer, const VkAllocationCallbacks*) {
  delete from_handle<Buffer>(buffer);
}

static void VKAPI_CALL kzGetBufferMemoryRequirements(VkDevice, VkBuffer buffer, VkMemoryRequirements* r) {
  /* api_impl.rs:5178-5182: size rounded up to the 64-byte buffer alignment, any memory type */
  Buffer* b = from_handle<Buffer>(buffer);
  r->alignment = 64;
  r->size = (b->size + 63) & ~(VkDeviceSize)63;
  r->memoryTypeBits = 0x3u;
}

static VkResult VKAPI_CALL kzBindBufferMemory(VkDevice, VkBuffer buffer, VkDeviceMemory memory, VkDeviceSize off) {
  Buffer* b = from_handle<Buffer>(buffer);
  DeviceMemory* m = from_handle<DeviceMemory>(memory);
  if (!m || off + b->size > m->size) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  b->mem = m;
  b->offset = off;
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzBindBufferMemory2(VkDevice device, uint32_t n, const VkBindBufferMemoryInfo* infos) {
  /* api_impl.rs:4975 vkBindBufferMemory2 */
  for (uint32_t i = 0; i < n; i++) {
    VkResult r = kzBindBufferMemory(device, infos[i].buffer, infos[i].memory, infos[i].memoryOffset);
    if (r != VK_SUCCESS) return r;
  }
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzCreateImage(VkDevice, const VkImageCreateInfo* ci, const VkAllocationCallbacks*,
                                         VkImage* out) {
  /* api_impl.rs:3851 vkCreateImage; image.rs:58-87 accepts only RGBA8, 1 mip, 1 sample.  This driver adds
   * B8G8R8A8_UNORM, the two 8-bit sRGB formats (one sample) and the depth formats; both tilings are
   * row-major. */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_IMAGE_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  uint32_t bpp = format_bpp(ci->format);
  const bool ms_ok = ci->samples == VK_SAMPLE_COUNT_4_BIT && !(ci->usage & VK_IMAGE_USAGE_SAMPLED_BIT) &&
                     (ci->format == VK_FORMAT_R8G8B8A8_UNORM || ci->format == VK_FORMAT_B8G8R8A8_UNORM ||
                      ci->format == VK_FORMAT_D32_SFLOAT);
  if (ci->imageType != VK_IMAGE_TYPE_2D || !bpp || ci->mipLevels != 1 || ci->arrayLayers != 1 ||
      (ci->samples != VK_SAMPLE_COUNT_1_BIT && !ms_ok) || ci->extent.width == 0 || ci->extent.height == 0 ||
      ci->extent.width > 8192 || ci->extent.height > 8192)
    return VK_ERROR_FORMAT_NOT_SUPPORTED;
  Image* img = new Image();
  img->format = ci->format;
  img->width = ci->extent.width;
  img->height = ci->extent.height;
  img->tiling = ci->tiling;
  img->usage = ci->usage;
  img->bpp = bpp;
  img->samples = ms_ok ? KZ_MS_SAMPLES : 1u;
  /* whole 32-bit words (a D16 row is cleared two texels per word); multisampled: the samples of a pixel
   * side by side */
  img->pitch = (img->width * bpp * img->samples + 3u) & ~3u;
  img->size = (VkDeviceSize)img->pitch * img->height;
  *out = to_handle<VkImage>(img);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyImage(VkDevice, VkImage image, const VkAllocationCallbacks*) {
  delete from_handle<Image>(image);
}

static void VKAPI_CALL kzGetImageMemoryRequirements(VkDevice, VkImage image, VkMemoryRequirements* r) {
  /* api_impl.rs:5123; 256-byte alignment so that rows start on vector-load boundaries */
  Image* img = from_handle<Image>(image);
  r->alignment = 256;
  r->size = (img->size + 255) & ~(VkDeviceSize)255;
  r->memoryTypeBits = 0x3u;
}

static VkResult VKAPI_CALL kzBindImageMemory(VkDevice, VkImage image, VkDeviceMemory memory, VkDeviceSize off) {
  Image* img = from_handle<Image>(image);
  DeviceMemory* m = from_handle<DeviceMemory>(memory);
  if (!m || off + img->size > m->size || (off & 15)) return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  img->mem = m;
  img->offset = off;
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzBindImageMemory2(VkDevice device, uint32_t n, const VkBindImageMemoryInfo* infos) {
  /* api_impl.rs:5013 vkBindImageMemory2 */
  for (uint32_t i = 0; i < n; i++) {
    VkResult r = kzBindImageMemory(device, infos[i].image, infos[i].memory, infos[i].memoryOffset);
    if (r != VK_SUCCESS) return r;
  }
  return VK_SUCCESS;
}

static void VKAPI_CALL kzGetImageSubresourceLayout(VkDevice, VkImage image, const VkImageSubresource*,
                                                   VkSubresourceLayout* l) {
  /* api_impl.rs:3904 */
  Image* img = from_handle<Image>(image);
  l->offset = 0;
  l->size = img->size;
  l->rowPitch = img->pitch;
  l->arrayPitch = img->size;
  l->depthPitch = img->size;
}

static VkResult VKAPI_CALL kzCreateImageView(VkDevice, const VkImageViewCreateInfo* ci, const VkAllocationCallbacks*,
                                             VkImageView* out) {
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_IMAGE_VIEW_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  Image* img = from_handle<Image>(ci->image);
  if (ci->format != img->format) return VK_ERROR_FORMAT_NOT_SUPPORTED;
  ImageView* v = new ImageView();
  v->image = img;
  v->format = ci->format;
  *out = to_handle<VkImageView>(v);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyImageView(VkDevice, VkImageView view, const VkAllocationCallbacks*) {
  delete from_handle<ImageView>(view);
}

/* ------------------------------------------------------------------------------------------------ */
/* render pass, framebuffer (render_pass.rs, api_impl.rs:4383-4434)                                 */

static VkResult VKAPI_CALL kzCreateRenderPass(VkDevice, const VkRenderPassCreateInfo* ci, const VkAllocationCallbacks*,
                                              VkRenderPass* out) {
  /* api_impl.rs:4402 vkCreateRenderPass (the reference ignores the create info, render_pass.rs:4) */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_RENDER_PASS_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  if (ci->subpassCount != 1) return VK_ERROR_FEATURE_NOT_PRESENT;
  const VkSubpassDescription& sp = ci->pSubpasses[0];
  if (sp.colorAttachmentCount > 1 || sp.inputAttachmentCount) return VK_ERROR_FEATURE_NOT_PRESENT;
  RenderPass* rp = new RenderPass();
  rp->atts.assign(ci->pAttachments, ci->pAttachments + ci->attachmentCount);
  if (sp.colorAttachmentCount == 1 && sp.pColorAttachments[0].attachment != VK_ATTACHMENT_UNUSED)
    rp->color_att = (int)sp.pColorAttachments[0].attachment;
  if (sp.pDepthStencilAttachment && sp.pDepthStencilAttachment->attachment != VK_ATTACHMENT_UNUSED)
    rp->depth_att = (int)sp.pDepthStencilAttachment->attachment;
  if (sp.colorAttachmentCount == 1 && sp.pResolveAttachments &&
      sp.pResolveAttachments[0].attachment != VK_ATTACHMENT_UNUSED)
    rp->resolve_att = (int)sp.pResolveAttachments[0].attachment;
  *out = to_handle<VkRenderPass>(rp);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyRenderPass(VkDevice, VkRenderPass rp, const VkAllocationCallbacks*) {
  delete from_handle<RenderPass>(rp);
}

static VkResult VKAPI_CALL kzCreateFramebuffer(VkDevice, const VkFramebufferCreateInfo* ci,
                                               const VkAllocationCallbacks*, VkFramebuffer* out) {
  /* api_impl.rs:4383 vkCreateFramebuffer */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_FRAMEBUFFER_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  Framebuffer* fb = new Framebuffer();
  fb->rp = from_handle<RenderPass>(ci->renderPass);
  for (uint32_t i = 0; i < ci->attachmentCount; i++) fb->views.push_back(from_handle<ImageView>(ci->pAttachments[i]));
  fb->width = ci->width;
  fb->height = ci->height;
  *out = to_handle<VkFramebuffer>(fb);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyFramebuffer(VkDevice, VkFramebuffer fb, const VkAllocationCallbacks*) {
  delete from_handle<Framebuffer>(fb);
}

/* ------------------------------------------------------------------------------------------------ */
/* shaders and pipelines (api_impl.rs:3946-4148, pipeline.rs)                                       */

static VkResult VKAPI_CALL kzCreateShaderModule(VkDevice, const VkShaderModuleCreateInfo* ci,
                                                const VkAllocationCallbacks*, VkShaderModule* out) {
  /* api_impl.rs:3946 vkCreateShaderModule copies the SPIR-V words (shader_module.rs:3-5) */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_SHADER_MODULE_CREATE_INFO || ci->codeSize % 4 || !ci->pCode)
    return VK_ERROR_INITIALIZATION_FAILED;
  ShaderModule* sm = new ShaderModule();
  sm->code.assign(ci->pCode, ci->pCode + ci->codeSize / 4);
  *out = to_handle<VkShaderModule>(sm);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyShaderModule(VkDevice, VkShaderModule sm, const VkAllocationCallbacks*) {
  delete from_handle<ShaderModule>(sm);
}

static VkResult VKAPI_CALL kzCreatePipelineCache(VkDevice, const VkPipelineCacheCreateInfo*,
                                                 const VkAllocationCallbacks*, VkPipelineCache* out) {
  *out = to_handle<VkPipelineCache>(new PipelineCache());
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyPipelineCache(VkDevice, VkPipelineCache c, const VkAllocationCallbacks*) {
  delete from_handle<PipelineCache>(c);
}

/* ------------------------------------------------------------------------------------------------ */
/* samplers and descriptor sets (api_impl.rs:4165-4339, descriptor_set.rs, sampler.rs)               */

static VkResult VKAPI_CALL kzCreateSampler(VkDevice, const VkSamplerCreateInfo* ci, const VkAllocationCallbacks*,
                                           VkSampler* out) {
  /* api_impl.rs:4165 vkCreateSampler.  Images have one mip level, so the level of detail selects only
   * between the min and mag filters: the driver takes samplers whose two filters agree, without
   * anisotropy or depth compare */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_SAMPLER_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  if (ci->magFilter != ci->minFilter || ci->anisotropyEnable || ci->compareEnable || ci->addressModeU > 4 ||
      ci->addressModeV > 4 || ci->borderColor > 5) {
    log_error("sampler: min and mag filters must agree; anisotropy and compare are not supported");
    return VK_ERROR_FEATURE_NOT_PRESENT;
  }
  Sampler* s = new Sampler();
  s->bits = (ci->magFilter == VK_FILTER_LINEAR ? (uint32_t)KZ_SAMP_LINEAR : 0u) |
            (ci->unnormalizedCoordinates ? (uint32_t)KZ_SAMP_UNNORMALIZED : 0u) |
            ((uint32_t)ci->addressModeU << KZ_SAMP_ADDR_U_SHIFT) | ((uint32_t)ci->addressModeV << KZ_SAMP_ADDR_V_SHIFT) |
            (((uint32_t)ci->borderColor / 2u) << KZ_SAMP_BORDER_SHIFT);
  *out = to_handle<VkSampler>(s);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroySampler(VkDevice, VkSampler s, const VkAllocationCallbacks*) {
  delete from_handle<Sampler>(s);
}

static VkResult VKAPI_CALL kzCreateDescriptorSetLayout(VkDevice, const VkDescriptorSetLayoutCreateInfo* ci,
                                                       const VkAllocationCallbacks*, VkDescriptorSetLayout* out) {
  /* api_impl.rs:4218; uniform and storage buffers (plain and dynamic; storage buffers are read-only to the
   * shaders) and combined image samplers */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_DESCRIPTOR_SET_LAYOUT_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  auto info = std::make_shared<SetLayoutInfo>();
  for (uint32_t i = 0; i < ci->bindingCount; i++) {
    const VkDescriptorSetLayoutBinding& b = ci->pBindings[i];
    if (b.descriptorType != VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER &&
        b.descriptorType != VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC &&
        b.descriptorType != VK_DESCRIPTOR_TYPE_STORAGE_BUFFER &&
        b.descriptorType != VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC &&
        b.descriptorType != VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER &&
        b.descriptorType != VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE && b.descriptorType != VK_DESCRIPTOR_TYPE_SAMPLER) {
      log_error("descriptor type %d is not supported (uniform and storage buffers, samplers, sampled images and "
                "combined image samplers are)",
                (int)b.descriptorType);
      return VK_ERROR_FEATURE_NOT_PRESENT;
    }
    if (b.binding >= KZ_MAX_DESC_BINDINGS) return VK_ERROR_FEATURE_NOT_PRESENT;
    SetBinding sb;
    sb.binding = b.binding;
    sb.type = b.descriptorType;
    sb.count = b.descriptorCount;
    if ((b.descriptorType == VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER || b.descriptorType == VK_DESCRIPTOR_TYPE_SAMPLER) &&
        b.pImmutableSamplers)
      for (uint32_t k = 0; k < b.descriptorCount; k++) sb.immutable.push_back(from_handle<Sampler>(b.pImmutableSamplers[k])->bits);
    info->bindings.push_back(sb);
  }
  std::sort(info->bindings.begin(), info->bindings.end(),
            [](const SetBinding& a, const SetBinding& b) { return a.binding < b.binding; });
  for (SetBinding& b : info->bindings) {
    b.first = info->descriptors;
    info->descriptors += b.count;
    if (b.type == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC || b.type == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC)
      info->dynamic += b.count;
  }
  if (info->descriptors > KZ_MAX_DESC_SLOTS) return VK_ERROR_FEATURE_NOT_PRESENT;
  DescriptorSetLayout* l = new DescriptorSetLayout();
  l->info = info;
  *out = to_handle<VkDescriptorSetLayout>(l);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyDescriptorSetLayout(VkDevice, VkDescriptorSetLayout l, const VkAllocationCallbacks*) {
  delete from_handle<DescriptorSetLayout>(l);
}

static VkResult VKAPI_CALL kzCreateDescriptorPool(VkDevice, const VkDescriptorPoolCreateInfo* ci,
                                                  const VkAllocationCallbacks*, VkDescriptorPool* out) {
  /* api_impl.rs:4258 */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_DESCRIPTOR_POOL_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  DescriptorPool* p = new DescriptorPool();
  p->max_sets = ci->maxSets;
  *out = to_handle<VkDescriptorPool>(p);
  return VK_SUCCESS;
}

static void free_pool_sets(DescriptorPool* p) {
  for (DescriptorSet* s : p->sets) delete s;
  p->sets.clear();
}

static void VKAPI_CALL kzDestroyDescriptorPool(VkDevice, VkDescriptorPool h, const VkAllocationCallbacks*) {
  DescriptorPool* p = from_handle<DescriptorPool>(h);
  if (!p) return;
  free_pool_sets(p);
  delete p;
}

static VkResult VKAPI_CALL kzResetDescriptorPool(VkDevice, VkDescriptorPool h, VkFlags) {
  /* api_impl.rs:4282 */
  free_pool_sets(from_handle<DescriptorPool>(h));
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzAllocateDescriptorSets(VkDevice, const VkDescriptorSetAllocateInfo* ai,
                                                    VkDescriptorSet* out) {
  /* api_impl.rs:4292: every set or none */
  if (!ai || ai->sType != VK_STRUCTURE_TYPE_DESCRIPTOR_SET_ALLOCATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  DescriptorPool* p = from_handle<DescriptorPool>(ai->descriptorPool);
  if (p->sets.size() + ai->descriptorSetCount > p->max_sets) {
    for (uint32_t i = 0; i < ai->descriptorSetCount; i++) out[i] = nullptr;
    return VK_ERROR_OUT_OF_POOL_MEMORY;
  }
  for (uint32_t i = 0; i < ai->descriptorSetCount; i++) {
    DescriptorSet* s = new DescriptorSet();
    s->layout = from_handle<DescriptorSetLayout>(ai->pSetLayouts[i])->info;
    s->entries.resize(s->layout->descriptors);
    for (const SetBinding& b : s->layout->bindings)
      for (uint32_t k = 0; k < b.count && k < b.immutable.size(); k++) {
        s->entries[b.first + k].sampler = b.immutable[k];
        /* a sampler binding with immutable samplers is complete without a write */
        if (b.type == VK_DESCRIPTOR_TYPE_SAMPLER) s->entries[b.first + k].written = true;
      }
    s->pool = p;
    p->sets.push_back(s);
    out[i] = to_handle<VkDescriptorSet>(s);
  }
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzFreeDescriptorSets(VkDevice, VkDescriptorPool h, uint32_t n, const VkDescriptorSet* sets) {
  /* api_impl.rs:4326 */
  DescriptorPool* p = from_handle<DescriptorPool>(h);
  for (uint32_t i = 0; i < n; i++) {
    DescriptorSet* s = from_handle<DescriptorSet>(sets[i]);
    if (!s) continue;
    p->sets.erase(std::remove(p->sets.begin(), p->sets.end(), s), p->sets.end());
    delete s;
  }
  return VK_SUCCESS;
}

/* the descriptors [element, element + count) of `binding` and, past its end, of the following bindings
 * (array element 0 on), as vkUpdateDescriptorSets (api_impl.rs:4339-4370) walks them; calls f(entry index) */
template <class F>
static bool walk_descriptors(const SetLayoutInfo& L, uint32_t binding, uint32_t element, uint32_t count, F f) {
  size_t bi = 0;
  while (bi < L.bindings.size() && L.bindings[bi].binding != binding) bi++;
  while (count) {
    if (bi >= L.bindings.size()) return false;
    const SetBinding& b = L.bindings[bi];
    if (element >= b.count) {
      element -= b.count;
      bi++;
      continue;
    }
    uint32_t n = std::min(count, b.count - element);
    for (uint32_t k = 0; k < n; k++) f(b.first + element + k, b);
    count -= n;
    element = 0;
    bi++;
  }
  return true;
}

static void VKAPI_CALL kzUpdateDescriptorSets(VkDevice, uint32_t nw, const VkWriteDescriptorSet* writes, uint32_t nc,
                                              const VkCopyDescriptorSet* copies) {
  for (uint32_t i = 0; i < nw; i++) {
    const VkWriteDescriptorSet& w = writes[i];
    DescriptorSet* s = from_handle<DescriptorSet>(w.dstSet);
    uint32_t k = 0;
    bool ok = walk_descriptors(*s->layout, w.dstBinding, w.dstArrayElement, w.descriptorCount,
                               [&](uint32_t e, const SetBinding& b) {
                                 DescriptorEntry& d = s->entries[e];
                                 if (b.type != w.descriptorType) return;
                                 d.written = true;
                                 if (w.descriptorType == VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER ||
                                     w.descriptorType == VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE ||
                                     w.descriptorType == VK_DESCRIPTOR_TYPE_SAMPLER) {
                                   if (w.descriptorType != VK_DESCRIPTOR_TYPE_SAMPLER)
                                     d.view = from_handle<ImageView>(w.pImageInfo[k].imageView);
                                   if (w.descriptorType != VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE && b.immutable.empty())
                                     d.sampler = from_handle<Sampler>(w.pImageInfo[k].sampler)->bits;
                                 } else {
                                   d.buffer = from_handle<Buffer>(w.pBufferInfo[k].buffer);
                                   d.offset = w.pBufferInfo[k].offset;
                                   d.range = w.pBufferInfo[k].range;
                                 }
                                 k++;
                               });
    if (!ok) log_error("vkUpdateDescriptorSets: write past the last binding of the set");
  }
  for (uint32_t i = 0; i < nc; i++) {
    const VkCopyDescriptorSet& c = copies[i];
    DescriptorSet* src = from_handle<DescriptorSet>(c.srcSet);
    DescriptorSet* dst = from_handle<DescriptorSet>(c.dstSet);
    std::vector<DescriptorEntry> tmp;
    walk_descriptors(*src->layout, c.srcBinding, c.srcArrayElement, c.descriptorCount,
                     [&](uint32_t e, const SetBinding&) { tmp.push_back(src->entries[e]); });
    size_t k = 0;
    walk_descriptors(*dst->layout, c.dstBinding, c.dstArrayElement, c.descriptorCount,
                     [&](uint32_t e, const SetBinding&) {
                       if (k < tmp.size()) dst->entries[e] = tmp[k++];
                     });
  }
}

static VkResult VKAPI_CALL kzCreatePipelineLayout(VkDevice, const VkPipelineLayoutCreateInfo* ci,
                                                  const VkAllocationCallbacks*, VkPipelineLayout* out) {
  /* api_impl.rs:4061 vkCreatePipelineLayout; push_constants_size (:4076-4080) = end of the last range;
   * descriptor slots numbered set by set (sets in order, each set's descriptors in binding order) */
  if (!ci || ci->sType != VK_STRUCTURE_TYPE_PIPELINE_LAYOUT_CREATE_INFO) return VK_ERROR_INITIALIZATION_FAILED;
  if (ci->setLayoutCount > KZ_MAX_DESC_SETS) return VK_ERROR_FEATURE_NOT_PRESENT;
  auto info = std::make_shared<PipelineLayoutInfo>();
  for (uint32_t i = 0; i < ci->setLayoutCount; i++) {
    info->slot_base[i] = info->slots;
    info->sets.push_back(from_handle<DescriptorSetLayout>(ci->pSetLayouts[i])->info);
    info->slots += info->sets.back()->descriptors;
  }
  if (info->slots > KZ_MAX_DESC_SLOTS) return VK_ERROR_FEATURE_NOT_PRESENT;
  PipelineLayout* l = new PipelineLayout();
  if (info->slots) l->info = info;
  for (uint32_t i = 0; i < ci->pushConstantRangeCount; i++) {
    uint32_t end = ci->pPushConstantRanges[i].offset + ci->pPushConstantRanges[i].size;
    if (end > l->push_size) l->push_size = end;
  }
  if (l->push_size > KZ_PUSH_BYTES) {
    delete l;
    return VK_ERROR_FEATURE_NOT_PRESENT;
  }
  *out = to_handle<VkPipelineLayout>(l);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyPipelineLayout(VkDevice, VkPipelineLayout l, const VkAllocationCallbacks*) {
  delete from_handle<PipelineLayout>(l);
}

static uint64_t g_pipeline_uid = 1;

static VkResult compile_stage(const VkPipelineShaderStageCreateInfo& st, ir::Stage stage,
                              std::shared_ptr<ir::Shader>& out) {
  ShaderModule* sm = from_handle<ShaderModule>(st.module);
  std::vector<std::pair<uint32_t, uint32_t>> spec;
  if (st.pSpecializationInfo) {
    const VkSpecializationInfo* si = st.pSpecializationInfo;
    for (uint32_t i = 0; i < si->mapEntryCount; i++) {
      const VkSpecializationMapEntry& e = si->pMapEntries[i];
      uint32_t v = 0;
      std::memcpy(&v, static_cast<const char*>(si->pData) + e.offset, e.size < 4 ? e.size : 4);
      spec.push_back({e.constantID, v});
    }
  }
  out = std::make_shared<ir::Shader>();
  std::string err = ir::translate_spirv(sm->code.data(), sm->code.size(), stage, st.pName, spec, *out);
  if (!err.empty()) {
    log_error("shader compile failed: %s", err.c_str());
    return VK_ERROR_INVALID_SHADER_NV;
  }
  return VK_SUCCESS;
}

static VkResult create_graphics_pipeline(const VkGraphicsPipelineCreateInfo& ci, Pipeline** out) {
  /* pipeline.rs:165-183 GraphicsPipeline::create collects the vertex and fragment stages and stops at
   * `unimplemented!()`; this builds the full pipeline state */
  Pipeline* p = new Pipeline();
  p->uid = __atomic_fetch_add(&g_pipeline_uid, 1, __ATOMIC_RELAXED);
  KzPipe& kp = p->pipe;
  std::memset(&kp, 0, sizeof kp);
  VkResult r = VK_SUCCESS;
  for (uint32_t i = 0; i < ci.stageCount && r == VK_SUCCESS; i++) {
    const VkPipelineShaderStageCreateInfo& st = ci.pStages[i];
    if (st.stage == VK_SHADER_STAGE_VERTEX_BIT) r = compile_stage(st, ir::Stage::Vertex, p->vs);
    else if (st.stage == VK_SHADER_STAGE_FRAGMENT_BIT) r = compile_stage(st, ir::Stage::Fragment, p->fs);
    else r = VK_ERROR_FEATURE_NOT_PRESENT;
  }
  if (r == VK_SUCCESS && !p->vs) r = VK_ERROR_INITIALIZATION_FAILED;
  if (r != VK_SUCCESS) {
    delete p;
    return r;
  }
  /* vertex input */
  if (ci.pVertexInputState) {
    const VkPipelineVertexInputStateCreateInfo& vi = *ci.pVertexInputState;
    for (uint32_t i = 0; i < vi.vertexBindingDescriptionCount; i++) {
      const VkVertexInputBindingDescription& b = vi.pVertexBindingDescriptions[i];
      if (b.binding >= KZ_MAX_BINDINGS) r = VK_ERROR_FEATURE_NOT_PRESENT;
      else {
        kp.binding_stride[b.binding] = b.stride;
        if (b.inputRate == VK_VERTEX_INPUT_RATE_INSTANCE) kp.binding_instanced |= 1u << b.binding;
      }
    }
    for (uint32_t i = 0; i < vi.vertexAttributeDescriptionCount && r == VK_SUCCESS; i++) {
      const VkVertexInputAttributeDescription& a = vi.pVertexAttributeDescriptions[i];
      uint32_t f = attr_format(a.format);
      if (a.location >= KZ_MAX_VS_INPUTS || a.binding >= KZ_MAX_BINDINGS || f == KZ_FMT_NONE ||
          kp.num_attrs >= KZ_MAX_VS_INPUTS) {
        r = VK_ERROR_FORMAT_NOT_SUPPORTED;
        break;
      }
      KzAttr& at = kp.attrs[kp.num_attrs++];
      at.location = a.location;
      at.binding = a.binding;
      at.format = f;
      at.offset = a.offset;
    }
  }
  if (ci.pInputAssemblyState && ci.pInputAssemblyState->topology != VK_PRIMITIVE_TOPOLOGY_TRIANGLE_LIST)
    r = VK_ERROR_FEATURE_NOT_PRESENT;
  if (ci.pDynamicState)
    for (uint32_t i = 0; i < ci.pDynamicState->dynamicStateCount; i++) {
      VkDynamicState d = ci.pDynamicState->pDynamicStates[i];
      if (d == VK_DYNAMIC_STATE_VIEWPORT) p->dyn_viewport = true;
      if (d == VK_DYNAMIC_STATE_SCISSOR) p->dyn_scissor = true;
      if (d == VK_DYNAMIC_STATE_BLEND_CONSTANTS) p->dyn_blend = true;
      if (d == VK_DYNAMIC_STATE_STENCIL_COMPARE_MASK) p->dyn_stencil |= 1u;
      if (d == VK_DYNAMIC_STATE_STENCIL_WRITE_MASK) p->dyn_stencil |= 2u;
      if (d == VK_DYNAMIC_STATE_STENCIL_REFERENCE) p->dyn_stencil |= 4u;
    }
  if (ci.pViewportState) {
    if (!p->dyn_viewport && ci.pViewportState->pViewports) p->viewport = ci.pViewportState->pViewports[0];
    if (!p->dyn_scissor && ci.pViewportState->pScissors) p->scissor = ci.pViewportState->pScissors[0];
  }
  kp.front_ccw = 1;
  if (ci.pRasterizationState) {
    const VkPipelineRasterizationStateCreateInfo& rs = *ci.pRasterizationState;
    if (rs.polygonMode != VK_POLYGON_MODE_FILL || rs.depthBiasEnable) r = VK_ERROR_FEATURE_NOT_PRESENT;
    kp.cull_mode = rs.cullMode;
    kp.front_ccw = rs.frontFace == VK_FRONT_FACE_COUNTER_CLOCKWISE;
    p->rasterizer_discard = rs.rasterizerDiscardEnable != 0;
  }
  if (ci.pMultisampleState) {
    /* 1 or 4 samples; per-sample shading, alpha to coverage / one and sample masks are not supported */
    const VkPipelineMultisampleStateCreateInfo& ms = *ci.pMultisampleState;
    if ((ms.rasterizationSamples != VK_SAMPLE_COUNT_1_BIT && ms.rasterizationSamples != VK_SAMPLE_COUNT_4_BIT) ||
        ms.sampleShadingEnable || ms.alphaToCoverageEnable || ms.alphaToOneEnable ||
        (ms.pSampleMask && (ms.pSampleMask[0] & 0xFu) != 0xFu))
      r = VK_ERROR_FEATURE_NOT_PRESENT;
  }
  if (ci.pDepthStencilState) {
    const VkPipelineDepthStencilStateCreateInfo& ds = *ci.pDepthStencilState;
    if (ds.depthBoundsTestEnable) r = VK_ERROR_FEATURE_NOT_PRESENT;
    if (ds.stencilTestEnable) {
      kp.stencil_test = 1;
      const VkStencilOpState* faces[2] = {&ds.front, &ds.back};
      for (int f = 0; f < 2; f++) {
        const VkStencilOpState& so = *faces[f];
        kp.stencil[2 * f] = (uint32_t)so.failOp | ((uint32_t)so.passOp << 3) | ((uint32_t)so.depthFailOp << 6) |
                            ((uint32_t)so.compareOp << 9);
        kp.stencil[2 * f + 1] = (so.compareMask & 0xFFu) | ((so.writeMask & 0xFFu) << 8) | ((so.reference & 0xFFu) << 16);
      }
    }
    kp.depth_test = ds.depthTestEnable;
    kp.depth_write = ds.depthWriteEnable;
    kp.depth_compare = ds.depthCompareOp;
  }
  kp.write_mask = 0xF;
  if (ci.pColorBlendState) {
    const VkPipelineColorBlendStateCreateInfo& cb = *ci.pColorBlendState;
    if (cb.logicOpEnable) r = VK_ERROR_FEATURE_NOT_PRESENT;
    if (cb.attachmentCount >= 1) {
      const VkPipelineColorBlendAttachmentState& a = cb.pAttachments[0];
      kp.blend_enable = a.blendEnable;
      kp.src_color = a.srcColorBlendFactor;
      kp.dst_color = a.dstColorBlendFactor;
      kp.color_op = a.colorBlendOp;
      kp.src_alpha = a.srcAlphaBlendFactor;
      kp.dst_alpha = a.dstAlphaBlendFactor;
      kp.alpha_op = a.alphaBlendOp;
      kp.write_mask = a.colorWriteMask;
    }
    for (int k = 0; k < 4; k++) kp.blend_const[k] = cb.blendConstants[k];
  }
  /* descriptor bindings the stages declare: each must be in the layout with a matching type and at least
   * as many array elements */
  PipelineLayout* pl = from_handle<PipelineLayout>(ci.layout);
  if (pl) p->layout = pl->info;
  for (const ir::Shader* sh : {p->vs.get(), p->fs.get()}) {
    if (!sh) continue;
    for (const ir::Interface::Binding& b : sh->iface.bindings) {
      const SetBinding* sb = p->layout && b.set < p->layout->sets.size() ? p->layout->sets[b.set]->find(b.binding)
                                                                         : nullptr;
      bool ok = sb && sb->count >= b.count &&
                (b.kind == 1   ? sb->type == VK_DESCRIPTOR_TYPE_COMBINED_IMAGE_SAMPLER
                 : b.kind == 3 ? sb->type == VK_DESCRIPTOR_TYPE_SAMPLED_IMAGE
                 : b.kind == 4 ? sb->type == VK_DESCRIPTOR_TYPE_SAMPLER
                 : b.kind == 2 ? (sb->type == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER ||
                                  sb->type == VK_DESCRIPTOR_TYPE_STORAGE_BUFFER_DYNAMIC)
                               : (sb->type == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER ||
                                  sb->type == VK_DESCRIPTOR_TYPE_UNIFORM_BUFFER_DYNAMIC));
      if (!ok) {
        log_error("pipeline: set %u binding %u of the shaders is missing from the pipeline layout or has another type",
                  b.set, b.binding);
        r = VK_ERROR_INITIALIZATION_FAILED;
      }
      p->bindings.push_back(b);
    }
  }
  /* interface between the stages */
  const ir::Interface& vif = p->vs->iface;
  kp.pos_input_mask = vif.pos_input_locations;
  kp.full_input_mask = vif.input_locations;
  if (p->fs) {
    const ir::Interface& fif = p->fs->iface;
    uint32_t slots = fif.input_slots, n = 0;
    while (slots >> n) n++;
    kp.num_varyings = n;
    kp.flat_mask = fif.flat_slots;
    kp.noperspective_mask = fif.noperspective_slots;
    kp.fs_discards = fif.discards;
    kp.fs_passthrough = ir::color_passthrough(p->fs->fn) ? 1u : 0u;
    kp.has_fs = 1;
    if (!fif.writes_color) kp.write_mask = 0;
  }
  if (r != VK_SUCCESS) {
    delete p;
    return r;
  }
  /* order-independent visibility resolve: no blending, no discard, and a depth rule that the
   * (depth, primitive) key reproduces */
  if (!kp.blend_enable && !kp.fs_discards && !kp.stencil_test) {
    if (!kp.depth_test) p->vis_key = KZ_VIS_LAST;
    else if (kp.depth_write) {
      switch (kp.depth_compare) {
        case VK_COMPARE_OP_LESS: p->vis_key = KZ_VIS_LESS; break;
        case VK_COMPARE_OP_LESS_OR_EQUAL: p->vis_key = KZ_VIS_LEQUAL; break;
        case VK_COMPARE_OP_GREATER: p->vis_key = KZ_VIS_GREATER; break;
        case VK_COMPARE_OP_GREATER_OR_EQUAL: p->vis_key = KZ_VIS_GEQUAL; break;
        default: break;
      }
    }
  }
  *out = p;
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzCreateGraphicsPipelines(VkDevice, VkPipelineCache, uint32_t n,
                                                     const VkGraphicsPipelineCreateInfo* cis,
                                                     const VkAllocationCallbacks*, VkPipeline* out) {
  /* api_impl.rs:4018 vkCreateGraphicsPipelines -> pipeline.rs:205-219 create_pipelines */
  VkResult result = VK_SUCCESS;
  for (uint32_t i = 0; i < n; i++) {
    Pipeline* p = nullptr;
    VkResult r = create_graphics_pipeline(cis[i], &p);
    out[i] = r == VK_SUCCESS ? to_handle<VkPipeline>(p) : nullptr;
    if (r != VK_SUCCESS) result = r;
  }
  return result;
}

static void VKAPI_CALL kzDestroyPipeline(VkDevice, VkPipeline p, const VkAllocationCallbacks*) {
  delete from_handle<Pipeline>(p);
}

/* ------------------------------------------------------------------------------------------------ */
/* fences and semaphores (api_impl.rs:3653-3720)                                                    */

static VkResult VKAPI_CALL kzCreateFence(VkDevice device, const VkFenceCreateInfo* ci, const VkAllocationCallbacks*,
                                         VkFence* out) {
  /* api_impl.rs:3653 vkCreateFence */
  Device* dev = from_handle<Device>(device);
  cudaSetDevice(dev->pd->cuda_device);
  Fence* f = new Fence();
  if (cudaEventCreateWithFlags(&f->ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    delete f;
    return VK_ERROR_OUT_OF_DEVICE_MEMORY;
  }
  f->signaled = ci && (ci->flags & VK_FENCE_CREATE_SIGNALED_BIT);
  *out = to_handle<VkFence>(f);
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroyFence(VkDevice, VkFence fence, const VkAllocationCallbacks*) {
  Fence* f = from_handle<Fence>(fence);
  if (!f) return;
  if (f->pending) cudaEventSynchronize(f->ev);
  cudaEventDestroy(f->ev);
  delete f;
}

static VkResult VKAPI_CALL kzResetFences(VkDevice, uint32_t n, const VkFence* fences) {
  for (uint32_t i = 0; i < n; i++) {
    Fence* f = from_handle<Fence>(fences[i]);
    f->signaled = false;
    f->error = VK_SUCCESS;
  }
  return VK_SUCCESS;
}

static VkResult VKAPI_CALL kzGetFenceStatus(VkDevice device, VkFence fence) {
  return fence_status(from_handle<Device>(device), from_handle<Fence>(fence));
}

static VkResult VKAPI_CALL kzWaitForFences(VkDevice device, uint32_t n, const VkFence* fences, VkBool32 all,
                                           uint64_t timeout) {
  /* api_impl.rs:3689 vkWaitForFences */
  return wait_fences(from_handle<Device>(device), n, fences, all, timeout);
}

static VkResult VKAPI_CALL kzCreateSemaphore(VkDevice, const VkSemaphoreCreateInfo*, const VkAllocationCallbacks*,
                                             VkSemaphore* out) {
  /* one in-order queue: semaphores order nothing the CUDA stream does not already order */
  *out = to_handle<VkSemaphore>(new Semaphore());
  return VK_SUCCESS;
}

static void VKAPI_CALL kzDestroySemaphore(VkDevice, VkSemaphore s, const VkAllocationCallbacks*) {
  delete from_handle<Semaphore>(s);
}

/* command-buffer functions live in kz_cmd.cpp */
extern "C" {
VkResult VKAPI_CALL kzCreateCommandPool(VkDevice, const VkCommandPoolCreateInfo*, const VkAllocationCallbacks*,
                                        VkCommandPool*);
void VKAPI_CALL kzDestroyCommandPool(VkDevice, VkCommandPool, const VkAllocationCallbacks*);
VkResult VKAPI_CALL kzResetCommandPool(VkDevice, VkCommandPool, VkCommandPoolResetFlags);
VkResult VKAPI_CALL kzAllocateCommandBuffers(VkDevice, const VkCommandBufferAllocateInfo*, VkCommandBuffer*);
void VKAPI_CALL kzFreeCommandBuffers(VkDevice, VkCommandPool, uint32_t, const VkCommandBuffer*);
VkResult VKAPI_CALL kzBeginCommandBuffer(VkCommandBuffer, const VkCommandBufferBeginInfo*);
VkResult VKAPI_CALL kzEndCommandBuffer(VkCommandBuffer);
VkResult VKAPI_CALL kzResetCommandBuffer(VkCommandBuffer, VkCommandBufferResetFlags);
void VKAPI_CALL kzCmdBindPipeline(VkCommandBuffer, VkPipelineBindPoint, VkPipeline);
void VKAPI_CALL kzCmdSetViewport(VkCommandBuffer, uint32_t, uint32_t, const VkViewport*);
void VKAPI_CALL kzCmdSetScissor(VkCommandBuffer, uint32_t, uint32_t, const VkRect2D*);
void VKAPI_CALL kzCmdSetBlendConstants(VkCommandBuffer, const float[4]);
void VKAPI_CALL kzCmdBindVertexBuffers(VkCommandBuffer, uint32_t, uint32_t, const VkBuffer*, const VkDeviceSize*);
void VKAPI_CALL kzCmdBindIndexBuffer(VkCommandBuffer, VkBuffer, VkDeviceSize, VkIndexType);
void VKAPI_CALL kzCmdPushConstants(VkCommandBuffer, VkPipelineLayout, VkShaderStageFlags, uint32_t, uint32_t,
                                   const void*);
void VKAPI_CALL kzCmdDraw(VkCommandBuffer, uint32_t, uint32_t, uint32_t, uint32_t);
void VKAPI_CALL kzCmdDrawIndirect(VkCommandBuffer, VkBuffer, VkDeviceSize, uint32_t, uint32_t);
void VKAPI_CALL kzCmdResolveImage(VkCommandBuffer, VkImage, VkImageLayout, VkImage, VkImageLayout, uint32_t,
                                  const VkImageResolve*);
void VKAPI_CALL kzCmdBindDescriptorSets(VkCommandBuffer, VkPipelineBindPoint, VkPipelineLayout, uint32_t, uint32_t,
                                        const VkDescriptorSet*, uint32_t, const uint32_t*);
void VKAPI_CALL kzCmdDrawIndexedIndirect(VkCommandBuffer, VkBuffer, VkDeviceSize, uint32_t, uint32_t);
void VKAPI_CALL kzCmdDrawIndirectCount(VkCommandBuffer, VkBuffer, VkDeviceSize, VkBuffer, VkDeviceSize, uint32_t,
                                       uint32_t);
void VKAPI_CALL kzCmdDrawIndexedIndirectCount(VkCommandBuffer, VkBuffer, VkDeviceSize, VkBuffer, VkDeviceSize,
                                              uint32_t, uint32_t);
void VKAPI_CALL kzCmdDrawIndexed(VkCommandBuffer, uint32_t, uint32_t, uint32_t, int32_t, uint32_t);
void VKAPI_CALL kzCmdBeginRenderPass(VkCommandBuffer, const VkRenderPassBeginInfo*, VkSubpassContents);
void VKAPI_CALL kzCmdEndRenderPass(VkCommandBuffer);
void VKAPI_CALL kzCmdClearColorImage(VkCommandBuffer, VkImage, VkImageLayout, const VkClearColorValue*, uint32_t,
                                     const VkImageSubresourceRange*);
void VKAPI_CALL kzCmdClearDepthStencilImage(VkCommandBuffer, VkImage, VkImageLayout, const VkClearDepthStencilValue*,
                                            uint32_t, const VkImageSubresourceRange*);
void VKAPI_CALL kzCmdPipelineBarrier(VkCommandBuffer, VkPipelineStageFlags, VkPipelineStageFlags, VkDependencyFlags,
                                     uint32_t, const VkMemoryBarrier*, uint32_t, const VkBufferMemoryBarrier*,
                                     uint32_t, const VkImageMemoryBarrier*);
void VKAPI_CALL kzCmdCopyBuffer(VkCommandBuffer, VkBuffer, VkBuffer, uint32_t, const VkBufferCopy*);
void VKAPI_CALL kzCmdCopyImageToBuffer(VkCommandBuffer, VkImage, VkImageLayout, VkBuffer, uint32_t,
                                       const VkBufferImageCopy*);
void VKAPI_CALL kzCmdCopyBufferToImage(VkCommandBuffer, VkBuffer, VkImage, VkImageLayout, uint32_t,
                                       const VkBufferImageCopy*);
void VKAPI_CALL kzCmdFillBuffer(VkCommandBuffer, VkBuffer, VkDeviceSize, VkDeviceSize, uint32_t);
void VKAPI_CALL kzCmdUpdateBuffer(VkCommandBuffer, VkBuffer, VkDeviceSize, VkDeviceSize, const void*);
void VKAPI_CALL kzCmdCopyImage(VkCommandBuffer, VkImage, VkImageLayout, VkImage, VkImageLayout, uint32_t,
                               const VkImageCopy*);
void VKAPI_CALL kzCmdClearAttachments(VkCommandBuffer, uint32_t, const VkClearAttachment*, uint32_t,
                                      const VkClearRect*);
void VKAPI_CALL kzCmdSetStencilCompareMask(VkCommandBuffer, VkFlags, uint32_t);
void VKAPI_CALL kzCmdSetStencilWriteMask(VkCommandBuffer, VkFlags, uint32_t);
void VKAPI_CALL kzCmdSetStencilReference(VkCommandBuffer, VkFlags, uint32_t);
}

/* ------------------------------------------------------------------------------------------------ */
/* dispatch (api_impl.rs:432-860 get_proc_address)                                                   */

struct ProcEntry {
  const char* name;
  PFN_vkVoidFunction fn;
};

#define KZ_PROC(name, fn) {name, reinterpret_cast<PFN_vkVoidFunction>(fn)}

static PFN_vkVoidFunction VKAPI_CALL kzGetInstanceProcAddr(VkInstance, const char* name);
static PFN_vkVoidFunction VKAPI_CALL kzGetDeviceProcAddr(VkDevice, const char* name);

static const ProcEntry kProcs[] = {
    KZ_PROC("vkGetInstanceProcAddr", kzGetInstanceProcAddr),
    KZ_PROC("vkGetDeviceProcAddr", kzGetDeviceProcAddr),
    KZ_PROC("vkCreateInstance", kzCreateInstance),
    KZ_PROC("vkDestroyInstance", kzDestroyInstance),
    KZ_PROC("vkEnumerateInstanceVersion", kzEnumerateInstanceVersion),
    KZ_PROC("vkEnumerateInstanceExtensionProperties", kzEnumerateInstanceExtensionProperties),
    KZ_PROC("vkEnumerateInstanceLayerProperties", kzEnumerateInstanceLayerProperties),
    KZ_PROC("vkEnumeratePhysicalDevices", kzEnumeratePhysicalDevices),
    KZ_PROC("vkGetPhysicalDeviceProperties", kzGetPhysicalDeviceProperties),
    KZ_PROC("vkGetPhysicalDeviceFeatures", kzGetPhysicalDeviceFeatures),
    KZ_PROC("vkGetPhysicalDeviceQueueFamilyProperties", kzGetPhysicalDeviceQueueFamilyProperties),
    KZ_PROC("vkGetPhysicalDeviceMemoryProperties", kzGetPhysicalDeviceMemoryProperties),
    KZ_PROC("vkGetPhysicalDeviceFormatProperties", kzGetPhysicalDeviceFormatProperties),
    KZ_PROC("vkGetPhysicalDeviceImageFormatProperties", kzGetPhysicalDeviceImageFormatProperties),
    KZ_PROC("vkEnumerateDeviceExtensionProperties", kzEnumerateDeviceExtensionProperties),
    KZ_PROC("vkEnumerateDeviceLayerProperties", kzEnumerateDeviceLayerProperties),
    KZ_PROC("vkCreateDevice", kzCreateDevice),
    KZ_PROC("vkDestroyDevice", kzDestroyDevice),
    KZ_PROC("vkGetDeviceQueue", kzGetDeviceQueue),
    KZ_PROC("vkDeviceWaitIdle", kzDeviceWaitIdle),
    KZ_PROC("vkQueueSubmit", kzQueueSubmit),
    KZ_PROC("vkQueueWaitIdle", kzQueueWaitIdle),
    KZ_PROC("vkAllocateMemory", kzAllocateMemory),
    KZ_PROC("vkFreeMemory", kzFreeMemory),
    KZ_PROC("vkMapMemory", kzMapMemory),
    KZ_PROC("vkUnmapMemory", kzUnmapMemory),
    KZ_PROC("vkFlushMappedMemoryRanges", kzFlushMappedMemoryRanges),
    KZ_PROC("vkInvalidateMappedMemoryRanges", kzInvalidateMappedMemoryRanges),
    KZ_PROC("vkCreateBuffer", kzCreateBuffer),
    KZ_PROC("vkDestroyBuffer", kzDestroyBuffer),
    KZ_PROC("vkGetBufferMemoryRequirements", kzGetBufferMemoryRequirements),
    KZ_PROC("vkBindBufferMemory", kzBindBufferMemory),
    KZ_PROC("vkBindBufferMemory2", kzBindBufferMemory2),
    KZ_PROC("vkBindBufferMemory2KHR", kzBindBufferMemory2),
    KZ_PROC("vkCreateImage", kzCreateImage),
    KZ_PROC("vkDestroyImage", kzDestroyImage),
    KZ_PROC("vkGetImageMemoryRequirements", kzGetImageMemoryRequirements),
    KZ_PROC("vkBindImageMemory", kzBindImageMemory),
    KZ_PROC("vkBindImageMemory2", kzBindImageMemory2),
    KZ_PROC("vkBindImageMemory2KHR", kzBindImageMemory2),
    KZ_PROC("vkGetImageSubresourceLayout", kzGetImageSubresourceLayout),
    KZ_PROC("vkCreateImageView", kzCreateImageView),
    KZ_PROC("vkDestroyImageView", kzDestroyImageView),
    KZ_PROC("vkCreateRenderPass", kzCreateRenderPass),
    KZ_PROC("vkDestroyRenderPass", kzDestroyRenderPass),
    KZ_PROC("vkCreateFramebuffer", kzCreateFramebuffer),
    KZ_PROC("vkDestroyFramebuffer", kzDestroyFramebuffer),
    KZ_PROC("vkCreateShaderModule", kzCreateShaderModule),
    KZ_PROC("vkDestroyShaderModule", kzDestroyShaderModule),
    KZ_PROC("vkCreatePipelineCache", kzCreatePipelineCache),
    KZ_PROC("vkDestroyPipelineCache", kzDestroyPipelineCache),
    KZ_PROC("vkCreatePipelineLayout", kzCreatePipelineLayout),
    KZ_PROC("vkCreateSampler", kzCreateSampler),
    KZ_PROC("vkDestroySampler", kzDestroySampler),
    KZ_PROC("vkCreateDescriptorSetLayout", kzCreateDescriptorSetLayout),
    KZ_PROC("vkDestroyDescriptorSetLayout", kzDestroyDescriptorSetLayout),
    KZ_PROC("vkCreateDescriptorPool", kzCreateDescriptorPool),
    KZ_PROC("vkDestroyDescriptorPool", kzDestroyDescriptorPool),
    KZ_PROC("vkResetDescriptorPool", kzResetDescriptorPool),
    KZ_PROC("vkAllocateDescriptorSets", kzAllocateDescriptorSets),
    KZ_PROC("vkFreeDescriptorSets", kzFreeDescriptorSets),
    KZ_PROC("vkUpdateDescriptorSets", kzUpdateDescriptorSets),
    KZ_PROC("vkCmdBindDescriptorSets", kzCmdBindDescriptorSets),
    KZ_PROC("vkDestroyPipelineLayout", kzDestroyPipelineLayout),
    KZ_PROC("vkCreateGraphicsPipelines", kzCreateGraphicsPipelines),
    KZ_PROC("vkDestroyPipeline", kzDestroyPipeline),
    KZ_PROC("vkCreateFence", kzCreateFence),
    KZ_PROC("vkDestroyFence", kzDestroyFence),
    KZ_PROC("vkResetFences", kzResetFences),
    KZ_PROC("vkGetFenceStatus", kzGetFenceStatus),
    KZ_PROC("vkWaitForFences", kzWaitForFences),
    KZ_PROC("vkCreateSemaphore", kzCreateSemaphore),
    KZ_PROC("vkDestroySemaphore", kzDestroySemaphore),
    KZ_PROC("vkCreateCommandPool", kzCreateCommandPool),
    KZ_PROC("vkDestroyCommandPool", kzDestroyCommandPool),
    KZ_PROC("vkResetCommandPool", kzResetCommandPool),
    KZ_PROC("vkAllocateCommandBuffers", kzAllocateCommandBuffers),
    KZ_PROC("vkFreeCommandBuffers", kzFreeCommandBuffers),
    KZ_PROC("vkBeginCommandBuffer", kzBeginCommandBuffer),
    KZ_PROC("vkEndCommandBuffer", kzEndCommandBuffer),
    KZ_PROC("vkResetCommandBuffer", kzResetCommandBuffer),
    KZ_PROC("vkCmdBindPipeline", kzCmdBindPipeline),
    KZ_PROC("vkCmdSetViewport", kzCmdSetViewport),
    KZ_PROC("vkCmdSetScissor", kzCmdSetScissor),
    KZ_PROC("vkCmdSetBlendConstants", kzCmdSetBlendConstants),
    KZ_PROC("vkCmdBindVertexBuffers", kzCmdBindVertexBuffers),
    KZ_PROC("vkCmdBindIndexBuffer", kzCmdBindIndexBuffer),
    KZ_PROC("vkCmdPushConstants", kzCmdPushConstants),
    KZ_PROC("vkCmdDraw", kzCmdDraw),
    KZ_PROC("vkCmdDrawIndirect", kzCmdDrawIndirect),
    KZ_PROC("vkCmdResolveImage", kzCmdResolveImage),
    KZ_PROC("vkCmdDrawIndexedIndirect", kzCmdDrawIndexedIndirect),
    KZ_PROC("vkCmdDrawIndirectCountKHR", kzCmdDrawIndirectCount),
    KZ_PROC("vkCmdDrawIndexedIndirectCountKHR", kzCmdDrawIndexedIndirectCount),
    KZ_PROC("vkCmdDrawIndirectCount", kzCmdDrawIndirectCount),
    KZ_PROC("vkCmdDrawIndexedIndirectCount", kzCmdDrawIndexedIndirectCount),
    KZ_PROC("vkCmdDrawIndexed", kzCmdDrawIndexed),
    KZ_PROC("vkCmdBeginRenderPass", kzCmdBeginRenderPass),
    KZ_PROC("vkCmdEndRenderPass", kzCmdEndRenderPass),
    KZ_PROC("vkCmdClearColorImage", kzCmdClearColorImage),
    KZ_PROC("vkCmdClearDepthStencilImage", kzCmdClearDepthStencilImage),
    KZ_PROC("vkCmdPipelineBarrier", kzCmdPipelineBarrier),
    KZ_PROC("vkCmdCopyBuffer", kzCmdCopyBuffer),
    KZ_PROC("vkCmdCopyImageToBuffer", kzCmdCopyImageToBuffer),
    KZ_PROC("vkCmdCopyBufferToImage", kzCmdCopyBufferToImage),
    KZ_PROC("vkCmdFillBuffer", kzCmdFillBuffer),
    KZ_PROC("vkCmdUpdateBuffer", kzCmdUpdateBuffer),
    KZ_PROC("vkCmdCopyImage", kzCmdCopyImage),
    KZ_PROC("vkCmdClearAttachments", kzCmdClearAttachments),
    KZ_PROC("vkCmdSetStencilCompareMask", kzCmdSetStencilCompareMask),
    KZ_PROC("vkCmdSetStencilWriteMask", kzCmdSetStencilWriteMask),
    KZ_PROC("vkCmdSetStencilReference", kzCmdSetStencilReference),
    KZ_PROC("vkCmdDrawIndirectCountAMD", kzCmdDrawIndirectCount),
    KZ_PROC("vkCmdDrawIndexedIndirectCountAMD", kzCmdDrawIndexedIndirectCount),
};

static PFN_vkVoidFunction lookup(const char* name) {
  if (!name) return nullptr;
  for (const ProcEntry& e : kProcs)
    if (!std::strcmp(e.name, name)) return e.fn;
  return nullptr;
}

static PFN_vkVoidFunction VKAPI_CALL kzGetInstanceProcAddr(VkInstance, const char* name) { return lookup(name); }
static PFN_vkVoidFunction VKAPI_CALL kzGetDeviceProcAddr(VkDevice, const char* name) { return lookup(name); }

}  // namespace kz

/* ------------------------------------------------------------------------------------------------ */
/* exported loader interface (vulkan-driver/src/lib.rs:38-130)                                      */

extern "C" KZ_API PFN_vkVoidFunction vk_icdGetInstanceProcAddr(VkInstance instance, const char* name) {
  return kz::kzGetInstanceProcAddr(instance, name);
}

extern "C" KZ_API VkResult vk_icdNegotiateLoaderICDInterfaceVersion(uint32_t* supported) {
  /* lib.rs:51-63: clamp to interface version 5 */
  if (*supported > 5u) *supported = 5u;
  return VK_SUCCESS;
}

extern "C" KZ_API PFN_vkVoidFunction vk_icdGetPhysicalDeviceProcAddr(VkInstance instance, const char* name) {
  /* lib.rs:68-130: only physical-device-level functions */
  static const char* kPhys[] = {"vkCreateDevice",
                                "vkEnumerateDeviceExtensionProperties",
                                "vkEnumerateDeviceLayerProperties",
                                "vkGetPhysicalDeviceFeatures",
                                "vkGetPhysicalDeviceFormatProperties",
                                "vkGetPhysicalDeviceImageFormatProperties",
                                "vkGetPhysicalDeviceMemoryProperties",
                                "vkGetPhysicalDeviceProperties",
                                "vkGetPhysicalDeviceQueueFamilyProperties"};
  if (!name) return nullptr;
  for (const char* n : kPhys)
    if (!std::strcmp(n, name)) return kz::kzGetInstanceProcAddr(instance, name);
  return nullptr;
}

extern "C" KZ_API int kzDriverSetOption(const char* key, const char* value) {
  kz::Options& o = kz::options();
  if (!key || !value) return -1;
  if (!std::strcmp(key, "mode")) {
    if (!std::strcmp(value, "persistent")) o.mode = 0;
    else if (!std::strcmp(value, "batched")) o.mode = 1;
    else if (!std::strcmp(value, "perdraw")) o.mode = 2;
    else return -1;
    return 0;
  }
  if (!std::strcmp(key, "tile")) {
    uint32_t t = (uint32_t)std::atoi(value);
    if (t != 8 && t != 16 && t != 32 && t != 64) return -1;
    o.tile = t;
    return 0;
  }
  if (!std::strcmp(key, "trace")) {
    o.trace = std::atoi(value);
    return 0;
  }
  if (!std::strcmp(key, "kernel_timing")) {
    if (std::strcmp(value, "0") && std::strcmp(value, "1")) return -1;
    o.kernel_timing = value[0] == '1';
    return 0;
  }
  if (!std::strcmp(key, "pdl")) {
    if (std::strcmp(value, "0") && std::strcmp(value, "1")) return -1;
    o.pdl = value[0] == '1';
    return 0;
  }
  if (!std::strcmp(key, "vector_fetch")) {
    if (std::strcmp(value, "0") && std::strcmp(value, "1")) return -1;
    o.vector_fetch = value[0] == '1';
    return 0;
  }
  if (!std::strcmp(key, "tma")) {
    if (std::strcmp(value, "0") && std::strcmp(value, "1")) return -1;
    o.tma = value[0] == '1';
    return 0;
  }
  if (!std::strcmp(key, "warp_px") || !std::strcmp(key, "job_blocks") || !std::strcmp(key, "geo_blocks")) {
    char* end = nullptr;
    unsigned long v = std::strtoul(value, &end, 10);
    if (!*value || *end) return -1;
    if (key[0] == 'w') {
      if (v < 1 || v > 4096) return -1;
      o.warp_px = (uint32_t)v;
    } else if (key[0] == 'j') {
      if (v < 1 || v > 32) return -1;
      o.job_blocks = (uint32_t)v;
    } else {
      if (v > 64) return -1;
      o.geo_blocks = (uint32_t)v;
    }
    return 0;
  }
  if (!std::strcmp(key, "barrier_ns")) {
    char* end = nullptr;
    unsigned long long v = std::strtoull(value, &end, 10);
    if (!*value || *end || v > 0xFFFFFFFFull) return -1;
    o.barrier_ns = (uint32_t)v;
    return 0;
  }
  if (!std::strcmp(key, "fault_alloc")) {
    o.fault_alloc = std::atol(value);
    kz::g_alloc_count = 0;
    return 0;
  }
  return -1;
}

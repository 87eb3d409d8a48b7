"""ctypes view of the Vulkan API exported by libkazan_driver.so.

The driver is a Vulkan ICD (the role of the reference's vulkan-driver crate, vulkan-driver/src/lib.rs).
With no Vulkan loader in this environment, callers load the library directly and resolve every vk*
function through vk_icdGetInstanceProcAddr, as a loader would.  Struct layouts follow
include/kz_vk_abi.h (the Vulkan specification's layouts).
"""
import ctypes
import os
from ctypes import (POINTER, Structure, Union, c_char, c_char_p, c_float, c_int, c_int32, c_size_t, c_uint8,
                    c_uint32, c_uint64, c_void_p)

PKG = os.path.dirname(os.path.abspath(__file__))
DRIVER_PATH = os.path.join(PKG, "_build", "libkazan_driver.so")

# ---- enumerants (Vulkan specification) ----
VK_SUCCESS = 0
VK_NOT_READY = 1
VK_TIMEOUT = 2
VK_INCOMPLETE = 5
VK_ERROR_OUT_OF_HOST_MEMORY = -1
VK_ERROR_OUT_OF_DEVICE_MEMORY = -2
VK_ERROR_INITIALIZATION_FAILED = -3
VK_ERROR_DEVICE_LOST = -4
VK_ERROR_FEATURE_NOT_PRESENT = -8
VK_ERROR_FORMAT_NOT_SUPPORTED = -11

ST_APPLICATION_INFO = 0
ST_INSTANCE_CREATE_INFO = 1
ST_DEVICE_QUEUE_CREATE_INFO = 2
ST_DEVICE_CREATE_INFO = 3
ST_SUBMIT_INFO = 4
ST_MEMORY_ALLOCATE_INFO = 5
ST_FENCE_CREATE_INFO = 8
ST_BUFFER_CREATE_INFO = 12
ST_IMAGE_CREATE_INFO = 14
ST_IMAGE_VIEW_CREATE_INFO = 15
ST_SHADER_MODULE_CREATE_INFO = 16
ST_PIPELINE_SHADER_STAGE_CREATE_INFO = 18
ST_PIPELINE_VERTEX_INPUT_STATE_CREATE_INFO = 19
ST_PIPELINE_INPUT_ASSEMBLY_STATE_CREATE_INFO = 20
ST_PIPELINE_VIEWPORT_STATE_CREATE_INFO = 22
ST_PIPELINE_RASTERIZATION_STATE_CREATE_INFO = 23
ST_PIPELINE_MULTISAMPLE_STATE_CREATE_INFO = 24
ST_PIPELINE_DEPTH_STENCIL_STATE_CREATE_INFO = 25
ST_PIPELINE_COLOR_BLEND_STATE_CREATE_INFO = 26
ST_PIPELINE_DYNAMIC_STATE_CREATE_INFO = 27
DYNAMIC_STATE_VIEWPORT, DYNAMIC_STATE_SCISSOR, DYNAMIC_STATE_BLEND_CONSTANTS = 0, 1, 4
DYNAMIC_STATE_STENCIL_COMPARE_MASK, DYNAMIC_STATE_STENCIL_WRITE_MASK, DYNAMIC_STATE_STENCIL_REFERENCE = 6, 7, 8
ST_GRAPHICS_PIPELINE_CREATE_INFO = 28
ST_PIPELINE_LAYOUT_CREATE_INFO = 30
ST_SAMPLER_CREATE_INFO = 31
ST_DESCRIPTOR_SET_LAYOUT_CREATE_INFO = 32
ST_DESCRIPTOR_POOL_CREATE_INFO = 33
ST_DESCRIPTOR_SET_ALLOCATE_INFO = 34
ST_WRITE_DESCRIPTOR_SET = 35
ST_COPY_DESCRIPTOR_SET = 36
DESCRIPTOR_SAMPLER = 0
DESCRIPTOR_COMBINED_IMAGE_SAMPLER = 1
DESCRIPTOR_SAMPLED_IMAGE = 2
DESCRIPTOR_UNIFORM_BUFFER = 6
DESCRIPTOR_UNIFORM_BUFFER_DYNAMIC = 8
DESCRIPTOR_STORAGE_BUFFER = 7
DESCRIPTOR_STORAGE_BUFFER_DYNAMIC = 9
FILTER_NEAREST, FILTER_LINEAR = 0, 1
ADDRESS_REPEAT, ADDRESS_MIRRORED_REPEAT, ADDRESS_CLAMP_TO_EDGE, ADDRESS_CLAMP_TO_BORDER, ADDRESS_MIRROR_CLAMP = 0, 1, 2, 3, 4
VK_ERROR_OUT_OF_POOL_MEMORY = -1000069000
ST_FRAMEBUFFER_CREATE_INFO = 37
ST_RENDER_PASS_CREATE_INFO = 38
ST_COMMAND_POOL_CREATE_INFO = 39
ST_COMMAND_BUFFER_ALLOCATE_INFO = 40
ST_COMMAND_BUFFER_BEGIN_INFO = 42
ST_RENDER_PASS_BEGIN_INFO = 43

FORMAT_R8G8B8A8_UNORM = 37
FORMAT_B8G8R8A8_UNORM = 44
FORMAT_R8G8B8A8_SRGB = 43
FORMAT_B8G8R8A8_SRGB = 50
COLOR_FORMATS = {"rgba8": FORMAT_R8G8B8A8_UNORM, "bgra8": FORMAT_B8G8R8A8_UNORM,
                 "rgba8_srgb": FORMAT_R8G8B8A8_SRGB, "bgra8_srgb": FORMAT_B8G8R8A8_SRGB}
FORMAT_R32G32_SFLOAT = 103
FORMAT_R32G32B32_SFLOAT = 106
FORMAT_R32G32B32A32_SFLOAT = 109
FORMAT_D32_SFLOAT = 126
FORMAT_D16_UNORM = 124
FORMAT_D24_UNORM_S8_UINT = 129
DEPTH_FORMATS = {"d32": FORMAT_D32_SFLOAT, "d16": FORMAT_D16_UNORM, "d24s8": FORMAT_D24_UNORM_S8_UINT}

IMAGE_TYPE_2D = 1
IMAGE_TILING_OPTIMAL = 0
IMAGE_TILING_LINEAR = 1
IMAGE_VIEW_TYPE_2D = 1
IMAGE_LAYOUT_UNDEFINED = 0
IMAGE_LAYOUT_GENERAL = 1
IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL = 2
IMAGE_LAYOUT_DEPTH_STENCIL_ATTACHMENT_OPTIMAL = 3
IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL = 6
IMAGE_LAYOUT_TRANSFER_DST_OPTIMAL = 7

BUFFER_USAGE_TRANSFER_SRC = 0x1
BUFFER_USAGE_TRANSFER_DST = 0x2
BUFFER_USAGE_UNIFORM = 0x10
BUFFER_USAGE_STORAGE = 0x20
BUFFER_USAGE_INDEX = 0x40
BUFFER_USAGE_VERTEX = 0x80
BUFFER_USAGE_INDIRECT = 0x100
IMAGE_USAGE_TRANSFER_SRC = 0x1
IMAGE_USAGE_TRANSFER_DST = 0x2
IMAGE_USAGE_SAMPLED = 0x4
IMAGE_USAGE_COLOR_ATTACHMENT = 0x10
IMAGE_USAGE_DEPTH_STENCIL_ATTACHMENT = 0x20
IMAGE_ASPECT_COLOR = 0x1
IMAGE_ASPECT_DEPTH = 0x2
IMAGE_ASPECT_STENCIL = 0x4

MEMORY_PROPERTY_DEVICE_LOCAL = 0x1
MEMORY_PROPERTY_HOST_VISIBLE = 0x2
MEMORY_PROPERTY_HOST_COHERENT = 0x4

SHADER_STAGE_VERTEX = 0x1
SHADER_STAGE_FRAGMENT = 0x10
TOPOLOGY_TRIANGLE_LIST = 3
POLYGON_MODE_FILL = 0
CULL_NONE = 0
CULL_FRONT = 1
CULL_BACK = 2
FRONT_FACE_CCW = 0
FRONT_FACE_CW = 1
COMPARE_NEVER, COMPARE_LESS, COMPARE_EQUAL, COMPARE_LEQUAL, COMPARE_GREATER, COMPARE_NOTEQUAL, \
    COMPARE_GEQUAL, COMPARE_ALWAYS = range(8)
BLEND_ZERO, BLEND_ONE = 0, 1
BLEND_SRC_ALPHA, BLEND_ONE_MINUS_SRC_ALPHA = 6, 7
BLEND_OP_ADD = 0
COLOR_MASK_RGBA = 0xF
DYNAMIC_VIEWPORT, DYNAMIC_SCISSOR = 0, 1
LOAD_OP_LOAD, LOAD_OP_CLEAR, LOAD_OP_DONT_CARE = 0, 1, 2
STORE_OP_STORE = 0
BIND_POINT_GRAPHICS = 0
COMMAND_BUFFER_LEVEL_PRIMARY = 0
INDEX_TYPE_UINT16, INDEX_TYPE_UINT32 = 0, 1
SUBPASS_CONTENTS_INLINE = 0
VERTEX_INPUT_RATE_VERTEX = 0
VERTEX_INPUT_RATE_INSTANCE = 1
FENCE_CREATE_SIGNALED = 0x1
SAMPLE_COUNT_1 = 0x1
ATTACHMENT_UNUSED = 0xFFFFFFFF


class VkError(RuntimeError):
    def __init__(self, what, code):
        super().__init__("%s failed with VkResult %d" % (what, code))
        self.code = code


def check(what, r):
    if r != VK_SUCCESS:
        raise VkError(what, r)
    return r


# ---- structures ----
class VkApplicationInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("pApplicationName", c_char_p), ("applicationVersion", c_uint32),
                ("pEngineName", c_char_p), ("engineVersion", c_uint32), ("apiVersion", c_uint32)]


class VkInstanceCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32),
                ("pApplicationInfo", POINTER(VkApplicationInfo)), ("enabledLayerCount", c_uint32),
                ("ppEnabledLayerNames", c_void_p), ("enabledExtensionCount", c_uint32),
                ("ppEnabledExtensionNames", c_void_p)]


_LIMIT_FIELDS = [
    ("maxImageDimension1D", c_uint32), ("maxImageDimension2D", c_uint32), ("maxImageDimension3D", c_uint32),
    ("maxImageDimensionCube", c_uint32), ("maxImageArrayLayers", c_uint32), ("maxTexelBufferElements", c_uint32),
    ("maxUniformBufferRange", c_uint32), ("maxStorageBufferRange", c_uint32), ("maxPushConstantsSize", c_uint32),
    ("maxMemoryAllocationCount", c_uint32), ("maxSamplerAllocationCount", c_uint32),
    ("bufferImageGranularity", c_uint64), ("sparseAddressSpaceSize", c_uint64),
    ("maxBoundDescriptorSets", c_uint32), ("maxPerStageDescriptorSamplers", c_uint32),
    ("maxPerStageDescriptorUniformBuffers", c_uint32), ("maxPerStageDescriptorStorageBuffers", c_uint32),
    ("maxPerStageDescriptorSampledImages", c_uint32), ("maxPerStageDescriptorStorageImages", c_uint32),
    ("maxPerStageDescriptorInputAttachments", c_uint32), ("maxPerStageResources", c_uint32),
    ("maxDescriptorSetSamplers", c_uint32), ("maxDescriptorSetUniformBuffers", c_uint32),
    ("maxDescriptorSetUniformBuffersDynamic", c_uint32), ("maxDescriptorSetStorageBuffers", c_uint32),
    ("maxDescriptorSetStorageBuffersDynamic", c_uint32), ("maxDescriptorSetSampledImages", c_uint32),
    ("maxDescriptorSetStorageImages", c_uint32), ("maxDescriptorSetInputAttachments", c_uint32),
    ("maxVertexInputAttributes", c_uint32), ("maxVertexInputBindings", c_uint32),
    ("maxVertexInputAttributeOffset", c_uint32), ("maxVertexInputBindingStride", c_uint32),
    ("maxVertexOutputComponents", c_uint32), ("maxTessellationGenerationLevel", c_uint32),
    ("maxTessellationPatchSize", c_uint32), ("maxTessellationControlPerVertexInputComponents", c_uint32),
    ("maxTessellationControlPerVertexOutputComponents", c_uint32),
    ("maxTessellationControlPerPatchOutputComponents", c_uint32),
    ("maxTessellationControlTotalOutputComponents", c_uint32),
    ("maxTessellationEvaluationInputComponents", c_uint32), ("maxTessellationEvaluationOutputComponents", c_uint32),
    ("maxGeometryShaderInvocations", c_uint32), ("maxGeometryInputComponents", c_uint32),
    ("maxGeometryOutputComponents", c_uint32), ("maxGeometryOutputVertices", c_uint32),
    ("maxGeometryTotalOutputComponents", c_uint32), ("maxFragmentInputComponents", c_uint32),
    ("maxFragmentOutputAttachments", c_uint32), ("maxFragmentDualSrcAttachments", c_uint32),
    ("maxFragmentCombinedOutputResources", c_uint32), ("maxComputeSharedMemorySize", c_uint32),
    ("maxComputeWorkGroupCount", c_uint32 * 3), ("maxComputeWorkGroupInvocations", c_uint32),
    ("maxComputeWorkGroupSize", c_uint32 * 3), ("subPixelPrecisionBits", c_uint32),
    ("subTexelPrecisionBits", c_uint32), ("mipmapPrecisionBits", c_uint32), ("maxDrawIndexedIndexValue", c_uint32),
    ("maxDrawIndirectCount", c_uint32), ("maxSamplerLodBias", c_float), ("maxSamplerAnisotropy", c_float),
    ("maxViewports", c_uint32), ("maxViewportDimensions", c_uint32 * 2), ("viewportBoundsRange", c_float * 2),
    ("viewportSubPixelBits", c_uint32), ("minMemoryMapAlignment", c_size_t),
    ("minTexelBufferOffsetAlignment", c_uint64), ("minUniformBufferOffsetAlignment", c_uint64),
    ("minStorageBufferOffsetAlignment", c_uint64), ("minTexelOffset", c_int32), ("maxTexelOffset", c_uint32),
    ("minTexelGatherOffset", c_int32), ("maxTexelGatherOffset", c_uint32), ("minInterpolationOffset", c_float),
    ("maxInterpolationOffset", c_float), ("subPixelInterpolationOffsetBits", c_uint32),
    ("maxFramebufferWidth", c_uint32), ("maxFramebufferHeight", c_uint32), ("maxFramebufferLayers", c_uint32),
    ("framebufferColorSampleCounts", c_uint32), ("framebufferDepthSampleCounts", c_uint32),
    ("framebufferStencilSampleCounts", c_uint32), ("framebufferNoAttachmentsSampleCounts", c_uint32),
    ("maxColorAttachments", c_uint32), ("sampledImageColorSampleCounts", c_uint32),
    ("sampledImageIntegerSampleCounts", c_uint32), ("sampledImageDepthSampleCounts", c_uint32),
    ("sampledImageStencilSampleCounts", c_uint32), ("storageImageSampleCounts", c_uint32),
    ("maxSampleMaskWords", c_uint32), ("timestampComputeAndGraphics", c_uint32), ("timestampPeriod", c_float),
    ("maxClipDistances", c_uint32), ("maxCullDistances", c_uint32), ("maxCombinedClipAndCullDistances", c_uint32),
    ("discreteQueuePriorities", c_uint32), ("pointSizeRange", c_float * 2), ("lineWidthRange", c_float * 2),
    ("pointSizeGranularity", c_float), ("lineWidthGranularity", c_float), ("strictLines", c_uint32),
    ("standardSampleLocations", c_uint32), ("optimalBufferCopyOffsetAlignment", c_uint64),
    ("optimalBufferCopyRowPitchAlignment", c_uint64), ("nonCoherentAtomSize", c_uint64)]


class VkPhysicalDeviceLimits(Structure):
    _fields_ = _LIMIT_FIELDS


class VkPhysicalDeviceProperties(Structure):
    _fields_ = [("apiVersion", c_uint32), ("driverVersion", c_uint32), ("vendorID", c_uint32), ("deviceID", c_uint32),
                ("deviceType", c_int), ("deviceName", c_char * 256), ("pipelineCacheUUID", c_uint8 * 16),
                ("limits", VkPhysicalDeviceLimits), ("sparseProperties", c_uint32 * 5)]


class VkMemoryType(Structure):
    _fields_ = [("propertyFlags", c_uint32), ("heapIndex", c_uint32)]


class VkMemoryHeap(Structure):
    _fields_ = [("size", c_uint64), ("flags", c_uint32)]


class VkPhysicalDeviceMemoryProperties(Structure):
    _fields_ = [("memoryTypeCount", c_uint32), ("memoryTypes", VkMemoryType * 32), ("memoryHeapCount", c_uint32),
                ("memoryHeaps", VkMemoryHeap * 16)]


class VkDeviceQueueCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("queueFamilyIndex", c_uint32),
                ("queueCount", c_uint32), ("pQueuePriorities", POINTER(c_float))]


class VkDeviceCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("queueCreateInfoCount", c_uint32),
                ("pQueueCreateInfos", POINTER(VkDeviceQueueCreateInfo)), ("enabledLayerCount", c_uint32),
                ("ppEnabledLayerNames", c_void_p), ("enabledExtensionCount", c_uint32),
                ("ppEnabledExtensionNames", c_void_p), ("pEnabledFeatures", c_void_p)]


class VkSubmitInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("waitSemaphoreCount", c_uint32),
                ("pWaitSemaphores", c_void_p), ("pWaitDstStageMask", c_void_p), ("commandBufferCount", c_uint32),
                ("pCommandBuffers", POINTER(c_void_p)), ("signalSemaphoreCount", c_uint32),
                ("pSignalSemaphores", c_void_p)]


class VkMemoryAllocateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("allocationSize", c_uint64), ("memoryTypeIndex", c_uint32)]


class VkMemoryRequirements(Structure):
    _fields_ = [("size", c_uint64), ("alignment", c_uint64), ("memoryTypeBits", c_uint32)]


class VkFenceCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32)]


class VkBufferCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("size", c_uint64), ("usage", c_uint32),
                ("sharingMode", c_int), ("queueFamilyIndexCount", c_uint32), ("pQueueFamilyIndices", c_void_p)]


class VkExtent3D(Structure):
    _fields_ = [("width", c_uint32), ("height", c_uint32), ("depth", c_uint32)]


class VkOffset3D(Structure):
    _fields_ = [("x", c_int32), ("y", c_int32), ("z", c_int32)]


class VkImageCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("imageType", c_int), ("format", c_int),
                ("extent", VkExtent3D), ("mipLevels", c_uint32), ("arrayLayers", c_uint32), ("samples", c_uint32),
                ("tiling", c_int), ("usage", c_uint32), ("sharingMode", c_int), ("queueFamilyIndexCount", c_uint32),
                ("pQueueFamilyIndices", c_void_p), ("initialLayout", c_int)]


class VkImageSubresource(Structure):
    _fields_ = [("aspectMask", c_uint32), ("mipLevel", c_uint32), ("arrayLayer", c_uint32)]


class VkSubresourceLayout(Structure):
    _fields_ = [("offset", c_uint64), ("size", c_uint64), ("rowPitch", c_uint64), ("arrayPitch", c_uint64),
                ("depthPitch", c_uint64)]


class VkImageSubresourceRange(Structure):
    _fields_ = [("aspectMask", c_uint32), ("baseMipLevel", c_uint32), ("levelCount", c_uint32),
                ("baseArrayLayer", c_uint32), ("layerCount", c_uint32)]


class VkImageSubresourceLayers(Structure):
    _fields_ = [("aspectMask", c_uint32), ("mipLevel", c_uint32), ("baseArrayLayer", c_uint32),
                ("layerCount", c_uint32)]


class VkImageViewCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("image", c_void_p),
                ("viewType", c_int), ("format", c_int), ("components", c_int * 4),
                ("subresourceRange", VkImageSubresourceRange)]


class VkShaderModuleCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("codeSize", c_size_t),
                ("pCode", c_void_p)]


class VkSpecializationMapEntry(Structure):
    _fields_ = [("constantID", c_uint32), ("offset", c_uint32), ("size", c_size_t)]


class VkSpecializationInfo(Structure):
    _fields_ = [("mapEntryCount", c_uint32), ("pMapEntries", POINTER(VkSpecializationMapEntry)),
                ("dataSize", c_size_t), ("pData", c_void_p)]


class VkPipelineShaderStageCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("stage", c_uint32),
                ("module", c_void_p), ("pName", c_char_p), ("pSpecializationInfo", POINTER(VkSpecializationInfo))]


class VkVertexInputBindingDescription(Structure):
    _fields_ = [("binding", c_uint32), ("stride", c_uint32), ("inputRate", c_int)]


class VkVertexInputAttributeDescription(Structure):
    _fields_ = [("location", c_uint32), ("binding", c_uint32), ("format", c_int), ("offset", c_uint32)]


class VkPipelineVertexInputStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32),
                ("vertexBindingDescriptionCount", c_uint32),
                ("pVertexBindingDescriptions", POINTER(VkVertexInputBindingDescription)),
                ("vertexAttributeDescriptionCount", c_uint32),
                ("pVertexAttributeDescriptions", POINTER(VkVertexInputAttributeDescription))]


class VkPipelineInputAssemblyStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("topology", c_int),
                ("primitiveRestartEnable", c_uint32)]


class VkViewport(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("width", c_float), ("height", c_float), ("minDepth", c_float),
                ("maxDepth", c_float)]


class VkOffset2D(Structure):
    _fields_ = [("x", c_int32), ("y", c_int32)]


class VkExtent2D(Structure):
    _fields_ = [("width", c_uint32), ("height", c_uint32)]


class VkRect2D(Structure):
    _fields_ = [("offset", VkOffset2D), ("extent", VkExtent2D)]


class VkPipelineViewportStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("viewportCount", c_uint32),
                ("pViewports", POINTER(VkViewport)), ("scissorCount", c_uint32), ("pScissors", POINTER(VkRect2D))]


class VkPipelineRasterizationStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("depthClampEnable", c_uint32),
                ("rasterizerDiscardEnable", c_uint32), ("polygonMode", c_int), ("cullMode", c_uint32),
                ("frontFace", c_int), ("depthBiasEnable", c_uint32), ("depthBiasConstantFactor", c_float),
                ("depthBiasClamp", c_float), ("depthBiasSlopeFactor", c_float), ("lineWidth", c_float)]


class VkPipelineMultisampleStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("rasterizationSamples", c_uint32),
                ("sampleShadingEnable", c_uint32), ("minSampleShading", c_float), ("pSampleMask", c_void_p),
                ("alphaToCoverageEnable", c_uint32), ("alphaToOneEnable", c_uint32)]


class VkStencilOpState(Structure):
    _fields_ = [("failOp", c_int), ("passOp", c_int), ("depthFailOp", c_int), ("compareOp", c_int),
                ("compareMask", c_uint32), ("writeMask", c_uint32), ("reference", c_uint32)]


class VkPipelineDepthStencilStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("depthTestEnable", c_uint32),
                ("depthWriteEnable", c_uint32), ("depthCompareOp", c_int), ("depthBoundsTestEnable", c_uint32),
                ("stencilTestEnable", c_uint32), ("front", VkStencilOpState), ("back", VkStencilOpState),
                ("minDepthBounds", c_float), ("maxDepthBounds", c_float)]


class VkPipelineColorBlendAttachmentState(Structure):
    _fields_ = [("blendEnable", c_uint32), ("srcColorBlendFactor", c_int), ("dstColorBlendFactor", c_int),
                ("colorBlendOp", c_int), ("srcAlphaBlendFactor", c_int), ("dstAlphaBlendFactor", c_int),
                ("alphaBlendOp", c_int), ("colorWriteMask", c_uint32)]


class VkPipelineColorBlendStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("logicOpEnable", c_uint32),
                ("logicOp", c_int), ("attachmentCount", c_uint32),
                ("pAttachments", POINTER(VkPipelineColorBlendAttachmentState)), ("blendConstants", c_float * 4)]


class VkPipelineDynamicStateCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("dynamicStateCount", c_uint32),
                ("pDynamicStates", POINTER(c_int))]


class VkGraphicsPipelineCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("stageCount", c_uint32),
                ("pStages", POINTER(VkPipelineShaderStageCreateInfo)),
                ("pVertexInputState", POINTER(VkPipelineVertexInputStateCreateInfo)),
                ("pInputAssemblyState", POINTER(VkPipelineInputAssemblyStateCreateInfo)),
                ("pTessellationState", c_void_p),
                ("pViewportState", POINTER(VkPipelineViewportStateCreateInfo)),
                ("pRasterizationState", POINTER(VkPipelineRasterizationStateCreateInfo)),
                ("pMultisampleState", POINTER(VkPipelineMultisampleStateCreateInfo)),
                ("pDepthStencilState", POINTER(VkPipelineDepthStencilStateCreateInfo)),
                ("pColorBlendState", POINTER(VkPipelineColorBlendStateCreateInfo)),
                ("pDynamicState", POINTER(VkPipelineDynamicStateCreateInfo)), ("layout", c_void_p),
                ("renderPass", c_void_p), ("subpass", c_uint32), ("basePipelineHandle", c_void_p),
                ("basePipelineIndex", c_int32)]


class VkPushConstantRange(Structure):
    _fields_ = [("stageFlags", c_uint32), ("offset", c_uint32), ("size", c_uint32)]


class VkPipelineLayoutCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("setLayoutCount", c_uint32),
                ("pSetLayouts", c_void_p), ("pushConstantRangeCount", c_uint32),
                ("pPushConstantRanges", POINTER(VkPushConstantRange))]


class VkAttachmentDescription(Structure):
    _fields_ = [("flags", c_uint32), ("format", c_int), ("samples", c_uint32), ("loadOp", c_int), ("storeOp", c_int),
                ("stencilLoadOp", c_int), ("stencilStoreOp", c_int), ("initialLayout", c_int),
                ("finalLayout", c_int)]


class VkAttachmentReference(Structure):
    _fields_ = [("attachment", c_uint32), ("layout", c_int)]


class VkSubpassDescription(Structure):
    _fields_ = [("flags", c_uint32), ("pipelineBindPoint", c_int), ("inputAttachmentCount", c_uint32),
                ("pInputAttachments", c_void_p), ("colorAttachmentCount", c_uint32),
                ("pColorAttachments", POINTER(VkAttachmentReference)), ("pResolveAttachments", c_void_p),
                ("pDepthStencilAttachment", POINTER(VkAttachmentReference)), ("preserveAttachmentCount", c_uint32),
                ("pPreserveAttachments", c_void_p)]


class VkRenderPassCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("attachmentCount", c_uint32),
                ("pAttachments", POINTER(VkAttachmentDescription)), ("subpassCount", c_uint32),
                ("pSubpasses", POINTER(VkSubpassDescription)), ("dependencyCount", c_uint32),
                ("pDependencies", c_void_p)]


class VkFramebufferCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("renderPass", c_void_p),
                ("attachmentCount", c_uint32), ("pAttachments", POINTER(c_void_p)), ("width", c_uint32),
                ("height", c_uint32), ("layers", c_uint32)]


class VkCommandPoolCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("queueFamilyIndex", c_uint32)]


class VkCommandBufferAllocateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("commandPool", c_void_p), ("level", c_int),
                ("commandBufferCount", c_uint32)]


class VkCommandBufferBeginInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("pInheritanceInfo", c_void_p)]


class VkClearColorValue(Union):
    _fields_ = [("float32", c_float * 4), ("int32", c_int32 * 4), ("uint32", c_uint32 * 4)]


class VkClearDepthStencilValue(Structure):
    _fields_ = [("depth", c_float), ("stencil", c_uint32)]


class VkClearValue(Union):
    _fields_ = [("color", VkClearColorValue), ("depthStencil", VkClearDepthStencilValue)]


class VkClearAttachment(Structure):
    _fields_ = [("aspectMask", c_uint32), ("colorAttachment", c_uint32), ("clearValue", VkClearValue)]


class VkClearRect(Structure):
    _fields_ = [("rect", VkRect2D), ("baseArrayLayer", c_uint32), ("layerCount", c_uint32)]


class VkRenderPassBeginInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("renderPass", c_void_p), ("framebuffer", c_void_p),
                ("renderArea", VkRect2D), ("clearValueCount", c_uint32), ("pClearValues", POINTER(VkClearValue))]


class VkImageCopy(Structure):
    _fields_ = [("srcSubresource", VkImageSubresourceLayers), ("srcOffset", VkOffset3D),
                ("dstSubresource", VkImageSubresourceLayers), ("dstOffset", VkOffset3D), ("extent", VkExtent3D)]


class VkImageResolve(Structure):
    _fields_ = [("srcSubresource", VkImageSubresourceLayers), ("srcOffset", VkOffset3D),
                ("dstSubresource", VkImageSubresourceLayers), ("dstOffset", VkOffset3D), ("extent", VkExtent3D)]


class VkSamplerCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("magFilter", c_int),
                ("minFilter", c_int), ("mipmapMode", c_int), ("addressModeU", c_int), ("addressModeV", c_int),
                ("addressModeW", c_int), ("mipLodBias", c_float), ("anisotropyEnable", c_uint32),
                ("maxAnisotropy", c_float), ("compareEnable", c_uint32), ("compareOp", c_int), ("minLod", c_float),
                ("maxLod", c_float), ("borderColor", c_int), ("unnormalizedCoordinates", c_uint32)]


class VkDescriptorSetLayoutBinding(Structure):
    _fields_ = [("binding", c_uint32), ("descriptorType", c_int), ("descriptorCount", c_uint32),
                ("stageFlags", c_uint32), ("pImmutableSamplers", c_void_p)]


class VkDescriptorSetLayoutCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("bindingCount", c_uint32),
                ("pBindings", POINTER(VkDescriptorSetLayoutBinding))]


class VkDescriptorPoolSize(Structure):
    _fields_ = [("type", c_int), ("descriptorCount", c_uint32)]


class VkDescriptorPoolCreateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("flags", c_uint32), ("maxSets", c_uint32),
                ("poolSizeCount", c_uint32), ("pPoolSizes", POINTER(VkDescriptorPoolSize))]


class VkDescriptorSetAllocateInfo(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("descriptorPool", c_void_p), ("descriptorSetCount", c_uint32),
                ("pSetLayouts", POINTER(c_void_p))]


class VkDescriptorImageInfo(Structure):
    _fields_ = [("sampler", c_void_p), ("imageView", c_void_p), ("imageLayout", c_int)]


class VkDescriptorBufferInfo(Structure):
    _fields_ = [("buffer", c_void_p), ("offset", c_uint64), ("range", c_uint64)]


class VkWriteDescriptorSet(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("dstSet", c_void_p), ("dstBinding", c_uint32),
                ("dstArrayElement", c_uint32), ("descriptorCount", c_uint32), ("descriptorType", c_int),
                ("pImageInfo", POINTER(VkDescriptorImageInfo)), ("pBufferInfo", POINTER(VkDescriptorBufferInfo)),
                ("pTexelBufferView", c_void_p)]


class VkCopyDescriptorSet(Structure):
    _fields_ = [("sType", c_int), ("pNext", c_void_p), ("srcSet", c_void_p), ("srcBinding", c_uint32),
                ("srcArrayElement", c_uint32), ("dstSet", c_void_p), ("dstBinding", c_uint32),
                ("dstArrayElement", c_uint32), ("descriptorCount", c_uint32)]


class VkExtensionProperties(Structure):
    _fields_ = [("extensionName", ctypes.c_char * 256), ("specVersion", c_uint32)]


class VkFormatProperties(Structure):
    _fields_ = [("linearTilingFeatures", c_uint32), ("optimalTilingFeatures", c_uint32), ("bufferFeatures", c_uint32)]


FORMAT_FEATURE_SAMPLED_IMAGE, FORMAT_FEATURE_COLOR_ATTACHMENT = 0x1, 0x80


class VkBufferCopy(Structure):
    _fields_ = [("srcOffset", c_uint64), ("dstOffset", c_uint64), ("size", c_uint64)]


class VkBufferImageCopy(Structure):
    _fields_ = [("bufferOffset", c_uint64), ("bufferRowLength", c_uint32), ("bufferImageHeight", c_uint32),
                ("imageSubresource", VkImageSubresourceLayers), ("imageOffset", VkOffset3D),
                ("imageExtent", VkExtent3D)]


# kernel kinds of kzGetKernelTimes (KZ_KERNEL_KIND_NAMES)
KERNEL_KINDS = ["kz_k_persistent", "kz_k_vis_init", "kz_k_vis_geometry", "kz_k_vis_large", "kz_k_vis_resolve",
                "kz_k_geometry", "kz_k_scan", "kz_k_bin", "kz_k_raster", "kz_k_clear", "kz_k_indirect",
                "kz_k_indirect_tables", "kz_k_resolve", "kz_k_persistent_vis", "kz_k_raster_direct",
                "kz_k_raster_ds", "kz_k_raster_ms"]


class KzCommandBufferStats(Structure):
    _fields_ = [("triangles", c_uint64), ("draws", c_uint32), ("segments", c_uint32), ("mode", c_uint32),
                ("tile", c_uint32), ("status", c_uint32), ("records", c_uint32), ("pairs", c_uint32),
                ("fragments", c_uint32), ("rec_cap", c_uint32), ("pair_cap", c_uint32), ("gpu_ms", c_float),
                ("launches", c_uint32)]


H = c_void_p
P = POINTER
_PROTOS = {
    "vkCreateInstance": (c_int, [P(VkInstanceCreateInfo), c_void_p, P(H)]),
    "vkDestroyInstance": (None, [H, c_void_p]),
    "vkEnumerateInstanceVersion": (c_int, [P(c_uint32)]),
    "vkEnumeratePhysicalDevices": (c_int, [H, P(c_uint32), P(H)]),
    "vkGetPhysicalDeviceProperties": (None, [H, P(VkPhysicalDeviceProperties)]),
    "vkGetPhysicalDeviceMemoryProperties": (None, [H, P(VkPhysicalDeviceMemoryProperties)]),
    "vkCreateDevice": (c_int, [H, P(VkDeviceCreateInfo), c_void_p, P(H)]),
    "vkDestroyDevice": (None, [H, c_void_p]),
    "vkGetDeviceQueue": (None, [H, c_uint32, c_uint32, P(H)]),
    "vkDeviceWaitIdle": (c_int, [H]),
    "vkQueueSubmit": (c_int, [H, c_uint32, P(VkSubmitInfo), H]),
    "vkQueueWaitIdle": (c_int, [H]),
    "vkAllocateMemory": (c_int, [H, P(VkMemoryAllocateInfo), c_void_p, P(H)]),
    "vkFreeMemory": (None, [H, H, c_void_p]),
    "vkMapMemory": (c_int, [H, H, c_uint64, c_uint64, c_uint32, P(c_void_p)]),
    "vkUnmapMemory": (None, [H, H]),
    "vkCreateBuffer": (c_int, [H, P(VkBufferCreateInfo), c_void_p, P(H)]),
    "vkDestroyBuffer": (None, [H, H, c_void_p]),
    "vkGetBufferMemoryRequirements": (None, [H, H, P(VkMemoryRequirements)]),
    "vkBindBufferMemory": (c_int, [H, H, H, c_uint64]),
    "vkCreateImage": (c_int, [H, P(VkImageCreateInfo), c_void_p, P(H)]),
    "vkDestroyImage": (None, [H, H, c_void_p]),
    "vkGetImageMemoryRequirements": (None, [H, H, P(VkMemoryRequirements)]),
    "vkBindImageMemory": (c_int, [H, H, H, c_uint64]),
    "vkGetImageSubresourceLayout": (None, [H, H, P(VkImageSubresource), P(VkSubresourceLayout)]),
    "vkCreateImageView": (c_int, [H, P(VkImageViewCreateInfo), c_void_p, P(H)]),
    "vkDestroyImageView": (None, [H, H, c_void_p]),
    "vkCreateRenderPass": (c_int, [H, P(VkRenderPassCreateInfo), c_void_p, P(H)]),
    "vkDestroyRenderPass": (None, [H, H, c_void_p]),
    "vkCreateFramebuffer": (c_int, [H, P(VkFramebufferCreateInfo), c_void_p, P(H)]),
    "vkDestroyFramebuffer": (None, [H, H, c_void_p]),
    "vkCreateShaderModule": (c_int, [H, P(VkShaderModuleCreateInfo), c_void_p, P(H)]),
    "vkDestroyShaderModule": (None, [H, H, c_void_p]),
    "vkCreatePipelineLayout": (c_int, [H, P(VkPipelineLayoutCreateInfo), c_void_p, P(H)]),
    "vkDestroyPipelineLayout": (None, [H, H, c_void_p]),
    "vkCreateGraphicsPipelines": (c_int, [H, H, c_uint32, P(VkGraphicsPipelineCreateInfo), c_void_p, P(H)]),
    "vkDestroyPipeline": (None, [H, H, c_void_p]),
    "vkCreateCommandPool": (c_int, [H, P(VkCommandPoolCreateInfo), c_void_p, P(H)]),
    "vkDestroyCommandPool": (None, [H, H, c_void_p]),
    "vkAllocateCommandBuffers": (c_int, [H, P(VkCommandBufferAllocateInfo), P(H)]),
    "vkFreeCommandBuffers": (None, [H, H, c_uint32, P(H)]),
    "vkBeginCommandBuffer": (c_int, [H, P(VkCommandBufferBeginInfo)]),
    "vkEndCommandBuffer": (c_int, [H]),
    "vkCmdBindPipeline": (None, [H, c_int, H]),
    "vkCmdSetViewport": (None, [H, c_uint32, c_uint32, P(VkViewport)]),
    "vkCmdSetScissor": (None, [H, c_uint32, c_uint32, P(VkRect2D)]),
    "vkCmdSetBlendConstants": (None, [H, P(ctypes.c_float)]),
    "vkCmdBindVertexBuffers": (None, [H, c_uint32, c_uint32, P(H), P(c_uint64)]),
    "vkCmdBindIndexBuffer": (None, [H, H, c_uint64, c_int]),
    "vkCmdPushConstants": (None, [H, H, c_uint32, c_uint32, c_uint32, c_void_p]),
    "vkCmdDraw": (None, [H, c_uint32, c_uint32, c_uint32, c_uint32]),
    "vkCmdDrawIndexed": (None, [H, c_uint32, c_uint32, c_uint32, c_int32, c_uint32]),
    "vkCmdDrawIndirect": (None, [H, H, c_uint64, c_uint32, c_uint32]),
    "vkCmdDrawIndexedIndirect": (None, [H, H, c_uint64, c_uint32, c_uint32]),
    "vkEnumerateDeviceExtensionProperties": (c_int, [H, ctypes.c_char_p, P(c_uint32), P(VkExtensionProperties)]),
    "vkGetPhysicalDeviceFeatures": (None, [H, P(c_uint32)]),
    "vkCmdResolveImage": (None, [H, H, c_int, H, c_int, c_uint32, P(VkImageResolve)]),
    "vkCmdCopyImage": (None, [H, H, c_int, H, c_int, c_uint32, P(VkImageCopy)]),
    "vkCmdUpdateBuffer": (None, [H, H, c_uint64, c_uint64, c_void_p]),
    "vkCmdClearAttachments": (None, [H, c_uint32, c_void_p, c_uint32, c_void_p]),
    "vkCmdSetStencilCompareMask": (None, [H, c_uint32, c_uint32]),
    "vkCmdSetStencilWriteMask": (None, [H, c_uint32, c_uint32]),
    "vkCmdSetStencilReference": (None, [H, c_uint32, c_uint32]),
    "vkCreateSampler": (c_int, [H, P(VkSamplerCreateInfo), c_void_p, P(H)]),
    "vkDestroySampler": (None, [H, H, c_void_p]),
    "vkCreateDescriptorSetLayout": (c_int, [H, P(VkDescriptorSetLayoutCreateInfo), c_void_p, P(H)]),
    "vkDestroyDescriptorSetLayout": (None, [H, H, c_void_p]),
    "vkCreateDescriptorPool": (c_int, [H, P(VkDescriptorPoolCreateInfo), c_void_p, P(H)]),
    "vkDestroyDescriptorPool": (None, [H, H, c_void_p]),
    "vkResetDescriptorPool": (c_int, [H, H, c_uint32]),
    "vkAllocateDescriptorSets": (c_int, [H, P(VkDescriptorSetAllocateInfo), P(H)]),
    "vkFreeDescriptorSets": (c_int, [H, H, c_uint32, P(H)]),
    "vkUpdateDescriptorSets": (None, [H, c_uint32, P(VkWriteDescriptorSet), c_uint32, P(VkCopyDescriptorSet)]),
    "vkCmdBindDescriptorSets": (None, [H, c_int, H, c_uint32, c_uint32, P(H), c_uint32, P(c_uint32)]),
    "vkCmdDrawIndirectCountKHR": (None, [H, H, c_uint64, H, c_uint64, c_uint32, c_uint32]),
    "vkCmdDrawIndexedIndirectCountKHR": (None, [H, H, c_uint64, H, c_uint64, c_uint32, c_uint32]),
    "vkCmdBeginRenderPass": (None, [H, P(VkRenderPassBeginInfo), c_int]),
    "vkCmdEndRenderPass": (None, [H]),
    "vkCmdClearColorImage": (None, [H, H, c_int, P(VkClearColorValue), c_uint32, P(VkImageSubresourceRange)]),
    "vkCmdClearDepthStencilImage": (None, [H, H, c_int, P(VkClearDepthStencilValue), c_uint32,
                                           P(VkImageSubresourceRange)]),
    "vkCmdCopyBuffer": (None, [H, H, H, c_uint32, P(VkBufferCopy)]),
    "vkCmdCopyImageToBuffer": (None, [H, H, c_int, H, c_uint32, P(VkBufferImageCopy)]),
    "vkCmdCopyBufferToImage": (None, [H, H, H, c_int, c_uint32, P(VkBufferImageCopy)]),
    "vkCmdFillBuffer": (None, [H, H, c_uint64, c_uint64, c_uint32]),
    "vkGetPhysicalDeviceFormatProperties": (None, [H, c_int, P(VkFormatProperties)]),
    "vkCreateFence": (c_int, [H, P(VkFenceCreateInfo), c_void_p, P(H)]),
    "vkDestroyFence": (None, [H, H, c_void_p]),
    "vkResetFences": (c_int, [H, c_uint32, P(H)]),
    "vkGetFenceStatus": (c_int, [H, H]),
    "vkWaitForFences": (c_int, [H, c_uint32, P(H), c_uint32, c_uint64]),
}

DRAW_PATH_ENTRY_POINTS = sorted(_PROTOS)


class Driver:
    """The ICD library with its vk* functions resolved through vk_icdGetInstanceProcAddr."""

    def __init__(self, path=None):
        path = path or DRIVER_PATH
        if not os.path.exists(path):
            raise RuntimeError("libkazan_driver.so is not built (run __graft_entry__.build())")
        self.lib = ctypes.CDLL(path)
        self.lib.vk_icdGetInstanceProcAddr.restype = c_void_p
        self.lib.vk_icdGetInstanceProcAddr.argtypes = [c_void_p, c_char_p]
        self.lib.vk_icdNegotiateLoaderICDInterfaceVersion.restype = c_int
        self.lib.vk_icdNegotiateLoaderICDInterfaceVersion.argtypes = [POINTER(c_uint32)]
        self.lib.vk_icdGetPhysicalDeviceProcAddr.restype = c_void_p
        self.lib.vk_icdGetPhysicalDeviceProcAddr.argtypes = [c_void_p, c_char_p]
        self.lib.kzDriverSetOption.restype = c_int
        self.lib.kzDriverSetOption.argtypes = [c_char_p, c_char_p]
        self.lib.kzGetQueueStream.restype = c_void_p
        self.lib.kzGetQueueStream.argtypes = [c_void_p]
        self.lib.kzGetCommandBufferStats.restype = c_int
        self.lib.kzGetCommandBufferStats.argtypes = [c_void_p, POINTER(KzCommandBufferStats)]
        self.lib.kzGetKernelTimes.restype = c_int
        self.lib.kzGetKernelTimes.argtypes = [c_void_p, POINTER(ctypes.c_double), POINTER(c_uint32), c_uint32,
                                              c_int]
        for name, (res, args) in _PROTOS.items():
            addr = self.lib.vk_icdGetInstanceProcAddr(None, name.encode())
            if not addr:
                raise RuntimeError("driver does not provide " + name)
            setattr(self, name, ctypes.CFUNCTYPE(res, *args)(addr))

    def set_option(self, key, value):
        if self.lib.kzDriverSetOption(key.encode(), str(value).encode()) != 0:
            raise ValueError("bad driver option %s=%s" % (key, value))

    def stats(self, cb):
        s = KzCommandBufferStats()
        check("kzGetCommandBufferStats", self.lib.kzGetCommandBufferStats(cb, ctypes.byref(s)))
        return s

    def kernel_times(self, cb, reset=False):
        """{kernel name: (summed ms, launches)} of a command buffer recorded with kernel_timing on"""
        ms = (ctypes.c_double * len(KERNEL_KINDS))()
        n = (c_uint32 * len(KERNEL_KINDS))()
        if self.lib.kzGetKernelTimes(cb, ms, n, len(KERNEL_KINDS), int(reset)) < 0:
            raise VkError("kzGetKernelTimes", -1)
        return {k: (ms[i], n[i]) for i, k in enumerate(KERNEL_KINDS) if n[i]}

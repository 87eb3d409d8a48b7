"""Drive the kazan GB300 driver through its Vulkan entry points: the calls an application (or the Vulkan
CTS through a loader) would make, issued directly against the ICD library.

  r = Renderer()                          instance, device, queue, command pool
  run = SceneRun(r, scene)                buffers, images, render pass, framebuffer, pipeline, command buffer
  run.submit(); color, depth = run.read()
"""
import ctypes
from ctypes import byref, c_float, c_uint32, c_uint64, c_void_p, pointer

import numpy as np

from . import vk
from .vk import check


class Buffer:
    def __init__(self, handle, memory, size, host_visible):
        self.handle, self.memory, self.size, self.host_visible = handle, memory, size, host_visible
        self.mapped = None


class Image:
    def __init__(self, handle, memory, view, width, height, fmt, host_visible, pitch):
        self.handle, self.memory, self.view = handle, memory, view
        self.width, self.height, self.format, self.host_visible, self.pitch = width, height, fmt, host_visible, pitch
        self.mapped = None


def _aspect(fmt):
    if fmt in (vk.FORMAT_D32_SFLOAT, vk.FORMAT_D16_UNORM):
        return vk.IMAGE_ASPECT_DEPTH
    if fmt == vk.FORMAT_D24_UNORM_S8_UINT:
        return vk.IMAGE_ASPECT_DEPTH | vk.IMAGE_ASPECT_STENCIL
    return vk.IMAGE_ASPECT_COLOR


class Renderer:
    def __init__(self, driver=None):
        self.drv = driver or vk.Driver()
        d = self.drv
        app = vk.VkApplicationInfo(vk.ST_APPLICATION_INFO, None, b"kazan_gb300", 1, b"kazan_gb300", 1,
                                   (1 << 22) | (1 << 12))
        ici = vk.VkInstanceCreateInfo(vk.ST_INSTANCE_CREATE_INFO, None, 0, pointer(app), 0, None, 0, None)
        self.instance = c_void_p()
        check("vkCreateInstance", d.vkCreateInstance(byref(ici), None, byref(self.instance)))
        n = c_uint32(0)
        check("vkEnumeratePhysicalDevices", d.vkEnumeratePhysicalDevices(self.instance, byref(n), None))
        if n.value == 0:
            d.vkDestroyInstance(self.instance, None)
            raise RuntimeError("no GPU: the driver exposes no physical device")
        pds = (c_void_p * n.value)()
        check("vkEnumeratePhysicalDevices", d.vkEnumeratePhysicalDevices(self.instance, byref(n), pds))
        self.physical = c_void_p(pds[0])
        self.props = vk.VkPhysicalDeviceProperties()
        d.vkGetPhysicalDeviceProperties(self.physical, byref(self.props))
        mp = vk.VkPhysicalDeviceMemoryProperties()
        d.vkGetPhysicalDeviceMemoryProperties(self.physical, byref(mp))
        self.host_type = self.device_type = None
        for i in range(mp.memoryTypeCount):
            f = mp.memoryTypes[i].propertyFlags
            if f & vk.MEMORY_PROPERTY_HOST_VISIBLE and self.host_type is None:
                self.host_type = i
            if f == vk.MEMORY_PROPERTY_DEVICE_LOCAL and self.device_type is None:
                self.device_type = i
        prio = c_float(1.0)
        qci = vk.VkDeviceQueueCreateInfo(vk.ST_DEVICE_QUEUE_CREATE_INFO, None, 0, 0, 1, pointer(prio))
        dci = vk.VkDeviceCreateInfo(vk.ST_DEVICE_CREATE_INFO, None, 0, 1, pointer(qci), 0, None, 0, None, None)
        self.device = c_void_p()
        check("vkCreateDevice", d.vkCreateDevice(self.physical, byref(dci), None, byref(self.device)))
        self.queue = c_void_p()
        d.vkGetDeviceQueue(self.device, 0, 0, byref(self.queue))
        pci = vk.VkCommandPoolCreateInfo(vk.ST_COMMAND_POOL_CREATE_INFO, None, 0x2, 0)
        self.pool = c_void_p()
        check("vkCreateCommandPool", d.vkCreateCommandPool(self.device, byref(pci), None, byref(self.pool)))
        fci = vk.VkFenceCreateInfo(vk.ST_FENCE_CREATE_INFO, None, 0)
        self.fence = c_void_p()
        check("vkCreateFence", d.vkCreateFence(self.device, byref(fci), None, byref(self.fence)))
        self._objects = []

    # ---------------------------------------------------------------------------------------------
    def close(self):
        d = self.drv
        if self.device:
            d.vkDeviceWaitIdle(self.device)
            for kind, h in reversed(self._objects):
                getattr(d, "vkDestroy" + kind if kind != "Memory" else "vkFreeMemory")(self.device, h, None)
            self._objects = []
            d.vkDestroyFence(self.device, self.fence, None)
            d.vkDestroyCommandPool(self.device, self.pool, None)
            d.vkDestroyDevice(self.device, None)
            d.vkDestroyInstance(self.instance, None)
            self.device = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def stream(self):
        return self.drv.lib.kzGetQueueStream(self.queue)

    # ---------------------------------------------------------------------------------------------
    def _alloc(self, req, host_visible):
        t = self.host_type if host_visible else self.device_type
        ai = vk.VkMemoryAllocateInfo(vk.ST_MEMORY_ALLOCATE_INFO, None, req.size, t)
        mem = c_void_p()
        check("vkAllocateMemory", self.drv.vkAllocateMemory(self.device, byref(ai), None, byref(mem)))
        self._objects.append(("Memory", mem))
        return mem

    def create_buffer(self, size, usage, host_visible=True):
        d = self.drv
        bci = vk.VkBufferCreateInfo(vk.ST_BUFFER_CREATE_INFO, None, 0, max(int(size), 4),
                                    usage | vk.BUFFER_USAGE_TRANSFER_SRC | vk.BUFFER_USAGE_TRANSFER_DST, 0, 0, None)
        h = c_void_p()
        check("vkCreateBuffer", d.vkCreateBuffer(self.device, byref(bci), None, byref(h)))
        req = vk.VkMemoryRequirements()
        d.vkGetBufferMemoryRequirements(self.device, h, byref(req))
        mem = self._alloc(req, host_visible)
        check("vkBindBufferMemory", d.vkBindBufferMemory(self.device, h, mem, 0))
        self._objects.append(("Buffer", h))
        return Buffer(h, mem, int(size), host_visible)

    def map(self, obj):
        if obj.mapped is None:
            p = c_void_p()
            check("vkMapMemory", self.drv.vkMapMemory(self.device, obj.memory, 0, 0xFFFFFFFFFFFFFFFF, 0, byref(p)))
            obj.mapped = p.value
        return obj.mapped

    def unmap(self, obj):
        if obj.mapped is not None:
            self.drv.vkUnmapMemory(self.device, obj.memory)
            obj.mapped = None

    def write_buffer(self, buf, array, keep_mapped=False):
        a = np.ascontiguousarray(array)
        if buf.host_visible:
            p = self.map(buf)
            ctypes.memmove(p, a.ctypes.data, a.nbytes)
            if not keep_mapped:
                self.unmap(buf)
            return
        staging = self.create_buffer(a.nbytes, 0, True)
        self.write_buffer(staging, a)
        cb = self.begin()
        region = vk.VkBufferCopy(0, 0, a.nbytes)
        self.drv.vkCmdCopyBuffer(cb, staging.handle, buf.handle, 1, byref(region))
        self.end_submit_wait(cb)
        self.free_command_buffer(cb)

    def create_image(self, width, height, fmt, usage, host_visible=True, samples=1):
        """samples 4: a multisampled attachment (optimal tiling; the samples of a pixel side by side in its
        host-visible memory, which the tests read directly)"""
        d = self.drv
        ici = vk.VkImageCreateInfo(vk.ST_IMAGE_CREATE_INFO, None, 0, vk.IMAGE_TYPE_2D, fmt,
                                   vk.VkExtent3D(width, height, 1), 1, 1, samples,
                                   vk.IMAGE_TILING_LINEAR if host_visible and samples == 1 else vk.IMAGE_TILING_OPTIMAL,
                                   usage | vk.IMAGE_USAGE_TRANSFER_SRC | vk.IMAGE_USAGE_TRANSFER_DST, 0, 0, None,
                                   vk.IMAGE_LAYOUT_UNDEFINED)
        h = c_void_p()
        check("vkCreateImage", d.vkCreateImage(self.device, byref(ici), None, byref(h)))
        req = vk.VkMemoryRequirements()
        d.vkGetImageMemoryRequirements(self.device, h, byref(req))
        mem = self._alloc(req, host_visible)
        check("vkBindImageMemory", d.vkBindImageMemory(self.device, h, mem, 0))
        self._objects.append(("Image", h))
        aspect = _aspect(fmt)
        vci = vk.VkImageViewCreateInfo(vk.ST_IMAGE_VIEW_CREATE_INFO, None, 0, h, vk.IMAGE_VIEW_TYPE_2D, fmt,
                                       (ctypes.c_int * 4)(0, 0, 0, 0), vk.VkImageSubresourceRange(aspect, 0, 1, 0, 1))
        view = c_void_p()
        check("vkCreateImageView", d.vkCreateImageView(self.device, byref(vci), None, byref(view)))
        self._objects.append(("ImageView", view))
        sub = vk.VkImageSubresource(aspect, 0, 0)
        lay = vk.VkSubresourceLayout()
        d.vkGetImageSubresourceLayout(self.device, h, byref(sub), byref(lay))
        img = Image(h, mem, view, width, height, fmt, host_visible, lay.rowPitch)
        img.samples = samples
        return img

    def read_image(self, img):
        n = img.pitch * img.height
        if img.host_visible:
            p = self.map(img)
            raw = np.ctypeslib.as_array((ctypes.c_uint8 * n).from_address(p)).copy()
        else:
            staging = self.create_buffer(n, 0, True)
            cb = self.begin()
            aspect = _aspect(img.format)
            region = vk.VkBufferImageCopy(0, 0, 0, vk.VkImageSubresourceLayers(aspect, 0, 0, 1),
                                          vk.VkOffset3D(0, 0, 0), vk.VkExtent3D(img.width, img.height, 1))
            self.drv.vkCmdCopyImageToBuffer(cb, img.handle, vk.IMAGE_LAYOUT_TRANSFER_SRC_OPTIMAL, staging.handle, 1,
                                            byref(region))
            self.end_submit_wait(cb)
            self.free_command_buffer(cb)
            p = self.map(staging)
            raw = np.ctypeslib.as_array((ctypes.c_uint8 * n).from_address(p)).copy()
            self.unmap(staging)
        # a host-visible image is read at its row pitch; a copy to a buffer packs rows tightly
        bpp = 2 if img.format == vk.FORMAT_D16_UNORM else 4
        ns = getattr(img, "samples", 1)
        if ns > 1:
            assert img.host_visible, "multisampled images are read through host-visible memory"
            raw = raw.reshape(img.height, img.pitch)[:, :img.width * bpp * ns].copy()
            if img.format == vk.FORMAT_D32_SFLOAT:
                return raw.view(np.float32).reshape(img.height, img.width, ns)
            return raw.reshape(img.height, img.width, ns, 4)
        raw = raw.reshape(img.height, img.pitch) if img.host_visible else raw[:img.height * img.width * bpp].reshape(
            img.height, img.width * bpp)
        if img.format == vk.FORMAT_D32_SFLOAT:
            return raw[:, :img.width * 4].copy().view(np.float32)
        if img.format == vk.FORMAT_D16_UNORM:
            return raw[:, :img.width * 2].copy().view(np.uint16)
        if img.format == vk.FORMAT_D24_UNORM_S8_UINT:
            return raw[:, :img.width * 4].copy().view(np.uint32)
        return raw[:, :img.width * 4].reshape(img.height, img.width, 4).copy()

    # ---------------------------------------------------------------------------------------------
    def begin(self):
        d = self.drv
        ai = vk.VkCommandBufferAllocateInfo(vk.ST_COMMAND_BUFFER_ALLOCATE_INFO, None, self.pool,
                                            vk.COMMAND_BUFFER_LEVEL_PRIMARY, 1)
        cb = c_void_p()
        check("vkAllocateCommandBuffers", d.vkAllocateCommandBuffers(self.device, byref(ai), byref(cb)))
        bi = vk.VkCommandBufferBeginInfo(vk.ST_COMMAND_BUFFER_BEGIN_INFO, None, 0, None)
        check("vkBeginCommandBuffer", d.vkBeginCommandBuffer(cb, byref(bi)))
        return cb

    def free_command_buffer(self, cb):
        self.drv.vkFreeCommandBuffers(self.device, self.pool, 1, byref(cb))

    def submit(self, cb, fence=None):
        arr = (c_void_p * 1)(cb)
        si = vk.VkSubmitInfo(vk.ST_SUBMIT_INFO, None, 0, None, None, 1, arr, 0, None)
        check("vkQueueSubmit", self.drv.vkQueueSubmit(self.queue, 1, byref(si), fence))

    def wait(self, timeout_ns=60_000_000_000):
        f = (c_void_p * 1)(self.fence)
        check("vkWaitForFences", self.drv.vkWaitForFences(self.device, 1, f, 1, timeout_ns))
        check("vkResetFences", self.drv.vkResetFences(self.device, 1, f))

    def submit_wait(self, cb):
        self.submit(cb, self.fence)
        self.wait()

    def end_submit_wait(self, cb):
        check("vkEndCommandBuffer", self.drv.vkEndCommandBuffer(cb))
        self.submit_wait(cb)

    # ---------------------------------------------------------------------------------------------
    def render_pass(self, color_fmt, depth, color_load=vk.LOAD_OP_CLEAR, depth_load=vk.LOAD_OP_CLEAR,
                    depth_fmt=vk.FORMAT_D32_SFLOAT, stencil_load=vk.LOAD_OP_CLEAR, samples=1):
        """colour (attachment 0) and depth (1) with `samples` samples; with 4 samples a single-sample resolve
        attachment (2) receives the colour at the end of the subpass"""
        atts = (vk.VkAttachmentDescription * 3)()
        atts[0] = vk.VkAttachmentDescription(0, color_fmt, samples, color_load, vk.STORE_OP_STORE, 2, 1,
                                             vk.IMAGE_LAYOUT_UNDEFINED, vk.IMAGE_LAYOUT_GENERAL)
        atts[1] = vk.VkAttachmentDescription(0, depth_fmt, samples, depth_load, vk.STORE_OP_STORE, stencil_load, 0,
                                             vk.IMAGE_LAYOUT_UNDEFINED, vk.IMAGE_LAYOUT_GENERAL)
        atts[2] = vk.VkAttachmentDescription(0, color_fmt, 1, vk.LOAD_OP_DONT_CARE, vk.STORE_OP_STORE, 2, 1,
                                             vk.IMAGE_LAYOUT_UNDEFINED, vk.IMAGE_LAYOUT_GENERAL)
        cref = vk.VkAttachmentReference(0, vk.IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL)
        dref = vk.VkAttachmentReference(1, vk.IMAGE_LAYOUT_DEPTH_STENCIL_ATTACHMENT_OPTIMAL)
        rref = vk.VkAttachmentReference(2, vk.IMAGE_LAYOUT_COLOR_ATTACHMENT_OPTIMAL)
        sp = vk.VkSubpassDescription(0, vk.BIND_POINT_GRAPHICS, 0, None, 1, pointer(cref),
                                     ctypes.cast(pointer(rref), c_void_p) if samples > 1 else None,
                                     pointer(dref) if depth else None, 0, None)
        rci = vk.VkRenderPassCreateInfo(vk.ST_RENDER_PASS_CREATE_INFO, None, 0,
                                        (2 if depth else 1) + (1 if samples > 1 else 0), atts, 1, pointer(sp), 0, None)
        h = c_void_p()
        check("vkCreateRenderPass", self.drv.vkCreateRenderPass(self.device, byref(rci), None, byref(h)))
        self._objects.append(("RenderPass", h))
        return h

    def framebuffer(self, rp, views, width, height):
        arr = (c_void_p * len(views))(*[v.value if isinstance(v, c_void_p) else v for v in views])
        fci = vk.VkFramebufferCreateInfo(vk.ST_FRAMEBUFFER_CREATE_INFO, None, 0, rp, len(views), arr, width, height, 1)
        h = c_void_p()
        check("vkCreateFramebuffer", self.drv.vkCreateFramebuffer(self.device, byref(fci), None, byref(h)))
        self._objects.append(("Framebuffer", h))
        return h

    def shader_module(self, words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        sci = vk.VkShaderModuleCreateInfo(vk.ST_SHADER_MODULE_CREATE_INFO, None, 0, w.nbytes, w.ctypes.data)
        h = c_void_p()
        check("vkCreateShaderModule", self.drv.vkCreateShaderModule(self.device, byref(sci), None, byref(h)))
        self._objects.append(("ShaderModule", h))
        return h

    def write_image(self, img, texels):
        """copy uint8 [h, w, 4] texels into a host-visible linear image, row by row at its pitch"""
        a = np.ascontiguousarray(texels, dtype=np.uint8)
        p = self.map(img)
        row = img.width * 4
        for y in range(img.height):
            ctypes.memmove(p + y * img.pitch, a[y].ctypes.data, row)
        self.unmap(img)

    # ---- samplers and descriptor sets ----
    def sampler(self, tex):
        """a VkSampler for scenes.Texture `tex` (min filter = mag filter)"""
        f = vk.FILTER_LINEAR if tex.linear else vk.FILTER_NEAREST
        ci = vk.VkSamplerCreateInfo(vk.ST_SAMPLER_CREATE_INFO, None, 0, f, f, 0, tex.address_u, tex.address_v,
                                    vk.ADDRESS_CLAMP_TO_EDGE, 0.0, 0, 1.0, 0, 0, 0.0, 0.0, 2 * tex.border,
                                    int(tex.unnormalized))
        h = c_void_p()
        check("vkCreateSampler", self.drv.vkCreateSampler(self.device, byref(ci), None, byref(h)))
        self._objects.append(("Sampler", h))
        return h

    def set_layout(self, bindings):
        """a descriptor set layout from [(binding, descriptor type, count)]"""
        arr = (vk.VkDescriptorSetLayoutBinding * len(bindings))(
            *[vk.VkDescriptorSetLayoutBinding(b, t, n, vk.SHADER_STAGE_VERTEX | vk.SHADER_STAGE_FRAGMENT, None)
              for b, t, n in bindings])
        ci = vk.VkDescriptorSetLayoutCreateInfo(vk.ST_DESCRIPTOR_SET_LAYOUT_CREATE_INFO, None, 0, len(bindings), arr)
        h = c_void_p()
        check("vkCreateDescriptorSetLayout", self.drv.vkCreateDescriptorSetLayout(self.device, byref(ci), None,
                                                                                  byref(h)))
        self._objects.append(("DescriptorSetLayout", h))
        return h

    def descriptor_sets(self, layout, n=1):
        """a pool holding `n` sets of `layout`; returns the sets"""
        sizes = (vk.VkDescriptorPoolSize * 3)(vk.VkDescriptorPoolSize(vk.DESCRIPTOR_COMBINED_IMAGE_SAMPLER, 64 * n),
                                              vk.VkDescriptorPoolSize(vk.DESCRIPTOR_UNIFORM_BUFFER, 64 * n),
                                              vk.VkDescriptorPoolSize(vk.DESCRIPTOR_UNIFORM_BUFFER_DYNAMIC, 64 * n))
        pci = vk.VkDescriptorPoolCreateInfo(vk.ST_DESCRIPTOR_POOL_CREATE_INFO, None, 0, n, 3, sizes)
        pool = c_void_p()
        check("vkCreateDescriptorPool", self.drv.vkCreateDescriptorPool(self.device, byref(pci), None, byref(pool)))
        self._objects.append(("DescriptorPool", pool))
        layouts = (c_void_p * n)(*([layout.value] * n))
        ai = vk.VkDescriptorSetAllocateInfo(vk.ST_DESCRIPTOR_SET_ALLOCATE_INFO, None, pool, n, layouts)
        sets = (c_void_p * n)()
        check("vkAllocateDescriptorSets", self.drv.vkAllocateDescriptorSets(self.device, byref(ai), sets))
        return [c_void_p(s) for s in sets]

    def write_image_descriptor(self, dset, binding, element, sampler, image, dtype=vk.DESCRIPTOR_COMBINED_IMAGE_SAMPLER):
        """a combined image sampler, or (dtype) a sampled image (sampler None) or a sampler (image None)"""
        ii = vk.VkDescriptorImageInfo(sampler, image.view if image is not None else None, vk.IMAGE_LAYOUT_GENERAL)
        w = vk.VkWriteDescriptorSet(vk.ST_WRITE_DESCRIPTOR_SET, None, dset, binding, element, 1,
                                    dtype, pointer(ii), None, None)
        self.drv.vkUpdateDescriptorSets(self.device, 1, byref(w), 0, None)

    def write_buffer_descriptor(self, dset, binding, buf, offset, size, dtype=vk.DESCRIPTOR_UNIFORM_BUFFER):
        bi = vk.VkDescriptorBufferInfo(buf.handle, offset, size)
        w = vk.VkWriteDescriptorSet(vk.ST_WRITE_DESCRIPTOR_SET, None, dset, binding, 0, 1, dtype, None, pointer(bi),
                                    None)
        self.drv.vkUpdateDescriptorSets(self.device, 1, byref(w), 0, None)

    def pipeline_layout(self, push_bytes, set_layouts=()):
        rng = vk.VkPushConstantRange(vk.SHADER_STAGE_VERTEX | vk.SHADER_STAGE_FRAGMENT, 0, push_bytes)
        sl = (c_void_p * max(1, len(set_layouts)))(*[s.value for s in set_layouts])
        lci = vk.VkPipelineLayoutCreateInfo(vk.ST_PIPELINE_LAYOUT_CREATE_INFO, None, 0, len(set_layouts),
                                            ctypes.cast(sl, c_void_p) if set_layouts else None,
                                            1 if push_bytes else 0, pointer(rng) if push_bytes else None)
        h = c_void_p()
        check("vkCreatePipelineLayout", self.drv.vkCreatePipelineLayout(self.device, byref(lci), None, byref(h)))
        self._objects.append(("PipelineLayout", h))
        return h

    def pipeline(self, scene, rp, layout, vs_words, fs_words, dynamic=(), instance_attr=None):
        """`dynamic`: VkDynamicState values the pipeline leaves to the command buffer; `instance_attr`:
        (location, format, stride) of an attribute read per instance from vertex binding 1"""
        vsm, fsm = self.shader_module(vs_words), self.shader_module(fs_words)
        stages = (vk.VkPipelineShaderStageCreateInfo * 2)()
        stages[0] = vk.VkPipelineShaderStageCreateInfo(vk.ST_PIPELINE_SHADER_STAGE_CREATE_INFO, None, 0,
                                                       vk.SHADER_STAGE_VERTEX, vsm, b"main", None)
        stages[1] = vk.VkPipelineShaderStageCreateInfo(vk.ST_PIPELINE_SHADER_STAGE_CREATE_INFO, None, 0,
                                                       vk.SHADER_STAGE_FRAGMENT, fsm, b"main", None)
        stride = scene.vertex_stride()
        binding = vk.VkVertexInputBindingDescription(0, stride, vk.VERTEX_INPUT_RATE_VERTEX)
        attrs = (vk.VkVertexInputAttributeDescription * 2)()
        if scene.shader == "color":
            attrs[0] = vk.VkVertexInputAttributeDescription(0, 0, vk.FORMAT_R32G32B32A32_SFLOAT, 0)
            attrs[1] = vk.VkVertexInputAttributeDescription(1, 0, vk.FORMAT_R32G32B32A32_SFLOAT, 16)
        elif scene.shader == "textured":
            attrs[0] = vk.VkVertexInputAttributeDescription(0, 0, vk.FORMAT_R32G32B32A32_SFLOAT, 0)
            attrs[1] = vk.VkVertexInputAttributeDescription(1, 0, vk.FORMAT_R32G32_SFLOAT, 16)
        else:
            attrs[0] = vk.VkVertexInputAttributeDescription(0, 0, vk.FORMAT_R32G32B32_SFLOAT, 0)
            attrs[1] = vk.VkVertexInputAttributeDescription(1, 0, vk.FORMAT_R32G32B32_SFLOAT, 12)
        nb, na = 1, 2
        if instance_attr is not None:
            loc, fmt, istride = instance_attr
            bindings = (vk.VkVertexInputBindingDescription * 2)(
                binding, vk.VkVertexInputBindingDescription(1, istride, vk.VERTEX_INPUT_RATE_INSTANCE))
            attrs3 = (vk.VkVertexInputAttributeDescription * 3)(
                attrs[0], attrs[1], vk.VkVertexInputAttributeDescription(loc, 1, fmt, 0))
            binding, attrs, nb, na = bindings, attrs3, 2, 3
        vis = vk.VkPipelineVertexInputStateCreateInfo(vk.ST_PIPELINE_VERTEX_INPUT_STATE_CREATE_INFO, None, 0, nb,
                                                      binding if nb > 1 else pointer(binding), na, attrs)
        ias = vk.VkPipelineInputAssemblyStateCreateInfo(vk.ST_PIPELINE_INPUT_ASSEMBLY_STATE_CREATE_INFO, None, 0,
                                                        vk.TOPOLOGY_TRIANGLE_LIST, 0)
        vp = vk.VkViewport(0.0, 0.0, float(scene.width), float(scene.height), 0.0, 1.0)
        sc = vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(scene.width, scene.height))
        vps = vk.VkPipelineViewportStateCreateInfo(vk.ST_PIPELINE_VIEWPORT_STATE_CREATE_INFO, None, 0, 1,
                                                   pointer(vp), 1, pointer(sc))
        rs = vk.VkPipelineRasterizationStateCreateInfo(vk.ST_PIPELINE_RASTERIZATION_STATE_CREATE_INFO, None, 0, 0, 0,
                                                       vk.POLYGON_MODE_FILL, scene.cull,
                                                       vk.FRONT_FACE_CCW if scene.front_ccw else vk.FRONT_FACE_CW,
                                                       0, 0.0, 0.0, 0.0, 1.0)
        ms = vk.VkPipelineMultisampleStateCreateInfo(vk.ST_PIPELINE_MULTISAMPLE_STATE_CREATE_INFO, None, 0,
                                                     scene.samples, 0, 0.0, None, 0, 0)
        faces = [vk.VkStencilOpState(), vk.VkStencilOpState()]
        if scene.stencil is not None:
            faces = [vk.VkStencilOpState(so.fail, so.pass_, so.depth_fail, so.compare, so.compare_mask, so.write_mask,
                                         so.reference) for so in (scene.stencil["front"], scene.stencil["back"])]
        ds = vk.VkPipelineDepthStencilStateCreateInfo(vk.ST_PIPELINE_DEPTH_STENCIL_STATE_CREATE_INFO, None, 0,
                                                      int(scene.depth_test), int(scene.depth_write),
                                                      scene.depth_compare, 0, int(scene.stencil is not None),
                                                      faces[0], faces[1], 0.0, 1.0)
        if scene.blend:
            att = vk.VkPipelineColorBlendAttachmentState(1, *scene.blend_factors(), scene.write_mask)
        else:
            att = vk.VkPipelineColorBlendAttachmentState(0, vk.BLEND_ONE, vk.BLEND_ZERO, vk.BLEND_OP_ADD,
                                                         vk.BLEND_ONE, vk.BLEND_ZERO, vk.BLEND_OP_ADD,
                                                         scene.write_mask)
        cbs = vk.VkPipelineColorBlendStateCreateInfo(vk.ST_PIPELINE_COLOR_BLEND_STATE_CREATE_INFO, None, 0, 0, 0, 1,
                                                     pointer(att), (c_float * 4)(*scene.blend_const))
        dyn_arr = (ctypes.c_int * max(1, len(dynamic)))(*dynamic)
        dyn = vk.VkPipelineDynamicStateCreateInfo(vk.ST_PIPELINE_DYNAMIC_STATE_CREATE_INFO, None, 0, len(dynamic),
                                                  dyn_arr)
        gci = vk.VkGraphicsPipelineCreateInfo(vk.ST_GRAPHICS_PIPELINE_CREATE_INFO, None, 0, 2, stages, pointer(vis),
                                              pointer(ias), None, pointer(vps), pointer(rs), pointer(ms), pointer(ds),
                                              pointer(cbs), pointer(dyn) if dynamic else None, layout, rp, 0, None, -1)
        h = c_void_p()
        check("vkCreateGraphicsPipelines",
              self.drv.vkCreateGraphicsPipelines(self.device, None, 1, byref(gci), None, byref(h)))
        self._objects.append(("Pipeline", h))
        return h


INDIRECT_STRIDE = 32  # bytes between the indirect commands of a SceneRun (larger than either command)


def indirect_commands(scene, instances=1):
    """the scene's draws as VkDrawIndirectCommand {vertexCount, instanceCount, firstVertex, firstInstance} or
    VkDrawIndexedIndirectCommand {indexCount, instanceCount, firstIndex, vertexOffset, firstInstance} words,
    one row of INDIRECT_STRIDE bytes per draw"""
    cmds = np.zeros((len(scene.draws), INDIRECT_STRIDE // 4), dtype=np.uint32)
    for i, dr in enumerate(scene.draws):
        if scene.indexed:
            cmds[i, :5] = [3 * dr.count, instances, dr.first, dr.vertex_offset & 0xFFFFFFFF, 0]
        else:
            cmds[i, :4] = [3 * dr.count, instances, dr.first, 0]
    return cmds


class SceneRun:
    """GPU resources and a recorded command buffer for one scene.

    indirect: None records vkCmdDraw / vkCmdDrawIndexed; "host" records the indirect variants over a
    host-visible buffer of commands written by the host; "device" over a device-local buffer that the same
    command buffer fills with vkCmdCopyBuffer before the render pass.  Draws with their own push constants
    become one indirect call each, the others one call of drawCount = len(draws).
    counts: with indirect, record the vkCmdDraw*IndirectCountKHR variants instead, with maxDrawCount as
    above and each call's draw count read from a host-visible buffer of one u32 per call (`counts` gives
    the initial words; the test rewrites them with write_buffer(run.count_buf, ...)).
    ubo_host_visible: the uniform buffer of a scene with `ubo` in host-visible memory (default: as
    host_visible).  buffers: (vertex buffer, index buffer) already holding the scene's data, shared instead
    of created.  vb_offset: bytes before the vertex data in its buffer (the vkCmdBindVertexBuffers offset)."""

    def __init__(self, r, scene, host_visible=False, mode=None, tile=None, keep_mapped=False, depth_host_visible=None,
                 indirect=None, counts=None, ubo_host_visible=None, buffers=None, vb_offset=0):
        self.r, self.scene = r, scene
        self.indirect = indirect
        d = r.drv
        if mode is not None:
            d.set_option("mode", mode)
        if tile is not None:
            d.set_option("tile", tile)
        self.vb_offset = vb_offset
        if buffers is not None:
            self.vb, self.ib = buffers
        else:
            # the vertex data starts `vb_offset` bytes into the buffer, where vkCmdBindVertexBuffers binds it
            data = np.ascontiguousarray(scene.vertices).view(np.uint8).ravel()
            if vb_offset:
                data = np.concatenate([np.zeros(vb_offset, np.uint8), data])
            self.vb = r.create_buffer(data.nbytes, vk.BUFFER_USAGE_VERTEX, host_visible)
            r.write_buffer(self.vb, data, keep_mapped=keep_mapped and host_visible)
            self.ib = None
            if scene.indexed:
                self.ib = r.create_buffer(scene.indices.nbytes, vk.BUFFER_USAGE_INDEX, host_visible)
                r.write_buffer(self.ib, scene.indices, keep_mapped=keep_mapped and host_visible)
        ns = scene.samples
        self.samples = None
        if ns > 1:
            # multisampled colour and depth in host-visible memory (read sample by sample by the tests); the
            # pass resolves the colour into self.color
            self.samples = r.create_image(scene.width, scene.height, vk.FORMAT_R8G8B8A8_UNORM,
                                          vk.IMAGE_USAGE_COLOR_ATTACHMENT, True, samples=ns)
        self.color = r.create_image(scene.width, scene.height, vk.COLOR_FORMATS[scene.color_format],
                                    vk.IMAGE_USAGE_COLOR_ATTACHMENT, host_visible)
        self.depth = r.create_image(scene.width, scene.height, vk.DEPTH_FORMATS[scene.depth_format],
                                    vk.IMAGE_USAGE_DEPTH_STENCIL_ATTACHMENT,
                                    (host_visible if depth_host_visible is None else depth_host_visible) or ns > 1,
                                    samples=ns)
        self.rp = r.render_pass(vk.COLOR_FORMATS[scene.color_format], True, depth_fmt=vk.DEPTH_FORMATS[scene.depth_format],
                                samples=ns)
        views = [self.samples.view, self.depth.view, self.color.view] if ns > 1 else [self.color.view, self.depth.view]
        self.fb = r.framebuffer(self.rp, views, scene.width, scene.height)
        # descriptor sets: the textured scene's sampler2D, or the Lambert matrices in a uniform buffer (one
        # 256-byte slot per draw, selected by a dynamic offset)
        self.set_layouts, self.dsets, self.ubo_buf, self.tex_image = [], [], None, None
        if scene.texture is not None:
            t = scene.texture
            th, tw = t.texels.shape[:2]
            self.tex_image = r.create_image(tw, th, vk.FORMAT_B8G8R8A8_UNORM if t.bgra else vk.FORMAT_R8G8B8A8_UNORM,
                                            vk.IMAGE_USAGE_SAMPLED, True)
            r.write_image(self.tex_image, t.texels)
            self.set_layouts = [r.set_layout([(0, vk.DESCRIPTOR_COMBINED_IMAGE_SAMPLER, 1)])]
            self.dsets = r.descriptor_sets(self.set_layouts[0])
            r.write_image_descriptor(self.dsets[0], 0, 0, r.sampler(t), self.tex_image)
        elif scene.ubo:
            mats = np.zeros((max(1, len(scene.draws)), 64), dtype=np.float32)
            for i, dr in enumerate(scene.draws):
                if dr.mvp is not None:
                    mats[i, :16] = dr.mvp
            self.ubo_buf = r.create_buffer(mats.nbytes, vk.BUFFER_USAGE_UNIFORM,
                                           host_visible if ubo_host_visible is None else ubo_host_visible)
            r.write_buffer(self.ubo_buf, mats)
            self.set_layouts = [r.set_layout([(0, vk.DESCRIPTOR_UNIFORM_BUFFER_DYNAMIC, 1)])]
            self.dsets = r.descriptor_sets(self.set_layouts[0])
            r.write_buffer_descriptor(self.dsets[0], 0, self.ubo_buf, 0, 64, vk.DESCRIPTOR_UNIFORM_BUFFER_DYNAMIC)
        push = 64 if scene.shader == "lambert" and not scene.ubo else 0
        self.layout = r.pipeline_layout(push, self.set_layouts)
        vs, fs = scene.shaders()
        self.pipe = r.pipeline(scene, self.rp, self.layout, vs, fs)
        self.cmds = self.cmd_staging = self.count_buf = None
        if indirect is not None and counts is not None:
            words = np.ascontiguousarray(counts, dtype=np.uint32).ravel()
            self.count_buf = r.create_buffer(words.nbytes, vk.BUFFER_USAGE_INDIRECT, True)
            r.write_buffer(self.count_buf, words)
        if indirect is not None:
            words = indirect_commands(scene)
            self.cmds = r.create_buffer(words.nbytes, vk.BUFFER_USAGE_INDIRECT, indirect == "host")
            if indirect == "host":
                r.write_buffer(self.cmds, words)
            else:
                self.cmd_staging = r.create_buffer(words.nbytes, vk.BUFFER_USAGE_TRANSFER_SRC, True)
                r.write_buffer(self.cmd_staging, words)
        self.cb = self.record()

    def record(self):
        r, s, d = self.r, self.scene, self.r.drv
        cb = r.begin()
        if self.cmd_staging is not None:
            region = vk.VkBufferCopy(0, 0, self.cmds.size)
            d.vkCmdCopyBuffer(cb, self.cmd_staging.handle, self.cmds.handle, 1, byref(region))
        clears = (vk.VkClearValue * 2)()
        clears[0].color.float32[:] = list(s.clear_color)
        clears[1].depthStencil.depth = s.clear_depth
        clears[1].depthStencil.stencil = s.clear_stencil
        rbi = vk.VkRenderPassBeginInfo(vk.ST_RENDER_PASS_BEGIN_INFO, None, self.rp, self.fb,
                                       vk.VkRect2D(vk.VkOffset2D(0, 0), vk.VkExtent2D(s.width, s.height)), 2, clears)
        d.vkCmdBeginRenderPass(cb, byref(rbi), vk.SUBPASS_CONTENTS_INLINE)
        d.vkCmdBindPipeline(cb, vk.BIND_POINT_GRAPHICS, self.pipe)
        if self.dsets and not s.ubo:
            sets = (c_void_p * 1)(self.dsets[0].value)
            d.vkCmdBindDescriptorSets(cb, vk.BIND_POINT_GRAPHICS, self.layout, 0, 1, sets, 0, None)
        bufs = (c_void_p * 1)(self.vb.handle.value)
        offs = (c_uint64 * 1)(self.vb_offset)
        d.vkCmdBindVertexBuffers(cb, 0, 1, bufs, offs)
        if self.ib is not None:
            d.vkCmdBindIndexBuffer(cb, self.ib.handle, 0, vk.INDEX_TYPE_UINT32)
        per_draw_push = any(dr.mvp is not None for dr in s.draws)
        if self.indirect is not None and not per_draw_push:
            self._indirect_call(cb, 0, 0, len(s.draws))
        for i, dr in enumerate(s.draws):
            if self.indirect is not None and not per_draw_push:
                break
            if dr.mvp is not None and s.ubo:
                sets = (c_void_p * 1)(self.dsets[0].value)
                offs = (c_uint32 * 1)(256 * i)
                d.vkCmdBindDescriptorSets(cb, vk.BIND_POINT_GRAPHICS, self.layout, 0, 1, sets, 1, offs)
            elif dr.mvp is not None:
                m = np.ascontiguousarray(dr.mvp, dtype=np.float32)
                d.vkCmdPushConstants(cb, self.layout, vk.SHADER_STAGE_VERTEX, 0, 64, m.ctypes.data)
            if self.indirect is not None:
                self._indirect_call(cb, i, i * INDIRECT_STRIDE, 1)
            elif s.indexed:
                d.vkCmdDrawIndexed(cb, 3 * dr.count, 1, dr.first, dr.vertex_offset, 0)
            else:
                d.vkCmdDraw(cb, 3 * dr.count, 1, dr.first, 0)
        d.vkCmdEndRenderPass(cb)
        check("vkEndCommandBuffer", d.vkEndCommandBuffer(cb))
        return cb

    def _indirect_call(self, cb, call, offset, draws):
        d, s = self.r.drv, self.scene
        if self.count_buf is None:
            fn = d.vkCmdDrawIndexedIndirect if s.indexed else d.vkCmdDrawIndirect
            fn(cb, self.cmds.handle, offset, draws, INDIRECT_STRIDE)
        else:
            fn = d.vkCmdDrawIndexedIndirectCountKHR if s.indexed else d.vkCmdDrawIndirectCountKHR
            fn(cb, self.cmds.handle, offset, self.count_buf.handle, 4 * call, draws, INDIRECT_STRIDE)

    def submit(self, wait=True):
        if wait:
            self.r.submit_wait(self.cb)
        else:
            self.r.submit(self.cb)

    def read(self):
        """(colour bytes in R, G, B, A order whatever the attachment's byte order, depth texels)"""
        color = self.r.read_image(self.color)
        if self.scene.color_format.startswith("bgra"):
            color = color[..., [2, 1, 0, 3]].copy()
        return color, self.r.read_image(self.depth)

    def stats(self):
        return self.r.drv.stats(self.cb)

"""ctypes binding of the shader backend's C ABI (include/kz_shader_backend.h), part of libkazan_driver.so:
SPIR-V -> IR (kzShaderCompile), IR -> PTX (kzShaderEmitPtx), PTX + pipeline kernels -> sm_103a image
(kzShaderLink), and the SPIR-V text dump (kzSpirvDisassemble)."""
import ctypes
from ctypes import POINTER, c_char_p, c_size_t, c_uint32, c_void_p

import numpy as np

from . import vk

VERTEX, FRAGMENT = 0, 4


class KzShaderInfo(ctypes.Structure):
    _fields_ = [(n, c_uint32) for n in ("stage", "input_locations", "pos_input_locations", "output_slots",
                                        "input_slots", "flat_slots", "noperspective_slots", "writes_position",
                                        "writes_color", "discards", "push_bytes", "ir_instructions",
                                        "ir_registers", "color_passthrough")]


class KzVertexInputLayout(ctypes.Structure):
    _fields_ = [("num_attrs", c_uint32), ("location", c_uint32 * 8), ("binding", c_uint32 * 8),
                ("format", c_uint32 * 8), ("offset", c_uint32 * 8), ("stride", c_uint32 * 8), ("instanced", c_uint32)]


class KzShaderBinding(ctypes.Structure):
    _fields_ = [(n, c_uint32) for n in ("set", "binding", "kind", "count", "bytes")]


class KzDescriptorSlots(ctypes.Structure):
    _fields_ = [("slot", (c_uint32 * 16) * 4)]


class ShaderError(RuntimeError):
    pass


_LIB = None


def lib(path=None):
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(path or vk.DRIVER_PATH)
        L.kzShaderCompile.argtypes = [c_void_p, c_size_t, c_uint32, c_char_p, c_void_p, c_void_p, c_uint32,
                                      POINTER(c_void_p), c_char_p, c_size_t]
        L.kzShaderCompile.restype = ctypes.c_int
        L.kzShaderInfo.argtypes = [c_void_p, POINTER(KzShaderInfo)]
        L.kzShaderDestroy.argtypes = [c_void_p]
        L.kzShaderEmitPtx.argtypes = [POINTER(c_void_p), POINTER(c_void_p), POINTER(KzVertexInputLayout), c_uint32,
                                      c_char_p, c_size_t]
        L.kzShaderEmitPtx.restype = c_size_t
        L.kzShaderEmitPtxDescriptors.argtypes = [POINTER(c_void_p), POINTER(c_void_p), POINTER(KzVertexInputLayout),
                                                 POINTER(KzDescriptorSlots), c_uint32, c_char_p, c_size_t]
        L.kzShaderEmitPtxDescriptors.restype = c_size_t
        L.kzShaderBindings.argtypes = [c_void_p, POINTER(KzShaderBinding), c_uint32]
        L.kzShaderBindings.restype = c_uint32
        L.kzShaderLink.argtypes = [c_char_p, c_void_p, c_size_t, POINTER(c_void_p), c_char_p, c_size_t]
        L.kzShaderLink.restype = ctypes.c_int
        L.kzCompiledCodeImage.argtypes = [c_void_p, POINTER(c_size_t)]
        L.kzCompiledCodeImage.restype = c_void_p
        L.kzCompiledCodeDestroy.argtypes = [c_void_p]
        L.kzSpirvDisassemble.argtypes = [c_void_p, c_size_t, c_char_p, c_size_t]
        L.kzSpirvDisassemble.restype = c_size_t
        _LIB = L
    return _LIB


class Shader:
    def __init__(self, words, stage, entry="main", spec=None):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        spec = spec or {}
        ids = (c_uint32 * max(1, len(spec)))(*spec.keys())
        vals = (c_uint32 * max(1, len(spec)))(*spec.values())
        err = ctypes.create_string_buffer(512)
        h = c_void_p()
        rc = lib().kzShaderCompile(w.ctypes.data, w.size, stage, entry.encode(), ids, vals, len(spec), ctypes.byref(h),
                                   err, 512)
        if rc != 0:
            raise ShaderError(err.value.decode())
        self.handle = h

    def bindings(self):
        """[(set, binding, kind, count, bytes)] of the descriptors the stage declares"""
        n = lib().kzShaderBindings(self.handle, None, 0)
        arr = (KzShaderBinding * max(1, n))()
        lib().kzShaderBindings(self.handle, arr, n)
        return [(b.set, b.binding, b.kind, b.count, b.bytes) for b in arr[:n]]

    def info(self):
        i = KzShaderInfo()
        lib().kzShaderInfo(self.handle, ctypes.byref(i))
        return {k: int(getattr(i, k)) for k, _ in KzShaderInfo._fields_}

    def __del__(self):
        if getattr(self, "handle", None):
            lib().kzShaderDestroy(self.handle)
            self.handle = None


def layout(attrs, strides, instanced=0):
    """attrs: list of (location, binding, format, offset)"""
    lay = KzVertexInputLayout()
    lay.num_attrs = len(attrs)
    for k, (loc, b, f, off) in enumerate(attrs):
        lay.location[k], lay.binding[k], lay.format[k], lay.offset[k] = loc, b, f, off
    for b, s in enumerate(strides):
        lay.stride[b] = s
    lay.instanced = instanced
    return lay


def descriptor_slots(mapping):
    """KzDescriptorSlots from {(set, binding): slot}"""
    d = KzDescriptorSlots()
    for s in range(4):
        for b in range(16):
            d.slot[s][b] = mapping.get((s, b), 0xFFFFFFFF)
    return d


def emit_ptx(pairs, layouts=None, slots=None):
    """pairs: list of (vertex Shader, fragment Shader or None); slots: per pair, {(set, binding): slot}"""
    n = len(pairs)
    vs = (c_void_p * n)(*[p[0].handle.value for p in pairs])
    fs = (c_void_p * n)(*[(p[1].handle.value if p[1] is not None else None) for p in pairs])
    lays = (KzVertexInputLayout * n)(*layouts) if layouts else None
    ds = (KzDescriptorSlots * n)(*[descriptor_slots(m) for m in slots]) if slots else None
    size = lib().kzShaderEmitPtxDescriptors(vs, fs, lays, ds, n, None, 0)
    buf = ctypes.create_string_buffer(size)
    lib().kzShaderEmitPtxDescriptors(vs, fs, lays, ds, n, buf, size)
    return buf.value.decode()


def link(ptx, pipeline_object=None):
    """returns the linked sm_103a image (bytes)"""
    err = ctypes.create_string_buffer(4096)
    h = c_void_p()
    if pipeline_object is None:
        rc = lib().kzShaderLink(ptx.encode(), None, 0, ctypes.byref(h), err, 4096)
    else:
        rc = lib().kzShaderLink(ptx.encode(), pipeline_object, len(pipeline_object), ctypes.byref(h), err, 4096)
    if rc != 0:
        raise ShaderError(err.value.decode())
    n = c_size_t()
    p = lib().kzCompiledCodeImage(h, ctypes.byref(n))
    img = ctypes.string_at(p, n.value)
    lib().kzCompiledCodeDestroy(h)
    return img


def disassemble(words):
    w = np.ascontiguousarray(words, dtype=np.uint32)
    n = lib().kzSpirvDisassemble(w.ctypes.data, w.size, None, 0)
    if n == 0:
        raise ShaderError("invalid SPIR-V module")
    buf = ctypes.create_string_buffer(n)
    lib().kzSpirvDisassemble(w.ctypes.data, w.size, buf, n)
    return buf.value.decode()

"""Python binding of the CPU oracle (kz_oracle.c).  TEST INFRASTRUCTURE ONLY.

Used by the tests, the smoke check and the CPU-baseline leg of bench.py as the checker; the driver never
loads it.  PARITY UNPINNED: the reference driver has no rasteriser (vulkan-driver/src/api_impl.rs:4632-4653
are `unimplemented!()`), so this oracle restates the Vulkan specification's rules (see kz_oracle.h).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkz_oracle.so")

SHADER = {"color": 0, "lambert": 1, "textured": 2}


class KzoTexture(ctypes.Structure):
    _fields_ = [("texels", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("pitch", ctypes.c_uint32), ("format", ctypes.c_uint32), ("sampler", ctypes.c_uint32)]


class KzoStencil(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("fail_op", "pass_op", "depth_fail_op", "compare_op", "compare_mask",
                                                "write_mask", "reference")]


DEPTH_FORMAT = {"d32": 0, "d16": 1, "d24s8": 2}


class KzoDraw(ctypes.Structure):
    _fields_ = [("shader", ctypes.c_uint32), ("vertices", ctypes.c_void_p), ("indices", ctypes.c_void_p),
                ("first", ctypes.c_uint32), ("vertex_offset", ctypes.c_int32), ("tri_count", ctypes.c_uint32),
                ("mvp", ctypes.c_float * 16), ("albedo", ctypes.c_float * 3), ("light", ctypes.c_float * 3),
                ("cull_mode", ctypes.c_uint32), ("front_ccw", ctypes.c_uint32), ("depth_test", ctypes.c_uint32),
                ("depth_write", ctypes.c_uint32), ("depth_compare", ctypes.c_uint32),
                ("blend_enable", ctypes.c_uint32), ("src_color", ctypes.c_uint32), ("dst_color", ctypes.c_uint32),
                ("color_op", ctypes.c_uint32), ("src_alpha", ctypes.c_uint32), ("dst_alpha", ctypes.c_uint32),
                ("alpha_op", ctypes.c_uint32), ("write_mask", ctypes.c_uint32), ("blend_const", ctypes.c_float * 4),
                ("viewport", ctypes.c_float * 6), ("scissor", ctypes.c_int32 * 4), ("tex", KzoTexture),
                ("stencil_test", ctypes.c_uint32), ("front", KzoStencil), ("back", KzoStencil),
                ("samples", ctypes.c_uint32), ("srgb", ctypes.c_uint32)]


class KzoStats(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_uint64), ("rejected", ctypes.c_uint64), ("clipped", ctypes.c_uint64),
                ("subtris", ctypes.c_uint64), ("fragments", ctypes.c_uint64), ("depth_pass", ctypes.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.kzo_render.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32, ctypes.POINTER(KzoDraw),
                                 ctypes.c_int, ctypes.POINTER(KzoStats)]
        L.kzo_render.restype = ctypes.c_int
        L.kzo_tex2d.argtypes = [ctypes.POINTER(KzoTexture), ctypes.c_float, ctypes.c_float,
                                ctypes.POINTER(ctypes.c_float)]
        L.kzo_render_ds.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32,
                                    ctypes.POINTER(KzoDraw), ctypes.c_int, ctypes.POINTER(KzoStats)]
        L.kzo_render_ds.restype = ctypes.c_int
        L.kzo_resolve.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        L.kzo_depth_value.argtypes = [ctypes.c_float, ctypes.c_uint32]
        L.kzo_depth_value.restype = ctypes.c_float
        L.kzo_unorm8.argtypes = [ctypes.c_float]
        L.kzo_unorm8.restype = ctypes.c_uint8
        L.kzo_clear_color.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_float)]
        L.kzo_clear_color_srgb.argtypes = L.kzo_clear_color.argtypes
        L.kzo_srgb8.argtypes = [ctypes.c_float]
        L.kzo_srgb8.restype = ctypes.c_uint8
        L.kzo_clear_depth.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                      ctypes.c_float]
        _LIB = L
    return _LIB


def texture_struct(t):
    """KzoTexture of a kazan_gb300.scenes.Texture (its texel array must stay alive)"""
    a = t.texels
    assert a.dtype == np.uint8 and a.flags.c_contiguous and a.ndim == 3 and a.shape[2] == 4
    return KzoTexture(a.ctypes.data, a.shape[1], a.shape[0], a.shape[1] * 4, 2 if t.bgra else 1, t.sampler_bits())


def tex2d(t, s, tc):
    """kzo_tex2d: the oracle's sample of Texture t at (s, tc), as float32 [4]"""
    ts = texture_struct(t)
    out = (ctypes.c_float * 4)()
    lib().kzo_tex2d(ctypes.byref(ts), float(s), float(tc), out)
    return np.array(out[:], dtype=np.float32)


def unorm8(v):
    return int(lib().kzo_unorm8(float(v)))


def clear_images(scene):
    """cleared colour and depth planes; the depth plane holds what the depth test compares (see kz_oracle.h)"""
    w, h = scene.width, scene.height
    color = np.empty((h, w, 4), dtype=np.uint8)
    depth = np.empty((h, w), dtype=np.float32)
    rect = (ctypes.c_int32 * 4)(0, 0, w, h)
    clear = lib().kzo_clear_color_srgb if getattr(scene, "srgb", False) else lib().kzo_clear_color
    clear(w, color.ctypes.data, rect, (ctypes.c_float * 4)(*scene.clear_color))
    fmt = DEPTH_FORMAT[scene.depth_format]
    lib().kzo_clear_depth(w, depth.ctypes.data, rect, lib().kzo_depth_value(scene.clear_depth, fmt))
    return color, depth


def packed_depth(depth, stencil, depth_format):
    """the depth attachment's texels from the oracle's planes: float32 (d32), uint16 (d16), or uint32 with the
    depth in bits 0..23 and the stencil in bits 24..31 (d24s8)"""
    if depth_format == "d16":
        return depth.astype(np.uint16)
    if depth_format == "d24s8":
        return depth.astype(np.uint32) | (stencil.astype(np.uint32) << 24)
    return depth


def make_draws(scene, draws=None):
    from kazan_gb300 import spirv_asm
    draws = scene.draws if draws is None else draws
    arr = (KzoDraw * max(1, len(draws)))()
    for i, d in enumerate(draws):
        k = arr[i]
        k.shader = SHADER[scene.shader]
        k.vertices = scene.vertices.ctypes.data
        k.indices = scene.indices.ctypes.data if scene.indices is not None else None
        k.first = d.first
        k.vertex_offset = d.vertex_offset
        k.tri_count = d.count
        if d.mvp is not None:
            k.mvp[:] = [float(x) for x in d.mvp]
        k.albedo[:] = [float(x) for x in spirv_asm.ALBEDO]
        k.light[:] = [float(x) for x in spirv_asm.LIGHT]
        k.cull_mode = scene.cull
        k.front_ccw = int(scene.front_ccw)
        k.depth_test = int(scene.depth_test)
        k.depth_write = int(scene.depth_write)
        k.depth_compare = scene.depth_compare
        k.blend_enable = int(scene.blend)
        k.src_color, k.dst_color, k.color_op, k.src_alpha, k.dst_alpha, k.alpha_op = scene.blend_factors()
        k.write_mask = scene.write_mask
        k.blend_const[:] = [float(x) for x in scene.blend_const]
        k.viewport[:] = [0.0, 0.0, float(scene.width), float(scene.height), 0.0, 1.0]
        k.scissor[:] = [0, 0, scene.width, scene.height]
        if scene.texture is not None:
            k.tex = texture_struct(scene.texture)
        k.samples = scene.samples
        k.srgb = int(getattr(scene, "srgb", False))
        if scene.stencil is not None:
            k.stencil_test = 1
            for face in ("front", "back"):
                so = scene.stencil[face]
                setattr(k, face, KzoStencil(so.fail, so.pass_, so.depth_fail, so.compare, so.compare_mask,
                                            so.write_mask, so.reference))
    return arr, len(draws)


def render_ms(scene, threads=1):
    """a 4x multisampled scene: (colour samples uint8 [H, W, 4, 4], depth samples float32 [H, W, 4], resolved
    colour uint8 [H, W, 4], stats)"""
    assert scene.samples == 4 and scene.depth_format == "d32"
    c1, d1 = clear_images(scene)
    color4 = np.ascontiguousarray(np.repeat(c1[:, :, None, :], 4, axis=2))
    depth4 = np.ascontiguousarray(np.repeat(d1[:, :, None], 4, axis=2))
    arr, n = make_draws(scene)
    st = KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, scene.width, scene.height)
    rc = lib().kzo_render_ds(scene.width, scene.height, color4.ctypes.data, depth4.ctypes.data, None, 0, area, n, arr,
                             threads, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("oracle failed")
    resolved = np.empty((scene.height, scene.width, 4), dtype=np.uint8)
    lib().kzo_resolve(scene.width, scene.height, color4.ctypes.data, resolved.ctypes.data)
    return color4, depth4, resolved, st.as_dict()


def render(scene, threads=1, draws=None, color=None, depth=None):
    """Render `scene` (a kazan_gb300.scenes.Scene) from cleared attachments; returns
    (color uint8 [H, W, 4], depth attachment texels [H, W] (float32 for d32, see packed_depth), stats dict)."""
    if scene.samples == 4:
        _, depth4, resolved, st = render_ms(scene, threads)
        return resolved, depth4, st
    if color is None or depth is None:
        color, depth = clear_images(scene)
    arr, n = make_draws(scene, draws)
    st = KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, scene.width, scene.height)
    stencil = None
    if scene.depth_format == "d24s8":
        stencil = np.full((scene.height, scene.width), scene.clear_stencil & 0xFF, dtype=np.uint8)
    rc = lib().kzo_render_ds(scene.width, scene.height, color.ctypes.data, depth.ctypes.data,
                             stencil.ctypes.data if stencil is not None else None, DEPTH_FORMAT[scene.depth_format],
                             area, n, arr, threads, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("oracle failed")
    return color, packed_depth(depth, stencil, scene.depth_format), st.as_dict()

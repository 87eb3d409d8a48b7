"""Seeded synthetic scenes of the draw-path workloads (generators in csrc/scene/kz_scene.c).

  small_soup      256x256, 2,048 non-indexed triangles, clip-space positions, pass-through colour shader,
                  depth LESS with writes, no culling, no blending (seed 1)
  single_large    1920x1080, 1,000,000 indexed triangles of a jittered latitude/longitude sphere mesh,
                  MVP push constant, Lambert fragment shader, back-face culling (seed 2)
  batched         2048x2048, 4,096 indexed draws with log-uniform triangle counts in [16, 65536], each its
                  own sphere mesh and MVP (random rotation, translation in [-5,5]^3) (seed 3)
  ordered_blend   1920x1080, 200,000 triangles with log-uniform pixel area in [4, 4096], alpha 0.5,
                  SRC_ALPHA / ONE_MINUS_SRC_ALPHA blending, depth LESS with writes off (seed 4)
Each generator takes its size parameters so tests can run the same scene family at smaller sizes.
"""
import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import spirv_asm

PKG = os.path.dirname(os.path.abspath(__file__))
_LIB = None

# camera distance of the single-large-draw sphere (kz_scene.c kz_mvp_single): the triangles that are
# rasterised -- front facing and at least partly inside the view frustum, 141,932 of the 1,000,000 -- then
# average 8.0 pixels of screen area on 1920x1080 (visible_triangles)
SINGLE_DISTANCE = 1.815


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(PKG, "_build", "libkz_scene.so")
        if not os.path.exists(path):
            raise RuntimeError("libkz_scene.so is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(path)
        f32p = ctypes.POINTER(ctypes.c_float)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.kz_scene_soup.argtypes = [ctypes.c_uint64, ctypes.c_uint32, f32p]
        L.kz_scene_blend.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_float, f32p]
        L.kz_mesh_dims.argtypes = [ctypes.c_uint32, u32p, u32p]
        L.kz_mesh_vertex_count.argtypes = [ctypes.c_uint32]
        L.kz_mesh_vertex_count.restype = ctypes.c_uint32
        L.kz_mesh_sphere.argtypes = [ctypes.c_uint64, ctypes.c_uint32, f32p, u32p]
        L.kz_mvp_single.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, f32p]
        L.kz_mvp_batched.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, f32p]
        L.kz_batched_counts.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, u32p]
        L.kz_batched_counts.restype = ctypes.c_uint64
        L.kz_rng_floats.argtypes = [ctypes.c_uint64, ctypes.c_uint32, f32p]
        L.kz_rng_first.argtypes = [ctypes.c_uint64]
        L.kz_rng_first.restype = ctypes.c_uint32
        _LIB = L
    return _LIB


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _up(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


@dataclass
class Draw:
    first: int                 # firstVertex (non-indexed) or firstIndex (indexed)
    count: int                 # triangles
    vertex_offset: int = 0     # vkCmdDrawIndexed vertexOffset
    mvp: Optional[np.ndarray] = None  # column-major float32[16] push constant (Lambert)


@dataclass
class StencilOp:
    """VkStencilOpState: VkStencilOp values and a VkCompareOp"""
    fail: int = 0
    pass_: int = 0
    depth_fail: int = 0
    compare: int = 7             # ALWAYS
    compare_mask: int = 0xFF
    write_mask: int = 0xFF
    reference: int = 0


@dataclass
class Texture:
    """a combined image sampler of one mip level: texels uint8 [h, w, 4] in the image's byte order"""
    texels: np.ndarray
    bgra: bool = False            # VK_FORMAT_B8G8R8A8_UNORM (else R8G8B8A8_UNORM)
    linear: bool = False          # VK_FILTER_LINEAR for both min and mag (else NEAREST)
    address_u: int = 0            # VkSamplerAddressMode
    address_v: int = 0
    border: int = 0               # 0 transparent black, 1 opaque black, 2 opaque white
    unnormalized: bool = False

    def sampler_bits(self):
        """KzSamplerBits (kz_raster_abi.h)"""
        return (int(self.linear) | (int(self.unnormalized) << 1) | (self.address_u << 4) | (self.address_v << 8) |
                (self.border << 12))


@dataclass
class Scene:
    name: str
    width: int
    height: int
    shader: str                # "color", "lambert" or "textured"
    vertices: np.ndarray       # float32 [V, 8] (color) or [V, 6] (lambert)
    indices: Optional[np.ndarray]
    draws: List[Draw]
    cull: int = 0
    front_ccw: bool = True
    depth_test: bool = True
    depth_write: bool = True
    depth_compare: int = 1     # VK_COMPARE_OP_LESS
    blend: bool = False
    blend_state: Optional[tuple] = None  # with blend: (srcColor, dstColor, colorOp, srcAlpha, dstAlpha, alphaOp) as
                                         # VkBlendFactor / VkBlendOp; None: SRC_ALPHA, ONE_MINUS_SRC_ALPHA, ADD
    blend_const: tuple = (0.0, 0.0, 0.0, 0.0)  # VkPipelineColorBlendStateCreateInfo::blendConstants
    write_mask: int = 0xF      # VkColorComponentFlags of the colour attachment
    clear_color: tuple = (0.0, 0.0, 0.0, 1.0)
    clear_depth: float = 1.0
    fs_words: Optional[np.ndarray] = field(default=None, repr=False)  # overrides the default fragment shader
    vs_words: Optional[np.ndarray] = field(default=None, repr=False)  # overrides the default vertex shader
    texture: Optional[Texture] = None  # "textured": the fragment shader's sampler2D (set 0, binding 0)
    ubo: bool = False          # "lambert": the matrices come from a uniform buffer (set 0, binding 0, dynamic
                               # offset per draw) instead of push constants
    depth_format: str = "d32"  # "d32" (D32_SFLOAT), "d16" (D16_UNORM) or "d24s8" (D24_UNORM_S8_UINT)
    stencil: Optional[dict] = None  # stencil test: {"front": StencilOp, "back": StencilOp} (d24s8 only)
    clear_stencil: int = 0
    samples: int = 1           # 1, or 4: multisampled colour and depth attachments, resolved at the end of the pass
    color_format: str = "rgba8"  # colour attachment: "rgba8", "bgra8", "rgba8_srgb" or "bgra8_srgb" (the sRGB
                                 # formats store sRGB-encoded red, green and blue)

    def blend_factors(self):
        """(srcColor, dstColor, colorOp, srcAlpha, dstAlpha, alphaOp) of the colour attachment's blend state"""
        return tuple(int(x) for x in self.blend_state) if self.blend_state is not None else (6, 7, 0, 6, 7, 0)

    @property
    def srgb(self):
        return self.color_format.endswith("_srgb")

    @property
    def triangles(self):
        return sum(d.count for d in self.draws)

    @property
    def indexed(self):
        return self.indices is not None

    def vertex_stride(self):
        return self.vertices.shape[1] * 4

    def shaders(self):
        if self.shader == "color":
            vs, fs = spirv_asm.color_vs(), spirv_asm.color_fs()
        elif self.shader == "textured":
            vs, fs = spirv_asm.textured_vs(), spirv_asm.textured_fs()
        else:
            vs, fs = spirv_asm.lambert_ubo_vs() if self.ubo else spirv_asm.lambert_vs(), spirv_asm.lambert_fs()
        if self.fs_words is not None:
            fs = self.fs_words
        if self.vs_words is not None:
            vs = self.vs_words
        return vs, fs

    def algorithmic_bytes(self):
        """algorithmic HBM bytes of one submission: 12 B of indices per indexed triangle, the vertex stride
        per vertex, 64 B of push constants per draw, and the framebuffer read and written once (colour and
        depth 4 B each per pixel; depth read but not written when depth writes are off)"""
        t_idx = self.triangles if self.indexed else 0
        v = len(self.vertices) if self.indexed else 3 * self.triangles
        push = 64 * len(self.draws) if self.shader == "lambert" else 0
        fb = self.width * self.height * ((4 + 4) * 2 if self.depth_write else (2 * 4 + 4))
        return 12 * t_idx + self.vertex_stride() * v + push + fb


def small_soup(seed=1, n=2048, width=256, height=256):
    v = np.empty((3 * n, 8), dtype=np.float32)
    lib().kz_scene_soup(seed, n, _fp(v))
    return Scene("small_soup", width, height, "color", v, None, [Draw(0, n)], cull=0)


def sphere_mesh(seed, tris):
    nv = lib().kz_mesh_vertex_count(tris)
    v = np.empty((nv, 6), dtype=np.float32)
    idx = np.empty(3 * tris, dtype=np.uint32)
    lib().kz_mesh_sphere(seed, tris, _fp(v), _up(idx))
    return v, idx


def mvp_single(width, height, dist=SINGLE_DISTANCE):
    m = np.empty(16, dtype=np.float32)
    lib().kz_mvp_single(width, height, dist, _fp(m))
    return m


def single_large(seed=2, tris=1_000_000, width=1920, height=1080, dist=SINGLE_DISTANCE):
    v, idx = sphere_mesh(seed, tris)
    return Scene("single_large", width, height, "lambert", v, idx,
                 [Draw(0, tris, 0, mvp_single(width, height, dist))], cull=2)


def visible_triangles(scene):
    """(count, mean screen area in pixels) of the triangles of an indexed Lambert scene that can be rasterised:
    front facing (counter-clockwise in framebuffer coordinates, y down) with all vertices in front of the eye
    and not all outside one plane of the view frustum.  A float64 restatement of the vertex shader's MVP
    transform and the viewport, for describing workloads (not bit-exact)."""
    v = np.asarray(scene.vertices, np.float64)
    idx = np.asarray(scene.indices, np.int64)
    pos = np.concatenate([v[:, :3], np.ones((len(v), 1))], axis=1)
    count, area_sum = 0, 0.0
    for dr in scene.draws:
        m = np.asarray(dr.mvp, np.float64).reshape(4, 4).T  # the push constant is column-major
        tri = idx[dr.first: dr.first + 3 * dr.count].reshape(-1, 3) + dr.vertex_offset  # first: firstIndex
        p = (pos @ m.T)[tri]  # [T, 3, 4]
        x, y, z, w = p[..., 0], p[..., 1], p[..., 2], p[..., 3]
        outside = (np.all(x > w, 1) | np.all(x < -w, 1) | np.all(y > w, 1) | np.all(y < -w, 1) | np.all(z < 0, 1) |
                   np.all(z > w, 1))
        ahead = np.all(w > 0, 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            sx = (x / w + 1.0) * scene.width / 2
            sy = (y / w + 1.0) * scene.height / 2
        a = 0.5 * ((sx[:, 1] - sx[:, 0]) * (sy[:, 2] - sy[:, 0]) - (sx[:, 2] - sx[:, 0]) * (sy[:, 1] - sy[:, 0]))
        vis = ahead & ~outside & (a < 0 if scene.front_ccw else a > 0)
        count += int(vis.sum())
        area_sum += float(np.abs(a[vis]).sum())
    return count, (area_sum / count if count else 0.0)


def batched_counts(seed=3, ndraws=4096, lo=16, hi=65536):
    c = np.empty(ndraws, dtype=np.uint32)
    lib().kz_batched_counts(seed, ndraws, lo, hi, _up(c))
    return c


def batched(seed=3, ndraws=4096, width=2048, height=2048, lo=16, hi=65536):
    counts = batched_counts(seed, ndraws, lo, hi)
    verts, inds, draws = [], [], []
    vbase = ibase = 0
    for i, t in enumerate(counts):
        v, idx = sphere_mesh(seed ^ (i + 1), int(t))
        m = np.empty(16, dtype=np.float32)
        lib().kz_mvp_batched(seed, i, width, height, _fp(m))
        verts.append(v)
        inds.append(idx)
        draws.append(Draw(ibase, int(t), vbase, m))
        vbase += len(v)
        ibase += len(idx)
    return Scene("batched", width, height, "lambert", np.concatenate(verts), np.concatenate(inds), draws, cull=2)


def ordered_blend(seed=4, n=200_000, width=1920, height=1080, amin=4.0, amax=4096.0, alpha=0.5):
    v = np.empty((3 * n, 8), dtype=np.float32)
    lib().kz_scene_blend(seed, n, width, height, amin, amax, alpha, _fp(v))
    return Scene("ordered_blend", width, height, "color", v, None, [Draw(0, n)], cull=0, depth_test=True,
                 depth_write=False, blend=True)


def textured(seed=6, n=4000, width=640, height=360, tex_w=61, tex_h=37, uv_lo=-1.5, uv_hi=2.5, size_lo=0.01,
             size_hi=0.6, **sampler):
    """n random triangles (vertices at log-uniform distances in [size_lo, size_hi] NDC from a centre) with
    per-vertex w in [0.5, 2] (perspective-correct texture coordinates) and coordinates in [uv_lo, uv_hi]
    (every address mode is exercised), over a random RGBA8 texture of tex_w x tex_h; `sampler` sets the
    Texture's filter and address fields"""
    rng = np.random.default_rng(seed)
    v = np.empty((3 * n, 6), dtype=np.float32)
    cx = rng.uniform(-1.1, 1.1, n)
    cy = rng.uniform(-1.1, 1.1, n)
    size = np.exp(rng.uniform(np.log(size_lo), np.log(size_hi), n))
    for k in range(3):
        ang = rng.uniform(0, 2 * np.pi, n)
        w = rng.uniform(0.5, 2.0, n)
        x = cx + size * np.cos(ang)
        y = cy + size * np.sin(ang)
        v[k::3, 0] = x * w
        v[k::3, 1] = y * w
        v[k::3, 2] = rng.uniform(0.05, 0.95, n) * w
        v[k::3, 3] = w
        v[k::3, 4] = rng.uniform(uv_lo, uv_hi, n)
        v[k::3, 5] = rng.uniform(uv_lo, uv_hi, n)
    texels = rng.integers(0, 256, (tex_h, tex_w, 4), dtype=np.uint8)
    return Scene("textured", width, height, "textured", v, None, [Draw(0, n)], cull=0,
                 texture=Texture(texels, **sampler))


def triangles_from(vertices_xyzw_rgba, width, height, **state):
    """a hand-made non-indexed colour scene (tests)"""
    v = np.ascontiguousarray(vertices_xyzw_rgba, dtype=np.float32).reshape(-1, 8)
    s = Scene("custom", width, height, "color", v, None, [Draw(0, len(v) // 3)])
    for k, val in state.items():
        setattr(s, k, val)
    return s

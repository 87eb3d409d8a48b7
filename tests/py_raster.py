"""A second, independent restatement of the draw path's rules in pure Python, for tiny scenes only.

It is test infrastructure: it checks the C oracle (oracle/kz_oracle.c) on hand-sized cases, using exact
rational arithmetic with one explicit round-to-nearest-even to binary32 per operation, so every fma is a
true single-rounding fma.  Coverage: colour pipeline (pass-through vertex shader, colour fragment shader),
non-indexed triangle lists, full-framebuffer viewport with depth range [0, 1], no culling, unless the
options below say otherwise.  Clipping: a triangle with all vertices beyond one plane of the view volume
(x > w, x < -w, y > w, y < -w, z < 0, z > w) is dropped; one with a vertex outside z >= 0, z <= w or the
guard band |x|, |y| <= 4w is clipped against those six planes in that order (Sutherland-Hodgman, a plane
skipped when no vertex is outside it), each new vertex on edge (inside i, outside o) being
fma(t, o_k - i_k, i_k) for every component with t = d_i / (d_i - d_o), d the plane's distance in binary32
(z, w - z, x + 4w, 4w - x, y + 4w, 4w - y); a polygon with a vertex at w <= 0 left is dropped, the rest
drawn as the fan (v0, v_i, v_i+1).

Rules (Vulkan specification, with the choices the spec leaves open fixed as the GPU path fixes them):
viewport x_f = fma(x * (1/w), W/2, W/2), snapped to 16.8 fixed point with round-to-nearest-even; signed
area S of the snapped vertices decides orientation; pixel (x, y) is sampled at (256 x + 128, 256 y + 128);
edge e runs from vertex e+1 to vertex e+2 and a pixel is covered when every edge function is > 0, or
== 0 on a top or left edge; depth z = fma(l2, z2 - z0, fma(l1, z1 - z0, z0)) with l_i = E_i * (1 / S),
tested with any VkCompareOp and written or not;
colour = perspective-correct interpolation q = fma(l2, 1/w2, fma(l1, 1/w1, l0 * 1/w0)),
c = fma(l2, c2/w2, fma(l1, c1/w1, l0 * c0/w0)) * (1 / q), stored as round(clamp(c, 0, 1) * 255) through
the colour write mask, or blended (the 15 single-source factors, the 5 ops, constants; blend_texel).
Optionally (render's `cull`, `front_ccw`, `viewport`, `scissor`): the polygon's area in framebuffer
coordinates a = -1/2 sum(x_i y_i+1 - x_i+1 y_i) decides facing (a > 0 is counter-clockwise), culled by
VkCullModeFlags; a viewport (x, y, width, height, minDepth, maxDepth) maps x_f = fma(x_d, w/2, x + w/2) and
z_f = fma(z_d, maxDepth - minDepth, minDepth) (each constant one binary32 operation), clamps depth to its
depth range, and admits pixel column p when p + 1/2 lies in [x, x + width) (rows likewise, for either sign
of the height); a scissor rectangle (x, y, width, height) admits its pixels.  D16 / D24 depth attachments
(`depth_format`) hold round(z * (2^n - 1)) of the binary32 product, compared and stored as integers; the
stencil test (`stencil`: per face (fail, pass, depth_fail, compare, compare_mask, write_mask, reference))
compares the masked reference with the masked stored value, then applies the VkStencilOp of its outcome
through the write mask, before the depth result decides whether the fragment goes on.  With `samples`=4
(the standard sample positions (3/8, 1/8), (7/8, 3/8), (1/8, 5/8), (5/8, 7/8) of a pixel) each sample has
its own coverage, depth and depth test; the fragment shader runs once at the pixel centre (extrapolated
when the centre lies outside) and its colour is written to every sample that passed.
"""
from fractions import Fraction
import math

import numpy as np

HALF = Fraction(1, 2)


def f32(q):
    """round an exact rational to the nearest binary32 value, ties to even (no overflow handling)"""
    q = Fraction(q)
    if q == 0:
        return Fraction(0)
    sign = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    e = max(e, -126)
    ulp = Fraction(2) ** (e - 23)
    m = a / ulp
    n = math.floor(m)
    r = m - n
    if r > HALF or (r == HALF and n % 2 == 1):
        n += 1
    return sign * n * ulp


def mul(a, b):
    return f32(a * b)


def fma(a, b, c):
    return f32(a * b + c)


def div(a, b):
    return f32(Fraction(a) / Fraction(b))


def rne(q):
    """round to the nearest integer, ties to even"""
    return round(Fraction(q))


def unorm8(v):
    c = min(max(v, Fraction(0)), Fraction(1))
    return int(rne(mul(c, Fraction(255))))


def depth_cmp(op, z, d):
    """VkCompareOp `op` of fragment depth z against stored depth d"""
    return [False, z < d, z == d, z <= d, z > d, z != d, z >= d, True][op]


def _factor(f, ch, s, d, k):
    """VkBlendFactor f for channel ch (the 15 single-source factors)"""
    one = Fraction(1)
    table = {0: lambda: Fraction(0), 1: lambda: one, 2: lambda: s[ch], 3: lambda: f32(one - s[ch]),
             4: lambda: d[ch], 5: lambda: f32(one - d[ch]), 6: lambda: s[3], 7: lambda: f32(one - s[3]),
             8: lambda: d[3], 9: lambda: f32(one - d[3]), 10: lambda: k[ch], 11: lambda: f32(one - k[ch]),
             12: lambda: k[3], 13: lambda: f32(one - k[3]),
             14: lambda: min(s[3], f32(one - d[3])) if ch < 3 else one}
    return table[f]()


def _blend_op(op, s, sf, d, df):
    """VkBlendOp with the products and fma the GPU path uses: ADD fma(s, sf, d df), SUBTRACT fma(s, sf, -(d df)),
    REVERSE_SUBTRACT fma(d, df, -(s sf)), MIN, MAX"""
    if op == 0:
        return fma(s, sf, mul(d, df))
    if op == 1:
        return fma(s, sf, -mul(d, df))
    if op == 2:
        return fma(d, df, -mul(s, sf))
    return min(s, d) if op == 3 else max(s, d)


def blend_texel(texel, out, factors, consts, write_mask):
    """the RGBA8 texel after blending fragment colour `out` (four exact binary32 values) into `texel`
    (unsigned normalized: source, destination and constants clamped to [0, 1]); factors = (srcColor, dstColor,
    colorOp, srcAlpha, dstAlpha, alphaOp)"""
    clamp = lambda v: min(max(v, Fraction(0)), Fraction(1))
    s = [clamp(v) for v in out]
    d = [div(int(t), 255) for t in texel]
    k = [clamp(Fraction(float(np.float32(c)))) for c in consts]
    res = list(texel)
    for ch in range(4):
        if not (write_mask >> ch) & 1:
            continue
        sf_i, df_i, op = (factors[0], factors[1], factors[2]) if ch < 3 else (factors[3], factors[4], factors[5])
        r = _blend_op(op, s[ch], _factor(sf_i, ch, s, d, k), d[ch], _factor(df_i, ch, s, d, k))
        res[ch] = unorm8(r)
    return res


def _plane_dist(p, plane):
    x, y, z, w = p[:4]
    g = 4 * w  # exact
    return [z, f32(w - z), f32(x + g), f32(g - x), f32(y + g), f32(g - y)][plane]


def clip_triangle(P):
    """the sub-triangles of triangle P (three lists of 8 exact binary32 values) after clipping, in fan order;
    [] when it is dropped"""
    if any(all(cond(p) for p in P) for cond in (lambda p: p[0] > p[3], lambda p: p[0] < -p[3],
                                               lambda p: p[1] > p[3], lambda p: p[1] < -p[3],
                                               lambda p: p[2] < 0, lambda p: p[2] > p[3])):
        return []
    if not any(_plane_dist(p, k) < 0 for p in P for k in range(6)):
        return [P]
    poly = [list(p) for p in P]
    for plane in range(6):
        if not any(_plane_dist(p, plane) < 0 for p in poly):
            continue
        out = []
        for i in range(len(poly)):
            p, q = poly[i], poly[(i + 1) % len(poly)]
            dp, dq = _plane_dist(p, plane), _plane_dist(q, plane)
            pin, qin = dp >= 0, dq >= 0
            if pin:
                out.append(p)
            if pin != qin:
                vi, vo = (p, q) if pin else (q, p)
                di, do = (dp, dq) if pin else (dq, dp)
                t = div(di, f32(di - do))
                out.append([fma(t, f32(vo[k] - vi[k]), vi[k]) for k in range(len(vi))])
        poly = out
        if len(poly) < 3:
            return []
    if not all(p[3] > 0 for p in poly):
        return []
    return [[poly[0], poly[i], poly[i + 1]] for i in range(1, len(poly) - 1)]


def _pixel_range(lo, extent):
    """first and one-past-last pixel p with p + 1/2 in [lo, lo + extent) (extent may be negative), from the
    binary32 operations ceil(lo - 1/2) and ceil((lo + extent) - 1/2)"""
    end = f32(lo + extent)
    a, b = (lo, end) if extent >= 0 else (end, lo)
    return math.ceil(f32(a - HALF)), math.ceil(f32(b - HALF))


DEPTH_BITS = {"d32": None, "d16": 16, "d24s8": 24}
MS_POS = [(96, 32), (224, 96), (32, 160), (160, 224)]  # sample offsets in 1/256 pixel


def stencil_op(op, s, write_mask, reference):
    """VkStencilOp on the stored 8-bit value s, through the write mask"""
    v = {0: s, 1: 0, 2: reference & 0xFF, 3: min(s + 1, 255), 4: max(s - 1, 0), 5: ~s & 0xFF, 6: (s + 1) & 0xFF,
         7: (s - 1) & 0xFF}[op]
    return (s & ~write_mask & 0xFF) | (v & write_mask & 0xFF)


def _pixel_ms(px, py, X, Y, dxs, dys, tl, inv_s, z0, dz1, dz2, zlo, zhi, IW, A, compare, depth_test, depth_write,
              depth4, color4, blend, blend_const, write_mask):
    """one pixel of a 4x multisampled attachment; returns 1 when a sample is covered"""
    def edges(sx, sy):
        return [dxs[e] * (sy - Y[(e + 1) % 3]) - dys[e] * (sx - X[(e + 1) % 3]) for e in range(3)]

    passed, zs, covered = [], {}, False
    for s, (ox, oy) in enumerate(MS_POS):
        E = edges(256 * px + ox, 256 * py + oy)
        if not all(E[e] > 0 or (E[e] == 0 and tl[e]) for e in range(3)):
            continue
        covered = True
        z = fma(mul(f32(E[2]), inv_s), dz2, fma(mul(f32(E[1]), inv_s), dz1, z0))
        zs[s] = min(max(z, zlo), zhi)
        if not depth_test or depth_cmp(compare, zs[s], depth4[py][px][s]):
            passed.append(s)
    if not covered:
        return 0
    if passed:
        E = edges(256 * px + 128, 256 * py + 128)  # the fragment shader at the pixel centre
        l = [mul(f32(E[e]), inv_s) for e in range(3)]
        q = fma(l[2], IW[2], fma(l[1], IW[1], mul(l[0], IW[0])))
        rq = div(1, q)
        out = [mul(fma(l[2], A[2][k], fma(l[1], A[1][k], mul(l[0], A[0][k]))), rq) for k in range(4)]
        for s in passed:
            if depth_test and depth_write:
                depth4[py][px][s] = zs[s]
            if blend is not None:
                color4[py, px, s] = blend_texel(color4[py, px, s], out, blend, blend_const, write_mask)
            else:
                for k in range(4):
                    if (write_mask >> k) & 1:
                        color4[py, px, s, k] = unorm8(out[k])
    return 1


def render(vertices, width, height, clear_color=(0.0, 0.0, 0.0, 1.0), clear_depth=1.0, compare=1, depth_write=True,
           blend=None, blend_const=(0.0, 0.0, 0.0, 0.0), write_mask=0xF, cull=0, front_ccw=True, viewport=None,
           scissor=None, depth_test=True, depth_format="d32", stencil=None, clear_stencil=0, samples=1):
    """vertices: float32 [3T, 8] (x, y, z, w, r, g, b, a); returns (colour uint8 [H, W, 4], depth float32
    [H, W], fragment count), and the stencil plane uint8 [H, W] fourth when `stencil` is given.  compare: the
    VkCompareOp of the depth test; blend: None, or the six blend factors and ops of blend_texel; cull:
    VkCullModeFlags; viewport: (x, y, width, height, minDepth, maxDepth), default the whole framebuffer with
    depths [0, 1]; scissor: (x, y, width, height); depth_format: "d32", "d16" or "d24s8" (the depth plane then
    holds the integer texel values); stencil: {"front": (...), "back": (...)} as in the module docstring;
    samples: 1, or 4 (D32, no stencil), which returns colour [H, W, 4 samples, 4] and depth [H, W, 4]."""
    v = np.asarray(vertices, dtype=np.float32).reshape(-1, 8)
    color = np.empty((height, width, 4), dtype=np.uint8)
    color[:] = [unorm8(Fraction(float(np.float32(c)))) for c in clear_color]
    bits = DEPTH_BITS[depth_format]

    def depth_value(z):
        return z if bits is None else Fraction(rne(mul(z, (1 << bits) - 1)))

    depth = [[depth_value(Fraction(float(np.float32(clear_depth))))] * width for _ in range(height)]
    sten = [[clear_stencil & 0xFF] * width for _ in range(height)]
    if samples == 4:
        assert bits is None and stencil is None
        color4 = np.repeat(color[:, :, None, :], 4, axis=2)
        depth4 = [[[depth[0][0]] * 4 for _ in range(width)] for _ in range(height)]
    vp = [Fraction(float(np.float32(c))) for c in (viewport or (0, 0, width, height, 0, 1))]
    hx, hy = mul(vp[2], HALF), mul(vp[3], HALF)
    ox, oy = f32(vp[0] + hx), f32(vp[1] + hy)
    pz, oz = f32(vp[5] - vp[4]), vp[4]
    zlo, zhi = min(vp[4], vp[5]), max(vp[4], vp[5])
    # the pixels a draw may touch: framebuffer, scissor and viewport
    rx0, rx1 = _pixel_range(vp[0], vp[2])
    ry0, ry1 = _pixel_range(vp[1], vp[3])
    rx0, ry0, rx1, ry1 = max(rx0, 0), max(ry0, 0), min(rx1, width), min(ry1, height)
    if scissor is not None:
        rx0, ry0 = max(rx0, scissor[0]), max(ry0, scissor[1])
        rx1, ry1 = min(rx1, scissor[0] + scissor[2]), min(ry1, scissor[1] + scissor[3])
    frags = 0
    pieces = []
    for t in range(len(v) // 3):
        pieces += clip_triangle([[Fraction(float(c)) for c in v[3 * t + j]] for j in range(3)])
    for P in pieces:
        X, Y, Z, IW, A = [], [], [], [], []
        for p in P:
            x, y, z, w = p[:4]
            iw = div(1, w)
            X.append(int(rne(mul(fma(mul(x, iw), hx, ox), 256))))
            Y.append(int(rne(mul(fma(mul(y, iw), hy, oy), 256))))
            Z.append(fma(mul(z, iw), pz, oz))
            IW.append(iw)
            A.append([mul(c, iw) for c in p[4:8]])
        S = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0])
        if S == 0:
            continue
        area = -Fraction(sum(X[i] * Y[(i + 1) % 3] - X[(i + 1) % 3] * Y[i] for i in range(3)), 2)
        front = area > 0 if front_ccw else area < 0
        if (cull & 2 and not front) or (cull & 1 and front):
            continue
        if S < 0:
            for arr in (X, Y, Z, IW, A):
                arr[1], arr[2] = arr[2], arr[1]
            S = -S
        lo, hi = (32, 224) if samples == 4 else (128, 128)  # the sample offsets' range
        bx0 = max(rx0, -((-(min(X) - hi)) // 256))
        by0 = max(ry0, -((-(min(Y) - hi)) // 256))
        bx1 = min(rx1 - 1, (max(X) - lo) // 256)
        by1 = min(ry1 - 1, (max(Y) - lo) // 256)
        inv_s = div(1, f32(S))
        z0, dz1, dz2 = Z[0], f32(Z[1] - Z[0]), f32(Z[2] - Z[0])
        tl, dxs, dys = [], [], []
        for e in range(3):
            a, b = (e + 1) % 3, (e + 2) % 3
            dx, dy = X[b] - X[a], Y[b] - Y[a]
            dxs.append(dx)
            dys.append(dy)
            tl.append(dy < 0 or (dy == 0 and dx > 0))
        for py in range(by0, by1 + 1):
            for px in range(bx0, bx1 + 1):
                if samples == 4:
                    frags += _pixel_ms(px, py, X, Y, dxs, dys, tl, inv_s, z0, dz1, dz2, zlo, zhi, IW, A, compare,
                                       depth_test, depth_write, depth4, color4, blend, blend_const, write_mask)
                    continue
                sx, sy = 256 * px + 128, 256 * py + 128
                E = []
                for e in range(3):
                    a = (e + 1) % 3
                    E.append(dxs[e] * (sy - Y[a]) - dys[e] * (sx - X[a]))
                if not all(E[e] > 0 or (E[e] == 0 and tl[e]) for e in range(3)):
                    continue
                frags += 1
                l = [mul(f32(E[e]), inv_s) for e in range(3)]
                z = fma(l[2], dz2, fma(l[1], dz1, z0))
                z = depth_value(min(max(z, zlo), zhi))
                dpass = not depth_test or depth_cmp(compare, z, depth[py][px])
                if stencil is not None:
                    fail, pas, dfail, cmp_op, cmask, wmask, ref = stencil["front" if front else "back"]
                    sv = sten[py][px]
                    if not depth_cmp(cmp_op, ref & cmask & 0xFF, sv & cmask):
                        sten[py][px] = stencil_op(fail, sv, wmask, ref)
                        continue
                    sten[py][px] = stencil_op(pas if dpass else dfail, sv, wmask, ref)
                if not dpass:
                    continue
                if depth_test and depth_write:
                    depth[py][px] = z
                q = fma(l[2], IW[2], fma(l[1], IW[1], mul(l[0], IW[0])))
                rq = div(1, q)
                out = [mul(fma(l[2], A[2][k], fma(l[1], A[1][k], mul(l[0], A[0][k]))), rq) for k in range(4)]
                if blend is not None:
                    color[py, px] = blend_texel(color[py, px], out, blend, blend_const, write_mask)
                else:
                    for k in range(4):
                        if (write_mask >> k) & 1:
                            color[py, px, k] = unorm8(out[k])
    if samples == 4:
        return color4, np.array([[[float(d) for d in px] for px in row] for row in depth4], dtype=np.float32), frags
    dep = np.array([[float(d) for d in row] for row in depth], dtype=np.float32)
    if stencil is not None:
        return color, dep, frags, np.array(sten, dtype=np.uint8)
    return color, dep, frags

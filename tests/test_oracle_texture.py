"""The oracle's texture sampling (kzo_tex2d, the rule the GPU's kz_tex2d follows) against an independent
numpy restatement of the Vulkan specification's texel selection: the wrapping operation of each address
mode, NEAREST (floor of the scaled coordinate), LINEAR (four texels around u - 0.5, v - 0.5, blended
lerp(lerp(t00, t10, a), lerp(t01, t11, a), b) with every float32 operation rounded), border colours, BGRA
byte order and unnormalized coordinates; plus known answers at texel centres."""
import itertools

import numpy as np
import pytest

from kazan_gb300 import scenes
from oracle import kz_oracle

F = np.float32


def _wrap(i, size, mode):
    if mode == 0:                                   # REPEAT
        return i % size
    if mode == 1:                                   # MIRRORED_REPEAT: (size - 1) - mirror((i mod 2size) - size)
        t = (i % (2 * size)) - size
        return size - 1 - (t if t >= 0 else -(1 + t))
    if mode == 3:                                   # CLAMP_TO_BORDER
        return -1 if i < 0 or i >= size else i
    if mode == 4:                                   # MIRROR_CLAMP_TO_EDGE
        m = i if i >= 0 else -(1 + i)
        return min(m, size - 1)
    return min(max(i, 0), size - 1)                 # CLAMP_TO_EDGE


def _to_int(x):
    # NaN and huge values: fmaxf/fminf keep the non-NaN operand
    x = F(-1.0e9) if np.isnan(x) else max(x, F(-1.0e9))
    return int(min(x, F(1.0e9)))


def _texel(t, i, j):
    if i < 0 or j < 0:
        c = F(1.0) if t.border == 2 else F(0.0)
        return [c, c, c, F(0.0) if t.border == 0 else F(1.0)]
    px = [F(int(b)) / F(255.0) for b in t.texels[j, i]]
    return [px[2], px[1], px[0], px[3]] if t.bgra else px


def _lerp(a, b, f):
    return F(a + F(f * F(b - a)))


def restated(t, s, tc):
    with np.errstate(invalid="ignore", over="ignore"):
        return _restated(t, s, tc)


def _restated(t, s, tc):
    h, w = t.texels.shape[:2]
    s, tc = F(s), F(tc)
    u, v = (s, tc) if t.unnormalized else (F(s * F(w)), F(tc * F(h)))
    if not t.linear:
        return _texel(t, _wrap(_to_int(np.floor(u)), w, t.address_u), _wrap(_to_int(np.floor(v)), h, t.address_v))
    u0, v0 = F(u - F(0.5)), F(v - F(0.5))
    fi, fj = F(np.floor(u0)), F(np.floor(v0))
    a = min(max(F(u0 - fi), F(0.0)), F(1.0)) if not np.isnan(u0 - fi) else F(0.0)
    b = min(max(F(v0 - fj), F(0.0)), F(1.0)) if not np.isnan(v0 - fj) else F(0.0)
    i0, j0 = _to_int(fi), _to_int(fj)
    x0, x1 = _wrap(i0, w, t.address_u), _wrap(i0 + 1, w, t.address_u)
    y0, y1 = _wrap(j0, h, t.address_v), _wrap(j0 + 1, h, t.address_v)
    t00, t10, t01, t11 = _texel(t, x0, y0), _texel(t, x1, y0), _texel(t, x0, y1), _texel(t, x1, y1)
    return [_lerp(_lerp(t00[k], t10[k], a), _lerp(t01[k], t11[k], a), b) for k in range(4)]


def _coords(rng, n, lo, hi):
    c = list(rng.uniform(lo, hi, n).astype(np.float32))
    return c + [F(0.0), F(1.0), F(-0.0), F(0.5), F(1e30), F(-1e30), F(np.inf), F(-np.inf), F(np.nan)]


@pytest.mark.parametrize("linear,mode,border,bgra,unnorm",
                         [(lin, m, b, bg, un) for lin, m in itertools.product((False, True), range(5))
                          for b, bg, un in ((m % 3, m == 2, False), (2 - m % 3, False, m == 4))])
def test_sampling_matches_restatement(linear, mode, border, bgra, unnorm):
    rng = np.random.default_rng(17 + 5 * mode + int(linear))
    tex = scenes.Texture(rng.integers(0, 256, (5, 7, 4), dtype=np.uint8), bgra=bgra, linear=linear,
                         address_u=mode, address_v=(mode + 2) % 5, border=border, unnormalized=unnorm)
    lo, hi = (-9.0, 16.0) if unnorm else (-2.5, 3.5)
    us, vs = _coords(rng, 150, lo, hi), _coords(rng, 150, lo, hi)
    for s, t in zip(us, vs[::-1]):
        got = kz_oracle.tex2d(tex, s, t)
        want = np.array(restated(tex, s, t), dtype=np.float32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (s, t, got, want)


def test_known_answers():
    texels = np.zeros((2, 2, 4), dtype=np.uint8)
    texels[0, 0] = (255, 0, 0, 255)
    texels[0, 1] = (0, 255, 0, 255)
    texels[1, 0] = (0, 0, 255, 255)
    texels[1, 1] = (255, 255, 255, 0)
    near = scenes.Texture(texels)
    # texel centres return the texel for both filters
    for (i, j) in itertools.product(range(2), range(2)):
        want = texels[j, i].astype(np.float32) / np.float32(255.0)
        assert np.array_equal(kz_oracle.tex2d(near, (i + 0.5) / 2, (j + 0.5) / 2), want)
        lin = scenes.Texture(texels, linear=True, address_u=2, address_v=2)
        assert np.array_equal(kz_oracle.tex2d(lin, (i + 0.5) / 2, (j + 0.5) / 2), want)
    # the centre of the texture blends the four texels equally
    lin = scenes.Texture(texels, linear=True, address_u=2, address_v=2)
    assert np.allclose(kz_oracle.tex2d(lin, 0.5, 0.5), texels.reshape(4, 4).mean(0) / 255.0, atol=1e-6)
    # repeat wraps, mirrored repeat reflects, clamp-to-border gives the border colour
    rep = scenes.Texture(texels, address_u=0, address_v=0)
    assert np.array_equal(kz_oracle.tex2d(rep, 1.25, 0.25), kz_oracle.tex2d(rep, 0.25, 0.25))
    mir = scenes.Texture(texels, address_u=1, address_v=1)
    assert np.array_equal(kz_oracle.tex2d(mir, 1.25, 0.25), kz_oracle.tex2d(mir, 0.75, 0.25))
    for border, want in ((0, [0, 0, 0, 0]), (1, [0, 0, 0, 1]), (2, [1, 1, 1, 1])):
        b = scenes.Texture(texels, address_u=3, address_v=3, border=border)
        assert np.array_equal(kz_oracle.tex2d(b, -0.25, 0.5), np.array(want, dtype=np.float32))
    # BGRA swaps the red and blue bytes
    bg = scenes.Texture(texels, bgra=True)
    assert np.array_equal(kz_oracle.tex2d(bg, 0.25, 0.25), np.array([0, 0, 1, 1], dtype=np.float32))

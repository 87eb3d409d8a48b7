"""The 8-bit sRGB tables (kazan_gb300/csrc/kz_srgb_table.h) against the sRGB transfer function evaluated
independently in float64 and in exact decimal arithmetic, and the oracle's sRGB encode and clear."""
import ctypes
import os
import re
import sys

import numpy as np

from oracle import kz_oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "kazan_gb300", "csrc")


def _table(name):
    text = open(os.path.join(CSRC, "kz_srgb_table.h")).read()
    body = text[text.index("#define " + name):]
    body = body[body.index("{") + 1:body.index("}")]
    return np.array([float.fromhex(v.strip().rstrip("f")) if "0x" in v else float(v.strip().rstrip("f"))
                     for v in re.sub(r"\\\s*\n", " ", body).split(",")], dtype=np.float32)


def srgb64(x):
    x = np.asarray(x, dtype=np.float64)
    return np.where(x <= 0.0031308, 12.92 * x, 1.055 * np.power(np.maximum(x, 0.0), 1.0 / 2.4) - 0.055)


def test_header_is_what_the_generator_writes():
    sys.path.insert(0, CSRC)
    try:
        import gen_srgb_table as gen
    finally:
        sys.path.pop(0)
    thr, dec = _table("KZ_SRGB_THRESHOLDS"), _table("KZ_SRGB_DECODE")
    assert len(thr) == 255 and len(dec) == 256
    assert np.array_equal(thr, np.array(gen.thresholds(), dtype=np.float32))
    assert np.array_equal(dec, np.array(gen.decode(), dtype=np.float32))


def test_steps_are_the_rounded_transfer_function():
    thr = _table("KZ_SRGB_THRESHOLDS")
    assert np.all(np.diff(thr) > 0)
    for k, t in enumerate(thr, start=1):
        below = np.nextafter(t, np.float32(0))
        assert 255 * srgb64(t) >= k - 0.5 - 1e-9 and 255 * srgb64(below) < k - 0.5 + 1e-9, k


def test_oracle_encode_matches_float64_formula():
    L = kz_oracle.lib()
    rng = np.random.default_rng(7)
    xs = np.concatenate([rng.random(20000, dtype=np.float32), rng.random(5000, dtype=np.float32) * 0.01,
                         np.float32([0.0, 1.0, 0.0031308, 1e-30, 0.9999999])])
    want = np.clip(np.rint(255 * srgb64(xs)), 0, 255)
    got = np.array([L.kzo_srgb8(float(x)) for x in xs])
    far = np.abs(255 * srgb64(xs) - np.floor(255 * srgb64(xs)) - 0.5) > 1e-6
    assert np.array_equal(got[far], want[far])
    assert [L.kzo_srgb8(v) for v in (-1.0, float("nan"), 2.0, float("inf"))] == [0, 0, 255, 255]


def test_decode_round_trips_and_is_correctly_rounded():
    L = kz_oracle.lib()
    dec = _table("KZ_SRGB_DECODE")
    assert [L.kzo_srgb8(float(v)) for v in dec] == list(range(256))
    c = np.arange(256) / 255.0
    exact = np.where(c <= 0.04045, c / 12.92, np.power((c + 0.055) / 1.055, 2.4))
    ulp = np.spacing(np.abs(dec)).astype(np.float64)
    assert np.all(np.abs(dec.astype(np.float64) - exact) <= 0.5 * ulp + 1e-12)


def test_oracle_srgb_clear():
    L = kz_oracle.lib()
    img = np.zeros((4, 6, 4), dtype=np.uint8)
    rect = (ctypes.c_int32 * 4)(1, 1, 5, 3)
    L.kzo_clear_color_srgb(6, img.ctypes.data, rect, (ctypes.c_float * 4)(0.5, 0.2140, 1.0, 0.6))
    assert list(img[2, 3]) == [188, 127, 255, kz_oracle.unorm8(0.6)]
    assert not img[0].any() and not img[:, 0].any()


def test_oracle_srgb_render_relates_to_unorm():
    """the same opaque scene stored as sRGB and as UNORM: alpha is the same; each red, green and blue code is
    the sRGB code of a value whose UNORM code is the UNORM image's (the transfer function lies above the
    identity, so sRGB >= UNORM, with equality at 0 and 255)"""
    import dataclasses

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from scene_cases import small_cases

    base = small_cases()["sphere"]
    u, _, _ = kz_oracle.render(dataclasses.replace(base, color_format="rgba8"), threads=4)
    s, _, _ = kz_oracle.render(dataclasses.replace(base, color_format="rgba8_srgb"), threads=4)
    assert np.array_equal(u[..., 3], s[..., 3])
    assert np.all(s[..., :3] >= u[..., :3])
    assert np.all(s[..., :3][u[..., :3] == 255] == 255)
    # a UNORM code k means v in [(k - 1/2)/255, (k + 1/2)/255): its sRGB code lies between those of the ends
    L = kz_oracle.lib()
    lo = np.array([L.kzo_srgb8(max(0.0, (k - 0.5) / 255)) for k in range(256)])
    hi = np.array([L.kzo_srgb8(min(1.0, (k + 0.5) / 255)) for k in range(256)])
    rgb_u, rgb_s = u[..., :3].astype(int), s[..., :3].astype(int)
    assert np.all((rgb_s >= lo[rgb_u]) & (rgb_s <= hi[rgb_u]))
    assert (rgb_s != rgb_u).any()

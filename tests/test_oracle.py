"""The CPU oracle (oracle/kz_oracle.c) on the CPU: checked against an independent pure-Python restatement
of the rules (tests/py_raster.py, exact rational arithmetic) on small scenes -- coverage and interpolation,
every depth compare op, every blend state, cull modes and facing, viewports and scissors, D16 / D24 depth
and the stencil test, 4x multisampling and its resolve, and clipping --, against properties that follow
from the rules by hand (watertight tessellations, no double coverage at shared vertices, invariance under
vertex rotation, UNORM8 rounding), and against its own committed golden digests.

The reference driver has no rasteriser to pin against (vulkan-driver/src/api_impl.rs:4632-4653 are
`unimplemented!()`); these checks are what pins the oracle."""
import hashlib
import json
import os
import struct

import numpy as np
import pytest

import py_raster
from kazan_gb300 import scenes
from oracle import kz_oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _pix_to_ndc(px, size):
    return 2.0 * px / size - 1.0


def _tri(points, size, z=0.5, w=1.0, rgba=(1.0, 0.5, 0.25, 1.0)):
    """three vertices given in pixel coordinates (x right, y down) -> clip-space rows"""
    rows = []
    for (x, y) in points:
        rows.append([_pix_to_ndc(x, size) * w, _pix_to_ndc(y, size) * w, z * w, w] + list(rgba))
    return rows


def _scene(rows, size):
    return scenes.triangles_from(np.array(rows, dtype=np.float32), size, size, clear_color=(0.0, 0.0, 0.0, 0.0))


def _both(rows, size):
    sc = _scene(rows, size)
    oc, od, st = kz_oracle.render(sc, threads=1)
    pc, pd, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color)
    return sc, (oc, od, st["fragments"]), (pc, pd, pf)


def _random_rows(seed, n, size, perspective):
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n):
        c = rng.uniform(-2, size + 2, 2)
        pts = [tuple(c + rng.normal(0, size / 5, 2)) for _ in range(3)]
        z = [float(rng.uniform(0.05, 0.95)) for _ in range(3)]
        w = [float(rng.uniform(0.5, 2.0)) if perspective else 1.0 for _ in range(3)]
        col = rng.uniform(0, 1, (3, 4))
        for j in range(3):
            x, y = pts[j]
            rows.append([_pix_to_ndc(x, size) * w[j], _pix_to_ndc(y, size) * w[j], z[j] * w[j], w[j]] + list(col[j]))
    return rows


@pytest.mark.parametrize("seed,perspective", [(1, False), (2, False), (3, True), (4, True)])
def test_oracle_matches_python_restatement(built, seed, perspective):
    size = 24
    _, (oc, od, of), (pc, pd, pf) = _both(_random_rows(seed, 12, size, perspective), size)
    assert of == pf
    assert np.array_equal(od.view(np.uint32), pd.view(np.uint32))
    assert np.array_equal(oc, pc)


def test_watertight_tessellation(built):
    """an 8x8 grid of cells over a 16-pixel square, each cell split in two: every pixel of the square is
    covered exactly once (no gaps, no double hits on shared edges)"""
    size, n, x0, s = 24, 8, 4.0, 2.0
    rows = []
    for i in range(n):
        for j in range(n):
            a, b = (x0 + i * s, x0 + j * s), (x0 + (i + 1) * s, x0 + j * s)
            c, d = (x0 + (i + 1) * s, x0 + (j + 1) * s), (x0 + i * s, x0 + (j + 1) * s)
            rows += _tri([a, b, c], size) + _tri([a, c, d], size)
    sc, (oc, od, of), (pc, pd, pf) = _both(rows, size)
    assert of == pf == 16 * 16
    covered = oc[..., 3] > 0
    assert covered[4:20, 4:20].all() and covered.sum() == 256
    assert np.array_equal(oc, pc)


def test_shared_vertex_on_pixel_centre(built):
    """a fan of 8 triangles around a pixel centre: the centre pixel is covered by exactly one of them"""
    size = 16
    cx, cy = 8.5, 8.5
    ring = [(cx + 5 * np.cos(a), cy + 5 * np.sin(a)) for a in np.linspace(0, 2 * np.pi, 9)[:-1]]
    rows = []
    for k in range(8):
        rows += _tri([(cx, cy), ring[k], ring[(k + 1) % 8]], size, z=0.1 + 0.1 * k)
    sc, (oc, od, of), (pc, pd, pf) = _both(rows, size)
    assert of == pf
    # count how many fan triangles cover the centre pixel with the oracle, one triangle at a time
    hits = 0
    for k in range(8):
        one = _scene(rows[3 * k:3 * k + 3], size)
        c, _, _ = kz_oracle.render(one)
        hits += int(c[8, 8, 3] > 0)
    assert hits == 1


def test_vertex_rotation_keeps_coverage(built):
    size = 24
    rows = _random_rows(7, 10, size, False)
    rot = []
    for t in range(len(rows) // 3):
        a, b, c = rows[3 * t:3 * t + 3]
        rot += [b, c, a]
    _, _, st1 = kz_oracle.render(_scene(rows, size))
    _, _, st2 = kz_oracle.render(_scene(rot, size))
    assert st1["fragments"] == st2["fragments"]
    # flat triangles (equal z, equal colour) give the same image under rotation
    flat = [r[:2] + [0.25 * r[3], r[3]] + [0.2, 0.4, 0.6, 1.0] for r in rows]
    flat_rot = [r[:2] + [0.25 * r[3], r[3]] + [0.2, 0.4, 0.6, 1.0] for r in rot]
    c1, d1, _ = kz_oracle.render(_scene(flat, size))
    c2, d2, _ = kz_oracle.render(_scene(flat_rot, size))
    assert np.array_equal(c1[..., 3] > 0, c2[..., 3] > 0)


def test_degenerate_and_offscreen_produce_nothing(built):
    size = 16
    rows = _tri([(2, 2), (6, 6), (10, 10)], size)            # collinear
    rows += _tri([(3, 3), (3, 3), (3, 3)], size)             # a point
    rows += _tri([(-20, 2), (-10, 2), (-15, 8)], size)       # left of the framebuffer
    rows += _tri([(2.6, 2.6), (2.9, 2.6), (2.6, 2.9)], size)  # misses every pixel centre
    _, _, st = kz_oracle.render(_scene(rows, size))
    assert st["fragments"] == 0


def _f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def test_unorm8_rounding_boundaries(built):
    for k in range(0, 255):
        mid = _f32((k + 0.5) / 255.0)
        for v in (mid, np.nextafter(np.float32(mid), np.float32(0)), np.nextafter(np.float32(mid), np.float32(1))):
            v = float(np.float32(v))
            assert kz_oracle.unorm8(v) == py_raster.unorm8(py_raster.Fraction(v)), v
    assert kz_oracle.unorm8(-1.0) == 0 and kz_oracle.unorm8(2.0) == 255 and kz_oracle.unorm8(float("nan")) in (0, 255)


def _digest(color, depth):
    return hashlib.sha256(color.tobytes()).hexdigest()[:32], hashlib.sha256(depth.tobytes()).hexdigest()[:32]


def test_oracle_golden_digests(built):
    """tests/golden/oracle_digests.json (made by tests/golden/make_oracle_golden.py) fixes the oracle's
    output on the small workloads, so a change to the oracle cannot pass silently"""
    with open(os.path.join(GOLDEN, "oracle_digests.json"), encoding="utf-8") as f:
        gold = json.load(f)
    import sys
    sys.path.insert(0, GOLDEN)
    import make_oracle_golden
    for name, scene in make_oracle_golden.cases().items():
        c, d, st = kz_oracle.render(scene, threads=4)
        cd, dd = _digest(c, d)
        assert gold[name] == {"color": cd, "depth": dd, "fragments": st["fragments"]}, name


def test_oracle_matches_python_on_plain_draw_prefix(built):
    """the first 8 triangles of the 2,048-triangle plain draw (seed 1), drawn at 40x40"""
    soup = scenes.small_soup()
    rows = soup.vertices[:24]
    size = 40
    sc = scenes.triangles_from(rows, size, size)
    oc, od, st = kz_oracle.render(sc, threads=1)
    pc, pd, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color)
    assert st["fragments"] == pf > 0
    assert np.array_equal(od.view(np.uint32), pd.view(np.uint32))
    assert np.array_equal(oc, pc)


def _state_rows(seed, n, size):
    """random triangles whose colours reach outside [0, 1] (clamped before blending and storing) and whose alpha
    varies, half of them coplanar at depth 0.25 (ties for EQUAL, LEQUAL and GEQUAL)"""
    rng = np.random.default_rng(seed)
    rows = []
    for t in range(n):
        c = rng.uniform(0, size, 2)
        pts = [tuple(c + rng.normal(0, size / 4, 2)) for _ in range(3)]
        z = [0.25] * 3 if t % 2 else [float(rng.uniform(0.05, 0.95)) for _ in range(3)]
        col = rng.uniform(-0.25, 1.25, (3, 4))
        for j in range(3):
            x, y = pts[j]
            rows.append([_pix_to_ndc(x, size), _pix_to_ndc(y, size), z[j], 1.0] + list(col[j]))
    return rows


def _compare_states(oc, od, pc, pd):
    assert np.array_equal(od.view(np.uint32), pd.view(np.uint32)), "depth differs"
    mism = np.argwhere(np.any(oc != pc, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s: oracle %s python %s" % (
        len(mism), mism[0], oc[tuple(mism[0])], pc[tuple(mism[0])])


@pytest.mark.parametrize("depth_write", [True, False])
@pytest.mark.parametrize("op", range(8))
def test_oracle_depth_compare_ops_match_python(built, op, depth_write):
    """every VkCompareOp, with and without depth writes, against the exact restatement"""
    from fixed_function_cases import CLEAR_DEPTH
    size = 16
    sc = scenes.triangles_from(np.array(_state_rows(10 + op, 10, size), dtype=np.float32), size, size,
                               clear_color=(0.1, 0.2, 0.3, 0.4), clear_depth=CLEAR_DEPTH[op], depth_compare=op,
                               depth_write=depth_write)
    oc, od, _ = kz_oracle.render(sc, threads=1)
    pc, pd, _ = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, clear_depth=sc.clear_depth,
                                 compare=op, depth_write=depth_write)
    _compare_states(oc, od, pc, pd)


@pytest.mark.parametrize("i", range(15))
def test_oracle_blend_states_match_python(built, i):
    """every blend factor in every slot, every op, constants and write masks, against the exact restatement"""
    from fixed_function_cases import BLEND_CONSTS, WRITE_MASKS, blend_states
    size = 16
    state = blend_states()[i]
    sc = scenes.triangles_from(np.array(_state_rows(40 + i, 10, size), dtype=np.float32), size, size,
                               clear_color=(0.3, 0.6, 0.9, 0.45), depth_compare=3, depth_write=False, blend=True,
                               blend_state=state, blend_const=BLEND_CONSTS[i % len(BLEND_CONSTS)],
                               write_mask=WRITE_MASKS[i % len(WRITE_MASKS)])
    oc, od, _ = kz_oracle.render(sc, threads=1)
    pc, pd, _ = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, compare=3, depth_write=False,
                                 blend=state, blend_const=sc.blend_const, write_mask=sc.write_mask)
    _compare_states(oc, od, pc, pd)


@pytest.mark.parametrize("front_ccw", [True, False])
@pytest.mark.parametrize("cull", range(4))
def test_oracle_cull_modes_match_python(built, cull, front_ccw):
    """VkCullModeFlags NONE / FRONT / BACK / FRONT_AND_BACK under both windings against the restatement, which
    decides facing from the specification's polygon area formula"""
    size = 16
    sc = scenes.triangles_from(np.array(_state_rows(70 + cull, 12, size), dtype=np.float32), size, size,
                               clear_color=(0.1, 0.2, 0.3, 0.4), cull=cull, front_ccw=front_ccw)
    oc, od, ost = kz_oracle.render(sc, threads=1)
    pc, pd, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, cull=cull,
                                  front_ccw=front_ccw)
    _compare_states(oc, od, pc, pd)
    assert ost["fragments"] == pf
    if cull == 3:
        assert pf == 0


# (x, y, width, height, minDepth, maxDepth) on a 24x24 framebuffer: the whole framebuffer; a fractional
# offset with a narrowed depth range; one reaching past the left edge with an inverted depth range; a
# y-flipped one
VIEWPORTS = [(0.0, 0.0, 24.0, 24.0, 0.0, 1.0), (3.5, 2.25, 15.0, 17.0, 0.2, 0.9), (-4.0, 3.0, 30.0, 16.0, 1.0, 0.0),
             (2.0, 21.0, 18.0, -17.5, 0.0, 1.0)]
SCISSORS = [(0, 0, 24, 24), (5, 3, 11, 14), (10, 0, 100, 100)]


@pytest.mark.parametrize("scissor", range(len(SCISSORS)))
@pytest.mark.parametrize("viewport", range(len(VIEWPORTS)))
def test_oracle_viewports_and_scissors_match_python(built, viewport, scissor):
    """the viewport transform (offsets, depth ranges, flips) and the pixel rectangle of viewport and scissor,
    against the restatement"""
    import ctypes
    size = 24
    vp, sci = VIEWPORTS[viewport], SCISSORS[scissor]
    sc = scenes.triangles_from(np.array(_random_rows(80 + viewport, 12, size, True), dtype=np.float32), size, size,
                               clear_color=(0.1, 0.2, 0.3, 0.4))
    col, dep = kz_oracle.clear_images(sc)
    arr, n = kz_oracle.make_draws(sc)
    arr[0].viewport[:] = list(vp)
    arr[0].scissor[:] = list(sci)
    ost = kz_oracle.KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, size, size)
    assert kz_oracle.lib().kzo_render_ds(size, size, col.ctypes.data, dep.ctypes.data, None, 0, area, n, arr, 1,
                                         ctypes.byref(ost)) == 0
    pc, pd, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, viewport=vp, scissor=sci)
    _compare_states(col, dep, pc, pd)
    assert ost.as_dict()["fragments"] == pf
    assert pf > 0


# per face (fail, pass, depth_fail, compare, compare_mask, write_mask, reference); VkStencilOp KEEP 0, ZERO 1,
# REPLACE 2, INCREMENT_AND_CLAMP 3, DECREMENT_AND_CLAMP 4, INVERT 5, INCREMENT_AND_WRAP 6, DECREMENT_AND_WRAP 7
STENCIL_CASES = {
    "count_overdraw": ({"front": (0, 6, 0, 7, 0xFF, 0xFF, 0), "back": (0, 6, 0, 7, 0xFF, 0xFF, 0)},
                       dict(depth_test=False, depth_write=False), 0),
    "first_wins": ({"front": (0, 3, 7, 2, 0xFF, 0xFF, 0), "back": (0, 3, 7, 2, 0xFF, 0xFF, 0)}, {}, 0),
    "faces_masks": ({"front": (1, 6, 4, 5, 0x03, 0x0F, 2), "back": (2, 5, 3, 6, 0xF0, 0xF3, 0x35)}, {}, 0x5A),
    "replace_greater": ({"front": (7, 2, 1, 4, 0xFF, 0xFF, 6), "back": (3, 2, 0, 3, 0xFF, 0xFF, 6)},
                        dict(depth_compare=3), 5),
}


@pytest.mark.parametrize("fmt,case", [("d16", None), ("d24s8", None)] + [("d24s8", c) for c in sorted(STENCIL_CASES)])
def test_oracle_depth_formats_and_stencil_match_python(built, fmt, case):
    """D16 and D24 depth (integer texels), and on D24S8 the stencil test with per-face ops, compare and write
    masks, against the restatement: colour, depth texels, stencil values and fragment counts"""
    import ctypes
    size = 16
    faces, state, clear_s = STENCIL_CASES[case] if case else (None, {}, 0)
    stencil = None
    if faces:
        stencil = {f: scenes.StencilOp(*faces[f]) for f in ("front", "back")}
    sc = scenes.triangles_from(np.array(_state_rows(90 + len(str(case)), 12, size), dtype=np.float32), size, size,
                               clear_color=(0.1, 0.2, 0.3, 0.4), clear_depth=0.6, depth_format=fmt,
                               stencil=stencil, clear_stencil=clear_s, **state)
    col, dep = kz_oracle.clear_images(sc)
    st_plane = np.full((size, size), clear_s & 0xFF, dtype=np.uint8) if fmt == "d24s8" else None
    arr, n = kz_oracle.make_draws(sc)
    ost = kz_oracle.KzoStats()
    area = (ctypes.c_int32 * 4)(0, 0, size, size)
    assert kz_oracle.lib().kzo_render_ds(size, size, col.ctypes.data, dep.ctypes.data,
                                         st_plane.ctypes.data if st_plane is not None else None,
                                         kz_oracle.DEPTH_FORMAT[fmt], area, n, arr, 1, ctypes.byref(ost)) == 0
    out = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, clear_depth=sc.clear_depth,
                           compare=sc.depth_compare, depth_write=sc.depth_write, depth_test=sc.depth_test,
                           depth_format=fmt, stencil=faces, clear_stencil=clear_s)
    pc, pd, pf = out[:3]
    _compare_states(col, dep, pc, pd)
    assert ost.as_dict()["fragments"] == pf
    if faces:
        assert np.array_equal(st_plane, out[3]), "stencil differs"
        assert len(np.unique(out[3])) >= 2


@pytest.mark.parametrize("blend", [False, True])
def test_oracle_multisampling_matches_python(built, blend):
    """4x multisampling: per-sample coverage, depth and depth test at the standard sample positions, one
    fragment-shader run at the pixel centre, colour to the passing samples; and the resolve, (s0 + s1 + s2 +
    s3 + 2) / 4 per channel"""
    size = 16
    state = dict(blend=True, blend_state=(6, 7, 0, 6, 7, 0), depth_compare=3, depth_write=False) if blend else {}
    sc = scenes.triangles_from(np.array(_state_rows(95 + int(blend), 10, size), dtype=np.float32), size, size,
                               clear_color=(0.1, 0.2, 0.3, 0.4), samples=4, **state)
    oc4, od4, ores, ost = kz_oracle.render_ms(sc, threads=1)
    pc4, pd4, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color, compare=sc.depth_compare,
                                    depth_write=sc.depth_write, blend=sc.blend_factors() if blend else None,
                                    samples=4)
    assert ost["fragments"] == pf
    assert np.array_equal(od4.view(np.uint32), pd4.view(np.uint32)), "sample depths differ"
    assert np.array_equal(oc4, pc4), "sample colours differ"
    resolved = ((pc4.astype(np.uint32).sum(axis=2) + 2) // 4).astype(np.uint8)
    assert np.array_equal(ores, resolved)
    # samples of one pixel differ along edges (partial coverage)
    assert np.any(np.any(pc4 != pc4[:, :, :1, :], axis=(2, 3)))


def _clip_rows(seed, n, size):
    """triangles reaching past the near and far planes, behind the eye (w < 0) and past the guard band"""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n):
        c = rng.uniform(-1.0, 1.0, 2)
        for _ in range(3):
            w = float(rng.choice([rng.uniform(0.5, 2.0), rng.uniform(-1.0, 0.3)]))
            xy = (c + rng.normal(0.0, 0.8, 2) * float(rng.choice([1.0, 8.0]))) * abs(w)
            z = float(rng.uniform(-0.6, 1.6)) * abs(w)
            rows.append([float(xy[0]), float(xy[1]), z, w] + list(rng.uniform(0, 1, 4)))
    return rows


@pytest.mark.parametrize("seed", range(6))
def test_oracle_clipping_matches_python(built, seed):
    """near, far and guard-band clipping, triangles behind the eye, fan triangulation of the clipped polygon,
    against the restatement's Sutherland-Hodgman clipper"""
    import scene_cases
    size = 24
    if seed == 0:
        sc = scene_cases.guard_band_and_near(width=size, height=size)
    else:
        sc = scenes.triangles_from(np.array(_clip_rows(seed, 14, size), dtype=np.float32), size, size,
                                   clear_color=(0.1, 0.2, 0.3, 0.4))
    oc, od, ost = kz_oracle.render(sc, threads=1)
    pc, pd, pf = py_raster.render(sc.vertices, size, size, clear_color=sc.clear_color)
    _compare_states(oc, od, pc, pd)
    assert ost["fragments"] == pf
    assert ost["clipped"] > 0 and pf > 0

"""Scenes shared by the oracle known-answer tests and the GPU parity tests."""
import numpy as np

from kazan_gb300 import scenes


def px_to_ndc(px, size):
    """framebuffer coordinate -> clip-space coordinate (w = 1, viewport covering the framebuffer)"""
    return np.float32(2.0 * px / size - 1.0)


def tri(verts_px, color, width, height, z=0.5):
    """one triangle given in framebuffer pixels -> 3 rows of (x, y, z, w, r, g, b, a)"""
    rows = []
    for (x, y) in verts_px:
        rows.append([px_to_ndc(x, width), px_to_ndc(y, height), z, 1.0] + list(color))
    return rows


def tessellated_square(n=7, width=64, height=64, seed=5):
    """an n x n grid of cells over a non-axis-aligned quad, two triangles per cell with random diagonal;
    every covered pixel must be covered exactly once"""
    rng = np.random.default_rng(seed)
    corners = np.array([[6.3, 4.1], [58.7, 9.9], [55.2, 60.6], [3.9, 52.3]])
    pts = np.empty((n + 1, n + 1, 2))
    for i in range(n + 1):
        for j in range(n + 1):
            u, v = j / n, i / n
            top = corners[0] * (1 - u) + corners[1] * u
            bot = corners[3] * (1 - u) + corners[2] * u
            pts[i, j] = top * (1 - v) + bot * v
    rows = []
    k = 0
    for i in range(n):
        for j in range(n):
            a, b, c, d = pts[i, j], pts[i, j + 1], pts[i + 1, j], pts[i + 1, j + 1]
            col = [((k * 37) % 255) / 255.0, ((k * 91) % 255) / 255.0, ((k * 53) % 255) / 255.0, 1.0]
            if rng.random() < 0.5:
                rows += tri([a, b, c], col, width, height) + tri([b, d, c], col[::-1], width, height)
            else:
                rows += tri([a, b, d], col, width, height) + tri([a, d, c], col[::-1], width, height)
            k += 1
    return scenes.triangles_from(np.array(rows, dtype=np.float32), width, height, depth_test=False,
                                 depth_write=False, clear_color=(0.5, 0.5, 0.5, 0.5))


def top_left_square(width=8, height=8):
    """a square whose corners sit exactly on pixel centres (1.5, 1.5) .. (5.5, 5.5): the top and left
    edges are inside, the bottom and right edges outside, so pixels x, y in [1, 5) are covered"""
    col = [1.0, 0.0, 0.0, 1.0]
    rows = tri([(1.5, 1.5), (5.5, 1.5), (1.5, 5.5)], col, width, height) + \
        tri([(5.5, 1.5), (5.5, 5.5), (1.5, 5.5)], col, width, height)
    return scenes.triangles_from(np.array(rows, dtype=np.float32), width, height)


def degenerate_and_offscreen(width=32, height=32):
    col = [0.0, 1.0, 0.0, 1.0]
    rows = tri([(2, 2), (10, 10), (18, 18)], col, width, height)            # zero area
    rows += tri([(40, 40), (60, 45), (50, 70)], col, width, height)         # off screen
    rows += tri([(3.2, 3.2), (3.4, 3.3), (3.3, 3.45)], col, width, height)  # covers no pixel centre
    rows += tri([(5, 20), (28, 22), (12, 30)], col, width, height)          # ordinary
    return scenes.triangles_from(np.array(rows, dtype=np.float32), width, height)


def guard_band_and_near(width=64, height=48):
    """triangles that need clipping: one far outside the guard band in x, one crossing z = 0, one
    crossing z = w (far plane); plus a reference triangle"""
    rows = []
    # x beyond 4w on one vertex (w = 1)
    rows += [[-0.5, -0.5, 0.3, 1.0, 1, 0, 0, 1], [9.0, -0.2, 0.3, 1.0, 0, 1, 0, 1], [-0.4, 0.6, 0.3, 1.0, 0, 0, 1, 1]]
    # near plane: one vertex with z < 0 and w < 0 (behind the eye)
    rows += [[-0.8, 0.7, 0.5, 1.0, 1, 1, 0, 1], [0.2, 0.9, 0.5, 1.0, 0, 1, 1, 1], [0.5, -0.5, -0.6, -0.7, 1, 0, 1, 1]]
    # far plane: one vertex with z > w
    rows += [[-0.9, -0.9, 0.2, 1.0, 0.5, 0.5, 0.5, 1], [-0.1, -0.95, 1.8, 1.2, 0.2, 0.9, 0.1, 1],
             [-0.6, -0.1, 0.9, 1.0, 0.9, 0.1, 0.6, 1]]
    # ordinary
    rows += [[0.1, 0.1, 0.4, 1.0, 0.3, 0.6, 0.9, 1], [0.9, 0.2, 0.6, 1.0, 0.3, 0.6, 0.9, 1],
             [0.5, 0.9, 0.5, 1.0, 0.3, 0.6, 0.9, 1]]
    return scenes.triangles_from(np.array(rows, dtype=np.float32), width, height)


def equal_depth_ties(width=40, height=40):
    """overlapping coplanar triangles at identical depth: under LESS the first one drawn must win"""
    rows = []
    for k in range(6):
        col = [k / 6.0, 1.0 - k / 6.0, 0.5, 1.0]
        rows += tri([(2 + k, 3), (37, 5 + k), (9, 36 - k)], col, width, height, z=0.25)
    return scenes.triangles_from(np.array(rows, dtype=np.float32), width, height)


def small_cases():
    """the draw-path scene families at sizes the oracle finishes in well under a second"""
    return {
        "soup": scenes.small_soup(),
        "sphere": scenes.single_large(tris=60_000, width=480, height=270, dist=1.30),
        "batched": scenes.batched(ndraws=48, width=512, height=512, lo=16, hi=4096),
        "blend": scenes.ordered_blend(n=4000, width=640, height=360, amin=4.0, amax=2048.0),
        "tess": tessellated_square(),
        "topleft": top_left_square(),
        "degenerate": degenerate_and_offscreen(),
        "clip": guard_band_and_near(),
        "ties": equal_depth_ties(),
    }

"""The seeded synthetic workloads: deterministic bytes for a seed, the shapes and counts each workload is
defined by (2,048-triangle plain draw, 1M-triangle single draw, 4,096-draw batched command buffer,
200K-triangle blend), and value ranges."""
import numpy as np

from kazan_gb300 import scenes


def test_plain_draw_is_deterministic_and_in_range():
    a, b = scenes.small_soup(), scenes.small_soup()
    assert np.array_equal(a.vertices, b.vertices)
    assert not np.array_equal(a.vertices, scenes.small_soup(seed=2).vertices)
    v = a.vertices
    assert v.shape == (3 * 2048, 8) and a.triangles == 2048 and (a.width, a.height) == (256, 256)
    assert (np.abs(v[:, :2]) <= 1).all() and (v[:, 2] >= 0).all() and (v[:, 2] <= 1).all() and (v[:, 3] == 1).all()
    assert (v[:, 4:] >= 0).all() and (v[:, 4:] <= 1).all()


def test_batched_counts():
    c = scenes.batched_counts()
    assert len(c) == 4096 and c.min() >= 16 and c.max() <= 65536
    assert int(c.sum()) == 32_650_790
    assert np.array_equal(c, scenes.batched_counts())


def test_sphere_mesh_is_closed_and_unit():
    v, idx = scenes.sphere_mesh(9, 5000)
    assert idx.max() < len(v) and len(idx) == 3 * 5000
    n = np.linalg.norm(v[:, 3:6], axis=1)
    assert np.allclose(n, 1.0, atol=1e-5)


def test_blend_scene_areas():
    s = scenes.ordered_blend(n=2000)
    v = s.vertices.reshape(-1, 3, 8)
    x = (v[:, :, 0] + 1) * s.width / 2
    y = (v[:, :, 1] + 1) * s.height / 2
    area = 0.5 * np.abs((x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0]))
    assert area.min() > 3.9 and area.max() < 4100
    assert np.allclose(v[:, :, 7], 0.5)


def test_visible_triangles_of_a_multi_draw_scene():
    """the visible-triangle count of a scene of several indexed draws reads each draw's indices from its
    firstIndex: a mesh drawn twice (the second draw's indices after the first's) counts twice"""
    import dataclasses
    one = scenes.single_large(tris=20_000, width=480, height=270)
    n1, area1 = scenes.visible_triangles(one)
    d = one.draws[0]
    twice = dataclasses.replace(one, indices=np.concatenate([one.indices, one.indices]),
                                draws=[d, scenes.Draw(3 * d.count, d.count, d.vertex_offset, d.mvp)])
    n2, area2 = scenes.visible_triangles(twice)
    assert n1 > 0 and n2 == 2 * n1 and abs(area2 - area1) < 1e-9

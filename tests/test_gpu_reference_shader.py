"""The reference's own vertex-shader fixture run in the draw path.  tests/golden/spirv/test.spv is the module
of the reference's decoder test and of its translator's simple_test (shader-compiler-translate-spirv-to-ir
/src/lib.rs:260-287, #[ignore]d there: the reference cannot translate it yet).  It sets gl_Position =
vec4(in.xyz, 1.0), converts in.z to a 64-bit unsigned integer and, unless that is 1, 2 or 8 (an OpSwitch on
the 64-bit value), stores 0.0 to gl_Position.x.  Here it is compiled by the project's SPIR-V -> PTX backend,
linked into the pipeline kernels and drawn; the oracle draws the same triangles with that shader restated in
numpy, through its pass-through shader.  Coverage (which pixels a fragment reaches, and how many fragments)
must agree exactly, on both raster paths, in every schedule: vertices with z in 1, 2, 8 or [1, 2) keep their
x, the others collapse onto x = 0, and z > 1 puts vertices beyond the far plane, so clipping is exercised."""
import dataclasses
import os

import numpy as np
import pytest

from kazan_gb300 import render, scenes
from kazan_gb300 import spirv_asm as sa
from oracle import kz_oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "spirv")
ZS = np.array([0.25, 0.5, 0.875, 1.0, 1.5, 2.0, 3.0, 8.0], dtype=np.float32)


def white_fs():
    """colour = (1, 1, 1, 1), no inputs"""
    m = sa.Module()
    m.capability(sa.CapShader)
    v4 = m.vec(m.f32(), 4)
    o = sa._io(m, sa.SCOutput, v4, 0)
    fn = sa._begin_main(m)
    one = m.cf(1.0)
    m.op(sa.OpStore, o, m.res(sa.OpCompositeConstruct, v4, one, one, one, one))
    sa._end_main(m)
    m.entry(sa.ExecFragment, fn, "main", [o])
    m.mode(fn, sa.ModeOriginUpperLeft)
    return m.to_words()


def reference_vs(xyz):
    """the fixture's vertex shader restated: (x if uint64(z) in {1, 2, 8} else 0, y, z, 1)"""
    xyz = np.asarray(xyz, dtype=np.float32)
    keep = np.isin(np.trunc(xyz[:, 2]).astype(np.uint64), [1, 2, 8])
    out = np.empty((len(xyz), 4), dtype=np.float32)
    out[:, 0] = np.where(keep, xyz[:, 0], np.float32(0.0))
    out[:, 1:3] = xyz[:, 1:3]
    out[:, 3] = 1.0
    return out


def _scenes(seed=11, n=800, size=160, blend=False):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1.0, 1.0, (n, 1, 2))
    xy = c + rng.normal(0.0, 0.25, (n, 3, 2))
    z = rng.choice(ZS, (n, 3))
    xyz = np.concatenate([xy, z[..., None]], axis=2).reshape(-1, 3).astype(np.float32)
    white = np.ones((len(xyz), 4), dtype=np.float32)
    state = dict(depth_test=False, depth_write=False, clear_color=(0.0, 0.0, 0.0, 0.0))
    if blend:
        state.update(blend=True)
    # the GPU scene feeds the fixture the raw positions (location 0; it reads x, y, z), the oracle the
    # restated outputs
    gpu = scenes.triangles_from(np.concatenate([xyz, np.ones((len(xyz), 1), np.float32), white], axis=1), size,
                                size, **state)
    words = np.fromfile(os.path.join(GOLDEN, "test.spv"), dtype="<u4")
    gpu = dataclasses.replace(gpu, vs_words=words, fs_words=white_fs())
    ref = scenes.triangles_from(np.concatenate([reference_vs(xyz), white], axis=1), size, size, **state)
    return gpu, ref


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
@pytest.mark.parametrize("blend", [False, True])
def test_reference_vertex_shader_fixture_in_the_draw_path(renderer, mode, blend):
    gpu, ref = _scenes(blend=blend)
    run = render.SceneRun(renderer, gpu, mode=mode, tile=16)
    run.submit()
    color, _ = run.read()
    stats = run.stats()
    renderer.free_command_buffer(run.cb)
    ref_c, _, st = kz_oracle.render(ref, threads=8)
    covered, ref_covered = np.any(color != 0, axis=-1), np.any(ref_c != 0, axis=-1)
    mism = np.argwhere(covered != ref_covered)
    assert mism.size == 0, "coverage differs at %d pixels, first %s" % (len(mism), mism[0])
    assert stats.status == 0
    assert stats.fragments == st["fragments"] % (1 << 32)
    assert np.all(color[covered] == 255)
    # both kinds of vertex occur: x kept and x collapsed, and some triangles reach past the far plane
    kept = np.isin(np.trunc(ZS).astype(np.uint64), [1, 2, 8])
    assert kept.any() and (~kept).any() and 0.1 < covered.mean() < 0.95

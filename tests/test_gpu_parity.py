"""GPU parity: every scene rendered through the driver's Vulkan entry points must equal the CPU oracle
bit for bit (colour bytes, depth bits) and cover the same number of fragments, in each execution mode
and for each bin tile size."""
import dataclasses

import numpy as np
import pytest

from kazan_gb300 import render, scenes
from oracle import kz_oracle

from scene_cases import small_cases

CASES = small_cases()


def _render(renderer, scene, mode, tile):
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    run.submit()
    color, depth = run.read()
    return color, depth, run.stats()


def _check(scene, color, depth, stats):
    ref_c, ref_d, st = kz_oracle.render(scene, threads=8)
    mism = np.argwhere(np.any(color != ref_c, axis=-1))
    assert mism.size == 0, "colour differs at %d pixels, first %s: gpu %s oracle %s" % (
        len(mism), mism[0], color[tuple(mism[0])], ref_c[tuple(mism[0])])
    assert np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32)), "depth differs"
    assert stats.status == 0
    assert stats.fragments == st["fragments"] % (1 << 32), (stats.fragments, st["fragments"])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched", "perdraw"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_parity_modes(renderer, case, mode):
    scene = CASES[case]
    color, depth, stats = _render(renderer, scene, mode, 16)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [8, 32, 64])
@pytest.mark.parametrize("case", ["soup", "batched", "blend", "clip"])
def test_parity_tiles(renderer, case, tile):
    scene = CASES[case]
    color, depth, stats = _render(renderer, scene, "persistent", tile)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
def test_resubmit_is_stable(renderer):
    """the same command buffer submitted three times gives the same image (clear-on-load each time)"""
    scene = CASES["batched"]
    run = render.SceneRun(renderer, scene, mode="persistent", tile=16)
    outs = []
    for _ in range(3):
        run.submit()
        outs.append(run.read())
    for c, d in outs[1:]:
        assert np.array_equal(c, outs[0][0]) and np.array_equal(d, outs[0][1])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "batched"])
def test_kernel_timing_keeps_parity_and_counts_launches(driver, renderer, mode):
    """kernel timing launches at submit instead of through a graph: same pixels, one timed entry per launch"""
    scene = CASES["batched"]
    driver.set_option("kernel_timing", 1)
    try:
        run = render.SceneRun(renderer, scene, mode=mode, tile=16)
    finally:
        driver.set_option("kernel_timing", 0)
    for _ in range(2):
        run.submit()
    color, depth = run.read()
    _check(scene, color, depth, run.stats())
    times = driver.kernel_times(run.cb, reset=True)
    assert sum(n for _, n in times.values()) == 2 * run.stats().launches
    assert all(ms > 0 for ms, _ in times.values())
    if mode == "persistent":  # an opaque pass: the persistent kernel with only the visibility phases
        assert "kz_k_persistent_vis" in times and "kz_k_vis_geometry" not in times
    assert driver.kernel_times(run.cb) == {}


def _oracle_equal(scene, color, depth):
    ref_c, ref_d, _ = kz_oracle.render(scene, threads=8)
    return np.array_equal(color, ref_c) and np.array_equal(depth.view(np.uint32), ref_d.view(np.uint32))


@pytest.mark.gpu
def test_host_visible_memory_rewritten_between_submissions(renderer):
    """host-visible inputs are uploaded by each submission (on the copy engine, after the queue's last use
    of that memory): rewriting the mapped vertex buffer between submissions changes the next image"""
    from kazan_gb300 import scenes
    a, b = scenes.small_soup(seed=11, n=300, width=96, height=96), scenes.small_soup(seed=12, n=300, width=96, height=96)
    run = render.SceneRun(renderer, a, host_visible=True, keep_mapped=True)
    for scene in (a, b, a):
        renderer.write_buffer(run.vb, scene.vertices, keep_mapped=True)
        run.submit()
        color, depth = run.read()
        assert _oracle_equal(scene, color, depth)


@pytest.mark.gpu
def test_double_buffered_submissions_in_flight(renderer):
    """two host-visible sets submitted back to back without waiting: each image is its own scene's"""
    from kazan_gb300 import scenes
    sc = [scenes.small_soup(seed=21 + i, n=500, width=128, height=128) for i in range(2)]
    runs = [render.SceneRun(renderer, s, host_visible=True, keep_mapped=True) for s in sc]
    for _ in range(3):
        for r in runs:
            r.submit(wait=False)
        renderer.drv.vkQueueWaitIdle(renderer.queue)
        for s, r in zip(sc, runs):
            color, depth = r.read()
            assert _oracle_equal(s, color, depth)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
def test_shaders_with_function_calls(renderer, mode):
    """shaders whose helpers are inlined by the translator, or that loop over a local array with run-time
    indices, render exactly what the straight-line shaders do"""
    import dataclasses
    import call_shaders
    soup = dataclasses.replace(CASES["soup"], fs_words=call_shaders.color_fs_calls())
    loops = dataclasses.replace(CASES["soup"], fs_words=call_shaders.color_fs_loops())
    lam = dataclasses.replace(CASES["batched"], vs_words=call_shaders.lambert_vs_calls())
    for scene in (soup, loops, lam):
        color, depth, stats = _render(renderer, scene, mode, 16)
        _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["batched", "blend", "clip"])
def test_chained_and_unchained_launches_agree(driver, renderer, case):
    """kernels chained by programmatic dependent launch (the default) and launched one after another
    render the same pixels; both match the oracle"""
    scene = CASES[case]
    outs = []
    for pdl in ("1", "0"):
        driver.set_option("pdl", pdl)
        try:
            run = render.SceneRun(renderer, scene, mode="batched", tile=16)
        finally:
            driver.set_option("pdl", "1")
        for _ in range(2):
            run.submit()
        color, depth = run.read()
        _check(scene, color, depth, run.stats())
        outs.append((color, depth))
        renderer.free_command_buffer(run.cb)
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.gpu
def test_per_draw_form_launches_geometry_per_draw(renderer):
    """the per-draw launch form: the key init and the resolve once per pass, the geometry and its
    large-triangle jobs once per draw"""
    scene = CASES["batched"]
    color, depth, stats = _render(renderer, scene, "perdraw", 16)
    _check(scene, color, depth, stats)
    assert stats.launches == 2 + 2 * len(scene.draws)


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [0, 4, 8, 12, 16, 48])
@pytest.mark.parametrize("case", ["soup", "sphere", "batched"])
def test_vertex_buffer_bind_offsets(renderer, case, offset):
    """vertex buffers bound at offsets that are and are not multiples of 16 bytes: the draws with 16-byte
    aligned bases fetch attributes with vector loads, the others word by word; the images are the same"""
    scene = CASES[case]
    run = render.SceneRun(renderer, scene, mode="batched", tile=16, vb_offset=offset)
    run.submit()
    color, depth = run.read()
    _check(scene, color, depth, run.stats())


def _blend_scene(width, height, seed=12):
    """3,000 blended triangles of 4 to 1,500 px, fewer on framebuffers so small that their clipped pieces
    would pass the 4,096 records one tile's bin sorts"""
    n = 3000 if width * height >= 16 * 16 else 1000
    return dataclasses.replace(scenes.ordered_blend(seed=seed, n=n, width=width, height=height, amin=4.0,
                                                    amax=1500.0), clear_color=(0.2, 0.3, 0.4, 0.5))


@pytest.mark.gpu
@pytest.mark.parametrize("tma", [1, 0])
@pytest.mark.parametrize("size", [(640, 360), (100, 37), (333, 200), (8, 8), (16, 16)])
@pytest.mark.parametrize("tile", [8, 16])
def test_tile_staging_by_tensor_copies(driver, renderer, size, tile, tma):
    """the ordered tile raster with each tile's colour and depth staged through TMA tensor copies (and, for
    comparison, with plain loads): partial tiles at the right and bottom edges, a width whose rows are not a
    multiple of 16 bytes (333: plain loads and stores), a framebuffer of one tile, and tiny framebuffers where
    most triangles are clipped into several pieces, many of them inside one tile without covering a sample
    (they are counted and binned by the same rule)"""
    scene = _blend_scene(*size)
    driver.set_option("tma", tma)
    try:
        color, depth, stats = _render(renderer, scene, "batched", tile)
    finally:
        driver.set_option("tma", 1)
    _check(scene, color, depth, stats)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "persistent"])
@pytest.mark.parametrize("tile", [8, 16, 32])
def test_heavily_clipped_blend_is_stable(renderer, mode, tile):
    """a 16x16 framebuffer under 3,000 triangles of up to 1,500 px: about 3,200 clipped pieces in the bins;
    three submissions give the oracle's image and fragment count each time"""
    scene = _blend_scene(16, 16)
    run = render.SceneRun(renderer, scene, mode=mode, tile=tile)
    for _ in range(3):
        run.submit()
        color, depth = run.read()
        _check(scene, color, depth, run.stats())


@pytest.mark.gpu
@pytest.mark.parametrize("knobs", [{"warp_px": 1}, {"warp_px": 16, "job_blocks": 1}, {"warp_px": 4096},
                                   {"job_blocks": 7}, {"job_blocks": 32}, {"geo_blocks": 1},
                                   {"warp_px": 96, "job_blocks": 8, "geo_blocks": 2}])
@pytest.mark.parametrize("mode", ["batched", "persistent", "perdraw"])
@pytest.mark.parametrize("case", ["soup", "sphere", "batched", "clip"])
def test_visibility_path_knobs(driver, renderer, case, mode, knobs):
    """the autotuner's knobs of the visibility path: the largest box a geometry warp rasterises (1 px: every
    triangle becomes large-triangle jobs; 4,096 px: nearly none), the 8x8 blocks per job and the geometry
    blocks per SM change which kernel covers a pixel, never the image"""
    scene = CASES[case]
    for k, v in knobs.items():
        driver.set_option(k, v)
    try:
        color, depth, stats = _render(renderer, scene, mode, 16)
    finally:
        driver.set_option("warp_px", 192)
        driver.set_option("job_blocks", 16)
        driver.set_option("geo_blocks", 0)
    _check(scene, color, depth, stats)

"""bench.py's roofline bookkeeping on the CPU: the algorithmic bytes of the dominant kernels, the committed
ncu figures it reads (DRAM traffic and warp instructions per launch of the 4,096-draw workload), and their
consistency with the workload's own counts."""
import importlib.util
import os

import pytest

from kazan_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_geometry_bytes_of_the_batched_workload(bench):
    """12 B of indices per triangle, 12 B of position per vertex and 64 B of push constants per draw"""
    sc = scenes.batched()
    b, formula = bench.kernel_bytes(sc, "kz_k_vis_geometry")
    assert formula == "12*T_indexed + 12*V + 64*draws"
    assert b == 12 * sc.triangles + 12 * len(sc.vertices) + 64 * len(sc.draws)
    assert sc.triangles == 32_650_790 and b == 593_263_408


def test_raster_bytes_follow_depth_writes(bench):
    blend = scenes.ordered_blend()
    b, _ = bench.kernel_bytes(blend, "kz_k_raster_direct")
    assert b == blend.width * blend.height * (2 * 4 + 4)  # colour read and written, depth read only
    single = scenes.single_large(tris=1000)
    assert bench.kernel_bytes(single, "kz_k_vis_resolve")[0] == single.width * single.height * 8


def test_committed_profile_figures(bench):
    """the DRAM traffic and instruction counts bench.py reports beside the live timing exist for the dominant
    kernel of the default workload, are per launch of the full workload (traffic between the algorithmic bytes
    and three times them), and are absent for other workloads"""
    traffic = bench.profiled_traffic("batched", "kz_k_vis_geometry")
    inst = bench.profiled_instructions("batched", "kz_k_vis_geometry")
    assert traffic and inst
    assert 593_263_408 < traffic < 3 * 593_263_408
    assert 10 < inst / 32_650_790 < 100  # warp instructions per triangle
    assert bench.profiled_traffic(None, "kz_k_vis_geometry") is None
    assert bench.profiled_instructions("blend", "kz_k_raster_direct") is None

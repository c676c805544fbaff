"""The bench line's roofline arithmetic on fixed inputs (no GPU): the stage
figures of a wavefront frame, which stage carries which traversal at each
fusion level, the dominant stage, and the DRAM traffic scaled from the ncu
bytes per ray."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


WORK = {"segments": 1000, "shadow_rays": 400, "nodes_visited": 10_000, "tris_tested": 5_000}
SH = {"shadow_nodes": 3_000, "shadow_tris": 2_000}
STAGES = {"extend_ms": 4.0, "shade_ms": 3.0, "shadow_ms": 2.0, "other_ms": 1.0, "iterations": 12}


def test_split_stages(bench):
    r = bench.stage_roofline({"fuse": 1, "refill": 8}, WORK, SH, STAGES, 80, 1000.0)
    ext_bytes = 1000 * 48 + (10_000 - 3_000) * 80 + (5_000 - 2_000) * 48
    sh_bytes = 400 * 48 + 3_000 * 80 + 2_000 * 48
    assert r["traversal"]["extend"]["algorithmic_bytes"] == ext_bytes
    assert r["traversal"]["shadow"]["algorithmic_bytes"] == sh_bytes
    # GB/s = bytes / (ms / 1e3) / 1e9; frac against the peak
    assert r["traversal"]["extend"]["achieved_gbs"] == pytest.approx(ext_bytes / 4e-3 / 1e9)
    assert r["traversal"]["extend"]["frac"] == pytest.approx(ext_bytes / 4e-3 / 1e9 / 1000.0)
    assert r["traversal"]["extend"]["kernel"] == "k_wf_extend_dyn"
    assert r["dominant"] == "extend"
    assert sum(r["share"].values()) == pytest.approx(1.0)
    assert r["share"]["extend"] == pytest.approx(0.4)
    assert r["frame_ms_host_loop"] == pytest.approx(10.0) and r["iterations"] == 12


def test_static_fetch_kernel_names(bench):
    r = bench.stage_roofline({"fuse": 1, "refill": 0}, WORK, SH, STAGES, 80, 1000.0)
    assert r["traversal"]["extend"]["kernel"] == "k_wf_extend"
    assert r["traversal"]["shadow"]["kernel"] == "k_wf_shadow"


def test_fused_levels_move_the_traversals(bench):
    # fuse 2: the shadow test runs inside shade; fuse 3: both traversals inside shade
    st2 = dict(STAGES, shadow_ms=0.0)
    r2 = bench.stage_roofline({"fuse": 2}, WORK, SH, st2, 80, 1000.0)
    assert set(r2["traversal"]) == {"extend", "shade"}
    st3 = dict(STAGES, extend_ms=0.0, shadow_ms=0.0)
    r3 = bench.stage_roofline({"fuse": 3}, WORK, SH, st3, 80, 1000.0)
    assert set(r3["traversal"]) == {"shade"} and r3["dominant"] == "shade"


def test_traffic_scales_with_the_stage_rays(bench):
    out = {"work": {"segments": 2_000_000, "shadow_rays": 1_000_000}}
    t = bench.traffic_dominant(out, "extend")
    assert t == pytest.approx(bench.DRAM_PER_RAY["extend"] * 2_000_000)
    assert bench.traffic_dominant(out, "shadow") is None  # no capture of that stage's bytes per ray
    assert bench.traffic_dominant({"work": {}}, "extend") is None

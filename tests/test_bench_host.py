"""The bench's roofline accounting on the CPU: the wavefront frame's algorithmic bytes from the traversal
counts a statistics-returning render reports (per segment, shadow record, node, triangle and shaded hit),
over the frame time, against the measured copy peak; and the ray cast's bytes per ray."""
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, str(ROOT))
    import bench as b

    return b


def test_segment_roofline_sums_the_wave_kernels_bytes(bench):
    st = {"rays": 1000, "shadow_rays": 400, "nodes_visited": 9000, "triangles_tested": 5000,
          "shadow_nodes_visited": 3000, "shadow_triangles_tested": 2000, "shaded_hits": 700}
    r = bench.segment_roofline(st, 2e-3)
    ext = 1000 * bench.SEG_BYTES + 9000 * bench.NODE_BYTES + 5000 * bench.TRI_BYTES
    sha = 400 * bench.SHADOW_REC_BYTES + 3000 * bench.NODE_BYTES + 2000 * bench.TRI_BYTES
    shade = 700 * bench.SHADE_BYTES + 300 * bench.MISS_BYTES
    assert r["extension_bytes"] == ext and r["shadow_bytes"] == sha and r["shade_bytes"] == shade
    assert r["bytes_per_frame"] == ext + sha + shade
    assert r["achieved"] == pytest.approx((ext + sha + shade) / 2e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["nodes_per_segment"] == 9.0 and r["tris_per_shadow_ray"] == 5.0
    peak, kind = bench._peak_hbm()
    assert r["peak"] == peak and r["peak_source"] == kind


def test_peak_comes_from_the_measured_file_when_present(bench):
    peak, kind = bench._peak_hbm()
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        assert kind == "measured" and peak == float(json.loads(p.read_text())["hbm_gbs"])
    else:
        assert kind == "fallback" and peak == bench.FALLBACK_HBM_GBS


def test_profiled_traffic_is_read_from_the_ray_cast_summary(bench):
    t = bench._profiled_traffic()
    assert t is not None and 1e7 < t < 1e10

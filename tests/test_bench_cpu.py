"""bench.py's CPU baseline (the oracle, timed on a small slab and scaled) on the
host: the reported phases add up, the one-thread variant runs on one thread
and leaves the oracle's thread setting as it was."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_cpu_sample_phases_and_single_thread(jfem, orc):
    sys.path.insert(0, str(ROOT))
    import bench
    before = orc.get_threads()
    r = bench.cpu_sample(jfem, (200, 20, 20), 50, 5)
    assert r["kind"] == "port" and r["unit"] == "s" and r["cores"] >= 1
    assert r["assembly_s"] > 0.0 and r["pcg_s"] > 0.0
    assert abs(r["value"] - (r["assembly_s"] + r["pcg_s"])) <= 1e-9 * r["value"]
    assert abs(r["pcg_s"] - r["s_per_iter"] * bench.FULL_PCG_ITERS) <= 1e-9 * r["pcg_s"]
    assert "Tet10 4x20x20 slab" in r["sample"] and "x50 in size" in r["sample"]
    assert r["scipy_pcg_s"] is not None and r["scipy_pcg_s"] > 0.0     # second, independent CPU point
    one = bench.cpu_sample(jfem, (200, 20, 20), 100, 3, threads=1)
    assert one["cores"] == 1 and one["value"] > 0.0
    assert orc.get_threads() == before

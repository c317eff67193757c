"""The reference algorithm's FP64 work per segment (the FLOP-counting
restatement: oracle/qs_oracle.c counts every +, -, *, / and sqrt of a double
on the tracking path as the reference writes it, and log / sin / cos / exp
calls apart), as committed in profiles/fp64_work_per_segment.json by
tests/golden/count_fp64_work.py and used by bench.py's
`roofline.fp64_algorithm`.

* The committed figures cover every benchmark workload and are of the
  order the algorithm implies: 24 facet dot products (120 operations), the
  full test of the facets facing the ray (about a dozen, 7 to 40 each), the
  segment's own bookkeeping, and a collision's ~70 on about 40% of segments.
* A fresh count of config1 (all 10 cycles) gives the committed numbers
  exactly: the counts are integers summed per thread, so they do not depend
  on the schedule.
* bench.py's arithmetic: achieved = operations per segment x segment rate,
  peak = 64 x the DFMA warp-instruction rate.
"""
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "tests" / "golden"))
DATA = ROOT / "profiles" / "fp64_work_per_segment.json"


def test_committed_counts_cover_the_workloads():
    data = json.loads(DATA.read_text())
    assert set(data["workloads"]) == {"config1", "config2", "config3", "config4", "config5"}
    for name, w in data["workloads"].items():
        assert w["segments"] > 1_000_000, name
        assert 300.0 < w["fp64_ops_per_segment"] < 600.0, name
        assert abs(w["fp64_ops_per_segment"] - w["fp64_ops"] / w["segments"]) < 0.01, name
        assert 0.5 < w["elementary_calls_per_segment"] < 2.0, name


def test_config1_count_is_reproduced():
    import count_fp64_work as cf
    want = json.loads(DATA.read_text())["workloads"]["config1"]
    got = cf.count_workload("config1")
    for key in ("segments", "fp64_ops", "elementary_calls"):
        assert got[key] == want[key], key


def test_bench_fp64_algorithm_roofline(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    per_seg = json.loads(DATA.read_text())["workloads"]["config2"]["fp64_ops_per_segment"]
    r = bench.fp64_work_roofline("config2", 2.0e9, 1.5e10)
    assert r["unit"] == "FLOP/s" and r["algorithm_fp64_ops_per_segment"] == per_seg
    assert abs(r["achieved"] - per_seg * 2.0e9) < 1.0 and r["peak"] == 64.0 * 1.5e10
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert bench.fp64_work_roofline("config2", 2.0e9, None) is None
    assert bench.fp64_work_roofline("no such workload", 2.0e9, 1.5e10) is None

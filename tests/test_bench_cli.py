"""bench.py's reference arm (the CPU port of the reference algorithm on the
host cores) runs without a GPU and prints one JSON line with the contract's
keys."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "config", "cpu_baseline", "e2e", "impl"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "segments/s"
    assert line["warmup"] >= 3 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1


def test_profile_figures_and_fp64_roofline(tmp_path, monkeypatch):
    """The per-segment ncu figures come from a machine-readable profile that
    records the hash of the kernel sources it was captured from; a capture of
    other sources is reported as stale, not used."""
    sys.path.insert(0, str(ROOT))
    import bench
    data, _ = bench.profile_figures()
    assert data["dram_bytes_per_segment"] > 0 and 1.0 < data["fp64_warp_instructions_per_segment"] < 50.0
    fake = tmp_path / "p.json"
    fake.write_text(json.dumps(dict(data, kernel_source_sha256=bench.kernel_source_hash())))
    monkeypatch.setattr(bench, "PROFILE_DATA", fake)
    assert bench.profile_figures()[1] is True
    fake.write_text(json.dumps(dict(data, kernel_source_sha256="0" * 64)))
    assert bench.profile_figures()[1] is False
    per_seg = data["fp64_warp_instructions_per_segment"]
    r = bench.fp64_roofline(per_seg, 2.0e9, 1.5e10)
    assert abs(r["achieved"] - per_seg * 2.0e9) < 1.0 and abs(r["frac"] - r["achieved"] / 1.5e10) < 1e-12
    assert bench.fp64_roofline(None, 2.0e9, 1.5e10) is None


def test_committed_profile_matches_kernel_sources():
    """The committed per-segment figures were captured from the kernel sources
    as they are: a change to track.cu / track_device.cuh needs a new capture
    (the ncu command recorded in the profile) before bench.py's FP64 roofline
    is reported again."""
    sys.path.insert(0, str(ROOT))
    import bench
    data, current = bench.profile_figures()
    assert current, ("kernel sources changed since the capture in " + str(bench.PROFILE_DATA.name) +
                     "; recapture with: " + data.get("captured", "?"))

"""Host-side pieces of the benchmark, on CPU: the algorithmic byte counts the
roofline divides by, the latency percentiles, the median of repeated passes,
the clock-record parser, the precision metric, the seeded workloads and the
reference arm's JSON line."""
import json
import os

import numpy as np
import pytest

import bench
from cyrsoxs_gb300 import workloads


def test_headline_algorithmic_bytes():
    # 256 x 512 x 512 voxels, 4 materials: 15 packed field volumes, 5 tensor entries
    w = workloads.workload("headline")
    V, P = 256 * 512 * 512, 512 * 512
    ab = lambda k: bench.algorithmic_bytes(k, w, 5, 36, 256, batch=50, npk=15)  # noqa: E731
    # a column pass reads and writes every packed volume once: 16.1 GB
    assert ab("k_fft_rows") == ab("k_fft_cols<y>") == 2 * 8 * 15 * V == 16_106_127_360
    # the z pass loads the 32-column tiles holding a plane the Ewald projection reads and stores
    # only those 8-plane boxes
    zl, zs = bench.zmask_fractions(w, w.energies)
    assert 0.7 < zl < 0.9 and 0.1 < zs < 0.25
    assert ab("k_fft_cols<z>") == 8 * 15 * V * (zl + zs)
    # the build reads 4 float4 materials and writes 15 complex volumes
    assert ab("k_build_fields") == (16 * 4 + 8 * 15) * V
    # Ewald: Z_j(k) and Z_j(-k) at two planes per pixel and energy, 3 Gram floats out
    assert ab("k_ewald_fields") == 50 * (4 * 8 * 15 * P + 12 * P)
    assert ab("k_rotate_gram") == 50 * (12 * P + 4 * P)
    assert ab("no_such_kernel") is None


def test_zmask_fractions_cover_the_sphere_and_the_dc_neighbours():
    # physSize 5 nm: the Ewald disc covers the detector, so every tile holds a read plane
    w = workloads.workload("c1")
    w = workloads.Workload("c1_z128", 128, 256, 256, 2, w.energies, w.angles, 5.0, 0, "sphere")
    zl, zs = bench.zmask_fractions(w, w.energies)
    assert zl == 1.0 and 0.0 < zs < 0.5
    # lengths without a masked z pass move everything
    assert bench.zmask_fractions(workloads.workload("z64"), [285.0]) == (1.0, 1.0)


def test_per_energy_bytes_count_kept_planes_only():
    w = workloads.workload("headline")
    P = 512 * 512
    full = bench.algorithmic_bytes("k_fft_rows", w, 5, 36, 256)
    pruned = bench.algorithmic_bytes("k_fft_rows", w, 5, 36, 127)
    assert full == 2 * 8 * 5 * 256 * P
    assert pruned * 256 == full * 127


def test_percentiles_are_nearest_rank():
    xs = [float(i) for i in range(1, 301)]
    assert bench._pct(xs, 0.50) == 150.0
    assert bench._pct(xs, 0.99) == 297.0
    # with 80 samples the 99th percentile is the slowest request itself
    assert bench._pct(xs[:80], 0.99) == 80.0
    s = bench._lat_summary([0.001, 0.002, 0.003])
    assert s == {"p50_ms": 2.0, "p99_ms": 3.0, "max_ms": 3.0}


def test_median_pass_returns_the_middle_run():
    times = iter([5.0, 1.0, 3.0, 2.0, 4.0])
    t, lat, all_t = bench._median_pass(lambda: (next(times), ["lat"]), 5)
    assert t == 3.0 and lat == ["lat"]
    assert all_t == [1.0, 2.0, 3.0, 4.0, 5.0]
    t, _, all_t = bench._median_pass(lambda: (7.0, []), 0)  # at least one pass
    assert t == 7.0 and all_t == [7.0]


def test_clock_record_parser():
    c = bench.ClockSampler()
    c.lines = [
        "0, 2070, 2070, 910.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2040, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage",
        "0, [N/A], 2070, 0, 0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.ClockSampler().summary()["samples"] == 0


def test_precision_metric_skips_nan_and_dim_pixels():
    ref = np.array([1.0, 2.0, np.nan, 1e-9, 4.0])
    got = np.array([1.0001, 2.0, np.nan, 5.0, np.nan])
    err, n = bench.rel_err(got, ref)
    assert n == 2  # the NaN pair, the pixel below 1e-6 of the peak and the one-sided NaN are left out
    assert err == pytest.approx(1e-4, rel=1e-6)


def test_peaks_fall_back_without_the_measured_file(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "HERE", str(tmp_path))
    assert bench.load_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6781.8}))
    assert bench.load_peaks() == (6781.8, "measured")
    assert bench.load_traffic("headline") == {}


def _smooth(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def test_serving_stream_is_seeded_with_a_share_of_arbitrary_sizes():
    a, b = workloads.serving_stream(300), workloads.serving_stream(300)
    assert [(t, w.nz, w.nx, w.num_material, len(w.energies)) for t, w in a] == \
           [(t, w.nz, w.nx, w.num_material, len(w.energies)) for t, w in b]
    times = [t for t, _ in a]
    assert all(t1 > t0 for t0, t1 in zip(times, times[1:]))
    rough = 0
    for _, w in a:
        assert w.nx == w.ny and 128 <= w.nx <= 512 and 32 <= w.nz <= 128
        rough += not (_smooth(w.nx) and _smooth(w.nz))
        assert 2 <= w.num_material <= 4 and 1 <= len(w.energies) <= 100 and 6 <= w.num_angles() <= 36
    assert 0.01 * len(a) <= rough <= 0.10 * len(a)  # about 5% arbitrary sizes (Bluestein transforms)


def test_batched_set_shapes():
    ws = workloads.batched_set()
    assert len(ws) == 64
    assert {w.nx for w in ws} <= {64, 128, 256} and {w.nz for w in ws} <= {16, 32, 64}
    assert all(w.nx == w.ny and w.num_material == 2 and len(w.energies) == 20 and w.num_angles() == 12 for w in ws)


def test_energy_shards_repeat_energies_beyond_the_list():
    es = [270.0, 280.0]
    shards = [bench.shard_energies(es, r, 2, 3) for r in range(2)]
    flat = shards[0] + shards[1]
    assert len(set(flat)) == 6 and shards[0][:2] == es


def test_reference_arm_prints_one_contract_line():
    # the reference arm (the FP64 port on the host cores) on the small workload: one JSON line with the
    # contract's keys, its own cpu_baseline, and an e2e with no device copies
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "small", "--steps", "2",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=root)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

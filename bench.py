#!/usr/bin/env python
"""Benchmark of the GB300 scattering engine: patterns/s on the 512^2 x 256
morphology (Z x Y x X = 256 x 512 x 512, 4 materials, 36 E angles).

A "pattern" is one Ewald-projected detector image [Ny][Nx] for one
(energy, k, E angle) - one pass of the reference's angle loop
(src/cudaMain.cu:611).  A step is one request: ENERGIES_PER_STEP energies of
the workload (all 50), every E angle, through the full path (polarization,
3D FFT, DC replacement, shift, Ewald projection, rotation, angle average,
detector warp).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

* value: device-resident throughput (morphology already in HBM), timed with
  CUDA events on the launch stream, max over ranks.  The morphology (4.3 GB)
  is larger than L2, so no flush is needed between steps.
* e2e: the same metric through the C ABI call cyr_cuda_main with host buffers
  (pinned), host->device copy of the morphology and device->host copy of the
  patterns inside the timed region, wall clock.
* roofline: per-kernel durations from CUDA events recorded around every
  launch on its stream during profiled steps; algorithmic bytes per launch from
  algorithmic_bytes() below; peak = measured HBM copy bandwidth.
* cpu_baseline: the FP64 CPU oracle (restatement of the reference's per-angle
  algorithm, OpenMP over all host threads) on a bounded sample (1 energy x 2
  E angles of the same morphology); the same sample checks the engine's
  precision at full size.
* --impl reference: the reference's algorithm on the host cores (the
  reference has no CPU path of its own, so this is the oracle port), one
  pattern per step.
Under torchrun, ranks take disjoint energy shards (weak scaling, no data-path
collective); only the timing uses the process group.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "patterns/s (512²×256, ≤1e-4 rel vs FP64) batched vs plain; p50/p99 latency"
ENERGIES_PER_STEP = 50  # one full request of the workload (50 energies x 36 E angles)
REF_CALLS = 5  # timed calls per side in the reference GPU comparison


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="headline", choices=["headline", "c2", "c4", "z64", "cube256", "c1", "small"])
    ap.add_argument("--energies-per-step", type=int, default=ENERGIES_PER_STEP)
    ap.add_argument("--strategy", type=int, default=0, choices=[0, 1, 2],
                    help="0 auto, 1 per-energy spectra, 2 field spectra once per request")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-served", action="store_true", help="skip the batched and serving measurements")
    ap.add_argument("--skip-reference-gpu", action="store_true",
                    help="skip timing the reference's own GPU build beside the engine")
    ap.add_argument("--skip-c4", action="store_true", help="skip the 256 x 1024 x 1024 precision samples")
    ap.add_argument("--skip-fp64", action="store_true", help="skip the comparison with the on-GPU FP64 pipeline")
    ap.add_argument("--served-only", action="store_true", help="only the batched and serving measurements")
    ap.add_argument("--slots", type=int, default=8, help="serving slots (requests in flight)")
    ap.add_argument("--no-groups", action="store_true", help="serve without request groups (one launch per request)")
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--served-reps", type=int, default=5, help="timed passes per batched mode (median reported)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard_energies(all_energies, rank, world, per_rank):
    """Disjoint, contiguous energy blocks per rank (as src/cudaMain.cu:499-503 splits energies over GPUs)."""
    need = per_rank * world
    es = [all_energies[i % len(all_energies)] + 0.001 * (i // len(all_energies)) for i in range(need)]
    return es[rank * per_rank:(rank + 1) * per_rank]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, interval_ms=50):
        self.index, self.interval = index, interval_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", f"-lms={self.interval}"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic(workload):
    """dram bytes per launch of each kernel from the committed ncu summary, or {}."""
    p = os.path.join(HERE, "profiles", f"traffic_{workload}.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


_ZMASK_CACHE = {}


def zmask_fractions(w, energies):
    """Shares of the FIELDS z pass's tiles it loads and of its 8-plane boxes it stores.

    The engine's k_zmask marks, per 16 columns and 8 planes, the spectrum planes the Ewald
    projection reads (each detector pixel's one or two planes, at its column and at the mirrored
    column for the unpacking, for every energy; k along z) and the DC neighbours; the z pass loads
    only tiles (32 columns for 128- and 256-point lines when nx allows, else 16) holding a mark and
    stores only marked boxes.  (1, 1) when the z pass takes no mask (other z lengths, nx not a
    multiple of 16)."""
    import numpy as np

    nx, ny, nz = w.nx, w.ny, w.nz
    if nz not in (128, 256, 512) or nx % 16:
        return 1.0, 1.0
    key = (nx, ny, nz, w.phys_size, tuple(float(e) for e in energies))
    if key in _ZMASK_CACHE:
        return _ZMASK_CACHE[key]
    f = np.float32
    start = f(-np.pi / w.phys_size)
    dx, dy, dz = (f((2 * np.pi / w.phys_size) / (n - 1)) for n in (nx, ny, nz))
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny))
    posx, posy = start + X.astype(f) * dx, start + Y.astype(f) * dy

    def igor(j, n):
        return np.where(j <= n // 2, n // 2 - j, n + n // 2 - j)

    ux, uy = igor(X, nx), igor(Y, ny)
    mx, my = np.where(ux > 0, nx - ux, 0), np.where(uy > 0, ny - uy, 0)
    boxes = np.zeros((ny, nx // 16, nz // 8), bool)
    for e in energies:
        kmag = f(2 * np.pi / f(1239.84197 / e))
        val = kmag * kmag - posx * posx - posy * posy
        ok = (val >= 0) & (X != nx - 1) & (Y != ny - 1)
        tz = ((-kmag + np.sqrt(np.maximum(val, f(0)))) - start) / dz
        z0 = np.where(tz <= 0, 0, tz).astype(np.int64)
        ok &= z0 < nz - 1
        for z in (z0, z0 + 1):
            uz = igor(np.minimum(z, nz - 1), nz)
            mz = np.where(uz > 0, nz - uz, 0)
            boxes[uy[ok], ux[ok] // 16, uz[ok] // 8] = True
            boxes[my[ok], mx[ok] // 16, mz[ok] // 8] = True
    for (x, y, z) in ((1 % nx, 0, 0), (nx - 1, 0, 0), (0, 1 % ny, 0), (0, ny - 1, 0), (0, 0, 1), (0, 0, nz - 1)):
        boxes[y, x // 16, z // 8] = True
    halves = 2 if nz in (128, 256) and nx % 32 == 0 else 1
    tiles = boxes.any(axis=2).reshape(ny, nx // (16 * halves), halves).any(axis=2)
    out = float(tiles.mean()), float(boxes.mean())
    _ZMASK_CACHE[key] = out
    return out


def algorithmic_bytes(kernel, w, nvol, nang, planes, batch=1, npk=0, energies=None):
    """Compulsory bytes per launch (each distinct element read once, written once).

    planes = z planes kept after the fused build + z FFT (nz when not pruned); for the FIELDS
    strategy nvol = packed field volumes, batch = energies per Ewald/rotation launch, and the z
    pass moves the tiles and plane boxes of zmask_fractions (over `energies`, default the
    workload's)."""
    V, P, M = w.nvox, w.nx * w.ny, w.num_material
    if npk:
        nq = 4 * (6 if nvol == 6 else 3)  # Gram bytes per pixel and energy (packed records)
        zload, zstore = zmask_fractions(w, w.energies if energies is None else energies)
        table = {
            "k_build_fields": (16 * M + 8 * npk) * V,
            "k_build_fields_rows": (16 * M + 8 * npk) * V,  # build fused with the x pass: one write
            "k_moments": 16 * M * P * math.ceil(w.nz / max(1, w.nz // 16)),  # every (nz / 16)-th z plane
            "k_fft_rows": 2 * 8 * npk * V,
            "k_fft_cols<y>": 2 * 8 * npk * V,
            "k_fft_cols<z>": 8 * npk * V * (zload + zstore),
            "k_fft_pass<x>": 2 * 8 * npk * V,
            "k_fft_pass<y>": 2 * 8 * npk * V,
            "k_fft_pass<z>": 2 * 8 * npk * V,
            # two planes of Z_j(k) and Z_j(-k) per pixel and energy, Gram maps out
            "k_ewald_fields": batch * (4 * 8 * npk * P + nq * P),
            "k_rotate_gram": batch * (nq * P + 4 * P),
            "k_rotate_average": batch * (4 * nang * P + 4 * P),
            "k_fill": batch * 4 * P,
            "k_warp": batch * 8 * P,
            "k_dc": 6 * 8 * npk,
        }
        return table.get(kernel)
    nq = 16 * (2 if nvol == 6 else 1)
    table = {
        "k_fft_rows": 2 * 8 * nvol * planes * P,
        "k_fft_cols<y>": 2 * 8 * nvol * planes * P,
        "k_fft_cols<z>": 2 * 8 * nvol * V,
        "k_ewald_angles": 2 * 8 * nvol * P + nq * P,
        "k_rotate_gram": nq * P + 4 * P,
        "k_build": (16 * M + 8 * nvol) * V,
        "k_build_fft_z": 16 * M * V + 8 * nvol * planes * P,
        "k_moments": 16 * M * V,
        "k_fft_pass<x>": 2 * 8 * nvol * planes * P,
        "k_fft_pass<y>": 2 * 8 * nvol * planes * P,
        "k_fft_pass<z>": 2 * 8 * nvol * V,
        "k_rotate_average": 4 * nang * P + 4 * P,
        "k_fill": 4 * P,
        "k_warp": 8 * P,
        "k_dc": 6 * 8 * nvol,
    }
    return table.get(kernel)


def rel_err(a, ref, thr=1e-6):
    import numpy as np

    both = ~np.isnan(a) & ~np.isnan(ref)
    peak = np.abs(ref[both]).max()
    sel = both & (np.abs(ref) > thr * peak)
    return float((np.abs(a[sel] - ref[sel]) / np.abs(ref[sel])).max()), int(sel.sum())


def run_reference(args):
    """The reference's algorithm on the host cores: the FP64 oracle port, all threads, one pattern per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np

    from cyrsoxs_gb300 import workloads
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle

    oracle.build()
    w = workloads.workload(args.workload)
    vox = workloads.voxels(w)
    opt_all = workloads.optical_constants(w)
    cores = oracle.num_threads()
    times = []
    for s in range(args.warmup + args.steps):
        e = s % len(w.energies)
        _, secs = oracle.run_arrays(nx=w.nx, ny=w.ny, nz=w.nz, energies=[w.energies[e]], optical=opt_all[e:e + 1],
                                    voxels=vox, angles=w.angles, phys_size=w.phys_size, angle_limit=1,
                                    energy_limit=1)
        if s >= args.warmup:
            times.append(secs)
    total = sum(times)
    value = len(times) / total
    line = {
        "metric": METRIC, "value": value, "unit": "patterns/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded morphology with the configuration's shapes and distributions)",
        "config": {"workload": f"{w.name}: Z x Y x X = {w.nz} x {w.ny} x {w.nx}, {w.num_material} materials, "
                               f"{w.num_angles()} E angles", "sample": "1 energy x 1 E angle per step"},
        "cpu_baseline": {"value": value, "unit": "patterns/s", "cores": cores, "kind": "port",
                         "sample": "1 energy x 1 E angle of the workload per step (per-angle algorithm, FP64)"},
        "e2e": {"value": value, "unit": "patterns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pick_energies(optical):
    """Indices of three energies of a workload's grid for the precision samples: the low edge
    of the range, the largest resonance (the largest summed delta and beta over the materials),
    and the least contrast (the smallest spread of n^2 between the materials)."""
    import numpy as np

    o = np.asarray(optical, np.float64)
    peak = int(np.argmax(o.sum(axis=(1, 2))))
    n2p = (1.0 - o[..., 0] + 1j * o[..., 1]) ** 2
    n2s = (1.0 - o[..., 2] + 1j * o[..., 3]) ** 2
    spread = (np.abs(n2p - n2p.mean(axis=1, keepdims=True)).sum(axis=1)
              + np.abs(n2s - n2s.mean(axis=1, keepdims=True)).sum(axis=1))
    least = int(np.argmin(spread))
    return {"low_edge": 0, "peak": peak, "least_contrast": least}


def precision_study(args, w, energies, optical, host_vox, strategy):
    """Full-size parity against the FP64 CPU oracle (the reference's per-angle algorithm):
    the benchmark morphology at three energies (low edge, largest resonance, least contrast)
    x 2 E angles; the first configuration in full (3 energies x 12 angles, both strategies);
    the 128 x 512 x 512 configuration and the 256 x 1024 x 1024 precision study at their
    largest resonance x 2 E angles.  Per entry: max relative error over pixels above 1e-6 of
    the oracle's peak, and whether the NaN masks are identical.  The first headline sample's
    oracle time is the CPU baseline."""
    import numpy as np
    import torch

    from cyrsoxs_gb300 import _native, workloads
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle

    oracle.build()
    entries, cpu = [], None

    def check(name, wl, es, opt, vox, angles, strat, per_energy_names=None):
        o = _native.Options(nx=wl.nx, ny=wl.ny, nz=wl.nz, num_material=wl.num_material, energies=es,
                            start_angle=angles[0], end_angle=angles[1], increment_angle=angles[2],
                            phys_size=wl.phys_size, strategy=strat)
        gpu = _native.cuda_main(o, opt, vox).astype(np.float64)
        ref, secs = oracle.run_arrays(nx=wl.nx, ny=wl.ny, nz=wl.nz, energies=es, optical=opt, voxels=vox,
                                      angles=angles, phys_size=wl.phys_size)
        nang = int(round((angles[1] - angles[0]) / angles[2] + 1))
        for i, e in enumerate(es):
            err, npx = rel_err(gpu[i], ref[i])
            entries.append({"config": name, "energy_eV": round(float(e), 4),
                            "energy_kind": per_energy_names[i] if per_energy_names else None,
                            "angles": nang, "strategy": {1: "per_energy", 2: "fields"}[strat],
                            "max_rel_err": err, "pixels": npx,
                            "nan_mask_equal": bool(np.array_equal(np.isnan(gpu[i]), np.isnan(ref[i])))})
        return secs

    two = lambda wl: (wl.angles[0], wl.angles[0] + wl.angles[2], wl.angles[2])  # noqa: E731
    # benchmark morphology: three energies x 2 angles; the first energy alone times the CPU baseline
    picks = pick_energies(optical)
    idx = sorted(set(picks.values()))
    kinds = {v: k for k, v in picks.items()}
    secs = check(w.name, w, [energies[0]], optical[:1], host_vox, two(w), strategy, ["low_edge"])
    cpu = {"value": 2.0 / secs, "unit": "patterns/s", "cores": oracle.num_threads(), "kind": "port",
           "seconds": secs, "sample": "1 energy x 2 E angles of the same morphology (per-angle algorithm, FP64)"}
    rest = [i for i in idx if i != 0]
    if rest:
        check(w.name, w, [energies[i] for i in rest], optical[rest], host_vox, two(w), strategy,
              [kinds[i] for i in rest])
    # first configuration in full, both strategies, on its anisotropic variant (the configuration's own
    # constants are identical for both materials: zero contrast, a pattern of rounding noise)
    c1 = workloads.workload("c1_aniso")
    v1, o1 = workloads.voxels(c1), workloads.optical_constants(c1)
    for strat in (1, 2):
        check("c1_aniso", c1, c1.energies, o1, v1, c1.angles, strat)
    del v1
    # 128 x 512 x 512 (and 256 x 1024 x 1024): the largest resonance, 2 angles
    for name in (("c2",) if args.skip_c4 else ("c2", "c4")):
        wl = workloads.workload(name)
        ol = workloads.optical_constants(wl)
        p = pick_energies(ol)["peak"]
        vl = workloads.voxels(wl)
        torch.cuda.empty_cache()
        check(name, wl, [wl.energies[p]], ol[p:p + 1], vl, two(wl), 2, ["peak"])
        del vl
        torch.cuda.empty_cache()
    worst = max(e["max_rel_err"] for e in entries)
    prec = {"max_rel_err_vs_fp64": worst, "nan_mask_equal": all(e["nan_mask_equal"] for e in entries),
            "entries": entries, "threshold": "pixels above 1e-6 of the oracle's peak",
            "oracle": "FP64 CPU restatement of the reference's per-angle algorithm"}
    return prec, cpu


def fp64_study(args):
    """Every energy and E angle of a full request against the on-GPU FP64 pipeline
    (cyr_simulate_device_fp64 on the same float4 morphology: the same float decisions, every
    amplitude in double): the benchmark request (50 energies x 36 angles), the 128 x 512 x 512
    request (50 x 36) and the 256 x 1024 x 1024 precision study (10 x 24).  Per request: the
    worst and the per-energy max relative error over pixels above 1e-6 of the FP64 peak, NaN
    masks, the FP32 request's time and its dominant kernel's algorithmic GB/s."""
    import numpy as np
    import torch

    from cyrsoxs_gb300 import _native, workloads

    peak, peak_kind = load_peaks()
    out = []
    names = ("headline", "c2") if args.skip_c4 else ("headline", "c2", "c4")
    cs = torch.cuda.current_stream()
    for name in names:
        w = workloads.workload(name)
        optical = workloads.optical_constants(w)
        vox = workloads.voxels_torch(w).contiguous()
        o = _native.Options(nx=w.nx, ny=w.ny, nz=w.nz, num_material=w.num_material, energies=w.energies,
                            start_angle=w.angles[0], end_angle=w.angles[1], increment_angle=w.angles[2],
                            phys_size=w.phys_size)
        P = w.nx * w.ny
        d32 = torch.empty(len(w.energies) * P, dtype=torch.float32, device="cuda")
        d64 = torch.empty(len(w.energies) * P, dtype=torch.float64, device="cuda")
        _native.simulate_device(o, optical, vox.data_ptr(), d32.data_ptr(), cs.cuda_stream)  # warm
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        _native.profile_begin(4096)
        t0.record(cs)
        _native.simulate_device(o, optical, vox.data_ptr(), d32.data_ptr(), cs.cuda_stream)
        t1.record(cs)
        torch.cuda.synchronize()
        kernels, _ = _native.profile_end()
        ms32 = t0.elapsed_time(t1)
        info = _native.plan_info(o)
        npk = info["packed_volumes"] if info["fields"] else 0
        eb = info["energy_batch"]
        batch = len(w.energies) / math.ceil(len(w.energies) / eb)
        ab = lambda k: algorithmic_bytes(k, w, info["nvol"], w.num_angles(), info["planes"], batch, npk)  # noqa: E731
        dom_name, (n_l, dom_ms, dom_c) = max(((k, v) for k, v in kernels.items() if ab(k)), key=lambda kv: kv[1][1])
        gbs = ab(dom_name) / (dom_ms / dom_c / 1000.0) / 1e9
        t2, t3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t2.record(cs)
        _native.simulate_device_fp64(o, optical, vox.data_ptr(), False, d64.data_ptr(), cs.cuda_stream)
        t3.record(cs)
        torch.cuda.synchronize()
        ms64 = t2.elapsed_time(t3)
        g32 = d32.view(len(w.energies), w.ny, w.nx).cpu().numpy().astype(np.float64)
        g64 = d64.view(len(w.energies), w.ny, w.nx).cpu().numpy()
        errs = [rel_err(g32[i], g64[i])[0] for i in range(len(w.energies))]
        masks = [bool(np.array_equal(np.isnan(g32[i]), np.isnan(g64[i]))) for i in range(len(w.energies))]
        out.append({"config": f"{name}: Z x Y x X = {w.nz} x {w.ny} x {w.nx}, {w.num_material} materials, "
                              f"{len(w.energies)} energies x {w.num_angles()} E angles (the whole request)",
                    "strategy": "fields" if info["fields"] else "per_energy",
                    "max_rel_err": max(errs), "nan_mask_equal": all(masks),
                    "per_energy_max_rel_err": [float(f"{e:.3e}") for e in errs],
                    "fp32_ms": ms32, "fp32_patterns_per_s": len(w.energies) * w.num_angles() / (ms32 / 1e3),
                    "fp64_ms": ms64,
                    "fp32_dominant_kernel": {"kernel": dom_name, "gbs": gbs, "frac_of_peak": gbs / peak,
                                             "peak": peak, "peak_source": peak_kind}})
        print("fp64_study", json.dumps(out[-1]), file=sys.stderr, flush=True)
        del vox, d32, d64
        torch.cuda.empty_cache()
    return {"oracle": "on-GPU FP64 pipeline (cyr_simulate_device_fp64), same morphology", "entries": out,
            "max_rel_err": max(e["max_rel_err"] for e in out), "nan_mask_equal": all(e["nan_mask_equal"] for e in out)}


def reference_gpu_baseline(args):
    """The reference's own GPU path, unmodified (src/cudaMain.cu with cuFFT, NPP and cuBLAS,
    built by oracle/ref/Makefile from the staged reference sources), timed on this GPU beside
    the engine on the same requests.

    Both sides are timed the same way: the wall clock around one full call from pinned host
    buffers (cudaMain / cudaMainStreams in the reference's harness, cyr_cuda_main here), after
    one untimed call; median of REF_CALLS timed calls (the shared host link shows occasional
    100 ms stalls on either side).  The first configuration runs in full, with the
    FP32 build (as shipped, --use_fast_math) for Algorithm 0 and 1 and the FP64 build for
    Algorithm 0; the larger shapes (128 x 512 x 512, 256 x 512 x 512 and 256 x 1024 x 1024) run a
    2-energy sample of their request (all E angles).
    The engine's output is also compared with the reference FP64 build's where that ran."""
    import tempfile

    import numpy as np
    import torch

    from cyrsoxs_gb300 import _native, workloads
    sys.path.insert(0, os.path.join(HERE, "tests", "golden"))
    import cases

    refdir = os.path.join(HERE, "oracle", "_ref")
    if not os.path.exists(os.path.join(refdir, "cyrsoxs_ref_fp32")):
        return {"unavailable": "the reference build (oracle/_ref) is missing: its sources were not staged"}
    specs = [("c1", None, 0, "fp32"), ("c1", None, 1, "fp32"), ("c1_aniso", None, 0, "fp64"),
             ("c2", 2, 0, "fp32"), ("c2", 2, 1, "fp32"), ("headline", 2, 0, "fp32"), ("c4", 2, 0, "fp32")]
    out, cache = [], {}

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
        t[...] = a
        return t

    with tempfile.TemporaryDirectory() as tmp:
        for name, nsample, algo, prec in specs:
            w = workloads.workload(name)
            es = w.energies if nsample is None else w.energies[:nsample]
            if name not in cache:
                cache.clear()
                torch.cuda.empty_cache()
                cache[name] = (pinned(workloads.voxels(w)), workloads.optical_constants(w)[:len(es)])
            vox, opt = cache[name]
            case = cases.Case(name, w.nx, w.ny, w.nz, w.num_material, list(es), angles=tuple(w.angles),
                              phys_size=w.phys_size, algorithm=algo, max_streams=1)
            entry = {"config": f"{name}: Z x Y x X = {w.nz} x {w.ny} x {w.nx}, {w.num_material} materials, "
                               f"{len(es)} energies x {w.num_angles()} E angles"
                               + (" (sample of the request)" if nsample else ""),
                     "algorithm": algo, "reference_build": prec, "patterns": len(es) * w.num_angles()}
            if not cases.reference_reads_in_bounds(case):
                entry["skipped"] = "the reference's Ewald gather would read outside the volume"
                out.append(entry)
                continue
            cpath = os.path.join(tmp, "c.case")
            rpath = os.path.join(tmp, "r.bin")
            cases.write_case_arrays(case, cpath, opt, vox)
            try:
                p = subprocess.run([os.path.join(refdir, f"cyrsoxs_ref_{prec}"), cpath, rpath, str(REF_CALLS)],
                                   capture_output=True, text=True, timeout=900)
            except subprocess.TimeoutExpired:
                entry["error"] = "reference run timed out"
                out.append(entry)
                continue
            if p.returncode != 0:
                entry["error"] = f"reference exit code {p.returncode}: {(p.stdout + p.stderr)[-300:]}"
                out.append(entry)
                continue
            rsec = [float(ln.split()[1]) for ln in p.stdout.splitlines() if ln.startswith("seconds ")]
            o = _native.Options(nx=w.nx, ny=w.ny, nz=w.nz, num_material=w.num_material, energies=list(es),
                                start_angle=w.angles[0], end_angle=w.angles[1], increment_angle=w.angles[2],
                                phys_size=w.phys_size, algorithm=algo)
            hout = torch.empty((len(es), 1, w.ny, w.nx), dtype=torch.float32, pin_memory=True).numpy()
            _native.cuda_main(o, opt, vox, out=hout)  # untimed
            esec = []
            for _ in range(REF_CALLS):
                t = time.perf_counter()
                _native.cuda_main(o, opt, vox, out=hout)
                esec.append(time.perf_counter() - t)
            ref_s, eng_s = statistics.median(rsec), statistics.median(esec)
            entry.update({"reference_s": ref_s, "reference_s_each": rsec, "engine_s": eng_s, "engine_s_each": esec,
                          "reference_patterns_per_s": entry["patterns"] / ref_s,
                          "engine_patterns_per_s": entry["patterns"] / eng_s, "engine_over_reference": ref_s / eng_s})
            if prec == "fp64":
                ref = np.fromfile(rpath, np.float64).reshape(hout.shape)
                err, npx = rel_err(hout.astype(np.float64), ref)
                # the FP64 build decides NaN pixels and Ewald planes in double, the engine in float as the
                # reference's FP32 build does: the masks may differ at the Ewald sphere's rim
                entry["engine_vs_reference_fp64"] = {
                    "max_rel_err": err, "pixels": npx,
                    "nan_mask_equal": bool(np.array_equal(np.isnan(hout), np.isnan(ref))),
                    "nan_mask_differing_pixels": int((np.isnan(hout) != np.isnan(ref)).sum())}
            out.append(entry)
            print("reference_gpu", json.dumps(entry), file=sys.stderr, flush=True)
    cache.clear()
    return {"timing": f"wall clock around one call from pinned host buffers, median of {REF_CALLS} after 1 untimed",
            "builds": "reference sources unmodified; FP32 with --use_fast_math as shipped, FP64 -DDOUBLE_PRECISION",
            "entries": out}


def _pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, max(0, int(math.ceil(q * len(xs))) - 1))]


def _lat_summary(lat_s):
    return {"p50_ms": 1000 * _pct(lat_s, 0.50), "p99_ms": 1000 * _pct(lat_s, 0.99), "max_ms": 1000 * max(lat_s)}


def _median_pass(fn, reps):
    """Run fn() reps times; return (seconds, latencies) of the median pass and all pass times."""
    runs = sorted((fn() for _ in range(max(1, reps))), key=lambda r: r[0])
    t, lat = runs[len(runs) // 2]
    return t, lat, [round(r[0], 5) for r in runs]


def served_benchmarks(args):
    """Batched and served throughput against the plain one-request-at-a-time
    path on the same GPU, with p50/p99 request latency.

    batched: the 64 uneven two-phase morphologies (20 energies x 12 E angles),
    all submitted at t = 0, device-resident (plain = cyr_simulate_device and a
    synchronisation per request, in order) and again from pinned host memory
    (plain = cyr_cuda_main per request); served = the serving engine
    (continuous batching over `--slots` slots, CUDA graphs, and request groups:
    queued same-shape requests on device buffers share one launch per kernel).
    serving: a seeded Poisson stream (200 requests/s) of requests of random
    size, materials, energies and angles with device-resident morphologies;
    plain = the same arrivals served one at a time in arrival order.  Each
    mode runs once untimed first (scratch, autotuning, graph capture); the
    batched modes are then timed `--served-reps` times and the median pass is
    reported, because one pass lasts only tens of milliseconds."""
    import torch

    from cyrsoxs_gb300 import _native, serving, workloads

    def opts_for(w, strategy=0):
        return _native.Options(nx=w.nx, ny=w.ny, nz=w.nz, num_material=w.num_material, energies=w.energies,
                               start_angle=w.angles[0], end_angle=w.angles[1], increment_angle=w.angles[2],
                               phys_size=w.phys_size, morphology_type=0, strategy=strategy)

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()

    out = {}
    cs = torch.cuda.current_stream()
    # ---- batched: 64 uneven morphologies ----
    reqs, per_energy_opts = [], []
    for w in workloads.batched_set():
        dv = workloads.voxels_torch(w).contiguous()
        hv = pinned((w.num_material, w.nz, w.ny, w.nx, 4))
        hv[...] = dv.cpu().numpy()
        per_energy_opts.append(opts_for(w, strategy=1))
        reqs.append((opts_for(w), workloads.optical_constants(w), dv,
                     torch.empty(len(w.energies) * w.ny * w.nx, dtype=torch.float32, device="cuda"), hv,
                     pinned((len(w.energies), 1, w.ny, w.nx)), len(w.energies) * w.num_angles()))
    torch.cuda.synchronize()
    patterns = sum(r[6] for r in reqs)

    def plain_batch(host, strategies=None):
        t0 = time.perf_counter()
        lat = []
        for i, (o, opt, dv, dout, hv, hout, _) in enumerate(reqs):
            if strategies is not None:
                o = strategies[i]
            if host:
                _native.cuda_main(o, opt, hv, out=hout)
            else:
                _native.simulate_device(o, opt, dv.data_ptr(), dout.data_ptr(), cs.cuda_stream)
                cs.synchronize()
            lat.append(time.perf_counter() - t0)
        return time.perf_counter() - t0, lat

    def served_batch(srv, host):
        t0 = time.perf_counter()
        if host:
            ids = [srv.submit(o, opt, hv, hout) for o, opt, dv, dout, hv, hout, _ in reqs]
        else:
            ids = [srv.submit(o, opt, dv.data_ptr(), dout.data_ptr(), device=True)
                   for o, opt, dv, dout, hv, hout, _ in reqs]
        lat = [srv.wait(i)[0] for i in ids]
        return time.perf_counter() - t0, lat

    for host, name, where in ((False, "batched", "device-resident morphologies and patterns"),
                              (True, "batched_host_buffers", "morphologies and patterns in pinned host memory "
                                                            "(host<->device copies inside the timed region)")):
        plain_batch(host)
        tp, lp, tpa = _median_pass(lambda: plain_batch(host), args.served_reps)
        with serving.Server(slots=args.slots, graphs=True, groups=not args.no_groups) as srv:
            served_batch(srv, host)
            ts, ls, tsa = _median_pass(lambda: served_batch(srv, host), args.served_reps)
            st = srv.stats()
        out[name] = {
            "config": "64 seeded two-phase Euler morphologies, X = Y in {64,128,256}, Z in {16,32,64}; 20 energies x "
                      f"12 E angles each; {where}; all requests at t = 0",
            "requests": len(reqs), "patterns": patterns,
            "passes": len(tpa),
            "plain": {"patterns_per_s": patterns / tp, "seconds": tp, "pass_seconds": tpa, **_lat_summary(lp)},
            "served": {"patterns_per_s": patterns / ts, "seconds": ts, "pass_seconds": tsa, "slots": args.slots,
                       "graphs": True, "groups": not args.no_groups,
                       "graph_replays": st["graph_replays"], "graph_captures": st["graph_captures"],
                       "group_runs": st["group_runs"], "grouped_requests": st["grouped_requests"],
                       **_lat_summary(ls)},
            "speedup": tp / ts,
        }
        if not host:
            # the share of the gain that is algorithmic: plain with the reference's per-energy schedule
            plain_batch(False, per_energy_opts)
            tpe, lpe, tpea = _median_pass(lambda: plain_batch(False, per_energy_opts), args.served_reps)
            out[name]["plain_per_energy"] = {"patterns_per_s": patterns / tpe, "seconds": tpe,
                                             "pass_seconds": tpea, **_lat_summary(lpe),
                                             "note": "strategy PER_ENERGY (spectra per energy, as the reference "
                                                     "schedules the path), one request at a time"}
            out[name]["speedup_vs_per_energy"] = tpe / ts
    del reqs
    # ---- serving: Poisson stream, device-resident morphologies ----
    # requests of the same shape read one shared device morphology (read-only), so that a
    # stream long enough for a meaningful p99 fits in HBM; each has its own optical constants
    stream_reqs, shared_vox = [], {}
    for arrival, w in workloads.serving_stream(args.serve_requests):
        key = (w.nz, w.ny, w.nx, w.num_material)
        if key not in shared_vox:
            shared_vox[key] = workloads.voxels_torch(w).contiguous()
        dv = shared_vox[key]
        dout = torch.empty(len(w.energies) * w.ny * w.nx, dtype=torch.float32, device="cuda")
        stream_reqs.append((arrival, opts_for(w), workloads.optical_constants(w), dv, dout,
                            len(w.energies) * w.num_angles()))
    torch.cuda.synchronize()
    spat = sum(r[5] for r in stream_reqs)

    def plain_stream(scale=1.0):
        t0 = time.perf_counter()
        lat = []
        for arrival, o, opt, dv, dout, _ in stream_reqs:
            arrival *= scale
            now = time.perf_counter() - t0
            if now < arrival:
                time.sleep(arrival - now)
            _native.simulate_device(o, opt, dv.data_ptr(), dout.data_ptr(), cs.cuda_stream)
            cs.synchronize()
            lat.append(time.perf_counter() - t0 - arrival)
        return time.perf_counter() - t0, lat

    def served_stream(srv, scale=1.0):
        t0 = time.perf_counter()
        ids, arrivals = [], []
        for arrival, o, opt, dv, dout, _ in stream_reqs:
            arrival *= scale
            now = time.perf_counter() - t0
            if now < arrival:
                time.sleep(arrival - now)
            ids.append(srv.submit(o, opt, dv.data_ptr(), dout.data_ptr(), device=True))
        lat = [srv.wait(i)[0] for i in ids]
        return time.perf_counter() - t0, lat

    plain_stream()
    tps, lps = plain_stream()
    # the same requests at higher arrival rates (the seeded arrival times scaled): where the capacity saturates
    sweep = []
    with serving.Server(slots=args.slots, groups=not args.no_groups) as srv:
        served_stream(srv)
        tss, lss = served_stream(srv)
        sst = srv.stats()
        for rate in (1000.0, 5000.0):
            scale = 200.0 / rate
            tpr, lpr = plain_stream(scale)
            tsr, lsr = served_stream(srv, scale)
            sweep.append({"rate_per_s": rate, "arrival_span_s": stream_reqs[-1][0] * scale,
                          "plain": {"patterns_per_s": spat / tpr, "seconds": tpr, **_lat_summary(lpr)},
                          "served": {"patterns_per_s": spat / tsr, "seconds": tsr, **_lat_summary(lsr)},
                          "speedup": tpr / tsr})
    mean_vox = sum(r[3].numel() // 4 for r in stream_reqs) / len(stream_reqs)
    out["serving"] = {
        "config": f"{len(stream_reqs)} requests, Poisson arrivals at 200/s (seeded); volume log-uniform in "
                  "[32x128^2, 128x512^2] (95% FFT-friendly sizes, 5% arbitrary), 2-4 materials, 1-100 energies, 6-36 E angles; "
                  f"device-resident morphologies (mean {mean_vox / 1e6:.1f} M voxels x materials; "
                  f"{len(shared_vox)} distinct shapes, requests of one shape share its morphology)",
        "requests": len(stream_reqs), "patterns": spat, "arrival_span_s": stream_reqs[-1][0],
        "plain": {"patterns_per_s": spat / tps, "seconds": tps, **_lat_summary(lps)},
        "served": {"patterns_per_s": spat / tss, "seconds": tss, "slots": args.slots, "groups": not args.no_groups,
                   "group_runs": sst["group_runs"], "grouped_requests": sst["grouped_requests"], **_lat_summary(lss)},
        "speedup": tps / tss,
        "rate_sweep": sweep,
    }
    del stream_reqs, shared_vox
    torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch

    rank, world, local = dist_env()
    if world != args.gpus:
        print(f"warning: --gpus {args.gpus} but WORLD_SIZE {world}", file=sys.stderr)
    torch.cuda.set_device(local)
    if args.served_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "served": served_benchmarks(args)}), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from cyrsoxs_gb300 import _native, workloads

    w = workloads.workload(args.workload)
    nang = w.num_angles()
    energies = shard_energies(w.energies, rank, world, args.energies_per_step)
    wstep = workloads.workload(args.workload, energies=energies)
    optical = workloads.optical_constants(wstep)
    vox = workloads.voxels_torch(w).contiguous()
    opts = _native.Options(nx=w.nx, ny=w.ny, nz=w.nz, num_material=w.num_material, energies=energies,
                           start_angle=w.angles[0], end_angle=w.angles[1], increment_angle=w.angles[2],
                           phys_size=w.phys_size, morphology_type=0, strategy=args.strategy)
    P = w.nx * w.ny
    out = torch.empty(len(energies) * P, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        _native.simulate_device(opts, optical, vox.data_ptr(), out.data_ptr(), sptr)

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # timed region: device-resident throughput
    step_ms = []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    barrier()
    total_ms = t0.elapsed_time(t1)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    if dist is not None:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    patterns = world * len(energies) * nang * args.steps
    value = patterns / (total_ms / 1000.0)

    # per-kernel durations (events around every launch on its stream)
    prof_steps = max(1, min(args.steps, 5))
    _native.profile_begin(4096)
    for _ in range(prof_steps):
        step()
    torch.cuda.synchronize()
    kernels, dropped = _native.profile_end()
    launches_per_step = sum(n for n, _, _ in kernels.values()) / prof_steps
    info = _native.plan_info(opts)
    nvol, planes = info["nvol"], info["planes"]
    npk = info["packed_volumes"] if info["fields"] else 0
    eb = info["energy_batch"]
    batch = len(energies) / math.ceil(len(energies) / eb)  # mean energies per batched launch
    ab = lambda k: algorithmic_bytes(k, w, nvol, nang, planes, batch, npk, energies)  # noqa: E731
    # dominant kernel: the largest share of the step among kernels with an algorithmic byte count
    dom = max(((k, v) for k, v in kernels.items() if ab(k)), key=lambda kv: kv[1][1])
    dom_name, (_, dom_ms, dom_n) = dom
    peak, peak_kind = load_peaks()
    dom_bytes = ab(dom_name)
    achieved = dom_bytes / (dom_ms / dom_n / 1000.0) / 1e9
    traffic = load_traffic(w.name).get(dom_name)
    # a "call" is one timed launch of the kernel's work (for Euler input the build kernels are
    # launched as a converted/trigonometric pair of which one returns at entry)
    kernel_table = {k: {"launches_per_step": n / prof_steps, "calls_per_step": c / prof_steps, "ms_per_call": ms / c,
                        "gbs": (ab(k) or 0) / (ms / c / 1000.0) / 1e9}
                    for k, (n, ms, c) in kernels.items()}

    result = {
        "metric": METRIC, "value": value, "unit": "patterns/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded morphology with the configuration's shapes and distributions)",
        "config": {"workload": f"{w.name}: Z x Y x X = {w.nz} x {w.ny} x {w.nx}, {w.num_material} materials (Euler), "
                               f"{nang} E angles ({w.angles[0]:g}:{w.angles[2]:g}:{w.angles[1]:g}), {len(energies)} energies per step per GPU, physSize "
                               f"{w.phys_size} nm, k = z",
                   "path": "plain (one request at a time, device-resident morphology)",
                   "l2": "inputs larger than L2 (morphology 4.3 GB)",
                   "patterns_per_step": world * len(energies) * nang},
        "latency_ms": {"p50_step": statistics.median(step_ms),
                       "p99_step": sorted(step_ms)[min(len(step_ms) - 1, int(math.ceil(0.99 * len(step_ms))) - 1)]},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": dom_bytes},
        "kernels": kernel_table,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "plan": info,
        "autotune": _native.tuning_report().strip().splitlines(),
        "clocks": None,
    }
    if rank == 0:
        result["clocks"] = clocks.summary()

    # e2e through the C ABI with host buffers (pinned), copies inside the timed region
    host_vox = torch.empty(vox.shape, dtype=torch.float32, pin_memory=True)
    host_vox.copy_(vox)
    host_vox_np = host_vox.numpy()
    del vox, out
    torch.cuda.empty_cache()
    host_out = torch.empty((len(energies), 1, w.ny, w.nx), dtype=torch.float32, pin_memory=True).numpy()
    _native.cuda_main(opts, optical, host_vox_np)  # warm (scratch allocation)
    e2e_times = []
    barrier()
    for _ in range(args.e2e_steps):
        t = time.perf_counter()
        _native.cuda_main(opts, optical, host_vox_np, out=host_out)
        e2e_times.append(time.perf_counter() - t)
    barrier()
    e2e_s = sum(e2e_times)
    if dist is not None:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    result["e2e"] = {"value": world * len(energies) * nang * args.e2e_steps / e2e_s, "unit": "patterns/s",
                     "h2d_bytes_per_step": int(host_vox_np.nbytes + optical.nbytes),
                     "d2h_bytes_per_step": int(host_out.nbytes), "steps": args.e2e_steps,
                     "step_ms": [round(t * 1e3, 2) for t in e2e_times],
                     "api": "cyr_cuda_main (host buffers)"}

    if rank == 0 and world == 1 and not args.skip_cpu:
        result["precision"], result["cpu_baseline"] = precision_study(args, w, energies, optical, host_vox_np,
                                                                      2 if info["fields"] else 1)
    if rank == 0 and world == 1 and not args.skip_fp64:
        result["precision_fp64_gpu"] = fp64_study(args)
    if rank == 0 and world == 1 and not args.skip_served:
        del host_vox, host_vox_np
        torch.cuda.empty_cache()
        result["served"] = served_benchmarks(args)
    if rank == 0 and world == 1 and not args.skip_reference_gpu:
        torch.cuda.empty_cache()
        result["reference_gpu"] = reference_gpu_baseline(args)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

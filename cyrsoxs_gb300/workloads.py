"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (no public dataset is involved).

* ``c1``: 2 materials on Z x Y x X = 32 x 256 x 256, physSize 5 nm; material 0
  is a sphere of radius 40 voxels (vfrac 1 inside) in a matrix of material 1;
  S = 0.5; theta, psi uniform random per voxel; 280/285/290 eV with
  delta = beta = 1e-3 + 5e-3 L(E) (Lorentzian at 285 eV, 1 eV wide);
  E angles 0:15:165.  Both materials get the same isotropic constants, so
  the dielectric tensor is (n^2 - 1) I everywhere and only the DC bin is
  non-zero: the patterns are rounding noise.  ``c1_aniso`` is the same case
  with the perpendicular resonance amplitude halved, which gives the
  orientation field contrast; precision is checked on it.
* ``c2`` / ``headline``: 4 materials; vfrac from seeded smooth random fields
  arg-maxed into 4 phases and smoothed over ~3 voxels; S ~ U(0, 1); a smooth
  random director field (theta = acos n_z, psi = atan2(n_y, n_x)); energies
  270-300 eV with 2 Lorentzian resonances per material; 36 E angles
  (0:5:175).  ``c2`` is 128 x 512 x 512 with physSize 2 nm; ``headline`` is
  the 512^2 x 256 shape (Z x Y x X = 256 x 512 x 512).
* ``c4``: the large precision study, 3 materials on Z x Y x X = 256 x 1024 x
  1024 with the same generators, 10 energies, 24 E angles (0:7.5:172.5).

Arrays come back in the engine's layout: voxels float32 [M][Z][Y][X][4]
(Euler s1 = (S, theta, psi, Vfrac)) and optical float32 [E][M][4]
(delta_par, beta_par, delta_perp, beta_perp).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    nz: int
    ny: int
    nx: int
    num_material: int
    energies: list
    angles: tuple
    phys_size: float
    seed: int = 0
    kind: str = "random"  # sphere | random
    extra: dict = field(default_factory=dict)

    @property
    def nvox(self) -> int:
        return self.nx * self.ny * self.nz

    def num_angles(self) -> int:
        s, e, d = self.angles
        return int(round((e - s) / d + 1)) if abs(e - s) > 1e-6 else 1


def _lorentz(e, e0, width):
    return 1.0 / (1.0 + ((e - e0) / (0.5 * width)) ** 2)


def workload(name: str, energies=None) -> Workload:
    if name == "c1":
        return Workload("c1", 32, 256, 256, 2, energies or [280.0, 285.0, 290.0], (0.0, 165.0, 15.0), 5.0, 0, "sphere")
    if name == "c1_aniso":
        return Workload("c1_aniso", 32, 256, 256, 2, energies or [280.0, 285.0, 290.0], (0.0, 165.0, 15.0), 5.0, 0,
                        "sphere", extra={"perp_amplitude": 0.5})
    if name == "c2":
        es = energies or [float(e) for e in np.linspace(270.0, 300.0, 50)]
        return Workload("c2", 128, 512, 512, 4, es, (0.0, 175.0, 5.0), 2.0, 2, "random")
    if name == "headline":
        es = energies or [float(e) for e in np.linspace(270.0, 300.0, 50)]
        return Workload("headline", 256, 512, 512, 4, es, (0.0, 175.0, 5.0), 2.0, 7, "random")
    if name == "z64":  # the c2 physics on a 64 x 512 x 512 grid: a profiling size (about 3.5 GB on the device)
        es = energies or [float(e) for e in np.linspace(270.0, 300.0, 50)]
        return Workload("z64", 64, 512, 512, 4, es, (0.0, 175.0, 5.0), 2.0, 2, "random")
    if name == "cube256":  # the headline physics on a 256^3 grid: a profiling size (about 3 GB on the device)
        es = energies or [float(e) for e in np.linspace(270.0, 300.0, 50)]
        return Workload("cube256", 256, 256, 256, 4, es, (0.0, 175.0, 5.0), 2.0, 5, "random")
    if name == "c4":  # large precision study: 3 materials on 256 x 1024 x 1024, 10 energies x 24 E angles
        es = energies or [float(e) for e in np.linspace(270.0, 300.0, 10)]
        return Workload("c4", 256, 1024, 1024, 3, es, (0.0, 172.5, 7.5), 2.0, 4, "random")
    if name == "small":
        return Workload("small", 16, 64, 64, 2, energies or [284.0, 286.0], (0.0, 150.0, 30.0), 5.0, 3, "random")
    raise ValueError(f"unknown workload {name}")


def batched_set(seed: int = 3) -> list:
    """The batched configuration: 64 seeded two-phase morphologies of uneven
    sizes, X = Y in {64, 128, 256} and Z in {16, 32, 64}, each with 20
    energies (280-290 eV) and 12 E angles (0:15:165), physSize 5 nm."""
    rng = np.random.Generator(np.random.PCG64(seed))
    es = [float(e) for e in np.linspace(280.0, 290.0, 20)]
    out = []
    for i in range(64):
        xy = int(rng.choice([64, 128, 256]))
        z = int(rng.choice([16, 32, 64]))
        out.append(Workload(f"batched_{i}", z, xy, xy, 2, es, (0.0, 165.0, 15.0), 5.0, seed=1000 + i))
    return out


def _smooth_sizes(lo: int, hi: int) -> list:
    """FFT-friendly sizes (2^a 3^b 5^c 7^d) in [lo, hi]."""
    out = []
    for n in range(lo, hi + 1):
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        if m == 1:
            out.append(n)
    return out


def serving_stream(n_requests: int, rate: float = 200.0, seed: int = 5) -> list:
    """The serving configuration: Poisson arrivals (mean `rate` per second) of
    requests whose volume is log-uniform between 32 x 128^2 and 128 x 512^2
    voxels, with 2-4 materials, 1-100 energies and 6-36 E angles.  95% of the
    sizes are quantised to FFT-friendly lengths (2^a 3^b 5^c 7^d); 5% keep
    arbitrary lengths (prime factors above 7 run as Bluestein transforms).
    Returns [(arrival_s, Workload)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    arbitrary = np.random.Generator(np.random.PCG64(seed + 1)).uniform(size=n_requests) < 0.05
    xy_sizes = _smooth_sizes(128, 512)
    z_sizes = _smooth_sizes(32, 128)
    t, out = 0.0, []
    for i in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        vol = math.exp(rng.uniform(math.log(32 * 128 * 128), math.log(128 * 512 * 512)))
        # split the volume between Z (a quarter of the XY side, as in the bounds) and X = Y
        side = (4.0 * vol) ** (1.0 / 3.0)
        xy = min(xy_sizes, key=lambda n: abs(math.log(n / side)))
        z = min(z_sizes, key=lambda n: abs(math.log(n / max(32.0, min(128.0, vol / (xy * xy))))))
        if arbitrary[i]:
            xy = int(min(512, max(128, round(side))))
            z = int(min(128, max(32, round(vol / (xy * xy)))))
        m = int(rng.integers(2, 5))
        ne = int(rng.integers(1, 101))
        na = int(rng.integers(6, 37))
        inc = 180.0 / na
        es = [float(e) for e in np.linspace(270.0, 300.0, ne)] if ne > 1 else [285.0]
        out.append((t, Workload(f"serve_{i}", z, xy, xy, m, es, (0.0, inc * (na - 1), inc), 2.0, seed=2000 + i)))
    return out


def optical_constants(w: Workload) -> np.ndarray:
    """[E][M][4] float32."""
    out = np.zeros((len(w.energies), w.num_material, 4), np.float64)
    if w.kind == "sphere":
        perp = w.extra.get("perp_amplitude", 1.0)
        for i, e in enumerate(w.energies):
            L = _lorentz(e, 285.0, 1.0)
            out[i, :, 0:2] = 1e-3 + 5e-3 * L
            out[i, :, 2:4] = 1e-3 + perp * 5e-3 * L
        return out.astype(np.float32)
    rng = np.random.Generator(np.random.PCG64(w.seed + 17))
    for m in range(w.num_material):
        e0 = rng.uniform(278.0, 292.0, 2)
        amp = rng.uniform(2e-3, 8e-3, 2)
        wid = rng.uniform(0.5, 2.0, 2)
        aniso = rng.uniform(0.3, 0.9)
        for i, e in enumerate(w.energies):
            L = sum(a * _lorentz(e, c, s) for a, c, s in zip(amp, e0, wid))
            base = 1e-3 * (1 + 0.2 * m)
            out[i, m] = (base + L, 0.4 * base + 0.5 * L, base + aniso * L, 0.4 * base + 0.5 * aniso * L)
    return out.astype(np.float32)


def _torch_device(prefer_cuda: bool):
    import torch

    return torch, torch.device("cuda" if (prefer_cuda and torch.cuda.is_available()) else "cpu")


def voxels_torch(w: Workload, prefer_cuda: bool = True):
    """The morphology as a torch float32 tensor [M][Z][Y][X][4] (on the GPU when available)."""
    torch, dev = _torch_device(prefer_cuda)
    import torch.nn.functional as F

    g = torch.Generator(device=dev)
    g.manual_seed(w.seed)
    M, Z, Y, X = w.num_material, w.nz, w.ny, w.nx
    out = torch.empty((M, Z, Y, X, 4), dtype=torch.float32, device=dev)
    if w.kind == "sphere":
        z = torch.arange(Z, device=dev, dtype=torch.float32).view(Z, 1, 1)
        y = torch.arange(Y, device=dev, dtype=torch.float32).view(1, Y, 1)
        x = torch.arange(X, device=dev, dtype=torch.float32).view(1, 1, X)
        d = torch.sqrt((x - X / 2) ** 2 + (y - Y / 2) ** 2 + (z - Z / 2) ** 2)
        inside = (d <= 40.0).float()
        fr = [inside, 1.0 - inside]
        for m in range(M):
            out[m, ..., 0] = 0.5
            out[m, ..., 1] = torch.rand((Z, Y, X), generator=g, device=dev) * math.pi
            out[m, ..., 2] = torch.rand((Z, Y, X), generator=g, device=dev) * (2 * math.pi)
            out[m, ..., 3] = fr[m] if m < 2 else 0.0
        return out

    def smooth(t, k):
        t = t.view(1, 1, Z, Y, X)
        for _ in range(2):
            t = F.avg_pool3d(t, k, stride=1, padding=k // 2, count_include_pad=False)
        return t.view(Z, Y, X)

    # phases: arg-max of smooth random fields, then smoothed over ~3 voxels
    best = None
    label = torch.zeros((Z, Y, X), dtype=torch.int64, device=dev)
    for m in range(M):
        f = smooth(torch.randn((Z, Y, X), generator=g, device=dev), 7)
        if best is None:
            best = f
        else:
            upd = f > best
            label[upd] = m
            best = torch.maximum(best, f)
    del best
    total = torch.zeros((Z, Y, X), dtype=torch.float32, device=dev)
    for m in range(M):
        v = smooth((label == m).float(), 3)
        out[m, ..., 3] = v
        total += v
    out[..., 3] /= total.clamp_min(1e-6)
    del total, label
    for m in range(M):
        out[m, ..., 0] = torch.rand((Z, Y, X), generator=g, device=dev)
        n = [smooth(torch.randn((Z, Y, X), generator=g, device=dev), 5) for _ in range(3)]
        norm = torch.sqrt(n[0] ** 2 + n[1] ** 2 + n[2] ** 2).clamp_min(1e-12)
        nz = (n[2] / norm).clamp(-1.0, 1.0)
        out[m, ..., 1] = torch.acos(nz)
        out[m, ..., 2] = torch.atan2(n[1], n[0]) % (2 * math.pi)
        del n, norm, nz
    return out


def voxels(w: Workload) -> np.ndarray:
    """The morphology as a numpy float32 array [M][Z][Y][X][4]."""
    return voxels_torch(w).cpu().numpy()

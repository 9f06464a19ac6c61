"""Seeded synthetic cases for the scattering path, shared by the golden-vector
script, the oracle tests and the GPU parity tests.

Every case is regenerated bit-identically from its seed (numpy PCG64), so only
the reference's outputs are stored as fixtures (``ref_<name>_fp32.bin``,
``ref_<name>_fp64.bin``), never the inputs.

A case mirrors what the reference's Python front end receives
(src/pymain.cpp:173-240): the InputData options, per-energy optical constants
[delta_par, beta_par, delta_perp, beta_perp] per material
(include/PyClass/RefractiveIndex.h:78-109) and the voxel array in the
reference's internal layout, Voxel::s1 per (material, z, y, x)
(include/Input/Input.h:59-94), after the VoxelData rule that zeroes theta and
psi where S == 0 (include/PyClass/VoxelData.h:164-170).

The case-file format is the one oracle/ref/ref_driver.cpp reads.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

EULER, VECTOR = 0, 1
NN, LINEAR = 0, 1
PARTIAL, FULL = 0, 1
LAB, MATERIAL = 1, 0  # the reference's ReferenceFrame bool values (include/Datatypes.h:77-82)


@dataclass
class Case:
    name: str
    nx: int
    ny: int
    nz: int
    num_material: int
    energies: list
    angles: tuple = (0.0, 165.0, 15.0)  # start, end, increment (degrees)
    phys_size: float = 5.0
    morphology: int = EULER
    windowing: int = 0
    interpolation: int = LINEAR
    scatter: int = PARTIAL
    rot_mask: int = 0
    algorithm: int = 0
    max_streams: int = 1
    frame: int = LAB
    case_type: int = 0
    kvecs: list = field(default_factory=lambda: [[0.0, 0.0, 1.0]])
    detector: tuple = (0.0, 0.0, 1.0)
    mode: int = 0  # 0 = full launch, 1 = computePolarization debug path
    pol_energy: float = 0.0
    pol_eangle: float = 0.0
    seed: int = 0
    geometry: str = "sphere"  # sphere | blobs
    aniso: float = 0.5  # perpendicular resonance amplitude relative to parallel


def lorentz(e, e0, width):
    return 1.0 / (1.0 + ((e - e0) / (0.5 * width)) ** 2)


def optical_constants(case: Case) -> np.ndarray:
    """[E][M][4] float32 optical constants with seeded Lorentzian resonances."""
    rng = np.random.Generator(np.random.PCG64(case.seed + 1000))
    out = np.zeros((len(case.energies), case.num_material, 4), np.float64)
    for m in range(case.num_material):
        e0 = 285.0 + rng.uniform(-3.0, 3.0)
        amp = 5e-3 * (1.0 + 0.5 * m)
        base = 1e-3 * (1.0 + 0.3 * m)
        for i, e in enumerate(case.energies):
            L = lorentz(e, e0, 1.0 + 0.2 * m)
            out[i, m, 0] = base + amp * L  # delta_par
            out[i, m, 1] = 0.4 * base + 0.6 * amp * L  # beta_par
            out[i, m, 2] = base + case.aniso * amp * L  # delta_perp
            out[i, m, 3] = 0.4 * base + 0.6 * case.aniso * amp * L  # beta_perp
    return out.astype(np.float32)


def _vfrac(case: Case, rng) -> np.ndarray:
    """[M][Z][Y][X] volume fractions that sum to 1."""
    nz, ny, nx, M = case.nz, case.ny, case.nx, case.num_material
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    if case.geometry == "sphere":
        r = 0.3 * min(nx, ny) if nz == 1 else 0.3 * min(nx, ny, max(nz, 2) * 2)
        d = np.sqrt((x - nx / 2 + 0.3) ** 2 + (y - ny / 2 - 0.2) ** 2 + ((z - nz / 2) * (nz > 1)) ** 2)
        inside = np.clip(r + 0.5 - d, 0.0, 1.0)  # one-voxel soft edge
        fr = [inside]
        rest = 1.0 - inside
        for m in range(1, M):
            share = rest / (M - 1)
            fr.append(share)
        return np.stack(fr).astype(np.float64)
    # seeded smooth random phases
    f = rng.standard_normal((M, nz, ny, nx))
    for _ in range(3):
        f = (f + np.roll(f, 1, 1) + np.roll(f, -1, 1) + np.roll(f, 1, 2) + np.roll(f, -1, 2)
             + np.roll(f, 1, 3) + np.roll(f, -1, 3)) / 7.0
    e = np.exp(3.0 * f / (f.std() + 1e-12))
    return e / e.sum(axis=0, keepdims=True)


def voxels(case: Case) -> np.ndarray:
    """[M][Z][Y][X][4] float32 in the reference's Voxel::s1 layout."""
    rng = np.random.Generator(np.random.PCG64(case.seed))
    vf = _vfrac(case, rng)
    M = case.num_material
    shape = (M, case.nz, case.ny, case.nx)
    out = np.zeros(shape + (4,), np.float32)
    S = rng.uniform(0.0, 1.0, shape)
    S[rng.uniform(size=shape) < 0.1] = 0.0  # exercise the S == 0 rule
    theta = rng.uniform(0.0, math.pi, shape)
    psi = rng.uniform(0.0, 2.0 * math.pi, shape)
    if case.morphology == EULER:
        theta = np.where(S != 0, theta, 0.0)
        psi = np.where(S != 0, psi, 0.0)
        out[..., 0] = S
        out[..., 1] = theta
        out[..., 2] = psi
        out[..., 3] = vf
    else:
        a = vf * S
        n = np.stack([np.cos(psi) * np.sin(theta), np.sin(psi) * np.sin(theta), np.cos(theta)], -1)
        s = np.sqrt(a)[..., None] * n
        out[..., 0:3] = s
        out[..., 3] = vf - a
    return out


def header_floats(case: Case):
    return (case.phys_size, case.angles[0], case.angles[1], case.angles[2], case.pol_energy, case.pol_eangle)


def write_case(case: Case, path: str) -> None:
    write_case_arrays(case, path, optical_constants(case), voxels(case))


def write_case_arrays(case: Case, path: str, opt: np.ndarray, vox: np.ndarray) -> None:
    """The case file of `case` with the given optical constants [E][M][4] and voxels [M][Z][Y][X][4]."""
    opt = np.ascontiguousarray(opt, np.float32)
    vox = np.ascontiguousarray(vox, np.float32)
    assert opt.shape == (len(case.energies), case.num_material, 4)
    assert vox.shape == (case.num_material, case.nz, case.ny, case.nx, 4)
    with open(path, "wb") as f:
        f.write(b"CYRCASE1")
        f.write(struct.pack("<6I", case.nx, case.ny, case.nz, case.num_material, len(case.energies), len(case.kvecs)))
        f.write(struct.pack("<10I", case.morphology, case.windowing, case.interpolation, case.scatter, case.rot_mask,
                            case.algorithm, case.max_streams, case.frame, case.case_type, case.mode))
        f.write(struct.pack("<6f", *header_floats(case)))
        f.write(struct.pack("<3f", *case.detector))
        f.write(np.asarray(case.energies, np.float32).tobytes())
        f.write(np.asarray(case.kvecs, np.float32).reshape(-1).tobytes())
        f.write(opt.tobytes())
        vox.tofile(f)


def num_angles(case: Case) -> int:
    """round((end - start) / inc + 1) in float, as src/cudaMain.cu:393-394."""
    s, e, d = (np.float32(v) for v in case.angles)
    if abs(float(s) - float(e)) < 1e-6:
        d = np.float32(1.0)
    return int(round(float((e - s) / d + np.float32(1.0))))


def output_shape(case: Case):
    if case.mode == 1:
        return (3, case.nz, case.ny, case.nx)
    return (len(case.energies), len(case.kvecs), case.ny, case.nx)


CASES = {
    c.name: c
    for c in [
        Case("euler_sphere", 32, 32, 16, 2, [280.0, 285.0, 290.0], seed=1),
        Case("euler_hanning_mask", 32, 32, 16, 2, [284.0, 286.5], angles=(0.0, 150.0, 30.0), windowing=1,
             rot_mask=1, seed=2, aniso=0.3),
        Case("vector_nn_full", 32, 32, 16, 3, [283.0, 287.0], morphology=VECTOR, interpolation=NN, scatter=FULL,
             seed=3, geometry="blobs"),
        Case("vector_linear", 32, 32, 16, 2, [285.0], morphology=VECTOR, seed=4, geometry="blobs",
             angles=(10.0, 100.0, 45.0)),
        Case("alg1_streams", 32, 32, 16, 2, [281.0, 289.0], algorithm=1, max_streams=2, seed=5, geometry="blobs"),
        Case("alg1_vector", 32, 32, 16, 2, [285.5], algorithm=1, max_streams=3, morphology=VECTOR, seed=6,
             rot_mask=1, geometry="blobs"),
        Case("nonsquare", 40, 24, 8, 2, [285.0, 290.0], seed=7, geometry="blobs", angles=(0.0, 90.0, 30.0)),
        Case("twod", 64, 64, 1, 2, [282.0, 285.0], seed=8, windowing=1),
        Case("twod_nn", 48, 48, 1, 2, [285.0], seed=9, interpolation=NN, rot_mask=1),
        Case("material_frame", 32, 32, 16, 2, [285.0], frame=MATERIAL, seed=10, geometry="blobs",
             angles=(0.0, 120.0, 40.0)),
        Case("odd_sizes", 20, 15, 7, 2, [284.0, 286.0], seed=11, geometry="blobs", angles=(0.0, 165.0, 55.0)),
        Case("single_angle", 32, 32, 16, 2, [285.0], seed=12, angles=(30.0, 30.0, 0.0)),
        Case("four_materials", 32, 32, 16, 4, [278.0, 285.0, 292.0], seed=13, geometry="blobs",
             angles=(0.0, 150.0, 30.0)),
        Case("beam_divergence", 32, 32, 16, 2, [285.0], case_type=1, kvecs=[[0.0, 0.15, 1.0], [0.1, 0.0, 1.0]],
             seed=14, geometry="blobs", angles=(0.0, 90.0, 45.0)),
        Case("grazing", 32, 32, 16, 2, [285.0], case_type=2, kvecs=[[0.0, 0.1, 1.0]], detector=(0.0, 0.1, 1.0),
             seed=15, geometry="blobs", angles=(0.0, 60.0, 30.0)),
        Case("pol_euler", 32, 32, 16, 2, [280.0, 285.0], mode=1, pol_energy=285.0, pol_eangle=90.0, seed=16,
             windowing=1),
        Case("pol_vector", 24, 20, 12, 3, [285.0], mode=1, pol_energy=285.0, pol_eangle=0.3, seed=17,
             morphology=VECTOR, geometry="blobs"),
        Case("pol_material", 16, 16, 8, 2, [285.0], mode=1, pol_energy=285.0, pol_eangle=1.1, seed=18,
             frame=MATERIAL, geometry="blobs"),
        Case("c1_slice", 256, 256, 32, 2, [285.0], seed=19),
    ]
}


def _normalize32(v):
    v = np.asarray(v, np.float32)
    n = np.float32(np.sqrt(np.float32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])))
    return v * np.float32(1.0 / float(n))


def reference_reads_in_bounds(case: Case, margin: float = 1e-2) -> bool:
    """True when the reference's Ewald gather stays inside the volume for this case.

    Restates the index arithmetic of include/uniaxial.h:876-947 (PARTIAL),
    :821-874 + :769-788 (FULL) and :739-753 (nearest neighbour) in float32.
    The reference reads plane Z+1 without checking Z+1 < Nz (and the NN index
    without any check), so a case is only run on a GPU when every valid pixel
    keeps its reads at least `margin` planes inside the volume.
    """
    if case.mode == 1 or case.nz == 1:
        return True
    f32 = np.float32
    start = -f32(math.pi / case.phys_size)
    dx = f32((2.0 * math.pi / case.phys_size) / (case.nx - 1))
    dy = f32((2.0 * math.pi / case.phys_size) / (case.ny - 1))
    dz = f32((2.0 * math.pi / case.phys_size) / (case.nz - 1))
    X, Y = np.meshgrid(np.arange(case.nx), np.arange(case.ny), indexing="xy")
    qx = start + X.astype(f32) * dx
    qy = start + Y.astype(f32) * dy
    valid_xy = (X != case.nx - 1) & (Y != case.ny - 1)
    kvs = [np.array([0, 0, 1], f32)] if case.case_type == 0 else [_normalize32(k) for k in case.kvecs]
    for e in case.energies:
        lam = f32(1239.84197 / f32(e))
        k = f32(2 * math.pi / lam)
        for kv in kvs:
            kx, ky, kz = k * kv[0], k * kv[1], k * kv[2]
            val = k * k - (kx + qx) * (kx + qx) - (ky + qy) * (ky + qy)
            ok = valid_xy & (val >= 0)
            t = ((-kz + np.sqrt(np.maximum(val, 0))) - start) / dz
            t = t[ok]
            if t.size == 0:
                continue
            if case.interpolation == NN:
                if np.round(t).max() > case.nz - 1 or t.max() > case.nz - 1 - 0.5 - margin:
                    return False
            else:
                lo = np.trunc(np.maximum(t - margin, 0))  # the smallest plane float rounding could pick
                hi = np.trunc(np.maximum(t + margin, 0))
                reads = lo <= case.nz - 1  # pixels that the Z > Nz-1 test does not NaN
                if reads.any() and (hi[reads] + 1).max() > case.nz - 1:
                    return False
    return True


# ---- isotropic morphologies: the analytical properties of the Born path ----
# With S = 0 every material is isotropic (phi_a = 0, include/uniaxial.h:58-169),
# and with n_par = n_perp = n the tensor Nr - phi I is vf (n^2 - 1) I, so the
# induced polarization is p = sum_m vf_m (n_m^2 - 1) E / 4 pi.  Two exact
# consequences, checked on the oracle and on the engine:
#  * scaling every (n_m^2 - 1) by one complex c scales every pattern by |c|^2;
#  * adding one constant C to every n_m^2 adds C (sum_m vf_m) E / 4 pi, which
#    for volume fractions summing to 1 is a constant field: it reaches only the
#    q = 0 bin, and the DC replacement (src/cudaMain.cu:123-176) overwrites that
#    bin from its neighbours, so the patterns do not change.

def isotropic_voxels(case: Case) -> np.ndarray:
    """The case's volume fractions with S = theta = psi = 0 (Euler layout)."""
    vf = _vfrac(case, np.random.Generator(np.random.PCG64(case.seed)))
    out = np.zeros((case.num_material, case.nz, case.ny, case.nx, 4), np.float32)
    out[..., 3] = vf
    return out


def constants_from_n2(n2: np.ndarray) -> np.ndarray:
    """[E][M] complex n^2 -> [E][M][4] float32 (delta, beta) with n_par = n_perp = sqrt(n^2)."""
    n = np.sqrt(np.asarray(n2, np.complex128))
    d, b = 1.0 - n.real, n.imag
    return np.stack([d, b, d, b], -1).astype(np.float32)


def n2_from_constants(optical: np.ndarray) -> np.ndarray:
    """[E][M][4] -> [E][M] complex n^2 of the parallel constants (n = 1 - delta + i beta)."""
    o = np.asarray(optical, np.float64)
    return (1.0 - o[..., 0] + 1j * o[..., 1]) ** 2

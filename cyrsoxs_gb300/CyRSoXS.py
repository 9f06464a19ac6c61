"""Drop-in replacement for the reference's pybind11 module ``CyRSoXS``
(usnistgov/cyrsoxs src/pymain.cpp:128-241), backed by the GB300 engine.

    from cyrsoxs_gb300 import CyRSoXS as cy

Same classes, methods, keyword names, enum values and array shapes; the same
print-and-return behaviour for validation errors (e.g.
include/Input/InputData.h:441-449).  Deliberate differences:

* Engine failures raise ``RuntimeError`` where the reference calls exit()
  (include/cudaHeaders.h:39-63) and takes the interpreter down.
* numpy views returned by ``dataToNumpy`` / ``writeAllToNumpy`` /
  ``writeToNumpy`` keep their buffer alive after ``clear()`` instead of
  dangling (the reference hands out views over memory it later deletes,
  include/PyClass/ScatteringPattern.h:121-130).
* HDF5 I/O (readFromH5, writeToH5, writeToHDF5) uses the package's own HDF5
  subset reader/writer (cyrsoxs_gb300.h5io) instead of libhdf5.
"""
from __future__ import annotations

import contextlib
import enum
import math
import os

import numpy as np
from numpy.lib.stride_tricks import as_strided

from . import _native

MAX_NUM_MATERIAL = 32
_f32 = np.float32


# ---------------------------------------------------------------------------
# Enums (src/pymain.cpp:137-171; include/Datatypes.h)
# ---------------------------------------------------------------------------
class InterpolationType(enum.IntEnum):
    NearestNeighour = 0
    Linear = 1


class FFTWindowing(enum.IntEnum):
    NoPadding = 0
    Hanning = 1


class ScatterApproach(enum.IntEnum):
    Partial = 0
    Full = 1


class MorphologyType(enum.IntEnum):
    EulerAngles = 0
    VectorMorphology = 1


class CaseType(enum.IntEnum):
    Default = 0
    BeamDivergence = 1
    GrazingIncidence = 2


class ReferenceFrame(enum.IntEnum):
    Material = 0
    Lab = 1


class MorphologyOrder(enum.IntEnum):
    ZYX = 0
    XYZ = 1


# export_values(): the enum members are also module attributes
for _e in (InterpolationType, FFTWindowing, ScatterApproach, MorphologyType, CaseType, ReferenceFrame, MorphologyOrder):
    for _m in _e:
        globals()[_m.name] = _m

_CASE_NAMES = ["Default", "BeamDivergence", "GrazingIncidence"]
_MORPH_NAMES = ["EulerAngles", "VectorMorphology"]
_INTERP_NAMES = ["Nearest Neighbour", "Trilinear interpolation"]
_WINDOW_NAMES = ["NONE", "HANNING"]
_FRAME_NAMES = ["MATERIAL", "LAB"]
_ALGO_NAMES = ["CommunicationMinimizing", "MemoryMinimizing"]
_PARAM_NAMES = ["ENERGY", "DIMENSION", "PHYSSIZE", "EANGLE", "KVectors", "MorphologyType", "CaseType",
                "DetectorCoord", "NUM_MATERIAL"]


def _feq(a, b) -> bool:
    """FEQUALS (include/Datatypes.h:151)."""
    return abs(float(a) - float(b)) < 1e-6


def _normalize(v):
    """normalizeVec in float (include/Rotation.h:490-493)."""
    v = np.asarray(v, _f32)
    n = _f32(math.sqrt(float(_f32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))))
    return (v * _f32(1.0 / float(n))).astype(_f32)


@contextlib.contextmanager
def ostream_redirect(stdout=True, stderr=True):
    """Accepted for API parity (src/pymain.cpp:136); the engine writes no C++ streams."""
    yield


# ---------------------------------------------------------------------------
# InputData (include/Input/InputData.h:430-615, PYBIND mode)
# ---------------------------------------------------------------------------
class InputData:
    def __init__(self, NumMaterial: int):
        self.NUM_MATERIAL = int(NumMaterial)
        self.energies: list = []
        self.startAngle = self.endAngle = self.incrementAngle = 0.0
        self.voxelDims = [0, 0, 0]
        self.physSize = 0.0
        self.caseType = 0
        self.morphologyType = 0
        self.morphologyOrder = -1
        self.kVectors: list = []
        self.detectorCoordinates = [0.0, 0.0, 1.0]
        self.algorithmType = 0
        self.numMaxStreams = 1
        self.interpolationType = int(InterpolationType.Linear)
        self.windowingType = int(FFTWindowing.NoPadding)
        self.rotMask = False
        self.openMP = 4
        self.scatterApproach = int(ScatterApproach.Partial)
        self.referenceFrame = True  # LAB
        self._set = [False] * len(_PARAM_NAMES)
        self._set[8] = True
        self._enable2D = False

    # required parameters
    def setEnergies(self, energies):
        e = sorted(float(_f32(x)) for x in energies)
        self.energies = e
        if any(a == b for a, b in zip(e, e[1:])):
            print("energies has duplicate entries . Can not add")
            return
        self._set[0] = True

    def setDimensions(self, Dims, MorphologyOrder):
        order = int(MorphologyOrder)
        d = [int(v) for v in Dims]
        if order == 1:  # XYZ
            self.voxelDims = [d[0], d[1], d[2]]
        elif order == 0:  # ZYX
            self.voxelDims = [d[2], d[1], d[0]]
        else:
            print("Invalid morphology order.")
            return
        self.morphologyOrder = order
        self._enable2D = self.voxelDims[2] == 1
        if self._enable2D:
            print("[INFO] 2D computation enabled")
        self._set[1] = True

    setDimension = setDimensions

    def setPhysSize(self, PhysSize):
        self.physSize = float(_f32(PhysSize))
        self._set[2] = True

    def setERotationAngle(self, StartAngle, EndAngle, IncrementAngle):
        self.startAngle, self.endAngle, self.incrementAngle = (float(_f32(v)) for v in (StartAngle, EndAngle,
                                                                                         IncrementAngle))
        if self.startAngle > self.endAngle:
            print("[ERROR]: Start EAngle cannot be greater than end EAngle")
            return
        if _feq(self.startAngle, self.endAngle):
            self.incrementAngle = 1.0
        elif _feq(self.incrementAngle, 0.0):
            print("[ERROR] :  Increment angle for Electric field rotation cannot be 0")
            return
        self._set[3] = True

    def setMorphologyType(self, morphologyType):
        self.morphologyType = int(morphologyType)
        self._set[5] = True

    def setCaseType(self, caseType):
        self.caseType = int(caseType)
        self._set[6] = True
        if self.caseType == 0:
            self.kVectors = [np.array([0, 0, 1], _f32)]
            self._set[4] = True
            self._set[7] = True

    def setKVectors(self, kVector):
        if self.caseType == 0:
            print("Cannot add kVectors for default case type")
            return
        self.kVectors.append(_normalize(kVector))
        self._set[4] = True
        if self.caseType == 1:
            self._set[7] = True

    def setDetectorCoordinates(self, detectorCoordinates):
        if self.caseType != 2:
            print("Cannot add Detector for default or Beam Divergence type")
            return
        self.detectorCoordinates = [float(_f32(v)) for v in detectorCoordinates]
        self._set[7] = True

    def setAlgorithm(self, AlgorithmID, MaxStreams=1):
        if int(AlgorithmID) >= 2:
            print("Incorrect AlgID.")
            return
        self.algorithmType = int(AlgorithmID)
        self.numMaxStreams = int(MaxStreams)

    def if2DComputation(self) -> bool:
        return self._enable2D

    def validate(self) -> bool:
        if not all(self._set):
            for name, ok in zip(_PARAM_NAMES, self._set):
                if not ok:
                    print("The value for ", name, "is not set")
        return all(self._set)

    def print(self):
        p = print
        p("Required options:")
        p("==================================================")
        p("NumMaterial          : ", self.NUM_MATERIAL)
        p("CaseType             : ", _CASE_NAMES[self.caseType])
        p("MorphologyType       : ", _MORPH_NAMES[self.morphologyType])
        X, Y, Z = self.voxelDims
        if self.morphologyOrder == 1:
            p("Dimensions [X Y Z]   :  [", X, ",", Y, ",", Z, "]")
        else:
            p("Dimensions [Z Y X]   :  [", Z, ",", Y, ",", X, "]")
        p("PhysSize             : ", self.physSize, "nm")
        p("Energy               : ", self.energies)
        p("ERotation Angle      : ", self.startAngle, " : ", self.incrementAngle, " : ", self.endAngle)
        p("Morphology Order     : ", ["ZYX", "XYZ"][self.morphologyOrder] if self.morphologyOrder in (0, 1) else "?")
        p("KVectorList           ")
        for k in self.kVectors:
            p("                     :  [", k[0], ",", k[1], ",", k[2], "]")
        p("\n")
        p("Optional options:")
        p("==================================================")
        p("Number of openMP threads : ", self.openMP)
        p("Interpolation Type       : ", _INTERP_NAMES[int(self.interpolationType)])
        p("Windowing Type           : ", _WINDOW_NAMES[int(self.windowingType)])
        p("Rotation Mask            : ", bool(self.rotMask))
        p("Reference Frame          : ", _FRAME_NAMES[int(bool(self.referenceFrame))])
        p("Algorithm                : ", _ALGO_NAMES[self.algorithmType])
        if self.algorithmType == 1:
            p("NumMaxStreams            : ", self.numMaxStreams)

    # engine options
    def _options(self) -> _native.Options:
        X, Y, Z = self.voxelDims
        kv = [np.asarray(k, _f32).tolist() for k in self.kVectors] or [[0.0, 0.0, 1.0]]
        return _native.Options(
            nx=X, ny=Y, nz=Z, num_material=self.NUM_MATERIAL, energies=self.energies, start_angle=self.startAngle,
            end_angle=self.endAngle, increment_angle=self.incrementAngle, phys_size=self.physSize,
            case_type=self.caseType, k_vectors=kv, detector=self.detectorCoordinates,
            morphology_type=self.morphologyType, ewald_interpolation=int(self.interpolationType),
            windowing=int(self.windowingType), scatter_approach=int(self.scatterApproach),
            algorithm=self.algorithmType, max_streams=self.numMaxStreams, rot_mask=int(bool(self.rotMask)),
            reference_frame=int(bool(self.referenceFrame)))

    @property
    def _nvox(self) -> int:
        return int(self.voxelDims[0]) * int(self.voxelDims[1]) * int(self.voxelDims[2])


# ---------------------------------------------------------------------------
# RefractiveIndex (include/PyClass/RefractiveIndex.h)
# ---------------------------------------------------------------------------
class RefractiveIndex:
    def __init__(self, inputData: InputData):
        self._input = inputData
        self._energies = list(inputData.energies)
        self._data = np.zeros((len(self._energies), inputData.NUM_MATERIAL, 4), _f32)  # delta/beta per energy
        self._valid = [False] * len(self._energies)

    def addData(self, OpticalConstants, Energy):
        M = self._input.NUM_MATERIAL
        vals = list(OpticalConstants)
        if len(vals) != M:
            print("Wrong input for Energy. Number not matching with number of Materials")
            return
        for v in vals:
            if len(v) != 4:
                print("Wrong number of input parameters. Parameters must be in the order of "
                      "(DeltaPara, BetaPara, DeltaPerp, , BetaPerp)")
                return
        E = float(_f32(Energy))
        idx = int(np.searchsorted(np.asarray(self._energies, _f32), _f32(E), side="left"))
        if idx >= len(self._energies) or not _feq(self._energies[idx], E):
            print("Bad Energy. Trying to add parameters for non-existent energy.")
            return
        self._data[idx] = np.asarray(vals, _f32)
        self._valid[idx] = True

    def validate(self) -> bool:
        if all(self._valid):
            return True
        for e, ok in zip(self._energies, self._valid):
            if not ok:
                print("Optical constants data missing for energy = ", e, "eV")
        return False

    def clear(self):
        self._data = np.zeros((0, self._input.NUM_MATERIAL, 4), _f32)

    def print(self):
        for i, e in enumerate(self._energies):
            print("Energy = ", e)
            for m in range(self._input.NUM_MATERIAL):
                d = self._data[i, m] if i < len(self._data) else np.zeros(4, _f32)
                npar = complex(1 - d[0], d[1])
                nper = complex(1 - d[2], d[3])
                print("Material = ", m, "npara = ", npar, "nperp = ", nper)

    def getRefractiveIndexData(self) -> np.ndarray:
        """[E][M][4] optical constants (delta_par, beta_par, delta_perp, beta_perp)."""
        return self._data


# ---------------------------------------------------------------------------
# VoxelData (include/PyClass/VoxelData.h)
# ---------------------------------------------------------------------------
def _xyz_to_zyx(a: np.ndarray, dims, ncomp: int) -> np.ndarray:
    """H5::XYZ_to_ZYX (include/Input/readH5.h:164-184): [X][Y][Z](c) -> [Z][Y][X](c)."""
    X, Y, Z = dims
    a = np.asarray(a).reshape((X, Y, Z) + ((ncomp,) if ncomp > 1 else ()))
    return np.ascontiguousarray(np.transpose(a, (2, 1, 0) + ((3,) if ncomp > 1 else ())))


class VoxelData:
    def __init__(self, InputData: InputData):
        self._input = InputData
        M = InputData.NUM_MATERIAL
        if M > MAX_NUM_MATERIAL:
            print("Maximum number of material is set to be 32. Please increase the number of materials. Exiting")
            self._voxel = None
            return
        self._voxel = np.zeros((M, InputData._nvox, 4), _f32)
        self._valid = [False] * M

    def _check(self, MaterialID, want_euler: bool) -> bool:
        inp = self._input
        if want_euler and inp.morphologyType != 0:
            print("Error: [Expected]: Euler Angles / Spherical Coordinates. [Found:] VectorMorphology\n")
            return False
        if not want_euler and inp.morphologyType == 0:
            print("Error: [Expected]: Vector Morphology [Found:] Euler Angles. Returning\n")
            return False
        if int(MaterialID) > inp.NUM_MATERIAL or int(MaterialID) == 0:
            raise RuntimeError(
                "Number of material does not match with the compiled version. matID must range from 1 to NUM_MATERIAL")
        if self._valid[int(MaterialID) - 1]:
            print("The material is already set. Please first reset to add the entries. Returning.")
            return False
        return True

    def _flat(self, a, ncomp=1):
        a = np.ascontiguousarray(a, dtype=_f32)
        if self._input.morphologyOrder == 1:
            a = _xyz_to_zyx(a, self._input.voxelDims, ncomp)
        return a.reshape(-1, ncomp) if ncomp > 1 else a.reshape(-1)

    def addVoxelData(self, *args, **kw):
        """Three overloads (src/pymain.cpp:205-211):
        (AlignedData, UnalignedData, MaterialID), (S, Theta, Psi, Vfrac, MaterialID), (Vfrac, MaterialID)."""
        names = list(kw)
        if "AlignedData" in kw or "UnalignedData" in kw or (len(args) + len(kw) == 3):
            return self._add_vector(*args, **kw)
        if "S" in kw or (len(args) + len(kw) == 5):
            return self._add_euler(*args, **kw)
        if len(args) + len(names) == 2:
            return self._add_vfrac(*args, **kw)
        raise TypeError("addVoxelData(): incompatible function arguments")

    def _add_vector(self, AlignedData, UnalignedData, MaterialID):
        if not self._check(MaterialID, want_euler=False):
            return
        n = self._input._nvox
        al = self._flat(np.asarray(AlignedData, _f32).reshape(-1)[: 3 * n], 3)
        un = self._flat(np.asarray(UnalignedData, _f32).reshape(-1)[:n])
        m = int(MaterialID) - 1
        self._voxel[m, :, 0:3] = al
        self._voxel[m, :, 3] = un
        self._valid[m] = True

    def _add_euler(self, S, Theta, Psi, Vfrac, MaterialID):
        if not self._check(MaterialID, want_euler=True):
            return
        n = self._input._nvox
        s, th, ps, vf = (self._flat(np.asarray(a, _f32).reshape(-1)[:n]) for a in (S, Theta, Psi, Vfrac))
        m = int(MaterialID) - 1
        aligned = s != 0  # theta and psi are zeroed where S == 0 (VoxelData.h:164-170)
        self._voxel[m, :, 0] = s
        self._voxel[m, :, 1] = np.where(aligned, th, 0)
        self._voxel[m, :, 2] = np.where(aligned, ps, 0)
        self._voxel[m, :, 3] = vf
        self._valid[m] = True

    def _add_vfrac(self, Vfrac, MaterialID):
        if not self._check(MaterialID, want_euler=True):
            return
        n = self._input._nvox
        m = int(MaterialID) - 1
        self._voxel[m, :, 0:3] = 0
        self._voxel[m, :, 3] = self._flat(np.asarray(Vfrac, _f32).reshape(-1)[:n])
        self._valid[m] = True

    def readFromH5(self, Filename):
        from . import h5io

        if any(self._valid):
            print("Some of the material is already set. Please first reset to continue. Returning.")
            return
        inp = self._input
        try:
            morph = h5io.read_morphology(Filename, inp.morphologyType)
        except (OSError, ValueError, KeyError) as exc:
            print("[HDF5 Error]:", exc)
            return
        if morph.num_material != inp.NUM_MATERIAL:
            print("[HDF5 Error]: Number of material.")
            return
        if morph.order != inp.morphologyOrder:
            print("[HDF5 Error]: Morphology Order mismatch.")
            return
        if not _feq(inp.physSize, morph.phys_size):
            print("[HDF5 Error]: PhysSize mismatch.")
            return
        if list(morph.dims_xyz) != list(inp.voxelDims):
            print("[HDF5 Error]: Dimension mismatch.")
            return
        self._voxel[:] = morph.voxels.reshape(self._voxel.shape)
        self._valid = [True] * inp.NUM_MATERIAL

    def reset(self):
        self._valid = [False] * self._input.NUM_MATERIAL

    def writeToH5(self):
        from . import h5io

        if not self.validate():
            return
        h5io.write_morphology_dump(self._input, self._voxel)

    def clear(self):
        self._voxel = None

    def validate(self) -> bool:
        for i, ok in enumerate(self._valid):
            if not ok:
                print("Voxel Data missing / corrupt for material = ", i + 1)
                return False
        if self._voxel is None or np.isnan(self._voxel).any():
            print("Nan Present in the morphology")
            return False
        return True

    def data(self) -> np.ndarray:
        return self._voxel


# ---------------------------------------------------------------------------
# ScatteringPattern (include/PyClass/ScatteringPattern.h)
# ---------------------------------------------------------------------------
class ScatteringPattern:
    def __init__(self, InputData: InputData):
        self._input = InputData
        X, Y, _ = InputData.voxelDims
        self._data = np.zeros(len(InputData.energies) * len(InputData.kVectors or [0]) * X * Y, _f32)

    def data(self) -> np.ndarray:
        return self._data

    def clear(self):
        self._data = None

    def writeToHDF5(self, dirName="HDF5"):
        from . import h5io

        h5io.write_scattering(self._input, self._data, dirName)

    def writeToVTI(self, dirName="VTI"):
        print("Not supported")  # include/utils.h:94-96

    def _energy_id(self, energy):
        es = self._input.energies
        if energy < es[0] or energy > es[-1]:
            return None
        i = int(np.searchsorted(np.asarray(es, _f32), _f32(energy), side="left"))
        return i if i < len(es) and _feq(es[i], energy) else None

    def dataToNumpy(self, Energy, kID=0):
        inp = self._input
        if inp.caseType == 0 and kID > 0:
            print("kID cannot be greater than 0 for Default")
            return np.array([], _f32)
        if kID >= len(inp.kVectors):
            print("[ERROR] kID = ", kID, " must be smaller than kVector Size = ", len(inp.kVectors))
            return np.array([], _f32)
        eid = self._energy_id(Energy)
        if eid is None:
            print("[ERROR]: Wrong EnergyID")
            return np.array([], _f32)
        k = inp.kVectors[kID]
        print("[INFO] kVector = [", k[0], ",", k[1], ",", k[2], "]")
        X, Y, _ = inp.voxelDims
        off = eid * X * Y * len(inp.kVectors) + kID * X * Y
        # shape (Ny, Nx) with strides (Ny, 1) elements, as the reference builds the view (:132-136)
        return as_strided(self._data[off:], shape=(Y, X), strides=(4 * Y, 4))

    writeToNumpy = dataToNumpy

    def writeAllToNumpy(self, kID=0):
        inp = self._input
        if inp.caseType == 0 and kID > 0:
            print("kID cannot be greater than 0 for Default")
            return np.array([], _f32)
        if kID >= len(inp.kVectors):
            print("[ERROR] kID = ", kID, " must be smaller than kVector Size = ", len(inp.kVectors))
            return np.array([], _f32)
        k = inp.kVectors[kID]
        print("[INFO] kVector = [", k[0], ",", k[1], ",", k[2], "]")
        X, Y, _ = inp.voxelDims
        # the reference ignores kID here and starts at the first image (:158-164)
        return as_strided(self._data, shape=(len(inp.energies), Y, X), strides=(4 * X * Y, 4 * Y, 4))


# ---------------------------------------------------------------------------
# Polarization (include/PyClass/Polarization.h)
# ---------------------------------------------------------------------------
class Polarization:
    def __init__(self, InputData: InputData):
        self._input = InputData
        X, Y, Z = InputData.voxelDims
        self._p = [np.zeros(X * Y * Z, np.complex64) for _ in range(3)]

    def clear(self):
        self._p = [None, None, None]

    def getData(self, id):
        if id not in (0, 1, 2):
            raise RuntimeError("Wrong id")
        return self._p[id]

    def writeToHDF5(self):
        from . import h5io

        h5io.write_polarization(self._input, self._p)

    def writeToNumpy(self, id):
        if id >= 3:
            print("Wrong id. Must be less than 2.")
            return np.array([], np.complex64)
        X, Y, Z = self._input.voxelDims
        return as_strided(self._p[id], shape=(Z, Y, X), strides=(8 * X * Y, 8 * Y, 8))


# ---------------------------------------------------------------------------
# Functions (src/pymain.cpp:47-126)
# ---------------------------------------------------------------------------
def launch(InputData, RefractiveIndexData, VoxelData, ScatteringPattern, WriteMetaData=True):
    """Runs the full simulation into ScatteringPattern (src/pymain.cpp:78-119)."""
    if not InputData.validate():
        print("Issues with Input Data")
        return
    if InputData.caseType != 0:
        print("This is an experimental feature which is not tested")
    if not RefractiveIndexData.validate():
        print("Issues with Energy data")
        return
    if not VoxelData.validate():
        print("Issues with Voxel Data input")
        return
    opts = InputData._options()
    out = _native.cuda_main(opts, RefractiveIndexData.getRefractiveIndexData(), VoxelData.data(),
                            streams_variant=InputData.algorithmType == 1)
    ScatteringPattern._data[: out.size] = out.reshape(-1)
    if WriteMetaData:
        _write_metadata(InputData)


def cleanup(RefractiveIndex, VoxelData, ScatteringPattern):
    VoxelData.clear()
    RefractiveIndex.clear()
    ScatteringPattern.clear()


def computePolarization(InputData, RefractiveIndex, VoxelData, Polarization, Energy, EAngle):
    """Polarization before the FFT; EAngle is used in radians, as the reference does
    (src/pymain.cpp:47-67 -> src/cudaMain.cu:1721)."""
    es = InputData.energies
    if Energy < es[0] or Energy > es[-1]:
        print("[ERROR]: Wrong Energy")
        return
    eid = int(np.searchsorted(np.asarray(es, _f32), _f32(Energy), side="left"))
    if not _feq(es[eid], Energy):
        print("[ERROR]: Wrong EnergyID")
        return
    px, py, pz = _native.compute_polarization(InputData._options(), RefractiveIndex.getRefractiveIndexData(),
                                              VoxelData.data(), float(EAngle), eid)
    for i, p in enumerate((px, py, pz)):
        Polarization._p[i][:] = p.reshape(-1)


def _write_metadata(inp: InputData, path: str = "CyRSoXS.log") -> None:
    """Run metadata next to the results (the role of printMetaData, include/utils.h:207-233)."""
    X, Y, Z = inp.voxelDims
    lines = [
        "CyRSoXS (GB300 engine): ",
        "=" * 89,
        f"Version              : {_native.version()}",
        "Size of Real         : 4",
        f"Number of material   : {inp.NUM_MATERIAL}",
        "",
        "Scaling Information:",
        "=" * 89,
        f"Number of pixel      :[{X},{Y}]",
        f"Q range              :[{-math.pi / inp.physSize},{math.pi / inp.physSize}]",
        "",
        "InputData : ",
        "=" * 89,
        f"CaseType             : {_CASE_NAMES[inp.caseType]}",
        f"Morphology Type      : {_MORPH_NAMES[inp.morphologyType]}",
        f"Reference Frame      : {_FRAME_NAMES[int(bool(inp.referenceFrame))]}({int(bool(inp.referenceFrame))})",
        f"Dimensions [Z Y X]   : [{Z} {Y} {X}]",
        f"PhysSize             : {inp.physSize}nm ",
        f"E Rotation Angle     : {inp.startAngle} : {inp.incrementAngle} : {inp.endAngle}",
        "Energies simulated   : [" + " ".join(str(e) for e in inp.energies) + " ]",
        f"Windowing Type       : {_WINDOW_NAMES[int(inp.windowingType)]}",
        f"Rotation Mask        : {int(bool(inp.rotMask))}",
        f"Interpolation Type   : {_INTERP_NAMES[int(inp.interpolationType)]}",
        "kVectors             : (" + "".join(f"[{k[0]},{k[1]},{k[2]}]" for k in inp.kVectors) + ")",
        f"Scatter Approach     : {['Partial', 'Full'][int(inp.scatterApproach)]}",
        f"Algorithm            : {_ALGO_NAMES[inp.algorithmType]}",
    ]
    try:
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
    except OSError:
        pass

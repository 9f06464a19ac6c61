"""The CyRSoXS command line on the GB300 engine:

    python -m cyrsoxs_gb300 <morphology.h5> [HDF5 output directory]

It does what the reference's executable does (src/main.cpp:107-173), from
the current directory:
* reads NumMaterial, the dimensions, the order and PhysSize from the
  morphology file;
* reads config.txt and Material1.txt .. Material<M>.txt;
* runs the simulation (cyr_cuda_main, or cyr_cuda_main_streams for
  Algorithm 1);
* writes HDF5/Energy_<E>.h5 (or the directory given), the optional morphology
  dump (DumpMorphology) and the run metadata CyRSoXS.log.

Input errors print a message and return a non-zero status instead of ending
the process from inside a library call.
"""
from __future__ import annotations

import sys

import numpy as np

from . import CyRSoXS as cy
from . import _native, config, h5io


def build_input(cfg: dict, morph: h5io.Morphology) -> cy.InputData:
    """InputData from the config settings and the morphology file's header."""
    inp = cy.InputData(NumMaterial=morph.num_material)
    inp.energies = list(cfg["energies"])  # in file order: Material<N>.txt indexes them so
    inp.startAngle, inp.incrementAngle, inp.endAngle = cfg["startAngle"], cfg["incrementAngle"], cfg["endAngle"]
    inp.voxelDims = list(morph.dims_xyz)
    inp.physSize = morph.phys_size
    inp.caseType = cfg["caseType"]
    inp.morphologyType = cfg["morphologyType"]
    inp.morphologyOrder = morph.order
    inp.kVectors = cfg["kVectors"]
    inp.detectorCoordinates = cfg["detectorCoordinates"]
    inp.algorithmType = int(cfg["algorithmType"])
    inp.numMaxStreams = int(cfg["numMaxStreams"])
    inp.interpolationType = int(cfg["ewaldsInterpolation"])
    inp.windowingType = int(cfg["windowingType"])
    inp.rotMask = bool(cfg["rotMask"])
    inp.scatterApproach = int(cfg["scatterApproach"])
    inp.referenceFrame = bool(cfg["referenceFrame"])
    return inp


def run(morphology_file: str, out_dir: str | None = None, config_file: str = "config.txt",
        material_dir: str = ".") -> int:
    try:
        cfg = config.read_config(config_file)
        morph = h5io.read_morphology(morphology_file, cfg["morphologyType"])
        optical = config.read_materials(morph.num_material, cfg["energies"], material_dir)
    except (config.ConfigError, OSError, KeyError, ValueError) as exc:
        print(exc)
        return 1
    if out_dir is not None:
        cfg["HDF5DirName"] = out_dir
    inp = build_input(cfg, morph)
    if inp.voxelDims[2] == 1:
        print("[INFO] 2D computation enabled")
    inp.print()
    if inp.caseType != 0:
        print("This is an experimental feature which is not tested. ")
    if cfg["dumpMorphology"]:
        h5io.write_morphology_dump(inp, morph.voxels)
    if np.isnan(morph.voxels).any():
        print("Nan detected in the morphology")
        return 1
    try:
        out = _native.cuda_main(inp._options(), optical, morph.voxels, streams_variant=inp.algorithmType == 1)
    except (_native.CyrError, ValueError, TypeError) as exc:
        print(exc)
        return 1
    h5io.write_scattering(inp, out, cfg["HDF5DirName"])
    cy._write_metadata(inp)
    print("Complete. Exiting ")
    return 0


def main(argv=None) -> int:
    args = sys.argv[1:] if argv is None else argv
    if len(args) < 1:
        print("Usage : python -m cyrsoxs_gb300 HDF5FileName HDF5OutputDirname [optional]")
        return 1
    return run(args[0], args[1] if len(args) > 1 else None)


if __name__ == "__main__":
    sys.exit(main())

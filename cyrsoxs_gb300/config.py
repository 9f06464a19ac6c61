"""Readers for the CyRSoXS text inputs, ``config.txt`` and ``Material<N>.txt``
(libconfig syntax; libconfig itself is not part of this stack).

The parser covers the libconfig subset these files use: settings
``name = value`` or ``name : value`` with an optional ``;`` or ``,``, scalar
numbers, strings and booleans, arrays ``[...]``, lists ``(...)``, groups
``{...}``, and ``#``, ``//`` and ``/* */`` comments.

``read_config`` follows the reference's InputData(filename) constructor
(include/Input/InputData.h:258-339); ``read_materials`` follows
readRefractiveIndexData (:341-379).
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

_TOKEN = re.compile(r"""
    (?P<ws>\s+|\#[^\n]*|//[^\n]*|/\*.*?\*/)
  | (?P<str>"(?:[^"\\]|\\.)*")
  | (?P<num>[+-]?(?:0[xX][0-9a-fA-F]+|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)L?)
  | (?P<name>[A-Za-z*][A-Za-z0-9_*\-]*)
  | (?P<punct>[=:;,\[\]\(\)\{\}])
""", re.VERBOSE | re.DOTALL)


class ConfigError(ValueError):
    pass


def _tokens(text):
    pos = 0
    out = []
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            line = text.count("\n", 0, pos) + 1
            raise ConfigError(f"parse error at line {line}: unexpected {text[pos:pos + 12]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind != "ws":
            out.append((kind, m.group(kind), text.count("\n", 0, m.start()) + 1))
    return out


class _Parser:
    def __init__(self, text):
        self.t = _tokens(text)
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None, 0)

    def take(self, want=None):
        tok = self.peek()
        if tok[0] is None or (want is not None and tok[1] != want):
            raise ConfigError(f"parse error at line {tok[2]}: expected {want!r}, found {tok[1]!r}")
        self.i += 1
        return tok

    def settings(self, end=None):
        out = {}
        while self.peek()[0] is not None and self.peek()[1] != end:
            kind, name, line = self.take()
            if kind != "name":
                raise ConfigError(f"parse error at line {line}: expected a setting name, found {name!r}")
            sep = self.take()
            if sep[1] not in ("=", ":"):
                raise ConfigError(f"parse error at line {sep[2]}: expected '=' or ':' after {name}")
            out[name] = self.value()
            if self.peek()[1] in (";", ","):
                self.take()
        return out

    def value(self):
        kind, v, line = self.peek()
        if v == "{":
            self.take("{")
            g = self.settings("}")
            self.take("}")
            return g
        if v in ("[", "("):
            close = "]" if v == "[" else ")"
            self.take(v)
            items = []
            while self.peek()[1] != close:
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take(close)
            return items
        self.take()
        if kind == "num":
            s = v.rstrip("L")
            if s.lower().startswith(("0x", "+0x", "-0x")):
                return int(s, 16)
            return float(s) if any(c in s for c in ".eE") else int(s)
        if kind == "str":
            return bytes(v[1:-1], "utf-8").decode("unicode_escape")
        if kind == "name" and v.lower() in ("true", "false"):
            return v.lower() == "true"
        raise ConfigError(f"parse error at line {line}: unexpected {v!r}")


def parse(text: str) -> dict:
    return _Parser(text).settings()


def parse_file(path: str) -> dict:
    try:
        with open(path) as f:
            text = f.read()
    except OSError as exc:
        raise ConfigError(f"Cannot read {path}") from exc
    return parse(text)


def _normalize(v):
    v = np.asarray(v, np.float32)
    return (v / np.float32(math.sqrt(float(np.dot(v.astype(np.float64), v.astype(np.float64)))))).astype(np.float32)


def read_config(path: str = "config.txt") -> dict:
    """The settings of config.txt as InputData holds them: required CaseType,
    Energies, EAngleRotation ([start, increment, end]) and MorphologyType;
    optional RotMask, EwaldsInterpolation, HDF5DirName, WindowingType,
    Algorithm, ScatterApproach, DumpMorphology, MaxStreams, ReferenceFrame;
    listKVectors (normalised) unless CaseType is 0; DetectorCoordinates
    (normalised) for grazing incidence."""
    cfg = parse_file(path)

    def req(key):
        if key not in cfg:
            raise ConfigError(f"[Input Error] No value corresponding to {key} found")
        return cfg[key]

    out = {"caseType": int(req("CaseType")), "energies": [float(e) for e in req("Energies")]}
    ang = [float(a) for a in req("EAngleRotation")]
    if len(ang) != 3:
        raise ConfigError("EAngleRotation needs 3 values")
    start, inc, end = ang
    if start > end:
        raise ConfigError("Start EAngle can not be greater than end EAngle")
    if inc == 0:
        if abs(start - end) > 1e-6:
            raise ConfigError("Increment angle = 0")
        inc = 1.0
    out.update(startAngle=start, incrementAngle=inc, endAngle=end, morphologyType=int(req("MorphologyType")))
    defaults = {"RotMask": ("rotMask", 0), "EwaldsInterpolation": ("ewaldsInterpolation", 1),
                "HDF5DirName": ("HDF5DirName", "HDF5"), "WindowingType": ("windowingType", 0),
                "Algorithm": ("algorithmType", 0), "ScatterApproach": ("scatterApproach", 0),
                "DumpMorphology": ("dumpMorphology", False), "MaxStreams": ("numMaxStreams", 1),
                "NumThreads": ("num_threads", 1)}
    for key, (field, dflt) in defaults.items():
        out[field] = cfg.get(key, dflt)
    rf = int(cfg.get("ReferenceFrame", 1))
    if rf not in (0, 1):
        raise ConfigError("Reference Frame must be 0 or 1")
    out["referenceFrame"] = rf
    if out["caseType"] == 0:
        out["kVectors"] = [[0.0, 0.0, 1.0]]
    else:
        if "listKVectors" not in cfg:
            raise ConfigError("[Input Error] No value corresponding to listKVectors found")
        out["kVectors"] = [_normalize(g["k"]).tolist() for g in cfg["listKVectors"]]
    if out["caseType"] == 2:
        out["detectorCoordinates"] = _normalize(req("DetectorCoordinates")).tolist()
    else:
        out["detectorCoordinates"] = [0.0, 0.0, 1.0]
    return out


def read_materials(num_material: int, energies, directory: str = ".") -> np.ndarray:
    """Optical constants [E][M][4] = (delta_par, beta_par, delta_perp, beta_perp)
    from Material1.txt .. Material<M>.txt, whose EnergyData<i> must match
    energy i within 1e-3 eV."""
    out = np.zeros((len(energies), num_material, 4), np.float32)
    for m in range(num_material):
        path = os.path.join(directory, f"Material{m + 1}.txt")
        cfg = parse_file(path)
        for i, e in enumerate(energies):
            g = cfg.get(f"EnergyData{i}")
            if g is None:
                raise ConfigError(f"[Input Error] No EnergyData{i} in {path}")
            if abs(float(g["Energy"]) - float(np.float32(e))) > 1e-3:
                raise ConfigError(f"[Input Error] No energy found for {e}")
            out[i, m] = (g["DeltaPara"], g["BetaPara"], g["DeltaPerp"], g["BetaPerp"])
    return out

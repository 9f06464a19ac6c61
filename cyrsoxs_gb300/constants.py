"""Optical-constant files for CyRSoXS: interpolate tabulated constants to the
simulated energies and write Material<N>.txt (the role of the reference's
scripts/generateConstants.py:28-150).

The table holds one row per tabulated energy with the energy and the four
constants in any column order (`columns` names them).  Duplicate energies
keep their first row; each requested energy is interpolated linearly between
the two tabulated energies that bracket it, and an energy outside the table
is an error.  A vacuum material has all four constants zero.
"""
from __future__ import annotations

import numpy as np

FIELDS = ("DeltaPara", "BetaPara", "DeltaPerp", "BetaPerp")


def interpolate(table, energies, columns=("Energy", "DeltaPara", "BetaPara", "DeltaPerp", "BetaPerp")) -> np.ndarray:
    """[E][4] = (delta_par, beta_par, delta_perp, beta_perp) at `energies`."""
    t = np.asarray(table, np.float64)
    col = {name: i for i, name in enumerate(columns)}
    order = np.argsort(t[:, col["Energy"]], kind="stable")
    t = t[order]
    e = t[:, col["Energy"]]
    keep = np.concatenate([[True], np.diff(e) != 0])  # first row of each duplicated energy
    t, e = t[keep], e[keep]
    req = np.asarray(energies, np.float64)
    if req.min() < e[0] or req.max() > e[-1]:
        raise ValueError(f"energies outside the tabulated range [{e[0]}, {e[-1]}]")
    return np.stack([np.interp(req, e, t[:, col[f]]) for f in FIELDS], axis=-1)


def write_material(path: str, energies, constants=None) -> None:
    """Material<N>.txt with one EnergyData<i> group per energy; constants
    [E][4] (delta_par, beta_par, delta_perp, beta_perp), or None for vacuum."""
    c = np.zeros((len(energies), 4)) if constants is None else np.asarray(constants, np.float64)
    with open(path, "w") as f:
        for i, e in enumerate(energies):
            f.write(f"EnergyData{i}:\n{{\nEnergy = {float(e)!r};\n")
            dp, bp, dq, bq = (float(v) for v in c[i])
            f.write(f"BetaPara = {bp!r};\nBetaPerp = {bq!r};\nDeltaPara = {dp!r};\nDeltaPerp = {dq!r};\n}}\n")

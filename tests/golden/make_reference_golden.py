"""Produces the golden vectors that pin the oracle: runs the reference's own
CUDA path (built unmodified by oracle/ref/Makefile into oracle/_ref/) on every
case of cases.py, in its FP32 (as shipped) and FP64 builds, and runs the NPP
warp probe on npp_cases.py.

Run on a machine with a GPU after `make -C oracle/ref REF_SRC=<reference tree>`:
    python tests/golden/make_reference_golden.py [outdir]
It writes ref_<case>_fp32.bin / ref_<case>_fp64.bin / npp_warp_out.bin and a
manifest (reference exit codes, run time, GPU name) into outdir (default:
tests/golden/, where the files are committed).  The inputs are not stored: cases.py
regenerates them from their seeds.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)

import cases  # noqa: E402
import npp_cases  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref")


def main(outdir: str) -> int:
    os.makedirs(outdir, exist_ok=True)
    manifest = {"cases": {}}
    try:
        manifest["gpu"] = subprocess.run(["nvidia-smi", "--query-gpu=name,driver_version", "--format=csv,noheader"],
                                         capture_output=True, text=True, timeout=60).stdout.strip()
    except Exception as exc:  # pragma: no cover - informational only
        manifest["gpu"] = f"unknown ({exc})"
    with tempfile.TemporaryDirectory() as tmp:
        for name, case in cases.CASES.items():
            if not cases.reference_reads_in_bounds(case):
                manifest["cases"][name] = "skipped: reference would read outside the volume"
                continue
            cpath = os.path.join(tmp, name + ".case")
            cases.write_case(case, cpath)
            entry = {}
            for prec in ("fp32", "fp64"):
                out = os.path.join(outdir, f"ref_{name}_{prec}.bin")
                t0 = time.time()
                p = subprocess.run([os.path.join(REF, f"cyrsoxs_ref_{prec}"), cpath, out], capture_output=True,
                                   text=True, timeout=600)
                entry[prec] = {"rc": p.returncode, "seconds": round(time.time() - t0, 3)}
                if p.returncode != 0:
                    entry[prec]["tail"] = (p.stdout + p.stderr)[-2000:]
                    if os.path.exists(out):
                        os.remove(out)
            manifest["cases"][name] = entry
            print(name, entry, flush=True)
        ppath = os.path.join(tmp, "npp.probe")
        npp_cases.write_probes(ppath)
        p = subprocess.run([os.path.join(REF, "npp_probe"), ppath, os.path.join(outdir, "npp_warp_out.bin")],
                           capture_output=True, text=True, timeout=600)
        manifest["npp_probe"] = {"rc": p.returncode, "tail": (p.stdout + p.stderr)[-2000:]}
        print("npp_probe", p.returncode, flush=True)
    with open(os.path.join(outdir, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    bad = [n for n, e in manifest["cases"].items() if isinstance(e, dict) and any(v["rc"] for v in e.values())]
    return 1 if bad or manifest["npp_probe"]["rc"] else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else HERE))

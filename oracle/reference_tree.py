"""Where the reference's source tree is, for the recipes and tests that read it.

Test infrastructure only.  The environment variable CYRSOXS_REFERENCE names
the tree; otherwise the copy that oracle/ref/stage_reference.sh placed in the
git-ignored reference-install folder baseline/_ref/cyrsoxs is used when it is
present.  There is no default location on the machine: with neither, the
callers skip what needs the reference.
"""
from __future__ import annotations

import os

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(REPO, "baseline", "_ref", "cyrsoxs")


def reference_tree() -> str | None:
    """The reference tree (a folder holding include/ and src/), or None."""
    for cand in (os.environ.get("CYRSOXS_REFERENCE"), STAGED):
        if cand and os.path.isdir(os.path.join(cand, "include")) and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def reference_file(*parts: str) -> str | None:
    """A file of the reference tree (e.g. reference_file("Data", "config.txt")), or None when absent."""
    tree = reference_tree()
    if tree is None:
        return None
    p = os.path.join(tree, *parts)
    return p if os.path.exists(p) else None

"""Where the golden generators find the reference tree.

``TM_REFERENCE`` names it; without that variable, a ``reference`` directory
beside the repository checkout is used. A generator stops with an error when
neither holds the reference's ``TensorMol`` package. Nothing at test time
reads the reference tree: only the generators call this.
"""
from __future__ import annotations

import os

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def reference_root() -> str:
    root = os.environ.get("TM_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
    if not os.path.isdir(os.path.join(root, "TensorMol")):
        raise SystemExit(f"reference tree not found at {root!r}: set TM_REFERENCE to the "
                         "directory that holds TensorMol/ and C_API/")
    return root

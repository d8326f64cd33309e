"""Generates tests/golden/cavity_lines.npz: the driven-cavity centre-line tables
the reference compares against in DrivenCavityLinesEval
(incompressible/navier_stokes_tools.h:572-729; data of Ghia, Ghia & Shin 1982 and
Botella & Peyret 1998 as printed there), read from the reference source.

Run from the repository root where the reference checkout is present:
    python tests/golden/make_cavity_tables.py
The GPU machine has no reference checkout; the fixture carries the tables there.
"""
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

NAMES = ["vertGhiaPosY", "vertGhia_100", "vertGhia_400", "vertGhia_1000", "horizGhiaPosX", "horizGhia100", "horizGhia400",
         "horizGhia1000", "vertBotella_1000", "horizBotella_1000"]


def tables(src: str) -> dict:
    out = {}
    for name in NAMES:
        m = re.search(r"const\s+number\s+" + re.escape(name) + r"\s*\[\s*\d+\s*\]\s*=\s*\{([^}]*)\}", src)
        if not m:
            raise SystemExit(f"table {name} not found")
        out[name] = np.array([float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()])
    return out


if __name__ == "__main__":
    ref = oracle.reference_root()
    if ref is None:
        sys.exit("the reference checkout is needed (NSREF_ROOT)")
    with open(os.path.join(ref, "incompressible", "navier_stokes_tools.h")) as f:
        t = tables(f.read())
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cavity_lines.npz")
    np.savez_compressed(path, **t)
    print(path, {k: v.shape for k, v in t.items()})

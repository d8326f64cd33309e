"""Generates tests/golden/reference_elements.npz from the REFERENCE's own code.

Run from the repository root, where the reference checkout is present:
    python tests/golden/make_reference_golden.py
It builds oracle/_ref/libnsfv1_ref.so (the unmodified reference sources
navier_stokes_fv1.cpp, stabilization.cpp, upwind.cpp, upwind_interface.cpp and
the NavierStokes base classes, compiled against the ugcore stand-in in
oracle/ugshim) and stores the reference's add_def_A_elem / add_jac_A_elem /
add_def_M_elem / add_jac_M_elem / add_rhs_elem outputs for every element type
x discretisation case on seeded distorted and affine elements. The GPU machine has
no reference checkout; these fixtures carry the reference's numbers there.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from _cases import DISC_CASES, DIM, POS_CASES, ROIDS, random_elements, random_local_u, ref_config  # noqa: E402

DT = 0.01


def fixtures():
    out = {}
    for tname, roid in ROIDS.items():
        dim = DIM[roid]
        n = 3 if roid == 8 else 5
        for ci, cfg in enumerate(DISC_CASES):
            seed = 5000 + 1000 * roid + ci
            corners = np.concatenate([random_elements(roid, n, seed), random_elements(roid, 2, seed + 7, affine=True)])
            u = random_local_u(roid, n + 2, seed + 1, zero_frac=0.2)
            uo = random_local_u(roid, n + 2, seed + 2) if cfg[3] else None
            r = oracle.ref_elem_batch(roid, ref_config(dim, cfg), corners, u, uo, DT)
            key = f"{tname}_{ci}"
            out[key + "_corners"] = corners
            out[key + "_u"] = u
            if uo is not None:
                out[key + "_uold"] = uo
            for k, v in r.items():
                out[key + "_" + k] = v
            # the same elements with the stabilisation as the convective upwind (set_pac_upwind)
            if not cfg[7]:
                r = oracle.ref_elem_batch(roid, dict(ref_config(dim, cfg), pac=True), corners, u, uo, DT)
                for k, v in r.items():
                    out[key + "_pac_" + k] = v
        # the positive upwind (non-diagonal stabilisation), with and without PAC
        for ci, cfg in enumerate(POS_CASES):
            seed = 9000 + 1000 * roid + ci
            corners = np.concatenate([random_elements(roid, n, seed), random_elements(roid, 2, seed + 7, affine=True)])
            u = random_local_u(roid, n + 2, seed + 1, zero_frac=0.2)
            uo = random_local_u(roid, n + 2, seed + 2) if cfg[3] else None
            key = f"{tname}_pos{ci}"
            out[key + "_corners"] = corners
            out[key + "_u"] = u
            if uo is not None:
                out[key + "_uold"] = uo
            for pac in (False, True):
                r = oracle.ref_elem_batch(roid, dict(ref_config(dim, cfg), pac=pac), corners, u, uo, DT)
                for k, v in r.items():
                    out[key + ("_pac_" if pac else "_") + k] = v
    return out


if __name__ == "__main__":
    if oracle.reference_root() is None:
        sys.exit("the reference checkout is needed (NSREF_ROOT)")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_elements.npz")
    np.savez_compressed(path, **fixtures())
    print(path, os.path.getsize(path))

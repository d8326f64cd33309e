"""Generates the committed golden fixtures of the oracle (tests/golden/*.npz).

Run from the repository root:  python tests/golden/make_golden.py
The fixtures pin the oracle's outputs (element-local callbacks for every
element type x configuration, and global defect / Jacobian / pattern /
colouring of two small meshes) so that the GPU machine, which has no reference
tree, checks the product against the same numbers.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from _cases import DISC_CASES, DIM, ROIDS, configure, random_elements, random_local_u  # noqa: E402
from plugin_navierstokes_gb300 import mesh  # noqa: E402

N_ELEM = 4
DT = 0.01


def element_fixtures():
    out = {}
    for tname, roid in ROIDS.items():
        dim = DIM[roid]
        for ci, cfg in enumerate(DISC_CASES):
            seed = 1000 * roid + ci
            corners = random_elements(roid, N_ELEM, seed)
            u = random_local_u(roid, N_ELEM, seed + 1, zero_frac=0.25)
            uo = random_local_u(roid, N_ELEM, seed + 2) if cfg[3] else None
            o = oracle.Oracle(dim)
            configure(o, dim, cfg)
            r = o.elem_batch(roid, corners, u, uo, DT)
            key = f"{tname}_{ci}"
            out[key + "_corners"] = corners
            out[key + "_u"] = u
            if uo is not None:
                out[key + "_uold"] = uo
            for k, v in r.items():
                out[key + "_" + k] = v
    return out


def mesh_fixtures():
    out = {}
    # 8 x 8 cavity, full upwind + FIELDS, nu = 0.01, at a seeded state
    roid, X, C = mesh.structured_quads(8)
    o = oracle.Oracle(2)
    configure(o, 2, DISC_CASES[0])
    o.set_mesh(roid, X, C)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    o.set_dirichlet(dofs, vals)
    U = (mesh.uniform(11, X.shape[0] * 3) * 2 - 1).reshape(-1, 3) * 0.5
    D, J = o.assemble(U)
    rp, ci = o.pattern()
    col, nc = o.coloring()
    Usol, st = o.newton(np.zeros_like(U), rtol=1e-10)
    out.update(quad_coords=X, quad_conn=C, quad_U=U, quad_D=D, quad_J=J, quad_rowptr=rp, quad_colidx=ci, quad_color=col,
               quad_dofs=dofs, quad_dvals=vals, quad_Usol=Usol, quad_newton_iters=st["iterations"])
    # 3 x 3 x 3 hexes, LPS + FLOW, nu = 0.0025, solenoidal state
    roid, X, C = mesh.structured_hexes(3)
    o = oracle.Oracle(3)
    configure(o, 3, DISC_CASES[1])
    o.set_mesh(roid, X, C)
    U = mesh.solenoidal_state(X, seed=1)
    D, J = o.assemble(U)
    rp, ci = o.pattern()
    col, nc = o.coloring()
    out.update(hex_coords=X, hex_conn=C, hex_U=U, hex_D=D, hex_J=J, hex_rowptr=rp, hex_colidx=ci, hex_color=col)
    # jittered triangles 6 x 6, transient full + FIELDS
    roid, X, C = mesh.jittered_triangles(6, seed=2)
    o = oracle.Oracle(2)
    configure(o, 2, DISC_CASES[0])
    o.set_mesh(roid, X, C)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    o.set_dirichlet(dofs, vals)
    U = (mesh.uniform(13, X.shape[0] * 3) * 2 - 1).reshape(-1, 3) * 0.5
    Uo = (mesh.uniform(14, X.shape[0] * 3) * 2 - 1).reshape(-1, 3) * 0.5
    D, J = o.assemble(U, Uo, DT)
    rp, ci = o.pattern()
    col, nc = o.coloring()
    out.update(tri_coords=X, tri_conn=C, tri_U=U, tri_Uold=Uo, tri_D=D, tri_J=J, tri_rowptr=rp, tri_colidx=ci, tri_color=col,
               tri_dofs=dofs, tri_dvals=vals)
    return out


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "elements.npz"), **element_fixtures())
    np.savez_compressed(os.path.join(here, "meshes.npz"), **mesh_fixtures())
    print("written")

"""The CPU oracle: geometry invariants, Jacobian consistency, golden fixtures."""
import os

import numpy as np
import pytest

import oracle
from _cases import DISC_CASES, DIM, NSH, ROIDS, configure, random_elements, random_local_u, rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
def test_geometry_invariants(roid):
    for e, corners in enumerate(random_elements(roid, 5, 77 + roid)):
        scvf, vol = oracle.geometry(roid, corners)
        dim = DIM[roid]
        for f in scvf:
            assert abs(f["shape"].sum() - 1.0) < 1e-14
            assert np.abs(f["grad"].sum(0)).max() < 1e-10
            # isoparametric: sum_k x_k (x) grad N_k = identity
            G = corners.T @ f["grad"][:, :dim]
            assert np.abs(G - np.eye(dim)).max() < 1e-10
            # normal oriented from -> to
            assert f["normal"][:dim] @ (corners[f["to"]] - corners[f["from"]]) > 0
        assert np.all(vol > 0)


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
def test_scv_volumes_partition_affine_element(roid):
    for corners in random_elements(roid, 4, 500 + roid, affine=True):
        _, vol = oracle.geometry(roid, corners)
        dim = DIM[roid]
        A = corners[1:dim + 1] - corners[0] if roid in (2, 4) else None
        if roid == 2:
            ref = abs(np.linalg.det(A)) / 2
        elif roid == 4:
            ref = abs(np.linalg.det(A)) / 6
        elif roid == 3:
            ref = abs(np.linalg.det(np.stack([corners[1] - corners[0], corners[3] - corners[0]])))
        else:
            ref = abs(np.linalg.det(np.stack([corners[1] - corners[0], corners[3] - corners[0], corners[4] - corners[0]])))
        assert abs(vol.sum() - ref) < 1e-13 * max(ref, 1e-30) * 10


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
@pytest.mark.parametrize("stab", ["fields", "without"])
@pytest.mark.parametrize("transient", [False, True])
def test_stokes_jacobian_is_defect_derivative(roid, stab, transient):
    """For Stokes flow with FIELDS (or no) stabilisation the defect is linear in
    u, so add_jac_A_elem must equal the derivative of add_def_A_elem (central
    differences). FLOW's cross terms are quadratic in u and the reference
    linearises them with the ip velocity frozen, so FLOW is not exact."""
    dim = DIM[roid]
    o = oracle.Oracle(dim)
    o.set_kinematic_viscosity(0.01)
    o.set_density(1.2)
    o.set_stokes(True)
    o.set_stabilization(stab)
    corners = random_elements(roid, 2, 300 + roid)
    u = random_local_u(roid, 2, 301 + roid)
    uo = random_local_u(roid, 2, 302 + roid) if transient else None
    r = o.elem_batch(roid, corners, u, uo, 0.01, want=("defA", "jacA"))
    n = u.shape[1]
    for e in range(2):
        J = r["jacA"][e].reshape(n, n)
        Jfd = np.zeros((n, n))
        h = 1e-6
        for j in range(n):
            up = u.copy(); um = u.copy()
            up[e, j] += h; um[e, j] -= h
            dp = o.elem_batch(roid, corners, up, uo, 0.01, want=("defA",))["defA"][e]
            dm = o.elem_batch(roid, corners, um, uo, 0.01, want=("defA",))["defA"][e]
            Jfd[:, j] = (dp - dm) / (2 * h)
        assert rel_err(J, Jfd) < 1e-7


def test_global_assembly_is_sum_of_element_callbacks():
    from plugin_navierstokes_gb300 import mesh
    roid, X, C = mesh.jittered_triangles(4, seed=5)
    o = oracle.Oracle(2)
    configure(o, 2, DISC_CASES[0])
    o.set_mesh(roid, X, C)
    U = (mesh.uniform(3, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    D, J = o.assemble(U)
    nsh, b = 3, 3
    loc = o.elem_batch(roid, X[C], U[C].transpose(0, 2, 1).reshape(len(C), -1), want=("defA", "jacA"))
    D2 = np.zeros_like(U)
    for e in range(len(C)):
        D2[C[e]] += loc["defA"][e].reshape(b, nsh).T
    assert rel_err(D, D2.ravel()) < 1e-14
    rp, ci = o.pattern()
    Jd = np.zeros((X.shape[0] * b, X.shape[0] * b))
    for r in range(X.shape[0]):
        for q in range(rp[r], rp[r + 1]):
            Jd[r * b:(r + 1) * b, ci[q] * b:(ci[q] + 1) * b] = J[q * 9:(q + 1) * 9].reshape(3, 3)
    J2 = np.zeros_like(Jd)
    for e in range(len(C)):
        Jl = loc["jacA"][e].reshape(b, nsh, b, nsh)
        for i in range(nsh):
            for j in range(nsh):
                J2[C[e][i] * b:(C[e][i] + 1) * b, C[e][j] * b:(C[e][j] + 1) * b] += Jl[:, i, :, j]
    assert rel_err(Jd, J2) < 1e-14


@pytest.mark.parametrize("gen", ["quads", "hexes", "tris"])
def test_pattern_and_coloring_properties(gen):
    from plugin_navierstokes_gb300 import mesh
    roid, X, C = {"quads": lambda: mesh.structured_quads(6), "hexes": lambda: mesh.structured_hexes(3),
                  "tris": lambda: mesh.jittered_triangles(5)}[gen]()
    o = oracle.Oracle(DIM[roid])
    o.set_mesh(roid, X, C)
    rp, ci = o.pattern()
    pairs = set()
    for r in range(X.shape[0]):
        cols = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(cols) > 0)
        pairs |= {(r, c) for c in cols}
    ref = {(a, b) for el in C for a in el for b in el}
    assert pairs == ref
    col, nc = o.coloring()
    for c in range(nc):
        nodes = C[col == c].ravel()
        assert len(nodes) == len(set(nodes.tolist()))
    if gen == "quads":
        assert nc == 4
    if gen == "hexes":
        assert nc == 8


def test_oracle_matches_golden_elements():
    g = np.load(os.path.join(GOLDEN, "elements.npz"))
    for tname, roid in ROIDS.items():
        for ci, cfg in enumerate(DISC_CASES):
            key = f"{tname}_{ci}"
            o = oracle.Oracle(DIM[roid])
            configure(o, DIM[roid], cfg)
            uo = g[key + "_uold"] if (key + "_uold") in g else None
            r = o.elem_batch(roid, g[key + "_corners"], g[key + "_u"], uo, 0.01)
            for k, v in r.items():
                assert rel_err(v, g[key + "_" + k]) < 1e-13, (key, k)


def test_oracle_matches_golden_meshes():
    from plugin_navierstokes_gb300 import mesh
    g = np.load(os.path.join(GOLDEN, "meshes.npz"))
    o = oracle.Oracle(2)
    configure(o, 2, DISC_CASES[0])
    o.set_mesh(3, g["quad_coords"], g["quad_conn"])
    o.set_dirichlet(g["quad_dofs"], g["quad_dvals"])
    D, J = o.assemble(g["quad_U"])
    assert rel_err(D, g["quad_D"]) < 1e-13 and rel_err(J, g["quad_J"]) < 1e-13
    rp, ci = o.pattern()
    assert np.array_equal(rp, g["quad_rowptr"]) and np.array_equal(ci, g["quad_colidx"])
    o3 = oracle.Oracle(3)
    configure(o3, 3, DISC_CASES[1])
    o3.set_mesh(8, g["hex_coords"], g["hex_conn"])
    D, J = o3.assemble(g["hex_U"])
    assert rel_err(D, g["hex_D"]) < 1e-13 and rel_err(J, g["hex_J"]) < 1e-13
    assert np.array_equal(o3.coloring()[0], g["hex_color"])


def test_full_upwind_limit_cycle_64():
    """Documented property of the reference discretisation: on the 64 x 64
    cavity with full upwind + FIELDS the Newton iteration enters a period-2
    cycle of the full-upwind switch at one SCVF and stalls near 1e-3."""
    pytest.importorskip("scipy")
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from plugin_navierstokes_gb300 import mesh
    roid, X, C = mesh.structured_quads(64)
    o = oracle.Oracle(2)
    o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("fields")
    o.set_mesh(roid, X, C)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    o.set_dirichlet(dofs, vals)
    rp, ci = o.pattern()
    n = X.shape[0]
    U = np.zeros(n * 3); U[dofs] = vals
    hist = []
    for _ in range(12):
        D, J = o.assemble(U)
        hist.append(np.linalg.norm(D))
        A = sp.bsr_matrix((J.reshape(-1, 3, 3), ci, rp), shape=(n * 3, n * 3)).tocsc()
        U = U - spl.spsolve(A, D)
    rel = np.array(hist) / hist[0]
    assert rel[-1] > 1e-4 and abs(rel[-1] - rel[-3]) < 1e-6 * rel[-1] * 1e3


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
def test_full_newton_jacobian_is_exact_without_upwind_and_stabilisation(roid):
    """Navier-Stokes with no upwind (flux through ip interpolation), no
    stabilisation and the full-Newton factor 1: the convective flux is
    rho (u_ip . n) u_ip and the reference's fixpoint + full-Newton parts of
    add_jac_A_elem (navier_stokes_fv1.cpp:377-550) form its exact derivative."""
    dim = DIM[roid]
    o = oracle.Oracle(dim)
    o.set_kinematic_viscosity(0.01)
    o.set_density(1.1)
    o.set_upwind("no")
    o.set_stabilization("without")
    o.set_exact_jacobian(1.0)
    corners = random_elements(roid, 2, 500 + roid)
    u = random_local_u(roid, 2, 501 + roid)
    r = o.elem_batch(roid, corners, u, None, 0.0, want=("defA", "jacA"))
    n = u.shape[1]
    for e in range(2):
        J = r["jacA"][e].reshape(n, n)
        Jfd = np.zeros((n, n))
        h = 1e-6
        for j in range(n):
            up = u.copy(); um = u.copy()
            up[e, j] += h; um[e, j] -= h
            dp = o.elem_batch(roid, corners, up, None, 0.0, want=("defA",))["defA"][e]
            dm = o.elem_batch(roid, corners, um, None, 0.0, want=("defA",))["defA"][e]
            Jfd[:, j] = (dp - dm) / (2 * h)
        assert rel_err(J, Jfd) < 1e-7


@pytest.mark.parametrize("roid", [2, 3, 4, 8])
@pytest.mark.parametrize("up,stab", [("lps", "flow"), ("full", "fields"), ("skewed", "fields")])
def test_assembly_is_translation_invariant(roid, up, stab):
    """Moving every corner by the same vector changes no geometric quantity the
    discretisation uses, so the element defect and Jacobian agree to rounding."""
    dim = DIM[roid]
    o = oracle.Oracle(dim)
    o.set_kinematic_viscosity(0.01)
    o.set_upwind(up)
    o.set_stabilization(stab)
    corners = random_elements(roid, 3, 600 + roid)
    u = random_local_u(roid, 3, 601 + roid)
    shift = np.array([0.37, -1.25, 2.5][:dim])
    r0 = o.elem_batch(roid, corners, u, None, 0.0, want=("defA", "jacA"))
    r1 = o.elem_batch(roid, corners + shift, u, None, 0.0, want=("defA", "jacA"))
    for k in ("defA", "jacA"):
        assert rel_err(r1[k], r0[k]) < 1e-11, (k, rel_err(r1[k], r0[k]))

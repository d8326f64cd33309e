"""GPU parity of the positive upwind (upwind.cpp:643-786) and the non-diagonal
FIELDS / FLOW stabilisation it selects (stabilization.cpp:244-403, 589-771).

The element callbacks are checked against the reference's own outputs
(tests/golden/reference_elements.npz, keys "<elem>_pos<i>") and the global
assembly (defect, FP64 / FP32 Jacobian, separate and fused entry points)
against the oracle, whose positive upwind is pinned to the reference by
tests/test_reference_pin.py.
Tolerance: max |gpu - ref| / max |ref| <= 1e-12 (FP64), 2e-5 (FP32 Jacobian).
"""
import os

import numpy as np
import pytest

import oracle
from _cases import DIM, NSH, POS_CASES, ROIDS, cfg_name, configure, random_elements, random_local_u, rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, mesh

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_elements.npz")
TOL64 = 1e-12
TOL32 = 2e-5


def _elem(cuda, roid, cfg, corners, u, uo, pac=False, stab_upwind=None):
    import torch
    dim = DIM[roid]
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, cfg)
    if stab_upwind:
        d.set_stabilization_upwind(stab_upwind)
    if pac:
        d.set_pac_upwind(True)
    n = corners.shape[0]
    nloc = (dim + 1) * NSH[roid]
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    out = {k: torch.zeros((n, nloc), dtype=torch.float64, device=cuda) for k in ("defA", "defM", "rhs")}
    out.update({k: torch.zeros((n, nloc * nloc), dtype=torch.float64, device=cuda) for k in ("jacA", "jacM")})
    d.elem_batch(roid, t(corners), t(u), None if uo is None else t(uo), 0.01, **out)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(POS_CASES)))
@pytest.mark.parametrize("pac", [False, True])
def test_positive_upwind_elements_match_reference_fixtures(cuda, tname, ci, pac):
    g = np.load(GOLDEN)
    roid = ROIDS[tname]
    key = f"{tname}_pos{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    r = _elem(cuda, roid, POS_CASES[ci], g[key + "_corners"], g[key + "_u"], uo, pac=pac)
    tag = "_pac_" if pac else "_"
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + tag + k]) <= TOL64, (key, pac, k, rel_err(r[k], g[key + tag + k]))


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("conv,stab_up,stab", [("pos", "lps", "flow"), ("full", "pos", "fields"), ("lps", "pos", "flow")])
def test_mixed_upwind_objects_match_oracle(cuda, tname, conv, stab_up, stab):
    """A positive upwind on only one of the convection and the stabilisation."""
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = (conv, stab, "raw", True, 1.0, False, False, False, False)
    corners = np.concatenate([random_elements(roid, 40, 1500 + roid), random_elements(roid, 8, 1600 + roid, affine=True)])
    u = random_local_u(roid, 48, 1700 + roid, zero_frac=0.1)
    uo = random_local_u(roid, 48, 1800 + roid)
    r = _elem(cuda, roid, cfg, corners, u, uo, stab_upwind=stab_up)
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    o.set_stabilization_upwind(stab_up)
    ref = o.elem_batch(roid, corners, u, uo, 0.01)
    for k in ref:
        assert rel_err(r[k], ref[k]) <= TOL64, (tname, conv, stab_up, k, rel_err(r[k], ref[k]))


def _mesh(gen):
    return {"quads": lambda: mesh.structured_quads(14), "hexes": lambda: mesh.structured_hexes(4),
            "tris": lambda: mesh.jittered_triangles(10, seed=7)}[gen]()


@pytest.mark.parametrize("gen", ["quads", "hexes", "tris"])
@pytest.mark.parametrize("ci", range(len(POS_CASES)))
def test_positive_upwind_global_assembly_matches_oracle(cuda, gen, ci):
    """Defect and Jacobian through every assembly entry point (FP64 and FP32
    values), Dirichlet rows included; repeated calls are bitwise identical."""
    import torch
    roid, X, C = _mesh(gen)
    dim = DIM[roid]
    cfg = POS_CASES[ci]
    b = dim + 1
    U = mesh.solenoidal_state(X, seed=21) if dim == 3 else (mesh.uniform(22, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    Uo = (U * 0.9) if cfg[3] else None
    dt = 0.02 if cfg[3] else 0.0
    o = oracle.Oracle(dim); configure(o, dim, cfg); o.set_mesh(roid, X, C)
    d = NavierStokesFV1(dim=dim); configure(d, dim, cfg); d.set_mesh(roid, X, C)
    if dim == 2:
        dofs, vals = mesh.cavity_dirichlet(X, 1.0)
        o.set_dirichlet(dofs, vals); d.set_dirichlet(dofs, vals)
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo.ravel(), dtype=torch.float64, device=cuda)
    D = torch.full_like(tu, float("nan"))
    J = torch.full((o.nnzb * b * b,), float("nan"), dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D, tuo, dt)
    d.assemble_jacobian(tu, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64, (gen, cfg_name(cfg))
    assert rel_err(J.cpu().numpy(), Jref) <= TOL64, (gen, cfg_name(cfg))
    D2, J2 = torch.empty_like(D), torch.empty_like(J)
    d.assemble_defect_jacobian(tu, D2, J2, tuo, dt)
    torch.cuda.synchronize()
    assert torch.equal(D, D2) and torch.equal(J, J2)
    J32 = torch.full((o.nnzb * b * b,), float("nan"), dtype=torch.float32, device=cuda)
    d.assemble_jacobian(tu, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32
    d.assemble_defect_jacobian(tu, D2, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32 and torch.equal(D, D2)


@pytest.mark.parametrize("stab", ["fields", "flow"])
def test_positive_upwind_newton_cavity(cuda, stab):
    """Newton on a 16 x 16 cavity with the positive upwind: the GPU solution's
    defect, evaluated by the oracle, meets the requested tolerance."""
    import torch
    roid, X, C = mesh.structured_quads(16)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,p", "Inner")
    o = oracle.Oracle(2)
    for disc in (d, o):
        disc.set_kinematic_viscosity(0.02)
        disc.set_upwind("pos")
        disc.set_stabilization(stab)
        disc.set_mesh(roid, X, C)
        disc.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-4)
    assert r["status"] == 0, r
    Dn, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert np.linalg.norm(Dn) <= 1.01e-8 * r["initial_defect"], (np.linalg.norm(Dn), r)

"""GPU post-processing (incompressible/navier_stokes_tools.h): vorticityFV1 and the
point evaluation against the oracle, and the lid-driven cavity's centre-line
values against the tables the reference compares with in DrivenCavityLinesEval
(tests/golden/cavity_lines.npz, made by make_cavity_tables.py from the reference
source). The cavity check rests on published data, not on the oracle.
Tolerances: vorticity and point values <= 1e-12 relative to the oracle (the
node sums run in colour order on the GPU, mesh order in the oracle); centre
lines of a 64 x 64 cavity at Re = 100 within 0.02 of the Ghia et al. values
(the oracle's 32 x 32 solution deviates by at most 0.023 / 0.024 for u / v).
"""
import os

import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, mesh, tools

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cavity_lines.npz")


def _setup(gen):
    roid, X, C = {"quads": lambda: mesh.structured_quads(12), "tris": lambda: mesh.jittered_triangles(10, seed=3),
                  "hexes": lambda: mesh.structured_hexes(4)}[gen]()
    dim = X.shape[1]
    d = NavierStokesFV1(dim=dim)
    o = oracle.Oracle(dim)
    for disc in (d, o):
        disc.set_kinematic_viscosity(0.01)
        disc.set_upwind("full")
        disc.set_stabilization("flow")
        disc.set_mesh(roid, X, C)
    return roid, X, C, d, o


@pytest.mark.parametrize("gen", ["quads", "tris", "hexes"])
def test_vorticity_matches_oracle(cuda, gen):
    import torch
    roid, X, C, d, o = _setup(gen)
    b = X.shape[1] + 1
    U = (mesh.uniform(41, X.shape[0] * b) * 2 - 1).reshape(-1, b)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    v = tools.vorticity(d, tu)
    v2 = tools.vorticity(d, tu)
    torch.cuda.synchronize()
    ref = o.vorticity(U)
    assert rel_err(v.cpu().numpy(), ref) <= 1e-12
    assert torch.equal(v, v2)
    # solid-body rotation (u, v) = (-y, x): curl 2 everywhere
    U[:, 0], U[:, 1] = -X[:, 1], X[:, 0]
    w = tools.vorticity(d, torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)).cpu().numpy()
    assert np.abs(w - 2.0).max() <= 1e-12


@pytest.mark.parametrize("gen", ["quads", "tris", "hexes"])
def test_point_evaluation_matches_oracle(cuda, gen):
    import torch
    roid, X, C, d, o = _setup(gen)
    dim = X.shape[1]
    b = dim + 1
    U = (mesh.uniform(43, X.shape[0] * b) * 2 - 1).reshape(-1, b)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    pts = mesh.uniform(44, 40 * dim).reshape(40, dim) * 1.1 - 0.05   # a few fall outside the unit box
    pts[:4] = X[[0, 3, 7, X.shape[0] - 1]]                             # mesh nodes
    for fct in range(b):
        got = tools.eval_at_points(d, tu, pts, fct)
        ref = o.eval_points(U, pts, fct)
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        ok = ~np.isnan(ref)
        assert ok.sum() >= 30 and rel_err(got[ok], ref[ok]) <= 1e-12
    assert np.allclose(tools.eval_at_points(d, tu, pts[:4], 0), U[[0, 3, 7, X.shape[0] - 1], 0], rtol=0, atol=1e-14)


def test_cavity_centre_lines_against_published_tables(cuda):
    """64 x 64 cavity at Re = 100 (lid speed 1, nu = 0.01), full upwind + FLOW, Newton on the
    GPU: centre-line velocities against the Ghia et al. values of the reference's tables."""
    import torch
    g = np.load(GOLDEN)
    roid, X, C = mesh.structured_quads(64)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(0.01)
    d.set_upwind("full")
    d.set_stabilization("flow")
    d.set_mesh(roid, X, C)
    d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, lin_max_iter=20000)
    assert r["status"] == 0
    res = tools.driven_cavity_lines_eval(d, u, g["vertGhiaPosY"], g["vertGhia_100"], g["horizGhiaPosX"], g["horizGhia100"])
    assert res["vertical"]["max_diff"] <= 0.02, res["vertical"]
    assert res["horizontal"]["max_diff"] <= 0.02, res["horizontal"]
    # the same lines through the oracle's point evaluation of the GPU solution
    o = oracle.Oracle(2)
    o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("flow"); o.set_mesh(roid, X, C)
    U = u.cpu().numpy()
    assert rel_err(res["vertical"]["measured"], o.eval_points(U, res["vertical"]["points"], 0)) <= 1e-12

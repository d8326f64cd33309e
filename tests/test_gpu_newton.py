"""GPU Newton (plain FP64 method and FP32-Jacobian mode) against the oracle."""
import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, mesh

pytestmark = pytest.mark.gpu


def _cavity(n, upwind="full", stab="fields", nu=0.01):
    roid, X, C = mesh.structured_quads(n)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    return roid, X, C, dofs, vals


@pytest.mark.parametrize("solver", ["bicgstab", "gmres"])
def test_newton_cavity_32_converges_and_matches_oracle(cuda, solver):
    import torch
    roid, X, C, dofs, vals = _cavity(32)
    o = oracle.Oracle(2); o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("fields")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    Uref, st = o.newton(np.zeros(X.shape[0] * 3), rtol=1e-10, lin_rtol=1e-3)
    assert st["status"] == 0
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(0.01); d.set_upwind("full"); d.set_stabilization("fields")
    d.set_mesh(roid, X, C); d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-10, lin_rtol=1e-3, linear_solver=solver, max_iter=60)
    assert r["status"] == 0 and r["final_defect"] <= 1e-10 * r["initial_defect"]
    assert abs(r["initial_defect"] - st["initial_defect"]) <= 1e-12 * st["initial_defect"]
    # both solve the same discrete problem to 1e-10: solutions agree far below the discretisation error
    assert rel_err(u.cpu().numpy(), Uref) < 1e-7
    # FP64 defect of the GPU solution, recomputed by the oracle
    D, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert np.linalg.norm(D) <= 2e-10 * st["initial_defect"]


def test_newton_fp32_jacobian_reaches_fp64_defect(cuda):
    import torch
    roid, X, C, dofs, vals = _cavity(32)
    d = NavierStokesFV1(dim=2)
    d.set_kinematic_viscosity(0.01); d.set_upwind("full"); d.set_stabilization("fields")
    d.set_mesh(roid, X, C); d.set_dirichlet(dofs, vals)
    u64 = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r64 = d.newton_solve(u64, rtol=1e-8, lin_rtol=1e-3)
    u32 = torch.zeros_like(u64)
    r32 = d.newton_solve(u32, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32")
    assert r32["status"] == 0 and r32["final_defect"] <= 1e-8 * r32["initial_defect"]
    o = oracle.Oracle(2); o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("fields")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    D, _ = o.assemble(u32.cpu().numpy(), jacobian=False)
    # the FP64 oracle defect of the FP32-Jacobian solution meets the same 1e-8 target
    assert np.linalg.norm(D) <= 1.01e-8 * r32["initial_defect"]
    assert rel_err(u32.cpu().numpy(), u64.cpu().numpy()) < 1e-5


def test_newton_3d_lps_flow_small(cuda):
    import torch
    roid, X, C = mesh.structured_hexes(6)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,w,p", "Inner")
    d.set_kinematic_viscosity(0.05); d.set_upwind("lps"); d.set_stabilization("flow")
    d.set_mesh(roid, X, C); d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 4, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, linear_solver="gmres", gmres_restart=40)
    assert r["status"] == 0
    o = oracle.Oracle(3); o.set_kinematic_viscosity(0.05); o.set_upwind("lps"); o.set_stabilization("flow")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    D, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert np.linalg.norm(D) <= 1.01e-8 * r["initial_defect"]


def test_newton_3d_fp32_jacobian_bicgstab(cuda):
    """The 3D FP32-Jacobian Newton with BiCGStab (4x4 blocks: the lane-per-corner
    FP32 Jacobian, the double-float block-Jacobi apply and the split-operand SpMV)
    reaches the FP64 oracle's 1e-8 defect reduction."""
    import torch
    roid, X, C = mesh.structured_hexes(6)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,w,p", "Inner")
    d.set_kinematic_viscosity(0.05); d.set_upwind("lps"); d.set_stabilization("flow")
    d.set_mesh(roid, X, C); d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 4, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, lin_max_iter=5000, jacobian_prec="f32")
    assert r["status"] == 0, r
    o = oracle.Oracle(3); o.set_kinematic_viscosity(0.05); o.set_upwind("lps"); o.set_stabilization("flow")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    D, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert np.linalg.norm(D) <= 1.01e-8 * r["initial_defect"]


def test_newton_reports_nonfinite(cuda):
    import torch
    roid, X, C, dofs, vals = _cavity(8)
    d = NavierStokesFV1(dim=2)
    d.set_kinematic_viscosity(0.01); d.set_upwind("full"); d.set_stabilization("fields")
    d.set_mesh(roid, X, C)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    u[7] = float("nan")
    r = d.newton_solve(u, raise_on_error=False)
    assert r["status"] == 6
    # the handle is still usable afterwards
    u.zero_()
    d.set_dirichlet(dofs, vals)
    r = d.newton_solve(u, rtol=1e-6, lin_rtol=1e-3)
    assert r["status"] == 0


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_transient_newton_on_jittered_triangles(cuda, prec):
    """Backward Euler on jittered triangles (the transient workload's construction
    at 32^2): every step reaches its Newton target, and the FP64 oracle defect of
    the end state of each step (with the previous state as u_old) meets it."""
    import torch
    roid, X, C = mesh.jittered_triangles(32, seed=2)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(0.001); d.set_upwind("full"); d.set_stabilization("fields")
    d.set_mesh(roid, X, C); d.set_dirichlet(dofs, vals)
    o = oracle.Oracle(2); o.set_kinematic_viscosity(0.001); o.set_upwind("full"); o.set_stabilization("fields")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    for _ in range(3):
        uo = u.clone()
        r = d.newton_solve(u, uo, dt=0.01, rtol=1e-6, lin_rtol=1e-4, lin_max_iter=5000, jacobian_prec=prec)
        assert r["status"] == 0, r
        D, _ = o.assemble(u.cpu().numpy(), uo.cpu().numpy(), 0.01, jacobian=False)
        assert np.linalg.norm(D) <= 1.01e-6 * r["initial_defect"], (np.linalg.norm(D), r)

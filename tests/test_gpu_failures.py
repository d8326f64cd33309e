"""Failure detection through status codes, with the failure planted on the host.

A zero diagonal block written into a Jacobian by the test (block-Jacobi entry
point), and a disc configured so that its own Jacobian has exactly singular
diagonal blocks (zero viscosity, Stokes, no stabilisation: the velocity rows of
every diagonal block are zero apart from the pressure column) must give
NSFV1_ERR_BREAKDOWN from the block-Jacobi preconditioner, the Newton solve and
the batched solve. The handle stays usable: the next call with valid data
succeeds. Nothing here faults or hangs the GPU.
"""
import numpy as np
import pytest

import oracle
from _cases import DISC_CASES, configure, rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, NSFV1Error, _capi, mesh

pytestmark = pytest.mark.gpu


def _quads_disc(n=12):
    roid, X, C = mesh.structured_quads(n)
    d = NavierStokesFV1("u,v,p")
    configure(d, 2, DISC_CASES[0])
    d.set_mesh(roid, X, C)
    return d, roid, X, C


@pytest.mark.parametrize("jdtype", ["f64", "f32"])
def test_block_jacobi_reports_a_planted_singular_block(cuda, jdtype):
    import torch
    d, roid, X, C = _quads_disc()
    nnzb = d.pattern_info()["nnz_blocks"]
    U = (mesh.uniform(21, X.shape[0] * 3) * 2 - 1)
    tu = torch.tensor(U, dtype=torch.float64, device=cuda)
    J = torch.empty(nnzb * 9, dtype=torch.float64 if jdtype == "f64" else torch.float32, device=cuda)
    d.assemble_jacobian(tu, J)
    r = torch.tensor(mesh.uniform(22, tu.numel()) - 0.5, dtype=torch.float64, device=cuda)
    z_ok = torch.empty_like(r)
    d.block_jacobi(J, r, z_ok)
    # zero the diagonal block of node 17
    rp, ci = d.pattern()
    q = int(rp[17] + np.nonzero(ci[rp[17]:rp[18]] == 17)[0][0])
    Jbad = J.clone()
    Jbad[q * 9:(q + 1) * 9] = 0
    z = torch.empty_like(r)
    with pytest.raises(NSFV1Error) as ex:
        d.block_jacobi(Jbad, r, z)
    assert ex.value.status == _capi.ERR_BREAKDOWN and "singular" in d.last_error()
    # the handle is still usable and gives the same result as before
    z2 = torch.empty_like(r)
    d.block_jacobi(J, r, z2)
    torch.cuda.synchronize()
    assert torch.equal(z2, z_ok)


def _singular_config(d):
    d.set_kinematic_viscosity(0.0)
    d.set_stokes(True)
    d.set_stabilization("without")
    d.set_upwind("full")


@pytest.mark.parametrize("jprec", ["f64", "f32"])
def test_newton_reports_singular_diagonal_blocks(cuda, jprec):
    import torch
    roid, X, C = mesh.structured_quads(8)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d = NavierStokesFV1("u,v,p")
    _singular_config(d)
    d.set_mesh(roid, X, C)
    d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, jacobian_prec=jprec, raise_on_error=False)
    assert r["status"] == _capi.ERR_BREAKDOWN, r
    assert "singular" in d.last_error()
    # the same handle, reconfigured, solves and meets the oracle defect target
    d.set_kinematic_viscosity(0.01)
    d.set_stokes(False)
    d.set_stabilization("flow")
    d.set_upwind("full")
    u.zero_()
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec=jprec)
    o = oracle.Oracle(2)
    o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("flow")
    o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
    D, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert r["status"] == 0 and np.linalg.norm(D) <= 1.01e-8 * r["initial_defect"]


def test_batched_newton_reports_singular_diagonal_blocks(cuda):
    import torch
    sizes, Re, lid = [8, 12], [100.0, 200.0], [1.0, 1.0]
    B = mesh.cavity_batch(sizes, Re, lid)
    d = NavierStokesFV1("u,v,p")
    _singular_config(d)
    d.set_mesh(B["elem_type"], B["coords"], B["conn"])
    d.set_instances(B["node_offsets"])
    d.set_dirichlet(B["dofs"], B["values"])
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    res = d.newton_solve_batched(u, rtol=1e-8, lin_max_iter=60, jacobian_prec="f32", raise_on_error=False)
    assert all(r["status"] == _capi.ERR_BREAKDOWN for r in res), res
    # usable afterwards with a regular configuration
    d.set_kinematic_viscosity(1.0)
    d.set_elem_viscosity(B["nu_elem"])
    d.set_stokes(False)
    d.set_stabilization("flow")
    d.set_upwind("full")
    u.zero_()
    res = d.newton_solve_batched(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32")
    assert all(r["status"] == 0 for r in res), res


def test_nonfinite_state_is_reported_and_the_handle_recovers(cuda):
    import torch
    d, roid, X, C = _quads_disc(8)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    d.set_dirichlet(dofs, vals)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    u[3 * 40] = float("inf")
    r = d.newton_solve(u, rtol=1e-8, raise_on_error=False)
    assert r["status"] == _capi.ERR_NONFINITE, r
    u.zero_()
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, raise_on_error=False)
    assert r["status"] == 0, r


@pytest.mark.parametrize("jdtype", ["f64", "f32"])
def test_bicgstab_breakdown_restarts_and_is_reported(cuda, jdtype):
    """A planted system on which BiCGStab breaks down at every start: identity
    diagonal blocks, the block (node 0, node 1) = -2 I, rhs = 1 on nodes 0 and 1.
    With r0 = rhs, v = J r0 is -1 on node 0 and +1 on node 1, so (r0, v) = 0:
    alpha breaks down, omega = (t, s) / (t, t) = 0, the residual does not move
    and every restart (shadow vector := residual) meets the same zero. The solve
    stops after 20 restarts with NSFV1_ERR_NOT_CONVERGED and x = 0; the handle
    then solves a well-posed system with the same pattern."""
    import torch
    d, roid, X, C = _quads_disc(2)
    rp, ci = d.pattern()
    b = 3
    dt_ = torch.float64 if jdtype == "f64" else torch.float32
    V = np.zeros((ci.size, b, b))
    for r in range(X.shape[0]):
        for q in range(rp[r], rp[r + 1]):
            if ci[q] == r:
                V[q] = np.eye(b)
    q01 = [q for q in range(rp[0], rp[1]) if ci[q] == 1]
    assert len(q01) == 1
    V[q01[0]] = -2.0 * np.eye(b)
    vals = torch.tensor(V.ravel(), dtype=dt_, device=cuda)
    rhs = torch.zeros(X.shape[0] * b, dtype=torch.float64, device=cuda)
    rhs[0:2 * b] = 1.0
    x = torch.full_like(rhs, float("nan"))
    res = d.linear_solve(vals, rhs, x, lin_rtol=1e-8, lin_max_iter=200, raise_on_error=False)
    assert res["status"] == _capi.ERR_NOT_CONVERGED, res
    assert res["restarts"] == 21 and res["iterations"] == 21, res
    assert res["relres"] == 1.0
    assert torch.count_nonzero(x).item() == 0
    # a well-posed system on the same handle: diagonal blocks only, one iteration
    V2 = np.zeros_like(V)
    for r in range(X.shape[0]):
        for q in range(rp[r], rp[r + 1]):
            if ci[q] == r:
                V2[q] = 2.0 * np.eye(b)
    vals2 = torch.tensor(V2.ravel(), dtype=dt_, device=cuda)
    rhs2 = torch.tensor(mesh.uniform(3, X.shape[0] * b) + 0.5, dtype=torch.float64, device=cuda)
    for solver in ("bicgstab", "gmres"):
        x2 = torch.empty_like(rhs2)
        res2 = d.linear_solve(vals2, rhs2, x2, lin_rtol=1e-10, linear_solver=solver)
        assert res2["status"] == 0 and res2["restarts"] == 0 and res2["iterations"] == 1, (solver, res2)
        assert torch.allclose(x2, rhs2 / 2.0, rtol=1e-14, atol=0.0)

"""Boundary-condition element discs: NavierStokesWall (zero-velocity Dirichlet
rows, incompressible/bnd/wall_impl.h:57-69), NavierStokesInflowFV1
(Dirichlet inflow velocity + the continuity equation's Neumann flux vel . n over
each boundary corner's dual face, incompressible/fv1/bnd/inflow_fv1_impl.h:57-82)
and NavierStokesNoNormalStressOutflowFV1 (tangential viscous, outgoing convective
and continuity fluxes over the outflow faces, incompressible/fv1/bnd/
no_normal_stress_outflow_fv1.cpp:343-504).

CPU: the oracle's inflow flux integrates to vel . n over the inflow boundary,
in 2D and 3D, and interior sides are refused. GPU: defect and Jacobian of a
channel (walls, inflow, natural outflow) match the oracle to 1e-12, stationary
and implicit Euler, and a Newton solve of the channel meets the oracle defect.
"""
import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import (NavierStokesFV1, NavierStokesInflowFV1, NavierStokesNoNormalStressOutflowFV1, NavierStokesWall,
                                      NSFV1Error, mesh)


def _channel(dim, n):
    if dim == 2:
        roid, X, C = mesh.structured_quads(n)
        X = X * np.array([2.0, 1.0])
    else:
        roid, X, C = mesh.structured_hexes(n)
        X = X * np.array([2.0, 1.0, 1.0])
    inflow = mesh.boundary_sides(roid, X, C, 0, 0.0)
    walls = np.unique(np.concatenate([mesh.boundary_nodes(X, a, v) for a in range(1, dim) for v in (0.0, 1.0)]))
    return roid, X, C, inflow, walls


def _setup(disc, dim, roid, X, C, inflow, walls, vel):
    disc.set_kinematic_viscosity(0.02)
    disc.set_upwind("lps" if dim == 3 else "full")
    disc.set_stabilization("flow" if dim == 3 else "fields")
    disc.set_mesh(roid, X, C)
    if isinstance(disc, oracle.Oracle):
        disc.add_wall(walls)
        disc.add_inflow(vel, inflow)
    else:
        NavierStokesWall(disc).add(walls)
        NavierStokesInflowFV1(disc).add(vel, inflow)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_inflow_flux_integrates_to_the_inflow(dim):
    roid, X, C, inflow, walls = _channel(dim, 6)
    o = oracle.Oracle(dim)
    vel = [1.5] + [0.0] * (dim - 1)
    _setup(o, dim, roid, X, C, inflow, walls, vel)
    U = np.zeros(X.shape[0] * (dim + 1))
    D, _ = o.assemble(U, jacobian=False)
    D = D.reshape(-1, dim + 1)
    # at rest only the inflow flux drives the continuity rows; its sum is vel . n over x = 0 (area 1)
    in_nodes = np.unique(inflow)
    assert abs(D[:, dim].sum() - (-1.5)) < 1e-13
    assert np.all(D[np.setdiff1d(np.arange(X.shape[0]), in_nodes), dim] == 0.0)
    # Dirichlet velocity rows: u - g on the inflow (the wall corners are later inflow rows: inflow wins)
    assert np.allclose(D[in_nodes, 0], -1.5)


def test_oracle_refuses_interior_sides():
    roid, X, C, inflow, walls = _channel(2, 4)
    o = oracle.Oracle(2)
    o.set_kinematic_viscosity(0.01); o.set_upwind("full"); o.set_stabilization("fields"); o.set_mesh(roid, X, C)
    interior = np.array([[C[0, 1], C[0, 2]]])   # the side shared by elements 0 and 1
    with pytest.raises(RuntimeError):
        o.add_inflow([1.0, 0.0], interior)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("transient", [False, True])
def test_channel_defect_and_jacobian_match_the_oracle(cuda, dim, transient):
    import torch
    roid, X, C, inflow, walls = _channel(dim, 8 if dim == 2 else 5)
    vel = [1.0, 0.25, -0.1][:dim]
    b = dim + 1
    d = NavierStokesFV1(dim=dim)
    o = oracle.Oracle(dim)
    for disc in (d, o):
        _setup(disc, dim, roid, X, C, inflow, walls, vel)
    U = (mesh.uniform(17, X.shape[0] * b) * 2 - 1)
    Uo = U * 0.7 if transient else None
    dt = 0.05 if transient else 0.0
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U, dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo, dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(Jref.size, dtype=torch.float64, device=cuda)
    d.assemble_defect_jacobian(tu, D, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= 1e-12
    assert rel_err(J.cpu().numpy(), Jref) <= 1e-12
    d.assemble_defect(tu, D, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= 1e-12


@pytest.mark.gpu
def test_channel_newton_meets_the_oracle_defect(cuda):
    """A 2 x 1 channel with walls, a plug inflow at x = 0 and the same plug profile
    prescribed at x = 2 through a second inflow disc (its continuity flux is the
    outflow: without an outflow disc the boundary control volumes would let no mass
    out), pressure pinned at one node: the GPU Newton meets the oracle defect."""
    import torch
    roid, X, C, inflow, walls = _channel(2, 16)
    outflow = mesh.boundary_sides(roid, X, C, 0, 2.0)
    d = NavierStokesFV1(dim=2)
    o = oracle.Oracle(2)
    for disc in (d, o):
        _setup(disc, 2, roid, X, C, inflow, walls, [1.0, 0.0])
        disc.add_dirichlet([2], [0.0])   # p at node 0
    NavierStokesInflowFV1(d).add([1.0, 0.0], outflow)
    o.add_inflow([1.0, 0.0], outflow)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-4, lin_max_iter=5000)
    Dn, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert r["status"] == 0 and np.linalg.norm(Dn) <= 1.01e-8 * r["initial_defect"], r


@pytest.mark.gpu
def test_inflow_rejects_interior_sides_and_bad_sizes(cuda):
    roid, X, C, inflow, walls = _channel(2, 4)
    d = NavierStokesFV1(dim=2)
    d.set_kinematic_viscosity(0.01); d.set_upwind("full"); d.set_stabilization("fields"); d.set_mesh(roid, X, C)
    with pytest.raises(NSFV1Error):
        NavierStokesInflowFV1(d).add([1.0, 0.0], np.array([[C[0, 1], C[0, 2]]]))
    with pytest.raises(NSFV1Error):
        NavierStokesInflowFV1(d).add([1.0, 0.0, 0.0], inflow)
    with pytest.raises(NSFV1Error):
        NavierStokesWall(d).add([X.shape[0] + 3])


def _dense(o, V, n_nodes, b):
    rp, ci = o.pattern()
    A = np.zeros((n_nodes * b, n_nodes * b))
    for r in range(n_nodes):
        for q in range(rp[r], rp[r + 1]):
            A[r * b:(r + 1) * b, ci[q] * b:(ci[q] + 1) * b] = V[q * b * b:(q + 1) * b * b].reshape(b, b)
    return A


@pytest.mark.parametrize("gen", ["quads", "tris", "hexes"])
def test_oracle_outflow_jacobian_is_the_derivative_of_its_defect(gen):
    """Without convection (Stokes) the outflow faces' Jacobian is exact: it equals the
    central difference of their defect."""
    roid, X, C = {"quads": lambda: mesh.structured_quads(3), "tris": lambda: mesh.jittered_triangles(3, seed=3),
                  "hexes": lambda: mesh.structured_hexes(2)}[gen]()
    dim = X.shape[1]
    b = dim + 1
    sides = mesh.boundary_sides(roid, X, C, 0, 1.0)

    def make(outflow):
        o = oracle.Oracle(dim)
        o.set_kinematic_viscosity(0.1); o.set_upwind("full"); o.set_stabilization("flow"); o.set_stokes(True)
        o.set_mesh(roid, X, C)
        if outflow:
            o.add_outflow(sides)
        return o

    with_, without = make(True), make(False)
    U = mesh.uniform(5, X.shape[0] * b) * 2 - 1
    Jb = _dense(with_, with_.assemble(U)[1], X.shape[0], b) - _dense(without, without.assemble(U)[1], X.shape[0], b)
    assert np.abs(Jb).max() > 0.05
    h = 1e-6
    fd = np.zeros_like(Jb)
    for k in range(U.size):
        e = np.zeros(U.size)
        e[k] = h
        bnd = lambda V: with_.assemble(V, jacobian=False)[0] - without.assemble(V, jacobian=False)[0]
        fd[:, k] = (bnd(U + e) - bnd(U - e)) / (2 * h)
    assert np.abs(fd - Jb).max() <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("transient", [False, True])
def test_outflow_channel_matches_the_oracle(cuda, dim, transient):
    """Walls, inflow and a no-normal-stress outflow at x = 2: defect and FP64 / FP32
    Jacobians through every assembly entry point."""
    import torch
    roid, X, C, inflow, walls = _channel(dim, 8 if dim == 2 else 4)
    outflow = mesh.boundary_sides(roid, X, C, 0, 2.0)
    vel = [1.0, 0.25, -0.1][:dim]
    b = dim + 1
    d = NavierStokesFV1(dim=dim)
    o = oracle.Oracle(dim)
    for disc in (d, o):
        _setup(disc, dim, roid, X, C, inflow, walls, vel)
    NavierStokesNoNormalStressOutflowFV1(d).add(outflow)
    o.add_outflow(outflow)
    U = (mesh.uniform(19, X.shape[0] * b) * 2 - 1)
    Uo = U * 0.7 if transient else None
    dt = 0.05 if transient else 0.0
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U, dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo, dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(Jref.size, dtype=torch.float64, device=cuda)
    d.assemble_defect_jacobian(tu, D, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= 1e-12 and rel_err(J.cpu().numpy(), Jref) <= 1e-12
    D2, J2 = torch.empty_like(D), torch.empty_like(J)
    d.assemble_defect(tu, D2, tuo, dt)
    d.assemble_jacobian(tu, J2, tuo, dt)
    torch.cuda.synchronize()
    assert torch.equal(D, D2) and rel_err(J2.cpu().numpy(), Jref) <= 1e-12
    J32 = torch.empty(Jref.size, dtype=torch.float32, device=cuda)
    d.assemble_jacobian(tu, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= 2e-5


@pytest.mark.gpu
def test_outflow_channel_newton_meets_the_oracle_defect(cuda):
    """A 2 x 1 channel with walls, a plug inflow and a no-normal-stress outflow (no
    pressure pin: the outflow fixes the pressure level): the GPU Newton meets the
    oracle defect, and the outflow profile is close to Poiseuille's (peak 1.5)."""
    import torch
    roid, X, C, inflow, walls = _channel(2, 16)
    outflow = mesh.boundary_sides(roid, X, C, 0, 2.0)
    d = NavierStokesFV1(dim=2)
    o = oracle.Oracle(2)
    for disc in (d, o):
        _setup(disc, 2, roid, X, C, inflow, walls, [1.0, 0.0])
    NavierStokesNoNormalStressOutflowFV1(d).add(outflow)
    o.add_outflow(outflow)
    u = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve(u, rtol=1e-8, lin_rtol=1e-4, lin_max_iter=5000)
    U = u.cpu().numpy()
    Dn, _ = o.assemble(U, jacobian=False)
    assert r["status"] == 0 and np.linalg.norm(Dn) <= 1.01e-8 * r["initial_defect"], r
    peak = U.reshape(-1, 3)[np.unique(outflow), 0].max()
    assert 1.35 < peak < 1.55

"""Batched Newton over independent cavity instances (one persistent GMRES
launch per Newton step) against per-instance oracle solves."""
import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, mesh

pytestmark = pytest.mark.gpu


def _batch(sizes, Re, lid, upwind="full", stab="flow"):
    B = mesh.cavity_batch(sizes, Re, lid)
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(1.0)   # replaced per element
    d.set_upwind(upwind); d.set_stabilization(stab)
    d.set_mesh(B["elem_type"], B["coords"], B["conn"])
    d.set_elem_viscosity(B["nu_elem"])
    d.set_instances(B["node_offsets"])
    d.set_dirichlet(B["dofs"], B["values"])
    return d, B


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("cluster", [1, 4])
def test_batched_newton_matches_oracle_per_instance(cuda, prec, cluster):
    import torch
    sizes = [8, 12, 16, 10, 20]
    Re = [50.0, 400.0, 100.0, 10.0, 800.0]
    lid = [1.0, 2.0, 0.5, 1.5, 1.0]
    d, B = _batch(sizes, Re, lid)
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    res = d.newton_solve_batched(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec=prec, cluster_size=cluster)
    U = u.cpu().numpy()
    offs = B["node_offsets"]
    for i, (N, re, u0) in enumerate(zip(sizes, Re, lid)):
        assert res[i]["status"] == 0, (i, res[i])
        roid, X, C = mesh.structured_quads(N)
        dofs, vals = mesh.cavity_dirichlet(X, u0)
        o = oracle.Oracle(2); o.set_kinematic_viscosity(u0 / re); o.set_upwind("full"); o.set_stabilization("flow")
        o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
        Ui = U[offs[i] * 3:offs[i + 1] * 3]
        D, _ = o.assemble(Ui, jacobian=False)
        # the per-instance FP64 oracle defect meets the target
        assert abs(res[i]["initial_defect"] - np.linalg.norm(o.assemble(_dir(Ui.size, dofs, vals), jacobian=False)[0])) <= 1e-10 * res[i]["initial_defect"]
        assert np.linalg.norm(D) <= 1.01e-8 * res[i]["initial_defect"], (i, np.linalg.norm(D), res[i])
        Uref, st = o.newton(np.zeros(Ui.size), rtol=1e-10, lin_rtol=1e-6, lin_maxit=20000)
        assert rel_err(Ui, Uref) < 1e-5


def _dir(n, dofs, vals):
    x = np.zeros(n)
    x[dofs] = vals
    return x


def test_batched_solution_is_deterministic(cuda):
    import torch
    d, B = _batch([8, 16, 12], [100.0, 300.0, 30.0], [1.0, 1.0, 2.0])
    u1 = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    u2 = torch.zeros_like(u1)
    r1 = d.newton_solve_batched(u1, rtol=1e-8, jacobian_prec="f32")
    r2 = d.newton_solve_batched(u2, rtol=1e-8, jacobian_prec="f32")
    assert torch.equal(u1, u2)
    assert [r["linear_iterations"] for r in r1] == [r["linear_iterations"] for r in r2]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_multigrid_batched_newton(cuda, prec):
    """Structured instances with the geometric multigrid preconditioner: every
    instance converges, meets the FP64 oracle defect target, and needs far fewer
    linear iterations than point-block Jacobi alone."""
    import torch
    sizes = [16, 32, 24, 48]
    Re = [100.0, 1000.0, 300.0, 800.0]
    lid = [1.0, 2.0, 0.5, 1.5]
    d, B = _batch(sizes, Re, lid)
    d.set_instance_grids(sizes)
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    res = d.newton_solve_batched(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec=prec, multigrid=True, max_iter=80)
    U = u.cpu().numpy()
    offs = B["node_offsets"]
    for i, (N, re, u0) in enumerate(zip(sizes, Re, lid)):
        assert res[i]["status"] == 0, (i, res[i])
        roid, X, C = mesh.structured_quads(N)
        dofs, vals = mesh.cavity_dirichlet(X, u0)
        o = oracle.Oracle(2); o.set_kinematic_viscosity(u0 / re); o.set_upwind("full"); o.set_stabilization("flow")
        o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
        D, _ = o.assemble(U[offs[i] * 3:offs[i + 1] * 3], jacobian=False)
        assert np.linalg.norm(D) <= 1.01e-8 * res[i]["initial_defect"], (i, res[i])
    # the V-cycle cuts the Krylov work by a large factor on the 48 x 48, Re 800 instance
    per_step_mg = res[3]["linear_iterations"] / max(res[3]["iterations"], 1)
    assert per_step_mg < 150, res[3]


def test_graph_replay_matches_direct_launches(cuda):
    """The captured per-step CUDA graph gives bit-identical iterates and counts."""
    import torch
    sizes = [16, 24, 32]
    d, B = _batch(sizes, [100.0, 500.0, 1000.0], [1.0, 0.7, 1.8])
    d.set_instance_grids(sizes)
    out = []
    for graph in (False, True):
        u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
        r = d.newton_solve_batched(u, rtol=1e-8, jacobian_prec="f32", graph=graph, max_iter=80)
        out.append((u, r))
    assert torch.equal(out[0][0], out[1][0])
    assert [x["linear_iterations"] for x in out[0][1]] == [x["linear_iterations"] for x in out[1][1]]


def test_adaptive_forcing_meets_the_oracle_target(cuda):
    """Eisenstat-Walker tolerances: every instance still reaches the FP64 oracle
    defect target, with fewer Krylov iterations than the fixed 1e-3 tolerance."""
    import torch
    sizes = [16, 32, 24]
    Re, lid = [200.0, 1000.0, 50.0], [1.0, 1.5, 2.0]
    d, B = _batch(sizes, Re, lid)
    d.set_instance_grids(sizes)
    lin = []
    for fmax in (0.0, 0.3):
        u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
        res = d.newton_solve_batched(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32", forcing_max=fmax, max_iter=100)
        U = u.cpu().numpy()
        offs = B["node_offsets"]
        for i, (N, re, u0) in enumerate(zip(sizes, Re, lid)):
            assert res[i]["status"] == 0, (fmax, i, res[i])
            roid, X, C = mesh.structured_quads(N)
            dofs, vals = mesh.cavity_dirichlet(X, u0)
            o = oracle.Oracle(2); o.set_kinematic_viscosity(u0 / re); o.set_upwind("full"); o.set_stabilization("flow")
            o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
            D, _ = o.assemble(U[offs[i] * 3:offs[i + 1] * 3], jacobian=False)
            assert np.linalg.norm(D) <= 1.01e-8 * res[i]["initial_defect"], (fmax, i, res[i])
        lin.append(sum(r["linear_iterations"] for r in res))
    assert lin[1] < lin[0], lin


def test_zero_reference_and_fallback(cuda):
    """defect_reference "zero": the target is relative to the zero iterate's
    defect; with zero_fallback a worse iterate restarts from zero, a better one
    is kept."""
    import torch
    sizes = [16, 16]
    Re, lid = [100.0, 100.0], [1.0, 1.0]
    d, B = _batch(sizes, Re, lid)
    n = B["coords"].shape[0] * 3
    u_ref = torch.zeros(n, dtype=torch.float64, device=cuda)
    r0 = d.newton_solve_batched(u_ref, rtol=1e-10, jacobian_prec="f64")
    zero_defect = r0[0]["initial_defect"]
    # instance 0: a slightly perturbed solution (better than zero), instance 1: garbage (worse)
    half = n // 2
    u = u_ref.clone()
    u[:half] += 1e-4 * torch.sin(torch.arange(half, dtype=torch.float64, device=cuda))
    u[half:] = 50.0
    res = d.newton_solve_batched(u, rtol=1e-8, jacobian_prec="f64", defect_reference="zero", zero_fallback=True)
    assert res[0]["initial_defect"] < 1e-2 * zero_defect
    assert abs(res[1]["initial_defect"] - r0[1]["initial_defect"]) <= 1e-12 * r0[1]["initial_defect"]
    for r in res:
        assert r["status"] == 0 and r["final_defect"] <= 1.0e-8 * zero_defect * 1.0000001
    assert res[0]["iterations"] < res[1]["iterations"]


def test_autotune_picks_a_candidate(cuda):
    import torch
    sizes = [16, 32, 24, 48]
    d, B = _batch(sizes, [100.0, 1000.0, 300.0, 800.0], [1.0, 2.0, 0.5, 1.5])
    d.set_instance_grids(sizes)
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    best, ms = d.batch_autotune(u, candidates=(2, 4, 8))
    assert best in (2, 4, 8) and len(ms) == 3 and all(t > 0 for t in ms)
    assert ms[(2, 4, 8).index(best)] == min(ms)
    assert torch.count_nonzero(u) == 0   # the iterate is untouched


def test_exact_jacobian_with_forcing_meets_the_oracle_target(cuda):
    """The fast path of the batched workload (exact-Jacobian factor 1, adaptive
    linear tolerances up to 0.3, FP32 Jacobian): every instance reaches the FP64
    oracle defect target of the plain discretisation."""
    import torch
    sizes = [16, 32, 24, 40]
    Re, lid = [200.0, 1000.0, 50.0, 700.0], [1.0, 1.5, 2.0, 0.6]
    B = mesh.cavity_batch(sizes, Re, lid)
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(1.0); d.set_upwind("full"); d.set_stabilization("flow"); d.set_exact_jacobian(1.0)
    d.set_mesh(B["elem_type"], B["coords"], B["conn"]); d.set_elem_viscosity(B["nu_elem"])
    d.set_instances(B["node_offsets"]); d.set_dirichlet(B["dofs"], B["values"]); d.set_instance_grids(sizes)
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    res = d.newton_solve_batched(u, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32", forcing_max=0.3, max_iter=80,
                                 defect_reference="zero", smooth_steps=3, coarse_steps=40)
    U = u.cpu().numpy()
    offs = B["node_offsets"]
    for i, (N, re, u0) in enumerate(zip(sizes, Re, lid)):
        assert res[i]["status"] == 0, (i, res[i])
        roid, X, C = mesh.structured_quads(N)
        dofs, vals = mesh.cavity_dirichlet(X, u0)
        o = oracle.Oracle(2); o.set_kinematic_viscosity(u0 / re); o.set_upwind("full"); o.set_stabilization("flow")
        o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
        D, _ = o.assemble(U[offs[i] * 3:offs[i + 1] * 3], jacobian=False)
        D0, _ = o.assemble(_dir(U[offs[i] * 3:offs[i + 1] * 3].size, dofs, vals), jacobian=False)
        assert np.linalg.norm(D) <= 1.01e-8 * np.linalg.norm(D0), (i, res[i])


def test_repartition_one_mesh_into_more_instances(cuda):
    """The same mesh of four cavities solved first as two instances (two cavities
    each), then as four: the batched solver's per-instance buffers follow the new
    partition, and every cavity meets its FP64 oracle defect target."""
    import torch
    sizes = [8, 8, 12, 12]
    Re = [100.0, 300.0, 50.0, 200.0]
    lid = [1.0, 1.5, 0.5, 2.0]
    d, B = _batch(sizes, Re, lid)
    offs = np.asarray(B["node_offsets"])
    d.set_instances([offs[0], offs[2], offs[4]])
    d.set_dirichlet(B["dofs"], B["values"])
    u2 = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    r2 = d.newton_solve_batched(u2, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32")
    assert len(r2) == 2 and all(r["status"] == 0 for r in r2)
    d.set_instances(offs)
    d.set_dirichlet(B["dofs"], B["values"])
    u4 = torch.zeros_like(u2)
    r4 = d.newton_solve_batched(u4, rtol=1e-8, lin_rtol=1e-3, jacobian_prec="f32")
    assert len(r4) == 4
    U = u4.cpu().numpy()
    for i, (N, re, u0) in enumerate(zip(sizes, Re, lid)):
        assert r4[i]["status"] == 0, (i, r4[i])
        roid, X, C = mesh.structured_quads(N)
        dofs, vals = mesh.cavity_dirichlet(X, u0)
        o = oracle.Oracle(2); o.set_kinematic_viscosity(u0 / re); o.set_upwind("full"); o.set_stabilization("flow")
        o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
        D, _ = o.assemble(U[offs[i] * 3:offs[i + 1] * 3], jacobian=False)
        assert np.linalg.norm(D) <= 1.01e-8 * r4[i]["initial_defect"], (i, np.linalg.norm(D), r4[i])

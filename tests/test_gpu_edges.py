"""Edge cases on the GPU: empty element batches, a single-element mesh, a batch
of one instance, one MLP point; each against the oracle or the obvious answer."""
import numpy as np
import pytest

import oracle
from _cases import rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, _capi, mesh

pytestmark = pytest.mark.gpu


def test_empty_element_batch_is_a_no_op(cuda):
    import torch
    d = NavierStokesFV1("u,v,p")
    d.set_kinematic_viscosity(0.01); d.set_upwind("full"); d.set_stabilization("fields")
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device=cuda)
    out = {k: z(0, 12) for k in ("defA", "defM", "rhs")}
    out.update({k: z(0, 144) for k in ("jacA", "jacM")})
    d.elem_batch(_capi.QUADRILATERAL, z(0, 4, 2), z(0, 12), None, 0.0, **out)
    torch.cuda.synchronize()


@pytest.mark.parametrize("roid", [_capi.TRIANGLE, _capi.QUADRILATERAL, _capi.TETRAHEDRON, _capi.HEXAHEDRON])
def test_single_element_mesh_matches_oracle(cuda, roid):
    import torch
    dim = 2 if roid in (_capi.TRIANGLE, _capi.QUADRILATERAL) else 3
    nsh = {_capi.TRIANGLE: 3, _capi.QUADRILATERAL: 4, _capi.TETRAHEDRON: 4, _capi.HEXAHEDRON: 8}[roid]
    ref = {_capi.TRIANGLE: [[0, 0], [1, 0], [0, 1]], _capi.QUADRILATERAL: [[0, 0], [1, 0], [1, 1], [0, 1]],
           _capi.TETRAHEDRON: [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]],
           _capi.HEXAHEDRON: [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]}[roid]
    rng = np.random.default_rng(roid)
    X = np.array(ref, float) * 0.3 + rng.uniform(-0.03, 0.03, (nsh, dim))
    C = np.arange(nsh, dtype=np.int32)[None, :]
    b = dim + 1
    U = rng.uniform(-1, 1, nsh * b)
    d = NavierStokesFV1(dim=dim); o = oracle.Oracle(dim)
    for disc in (d, o):
        disc.set_kinematic_viscosity(0.01); disc.set_upwind("lps"); disc.set_stabilization("flow")
        disc.set_mesh(roid, X, C)
    tu = torch.tensor(U, dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(nsh * nsh * b * b, dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D)
    d.assemble_jacobian(tu, J)
    Do, Jo = o.assemble(U)
    assert rel_err(D.cpu().numpy(), Do) <= 1e-12 and rel_err(J.cpu().numpy(), Jo) <= 1e-12


def test_batch_of_one_instance_matches_the_single_solver(cuda):
    import torch
    B = mesh.cavity_batch([24], [200.0], [1.0])
    d = NavierStokesFV1("u,v,p")
    d.set_kinematic_viscosity(1.0); d.set_upwind("full"); d.set_stabilization("flow")
    d.set_mesh(B["elem_type"], B["coords"], B["conn"]); d.set_elem_viscosity(B["nu_elem"])
    d.set_instances(B["node_offsets"]); d.set_dirichlet(B["dofs"], B["values"]); d.set_instance_grids([24])
    u = torch.zeros(B["coords"].shape[0] * 3, dtype=torch.float64, device=cuda)
    r = d.newton_solve_batched(u, rtol=1e-8)
    assert len(r) == 1 and r[0]["status"] == 0
    o = oracle.Oracle(2); o.set_kinematic_viscosity(1.0 / 200.0); o.set_upwind("full"); o.set_stabilization("flow")
    o.set_mesh(B["elem_type"], B["coords"], B["conn"]); o.set_dirichlet(B["dofs"], B["values"])
    D, _ = o.assemble(u.cpu().numpy(), jacobian=False)
    assert np.linalg.norm(D) <= 1.01e-8 * r[0]["initial_defect"]


def test_mlp_single_point(cuda):
    import torch

    from oracle import mlp_oracle as mo
    from plugin_navierstokes_gb300.warm_start import CoordinateMLP
    p = mo.init_params(3, film_scale=0.2)
    m = CoordinateMLP(max_points=128, max_slots=2)
    m.set_params(p)
    xy = np.array([[0.25, 0.75]], np.float32)
    cond = np.array([[0.3, -0.4]], np.float32)
    out = torch.empty((1, 3), dtype=torch.float32, device=cuda)
    m.forward(torch.from_numpy(xy).to(cuda), np.array([0, 1]), cond, out)
    ref, _ = mo.forward(p, xy, np.array([0, 1]), cond, use_bf16=True)
    assert np.abs(out.double().cpu().numpy() - ref).max() <= 2e-3 * max(1.0, np.abs(ref).max())

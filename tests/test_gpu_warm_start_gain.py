"""What the trained network gains: a warm start learned from plain-method solves
of small cavities needs fewer Krylov iterations (and no more Newton steps) than
the zero initial iterate on held-out cavities, while every instance still meets
1e-8 of its zero-iterate defect (the same target for both)."""
import numpy as np
import pytest

import oracle
from plugin_navierstokes_gb300 import mesh

pytestmark = pytest.mark.gpu


def _draws(n, seed, re_max):
    r = mesh.uniform(seed, 2 * n).reshape(n, 2)
    return np.exp(np.log(10.0) + r[:, 0] * (np.log(re_max) - np.log(10.0))), 0.5 + 1.5 * r[:, 1]


def test_learned_warm_start_gain(cuda):
    import torch

    from plugin_navierstokes_gb300.warm_start import CavityBatch, CoordinateMLP, generate_training_set

    N = 32
    Re, lid = _draws(48, 41, 300.0)
    coords, targets, cond, res = generate_training_set(Re, lid, N=N, batch=48)
    assert all(r["status"] == 0 for r in res)
    m = CoordinateMLP(max_points=8192, max_slots=16, seed=4)
    hist = m.train(coords, targets, cond, steps=2500, slots=16, points_per_slot=512, lr=2e-3, lr_final=2e-5, seed=4)
    assert hist[-50:].mean() < 0.02 * hist[:10].mean()
    Re_t, lid_t = _draws(12, 43, 300.0)
    cb = CavityBatch(np.full(12, N), Re_t, lid_t)
    cb.cluster_size = 4
    out = {}
    for name in ("zero", "learned"):
        u = cb.zeros()
        if name == "learned":
            cb.predict(m, u)
        r = cb.solve(u, "f32", zero_fallback=(name == "learned"))
        assert all(x["status"] == 0 for x in r), (name, r)
        U = u.cpu().numpy()
        for i in range(12):
            roid, X, C = mesh.structured_quads(N)
            dofs, vals = mesh.cavity_dirichlet(X, float(lid_t[i]))
            o = oracle.Oracle(2)
            o.set_kinematic_viscosity(float(lid_t[i] / Re_t[i])); o.set_upwind("full"); o.set_stabilization("flow")
            o.set_mesh(roid, X, C); o.set_dirichlet(dofs, vals)
            D, _ = o.assemble(U[cb.node_offsets[i] * 3:cb.node_offsets[i + 1] * 3], jacobian=False)
            x0 = np.zeros(X.shape[0] * 3)
            x0[dofs] = vals
            D0, _ = o.assemble(x0, jacobian=False)
            assert np.linalg.norm(D) <= 1.01e-8 * np.linalg.norm(D0), (name, i)
        out[name] = (sum(x["iterations"] for x in r), sum(x["linear_iterations"] for x in r),
                     float(np.median([x["initial_defect"] for x in r])))
    # the network's iterate starts far closer than zero, and the solves need less work
    assert out["learned"][2] < 0.5 * out["zero"][2], out
    assert out["learned"][0] <= out["zero"][0], out
    assert out["learned"][1] < out["zero"][1], out

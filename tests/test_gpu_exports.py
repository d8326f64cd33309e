"""GPU parity of the data exports (ex_nodal_velocity, ex_velocity_grad,
ex_velocity_ip, ex_nodal_pressure, ex_pressure_grad; navier_stokes_fv1.cpp:894-1491)
against the oracle, whose exports are pinned to the reference's own by
tests/test_reference_pin.py. Values and derivatives at the SCVF ips, the SCV ips
and given local points, for every discretisation case including the positive
upwind. Tolerance: max |gpu - oracle| / max |oracle| <= 1e-12 per array.
"""
import numpy as np
import pytest

import oracle
from _cases import DIM, DISC_CASES, NSH, POS_CASES, ROIDS, cfg_name, configure, random_elements, random_local_u, rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, NSFV1Error

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES) + len(POS_CASES)))
def test_exports_match_oracle(cuda, tname, ci):
    import torch
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = (DISC_CASES + POS_CASES)[ci]
    corners = np.concatenate([random_elements(roid, 30, 3000 + ci + roid), random_elements(roid, 6, 3100 + ci, affine=True)])
    u = random_local_u(roid, 36, 3200 + ci, zero_frac=0.1)
    uo = random_local_u(roid, 36, 3300 + ci) if cfg[3] else None
    lips = np.random.default_rng(ci + roid).random((7, dim)) * (0.3 if roid in (2, 4) else 1.0)
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, cfg)
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    exports = [d.velocity(), d.velocity_grad(), d.velocity_ip(), d.pressure(), d.pressure_grad()]
    for which, ex in enumerate(exports):
        for kind, pts in ((0, "scvf"), (1, "scv"), (2, lips)):
            v, der = ex.evaluate(roid, t(corners), t(u), None if uo is None else t(uo), 0.01, pts, derivs=True)
            torch.cuda.synchronize()
            rv, rd = o.export(which, roid, corners, u, uo, 0.01, kind, lips if kind == 2 else None)
            assert rel_err(v.cpu().numpy(), rv) <= TOL, (tname, cfg_name(cfg), oracle.EXPORTS[which], kind, "values")
            assert rel_err(der.cpu().numpy(), rd) <= TOL, (tname, cfg_name(cfg), oracle.EXPORTS[which], kind, "derivs")
            # values alone give the same numbers
            v2, _ = ex.evaluate(roid, t(corners), t(u), None if uo is None else t(uo), 0.01, pts, derivs=False)
            torch.cuda.synchronize()
            assert torch.equal(v, v2)


def test_export_arguments_are_checked(cuda):
    import torch
    d = NavierStokesFV1(dim=2)
    configure(d, 2, DISC_CASES[0])
    c = torch.zeros((1, 4, 2), dtype=torch.float64, device=cuda)
    u = torch.zeros((1, 12), dtype=torch.float64, device=cuda)
    v = torch.zeros((1, 70, 2), dtype=torch.float64, device=cuda)
    with pytest.raises(NSFV1Error):
        d.export(9, 3, c, u, v)
    with pytest.raises(NSFV1Error):
        d.export(0, 3, c, u, v, points=np.zeros((65, 2)))
    with pytest.raises(NSFV1Error):
        d.export(0, 8, c, u, v)

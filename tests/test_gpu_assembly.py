"""GPU parity of the FV1 assembly against the oracle and the golden fixtures.

Tolerance (FP64 path): max |gpu - ref| / max |ref| <= 1e-12 per output array.
FP32-Jacobian mode: <= 2e-5 against the FP64 oracle Jacobian.
Integer data (pattern, colouring): bit-exact.
"""
import os

import numpy as np
import pytest

import oracle
from _cases import DISC_CASES, DIM, NSH, ROIDS, cfg_name, configure, random_elements, random_local_u, rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, NSFV1Error, mesh

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12
TOL32 = 2e-5


def _gpu_elem(cuda, roid, cfg, corners, u, uo, dt=0.01):
    import torch
    dim = DIM[roid]
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, cfg)
    n = corners.shape[0]
    nloc = (dim + 1) * NSH[roid]
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    out = {k: torch.zeros((n, nloc), dtype=torch.float64, device=cuda) for k in ("defA", "defM", "rhs")}
    out.update({k: torch.zeros((n, nloc * nloc), dtype=torch.float64, device=cuda) for k in ("jacA", "jacM")})
    d.elem_batch(roid, t(corners), t(u), None if uo is None else t(uo), dt, **out)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_element_callbacks_match_golden(cuda, tname, ci):
    g = np.load(os.path.join(GOLDEN, "elements.npz"))
    roid = ROIDS[tname]
    key = f"{tname}_{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    r = _gpu_elem(cuda, roid, DISC_CASES[ci], g[key + "_corners"], g[key + "_u"], uo)
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + "_" + k]) <= TOL64, (key, cfg_name(DISC_CASES[ci]), k, rel_err(r[k], g[key + "_" + k]))


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_element_callbacks_match_reference_fixtures(cuda, tname, ci):
    """The GPU element callbacks against the numbers of the reference's own
    code (tests/golden/reference_elements.npz, made by make_reference_golden.py
    from the reference sources compiled against the ugcore stand-in)."""
    g = np.load(os.path.join(GOLDEN, "reference_elements.npz"))
    roid = ROIDS[tname]
    key = f"{tname}_{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    r = _gpu_elem(cuda, roid, DISC_CASES[ci], g[key + "_corners"], g[key + "_u"], uo)
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + "_" + k]) <= TOL64, (key, cfg_name(DISC_CASES[ci]), k, rel_err(r[k], g[key + "_" + k]))


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", [i for i, c in enumerate(DISC_CASES) if not c[7]])
def test_pac_element_callbacks_match_reference_fixtures(cuda, tname, ci):
    """set_pac_upwind(true) on the GPU against the reference's own PAC outputs."""
    import torch
    g = np.load(os.path.join(GOLDEN, "reference_elements.npz"))
    roid = ROIDS[tname]
    dim = DIM[roid]
    key = f"{tname}_{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, DISC_CASES[ci])
    d.set_pac_upwind(True)
    corners, u = g[key + "_corners"], g[key + "_u"]
    n = corners.shape[0]
    nloc = (dim + 1) * NSH[roid]
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    out = {k: torch.zeros((n, nloc), dtype=torch.float64, device=cuda) for k in ("defA", "defM", "rhs")}
    out.update({k: torch.zeros((n, nloc * nloc), dtype=torch.float64, device=cuda) for k in ("jacA", "jacM")})
    d.elem_batch(roid, t(corners), t(u), None if uo is None else t(uo), 0.01, **out)
    torch.cuda.synchronize()
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        r = out[k].cpu().numpy()
        assert rel_err(r, g[key + "_pac_" + k]) <= TOL64, (key, "pac", k, rel_err(r, g[key + "_pac_" + k]))


@pytest.mark.parametrize("gen", ["quads", "hexes", "tris"])
@pytest.mark.parametrize("cfgi", [1, 2, 3])
def test_pac_global_assembly_matches_oracle(cuda, gen, cfgi):
    """PAC through the global kernels (separate and fused, FP64 and FP32 values)."""
    import torch
    roid, X, C = {"quads": lambda: mesh.structured_quads(12), "hexes": lambda: mesh.structured_hexes(4),
                  "tris": lambda: mesh.jittered_triangles(10, seed=6)}[gen]()
    dim = DIM[roid]
    cfg = DISC_CASES[cfgi]
    b = dim + 1
    U = mesh.solenoidal_state(X, seed=13) if dim == 3 else (mesh.uniform(14, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    Uo = (U * 0.85) if cfg[3] else None
    dt = 0.02 if cfg[3] else 0.0
    o = oracle.Oracle(dim); configure(o, dim, cfg); o.set_pac_upwind(True); o.set_mesh(roid, X, C)
    d = NavierStokesFV1(dim=dim); configure(d, dim, cfg); d.set_pac_upwind(True); d.set_mesh(roid, X, C)
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo.ravel(), dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(o.nnzb * b * b, dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D, tuo, dt)
    d.assemble_jacobian(tu, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64 and rel_err(J.cpu().numpy(), Jref) <= TOL64
    d.assemble_defect_jacobian(tu, D, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64 and rel_err(J.cpu().numpy(), Jref) <= TOL64
    J32 = torch.empty(o.nnzb * b * b, dtype=torch.float32, device=cuda)
    d.assemble_jacobian(tu, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32
    d.assemble_defect_jacobian(tu, D, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_element_callbacks_match_oracle_random(cuda, tname, ci):
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = DISC_CASES[ci]
    n = 257
    corners = random_elements(roid, n, 9000 + 17 * ci + roid)
    u = random_local_u(roid, n, 9100 + ci, zero_frac=0.1)
    uo = random_local_u(roid, n, 9200 + ci) if cfg[3] else None
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    ref = o.elem_batch(roid, corners, u, uo, 0.01)
    r = _gpu_elem(cuda, roid, cfg, corners, u, uo)
    for k in ref:
        assert rel_err(r[k], ref[k]) <= TOL64, (tname, cfg_name(cfg), k, rel_err(r[k], ref[k]))


def _setup_mesh_pair(name, g):
    if name == "quad":
        roid, dim, cfg, U, Uo, dt = 3, 2, DISC_CASES[0], g["quad_U"], None, 0.0
    elif name == "hex":
        roid, dim, cfg, U, Uo, dt = 8, 3, DISC_CASES[1], g["hex_U"], None, 0.0
    else:
        roid, dim, cfg, U, Uo, dt = 2, 2, DISC_CASES[0], g["tri_U"], g["tri_Uold"], 0.01
    return roid, dim, cfg, U, Uo, dt


@pytest.mark.parametrize("name", ["quad", "hex", "tri"])
def test_global_assembly_matches_golden(cuda, name):
    import torch
    g = np.load(os.path.join(GOLDEN, "meshes.npz"))
    roid, dim, cfg, U, Uo, dt = _setup_mesh_pair(name, g)
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, cfg)
    d.set_mesh(roid, g[name + "_coords"], g[name + "_conn"])
    if name + "_dofs" in g:
        d.set_dirichlet(g[name + "_dofs"], g[name + "_dvals"])
    rp, ci = d.pattern()
    assert np.array_equal(rp, g[name + "_rowptr"]) and np.array_equal(ci, g[name + "_colidx"])
    assert np.array_equal(d.coloring(), g[name + "_color"])
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo.ravel(), dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    b = dim + 1
    J = torch.empty(ci.size * b * b, dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D, tuo, dt)
    d.assemble_jacobian(tu, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), g[name + "_D"]) <= TOL64
    assert rel_err(J.cpu().numpy(), g[name + "_J"]) <= TOL64
    # FP32-Jacobian mode against the FP64 oracle Jacobian
    J32 = torch.empty(ci.size * b * b, dtype=torch.float32, device=cuda)
    d.assemble_jacobian(tu, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), g[name + "_J"]) <= TOL32
    # determinism: a second run is bitwise identical
    D2 = torch.empty_like(tu)
    J2 = torch.empty_like(J)
    d.assemble_defect(tu, D2, tuo, dt)
    d.assemble_jacobian(tu, J2, tuo, dt)
    torch.cuda.synchronize()
    assert torch.equal(D, D2) and torch.equal(J, J2)


@pytest.mark.parametrize("gen,cfgi", [("quads", 0), ("quads", 3), ("hexes", 1), ("hexes", 2), ("tris", 4)])
def test_global_assembly_matches_oracle(cuda, gen, cfgi):
    import torch
    roid, X, C = {"quads": lambda: mesh.structured_quads(24), "hexes": lambda: mesh.structured_hexes(6),
                  "tris": lambda: mesh.jittered_triangles(16, seed=4)}[gen]()
    dim = DIM[roid]
    cfg = DISC_CASES[cfgi]
    b = dim + 1
    U = mesh.solenoidal_state(X, seed=7) if dim == 3 else (mesh.uniform(8, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    Uo = (U * 0.9) if cfg[3] else None
    dt = 0.01 if cfg[3] else 0.0
    o = oracle.Oracle(dim); configure(o, dim, cfg); o.set_mesh(roid, X, C)
    d = NavierStokesFV1(dim=dim); configure(d, dim, cfg); d.set_mesh(roid, X, C)
    if dim == 2:
        dofs, vals = mesh.cavity_dirichlet(X, 1.0)
        o.set_dirichlet(dofs, vals); d.set_dirichlet(dofs, vals)
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo.ravel(), dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(o.nnzb * b * b, dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D, tuo, dt)
    d.assemble_jacobian(tu, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64
    assert rel_err(J.cpu().numpy(), Jref) <= TOL64


def test_bsr_spmv_matches_oracle(cuda):
    import torch
    g = np.load(os.path.join(GOLDEN, "meshes.npz"))
    o = oracle.Oracle(3); configure(o, 3, DISC_CASES[1]); o.set_mesh(8, g["hex_coords"], g["hex_conn"])
    d = NavierStokesFV1(dim=3); configure(d, 3, DISC_CASES[1]); d.set_mesh(8, g["hex_coords"], g["hex_conn"])
    x = mesh.uniform(5, g["hex_U"].size) - 0.5
    y_ref = o.bsr_mv(g["hex_J"], x)
    for dt_ in (torch.float64, torch.float32):
        V = torch.tensor(g["hex_J"], dtype=dt_, device=cuda)
        tx = torch.tensor(x, dtype=torch.float64, device=cuda)
        ty = torch.empty_like(tx)
        d.bsr_mv(V, tx, ty)
        torch.cuda.synchronize()
        assert rel_err(ty.cpu().numpy(), y_ref) <= (TOL64 if dt_ == torch.float64 else TOL32)
        if dt_ == torch.float32:
            # the BiCGStab form: x split once into float pairs, the same product bit for bit
            xs = d.split_vector(tx)
            ys = torch.empty_like(tx)
            d.bsr_mv_split(V, xs, ys)
            torch.cuda.synchronize()
            assert torch.equal(ys, ty)
            h, l = xs.view(-1, 2)[:, 0].double(), xs.view(-1, 2)[:, 1].double()
            assert float(((h + l - tx).abs() / tx.abs().clamp_min(1e-300)).max()) <= 2.0 ** -46


def test_lps_no_cut_side_is_reported(cuda):
    """An element whose corner coordinate is NaN makes every LPS ray test fail:
    the call returns NSFV1_ERR_GEOMETRY (the reference's UG_THROW "Cannot find
    cut side"), and the handle stays usable."""
    import torch
    d = NavierStokesFV1(dim=2)
    d.set_kinematic_viscosity(0.01); d.set_upwind("lps"); d.set_stabilization("fields")
    corners = torch.tensor([[[0, 0], [1, 0], [1, float("nan")], [0, 1.0]]], dtype=torch.float64, device=cuda)
    u = torch.ones((1, 12), dtype=torch.float64, device=cuda)
    dA = torch.zeros((1, 12), dtype=torch.float64, device=cuda)
    with pytest.raises(NSFV1Error):
        d.elem_batch(3, corners, u, defA=dA)
    ok = torch.tensor(random_elements(3, 1, 1), dtype=torch.float64, device=cuda)
    d.elem_batch(3, ok, u, defA=dA)


@pytest.mark.parametrize("gen", ["quads", "hexes"])
def test_block_jacobi_matches_numpy(cuda, gen):
    import torch
    roid, X, C = {"quads": lambda: mesh.structured_quads(12), "hexes": lambda: mesh.structured_hexes(4)}[gen]()
    dim = DIM[roid]
    b = dim + 1
    d = NavierStokesFV1(dim=dim); configure(d, dim, DISC_CASES[0] if dim == 2 else DISC_CASES[1]); d.set_mesh(roid, X, C)
    U = mesh.solenoidal_state(X, seed=3) if dim == 3 else (mesh.uniform(8, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    rp, ci = d.pattern()
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    J = torch.empty(ci.size * b * b, dtype=torch.float64, device=cuda)
    d.assemble_jacobian(tu, J)
    r = torch.tensor(mesh.uniform(4, tu.numel()) - 0.5, dtype=torch.float64, device=cuda)
    z = torch.empty_like(r)
    d.block_jacobi(J, r, z)
    torch.cuda.synchronize()
    Jh = J.cpu().numpy().reshape(-1, b, b)
    diag = np.array([Jh[rp[i] + np.searchsorted(ci[rp[i]:rp[i + 1]], i)] for i in range(X.shape[0])])
    zref = np.einsum("nij,nj->ni", np.linalg.inv(diag), r.cpu().numpy().reshape(-1, b)).ravel()
    assert rel_err(z.cpu().numpy(), zref) <= TOL64


def test_assembly_cta_size_is_bitwise_neutral_and_autotuned(cuda):
    """The colour scatter is order-free, so the assembly CTA size changes no bit;
    the assembly autotuner keeps one of its candidates."""
    import torch
    from plugin_navierstokes_gb300 import NavierStokesFV1, mesh
    roid, X, C = mesh.structured_hexes(6)
    U = mesh.solenoidal_state(X, seed=1)
    d = NavierStokesFV1("u,v,w,p", "Inner")
    d.set_kinematic_viscosity(0.0025); d.set_upwind("lps"); d.set_stabilization("flow")
    d.set_mesh(roid, X, C)
    nnzb = d.pattern_info()["nnz_blocks"]
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    out = []
    for t in (32, 64, 96, 128):
        d.set_assembly_threads(t)
        D = torch.empty_like(tu)
        J = torch.empty(nnzb * 16, dtype=torch.float64, device=cuda)
        d.assemble_defect(tu, D)
        d.assemble_jacobian(tu, J)
        out.append((D, J))
    for D, J in out[1:]:
        assert torch.equal(D, out[0][0]) and torch.equal(J, out[0][1])
    best, ms = d.assembly_autotune(tu, "f64", (32, 64, 128))
    assert best in (32, 64, 128) and len(ms) == 3 and ms[(32, 64, 128).index(best)] == min(ms)


def test_fp32_3d_jacobian_needs_16_byte_alignment(cuda):
    import torch
    from plugin_navierstokes_gb300 import NSFV1Error, NavierStokesFV1, mesh
    roid, X, C = mesh.structured_hexes(2)
    d = NavierStokesFV1("u,v,w,p", "Inner")
    d.set_kinematic_viscosity(0.0025); d.set_upwind("lps"); d.set_stabilization("flow")
    d.set_mesh(roid, X, C)
    nnzb = d.pattern_info()["nnz_blocks"]
    tu = torch.zeros(X.shape[0] * 4, dtype=torch.float64, device=cuda)
    J = torch.zeros(nnzb * 16 + 4, dtype=torch.float32, device=cuda)
    with pytest.raises(NSFV1Error):
        d.assemble_jacobian(tu, J[1:])
    d.assemble_jacobian(tu, J[4:])   # 16-byte offset: fine


@pytest.mark.parametrize("gen", ["quads", "hexes", "tris"])
@pytest.mark.parametrize("cfgi", range(len(DISC_CASES)))
def test_fused_defect_jacobian_matches_oracle(cuda, gen, cfgi):
    """nsfv1_assemble_defect_jacobian (one pass for both outputs) against the oracle,
    for every discretisation case, stationary or implicit Euler as the case says."""
    import torch
    roid, X, C = {"quads": lambda: mesh.structured_quads(16), "hexes": lambda: mesh.structured_hexes(5),
                  "tris": lambda: mesh.jittered_triangles(12, seed=5)}[gen]()
    dim = DIM[roid]
    cfg = DISC_CASES[cfgi]
    b = dim + 1
    U = mesh.solenoidal_state(X, seed=9) if dim == 3 else (mesh.uniform(11, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    Uo = (U * 0.8) if cfg[3] else None
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
    d.assemble_defect_jacobian(tu, D, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64, (gen, cfg_name(cfg))
    assert rel_err(J.cpu().numpy(), Jref) <= TOL64, (gen, cfg_name(cfg))
    # FP32 values through the same entry point (FP64 defect + FP32 Jacobian)
    D32 = torch.full_like(tu, float("nan"))
    J32 = torch.full((o.nnzb * b * b,), float("nan"), dtype=torch.float32, device=cuda)
    d.assemble_defect_jacobian(tu, D32, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D32.cpu().numpy(), Dref) <= TOL64
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32
    # with FP32 values the call is the FP64 defect and the FP32 Jacobian of the separate calls,
    # bit for bit, and repeatable
    Ds, J32s = torch.empty_like(D), torch.empty_like(J32)
    d.assemble_defect(tu, Ds, tuo, dt)
    d.assemble_jacobian(tu, J32s, tuo, dt)
    torch.cuda.synchronize()
    assert torch.equal(Ds, D32) and torch.equal(J32s, J32)
    # determinism of the fused pass
    D2, J2 = torch.empty_like(D), torch.empty_like(J)
    d.assemble_defect_jacobian(tu, D2, J2, tuo, dt)
    torch.cuda.synchronize()
    assert torch.equal(D, D2) and torch.equal(J, J2)


def test_pattern_and_coloring_bit_exact_at_benchmark_size(cuda):
    """The 64^3 hexahedral benchmark mesh: block-CSR pattern (7,189,057 blocks) and
    element colouring of the handle, bit-exact with the oracle's."""
    roid, X, C = mesh.structured_hexes(64)
    d = NavierStokesFV1(dim=3); configure(d, 3, DISC_CASES[1]); d.set_mesh(roid, X, C)
    o = oracle.Oracle(3); configure(o, 3, DISC_CASES[1]); o.set_mesh(roid, X, C)
    rp, ci = d.pattern()
    orp, oci = o.pattern()
    assert ci.size == 193 ** 3
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    col = d.coloring()
    ocol, onc = o.coloring()
    assert np.array_equal(col, ocol) and d.pattern_info()["n_colors"] == onc


@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_prism_mesh_assembly_matches_oracle(cuda, ci):
    """Prisms (the reference registers them, navier_stokes_fv1.cpp:1541-1544) on an extruded
    jittered triangulation: defect and FP64 / FP32 Jacobians through the separate and the
    fused entry points, pattern and colouring bit-exact."""
    import torch
    roid, X, C = mesh.extruded_prisms(4, 3, seed=8)
    cfg = DISC_CASES[ci]
    b = 4
    U = mesh.solenoidal_state(X, seed=15)
    Uo = (U * 0.8) if cfg[3] else None
    dt = 0.02 if cfg[3] else 0.0
    o = oracle.Oracle(3); configure(o, 3, cfg); o.set_mesh(roid, X, C)
    d = NavierStokesFV1(dim=3); configure(d, 3, cfg); d.set_mesh(roid, X, C)
    rp, cix = d.pattern()
    orp, oci = o.pattern()
    assert np.array_equal(rp, orp) and np.array_equal(cix, oci) and np.array_equal(d.coloring(), o.coloring()[0])
    Dref, Jref = o.assemble(U, Uo, dt)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    tuo = None if Uo is None else torch.tensor(Uo.ravel(), dtype=torch.float64, device=cuda)
    D = torch.empty_like(tu)
    J = torch.empty(o.nnzb * b * b, dtype=torch.float64, device=cuda)
    d.assemble_defect(tu, D, tuo, dt)
    d.assemble_jacobian(tu, J, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D.cpu().numpy(), Dref) <= TOL64 and rel_err(J.cpu().numpy(), Jref) <= TOL64, cfg_name(cfg)
    D2, J2 = torch.empty_like(D), torch.empty_like(J)
    d.assemble_defect_jacobian(tu, D2, J2, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(D2.cpu().numpy(), Dref) <= TOL64 and rel_err(J2.cpu().numpy(), Jref) <= TOL64
    J32 = torch.empty(o.nnzb * b * b, dtype=torch.float32, device=cuda)
    d.assemble_jacobian(tu, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32
    d.assemble_defect_jacobian(tu, D2, J32, tuo, dt)
    torch.cuda.synchronize()
    assert rel_err(J32.double().cpu().numpy(), Jref) <= TOL32

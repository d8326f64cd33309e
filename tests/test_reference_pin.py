"""The oracle pinned to the reference's own code.

The reference's FV1 sources (navier_stokes_fv1.cpp, stabilization.cpp,
upwind.cpp, upwind_interface.cpp and the NavierStokes base classes) are
compiled unmodified against the ugcore stand-in in oracle/ugshim into
oracle/_ref/libnsfv1_ref.so. Its element callbacks produced the committed
fixtures tests/golden/reference_elements.npz (make_reference_golden.py); the
oracle must reproduce them, and, where the reference checkout is present, it
must match the reference live on further seeded elements and the two
restatements of ugcore's FV1 geometry must agree.
Tolerance: max |oracle - reference| / max |reference| <= 1e-12 per array
(measured about 2e-14).
"""
import os

import numpy as np
import pytest

import oracle
from _cases import DISC_CASES, DIM, NSH, POS_CASES, ROIDS, cfg_name, configure, random_elements, random_local_u, ref_config, rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_elements.npz")
TOL = 1e-12
has_ref = oracle.reference_root() is not None


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_oracle_reproduces_the_reference_fixtures(tname, ci):
    g = np.load(GOLDEN)
    roid = ROIDS[tname]
    dim = DIM[roid]
    key = f"{tname}_{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    o = oracle.Oracle(dim)
    configure(o, dim, DISC_CASES[ci])
    r = o.elem_batch(roid, g[key + "_corners"], g[key + "_u"], uo, 0.01)
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + "_" + k]) <= TOL, (key, cfg_name(DISC_CASES[ci]), k, rel_err(r[k], g[key + "_" + k]))


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", [i for i, c in enumerate(DISC_CASES) if not c[7]])
def test_oracle_pac_reproduces_the_reference_fixtures(tname, ci):
    """set_pac_upwind(true): the stabilised velocity as the convective upwind."""
    g = np.load(GOLDEN)
    roid = ROIDS[tname]
    dim = DIM[roid]
    key = f"{tname}_{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    o = oracle.Oracle(dim)
    configure(o, dim, DISC_CASES[ci])
    o.set_pac_upwind(True)
    r = o.elem_batch(roid, g[key + "_corners"], g[key + "_u"], uo, 0.01)
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + "_pac_" + k]) <= TOL, (key, "pac", k, rel_err(r[k], g[key + "_pac_" + k]))


@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(POS_CASES)))
@pytest.mark.parametrize("pac", [False, True])
def test_oracle_positive_upwind_reproduces_the_reference_fixtures(tname, ci, pac):
    """The positive upwind (ip shapes) and the non-diagonal FIELDS / FLOW branches."""
    g = np.load(GOLDEN)
    roid = ROIDS[tname]
    dim = DIM[roid]
    key = f"{tname}_pos{ci}"
    uo = g[key + "_uold"] if (key + "_uold") in g else None
    o = oracle.Oracle(dim)
    configure(o, dim, POS_CASES[ci])
    if pac:
        o.set_pac_upwind(True)
    r = o.elem_batch(roid, g[key + "_corners"], g[key + "_u"], uo, 0.01)
    tag = "_pac_" if pac else "_"
    for k in ("defA", "jacA", "defM", "jacM", "rhs"):
        assert rel_err(r[k], g[key + tag + k]) <= TOL, (key, pac, k, rel_err(r[k], g[key + tag + k]))


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(POS_CASES)))
def test_oracle_positive_upwind_matches_the_reference_live(tname, ci):
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = POS_CASES[ci]
    n = 40
    corners = np.concatenate([random_elements(roid, n, 700 + 11 * ci + roid), random_elements(roid, 8, 800 + ci, affine=True)])
    u = random_local_u(roid, n + 8, 900 + ci, zero_frac=0.1)
    uo = random_local_u(roid, n + 8, 950 + ci) if cfg[3] else None
    for pac in (False, True):
        o = oracle.Oracle(dim)
        configure(o, dim, cfg)
        if pac:
            o.set_pac_upwind(True)
        mine = o.elem_batch(roid, corners, u, uo, 0.01)
        ref = oracle.ref_elem_batch(roid, dict(ref_config(dim, cfg), pac=pac), corners, u, uo, 0.01)
        for k in ref:
            assert rel_err(mine[k], ref[k]) <= TOL, (tname, cfg_name(cfg), pac, k, rel_err(mine[k], ref[k]))


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("conv,stab_up,stab", [("pos", "lps", "flow"), ("full", "pos", "fields"), ("lps", "pos", "flow")])
def test_oracle_mixed_upwind_objects_match_the_reference_live(tname, conv, stab_up, stab):
    """Convection and stabilisation with upwind objects of different kinds (one of them positive)."""
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = (conv, stab, "raw", True, 1.0, False, False, False, False)
    n = 24
    corners = random_elements(roid, n, 1200 + roid)
    u = random_local_u(roid, n, 1300 + roid)
    uo = random_local_u(roid, n, 1400 + roid)
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    o.set_stabilization_upwind(stab_up)
    mine = o.elem_batch(roid, corners, u, uo, 0.01)
    ref = oracle.ref_elem_batch(roid, dict(ref_config(dim, cfg), stab_upwind=stab_up), corners, u, uo, 0.01)
    for k in ref:
        assert rel_err(mine[k], ref[k]) <= TOL, (tname, conv, stab_up, k, rel_err(mine[k], ref[k]))


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_oracle_matches_the_reference_live(tname, ci):
    roid = ROIDS[tname]
    dim = DIM[roid]
    cfg = DISC_CASES[ci]
    n = 48
    corners = np.concatenate([random_elements(roid, n, 300 + 11 * ci + roid), random_elements(roid, 8, 400 + ci, affine=True)])
    u = random_local_u(roid, n + 8, 500 + ci, zero_frac=0.1)
    uo = random_local_u(roid, n + 8, 600 + ci) if cfg[3] else None
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    mine = o.elem_batch(roid, corners, u, uo, 0.01)
    ref = oracle.ref_elem_batch(roid, ref_config(dim, cfg), corners, u, uo, 0.01)
    for k in ref:
        assert rel_err(mine[k], ref[k]) <= TOL, (tname, cfg_name(cfg), k, rel_err(mine[k], ref[k]))


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
def test_geometry_restatements_agree(tname):
    """ugcore's FV1Geometry is restated twice (the oracle and the stand-in the
    reference is compiled against); both give the same dual mesh."""
    roid = ROIDS[tname]
    for e, c in enumerate(random_elements(roid, 6, 70 + roid)):
        a, va = oracle.geometry(roid, c)
        b, vb = oracle.ref_geometry(roid, c)
        for x, y in zip(a, b):
            assert (x["from"], x["to"]) == (y["from"], y["to"])
            for k in ("ip", "normal", "shape", "grad"):
                assert np.abs(x[k] - y[k]).max() <= 1e-13 * max(1.0, np.abs(y[k]).max()), (tname, e, k)
        assert np.abs(va - vb).max() <= 1e-13 * np.abs(vb).max()


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
def test_reference_rejects_what_the_product_rejects():
    """Unknown ids raise in the reference (UG_THROW) as they do in the oracle."""
    roid = ROIDS["quad"]
    c = random_elements(roid, 1, 3)
    u = random_local_u(roid, 1, 4)
    for bad in ({"upwind": "weighted", "stab": "fields"}, {"upwind": "full", "stab": "supg"},
                {"upwind": "full", "stab": "fields", "diff_length": "bogus"}):
        with pytest.raises(RuntimeError):
            oracle.ref_elem_batch(roid, dict(ref_config(2, DISC_CASES[0]), **bad), c, u)


def _ref_cavity_newton(n, stab, max_it):
    """Newton with exact sparse solves on the n x n lid-driven cavity (nu 0.01, full
    upwind), every defect and Jacobian assembled from the REFERENCE's element
    callbacks (gather / scatter in numpy, Dirichlet rows = identity); backtracking
    halves the step until ||d|| decreases. Returns the relative defect history."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from plugin_navierstokes_gb300 import mesh

    roid, X, C = mesh.structured_quads(n)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    cfg = {"nu": 0.01, "rho": 1.0, "upwind": "full", "stab": stab}
    E, nsh = C.shape
    b = 3
    idx = (C[:, None, :] * b + np.arange(b)[None, :, None]).reshape(E, b * nsh)
    rows = np.broadcast_to(idx[:, :, None], (E, b * nsh, b * nsh)).ravel()
    cols = np.broadcast_to(idx[:, None, :], (E, b * nsh, b * nsh)).ravel()
    keep = ~np.isin(rows, dofs)

    def assemble(U, jac):
        uloc = U.reshape(-1, b)[C].transpose(0, 2, 1).reshape(E, b * nsh)
        r = oracle.ref_elem_batch(roid, cfg, X[C], uloc, want=("defA", "jacA") if jac else ("defA",))
        D = np.zeros(U.size)
        np.add.at(D, idx.ravel(), r["defA"].ravel())
        D[dofs] = U[dofs] - vals
        if not jac:
            return D, None
        J = sp.coo_matrix((np.concatenate([r["jacA"].ravel()[keep], np.ones(dofs.size)]),
                           (np.concatenate([rows[keep], dofs]), np.concatenate([cols[keep], dofs]))), shape=(U.size, U.size))
        return D, J.tocsc()

    U = np.zeros(X.shape[0] * b)
    U[dofs] = vals
    D, J = assemble(U, True)
    d0 = np.linalg.norm(D)
    hist = []
    for _ in range(max_it):
        du = spl.spsolve(J, D)
        lam = 1.0
        for k in range(7):
            Ut = U - lam * du
            Dt, _ = assemble(Ut, False)
            if np.linalg.norm(Dt) < np.linalg.norm(D) or k == 6:
                break
            lam *= 0.5
        U = Ut
        D, J = assemble(U, True)
        hist.append(np.linalg.norm(D) / d0)
        if hist[-1] < 1e-8:
            break
    return hist


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
def test_64_cavity_full_upwind_fields_stalls_with_the_reference_code():
    """The finding behind the cavity workloads' FLOW setting, re-derived with the
    reference's own upwind (tie -> 'to', upwind.cpp:161) and FIELDS code: with
    full upwind + FIELDS the 64 x 64 cavity (nu 0.01) never reaches a relative
    defect of 1e-8 (it cycles between about 2e-4 and 1e-3), while full upwind +
    FLOW converges in about 12 exact Newton steps."""
    fields = _ref_cavity_newton(64, "fields", 30)
    assert min(fields) > 1e-5, fields
    assert max(fields[-10:]) > 2 * min(fields[-10:])   # no monotone progress: a cycle
    flow = _ref_cavity_newton(64, "flow", 20)
    assert flow[-1] < 1e-8 and len(flow) <= 15, flow


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("which", range(5))
def test_oracle_exports_match_the_reference_live(tname, which):
    """The data exports (navier_stokes_fv1.cpp:894-1491): values and derivatives at
    the SCVF ips, the SCV ips and given local points, for both stabilisations with
    and without the positive upwind (diagonal and non-diagonal branches)."""
    roid = ROIDS[tname]
    dim = DIM[roid]
    rng = np.random.default_rng(which + 10 * roid)
    lips = rng.random((5, dim)) * (0.3 if roid in (2, 4) else 1.0)
    cases = [DISC_CASES[i] for i in (0, 1, 2, 3, 5)] + [POS_CASES[i] for i in (0, 1, 4)]
    for ci, cfg in enumerate(cases):
        corners = np.concatenate([random_elements(roid, 6, 2000 + ci + roid), random_elements(roid, 2, 2100 + ci, affine=True)])
        u = random_local_u(roid, 8, 2200 + ci)
        uo = random_local_u(roid, 8, 2300 + ci) if cfg[3] else None
        for kind in (0, 1, 2):
            o = oracle.Oracle(dim)
            configure(o, dim, cfg)
            v, d = o.export(which, roid, corners, u, uo, 0.01, kind, lips if kind == 2 else None)
            rv, rd = oracle.ref_export(which, roid, ref_config(dim, cfg), corners, u, uo, 0.01, kind, lips if kind == 2 else None)
            assert rel_err(v, rv) <= TOL and rel_err(d, rd) <= TOL, (tname, oracle.EXPORTS[which], cfg_name(cfg), kind)


@pytest.mark.skipif(not has_ref, reason="reference checkout not present")
@pytest.mark.parametrize("tname", list(ROIDS))
@pytest.mark.parametrize("ci", range(len(DISC_CASES)))
def test_oracle_outflow_matches_the_reference_live(tname, ci):
    """NavierStokesNoNormalStressOutflowFV1 (no_normal_stress_outflow_fv1.cpp:343-504) on
    elements with random outflow sides: the reference's own disc, on the stand-in's
    boundary faces, against the oracle's element-level evaluation."""
    roid = ROIDS[tname]
    dim = DIM[roid]
    nside = {2: 3, 3: 4, 4: 4, 6: 5, 8: 6}[roid]
    cfg = DISC_CASES[ci]
    corners = np.concatenate([random_elements(roid, 16, 900 + ci + roid), random_elements(roid, 4, 950 + ci, affine=True)])
    u = random_local_u(roid, 20, 990 + ci)
    masks = np.random.default_rng(ci + roid).integers(1, 2 ** nside, 20)
    o = oracle.Oracle(dim)
    configure(o, dim, cfg)
    d, J = o.outflow_elem(roid, corners, u, masks)
    rd, rJ = oracle.ref_outflow(roid, ref_config(dim, cfg), corners, u, masks)
    assert np.abs(rd).max() > 0 and rel_err(d, rd) <= TOL and rel_err(J, rJ) <= TOL, (tname, cfg_name(cfg))

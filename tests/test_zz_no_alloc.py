"""The allocation-free block-Jacobi entry point (nsfv1_block_jacobi_noalloc).

It serves callers that cannot allocate device memory (all of their memory is
handed out by their own pool allocator): its scratch is a fixed array inside
the library. Like the allocating entry point, each call waits for its stream
to read the singular-block flag. The test
calls it through the C ABI twice in a row and checks it against the allocating
entry point nsfv1_block_jacobi, within the FP64 tolerance of the parity tests
(max |a - b| / max |b| <= 1e-12), and checks that a mesh above the stated
limit is refused. This file sorts last so that a run stopping at the first
failure has run every other test.
"""
import numpy as np
import pytest

from _cases import DISC_CASES, DIM, configure, rel_err
from plugin_navierstokes_gb300 import NavierStokesFV1, _capi, mesh

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def _noalloc(d, vals, r, z):
    import torch

    prec = _capi.F64 if vals.dtype == torch.float64 else _capi.F32
    stream = torch.cuda.current_stream().cuda_stream
    return d._lib.nsfv1_block_jacobi_noalloc(d._h, vals.data_ptr(), prec, r.data_ptr(), z.data_ptr(), stream)


@pytest.mark.parametrize("gen,jdtype", [("quads", "f64"), ("quads", "f32"), ("hexes", "f64"), ("hexes", "f32")])
def test_noalloc_matches_allocating_entry_point(cuda, gen, jdtype):
    import torch

    roid, X, C = {"quads": lambda: mesh.structured_quads(24), "hexes": lambda: mesh.structured_hexes(6)}[gen]()
    dim = DIM[roid]
    b = dim + 1
    d = NavierStokesFV1(dim=dim)
    configure(d, dim, DISC_CASES[0] if dim == 2 else DISC_CASES[1])
    d.set_mesh(roid, X, C)
    U = mesh.solenoidal_state(X, seed=3) if dim == 3 else (mesh.uniform(8, X.shape[0] * 3) * 2 - 1).reshape(-1, 3)
    nnzb = d.pattern_info()["nnz_blocks"]
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=cuda)
    J = torch.empty(nnzb * b * b, dtype=torch.float64 if jdtype == "f64" else torch.float32, device=cuda)
    d.assemble_jacobian(tu, J)
    for call, seed in enumerate((4, 5)):
        r = torch.tensor(mesh.uniform(seed, tu.numel()) - 0.5, dtype=torch.float64, device=cuda)
        z_ref = torch.empty_like(r)
        d.block_jacobi(J, r, z_ref)
        z = torch.full_like(r, float("nan"))
        assert _noalloc(d, J, r, z) == _capi.OK, d.last_error()
        torch.cuda.synchronize()
        assert rel_err(z.cpu().numpy(), z_ref.cpu().numpy()) <= TOL64, (gen, jdtype, call)


def test_noalloc_rejects_meshes_above_the_limit(cuda):
    import torch

    n = 182   # 183^2 = 33489 nodes > 32768
    roid, X, C = mesh.structured_quads(n)
    assert X.shape[0] > _capi.NOALLOC_MAX_NODES
    d = NavierStokesFV1(dim=2)
    configure(d, 2, DISC_CASES[0])
    d.set_mesh(roid, X, C)
    nnzb = d.pattern_info()["nnz_blocks"]
    J = torch.zeros(nnzb * 9, dtype=torch.float64, device=cuda)
    r = torch.zeros(X.shape[0] * 3, dtype=torch.float64, device=cuda)
    z = torch.zeros_like(r)
    assert _noalloc(d, J, r, z) == _capi.ERR_ARGUMENT
    assert "at most 32768" in d.last_error()


def test_noalloc_reports_a_planted_singular_block_and_recovers(cuda):
    """A zero diagonal block written into the Jacobian by the test gives
    NSFV1_ERR_BREAKDOWN from the allocation-free entry point, as from the
    allocating one; the next call with the valid Jacobian matches again."""
    import torch

    roid, X, C = mesh.structured_quads(12)
    d = NavierStokesFV1(dim=2)
    configure(d, 2, DISC_CASES[0])
    d.set_mesh(roid, X, C)
    nnzb = d.pattern_info()["nnz_blocks"]
    tu = torch.tensor(mesh.uniform(31, X.shape[0] * 3) * 2 - 1, dtype=torch.float64, device=cuda)
    J = torch.empty(nnzb * 9, dtype=torch.float64, device=cuda)
    d.assemble_jacobian(tu, J)
    rp, ci = d.pattern()
    q = int(rp[20] + np.nonzero(ci[rp[20]:rp[21]] == 20)[0][0])
    Jbad = J.clone()
    Jbad[q * 9:(q + 1) * 9] = 0
    r = torch.tensor(mesh.uniform(32, tu.numel()) - 0.5, dtype=torch.float64, device=cuda)
    z = torch.empty_like(r)
    assert _noalloc(d, Jbad, r, z) == _capi.ERR_BREAKDOWN
    assert "singular" in d.last_error()
    z_ref = torch.empty_like(r)
    d.block_jacobi(J, r, z_ref)
    assert _noalloc(d, J, r, z) == _capi.OK, d.last_error()
    torch.cuda.synchronize()
    assert rel_err(z.cpu().numpy(), z_ref.cpu().numpy()) <= TOL64

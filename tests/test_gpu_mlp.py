"""Tensor-core GEMM and the warm-start MLP on the GPU against the CPU oracle.

GEMM: BF16 operands, FP32 accumulation; compared with a float64 product of the
same BF16 values (relative tolerance 1e-5: only the summation order differs).
MLP forward / gradient: compared with oracle/mlp_oracle.py, which applies the
GPU path's BF16 roundings at the same places; the tolerance (2e-3 relative L2
per output, 1e-2 per gradient block) covers FP32 summation order and the rare
BF16 rounding flips that it causes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_pair(torch, cuda, M, N, K, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    return A.to(cuda), B.to(cuda), A.double(), B.double()


@pytest.mark.parametrize("M,N,K,splits", [(128, 256, 64, 1), (256, 64, 1024, 4), (384, 128, 192, 1), (256, 256, 4096, 8),
                                          (512, 512, 256, 1), (128, 64, 640, 3), (65536, 256, 256, 1)])
def test_gemm_bf16_matches_float64(cuda, M, N, K, splits):
    import torch

    from plugin_navierstokes_gb300.warm_start import gemm_bf16

    A, B, Ad, Bd = _bf16_pair(torch, cuda, M, N, K, M + N + K)
    C = gemm_bf16(A, B, splits=splits)
    torch.cuda.synchronize()
    got = C.double().sum(0).cpu()
    ref = Ad @ Bd.T
    err = (got - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err
    # every split is a partial over its own K chunk
    assert C.shape[0] >= 1


def _mlp_case(seed, P, slots):
    from oracle import mlp_oracle as mo

    rng = np.random.default_rng(seed)
    p = mo.init_params(seed, film_scale=0.3)
    xy = rng.uniform(0, 1, (P, 2)).astype(np.float32)
    sp = np.array(slots, np.int32)
    cond = rng.uniform(-1, 1, (len(slots) - 1, 2)).astype(np.float32)
    target = rng.uniform(-1, 1, (P, 3)).astype(np.float32)
    return p, xy, sp, cond, target


@pytest.mark.parametrize("P,slots", [(300, (0, 100, 300)), (128, (0, 128)), (1000, (0, 1, 500, 999, 1000))])
def test_mlp_forward_matches_oracle(cuda, P, slots):
    import torch

    from oracle import mlp_oracle as mo
    from plugin_navierstokes_gb300.warm_start import CoordinateMLP

    p, xy, sp, cond, _ = _mlp_case(P, P, slots)
    m = CoordinateMLP(max_points=1024, max_slots=8)
    m.set_params(p)
    out = torch.empty((P, 3), dtype=torch.float32, device=cuda)
    m.forward(torch.from_numpy(xy).to(cuda), sp, cond, out)
    torch.cuda.synchronize()
    ref, _ = mo.forward(p, xy, sp, cond, use_bf16=True)
    got = out.double().cpu().numpy()
    for c in range(3):
        e = np.linalg.norm(got[:, c] - ref[:, c]) / np.linalg.norm(ref[:, c])
        assert e < 2e-3, (c, e)


def test_mlp_gradient_matches_oracle(cuda):
    import torch

    from oracle import mlp_oracle as mo
    from plugin_navierstokes_gb300.warm_start import CoordinateMLP

    P = 700
    p, xy, sp, cond, target = _mlp_case(11, P, (0, 200, 450, 700))
    m = CoordinateMLP(max_points=1024, max_slots=8)
    m.set_params(p)
    grad = torch.empty(m.num_params, dtype=torch.float32, device=cuda)
    loss = m.loss_grad(torch.from_numpy(xy).to(cuda), sp, cond, torch.from_numpy(target).to(cuda), grad)
    torch.cuda.synchronize()
    lref, gref = mo.loss_grad(p, xy, sp, cond, target, use_bf16=True)
    assert abs(loss - lref) <= 1e-3 * lref
    g = grad.double().cpu().numpy()
    off, total = mo.offsets()
    assert g.size == total
    for key, (o, size) in off.items():
        r = gref[o:o + size]
        e = np.linalg.norm(g[o:o + size] - r) / max(np.linalg.norm(r), 1e-30)
        assert e < 1e-2, (key, e)
    # the parameters are not changed by a gradient evaluation
    assert np.array_equal(m.get_params(), p)


def _synthetic_dataset(torch, cuda, n_train=16, n=17):
    """Targets of a smooth conditioned field on an n x n node grid."""
    from oracle import mlp_oracle as mo

    x = np.linspace(0, 1, n)
    X, Y = np.meshgrid(x, x, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float32)
    rng = np.random.default_rng(5)
    re = np.exp(rng.uniform(np.log(10), np.log(1000), n_train))
    lid = rng.uniform(0.5, 2.0, n_train)
    cond = np.stack([mo.condition(r, l) for r, l in zip(re, lid)]).astype(np.float32)
    t = np.zeros((n_train, n * n, 3), np.float32)
    for k in range(n_train):
        a = cond[k, 0]
        t[k, :, 0] = np.sin(np.pi * X.ravel()) * np.sin(np.pi * Y.ravel()) * (1 + 0.3 * a)
        t[k, :, 1] = np.cos(np.pi * X.ravel()) * Y.ravel() * (1 - 0.2 * a)
        t[k, :, 2] = 0.1 * (X.ravel() - 0.5) * a
    return (torch.from_numpy(coords).to(cuda), torch.from_numpy(t).to(cuda), torch.from_numpy(cond).to(cuda))


def test_mlp_training_reduces_loss_and_is_deterministic(cuda):
    import torch

    from plugin_navierstokes_gb300.warm_start import CoordinateMLP

    coords, t, cond = _synthetic_dataset(torch, cuda)
    runs = []
    for _ in range(2):
        m = CoordinateMLP(max_points=4096, max_slots=16, seed=4)
        hist = m.train(coords, t, cond, steps=300, slots=8, points_per_slot=256, lr=2e-3, lr_final=1e-4, seed=9)
        runs.append((hist, m.get_params()))
    hist = runs[0][0]
    assert np.all(np.isfinite(hist))
    assert hist[-20:].mean() < 0.05 * hist[:5].mean(), (hist[:5], hist[-20:])
    assert np.array_equal(runs[0][1], runs[1][1])

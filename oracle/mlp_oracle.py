"""CPU restatement of the warm-start coordinate MLP (test infrastructure only).

Forward, loss and backward of the network of plugin_navierstokes_gb300's
nsfv1_mlp_* entry points, in float64 numpy, with the BF16 roundings of the GPU
path applied at the same places (GEMM operands: features, hidden activations,
weights, output and data gradients) when ``bf16=True``; with ``bf16=False`` it
is the exact float64 network, used to check this file's backward pass against
finite differences. The learned warm start has no counterpart in the reference
(it starts Newton from the caller's iterate), so this oracle is pinned by the
finite-difference check, not by reference vectors.

Parameter layout (float32 flat vector): per layer l = 0..3
[W_l (256 x in_l), b_l (256), Gw_l (256 x 2), Gb_l (256), Bw_l (256 x 2), Bb_l (256)],
then Wh (3 x 256), bh (3); in_0 = 64, in_l = 256 otherwise.
"""
from __future__ import annotations

import numpy as np

W, L, F, OUT = 256, 4, 16, 3


def layer_in(l: int) -> int:
    return 4 * F if l == 0 else W


def offsets():
    off, o = {}, 0
    for l in range(L):
        for name, size in (("W", W * layer_in(l)), ("b", W), ("Gw", 2 * W), ("Gb", W), ("Bw", 2 * W), ("Bb", W)):
            off[(name, l)] = (o, size)
            o += size
    off[("Wh", 0)] = (o, OUT * W)
    o += OUT * W
    off[("bh", 0)] = (o, OUT)
    o += OUT
    return off, o


def unpack(p: np.ndarray):
    off, _ = offsets()
    g = {}
    for (name, l), (o, size) in off.items():
        v = p[o:o + size].astype(np.float64)
        if name == "W":
            v = v.reshape(W, layer_in(l))
        elif name in ("Gw", "Bw"):
            v = v.reshape(W, 2)
        elif name == "Wh":
            v = v.reshape(OUT, W)
        g[(name, l)] = v
    return g


def pack(g) -> np.ndarray:
    off, total = offsets()
    p = np.zeros(total, np.float64)
    for key, (o, size) in off.items():
        p[o:o + size] = np.asarray(g[key]).ravel()
    return p


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even) via float32, returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def condition(re, lid):
    return np.array([(np.log(re) - np.log(100.0)) / np.log(10.0), (lid - 1.25) / 0.75], np.float32)


def features(xy: np.ndarray) -> np.ndarray:
    k = np.arange(1, F + 1, dtype=np.float64)
    ax = np.pi * xy[:, 0:1].astype(np.float64) * k
    ay = np.pi * xy[:, 1:2].astype(np.float64) * k
    f = np.stack([np.sin(ax), np.cos(ax), np.sin(ay), np.cos(ay)], axis=2)   # [P, F, 4]
    return f.reshape(xy.shape[0], 4 * F)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(p: np.ndarray, xy: np.ndarray, slot_ptr, cond: np.ndarray, use_bf16: bool = True):
    """Returns (out [P, 3], cache) for points xy [P, 2] in slots slot_ptr."""
    rnd = bf16 if use_bf16 else (lambda v: np.asarray(v, np.float64))
    g = unpack(p)
    P = xy.shape[0]
    slot = np.repeat(np.arange(len(slot_ptr) - 1), np.diff(slot_ptr))
    c = cond.astype(np.float64)[slot]                       # [P, 2]
    h = rnd(features(xy))
    cache = {"h": [h], "a": [], "gamma": [], "beta": [], "slot": slot, "c": c}
    for l in range(L):
        Wl = rnd(g[("W", l)])
        a = h @ Wl.T
        gam = 1.0 + c @ g[("Gw", l)].T + g[("Gb", l)]
        bet = c @ g[("Bw", l)].T + g[("Bb", l)]
        z = gam * (a + g[("b", l)]) + bet
        h = rnd(z * _sig(z))
        cache["a"].append(a)
        cache["gamma"].append(gam)
        cache["beta"].append(bet)
        cache["h"].append(h)
    out = h @ rnd(g[("Wh", 0)]).T + g[("bh", 0)]
    return out, cache


def loss_grad(p: np.ndarray, xy: np.ndarray, slot_ptr, cond: np.ndarray, target: np.ndarray, use_bf16: bool = True):
    """(loss, gradient flat float64) of the mean squared error over points and channels."""
    rnd = bf16 if use_bf16 else (lambda v: np.asarray(v, np.float64))
    g = unpack(p)
    out, cache = forward(p, xy, slot_ptr, cond, use_bf16)
    P = xy.shape[0]
    r = out - target.astype(np.float64)
    loss = float(np.sum(r * r) / (3.0 * P))
    dout = rnd(2.0 * r / (3.0 * P))
    gr = {k: np.zeros_like(v) for k, v in g.items()}
    gr[("bh", 0)] = (2.0 * r / (3.0 * P)).sum(axis=0)
    gr[("Wh", 0)] = dout.T @ cache["h"][L]
    dh = dout @ rnd(g[("Wh", 0)])
    nslot = len(slot_ptr) - 1
    slot, c = cache["slot"], cache["c"]
    cs = cond.astype(np.float64)
    for l in range(L - 1, -1, -1):
        a, gam, bet = cache["a"][l], cache["gamma"][l], cache["beta"][l]
        ab = a + g[("b", l)]
        z = gam * ab + bet
        s = _sig(z)
        dz = dh * s * (1.0 + z * (1.0 - s))
        da_exact = dz * gam
        da = rnd(da_exact)
        gr[("b", l)] = da_exact.sum(axis=0)
        dgam = np.zeros((nslot, W))
        dbet = np.zeros((nslot, W))
        np.add.at(dgam, slot, dz * ab)
        np.add.at(dbet, slot, dz)
        gr[("Gw", l)] = dgam.T @ cs
        gr[("Gb", l)] = dgam.sum(axis=0)
        gr[("Bw", l)] = dbet.T @ cs
        gr[("Bb", l)] = dbet.sum(axis=0)
        gr[("W", l)] = da.T @ cache["h"][l]
        dh = da @ rnd(g[("W", l)])
    return loss, pack(gr)


def init_params(seed: int = 0, film_scale: float = 0.0) -> np.ndarray:
    """A random parameter vector (numpy PRNG; for tests)."""
    rng = np.random.default_rng(seed)
    g = {}
    for l in range(L):
        b = np.sqrt(6.0 / layer_in(l))
        g[("W", l)] = rng.uniform(-b, b, (W, layer_in(l)))
        g[("b", l)] = rng.uniform(-0.1, 0.1, W)
        g[("Gw", l)] = rng.uniform(-film_scale, film_scale, (W, 2))
        g[("Gb", l)] = rng.uniform(-film_scale, film_scale, W)
        g[("Bw", l)] = rng.uniform(-film_scale, film_scale, (W, 2))
        g[("Bb", l)] = rng.uniform(-film_scale, film_scale, W)
    bh = np.sqrt(3.0 / W)
    g[("Wh", 0)] = rng.uniform(-bh, bh, (OUT, W))
    g[("bh", 0)] = rng.uniform(-0.1, 0.1, OUT)
    return pack(g).astype(np.float32)

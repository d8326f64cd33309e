"""Meshes, boundary rows and seeded states of the cavity workloads.

Node numbering is lexicographic (x fastest). Corner orders follow the ugcore
reference elements: quadrilateral (0,0),(1,0),(1,1),(0,1); hexahedron bottom
face counter-clockwise then top face; triangles counter-clockwise.
The PRNG is splitmix64 with 53-bit uniform doubles, so every input is
reproducible from its seed on any host.
"""
from __future__ import annotations

import numpy as np

from ._capi import HEXAHEDRON, PRISM, QUADRILATERAL, TETRAHEDRON, TRIANGLE

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n consecutive splitmix64 outputs of the stream seeded with ``seed``."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + _GOLDEN * (np.arange(1, n + 1, dtype=np.uint64))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int) -> np.ndarray:
    """n uniform doubles in [0, 1) from the top 53 bits of splitmix64."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def structured_quads(n: int, length: float = 1.0):
    """n x n quadrilaterals on [0, length]^2: (coords[(n+1)^2, 2], conn[n^2, 4])."""
    m = n + 1
    x = np.arange(m, dtype=np.float64) * (length / n)
    X, Y = np.meshgrid(x, x, indexing="xy")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    n0 = (j * m + i).ravel()
    conn = np.stack([n0, n0 + 1, n0 + m + 1, n0 + m], axis=1).astype(np.int32)
    return QUADRILATERAL, coords, conn


def structured_hexes(n: int, length: float = 1.0):
    """n^3 hexahedra on [0, length]^3: (coords[(n+1)^3, 3], conn[n^3, 8])."""
    m = n + 1
    x = np.arange(m, dtype=np.float64) * (length / n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    n0 = (k * m * m + j * m + i).ravel()
    s = m * m
    conn = np.stack([n0, n0 + 1, n0 + m + 1, n0 + m, n0 + s, n0 + s + 1, n0 + s + m + 1, n0 + s + m], axis=1).astype(np.int32)
    return HEXAHEDRON, coords, conn


def jittered_triangles(n: int, seed: int = 2, jitter: float = 0.2):
    """n x n grid on [0,1]^2 with every node moved by U[-jitter h, jitter h] per
    coordinate (boundary nodes only tangentially, corners fixed), each cell split
    along (0,2) when i+j is even and along (1,3) otherwise: 2 n^2 triangles."""
    m = n + 1
    h = 1.0 / n
    x = np.arange(m, dtype=np.float64) * h
    X, Y = np.meshgrid(x, x, indexing="xy")
    r = uniform(seed, 2 * m * m).reshape(m * m, 2)
    dx = (2.0 * r[:, 0] - 1.0) * jitter * h
    dy = (2.0 * r[:, 1] - 1.0) * jitter * h
    X = X.ravel().copy()
    Y = Y.ravel().copy()
    onx = (X == 0.0) | (X == 1.0)
    ony = (Y == 0.0) | (Y == 1.0)
    X = np.where(onx, X, X + dx)
    Y = np.where(ony, Y, Y + dy)
    coords = np.stack([X, Y], axis=1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    q0 = (j * m + i).ravel()
    q1, q2, q3 = q0 + 1, q0 + m + 1, q0 + m
    even = ((i + j).ravel() % 2) == 0
    t1 = np.where(even[:, None], np.stack([q0, q1, q2], 1), np.stack([q0, q1, q3], 1))
    t2 = np.where(even[:, None], np.stack([q0, q2, q3], 1), np.stack([q1, q2, q3], 1))
    conn = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int32)
    return TRIANGLE, coords, conn


def extruded_prisms(n: int, nz: int | None = None, seed: int = 2, jitter: float = 0.2):
    """The jittered n x n triangulation of [0,1]^2 (jittered_triangles) extruded to
    nz layers in z (nz = n by default): 2 n^2 nz prisms, corners (t0, t1, t2) of a
    layer's bottom then the same of its top (the reference prism's order)."""
    nz = n if nz is None else nz
    _, xy, tri = jittered_triangles(n, seed=seed, jitter=jitter)
    # counter-clockwise triangles (positive orientation of the bottom face seen from above)
    a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
    cw = ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])) < 0
    tri = np.where(cw[:, None], tri[:, [0, 2, 1]], tri)
    nn = xy.shape[0]
    z = np.arange(nz + 1, dtype=np.float64) / nz
    coords = np.concatenate([np.column_stack([xy, np.full(nn, zk)]) for zk in z])
    layers = [np.concatenate([tri + k * nn, tri + (k + 1) * nn], axis=1) for k in range(nz)]
    return PRISM, coords, np.concatenate(layers).astype(np.int32)


def cavity_dirichlet(coords: np.ndarray, lid: float = 1.0, tol: float = 1e-12):
    """Lid-driven cavity rows on [0,1]^dim: every boundary node has Dirichlet
    velocity; the lid (y = 1, excluding the nodes on the other walls) moves with
    u = lid, all other boundary velocities are 0; p is pinned to 0 at node 0.
    Returns (dofs = node * b + fct, values)."""
    n, dim = coords.shape
    b = dim + 1
    on = np.zeros(n, bool)
    for d in range(dim):
        on |= (np.abs(coords[:, d]) < tol) | (np.abs(coords[:, d] - 1.0) < tol)
    lidn = np.abs(coords[:, 1] - 1.0) < tol
    for d in range(dim):
        if d != 1:
            lidn &= (np.abs(coords[:, d]) > tol) & (np.abs(coords[:, d] - 1.0) > tol)
    nodes = np.nonzero(on)[0]
    dofs = (nodes[:, None] * b + np.arange(dim)[None, :]).ravel()
    vals = np.zeros((nodes.size, dim))
    vals[:, 0] = np.where(lidn[nodes], lid, 0.0)
    dofs = np.concatenate([dofs, [0 * b + dim]]).astype(np.int32)
    vals = np.concatenate([vals.ravel(), [0.0]])
    order = np.argsort(dofs, kind="stable")
    return dofs[order], vals[order]


def solenoidal_state(coords: np.ndarray, seed: int = 1, n_modes: int = 8, kmax: int = 4) -> np.ndarray:
    """Seeded 3D state [n, 4]: (u, v, w) = curl A with
    A_c = sum_k sin(2 pi m_ck . x + phi_ck) / (2 pi |m_ck|), m_ck in Z^3 with
    1 <= |m_ck|_inf <= kmax, phi ~ U[0, 2 pi) (divergence free, each term of
    amplitude <= 1), and p ~ U[-1, 1]."""
    n = coords.shape[0]
    r = uniform(seed, 3 * n_modes * 4 + n)
    m = np.floor(r[: 3 * n_modes * 3].reshape(3, n_modes, 3) * (2 * kmax + 1)).astype(np.int64) - kmax
    m[np.all(m == 0, axis=2)] = np.array([1, 0, 0])
    phi = r[3 * n_modes * 3: 3 * n_modes * 4].reshape(3, n_modes) * (2.0 * np.pi)
    p = 2.0 * r[3 * n_modes * 4:] - 1.0
    x = coords
    # grad A_c [n, 3]
    G = np.zeros((3, n, 3))
    for c in range(3):
        for k in range(n_modes):
            mk = m[c, k].astype(np.float64)
            arg = 2.0 * np.pi * (x @ mk) + phi[c, k]
            G[c] += np.cos(arg)[:, None] * (mk / np.linalg.norm(mk))[None, :]
    u = G[2][:, 1] - G[1][:, 2]
    v = G[0][:, 2] - G[2][:, 0]
    w = G[1][:, 0] - G[0][:, 1]
    return np.stack([u, v, w, p], axis=1)


CAVITY_SIZES = (32, 48, 64, 96, 128, 192, 256)


def draw_cavity_params(n_inst: int, seed: int = 3, sizes=CAVITY_SIZES, re_range=(10.0, 1000.0), lid_range=(0.5, 2.0)):
    """Seeded draws of the batched-cavity workload: mesh side N uniform over
    ``sizes``, Re log-uniform in ``re_range``, lid speed uniform in ``lid_range``;
    the viscosity of the unit cavity is nu = lid / Re."""
    r = uniform(seed, 3 * n_inst).reshape(n_inst, 3)
    N = np.array(sizes)[np.minimum((r[:, 0] * len(sizes)).astype(int), len(sizes) - 1)]
    Re = np.exp(np.log(re_range[0]) + r[:, 1] * (np.log(re_range[1]) - np.log(re_range[0])))
    lid = lid_range[0] + r[:, 2] * (lid_range[1] - lid_range[0])
    return N, Re, lid


def cavity_batch(sizes, Re, lid):
    """Independent lid-driven cavities (unit squares, quadrilaterals) as one mesh:
    returns dict(elem_type, coords, conn, node_offsets, nu_elem, dofs, values)."""
    coords, conns, offs, nus, dofs, vals = [], [], [0], [], [], []
    for N, re, u0 in zip(sizes, Re, lid):
        _, X, C = structured_quads(int(N))
        d, v = cavity_dirichlet(X, float(u0))
        base = offs[-1]
        coords.append(X)
        conns.append(C + base)
        dofs.append(d + base * 3)
        vals.append(v)
        nus.append(np.full(C.shape[0], float(u0) / float(re)))
        offs.append(base + X.shape[0])
    return {"elem_type": QUADRILATERAL, "coords": np.concatenate(coords), "conn": np.concatenate(conns).astype(np.int32),
            "node_offsets": np.array(offs, np.int32), "nu_elem": np.concatenate(nus),
            "dofs": np.concatenate(dofs).astype(np.int32), "values": np.concatenate(vals)}


# element sides in ugcore's reference order (corner ids of each side)
_SIDES = {
    TRIANGLE: [[0, 1], [1, 2], [2, 0]],
    QUADRILATERAL: [[0, 1], [1, 2], [2, 3], [3, 0]],
    TETRAHEDRON: [[0, 2, 1], [0, 1, 3], [1, 2, 3], [0, 3, 2]],
    HEXAHEDRON: [[0, 3, 2, 1], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [0, 4, 7, 3], [4, 5, 6, 7]],
}


def boundary_sides(elem_type: int, coords: np.ndarray, conn: np.ndarray, axis: int, value: float, tol: float = 1e-12) -> np.ndarray:
    """Node lists of the element sides that lie on the plane coords[:, axis] == value
    (corners in the element's side order), e.g. the inflow boundary of a channel
    for NavierStokesInflowFV1.add."""
    out = []
    on = np.abs(coords[:, axis] - value) <= tol
    for s in _SIDES[elem_type]:
        nodes = conn[:, s]
        hit = np.all(on[nodes], axis=1)
        out.append(nodes[hit])
    return np.concatenate(out).astype(np.int32) if out else np.zeros((0, len(_SIDES[elem_type][0])), np.int32)


def boundary_nodes(coords: np.ndarray, axis: int, value: float, tol: float = 1e-12) -> np.ndarray:
    """Ids of the nodes on the plane coords[:, axis] == value."""
    return np.nonzero(np.abs(coords[:, axis] - value) <= tol)[0].astype(np.int32)

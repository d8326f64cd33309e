"""Seeded element-level and mesh-level parity cases shared by the golden
fixture generator and the GPU parity tests."""
from __future__ import annotations

import numpy as np

from plugin_navierstokes_gb300.mesh import uniform

ROIDS = {"tri": 2, "quad": 3, "tet": 4, "prism": 6, "hex": 8}
NSH = {2: 3, 3: 4, 4: 4, 6: 6, 8: 8}
DIM = {2: 2, 3: 2, 4: 3, 6: 3, 8: 3}
REF = {
    2: np.array([[0, 0], [1, 0], [0, 1.0]]),
    3: np.array([[0, 0], [1, 0], [1, 1], [0, 1.0]]),
    4: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]),
    6: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1.0]]),
    8: np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1.0]]),
}

# (upwind, stabilisation, diff length, transient, exact jacobian, peclet, laplace, stokes, source)
DISC_CASES = [
    ("full", "fields", "raw", False, 0.0, False, False, False, False),
    ("lps", "flow", "raw", False, 0.0, False, False, False, False),
    ("no", "fields", "fivepoint", True, 1.0, False, False, False, True),
    ("skewed", "flow", "cor", False, 1.0, True, False, False, False),
    ("lps", "fields", "raw", True, 0.0, False, True, False, True),
    ("full", "without", "raw", False, 1.0, True, False, False, False),
    ("full", "flow", "raw", False, 0.0, False, False, True, False),
]

# the positive upwind (ip shapes: the non-diagonal FIELDS / FLOW branches)
POS_CASES = [
    ("pos", "fields", "raw", False, 0.0, False, False, False, False),
    ("pos", "flow", "raw", True, 1.0, False, False, False, True),
    ("pos", "fields", "cor", True, 1.0, True, False, False, False),
    ("pos", "flow", "fivepoint", False, 0.0, False, True, False, False),
    ("pos", "without", "raw", False, 1.0, False, False, False, False),
]


def random_elements(roid: int, n: int, seed: int, h: float = 0.1, jitter: float = 0.15, affine: bool = False) -> np.ndarray:
    """n distorted copies of the reference element scaled by h (corner jitter
    U[-jitter h, jitter h]; affine=True applies one random affine map instead)."""
    dim = DIM[roid]
    nsh = NSH[roid]
    r = uniform(seed, n * (nsh * dim + dim * dim + dim)).reshape(n, -1)
    out = np.empty((n, nsh, dim))
    for e in range(n):
        off = r[e, :dim] * 3.0
        if affine:
            A = np.eye(dim) + (r[e, dim:dim + dim * dim].reshape(dim, dim) - 0.5) * 0.4
            out[e] = off + h * REF[roid] @ A.T
        else:
            jit = (r[e, dim + dim * dim:dim + dim * dim + nsh * dim].reshape(nsh, dim) * 2 - 1) * jitter
            out[e] = off + h * (REF[roid] + jit)
    return out


def random_local_u(roid: int, n: int, seed: int, zero_frac: float = 0.0) -> np.ndarray:
    b = DIM[roid] + 1
    nsh = NSH[roid]
    u = uniform(seed, n * b * nsh).reshape(n, b * nsh) * 2 - 1
    if zero_frac > 0:
        u[: int(n * zero_frac), : DIM[roid] * nsh] = 0.0
    return u


def configure(disc, dim: int, cfg) -> None:
    """Apply a DISC_CASES entry to a disc (oracle or product: same method names)."""
    up, stab, dl, transient, exact, peclet, laplace, stokes, source = cfg
    disc.set_kinematic_viscosity(0.01 if dim == 2 else 0.0025)
    disc.set_density(1.0 if not source else 1.3)
    disc.set_upwind(up)
    disc.set_stabilization(stab, dl)
    disc.set_exact_jacobian(exact)
    disc.set_peclet_blend(peclet)
    disc.set_laplace(laplace)
    disc.set_stokes(stokes)
    if source:
        disc.set_source([0.3, -0.2, 0.1][:dim])


def ref_config(dim: int, cfg) -> dict:
    """The same DISC_CASES entry as a configuration of the reference library
    (oracle.ref_elem_batch); values as in configure()."""
    up, stab, dl, transient, exact, peclet, laplace, stokes, source = cfg
    return {"nu": 0.01 if dim == 2 else 0.0025, "rho": 1.0 if not source else 1.3, "full_newton": exact,
            "source": [0.3, -0.2, 0.1][:dim] if source else None, "stokes": stokes, "laplace": laplace, "peclet": peclet,
            "upwind": up, "stab": stab, "diff_length": dl}


def cfg_name(cfg) -> str:
    up, stab, dl, transient, exact, peclet, laplace, stokes, source = cfg
    return f"{up}-{stab}-{dl}" + ("-tr" if transient else "") + ("-ex" if exact else "") + ("-pe" if peclet else "") + \
        ("-lap" if laplace else "") + ("-stokes" if stokes else "") + ("-src" if source else "")


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| (norm-wise relative error used by the parity tests)."""
    den = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b))) / den if den > 0 else float(np.max(np.abs(a - b))) if a.size else 0.0

"""Post-processing of an FV1 solution (incompressible/navier_stokes_tools.h).

vorticity() and the point evaluation run on the GPU through the C ABI
(nsfv1_vorticity, nsfv1_eval_points). driven_cavity_lines_eval() is the
reference's DrivenCavityLinesEval / DrivenCavityEvalAtPoints
(navier_stokes_tools.h:540-729) for the unit lid-driven cavity: the first
velocity component on the vertical centre line x = 0.5 and the second on the
horizontal centre line y = 0.5, against tabulated values. The reference carries
its comparison tables (Ghia, Ghia & Shin 1982; Botella & Peyret 1998; Erturk et
al. 2005) in its source; here the caller passes the table to compare with.
"""
from __future__ import annotations

import numpy as np


def vorticity(disc, u, vort=None, stream=None):
    """vorticityFV1 (navier_stokes_tools.h:387-525): one value per node (device tensor)."""
    import torch

    if vort is None:
        vort = torch.empty(u.numel() // (disc.dim + 1), dtype=torch.float64, device=u.device)
    disc.vorticity(u, vort, stream)
    return vort


def eval_at_points(disc, u, points, fct: int) -> np.ndarray:
    """Function fct (0..dim) of the P1 solution at global points [n][dim] (host array in,
    host array out; NaN outside the mesh)."""
    import torch

    pts = torch.tensor(np.ascontiguousarray(points, np.float64), device=u.device)
    return disc.eval_points(u, pts, fct).cpu().numpy()


def driven_cavity_lines_eval(disc, u, vert_pos, vert_ref, horiz_pos, horiz_ref, vel_cmp=(0, 1)) -> dict:
    """u_x on x = 0.5 at the heights vert_pos against vert_ref, u_y on y = 0.5 at the
    abscissae horiz_pos against horiz_ref (DrivenCavityLinesEval, navier_stokes_tools.h:
    572-729). Returns per line the rows (position, measured, reference, |difference|)
    and the maximum and average difference, as DrivenCavityEvalAtPoints prints them."""
    out = {}
    for name, pos, ref, cmp, fixed_axis in (("vertical", vert_pos, vert_ref, vel_cmp[0], 0),
                                             ("horizontal", horiz_pos, horiz_ref, vel_cmp[1], 1)):
        pos = np.asarray(pos, np.float64)
        ref = np.asarray(ref, np.float64)
        pts = np.empty((pos.size, 2))
        pts[:, fixed_axis] = 0.5
        pts[:, 1 - fixed_axis] = pos
        val = eval_at_points(disc, u, pts, cmp)
        diff = np.abs(ref - val)
        out[name] = {"points": pts, "measured": val, "reference": ref, "difference": diff,
                     "max_diff": float(diff.max()), "avg_diff": float(diff.mean())}
    return out

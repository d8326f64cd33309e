"""GB300-native FV1 incompressible Navier-Stokes assembly + Newton path.

Drop-in for the NavierStokesFV1 element disc of UG4 plugin_NavierStokes: the
native library libnsfv1_gb300.so (hand-written sm_103a CUDA behind a C ABI,
include/nsfv1_gb300.h) does all compute; this package binds it and mirrors the
reference's NavierStokesFV1 interface.
"""
from . import _capi, mesh
from ._capi import NSFV1Error
from .navier_stokes_fv1 import (DataExport, NavierStokesFV1, NavierStokesInflowFV1, NavierStokesNoNormalStressOutflowFV1, NavierStokesWall,
                                mesh_pattern)

__all__ = ["DataExport", "NavierStokesFV1", "NavierStokesInflowFV1", "NavierStokesNoNormalStressOutflowFV1", "NavierStokesWall", "NSFV1Error",
           "mesh", "mesh_pattern", "_capi"]

"""GB300 (sm_103a) implementation of poroMec's per-time-step Biot hot path.

The product is the C-ABI library built from ``poromec_gb300/csrc`` (see
``include/poromec_gb300.h``); :mod:`poromec_gb300.capi` binds it and mirrors
the reference's element/solver call surface, :mod:`poromec_gb300.meshgen`
builds the seeded benchmark problems.
"""
from . import meshgen  # noqa: F401
from .capi import Mesh, PMError, StepInfo, from_problem, load, matvec_csrd_dev, reord  # noqa: F401

__all__ = ["Mesh", "PMError", "StepInfo", "from_problem", "load", "matvec_csrd_dev", "meshgen"]

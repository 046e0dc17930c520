"""GB300-native MicroFC hot path: the 5-equation diffuse-interface RHS and
TVD Runge-Kutta step as fused sm_103a CUDA kernels behind a C ABI.

Public API:

* :class:`Case`, :class:`Patch` -- case-file inputs (reference namelist keys)
* :mod:`microfc_gb300.cases` -- the benchmark cases
* :mod:`microfc_gb300.preprocess` -- grid and initial condition (pre_process)
* :class:`Simulation` -- device-resident solver (s_compute_rhs, s_*_tvd_rk, run)
* :mod:`microfc_gb300.io` -- the reference's data files (p_all/p<rank>/<t>/)
"""
from .case import Case, Patch  # noqa: F401
from .solver import Simulation  # noqa: F401
from . import cases, preprocess  # noqa: F401

__all__ = ["Case", "Patch", "Simulation", "cases", "preprocess"]

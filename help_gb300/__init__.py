"""help_gb300: GB300-native normal-equations backend for the HELP interior-point LP solver.

Public entry points:

* :class:`help_gb300.backend.GpuNormalEquations` -- the four boundary
  operations of the reference's PCG backend (LinearEquation_Construct,
  RenewLinearEquation, SolveLinearEquation, LinearEquation_Destruct) on one
  GB300, over the C ABI of ``libhelp_gpu.so`` (include/help_gpu.h);
* :func:`help_gb300.lp.make_lp` -- the seeded benchmark instances;
  :func:`help_gb300.lp.read_mps` / :func:`help_gb300.lp.read_bin` -- LPs
  from files;
* :func:`help_gb300.lp.remove_dependent_rows` -- the dependent-row presolve
  (the reference's Presolve_Lindep.cpp), with
  :func:`help_gb300.lp.expand_duals` to map duals back;
* :func:`help_gb300.hsd.solve_lp` -- the HSD interior-point driver over any
  backend (``presolve_lindep=True`` runs the presolve first).
"""
__all__ = ["backend", "lp", "hsd", "native", "build"]

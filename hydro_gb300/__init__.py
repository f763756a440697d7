"""GB300-native (sm_103a) implementation of hydro's time-step hot path.

Host side of the drop-in: ctypes bindings of the C-ABI in include/hydro_gpu.h
(``capi``), case builders (``cases``) and the Python mirror of the
reference's FluidSolver / AdvectionSolverMulti / hydro<Mesh>::step interface
(``solver``).  The compute path is libhydro_gpu.so (CUDA, built in-tree by
``build``).
"""
__version__ = "0.1.0"

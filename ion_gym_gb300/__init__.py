"""ion_gym_gb300 -- ion_gym's 3-D finite-difference Laplace field solve on
one NVIDIA GB300 (sm_103a).

Public modules:
  ion_gym_gb300.physics.solver3d     drop-in for ion_gym.physics.solver3d
  ion_gym_gb300.physics.multigrid3d  drop-in for ion_gym.physics.multigrid3d
  ion_gym_gb300.io.fa_cache          the basis-cache layout (store / load)

The compute path is libigsolve.so (C-ABI: include/igsolve.h), built in-tree
by ion_gym_gb300.build.build().
"""
__version__ = "0.1.0"

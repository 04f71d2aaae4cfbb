"""The field-solve modules: solver3d (SOR, basis loop, theta builders) and
multigrid3d (cascadic and V-cycle multigrid, the basis door, the stop flag),
drop-ins for ion_gym.physics.solver3d and ion_gym.physics.multigrid3d."""

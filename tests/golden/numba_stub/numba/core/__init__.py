"""Stub sub-package: ion_gym.physics imports numba.core.config."""

"""Stub of numba.core.config: only CACHE_DIR is read or written."""
CACHE_DIR = ""

"""Field-cache I/O in the reference layout."""

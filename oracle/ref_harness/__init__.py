"""Harness that runs the reference's own kernels on a GPU (test infrastructure)."""

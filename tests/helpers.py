"""Tolerances used by the parity tests (relative, per field)."""
# Parity bar for FP64 results against the oracle / the reference JAX.
TOL = 1e-10

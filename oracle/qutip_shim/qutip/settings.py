"""Tolerance used by Qobj equality and Hermiticity checks (QuTiP 4.7.2 default)."""
atol = 1e-12

"""Shared numerical tolerance of the XPBD kernels (xpbd_gpu/constants.py:3 of the reference)."""

EPSILON = 1e-12

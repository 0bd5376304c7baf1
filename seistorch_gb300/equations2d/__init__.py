"""Equation modules with seistorch's ``_time_step`` signatures
(seistorch/equations2d), backed by the native kernels."""

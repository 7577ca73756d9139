"""Test-only shim: NumPy 2 removed np.alltrue, which the reference tests use."""
import numpy as np

if not hasattr(np, "alltrue"):
    np.alltrue = np.all

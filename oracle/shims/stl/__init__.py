"""Placeholder for numpy-stl (oracle test infrastructure only)."""
from . import mesh  # noqa: F401

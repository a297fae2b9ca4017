"""Placeholder for matplotlib.animation (oracle test infrastructure only)."""

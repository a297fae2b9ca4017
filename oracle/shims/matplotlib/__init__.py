"""Placeholder for matplotlib (oracle test infrastructure only)."""

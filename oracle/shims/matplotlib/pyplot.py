"""Placeholder for matplotlib.pyplot (oracle test infrastructure only)."""


def __getattr__(name):
    raise RuntimeError("matplotlib is not available in this environment")

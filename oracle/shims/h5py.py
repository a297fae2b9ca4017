"""Placeholder for h5py (oracle test infrastructure only)."""


class File:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("h5py is not available in this environment")

"""Placeholder for numpy-stl's mesh module (oracle test infrastructure only)."""


class Mesh:
    @staticmethod
    def from_file(*args, **kwargs):
        raise RuntimeError("numpy-stl is not available in this environment")

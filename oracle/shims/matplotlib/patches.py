"""Placeholder for matplotlib.patches (oracle test infrastructure only)."""


class Ellipse:
    pass


class Polygon:
    pass

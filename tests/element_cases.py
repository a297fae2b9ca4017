"""Domains with every analytic element of pylbm (pylbm/elements/*.py).

``cases(ns)`` builds the dictionaries with the element classes of the
namespace ``ns``: the reference package (tests/golden/make_element_golden.py
records its Domain arrays) or pylbm_gb300.geometry (the tests build the same
domains on the host and on the device and compare).  Solid and fluid
elements, overlaps, tilted axes and several labels per element are covered.
"""


def cases(ns):
    return {
        "ellipse_triangle_d2q9": {
            "box": {"x": [0.0, 2.0], "y": [0.0, 1.0], "label": 0},
            "space_step": 1.0 / 40,
            "schemes": [{"velocities": list(range(9))}],
            "elements": [
                ns.Ellipse([0.53, 0.48], [0.25, 0.1], [-0.04, 0.1], label=1),
                ns.Triangle([1.1, 0.15], [0.5, 0.12], [0.15, 0.6], label=[2, 3, 4]),
                ns.Ellipse([1.32, 0.37], [0.06, 0.0], [0.0, 0.04], label=5, isfluid=True),
                ns.Triangle([0.2, 0.7], [0.3, 0.0], [0.0, 0.25], label=6),
            ],
        },
        "triangle_d2q13": {
            "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": [0, 1, 2, 3]},
            "space_step": 1.0 / 48,
            "schemes": [{"velocities": list(range(13))}],
            "elements": [
                ns.Triangle([0.31, 0.22], [0.41, 0.07], [-0.12, 0.5], label=[4, 5, 6]),
                ns.Ellipse([0.7, 0.7], [0.1, 0.1], [-0.05, 0.05], label=7),
            ],
        },
        "ellipsoid_cylinder_d3q19": {
            "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": 0},
            "space_step": 1.0 / 24,
            "schemes": [{"velocities": list(range(19))}],
            "elements": [
                ns.Ellipsoid([0.3, 0.35, 0.4], [0.15, 0.05, 0.0], [-0.02, 0.06, 0.0], [0.0, 0.0, 0.12], label=1),
                ns.CylinderCircle([0.68, 0.62, 0.5], [0.12, 0.0, 0.0], [0.0, 0.0, 0.12], [0.03, 0.2, 0.02],
                                  label=[2, 3, 4]),
            ],
        },
        "cylinders_d3q27": {
            "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": 0},
            "space_step": 1.0 / 20,
            "schemes": [{"velocities": list(range(27))}],
            "elements": [
                ns.CylinderEllipse([0.3, 0.3, 0.5], [0.15, 0.0, 0.0], [0.0, 0.08, 0.0], [0.02, 0.03, 0.3],
                                   label=[1, 2, 3]),
                ns.CylinderTriangle([0.55, 0.55, 0.2], [0.3, 0.05, 0.0], [0.02, 0.3, 0.0], [0.0, 0.0, 0.15],
                                    label=[4, 5, 6, 7, 8]),
                ns.Parallelepiped([0.12, 0.62, 0.55], [0.25, 0.0, 0.0], [0.05, 0.22, 0.0], [0.0, 0.04, 0.3],
                                  label=[9, 10, 11, 12, 13, 14]),
                # a fluid cavity carved out of the parallelepiped
                ns.Ellipsoid([0.27, 0.75, 0.7], [0.06, 0.0, 0.0], [0.0, 0.05, 0.0], [0.0, 0.0, 0.07], label=15,
                             isfluid=True),
            ],
        },
    }

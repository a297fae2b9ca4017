"""Fixture of pylbm's own Domain built with every analytic element.

Run in a container where the reference sources are available (read-only):

    PYTHONDONTWRITEBYTECODE=1 \
    PYTHONPATH=oracle/shims:$PYLBM_REFERENCE python tests/golden/make_element_golden.py

For each case of tests/element_cases.py the reference's Domain
(pylbm/domain.py:87-620 with the element classes of pylbm/elements/) is built
and its arrays are recorded: in_or_out (as "is fluid"), and every link whose
flag is not 999 (velocity index, node index, distance, flag).  The result is
elements.npz beside this script.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
sys.path.insert(0, TESTS)

import pylbm  # noqa: E402  (reference, through the shims)

import element_cases  # noqa: E402


def main():
    out = {}
    for name, dico in element_cases.cases(pylbm).items():
        dom = pylbm.Domain(dico)
        fluid = dom.in_or_out == dom.valin
        links = np.nonzero(dom.flag != dom.valin)
        flat = np.ravel_multi_index(links[1:], dom.flag.shape[1:])
        out[name + "/fluid"] = fluid
        out[name + "/u"] = links[0].astype(np.int16)
        out[name + "/node"] = flat.astype(np.int32)
        out[name + "/distance"] = dom.distance[links]
        out[name + "/flag"] = dom.flag[links].astype(np.int16)
        out[name + "/velocities"] = np.asarray([v.v for v in dom.stencil.unique_velocities])
        print(name, fluid.shape, "links", flat.size, "labels", np.unique(dom.flag[links]))
    np.savez_compressed(os.path.join(HERE, "elements.npz"), **out)


if __name__ == "__main__":
    main()

"""The routine names and parameter names of ``CudaModule`` against pylbm's.

pylbm binds every generated routine's arguments by the names
``inspect.getfullargspec`` returns (pylbm/symbolic.py:288-299).  The fixture
ref_signatures.json holds those names for the reference's own Cython modules
(tests/golden/make_signatures.py); the CUDA module must offer every routine
of the hot path under the same name with the same parameter names."""
import inspect
import json
import os

import pytest

import demo_cases
from conftest import GOLDEN
from pylbm_gb300 import workloads as W
from pylbm_gb300.generator import _routine, routine_signatures
from pylbm_gb300.scheme import Scheme

CASES = {
    "cavity_d2q9": lambda: W.cavity(n=32),
    "disc_flow_d2q9": lambda: W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0),
    "poiseuille_vec": lambda: demo_cases.poiseuille_vec(),
    "euler_1d": lambda: demo_cases.euler_1d(),
    "poiseuille_3d": lambda: demo_cases.poiseuille_3d(),
    "karman_geier": lambda: demo_cases.karman_vortex_street(dx=1.0 / 32),
    "tgv3d_d3q19": lambda: W.tgv3d(n=8),
    "advection_reaction_1d": lambda: demo_cases.advection_reaction_1d(),
}

with open(os.path.join(GOLDEN, "ref_signatures.json")) as fh:
    REF = json.load(fh)


@pytest.mark.parametrize("case", sorted(REF))
def test_routine_parameter_names_match_reference(case):
    ours = routine_signatures(Scheme(CASES[case]()))
    ref = REF[case]["routines"]
    assert set(ref) <= set(ours), set(ref) - set(ours)
    for name, args in ref.items():
        if name in ours:
            assert sorted(ours[name]) == sorted(args), (name, ours[name], args)


def test_routines_introspect_like_generated_functions():
    seen = []
    fn = _routine("bounce_back", ["f", "iload0", "istore", "ncond", "nx", "ny", "rhs"],
                  lambda **kw: seen.append(sorted(kw)))
    assert fn.__name__ == "bounce_back"
    args = inspect.getfullargspec(fn).args
    assert args == ["f", "iload0", "istore", "ncond", "nx", "ny", "rhs"]
    # call_genfunction: keep only the routine's names from a larger namespace
    namespace = {a: i for i, a in enumerate(args)}
    namespace.update(self=None, dim=2, fcopy=None)
    fn(**{k: namespace[k] for k in args})
    assert seen == [sorted(args)]
    with pytest.raises(TypeError):
        fn(f=1)


def test_update_routines_per_axis():
    sig = routine_signatures(Scheme(W.tgv3d(n=8)))
    assert [n for n in sorted(sig) if n.startswith("update_")] == ["update_x", "update_y", "update_z"]
    sig1 = routine_signatures(Scheme(demo_cases.euler_1d()))
    assert [n for n in sorted(sig1) if n.startswith("update_")] == ["update_x"]


def test_parameter_names_of_runtime_symbols():
    """A scheme with run-time parameters: the step takes all of them, the
    equilibrium those of m_eq, and 'lambda' is passed as 'lambda_'
    (pylbm/algorithm/base.py:656-662)."""
    import sympy as sp
    omega, lam = sp.symbols("omega, lambda")
    d = W.shear_layer(n=16, omega=omega)
    sig = routine_signatures(Scheme(d))
    assert "omega" in sig["one_time_step"] and "omega" in sig["relaxation"]
    assert "omega" not in sig["equilibrium"] and "omega" not in sig["f2m"]
    from pylbm_gb300.generator import _arg_name
    assert _arg_name(str(lam)) == "lambda_" and _arg_name("omega") == "omega"

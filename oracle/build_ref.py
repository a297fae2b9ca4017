"""Recipe: the reference's own generated kernels, as C, in oracle/_ref/.

TEST INFRASTRUCTURE ONLY (the CPU baseline of bench.py --impl reference).

pylbm has no hand-written kernels: for each scheme it generates a Cython
module (pylbm/generator/autowrap.py:52-136, printer
pylbm/generator/printing/cython.py) and builds it with setuptools.  This
script runs the reference pylbm (read-only sources, import shims from
oracle/shims) with ``codegen_option={'directory': oracle/_ref/<name>}`` so
that its generator writes ``wrapped_module_0.pyx`` and Cython translates it
to ``wrapped_module_0.c`` there.  The C file is plain CPython-extension C: on
a machine without Cython (the GPU host) ``compile_ref()`` builds it with gcc
against the Python headers, which is what setuptools would do.

Run here (where the reference sources and Cython exist):

    python oracle/build_ref.py

Outputs go only to oracle/_ref/ (git-ignored).
"""
import glob
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: $PYLBM_REFERENCE, else a "reference" folder beside this repository
REFERENCE_SOURCES = os.environ.get("PYLBM_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")

WORKLOADS = {
    # name: (workload builder, kwargs) -- the scheme decides the module; the
    # grid size is passed at call time
    "tgv3d": ("tgv3d", {"n": 8}),
    "cavity": ("cavity", {"n": 8}),
}


def generate():
    """Run the reference generator for every workload (needs the reference)."""
    sys.path.insert(0, os.path.join(HERE, "shims"))
    sys.path.insert(0, REFERENCE_SOURCES)
    sys.path.insert(0, ROOT)
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    import pylbm  # the reference
    from pylbm_gb300 import workloads as W

    for name, (fn, kw) in WORKLOADS.items():
        out = os.path.join(REF_DIR, name)
        os.makedirs(out, exist_ok=True)
        kwargs = dict(kw)
        if fn == "cavity":
            kwargs["bc"] = pylbm.bc
        dico = getattr(W, fn)(**kwargs)
        dico["generator"] = "cython"
        dico["codegen_option"] = {"directory": out, "generate": True}
        pylbm.Simulation(dico)
        print("generated", out, sorted(os.listdir(out)))


def module_dir(name):
    return os.path.join(REF_DIR, name)


def compile_ref(name, force=False):
    """Build oracle/_ref/<name>/wrapped_module_0.c for this machine; return the directory."""
    d = module_dir(name)
    src = os.path.join(d, "wrapped_module_0.c")
    if not os.path.exists(src):
        return None
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    out = os.path.join(d, "wrapped_module_0" + suffix)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return d
    inc = sysconfig.get_paths()["include"]
    # same optimisation level as the reference's setup (pylbm/generator/autowrap.py:93-136)
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-w", f"-I{inc}", "-o", out + ".tmp", src]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(out + ".tmp", out)
    # a module built elsewhere (other platform tag) must not shadow this one
    for other in glob.glob(os.path.join(d, "wrapped_module_0.cpython-*.so")):
        if other != out:
            os.unlink(other)
    return d


def load(name):
    """Import the reference's generated module for ``name`` (None if unavailable)."""
    d = compile_ref(name)
    if d is None:
        return None
    import importlib.util
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    spec = importlib.util.spec_from_file_location("wrapped_module_0", os.path.join(d, "wrapped_module_0" + suffix))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    generate()
    for n in WORKLOADS:
        print("compiled", compile_ref(n, force=True))

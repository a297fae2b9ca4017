"""ctypes binding of the C ABI (include/lbm_gb300.h) and the module builder.

``core()`` loads ``liblbm_gb300.so`` (device memory, halo, boundary kernels,
sums).  ``SchemeModule`` compiles the per-scheme translation unit produced by
``codegen.SchemeSource`` with nvcc for sm_103a into
``pylbm_gb300/_jit/lbm_scheme_<hash>.so`` and loads it, the way pylbm compiles
and imports one generated module per scheme (pylbm/generator/autowrap.py:52-136).
Every call checks the returned status and raises ``LbmError`` with the
library's message; there is no host fallback.
"""
import ctypes
import hashlib
import os
import shutil
import subprocess
import tempfile
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), "include")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
JIT_DIR = os.environ.get("PYLBM_GB300_JIT_DIR", os.path.join(PKG_DIR, "_jit"))
CORE_NAME = "liblbm_gb300.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

LBM_MAX_Q = 64
DTYPES = {"float64": 0, "float32": 1, "float16": 2, "bfloat16": 3}
DTYPE_SIZE = {"float64": 8, "float32": 4, "float16": 2, "bfloat16": 2}
H2D, D2H, D2D = 0, 1, 2


class LbmError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"[lbm status {code}] {msg}")
        self.code = code


class Lattice(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("nv", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("n", ctypes.c_int32 * 3),
        ("halo", ctypes.c_int32 * 3),
        ("stride", ctypes.c_int64 * 3),
        ("vstride", ctypes.c_int64),
        ("origin", ctypes.c_int64),
        ("elements", ctypes.c_int64),
        ("shift", ctypes.c_double * LBM_MAX_Q),
    ]


LBM_MAX_PRM = 8
LBM_INSTANCE_PAIRS = 1
LBM_ELEMENT_CIRCLE = 1
LBM_ELEMENT_PARALLELOGRAM = 2
LBM_ELEMENT_SPHERE = 3
LBM_ELEMENT_ELLIPSE = 4
LBM_ELEMENT_TRIANGLE = 5
LBM_ELEMENT_ELLIPSOID = 6
LBM_ELEMENT_CYLINDER = 7


class DomainDesc(ctypes.Structure):
    """lbm_domain (include/lbm_gb300.h)."""
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("nu", ctypes.c_int32),
        ("n", ctypes.c_int32 * 3),
        ("halo", ctypes.c_int32 * 3),
        ("vel", (ctypes.c_int32 * 3) * LBM_MAX_Q),
        ("dx", ctypes.c_double),
    ]


LBM_BC_KIND = {"bounce_back": 1, "anti_bounce_back": 2, "neumann": 3, "bouzidi_bounce_back": 4,
               "bouzidi_anti_bounce_back": 5, "ghost_copy": 6}
LBM_BC_FLOAT_FORM = 1
LBM_BC_FLAT = 2


class BcMethod(ctypes.Structure):
    """lbm_bc_method (include/lbm_gb300.h)."""
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("ncond", ctypes.c_int32),
        ("first", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("iload0", ctypes.c_void_p),
        ("iload1", ctypes.c_void_p),
        ("istore", ctypes.c_void_p),
        ("rhs", ctypes.c_void_p),
        ("dist", ctypes.c_void_p),
    ]


class ElementDesc(ctypes.Structure):
    """lbm_element (include/lbm_gb300.h)."""
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("isfluid", ctypes.c_int32),
        ("label", ctypes.c_int32 * 6),
        ("p", ctypes.c_double * 24),
        ("lo", ctypes.c_int32 * 3),
        ("hi", ctypes.c_int32 * 3),
        ("vq", (ctypes.c_double * 4) * LBM_MAX_Q),
    ]


class Instance(ctypes.Structure):
    """lbm_instance of include/lbm_gb300.h (one member of an ensemble)."""

    _fields_ = [
        ("offset", ctypes.c_int64 * 2),
        ("n", ctypes.c_int32 * 3),
        ("halo", ctypes.c_int32 * 3),
        ("stride", ctypes.c_int64 * 3),
        ("vstride", ctypes.c_int64),
        ("origin", ctypes.c_int64),
        ("rows", ctypes.c_int32),
        ("col_tiles", ctypes.c_int32),
        ("tile_begin", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("prm", ctypes.c_double * LBM_MAX_PRM),
    ]


def device_info():
    """(multiprocessor count, device name) of the current device."""
    sm = ctypes.c_int32()
    name = ctypes.create_string_buffer(256)
    check(core().lbm_device_info(ctypes.byref(sm), name, 256))
    return sm.value, name.value.decode()


def nvcc_path():
    for cand in (os.environ.get("NVCC"),
                 os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"),
                 shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise LbmError(-1, "nvcc not found (set CUDA_HOME or NVCC)")


def _nvcc_shared(sources, out, extra=()):
    """Compile CUDA sources into a shared library, atomically replacing ``out``."""
    os.makedirs(os.path.dirname(out), exist_ok=True)
    fd, tmp = tempfile.mkstemp(suffix=".so", dir=os.path.dirname(out))
    os.close(fd)
    cmd = [nvcc_path(), *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-o", tmp, *extra, *sources]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        os.unlink(tmp)
        raise LbmError(-1, "nvcc failed:\n" + " ".join(cmd) + "\n" + proc.stderr[-4000:])
    os.replace(tmp, out)
    return out


def build_core(force=False):
    out = os.path.join(LIB_DIR, CORE_NAME)
    srcs = [os.path.join(CSRC, "lbm_core.cu"), os.path.join(CSRC, "lbm_closure.cu"), os.path.join(CSRC, "lbm_domain.cu")]
    deps = srcs + [os.path.join(CSRC, f) for f in ("lbm_common.cuh", "lbm_mlp.cuh")] + \
        [os.path.join(INCLUDE, "lbm_gb300.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    return _nvcc_shared(srcs, out)


_core = None
_core_lock = threading.Lock()


def _sig(lib, name, res, args):
    fn = getattr(lib, name)
    fn.restype = res
    fn.argtypes = args
    return fn


def core():
    """The loaded liblbm_gb300.so (built on first use if missing)."""
    global _core
    with _core_lock:
        if _core is None:
            path = os.path.join(LIB_DIR, CORE_NAME)
            if not os.path.exists(path):
                build_core()
            lib = ctypes.CDLL(path)
            P, I32, I64, SZ = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
            LP = ctypes.POINTER(Lattice)
            _sig(lib, "lbm_version", ctypes.c_char_p, [])
            _sig(lib, "lbm_last_error", ctypes.c_char_p, [])
            _sig(lib, "lbm_lattice_init", I32, [LP, I32, I32, I32, P, P])
            _sig(lib, "lbm_device_count", I32, [ctypes.POINTER(I32)])
            _sig(lib, "lbm_set_device", I32, [I32])
            _sig(lib, "lbm_device_info", I32, [ctypes.POINTER(I32), ctypes.c_char_p, I32])
            _sig(lib, "lbm_device_synchronize", I32, [])
            _sig(lib, "lbm_alloc", I32, [ctypes.POINTER(P), SZ])
            _sig(lib, "lbm_free", I32, [P])
            _sig(lib, "lbm_memcpy", I32, [P, P, SZ, I32, P])
            _sig(lib, "lbm_memset", I32, [P, I32, SZ, P])
            _sig(lib, "lbm_stream_create", I32, [ctypes.POINTER(P)])
            _sig(lib, "lbm_stream_destroy", I32, [P])
            _sig(lib, "lbm_stream_synchronize", I32, [P])
            _sig(lib, "lbm_host_alloc", I32, [ctypes.POINTER(P), SZ])
            _sig(lib, "lbm_host_free", I32, [P])
            _sig(lib, "lbm_host_device_pointer", I32, [P, ctypes.POINTER(P)])
            _sig(lib, "lbm_event_create", I32, [ctypes.POINTER(P)])
            _sig(lib, "lbm_event_destroy", I32, [P])
            _sig(lib, "lbm_event_record", I32, [P, P])
            _sig(lib, "lbm_event_elapsed_ms", I32, [P, P, ctypes.POINTER(ctypes.c_float)])
            _sig(lib, "lbm_graph_begin", I32, [P])
            _sig(lib, "lbm_graph_end", I32, [P, ctypes.POINTER(P)])
            _sig(lib, "lbm_graph_launch", I32, [P, P])
            _sig(lib, "lbm_graph_destroy", I32, [P])
            _sig(lib, "lbm_update_halo", I32, [P, LP, P])
            _sig(lib, "lbm_update_halo_axis", I32, [P, LP, I32, P])
            _sig(lib, "lbm_gather", I32, [P, LP, I32, P, P, P, P, P])
            _sig(lib, "lbm_copy_planes", I32, [P, LP, I32, I32, I32, P, I32, P])
            _sig(lib, "lbm_fp64_fma_scratch_bytes", I32, [ctypes.POINTER(SZ)])
            _sig(lib, "lbm_fp64_fma_rate", I32, [P, I32, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.POINTER(ctypes.c_float), P])
            _sig(lib, "lbm_bounce_back", I32, [P, P, P, I32, P, LP, I32, P])
            _sig(lib, "lbm_anti_bounce_back", I32, [P, P, P, I32, P, LP, I32, P])
            _sig(lib, "lbm_neumann", I32, [P, P, P, I32, LP, I32, P])
            _sig(lib, "lbm_bouzidi_bounce_back", I32, [P, P, P, P, I32, P, P, LP, P, P])
            DP = ctypes.POINTER(DomainDesc)
            _sig(lib, "lbm_domain_reset", I32, [DP, P, P, P, P])
            _sig(lib, "lbm_domain_box", I32, [DP, P, P, P, P])
            _sig(lib, "lbm_domain_element", I32, [DP, ctypes.POINTER(ElementDesc), P, P, P, P, P])
            _sig(lib, "lbm_domain_clean", I32, [DP, P, P, P, P])
            _sig(lib, "lbm_links_block", I32, [])
            _sig(lib, "lbm_links_count", I32, [DP, P, I32, I32, P, P])
            _sig(lib, "lbm_links_fill", I32, [DP, P, P, I32, I32, P, P, P, P, P])
            _sig(lib, "lbm_boundary_batch", I32, [P, LP, P, I32, I32, P])
            _sig(lib, "lbm_bouzidi_anti_bounce_back", I32, [P, P, P, P, I32, P, P, LP, I32, P])
            _sig(lib, "lbm_population_sums_scratch_bytes", I32, [LP, ctypes.POINTER(SZ)])
            _sig(lib, "lbm_population_sums", I32, [P, LP, P, P, P, SZ, P])
            _sig(lib, "lbm_population_sums_noalloc", I32, [P, LP, P, P, P])
            _sig(lib, "lbm_restrict", I32, [P, LP, P, I32, P])
            _sig(lib, "lbm_population_sums_noalloc_max_bytes", SZ, [])
            F32 = ctypes.c_float
            _sig(lib, "lbm_mlp_sizes", I32, [ctypes.POINTER(I32), ctypes.POINTER(I32)])
            _sig(lib, "lbm_mlp_scratch_bytes", I32, [I32, ctypes.POINTER(SZ)])
            _sig(lib, "lbm_mlp_sync_weights", I32, [P, P, P])
            _sig(lib, "lbm_mlp_forward", I32, [P, I32, P, P, P, P])
            _sig(lib, "lbm_mlp_forward_tc", I32, [P, I32, P, P, P])
            _sig(lib, "lbm_mlp_tc_timeouts", I32, [ctypes.POINTER(ctypes.c_uint32)])
            _sig(lib, "lbm_mlp_gradients_tc", I32, [P, P, I32, P, P, P, P])
            _sig(lib, "lbm_mlp_vjp_tc", I32, [P, P, I32, P, P, P, P])
            _sig(lib, "lbm_mlp_gradients", I32, [P, P, I32, P, P, P, P, P, SZ, P])
            _sig(lib, "lbm_mlp_adam", I32, [P, P, P, P, F32, F32, F32, F32, I32, P, P])
            _core = lib
    return _core


def check(rc, lib=None, getter="lbm_last_error"):
    if rc != 0:
        lib = lib or core()
        msg = getattr(lib, getter)()
        raise LbmError(rc, msg.decode() if msg else "unknown error")


def lattice(dim, nv, dtype, n, halo, shift=None):
    lat = Lattice()
    n3 = (ctypes.c_int32 * 3)(*[int(x) for x in n] + [1] * (3 - len(n)))
    h3 = (ctypes.c_int32 * 3)(*[int(x) for x in halo] + [0] * (3 - len(halo)))
    check(core().lbm_lattice_init(ctypes.byref(lat), dim, nv, DTYPES[dtype], ctypes.cast(n3, ctypes.c_void_p),
                                  ctypes.cast(h3, ctypes.c_void_p)))
    if shift is not None:
        for k, v in enumerate(shift):
            lat.shift[k] = float(v)
    return lat


class DeviceBuffer:
    """Device allocation owned from Python (lbm_alloc / lbm_free)."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(core().lbm_alloc(ctypes.byref(p), self.nbytes))
        self.ptr = p.value

    def free(self):
        if getattr(self, "ptr", None):
            core().lbm_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return ctypes.c_void_p(self.ptr)

    def upload(self, array, stream=None, offset=0):
        a = np.ascontiguousarray(array)
        if a.nbytes + offset > self.nbytes:
            raise ValueError("upload larger than the buffer")
        check(core().lbm_memcpy(ctypes.c_void_p(self.ptr + offset), a.ctypes.data_as(ctypes.c_void_p), a.nbytes,
                                H2D, stream))
        check(core().lbm_stream_synchronize(stream))
        return a

    def download(self, out, stream=None, offset=0):
        if not out.flags["C_CONTIGUOUS"]:
            raise ValueError("download target must be C-contiguous")
        if out.nbytes + offset > self.nbytes:
            raise ValueError("download larger than the buffer")
        check(core().lbm_memcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr + offset),
                                out.nbytes, D2H, stream))
        check(core().lbm_stream_synchronize(stream))
        return out

    def zero(self, stream=None):
        check(core().lbm_memset(self.handle, 0, self.nbytes, stream))


class Event:
    """CUDA event (lbm_event_*) for device-side timing on a stream."""

    def __init__(self):
        p = ctypes.c_void_p()
        check(core().lbm_event_create(ctypes.byref(p)))
        self.ptr = p.value

    def record(self, stream=None):
        check(core().lbm_event_record(ctypes.c_void_p(self.ptr), stream))

    def elapsed_ms(self, end):
        ms = ctypes.c_float()
        check(core().lbm_event_elapsed_ms(ctypes.c_void_p(self.ptr), ctypes.c_void_p(end.ptr), ctypes.byref(ms)))
        return float(ms.value)

    def __del__(self):
        try:
            if self.ptr:
                core().lbm_event_destroy(ctypes.c_void_p(self.ptr))
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array."""

    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        check(core().lbm_host_alloc(ctypes.byref(p), int(nbytes)))
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def array(self, dtype, count=None):
        dtype = np.dtype(dtype)
        count = self.nbytes // dtype.itemsize if count is None else count
        buf = (ctypes.c_char * (count * dtype.itemsize)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype, count=count)

    def free(self):
        if self.ptr:
            core().lbm_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def mapped_device_pointer(array):
    """Device address of a C-contiguous numpy array in page-locked host memory
    (``pinned_empty``), or None: kernels can then read or write it directly
    over the host link instead of a staged copy."""
    if not isinstance(array, np.ndarray) or not array.flags["C_CONTIGUOUS"] or not isinstance(array, _PinnedArray):
        return None
    dev = ctypes.c_void_p()
    if core().lbm_host_device_pointer(ctypes.c_void_p(array.ctypes.data), ctypes.byref(dev)) != 0:
        return None
    return dev


def fp64_fma_rate(iters=4096, stream=None):
    """Measured FP64 FMA rate of the current device in flop/s (lbm_fp64_fma_rate)."""
    lib = core()
    size = ctypes.c_size_t()
    check(lib.lbm_fp64_fma_scratch_bytes(ctypes.byref(size)))
    scratch = DeviceBuffer(size.value)
    rate, ms = ctypes.c_double(), ctypes.c_float()
    check(lib.lbm_fp64_fma_rate(scratch.handle, int(iters), ctypes.byref(rate), ctypes.byref(ms), stream))
    scratch.free()
    return float(rate.value)


class _PinnedArray(np.ndarray):
    """numpy array over page-locked memory; keeps its PinnedBuffer alive."""


def pinned_empty(shape, dtype=np.float64):
    """Uninitialised numpy array in page-locked host memory.

    Host-device copies from or into such an array run at the link's full
    rate (pageable memory is staged through driver buffers); pass it to
    ``Simulation.m_halo[...] = array`` or ``Simulation.fields(out=array)``.
    """
    dtype = np.dtype(dtype)
    shape = tuple(int(n) for n in np.atleast_1d(shape))
    count = int(np.prod(shape))
    buf = PinnedBuffer(max(count * dtype.itemsize, 1))
    arr = buf.array(dtype, count).reshape(shape).view(_PinnedArray)
    arr._pinned = buf
    return arr


class SchemeModule:
    """Compiled per-scheme module (lbm_scheme_<hash>.so)."""

    _cache = {}
    _lock = threading.Lock()

    def __init__(self, source_obj, storage, compute):
        self.src = source_obj
        self.storage = storage
        self.compute = compute
        text = source_obj.module_source(storage, compute)
        deps = "".join(open(os.path.join(CSRC, f)).read()
                       for f in ("lbm_common.cuh", "lbm_mlp.cuh", "lbm_tc.cuh", "scheme_kernels.cuh"))
        deps += open(os.path.join(INCLUDE, "lbm_gb300.h")).read()
        flags = list(getattr(source_obj, "nvcc_flags", []))
        key = hashlib.sha256((text + deps + " ".join(ARCH_FLAGS + flags)).encode()).hexdigest()[:20]
        self.key = key
        self.path = os.path.join(JIT_DIR, f"lbm_scheme_{key}.so")
        with SchemeModule._lock:
            lib = SchemeModule._cache.get(key)
            if lib is None:
                if not os.path.exists(self.path):
                    os.makedirs(JIT_DIR, exist_ok=True)
                    cu = os.path.join(JIT_DIR, f"lbm_scheme_{key}.cu")
                    with open(cu + ".tmp", "w") as fh:
                        fh.write(text)
                    os.replace(cu + ".tmp", cu)
                    _nvcc_shared([cu], self.path, extra=flags)
                lib = ctypes.CDLL(self.path)
                self._bind(lib)
                SchemeModule._cache[key] = lib
        self.lib = lib
        nv, dim, nprm, st, cp = (ctypes.c_int32() for _ in range(5))
        shift = (ctypes.c_double * LBM_MAX_Q)()
        mref = (ctypes.c_double * LBM_MAX_Q)()
        self.call(lib.lbm_scheme_describe(ctypes.byref(nv), ctypes.byref(dim), ctypes.byref(nprm), ctypes.byref(st),
                                          ctypes.byref(cp), shift, mref))
        self.nv, self.dim, self.nprm = nv.value, dim.value, nprm.value
        self.shift = np.array(shift[:self.nv])
        self.mref = np.array(mref[:self.nv])

    @staticmethod
    def _bind(lib):
        P, I32 = ctypes.c_void_p, ctypes.c_int32
        LP = ctypes.POINTER(Lattice)
        _sig(lib, "lbm_scheme_last_error", ctypes.c_char_p, [])
        _sig(lib, "lbm_scheme_describe", I32, [P, P, P, P, P, P, P])
        _sig(lib, "lbm_one_time_step", I32, [P, P, LP, P, P])
        _sig(lib, "lbm_one_time_step_periodic", I32, [P, P, LP, P, P])
        _sig(lib, "lbm_one_time_step_walls", I32, [P, P, LP, P, P, P, P])
        _sig(lib, "lbm_transport", I32, [P, P, LP, P])
        _sig(lib, "lbm_f2m", I32, [P, LP, P, LP, P])
        _sig(lib, "lbm_f2m_conserved", I32, [P, LP, P, LP, P])
        _sig(lib, "lbm_m2f", I32, [P, LP, P, LP, P])
        _sig(lib, "lbm_equilibrium", I32, [P, LP, P, P])
        _sig(lib, "lbm_relaxation", I32, [P, LP, P, P])
        _sig(lib, "lbm_source_term", I32, [P, LP, P, P])
        _sig(lib, "lbm_init_conserved", I32, [P, LP, P, LP, P, P])
        _sig(lib, "lbm_f2m_conserved_dense", I32, [P, LP, P, P])
        _sig(lib, "lbm_scheme_set_step_variant", I32, [I32])
        _sig(lib, "lbm_scheme_wait_timeouts", I32, [ctypes.POINTER(ctypes.c_uint32)])
        _sig(lib, "lbm_scheme_set_closure_tc_occupancy", I32, [I32])
        _sig(lib, "lbm_scheme_closure_tc_occupancy", I32, [ctypes.POINTER(ctypes.c_int32)] * 2)
        _sig(lib, "lbm_ensemble_step", I32, [P, P, P, I32, I32, I32, I32, I32, P])
        _sig(lib, "lbm_ensemble_step_pairs", I32, [P, P, P, I32, I32, I32, I32, I32, P])
        _sig(lib, "lbm_one_time_step_periodic_closure", I32, [P, P, LP, P, P, P, P, P, P, P, I32, P])
        _sig(lib, "lbm_one_time_step_periodic_closure_tc", I32, [P, P, LP, P, P, P, P, P, P, P])

    def call(self, rc):
        check(rc, self.lib, "lbm_scheme_last_error")

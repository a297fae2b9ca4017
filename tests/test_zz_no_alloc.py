"""The allocation-free population sums against the allocating entry point.

``lbm_population_sums_noalloc`` serves callers that cannot call cudaMalloc
(an application whose memory manager owns all device memory, or a loop that
cannot take cudaMalloc's implicit synchronisation): its scratch is a fixed
device array inside liblbm_gb300.so.  This file is collected last, so a run
that stops at the first failure has already run every other test; it also
passes on its own in a fresh process (the first call sets the array up).
"""
import ctypes

import numpy as np
import pytest

from pylbm_gb300 import Simulation, runtime
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _read(buf, nv):
    host = np.empty(nv + 1, dtype=np.float64)
    buf.download(host)
    flag = int(np.frombuffer(host[nv:].tobytes()[:4], dtype=np.int32)[0])
    return host[:nv].copy(), flag


def test_noalloc_sums_match_allocating_sums_twice():
    core = runtime.core()
    sim = Simulation(W.shear_layer(n=96), dtype="float32")
    nv = sim.scheme.nv
    lat = ctypes.byref(sim._lat)
    size = ctypes.c_size_t()
    runtime.check(core.lbm_population_sums_scratch_bytes(lat, ctypes.byref(size)))
    assert size.value <= core.lbm_population_sums_noalloc_max_bytes()
    scratch = runtime.DeviceBuffer(size.value)
    out_ref = runtime.DeviceBuffer(8 * (nv + 1))
    out_na = runtime.DeviceBuffer(8 * (nv + 1))
    results = []
    for call in range(2):
        sim.run(5 + 10 * call)  # different contents for the second call
        sim.synchronize()
        runtime.check(core.lbm_population_sums(sim._F.handle, lat, out_ref.handle,
                                               ctypes.c_void_p(out_ref.ptr + 8 * nv), scratch.handle,
                                               size.value, sim._stream))
        runtime.check(core.lbm_population_sums_noalloc(sim._F.handle, lat, out_na.handle,
                                                       ctypes.c_void_p(out_na.ptr + 8 * nv), sim._stream))
        sim.synchronize()
        ref, ref_flag = _read(out_ref, nv)
        got, got_flag = _read(out_na, nv)
        assert got_flag == ref_flag == 0
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-12)
        results.append(got)
    assert not np.array_equal(results[0], results[1])


def test_noalloc_rejects_lattice_beyond_builtin_scratch():
    core = runtime.core()
    # 64 populations over 4096 row blocks need 2 MiB of partials, twice the built-in array
    lat = runtime.lattice(3, 64, "float32", [256, 256, 64], [1, 1, 1])
    size = ctypes.c_size_t()
    runtime.check(core.lbm_population_sums_scratch_bytes(ctypes.byref(lat), ctypes.byref(size)))
    assert size.value > core.lbm_population_sums_noalloc_max_bytes()
    dummy = runtime.DeviceBuffer(256)
    out = runtime.DeviceBuffer(8 * 65)
    rc = core.lbm_population_sums_noalloc(dummy.handle, ctypes.byref(lat), out.handle,
                                          ctypes.c_void_p(out.ptr + 8 * 64), None)
    assert rc == 1
    assert b"built-in scratch" in core.lbm_last_error()

"""generator='cuda' inside pylbm itself: the backend binding, applied at run time.

``install()`` adds the backend 'CUDA' to an imported pylbm package without
editing its files, so that pylbm's own ``Simulation(dico)`` with
``dico['generator'] = 'cuda'`` runs its time loop -- ``one_time_step``,
``boundary_condition``, ``Array.update``, the boundary methods'
``update``, ``m[...]`` / ``F[...]`` -- through this package's kernels, by
pylbm's own ``call_genfunction`` (pylbm/symbolic.py:288-299).  Each patch is
the change a pylbm maintainer would make at that place:

====================================  ==============================================
pylbm (reference)                     'CUDA' backend
====================================  ==============================================
storage.py:63-125 ``Array``           ``CudaArray``: the values live in a
                                      ``generator.DeviceArray`` ([nv, x, y, z]);
                                      the host mirror ``array_cpu`` is refreshed
                                      from the device when read and written back
                                      when assigned (what the LOOPY path does
                                      with pyopencl arrays)
container.py:94-106                   ``CudaContainer``: F, Fnew, m as
                                      ``CudaArray`` in structure-of-arrays order
simulation.py:165-171                 ``_get_container`` maps 'CUDA' to it
generator/generator.py:19-35          ``add_routine`` records the routine name
                                      (the CUDA module has every routine);
                                      ``compile`` loads ``generator.CudaModule``
                                      of the scheme
algorithm/base.py:91, scheme.py:136   the scheme's dictionary reaches the
                                      generator (what ``compile`` builds from)
boundary.py:378-397 ``move2gpu``      boundary lists uploaded with ``to_device``
validator.py:327-328                  'cuda' accepted as a generator
====================================  ==============================================

Populations are float64 (pylbm's dtype), computed in the reference
generator's printed forms where the scheme allows (the FP64 parity path).
"""
import numpy as np
import sympy as sp

from .generator import CudaModule, DeviceArray, to_device

BACKEND = "CUDA"


class CudaDevice:
    """What the backend places on the device: the scheme's module, the
    population/moment arrays and the boundary lists."""

    @staticmethod
    def module(dico):
        return CudaModule(dico, storage="float64")

    @staticmethod
    def array(nv, nspace, vmax):
        return DeviceArray(nv, nspace, vmax, "float64")

    @staticmethod
    def to_device(host):
        return to_device(host)


def install(pylbm=None, device=None):
    """Add the 'CUDA' backend to ``pylbm`` (the imported reference package,
    imported here when None); returns the package.  ``device`` supplies the
    module, arrays and list uploads (default ``CudaDevice``; a stand-in with
    the same three functions lets the binding run where no GPU is present).
    Installing twice replaces the device."""
    if pylbm is None:
        import pylbm
    dev = device or CudaDevice
    if getattr(pylbm, "_cuda_backend_installed", False):
        pylbm._cuda_backend_device[0] = dev
        return pylbm
    current = [dev]  # read at call time: a later install() swaps the device
    from pylbm import boundary as bd
    from pylbm import container as ct
    from pylbm import scheme as sc
    from pylbm import simulation as sm
    from pylbm import storage as st
    from pylbm.algorithm import base as ab
    from pylbm.generator import generator as gen

    Array = st.Array

    class CudaArray(Array):
        """pylbm's Array whose values live on the device."""

        def __init__(self, nv, gspace_size, vmax, sorder=None, mpi_topo=None, dtype=np.double,
                     gpu_support=False):
            self._device = None
            super().__init__(nv, gspace_size, vmax, sorder, mpi_topo, dtype, gpu_support=False)
            if list(self.index) != list(range(self.dim + 1)):
                raise ValueError("the CUDA backend stores arrays as [nv, x, y(, z)]")
            self.gpu_support = BACKEND
            self.array = self._device = current[0].array(nv, self.region_size, vmax)

        # the host mirror follows the device whenever pylbm reads it
        @property
        def swaparray(self):
            if self._device is not None:
                self.array_cpu[...] = self._device.get()
            return self._swap

        @swaparray.setter
        def swaparray(self, value):
            self._swap = value

        @property
        def nspace(self):
            return self._swap.shape[1:]

        @property
        def nv(self):
            return self._swap.shape[0]

        def __getitem__(self, key):
            sw = self.swaparray
            return sw[self.consm[key]] if isinstance(key, sp.Symbol) else sw[key]

        def __setitem__(self, key, values):
            sw = self.swaparray
            sw[self.consm[key] if isinstance(key, sp.Symbol) else key] = values
            self._device.set(self.array_cpu)

        def _in(self, key):
            sw = self.swaparray
            inner = tuple(slice(v, -v) for v in self.vmax)
            plane = sw[self.consm[key]] if isinstance(key, (sp.Symbol, sp.IndexedBase)) else sw[key]
            return plane[inner]

    def _array_new(cls, *args, **kwargs):
        if cls is Array and kwargs.get("gpu_support") == BACKEND:
            return object.__new__(CudaArray)
        return object.__new__(cls)

    Array.__new__ = staticmethod(_array_new)

    class CudaContainer(ct.BaseContainer):
        """Populations F, Fnew and moments m on the device, [nv, x, y(, z)]."""

        gpu_support = BACKEND

        def __init__(self, domain, scheme, sorder=None):
            super().__init__(domain, scheme, list(range(domain.dim + 1)), st.SOA)
            self.Fnew = Array(self.nv, self.nspace, self.vmax, self.sorder, self.mpi_topo,
                              gpu_support=self.gpu_support)
            self.Fnew.set_conserved_moments(scheme.consm)

        def move2gpu(self, array):
            # the kernels do not read the fluid/solid map
            return array

    orig_get_container = sm.Simulation._get_container

    def _get_container(self, sorder):
        if self.generator.backend == BACKEND:
            return CudaContainer(self.domain, self.scheme, sorder)
        return orig_get_container(self, sorder)

    sm.Simulation._get_container = _get_container

    orig_add_routine = gen.Generator.add_routine
    orig_compile = gen.Generator.compile

    def add_routine(self, name_expr, local_vars=None, settings={}):
        if self.backend == BACKEND:
            self.routines[name_expr[0]] = None
            return
        return orig_add_routine(self, name_expr, local_vars, settings)

    def compile(self):
        if self.backend == BACKEND:
            self.module = current[0].module(self.cuda_scheme_dico)
            return
        return orig_compile(self)

    gen.Generator.add_routine = add_routine
    gen.Generator.compile = compile

    orig_scheme_init = sc.Scheme.__init__

    def scheme_init(self, dico, *args, **kwargs):
        orig_scheme_init(self, dico, *args, **kwargs)
        self.dico = dico

    sc.Scheme.__init__ = scheme_init

    orig_algo_init = ab.BaseAlgorithm.__init__

    def algo_init(self, scheme, sorder, generator, settings=None):
        orig_algo_init(self, scheme, sorder, generator, settings)
        if generator.backend == BACKEND:
            generator.cuda_scheme_dico = scheme.dico

    ab.BaseAlgorithm.__init__ = algo_init

    orig_move2gpu = bd.BoundaryMethod.move2gpu

    def move2gpu(self):
        if self.generator.backend.upper() == BACKEND:
            up = current[0].to_device
            self.rhs = up(self.rhs)
            if hasattr(self, "s"):
                self.s = up(self.s)
            self.istore = up(self.istore)
            self.iload = [up(il) for il in self.iload]
            return
        return orig_move2gpu(self)

    bd.BoundaryMethod.move2gpu = move2gpu

    orig_validate = sm.validate

    def validate(dico, name):
        if str(dico.get("generator", "")).upper() == BACKEND:
            dico = dict(dico)
            dico["generator"] = "cython"  # the same schema with the new backend allowed
        return orig_validate(dico, name)

    sm.validate = validate
    pylbm._cuda_backend_installed = True
    pylbm._cuda_backend_device = current
    return pylbm

"""RIME v4 solver: dimension / array / property registry on one GPU.

Mirrors the reference's v4 ``RimeSolver`` (``montblanc/impl/rime/v4/RimeSolver.py``
on top of ``solvers/rime_solver.py`` and ``solvers/mb_cuda_solver.py``):

* dimensions carry (global size, local size, lower extent, upper extent);
* every v4 array is a device tensor attribute (``slvr.uvw`` ...), with
  generated ``transfer_<name>(ndarray)`` / ``retrieve_<name>()`` methods;
* every property is an attribute with a ``set_<name>`` setter;
* ``solve()`` runs the pipeline on the solver's stream.

Arrays are torch tensors (complex arrays as complex64/complex128, which are
interleaved in memory like the reference's float2/double2).  PyTorch only
owns the memory; every computation is a call into the CUDA library.
"""
import types

import numpy as np
import torch

from . import _cabi
from .config import ARRAYS, PROPERTIES, STAGE_SCRATCH, Options, gen_cfg
from .pipeline import Pipeline
from .src_types import sources_to_nr_vars


def nr_of_baselines(na, auto_correlations=False):
    """montblanc/util/__init__.py:42-50"""
    return na * (na + 1) // 2 if auto_correlations else na * (na - 1) // 2


class Dimension(object):
    __slots__ = ('name', 'global_size', 'local_size', 'lower_extent', 'upper_extent', 'description')

    def __init__(self, name, size, description=''):
        self.name = name
        self.global_size = self.local_size = self.upper_extent = int(size)
        self.lower_extent = 0
        self.description = description

    @property
    def extent_size(self):
        return self.upper_extent - self.lower_extent


def default_pipeline(cfg):
    from .nodes import RimeV4Fused
    return Pipeline([RimeV4Fused()])


def stage_pipeline(cfg=None):
    """The reference's four-node v4 pipeline (impl/rime/v4/RimeSolver.py:36-40)."""
    from .nodes import RimeBSqrt, RimeEBeam, RimeEKBSqrt, RimeSumCoherencies
    return Pipeline([RimeBSqrt(), RimeEBeam(), RimeEKBSqrt(), RimeSumCoherencies()])


class RimeSolver(object):
    def __init__(self, slvr_cfg):
        cfg = gen_cfg(**slvr_cfg)
        self._slvr_cfg = cfg
        if cfg[Options.DTYPE] == Options.DTYPE_FLOAT:
            self.ft, self.ct = np.float32, np.complex64
            self.tft, self.tct = torch.float32, torch.complex64
        else:
            self.ft, self.ct = np.float64, np.complex128
            self.tft, self.tct = torch.float64, torch.complex128
        self.device = torch.device(cfg.get(Options.DEVICE, 'cuda'))
        if self.device.type != 'cuda':
            raise ValueError('montblanc_gb300 solvers run on a CUDA device (got %s)' % self.device)
        if not torch.cuda.is_available():
            raise RuntimeError('montblanc_gb300 found no CUDA device')
        self._use_weight_vector = bool(cfg.get(Options.WEIGHT_VECTOR, False))
        self._vis_output = cfg.get(Options.VISIBILITY_OUTPUT, Options.VISIBILITY_OUTPUT_MODEL)
        self._autocor = bool(cfg.get(Options.AUTO_CORRELATIONS, False))
        self.rime_mode = cfg.get(Options.RIME_MODE, 'native')
        self._dims = {}
        self._arrays = {}
        self._properties = {}
        self.stream = None
        self.register_default_dimensions()
        self.register_dimension('beam_lw', cfg[Options.E_BEAM_WIDTH], 'E beam cube l width')
        self.register_dimension('beam_mh', cfg[Options.E_BEAM_HEIGHT], 'E beam cube m height')
        self.register_dimension('beam_nud', cfg[Options.E_BEAM_DEPTH], 'E beam cube nu depth')
        for name, _, default in PROPERTIES:
            self.register_property(name, default)
        self.create_arrays(cfg.get(Options.DATA_SOURCE, Options.DATA_SOURCE_DEFAULT))
        self.pipeline = cfg.get(Options.PIPELINE) or default_pipeline(cfg)

    # ---- dimensions -----------------------------------------------------
    def register_dimension(self, name, size, description=''):
        self._dims[name] = Dimension(name, size, description)

    def register_default_dimensions(self):
        """solvers/rime_solver.py:101-161"""
        cfg = self._slvr_cfg
        ntime, na, nchan, npol = cfg[Options.NTIME], cfg[Options.NA], cfg[Options.NCHAN], cfg[Options.NPOL]
        self.register_dimension('ntime', ntime, 'Timesteps')
        self.register_dimension('na', na, 'Antenna')
        self.register_dimension('nbands', cfg.get(Options.NBANDS, 1), 'Bands')
        self.register_dimension('nchan', nchan, 'Channels')
        self.register_dimension('npol', npol, 'Polarisations')
        nbl = cfg.get(Options.NBL, nr_of_baselines(na, self._autocor))
        self.register_dimension('nbl', nbl, 'Baselines')
        self.register_dimension('npolchan', nchan * npol, 'Polarised channels')
        self.register_dimension('nvis', ntime * nbl * nchan, 'Visibilities')
        nr = sources_to_nr_vars(cfg.get(Options.SOURCES) or {})
        self.register_dimension('nsrc', sum(nr.values()), 'Sources (total)')
        for var, n in nr.items():
            self.register_dimension(var, n, var)

    def dimensions(self):
        return self._dims

    def dim_local_size(self, *names):
        v = tuple(self._dims[n].local_size for n in names)
        return v[0] if len(v) == 1 else v

    def dim_global_size(self, *names):
        v = tuple(self._dims[n].global_size for n in names)
        return v[0] if len(v) == 1 else v

    def dim_extents(self, *names):
        v = tuple((self._dims[n].lower_extent, self._dims[n].upper_extent) for n in names)
        return v[0] if len(v) == 1 else v

    def update_dimension(self, name, **kw):
        d = self._dims[name]
        for k, val in kw.items():
            setattr(d, k, int(val))

    def mb_dims(self):
        d = _cabi.MbDims()
        for n in _cabi.DIM_NAMES:
            x = self._dims[n]
            setattr(d, n, _cabi.MbDim(x.global_size, x.local_size, x.lower_extent, x.upper_extent))
        return d

    # ---- properties -----------------------------------------------------
    def register_property(self, name, default):
        self._properties[name] = default
        setattr(self, name, float(default))
        setattr(self, 'set_' + name, types.MethodType(lambda s, v, n=name: setattr(s, n, float(v)), self))

    def properties(self):
        return dict((n, getattr(self, n)) for n in self._properties)

    def mb_props(self):
        return _cabi.make_props(**{n: getattr(self, n) for n in _cabi.PROP_NAMES})

    # ---- arrays ---------------------------------------------------------
    def _shape(self, sym):
        return tuple(self._dims[s].local_size if isinstance(s, str) else s for s in sym)

    def _torch_dtype(self, dt):
        return {'ft': self.tft, 'ct': self.tct, 'int32': torch.int32, 'uint8': torch.uint8}[dt]

    def _np_dtype(self, dt):
        return {'ft': self.ft, 'ct': self.ct, 'int32': np.int32, 'uint8': np.uint8}[dt]

    def create_arrays(self, data_source=Options.DATA_SOURCE_DEFAULT):
        for name, (sym, dt, default) in ARRAYS.items():
            if name in STAGE_SCRATCH:
                continue
            self.create_array(name, data_source)

    def create_array(self, name, data_source=Options.DATA_SOURCE_DEFAULT):
        sym, dt, default = ARRAYS[name]
        shape = self._shape(sym)
        host = np.zeros(shape, dtype=self._np_dtype(dt))
        if data_source == Options.DATA_SOURCE_TEST:
            from . import testdata
            testdata.fill(self, name, host)
        elif data_source != Options.DATA_SOURCE_EMPTY and default is not None and host.size:
            if callable(default):
                host[...] = default(self, host)
            else:
                host[...] = default
        t = torch.from_numpy(host).to(self.device)
        self._arrays[name] = t
        setattr(self, name, t)
        return t

    def ensure_array(self, name):
        if name not in self._arrays:
            self.create_array(name, Options.DATA_SOURCE_EMPTY)
        return self._arrays[name]

    def arrays(self):
        return dict(self._arrays)

    def transfer(self, name, npary):
        t = self._arrays[name]
        src = torch.as_tensor(np.ascontiguousarray(npary))
        if tuple(src.shape) != tuple(t.shape):
            raise ValueError("Supplied array '%s' shape %s does not match the expected shape %s"
                             % (name, tuple(src.shape), tuple(t.shape)))
        t.copy_(src.to(t.dtype))

    def retrieve(self, name):
        return self._arrays[name].cpu().numpy()

    def __getattr__(self, attr):
        # transfer_<name> / retrieve_<name>, as generated by mb_cuda_solver.py:67-124
        if attr.startswith('transfer_'):
            name = attr[len('transfer_'):]
            if name in ARRAYS:
                return lambda npary: (self.ensure_array(name), self.transfer(name, npary))[-1]
        elif attr.startswith('retrieve_'):
            name = attr[len('retrieve_'):]
            if name in ARRAYS:
                def retrieve():
                    self.ensure_array(name)
                    return self.retrieve(name)
                return retrieve
        raise AttributeError(attr)

    # ---- options --------------------------------------------------------
    def is_float(self):
        return self.ft == np.float32

    def is_double(self):
        return self.ft == np.float64

    def mb_dtype(self):
        return _cabi.MB_FLOAT32 if self.is_float() else _cabi.MB_FLOAT64

    def use_weight_vector(self):
        return self._use_weight_vector

    def outputs_residuals(self):
        return self._vis_output == Options.VISIBILITY_OUTPUT_RESIDUALS

    def outputs_model_visibilities(self):
        return self._vis_output == Options.VISIBILITY_OUTPUT_MODEL

    def is_autocorrelated(self):
        return self._autocor

    def mb_options(self):
        o = 0
        if self.use_weight_vector():
            o |= _cabi.MB_APPLY_WEIGHTS
        if self.outputs_residuals():
            o |= _cabi.MB_RESIDUALS
        return o

    def config(self):
        return self._slvr_cfg

    def default_base_ant_pairs(self):
        """solvers/rime_solver.py:92-99"""
        return np.triu_indices(self.dim_local_size('na'), 0 if self._autocor else 1)

    def default_ant_pairs(self):
        """impl/rime/v4/ant_pairs.py:23-37"""
        ntime, nbl = self.dim_local_size('ntime', 'nbl')
        a0, a1 = (a[:nbl] for a in self.default_base_ant_pairs())
        return np.tile(a0, ntime).reshape(ntime, nbl), np.tile(a1, ntime).reshape(ntime, nbl)

    # ---- execution ------------------------------------------------------
    def stream_handle(self, stream=None):
        s = stream if stream is not None else (self.stream or torch.cuda.current_stream(self.device))
        return ctypes_void_p(s.cuda_stream)

    def workspace(self, nbytes, key='fused'):
        """A cached device buffer of at least ``nbytes`` (256-byte aligned)."""
        cache = self.__dict__.setdefault('_workspaces', {})
        buf = cache.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)
            cache[key] = buf
        return buf

    def set_X2(self, value):
        self.X2 = float(value)

    def solve(self):
        ok = self.pipeline.execute(self, self.stream)
        if not ok and self.pipeline.last_error is not None:
            raise self.pipeline.last_error
        return ok

    def initialise(self):
        ok = self.pipeline.initialise(self, self.stream)
        if not ok and self.pipeline.last_error is not None:
            raise self.pipeline.last_error
        return ok

    def shutdown(self):
        return self.pipeline.shutdown(self, self.stream)

    def __enter__(self):
        self.initialise()
        return self

    def __exit__(self, etype, value, tb):
        self.shutdown()


def ctypes_void_p(x):
    import ctypes
    return ctypes.c_void_p(int(x))


def ptr(t):
    """Device address of a contiguous tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_contiguous():
        raise ValueError('arrays passed to the CUDA library must be contiguous')
    return t.data_ptr() if t.numel() else None

"""Load the reference's own v4 CPU solver behind minimal shims.

Used only by ``make_golden.py`` in a container where the reference checkout is
mounted.  The reference is Python 2 era code whose CPU path
(``montblanc/impl/rime/v4/cpu/CPUSolver.py``) still parses under Python 3,
but its imports need packages that are not installed here (``numexpr``,
``hypercube``, ``pycuda``).  This module provides stand-ins that hold no RIME
arithmetic:

* ``numexpr.evaluate`` evaluates the expression string with NumPy;
* ``montblanc`` / ``montblanc.util`` / ``montblanc.config`` /
  ``montblanc.solvers`` provide the constants, ``random_like``, the beam-cube
  option keys and a small dimension/array/property registry standing in for
  ``hypercube`` + ``MontblancNumpySolver``;
* the real ``impl/rime/v4/{config,ant_pairs}.py`` and ``cpu/CPUSolver.py``
  are loaded unmodified from the reference tree;
* ``ap_idx`` results are converted from lists to tuples, because NumPy 2
  rejects a list of index arrays as a fancy index.
"""
import importlib.util
import logging
import os
import sys
import types

import numpy as np

#: The reference checkout's ``montblanc`` package directory: the
#: MONTBLANC_REFERENCE environment variable names the checkout (default
#: /root/reference); ``set_reference_root`` overrides it before first use.
REF_ROOT = os.path.join(os.environ.get('MONTBLANC_REFERENCE', '/root/reference'), 'montblanc')


def set_reference_root(checkout):
    """Load the reference from the checkout at ``checkout`` (call before
    the first ``reference_solver``)."""
    global REF_ROOT
    if _CPUSolver is not None:
        raise RuntimeError('the reference CPUSolver is already loaded from %s' % REF_ROOT)
    REF_ROOT = os.path.join(checkout, 'montblanc')


def _numexpr_module():
    ne = types.ModuleType('numexpr')

    def evaluate(expr, local_dict=None, out=None, **_):
        ns = {'exp': np.exp, 'sqrt': np.sqrt, 'where': np.where,
              'sum': lambda x, axis=None: np.sum(x, axis=axis)}
        ns.update(local_dict or {})
        res = eval(expr, {'__builtins__': {}}, ns)
        if out is not None:
            out[...] = res
            return out
        return np.asarray(res)

    ne.evaluate = evaluate
    return ne


class _Constants:
    C = 299792458


class _Options:
    E_BEAM_WIDTH = 'beam_lw'
    E_BEAM_HEIGHT = 'beam_mh'
    E_BEAM_DEPTH = 'beam_nud'
    WEIGHT_VECTOR = 'weight_vector'
    VISIBILITY_OUTPUT = 'vis_output'


class _NumpySolver:
    """Dimension / array / property registry (the part of hypercube the CPU
    solver touches)."""

    def __init__(self, slvr_cfg):
        self._cfg = slvr_cfg
        self._dims = {}
        self.ft = np.float64
        self.ct = np.complex128

    # dimensions
    def register_dimension(self, name, size, **_):
        self._dims[name] = int(size)

    def register_default_dimensions(self):
        c = self._cfg
        na = c['na']
        self.register_dimension('ntime', c['ntime'])
        self.register_dimension('na', na)
        self.register_dimension('nchan', c['nchan'])
        self.register_dimension('npol', 4)
        self.register_dimension('nbl', c.get('nbl', na * (na - 1) // 2))
        self.register_dimension('npolchan', 4 * c['nchan'])
        srcs = c['sources']
        self.register_dimension('npsrc', srcs.get('point', 0))
        self.register_dimension('ngsrc', srcs.get('gaussian', 0))
        self.register_dimension('nssrc', srcs.get('sersic', 0))
        self.register_dimension('nsrc', sum(srcs.values()))

    def dim_local_size(self, *names):
        vals = tuple(self._dims[n] for n in names)
        return vals[0] if len(vals) == 1 else vals

    dim_global_size = dim_local_size

    # properties
    def register_properties(self, props):
        for p in props:
            setattr(self, p['name'], float(p['default']))
            setattr(self, 'set_' + p['name'],
                    (lambda n: (lambda v: setattr(self, n, float(v))))(p['name']))

    # arrays
    def register_arrays(self, arrays):
        self._arrays = arrays

    def create_arrays(self):
        tmap = {'ft': self.ft, 'ct': self.ct}
        for a in self._arrays:
            shape = tuple(self._dims[s] if isinstance(s, str) else s for s in a['shape'])
            dt = tmap.get(a['dtype'], a['dtype'])
            setattr(self, a['name'], np.zeros(shape, dtype=dt))

    def default_base_ant_pairs(self):
        return np.triu_indices(self._dims['na'], 1)

    def use_weight_vector(self):
        return bool(self._cfg.get('weight_vector', False))

    def outputs_residuals(self):
        return self._cfg.get('vis_output', 'model') == 'residuals'


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


_CPUSolver = None


def reference_cpu_solver_class():
    """Install the shims (once) and return the reference's CPUSolver class."""
    global _CPUSolver
    if _CPUSolver is not None:
        return _CPUSolver
    sys.modules['numexpr'] = _numexpr_module()
    mb = types.ModuleType('montblanc')
    mb.__path__ = []
    mb.constants = _Constants()
    mb.log = logging.getLogger('montblanc-ref')
    sys.modules['montblanc'] = mb
    util = types.ModuleType('montblanc.util')

    def random_like(ary=None, shape=None, dtype=None):
        if ary is not None:
            shape, dtype = ary.shape, ary.dtype
        if np.issubdtype(dtype, np.complexfloating):
            return (np.random.random(shape) + 1j * np.random.random(shape)).astype(dtype)
        return np.random.random(shape).astype(dtype)

    def rethrow_attribute_exception(e):
        raise e

    util.random_like = random_like
    util.rethrow_attribute_exception = rethrow_attribute_exception
    sys.modules['montblanc.util'] = util
    mb.util = util
    cfg = types.ModuleType('montblanc.config')
    cfg.RimeSolverConfig = _Options
    sys.modules['montblanc.config'] = cfg
    solvers = types.ModuleType('montblanc.solvers')
    solvers.MontblancNumpySolver = _NumpySolver
    sys.modules['montblanc.solvers'] = solvers
    for pkg in ('montblanc.impl', 'montblanc.impl.rime', 'montblanc.impl.rime.v4',
                'montblanc.impl.rime.v4.cpu'):
        m = types.ModuleType(pkg)
        m.__path__ = []
        sys.modules[pkg] = m
    _load('montblanc.impl.rime.v4.config', REF_ROOT + '/impl/rime/v4/config.py')
    _load('montblanc.impl.rime.v4.ant_pairs', REF_ROOT + '/impl/rime/v4/ant_pairs.py')
    mod = _load('montblanc.impl.rime.v4.cpu.CPUSolver',
                REF_ROOT + '/impl/rime/v4/cpu/CPUSolver.py')
    _CPUSolver = mod.CPUSolver
    return _CPUSolver


ARRAY_NAMES = ('uvw', 'antenna1', 'antenna2', 'frequency', 'ref_frequency',
               'parallactic_angles', 'point_errors', 'antenna_scaling', 'E_beam',
               'G_term', 'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape',
               'flag', 'weight_vector', 'observed_vis')
PROP_NAMES = ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm',
              'beam_lfreq', 'beam_ul', 'beam_um', 'beam_ufreq')


def reference_solver(P):
    """Build a reference CPUSolver holding the arrays of problem dict ``P``."""
    CPUSolver = reference_cpu_solver_class()
    ntime, na = P['uvw'].shape[:2]
    lw, mh, nud = P['E_beam'].shape[:3]
    cfg = {'ntime': ntime, 'na': na, 'nchan': P['frequency'].shape[0],
           'nbl': P['antenna1'].shape[1],
           'sources': {'point': P['npsrc'], 'gaussian': P['ngsrc'], 'sersic': P['nssrc']},
           'beam_lw': lw, 'beam_mh': mh, 'beam_nud': nud,
           'weight_vector': P['use_weight_vector'],
           'vis_output': 'residuals' if P['residuals'] else 'model'}
    slvr = CPUSolver(cfg)
    raw_ap_idx = slvr.ap_idx

    def ap_idx(*a, **k):
        i0, i1 = raw_ap_idx(*a, **k)
        return tuple(i0), tuple(i1)

    slvr.ap_idx = ap_idx
    for n in ARRAY_NAMES:
        getattr(slvr, n)[...] = P[n]
    for n in PROP_NAMES:
        getattr(slvr, 'set_' + n)(P[n])
    return slvr

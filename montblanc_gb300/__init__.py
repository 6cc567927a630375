"""montblanc_gb300: the RIME v4 chi^2 (+ gradient) hot path of Montblanc on
NVIDIA GB300 (sm_103a), behind the reference's Python entry points.

    import montblanc_gb300 as montblanc
    cfg = montblanc.rime_solver_cfg(na=14, ntime=10, nchan=16,
                                    sources=montblanc.sources(point=20, gaussian=10),
                                    dtype='double', data_source='default')
    with montblanc.rime_solver(cfg) as slvr:
        slvr.transfer_lm(lm) ...
        slvr.solve()
        print(slvr.X2)

The CUDA library (``libmbrime.so``, C ABI in include/montblanc_gb300.h) is
loaded on first use of a solver / problem; there is no CPU fallback.
"""
from . import src_types
from .config import Options, gen_cfg
from .node import Node, NullNode
from .pipeline import Pipeline, PipeLineError

__version__ = '0.1.0'


class _Constants(object):
    @property
    def C(self):
        """Speed of light in m/s (montblanc/__init__.py:52-59)."""
        return 299792458


constants = _Constants()


def source_types():
    return src_types.source_types()


def sources(**kwargs):
    """{type: count} for point / gaussian / sersic sources (montblanc/__init__.py:75-92)."""
    return src_types.default_sources(**kwargs)


def rime_solver_cfg(**kwargs):
    """Solver configuration dict (montblanc/__init__.py:96-126).  Unlike the
    reference the data source defaults to 'default': a MeasurementSet is read
    only when data_source='ms' and msfile are given."""
    cfg = gen_cfg(**kwargs)
    cfg.setdefault(Options.DATA_SOURCE, Options.DATA_SOURCE_DEFAULT)
    return cfg


def rime_solver(slvr_cfg):
    """Return a RIME solver for ``slvr_cfg`` (montblanc/factory.py:150-183):
    version 'v4' a device-resident ``RimeSolver``, version 'v5' the streaming
    ``CompositeRimeSolver`` over host arrays."""
    version = slvr_cfg.get(Options.VERSION, Options.DEFAULT_VERSION)
    if version not in (Options.VERSION_FOUR, Options.VERSION_FIVE):
        raise ValueError('Invalid version %s (this package implements the v4 path)' % version)
    if version == Options.VERSION_FIVE:
        from .composite import CompositeRimeSolver as cls
    else:
        from .solver import RimeSolver as cls
    if slvr_cfg.get(Options.DATA_SOURCE) == Options.DATA_SOURCE_MS:
        return rime_solver_from_ms(cls, slvr_cfg)
    return cls(slvr_cfg)


def rime_solver_from_ms(cls, slvr_cfg):
    """A solver of class ``cls`` sized by, and holding the arrays of, the
    MeasurementSet ``slvr_cfg['msfile']`` (montblanc/factory.py:113-148)."""
    from .ms import MeasurementSetLoader
    if Options.MS_FILE not in slvr_cfg:
        raise KeyError("%s is '%s' in the solver configuration, but no MeasurementSet is given in the %s key"
                       % (Options.DATA_SOURCE, Options.DATA_SOURCE_MS, Options.MS_FILE))
    cfg = dict(slvr_cfg)
    with MeasurementSetLoader(cfg[Options.MS_FILE], auto_correlations=cfg.get(Options.AUTO_CORRELATIONS,
                                                                              False)) as loader:
        ntime, nbl, na, nbands, nchan = loader.get_dims()
        cfg.update({Options.NTIME: ntime, Options.NA: na, Options.NBL: nbl, Options.NBANDS: nbands,
                    Options.NCHAN: nchan})
        slvr = cls(cfg)
        loader.load(slvr, cfg)
        return slvr


def __getattr__(name):
    # Lazily import the CUDA-backed pieces so that configuration helpers work
    # without loading the library.
    if name in ('RimeBSqrt', 'RimeEBeam', 'RimeEKBSqrt', 'RimeSumCoherencies', 'RimeReduction',
                'RimeV4Fused'):
        from . import nodes
        return getattr(nodes, name)
    if name in ('RimeSolver', 'stage_pipeline', 'default_pipeline'):
        from . import solver
        return getattr(solver, name)
    if name in ('RimeProblem', 'rime_chi2'):
        from . import rime
        return getattr(rime, name)
    raise AttributeError(name)

"""Solver configuration keys and the v4 array / property specification.

The option names, defaults and valid values are the reference's
(``montblanc/slvr_config.py:61-255``, ``montblanc/impl/rime/slvr_config.py:35-201``)
so that a configuration dict written for the reference configures this
solver the same way.  Only the keys that matter to the RIME v4 path, the
streaming (v5) driver and MeasurementSet input are interpreted; others are
accepted and ignored.

``ARRAYS`` and ``PROPERTIES`` restate the v4 array/property table of
``montblanc/impl/rime/v4/config.py:54-69, 131-247``: names, symbolic shapes,
dtypes ('ft' = float type, 'ct' = complex type) and default fills.
"""
import numpy as np

LIGHTSPEED = 299792458.0


class Options:
    # montblanc/slvr_config.py
    MODE = 'mode'
    SOURCES = 'sources'
    NTIME = 'ntime'
    NA = 'na'
    NBL = 'nbl'
    NCHAN = 'nchan'
    NBANDS = 'nbands'
    NPOL = 'npol'
    NSRC = 'nsrc'
    DTYPE = 'dtype'
    DTYPE_FLOAT = 'float'
    DTYPE_DOUBLE = 'double'
    AUTO_CORRELATIONS = 'auto_correlations'
    DATA_SOURCE = 'data_source'
    DATA_SOURCE_DEFAULT = 'default'
    DATA_SOURCE_MS = 'ms'
    DATA_SOURCE_TEST = 'test'
    DATA_SOURCE_EMPTY = 'empty'
    MS_FILE = 'msfile'
    CONTEXT = 'context'
    INIT_WEIGHTS = 'init_weights'
    INIT_WEIGHTS_NONE = None
    INIT_WEIGHTS_SIGMA = 'sigma'
    INIT_WEIGHTS_WEIGHT = 'weight'
    # montblanc/impl/rime/slvr_config.py
    E_BEAM_WIDTH = 'beam_lw'
    E_BEAM_HEIGHT = 'beam_mh'
    E_BEAM_DEPTH = 'beam_nud'
    WEIGHT_VECTOR = 'weight_vector'
    SOURCE_BATCH_SIZE = 'source_batch_size'
    NSOLVERS = 'nsolvers'
    VISIBILITY_OUTPUT = 'vis_output'
    VISIBILITY_OUTPUT_MODEL = 'model'
    VISIBILITY_OUTPUT_RESIDUALS = 'residuals'
    VISIBILITY_WRITE_MODE = 'vis_write_mode'
    VISIBILITY_WRITE_MODE_OVERWRITE = 'overwrite'
    VISIBILITY_WRITE_MODE_SUM = 'sum'
    VERSION = 'version'
    VERSION_FOUR = 'v4'
    VERSION_FIVE = 'v5'
    DEFAULT_VERSION = VERSION_FOUR
    # keys of this implementation
    RIME_MODE = 'rime_mode'          # 'native' | 'split_tf32' | 'split_bf16'
    DEVICE = 'device'                # torch device string, default 'cuda'
    PIPELINE = 'pipeline'


DEFAULTS = {
    Options.MODE: 'chi-squared',
    Options.NTIME: 10,
    Options.NA: 7,
    Options.NCHAN: 16,
    Options.NBANDS: 1,
    Options.NPOL: 4,
    Options.DTYPE: Options.DTYPE_DOUBLE,
    Options.AUTO_CORRELATIONS: False,
    Options.E_BEAM_WIDTH: 50,
    Options.E_BEAM_HEIGHT: 50,
    Options.E_BEAM_DEPTH: 50,
    Options.WEIGHT_VECTOR: False,
    Options.SOURCE_BATCH_SIZE: 500,
    Options.NSOLVERS: 2,
    Options.VISIBILITY_OUTPUT: Options.VISIBILITY_OUTPUT_MODEL,
    Options.VISIBILITY_WRITE_MODE: Options.VISIBILITY_WRITE_MODE_OVERWRITE,
    Options.VERSION: Options.VERSION_FOUR,
    Options.RIME_MODE: 'native',
    Options.DEVICE: 'cuda',
}

VALID = {
    Options.DTYPE: (Options.DTYPE_FLOAT, Options.DTYPE_DOUBLE),
    Options.WEIGHT_VECTOR: (True, False),
    Options.VISIBILITY_OUTPUT: (Options.VISIBILITY_OUTPUT_MODEL, Options.VISIBILITY_OUTPUT_RESIDUALS),
    Options.VISIBILITY_WRITE_MODE: (Options.VISIBILITY_WRITE_MODE_OVERWRITE, Options.VISIBILITY_WRITE_MODE_SUM),
    Options.VERSION: (Options.VERSION_FOUR, Options.VERSION_FIVE),
    Options.RIME_MODE: ('native', 'split_tf32', 'split_bf16'),
    Options.DATA_SOURCE: (Options.DATA_SOURCE_DEFAULT, Options.DATA_SOURCE_MS, Options.DATA_SOURCE_TEST,
                          Options.DATA_SOURCE_EMPTY),
    Options.INIT_WEIGHTS: (Options.INIT_WEIGHTS_NONE, Options.INIT_WEIGHTS_SIGMA, Options.INIT_WEIGHTS_WEIGHT),
}


class SolverConfiguration(dict):
    """A plain dict of solver options (the reference's gen_cfg result)."""


def gen_cfg(**kwargs):
    cfg = SolverConfiguration(DEFAULTS)
    cfg.update(kwargs)
    for k, valid in VALID.items():
        if k in cfg and cfg[k] not in valid:
            raise ValueError("Option '%s' = %r is not one of %r" % (k, cfg[k], valid))
    return cfg


FWHM2INT = 1.0 / np.sqrt(np.log(256.0))

#: (name, dtype, default) -- montblanc/impl/rime/v4/config.py:54-69
PROPERTIES = (
    ('gauss_scale', 'ft', FWHM2INT * np.sqrt(2.0) * np.pi / LIGHTSPEED),
    ('two_pi_over_c', 'ft', 2.0 * np.pi / LIGHTSPEED),
    ('sigma_sqrd', 'ft', 1.0),
    ('X2', 'ft', 0.0),
    ('beam_ll', 'ft', -0.5),
    ('beam_lm', 'ft', -0.5),
    ('beam_lfreq', 'ft', 1.3e9),
    ('beam_ul', 'ft', 0.5),
    ('beam_um', 'ft', 0.5),
    ('beam_ufreq', 'ft', 1.5e9),
)


def _default_ant1(slvr, ary):
    return slvr.default_ant_pairs()[0]


def _default_ant2(slvr, ary):
    return slvr.default_ant_pairs()[1]


def _linspace_freq(slvr, ary):
    return np.linspace(1e9, 2e9, ary.shape[0])


#: name -> (symbolic shape, dtype, default).  Scratch / output arrays have
#: default None (zero-filled).  montblanc/impl/rime/v4/config.py:131-247
ARRAYS = {
    'uvw': (('ntime', 'na', 3), 'ft', 0.0),
    'antenna1': (('ntime', 'nbl'), 'int32', _default_ant1),
    'antenna2': (('ntime', 'nbl'), 'int32', _default_ant2),
    'frequency': (('nchan',), 'ft', _linspace_freq),
    'ref_frequency': (('nchan',), 'ft', 1.4e9),
    'parallactic_angles': (('ntime', 'na'), 'ft', 0.0),
    'point_errors': (('ntime', 'na', 'nchan', 2), 'ft', 0.0),
    'antenna_scaling': (('na', 'nchan', 2), 'ft', 1.0),
    'E_beam': (('beam_lw', 'beam_mh', 'beam_nud', 4), 'ct', np.array([1, 0, 0, 1])),
    'G_term': (('ntime', 'na', 'nchan', 4), 'ct', np.array([1, 0, 0, 1])),
    'lm': (('nsrc', 2), 'ft', 0.0),
    'stokes': (('nsrc', 'ntime', 4), 'ft', np.array([1, 0, 0, 0])),
    'alpha': (('nsrc', 'ntime'), 'ft', 0.8),
    'gauss_shape': ((3, 'ngsrc'), 'ft', np.array([0, 0, 1])[:, None]),
    'sersic_shape': ((3, 'nssrc'), 'ft', np.array([0, 0, 0])[:, None]),
    'flag': (('ntime', 'nbl', 'nchan', 4), 'uint8', 0),
    'weight_vector': (('ntime', 'nbl', 'nchan', 4), 'ft', 1.0),
    'observed_vis': (('ntime', 'nbl', 'nchan', 4), 'ct', 0.0),
    # scratch and outputs
    'B_sqrt': (('nsrc', 'ntime', 'nchan', 4), 'ct', None),
    'jones': (('nsrc', 'ntime', 'na', 'nchan', 4), 'ct', None),
    'model_vis': (('ntime', 'nbl', 'nchan', 4), 'ct', None),
    'chi_sqrd_result': (('ntime', 'nbl', 'nchan'), 'ft', None),
}

#: Arrays only the per-stage pipeline needs (allocated on demand).
STAGE_SCRATCH = ('B_sqrt', 'jones')

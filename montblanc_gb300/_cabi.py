"""ctypes binding of the C ABI declared in include/montblanc_gb300.h.

The library is loaded from the package directory (``libmbrime.so``), built
with nvcc on first use if it is missing or stale.  There is no fallback: if
the library cannot be built or loaded, importing this module raises.
"""
import ctypes
import os

from . import _build


class MontblancError(RuntimeError):
    """Raised when an entry point returns a status other than MB_OK."""

    def __init__(self, status, name, message):
        self.status = status
        super().__init__('%s failed with %s: %s' % (name, STATUS_NAMES.get(status, status), message))


MB_OK = 0
STATUS_NAMES = {0: 'MB_OK', 1: 'MB_ERR_NULL_PTR', 2: 'MB_ERR_BAD_SHAPE', 3: 'MB_ERR_BAD_EXTENT',
                4: 'MB_ERR_UNSUPPORTED_DTYPE', 5: 'MB_ERR_CUDA', 6: 'MB_ERR_TIMEOUT',
                7: 'MB_ERR_WORKSPACE', 8: 'MB_ERR_INVALID_ARG', 9: 'MB_ERR_UNSUPPORTED'}

MB_FLOAT32, MB_FLOAT64 = 0, 1
MB_MODE_NATIVE, MB_MODE_SPLIT_TF32, MB_MODE_SPLIT_BF16 = 0, 1, 2
MODES = {'native': MB_MODE_NATIVE, 'split_tf32': MB_MODE_SPLIT_TF32, 'split_bf16': MB_MODE_SPLIT_BF16}
MB_APPLY_WEIGHTS = 0x1
MB_RESIDUALS = 0x2
MB_SOURCE_TILE_SHIFT = 8
MB_SOURCE_TILE_MASK = 0x3 << MB_SOURCE_TILE_SHIFT
SOURCE_TILES = {0: 0, 8: 0x1 << MB_SOURCE_TILE_SHIFT, 16: 0x2 << MB_SOURCE_TILE_SHIFT,
                32: 0x3 << MB_SOURCE_TILE_SHIFT}


def source_tile_bits(tile):
    """Option bits asking the CUDA-core kernels for ``tile`` sources per
    shared-memory tile (0: the library's default)."""
    if tile not in SOURCE_TILES:
        raise ValueError('source tile %r is not one of %s' % (tile, sorted(SOURCE_TILES)))
    return SOURCE_TILES[tile]
MB_TC_SELFTEST_A_IN_TMEM = 0x10

DIM_NAMES = ('ntime', 'na', 'nbl', 'nchan', 'npol', 'npolchan', 'nsrc', 'npsrc', 'ngsrc', 'nssrc',
             'beam_lw', 'beam_mh', 'beam_nud')
PROP_NAMES = ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm', 'beam_lfreq',
              'beam_ul', 'beam_um', 'beam_ufreq')
INPUT_NAMES = ('uvw', 'antenna1', 'antenna2', 'frequency', 'ref_frequency', 'parallactic_angles',
               'point_errors', 'antenna_scaling', 'E_beam', 'G_term', 'lm', 'stokes', 'alpha',
               'gauss_shape', 'sersic_shape', 'flag', 'weight_vector', 'observed_vis')
GRAD_NAMES = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term')


class MbDim(ctypes.Structure):
    _fields_ = [('global_size', ctypes.c_uint32), ('local_size', ctypes.c_uint32),
                ('lower_extent', ctypes.c_uint32), ('upper_extent', ctypes.c_uint32)]


class MbDims(ctypes.Structure):
    _fields_ = [(n, MbDim) for n in DIM_NAMES]


class MbProps(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in PROP_NAMES]


class MbRimeInputs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in INPUT_NAMES]


class MbRimeGrads(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in GRAD_NAMES]


class MbBatchSet(ctypes.Structure):
    _fields_ = [('npsrc', ctypes.c_uint32), ('ngsrc', ctypes.c_uint32), ('nssrc', ctypes.c_uint32),
                ('mode', ctypes.c_uint32), ('options', ctypes.c_uint32), ('reserved', ctypes.c_uint32),
                ('lm', ctypes.c_void_p), ('stokes', ctypes.c_void_p), ('alpha', ctypes.c_void_p),
                ('gauss_shape', ctypes.c_void_p), ('sersic_shape', ctypes.c_void_p), ('grads', MbRimeGrads)]


# (name, restype, argtypes) of every exported function.
_vp, _sz, _u32, _i32, _dbl = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int, ctypes.c_double
_pdims, _pprops = ctypes.POINTER(MbDims), ctypes.POINTER(MbProps)
SIGNATURES = {
    'mb_version': (ctypes.c_char_p, []),
    'mb_last_error_string': (ctypes.c_char_p, []),
    'mb_status_string': (ctypes.c_char_p, [_i32]),
    'mb_bsqrt': (_i32, [_i32, _pdims, _vp, _vp, _vp, _vp, _vp, _vp]),
    'mb_ebeam': (_i32, [_i32, _pdims, _pprops, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'mb_ekb_sqrt': (_i32, [_i32, _pdims, _pprops, _vp, _vp, _vp, _vp, _vp, _vp]),
    'mb_sum_coherencies': (_i32, [_i32, _pdims, _pprops, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                  _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'mb_reduce_chi2_workspace_size': (_sz, [_pdims]),
    'mb_reduce_chi2': (_i32, [_i32, _pdims, _vp, _dbl, _vp, _vp, _sz, _vp]),
    'mb_rime_workspace_size': (_sz, [_i32, _i32, _pdims, _i32]),
    'mb_rime_forward': (_i32, [_i32, _i32, _pdims, _pprops, _u32, ctypes.POINTER(MbRimeInputs), _vp,
                               _vp, _vp, _i32, _vp, _sz, _vp]),
    'mb_rime_adjoint': (_i32, [_i32, _i32, _pdims, _pprops, _u32, ctypes.POINTER(MbRimeInputs), _dbl,
                               ctypes.POINTER(MbRimeGrads), _vp, _sz, _vp]),
    'mb_rime_status': (_i32, [_i32, _i32, _pdims, _i32, _vp, _sz, _vp]),
    'mb_rime_batch_workspace_size': (_sz, [_i32, _pdims, ctypes.POINTER(MbBatchSet), _i32]),
    'mb_rime_batch_prepare': (_i32, [_i32, _pdims, ctypes.POINTER(MbBatchSet), _i32, _vp, _sz, _vp]),
    'mb_rime_batch': (_i32, [_i32, _pdims, _pprops, _u32, ctypes.POINTER(MbRimeInputs),
                             ctypes.POINTER(MbBatchSet), _i32, _vp, _dbl, _vp, _sz, _vp]),
    'mb_set_wait_limit': (_i32, [_u32]),
    'mb_default_wait_limit': (_u32, []),
    'mb_tc_selftest': (_i32, [_vp, _vp, _i32, _i32, _vp, _vp, _vp]),
    'mb_wait_selftest': (_i32, [_u32, _vp, _vp]),
    'mb_rime_noalloc_max_units': (_sz, []),
    'mb_rime_forward_noalloc': (_i32, [_i32, _pdims, _pprops, _u32, ctypes.POINTER(MbRimeInputs), _vp, _vp,
                                       _vp, _vp]),
    'mb_kernel_launches': (ctypes.c_uint64, []),
    'mb_kernel_timing': (_i32, [_i32]),
    'mb_kernel_time': (_i32, [ctypes.c_char_p, ctypes.POINTER(_dbl), ctypes.POINTER(ctypes.c_int64)]),
    'mb_kernel_timing_reset': (_i32, []),
    'mb_kernel_timing_name': (ctypes.c_char_p, [_i32]),
}


def _load():
    path = _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()
LIB_PATH = _build.LIB


def check(status, name):
    if status != MB_OK:
        raise MontblancError(status, name, lib.mb_last_error_string().decode())


def call(name, *args):
    """Call an mb_status-returning entry point and raise on failure."""
    check(getattr(lib, name)(*args), name)


def make_dims(ntime, na, nbl, nchan, npsrc, ngsrc=0, nssrc=0, beam=(1, 1, 1), extents=None, globals_=None):
    """Build an MbDims.  ``extents`` maps a dimension name to (lower, upper);
    ``globals_`` maps a dimension name to its global size (defaults: local)."""
    sizes = {'ntime': ntime, 'na': na, 'nbl': nbl, 'nchan': nchan, 'npol': 4, 'npolchan': 4 * nchan,
             'nsrc': npsrc + ngsrc + nssrc, 'npsrc': npsrc, 'ngsrc': ngsrc, 'nssrc': nssrc,
             'beam_lw': beam[0], 'beam_mh': beam[1], 'beam_nud': beam[2]}
    extents = extents or {}
    globals_ = globals_ or {}
    d = MbDims()
    for n in DIM_NAMES:
        local = int(sizes[n])
        lo, hi = extents.get(n, (0, local))
        setattr(d, n, MbDim(int(globals_.get(n, local)), local, int(lo), int(hi)))
    return d


def make_props(**kw):
    p = MbProps()
    for n in PROP_NAMES:
        setattr(p, n, float(kw[n]))
    return p


def version():
    return lib.mb_version().decode()


def kernel_launches():
    """Kernels this library has launched in this process."""
    return int(lib.mb_kernel_launches())


class KernelTimer:
    """Per-kernel CUDA-event timing of the library's launches while active.

    ``with KernelTimer() as kt: ...`` records an event pair on the launch
    stream around every launch inside the block; ``kt.times()`` maps each
    kernel name to (total ms, launches) and ``kt.launches`` is the number of
    launches the block made.
    """

    def __enter__(self):
        call('mb_kernel_timing_reset')
        self._n0 = kernel_launches()
        call('mb_kernel_timing', 1)
        return self

    def __exit__(self, *exc):
        call('mb_kernel_timing', 0)
        self.launches = kernel_launches() - self._n0
        return False

    def times(self):
        out = {}
        i = 0
        while True:
            name = lib.mb_kernel_timing_name(i)
            if name is None:
                break
            ms, n = ctypes.c_double(), ctypes.c_int64()
            call('mb_kernel_time', name, ctypes.byref(ms), ctypes.byref(n))
            if n.value:
                out[name.decode()] = (ms.value, n.value)
            i += 1
        return out


def exported_symbols():
    return tuple(SIGNATURES)


def lib_path():
    return os.path.abspath(LIB_PATH)

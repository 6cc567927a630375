"""The C ABI library: builds, loads and exports every declared symbol;
argument validation fails cleanly without touching the GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'montblanc_gb300.h')


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'^\s*(?:const char\*|mb_status|size_t|uint64_t|uint32_t)\s+(mb_\w+)\s*\(', text, re.M)))


def test_header_declares_entry_points():
    fns = declared_functions()
    for f in ('mb_bsqrt', 'mb_ebeam', 'mb_ekb_sqrt', 'mb_sum_coherencies', 'mb_reduce_chi2',
              'mb_rime_forward', 'mb_rime_adjoint', 'mb_rime_workspace_size', 'mb_last_error_string'):
        assert f in fns


def test_library_exports_every_declared_symbol():
    from montblanc_gb300 import _cabi
    lib = ctypes.CDLL(_cabi.lib_path())
    for f in declared_functions():
        assert hasattr(lib, f), f
    assert set(declared_functions()) == set(_cabi.exported_symbols())
    assert 'sm_103a' in _cabi.version()


def test_null_pointer_is_rejected():
    from montblanc_gb300 import _cabi
    d = _cabi.make_dims(2, 3, 3, 4, 2)
    st = _cabi.lib.mb_bsqrt(_cabi.MB_FLOAT64, ctypes.byref(d), None, None, None, None, None, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_NULL_PTR'
    assert b'stokes' in _cabi.lib.mb_last_error_string()


def test_bad_extent_is_rejected():
    from montblanc_gb300 import _cabi
    d = _cabi.make_dims(2, 3, 3, 4, 2, extents={'ntime': (1, 5)})
    fake = ctypes.c_void_p(16)
    st = _cabi.lib.mb_bsqrt(_cabi.MB_FLOAT64, ctypes.byref(d), fake, fake, fake, fake, fake, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_BAD_EXTENT'


def test_bad_shape_and_dtype_are_rejected():
    from montblanc_gb300 import _cabi
    d = _cabi.make_dims(2, 3, 3, 4, 2)
    d.npolchan.local_size = d.npolchan.global_size = 7
    d.npolchan.upper_extent = 7
    fake = ctypes.c_void_p(16)
    st = _cabi.lib.mb_bsqrt(_cabi.MB_FLOAT64, ctypes.byref(d), fake, fake, fake, fake, fake, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_BAD_SHAPE'
    d = _cabi.make_dims(2, 3, 3, 4, 2)
    st = _cabi.lib.mb_bsqrt(7, ctypes.byref(d), fake, fake, fake, fake, fake, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_UNSUPPORTED_DTYPE'


def test_workspace_is_checked():
    from montblanc_gb300 import _cabi
    d = _cabi.make_dims(2, 3, 3, 4, 2, beam=(2, 2, 2))
    n = _cabi.lib.mb_rime_workspace_size(_cabi.MB_FLOAT32, 0, ctypes.byref(d), 1)
    assert n > 0
    assert _cabi.lib.mb_rime_workspace_size(_cabi.MB_FLOAT32, 0, ctypes.byref(d), 0) < n
    fake = ctypes.c_void_p(256)
    inp = _cabi.MbRimeInputs()
    for name in _cabi.INPUT_NAMES:
        setattr(inp, name, 256)
    p = _cabi.make_props(gauss_scale=1, two_pi_over_c=1, sigma_sqrd=1, beam_ll=-1, beam_lm=-1,
                         beam_lfreq=1, beam_ul=1, beam_um=1, beam_ufreq=2)
    x2 = ctypes.c_void_p(256)
    st = _cabi.lib.mb_rime_forward(_cabi.MB_FLOAT32, 0, ctypes.byref(d), ctypes.byref(p), 0, ctypes.byref(inp),
                                   None, None, x2, 1, fake, n - 1, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_WORKSPACE'
    st = _cabi.lib.mb_rime_forward(_cabi.MB_FLOAT64, 1, ctypes.byref(d), ctypes.byref(p), 0, ctypes.byref(inp),
                                   None, None, x2, 0, fake, 1 << 30, None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_UNSUPPORTED'


def test_python_error_mapping():
    from montblanc_gb300 import _cabi
    d = _cabi.make_dims(2, 3, 3, 4, 2)
    with pytest.raises(_cabi.MontblancError, match='MB_ERR_NULL_PTR'):
        _cabi.call('mb_bsqrt', _cabi.MB_FLOAT64, ctypes.byref(d), None, None, None, None, None, None)


def test_kernel_timing_without_launches():
    """Timing switches on and off and reports nothing when nothing launched;
    rejected calls launch nothing, so the launch counter does not move."""
    from montblanc_gb300 import _cabi
    n0 = _cabi.kernel_launches()
    with _cabi.KernelTimer() as kt:
        d = _cabi.make_dims(2, 3, 3, 4, 2)
        _cabi.lib.mb_bsqrt(_cabi.MB_FLOAT64, ctypes.byref(d), None, None, None, None, None, None)
    assert kt.launches == 0
    assert kt.times() == {}
    assert _cabi.kernel_launches() == n0
    ms, n = ctypes.c_double(-1.0), ctypes.c_int64(-1)
    _cabi.call('mb_kernel_time', None, ctypes.byref(ms), ctypes.byref(n))
    assert (ms.value, n.value) == (0.0, 0)
    st = _cabi.lib.mb_kernel_time(None, None, ctypes.byref(n))
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_NULL_PTR'


def test_source_tile_options():
    """Tile bits pass option validation (the call then stops at the short
    workspace); unknown bits are rejected; the header and Python agree."""
    from montblanc_gb300 import _cabi
    text = open(HEADER).read()
    assert re.search(r'#define MB_SOURCE_TILE_SHIFT 8\b', text)
    assert _cabi.MB_SOURCE_TILE_MASK == 0x3 << 8
    assert [_cabi.source_tile_bits(t) >> 8 for t in (0, 8, 16, 32)] == [0, 1, 2, 3]
    with pytest.raises(ValueError):
        _cabi.source_tile_bits(12)
    d = _cabi.make_dims(2, 3, 3, 4, 2, beam=(2, 2, 2))
    n = _cabi.lib.mb_rime_workspace_size(_cabi.MB_FLOAT32, 0, ctypes.byref(d), 0)
    inp = _cabi.MbRimeInputs()
    for name in _cabi.INPUT_NAMES:
        setattr(inp, name, 256)
    p = _cabi.make_props(gauss_scale=1, two_pi_over_c=1, sigma_sqrd=1, beam_ll=-1, beam_lm=-1,
                         beam_lfreq=1, beam_ul=1, beam_um=1, beam_ufreq=2)
    x2, fake = ctypes.c_void_p(256), ctypes.c_void_p(256)
    for opts, want in ((_cabi.source_tile_bits(32), 'MB_ERR_WORKSPACE'), (1 << 12, 'MB_ERR_INVALID_ARG')):
        st = _cabi.lib.mb_rime_forward(_cabi.MB_FLOAT32, 0, ctypes.byref(d), ctypes.byref(p), opts,
                                       ctypes.byref(inp), None, None, x2, 0, fake, n - 1, None)
        assert _cabi.STATUS_NAMES[st] == want, (opts, _cabi.STATUS_NAMES[st])


def test_batch_plan_validation():
    """mb_rime_batch_workspace_size (host-side planning, no launch): a valid
    batch of sets has a workspace that grows with its sets; arrays above 64
    antennas, split modes on FP64 data, non-tile option bits and sets
    without source arrays are refused with 0 and a message."""
    from montblanc_gb300 import _cabi
    lib = _cabi.lib
    dummy = ctypes.c_void_p(0x1000)

    def sets(specs):
        arr = (_cabi.MbBatchSet * max(len(specs), 1))()
        for i, (npt, ng, ns, mode, opts) in enumerate(specs):
            b = arr[i]
            b.npsrc, b.ngsrc, b.nssrc, b.mode, b.options, b.reserved = npt, ng, ns, mode, opts, 0
            b.lm = b.stokes = b.alpha = dummy
            b.gauss_shape = dummy if ng else None
            b.sersic_shape = dummy if ns else None
        return arr, len(specs)

    def size(na, specs, dtype=_cabi.MB_FLOAT32):
        d = _cabi.make_dims(4, na, na * (na - 1) // 2, 3, 0, beam=(8, 8, 4))
        arr, n = sets(specs)
        return lib.mb_rime_batch_workspace_size(dtype, ctypes.byref(d), arr, n)

    tc, nat = _cabi.MB_MODE_SPLIT_TF32, _cabi.MB_MODE_NATIVE
    one = size(27, [(10, 2, 1, tc, 0)])
    two = size(27, [(10, 2, 1, tc, 0), (5, 0, 0, nat, _cabi.source_tile_bits(16))])
    assert 0 < one < two
    assert size(65, [(10, 0, 0, nat, 0)]) == 0
    assert '64 antennas' in lib.mb_last_error_string().decode()
    assert size(27, [(10, 0, 0, tc, 0)], dtype=_cabi.MB_FLOAT64) == 0
    assert 'FLOAT32' in lib.mb_last_error_string().decode()
    assert size(27, [(10, 0, 0, nat, _cabi.MB_APPLY_WEIGHTS)]) == 0
    assert 'source-tile' in lib.mb_last_error_string().decode()
    arr, n = sets([(10, 0, 0, nat, 0)])
    arr[0].lm = None
    d = _cabi.make_dims(4, 27, 351, 3, 0, beam=(8, 8, 4))
    assert lib.mb_rime_batch_workspace_size(_cabi.MB_FLOAT32, ctypes.byref(d), arr, n) == 0
    assert 'lm' in lib.mb_last_error_string().decode()

"""mb_rime_forward_noalloc: the allocation-free forward for callers that may
not allocate device memory (their own pool or framework owns it, or a
cudaMalloc would stall a latency-bound pipeline).  Called through the C ABI
and compared with mb_rime_forward on two calls in a row; the second call
must not see stale partial sums of the first (the static scratch array is
shared by all calls).  Collected last so that a failure here leaves the
rest of the suite already run."""
import ctypes

import numpy as np
import pytest

import golden_io
from gpu_helpers import TOL

pytestmark = pytest.mark.gpu


def _run(prob, fn, model_vis, chi2, x2):
    import torch
    from montblanc_gb300 import _cabi
    d = prob.dims()
    inp = prob.inputs()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if fn == 'noalloc':
        st = _cabi.lib.mb_rime_forward_noalloc(prob.mb_dtype, ctypes.byref(d), ctypes.byref(prob.mb_props()),
                                               prob.options(), ctypes.byref(inp), model_vis.data_ptr(),
                                               chi2.data_ptr(), x2.data_ptr(), stream)
    else:
        ws = prob.workspace('native', False)
        st = _cabi.lib.mb_rime_forward(prob.mb_dtype, 0, ctypes.byref(d), ctypes.byref(prob.mb_props()),
                                       prob.options(), ctypes.byref(inp), model_vis.data_ptr(), chi2.data_ptr(),
                                       x2.data_ptr(), 0, ws.data_ptr(), ws.numel(), stream)
    _cabi.check(st, fn)
    torch.cuda.synchronize()


@pytest.mark.parametrize('dtype', ['double', 'float'])
def test_noalloc_matches_workspace_forward_twice(dtype):
    # Same tolerances as the other parity tests: the allocation-free path
    # forms the beam and phase terms without the workspace tables, so FP32
    # results differ in rounding.
    tol = TOL[dtype]
    import torch
    from montblanc_gb300.rime import RimeProblem
    problems = [RimeProblem.from_numpy(golden_io.load(n)[0], dtype=dtype)
                for n in ('small_fp64', 'perm_p3_g3_s3_w1')]
    for prob in problems:  # two calls in a row, different shapes
        v_ref, c_ref = prob.empty_vis(), prob.empty_chi2()
        x_ref = torch.zeros(1, dtype=torch.float64, device='cuda')
        _run(prob, 'workspace', v_ref, c_ref, x_ref)
        for _ in range(2):
            v, c = prob.empty_vis(), prob.empty_chi2()
            x = torch.full((1,), float('nan'), dtype=torch.float64, device='cuda')
            _run(prob, 'noalloc', v, c, x)
            assert golden_io.rel_err(v.cpu().numpy(), v_ref.cpu().numpy()) <= tol['vis']
            assert golden_io.rel_err(c.cpu().numpy(), c_ref.cpu().numpy()) <= tol['terms']
            assert abs(x.item() - x_ref.item()) <= tol['X2'] * abs(x_ref.item())


@pytest.mark.parametrize('dtype', ['double', 'float'])
def test_noalloc_source_batches(dtype):
    """Two source batches through the allocation-free entry, the second
    accumulating onto the partial sums the first left in model_vis, give the
    reference's one-call result."""
    import torch
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load('perm_p3_g3_s3_w0')
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    vis, chi2 = prob.empty_vis(), prob.empty_chi2()
    x2 = torch.zeros(1, dtype=torch.float64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for lo, hi, ext in ((0, 4, {'npsrc': (0, 3), 'ngsrc': (0, 1), 'nssrc': (0, 0)}),
                        (4, 9, {'npsrc': (0, 0), 'ngsrc': (0, 2), 'nssrc': (0, 3)})):
        sl = slice(lo, hi)
        ov = {'lm': prob.arrays['lm'][sl].contiguous(), 'stokes': prob.arrays['stokes'][sl].contiguous(),
              'alpha': prob.arrays['alpha'][sl].contiguous()}
        gl = max(lo, 3) - 3
        gs = torch.zeros_like(prob.arrays['gauss_shape'])
        gs[:, :3 - gl] = prob.arrays['gauss_shape'][:, gl:]
        ov['gauss_shape'] = gs
        e = dict(ext)
        e['nsrc'] = (lo, hi)
        d = _cabi.make_dims(prob.ntime, prob.na, prob.nbl, prob.nchan, 3, 3, 3, beam=prob.beam,
                            extents=e, globals_={'nsrc': 9})
        d.nsrc.local_size = 9
        inp = prob.inputs(**ov)
        st = _cabi.lib.mb_rime_forward_noalloc(prob.mb_dtype, ctypes.byref(d), ctypes.byref(prob.mb_props()),
                                               prob.options(), ctypes.byref(inp), vis.data_ptr(), chi2.data_ptr(),
                                               x2.data_ptr(), stream)
        _cabi.check(st, 'mb_rime_forward_noalloc')
    torch.cuda.synchronize()
    assert golden_io.rel_err(vis.cpu().numpy(), ref['vis_out']) < TOL[dtype]['vis']
    assert golden_io.rel_err(chi2.cpu().numpy(), ref['chi_sqrd_terms']) < TOL[dtype]['terms']
    assert abs(x2.item() - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


def test_noalloc_zero_extent():
    """No (time, channel) units: chi^2 is 0 and nothing else is touched."""
    import torch
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, _ = golden_io.load('small_fp64')
    prob = RimeProblem.from_numpy(P, dtype='float')
    d = _cabi.make_dims(prob.ntime, prob.na, prob.nbl, prob.nchan, prob.npsrc, prob.ngsrc, prob.nssrc,
                        beam=prob.beam, extents={'ntime': (0, 0)})
    vis = prob.empty_vis().fill_(7.0)
    x2 = torch.full((1,), float('nan'), dtype=torch.float64, device='cuda')
    inp = prob.inputs()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = _cabi.lib.mb_rime_forward_noalloc(prob.mb_dtype, ctypes.byref(d), ctypes.byref(prob.mb_props()), 0,
                                           ctypes.byref(inp), vis.data_ptr(), None, x2.data_ptr(), stream)
    _cabi.check(st, 'mb_rime_forward_noalloc')
    torch.cuda.synchronize()
    assert x2.item() == 0.0
    assert bool((vis == 7.0).all())


def test_noalloc_rejects_too_many_units():
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, _ = golden_io.load('small_fp64')
    prob = RimeProblem.from_numpy(P, dtype='float')
    maxu = _cabi.lib.mb_rime_noalloc_max_units()
    d = _cabi.make_dims(maxu + 1, prob.na, prob.nbl, 1, prob.npsrc, prob.ngsrc, prob.nssrc, beam=prob.beam)
    inp = prob.inputs()
    x2 = prob.empty_chi2()
    st = _cabi.lib.mb_rime_forward_noalloc(prob.mb_dtype, ctypes.byref(d), ctypes.byref(prob.mb_props()), 0,
                                           ctypes.byref(inp), None, None, x2.data_ptr(), None)
    assert _cabi.STATUS_NAMES[st] == 'MB_ERR_UNSUPPORTED'
    assert b'at most' in _cabi.lib.mb_last_error_string()

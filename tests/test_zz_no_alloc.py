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

"""Tensor-core operand path (staging layout, descriptors, tcgen05.mma,
TMEM readout) against an FP64 matrix product."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# One accumulator over all of K: the tensor core's FP32 accumulation rounds
# toward zero, adding ~2.5e-8 relative per accumulation (3 per 8 TF32 / 16
# BF16 values of K); BF16 hi + lo also has a ~5e-6 representation floor.
@pytest.mark.parametrize('mode,K,tol', [('split_tf32', 32, 2e-6), ('split_tf32', 256, 5e-6),
                                        ('split_bf16', 64, 5e-5), ('split_bf16', 256, 5e-5)])
def test_split_gemm_selftest(mode, K, tol):
    import torch
    from montblanc_gb300 import _cabi
    g = torch.Generator(device='cpu').manual_seed(K)
    A = torch.randn(128, K, generator=g, dtype=torch.float64)
    B = torch.randn(128, K, generator=g, dtype=torch.float64)
    A32, B32 = A.float().cuda(), B.float().cuda()
    D = torch.zeros(128, 128, dtype=torch.float32, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    _cabi.call('mb_tc_selftest', A32.data_ptr(), B32.data_ptr(), K, _cabi.MODES[mode], D.data_ptr(),
               status.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert status.item() == 0
    ref = (A32.double().cpu() @ B32.double().cpu().T).numpy()
    got = D.cpu().double().numpy()
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err < tol, err
    # a plain FP32 product of the same operands is far less accurate for BF16 operands
    assert np.isfinite(got).all()


@pytest.mark.parametrize('K', [64, 256])
def test_split_gemm_selftest_a_in_tmem(K):
    """BF16 split product with the A operand read from tensor memory equals
    the same product with A from shared memory (and the FP64 product)."""
    import torch
    from montblanc_gb300 import _cabi
    g = torch.Generator(device='cpu').manual_seed(K + 1)
    A32 = torch.randn(128, K, generator=g, dtype=torch.float64).float().cuda()
    B32 = torch.randn(128, K, generator=g, dtype=torch.float64).float().cuda()
    out = {}
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for flag in (0, _cabi.MB_TC_SELFTEST_A_IN_TMEM):
        D = torch.zeros(128, 128, dtype=torch.float32, device='cuda')
        status = torch.zeros(1, dtype=torch.int32, device='cuda')
        _cabi.call('mb_tc_selftest', A32.data_ptr(), B32.data_ptr(), K, _cabi.MODES['split_bf16'] | flag,
                   D.data_ptr(), status.data_ptr(), stream)
        torch.cuda.synchronize()
        assert status.item() == 0
        out[flag] = D.cpu().double().numpy()
    ref = (A32.double().cpu() @ B32.double().cpu().T).numpy()
    got = out[_cabi.MB_TC_SELFTEST_A_IN_TMEM]
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 5e-5
    assert np.max(np.abs(got - out[0])) <= 1e-6 * np.max(np.abs(ref))


SPLIT_TOL = {'split_tf32': {'vis': 2e-5, 'terms': 1e-3, 'X2': 1e-4},
             'split_bf16': {'vis': 2e-4, 'terms': 1e-2, 'X2': 1e-3}}


@pytest.mark.parametrize('mode', ['split_tf32', 'split_bf16'])
@pytest.mark.parametrize('name', ['small_fp64', 'perm_p3_g0_s0_w1', 'perm_p3_g3_s3_w0', 'residual_w1',
                                  'ebeam_odd'])
def test_split_forward_matches_reference(mode, name):
    """Point sources on the tensor cores (extended sources on the CUDA cores)
    against the reference's own outputs."""
    import golden_io
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load(name)
    prob = RimeProblem.from_numpy(P, dtype='float')
    vis, chi2 = prob.empty_vis(), prob.empty_chi2()
    x2 = prob.forward(mode=mode, model_vis=vis, chi_sqrd_result=chi2).item()
    tol = SPLIT_TOL[mode]
    assert golden_io.rel_err(vis.cpu().numpy(), ref['vis_out']) < tol['vis']
    assert golden_io.rel_err(chi2.cpu().numpy(), ref['chi_sqrd_terms']) < tol['terms']
    assert abs(x2 - ref['X2']) <= tol['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('mode', ['split_tf32', 'split_bf16'])
def test_split_forward_many_sources_against_fp64(mode):
    """300 point + 20 gaussian sources (several accumulation groups and a
    partial last stage) against the FP64 path on the same FP32 inputs."""
    import numpy as np
    from montblanc_gb300 import synth
    from montblanc_gb300.rime import RimeProblem
    P = synth.make_problem(ntime=3, na=27, nchan=4, npsrc=301, ngsrc=20, seed=5, flag_fraction=0.05,
                           antenna_scaling_noise=0.02)
    for k in ('uvw', 'frequency', 'ref_frequency', 'parallactic_angles', 'point_errors', 'antenna_scaling',
              'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'weight_vector'):
        P[k] = P[k].astype(np.float32).astype(np.float64)
    for k in ('E_beam', 'G_term'):
        P[k] = P[k].astype(np.complex64).astype(np.complex128)
    p64 = RimeProblem.from_numpy(P, dtype='double')
    v64 = p64.empty_vis()
    p64.forward(model_vis=v64)
    P['observed_vis'] = (v64.cpu().numpy() + 0.1).astype(np.complex64).astype(np.complex128)
    p64 = RimeProblem.from_numpy(P, dtype='double')
    p32 = RimeProblem.from_numpy(P, dtype='float')
    v64, v32, vn = p64.empty_vis(), p32.empty_vis(), p32.empty_vis()
    x64 = p64.forward(model_vis=v64).item()
    x32 = p32.forward(mode=mode, model_vis=v32).item()
    p32.forward(mode='native', model_vis=vn)
    a, b, c = v32.cpu().numpy(), v64.cpu().numpy(), vn.cpu().numpy()
    err = np.linalg.norm(a - b) / np.linalg.norm(b)
    err_native = np.linalg.norm(c - b) / np.linalg.norm(b)
    assert err < (2e-6 if mode == 'split_tf32' else 5e-5), (err, err_native)
    assert abs(x32 - x64) <= 1e-3 * abs(x64)


@pytest.mark.parametrize('limit', [0, 1 << 10])
def test_bounded_wait_gives_up_and_the_context_stays_usable(limit):
    """A wait on an mbarrier that nothing arrives on gives up after its poll
    limit, reports it, frees its TMEM; the tensor-core kernels run
    correctly right after it."""
    import torch
    from montblanc_gb300 import _cabi
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _cabi.call('mb_wait_selftest', limit, status.data_ptr(), stream)
    torch.cuda.synchronize()
    assert status.item() == 1
    g = torch.Generator(device='cpu').manual_seed(3)
    A = torch.randn(128, 64, generator=g).cuda()
    B = torch.randn(128, 64, generator=g).cuda()
    D = torch.zeros(128, 128, dtype=torch.float32, device='cuda')
    status.zero_()
    _cabi.call('mb_tc_selftest', A.data_ptr(), B.data_ptr(), 64, _cabi.MODES['split_tf32'], D.data_ptr(),
               status.data_ptr(), stream)
    torch.cuda.synchronize()
    assert status.item() == 0
    ref = (A.double() @ B.double().T)
    assert float((D.double() - ref).abs().max() / ref.abs().max()) < 5e-6


def test_fused_timeout_reaches_the_host():
    """With the poll limit of the tensor-core kernels' pipeline waits at 0,
    every such wait gives up at once: the forward's chi^2 is NaN and
    mb_rime_status reports MB_ERR_TIMEOUT, and so does an adjoint after it
    (which then does no work).  An adjoint after a good forward gives up on
    its own waits and reports it too.  With the default limit restored the
    same problem runs correctly in the same context."""
    import math
    import torch
    import golden_io
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load('small_fp64')
    prob = RimeProblem.from_numpy(P, dtype='float')
    good = prob.forward(mode='split_tf32', want_grad=True).item()
    prob.adjoint(mode='split_tf32')
    prob.check('split_tf32', True)
    default = _cabi.lib.mb_default_wait_limit()
    try:
        _cabi.call('mb_set_wait_limit', 0)
        x2 = prob.forward(mode='split_tf32', want_grad=True).item()
        assert math.isnan(x2)
        with pytest.raises(_cabi.MontblancError) as e:
            prob.check('split_tf32', True)
        assert e.value.status == 6  # MB_ERR_TIMEOUT
        prob.adjoint(mode='split_tf32')
        with pytest.raises(_cabi.MontblancError):
            prob.check('split_tf32', True)
        # a good forward, then an adjoint whose own waits give up
        _cabi.call('mb_set_wait_limit', default)
        prob.forward(mode='split_tf32', want_grad=True)
        torch.cuda.synchronize()
        _cabi.call('mb_set_wait_limit', 0)
        prob.adjoint(mode='split_tf32')
        with pytest.raises(_cabi.MontblancError):
            prob.check('split_tf32', True)
    finally:
        torch.cuda.synchronize()
        _cabi.call('mb_set_wait_limit', default)
    x2 = prob.forward(mode='split_tf32', want_grad=True).item()
    g = prob.adjoint(mode='split_tf32')
    prob.check('split_tf32', True)
    assert x2 == good
    assert abs(x2 - ref['X2']) <= 1e-4 * abs(ref['X2'])
    assert all(torch.isfinite(v).all() for v in g.values())

"""Arrays wider than the fused kernels' 64-antenna tile, evaluated as antenna
sub-arrays (one launch per pair of 32-antenna blocks, each baseline owned by
one launch), against the reference's own forward and the FP64 oracle
gradient.

Fixtures (tests/golden/make_golden.py, case_wide_arrays): 128 antennas
(8128 baselines, four blocks) and 75 antennas (a ragged last block of 11),
weights, flags and point, gaussian and sersic sources; gradients at the
truth and at source positions displaced from it.

Bounds: FP64 as for the benchmarked units (1e-10 forward, 1e-9 gradients);
the FP32 forms' bounds sit above the values measured on these fixtures,
which are given beside them.
"""
import numpy as np
import pytest

import golden_io
from gpu_helpers import TOL
from test_units_gpu import PARAMS, evaluate, norm_err, oracle_grads

pytestmark = pytest.mark.gpu
WIDE = ('wide_na128', 'wide_na75')

#: Norm-wise relative model-visibility error against the reference
#: (measured, 128 / 75 antennas: plain FP32 2.5e-7 / 2.3e-7, TF32 split
#: 4.2e-7 / 3.6e-7, BF16 split 4.3e-6 / 4.3e-6).
VIS_BOUND = {'native': 1e-6, 'split_tf32': 1e-6, 'split_bf16': 1e-5}
#: Relative chi^2 error (measured: 9.9e-8 / 2.1e-7, 4.9e-7 / 4.4e-7,
#: 5.9e-6 / 7.2e-6).
X2_BOUND = {'native': 1e-5, 'split_tf32': 1e-5, 'split_bf16': 2e-4}
#: Norm-wise relative gradient error (worst parameter) at the displaced
#: sources (measured: 2.2e-3 / 2.0e-4, 2.2e-3 / 4.6e-4, 3.0e-3 / 7.6e-4).
#: These problems have few (time, channel) units, so each source's gradient
#: sums few visibilities and stays close to the noise: the FP32 model error
#: reaches it amplified (the FP64 path agrees with the oracle to 3e-11).
GRAD_BOUND = {'native': 5e-3, 'split_tf32': 5e-3, 'split_bf16': 6e-3}


@pytest.mark.parametrize('name', WIDE)
def test_fp64_forward_matches_reference(name):
    P, ref, vis, terms, x2, _ = evaluate(name, 'double')
    assert golden_io.rel_err(vis, ref['vis_out']) < TOL['double']['vis']
    assert golden_io.rel_err(terms, ref['chi_sqrd_terms']) < golden_io.terms_tol(P, ref, 1e-12, 1e-10)
    assert abs(x2 - ref['X2']) <= TOL['double']['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('mode', ['native', 'split_tf32', 'split_bf16'])
@pytest.mark.parametrize('name', WIDE)
def test_fp32_forward_error_bound(name, mode):
    _, ref, vis, _, x2, _ = evaluate(name, 'float', mode)
    err = norm_err(vis, ref['vis_out'])
    assert err < VIS_BOUND[mode], err
    assert abs(x2 - ref['X2']) <= X2_BOUND[mode] * abs(ref['X2']), (x2, ref['X2'])


@pytest.mark.parametrize('displaced', [False, True])
@pytest.mark.parametrize('name', WIDE)
def test_fp64_adjoint_matches_oracle(name, displaced):
    _, ref, _, _, _, g = evaluate(name, 'double', want_grad=True, displaced=displaced)
    og = oracle_grads(ref, displaced)
    for k in PARAMS:
        if og[k].size:
            assert norm_err(g[k], og[k]) < 1e-9, (k, norm_err(g[k], og[k]))


@pytest.mark.parametrize('mode', ['native', 'split_tf32', 'split_bf16'])
@pytest.mark.parametrize('name', WIDE)
def test_fp32_gradient_error_bound(name, mode):
    _, ref, _, _, _, g = evaluate(name, 'float', mode, want_grad=True, displaced=True)
    og = oracle_grads(ref, True)
    for k in PARAMS:
        if og[k].size:
            err = norm_err(g[k], og[k])
            assert err < GRAD_BOUND[mode], (k, err)


def test_sub_arrays_launch_per_block_pair():
    """128 antennas run as 6 launches of the forward kernel, one per pair of
    its four 32-antenna blocks."""
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, _ = golden_io.load('wide_na128')
    prob = RimeProblem.from_numpy(P, dtype='float')
    import torch
    with _cabi.KernelTimer() as kt:
        prob.forward(mode='split_tf32')
        torch.cuda.synchronize()
    assert kt.times()['coh_tc_fwd_kernel'][1] == 6


@pytest.mark.parametrize('dtype', ['double', 'float'])
def test_sub_arrays_with_source_batches(dtype):
    """The reference's source batches (nsrc extents, partial sums carried in
    model_vis) on a 75-antenna array split into sub-arrays: 12 point sources,
    then 4 point, 4 gaussian and 4 sersic sources, against the reference's
    one-pass result."""
    import ctypes
    import torch
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load('wide_na75')
    assert (P['npsrc'], P['ngsrc'], P['nssrc']) == (16, 4, 4)
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    vis, chi2 = prob.empty_vis(), prob.empty_chi2()
    x2 = torch.zeros(1, dtype=torch.float64, device='cuda')
    ws = prob.workspace('native', False)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for lo, hi, ext in ((0, 12, {'npsrc': (0, 12), 'ngsrc': (0, 0), 'nssrc': (0, 0)}),
                        (12, 24, {'npsrc': (0, 4), 'ngsrc': (0, 4), 'nssrc': (0, 4)})):
        sl = slice(lo, hi)
        ov = {'lm': prob.arrays['lm'][sl].contiguous(), 'stokes': prob.arrays['stokes'][sl].contiguous(),
              'alpha': prob.arrays['alpha'][sl].contiguous()}
        e = dict(ext)
        e['nsrc'] = (lo, hi)
        d = _cabi.make_dims(prob.ntime, prob.na, prob.nbl, prob.nchan, 16, 4, 4, beam=prob.beam,
                            extents=e, globals_={'nsrc': 24})
        inp = prob.inputs(**ov)
        _cabi.call('mb_rime_forward', prob.mb_dtype, 0, ctypes.byref(d), ctypes.byref(prob.mb_props()),
                   prob.options(), ctypes.byref(inp), vis.data_ptr(), chi2.data_ptr(), x2.data_ptr(), 0,
                   ws.data_ptr(), ws.numel(), stream)
    assert golden_io.rel_err(vis.cpu().numpy(), ref['vis_out']) < TOL[dtype]['vis']
    assert abs(x2.item() - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('na', [32, 33, 65])
def test_antenna_count_edges(na):
    """The edges of the kernels' antenna layouts against the FP64 oracle:
    32 antennas (two channels per tensor-core CTA, exactly full), 33 (one
    channel per CTA), 65 (three sub-arrays, the last block one antenna);
    FP64 forward and adjoint, the TF32 split forward."""
    from montblanc_gb300 import synth
    from montblanc_gb300.rime import RimeProblem
    from oracle import adjoint as OA
    from oracle import rime_v4 as O
    P = synth.make_problem(ntime=2, na=na, nchan=3, npsrc=9, ngsrc=2, nssrc=1, seed=na, beam_shape=(12, 12, 6),
                           flag_fraction=0.05)
    model, _, _ = O.forward(P)
    synth.add_noise(P, model, sigma=0.1, seed=na + 1)
    # inputs representable in FP32, so that the FP32 run and the oracle see
    # the same values (the phase of a rounded uvw differs by ~1e-4 rad)
    for k, v in P.items():
        if isinstance(v, np.ndarray) and v.dtype == np.float64:
            P[k] = v.astype(np.float32).astype(np.float64)
        elif isinstance(v, np.ndarray) and v.dtype == np.complex128:
            P[k] = v.astype(np.complex64).astype(np.complex128)
    ref_vis, _, ref_x2 = O.forward(P)
    ref_x2g, ref_g = OA.chi2_grad(P)
    prob = RimeProblem.from_numpy(P, dtype='double')
    vis = prob.empty_vis()
    x2 = prob.forward(model_vis=vis, want_grad=True).item()
    g = {k: v.cpu().numpy() for k, v in prob.adjoint().items()}
    assert golden_io.rel_err(vis.cpu().numpy(), ref_vis) < 1e-10
    assert abs(x2 - ref_x2) <= 1e-10 * abs(ref_x2)
    for k, r in ref_g.items():
        if r.size:
            assert norm_err(g[k], r) < 1e-9, (k, norm_err(g[k], r))
    p32 = RimeProblem.from_numpy(P, dtype='float')
    v32 = p32.empty_vis()
    x2s = p32.forward(mode='split_tf32', model_vis=v32).item()
    assert norm_err(v32.cpu().numpy(), ref_vis) < VIS_BOUND['split_tf32']
    assert abs(x2s - ref_x2) <= X2_BOUND['split_tf32'] * abs(ref_x2)

"""Fused forward (mb_rime_forward) against the reference's outputs."""
import numpy as np
import pytest

import golden_io
from gpu_helpers import TOL, solver_for
from oracle import rime_v4 as O

pytestmark = pytest.mark.gpu
DTYPES = ('double', 'float')
CASES = [n for n in golden_io.names() if n != 'given_jones']


@pytest.mark.parametrize('dtype', DTYPES)
@pytest.mark.parametrize('name', CASES)
def test_fused_solver_matches_reference(name, dtype):
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    with solver_for(P, dtype, mb.Pipeline([mb.RimeV4Fused()])) as s:
        s.solve()
        assert golden_io.rel_err(s.retrieve_model_vis(), ref['vis_out']) < TOL[dtype]['vis']
        # chi^2 terms: the model's agreement amplified by max|model| / max|residual|
        vis_rel = 1e-12 if dtype == 'double' else 2e-7
        assert golden_io.rel_err(s.retrieve_chi_sqrd_result(), ref['chi_sqrd_terms']) < \
            golden_io.terms_tol(P, ref, vis_rel, TOL[dtype]['terms'])
        assert abs(s.X2 - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('dtype', DTYPES)
def test_fused_chi2_only(dtype):
    """model_vis and chi_sqrd_result may be omitted (NULL)."""
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load('small_fp64')
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    x2 = prob.forward().item()
    assert abs(x2 - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('dtype, mode', [(d, 0) for d in DTYPES] + [('float', 1)])
def test_fused_source_batches(dtype, mode):
    """Fused forward over two source batches accumulating in model_vis (mode
    1, the TF32 split form: its extended sources' CUDA-core forward adds to
    the first batch's partial sums, the tensor-core forward adds its point
    sources to that)."""
    import montblanc_gb300 as mb
    from montblanc_gb300.rime import RimeProblem
    from montblanc_gb300 import _cabi
    import ctypes
    import torch
    P, ref = golden_io.load('perm_p3_g3_s3_w0')
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    vis = prob.empty_vis()
    chi2 = prob.empty_chi2()
    x2 = torch.zeros(1, dtype=torch.float64, device='cuda')
    ws = prob.workspace('native' if mode == 0 else 'split_tf32', False)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for lo, hi, ext in ((0, 4, {'npsrc': (0, 3), 'ngsrc': (0, 1), 'nssrc': (0, 0)}),
                        (4, 9, {'npsrc': (0, 0), 'ngsrc': (0, 2), 'nssrc': (0, 3)})):
        # present the batch's sources at the front of each parameter array
        sl = slice(lo, hi)
        ov = {'lm': prob.arrays['lm'][sl].contiguous(), 'stokes': prob.arrays['stokes'][sl].contiguous(),
              'alpha': prob.arrays['alpha'][sl].contiguous()}
        gl = max(lo, 3) - 3
        gs = torch.zeros_like(prob.arrays['gauss_shape'])  # keeps the local row stride of 3
        gs[:, :3 - gl] = prob.arrays['gauss_shape'][:, gl:]
        ov['gauss_shape'] = gs
        e = dict(ext)
        e['nsrc'] = (lo, hi)
        d = _cabi.make_dims(prob.ntime, prob.na, prob.nbl, prob.nchan, 3, 3, 3, beam=prob.beam,
                            extents=e, globals_={'nsrc': 9})
        d.nsrc.local_size = 9
        inp = prob.inputs(**ov)
        _cabi.call('mb_rime_forward', prob.mb_dtype, mode, ctypes.byref(d), ctypes.byref(prob.mb_props()),
                   prob.options(), ctypes.byref(inp), vis.data_ptr(), chi2.data_ptr(), x2.data_ptr(), 0,
                   ws.data_ptr(), ws.numel(), stream)
    assert golden_io.rel_err(vis.cpu().numpy(), ref['vis_out']) < TOL[dtype]['vis']
    assert abs(x2.item() - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


def test_fused_non_default_antenna_pairs():
    """Baselines in arbitrary order, including swapped (q, p) pairs and an
    autocorrelation, against the oracle (which follows antenna1/antenna2)."""
    from montblanc_gb300.rime import RimeProblem
    P, _ = golden_io.load('perm_p3_g3_s3_w1')
    rng = np.random.default_rng(11)
    a1, a2 = P['antenna1'].copy(), P['antenna2'].copy()
    for t in range(a1.shape[0]):
        perm = rng.permutation(a1.shape[1])
        a1[t], a2[t] = a1[t][perm], a2[t][perm]
        swap = rng.random(a1.shape[1]) < 0.5
        a1[t][swap], a2[t][swap] = a2[t][swap].copy(), a1[t][swap].copy()
        a2[t][0] = a1[t][0]  # one autocorrelation per time step
    P['antenna1'], P['antenna2'] = a1, a2
    out, terms, X2 = O.forward(P, src_chunk=9)
    prob = RimeProblem.from_numpy(P, dtype='double')
    vis, chi2 = prob.empty_vis(), prob.empty_chi2()
    x2 = prob.forward(model_vis=vis, chi_sqrd_result=chi2).item()
    assert golden_io.rel_err(vis.cpu().numpy(), out) < 1e-10
    assert golden_io.rel_err(chi2.cpu().numpy(), terms) < 1e-10
    assert abs(x2 - X2) <= 1e-10 * abs(X2)


def test_kernel_timer_reports_the_fused_launches():
    """Per-kernel event timing sees the fused kernels of one forward."""
    from montblanc_gb300 import _cabi
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load('small_fp64')
    prob = RimeProblem.from_numpy(P, dtype='float')
    prob.forward()
    with _cabi.KernelTimer() as kt:
        x2 = prob.forward().item()
    times = kt.times()
    assert 'coh_fwd_kernel' in times and 'sum_partials_kernel' in times
    assert kt.launches == sum(n for _, n in times.values())
    assert all(ms >= 0.0 for ms, _ in times.values())
    assert abs(x2 - ref['X2']) <= TOL['float']['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('mode', ['native', 'split_tf32'])
def test_fp32_phase_on_long_baselines(mode):
    """Baselines thousands of kilometres long (about 2e6 phase cycles): the
    FP32 forms reduce phi nu / c from FP32 pairs of the FP64 path length, and
    their model visibilities keep their usual error against the FP64 oracle
    (a phase argument formed in FP32 would be off by whole cycles here)."""
    from montblanc_gb300 import synth
    from montblanc_gb300.rime import RimeProblem
    from test_units_gpu import norm_err
    P = synth.make_problem(ntime=2, na=12, nchan=4, npsrc=10, seed=5, beam_shape=(12, 12, 6))
    P['uvw'] = P['uvw'] * 5000.0
    # inputs representable in FP32, so that both see the same values
    for k, v in P.items():
        if isinstance(v, np.ndarray) and v.dtype == np.float64:
            P[k] = v.astype(np.float32).astype(np.float64)
        elif isinstance(v, np.ndarray) and v.dtype == np.complex128:
            P[k] = v.astype(np.complex64).astype(np.complex128)
    l, m = P['lm'][:, 0], P['lm'][:, 1]
    phi = (P['uvw'][..., 0][:, None] * l[None, :, None] + P['uvw'][..., 1][:, None] * m[None, :, None] +
           P['uvw'][..., 2][:, None] * (np.sqrt(1 - l * l - m * m) - 1)[None, :, None])
    assert np.abs(phi).max() * P['frequency'].max() / 299792458.0 > 1e6
    ref_vis, _, _ = O.forward(P)
    prob = RimeProblem.from_numpy(P, dtype='float')
    vis = prob.empty_vis()
    prob.forward(mode=mode, model_vis=vis)
    assert norm_err(vis.cpu().numpy(), ref_vis) < 1e-6

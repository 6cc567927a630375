"""The CUDA paths on sampled (time, channel) units of the two benchmarked
workloads, against the reference's own outputs and the FP64 oracle gradient.

Fixtures (tests/golden/make_golden.py, case_sampled_units): all sources and
baselines of
  * units_medium_mixed: 3 times x 3 channels of the 100 x 27 x 64 workload,
    1000 point + 200 gaussian + 50 sersic sources;
  * units_large_point: 2 times x 3 channels of the 200 x 64 x 256 workload,
    20 000 point + 500 gaussian sources (the benchmark's own units: same
    generator and seed).
Forward outputs come from the reference's CPUSolver run per source batch;
gradients from oracle/adjoint.py (the reference has none), at the truth and
at source positions displaced from it.

Bounds:
  * FP64: 1e-10 relative (max-normalised) for model visibilities, chi^2
    terms and chi^2; gradients 1e-9 (norm-wise) of the oracle's.
  * plain FP32 (CUDA cores): the reference's float tolerances.
  * split precision: relative model-visibility error (norm-wise) below
    1e-6 for the TF32 split, 1e-5 for the BF16 split (its hi + lo operands
    carry 16 significant bits).
  * chi^2 and gradients of the FP32 forms: the bounds below, each set above
    the measured value with the measurement beside it.
"""
import numpy as np
import pytest

import golden_io
from gpu_helpers import TOL

pytestmark = pytest.mark.gpu
UNITS = ('units_medium_mixed', 'units_large_point')
PARAMS = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term')

#: Norm-wise relative error of the model visibilities against FP64
#: (measured: plain FP32 2.6e-7, TF32 split 8.1e-7, BF16 split 4.6e-6).
VIS_BOUND = {'native': 1e-6, 'split_tf32': 1e-6, 'split_bf16': 1e-5}
#: Relative chi^2 error against FP64 (measured on the 20 500-source units:
#: 6.5e-6, 2.0e-5, 6.4e-4).  chi^2 sums squared residuals that are small
#: against the model (max|model| / max|residual| = 7000 there), so it
#: carries the model's error amplified.
X2_BOUND = {'native': 2e-5, 'split_tf32': 5e-5, 'split_bf16': 2e-3}
#: Norm-wise relative gradient error against the FP64 oracle, worst
#: parameter.  At the displaced source positions the residual is model
#: mismatch (measured: plain FP32 2.3e-5, TF32 split 4.2e-4, BF16 split
#: 4.8e-4); at the truth the gradient is a noise-level sum and the forward
#: model's error biases it (1.9e-3, 2.4e-2, 3.0e-2).  The split forms' worst
#: parameter is G: the tensor core's FP32 accumulation truncates toward zero,
#: shrinking the model coherently, and d chi^2 / dG = sum M V^H adds that
#: shrink up coherently where round-to-nearest FP32 errors average out.
GRAD_BOUND_DISPLACED = {'native': 5e-5, 'split_tf32': 1e-3, 'split_bf16': 1e-3}
GRAD_BOUND_TRUTH = {'native': 5e-3, 'split_tf32': 5e-2, 'split_bf16': 6e-2}


def norm_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def evaluate(name, dtype, mode='native', want_grad=False, displaced=False):
    """Forward (and adjoint) of fixture ``name`` on the GPU: (P, ref, vis,
    chi^2 terms, X2, grads)."""
    from montblanc_gb300.rime import RimeProblem
    P, ref = golden_io.load(name)
    if displaced:
        P['lm'] = ref['displaced_lm']
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    vis, terms = prob.empty_vis(), prob.empty_chi2()
    x2 = prob.forward(mode=mode, model_vis=vis, chi_sqrd_result=terms, want_grad=want_grad).item()
    grads = prob.adjoint(mode=mode) if want_grad else None
    if grads is not None:
        grads = {k: v.cpu().numpy() for k, v in grads.items()}
    return P, ref, vis.cpu().numpy(), terms.cpu().numpy(), x2, grads


def oracle_grads(ref, displaced):
    pre = 'displaced_grad_' if displaced else 'grad_'
    return {k: ref[pre + k] for k in PARAMS}


@pytest.mark.parametrize('name', UNITS)
def test_fp64_forward_matches_reference(name):
    P, ref, vis, terms, x2, _ = evaluate(name, 'double')
    assert golden_io.rel_err(vis, ref['vis_out']) < TOL['double']['vis']
    # chi^2 terms: the model's agreement amplified by max|model| / max|residual|
    assert golden_io.rel_err(terms, ref['chi_sqrd_terms']) < golden_io.terms_tol(P, ref, 1e-12, 1e-10)
    assert abs(x2 - ref['X2']) <= TOL['double']['X2'] * abs(ref['X2'])


@pytest.mark.parametrize('name', UNITS)
def test_fp32_forward_within_float_tolerance(name):
    P, ref, vis, terms, x2, _ = evaluate(name, 'float')
    assert golden_io.rel_err(vis, ref['vis_out']) < TOL['float']['vis']
    assert norm_err(vis, ref['vis_out']) < VIS_BOUND['native']
    assert golden_io.rel_err(terms, ref['chi_sqrd_terms']) < golden_io.terms_tol(P, ref, 2e-7, TOL['float']['terms'])
    assert abs(x2 - ref['X2']) <= X2_BOUND['native'] * abs(ref['X2'])


@pytest.mark.parametrize('mode', ['split_tf32', 'split_bf16'])
@pytest.mark.parametrize('name', UNITS)
def test_split_forward_error_bound(name, mode):
    _, ref, vis, terms, x2, _ = evaluate(name, 'float', mode)
    err = norm_err(vis, ref['vis_out'])
    assert err < VIS_BOUND[mode], err
    assert abs(x2 - ref['X2']) <= X2_BOUND[mode] * abs(ref['X2']), (x2, ref['X2'])


@pytest.mark.parametrize('displaced', [False, True])
@pytest.mark.parametrize('name', UNITS)
def test_fp64_adjoint_matches_oracle(name, displaced):
    _, ref, _, _, _, g = evaluate(name, 'double', want_grad=True, displaced=displaced)
    og = oracle_grads(ref, displaced)
    for k in PARAMS:
        if og[k].size:
            assert norm_err(g[k], og[k]) < 1e-9, (k, norm_err(g[k], og[k]))


@pytest.mark.parametrize('mode', ['native', 'split_tf32', 'split_bf16'])
@pytest.mark.parametrize('displaced', [False, True])
@pytest.mark.parametrize('name', UNITS)
def test_fp32_gradient_error_bound(name, displaced, mode):
    """Plain FP32 and split-precision gradients against the FP64 oracle."""
    _, ref, _, _, _, g = evaluate(name, 'float', mode, want_grad=True, displaced=displaced)
    og = oracle_grads(ref, displaced)
    bound = (GRAD_BOUND_DISPLACED if displaced else GRAD_BOUND_TRUTH)[mode]
    for k in PARAMS:
        if og[k].size:
            err = norm_err(g[k], og[k])
            assert err < bound, (k, err)

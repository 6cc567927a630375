"""GPU adjoint (mb_rime_adjoint) and the autograd wrapper against the FP64
NumPy gradient and against central finite differences of the GPU FP64
forward at the medium workload size."""
import numpy as np
import pytest

from montblanc_gb300 import synth
from oracle import adjoint as OA
from oracle import rime_v4 as O

pytestmark = pytest.mark.gpu
PARAMS = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term')


def small_problem(seed, use_w, residuals=False, na=6, np_=4, ng=3, ns=2, offset=0.0):
    """Observed = model + noise; with ``offset`` > 0 the gradient is then
    evaluated at source positions displaced by N(0, offset) from the truth.

    At the truth the gradient is a noise-level quantity, and the ~1e-6
    relative FP32 error of the model biases it by about sqrt(N) dM / sigma
    (~1e-3 relative here); FP32 gradients are therefore checked away from
    the optimum, where their relative error is meaningful."""
    P = synth.make_problem(ntime=3, na=na, nchan=5, npsrc=np_, ngsrc=ng, nssrc=ns, seed=seed,
                           beam_shape=(12, 12, 6), random_weights=True, flag_fraction=0.15,
                           antenna_scaling_noise=0.05, use_weight_vector=use_w, residuals=residuals)
    model, _, _ = O.forward(P)
    synth.add_noise(P, model, sigma=0.5, seed=seed + 1)
    P['sigma_sqrd'] = 0.7
    if offset:
        P['lm'] = P['lm'] + np.random.default_rng(seed + 2).normal(0.0, offset, P['lm'].shape)
    return P


def grad_err(g, ref):
    den = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(g - ref)) / den)


@pytest.mark.parametrize('dtype,tol', [('double', 1e-9), ('float', 2e-3)])
@pytest.mark.parametrize('seed,use_w,resid', [(21, True, False), (22, False, False), (23, True, True)])
def test_adjoint_matches_numpy_gradient(dtype, tol, seed, use_w, resid):
    from montblanc_gb300.rime import RimeProblem
    P = small_problem(seed, use_w, resid, offset=0.0 if dtype == 'double' else 2e-4)
    chi2, ref = OA.chi2_grad(P)
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    x2, g = prob.chi2_and_grad()
    assert abs(x2.item() - chi2) <= (1e-10 if dtype == 'double' else 1e-4) * abs(chi2)
    for k in PARAMS:
        if ref[k].size == 0:
            continue
        err = grad_err(g[k].cpu().numpy(), ref[k])
        assert err < tol, (k, err)


def test_adjoint_point_only_and_extended_only():
    from montblanc_gb300.rime import RimeProblem
    for np_, ng, ns in ((5, 0, 0), (0, 3, 3)):
        P = small_problem(31 + np_, True, np_=np_, ng=ng, ns=ns)
        _, ref = OA.chi2_grad(P)
        _, g = RimeProblem.from_numpy(P, dtype='double').chi2_and_grad()
        for k in PARAMS:
            if ref[k].size:
                assert grad_err(g[k].cpu().numpy(), ref[k]) < 1e-9, k


def test_autograd_function():
    import torch
    from montblanc_gb300.rime import RimeProblem, rime_chi2
    P = small_problem(41, True)
    _, ref = OA.chi2_grad(P)
    prob = RimeProblem.from_numpy(P, dtype='double')
    ps = {k: prob.arrays[k].clone().requires_grad_(True) for k in PARAMS}
    x2 = rime_chi2(prob, *(ps[k] for k in PARAMS))
    (3.0 * x2).backward()
    for k in PARAMS:
        if ref[k].size:
            assert grad_err(ps[k].grad.cpu().numpy(), 3.0 * ref[k]) < 1e-9, k


def test_gradient_finite_differences_medium_workload():
    """50 random parameters of the medium workload (100 times, 27 antennas,
    64 channels, 1000 point + 200 gaussian + 50 sersic sources), central
    differences with a 1e-6 relative step of the FP64 GPU forward."""
    import torch
    from montblanc_gb300.rime import RimeProblem
    P = synth.make_problem(**synth.WORKLOADS['medium_mixed'], seed=2024)
    prob = RimeProblem.from_numpy(P, dtype='double')
    model = prob.empty_vis()
    prob.forward(model_vis=model)
    P['observed_vis'] = model.cpu().numpy()
    synth.add_noise(P, P['observed_vis'], sigma=0.1, seed=2025)
    prob.arrays['observed_vis'].copy_(torch.as_tensor(P['observed_vis']))
    x2, g = prob.chi2_and_grad()
    rng = np.random.default_rng(7)
    names = ['lm'] * 10 + ['stokes'] * 10 + ['alpha'] * 8 + ['gauss_shape'] * 8 + ['sersic_shape'] * 6 + \
            ['G_term'] * 8
    checked = 0
    for name in names:
        arr = prob.arrays[name]
        idx = tuple(int(rng.integers(0, n)) for n in arr.shape)
        x0 = arr[idx].item()
        imag = name == 'G_term' and rng.random() < 0.5
        mag = abs(x0) if abs(x0) > 0 else 1.0
        h = 1e-6 * mag
        d = 1j * h if imag else h
        arr[idx] = x0 + d
        fp = prob.forward().item()
        arr[idx] = x0 - d
        fm = prob.forward().item()
        arr[idx] = x0
        num = (fp - fm) / (2 * h)
        an = g[name][idx].item()
        an = an.imag if imag else (an.real if isinstance(an, complex) else an)
        # rounding floor of a central difference of a chi^2 of this size
        fd_noise = 8 * np.finfo(np.float64).eps * abs(x2.item()) / h
        assert abs(an - num) <= 1e-4 * abs(num) + fd_noise, (name, idx, an, num, fd_noise)
        checked += abs(num) > 10 * fd_noise
    # most of the 50 draws must be far enough above the FD floor to count
    assert checked >= 25, checked


@pytest.mark.parametrize('mode', ['split_tf32', 'split_bf16'])
@pytest.mark.parametrize('seed,use_w,mix', [(51, True, (5, 3, 2)), (52, False, (7, 0, 0)),
                                            (53, True, (0, 2, 2))])
def test_split_adjoint_matches_numpy_gradient(mode, seed, use_w, mix):
    """Point-source dJ = Y J on the tensor cores (BF16 hi + lo operands),
    extended sources on the CUDA cores, against the FP64 NumPy gradient."""
    from montblanc_gb300.rime import RimeProblem
    np_, ng, ns = mix
    P = small_problem(seed, use_w, np_=np_, ng=ng, ns=ns, offset=2e-4)
    chi2, ref = OA.chi2_grad(P)
    prob = RimeProblem.from_numpy(P, dtype='float')
    x2, g = prob.chi2_and_grad(mode=mode)
    assert abs(x2.item() - chi2) <= 1e-4 * abs(chi2)
    for k in PARAMS:
        if ref[k].size == 0:
            continue
        err = grad_err(g[k].cpu().numpy(), ref[k])
        assert err < 2e-3, (k, err)

"""The FP64 NumPy adjoint against central finite differences of the forward
oracle (the reference has no gradient, so this pins the adjoint oracle)."""
import numpy as np
import pytest

from montblanc_gb300 import synth
from oracle import adjoint as A
from oracle import rime_v4 as O


def problem(seed=5, use_weight_vector=True, residuals=False):
    P = synth.make_problem(ntime=3, na=5, nchan=4, npsrc=3, ngsrc=2, nssrc=2, seed=seed,
                           beam_shape=(12, 12, 6), random_weights=True, flag_fraction=0.15,
                           antenna_scaling_noise=0.05, use_weight_vector=use_weight_vector,
                           residuals=residuals)
    model, _, _ = O.forward(P)
    synth.add_noise(P, model, sigma=0.5, seed=seed + 1)
    P['sigma_sqrd'] = 0.7
    return P


def chi2_of(P):
    return O.forward(P, src_chunk=7)[2]


def fd(P, name, idx, rel=1e-6, imag=False):
    x = P[name]
    x0 = x[idx]
    h = rel * max(abs(x0), 1e-3 if name != 'lm' else 1e-2)
    d = 1j * h if imag else h
    x[idx] = x0 + d
    fp = chi2_of(P)
    x[idx] = x0 - d
    fm = chi2_of(P)
    x[idx] = x0
    return (fp - fm) / (2 * h)


@pytest.mark.parametrize('use_w', [True, False])
def test_adjoint_oracle_matches_finite_differences(use_w):
    P = problem(use_weight_vector=use_w)
    chi2, g = A.chi2_grad(P, src_chunk=3)
    assert abs(chi2 - chi2_of(P)) <= 1e-12 * abs(chi2)
    rng = np.random.default_rng(0)
    checks = []
    for name in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term'):
        shape = P[name].shape
        for _ in range(5):
            idx = tuple(int(rng.integers(0, n)) for n in shape)
            if name == 'G_term':
                checks.append((g[name][idx].real, fd(P, name, idx)))
                checks.append((g[name][idx].imag, fd(P, name, idx, imag=True)))
            else:
                checks.append((g[name][idx], fd(P, name, idx)))
    scale = max(abs(a) for a, _ in checks)
    for an, num in checks:
        assert abs(an - num) <= 1e-6 * abs(num) + 1e-7 * scale, (an, num)


def test_adjoint_residual_mode_same_gradient():
    P = problem(seed=9)
    c1, g1 = A.chi2_grad(P)
    P['residuals'] = True
    c2, g2 = A.chi2_grad(P)
    assert abs(c1 - c2) < 1e-12 * abs(c1)
    for k in g1:
        assert np.allclose(g1[k], g2[k], rtol=1e-12, atol=0)

"""The CPU oracle against fixtures produced by the reference's own CPUSolver."""
import numpy as np
import pytest

import golden_io
from oracle import rime_v4 as O

ALL = golden_io.names()


def test_fixtures_present():
    assert 'small_fp64' in ALL
    assert len([n for n in ALL if n.startswith('perm_')]) == 14


@pytest.mark.parametrize('name', ALL)
def test_oracle_matches_reference(name):
    P, ref = golden_io.load(name)
    jones = P.get('jones')
    out, terms, X2 = O.forward(P, src_chunk=8, jones=jones)
    # chi^2 terms are squared residuals of nearly equal quantities, so their
    # relative error is that of the model amplified by max|model| /
    # max|residual| (7000 on the 20 500-source units: sums over sources in
    # a different order than the reference's differ by ~1e-14); 1e-10 is
    # the FP64 bar where that amplification is small.
    assert golden_io.rel_err(out, ref['vis_out']) < 1e-11
    assert golden_io.rel_err(terms, ref['chi_sqrd_terms']) < golden_io.terms_tol(P, ref, 1e-13, 1e-10)
    assert abs(X2 - ref['X2']) <= 1e-10 * abs(ref['X2'])
    if 'B_sqrt' in ref:
        assert golden_io.rel_err(O.brightness_sqrt(O.brightness(P)), ref['B_sqrt']) < 1e-13
    ts = slice(*ref['time_slice']) if 'time_slice' in ref else slice(None)
    if 'E_term' in ref:
        assert golden_io.rel_err(O.e_beam(P, times=ts), ref['E_term']) < 1e-12
    if 'jones' in ref:
        assert golden_io.rel_err(O.ekb_sqrt_per_antenna(P, times=ts), ref['jones']) < 1e-11


def test_brightness_sqrt_identities():
    """sqrt(B) sqrt(B) = B and sqrt(B) Hermitian (test_rime_v4.py:279-342)."""
    P, _ = golden_io.load('small_fp64')
    B = O.brightness(P)
    S = O.brightness_sqrt(B)
    S2 = O.jones_mul(S, S)
    assert golden_io.rel_err(S2, B) < 1e-13
    Sm = S.reshape(S.shape[:-1] + (2, 2))
    assert np.allclose(Sm, np.conj(np.swapaxes(Sm, -1, -2)), rtol=0, atol=1e-14)


def test_sqrt_multiply_identity():
    """(J_p sqrt B)(J_q sqrt B)^H = J_p B J_q^H (test_rime_v4.py:422-503)."""
    rng = np.random.default_rng(3)
    J = rng.random((50, 4)) + 1j * rng.random((50, 4))
    K = rng.random((50, 4)) + 1j * rng.random((50, 4))
    P, _ = golden_io.load('small_fp64')
    B = O.brightness(P)[:50 // 10].reshape(-1, 4)[:50]
    S = O.brightness_sqrt(B)
    lhs = O.jones_mul_h(O.jones_mul(J, S), O.jones_mul(K, S))
    rhs = O.jones_mul_h(O.jones_mul(J, B), K)
    assert golden_io.rel_err(lhs, rhs) < 1e-13


def test_jones_multiply_against_matmul():
    """test_rime_v4.py:505-529"""
    rng = np.random.default_rng(4)
    A = rng.random((100, 4)) + 1j * rng.random((100, 4))
    B = rng.random((100, 4)) + 1j * rng.random((100, 4))
    Am, Bm = A.reshape(-1, 2, 2), B.reshape(-1, 2, 2)
    assert np.allclose(O.jones_mul(A, B).reshape(-1, 2, 2), Am @ Bm)
    assert np.allclose(O.jones_mul_h(A, B).reshape(-1, 2, 2), Am @ np.conj(np.swapaxes(Bm, 1, 2)))


def test_source_chunking_is_linear():
    """Summing source chunks gives the same visibilities (v5 batching premise)."""
    P, _ = golden_io.load('perm_p3_g3_s3_w1')
    a = O.ekb_vis(P, src_chunk=9)
    b = O.ekb_vis(P, src_chunk=2, time_chunk=1)
    assert golden_io.rel_err(b, a) < 1e-13

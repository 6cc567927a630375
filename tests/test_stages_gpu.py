"""Per-stage nodes (RimeBSqrt, RimeEBeam, RimeEKBSqrt, RimeSumCoherencies,
RimeReduction) against the reference's own outputs, in the style of
montblanc/tests/test_rime_v4.py: one node at a time through its pipeline."""
import numpy as np
import pytest

import golden_io
from gpu_helpers import TOL, solver_for

pytestmark = pytest.mark.gpu
DTYPES = ('double', 'float')


def _pipeline(*nodes):
    import montblanc_gb300 as mb
    return mb.Pipeline(list(nodes))


@pytest.mark.parametrize('dtype', DTYPES)
@pytest.mark.parametrize('name', ['small_fp64', 'perm_p3_g3_s3_w0', 'residual_w1'])
def test_b_sqrt(name, dtype):
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    with solver_for(P, dtype, _pipeline(mb.RimeBSqrt())) as s:
        s.solve()
        got = s.retrieve_B_sqrt()
    assert golden_io.rel_err(got, ref['B_sqrt']) < TOL[dtype]['bsqrt']
    # sqrt(B) is Hermitian and squares to B (test_rime_v4.py:296-315)
    S = got.astype(np.complex128).reshape(got.shape[:-1] + (2, 2))
    assert np.allclose(S, np.conj(np.swapaxes(S, -1, -2)), atol=1e-6)


@pytest.mark.parametrize('dtype', DTYPES)
@pytest.mark.parametrize('name', ['ebeam_odd', 'ebeam_2x2x2', 'small_fp64'])
def test_e_beam(name, dtype):
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    with solver_for(P, dtype, _pipeline(mb.RimeEBeam())) as s:
        s.solve()
        got = s.retrieve_jones()
    if 'time_slice' in ref:
        got = got[:, slice(*ref['time_slice'])]
    tol = 1e-10 if dtype == 'double' else 1e-4
    assert golden_io.rel_err(got, ref['E_term']) < tol
    assert np.count_nonzero(ref['E_term']) / ref['E_term'].size > 0.85


@pytest.mark.parametrize('dtype', DTYPES)
@pytest.mark.parametrize('name', ['ebeam_odd', 'perm_p3_g3_s3_w1', 'small_fp64'])
def test_ekb_sqrt(name, dtype):
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    with solver_for(P, dtype, _pipeline(mb.RimeEBeam(), mb.RimeBSqrt(), mb.RimeEKBSqrt())) as s:
        s.solve()
        got = s.retrieve_jones()
    if 'time_slice' in ref:
        got = got[:, slice(*ref['time_slice'])]
    assert golden_io.rel_err(got, ref['jones']) < TOL[dtype]['jones']


def _check_vis(s, ref, dtype):
    assert golden_io.rel_err(s.retrieve_model_vis(), ref['vis_out']) < TOL[dtype]['vis']
    assert golden_io.rel_err(s.retrieve_chi_sqrd_result(), ref['chi_sqrd_terms']) < TOL[dtype]['terms']
    assert abs(s.X2 - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])


SUM_CASES = [n for n in golden_io.names() if n.startswith(('perm_', 'residual_'))] + ['given_jones']


@pytest.mark.parametrize('dtype', DTYPES)
@pytest.mark.parametrize('name', SUM_CASES)
def test_sum_coherencies(name, dtype):
    """Coherency sum + G + chi^2 on the reference's per-antenna terms for
    every source-type mix, weights on/off and residual output
    (test_rime_v4.py:181-277)."""
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    jones = P['jones'] if 'jones' in P else ref['jones']
    with solver_for(P, dtype, _pipeline(mb.RimeSumCoherencies())) as s:
        s.transfer_jones(jones)
        s.solve()
        _check_vis(s, ref, dtype)


@pytest.mark.parametrize('dtype', DTYPES)
def test_four_node_pipeline(dtype):
    """The reference's default v4 pipeline end to end."""
    import montblanc_gb300 as mb
    P, ref = golden_io.load('small_fp64')
    with solver_for(P, dtype, mb.stage_pipeline()) as s:
        s.solve()
        _check_vis(s, ref, dtype)


@pytest.mark.parametrize('dtype', DTYPES)
def test_source_batches_accumulate(dtype):
    """Two source batches (lower/upper extents) give the single-batch result
    (RimeSumCoherencies.py:185-190, 311-316)."""
    import montblanc_gb300 as mb
    P, ref = golden_io.load('perm_p3_g3_s3_w1')
    jones = ref['jones']
    with solver_for(P, dtype, _pipeline(mb.RimeSumCoherencies())) as s:
        nsrc = s.dim_global_size('nsrc')
        # batch 1: point sources [0, 3)
        s.transfer_jones(jones)
        for dim, lo, hi in (('nsrc', 0, 3), ('npsrc', 0, 3), ('ngsrc', 0, 0), ('nssrc', 0, 0)):
            s.update_dimension(dim, lower_extent=lo, upper_extent=hi)
        s.solve()
        # batch 2: the remaining sources, presented as a shifted array
        shifted = np.zeros_like(jones)
        shifted[:nsrc - 3] = jones[3:]
        s.transfer_jones(shifted)
        g = P['gauss_shape']
        x = P['sersic_shape']
        s.update_dimension('nsrc', lower_extent=3, upper_extent=nsrc)
        s.update_dimension('npsrc', lower_extent=0, upper_extent=0)
        s.update_dimension('ngsrc', lower_extent=0, upper_extent=3)
        s.update_dimension('nssrc', lower_extent=0, upper_extent=3)
        s.solve()
        _check_vis(s, ref, dtype)


@pytest.mark.parametrize('dtype', DTYPES)
def test_rime_reduction(dtype):
    import montblanc_gb300 as mb
    P, ref = golden_io.load('perm_p3_g3_s0_w1')
    with solver_for(P, dtype, _pipeline(mb.RimeSumCoherencies())) as s:
        s.transfer_jones(ref['jones'])
        s.solve()
        red = mb.RimeReduction()
        red.initialise(s)
        x2 = red.execute(s).item()
    assert abs(x2 - ref['X2']) <= TOL[dtype]['X2'] * abs(ref['X2'])

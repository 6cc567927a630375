"""Streaming (v5-semantics) solver: chunk and batch planning and array
handling on the CPU; on the GPU, agreement with the device-resident v4
solver and the reference's v5 behaviours (montblanc/tests/test_rime_v5.py:
73-151: visibility write modes, supplied arrays)."""
import numpy as np
import pytest

from montblanc_gb300 import composite as C


def test_vis_chunks_cover_the_space_once():
    for ntime, nchan, nt, nc in ((7, 5, 3, 2), (10, 16, 10, 16), (1, 1, 4, 4), (9, 4, 2, 3)):
        seen = np.zeros((ntime, nchan), dtype=int)
        for t0, t1, c0, c1 in C.gen_vis_chunks(ntime, nchan, nt, nc):
            assert 0 <= t0 < t1 <= ntime and 0 <= c0 < c1 <= nchan
            assert t1 - t0 <= nt and c1 - c0 <= nc
            seen[t0:t1, c0:c1] += 1
        assert (seen == 1).all()


@pytest.mark.parametrize('counts,batch', [((10, 10, 10), 7), ((3, 0, 5), 2), ((0, 4, 0), 10), ((5, 5, 5), 1)])
def test_source_batches_follow_type_order(counts, batch):
    c = dict(zip(('npsrc', 'ngsrc', 'nssrc'), counts))
    types = np.repeat([0, 1, 2], counts)
    index = np.concatenate([np.arange(n) for n in counts])
    covered = []
    for s0, s1, per in C.gen_source_batches(c, batch):
        assert s1 - s0 == sum(n for _, n in per.values()) and s1 - s0 <= batch
        k = s0
        for ti, v in enumerate(('npsrc', 'ngsrc', 'nssrc')):
            first, n = per[v]
            for j in range(n):
                assert types[k] == ti and index[k] == first + j
                k += 1
        covered.extend(range(s0, s1))
    assert covered == list(range(sum(counts)))


def test_plan_chunks_fits_the_budget():
    def per(nt, nc):
        return nt * nc * 1000 + 100
    for budget in (2500, 10_000, 123_456, 10**9):
        nt, nc = C.plan_chunks(64, 32, per, budget, 2)
        assert 1 <= nt <= 64 and 1 <= nc <= 32
        assert per(nt, nc) * 2 <= budget
    assert C.plan_chunks(64, 32, per, 10**9, 2) == (64, 32)
    with pytest.raises(ValueError):
        C.plan_chunks(64, 32, per, 1000, 2)


def _cfg(**kw):
    import montblanc_gb300 as mb
    base = dict(na=7, ntime=6, nchan=5, sources=mb.sources(point=4, gaussian=3, sersic=2),
                beam_lw=9, beam_mh=8, beam_nud=5, dtype='double', version='v5', data_source='test',
                vis_chunk=(4, 2), source_batch_size=4, nsolvers=2)
    base.update(kw)
    return mb.rime_solver_cfg(**base)


def test_supplied_and_ignored_arrays():
    """Supplied arrays are used as given (dtype kept), bad shapes raise
    ValueError, ignored arrays are not created (test_rime_v5.py:107-151)."""
    import montblanc_gb300 as mb
    uvw = np.zeros((6, 7, 3), dtype=np.float32)
    vis = np.zeros((6, 21, 5, 4), dtype=np.complex64)
    s = mb.rime_solver(_cfg(array_cfg={'supplied': {'uvw': uvw, 'model_vis': vis}, 'ignore': ['weight_vector']}))
    assert isinstance(s, C.CompositeRimeSolver)
    assert s.uvw is uvw and s.model_vis.dtype == np.complex64
    assert s.observed_vis.dtype == np.complex128
    assert np.count_nonzero(s.lm) > 0.9 * s.lm.size
    assert 'weight_vector' not in s.arrays()
    with pytest.raises(ValueError):
        mb.rime_solver(_cfg(array_cfg={'supplied': {'uvw': np.zeros((6, 6, 3))}}))
    with pytest.raises(ValueError):
        mb.rime_solver(_cfg(array_cfg={'supplied': {'not_an_array': np.zeros(3)}}))
    assert s.chunk_shape() == (4, 2)
    assert len(s.vis_chunks()) == 2 * 3 and len(s.source_batches()) == 3


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
ARRAYS = ('uvw', 'antenna1', 'antenna2', 'frequency', 'ref_frequency', 'parallactic_angles', 'point_errors',
          'antenna_scaling', 'E_beam', 'G_term', 'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'flag',
          'weight_vector', 'observed_vis')


def _v4_twin(s5, dtype, **kw):
    """A device-resident v4 solver holding the v5 solver's arrays."""
    import montblanc_gb300 as mb
    d = s5.dimensions()
    c = mb.rime_solver_cfg(na=d['na'].local_size, ntime=d['ntime'].local_size, nchan=d['nchan'].local_size,
                           sources=mb.sources(point=d['npsrc'].local_size, gaussian=d['ngsrc'].local_size,
                                              sersic=d['nssrc'].local_size),
                           beam_lw=d['beam_lw'].local_size, beam_mh=d['beam_mh'].local_size,
                           beam_nud=d['beam_nud'].local_size, dtype=dtype, data_source='empty', **kw)
    s4 = mb.rime_solver(c)
    for n in ARRAYS:
        if n in s5.arrays():
            getattr(s4, 'transfer_' + n)(s5.arrays()[n])
    return s4


@pytest.mark.gpu
@pytest.mark.parametrize('dtype,wv,out', [('double', True, 'model'), ('double', False, 'residuals'),
                                          ('float', True, 'model')])
def test_streaming_matches_resident_solver(dtype, wv, out):
    """Chunked (time x channel) and source-batched solve == one v4 solve."""
    import montblanc_gb300 as mb
    np.random.seed(5)
    s5 = mb.rime_solver(_cfg(dtype=dtype, weight_vector=wv, vis_output=out))
    s5.set_sigma_sqrd(2.5)
    s5.solve()
    with _v4_twin(s5, dtype, weight_vector=wv, vis_output=out) as s4:
        s4.set_sigma_sqrd(2.5)
        s4.solve()
        ref = s4.retrieve_model_vis()
        tol = 1e-10 if dtype == 'double' else 2e-5
        assert np.abs(s5.model_vis - ref).max() <= tol * np.abs(ref).max()
        assert abs(s5.X2 - s4.X2) <= (1e-10 if dtype == 'double' else 1e-4) * abs(s4.X2)


@pytest.mark.gpu
def test_visibility_write_mode():
    """test_rime_v5.py:73-104: overwrite repeats, sum accumulates."""
    import montblanc_gb300 as mb
    np.random.seed(6)
    s = mb.rime_solver(_cfg(vis_write_mode='overwrite'))
    s.solve()
    vis = s.model_vis.copy()
    s.solve()
    assert np.allclose(vis, s.model_vis)
    np.random.seed(6)
    s = mb.rime_solver(_cfg(vis_write_mode='sum'))
    s.solve()
    vis = s.model_vis.copy()
    for _ in range(4):
        s.solve()
    assert np.allclose(5 * vis, s.model_vis)


@pytest.mark.gpu
def test_single_precision_supplied_arrays_on_double_solver():
    """test_rime_v5.py:139-151: complex64 model_vis and float32 uvw supplied
    to a double-precision solver."""
    import montblanc_gb300 as mb
    np.random.seed(7)
    vis = np.zeros((6, 21, 5, 4), dtype=np.complex64)
    s = mb.rime_solver(_cfg(array_cfg={'supplied': {'model_vis': vis}}))
    assert s.model_vis.dtype == np.complex64 and s.observed_vis.dtype == np.complex128
    s.solve()
    with _v4_twin(s, 'double') as s4:
        s4.solve()
        ref = s4.retrieve_model_vis()
        assert np.abs(s.model_vis - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.gpu
def test_streaming_gradient_matches_whole_problem():
    """chi^2 and its gradient streamed in chunks == one fused call."""
    import montblanc_gb300 as mb
    from montblanc_gb300.rime import RimeProblem
    np.random.seed(8)
    s = mb.rime_solver(_cfg(weight_vector=True))
    grads = s.solve_with_gradient()
    A = s.arrays()
    P = {n: A[n] for n in ARRAYS}
    d = s.dimensions()
    P.update(npsrc=d['npsrc'].local_size, ngsrc=d['ngsrc'].local_size, nssrc=d['nssrc'].local_size,
             use_weight_vector=True, residuals=False)
    for n in ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm', 'beam_lfreq', 'beam_ul',
              'beam_um', 'beam_ufreq'):
        P[n] = float(getattr(s, n))
    prob = RimeProblem.from_numpy(P, dtype='double')
    x2, g = prob.chi2_and_grad()
    assert abs(s.X2 - x2.item()) <= 1e-10 * abs(x2.item())
    for n in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term'):
        ref = g[n].cpu().numpy()
        assert np.abs(grads[n] - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1e-300), n


@pytest.mark.gpu
@pytest.mark.parametrize('name, chunk, nbatch', [('units_medium_mixed', (2, 2), 5), ('wide_na75', (2, 1), 1)])
def test_streaming_matches_reference_fixture(name, chunk, nbatch):
    """The streamed solve of 3 time steps x 3 channels of the 100 x 27 x 64
    workload (all 1250 sources, tests/golden/units_medium_mixed, outputs of
    the reference's CPUSolver) in (2, 2) visibility chunks and 300-source
    batches, and the 75-antenna array of tests/golden/wide_na75 (weights,
    flags; antenna sub-arrays inside each chunk): model visibilities,
    chi^2 terms and chi^2 against the reference, the streamed gradient
    against the FP64 oracle's."""
    import golden_io
    import montblanc_gb300 as mb
    P, ref = golden_io.load(name)
    ntime, na = P['uvw'].shape[:2]
    lw, mh, nud = P['E_beam'].shape[:3]
    supplied = {n: P[n] for n in ARRAYS}
    cfg = mb.rime_solver_cfg(na=na, ntime=ntime, nchan=P['frequency'].shape[0], nbl=P['antenna1'].shape[1],
                             sources=mb.sources(point=P['npsrc'], gaussian=P['ngsrc'], sersic=P['nssrc']),
                             beam_lw=lw, beam_mh=mh, beam_nud=nud, dtype='double', version='v5',
                             data_source='empty', vis_chunk=chunk, source_batch_size=300, nsolvers=2,
                             weight_vector=bool(P['use_weight_vector']), array_cfg={'supplied': supplied})
    s = mb.rime_solver(cfg)
    for n in ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm', 'beam_lfreq', 'beam_ul',
              'beam_um', 'beam_ufreq'):
        getattr(s, 'set_' + n)(P[n])
    assert len(s.vis_chunks()) == 4 and len(s.source_batches()) == nbatch
    s.solve()
    assert golden_io.rel_err(s.model_vis, ref['vis_out']) < 1e-10
    assert abs(s.X2 - ref['X2']) <= 1e-10 * abs(ref['X2'])
    grads = s.solve_with_gradient()
    assert abs(s.X2 - ref['X2']) <= 1e-10 * abs(ref['X2'])
    for n in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term'):
        g = ref['grad_' + n]
        assert np.linalg.norm(grads[n] - g) <= 1e-9 * np.linalg.norm(g), n

"""MeasurementSet input (montblanc/impl/common/loaders/loaders.py:35-137,
montblanc/impl/rime/v4/loaders/loaders.py:49-246) on an in-memory
MeasurementSet whose rows are shuffled and include auto-correlations, a
second field and two bands mapped through DATA_DESCRIPTION.  The expected
arrays are built from the generating values, not from the loader's logic."""
import numpy as np
import pytest

from montblanc_gb300 import ms, util

NA, NTIME, CPB = 5, 3, 3
SPW_OF_DDID = np.array([1, 0])  # data description 0 -> band 1, 1 -> band 0


def _ms(seed=0, weight_spectrum=True, sigma=True, ra=-0.4, num_chan=(CPB, CPB)):
    rng = np.random.default_rng(seed)
    lat, lon = np.radians(-30.7), np.radians(21.4)
    a, f = util.WGS84_A, util.WGS84_F
    e2 = f * (2 - f)
    nrad = a / np.sqrt(1 - e2 * np.sin(lat) ** 2)
    centre = np.array([nrad * np.cos(lat) * np.cos(lon), nrad * np.cos(lat) * np.sin(lon), nrad * (1 - e2) * np.sin(lat)])
    pos = centre + rng.normal(0, 500.0, (NA, 3))
    times = 4.9e9 + np.arange(NTIME) * 8.0
    ant_uvw = rng.normal(0, 300.0, (NTIME, NA, 3))
    freqs = np.array([1.30e9, 1.31e9, 1.32e9, 1.40e9, 1.41e9, 1.42e9]).reshape(2, CPB)
    rows = []
    for ti in range(NTIME):
        for p in range(NA):
            for q in range(p, NA):
                for ddid in (0, 1):
                    for field in (0, 1):
                        rows.append((ti, p, q, ddid, field))
    rows = [rows[i] for i in rng.permutation(len(rows))]
    n = len(rows)
    ti, p, q, dd, fld = (np.array(c) for c in zip(*rows))
    cols = {'TIME': times[ti], 'ANTENNA1': p, 'ANTENNA2': q, 'DATA_DESC_ID': dd, 'FIELD_ID': fld,
            'UVW': ant_uvw[ti, q] - ant_uvw[ti, p],
            'DATA': rng.normal(size=(n, CPB, 4)) + 1j * rng.normal(size=(n, CPB, 4)),
            'FLAG': rng.uniform(size=(n, CPB, 4)) < 0.2,
            'FLAG_ROW': rng.uniform(size=n) < 0.1,
            'WEIGHT': rng.uniform(0.5, 2.0, (n, 4))}
    if weight_spectrum:
        cols['WEIGHT_SPECTRUM'] = rng.uniform(0.5, 2.0, (n, CPB, 4))
    if sigma:
        cols['SIGMA'] = rng.uniform(0.1, 0.3, (n, 4))
    tables = {
        'MAIN': cols,
        'ANTENNA': {'POSITION': pos},
        'SPECTRAL_WINDOW': {'CHAN_FREQ': freqs, 'NUM_CHAN': np.array(num_chan), 'REF_FREQUENCY': freqs[:, 0]},
        'FIELD': {'PHASE_DIR': np.array([[[ra, -0.5]], [[1.0, 0.2]]])},
        'DATA_DESCRIPTION': {'SPECTRAL_WINDOW_ID': SPW_OF_DDID},
    }
    truth = dict(pos=pos, times=times, ant_uvw=ant_uvw, freqs=freqs, rows=rows, ra=ra)
    return tables, truth


def _expected_vis(tables, truth, name, auto=False):
    """(ntime, nbl, nchan, 4) array of main-table column ``name``, placed by
    looking up each (time, p, q, band, channel) directly."""
    cols = tables['MAIN']
    pairs = [(p, q) for p in range(NA) for q in range(p if auto else p + 1, NA)]
    out = np.zeros((NTIME, len(pairs), 2 * CPB) + cols[name].shape[2:], dtype=cols[name].dtype)
    for r, (ti, p, q, dd, fld) in enumerate(truth['rows']):
        if fld != 0 or (p, q) not in pairs:
            continue
        band = SPW_OF_DDID[dd]
        out[ti, pairs.index((p, q)), band * CPB:(band + 1) * CPB] = cols[name][r]
    return out, pairs


def test_dims_and_frequencies():
    tables, truth = _ms()
    with ms.MeasurementSetLoader(tables) as L:
        assert L.get_dims() == (NTIME, NA * (NA - 1) // 2, NA, 2, 2 * CPB)
        A = L.arrays()
    np.testing.assert_array_equal(A['frequency'], truth['freqs'].reshape(-1))
    np.testing.assert_array_equal(A['ref_frequency'], np.repeat(truth['freqs'][:, 0], CPB))
    with ms.MeasurementSetLoader(tables, auto_correlations=True) as L:
        assert L.get_dims()[:3] == (NTIME, NA * (NA + 1) // 2, NA)


def test_uvw_antennas_and_parallactic_angles():
    tables, truth = _ms()
    A = ms.MeasurementSetLoader(tables).arrays()
    pairs = [(p, q) for p in range(NA) for q in range(p + 1, NA)]
    np.testing.assert_array_equal(A['antenna1'], np.tile([p for p, _ in pairs], (NTIME, 1)))
    np.testing.assert_array_equal(A['antenna2'], np.tile([q for _, q in pairs], (NTIME, 1)))
    assert A['antenna1'].dtype == np.int32
    # antenna 0 at the origin, the rest relative to it; baselines are differences
    np.testing.assert_allclose(A['uvw'], truth['ant_uvw'] - truth['ant_uvw'][:, :1], atol=1e-9)
    for j, (p, q) in enumerate(pairs):
        np.testing.assert_allclose(A['uvw'][:, q] - A['uvw'][:, p],
                                   truth['ant_uvw'][:, q] - truth['ant_uvw'][:, p], atol=1e-9)
    ref = util.parallactic_angles(np.array([truth['ra'] + 2 * np.pi, -0.5]), truth['pos'], truth['times'])
    np.testing.assert_allclose(A['parallactic_angles'], ref, atol=1e-12)
    assert A['parallactic_angles'].shape == (NTIME, NA)


def test_visibilities_and_flags():
    tables, truth = _ms()
    A = ms.MeasurementSetLoader(tables).arrays()
    vis, _ = _expected_vis(tables, truth, 'DATA')
    np.testing.assert_array_equal(A['observed_vis'], vis)
    flag, _ = _expected_vis(tables, truth, 'FLAG')
    cols = tables['MAIN']
    tables['MAIN'] = dict(cols, FLAG=np.broadcast_to(cols['FLAG_ROW'][:, None, None], cols['FLAG'].shape))
    frow, _ = _expected_vis(tables, truth, 'FLAG')
    np.testing.assert_array_equal(A['flag'], (flag | frow).astype(np.uint8))
    assert 'weight_vector' not in A


@pytest.mark.parametrize('init,spectrum,sigma,source', [('weight', True, True, 'WEIGHT_SPECTRUM'),
                                                        ('weight', False, True, 'WEIGHT'),
                                                        ('sigma', True, True, 'SIGMA'),
                                                        ('sigma', True, False, None)])
def test_weight_initialisation(init, spectrum, sigma, source):
    tables, truth = _ms(weight_spectrum=spectrum, sigma=sigma)
    A = ms.MeasurementSetLoader(tables).arrays(init_weights=init)
    cols = tables['MAIN']
    if source is None:
        expected = np.ones_like(A['weight_vector'])
    else:
        col = cols[source]
        if col.ndim == 2:  # per row and correlation: the same for every channel
            tables['MAIN'] = dict(cols, **{source: np.repeat(col[:, None, :], CPB, axis=1)})
        expected, _ = _expected_vis(tables, truth, source)
    np.testing.assert_array_equal(A['weight_vector'], expected)


def test_rejects_unequal_bands_and_missing_tables():
    tables, _ = _ms(num_chan=(CPB, CPB + 1))
    with pytest.raises(ValueError):
        ms.MeasurementSetLoader(tables)
    tables, _ = _ms()
    del tables['FIELD']
    with pytest.raises(KeyError):
        ms.MeasurementSetLoader(tables)
    with pytest.raises(ValueError):
        ms.MeasurementSetLoader(_ms()[0]).arrays(init_weights='bogus')


def test_path_needs_casacore(tmp_path):
    try:
        import casacore.tables  # noqa: F401
        pytest.skip('python-casacore is installed')
    except ImportError:
        pass
    with pytest.raises(ImportError):
        ms.MeasurementSetLoader(str(tmp_path / 'missing.ms'))


def test_factory_requires_msfile():
    import montblanc_gb300 as mb
    with pytest.raises(KeyError):
        mb.rime_solver(mb.rime_solver_cfg(data_source='ms'))


@pytest.mark.gpu
@pytest.mark.parametrize('version', ['v4', 'v5'])
def test_solver_from_measurement_set(version):
    """rime_solver(data_source='ms') sizes the solver from the MeasurementSet,
    holds the loader's arrays (cast to the solver's dtypes) and solves."""
    import montblanc_gb300 as mb
    tables, _ = _ms()
    cfg = mb.rime_solver_cfg(data_source='ms', msfile=tables, sources=mb.sources(point=3, gaussian=1),
                             dtype='double', version=version, init_weights='weight', weight_vector=True)
    s = mb.rime_solver(cfg)
    d = s.dimensions()
    assert (d['ntime'].global_size, d['na'].global_size, d['nbl'].global_size, d['nchan'].global_size) == \
        (NTIME, NA, NA * (NA - 1) // 2, 2 * CPB)
    A = ms.MeasurementSetLoader(tables).arrays(init_weights='weight')
    got = s.arrays()
    for name in ('uvw', 'antenna1', 'frequency', 'observed_vis', 'flag', 'weight_vector'):
        g = got[name]
        g = g.cpu().numpy() if hasattr(g, 'cpu') else np.asarray(g)
        np.testing.assert_array_equal(g, A[name].astype(g.dtype))
    s.solve()
    assert np.isfinite(s.X2)


def test_path_branch_with_a_casacore_stand_in(monkeypatch):
    """A MeasurementSet path goes through casacore.tables: table(path) for
    MAIN and table('path::NAME') for each sub-table, opened read-only, then
    colnames / getcol / nrows / close.  A stand-in module serves the
    in-memory tables under those names."""
    import sys
    import types
    tables, truth = _ms()
    opened, closed = [], []

    class Table(object):
        def __init__(self, path, ack=True, readonly=False):
            assert ack is False and readonly is True
            name = path.split('::')[1] if '::' in path else 'MAIN'
            assert path.split('::')[0] == '/data/obs.ms'
            self.cols = tables[name]
            opened.append(name)

        def colnames(self):
            return list(self.cols)

        def getcol(self, name):
            return self.cols[name]

        def nrows(self):
            return len(next(iter(self.cols.values())))

        def close(self):
            closed.append(1)

    mod = types.ModuleType('casacore.tables')
    mod.table = Table
    pkg = types.ModuleType('casacore')
    pkg.tables = mod
    monkeypatch.setitem(sys.modules, 'casacore', pkg)
    monkeypatch.setitem(sys.modules, 'casacore.tables', mod)
    with ms.MeasurementSetLoader('/data/obs.ms') as L:
        assert L.get_dims() == (NTIME, NA * (NA - 1) // 2, NA, 2, 2 * CPB)
        A = L.arrays(init_weights='weight')
    assert sorted(opened) == sorted(['MAIN'] + list(ms.SUBTABLES))
    assert len(closed) == len(opened)
    B = ms.MeasurementSetLoader(tables).arrays(init_weights='weight')
    for k in B:
        np.testing.assert_array_equal(A[k], B[k])

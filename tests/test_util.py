"""Sky-model parsing and parallactic angles (host-side input preparation).

The sky-model case is the reference's known-answer test
(montblanc/tests/test_utils.py:164-203).  Parallactic angles have no
casacore here, so the formula is checked against an independent vector
construction, the geodetic conversion by its inverse, and sidereal time
against its published value at J2000.0."""
import numpy as np
import pytest

from montblanc_gb300 import util


def _write(tmp_path, text):
    p = tmp_path / 'sky.txt'
    p.write_text(text)
    return str(p)


def test_sky_model_known_answer(tmp_path):
    fn = _write(tmp_path, '# format npsrc: l, m, I, Q, U, V\n'
                          '11, 12, 13, 14, 15, 16\n'
                          '21, 22, 23, 24, 25, 26\n'
                          '# format ngsrc: l, m, I, Q, U, V, el, em, eR\n'
                          '31, 32, 33, 34, 35, 36, 37, 38, 39\n'
                          '41, 42, 43, 44, 45, 46, 47, 48, 49\n')
    r = util.parse_sky_model(fn)
    A, S = r.arrays, r.src_counts
    assert S == {'npsrc': 2, 'ngsrc': 2}
    assert A['l'] == ['11', '21', '31', '41'] and A['m'] == ['12', '22', '32', '42']
    assert A['I'] == ['13', '23', '33', '43'] and A['V'] == ['16', '26', '36', '46']
    assert A['el'] == ['37', '47'] and A['em'] == ['38', '48'] and A['eR'] == ['39', '49']
    ft = np.float32
    shape = (2, S['npsrc'] + S['ngsrc'])
    ary = r.shape_arrays(['l', 'm'], shape, ft)
    assert ary.shape == shape and ary.dtype == ft
    assert np.all(ary[0] == ((np.arange(4) + 1) * 10 + 1).astype(ft))
    assert np.all(ary[1] == ((np.arange(4) + 1) * 10 + 2).astype(ft))


def test_sky_model_arrays_order_defaults_and_blank_lines(tmp_path):
    fn = _write(tmp_path, '# format ngsrc: l, m, I, el, em, eR\n'
                          '0.01, 0.02, 3.0, 1e-5, 2e-5, 0.7\n'
                          '\n'
                          '# format npsrc: l, m, I, Q, U, V, alpha\n'
                          '0.03, 0.04, 2.0, 0.1, 0.2, 0.3, -0.7\n'
                          '0.05, 0.06, 1.0, 0.0, 0.0, 0.0, 0.5, 99\n'
                          '# format nssrc: l, m, I, e1, e2, eS\n'
                          '0.07, 0.08, 4.0, 0.1, -0.2, 3e-5\n')
    r = util.parse_sky_model(fn)
    out = util.sky_model_arrays(r, ntime=3)
    assert out['sources'] == {'point': 2, 'gaussian': 1, 'sersic': 1}
    # point sources first (file order within a type), then gaussian, sersic
    np.testing.assert_array_equal(out['lm'], [[0.03, 0.04], [0.05, 0.06], [0.01, 0.02], [0.07, 0.08]])
    assert out['stokes'].shape == (4, 3, 4) and out['alpha'].shape == (4, 3)
    np.testing.assert_array_equal(out['stokes'][0, 2], [2.0, 0.1, 0.2, 0.3])
    np.testing.assert_array_equal(out['stokes'][2, 0], [3.0, 0.0, 0.0, 0.0])  # Q, U, V default 0
    np.testing.assert_array_equal(out['alpha'][:, 1], [-0.7, 0.5, 0.0, 0.0])
    np.testing.assert_array_equal(out['gauss_shape'][:, 0], [1e-5, 2e-5, 0.7])
    np.testing.assert_array_equal(out['sersic_shape'][:, 0], [0.1, -0.2, 3e-5])


def test_sky_model_rejects_unknown_source_type(tmp_path):
    fn = _write(tmp_path, '# format nqsrc: l, m, I\n0.1, 0.2, 1\n')
    with pytest.raises(ValueError):
        util.sky_model_arrays(util.parse_sky_model(fn), ntime=1)


def _pa_by_vectors(H, dec, lat):
    """Position angle (north through east) of the zenith seen from the
    direction (H, dec), from unit vectors in the (hour-angle) equatorial frame."""
    def unit(h, d):
        # x towards the meridian on the equator, y towards hour angle -6 h (east), z the pole
        return np.array([np.cos(d) * np.cos(h), -np.cos(d) * np.sin(h), np.sin(d)])
    s = unit(H, dec)
    zen = unit(0.0, lat)
    pole = np.array([0.0, 0.0, 1.0])
    north = pole - s * (s @ pole)
    north /= np.linalg.norm(north)
    east = np.cross(pole, s)
    east /= np.linalg.norm(east)
    return np.arctan2(zen @ east, zen @ north)


def test_parallactic_angle_formula_against_vectors():
    rng = np.random.default_rng(1)
    for _ in range(200):
        H = rng.uniform(-np.pi, np.pi)
        dec = rng.uniform(-1.4, 1.4)
        lat = rng.uniform(-1.4, 1.4)
        q = util.parallactic_angle(H, dec, lat)
        ref = _pa_by_vectors(H, dec, lat)
        assert abs(np.angle(np.exp(1j * (q - ref)))) < 1e-12
    # transit south of the zenith: 0; antisymmetric in the hour angle
    assert abs(util.parallactic_angle(0.0, -0.5, -0.3)) < 1e-15
    assert abs(util.parallactic_angle(0.7, -0.5, -0.3) + util.parallactic_angle(-0.7, -0.5, -0.3)) < 1e-15


def test_geodetic_round_trip():
    rng = np.random.default_rng(2)
    lon = rng.uniform(-np.pi, np.pi, 50)
    lat = rng.uniform(-1.5, 1.5, 50)
    h = rng.uniform(-100.0, 5000.0, 50)
    e2 = util.WGS84_F * (2 - util.WGS84_F)
    nrad = util.WGS84_A / np.sqrt(1 - e2 * np.sin(lat) ** 2)
    xyz = np.stack([(nrad + h) * np.cos(lat) * np.cos(lon), (nrad + h) * np.cos(lat) * np.sin(lon),
                    (nrad * (1 - e2) + h) * np.sin(lat)], axis=1)
    lo, la, hh = util.itrf_to_geodetic(xyz)
    np.testing.assert_allclose(lo, lon, atol=1e-12)
    np.testing.assert_allclose(la, lat, atol=1e-12)
    np.testing.assert_allclose(hh, h, atol=1e-5)


def test_gmst_at_j2000():
    """GMST at 2000-01-01 12:00 UT1 is 18h41m50.548s (280.46062 deg)."""
    t = 51544.5 * 86400.0
    g = np.degrees(util.gmst(t))
    assert abs(g - 280.46061837) < 2e-5
    # one sidereal day later the angle repeats
    assert abs(np.angle(np.exp(1j * (util.gmst(t + 86164.0905) - util.gmst(t))))) < 1e-6


def test_precession_is_a_rotation():
    t = np.array([51544.5 * 86400.0, 60000.0 * 86400.0])
    ra, dec = util.precess_j2000(np.array([1.0, 1.0]), np.array([-0.4, -0.4]), t)
    assert abs(ra[0] - 1.0) < 1e-6 and abs(dec[0] + 0.4) < 1e-6
    # separations are preserved
    a = util.precess_j2000(0.3, 0.2, t[1])
    b = util.precess_j2000(2.1, -0.9, t[1])

    def vec(r, d):
        return np.array([np.cos(d) * np.cos(r), np.cos(d) * np.sin(r), np.sin(d)])
    assert abs(vec(*a) @ vec(*b) - vec(0.3, 0.2) @ vec(2.1, -0.9)) < 1e-12


def test_parallactic_angles_shape_and_transit():
    # antenna on the equator at longitude 0 looking at dec -30 deg
    pos = np.array([[util.WGS84_A, 0.0, 0.0], [util.WGS84_A * np.cos(0.3), util.WGS84_A * np.sin(0.3), 0.0]])
    t0 = 59000.0 * 86400.0
    times = t0 + np.arange(5) * 3600.0
    fc = np.array([1.2, -np.pi / 6])
    pa = util.parallactic_angles(fc, pos, times)
    assert pa.shape == (5, 2) and np.isfinite(pa).all()
    # from the equator the zenith lies on the hour circle through the pole, at +-90 deg off transit
    ra_d, dec_d = util.precess_j2000(fc[0], fc[1], times)
    ha = util.gmst(times) - ra_d
    np.testing.assert_allclose(pa[:, 0], util.parallactic_angle(ha, dec_d, 0.0), atol=1e-12)


def test_parallactic_angle_error_from_omitted_terms():
    """Moving the direction by the summed omitted terms (nutation,
    aberration, UT1 - UTC, polar motion: 60.9" = 2.95e-4 rad) changes the
    parallactic angle by no more than e (tan(elevation) + |tan(dec)|).  For
    the generator's field (dec -30 deg) at elevations up to 60 degrees that
    is 6.8e-4 rad, which moves a source 0.07 rad from the field centre by
    4.8e-5 rad on the beam and changes the synthetic 50 x 50 x 32 beam's E
    by at most 1.5e-3 of its largest value (5e-5 norm-wise over the sources
    of the test sky)."""
    from montblanc_gb300 import util, synth
    from oracle import rime_v4 as O
    e = util.omitted_direction_error()
    assert abs(e - 60.89762 * util.ARCSEC) < 1e-12
    lat = np.deg2rad(-30.0)
    rng = np.random.default_rng(3)
    for _ in range(4000):
        H = rng.uniform(-np.pi, np.pi)
        dec = rng.uniform(-np.deg2rad(80.0), np.deg2rad(80.0))
        sin_el = np.sin(lat) * np.sin(dec) + np.cos(lat) * np.cos(dec) * np.cos(H)
        el = np.arcsin(sin_el)
        if not (0.0 < el <= np.deg2rad(80.0)):
            continue
        chi = util.parallactic_angle(H, dec, lat)
        bound = util.parallactic_angle_error_bound(el, dec)
        for ang in np.linspace(0, 2 * np.pi, 8, endpoint=False):  # displacement by e in any direction
            dH, dd = e * np.cos(ang) / np.cos(dec), e * np.sin(ang)
            d = np.angle(np.exp(1j * (util.parallactic_angle(H + dH, dec + dd, lat) - chi)))
            assert abs(d) <= 1.02 * bound + 1e-12, (np.rad2deg(el), np.rad2deg(dec), d, bound)
    field = float(util.parallactic_angle_error_bound(np.deg2rad(60.0), np.deg2rad(-30.0)))
    assert 6.7e-4 < field < 6.9e-4
    # its effect on E for the synthetic beam and the sky of the test workloads
    P = synth.make_problem(ntime=2, na=3, nchan=2, npsrc=200, seed=5)
    E0 = O.e_beam(P)
    P['parallactic_angles'] = P['parallactic_angles'] + field
    E1 = O.e_beam(P)
    rel = np.max(np.abs(E1 - E0)) / np.max(np.abs(E0))
    assert rel < 1.5e-3, rel
    assert np.linalg.norm(E1 - E0) / np.linalg.norm(E0) < 6e-5

"""Seeded synthetic RIME v4 problems.

No measurement set or FITS beam is available, so every workload is generated
here from a seed.  The generator produces the reference's v4 arrays
(``montblanc/impl/rime/v4/config.py:131-247``) with physically shaped values:

* channels spanning 1.4-1.5 GHz, reference frequency 1.4 GHz;
* antennas at uniform random east/north positions within +-1.5 km, with
  per-antenna uvw from earth-rotation tracks at declination -30 deg over
  10 hours (antenna 0 at the origin, as the reference's MS loader stores
  them, ``impl/rime/v4/loaders/loaders.py:92-111``);
* parallactic angles from the same track;
* sources with l, m ~ U(-0.05, 0.05), I ~ U(1, 10), Q, U, V = I * U(-0.1, 0.1),
  alpha ~ U(-0.8, 0.8);
* gaussian shapes el, em ~ U(0, 1e-4), R ~ U(0.5, 1); sersic e1, e2 ~
  U(-0.3, 0.3), scale ~ U(1e-5, 1e-4);
* a 50x50x32 complex 2x2 beam cube: a cos^3 taper on the diagonal plus
  N(0, 0.01) complex ripple on every correlation;
* pointing errors N(0, 1e-3); G = identity + N(0, 0.05) complex;
* unit weights and no flags unless asked for.

``observed_vis`` is left at zero; callers fill it with a model plus noise
(``add_noise``) once they have a forward model to hand.
"""
import numpy as np

LIGHTSPEED = 299792458.0
FWHM2INT = 1.0 / np.sqrt(np.log(256.0))

#: Default scalar properties, as in montblanc/impl/rime/v4/config.py:54-69.
DEFAULT_PROPS = {
    'gauss_scale': FWHM2INT * np.sqrt(2.0) * np.pi / LIGHTSPEED,
    'two_pi_over_c': 2.0 * np.pi / LIGHTSPEED,
    'sigma_sqrd': 1.0,
    'beam_ll': -0.5, 'beam_lm': -0.5, 'beam_lfreq': 1.3e9,
    'beam_ul': 0.5, 'beam_um': 0.5, 'beam_ufreq': 1.5e9,
}

#: Workload shapes used throughout (time steps, antennas, channels, sources).
WORKLOADS = {
    'small_fp64': dict(ntime=10, na=14, nchan=16, npsrc=20, ngsrc=10, nssrc=0),
    'medium_mixed': dict(ntime=100, na=27, nchan=64, npsrc=1000, ngsrc=200, nssrc=50),
    'large_point': dict(ntime=200, na=64, nchan=256, npsrc=20000, ngsrc=500, nssrc=0),
    # the large problem's antennas on fewer times, channels and sources, its
    # visibility and operand arrays still larger than L2: the ncu case
    'profile_point': dict(ntime=32, na=64, nchan=64, npsrc=4000, ngsrc=50, nssrc=0),
}


def nr_of_baselines(na, auto_correlations=False):
    return na * (na + 1) // 2 if auto_correlations else na * (na - 1) // 2


def _track(rng, ntime, na, dec=np.deg2rad(-30.0), lat=np.deg2rad(-30.0), hours=10.0):
    east = rng.uniform(-1500.0, 1500.0, size=na)
    north = rng.uniform(-1500.0, 1500.0, size=na)
    east[0] = 0.0
    north[0] = 0.0
    # Local east/north/up -> equatorial XYZ (up = 0)
    X = -np.sin(lat) * north
    Y = east
    Z = np.cos(lat) * north
    H = np.deg2rad(15.0) * np.linspace(-hours / 2, hours / 2, ntime)
    sH, cH = np.sin(H)[:, None], np.cos(H)[:, None]
    u = sH * X[None] + cH * Y[None]
    v = -np.sin(dec) * cH * X[None] + np.sin(dec) * sH * Y[None] + np.cos(dec) * Z[None]
    w = np.cos(dec) * cH * X[None] - np.cos(dec) * sH * Y[None] + np.sin(dec) * Z[None]
    uvw = np.stack([u, v, w], axis=-1)
    pa = np.arctan2(np.sin(H) * np.cos(lat),
                    np.sin(lat) * np.cos(dec) - np.cos(lat) * np.sin(dec) * np.cos(H))
    return uvw, np.repeat(pa[:, None], na, axis=1)


def beam_cube(rng, lw=50, mh=50, nud=32, props=DEFAULT_PROPS):
    l = np.linspace(props['beam_ll'], props['beam_ul'], lw)
    m = np.linspace(props['beam_lm'], props['beam_um'], mh)
    f = np.linspace(props['beam_lfreq'], props['beam_ufreq'], nud)
    r = np.sqrt(l[:, None] ** 2 + m[None, :] ** 2)
    arg = np.minimum(r[:, :, None] * 2.0 * (f[None, None, :] / 1.4e9), np.pi / 2)
    taper = np.cos(arg) ** 3
    E = (rng.normal(0.0, 0.01, size=(lw, mh, nud, 4))
         + 1j * rng.normal(0.0, 0.01, size=(lw, mh, nud, 4)))
    E[..., 0] += taper
    E[..., 3] += taper
    return E


def make_problem(ntime, na, nchan, npsrc, ngsrc=0, nssrc=0, seed=0,
                 beam_shape=(50, 50, 32), use_weight_vector=False,
                 residuals=False, random_weights=False, flag_fraction=0.0,
                 antenna_scaling_noise=0.0, auto_correlations=False, vis_arrays=True):
    """Return a problem dict of float64/complex128 NumPy arrays.

    With ``vis_arrays=False`` the visibility-sized arrays (flag,
    weight_vector, observed_vis) are left out, for callers that create them
    on the device."""
    rng = np.random.default_rng(seed)
    nsrc = npsrc + ngsrc + nssrc
    nbl = nr_of_baselines(na, auto_correlations)
    P = dict(DEFAULT_PROPS)
    P.update(npsrc=npsrc, ngsrc=ngsrc, nssrc=nssrc,
             use_weight_vector=use_weight_vector, residuals=residuals)
    uvw, pa = _track(rng, ntime, na)
    P['uvw'] = uvw
    P['parallactic_angles'] = pa
    k = 0 if auto_correlations else 1
    a1, a2 = np.triu_indices(na, k)
    P['antenna1'] = np.tile(a1.astype(np.int32), (ntime, 1))
    P['antenna2'] = np.tile(a2.astype(np.int32), (ntime, 1))
    P['frequency'] = np.linspace(1.4e9, 1.5e9, nchan)
    P['ref_frequency'] = np.full(nchan, 1.4e9)
    P['point_errors'] = rng.normal(0.0, 1e-3, size=(ntime, na, nchan, 2))
    P['antenna_scaling'] = 1.0 + antenna_scaling_noise * rng.normal(size=(na, nchan, 2))
    P['E_beam'] = beam_cube(rng, *beam_shape)
    G = (rng.normal(0.0, 0.05, size=(ntime, na, nchan, 4))
         + 1j * rng.normal(0.0, 0.05, size=(ntime, na, nchan, 4)))
    G[..., 0] += 1.0
    G[..., 3] += 1.0
    P['G_term'] = G
    P['lm'] = rng.uniform(-0.05, 0.05, size=(nsrc, 2))
    I = rng.uniform(1.0, 10.0, size=nsrc)
    QUV = I[:, None] * rng.uniform(-0.1, 0.1, size=(nsrc, 3))
    stokes = np.concatenate([I[:, None], QUV], axis=1)
    P['stokes'] = np.repeat(stokes[:, None, :], ntime, axis=1).copy()
    P['alpha'] = np.repeat(rng.uniform(-0.8, 0.8, size=nsrc)[:, None], ntime, axis=1).copy()
    P['gauss_shape'] = np.stack([rng.uniform(0.0, 1e-4, ngsrc),
                                 rng.uniform(0.0, 1e-4, ngsrc),
                                 rng.uniform(0.5, 1.0, ngsrc)])
    P['sersic_shape'] = np.stack([rng.uniform(-0.3, 0.3, nssrc),
                                  rng.uniform(-0.3, 0.3, nssrc),
                                  rng.uniform(1e-5, 1e-4, nssrc)])
    vshape = (ntime, nbl, nchan, 4)
    if not vis_arrays:
        return P
    P['flag'] = (rng.random(vshape) < flag_fraction).astype(np.uint8)
    P['weight_vector'] = rng.random(vshape) if random_weights else np.ones(vshape)
    P['observed_vis'] = np.zeros(vshape, dtype=np.complex128)
    return P


def add_noise(P, model_vis, sigma=0.1, seed=1):
    """observed = model + N(0, sigma) complex noise (the generator's rule)."""
    rng = np.random.default_rng(seed)
    noise = rng.normal(0.0, sigma, model_vis.shape) + 1j * rng.normal(0.0, sigma, model_vis.shape)
    P['observed_vis'] = model_vis + noise
    return P


def dims_of(P):
    """(ntime, na, nbl, nchan, nsrc) of a problem dict."""
    ntime, na = P['uvw'].shape[:2]
    return ntime, na, P['antenna1'].shape[1], P['frequency'].shape[0], P['lm'].shape[0]

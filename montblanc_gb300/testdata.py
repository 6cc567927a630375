"""Random 'test' fills for the v4 arrays (data_source='test').

Same distributions as the reference's ``test=`` initialisers
(montblanc/impl/rime/v4/config.py:71-247): a circle of antennas for uvw,
uniform random Stokes with I^2 >= Q^2 + U^2 + V^2, uniform random beam
cube, G, weights and observed visibilities, random 0/1 flags, a fixed
1 arcsec sersic scale.  Uses numpy's global random state, as the reference
does.
"""
import numpy as np


def _random_like(ary):
    if np.iscomplexobj(ary):
        return np.random.random(ary.shape) + 1j * np.random.random(ary.shape)
    return np.random.random(ary.shape)


def _uvw(slvr, ary):
    ntime, na = ary.shape[:2]
    ant = 2 * np.pi * np.arange(na) / float(na)
    tim = np.arange(ntime) / float(ntime)
    ta = tim[:, None] * ant[None, :]
    ary[:, :, 0] = 10 * np.sin(ta)
    ary[:, :, 1] = 10 * np.sin(ta)
    ary[:, :, 2] = np.random.random((ntime, na)) * 0.1
    ary[:, 0, :] = 0
    return ary


def _stokes(slvr, ary):
    noise = np.random.random(ary.shape[:2]) * 0.1
    Q = np.random.random(ary.shape[:2]) - 0.5
    U = np.random.random(ary.shape[:2]) - 0.5
    V = np.random.random(ary.shape[:2]) - 0.5
    ary[..., 0] = np.sqrt(Q ** 2 + U ** 2 + V ** 2 + noise)
    ary[..., 1], ary[..., 2], ary[..., 3] = Q, U, V
    return ary


def _gauss(slvr, ary):
    ary[...] = np.random.random(ary.shape)
    return ary


def _sersic(slvr, ary):
    ary[0] = 0
    ary[1] = 0
    ary[2] = np.pi / 648000
    return ary


TEST_FILLS = {
    'uvw': _uvw,
    'antenna1': lambda s, a: s.default_ant_pairs()[0],
    'antenna2': lambda s, a: s.default_ant_pairs()[1],
    'frequency': lambda s, a: np.linspace(1e9, 2e9, a.shape[0]),
    'ref_frequency': lambda s, a: 1.4e9,
    'parallactic_angles': lambda s, a: _random_like(a) * np.pi,
    'point_errors': lambda s, a: (_random_like(a) - 0.5) * 1e-2,
    'antenna_scaling': lambda s, a: _random_like(a),
    'E_beam': lambda s, a: _random_like(a),
    'G_term': lambda s, a: _random_like(a),
    'lm': lambda s, a: (_random_like(a) - 0.5) * 1e-1,
    'stokes': _stokes,
    'alpha': lambda s, a: _random_like(a) * 0.1,
    'gauss_shape': _gauss,
    'sersic_shape': _sersic,
    'flag': lambda s, a: np.random.randint(0, 2, size=a.shape),
    'weight_vector': lambda s, a: _random_like(a),
    'observed_vis': lambda s, a: _random_like(a),
}


def fill(slvr, name, ary):
    fn = TEST_FILLS.get(name)
    if fn is not None and ary.size:
        out = fn(slvr, ary)
        if out is not None and out is not ary:
            ary[...] = out

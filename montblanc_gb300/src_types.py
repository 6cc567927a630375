"""Source types and their counting variables (montblanc/src_types.py:27-189).

Sources are always ordered point, gaussian, sersic.
"""
from collections import OrderedDict

SOURCE_VAR_TYPES = OrderedDict([('point', 'npsrc'), ('gaussian', 'ngsrc'), ('sersic', 'nssrc')])


def source_types():
    return list(SOURCE_VAR_TYPES.keys())


def source_nr_vars():
    return list(SOURCE_VAR_TYPES.values())


def default_sources(**kwargs):
    """Ordered {type: count}; unknown types are rejected, and one point source
    is added when every count is zero (src_types.py:46-89)."""
    bad = [t for t in kwargs if t not in SOURCE_VAR_TYPES]
    if bad:
        raise KeyError('Unknown source type(s) %s; valid types are %s' % (bad, source_types()))
    S = OrderedDict()
    for k in SOURCE_VAR_TYPES:
        try:
            S[k] = int(kwargs.get(k, 0))
        except ValueError:
            raise TypeError('Supplied value %r for source %s cannot be converted to an integer'
                            % (kwargs.get(k), k))
    if sum(S.values()) == 0:
        S['point'] = 1
    return S


def sources_to_nr_vars(sources):
    S = default_sources(**sources)
    return OrderedDict((SOURCE_VAR_TYPES[k], v) for k, v in S.items())

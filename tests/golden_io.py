"""Load the golden fixtures in tests/golden into problem dicts."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def names(prefix=''):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + '*.npz')))


def load(name):
    """Return (problem dict with float64/complex128 inputs, outputs dict)."""
    z = np.load(os.path.join(GOLDEN, name + '.npz'))
    P, out = {}, {}
    for k in z.files:
        v = z[k]
        if k.startswith('in_'):
            n = k[3:]
            if v.dtype == np.float32:
                v = v.astype(np.float64)
            elif v.dtype == np.complex64:
                v = v.astype(np.complex128)
            P[n] = v
        elif k.startswith('prop_'):
            P[k[5:]] = float(v)
        elif k.startswith('opt_'):
            P[k[4:]] = v.item()
        elif k.startswith('out_'):
            out[k[4:]] = v
    return P, out


def rel_err(a, b):
    """max |a - b| / max |b| (norm-free, robust for tiny entries)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def conditioning(P, ref):
    """kappa = max |model| / max |observed - model|: a chi^2 term is the
    square of a residual that is small against the model, so a relative
    error e of the model visibilities becomes a relative error of about
    2 e kappa in the chi^2 terms."""
    vis = np.asarray(ref['vis_out'])
    res = np.asarray(P['observed_vis']) - vis
    return float(np.max(np.abs(vis)) / max(np.max(np.abs(res)), 1e-300))


def terms_tol(P, ref, vis_rel, floor):
    """Bound on rel_err of the chi^2 terms implied by model visibilities
    that agree to ``vis_rel`` (relative), never below ``floor``."""
    return max(floor, 2.0 * vis_rel * conditioning(P, ref))

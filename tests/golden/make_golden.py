"""Generate the golden fixtures in this directory from the reference itself.

Run in a container where the reference checkout is mounted at
/root/reference (the GPU machines do not have it):

    python tests/golden/make_golden.py

Each fixture is produced by the reference's own v4 ``CPUSolver``
(``montblanc/impl/rime/v4/cpu/CPUSolver.py``), loaded through ``ref_shim``.
Inputs come from the seeded generator in ``montblanc_gb300.synth`` (or from
random fills in the style of the reference's unit tests,
``montblanc/tests/test_rime_v4.py``), rounded to float32-representable values
so that they are stored losslessly as float32/complex64 and so that FP32 and
FP64 runs see the same inputs.  Outputs are stored in float64/complex128.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from montblanc_gb300 import synth  # noqa: E402
import ref_shim  # noqa: E402

FLOAT_ARRAYS = ('uvw', 'frequency', 'ref_frequency', 'parallactic_angles', 'point_errors',
                'antenna_scaling', 'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape',
                'weight_vector')
COMPLEX_ARRAYS = ('E_beam', 'G_term', 'observed_vis')


def to_f32_exact(P):
    for k in FLOAT_ARRAYS:
        P[k] = P[k].astype(np.float32).astype(np.float64)
    for k in COMPLEX_ARRAYS:
        P[k] = P[k].astype(np.complex64).astype(np.complex128)
    for k in ref_shim.PROP_NAMES:
        P[k] = float(np.float32(P[k]))
    return P


def reference_outputs(P, jones=None):
    s = ref_shim.reference_solver(P)
    out = {}
    if jones is None:
        out['B_sqrt'] = s.compute_b_sqrt_jones()
        out['E_term'] = s.compute_E_beam()
        jones = s.compute_ekb_sqrt_jones_per_ant()
        out['jones'] = jones
    vis = s.compute_ekb_vis(s.compute_ekb_jones_per_bl(jones))
    out['vis_out'] = s.compute_gekb_vis(vis)
    out['chi_sqrd_terms'] = s.compute_chi_sqrd_sum_terms(out['vis_out'])
    out['X2'] = np.float64(s.compute_chi_sqrd(out['chi_sqrd_terms']))
    return out


def save(name, P, out, keep=('B_sqrt', 'E_term', 'jones'), time_slice=None, jones_in=None):
    rec = {}
    for k in FLOAT_ARRAYS:
        rec['in_' + k] = P[k].astype(np.float32)
    for k in COMPLEX_ARRAYS:
        rec['in_' + k] = P[k].astype(np.complex64)
    rec['in_antenna1'] = P['antenna1']
    rec['in_antenna2'] = P['antenna2']
    rec['in_flag'] = P['flag']
    for k in ref_shim.PROP_NAMES:
        rec['prop_' + k] = np.float64(P[k])
    for k in ('npsrc', 'ngsrc', 'nssrc'):
        rec['opt_' + k] = np.int64(P[k])
    rec['opt_use_weight_vector'] = np.bool_(P['use_weight_vector'])
    rec['opt_residuals'] = np.bool_(P['residuals'])
    if jones_in is not None:
        rec['in_jones'] = jones_in.astype(np.complex64)
    for k in ('vis_out', 'chi_sqrd_terms', 'X2'):
        rec['out_' + k] = out[k]
    for k in keep:
        if k in out:
            v = out[k]
            if time_slice is not None and k in ('E_term', 'jones'):
                v = v[:, time_slice]
            rec['out_' + k] = v
    if time_slice is not None:
        rec['out_time_slice'] = np.array([time_slice.start, time_slice.stop])
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
    print(name, sum(v.nbytes for v in rec.values()) // 1024, 'KiB raw')


def case_small_fp64():
    """The 10 time x 14 antenna x 16 channel, 20 point + 10 gaussian problem."""
    P = to_f32_exact(synth.make_problem(10, 14, 16, 20, 10, 0, seed=1234))
    model = reference_outputs(P)['vis_out']
    synth.add_noise(P, model, sigma=0.1, seed=99)
    P = to_f32_exact(P)
    out = reference_outputs(P)
    save('small_fp64', P, out, time_slice=slice(0, 1))


def _unit_test_style(npsrc, ngsrc, nssrc, seed, weight_vector, residuals,
                     ntime=4, na=6, nchan=8, beam=(12, 12, 6)):
    """Random fills in the style of the reference's 'test' initialisers
    (montblanc/impl/rime/v4/config.py:131-247) on a physically shaped base."""
    P = synth.make_problem(ntime, na, nchan, npsrc, ngsrc, nssrc, seed=seed,
                           beam_shape=beam, use_weight_vector=weight_vector,
                           residuals=residuals, random_weights=True, flag_fraction=0.2,
                           antenna_scaling_noise=0.05)
    rng = np.random.default_rng(seed + 7)
    P['sigma_sqrd'] = float(rng.uniform(0.5, 1.5))
    P['parallactic_angles'] = rng.random(P['parallactic_angles'].shape) * np.pi
    P['point_errors'] = (rng.random(P['point_errors'].shape) - 0.5) * 1e-2
    P['lm'] = (rng.random(P['lm'].shape) - 0.5) * 1e-1
    P['beam_ll'] = P['beam_lm'] = -1.0
    P['beam_ul'] = P['beam_um'] = 1.0
    P['observed_vis'] = rng.random(P['observed_vis'].shape) + 1j * rng.random(P['observed_vis'].shape)
    return to_f32_exact(P)


def case_source_permutations():
    """All non-empty {0,3}^3 point/gaussian/sersic mixes x weight vector on/off,
    plus residual output (test_rime_v4.py:44-93, 224-277)."""
    seed = 100
    for wv in (False, True):
        for p in (0, 3):
            for g in (0, 3):
                for s in (0, 3):
                    if p == g == s == 0:
                        continue
                    seed += 1
                    P = _unit_test_style(p, g, s, seed, wv, False)
                    out = reference_outputs(P)
                    save('perm_p%d_g%d_s%d_w%d' % (p, g, s, int(wv)), P, out,
                         keep=('B_sqrt', 'jones'))
    for wv in (False, True):
        seed += 1
        P = _unit_test_style(3, 3, 3, seed, wv, True)
        save('residual_w%d' % int(wv), P, reference_outputs(P), keep=('B_sqrt', 'jones'))


def case_ebeam_edges():
    """Odd beam-cube sizes and the 2x2x2 cube (test_rime_v4.py:344-420)."""
    for name, beam in (('ebeam_odd', (13, 17, 11)), ('ebeam_2x2x2', (2, 2, 2))):
        P = _unit_test_style(4, 3, 0, 500 + beam[0], False, False, ntime=3, na=5,
                             nchan=8, beam=beam)
        save(name, P, reference_outputs(P), keep=('E_term', 'jones'))


def case_given_jones():
    """Coherency sum on random per-antenna Jones terms
    (test_rime_v4.py:181-222)."""
    P = _unit_test_style(3, 3, 3, 777, True, False)
    rng = np.random.default_rng(778)
    nsrc = 9
    ntime, na = P['uvw'].shape[:2]
    nchan = P['frequency'].shape[0]
    shape = (nsrc, ntime, na, nchan, 4)
    J = (rng.random(shape) + 1j * rng.random(shape)).astype(np.complex64).astype(np.complex128)
    out = reference_outputs(P, jones=J)
    save('given_jones', P, out, keep=(), jones_in=J)


if __name__ == '__main__':
    np.random.seed(0)
    case_small_fp64()
    case_source_permutations()
    case_ebeam_edges()
    case_given_jones()

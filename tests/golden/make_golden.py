"""Generate the golden fixtures in this directory from the reference itself.

Run in a container where the reference checkout is mounted (the GPU
machines do not have it); the checkout is /root/reference unless the
MONTBLANC_REFERENCE environment variable or ``--reference PATH`` names
another:

    python tests/golden/make_golden.py [--reference PATH] [--only NAME ...]

Each fixture is produced by the reference's own v4 ``CPUSolver``
(``montblanc/impl/rime/v4/cpu/CPUSolver.py``), loaded through ``ref_shim``.
Inputs come from the seeded generator in ``montblanc_gb300.synth`` (or from
random fills in the style of the reference's unit tests,
``montblanc/tests/test_rime_v4.py``), rounded to float32-representable values
so that they are stored losslessly as float32/complex64 and so that FP32 and
FP64 runs see the same inputs.  Outputs are stored in float64/complex128.
"""
import argparse
import multiprocessing as mp
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


# ---------------------------------------------------------------------------
# Sampled (time, channel) units of the two large workloads
# ---------------------------------------------------------------------------
def sample_units(P, times, chans):
    """The problem restricted to the given time steps and channels, all
    sources and baselines: the visibilities of these units are exactly those
    of the full problem (units are independent)."""
    t, c = np.asarray(times), np.asarray(chans)
    Q = dict(P)
    for k in ('uvw', 'parallactic_angles', 'antenna1', 'antenna2'):
        Q[k] = P[k][t]
    Q['frequency'] = P['frequency'][c]
    Q['ref_frequency'] = P['ref_frequency'][c]
    Q['point_errors'] = P['point_errors'][t][:, :, c]
    Q['antenna_scaling'] = P['antenna_scaling'][:, c]
    Q['G_term'] = P['G_term'][t][:, :, c]
    Q['stokes'] = P['stokes'][:, t]
    Q['alpha'] = P['alpha'][:, t]
    nbl = P['antenna1'].shape[1]
    shape = (len(t), nbl, len(c), 4)
    Q['flag'] = np.zeros(shape, np.uint8)
    Q['weight_vector'] = np.ones(shape)
    Q['observed_vis'] = np.zeros(shape, np.complex128)
    return Q


def source_batch(P, s0, s1):
    """The sub-problem holding sources [s0, s1) (any mix of types)."""
    npsrc, ngsrc = P['npsrc'], P['ngsrc']
    Q = dict(P)
    Q['lm'], Q['stokes'], Q['alpha'] = P['lm'][s0:s1], P['stokes'][s0:s1], P['alpha'][s0:s1]
    p0, p1 = min(s0, npsrc), min(s1, npsrc)
    g0, g1 = min(max(s0 - npsrc, 0), ngsrc), min(max(s1 - npsrc, 0), ngsrc)
    x0, x1 = max(s0 - npsrc - ngsrc, 0), max(s1 - npsrc - ngsrc, 0)
    Q['npsrc'], Q['ngsrc'], Q['nssrc'] = p1 - p0, g1 - g0, x1 - x0
    Q['gauss_shape'] = P['gauss_shape'][:, g0:g1]
    Q['sersic_shape'] = P['sersic_shape'][:, x0:x1]
    return Q


def _batch_vis(args):
    P, s0, s1 = args
    s = ref_shim.reference_solver(source_batch(P, s0, s1))
    return s.compute_ekb_vis(s.compute_ekb_jones_per_bl(s.compute_ekb_sqrt_jones_per_ant()))


def reference_outputs_batched(P, batch=256, processes=None):
    """The reference's forward over source batches (CPUSolver chunked over
    sources: the sum over sources is linear and G is applied after it):
    compute_ekb_vis per batch, summed, then compute_gekb_vis,
    compute_chi_sqrd_sum_terms and compute_chi_sqrd on the sum."""
    nsrc = P['lm'].shape[0]
    jobs = [(P, s0, min(nsrc, s0 + batch)) for s0 in range(0, nsrc, batch)]
    with mp.get_context('fork').Pool(processes or os.cpu_count()) as pool:
        parts = pool.map(_batch_vis, jobs, chunksize=1)
    vis = np.sum(parts, axis=0)
    s = ref_shim.reference_solver(source_batch(P, 0, min(nsrc, 1)))
    out = {'vis_out': s.compute_gekb_vis(vis)}
    out['chi_sqrd_terms'] = s.compute_chi_sqrd_sum_terms(out['vis_out'])
    out['X2'] = np.float64(s.compute_chi_sqrd(out['chi_sqrd_terms']))
    return out


def _grad_part(args):
    from oracle import adjoint as OA
    P, s0, s1, gV_P = args
    return OA.chi2_grad_sources(gV_P, s0, s1)


def oracle_gradient(P, batch=256, processes=None):
    """FP64 gradient of chi^2 from the oracle (oracle/adjoint.py, pinned by
    central finite differences): the reference has no gradient."""
    from oracle import adjoint as OA
    nsrc = P['lm'].shape[0]
    base = OA.chi2_grad_prepare(P, src_chunk=batch)
    jobs = [(P, s0, min(nsrc, s0 + batch), base) for s0 in range(0, nsrc, batch)]
    with mp.get_context('fork').Pool(processes or os.cpu_count()) as pool:
        parts = pool.map(_grad_part, jobs, chunksize=1)
    return OA.chi2_grad_combine(base, parts)


#: (fixture name, workload, time steps, channels) of the sampled units.
SAMPLED = (
    ('units_medium_mixed', 'medium_mixed', [0, 41, 99], [0, 27, 63]),
    ('units_large_point', 'large_point', [0, 199], [0, 128, 255]),
)
#: Seed of the benchmark's workloads (bench.py --seed default), so the
#: sampled units are units of the workload the benchmark times.
BENCH_SEED = 20261203


def case_sampled_units(only=None):
    """(time, channel) units of the 100 x 27 x 64 mixed workload (1000 point
    + 200 gaussian + 50 sersic sources) and of the 200 x 64 x 256 point
    workload (20 000 point + 500 gaussian), all sources and baselines: the
    reference's forward (per source batch) and the oracle's FP64 gradient."""
    for name, wl, times, chans in SAMPLED:
        if only and name not in only:
            continue
        spec = synth.WORKLOADS[wl]
        P = synth.make_problem(**spec, seed=BENCH_SEED, vis_arrays=False)
        Q = to_f32_exact(sample_units(P, times, chans))
        model = reference_outputs_batched(Q)['vis_out']
        synth.add_noise(Q, model, sigma=0.1, seed=BENCH_SEED + 5)
        Q = to_f32_exact(Q)
        out = reference_outputs_batched(Q)
        x2g, grads = oracle_gradient(Q)
        for k, v in grads.items():
            out['grad_' + k] = v
        out['grad_X2'] = np.float64(x2g)
        out['sample_times'] = np.array(times)
        out['sample_chans'] = np.array(chans)
        keep = tuple(k for k in out if k.startswith(('grad_', 'sample_')))
        save(name, Q, out, keep=keep)


#: Standard deviation (rad) of the source displacement of the displaced
#: gradients: phase errors of ~0.01-0.1 rad on the longest baselines, so
#: the residual is model mismatch well above the N(0, 0.1) noise.
DISPLACEMENT = 3e-7


def case_displaced_gradients(only=None):
    """Adds to each sampled-unit fixture the oracle gradient at source
    positions displaced by N(0, DISPLACEMENT) from the truth (same observed
    visibilities).  At the truth the gradient is a noise-level sum; away
    from it the residual is dominated by the model, and gradient errors of
    the FP32 forms are relative to a signal."""
    for name, _, _, _ in SAMPLED:
        if only and name not in only:
            continue
        path = os.path.join(HERE, name + '.npz')
        z = dict(np.load(path))
        P, _ = load_fixture(z)
        rng = np.random.default_rng(BENCH_SEED + 9)
        lm = P['lm'] + rng.normal(0.0, DISPLACEMENT, P['lm'].shape)
        P['lm'] = lm.astype(np.float32).astype(np.float64)
        _, grads = oracle_gradient(P)
        z['out_displaced_lm'] = P['lm'].astype(np.float32)
        for k, v in grads.items():
            z['out_displaced_grad_' + k] = v
        np.savez_compressed(path, **z)
        print(name, 'displaced gradients added')


#: Arrays wider than the fused kernels' 64-antenna tile, evaluated as
#: antenna sub-arrays: 128 antennas (four blocks of 32) and 75 antennas (a
#: ragged last block of 11), with weights, flags and all three source types.
WIDE = (
    ('wide_na128', dict(ntime=2, na=128, nchan=3, npsrc=24, ngsrc=6, nssrc=3)),
    ('wide_na75', dict(ntime=3, na=75, nchan=2, npsrc=16, ngsrc=4, nssrc=4)),
)


def case_wide_arrays(only=None):
    """The reference's forward and the oracle's FP64 gradient (at the truth
    and at displaced source positions) on the WIDE problems."""
    for k, (name, shape) in enumerate(WIDE):
        if only and name not in only:
            continue
        P = to_f32_exact(synth.make_problem(**shape, seed=BENCH_SEED + 40 + k, beam_shape=(24, 24, 8),
                                            use_weight_vector=True, random_weights=True, flag_fraction=0.05))
        model = reference_outputs_batched(P)['vis_out']
        synth.add_noise(P, model, sigma=0.1, seed=BENCH_SEED + 50 + k)
        P = to_f32_exact(P)
        out = reference_outputs_batched(P)
        x2g, grads = oracle_gradient(P)
        for g, v in grads.items():
            out['grad_' + g] = v
        out['grad_X2'] = np.float64(x2g)
        rng = np.random.default_rng(BENCH_SEED + 60 + k)
        P2 = dict(P)
        P2['lm'] = (P['lm'] + rng.normal(0.0, DISPLACEMENT, P['lm'].shape)).astype(np.float32).astype(np.float64)
        _, dgrads = oracle_gradient(P2)
        out['displaced_lm'] = P2['lm'].astype(np.float32)
        for g, v in dgrads.items():
            out['displaced_grad_' + g] = v
        keep = tuple(g for g in out if g.startswith(('grad_', 'displaced_')))
        save(name, P, out, keep=keep)


def load_fixture(z):
    """Problem dict (float64 / complex128) and outputs of a fixture's arrays."""
    P, out = {}, {}
    for k, v in z.items():
        if k.startswith('in_'):
            if v.dtype == np.float32:
                v = v.astype(np.float64)
            elif v.dtype == np.complex64:
                v = v.astype(np.complex128)
            P[k[3:]] = v
        elif k.startswith('prop_'):
            P[k[5:]] = float(v)
        elif k.startswith('opt_'):
            P[k[4:]] = v.item()
        elif k.startswith('out_'):
            out[k[4:]] = v
    return P, out


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', help='reference checkout (default: MONTBLANC_REFERENCE or /root/reference)')
    ap.add_argument('--only', nargs='*', help='fixture names to regenerate')
    ap.add_argument('--displaced-only', action='store_true',
                    help='only add the displaced gradients to existing sampled-unit fixtures')
    args = ap.parse_args()
    if args.reference:
        ref_shim.set_reference_root(args.reference)
    np.random.seed(0)
    only = set(args.only or ())
    if not only:
        case_small_fp64()
        case_source_permutations()
        case_ebeam_edges()
        case_given_jones()
    if not args.displaced_only:
        case_sampled_units(only)
    case_displaced_gradients(only)
    if not args.displaced_only:
        case_wide_arrays(only)

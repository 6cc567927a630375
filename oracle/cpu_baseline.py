"""CPU baseline timing of the oracle (test / benchmark infrastructure only).

Times the FP64 NumPy restatement of the reference's CPU path
(``oracle/rime_v4.py``, forward chi^2) plus the FP64 NumPy gradient
(``oracle/adjoint.py``) on a bounded sample of a workload: a set of
independent (time, channel) units, each with all antennas and a subset of
the sources, spread over a process pool (spawn start method) on the host
cores.  Only bench.py's CPU-baseline leg and its reference arm use this.
"""
import multiprocessing as mp
import os
import time

import numpy as np

from . import adjoint as OA


def _unit_worker(args):
    P = args
    t0 = time.perf_counter()
    chi2, _ = OA.chi2_grad(P, src_chunk=32)
    return chi2, time.perf_counter() - t0


def sample_mix(P_full, nsrc_sample):
    """(point, gaussian, sersic) counts of a sample of ``nsrc_sample``
    sources in the problem's proportions (every type present keeps at least
    one source)."""
    counts = [P_full['npsrc'], P_full['ngsrc'], P_full['nssrc']]
    total = sum(counts)
    n = min(nsrc_sample, total)
    mix = [min(c, max(1 if c else 0, int(round(n * c / total)))) for c in counts]
    i = int(np.argmax(counts))
    mix[i] = min(counts[i], mix[i] + n - sum(mix))
    return tuple(mix)


def make_units(P_full, obs, units, nsrc_sample):
    """Sub-problems of one time step x one channel with ``nsrc_sample``
    sources: the first sources of each type, in the problem's proportions
    (sample_mix).

    ``obs(t, ch)`` returns the observed visibilities (nbl, 4) of a unit."""
    npsrc, ngsrc = P_full['npsrc'], P_full['ngsrc']
    ns_p, ns_g, ns_s = sample_mix(P_full, nsrc_sample)
    sel = np.r_[0:ns_p, npsrc:npsrc + ns_g, npsrc + ngsrc:npsrc + ngsrc + ns_s]
    out = []
    for (t, ch) in units:
        P = {k: P_full[k] for k in ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm',
                                    'beam_lfreq', 'beam_ul', 'beam_um', 'beam_ufreq', 'E_beam',
                                    'antenna_scaling')}
        P['antenna_scaling'] = P_full['antenna_scaling'][:, ch:ch + 1]
        P.update(npsrc=ns_p, ngsrc=ns_g, nssrc=ns_s, use_weight_vector=False, residuals=False)
        P['uvw'] = P_full['uvw'][t:t + 1]
        P['parallactic_angles'] = P_full['parallactic_angles'][t:t + 1]
        P['antenna1'] = P_full['antenna1'][t:t + 1]
        P['antenna2'] = P_full['antenna2'][t:t + 1]
        P['frequency'] = P_full['frequency'][ch:ch + 1]
        P['ref_frequency'] = P_full['ref_frequency'][ch:ch + 1]
        P['point_errors'] = P_full['point_errors'][t:t + 1, :, ch:ch + 1]
        P['G_term'] = P_full['G_term'][t:t + 1, :, ch:ch + 1]
        P['lm'] = P_full['lm'][sel]
        P['stokes'] = P_full['stokes'][sel][:, t:t + 1]
        P['alpha'] = P_full['alpha'][sel][:, t:t + 1]
        P['gauss_shape'] = P_full['gauss_shape'][:, :ns_g]
        P['sersic_shape'] = P_full['sersic_shape'][:, :ns_s]
        nbl = P['antenna1'].shape[1]
        P['flag'] = np.zeros((1, nbl, 1, 4), np.uint8)
        P['weight_vector'] = np.ones((1, nbl, 1, 4))
        P['observed_vis'] = np.asarray(obs(t, ch), dtype=np.complex128).reshape(1, nbl, 1, 4)
        out.append(P)
    return out


def time_units(problems, processes=None):
    """Run chi2_grad on every unit in a spawn pool; return (wall s, procs)."""
    procs = processes or os.cpu_count() or 1
    procs = max(1, min(procs, len(problems)))
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    os.environ.setdefault('OPENBLAS_NUM_THREADS', '1')
    ctx = mp.get_context('spawn')
    with ctx.Pool(procs) as pool:
        pool.map(_unit_worker, problems[:procs])  # warm the workers (imports)
        t0 = time.perf_counter()
        pool.map(_unit_worker, problems)
        wall = time.perf_counter() - t0
    return wall, procs

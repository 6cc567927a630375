#!/usr/bin/env python
"""Benchmark: source.vis terms/s of the RIME v4 chi^2 + full gradient.

One step = one fused forward chi^2 (mb_rime_forward, want_grad=1) plus the
adjoint (mb_rime_adjoint) over the whole workload, inputs resident on the
GPU.  terms/step = nsrc * ntime * nbl * nchan.

Default workload (the largest one of the suite, and the one the
split-precision target is stated on): 200 time steps, 64 antennas
(2016 baselines), 256 channels, 20000 point + 500 gaussian sources, FP32
data, unit weights, no flags; observed = model + N(0, 0.1) complex noise.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode MODE]
                    [--workload NAME] [--impl reference]

With --gpus N > 1 (one process per GPU under torch.distributed.run) every
rank evaluates its own replica of the workload: the path needs no
collective, so the job total is N * terms / (max over ranks of the time).

Prints one JSON line (rank 0).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'source·vis terms/s for χ²+grad, split-prec vs plain FP32, at stated FP64 error'
UNIT = 'source·vis terms/s'

# Algorithmic work per source.vis term: one 2x2 complex J_p J_q^H product with
# its accumulation, 64 flops, in the forward; the adjoint's X.A contraction
# (d chi^2 / dJ_a = sum_b Y_ab J_b), 64 flops.  chi^2 + gradient: 128.
FLOPS_FWD = 64
FLOPS_ADJ = 64
SM_COUNT = 152

# What ncu shows for the dominant kernels (profiles/*.md of the same build:
# one --set full capture of one launch on the profile_point workload).
NCU_LIMITER = {
    'coh_tc_adj_kernel': {
        'source': 'profiles/coh_tc_adj_kernel_profile_point.md',
        'limiter': 'CUDA-core issue and latency of the per-(source, antenna) producer and chain',
        'sm__pipe_tensor_cycles_active': 0.115, 'smsp__issue_active': 0.392,
        'pipe_fma_cycles': 0.246, 'pipe_alu': 0.284, 'pipe_fp64': 0.018, 'pipe_xu': 0.034,
        'thread_instructions_per_item': 647},
    'coh_tc_fwd_kernel': {
        'source': 'profiles/coh_tc_fwd_kernel_profile_point.md',
        'limiter': 'CUDA-core issue and latency of the per-(source, antenna) producer; TMEM drains',
        'sm__pipe_tensor_cycles_active': 0.352, 'smsp__issue_active': 0.436,
        'pipe_fma_cycles': 0.204, 'pipe_alu': 0.345, 'pipe_fp64': 0.003, 'pipe_xu': 0.048,
        'thread_instructions_per_item': 510},
}

# DRAM bytes per launch from a one-kernel ncu capture on the profile_point
# workload (32 x 64 x 64 units, 4000 point + 50 gaussian sources; profiles/
# dram_bytes_profile_point.md), split into the part that scales with the
# (time, channel) units and the part that scales with the (time, source,
# antenna) path lengths, read once per time step from DRAM (the units of one
# time step run together and share them in L2).
NCU_DRAM = {
    # kernel: (bytes per unit, bytes per (time, source, antenna)); the
    # profile_point launch moved 475.5 MB (forward) and 221.6 MB (adjoint)
    # over 2048 units and 32 x 4050 x 64 8-byte path lengths (66.4 MB)
    'coh_tc_fwd_kernel': (199.7e3, 8.0),
    'coh_tc_adj_kernel': (75.8e3, 8.0),
}


def dram_traffic(kernel, workload):
    """Modelled DRAM bytes per launch of ``kernel`` on ``workload`` (None if
    the kernel has no capture)."""
    from montblanc_gb300 import synth
    if kernel not in NCU_DRAM:
        return None
    w = synth.WORKLOADS[workload]
    per_unit, per_tsa = NCU_DRAM[kernel]
    units = w['ntime'] * w['nchan']
    tsa = w['ntime'] * (w['npsrc'] + w['ngsrc'] + w['nssrc']) * w['na']
    return per_unit * units + per_tsa * tsa


def workload_terms(name):
    """(point-source terms, extended-source terms) of one chi^2 evaluation."""
    from montblanc_gb300 import synth
    w = synth.WORKLOADS[name]
    vis = w['ntime'] * synth.nr_of_baselines(w['na']) * w['nchan']
    return w['npsrc'] * vis, (w['ngsrc'] + w['nssrc']) * vis


def kernel_work(workload, mode):
    """Algorithmic flops per launch of each coherency kernel: FLOPS_FWD per
    source.vis term for the forward kernels, FLOPS_ADJ per term for the
    adjoint kernels, over the sources each kernel handles (split modes: the
    tensor-core kernels take the point sources, the forward kernel also the
    extended ones; the CUDA-core adjoint the extended sources)."""
    pt, et = workload_terms(workload)
    split = mode != 'native'
    return {
        'coh_tc_fwd_kernel': FLOPS_FWD * (pt + et),
        'coh_fwd_kernel': FLOPS_FWD * (pt + et),
        'coh_tc_adj_kernel': FLOPS_ADJ * pt,
        'coh_adj_kernel': FLOPS_ADJ * (et if split else pt + et),
    }


def fp32_peak_tflops(clk):
    """FP32 CUDA-core peak at the sampled SM clock (152 SMs x 128 FMA)."""
    sm_mhz = clk.get('sm_mhz') or 2070.0
    return SM_COUNT * 128 * 2 * sm_mhz * 1e6 / 1e12


def roofline(workload, mode, kernels, peak, peak_src, clk):
    """Roofline of the kernel with the largest share of the timed steps.

    achieved = algorithmic flops per launch / mean CUDA-event duration of
    that kernel's launches in the timed region (events on its launch
    stream), against the measured sustained bf16 tensor peak for the
    tensor-core forms (the roof of the contraction they execute) and the
    FP32 CUDA-core peak at the sampled clock for the plain form.  The bound
    is the roof the kernel's arithmetic intensity puts it under; ``limiter``
    is what ncu shows holding it below that roof."""
    work = kernel_work(workload, mode)
    name = max(kernels, key=lambda k: kernels[k][0])
    ms, n = kernels[name]
    per_launch_ms = ms / n
    flops = work.get(name)
    if mode == 'native':
        out = {'bound': 'fp32 (CUDA cores)', 'peak': fp32_peak_tflops(clk),
               'peak_source': 'FP32 CUDA-core peak at the sampled SM clock'}
    else:
        out = {'bound': 'tensor', 'peak': peak,
               'peak_source': '%s bf16 sustained (MEASURED_PEAKS.json)' % peak_src}
    out.update({'kernel': name, 'launch_ms': per_launch_ms, 'unit': 'TFLOP/s',
                'traffic': dram_traffic(name, workload),
                'traffic_source': 'profiles/dram_bytes_profile_point.md, scaled by units and path lengths'})
    if name in NCU_LIMITER:
        out['limiter'] = NCU_LIMITER[name]
    if flops is None:
        out.update({'achieved': None, 'frac': None})
        return out
    achieved = flops / (per_launch_ms * 1e-3) / 1e12
    out.update({'achieved': achieved, 'frac': achieved / out['peak'], 'algorithmic_flops_per_launch': flops,
                'flops_per_term': FLOPS_ADJ if 'adj' in name else FLOPS_FWD})
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', choices=('ours', 'reference'), default='ours')
    ap.add_argument('--workload', default='large_point')
    ap.add_argument('--mode', default='split_tf32', help="native | split_tf32 | split_bf16")
    ap.add_argument('--no-plain', action='store_true', help='skip timing the plain FP32 CUDA-core form')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-batch', action='store_true', help='skip the batched-likelihood measurement')
    ap.add_argument('--seed', type=int, default=20261203)
    return ap.parse_args()


def workload_desc(name):
    from montblanc_gb300 import synth
    w = synth.WORKLOADS[name]
    nbl = synth.nr_of_baselines(w['na'])
    return ('%s: ntime %d, na %d (nbl %d), nchan %d, %d point + %d gaussian + %d sersic sources, FP32 data'
            % (name, w['ntime'], w['na'], nbl, w['nchan'], w['npsrc'], w['ngsrc'], w['nssrc']))


def terms_of(name):
    from montblanc_gb300 import synth
    w = synth.WORKLOADS[name]
    return (w['npsrc'] + w['ngsrc'] + w['nssrc']) * w['ntime'] * synth.nr_of_baselines(w['na']) * w['nchan']


# ---------------------------------------------------------------------------
# distributed plumbing
# ---------------------------------------------------------------------------
def dist_init(n):
    """(world size, rank, local rank) from the launcher's environment; with
    more than one rank, a process group over NCCL (one GPU per rank), or
    over gloo where no GPU is visible (host-side tests of the replica
    plumbing)."""
    import torch
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if ws > 1:
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group('nccl', device_id=torch.device('cuda', local))
        else:
            dist.init_process_group('gloo')
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    """The largest x over the ranks (the slowest replica's time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(ws, terms_per_rank, ms_max):
    """Whole-job throughput of ws replicas that each process terms_per_rank
    terms per step, timed by the slowest rank (weak scaling)."""
    return ws * terms_per_rank / (ms_max * 1e-3)


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class Clocks(object):
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self):
        self.lines = []
        self.proc = None

    def start(self):
        idx = os.environ.get('CUDA_VISIBLE_DEVICES', '0').split(',')[0] or '0'
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', idx, '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': smax,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def build_workload(name, seed):
    import torch
    from montblanc_gb300 import synth
    from montblanc_gb300.rime import RimeProblem
    spec = synth.WORKLOADS[name]
    P = synth.make_problem(**spec, seed=seed, vis_arrays=False)
    prob = RimeProblem.from_numpy(P, dtype='float', device='cuda')
    model = prob.empty_vis()
    prob.forward(mode='native', model_vis=model)
    g = torch.Generator(device='cuda')
    g.manual_seed(seed + 1)
    noise = torch.randn(model.shape, dtype=torch.complex64, device='cuda', generator=g)
    model.add_(noise, alpha=0.1 * math.sqrt(2.0))  # N(0, 0.1) on re and im
    prob.arrays['observed_vis'] = model
    torch.cuda.synchronize()
    return P, prob


def batched_likelihood(seed, nsets=256, reps=2):
    """256 parameter sets (per-set source counts log-uniform in 10..5000,
    point / gaussian / sersic mix) against one 100 x 27 x 64 observation:
    chi^2 + gradient of every set per batch, the form and source tile
    autotuned per set, all sets of a form in one forward and one adjoint
    launch (mb_rime_batch), the batch captured as one CUDA graph and
    replayed.  Errors against the FP64 form on the smallest, median and
    largest sets."""
    import numpy as np
    import torch
    from montblanc_gb300 import synth
    from montblanc_gb300.batch import RimeBatch, make_sets
    from montblanc_gb300.rime import RimeProblem
    spec = synth.WORKLOADS['medium_mixed']
    P = synth.make_problem(**spec, seed=seed, vis_arrays=True)
    prob = RimeProblem.from_numpy(P, dtype='float', device='cuda')
    model = prob.empty_vis()
    prob.forward(mode='native', model_vis=model)
    g = torch.Generator(device='cuda')
    g.manual_seed(seed + 1)
    model.add_(torch.randn(model.shape, dtype=torch.complex64, device='cuda', generator=g), alpha=0.1 * math.sqrt(2.0))
    P['observed_vis'] = model.cpu().numpy()
    del prob, model
    sets = make_sets(P, nsets, seed=seed + 2)
    b = RimeBatch(P, sets, dtype='float')
    t0 = time.time()
    forms = b.autotune()
    tune_s = time.time() - t0
    b.capture()
    b.run()
    torch.cuda.synchronize()
    from montblanc_gb300 import _cabi
    l0 = _cabi.lib.mb_kernel_launches()
    b.enqueue()
    torch.cuda.synchronize()
    launches = int(_cabi.lib.mb_kernel_launches() - l0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.run()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    x2 = b.X2.cpu().numpy()
    n = np.array([sum(c) for c in b.counts])
    pick = sorted({int(np.argmin(n)), int(np.argsort(n)[len(n) // 2]), int(np.argmax(n))})
    ref = RimeBatch(P, [sets[i] for i in pick], dtype='double')
    ref.forms = ['native'] * len(pick)
    ref_x2 = ref.run().cpu().numpy()
    x2_err, g_err = [], []
    for j, i in enumerate(pick):
        x2_err.append(abs(x2[i] - ref_x2[j]) / abs(ref_x2[j]))
        g32, g64 = b.set_grads(i), ref.set_grads(j)
        num = sum(float(np.sum((g32[k] - g64[k]) ** 2)) for k in ('lm', 'stokes', 'alpha'))
        den = sum(float(np.sum(g64[k] ** 2)) for k in ('lm', 'stokes', 'alpha'))
        g_err.append(math.sqrt(num / den))
    return {'workload': '%d sets x (ntime 100, na 27, nchan 64), per-set nsrc log-uniform 10..5000 '
                        '(%d sources in all), shared observation' % (nsets, int(n.sum())),
            'sets_per_s': nsets / (ms * 1e-3), 'terms_per_s': b.terms() / (ms * 1e-3), 'ms_per_batch': ms,
            'execution': 'one CUDA graph replay per batch of %d kernel launches: shared tables, one forward and '
                         'one adjoint launch per (form, source tile) over all its sets\' (time, channel) units, '
                         'the chi^2 sums, the gradients' % launches,
            'launches_per_batch': launches,
            'forms': {f: forms.count(f) for f in set(forms)},
            'choices': {'%s/%d' % c: n_c for c, n_c in
                        ((c, list(zip(b.forms, b.tiles)).count(c)) for c in set(zip(b.forms, b.tiles)))},
            'autotune_s': tune_s,
            'autotune_ms_by_nsrc': b.tune_times,
            'errors_vs_fp64': {'sets': [int(n[i]) for i in pick], 'chi2_rel': x2_err, 'grad_rel_norm': g_err}}


def subset_problem(P, prob, times, chans):
    """The same sky and antennas on a few (time, channel) units, for the
    error measurement against the FP64 path."""
    import numpy as np
    Q = dict(P)
    t = np.asarray(times)
    c = np.asarray(chans)
    Q['uvw'] = P['uvw'][t]
    Q['parallactic_angles'] = P['parallactic_angles'][t]
    Q['antenna1'] = P['antenna1'][t]
    Q['antenna2'] = P['antenna2'][t]
    Q['frequency'] = P['frequency'][c]
    Q['ref_frequency'] = P['ref_frequency'][c]
    Q['point_errors'] = P['point_errors'][t][:, :, c]
    Q['antenna_scaling'] = P['antenna_scaling'][:, c]
    Q['G_term'] = P['G_term'][t][:, :, c]
    Q['stokes'] = P['stokes'][:, t]
    Q['alpha'] = P['alpha'][:, t]
    obs = prob.arrays['observed_vis'][t][:, :, c].cpu().numpy()
    Q['observed_vis'] = obs
    Q['flag'] = np.zeros(obs.shape, np.uint8)
    return Q


ERROR_FIXTURES = (
    ('units_medium_mixed', '3 time steps x 3 channels of the 100 x 27 x 64 workload, all 1250 sources '
                           '(1000 point + 200 gaussian + 50 sersic) and 351 baselines'),
    ('units_large_point', '2 time steps x 3 channels of the 200 x 64 x 256 workload (this benchmark\'s '
                          'generator and seed), all 20500 sources and 2016 baselines'),
)
GRAD_NAMES = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term')


def errors_vs_reference(modes):
    """Errors of each form against the reference on sampled units of the two
    large workloads (tests/golden fixtures: the reference's CPUSolver
    outputs, run per source batch, and the FP64 oracle's gradients at the
    truth and at displaced source positions; the reference has no
    gradient).  Norm-wise relative errors; chi^2 relative."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, 'tests'))
    import golden_io
    from montblanc_gb300.rime import RimeProblem

    def nerr(a, b):
        return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))

    out = {}
    for name, desc in ERROR_FIXTURES:
        P, ref = golden_io.load(name)
        res = {'sample': desc, 'reference': 'reference CPUSolver forward; FP64 oracle gradient'}
        for dtype, mode in [('double', 'native'), ('float', 'native')] + [('float', m) for m in modes]:
            key = 'fp64' if dtype == 'double' else ('plain_fp32' if mode == 'native' else mode)
            r = {}
            for disp in (False, True):
                Q = dict(P)
                if disp:
                    Q['lm'] = ref['displaced_lm']
                prob = RimeProblem.from_numpy(Q, dtype=dtype)
                vis = prob.empty_vis()
                x2 = prob.forward(mode=mode, model_vis=vis, want_grad=True).item()
                g = prob.adjoint(mode=mode)
                prob.check(mode, True)
                pre = 'displaced_grad_' if disp else 'grad_'
                ge = {k: nerr(g[k].cpu().numpy(), ref[pre + k]) for k in GRAD_NAMES if ref[pre + k].size}
                if disp:
                    r['grad_displaced_rel_norm'] = ge
                else:
                    r['vis_rel_norm'] = nerr(vis.cpu().numpy(), ref['vis_out'])
                    r['chi2_rel'] = abs(x2 - float(ref['X2'])) / abs(float(ref['X2']))
                    r['grad_truth_rel_norm'] = ge
            res[key] = r
        out[name] = res
    return out


# ---------------------------------------------------------------------------
# timing
# ---------------------------------------------------------------------------
def time_resident(prob, mode, steps, warmup, ws, kernels=None):
    """Device-resident chi^2 + gradient; returns (ms/step, fwd ms, adj ms).

    With ``kernels`` (a dict), the library's per-kernel CUDA-event times of
    the timed steps are stored in it, {name: (total ms, launches)}, and the
    number of library launches under the key '_launches'."""
    import torch
    from montblanc_gb300 import _cabi
    stream = torch.cuda.current_stream()
    grads = prob.empty_grads()

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        prob.forward(mode=mode, want_grad=True)
        if ev:
            ev[1].record(stream)
        prob.adjoint(mode=mode, grads=grads)
        if ev:
            ev[2].record(stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    with _cabi.KernelTimer() as kt:
        for i in range(steps):
            step(evs[i])
        torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    if kernels is not None:
        kernels.update(kt.times())
        kernels['_launches'] = kt.launches
    total = evs[0][0].elapsed_time(evs[-1][2])
    fwd = [e[0].elapsed_time(e[1]) for e in evs]
    adj = [e[1].elapsed_time(e[2]) for e in evs]
    return total / steps, statistics.mean(fwd), statistics.mean(adj)


def time_plain_slice(P, prob, ws, workload, clk, ntime=20, steps=3, warmup=1):
    """The plain FP32 CUDA-core form on the first ``ntime`` time steps of
    the workload (its throughput per term does not depend on the time
    extent), ``steps`` timed steps after ``warmup``, with its own roofline
    against the FP32 CUDA-core peak.  The form runs at its faster source tile
    (16 or 32 sources per shared-memory tile, one timed step each)."""
    import torch
    from montblanc_gb300.rime import RimeProblem
    nt = min(ntime, prob.ntime)
    Q = subset_problem(P, prob, list(range(nt)), list(range(prob.nchan)))
    sub = RimeProblem.from_numpy(Q, dtype='float')
    terms = prob.nsrc * nt * prob.nbl * prob.nchan
    tile_ms = {}
    for tile in (16, 32):
        sub.source_tile = tile
        tile_ms[tile] = max_over_ranks(ws, time_resident(sub, 'native', 1, 1, ws, {})[0])
    sub.source_tile = min(tile_ms, key=tile_ms.get)
    kernels = {}
    ms, fwd, adj = time_resident(sub, 'native', steps, warmup, ws, kernels)
    sub.check('native', True)
    ms = max_over_ranks(ws, ms)
    kernels.pop('_launches', None)
    pt, et = workload_terms(workload)
    scale = nt / prob.ntime  # the slice's share of the workload's terms
    work = {'coh_fwd_kernel': FLOPS_FWD * (pt + et) * scale, 'coh_adj_kernel': FLOPS_ADJ * (pt + et) * scale}
    peak = fp32_peak_tflops(clk)
    rl = {}
    for k, (kms, n) in kernels.items():
        if k in work:
            ach = work[k] / (kms / n * 1e-3) / 1e12
            rl[k] = {'achieved': ach, 'unit': 'TFLOP/s', 'peak': peak, 'frac': ach / peak,
                     'bound': 'fp32 (CUDA cores)', 'launch_ms': kms / n}
    step_ach = (FLOPS_FWD + FLOPS_ADJ) * terms / (ms * 1e-3) / 1e12
    out = {'value': ws * terms / (ms * 1e-3), 'unit': UNIT, 'ms_per_step': ms, 'forward_ms': fwd,
           'adjoint_ms': adj, 'mode': 'native', 'steps': steps, 'warmup': warmup,
           'sample': 'first %d of %d time steps, all sources, baselines and channels' % (nt, prob.ntime),
           'source_tile': sub.source_tile, 'source_tile_ms': tile_ms,
           'roofline': {'step_achieved_tflops': step_ach, 'fp32_peak_tflops_at_clock': peak,
                        'step_frac': step_ach / peak, 'kernels': rl},
           'kernels_ms_per_step': {k: v[0] / steps for k, v in sorted(kernels.items())}}
    del sub
    torch.cuda.empty_cache()
    return out


def time_fp64_forward(P, prob, ws, ntime=1, steps=1, warmup=1):
    """The reference's default configuration through the drop-in path: the
    FP64 forward (model visibilities, chi^2 terms and chi^2, no gradient)
    of the CUDA-core kernels on the first ``ntime`` time steps of the
    workload, all channels, sources and baselines."""
    import torch
    from montblanc_gb300.rime import RimeProblem
    nt = min(ntime, prob.ntime)
    Q = subset_problem(P, prob, list(range(nt)), list(range(prob.nchan)))
    sub = RimeProblem.from_numpy(Q, dtype='double')
    vis, terms = sub.empty_vis(), sub.empty_chi2()
    for _ in range(warmup):
        sub.forward(mode='native', model_vis=vis, chi_sqrd_result=terms)
    torch.cuda.synchronize()
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        sub.forward(mode='native', model_vis=vis, chi_sqrd_result=terms)
    e1.record()
    e1.synchronize()
    ms = max_over_ranks(ws, e0.elapsed_time(e1) / steps)
    n = prob.nsrc * nt * prob.nbl * prob.nchan
    del sub, vis, terms
    torch.cuda.empty_cache()
    return {'value': ws * n / (ms * 1e-3), 'unit': UNIT, 'ms_per_step': ms, 'steps': steps, 'warmup': warmup,
            'what': 'FP64 forward (chi^2, model visibilities, chi^2 terms; no gradient), mode native, the '
                    'drop-in rime_solver default', 'terms_per_step': n,
            'sample': 'first %d of %d time steps, all sources, baselines and channels' % (nt, prob.ntime)}


def time_e2e(prob, mode, steps, warmup, ws):
    """Through the public API with host buffers: every step copies its
    inputs from pinned host memory and reads chi^2 and all gradients back
    into pinned host memory.  ``HostFeed`` puts the copies on their own
    streams with double-buffered device inputs, so the copies of step i+1
    and the read-back of step i-1 overlap the kernels of step i; the timed
    region runs from the first step's copy-in to the last step's read-back.
    Returns (ms per step, bytes in, bytes out per step, phase times)."""
    import torch
    from montblanc_gb300.rime import HostFeed
    names = ['observed_vis', 'flag', 'G_term', 'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape']
    host = {n: prob.arrays[n].cpu().pin_memory() for n in names}
    feed = HostFeed(prob, names, mode=mode, depth=2)
    grads = prob.empty_grads()
    outs = [({n: torch.empty(g.shape, dtype=g.dtype).pin_memory() for n, g in grads.items()},
             torch.empty(1, dtype=torch.float64).pin_memory()) for _ in range(2)]
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = 8 + sum(t.numel() * t.element_size() for t in outs[0][0].values())

    for i in range(max(1, warmup)):
        feed.submit(host, outs[i % 2][1], outs[i % 2][0])
    feed.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(steps)]
    start.record(feed.h2d)
    for i in range(steps):
        last = feed.submit(host, outs[i % 2][1], outs[i % 2][0], events=evs[i])
    last.synchronize()
    total = start.elapsed_time(evs[-1][3])
    feed.synchronize()
    barrier(ws)
    phases = {'h2d_ms': statistics.mean(e[0].elapsed_time(e[1]) for e in evs),
              'd2h_ms': statistics.mean(e[2].elapsed_time(e[3]) for e in evs),
              'overlap': 'HostFeed: copies on their own streams, double-buffered device inputs; the copies of '
                         'step i+1 and the read-back of step i-1 run under the kernels of step i'}
    return total / steps, h2d, d2h, phases


def cpu_baseline(P, prob, max_units=None):
    """The FP64 oracle (forward + gradient) on the host cores over a bounded
    sample: (time, channel) units with all antennas and 2000 sources drawn
    from every source type in the workload's proportions."""
    from oracle import cpu_baseline as C
    cores = os.cpu_count() or 1
    nunits = max_units or 2 * cores
    nsample = min(2000, prob.nsrc)
    units = [((7 * i) % prob.ntime, (13 * i) % prob.nchan) for i in range(nunits)]
    obs = prob.arrays['observed_vis']
    probs = C.make_units(P, lambda t, ch: obs[t, :, ch].cpu().numpy(), units, nsample)
    wall, procs = C.time_units(probs, cores)
    terms = nunits * nsample * prob.nbl
    mix = C.sample_mix(P, nsample)
    return {'value': terms / wall, 'unit': UNIT, 'cores': procs, 'kind': 'port',
            'sample': '%d (time, channel) units x %d sources (%d point + %d gaussian + %d sersic) x %d baselines, '
                      'FP64 NumPy chi^2 + gradient (the oracle, a NumPy restatement of the reference\'s '
                      'CPUSolver: the reference tree is not on the GPU machines), %.1f s wall'
                      % (nunits, nsample, mix[0], mix[1], mix[2], prob.nbl, wall)}


def peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            m = json.load(f)
        return m['bf16_tflops'], m['bf16_tflops_sustained'], m['hbm_gbs'], 'measured'
    except (OSError, KeyError, ValueError):
        return 1900.0, 1700.0, 6800.0, 'fallback'


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference arm: the CPU restatement of the reference's v4 path
    (FP64 NumPy, forward + gradient) on the host cores, same workload."""
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    import numpy as np
    from montblanc_gb300 import synth
    from oracle import cpu_baseline as C
    from oracle import rime_v4 as O
    spec = synth.WORKLOADS[args.workload]
    P = synth.make_problem(**spec, seed=args.seed, vis_arrays=False)
    cores = os.cpu_count() or 1
    nsample = min(2000, spec['npsrc'] + spec['ngsrc'] + spec['nssrc'])
    nbl = P['antenna1'].shape[1]
    rng = np.random.default_rng(args.seed)
    times = []
    for step in range(args.warmup + args.steps):
        units = [(int(rng.integers(P['uvw'].shape[0])), int(rng.integers(P['frequency'].shape[0])))
                 for _ in range(cores)]
        probs = C.make_units(P, lambda t, ch: rng.normal(0, 0.1, (nbl, 4)) + 0j, units, nsample)
        wall, procs = C.time_units(probs, cores)
        if step >= args.warmup:
            times.append(wall)
    terms = cores * nsample * nbl
    value = terms / statistics.mean(times)
    mix = C.sample_mix(P, nsample)
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * statistics.mean(times),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic',
            'config': run_config(args, 1),
            'form': 'CPU FP64 chi^2 + gradient: the oracle, a NumPy restatement of the reference\'s v4 CPUSolver '
                    '(the reference tree is not on the GPU machines; the restatement is faster than the '
                    'reference\'s own code, so the ratio against it is conservative)',
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': procs, 'kind': 'port',
                             'sample': 'per step %d (time, channel) units x %d sources (%d point + %d gaussian '
                                       '+ %d sersic, in the workload\'s proportions) x %d baselines'
                                       % (cores, nsample, mix[0], mix[1], mix[2], nbl)},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def run_config(args, ws):
    """The workload configuration both arms report."""
    from montblanc_gb300 import synth
    w = synth.WORKLOADS[args.workload]
    nvis = w['ntime'] * synth.nr_of_baselines(w['na']) * w['nchan']
    return {'workload': workload_desc(args.workload), 'mode': args.mode, 'terms_per_step': terms_of(args.workload),
            'l2': 'inputs larger than L2 (observed_vis alone %.1f GB)' % (nvis * 4 * 8 / 1e9),
            'phase': 'FP64 path length; FP32 forms reduce phi nu / c as a double-float product', 'replicas': ws}


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    import torch
    ws, rank, local = dist_init(args.gpus)
    P, prob = build_workload(args.workload, args.seed + rank)
    terms = terms_of(args.workload)

    clocks = Clocks()
    clocks.start()
    kernels = {}
    ms, fwd_ms, adj_ms = time_resident(prob, args.mode, args.steps, args.warmup, ws, kernels)
    clk = clocks.stop()
    prob.check(args.mode, True)  # no bounded device wait gave up
    ms_max = max_over_ranks(ws, ms)
    value = whole_job_value(ws, terms, ms_max)

    plain = fp64_fwd = None
    if not args.no_plain and args.mode != 'native':
        # The plain FP32 CUDA-core form on the first 20 time steps of the same
        # workload (throughput per term does not depend on the time extent).
        plain = time_plain_slice(P, prob, ws, args.workload, clk)
        fp64_fwd = time_fp64_forward(P, prob, ws)
    e2e = None
    if not args.no_e2e:
        ems, h2d, d2h, phases = time_e2e(prob, args.mode, args.steps, 1, ws)
        ems = max_over_ranks(ws, ems)
        e2e = {'value': ws * terms / (ems * 1e-3), 'unit': UNIT, 'h2d_bytes_per_step': h2d,
               'd2h_bytes_per_step': d2h, 'ms_per_step': ems}
        e2e.update(phases)

    if rank != 0:
        return
    errs = errors_vs_reference(sorted({args.mode, 'split_tf32', 'split_bf16'} - {'native'}))
    burst, sustained, hbm, src = peaks()
    launches = kernels.pop('_launches')
    rl = roofline(args.workload, args.mode, kernels, sustained, src, clk)
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_max, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32' if args.mode == 'native' else 'f32 (%s products)' % args.mode,
        'data': 'synthetic (seeded generator; observed = model + N(0,0.1) noise)',
        'config': run_config(args, ws),
        'forward_ms': fwd_ms, 'adjoint_ms': adj_ms,
        'roofline': rl,
        'kernels_ms_per_step': {k: v[0] / args.steps for k, v in sorted(kernels.items())},
        'errors_vs_reference': errs,
        'gpu_launches': launches,
        'clocks': clk,
    }
    if fp64_fwd:
        line['fp64_forward'] = fp64_fwd
    if plain:
        line['plain_fp32'] = plain
        line['split_over_plain'] = value / plain['value']
        line['roofline_plain_fp32'] = plain['roofline']
    if e2e:
        line['e2e'] = e2e
    if not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(P, prob)
    if not args.no_batch:
        line['batched'] = batched_likelihood(args.seed)
    print(json.dumps(line))


if __name__ == '__main__':
    main()

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

# Algorithmic work per source.vis term: a 2x2 complex J_p J_q^H product with
# accumulation (64 flops) forward; the two 2x2 complex products of the
# adjoint, d/dJ_p += gV J_q and d/dJ_q += gV^H J_p (128 flops).
FLOPS_FWD = 64
FLOPS_ADJ = 128
SM_COUNT = 152

# DRAM traffic (bytes) per launch of the dominant kernel from ncu captures,
# keyed by (kernel, workload, mode).
NCU_TRAFFIC = {
    # ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum (one pass), the
    # timed step of `bench.py --steps 1 --warmup 1 --no-e2e --no-cpu
    # --no-plain --no-batch`
    ('coh_tc_adj_kernel', 'large_point', 'split_tf32'): 9.34e9 + 0.199e9,
    ('coh_tc_fwd_kernel', 'large_point', 'split_tf32'): 6.29e9 + 3.42e9,
    # the same with --workload profile_point
    ('coh_tc_adj_kernel', 'profile_point', 'split_tf32'): 351.6e6 + 4.1e6,
    ('coh_tc_fwd_kernel', 'profile_point', 'split_tf32'): 229.3e6 + 108.9e6,
}


def workload_terms(name):
    """(point-source terms, extended-source terms) of one chi^2 evaluation."""
    from montblanc_gb300 import synth
    w = synth.WORKLOADS[name]
    vis = w['ntime'] * synth.nr_of_baselines(w['na']) * w['nchan']
    return w['npsrc'] * vis, (w['ngsrc'] + w['nssrc']) * vis


def roofline(workload, mode, kernels, peak, peak_src, clk):
    """Roofline of the kernel with the largest share of the timed steps.

    achieved = algorithmic flops per launch / mean CUDA-event duration of
    that kernel's launches in the timed region (events on its launch
    stream).  Algorithmic flops: FLOPS_FWD per source.vis term for the
    forward coherency kernels, FLOPS_ADJ per term for the adjoint kernels,
    over the sources each kernel handles (split modes: the tensor-core
    kernels take the point sources; the CUDA-core adjoint the rest)."""
    pt, et = workload_terms(workload)
    split = mode != 'native'
    work = {
        'coh_tc_fwd_kernel': FLOPS_FWD * (pt + et),
        'coh_fwd_kernel': FLOPS_FWD * (pt + et),
        'coh_tc_adj_kernel': FLOPS_ADJ * pt,
        'coh_adj_kernel': FLOPS_ADJ * (et if split else pt + et),
    }
    name = max(kernels, key=lambda k: kernels[k][0])
    ms, n = kernels[name]
    per_launch_ms = ms / n
    flops = work.get(name)
    sm_mhz = clk.get('sm_mhz') or 2070.0
    fp32_peak = SM_COUNT * 128 * 2 * sm_mhz * 1e6 / 1e12
    out = {'bound': 'tensor', 'kernel': name, 'launch_ms': per_launch_ms, 'unit': 'TFLOP/s',
           'peak': peak, 'peak_source': '%s bf16 sustained (MEASURED_PEAKS.json)' % peak_src,
           'traffic': NCU_TRAFFIC.get((name, workload, mode))}
    if flops is None:
        out.update({'achieved': None, 'frac': None})
        return out
    achieved = flops / (per_launch_ms * 1e-3) / 1e12
    out.update({'achieved': achieved, 'frac': achieved / peak, 'algorithmic_flops_per_launch': flops,
                'fp32_simt_peak_tflops_at_clock': fp32_peak, 'fp32_simt_frac': achieved / fp32_peak})
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
    autotuned per set,
    the batch captured as one CUDA graph and replayed.  Errors against the
    FP64 form on the smallest, median and largest sets."""
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
            'execution': 'one CUDA graph replay per batch (forward + adjoint of every set)',
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


def errors_vs_fp64(P, prob, mode):
    """Visibility, chi^2 and gradient errors of ``mode`` against the FP64
    GPU path (itself within 1e-10 of the reference CPU path) on 2 time steps
    x 3 channels of the workload with every source and antenna."""
    import numpy as np
    import torch
    from montblanc_gb300.rime import RimeProblem
    Q = subset_problem(P, prob, [0, prob.ntime - 1], [0, prob.nchan // 2, prob.nchan - 1])
    # the FP64 reference sees the same FP32 data, so the error is the method's
    for k, v in list(Q.items()):
        if isinstance(v, np.ndarray) and v.dtype == np.float64:
            Q[k] = v.astype(np.float32).astype(np.float64)
        elif isinstance(v, np.ndarray) and v.dtype == np.complex128:
            Q[k] = v.astype(np.complex64).astype(np.complex128)
    p64 = RimeProblem.from_numpy(Q, dtype='double')
    p32 = RimeProblem.from_numpy(Q, dtype='float')
    v64, v32 = p64.empty_vis(), p32.empty_vis()
    x64, g64 = p64.forward(model_vis=v64, want_grad=True).item(), None
    g64 = p64.adjoint()
    x32 = p32.forward(mode=mode, model_vis=v32, want_grad=True).item()
    g32 = p32.adjoint(mode=mode)
    a, b = v32.cpu().numpy().astype(np.complex128), v64.cpu().numpy()
    # the outputs are residual-free model visibilities (vis_output='model')
    out = {'vis_rel_norm': float(np.linalg.norm(a - b) / np.linalg.norm(b)),
           'vis_rel_max': float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
           'chi2_rel': abs(x32 - x64) / abs(x64)}
    for k in ('lm', 'stokes', 'G_term'):
        ga, gb = g32[k].cpu().numpy().astype(np.complex128), g64[k].cpu().numpy()
        out['grad_%s_rel_norm' % k] = float(np.linalg.norm(ga - gb) / np.linalg.norm(gb))
    out['sample'] = '2 time steps x 3 channels, all %d sources and %d antennas' % (prob.nsrc, prob.na)
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


def time_plain_slice(P, prob, ws, ntime=20):
    import numpy as np
    import torch
    from montblanc_gb300.rime import RimeProblem
    nt = min(ntime, prob.ntime)
    Q = subset_problem(P, prob, list(range(nt)), list(range(prob.nchan)))
    sub = RimeProblem.from_numpy(Q, dtype='float')
    terms = prob.nsrc * nt * prob.nbl * prob.nchan
    ms, fwd, adj = time_resident(sub, 'native', 1, 1, ws)
    ms = max_over_ranks(ws, ms)
    out = {'value': ws * terms / (ms * 1e-3), 'unit': UNIT, 'ms_per_step': ms, 'forward_ms': fwd,
           'adjoint_ms': adj, 'mode': 'native',
           'sample': 'first %d of %d time steps, all sources, baselines and channels' % (nt, prob.ntime)}
    del sub
    torch.cuda.empty_cache()
    return out


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
    sample: (time, channel) units with all antennas and 2000 sources."""
    from oracle import cpu_baseline as C
    cores = os.cpu_count() or 1
    nunits = max_units or 2 * cores
    nsample = min(2000, prob.nsrc)
    units = [((7 * i) % prob.ntime, (13 * i) % prob.nchan) for i in range(nunits)]
    obs = prob.arrays['observed_vis']
    probs = C.make_units(P, lambda t, ch: obs[t, :, ch].cpu().numpy(), units, nsample)
    wall, procs = C.time_units(probs, cores)
    terms = nunits * nsample * prob.nbl
    return {'value': terms / wall, 'unit': UNIT, 'cores': procs, 'kind': 'port',
            'sample': '%d (time, channel) units x %d sources x %d baselines, FP64 NumPy chi^2 + gradient, '
                      '%.1f s wall' % (nunits, nsample, prob.nbl, wall)}


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
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * statistics.mean(times),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic',
            'config': {'workload': workload_desc(args.workload), 'form': 'CPU FP64 (reference algorithm)'},
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': procs, 'kind': 'port',
                             'sample': 'per step %d (time, channel) units x %d sources x %d baselines'
                                       % (cores, nsample, nbl)},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


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
    ms_max = max_over_ranks(ws, ms)
    value = whole_job_value(ws, terms, ms_max)

    plain = None
    if not args.no_plain and args.mode != 'native':
        # The plain FP32 CUDA-core form on the first 20 time steps of the same
        # workload (throughput per term does not depend on the time extent).
        plain = time_plain_slice(P, prob, ws)
    e2e = None
    if not args.no_e2e:
        ems, h2d, d2h, phases = time_e2e(prob, args.mode, args.steps, 1, ws)
        ems = max_over_ranks(ws, ems)
        e2e = {'value': ws * terms / (ems * 1e-3), 'unit': UNIT, 'h2d_bytes_per_step': h2d,
               'd2h_bytes_per_step': d2h, 'ms_per_step': ems}
        e2e.update(phases)

    if rank != 0:
        return
    errs = errors_vs_fp64(P, prob, args.mode)
    burst, sustained, hbm, src = peaks()
    launches = kernels.pop('_launches')
    rl = roofline(args.workload, args.mode, kernels, sustained, src, clk)
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_max, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32' if args.mode == 'native' else 'f32 (%s products)' % args.mode,
        'data': 'synthetic (seeded generator; observed = model + N(0,0.1) noise)',
        'config': {'workload': workload_desc(args.workload), 'mode': args.mode, 'terms_per_step': terms,
                   'l2': 'inputs larger than L2 (observed_vis alone %.1f GB)'
                         % (prob.arrays['observed_vis'].numel() * 8 / 1e9),
                   'phase': 'FP64 argument and range reduction', 'replicas': ws},
        'forward_ms': fwd_ms, 'adjoint_ms': adj_ms,
        'roofline': rl,
        'kernels_ms_per_step': {k: v[0] / args.steps for k, v in sorted(kernels.items())},
        'errors_vs_fp64': errs,
        'gpu_launches': launches,
        'clocks': clk,
    }
    if plain:
        line['plain_fp32'] = plain
        line['split_over_plain'] = value / plain['value']
    if e2e:
        line['e2e'] = e2e
    if not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(P, prob)
    if not args.no_batch:
        line['batched'] = batched_likelihood(args.seed)
    print(json.dumps(line))


if __name__ == '__main__':
    main()

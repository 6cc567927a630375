"""Batched likelihood: chi^2 and its gradient for many parameter sets
against one observation.

A sampler proposes many source models at once; every proposal shares the
observation (uvw, antenna pairs, frequencies, beam, pointing, G, flags,
weights, observed visibilities) and differs only in its sources (lm,
Stokes, alpha, shapes), with its own source counts.  ``RimeBatch`` keeps the
observation on the device once, the sets' parameters in concatenated device
arrays, and evaluates every set's chi^2 and gradient with ``mb_rime_batch``:
all sets of one kernel form run as one forward launch and one adjoint
launch whose CTAs are the sets' (time, channel) units (largest sets first),
so a batch is a fixed handful of launches (shared tables, one forward and
one adjoint per (form, source tile), the chi^2 sums, the gradients), which
``capture`` records once as a CUDA graph and ``run`` replays.

The kernel form of each set (CUDA-core ``native`` or tensor-core
``split_tf32``) and the source tile of its CUDA-core kernels (sources per
shared-memory tile: 8, 16 or 32) are chosen by ``autotune``, which times
every candidate on representative sets of each source-count range and keeps
the fastest: small source counts favour the CUDA-core tiles, large ones the
tensor cores.
"""
import ctypes

import numpy as np
import torch

from . import _cabi
from .solver import ptr

SHARED_FLOAT = ('uvw', 'frequency', 'ref_frequency', 'parallactic_angles', 'point_errors',
                'antenna_scaling', 'weight_vector')
SHARED_COMPLEX = ('E_beam', 'G_term', 'observed_vis')
PER_SET = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape')
FORMS = ('native', 'split_tf32')
#: (form, source tile) pairs the autotuner times by default; tile 0 is the
#: library default.  The tile only concerns the CUDA-core kernels: all of a
#: native set, the extended sources' adjoint of a split set.
CANDIDATES = (('native', 8), ('native', 16), ('native', 32), ('split_tf32', 0), ('split_tf32', 16))


def make_sets(P, nsets, seed=0, lo=10, hi=5000, gauss_fraction=0.16, sersic_fraction=0.04):
    """Synthetic proposals for observation P: per set a source count
    log-uniform in [lo, hi], split into point / gaussian / sersic sources,
    parameters drawn like montblanc_gb300.synth draws them."""
    rng = np.random.default_rng(seed)
    ntime = P['uvw'].shape[0]
    sets = []
    for _ in range(nsets):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        ng = int(round(n * gauss_fraction))
        ns = int(round(n * sersic_fraction))
        npt = max(n - ng - ns, 0)
        tot = npt + ng + ns
        I = rng.uniform(1.0, 10.0, tot)
        stokes = np.concatenate([I[:, None], I[:, None] * rng.uniform(-0.1, 0.1, (tot, 3))], axis=1)
        sets.append({
            'npsrc': npt, 'ngsrc': ng, 'nssrc': ns,
            'lm': rng.uniform(-0.05, 0.05, (tot, 2)),
            'stokes': np.repeat(stokes[:, None, :], ntime, axis=1),
            'alpha': np.repeat(rng.uniform(-0.8, 0.8, tot)[:, None], ntime, axis=1),
            'gauss_shape': np.stack([rng.uniform(0, 1e-4, ng), rng.uniform(0, 1e-4, ng), rng.uniform(0.5, 1, ng)]),
            'sersic_shape': np.stack([rng.uniform(-0.3, 0.3, ns), rng.uniform(-0.3, 0.3, ns),
                                      rng.uniform(1e-5, 1e-4, ns)]),
        })
    return sets


class RimeBatch(object):
    """chi^2 + gradient of ``sets`` (list of dicts with npsrc, ngsrc, nssrc
    and the PER_SET arrays) against the observation in ``P`` (a problem
    dict as montblanc_gb300.synth makes, without source arrays needed)."""

    def __init__(self, P, sets, dtype='float', device='cuda', want_G_grad=False):
        self.dtype = dtype
        self.mb_dtype = _cabi.MB_FLOAT64 if dtype == 'double' else _cabi.MB_FLOAT32
        self.tft = torch.float64 if dtype == 'double' else torch.float32
        self.tct = torch.complex128 if dtype == 'double' else torch.complex64
        self.device = torch.device(device)
        self.use_weight_vector = bool(P.get('use_weight_vector', False))
        self.residuals = bool(P.get('residuals', False))
        self.props = {k: float(P[k]) for k in _cabi.PROP_NAMES}
        ntime, na = P['uvw'].shape[:2]
        self.ntime, self.na = int(ntime), int(na)
        self.nbl = int(P['antenna1'].shape[1])
        self.nchan = int(P['frequency'].shape[0])
        self.beam = tuple(int(x) for x in P['E_beam'].shape[:3])
        dev = self.device
        sh = {}
        for k in SHARED_FLOAT:
            if k == 'weight_vector' and not self.use_weight_vector:
                sh[k] = None
                continue
            sh[k] = torch.as_tensor(np.ascontiguousarray(P[k])).to(device=dev, dtype=self.tft)
        for k in SHARED_COMPLEX:
            sh[k] = torch.as_tensor(np.ascontiguousarray(P[k])).to(device=dev, dtype=self.tct)
        for k in ('antenna1', 'antenna2'):
            sh[k] = torch.as_tensor(np.ascontiguousarray(P[k], dtype=np.int32)).to(dev)
        vshape = (self.ntime, self.nbl, self.nchan, 4)
        sh['flag'] = (torch.as_tensor(np.ascontiguousarray(P['flag'], dtype=np.uint8)).to(dev)
                      if 'flag' in P else torch.zeros(vshape, dtype=torch.uint8, device=dev))
        self.shared = sh
        # concatenated per-set parameters; a set's gaussian / sersic block is
        # its own (3, n) matrix, so its row stride is its own count
        self.counts = [(int(s['npsrc']), int(s['ngsrc']), int(s['nssrc'])) for s in sets]
        self.nsets = len(sets)
        nsrc = np.array([sum(c) for c in self.counts])
        self.src_off = np.concatenate([[0], np.cumsum(nsrc)])
        self.g_off = np.concatenate([[0], np.cumsum([3 * c[1] for c in self.counts])])
        self.x_off = np.concatenate([[0], np.cumsum([3 * c[2] for c in self.counts])])

        def cat(name):
            parts = [np.asarray(s[name], dtype=np.float64).reshape(-1) for s in sets]
            flat = np.concatenate(parts) if parts else np.zeros(0)
            return torch.as_tensor(flat).to(device=dev, dtype=self.tft)
        self.params = {n: cat(n) for n in PER_SET}
        self.grads = {n: torch.zeros_like(t) for n, t in self.params.items()}
        self.grad_G = (torch.zeros((self.nsets,) + tuple(sh['G_term'].shape), dtype=self.tct, device=dev)
                       if want_G_grad else None)
        self.X2 = torch.zeros(self.nsets, dtype=torch.float64, device=dev)
        self.forms = ['split_tf32' if dtype == 'float' else 'native'] * self.nsets
        self.tiles = [0] * self.nsets
        self._graph = None
        self._ws = None        # single-set workspace (autotuner timings)
        self._bws = None       # batch workspace
        self._prepared = None  # (forms, tiles) the batch workspace's tables were written for

    # ---- per-set call arguments -------------------------------------------------
    def _dims(self, i):
        npt, ng, ns = self.counts[i]
        return _cabi.make_dims(self.ntime, self.na, self.nbl, self.nchan, npt, ng, ns, beam=self.beam)

    def _options(self, i=None):
        o = _cabi.source_tile_bits(self.tiles[i]) if i is not None else 0
        if self.use_weight_vector:
            o |= _cabi.MB_APPLY_WEIGHTS
        if self.residuals:
            o |= _cabi.MB_RESIDUALS
        return o

    def _set_ptrs(self, store, i):
        es = torch.tensor([], dtype=self.tft).element_size()
        s0 = int(self.src_off[i])
        nt = self.ntime
        return {'lm': ptr(store['lm']) + s0 * 2 * es,
                'stokes': ptr(store['stokes']) + s0 * nt * 4 * es,
                'alpha': ptr(store['alpha']) + s0 * nt * es,
                'gauss_shape': ptr(store['gauss_shape']) + int(self.g_off[i]) * es if self.counts[i][1] else None,
                'sersic_shape': ptr(store['sersic_shape']) + int(self.x_off[i]) * es if self.counts[i][2] else None}

    def _inputs(self, i):
        x = _cabi.MbRimeInputs()
        p = self._set_ptrs(self.params, i)
        for n in _cabi.INPUT_NAMES:
            setattr(x, n, p[n] if n in p else ptr(self.shared.get(n)))
        return x

    def _grad_struct(self, i):
        g = _cabi.MbRimeGrads()
        p = self._set_ptrs(self.grads, i)
        for n in _cabi.GRAD_NAMES:
            if n == 'G_term':
                setattr(g, n, ptr(self.grad_G[i]) if self.grad_G is not None else None)
            else:
                setattr(g, n, p[n])
        return g

    def workspace(self):
        need = 0
        for i in range(self.nsets):
            d = self._dims(i)
            need = max(need, _cabi.lib.mb_rime_workspace_size(self.mb_dtype, _cabi.MODES[self.forms[i]],
                                                             ctypes.byref(d), 1))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.device)
        return self._ws

    def enqueue_set(self, i, stream=None):
        """Forward chi^2 (into X2[i]) and gradient of set i on the stream."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        handle = ctypes.c_void_p(s.cuda_stream)
        d = self._dims(i)
        mode = _cabi.MODES[self.forms[i]]
        props = _cabi.make_props(**self.props)
        inp = self._inputs(i)
        ws = self._ws
        _cabi.call('mb_rime_forward', self.mb_dtype, mode, ctypes.byref(d), ctypes.byref(props), self._options(i),
                   ctypes.byref(inp), None, None, ptr(self.X2) + 8 * i, 1, ptr(ws), ws.numel(), handle)
        g = self._grad_struct(i)
        _cabi.call('mb_rime_adjoint', self.mb_dtype, mode, ctypes.byref(d), ctypes.byref(props), self._options(i),
                   ctypes.byref(inp), 1.0, ctypes.byref(g), ptr(ws), ws.numel(), handle)

    # ---- the batched call ---------------------------------------------------------
    def _batch_sets(self):
        arr = (_cabi.MbBatchSet * max(self.nsets, 1))()
        for i in range(self.nsets):
            npt, ng, ns = self.counts[i]
            b = arr[i]
            b.npsrc, b.ngsrc, b.nssrc = npt, ng, ns
            b.mode = _cabi.MODES[self.forms[i]]
            b.options = _cabi.source_tile_bits(self.tiles[i]) if self.tiles[i] else 0
            b.reserved = 0
            p = self._set_ptrs(self.params, i)
            b.lm, b.stokes, b.alpha = p['lm'], p['stokes'], p['alpha']
            b.gauss_shape, b.sersic_shape = p['gauss_shape'], p['sersic_shape']
            b.grads = self._grad_struct(i)
        return arr

    def prepare(self, stream=None):
        """Size the batch workspace and write its per-set table and launch
        lists (synchronous; done again only when forms or tiles change)."""
        key = (tuple(self.forms), tuple(self.tiles))
        if self._prepared == key:
            return
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        self._sets_c = self._batch_sets()
        d = self._dims(0) if self.nsets else _cabi.make_dims(self.ntime, self.na, self.nbl, self.nchan, 0,
                                                             beam=self.beam)
        self._obs_dims = d
        need = _cabi.lib.mb_rime_batch_workspace_size(self.mb_dtype, ctypes.byref(d), self._sets_c, self.nsets)
        if need == 0 and self.nsets:
            raise _cabi.MontblancError(_cabi.MB_ERR_INVALID_ARG, 'mb_rime_batch_workspace_size',
                                       _cabi.lib.mb_last_error_string().decode())
        if self._bws is None or self._bws.numel() < need:
            self._bws = None
            self._bws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.device)
        _cabi.call('mb_rime_batch_prepare', self.mb_dtype, ctypes.byref(d), self._sets_c, self.nsets,
                   ptr(self._bws), self._bws.numel(), ctypes.c_void_p(s.cuda_stream))
        self._inputs_c = self._inputs(0) if self.nsets else None
        self._props_c = _cabi.make_props(**self.props)
        self._prepared = key

    def enqueue(self, stream=None):
        """chi^2 (into X2) and gradients of every set: one mb_rime_batch call."""
        self.prepare(stream)
        if self.nsets == 0:
            return
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _cabi.call('mb_rime_batch', self.mb_dtype, ctypes.byref(self._obs_dims), ctypes.byref(self._props_c),
                   self._options(), ctypes.byref(self._inputs_c), self._sets_c, self.nsets, ptr(self.X2), 1.0,
                   ptr(self._bws), self._bws.numel(), ctypes.c_void_p(s.cuda_stream))

    # ---- tuning and graphs -------------------------------------------------------------
    def _time_set(self, i, form, reps, tile=0):
        self.forms[i] = form
        self.tiles[i] = tile
        self.workspace()
        self.enqueue_set(i)
        torch.cuda.synchronize(self.device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            self.enqueue_set(i)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def autotune(self, forms=None, buckets=8, reps=2, candidates=None):
        """Choose the kernel form and source tile of every set by measurement.

        Sets are grouped into ``buckets`` ranges of log source count; the set
        at each bucket's median is timed with every candidate (form, source
        tile) pair (CUDA events, after one warm-up) and the bucket takes the
        fastest.  ``forms`` restricts the candidates to those forms;
        ``buckets=None`` times every set.  Returns the per-set forms (the
        tiles are in ``self.tiles``)."""
        cands = list(candidates or CANDIDATES)
        if forms is not None:
            cands = [c for c in cands if c[0] in forms]
        if self.dtype != 'float':
            cands = [c for c in cands if c[0] == 'native'] or [('native', 0)]
        n = np.array([sum(c) for c in self.counts])
        if buckets is None or buckets >= self.nsets:
            groups = [[i] for i in range(self.nsets)]
        else:
            edges = np.quantile(np.log(n), np.linspace(0.0, 1.0, buckets + 1))
            idx = np.clip(np.searchsorted(edges, np.log(n), side='right') - 1, 0, buckets - 1)
            groups = [list(np.nonzero(idx == b)[0]) for b in range(buckets)]
            groups = [g for g in groups if g]
        forms_out, tiles_out = list(self.forms), list(self.tiles)
        self.tune_times = {}
        for g in groups:
            rep_set = int(g[np.argsort(n[g])[len(g) // 2]])
            t = [self._time_set(rep_set, f, reps, tile) for f, tile in cands]
            best = cands[int(np.argmin(t))]
            self.tune_times[int(n[rep_set])] = {'%s/%d' % c: ms for c, ms in zip(cands, t)}
            for i in g:
                forms_out[i], tiles_out[i] = best
        self.forms, self.tiles = forms_out, tiles_out
        self._graph = None
        return forms_out

    def capture(self):
        """Capture the whole batch as one CUDA graph (forms fixed)."""
        self.prepare()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode='relaxed'):
            self.enqueue()
        self._graph = g
        return g

    def run(self):
        """chi^2 (device float64, one per set) and gradients of every set;
        gradients land in ``self.grads`` (concatenated like the parameters)
        and, if asked for, ``self.grad_G``."""
        if self._graph is not None:
            self._graph.replay()
        else:
            self.enqueue()
        return self.X2

    # ---- views -----------------------------------------------------------------------
    def set_grads(self, i):
        """Host copies of set i's gradients in the v4 shapes."""
        npt, ng, ns = self.counts[i]
        n = npt + ng + ns
        s0, s1 = int(self.src_off[i]), int(self.src_off[i + 1])
        nt = self.ntime
        out = {'lm': self.grads['lm'][2 * s0:2 * s1].view(n, 2),
               'stokes': self.grads['stokes'][4 * nt * s0:4 * nt * s1].view(n, nt, 4),
               'alpha': self.grads['alpha'][nt * s0:nt * s1].view(n, nt),
               'gauss_shape': self.grads['gauss_shape'][int(self.g_off[i]):int(self.g_off[i + 1])].view(3, ng),
               'sersic_shape': self.grads['sersic_shape'][int(self.x_off[i]):int(self.x_off[i + 1])].view(3, ns)}
        if self.grad_G is not None:
            out['G_term'] = self.grad_G[i]
        return {k: v.cpu().numpy() for k, v in out.items()}

    def terms(self):
        """source.vis terms of one evaluation of the whole batch."""
        return int(self.src_off[-1]) * self.ntime * self.nbl * self.nchan

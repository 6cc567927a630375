"""Streaming RIME solver on one GPU: the reference's v5 driver semantics.

The reference's ``CompositeRimeSolver``
(``montblanc/impl/rime/v5/CompositeRimeSolver.py``) keeps the whole problem
in host (NumPy) arrays, cuts the visibility space into chunks sized by a
device-memory budget (``_gen_vis_slices``, :284-339), runs each chunk's
sources in batches of ``source_batch_size`` (``_gen_source_slices``,
:230-282) with the partial sums carried in the model visibilities, copies
each chunk's model visibilities and chi^2 back asynchronously, and writes
them into the host ``model_vis`` by overwriting or summing
(``vis_write_mode``, :1122-1131).  chi^2 is the sum over chunks, divided by
sigma^2 when no weight vector is used (:1207-1213).

Here the same contract runs on one GB300:

* host arrays are NumPy arrays named as the v4 arrays; arrays supplied in
  ``array_cfg['supplied']`` are used as given (shape checked, dtype kept),
  arrays listed in ``array_cfg['ignore']`` are not created;
* the visibility space is cut into (time, channel) chunks.  Baselines are
  not cut: the fused kernels consume whole (time, channel) units, and one
  unit needs only ``nbl * 4`` visibilities on the device, so time and
  channel chunking alone fit any problem into any budget;
* ``nsolvers`` chunk slots, each with its own CUDA stream, device buffers
  and pinned host staging buffers, are used round robin, so the host-side
  staging and write-back of one chunk overlaps the device work of others;
* every source batch of a chunk is one ``mb_rime_forward`` call whose nsrc
  extents mark it as the first / a middle / the last batch (the kernels
  accumulate partial sums in the chunk's model visibilities and apply G,
  flags and chi^2 after the last batch);
* ``solve_with_gradient`` streams chi^2 and its gradient in the same
  chunks (sources are not batched there: the adjoint needs the complete
  model of its chunk).
"""
import ctypes

import numpy as np
import torch

from . import _cabi
from .config import ARRAYS, PROPERTIES, STAGE_SCRATCH, Options, gen_cfg
from .solver import Dimension, nr_of_baselines, ptr
from .src_types import source_nr_vars, sources_to_nr_vars

#: Extra configuration keys of the streaming solver.
VIS_CHUNK = 'vis_chunk'        # (ntime, nchan) per chunk, overrides the budget
MEM_BUDGET = 'mem_budget'      # device bytes for all chunk slots

#: Arrays whose leading dims are sliced per chunk: name -> (time axis,
#: channel axis) within the array (None: not sliced along that dimension).
CHUNK_AXES = {
    'uvw': (0, None), 'antenna1': (0, None), 'antenna2': (0, None),
    'parallactic_angles': (0, None), 'point_errors': (0, 2), 'antenna_scaling': (None, 1),
    'frequency': (None, 0), 'ref_frequency': (None, 0), 'G_term': (0, 2),
    'stokes': (1, None), 'alpha': (1, None), 'flag': (0, 2), 'weight_vector': (0, 2),
    'observed_vis': (0, 2), 'model_vis': (0, 2),
}
#: Arrays copied to the device whole, once per solve.
WHOLE = ('lm', 'gauss_shape', 'sersic_shape', 'E_beam')
#: Visibility-shaped outputs of a chunk.
OUTPUTS = ('model_vis',)


def gen_vis_chunks(ntime, nchan, nt, nc):
    """(t0, t1, c0, c1) of every chunk, time-major like the reference's
    ``_gen_vis_slices`` (CompositeRimeSolver.py:308-337)."""
    for t0 in range(0, ntime, nt):
        for c0 in range(0, nchan, nc):
            yield t0, min(t0 + nt, ntime), c0, min(c0 + nc, nchan)


def gen_source_batches(counts, batch):
    """Source batches over the point, gaussian, sersic ordering.

    ``counts`` maps npsrc / ngsrc / nssrc to their totals.  Yields
    (s0, s1, {var: (first index of the type in the batch, count)}), like the
    reference's ``_gen_source_slices`` with ``source_range_slices``
    (CompositeRimeSolver.py:230-282)."""
    nsrc = sum(counts[v] for v in source_nr_vars())
    batch = max(1, int(batch))
    for s0 in range(0, nsrc, batch):
        s1 = min(s0 + batch, nsrc)
        per = {}
        start = 0
        for v in source_nr_vars():
            lo, hi = start, start + counts[v]
            a, b = max(lo, s0), min(hi, s1)
            per[v] = (a - lo, max(0, b - a))
            start = hi
        yield s0, s1, per


def chunk_bytes(nt, nc, na, nbl, nsrc, ft_bytes, weights):
    """Device bytes one chunk slot holds for an (nt, nc) chunk: the sliced
    arrays plus the fused forward's workspace estimate."""
    ct = 2 * ft_bytes
    vis = nt * nbl * nc * 4
    per_vis = 2 * ct + 1 + (ft_bytes if weights else 0)  # observed + model, flag, weight
    b = vis * per_vis
    b += nt * na * nc * (4 * ct + 2 * ft_bytes)           # G, pointing errors
    b += nt * (na * (3 + 1) * ft_bytes + 2 * nbl * 4)     # uvw, pa, antenna pairs
    b += nsrc * nt * 5 * ft_bytes                         # stokes, alpha
    b += nt * nbl * nc * ft_bytes                         # chi^2 terms
    b += nt * nsrc * na * 8                               # path lengths (8 bytes each)
    b += nt * nc * 8 + (1 << 16)
    return b


def plan_chunks(ntime, nchan, per_chunk_bytes, budget, nslots):
    """Largest (nt, nc), whole channels preferred, whose nslots slots fit in
    budget bytes.  per_chunk_bytes(nt, nc) gives one slot's size."""
    if per_chunk_bytes(1, 1) * nslots > budget:
        raise ValueError('memory budget %d bytes cannot hold %d slots of one (time, channel) unit'
                         % (budget, nslots))
    nc = nchan
    while nc > 1 and per_chunk_bytes(1, nc) * nslots > budget:
        nc = (nc + 1) // 2
    nt = 1
    while nt < ntime and per_chunk_bytes(min(2 * nt, ntime), nc) * nslots <= budget:
        nt = min(2 * nt, ntime)
    return nt, nc


class _Slot(object):
    """Device buffers, pinned staging buffers and the stream of one chunk slot."""

    def __init__(self, device):
        self.stream = torch.cuda.Stream(device=device)
        self.dev = {}
        self.pin = {}
        self.event = None
        self.pending = None  # (t0, t1, c0, c1, x2 pinned, outputs)

    def buffer(self, kind, name, shape, dtype, device):
        store = self.dev if kind == 'dev' else self.pin
        n = int(np.prod(shape)) if len(shape) else 1
        buf = store.get(name)
        if buf is None or buf.numel() < n or buf.dtype != dtype:
            if kind == 'dev':
                buf = torch.empty(max(n, 1), dtype=dtype, device=device)
            else:
                buf = torch.empty(max(n, 1), dtype=dtype, pin_memory=True)
            store[name] = buf
        return buf[:n].view(shape)


class CompositeRimeSolver(object):
    """Host-resident RIME v4 problem solved in streamed (time, channel)
    chunks with batched sources; see the module docstring."""

    def __init__(self, slvr_cfg):
        cfg = gen_cfg(**slvr_cfg)
        self._slvr_cfg = cfg
        if cfg[Options.DTYPE] == Options.DTYPE_FLOAT:
            self.ft, self.ct = np.float32, np.complex64
            self.tft, self.tct = torch.float32, torch.complex64
        else:
            self.ft, self.ct = np.float64, np.complex128
            self.tft, self.tct = torch.float64, torch.complex128
        self.device = torch.device(cfg.get(Options.DEVICE, 'cuda'))
        self._use_weight_vector = bool(cfg.get(Options.WEIGHT_VECTOR, False))
        self._vis_output = cfg.get(Options.VISIBILITY_OUTPUT, Options.VISIBILITY_OUTPUT_MODEL)
        self._write_mode = cfg.get(Options.VISIBILITY_WRITE_MODE, Options.VISIBILITY_WRITE_MODE_OVERWRITE)
        self._autocor = bool(cfg.get(Options.AUTO_CORRELATIONS, False))
        self.rime_mode = cfg.get(Options.RIME_MODE, 'native')
        self.source_batch_size = int(cfg.get(Options.SOURCE_BATCH_SIZE, 500))
        self.nsolvers = max(1, int(cfg.get(Options.NSOLVERS, 2)))
        self._dims = {}
        self._register_dimensions()
        self._properties = {name: self.ft(default) for name, _, default in PROPERTIES}
        for name, value in self._properties.items():
            setattr(self, name, value)
        array_cfg = cfg.get('array_cfg', {}) or {}
        self._create_arrays(cfg.get(Options.DATA_SOURCE, Options.DATA_SOURCE_DEFAULT),
                            array_cfg.get('supplied') or {}, array_cfg.get('ignore') or ())
        self._chunk = cfg.get(VIS_CHUNK)
        self._budget = cfg.get(MEM_BUDGET)
        self._slots = None

    # ---- dimensions -------------------------------------------------------
    def _register_dimensions(self):
        cfg = self._slvr_cfg
        ntime, na, nchan, npol = cfg[Options.NTIME], cfg[Options.NA], cfg[Options.NCHAN], cfg[Options.NPOL]
        nbl = cfg.get(Options.NBL, nr_of_baselines(na, self._autocor))
        sizes = [('ntime', ntime), ('na', na), ('nbl', nbl), ('nchan', nchan), ('npol', npol),
                 ('npolchan', nchan * npol), ('nvis', ntime * nbl * nchan),
                 ('beam_lw', cfg[Options.E_BEAM_WIDTH]), ('beam_mh', cfg[Options.E_BEAM_HEIGHT]),
                 ('beam_nud', cfg[Options.E_BEAM_DEPTH])]
        nr = sources_to_nr_vars(cfg.get(Options.SOURCES) or {})
        sizes.append(('nsrc', sum(nr.values())))
        sizes.extend(nr.items())
        for name, n in sizes:
            self._dims[name] = Dimension(name, n)

    def dim_local_size(self, *names):
        v = tuple(self._dims[n].local_size for n in names)
        return v[0] if len(v) == 1 else v

    def dimensions(self):
        return self._dims

    # ---- arrays -------------------------------------------------------------
    def _np_dtype(self, dt):
        return {'ft': self.ft, 'ct': self.ct, 'int32': np.int32, 'uint8': np.uint8}[dt]

    def _shape(self, sym):
        return tuple(self._dims[s].local_size if isinstance(s, str) else s for s in sym)

    def default_base_ant_pairs(self):
        """solvers/rime_solver.py:92-99"""
        return np.triu_indices(self.dim_local_size('na'), 0 if self._autocor else 1)

    def default_ant_pairs(self):
        """impl/rime/v4/ant_pairs.py:23-37"""
        ntime, nbl = self.dim_local_size('ntime', 'nbl')
        a0, a1 = (a[:nbl] for a in self.default_base_ant_pairs())
        return np.tile(a0, ntime).reshape(ntime, nbl), np.tile(a1, ntime).reshape(ntime, nbl)

    def _create_arrays(self, data_source, supplied, ignore):
        self._arrays = {}
        unknown = [n for n in supplied if n not in ARRAYS]
        if unknown:
            raise ValueError('Supplied arrays %s are not v4 arrays' % unknown)
        for name, (sym, dt, default) in ARRAYS.items():
            if name in STAGE_SCRATCH or name in ignore:
                continue
            shape = self._shape(sym)
            if name in supplied:
                ary = np.asarray(supplied[name])
                if tuple(ary.shape) != shape:
                    raise ValueError("Supplied array '%s' has shape %s, expected %s"
                                     % (name, tuple(ary.shape), shape))
                host = ary
            else:
                host = np.zeros(shape, dtype=self._np_dtype(dt))
                if data_source == Options.DATA_SOURCE_TEST:
                    from . import testdata
                    testdata.fill(self, name, host)
                elif data_source != Options.DATA_SOURCE_EMPTY and default is not None and host.size:
                    host[...] = default(self, host) if callable(default) else default
            self._arrays[name] = host
            setattr(self, name, host)

    def arrays(self):
        return dict(self._arrays)

    def transfer(self, name, npary):
        """Copy npary into the host array ``name`` (shape checked)."""
        ary = self._arrays[name]
        npary = np.asarray(npary)
        if npary.shape != ary.shape:
            raise ValueError("Array '%s' has shape %s, expected %s" % (name, npary.shape, ary.shape))
        ary[...] = npary

    def __getattr__(self, attr):
        if attr.startswith('transfer_') and attr[len('transfer_'):] in ARRAYS:
            name = attr[len('transfer_'):]
            return lambda npary: self.transfer(name, npary)
        if attr.startswith('retrieve_') and attr[len('retrieve_'):] in ARRAYS:
            name = attr[len('retrieve_'):]
            return lambda: self._arrays[name].copy()
        if attr.startswith('set_') and attr[len('set_'):] in self.__dict__.get('_properties', {}):
            name = attr[len('set_'):]
            return lambda value: self.set_property(name, value)
        raise AttributeError(attr)

    def config(self):
        return self._slvr_cfg

    # ---- properties / options ---------------------------------------------
    def set_property(self, name, value):
        self._properties[name] = self.ft(value)
        setattr(self, name, self.ft(value))

    def set_X2(self, value):
        self.X2 = float(value)

    def use_weight_vector(self):
        return self._use_weight_vector

    def outputs_residuals(self):
        return self._vis_output == Options.VISIBILITY_OUTPUT_RESIDUALS

    def mb_dtype(self):
        return _cabi.MB_FLOAT32 if self.ft == np.float32 else _cabi.MB_FLOAT64

    def mb_options(self):
        o = 0
        if self._use_weight_vector:
            o |= _cabi.MB_APPLY_WEIGHTS
        if self.outputs_residuals():
            o |= _cabi.MB_RESIDUALS
        return o

    def mb_props(self):
        return _cabi.make_props(**{n: float(getattr(self, n)) for n in _cabi.PROP_NAMES})

    # ---- chunk plan -----------------------------------------------------------
    def chunk_shape(self):
        """(ntime, nchan) of the visibility chunks."""
        ntime, nchan, na, nbl, nsrc = self.dim_local_size('ntime', 'nchan', 'na', 'nbl', 'nsrc')
        if self._chunk is not None:
            nt, nc = (int(x) for x in self._chunk)
            return max(1, min(nt, ntime)), max(1, min(nc, nchan))
        budget = self._budget
        if budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget = free // 2
        fb = np.dtype(self.ft).itemsize

        def per(nt, nc):
            return chunk_bytes(nt, nc, na, nbl, nsrc, fb, self._use_weight_vector)

        return plan_chunks(ntime, nchan, per, int(budget), self.nsolvers)

    def vis_chunks(self):
        nt, nc = self.chunk_shape()
        return list(gen_vis_chunks(self.dim_local_size('ntime'), self.dim_local_size('nchan'), nt, nc))

    def source_batches(self):
        counts = {v: self.dim_local_size(v) for v in source_nr_vars()}
        return list(gen_source_batches(counts, self.source_batch_size))

    # ---- device staging -----------------------------------------------------------
    def _torch_dtype(self, ary):
        return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
                np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128,
                np.dtype(np.int32): torch.int32, np.dtype(np.uint8): torch.uint8}[np.dtype(ary.dtype)]

    def _compute_dtype(self, name):
        dt = ARRAYS[name][1]
        return {'ft': self.tft, 'ct': self.tct, 'int32': torch.int32, 'uint8': torch.uint8}[dt]

    def _host_slice(self, name, t0, t1, c0, c1):
        ary = self._arrays[name]
        ta, ca = CHUNK_AXES[name]
        idx = [slice(None)] * ary.ndim
        if ta is not None:
            idx[ta] = slice(t0, t1)
        if ca is not None:
            idx[ca] = slice(c0, c1)
        return ary[tuple(idx)]

    def _stage(self, slot, name, host):
        """Copy host (any layout) through the slot's pinned buffer to its
        device buffer, converted to the compute dtype, on the slot stream."""
        pin = slot.buffer('pin', name, host.shape, self._torch_dtype(host), None)
        np.copyto(pin.numpy(), host)
        dev = slot.buffer('dev', name, host.shape, self._compute_dtype(name), self.device)
        if pin.dtype == dev.dtype:
            dev.copy_(pin, non_blocking=True)
        else:
            raw = slot.buffer('dev', name + '.raw', host.shape, pin.dtype, self.device)
            raw.copy_(pin, non_blocking=True)
            dev.copy_(raw)
        return dev

    def _upload_whole(self):
        """Arrays used whole by every chunk, on the current stream."""
        self._whole = {}
        for name in WHOLE:
            if name in self._arrays:
                host = np.ascontiguousarray(self._arrays[name])
                self._whole[name] = torch.from_numpy(host).to(self.device).to(self._compute_dtype(name))

    def _slots_ready(self):
        if self._slots is None:
            self._slots = [_Slot(self.device) for _ in range(self.nsolvers)]
        return self._slots

    def _chunk_dims(self, t0, t1, c0, c1, src=None):
        """mb_dims of a chunk; src = (s0, s1, per-type (first, count)) for a
        source batch (parameter pointers then start at the batch)."""
        na, nbl, npol = self.dim_local_size('na', 'nbl', 'npol')
        nt, nc = t1 - t0, c1 - c0
        d = _cabi.MbDims()
        sizes = {'ntime': nt, 'na': na, 'nbl': nbl, 'nchan': nc, 'npol': npol, 'npolchan': nc * npol,
                 'beam_lw': self.dim_local_size('beam_lw'), 'beam_mh': self.dim_local_size('beam_mh'),
                 'beam_nud': self.dim_local_size('beam_nud')}
        for n, v in sizes.items():
            setattr(d, n, _cabi.MbDim(v, v, 0, v))
        nsrc = self.dim_local_size('nsrc')
        if src is None:
            setattr(d, 'nsrc', _cabi.MbDim(nsrc, nsrc, 0, nsrc))
            for v in source_nr_vars():
                n = self.dim_local_size(v)
                setattr(d, v, _cabi.MbDim(n, n, 0, n))
        else:
            s0, s1, per = src
            setattr(d, 'nsrc', _cabi.MbDim(nsrc, nsrc, s0, s1))
            for v in source_nr_vars():
                n = self.dim_local_size(v)
                setattr(d, v, _cabi.MbDim(n, n, 0, per[v][1]))
        return d

    def _inputs(self, dev, src=None):
        """MbRimeInputs of a chunk; for a source batch the per-source
        pointers start at the batch's first source (of each type)."""
        x = _cabi.MbRimeInputs()
        for n in _cabi.INPUT_NAMES:
            t = dev.get(n, self._whole.get(n))
            if n == 'weight_vector' and not self._use_weight_vector:
                t = None
            setattr(x, n, ptr(t))
        if src is not None:
            s0, s1, per = src
            fsz = torch.tensor([], dtype=self.tft).element_size()
            nt = dev['alpha'].shape[1]
            x.lm = ptr(self._whole['lm']) + s0 * 2 * fsz
            x.stokes = ptr(dev['stokes']) + s0 * nt * 4 * fsz
            x.alpha = ptr(dev['alpha']) + s0 * nt * fsz
            if 'gauss_shape' in self._whole and self._whole['gauss_shape'].numel():
                x.gauss_shape = ptr(self._whole['gauss_shape']) + per['ngsrc'][0] * fsz
            if 'sersic_shape' in self._whole and self._whole['sersic_shape'].numel():
                x.sersic_shape = ptr(self._whole['sersic_shape']) + per['nssrc'][0] * fsz
        return x

    def _workspace(self, slot, dims, want_grad):
        n = _cabi.lib.mb_rime_workspace_size(self.mb_dtype(), _cabi.MODES[self.rime_mode], ctypes.byref(dims),
                                             int(want_grad))
        return slot.buffer('dev', 'workspace' + ('.grad' if want_grad else ''), (max(n, 256),), torch.uint8,
                           self.device)

    def _enqueue_chunk(self, slot, t0, t1, c0, c1, want_grad=False):
        """Stage a chunk, run its source batches (or the forward + adjoint),
        and queue the copies of its outputs to pinned memory."""
        with torch.cuda.stream(slot.stream):
            dev = {}
            for name in CHUNK_AXES:
                if name in OUTPUTS or name not in self._arrays:
                    continue
                if name == 'weight_vector' and not self._use_weight_vector:
                    continue
                dev[name] = self._stage(slot, name, np.ascontiguousarray(self._host_slice(name, t0, t1, c0, c1)))
            nt, nc = t1 - t0, c1 - c0
            nbl = self.dim_local_size('nbl')
            model = slot.buffer('dev', 'model_vis', (nt, nbl, nc, 4), self.tct, self.device)
            x2 = slot.buffer('dev', 'X2', (1,), torch.float64, self.device)
            handle = ctypes.c_void_p(slot.stream.cuda_stream)
            mode = _cabi.MODES[self.rime_mode]
            grads = None
            if not want_grad:
                batches = self.source_batches()
                ws = self._workspace(slot, self._chunk_dims(t0, t1, c0, c1), False)
                for src in batches:
                    d = self._chunk_dims(t0, t1, c0, c1, src if len(batches) > 1 else None)
                    inp = self._inputs(dev, src if len(batches) > 1 else None)
                    _cabi.call('mb_rime_forward', self.mb_dtype(), mode, ctypes.byref(d),
                               ctypes.byref(self.mb_props()), self.mb_options(), ctypes.byref(inp),
                               model.data_ptr(), None, x2.data_ptr(), 0, ws.data_ptr(), ws.numel(), handle)
            else:
                d = self._chunk_dims(t0, t1, c0, c1)
                ws = self._workspace(slot, d, True)
                inp = self._inputs(dev)
                _cabi.call('mb_rime_forward', self.mb_dtype(), mode, ctypes.byref(d),
                           ctypes.byref(self.mb_props()), self.mb_options(), ctypes.byref(inp),
                           model.data_ptr(), None, x2.data_ptr(), 1, ws.data_ptr(), ws.numel(), handle)
                grads = self._chunk_grads(slot, dev, nt, nc)
                g = _cabi.MbRimeGrads()
                for n in _cabi.GRAD_NAMES:
                    setattr(g, n, ptr(grads.get(n)))
                _cabi.call('mb_rime_adjoint', self.mb_dtype(), mode, ctypes.byref(d),
                           ctypes.byref(self.mb_props()), self.mb_options(), ctypes.byref(inp), 1.0,
                           ctypes.byref(g), ws.data_ptr(), ws.numel(), handle)
            out_pin = slot.buffer('pin', 'out.model_vis', (nt, nbl, nc, 4), self.tct, None)
            out_pin.copy_(model, non_blocking=True)
            x2_pin = slot.buffer('pin', 'out.X2', (1,), torch.float64, None)
            x2_pin.copy_(x2, non_blocking=True)
            grads_pin = None
            if grads is not None:
                grads_pin = {}
                for n, t in grads.items():
                    p = slot.buffer('pin', 'out.' + n, tuple(t.shape), t.dtype, None)
                    p.copy_(t, non_blocking=True)
                    grads_pin[n] = p
            slot.event = torch.cuda.Event()
            slot.event.record(slot.stream)
        slot.pending = (t0, t1, c0, c1, x2_pin, out_pin, grads_pin)

    def _chunk_grads(self, slot, dev, nt, nc):
        nsrc, na = self.dim_local_size('nsrc', 'na')
        g = {'lm': slot.buffer('dev', 'g.lm', (nsrc, 2), self.tft, self.device),
             'stokes': slot.buffer('dev', 'g.stokes', (nsrc, nt, 4), self.tft, self.device),
             'alpha': slot.buffer('dev', 'g.alpha', (nsrc, nt), self.tft, self.device),
             'G_term': slot.buffer('dev', 'g.G_term', (nt, na, nc, 4), self.tct, self.device)}
        ng, ns = self.dim_local_size('ngsrc', 'nssrc')
        if ng:
            g['gauss_shape'] = slot.buffer('dev', 'g.gauss', (3, ng), self.tft, self.device)
        if ns:
            g['sersic_shape'] = slot.buffer('dev', 'g.sersic', (3, ns), self.tft, self.device)
        return g

    def _harvest(self, slot, write, grads_out=None):
        """Wait for a slot's chunk and fold its outputs into the host arrays."""
        if slot.pending is None:
            return 0.0
        slot.event.synchronize()
        t0, t1, c0, c1, x2_pin, out_pin, grads_pin = slot.pending
        slot.pending = None
        mv = self._arrays.get('model_vis')
        if mv is not None:
            write(mv[t0:t1, :, c0:c1, :], out_pin.numpy())
        if grads_out is not None and grads_pin is not None:
            grads_out['lm'] += grads_pin['lm'].numpy()
            grads_out['stokes'][:, t0:t1, :] += grads_pin['stokes'].numpy()
            grads_out['alpha'][:, t0:t1] += grads_pin['alpha'].numpy()
            grads_out['G_term'][t0:t1, :, c0:c1, :] = grads_pin['G_term'].numpy()
            for n in ('gauss_shape', 'sersic_shape'):
                if n in grads_pin:
                    grads_out[n] += grads_pin[n].numpy()
        return float(x2_pin.numpy()[0])

    def _run(self, want_grad):
        if self._write_mode == Options.VISIBILITY_WRITE_MODE_SUM:
            def write(dst, src):
                dst += src
        else:
            def write(dst, src):
                dst[...] = src
        grads_out = None
        if want_grad:
            nsrc, ntime, na, nchan = self.dim_local_size('nsrc', 'ntime', 'na', 'nchan')
            ng, ns = self.dim_local_size('ngsrc', 'nssrc')
            grads_out = {'lm': np.zeros((nsrc, 2)), 'stokes': np.zeros((nsrc, ntime, 4)),
                         'alpha': np.zeros((nsrc, ntime)),
                         'G_term': np.zeros((ntime, na, nchan, 4), dtype=np.complex128)}
            if ng:
                grads_out['gauss_shape'] = np.zeros((3, ng))
            if ns:
                grads_out['sersic_shape'] = np.zeros((3, ns))
        slots = self._slots_ready()
        self._upload_whole()
        torch.cuda.current_stream(self.device).synchronize()  # the slot streams read these
        X2 = 0.0
        for i, (t0, t1, c0, c1) in enumerate(self.vis_chunks()):
            slot = slots[i % len(slots)]
            X2 += self._harvest(slot, write, grads_out)
            self._enqueue_chunk(slot, t0, t1, c0, c1, want_grad)
        for slot in slots:
            X2 += self._harvest(slot, write, grads_out)
        # each chunk's chi^2 already carries 1 / sigma^2 when no weights apply
        self.set_X2(X2)
        return grads_out

    def solve(self):
        """chi^2 over all chunks into X2; model (or residual) visibilities
        into model_vis, overwritten or summed per vis_write_mode."""
        self._run(False)
        return True

    def solve_with_gradient(self):
        """Like solve, plus d chi^2 / d(lm, stokes, alpha, gauss_shape,
        sersic_shape, G_term) as host arrays (FP64 / complex128)."""
        return self._run(True)

    def initialise(self):
        return True

    def shutdown(self):
        self._slots = None
        return True

    def __enter__(self):
        self.initialise()
        return self

    def __exit__(self, etype, value, tb):
        self.shutdown()

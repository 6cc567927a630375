"""Functional entry to the fused chi^2 / gradient path.

``RimeProblem`` holds one problem's device arrays (named as the reference's
v4 arrays), its dims/props/options, and a workspace, and calls
``mb_rime_forward`` / ``mb_rime_adjoint``.  ``rime_chi2`` wraps the pair as
a ``torch.autograd.Function`` whose differentiable inputs are the source
parameters and G.
"""
import ctypes

import numpy as np
import torch

from . import _cabi
from .solver import ptr

FLOAT_INPUTS = ('uvw', 'frequency', 'ref_frequency', 'parallactic_angles', 'point_errors',
                'antenna_scaling', 'lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'weight_vector')
COMPLEX_INPUTS = ('E_beam', 'G_term', 'observed_vis')
PARAMS = ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term')


class RimeProblem(object):
    def __init__(self, arrays, props, npsrc, ngsrc, nssrc, use_weight_vector=False, residuals=False,
                 dtype='double', device='cuda'):
        self.dtype = dtype
        self.mb_dtype = _cabi.MB_FLOAT64 if dtype == 'double' else _cabi.MB_FLOAT32
        self.tft = torch.float64 if dtype == 'double' else torch.float32
        self.tct = torch.complex128 if dtype == 'double' else torch.complex64
        self.device = torch.device(device)
        self.arrays = arrays
        self.props = dict(props)
        self.npsrc, self.ngsrc, self.nssrc = int(npsrc), int(ngsrc), int(nssrc)
        self.use_weight_vector = bool(use_weight_vector)
        self.residuals = bool(residuals)
        ntime, na = arrays['uvw'].shape[:2]
        self.ntime, self.na = int(ntime), int(na)
        self.nbl = int(arrays['antenna1'].shape[1])
        self.nchan = int(arrays['frequency'].shape[0])
        self.nsrc = self.npsrc + self.ngsrc + self.nssrc
        self.beam = tuple(int(x) for x in arrays['E_beam'].shape[:3])
        self._ws = {}
        self._x2 = torch.zeros(1, dtype=torch.float64, device=self.device)
        # sources per shared-memory tile of the CUDA-core kernels (0: default)
        self.source_tile = 0

    # ---- construction -----------------------------------------------------
    @classmethod
    def from_numpy(cls, P, dtype='double', device='cuda', pin=False):
        """Copy a problem dict of NumPy arrays (see montblanc_gb300.synth) to
        the device in the requested precision."""
        tft = torch.float64 if dtype == 'double' else torch.float32
        tct = torch.complex128 if dtype == 'double' else torch.complex64
        arrays = {}
        ntime, nbl, nchan = P['antenna1'].shape[0], P['antenna1'].shape[1], P['frequency'].shape[0]
        vshape = (ntime, nbl, nchan, 4)
        for k in FLOAT_INPUTS:
            if k == 'weight_vector' and k not in P:
                # only read when weights are applied
                arrays[k] = (torch.ones(vshape, dtype=tft, device=device)
                             if P.get('use_weight_vector', False) else None)
                continue
            arrays[k] = torch.as_tensor(np.ascontiguousarray(P[k])).to(device=device, dtype=tft)
        for k in COMPLEX_INPUTS:
            if k == 'observed_vis' and k not in P:
                arrays[k] = torch.zeros(vshape, dtype=tct, device=device)
                continue
            arrays[k] = torch.as_tensor(np.ascontiguousarray(P[k])).to(device=device, dtype=tct)
        arrays['antenna1'] = torch.as_tensor(np.ascontiguousarray(P['antenna1'], dtype=np.int32)).to(device)
        arrays['antenna2'] = torch.as_tensor(np.ascontiguousarray(P['antenna2'], dtype=np.int32)).to(device)
        if 'flag' in P:
            arrays['flag'] = torch.as_tensor(np.ascontiguousarray(P['flag'], dtype=np.uint8)).to(device)
        else:
            arrays['flag'] = torch.zeros(vshape, dtype=torch.uint8, device=device)
        props = {k: float(P[k]) for k in _cabi.PROP_NAMES}
        return cls(arrays, props, P['npsrc'], P['ngsrc'], P['nssrc'], P.get('use_weight_vector', False),
                   P.get('residuals', False), dtype=dtype, device=device)

    def dims(self, src_extent=None):
        ext = {}
        glob = {}
        if src_extent is not None:
            ext['nsrc'] = src_extent
            glob['nsrc'] = self.nsrc
        return _cabi.make_dims(self.ntime, self.na, self.nbl, self.nchan, self.npsrc, self.ngsrc, self.nssrc,
                               beam=self.beam, extents=ext, globals_=glob)

    def mb_props(self):
        return _cabi.make_props(**self.props)

    def options(self):
        o = _cabi.source_tile_bits(self.source_tile)
        if self.use_weight_vector:
            o |= _cabi.MB_APPLY_WEIGHTS
        if self.residuals:
            o |= _cabi.MB_RESIDUALS
        return o

    def inputs(self, **override):
        x = _cabi.MbRimeInputs()
        for n in _cabi.INPUT_NAMES:
            t = override.get(n, self.arrays.get(n))
            setattr(x, n, ptr(t))
        return x

    def workspace(self, mode, want_grad):
        d = self.dims()
        n = _cabi.lib.mb_rime_workspace_size(self.mb_dtype, _cabi.MODES[mode], ctypes.byref(d), int(want_grad))
        key = (mode, bool(want_grad))
        buf = self._ws.get(key)
        if buf is None or buf.numel() < n:
            buf = torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)
            self._ws[key] = buf
        return buf

    def empty_vis(self):
        return torch.empty((self.ntime, self.nbl, self.nchan, 4), dtype=self.tct, device=self.device)

    def empty_chi2(self):
        return torch.empty((self.ntime, self.nbl, self.nchan), dtype=self.tft, device=self.device)

    # ---- calls --------------------------------------------------------------
    def forward(self, mode='native', want_grad=False, model_vis=None, chi_sqrd_result=None, stream=None,
                X2=None, overrides=None):
        """Launch the fused forward; returns the device chi^2 (1-element
        float64 tensor).  No host synchronisation."""
        d = self.dims()
        ws = self.workspace(mode, want_grad)
        inp = self.inputs(**(overrides or {}))
        out = self._x2 if X2 is None else X2
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _cabi.call('mb_rime_forward', self.mb_dtype, _cabi.MODES[mode], ctypes.byref(d),
                   ctypes.byref(self.mb_props()), self.options(), ctypes.byref(inp), ptr(model_vis),
                   ptr(chi_sqrd_result), ptr(out), int(want_grad), ptr(ws), ws.numel(),
                   ctypes.c_void_p(s.cuda_stream))
        return out

    def empty_grads(self):
        return {
            'lm': torch.empty_like(self.arrays['lm']),
            'stokes': torch.empty_like(self.arrays['stokes']),
            'alpha': torch.empty_like(self.arrays['alpha']),
            'gauss_shape': torch.empty_like(self.arrays['gauss_shape']),
            'sersic_shape': torch.empty_like(self.arrays['sersic_shape']),
            'G_term': torch.empty_like(self.arrays['G_term']),
        }

    def adjoint(self, mode='native', grad_scale=1.0, grads=None, stream=None, overrides=None):
        """Launch the adjoint after ``forward(..., want_grad=True)``; returns
        a dict of gradient tensors (same shapes/dtypes as the parameters)."""
        d = self.dims()
        ws = self.workspace(mode, True)
        inp = self.inputs(**(overrides or {}))
        g = grads if grads is not None else self.empty_grads()
        mg = _cabi.MbRimeGrads()
        for n in _cabi.GRAD_NAMES:
            setattr(mg, n, ptr(g.get(n)))
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _cabi.call('mb_rime_adjoint', self.mb_dtype, _cabi.MODES[mode], ctypes.byref(d),
                   ctypes.byref(self.mb_props()), self.options(), ctypes.byref(inp), float(grad_scale),
                   ctypes.byref(mg), ptr(ws), ws.numel(), ctypes.c_void_p(s.cuda_stream))
        return g

    def chi2_and_grad(self, mode='native', stream=None):
        x2 = self.forward(mode=mode, want_grad=True, stream=stream)
        g = self.adjoint(mode=mode, stream=stream)
        return x2, g

    def check(self, mode='native', want_grad=False, stream=None):
        """Synchronise and raise MontblancError (MB_ERR_TIMEOUT) if a bounded
        wait of the last forward / adjoint in (mode, want_grad) gave up."""
        d = self.dims()
        ws = self.workspace(mode, want_grad)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _cabi.call('mb_rime_status', self.mb_dtype, _cabi.MODES[mode], ctypes.byref(d), int(want_grad), ptr(ws),
                   ws.numel(), ctypes.c_void_p(s.cuda_stream))


class _RimeChi2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, problem, mode, lm, stokes, alpha, gauss_shape, sersic_shape, G_term):
        ov = {'lm': lm.detach().contiguous(), 'stokes': stokes.detach().contiguous(),
              'alpha': alpha.detach().contiguous(), 'gauss_shape': gauss_shape.detach().contiguous(),
              'sersic_shape': sersic_shape.detach().contiguous(), 'G_term': G_term.detach().contiguous()}
        x2 = problem.forward(mode=mode, want_grad=True, X2=torch.empty(1, dtype=torch.float64,
                                                                      device=problem.device), overrides=ov)
        ctx.problem, ctx.mode, ctx.ov = problem, mode, ov
        return x2[0].clone()

    @staticmethod
    def backward(ctx, gout):
        g = ctx.problem.adjoint(mode=ctx.mode, grad_scale=1.0, overrides=ctx.ov)
        s = gout.to(torch.float64)
        out = [(g[n] * s.to(g[n].real.dtype if g[n].is_complex() else g[n].dtype)) for n in PARAMS]
        return (None, None) + tuple(out)


def rime_chi2(problem, lm, stokes, alpha, gauss_shape, sersic_shape, G_term, mode='native'):
    """Differentiable chi^2 of ``problem`` at the given parameters.

    Gradients flow to lm, stokes, alpha, gauss_shape, sersic_shape and
    G_term; the complex gradient of G_term is d/dRe + i d/dIm, torch's
    convention for real-valued losses.  K and E are recomputed in the
    backward pass rather than stored."""
    return _RimeChi2.apply(problem, mode, lm, stokes, alpha, gauss_shape, sersic_shape, G_term)


class HostFeed(object):
    """chi^2 and gradient of a sequence of input sets that live in host
    memory, with the transfers overlapped with the kernels.

    Each ``submit`` copies one set of host arrays (``names``: any of the
    problem's input arrays, e.g. observed_vis, flag, G_term and the source
    parameters) to the device on a host-to-device stream, runs the fused
    forward and adjoint on a compute stream once that copy has landed, and
    copies chi^2 and the gradients back into the caller's host tensors on a
    device-to-host stream.  ``depth`` sets of device buffers rotate, so the
    copies of set i+1 and the read-back of set i-1 run while the kernels of
    set i do.  Host tensors should be pinned for the copies to be
    asynchronous; a submitted set's host inputs and outputs must stay alive
    and untouched until its ``done`` event has completed."""

    def __init__(self, problem, names, mode='native', depth=2, grad_scale=1.0):
        for n in names:
            if n not in _cabi.INPUT_NAMES or problem.arrays.get(n) is None:
                raise ValueError('%s is not an input array of this problem' % n)
        if depth < 1:
            raise ValueError('depth must be at least 1')
        self.problem, self.mode, self.names = problem, mode, tuple(names)
        self.grad_scale = float(grad_scale)
        dev = problem.device
        self.h2d = torch.cuda.Stream(dev)
        self.compute = torch.cuda.Stream(dev)
        self.d2h = torch.cuda.Stream(dev)
        self.slots = []
        for _ in range(depth):
            self.slots.append({
                'inputs': {n: torch.empty_like(problem.arrays[n]) for n in self.names},
                'grads': problem.empty_grads(),
                'x2': torch.zeros(1, dtype=torch.float64, device=dev),
                'loaded': torch.cuda.Event(enable_timing=True),
                'computed': torch.cuda.Event(enable_timing=True),
                'done': torch.cuda.Event(enable_timing=True),
                'used': False,
            })
        self.count = 0

    def submit(self, host_inputs, x2_out, grads_out, events=None):
        """Queue one set: ``host_inputs`` {name: host tensor} for every name
        of the feed, ``x2_out`` a 1-element float64 host tensor and
        ``grads_out`` {name: host tensor} (any subset of the gradient names)
        receiving the results.  Returns the event recorded after the
        read-back.  ``events``, if given, is a list of four timing events
        recorded before and after the copy in, after the kernels and after
        the read-back."""
        s = self.slots[self.count % len(self.slots)]
        self.count += 1
        p = self.problem
        with torch.cuda.stream(self.h2d):
            if s['used']:
                self.h2d.wait_event(s['computed'])   # the previous set's kernels read these buffers
            if events:
                events[0].record(self.h2d)
            for n in self.names:
                s['inputs'][n].copy_(host_inputs[n], non_blocking=True)
            s['loaded'].record(self.h2d)
            if events:
                events[1].record(self.h2d)
        self.compute.wait_event(s['loaded'])
        if s['used']:
            self.compute.wait_event(s['done'])       # the previous set's gradients have been read back
        x2 = p.forward(mode=self.mode, want_grad=True, X2=s['x2'], stream=self.compute, overrides=s['inputs'])
        p.adjoint(mode=self.mode, grad_scale=self.grad_scale, grads=s['grads'], stream=self.compute,
                  overrides=s['inputs'])
        s['computed'].record(self.compute)
        if events:
            events[2].record(self.compute)
        with torch.cuda.stream(self.d2h):
            self.d2h.wait_event(s['computed'])
            x2_out.copy_(x2, non_blocking=True)
            for n, t in grads_out.items():
                t.copy_(s['grads'][n], non_blocking=True)
            s['done'].record(self.d2h)
            if events:
                events[3].record(self.d2h)
        s['used'] = True
        return s['done']

    def synchronize(self):
        for st in (self.h2d, self.compute, self.d2h):
            st.synchronize()

"""Pipeline nodes: the reference's v4 stages and the v5 reduction, each a
thin call into the CUDA library, plus a fused forward node.

Each node reads the solver's arrays by name and launches on the given
stream (a torch.cuda.Stream; None = the solver's / current stream).
"""
import ctypes

import torch

from . import _cabi
from .node import Node
from .solver import ptr


def _stream(solver, stream):
    return solver.stream_handle(stream)


class RimeBSqrt(Node):
    """B_sqrt(nsrc, ntime, nchan, 4) from stokes and alpha
    (montblanc/impl/rime/v4/gpu/RimeBSqrt.py:151-228)."""

    def initialise(self, solver, stream=None):
        solver.ensure_array('B_sqrt')

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        _cabi.call('mb_bsqrt', s.mb_dtype(), ctypes.byref(s.mb_dims()), ptr(s.stokes), ptr(s.alpha),
                   ptr(s.frequency), ptr(s.ref_frequency), ptr(s.B_sqrt), _stream(s, stream))

    def post_execution(self, solver, stream=None):
        pass


class RimeEBeam(Node):
    """jones <- beam-cube E term (montblanc/impl/rime/v4/gpu/RimeEBeam.py:373-463)."""

    def initialise(self, solver, stream=None):
        solver.ensure_array('jones')

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        _cabi.call('mb_ebeam', s.mb_dtype(), ctypes.byref(s.mb_dims()), ctypes.byref(s.mb_props()),
                   ptr(s.lm), ptr(s.parallactic_angles), ptr(s.point_errors), ptr(s.antenna_scaling),
                   ptr(s.frequency), ptr(s.E_beam), ptr(s.jones), _stream(s, stream))

    def post_execution(self, solver, stream=None):
        pass


class RimeEKBSqrt(Node):
    """jones <- jones . (K * B_sqrt) (montblanc/impl/rime/v4/gpu/RimeEKBSqrt.py:201-276)."""

    def initialise(self, solver, stream=None):
        solver.ensure_array('jones')
        solver.ensure_array('B_sqrt')

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        _cabi.call('mb_ekb_sqrt', s.mb_dtype(), ctypes.byref(s.mb_dims()), ctypes.byref(s.mb_props()),
                   ptr(s.uvw), ptr(s.lm), ptr(s.frequency), ptr(s.B_sqrt), ptr(s.jones), _stream(s, stream))

    def post_execution(self, solver, stream=None):
        pass


class RimeSumCoherencies(Node):
    """Coherency sum, G, flags, residuals, chi^2 terms and the chi^2 scalar
    (montblanc/impl/rime/v4/gpu/RimeSumCoherencies.py:434-539).

    As in the reference, the chi^2 scalar is read back to the host (a
    device->host synchronisation) and divided by sigma_sqrd unless a weight
    vector is in use."""

    def initialise(self, solver, stream=None):
        solver.ensure_array('jones')
        self._x2 = torch.zeros(1, dtype=torch.float64, device=solver.device)

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        d = s.mb_dims()
        h = _stream(s, stream)
        _cabi.call('mb_sum_coherencies', s.mb_dtype(), ctypes.byref(d), ctypes.byref(s.mb_props()),
                   s.mb_options(), ptr(s.uvw), ptr(s.gauss_shape), ptr(s.sersic_shape), ptr(s.frequency),
                   ptr(s.antenna1), ptr(s.antenna2), ptr(s.jones), ptr(s.flag), ptr(s.weight_vector),
                   ptr(s.observed_vis), ptr(s.G_term), ptr(s.model_vis), ptr(s.chi_sqrd_result), h)
        if d.nsrc.upper_extent < d.nsrc.global_size:
            return
        ws = s.workspace(_cabi.lib.mb_reduce_chi2_workspace_size(ctypes.byref(d)), key='reduce')
        _cabi.call('mb_reduce_chi2', s.mb_dtype(), ctypes.byref(d), ptr(s.chi_sqrd_result), 1.0,
                   ptr(self._x2), ptr(ws), ws.numel(), h)
        x2 = self._x2.item()
        s.set_X2(x2 if s.use_weight_vector() else x2 / s.sigma_sqrd)

    def post_execution(self, solver, stream=None):
        pass


class RimeReduction(Node):
    """Sum of chi_sqrd_result over the active extents, returned as a device
    scalar without a host synchronisation
    (montblanc/impl/rime/v5/gpu/RimeReduction.py:26-64)."""

    def initialise(self, solver, stream=None):
        pass

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        d = s.mb_dims()
        out = torch.empty(1, dtype=torch.float64, device=s.device)
        ws = s.workspace(_cabi.lib.mb_reduce_chi2_workspace_size(ctypes.byref(d)), key='reduce')
        _cabi.call('mb_reduce_chi2', s.mb_dtype(), ctypes.byref(d), ptr(s.chi_sqrd_result), 1.0, ptr(out),
                   ptr(ws), ws.numel(), _stream(s, stream))
        return out

    def post_execution(self, solver, stream=None):
        pass


def rime_inputs(s, **override):
    """MbRimeInputs pointing at the solver's arrays (or overriding tensors)."""
    x = _cabi.MbRimeInputs()
    for n in _cabi.INPUT_NAMES:
        t = override.get(n, getattr(s, n))
        setattr(x, n, ptr(t))
    return x


class RimeV4Fused(Node):
    """The whole v4 forward (B_sqrt, E, K, coherency sum, G, chi^2) in one
    fused pass per (time, channel), without the per-antenna jones array.
    Writes model_vis, chi_sqrd_result and X2 like the four-node pipeline.
    ``mode`` selects the arithmetic ('native', 'split_tf32', 'split_bf16');
    default: the solver's ``rime_mode`` option."""

    def __init__(self, mode=None):
        super(RimeV4Fused, self).__init__()
        self.mode = mode

    def initialise(self, solver, stream=None):
        self._x2 = torch.zeros(1, dtype=torch.float64, device=solver.device)

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        s = solver
        d = s.mb_dims()
        mode = _cabi.MODES[self.mode or s.rime_mode]
        nbytes = _cabi.lib.mb_rime_workspace_size(s.mb_dtype(), mode, ctypes.byref(d), 0)
        ws = s.workspace(nbytes)
        inputs = rime_inputs(s)
        _cabi.call('mb_rime_forward', s.mb_dtype(), mode, ctypes.byref(d), ctypes.byref(s.mb_props()),
                   s.mb_options(), ctypes.byref(inputs), ptr(s.model_vis), ptr(s.chi_sqrd_result),
                   ptr(self._x2), 0, ptr(ws), ws.numel(), _stream(s, stream))
        if d.nsrc.upper_extent < d.nsrc.global_size:
            return
        # reads chi^2 back (a host synchronisation, like the reference's
        # .get()), after checking that no bounded device wait gave up
        _cabi.call('mb_rime_status', s.mb_dtype(), mode, ctypes.byref(d), 0, ptr(ws), ws.numel(),
                   _stream(s, stream))
        s.set_X2(self._x2.item())

    def post_execution(self, solver, stream=None):
        pass

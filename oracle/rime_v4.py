"""CPU oracle for the RIME v4 forward path (test infrastructure only).

This module is a NumPy restatement of the reference's CPU solver
(``montblanc/impl/rime/v4/cpu/CPUSolver.py``).  It exists so that the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` can check
and time the CUDA path.  The product never imports it.

Parity status: pinned.  ``tests/golden/make_golden.py`` runs the reference's
own ``CPUSolver`` (behind small shims for its missing dependencies) on seeded
inputs and stores the outputs as fixtures; ``tests/test_oracle_golden.py``
checks this module against them.

A problem is a plain dict of NumPy arrays named like the reference's arrays
(``montblanc/impl/rime/v4/config.py:131-247``) plus the scalar properties
(``config.py:54-69``) and the options ``npsrc``, ``ngsrc``, ``nssrc``,
``use_weight_vector`` and ``residuals``.  Every function accepts an optional
source slice and time slice so that large problems can be evaluated in chunks
(the sum over sources is linear and G is applied after it).
"""
import numpy as np

LIGHTSPEED = 299792458.0  # montblanc/__init__.py:52-59


def _src(P, s):
    return slice(None) if s is None else s


def brightness(P, srcs=None, times=None):
    """B(s,t,ch) = [[I+Q, U+iV], [U-iV, I-Q]] * (nu/nu_ref)**alpha.

    Follows CPUSolver.compute_b_jones (CPUSolver.py:235-265).
    Returns (nsrc, ntime, nchan, 4) complex.
    """
    S = P['stokes'][_src(P, srcs)][:, _src(P, times)]
    a = P['alpha'][_src(P, srcs)][:, _src(P, times)]
    I, Q, U, V = S[..., 0], S[..., 1], S[..., 2], S[..., 3]
    B = np.stack([I + Q, U + 1j * V, U - 1j * V, I - Q], axis=-1)
    ratio = P['frequency'] / P['ref_frequency']
    power = ratio[None, None, :] ** a[:, :, None]
    return B[:, :, None, :] * power[..., None]


def brightness_sqrt(B):
    """Square root of a brightness matrix with real, non-negative trace/det.

    Follows CPUSolver.compute_b_sqrt_jones (CPUSolver.py:267-317):
    s = sqrt(det), t = sqrt(trace + 2 s), sqrt(B) = (B + s*I) / t, with
    t := 1 where s == t == 0.
    """
    B = np.array(B, copy=True)
    trace = (B[..., 0] + B[..., 3]).real
    det = (B[..., 0] * B[..., 3] - B[..., 1] * B[..., 2]).real
    assert np.all(trace >= 0.0) and np.all(det >= 0.0)
    s = np.sqrt(det)
    t = np.sqrt(trace + 2 * s)
    t[(s == 0.0) & (t == 0.0)] = 1.0
    B[..., 0] += s
    B[..., 3] += s
    return B / t[..., None]


def phase_scalar(P, srcs=None, times=None):
    """K(s,t,a,ch) = exp(-2 pi i (u l + v m + w (n - 1)) nu / c).

    Follows CPUSolver.compute_k_jones_scalar_per_ant (CPUSolver.py:162-195).
    Returns (nsrc, ntime, na, nchan) complex.
    """
    lm = P['lm'][_src(P, srcs)]
    uvw = P['uvw'][_src(P, times)]
    l, m = lm[:, 0], lm[:, 1]
    n = np.sqrt(1.0 - l ** 2 - m ** 2) - 1.0
    phase = (l[:, None, None] * uvw[None, :, :, 0]
             + m[:, None, None] * uvw[None, :, :, 1]
             + n[:, None, None] * uvw[None, :, :, 2])
    arg = -2.0 * np.pi * phase[..., None] * P['frequency'][None, None, None, :] / LIGHTSPEED
    return np.exp(1j * arg)


def beam_grid_channel(P):
    """Channel grid coordinates of the beam cube (CPUSolver.py:408-414)."""
    nud = P['E_beam'].shape[2]
    vch = (nud - 1) * (P['frequency'] - P['beam_lfreq']) / (P['beam_ufreq'] - P['beam_lfreq'])
    vch = np.clip(vch, 0.0, nud - 1)
    g0 = np.floor(vch)
    g1 = np.minimum(g0 + 1.0, nud - 1)
    return g0.astype(np.int64), g1.astype(np.int64), vch - g0


def beam_grid_lm(P, srcs=None, times=None):
    """Rotated, offset and scaled source positions on the beam grid.

    Follows CPUSolver.compute_E_beam (CPUSolver.py:367-406).  Returns the
    clipped grid coordinates (vl, vm), each (nsrc, ntime, na, nchan).
    """
    lm = P['lm'][_src(P, srcs)]
    pa = P['parallactic_angles'][_src(P, times)]
    pe = P['point_errors'][_src(P, times)]
    sc = P['antenna_scaling']
    nl, nm = P['E_beam'].shape[0], P['E_beam'].shape[1]
    sint, cost = np.sin(pa), np.cos(pa)
    l0 = lm[:, 0][:, None, None]
    m0 = lm[:, 1][:, None, None]
    l = (l0 * cost[None] - m0 * sint[None])[..., None] + pe[None, ..., 0]
    m = (l0 * sint[None] + m0 * cost[None])[..., None] + pe[None, ..., 1]
    l = l * sc[None, None, :, :, 0]
    m = m * sc[None, None, :, :, 1]
    vl = np.clip((nl - 1) * (l - P['beam_ll']) / (P['beam_ul'] - P['beam_ll']), 0.0, nl - 1)
    vm = np.clip((nm - 1) * (m - P['beam_lm']) / (P['beam_um'] - P['beam_lm']), 0.0, nm - 1)
    return vl, vm


def e_beam(P, srcs=None, times=None):
    """Trilinearly interpolated, amplitude-renormalised beam E(s,t,a,ch,pol).

    Follows CPUSolver.compute_E_beam / trilinear_interpolate
    (CPUSolver.py:319-475): 8 corner gathers weighted by the simplified
    trilinear weights, then E = sum * (sum of weighted |E|) / |sum| with the
    normalisation set to 1 where 1/|sum| is not finite.
    """
    E = P['E_beam']
    nl, nm = E.shape[0], E.shape[1]
    vl, vm = beam_grid_lm(P, srcs, times)
    gl0 = np.floor(vl)
    gl1 = np.minimum(gl0 + 1.0, nl - 1)
    ld = vl - gl0
    gm0 = np.floor(vm)
    gm1 = np.minimum(gm0 + 1.0, nm - 1)
    md = vm - gm0
    gc0, gc1, chd = beam_grid_channel(P)
    chd = chd[None, None, None, :]
    acc = np.zeros(vl.shape + (4,), dtype=np.complex128)
    amp = np.zeros(vl.shape + (4,), dtype=np.float64)
    corners = [
        (gl0, gm0, gc0, (1 - ld) * (1 - md) * (1 - chd)),
        (gl1, gm0, gc0, ld * (1 - md) * (1 - chd)),
        (gl0, gm1, gc0, (1 - ld) * md * (1 - chd)),
        (gl1, gm1, gc0, ld * md * (1 - chd)),
        (gl0, gm0, gc1, (1 - ld) * (1 - md) * chd),
        (gl1, gm0, gc1, ld * (1 - md) * chd),
        (gl0, gm1, gc1, (1 - ld) * md * chd),
        (gl1, gm1, gc1, ld * md * chd),
    ]
    for gl, gm, gc, w in corners:
        vals = E[gl.astype(np.int64), gm.astype(np.int64), gc[None, None, None, :]]
        acc += w[..., None] * vals
        amp += w[..., None] * np.abs(vals)
    with np.errstate(divide='ignore', invalid='ignore'):
        norm = 1.0 / np.abs(acc)
    norm[~np.isfinite(norm)] = 1.0
    return acc * (norm * amp)


def jones_mul(A, B):
    """2x2 product of row-major [00,01,10,11] Jones arrays (CPUSolver.py:518-541)."""
    a = A.reshape(A.shape[:-1] + (2, 2))
    b = B.reshape(B.shape[:-1] + (2, 2))
    r = np.matmul(a, b)
    return r.reshape(r.shape[:-2] + (4,))


def jones_mul_h(A, B):
    """A @ B^H for row-major Jones arrays (CPUSolver.py:529-531)."""
    a = A.reshape(A.shape[:-1] + (2, 2))
    b = B.reshape(B.shape[:-1] + (2, 2))
    r = np.matmul(a, np.conj(np.swapaxes(b, -1, -2)))
    return r.reshape(r.shape[:-2] + (4,))


def ekb_sqrt_per_antenna(P, srcs=None, times=None):
    """J(s,t,a,ch) = E . (K * sqrt(B)).

    Follows CPUSolver.compute_kb_sqrt_jones_per_ant and
    compute_ekb_sqrt_jones_per_ant (CPUSolver.py:217-233, 543-560).
    """
    K = phase_scalar(P, srcs, times)
    Bs = brightness_sqrt(brightness(P, srcs, times))
    KB = K[..., None] * Bs[:, :, None, :, :]
    return jones_mul(e_beam(P, srcs, times), KB)


def baseline_uvw(P, times=None):
    """Per-baseline uvw = uvw[antenna2] - uvw[antenna1] (CPUSolver.py:69-79)."""
    tsl = _src(P, times)
    uvw = P['uvw'][tsl]
    a1 = P['antenna1'][tsl]
    a2 = P['antenna2'][tsl]
    t = np.arange(uvw.shape[0])[:, None]
    return uvw[t, a2] - uvw[t, a1]


def gaussian_shape(P, gsrcs, times=None):
    """Gaussian shape factors (ngsrc, ntime, nbl, nchan) (CPUSolver.py:59-103)."""
    buvw = baseline_uvw(P, times)
    u, v = buvw[..., 0], buvw[..., 1]
    el, em, R = (P['gauss_shape'][k][gsrcs] for k in range(3))
    u1 = em[:, None, None] * u[None] - el[:, None, None] * v[None]
    v1 = el[:, None, None] * u[None] + em[:, None, None] * v[None]
    k = (P['gauss_scale'] * P['frequency'])[None, None, None, :]
    return np.exp(-((u1[..., None] * k * R[:, None, None, None]) ** 2 + (v1[..., None] * k) ** 2))


def sersic_shape(P, ssrcs, times=None):
    """Sersic shape factors (nssrc, ntime, nbl, nchan) (CPUSolver.py:105-160)."""
    buvw = baseline_uvw(P, times)
    u, v = buvw[..., 0], buvw[..., 1]
    e1, e2, R = (P['sersic_shape'][k][ssrcs] for k in range(3))
    u1 = (1.0 + e1)[:, None, None] * u[None] + e2[:, None, None] * v[None]
    v1 = e2[:, None, None] * u[None] + (1.0 - e1)[:, None, None] * v[None]
    k = (P['two_pi_over_c'] * P['frequency'])[None, None, None, :]
    Rs = (R / (1.0 - e1 * e1 - e2 * e2))[:, None, None, None]
    den = 1.0 + (u1[..., None] * k * Rs) ** 2 + (v1[..., None] * k * Rs) ** 2
    return 1.0 / (den * np.sqrt(den))


def source_shape(P, s0, s1, times=None):
    """Shape factor for global sources [s0, s1): 1 for point sources,
    gaussian / sersic factors for the others (CPUSolver.py:585-597).
    Returns (s1-s0, ntime, nbl, nchan) or None if all are point sources."""
    npsrc, ngsrc = P['npsrc'], P['ngsrc']
    if s1 <= npsrc:
        return None
    buvw = baseline_uvw(P, times)
    ntime, nbl = buvw.shape[0], buvw.shape[1]
    out = np.ones((s1 - s0, ntime, nbl, P['frequency'].shape[0]))
    g0, g1 = max(s0, npsrc), min(s1, npsrc + ngsrc)
    if g1 > g0:
        out[g0 - s0:g1 - s0] = gaussian_shape(P, slice(g0 - npsrc, g1 - npsrc), times)
    x0, x1 = max(s0, npsrc + ngsrc), s1
    if x1 > x0:
        out[x0 - s0:x1 - s0] = sersic_shape(P, slice(x0 - npsrc - ngsrc, x1 - npsrc - ngsrc), times)
    return out


def ekb_vis(P, src_chunk=64, time_chunk=None, jones=None):
    """Sum over sources of shape * J_p J_q^H per (t, bl, ch).

    Follows CPUSolver.compute_ekb_jones_per_bl and compute_ekb_vis
    (CPUSolver.py:562-634), evaluated in source and time chunks.  If
    ``jones`` (nsrc, ntime, na, nchan, 4) is given it is used in place of
    the computed per-antenna terms (as the reference's coherency test does,
    tests/test_rime_v4.py:181-222).
    """
    nsrc = P['lm'].shape[0]
    ntime = P['uvw'].shape[0]
    nbl = P['antenna1'].shape[1]
    nchan = P['frequency'].shape[0]
    time_chunk = time_chunk or ntime
    vis = np.zeros((ntime, nbl, nchan, 4), dtype=np.complex128)
    for t0 in range(0, ntime, time_chunk):
        t1 = min(ntime, t0 + time_chunk)
        tsl = slice(t0, t1)
        a1 = P['antenna1'][tsl]
        a2 = P['antenna2'][tsl]
        tt = np.arange(t1 - t0)[:, None]
        for s0 in range(0, nsrc, src_chunk):
            s1 = min(nsrc, s0 + src_chunk)
            if jones is None:
                J = ekb_sqrt_per_antenna(P, slice(s0, s1), tsl)
            else:
                J = jones[s0:s1, tsl]
            Jp = J[:, tt, a1]
            Jq = J[:, tt, a2]
            X = jones_mul_h(Jp, Jq)
            shp = source_shape(P, s0, s1, tsl)
            if shp is not None:
                X = X * shp[..., None]
            vis[tsl] += X.sum(axis=0)
    return vis


def gekb_vis(P, vis):
    """Apply G_p V G_q^H, flagging, and model/residual output.

    Follows CPUSolver.compute_gekb_vis (CPUSolver.py:636-676).
    """
    t = np.arange(vis.shape[0])[:, None]
    Gp = P['G_term'][t, P['antenna1']]
    Gq = P['G_term'][t, P['antenna2']]
    M = jones_mul_h(jones_mul(Gp, vis), Gq)
    flagged = P['flag'] > 0
    if P.get('residuals', False):
        return (P['observed_vis'] - M) * np.where(flagged, 0.0, 1.0)
    M = np.array(M, copy=True)
    M[flagged] = 0
    return M


def chi_sqrd_terms(P, vis_out):
    """Weighted squared residuals summed over polarisations (ntime,nbl,nchan).

    Follows CPUSolver.compute_chi_sqrd_sum_terms (CPUSolver.py:678-722).
    """
    if P.get('residuals', False):
        d = vis_out
    else:
        d = (P['observed_vis'] - vis_out) * np.where(P['flag'] > 0, 0.0, 1.0)
    re = d.real ** 2
    im = d.imag ** 2
    if P.get('use_weight_vector', False):
        re = re * P['weight_vector']
        im = im * P['weight_vector']
    return re.sum(axis=3) + im.sum(axis=3)


def chi_sqrd(P, terms):
    """Sum of the terms, divided by sigma^2 without a weight vector (CPUSolver.py:724-737)."""
    s = terms.sum()
    return s if P.get('use_weight_vector', False) else s / P['sigma_sqrd']


def forward(P, src_chunk=64, time_chunk=None, jones=None):
    """Full v4 forward: returns (model-or-residual vis, chi^2 terms, chi^2)."""
    v = ekb_vis(P, src_chunk=src_chunk, time_chunk=time_chunk, jones=jones)
    out = gekb_vis(P, v)
    terms = chi_sqrd_terms(P, out)
    return out, terms, chi_sqrd(P, terms)

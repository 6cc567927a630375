"""FP64 NumPy gradient of the RIME v4 chi^2 (test infrastructure only).

The reference has no gradient, so this module is written from the forward
formulas in ``oracle/rime_v4.py`` (which restate
``montblanc/impl/rime/v4/cpu/CPUSolver.py``).  It is itself pinned by central
finite differences of the forward oracle (tests/test_adjoint_oracle.py).

Conventions: for a real parameter x the result is d chi^2 / dx; for the
complex G_term it is d chi^2 / dRe + i d chi^2 / dIm.  Source parameters are
the arrays lm (nsrc, 2), stokes (nsrc, ntime, 4), alpha (nsrc, ntime),
gauss_shape (3, ngsrc) and sersic_shape (3, nssrc).

Chain (per source s, time t, antenna a, channel ch):
  chi^2 = scale * sum w |O - M|^2 ,  M = G_p V G_q^H ,  V = sum_s c J_p J_q^H
  gM = -2 scale w (O - M)  (zero where flagged)
  gV = G_p^H gM G_q ,  gG_p += gM G_q V^H ,  gG_q += gM^H G_p V
  gJ_p += c gV J_q ,  gJ_q += c gV^H J_p ,  gc = Re <gV, J_p J_q^H>
  J = E (K sqrt(B)) :  gE = gJ (K sqrt(B))^H ,  g(K sqrt(B)) = E^H gJ
"""
import numpy as np

from . import rime_v4 as O


def _herm(X):
    x = X.reshape(X.shape[:-1] + (2, 2))
    return np.conj(np.swapaxes(x, -1, -2)).reshape(X.shape)


def _re_inner(X, Y):
    """Re sum_ij conj(X_ij) Y_ij over the trailing Jones axis."""
    return np.sum((np.conj(X) * Y).real, axis=-1)


def beam_with_grad(P, srcs=None, times=None):
    """E(s,t,a,ch,4) and its derivatives with respect to the source l and m.

    Same interpolation as rime_v4.e_beam; derivatives vanish where the grid
    coordinate was clipped to the cube edge."""
    lm = P['lm'][O._src(P, srcs)]
    pa = P['parallactic_angles'][O._src(P, times)]
    pe = P['point_errors'][O._src(P, times)]
    sc = P['antenna_scaling']
    E_beam = P['E_beam']
    nl, nm = E_beam.shape[:2]
    sint, cost = np.sin(pa), np.cos(pa)
    l0 = lm[:, 0][:, None, None]
    m0 = lm[:, 1][:, None, None]
    l = ((l0 * cost[None] - m0 * sint[None])[..., None] + pe[None, ..., 0]) * sc[None, None, :, :, 0]
    m = ((l0 * sint[None] + m0 * cost[None])[..., None] + pe[None, ..., 1]) * sc[None, None, :, :, 1]
    kl = (nl - 1) / (P['beam_ul'] - P['beam_ll'])
    km = (nm - 1) / (P['beam_um'] - P['beam_lm'])
    vl_raw = (nl - 1) * (l - P['beam_ll']) / (P['beam_ul'] - P['beam_ll'])
    vm_raw = (nm - 1) * (m - P['beam_lm']) / (P['beam_um'] - P['beam_lm'])
    in_l = (vl_raw > 0) & (vl_raw < nl - 1)
    in_m = (vm_raw > 0) & (vm_raw < nm - 1)
    vl = np.clip(vl_raw, 0.0, nl - 1)
    vm = np.clip(vm_raw, 0.0, nm - 1)
    gl0 = np.floor(vl)
    gl1 = np.minimum(gl0 + 1, nl - 1)
    ld = vl - gl0
    gm0 = np.floor(vm)
    gm1 = np.minimum(gm0 + 1, nm - 1)
    md = vm - gm0
    gc0, gc1, chd = O.beam_grid_channel(P)
    cd = chd[None, None, None, :]
    shape = vl.shape + (4,)
    S = np.zeros(shape, complex)
    A = np.zeros(shape)
    Sl = np.zeros(shape, complex)
    Al = np.zeros(shape)
    Sm = np.zeros(shape, complex)
    Am = np.zeros(shape)
    for hl in (0, 1):
        for hm in (0, 1):
            for hc in (0, 1):
                il = (gl1 if hl else gl0).astype(np.int64)
                im = (gm1 if hm else gm0).astype(np.int64)
                ic = (gc1 if hc else gc0)[None, None, None, :]
                fl = ld if hl else 1 - ld
                fm = md if hm else 1 - md
                fc = cd if hc else 1 - cd
                w = fl * fm * fc
                wl = (1 if hl else -1) * fm * fc
                wm = fl * (1 if hm else -1) * fc
                e = E_beam[il, im, ic]
                ab = np.abs(e)
                S += w[..., None] * e
                A += w[..., None] * ab
                Sl += wl[..., None] * e
                Al += wl[..., None] * ab
                Sm += wm[..., None] * e
                Am += wm[..., None] * ab
    r = np.abs(S)
    with np.errstate(divide='ignore', invalid='ignore'):
        inv = 1.0 / r
    ok = np.isfinite(inv)
    inv = np.where(ok, inv, 0.0)
    E = np.where(ok, S * A * inv, S * A)

    def dnorm(dS, dA):
        dr = (np.conj(S) * dS).real * inv
        with_norm = (dS * A + S * dA) * inv - S * A * dr * inv * inv
        return np.where(ok, with_norm, dS * A + S * dA)

    dE_ld = dnorm(Sl, Al)
    dE_md = dnorm(Sm, Am)
    # d(vl)/d(l0), d(vl)/d(m0), d(vm)/d(l0), d(vm)/d(m0)
    a_l = sc[None, None, :, :, 0]
    a_m = sc[None, None, :, :, 1]
    c = cost[None, :, :, None]
    s_ = sint[None, :, :, None]
    dvl_dl = np.where(in_l, kl * a_l * c, 0.0)
    dvl_dm = np.where(in_l, -kl * a_l * s_, 0.0)
    dvm_dl = np.where(in_m, km * a_m * s_, 0.0)
    dvm_dm = np.where(in_m, km * a_m * c, 0.0)
    dE_dl = dE_ld * dvl_dl[..., None] + dE_md * dvm_dl[..., None]
    dE_dm = dE_ld * dvl_dm[..., None] + dE_md * dvm_dm[..., None]
    return E, dE_dl, dE_dm


def brightness_sqrt_grads(P, gBs, srcs=None, times=None):
    """Chain g(sqrt B) (s,t,ch,4) to stokes (s,t,4) and alpha (s,t).

    sqrt(B) = sqrt(p) (B0 + s0 I) / sqrt(2 (I + s0)), p = (nu/nu_ref)^alpha,
    s0 = sqrt(I^2 - Q^2 - U^2 - V^2)."""
    S = P['stokes'][O._src(P, srcs)][:, O._src(P, times)]
    a = P['alpha'][O._src(P, srcs)][:, O._src(P, times)]
    I, Q, U, V = (S[..., k][..., None] for k in range(4))
    ratio = (P['frequency'] / P['ref_frequency'])[None, None, :]
    p = ratio ** a[..., None]
    Bs = O.brightness_sqrt(O.brightness(P, srcs, times))
    s0 = np.sqrt(np.maximum(I * I - Q * Q - U * U - V * V, 0.0))
    pt = p / np.sqrt(2 * p * (I + s0))
    GB = _re_inner(gBs, Bs)
    tr1 = gBs[..., 0].real + gBs[..., 3].real
    q2 = GB / (2 * s0 * (I + s0))
    gI = pt * (1 + I / s0) * tr1 - GB / (2 * s0)
    gQ = pt * ((gBs[..., 0].real - gBs[..., 3].real) - (Q / s0) * tr1) + q2 * Q
    gU = pt * ((gBs[..., 1].real + gBs[..., 2].real) - (U / s0) * tr1) + q2 * U
    gV = pt * ((gBs[..., 1].imag - gBs[..., 2].imag) - (V / s0) * tr1) + q2 * V
    g_stokes = np.stack([gI.sum(-1), gQ.sum(-1), gU.sum(-1), gV.sum(-1)], axis=-1)
    g_alpha = (GB * 0.5 * np.log(ratio)).sum(-1)
    return g_stokes, g_alpha


def shape_grads(P, s0, s1, times=None):
    """Shape factors c (n, t, bl, ch) and dc / d(3 params) (n, 3, t, bl, ch)
    for global sources [s0, s1) (zeros for point sources)."""
    npsrc, ngsrc = P['npsrc'], P['ngsrc']
    buvw = O.baseline_uvw(P, times)
    u = buvw[..., 0][None, :, :, None]
    v = buvw[..., 1][None, :, :, None]
    nt, nbl = buvw.shape[:2]
    nch = P['frequency'].shape[0]
    c = np.ones((s1 - s0, nt, nbl, nch))
    d = np.zeros((s1 - s0, 3, nt, nbl, nch))
    f = P['frequency'][None, None, None, :]
    for s in range(s0, s1):
        i = s - s0
        if s < npsrc:
            continue
        if s < npsrc + ngsrc:
            el, em, R = (P['gauss_shape'][k][s - npsrc] for k in range(3))
            k = P['gauss_scale'] * f
            a1 = u * em - v * el
            u1 = a1 * k * R
            v1 = (u * el + v * em) * k
            cc = np.exp(-(u1 ** 2 + v1 ** 2))
            c[i] = cc[0]
            d[i, 0] = (-2 * cc * (u1 * (-v * k * R) + v1 * (u * k)))[0]
            d[i, 1] = (-2 * cc * (u1 * (u * k * R) + v1 * (v * k)))[0]
            d[i, 2] = (-2 * cc * (u1 * a1 * k))[0]
        else:
            e1, e2, R = (P['sersic_shape'][k][s - npsrc - ngsrc] for k in range(3))
            k = P['two_pi_over_c'] * f
            den = 1 - e1 * e1 - e2 * e2
            Sc = R / den
            a1 = u * (1 + e1) + v * e2
            b1 = u * e2 + v * (1 - e1)
            u1, v1 = a1 * k * Sc, b1 * k * Sc
            dd = 1 + u1 ** 2 + v1 ** 2
            cc = 1 / (dd * np.sqrt(dd))
            dS1, dS2 = Sc * 2 * e1 / den, Sc * 2 * e2 / den
            k3 = -3 * cc / dd
            c[i] = cc[0]
            d[i, 0] = (k3 * (u1 * k * (u * Sc + a1 * dS1) + v1 * k * (-v * Sc + b1 * dS1)))[0]
            d[i, 1] = (k3 * (u1 * k * (v * Sc + a1 * dS2) + v1 * k * (u * Sc + b1 * dS2)))[0]
            d[i, 2] = (k3 * (u1 * a1 * k / den + v1 * b1 * k / den))[0]
    return c, d


def chi2_grad_prepare(P, src_chunk=16):
    """The per-visibility part of the gradient: chi^2, gV = d chi^2 / dV and
    d chi^2 / dG (a dict the per-source part reads)."""
    ntime = P['uvw'].shape[0]
    a1, a2 = P['antenna1'], P['antenna2']
    tt = np.arange(ntime)[:, None]
    V = O.ekb_vis(P, src_chunk=src_chunk)
    Gp = P['G_term'][tt, a1]
    Gq = P['G_term'][tt, a2]
    M = O.jones_mul_h(O.jones_mul(Gp, V), Gq)
    mask = P['flag'] > 0
    Ov = np.where(mask, 0.0, P['observed_vis'])
    M = np.where(mask, 0.0, M)
    R = Ov - M
    use_w = P.get('use_weight_vector', False)
    w = P['weight_vector'] if use_w else 1.0
    scale = 1.0 if use_w else 1.0 / P['sigma_sqrd']
    chi2 = scale * np.sum(w * (R.real ** 2 + R.imag ** 2))
    gM = np.where(mask, 0.0, -2.0 * scale * w * R)
    gV = O.jones_mul(O.jones_mul(_herm(Gp), gM), Gq)
    gG = np.zeros_like(P['G_term'])
    dGp = O.jones_mul(gM, O.jones_mul_h(Gq, V))
    dGq = O.jones_mul(_herm(gM), O.jones_mul(Gp, V))
    for t in range(ntime):
        np.add.at(gG[t], a1[t], dGp[t])
        np.add.at(gG[t], a2[t], dGq[t])
    return {'P': P, 'chi2': chi2, 'gV': gV, 'gG': gG}


def chi2_grad_sources(base, s0, s1):
    """Gradients of the source parameters of sources [s0, s1), from
    chi2_grad_prepare's gV: (g_lm, g_stokes, g_alpha, g_shape) for those
    sources, g_shape (3, s1 - s0) (zero for point sources)."""
    P, gV = base['P'], base['gV']
    ntime = P['uvw'].shape[0]
    a1, a2 = P['antenna1'], P['antenna2']
    tt = np.arange(ntime)[:, None]
    f = P['frequency']
    uvw = P['uvw']
    sl = slice(s0, s1)
    K = O.phase_scalar(P, sl)
    Bs = O.brightness_sqrt(O.brightness(P, sl))
    E, dE_dl, dE_dm = beam_with_grad(P, sl)
    KB = K[..., None] * Bs[:, :, None]
    J = O.jones_mul(E, KB)
    Jp, Jq = J[:, tt, a1], J[:, tt, a2]
    c, dc = shape_grads(P, s0, s1)
    gJ = np.zeros_like(J)
    cp = O.jones_mul(gV[None], Jq) * c[..., None]
    cq = O.jones_mul(_herm(gV)[None], Jp) * c[..., None]
    for t in range(ntime):
        np.add.at(gJ[:, t], (slice(None), a1[t]), cp[:, t])
        np.add.at(gJ[:, t], (slice(None), a2[t]), cq[:, t])
    gc = _re_inner(gV[None], O.jones_mul_h(Jp, Jq))
    g_shape = np.einsum('stbc,sktbc->ks', gc, dc)
    gE = O.jones_mul_h(gJ, KB)
    gKB = O.jones_mul(_herm(E), gJ)
    gK = np.sum(np.conj(Bs)[:, :, None] * gKB, axis=-1)
    gBs = (np.conj(K)[..., None] * gKB).sum(axis=2)
    l, m = P['lm'][sl, 0], P['lm'][sl, 1]
    nf = np.sqrt(1 - l ** 2 - m ** 2)
    dphase = -2j * np.pi * f / O.LIGHTSPEED
    dK = K * dphase[None, None, None, :]
    dphi_dl = uvw[None, :, :, 0] - uvw[None, :, :, 2] * (l / nf)[:, None, None]
    dphi_dm = uvw[None, :, :, 1] - uvw[None, :, :, 2] * (m / nf)[:, None, None]
    gphi = (np.conj(gK) * dK).real
    g_lm = np.stack([(gphi * dphi_dl[..., None]).sum(axis=(1, 2, 3)) + _re_inner(gE, dE_dl).sum(axis=(1, 2, 3)),
                     (gphi * dphi_dm[..., None]).sum(axis=(1, 2, 3)) + _re_inner(gE, dE_dm).sum(axis=(1, 2, 3))],
                    axis=-1)
    g_stokes, g_alpha = brightness_sqrt_grads(P, gBs, sl)
    return s0, s1, g_lm, g_stokes, g_alpha, g_shape


def chi2_grad_combine(base, parts):
    """(chi^2, dict of gradients) from chi2_grad_prepare and the
    chi2_grad_sources results of batches covering every source once."""
    P = base['P']
    npsrc, ngsrc = P['npsrc'], P['ngsrc']
    g_lm = np.zeros_like(P['lm'])
    g_stokes = np.zeros_like(P['stokes'])
    g_alpha = np.zeros_like(P['alpha'])
    g_gauss = np.zeros_like(P['gauss_shape'])
    g_sersic = np.zeros_like(P['sersic_shape'])
    for s0, s1, gl, gs, ga, gsh in parts:
        g_lm[s0:s1] += gl
        g_stokes[s0:s1] += gs
        g_alpha[s0:s1] += ga
        for s in range(s0, s1):
            if npsrc <= s < npsrc + ngsrc:
                g_gauss[:, s - npsrc] += gsh[:, s - s0]
            elif s >= npsrc + ngsrc:
                g_sersic[:, s - npsrc - ngsrc] += gsh[:, s - s0]
    return base['chi2'], {'lm': g_lm, 'stokes': g_stokes, 'alpha': g_alpha, 'gauss_shape': g_gauss,
                          'sersic_shape': g_sersic, 'G_term': base['gG']}


def chi2_grad(P, src_chunk=16):
    """Return (chi^2, dict of gradients) in FP64."""
    base = chi2_grad_prepare(P, src_chunk)
    nsrc = P['lm'].shape[0]
    parts = [chi2_grad_sources(base, s0, min(nsrc, s0 + src_chunk)) for s0 in range(0, nsrc, src_chunk)]
    return chi2_grad_combine(base, parts)

"""Batched likelihood over many parameter sets sharing one observation
(mb_rime_batch): per-set results equal single-problem calls and the FP64
oracle, a batch is a fixed number of launches whatever its size, graph
replay equals eager execution, the autotuner picks a valid form per set."""
import numpy as np
import pytest

from montblanc_gb300 import synth

pytestmark = pytest.mark.gpu


def _observation():
    P = synth.make_problem(ntime=4, na=7, nchan=3, npsrc=2, ngsrc=1, nssrc=1, seed=3, use_weight_vector=True,
                           random_weights=True, flag_fraction=0.05, beam_shape=(9, 8, 5))
    rng = np.random.default_rng(4)
    P['observed_vis'] = rng.normal(0, 1, P['observed_vis'].shape) + 1j * rng.normal(0, 1, P['observed_vis'].shape)
    return P


def _single(P, s, dtype, form):
    from montblanc_gb300.rime import RimeProblem
    Q = dict(P)
    for k in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'npsrc', 'ngsrc', 'nssrc'):
        Q[k] = s[k]
    prob = RimeProblem.from_numpy(Q, dtype=dtype)
    x2, g = prob.chi2_and_grad(mode=form)
    return x2.item(), {k: v.cpu().numpy() for k, v in g.items()}


@pytest.mark.parametrize('dtype,form', [('double', 'native'), ('float', 'native'), ('float', 'split_tf32')])
def test_batch_matches_single_problems(dtype, form):
    from montblanc_gb300.batch import RimeBatch, make_sets
    P = _observation()
    sets = make_sets(P, 5, seed=1, lo=3, hi=40)
    b = RimeBatch(P, sets, dtype=dtype, want_G_grad=True)
    b.forms = [form] * b.nsets
    x2 = b.run().cpu().numpy()
    tol = 1e-12 if dtype == 'double' else 1e-5
    for i, s in enumerate(sets):
        ref_x2, ref_g = _single(P, s, dtype, form)
        assert abs(x2[i] - ref_x2) <= tol * abs(ref_x2)
        g = b.set_grads(i)
        for k in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'G_term'):
            assert g[k].shape == ref_g[k].shape, (i, k)
            if ref_g[k].size == 0:
                continue
            scale = max(np.abs(ref_g[k]).max(), 1e-30)
            assert np.abs(g[k] - ref_g[k]).max() <= tol * scale, (i, k)


def test_graph_replay_and_autotune():
    import torch
    from montblanc_gb300.batch import CANDIDATES, FORMS, RimeBatch, make_sets
    P = _observation()
    sets = make_sets(P, 6, seed=2, lo=3, hi=60)
    b = RimeBatch(P, sets, dtype='float')
    forms = b.autotune()
    assert len(forms) == 6 and all(f in FORMS for f in forms)
    assert all(c in CANDIDATES for c in zip(b.forms, b.tiles))
    assert all(len(v) == len(CANDIDATES) for v in b.tune_times.values())
    eager = b.run().clone()
    g_eager = {k: v.clone() for k, v in b.grads.items()}
    b.capture()
    b.X2.zero_()
    for v in b.grads.values():
        v.zero_()
    for _ in range(2):
        replay = b.run()
    torch.cuda.synchronize()
    assert torch.equal(replay, eager)
    for k in g_eager:
        assert torch.allclose(b.grads[k], g_eager[k], rtol=1e-5, atol=1e-6 * float(g_eager[k].abs().max() + 1e-30))


@pytest.mark.parametrize('dtype,form,tile', [('float', 'native', 8), ('float', 'native', 32),
                                             ('double', 'native', 32), ('float', 'split_tf32', 8)])
def test_source_tiles_leave_results_unchanged(dtype, form, tile):
    """The source tile of the CUDA-core kernels only changes the order of
    summation."""
    from montblanc_gb300.batch import RimeBatch, make_sets
    P = _observation()
    sets = make_sets(P, 3, seed=5, lo=20, hi=70)
    a = RimeBatch(P, sets, dtype=dtype)
    b = RimeBatch(P, sets, dtype=dtype)
    a.forms = b.forms = [form] * 3
    b.tiles = [tile] * 3
    xa, xb = a.run().cpu().numpy(), b.run().cpu().numpy()
    tol = 1e-12 if dtype == 'double' else 2e-6
    assert np.all(np.abs(xa - xb) <= tol * np.abs(xa))
    for i in range(3):
        ga, gb = a.set_grads(i), b.set_grads(i)
        for k in ('lm', 'stokes', 'gauss_shape', 'sersic_shape'):
            if ga[k].size:
                assert np.abs(ga[k] - gb[k]).max() <= 10 * tol * max(np.abs(ga[k]).max(), 1e-30), (i, k)


def _with_set(P, s):
    Q = dict(P)
    for k in ('lm', 'stokes', 'alpha', 'gauss_shape', 'sersic_shape', 'npsrc', 'ngsrc', 'nssrc'):
        Q[k] = s[k]
    return Q


def _empty_set(P, npsrc=0, ngsrc=0, nssrc=0, seed=0):
    """A set with the given counts, parameters drawn like make_sets does."""
    from montblanc_gb300.batch import make_sets
    s = make_sets(P, 1, seed=seed, lo=40, hi=41)[0]
    n = npsrc + ngsrc + nssrc
    out = {'npsrc': npsrc, 'ngsrc': ngsrc, 'nssrc': nssrc,
           'lm': s['lm'][:n], 'stokes': s['stokes'][:n], 'alpha': s['alpha'][:n],
           'gauss_shape': s['gauss_shape'][:, :ngsrc], 'sersic_shape': s['sersic_shape'][:, :nssrc]}
    return out


#: chi^2 (relative) and gradient (norm-wise relative, worst parameter) bounds
#: against the FP64 oracle.
ORACLE_TOL = {'double': (1e-10, 1e-9), 'float': (1e-5, 1e-3)}


@pytest.mark.parametrize('dtype', ['double', 'float'])
def test_batch_sets_match_oracle(dtype):
    """Sets of one batch against the FP64 oracle (chi^2 and every gradient):
    three generated sets, a set without sources and one with extended sources
    only; in FP32 the sets mix the CUDA-core and TF32 split forms and source
    tiles, so the batch runs several forward and adjoint launches."""
    from montblanc_gb300.batch import RimeBatch, make_sets
    from oracle import adjoint as OA
    from oracle import rime_v4 as O
    P = _observation()
    sets = make_sets(P, 3, seed=11, lo=8, hi=30) + [_empty_set(P), _empty_set(P, ngsrc=3, nssrc=2, seed=2)]
    b = RimeBatch(P, sets, dtype=dtype, want_G_grad=True)
    if dtype == 'float':
        b.forms = ['native', 'split_tf32', 'split_tf32', 'split_tf32', 'split_tf32']
        b.tiles = [16, 0, 8, 0, 32]
    x2 = b.run().cpu().numpy()
    tx2, tg = ORACLE_TOL[dtype]
    for i, s in enumerate(sets):
        Q = _with_set(P, s)
        if s['npsrc'] + s['ngsrc'] + s['nssrc'] == 0:
            ref_x2 = O.chi_sqrd(Q, O.chi_sqrd_terms(Q, np.zeros_like(P['observed_vis'])))
            assert abs(x2[i] - ref_x2) <= tx2 * abs(ref_x2), (i, x2[i], ref_x2)
            assert not np.any(b.set_grads(i)['G_term'] != b.set_grads(i)['G_term'])  # finite
            continue
        ref_x2, ref_g = OA.chi2_grad(Q)
        assert abs(x2[i] - ref_x2) <= tx2 * abs(ref_x2), (i, x2[i], ref_x2)
        g = b.set_grads(i)
        for k, r in ref_g.items():
            if r.size == 0:
                continue
            err = np.linalg.norm(g[k] - r) / np.linalg.norm(r)
            assert err <= tg, (i, k, err)


def test_batch_launches_do_not_grow_with_sets():
    """A batch is a fixed set of launches (shared tables, one forward and one
    adjoint launch per kernel form, the chi^2 sums, the gradients): 2 and 8
    sets of the same forms launch the same kernels."""
    import torch
    from montblanc_gb300 import _cabi
    from montblanc_gb300.batch import RimeBatch, make_sets
    P = _observation()
    counts = []
    for n in (2, 8):
        sets = make_sets(P, n, seed=3, lo=30, hi=60)
        b = RimeBatch(P, sets, dtype='float')
        b.forms = ['split_tf32'] * n
        b.prepare()
        torch.cuda.synchronize()
        l0 = _cabi.lib.mb_kernel_launches()
        b.run()
        torch.cuda.synchronize()
        counts.append(_cabi.lib.mb_kernel_launches() - l0)
    # beam plane, path lengths, sqrt(B) table, extended sources' forward,
    # tensor-core forward, chi^2 sums, point- and extended-source adjoints,
    # gradients
    assert counts == [9, 9], counts

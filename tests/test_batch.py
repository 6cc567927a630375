"""Batched likelihood over many parameter sets sharing one observation:
per-set results equal single-problem calls, graph replay equals eager
execution, the autotuner picks a valid form per set."""
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

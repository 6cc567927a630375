"""HostFeed: chi^2 and gradients of input sets held in host memory, with the
copies overlapped with the kernels, equal the same sets run one at a time
through RimeProblem."""
import numpy as np
import pytest

from montblanc_gb300 import synth


class _FakeProblem(object):
    arrays = {'observed_vis': object(), 'weight_vector': None}


def test_hostfeed_rejects_unknown_and_absent_arrays():
    from montblanc_gb300.rime import HostFeed
    with pytest.raises(ValueError):
        HostFeed(_FakeProblem(), ['not_an_array'])
    with pytest.raises(ValueError):
        HostFeed(_FakeProblem(), ['weight_vector'])   # absent: weights not applied
    with pytest.raises(ValueError):
        HostFeed(_FakeProblem(), ['observed_vis'], depth=0)


def _sets(P, n, rng):
    out = []
    for _ in range(n):
        s = {'observed_vis': P['observed_vis'] + 0.3 * (rng.normal(size=P['observed_vis'].shape)
                                                        + 1j * rng.normal(size=P['observed_vis'].shape)),
             'lm': P['lm'] + rng.normal(0, 1e-4, P['lm'].shape),
             'stokes': P['stokes'] * rng.uniform(0.8, 1.2, P['stokes'].shape),
             'flag': (rng.uniform(size=P['observed_vis'].shape) < 0.05).astype(np.uint8)}
        out.append(s)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize('dtype,mode,depth', [('double', 'native', 2), ('float', 'split_tf32', 2),
                                              ('float', 'native', 1)])
def test_hostfeed_matches_sequential_calls(dtype, mode, depth):
    import torch
    from montblanc_gb300.rime import HostFeed, RimeProblem
    P = synth.make_problem(ntime=3, na=9, nchan=4, npsrc=6, ngsrc=2, nssrc=1, seed=11, beam_shape=(9, 8, 5))
    rng = np.random.default_rng(12)
    sets = _sets(P, 4, rng)
    prob = RimeProblem.from_numpy(P, dtype=dtype)
    names = ['observed_vis', 'lm', 'stokes', 'flag']
    host = []
    for s in sets:
        h = {}
        for n in names:
            ref = prob.arrays[n]
            h[n] = torch.as_tensor(np.ascontiguousarray(s[n])).to(ref.dtype).pin_memory()
        host.append(h)
    feed = HostFeed(prob, names, mode=mode, depth=depth)
    outs = []
    done = []
    for h in host:
        g = {n: torch.empty(t.shape, dtype=t.dtype).pin_memory() for n, t in prob.empty_grads().items()}
        x2 = torch.empty(1, dtype=torch.float64).pin_memory()
        done.append(feed.submit(h, x2, g))
        outs.append((x2, g))
    for ev in done:
        ev.synchronize()
    tol = 1e-12 if dtype == 'double' else 1e-6
    for h, (x2, g) in zip(host, outs):
        for n in names:
            prob.arrays[n].copy_(h[n])
        rx2, rg = prob.chi2_and_grad(mode=mode)
        torch.cuda.synchronize()
        assert abs(x2.item() - rx2.item()) <= tol * abs(rx2.item())
        for n in rg:
            a, b = g[n].numpy(), rg[n].cpu().numpy()
            if b.size:
                assert np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300), n

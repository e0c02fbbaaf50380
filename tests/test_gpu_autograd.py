"""The torch.autograd binding of the pair adjoint (gain_autograd.line_strengths over
gain_adjoint_pair_prec): torch.autograd.gradcheck (central differences of every entry) on a
small pair, and a log-ratio loss L = sum w (log S - log S_t)^2 of the kind dipole-surface
refinement minimises, against central differences (h = 1e-6) on sampled entries and against
the exact directional derivative (S is quadratic in mu, so amp(d) is the forward pass of the
dipole d), in FP64 and FP32 adjoint arithmetic."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def _setup(rule="c4", nv=12):
    import gainls
    import synth
    p = synth.make_problem(nv, [2, 3], rule, blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    return p, eng, lo, up


@pytest.mark.parametrize("rule", ["c4", "c4r"])
def test_gradcheck_weighted_sum(built_lib, rule):
    import torch
    import gain_autograd
    p, eng, lo, up = _setup(rule, nv=8)
    w = torch.from_numpy(np.random.default_rng(5).standard_normal((len(lo), len(up))))
    mu = torch.tensor(p.dipole, dtype=torch.float64, requires_grad=True)

    def f(m):
        return (w * gain_autograd.line_strengths(m, eng, (0, 0, 1, 1), lo, up)).sum()

    assert torch.autograd.gradcheck(f, (mu,), eps=1e-6, atol=1e-7, rtol=1e-6, check_undefined_grad=False,
                                    nondet_tol=1e-10)   # the adjoint sums with atomic adds
    eng.close()


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("f32", 2e-5)])
def test_log_ratio_loss(built_lib, precision, tol):
    import torch
    import gain_autograd
    p, eng, lo, up = _setup()
    rng = np.random.default_rng(77)
    pair = (0, 0, 1, 1)
    mu0 = torch.tensor(p.dipole, dtype=torch.float64)
    mu_t = mu0 * (1.0 + 0.01 * torch.from_numpy(rng.standard_normal(p.dipole.shape)))
    with torch.no_grad():
        S_t = gain_autograd.line_strengths(mu_t, eng, pair, lo, up)
    S0 = gain_autograd.line_strengths(mu0, eng, pair, lo, up).detach()
    mask = (S0 > 1e-10 * S0.max()) & (S_t > 1e-10 * S_t.max())

    def loss_of(m):
        S = gain_autograd.line_strengths(m, eng, pair, lo, up, precision=precision)
        return ((torch.log(S[mask]) - torch.log(S_t[mask])) ** 2).sum()

    mu = mu0.clone().requires_grad_(True)
    L = loss_of(mu)
    L.backward()
    g = mu.grad.numpy().reshape(-1)
    gmax = np.abs(g).max()
    assert gmax > 0
    # exact directional derivative: dL = sum 2 r / S * 2 amp amp(d), amp(d) = the pair's
    # amplitudes with the dipole d (amp is linear in mu)
    import gainls
    eng.upload_dipole(p.dipole.reshape(-1), p.dipole.shape[-1], 0, p.dipole.shape[-1], p.dipole.shape[-1])
    eng.run_pair(*pair, lo, up, gainls.PATH_PLAIN_FP64)
    amp = eng.fetch_amp().copy()
    S = amp ** 2
    r = np.zeros_like(S)
    r[mask.numpy()] = (np.log(S) - np.log(S_t.numpy()))[mask.numpy()]
    for _ in range(3):
        d = rng.standard_normal(p.dipole.shape)
        eng.upload_dipole(np.ascontiguousarray(d).reshape(-1), d.shape[-1], 0, d.shape[-1], d.shape[-1])
        eng.run_pair(*pair, lo, up, gainls.PATH_PLAIN_FP64)
        ad = eng.fetch_amp()
        exact = float(np.sum(2.0 * r / np.where(S > 0, S, 1.0) * 2.0 * amp * ad))
        terms = float(np.sum(np.abs(2.0 * r / np.where(S > 0, S, 1.0) * 2.0 * amp * ad)))
        assert abs(float(np.dot(g, d.reshape(-1))) - exact) <= tol * terms
    # central differences (h = 1e-6) on sampled entries with a non-negligible gradient
    if precision == "f64":
        idx = rng.choice(np.flatnonzero(np.abs(g) > 1e-3 * gmax), size=12, replace=False)
        h = 1e-6
        for k in idx:
            e = torch.zeros(mu0.numel(), dtype=torch.float64)
            e[k] = h
            e = e.view_as(mu0)
            with torch.no_grad():
                fd = (loss_of(mu0 + e) - loss_of(mu0 - e)).item() / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 * gmax + 1e-5 * abs(g[k]), (k, fd, g[k])
    eng.close()

"""The hand-written adjoint of the fixed-set coefficient estimate (config 4).

With the identified frequencies held fixed, Iterate's coefficient estimate
(src/iterate.cc:146-171) is a linear map c = A x (``mpsft_estimate``);
``mpsft_adjoint`` applies A^H. Checked here:

  * the estimate against the same formula on the oracle's FP64 bins (1e-10);
  * the adjoint identity <A x, g> = <x, A^H g> (1e-12 relative);
  * dL/dx of L = ||c - c_target||^2 through a torch.autograd.Function
    (forward = estimate, backward = adjoint) against central finite
    differences, h = 1e-3 in FP64, on 64 sample indices (1e-7 relative);
  * against the dense-DFT-row gradient: for identified modes in distinct bins
    inside the window's passband, n D_S (A^H g) = g up to window leakage
    (D_S = the DFT rows of the set, 1e-4 relative).
"""
from __future__ import annotations

import numpy as np
import pytest

import mpsft_gb300 as m

pytestmark = pytest.mark.gpu


def _tone_signal(n, k, coef, sigma, rng):
    j = np.arange(n)
    x = np.zeros(n, np.complex128)
    for kk, cc in zip(k, coef):
        x += cc * np.exp(2j * np.pi * ((kk * j) % n) / n)
    x += sigma * (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    return x


def _setup(ctx, n, bins, delta, trials, seed):
    rng = np.random.default_rng(seed)
    a = int(rng.integers(1, n)) | 1
    b, c = int(rng.integers(0, n)), int(rng.integers(0, n))
    q = [int(v) for v in rng.integers(0, n, trials)]
    bits = m.num_bits(n, bins)
    return ctx.estimate_setup(bins, bits, delta, a, b, c, q)


def _reference_estimate(port, x, su, k0):
    """The estimate formula on the oracle's FP64 bins of every trial."""
    n, B, L = x.size, su.bins, su.bits
    T = su.trials
    U = [port.bin_in_time(x, B, L, su.window_delta, su.a, su.b, su.c, su.q[t])
         for t in range(T)]
    out = []
    for kk in k0:
        k1 = (su.a * int(kk) + su.b) % n
        beta = (k1 * B) // n
        xi0 = k1 / n - (beta + 0.5) / B
        wf = port.sample_in_freq(n, B, su.window_delta, xi0)
        acc = 0j
        for t in range(T):
            for r in range(1 + 2 * L):
                off = 0 if r == 0 else ((B << ((r - 1) // 2)) * (1 if r % 2 else -1))
                tau = su.q[t] + off
                acc += U[t][r, beta] * np.exp(-2j * np.pi * ((tau * k1) % n) / n)
        ph = np.exp(-2j * np.pi * ((su.c * int(kk)) % n) / n)
        out.append(acc * ph / (wf * T * (1 + 2 * L)))
    return np.array(out)


def test_estimate_matches_oracle(ctx, port):
    n, rng = 1 << 14, np.random.default_rng(3)
    k = rng.choice(n, 20, replace=False)
    x = _tone_signal(n, k, np.exp(2j * np.pi * rng.random(20)), 1e-3, rng)
    su = _setup(ctx, n, 101, 1e-6, 3, 5)
    sig = ctx.upload(x)
    got = ctx.estimate(sig, su, k)
    want = _reference_estimate(port, x, su, k)
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()


def test_estimate_complex64_config4(ctx, port):
    """Config 4's input type: the estimate of a complex64 signal (FP64
    arithmetic on the exactly widened samples) equals that of the same
    samples in complex128 bit for bit, and the oracle's to FP64 rounding."""
    n, S = 1 << 20, 200
    rng = np.random.default_rng(11)
    k = rng.choice(n, S, replace=False)
    x64 = _tone_signal(n, k, np.exp(2j * np.pi * rng.random(S)), 1e-6,
                       rng).astype(np.complex64)
    su = _setup(ctx, n, 2 * S + 1, 1e-5, 3, 21)
    s64 = ctx.upload(x64)
    s128 = ctx.upload(x64.astype(np.complex128))
    got = ctx.estimate(s64, su, k)
    assert np.array_equal(got, ctx.estimate(s128, su, k))
    want = _reference_estimate(port, x64.astype(np.complex128), su, k)
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()
    s64.free()
    s128.free()


@pytest.mark.parametrize("n", [1 << 16, 65537])
def test_adjoint_identity(ctx, n):
    rng = np.random.default_rng(7)
    su = _setup(ctx, n, 401, 1e-5, 3, 11)
    k0 = rng.choice(n, 60, replace=False).astype(np.int32)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = rng.standard_normal(60) + 1j * rng.standard_normal(60)
    ax = ctx.estimate(ctx.upload(x), su, k0)
    ahg = ctx.adjoint(n, su, k0, g)
    lhs = np.vdot(g, ax)          # <A x, g> = g^H A x
    rhs = np.vdot(ahg, x)         # <x, A^H g> = (A^H g)^H x
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(g) * np.linalg.norm(ax) * 10
    assert np.count_nonzero(ahg) > 0


class _Estimate:
    """torch.autograd.Function: forward = mpsft_estimate, backward = mpsft_adjoint."""

    @staticmethod
    def make(ctx, su, k0, n):
        import torch

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(fctx, x):
                sig = ctx.upload(x.detach().cpu().numpy().astype(np.complex128))
                c = ctx.estimate(sig, su, k0)
                sig.free()
                return torch.from_numpy(c)

            @staticmethod
            def backward(fctx, grad_c):
                g = grad_c.detach().cpu().numpy().astype(np.complex128)
                return torch.from_numpy(ctx.adjoint(n, su, k0, g))

        return Fn


def test_gradient_finite_differences(ctx):
    import torch

    # config 4: N = 2^20, S = 200 unit modes, loss ||c - c_target||^2
    n, S = 1 << 20, 200
    rng = np.random.default_rng(4)
    k = rng.choice(n, S, replace=False).astype(np.int32)
    x = _tone_signal(n, k, np.exp(2j * np.pi * rng.random(S)), 1e-6, rng)
    c_target = (rng.standard_normal(S) + 1j * rng.standard_normal(S)) / np.sqrt(2)
    su = _setup(ctx, n, 2 * S + 1, 1e-5, 3, 21)
    fn = _Estimate.make(ctx, su, k, n)
    xt = torch.from_numpy(x.copy()).requires_grad_(True)
    loss = (fn.apply(xt) - torch.from_numpy(c_target)).abs().pow(2).sum()
    loss.backward()
    grad = xt.grad.numpy()
    sig = ctx.upload(x)

    def L(xv):
        sig.write(xv)
        return float(np.sum(np.abs(ctx.estimate(sig, su, k) - c_target) ** 2))

    support = np.flatnonzero(grad)
    idx = np.concatenate([rng.choice(support, 48, replace=False),
                          rng.choice(n, 16, replace=False)])
    h = 1e-3
    fd = []
    for j in idx:
        e = np.zeros(n, np.complex128)
        e[j] = h
        d_re = (L(x + e) - L(x - e)) / (2 * h)
        d_im = (L(x + 1j * e) - L(x - 1j * e)) / (2 * h)
        fd.append(d_re + 1j * d_im)
    fd = np.array(fd)
    err = np.abs(fd - grad[idx]).max() / np.abs(grad[idx]).max()
    print(f"max |FD - adjoint| / max |grad| = {err:.2e}")
    assert err < 1e-7


def test_gradient_matches_dense_dft_rows(ctx):
    n, S = 1 << 20, 200
    rng = np.random.default_rng(8)
    k = rng.choice(n, S, replace=False).astype(np.int64)
    B = 8 * S + 1
    su = _setup(ctx, n, B, 1e-5, 3, 31)
    # the modes an iteration would identify: alone in their bin and inside the
    # window's passband (|xi0| < B / 4 of a bin)
    k1 = (su.a * k + su.b) % n
    beta = (k1 * B) // n
    xi0 = k1 / n - (beta + 0.5) / B
    _, cnt = np.unique(beta, return_counts=True)
    alone = np.isin(beta, np.unique(beta)[cnt == 1])
    keep = alone & (np.abs(xi0) < 0.2 / B)
    ks = k[keep].astype(np.int32)
    assert ks.size >= 20
    g = rng.standard_normal(ks.size) + 1j * rng.standard_normal(ks.size)
    ahg = ctx.adjoint(n, su, ks, g)
    # n D_S (A^H g), D_S = rows (1/n) e^{-2 pi i j k / n}
    j = np.arange(n)
    proj = np.array([np.sum(ahg * np.exp(-2j * np.pi * ((j * kk) % n) / n))
                     for kk in ks])
    err = np.linalg.norm(proj - g) / np.linalg.norm(g)
    print(f"||n D_S A^H g - g|| / ||g|| = {err:.2e} over {ks.size} modes")
    assert err < 1e-4

"""The MLP oracle's backward pass against finite differences (CPU)."""
import numpy as np


def test_oracle_gradient_finite_differences():
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.2, M.NPAR).astype(np.float32)
    w = M.bf16(w).astype(np.float32)  # on the BF16 grid: rounding is then the identity
    x = rng.normal(0, 1, (64, 4))
    t = rng.normal(0, 0.3, 64)
    loss, g = M.loss_and_grad(w, x, t)
    # perturb weights that stay on the bf16 grid: compare directional derivatives
    # with a smooth surrogate (no rounding) instead
    def f(wf):
        W1, b1, W2, b2, W3, b3, W4, b4 = (wf[M.OW1:M.OB1].reshape(64, 4), wf[M.OB1:M.OW2],
                                          wf[M.OW2:M.OB2].reshape(64, 64), wf[M.OB2:M.OW3],
                                          wf[M.OW3:M.OB3].reshape(64, 64), wf[M.OB3:M.OW4],
                                          wf[M.OW4:M.OB4].reshape(1, 64), wf[M.OB4:])
        a = M.silu(x @ W1.T + b1); a = M.silu(a @ W2.T + b2); a = M.silu(a @ W3.T + b3)
        return np.mean(((a @ W4.T + b4)[:, 0] - t) ** 2)
    wd = w.astype(np.float64)
    assert abs(f(wd) - loss) < 1e-12
    for _ in range(5):
        dvec = rng.normal(0, 1, M.NPAR)
        eps = 1e-6
        fd = (f(wd + eps * dvec) - f(wd - eps * dvec)) / (2 * eps)
        assert abs(fd - g @ dvec) <= 1e-6 * max(1.0, abs(fd))

"""CPU oracle of the cooling-surrogate MLP (test infrastructure only).

Float64 NumPy forward and backward of the 4 -> 64 -> 64 -> 64 -> 1 SiLU
network with the weights rounded to BF16, as the GPU kernels use them, and
optionally the BF16 roundings of the tensor-core training pass; used to
check the GPU gradients and inference.
"""
from __future__ import annotations

import numpy as np

H, NIN = 64, 4
OW1 = 0
OB1 = OW1 + H * NIN
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + H * H
OW4 = OB3 + H
OB4 = OW4 + H
NPAR = OB4 + 1


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even)."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = bf16(w)
    return (w[OW1:OB1].reshape(H, NIN), w[OB1:OW2], w[OW2:OB2].reshape(H, H), w[OB2:OW3],
            w[OW3:OB3].reshape(H, H), w[OB3:OW4], w[OW4:OB4].reshape(1, H), w[OB4:NPAR])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_and_grad(w, x, t, bf16_operands=False):
    """Loss and gradient of one batch. bf16_operands restates the
    tensor-core training pass (torch_gb300/csrc/mlp.cu, k_mlp_train_tc):
    the inputs, the activations and the gradient operands of the MMAs (dy for
    layer 4, dz for layers 1-3) rounded to BF16, every product accumulated
    exactly; without it, the exact network with BF16 weights."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(w)
    q = bf16 if bf16_operands else (lambda a: np.asarray(a, np.float64))
    x = q(x)
    t = np.asarray(t, np.float64)
    z1 = x @ W1.T + b1; a1 = q(silu(z1))
    z2 = a1 @ W2.T + b2; a2 = q(silu(z2))
    z3 = a2 @ W3.T + b3; a3 = q(silu(z3))
    y = (a3 @ W4.T + b4)[:, 0]
    n = x.shape[0]
    r = y - t
    loss = np.mean(r * r)
    dy = (2.0 * r / n)[:, None]
    g = np.zeros(NPAR)
    dyq = q(dy)
    g[OW4:OB4] = (dyq.T @ a3).ravel(); g[OB4] = dyq.sum()
    d3 = q((dy @ W4) * dsilu(z3))
    g[OW3:OB3] = (d3.T @ a2).ravel(); g[OB3:OW4] = d3.sum(0)
    d2 = q((d3 @ W3) * dsilu(z2))
    g[OW2:OB2] = (d2.T @ a1).ravel(); g[OB2:OW3] = d2.sum(0)
    d1 = q((d2 @ W2) * dsilu(z1))
    g[OW1:OB1] = (d1.T @ x).ravel(); g[OB1:OW2] = d1.sum(0)
    return loss, g


def forward(w, x):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(w)
    a = silu(np.asarray(x, np.float64) @ W1.T + b1)
    a = silu(a @ W2.T + b2)
    a = silu(a @ W3.T + b3)
    return (a @ W4.T + b4)[:, 0]

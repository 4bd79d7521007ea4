"""Test infrastructure: numpy (FP64) restatement of the learned initial guess /
preconditioner model, used only to check the GPU training kernels' loss and
gradients.  The model itself has no counterpart in the reference.

Model:   X (B x 64 site descriptors) -> Y = W3 gelu(W2 gelu(W1 X + b1) + b2) + b3
         (B x 4), GELU(x) = x/2 (1 + erf(x / sqrt 2)).
Guess:   mu0_i = Y_i0 v1_i + Y_i1 v2_i + Y_i2 v3_i  (equivariant basis vectors)
Precond: z_i = a_i + Y_i3 w_i                      (a = alpha r, w = alpha T_near alpha r)
Loss:    (1/B) sum_i |mu0_i - mu*_i|^2 / s_i + lam (1/B) sum_i |a_i + Y_i3 w_i - e_i|^2 / t_i

A target row holds v1 v2 v3 mu* a w e (7 x 3 values), s, t and one pad value.
"""
import numpy as np
from scipy.special import erf

SQRT2 = np.sqrt(2.0)
INV_SQRT_2PI = 1.0 / np.sqrt(2.0 * np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / SQRT2))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / SQRT2)) + x * np.exp(-0.5 * x * x) * INV_SQRT_2PI


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = params
    Z1 = X @ W1.T + b1
    H1 = gelu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = gelu(Z2)
    Y = H2 @ W3.T + b3
    return Y, (X, Z1, H1, Z2, H2)


def loss_and_grads(params, X, T, lam=1.0):
    W1, b1, W2, b2, W3, b3 = params
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    B = X.shape[0]
    Y, (X, Z1, H1, Z2, H2) = forward([np.asarray(p, np.float64) for p in params], X)
    v1, v2, v3, mu, a, w, e = (T[:, 3 * k:3 * k + 3] for k in range(7))
    s, t = T[:, 21], T[:, 22]
    mu0 = Y[:, 0:1] * v1 + Y[:, 1:2] * v2 + Y[:, 2:3] * v3
    dg = mu0 - mu
    dp = a + Y[:, 3:4] * w - e
    L = (np.sum(dg * dg, axis=1) / s).sum() / B + lam * (np.sum(dp * dp, axis=1) / t).sum() / B
    dY = np.zeros_like(Y)
    for k, v in enumerate((v1, v2, v3)):
        dY[:, k] = 2.0 * np.sum(dg * v, axis=1) / s / B
    dY[:, 3] = 2.0 * lam * np.sum(dp * w, axis=1) / t / B
    dW3 = dY.T @ H2
    db3 = dY.sum(0)
    dZ2 = (dY @ np.asarray(W3, np.float64)) * gelu_grad(Z2)
    dW2 = dZ2.T @ H1
    db2 = dZ2.sum(0)
    dZ1 = (dZ2 @ np.asarray(W2, np.float64)) * gelu_grad(Z1)
    dW1 = dZ1.T @ X
    db1 = dZ1.sum(0)
    return L, [dW1, db1, dW2, db2, dW3, db3]

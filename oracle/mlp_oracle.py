"""Float64 restatement of the bin-capacity model (TEST INFRASTRUCTURE ONLY).

Checks the GPU forward and backward kernels of
custom-gpgpu-rasterizer_gb300/csrc/gbr_predict.cu: the same 12-64-64-1 MLP
(ReLU, softplus output), parameters stored as BF16 and evaluated here in
float64, loss (log1p(l) - log1p(count))^2 summed over samples.  Parameter
layout (csrc/gbr_predict.h): W1[12][64], b1[64], W2[64][64], b2[64],
W3[64], b3.
"""
import numpy as np

F, H = 12, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + F * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NUM_PARAMS = OFF_B3 + 1


def bf16_to_f64(w_u16: np.ndarray) -> np.ndarray:
    return (w_u16.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def f32_to_bf16(w: np.ndarray) -> np.ndarray:
    """Round to nearest even, as __float2bfloat16_rn."""
    u = np.asarray(w, np.float32).view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return rounded.astype(np.uint16)


def unpack(w):
    W1 = w[OFF_W1:OFF_B1].reshape(F, H)
    b1 = w[OFF_B1:OFF_W2]
    W2 = w[OFF_W2:OFF_B2].reshape(H, H)
    b2 = w[OFF_B2:OFF_W3]
    W3 = w[OFF_W3:OFF_B3]
    b3 = w[OFF_B3]
    return W1, b1, W2, b2, W3, b3


def softplus(y):
    return np.where(y > 20, y, np.log1p(np.exp(np.minimum(y, 20))))


def predict(w_u16, X):
    W1, b1, W2, b2, W3, b3 = unpack(bf16_to_f64(w_u16))
    h1 = np.maximum(X @ W1 + b1, 0)
    h2 = np.maximum(h1 @ W2 + b2, 0)
    return softplus(h2 @ W3 + b3)


def loss_grad(w_u16, X, y):
    """(loss summed over samples, gradient wrt the parameters)."""
    w = bf16_to_f64(w_u16)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    a1 = X @ W1 + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0)
    out = h2 @ W3 + b3
    lam = softplus(out)
    d = np.log1p(lam) - np.log1p(y)
    loss = float((d * d).sum())
    g = 2 * d / (1 + lam) / (1 + np.exp(-out))
    grad = np.zeros(NUM_PARAMS)
    grad[OFF_W3:OFF_B3] = h2.T @ g
    grad[OFF_B3] = g.sum()
    dh2 = np.outer(g, W3) * (a2 > 0)
    grad[OFF_W2:OFF_B2] = (h1.T @ dh2).reshape(-1)
    grad[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (a1 > 0)
    grad[OFF_W1:OFF_B1] = (X.T @ dh1).reshape(-1)
    grad[OFF_B1:OFF_W2] = dh1.sum(0)
    return loss, grad

"""FP64 numpy oracle of the MLP surrogate's forward, backward and Adam step —
TEST INFRASTRUCTURE ONLY.  BF16 rounding (round to nearest even on the upper
16 bits of an IEEE float32) is applied at the same points as the device:
inputs, weights, activations and backward deltas are BF16, accumulation and
pre-activations are wider.  GELU is the erf form z * Phi(z)."""
import numpy as np
from scipy.special import erf


def bf16(x):
    """Round float32 values to bfloat16 (returned as float64)."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def hidden(x16, w16, b):
    """z = x16 @ w16^T + b; a16 = bf16(gelu(z))."""
    z = x16 @ w16.T + b
    return z, bf16(gelu(z))


def back(dy16, w16, z):
    """delta16 = bf16((dy16 @ w16) * gelu'(z))."""
    return bf16((dy16 @ w16) * gelu_grad(z))


def adam(w, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1**step)
    vh = v / (1 - b2**step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def predict(q, mu_q, inv_q, mu_g, sig_g, W, b):
    """Surrogate gradient at positions q [d][C] with weights W (FP32 masters,
    rounded to BF16 here) and biases b: the output layer reads [h2 | x]."""
    x = bf16(((q.T - mu_q) * inv_q).astype(np.float32))
    w16 = [bf16(w) for w in W]
    _, a1 = hidden(x, w16[0], b[0])
    _, a2 = hidden(a1, w16[1], b[1])
    y = np.c_[a2, x] @ w16[2].T + b[2]
    return (y * sig_g + mu_g).T

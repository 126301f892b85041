"""FP64 numpy oracle of the surrogates (the MLP's forward, backward and Adam
step; the scalar potential's gradient pass and double backpropagation) —
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


# ---- scalar-potential surrogate ---------------------------------------------
# f(x) = w3 . gelu(W2 gelu(W1 x + b1) + b2) + x^T A x / 2 + beta . x, with the
# leapfrog driven by grad_q f = grad_x f / s.  Two forms: exact FP64 (for
# finite-difference checks) and the device's rounding points (BF16 inputs,
# weights, activations and deltas; FP32-or-wider accumulation).


def gelu_grad2(z):
    return np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi) * (2.0 - z * z)


def potential_value(x, W1, b1, W2, b2, w3, A, beta):
    """f at rows of x [B][d] (FP64, no rounding)."""
    a2 = gelu(gelu(x @ W1.T + b1) @ W2.T + b2)
    return a2 @ w3 + 0.5 * np.sum((x @ A) * x, axis=1) + x @ beta


def potential_grad(x, W1, b1, W2, b2, w3, A, beta):
    """grad_x f at rows of x [B][d] (FP64, no rounding)."""
    z1 = x @ W1.T + b1
    z2 = gelu(z1) @ W2.T + b2
    delta2 = w3 * gelu_grad(z2)
    delta1 = (delta2 @ W2) * gelu_grad(z1)
    return delta1 @ W1 + x @ A + beta


def potential_loss_grads(x, t, scale, shift, W1, b1, W2, b2, w3, A, beta):
    """Loss 0.5/B sum |y - t|^2 of y = scale * grad_x f + shift and its
    gradients with respect to W1, b1, W2, b2, w3 (FP64, no rounding), by the
    double backpropagation the device runs."""
    B = x.shape[0]
    z1 = x @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    delta2 = w3 * gelu_grad(z2)
    u1 = delta2 @ W2
    delta1 = u1 * gelu_grad(z1)
    gx = delta1 @ W1 + x @ A + beta
    y = scale * gx + shift
    loss = 0.5 * np.sum((y - t) ** 2) / B
    e = scale * (y - t) / B
    dbar1 = e @ W1.T
    ubar1 = dbar1 * gelu_grad(z1)
    zbar1 = dbar1 * u1 * gelu_grad2(z1)
    dbar2 = ubar1 @ W2.T
    gw3 = np.sum(dbar2 * gelu_grad(z2), axis=0)
    zbar2 = dbar2 * w3 * gelu_grad2(z2)
    abar1 = zbar2 @ W2
    zbar1 = zbar1 + abar1 * gelu_grad(z1)
    gW1 = delta1.T @ e + zbar1.T @ x
    gW2 = delta2.T @ ubar1 + zbar2.T @ a1
    return loss, {"W1": gW1, "b1": zbar1.sum(0), "W2": gW2, "b2": zbar2.sum(0), "w3": gw3}


def potential_value_loss_grads(x, t, weight, W1, b1, W2, b2, w3):
    """Value-matching loss 0.5 weight mean_b (r_b - rbar)^2 with
    r_b = w3 . GELU(W2 GELU(W1 x_b + b1) + b2) - t_b (t_b: the exact misfit
    minus the fixed quadratic part) and its gradients with respect to
    W1, b1, W2, b2, w3 (FP64, no rounding; plain backpropagation)."""
    B = x.shape[0]
    z1 = x @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    a2 = gelu(z2)
    r = a2 @ w3 - t
    c = r - r.mean()
    loss = 0.5 * weight * np.sum(c * c) / B
    dv = weight * c / B
    delta2 = w3 * gelu_grad(z2)
    delta1 = (delta2 @ W2) * gelu_grad(z1)
    dz2 = dv[:, None] * delta2
    dz1 = dv[:, None] * delta1
    return loss, {"W1": dz1.T @ x, "b1": dz1.sum(0), "W2": dz2.T @ a1, "b2": dz2.sum(0), "w3": dv @ a2}


def potential_predict(q, mu_q, s_q, mu_g, sig_g, W1, b1, W2, b2, w3, A, beta):
    """Surrogate gradient grad_q f at positions q [d][C] with the device's
    rounding points: x, W1, W2 and the scaled output matrix [W1^T | A] / (s
    sig_g) in BF16, activations and deltas in BF16."""
    x = bf16(((q.T - mu_q) / s_q).astype(np.float32))
    D = 1.0 / (s_q * sig_g)
    w1, w2 = bf16(W1), bf16(W2)
    z1 = x @ w1.T + b1
    a1 = bf16(gelu(z1))
    z2 = a1 @ w2.T + b2
    delta2 = bf16(w3 * gelu_grad(z2))
    delta1 = bf16((delta2 @ bf16(W2.T).T) * gelu_grad(z1))
    wg = bf16(np.c_[(D[:, None] * W1.T), D[:, None] * A])  # [d][h1 + d]
    bias = D * beta - mu_g / sig_g
    y = np.c_[delta1, x] @ wg.T + bias
    return (y * sig_g + mu_g).T

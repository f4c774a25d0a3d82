"""CPU oracle of the learned correction's MLP — TEST INFRASTRUCTURE ONLY.

Follows the reference's CPU neural math for the pieces it has:
LINEAR forward/backward (src/gfx/neural_math.cpp:119-132 and its backward),
the mean squared error, and Adam (neural_math.cpp:1177-1208); the central
finite-difference gradient check follows tests/gradient_check.h:22-60
(double precision, step 1e-5, error scaled by the typical gradient size).
GELU (Hendrycks & Gimpel 2016, z Phi(z) with erf(z / sqrt 2) taken as
tanh(a z + b z^3), a = sqrt(2 / pi), b = 0.044715 a) and BF16 rounding (round
to nearest even of the FP32 value) are new here (the reference has neither);
the GPU evaluates the tanh with the hardware's approximate tanh.

`forward(..., bf16=True)` rounds where the GPU rounds: the normalised input,
the weights and both hidden activations become BF16 before each product,
with products summed in double.
"""
from __future__ import annotations

import math

import numpy as np

IN, HIDDEN, OUT = 32, 128, 3
W1, B1 = 0, HIDDEN * IN
W2 = B1 + HIDDEN
B2 = W2 + HIDDEN * HIDDEN
W3 = B2 + HIDDEN
B3 = W3 + OUT * HIDDEN
PARAMS = B3 + OUT

_erf = np.vectorize(math.erf)


def bf16(x) -> np.ndarray:
    """Round FP32 values to BF16 (nearest even); returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    return (p[W1:B1].reshape(HIDDEN, IN), p[B1:W2], p[W2:B2].reshape(HIDDEN, HIDDEN), p[B2:W3],
            p[W3:B3].reshape(OUT, HIDDEN), p[B3:PARAMS])


GELU_A = math.sqrt(2.0 / math.pi)
GELU_B = 0.044715 * GELU_A


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(z * (GELU_A + GELU_B * z * z)))


def gelu_grad(z):
    t = np.tanh(z * (GELU_A + GELU_B * z * z))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * (GELU_A + 3.0 * GELU_B * z * z)


def gelu_erf(z):
    """The exact erf form, for comparing the approximation against it."""
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def normalise(features, mean, std):
    """(f - mean) * (1 / std) in float32, as the GPU kernel computes it."""
    f = np.asarray(features, np.float32)
    inv = (np.float32(1.0) / np.asarray(std, np.float32)).astype(np.float32)
    return ((f - np.asarray(mean, np.float32)) * inv).astype(np.float32)


def forward(params, features, mean, std, scale, bf16_rounding=True):
    """Returns (y, cache): y is the network output before scaling."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    x = normalise(features, mean, std)
    r = (lambda a: bf16(a).astype(np.float64)) if bf16_rounding else (lambda a: np.asarray(a, np.float64))
    x = r(x)
    if bf16_rounding:
        w1r, w2r, w3r = r(w1.astype(np.float32)), r(w2.astype(np.float32)), r(w3.astype(np.float32))
    else:
        w1r, w2r, w3r = w1, w2, w3
    z1 = x @ w1r.T + b1
    h1 = r(gelu(z1).astype(np.float32)) if bf16_rounding else gelu(z1)
    z2 = h1 @ w2r.T + b2
    h2 = r(gelu(z2).astype(np.float32)) if bf16_rounding else gelu(z2)
    y = h2 @ w3r.T + b3
    cache = dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, w1=w1r, w2=w2r, w3=w3r)
    return y, cache


def loss_and_grad(params, features, targets, mean, std, scale, bf16_rounding=True, bf16_grads=False):
    """Mean squared error on normalised targets and its gradient (double).

    bf16_grads rounds the backward's operands to BF16 where the GPU's
    tensor-core backward does: dY on its way into the W3 gradient (its bias
    gradient sums the unrounded dY), dZ2 (computed from the unrounded dY)
    into the W2 and b2 gradients and into dH1 = dZ2 W2, and dZ1 into the W1
    and b1 gradients."""
    y, c = forward(params, features, mean, std, scale, bf16_rounding)
    t = np.asarray(targets, np.float64) / np.asarray(scale, np.float64)
    n = y.shape[0]
    e = y - t
    loss = float((e * e).sum() / (n * OUT))
    dy = 2.0 * e / (n * OUT)
    r = (lambda a: bf16(np.asarray(a, np.float32)).astype(np.float64)) if bf16_grads else (lambda a: a)
    g = np.zeros(PARAMS)
    g[W3:B3] = (r(dy).T @ c["h2"]).reshape(-1)
    g[B3:PARAMS] = dy.sum(0)
    dz2 = r((dy @ c["w3"]) * gelu_grad(c["z2"]))
    g[W2:B2] = (dz2.T @ c["h1"]).reshape(-1)
    g[B2:W3] = dz2.sum(0)
    dz1 = r((dz2 @ c["w2"]) * gelu_grad(c["z1"]))
    g[W1:B1] = (dz1.T @ c["x"]).reshape(-1)
    g[B1:W2] = dz1.sum(0)
    return loss, g


def relative_error(a: float, b: float, typical: float) -> float:
    """tests/gradient_check.h:22-25: scaled by the typical gradient size."""
    scale = max(abs(a), abs(b), 0.05 * typical, 1.0e-6)
    return abs(a - b) / scale


def finite_difference_check(params, features, targets, mean, std, scale, indices, h=1.0e-5):
    """Worst relative error between the analytic gradient (double, no BF16)
    and central differences at the given parameter indices."""
    p = np.asarray(params, np.float64).copy()
    _, g = loss_and_grad(p, features, targets, mean, std, scale, bf16_rounding=False)
    typical = float(np.abs(g).max())
    worst = 0.0
    for i in indices:
        keep = p[i]
        p[i] = keep + h
        plus, _ = loss_and_grad(p, features, targets, mean, std, scale, bf16_rounding=False)
        p[i] = keep - h
        minus, _ = loss_and_grad(p, features, targets, mean, std, scale, bf16_rounding=False)
        p[i] = keep
        worst = max(worst, relative_error(g[i], (plus - minus) / (2.0 * h), typical))
    return worst


def adam_step(params, grads, first, second, step, lr, beta1=0.9, beta2=0.999, epsilon=1e-8):
    """adamCorrections + adamStep (neural_math.cpp:1177-1208), float32."""
    f32 = np.float32
    c1 = f32(1.0) - f32(beta1) ** f32(step)
    c2 = f32(1.0) - f32(beta2) ** f32(step)
    g = np.asarray(grads, np.float32)
    first[:] = f32(beta1) * first + (f32(1.0) - f32(beta1)) * g
    second[:] = f32(beta2) * second + (f32(1.0) - f32(beta2)) * g * g
    params[:] = params - f32(lr) * (first / c1) / (np.sqrt(second / c2) + f32(epsilon))
    return params

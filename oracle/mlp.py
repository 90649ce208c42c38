"""FP64 reference of the learned proposal (TEST INFRASTRUCTURE ONLY).

The learned proposal has no counterpart in the reference: a small MLP maps a
site's six neighbour directors and the temperature (19 inputs) to the mean
axis mu (3) and log-concentration l (1) of an antipodally symmetric von
Mises-Fisher mixture on the sphere,

    q(n' | nbrs) = C(kappa) cosh(kappa * muhat . n'),  C(kappa) = kappa / (4 pi sinh kappa),

(half vMF(muhat, kappa) + half vMF(-muhat, kappa), invariant under n -> -n
like the nematic energy).  Because mu and kappa depend only on the
neighbours, Metropolis-Hastings with this independence proposal accepts
n -> n' with probability

    min(1, exp(-dE/T) * cosh(kappa muhat.n) / cosh(kappa muhat.n')).

This module restates, in FP64 NumPy: the MLP (19 -> 64 -> 64 -> 4, GELU with
the tanh form), its negative log-likelihood loss and gradients (checked here
by finite differences), the mixture's log density, its exact inverse-CDF
sampler (Wood 1994 for the 3-sphere case), and the MH log ratio.
"""
from __future__ import annotations

import numpy as np

D_IN, D_H, D_OUT = 19, 64, 4
K_IN = 32  # inputs padded to a multiple of 16 for the BF16 tensor-core tiles
N_OUT = 8  # outputs padded to one 8-wide tile
LOGK_MIN, LOGK_MAX = -4.0, 6.0
GELU_C = 0.7978845608028654  # sqrt(2/pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    u = GELU_C * (x + 0.044715 * x ** 3)
    t = np.tanh(u)
    du = GELU_C * (1.0 + 3 * 0.044715 * x ** 2)
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * du


def init_params(rng: np.random.Generator, scale: float = 1.0):
    """Weights as (W1 [19,64], b1 [64], W2 [64,64], b2 [64], W3 [64,4], b3 [4])."""
    W1 = rng.normal(0, scale / np.sqrt(D_IN), (D_IN, D_H))
    W2 = rng.normal(0, scale / np.sqrt(D_H), (D_H, D_H))
    W3 = rng.normal(0, scale / np.sqrt(D_H), (D_H, D_OUT))
    return [W1, np.zeros(D_H), W2, np.zeros(D_H), W3, np.zeros(D_OUT)]


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = params
    H1 = X @ W1 + b1
    A1 = gelu(H1)
    H2 = A1 @ W2 + b2
    A2 = gelu(H2)
    Y = A2 @ W3 + b3
    return Y, (X, H1, A1, H2, A2)


def log_cosh(x):
    ax = np.abs(x)
    return ax + np.log1p(np.exp(-2.0 * ax)) - np.log(2.0)


def log_sinh(k):
    return k + np.log1p(-np.exp(-2.0 * k)) - np.log(2.0)


def split_out(Y):
    """mu-hat, kappa, |mu|, the clamped log-kappa and whether it was clamped."""
    mu = Y[:, :3]
    nm = np.linalg.norm(mu, axis=1)
    muhat = mu / np.maximum(nm, 1e-12)[:, None]
    l = np.clip(Y[:, 3], LOGK_MIN, LOGK_MAX)
    clamped = (Y[:, 3] < LOGK_MIN) | (Y[:, 3] > LOGK_MAX)
    return muhat, np.exp(l), nm, l, clamped


def log_density(Y, n):
    """log q(n) of the antipodal mixture for outputs Y and unit vectors n."""
    muhat, k, _, _, _ = split_out(Y)
    m = np.sum(muhat * n, axis=1)
    return np.log(k) - np.log(4 * np.pi) - log_sinh(k) + log_cosh(k * m)


def nll_and_grad(params, X, n):
    """Mean negative log density of targets n and its gradient w.r.t. params."""
    Y, (X_, H1, A1, H2, A2) = forward(params, X)
    B = X.shape[0]
    muhat, k, nm, l, clamped = split_out(Y)
    m = np.sum(muhat * n, axis=1)
    loss = -np.mean(log_density(Y, n))
    th = np.tanh(k * m)
    coth = 1.0 / np.tanh(k)
    dL_dk = (-1.0 / k + coth - m * th) / B
    dL_dl = np.where(clamped, 0.0, dL_dk * k)
    dL_dm = (-k * th) / B
    dL_dmu = dL_dm[:, None] * (n - m[:, None] * muhat) / np.maximum(nm, 1e-12)[:, None]
    dY = np.concatenate([dL_dmu, dL_dl[:, None]], axis=1)
    W1, b1, W2, b2, W3, b3 = params
    gW3 = A2.T @ dY
    gb3 = dY.sum(0)
    dA2 = dY @ W3.T
    dH2 = dA2 * gelu_grad(H2)
    gW2 = A1.T @ dH2
    gb2 = dH2.sum(0)
    dA1 = dH2 @ W2.T
    dH1 = dA1 * gelu_grad(H1)
    gW1 = X_.T @ dH1
    gb1 = dH1.sum(0)
    return loss, [gW1, gb1, gW2, gb2, gW3, gb3]


def sample(Y, u_w, u_phi, u_sign):
    """Draws from the antipodal mixture: w = cos(angle to muhat) by the exact
    inverse CDF w = 1 + log(1 - (1-u)(1-exp(-2 kappa)))/kappa, an azimuth
    2 pi u_phi about muhat, and the sign flip with probability 1/2."""
    muhat, k, _, _, _ = split_out(Y)
    w = 1.0 + np.log1p(-(1.0 - u_w) * (-np.expm1(-2.0 * k))) / k
    w = np.clip(w, -1.0, 1.0)
    # an orthonormal pair perpendicular to muhat
    a = np.where(np.abs(muhat[:, 0:1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    e1 = np.cross(muhat, a)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(muhat, e1)
    phi = 2 * np.pi * u_phi
    r = np.sqrt(np.maximum(0.0, 1 - w * w))
    v = w[:, None] * muhat + r[:, None] * (np.cos(phi)[:, None] * e1 + np.sin(phi)[:, None] * e2)
    return np.where((u_sign < 0.5)[:, None], v, -v)


def mh_log_ratio(Y, n_old, n_new, dE, T):
    """log of exp(-dE/T) q(n_old)/q(n_new)."""
    muhat, k, _, _, _ = split_out(Y)
    return -dE / T + log_cosh(k * np.sum(muhat * n_old, 1)) - log_cosh(k * np.sum(muhat * n_new, 1))


def features(nbrs: np.ndarray, T) -> np.ndarray:
    """Network input: the six neighbour directors (x+, x-, y+, y-, z+, z-; 18
    numbers) then T."""
    B = nbrs.shape[0]
    T = np.broadcast_to(np.asarray(T, np.float64), (B,))
    return np.concatenate([nbrs.reshape(B, 18), T[:, None]], axis=1)


def pack_weights(params):
    """Flat FP32 layout the engine takes: W1 [32 x 64] (rows 19..31 zero),
    b1 [64], W2 [64 x 64], b2 [64], W3 [64 x 8] (cols 4..7 zero), b3 [8]."""
    W1, b1, W2, b2, W3, b3 = params
    W1p = np.zeros((K_IN, D_H))
    W1p[:D_IN] = W1
    W3p = np.zeros((D_H, N_OUT))
    W3p[:, :D_OUT] = W3
    b3p = np.zeros(N_OUT)
    b3p[:D_OUT] = b3
    return np.concatenate([W1p.ravel(), b1, W2.ravel(), b2, W3p.ravel(), b3p]).astype(np.float32)


def unpack_weights(flat):
    flat = np.asarray(flat, np.float64)
    o = 0

    def take(n, shape):
        nonlocal o
        x = flat[o:o + n].reshape(shape)
        o += n
        return x

    W1p = take(K_IN * D_H, (K_IN, D_H))
    b1 = take(D_H, (D_H,))
    W2 = take(D_H * D_H, (D_H, D_H))
    b2 = take(D_H, (D_H,))
    W3p = take(D_H * N_OUT, (D_H, N_OUT))
    b3p = take(N_OUT, (N_OUT,))
    return [W1p[:D_IN], b1, W2, b2, W3p[:, :D_OUT], b3p[:D_OUT]]


N_PARAMS = K_IN * D_H + D_H + D_H * D_H + D_H + D_H * N_OUT + N_OUT


def bf16_round(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu_bf16_arith(h):
    """GELU as the engine's inference kernel evaluates it: packed BF16
    arithmetic, every operation rounded to bfloat16 (tanh itself exact here,
    approximate in hardware), constants rounded to bfloat16."""
    c = bf16_round(GELU_C)
    c3 = bf16_round(GELU_C * 0.044715)
    x = bf16_round(h)
    x2 = bf16_round(x * x)
    t = bf16_round(x2 * c3 + c)
    u = bf16_round(x * t)
    th = bf16_round(np.tanh(u))
    hh = bf16_round(x * 0.5)
    return bf16_round(hh * th + hh)


def forward_bf16(params, X):
    """The forward pass with the engine's roundings: inputs, weights and hidden
    activations as bfloat16, FP32-exact products accumulated in FP64, GELU in
    BF16 arithmetic (gelu_bf16_arith)."""
    W1, b1, W2, b2, W3, b3 = params
    H1 = bf16_round(X) @ bf16_round(W1) + b1
    A1 = gelu_bf16_arith(H1)
    H2 = A1 @ bf16_round(W2) + b2
    A2 = gelu_bf16_arith(H2)
    return A2 @ bf16_round(W3) + b3

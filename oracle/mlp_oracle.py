"""Float64 restatement of the learned-radius network -- TEST INFRASTRUCTURE ONLY.

Independent CPU computation of the radius network's forward pass and of the
gradient of its training loss, used by the tests to check the library's GPU
training and inference kernels. It applies the same BF16 roundings the GPU
path applies (weights, inputs and the first hidden layer; round to nearest
even), and computes everything else in float64.

Parameter layout (float32 vector of 5313): W1[64][16], b1[64], W2[64][64],
b2[64], w3[64], b3. Loss: mean squared error between the network output and
the standardised target; the gradient of the mean is returned together with
the summed squared error.
"""
from __future__ import annotations

import numpy as np

F, H = 16, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
N_PARAMS = OFF_B3 + 1


def bf16_round(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params):
    p = bf16_round(np.asarray(params, np.float32)).astype(np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, F), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(params, X):
    """Standardised network output for features X (n, 16); plus the activations."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    x = bf16_round(X).astype(np.float64)
    z1 = x @ W1.T + b1
    a1 = bf16_round((z1 * _sig(z1)).astype(np.float32)).astype(np.float64)
    z2 = a1 @ W2.T + b2
    a2 = z2 * _sig(z2)
    y = a2 @ w3 + b3
    return y, dict(x=x, z1=z1, a1=a1, z2=z2, a2=a2)


def _dsilu(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def gradients(params, X, Y):
    """(gradient of mean((y - Y)^2) w.r.t. the parameters, summed squared error)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    y, a = forward(params, X)
    n = X.shape[0]
    e = y - np.asarray(Y, np.float64)
    dy = 2.0 * e / n
    g = np.zeros(N_PARAMS, np.float64)
    g[OFF_W3:OFF_B3] = a["a2"].T @ dy
    g[OFF_B3] = dy.sum()
    dz2 = dy[:, None] * w3[None, :] * _dsilu(a["z2"])
    g[OFF_W2:OFF_B2] = (dz2.T @ a["a1"]).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    dz1 = (dz2 @ W2) * _dsilu(a["z1"])  # the BF16 rounding of a1 is passed straight through
    g[OFF_W1:OFF_B1] = (dz1.T @ a["x"]).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    return g, float(np.sum(e * e))

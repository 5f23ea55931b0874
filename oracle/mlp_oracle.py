"""mlp_oracle.py - FP64 CPU restatement of the move-proposal network.

TEST INFRASTRUCTURE ONLY: the checker of the GPU forward / backward kernels
of gala-mg_gb300/csrc/proposal.cu (k_mlp_grad, k_mlp_logits, the inference of
k_prop_step).  The engine never calls it.  The network has no counterpart in
the reference (LinXi-lx/GALA-mg), so its parity is pinned by finite
differences of this oracle's own loss (tests/test_oracle.py), not by a
reference vector.

Network: x (8) -> relu(W1 x + b1) (32) -> relu(W2 h1 + b2) (32) -> w3 h2 + b3.
Parameter vector layout (1377 floats): W1[32][8], b1[32], W2[32][32], b2[32],
w3[32], b3.  Loss: sum over samples of wt * (softplus(out) - y * out), the
binary cross-entropy of sigmoid(out), wt = pos_weight for y = 1, else 1.
"""
import numpy as np

N_IN, N_H = 8, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_H
N_PARAMS = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(N_H, N_IN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(N_H, N_H)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def forward(p, X):
    """Logits of the rows of X (FP64)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ w3 + b3


def bf16_round(p):
    """Round float32 values to bfloat16 (round to nearest even), as
    __float2bfloat16_rn does for finite inputs."""
    a = np.ascontiguousarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (a >> 16) & 1
    r = ((a + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def loss_and_grad(p, X, Y, pos_weight=1.0):
    """Summed weighted BCE and its gradient with respect to p (FP64)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    out = h2 @ w3 + b3
    wt = np.where(Y > 0.5, pos_weight, 1.0)
    sp = np.logaddexp(0.0, out)  # softplus
    loss = float(np.sum(wt * (sp - Y * out)))
    dout = wt * (1.0 / (1.0 + np.exp(-out)) - Y)
    g = np.zeros(N_PARAMS, dtype=np.float64)
    g[OFF_W3:OFF_B3] = dout @ h2
    g[OFF_B3] = dout.sum()
    dz2 = (dout[:, None] * w3[None, :]) * (z2 > 0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    g[OFF_W1:OFF_B1] = (dz1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    return loss, g

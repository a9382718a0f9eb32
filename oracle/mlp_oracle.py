"""Float64 restatement of the hybrid classifier's network and loss.

TEST INFRASTRUCTURE ONLY (tests/ import it to check the GPU forward and
training kernels of fiesta_gb300/csrc/fst_hybrid.cu).

Network: 20 -> 32 -> 32 -> 1, ReLU, ReLU, sigmoid.  Parameters packed as
W1[32][20], b1[32], W2[32][32], b2[32], w3[32], b3 (include/fst.h).
Loss: mean over samples of w * (softplus(z) - y z), w = pos_weight if y = 1.
"""
import numpy as np

NI, NH = 20, 32
NP = NH * NI + NH + NH * NH + NH + NH + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + NH * NI].reshape(NH, NI); o += NH * NI
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / NI), (NH, NI))
    W2 = rng.normal(0, np.sqrt(2.0 / NH), (NH, NH))
    w3 = rng.normal(0, np.sqrt(1.0 / NH), NH)
    return pack(W1, np.zeros(NH), W2, np.zeros(NH), w3, 0.0)


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ w3 + b3
    return z, (X, a1, h1, a2, h2)


def prob(p, X):
    z, _ = forward(p, X)
    return 1.0 / (1.0 + np.exp(-z))


def loss_grad(p, X, y, pos_weight=1.0):
    z, (X, a1, h1, a2, h2) = forward(p, X)
    y = np.asarray(y, dtype=np.float64)
    w = np.where(y > 0.5, pos_weight, 1.0)
    sp = np.logaddexp(0.0, z)
    n = len(y)
    loss = np.sum(w * (sp - y * z)) / n
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / n
    W1, b1, W2, b2, w3, b3 = unpack(p)
    gw3 = h2.T @ dz
    gb3 = dz.sum()
    d2 = np.outer(dz, w3) * (a2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    return loss, pack(gW1, gb1, gW2, gb2, gw3, gb3)

"""CPU restatement of the preconditioner network's forward pass, loss and
gradient, with the BF16 roundings of the tensor-core kernels (inputs,
weights, hidden activations and backpropagated errors rounded to BF16;
products accumulated in FP32 or wider), and of its per-atom inputs
(descriptors).  TEST INFRASTRUCTURE ONLY: the checker of mappg_mlp_grad,
mappg_mlp_predict and mappg_sys_descriptors.

Layout of the parameter vector (10496 floats): W1 [64][64] | W2 [64][80] |
W3 [16][80], row-major [unit][input]; input 33 of W1 and input 64 of W2, W3
are the biases (constant-one inputs).  Outputs: softplus of the first three
units of layer 3.  Loss: mean over atoms and outputs of (log y - log t)^2.
"""
import numpy as np

NIN, NH, NHK, NOUT = 64, 64, 80, 16
SIZES = (NH * NIN, NH * NHK, NOUT * NHK)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def unpack(w):
    w = np.asarray(w, dtype=np.float32)
    a, b, c = SIZES
    return w[:a].reshape(NH, NIN), w[a:a + b].reshape(NH, NHK), w[a + b:].reshape(NOUT, NHK)


def inputs(feat, mean, sdev):
    n = feat.shape[0]
    X = np.zeros((n, NIN), dtype=np.float32)
    X[:, :33] = (np.asarray(feat, np.float32) - mean) / sdev
    X[:, 33] = 1.0
    return bf16(X)


def softplus(z):
    return np.where(z > 20.0, z, np.log1p(np.exp(np.minimum(z, 20.0))))


def forward(w, X):
    W1, W2, W3 = (bf16(m).astype(np.float64) for m in unpack(w))
    n = X.shape[0]
    H1 = np.zeros((n, NHK), np.float32)
    H1[:, :NH] = bf16(np.tanh(X.astype(np.float64) @ W1.T))
    H1[:, NH] = 1.0
    H2 = np.zeros((n, NHK), np.float32)
    H2[:, :NH] = bf16(np.tanh(H1.astype(np.float64) @ W2.T))
    H2[:, NH] = 1.0
    Z3 = H2.astype(np.float64) @ W3.T
    return H1, H2, Z3


def loss_grad(w, X, T):
    """Loss and gradient (same layout as w) of the mean squared log error."""
    W1, W2, W3 = (bf16(m).astype(np.float64) for m in unpack(w))
    n = X.shape[0]
    H1, H2, Z3 = forward(w, X)
    z = Z3[:, :3]
    y = softplus(z)
    r = np.log(y) - np.log(T)
    loss = np.sum(r * r) / (3 * n)
    dz3 = np.zeros((n, NOUT))
    dz3[:, :3] = 2.0 * r / y / (1.0 + np.exp(-z)) / (3 * n)
    dz3 = bf16(dz3).astype(np.float64)
    dh2 = dz3 @ W3[:, :NH]
    dz2 = bf16(dh2 * (1.0 - H2[:, :NH].astype(np.float64) ** 2)).astype(np.float64)
    dh1 = dz2 @ W2[:, :NH]
    dz1 = bf16(dh1 * (1.0 - H1[:, :NH].astype(np.float64) ** 2)).astype(np.float64)
    g3 = dz3.T @ H2.astype(np.float64)
    g2 = dz2.T @ H1.astype(np.float64)
    g1 = dz1.T @ X.astype(np.float64)
    return loss, np.concatenate([g1.ravel(), g2.ravel(), g3.ravel()])


# the network's per-atom inputs (k_descriptors)
DESC_R, DESC_RC, DESC_W = 16, 5.5, 0.3
DESC_CENTRES = 2.0 + 3.5 * np.arange(DESC_R) / 15.0


def descriptors(H, x, elem, rho):
    """Per-atom inputs as k_descriptors forms them, in FP64: 16 Gaussian
    radial functions (centres 2.0-5.5 A in 15 equal steps, width 0.3 A)
    times the cosine cutoff 0.5 (1 + cos(pi r / 5.5)), summed over the
    neighbours of element 0 (columns 0-15) and of element 1 (columns 16-31)
    within 5.5 A, every periodic image counted; column 32 is the host
    density rho (passed in: the oracle's per-atom EAM density).  H: rows are
    the cell vectors.  Brute force over images: for test-sized cells."""
    H = np.asarray(H, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    elem = np.asarray(elem)
    n = len(x)
    # image range per cell vector: the spacing of its lattice planes
    vol = abs(np.linalg.det(H))
    reach = []
    for k in range(3):
        a, b = H[(k + 1) % 3], H[(k + 2) % 3]
        reach.append(int(np.ceil(DESC_RC / (vol / np.linalg.norm(np.cross(a, b))))) + 1)
    shifts = np.array([(i, j, k) for i in range(-reach[0], reach[0] + 1) for j in range(-reach[1], reach[1] + 1)
                       for k in range(-reach[2], reach[2] + 1)], dtype=np.float64) @ H
    out = np.zeros((n, 2 * DESC_R + 1))
    for i in range(n):
        d = x[i][None, None, :] - (x[None, :, :] + shifts[:, None, :])  # [shift][j][3]
        r = np.sqrt(np.sum(d * d, axis=2))
        keep = (r < DESC_RC) & (r > 0.0)
        sh, j = np.nonzero(keep)
        rr = r[sh, j]
        fc = 0.5 * (1.0 + np.cos(np.pi * rr / DESC_RC))
        g = np.exp(-(rr[:, None] - DESC_CENTRES[None, :]) ** 2 / (2.0 * DESC_W * DESC_W)) * fc[:, None]
        for e in (0, 1):
            out[i, e * DESC_R:(e + 1) * DESC_R] = g[elem[j] == e].sum(axis=0)
    out[:, 2 * DESC_R] = rho
    return out

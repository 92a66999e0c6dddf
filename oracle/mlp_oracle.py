"""CPU oracle of the proposal network (TEST INFRASTRUCTURE ONLY): numpy forward
and backward of the 16-32-32-1 ReLU MLP with the GPU kernels' BF16 rounding
points (features and weights rounded to BF16; hidden activations and
activation gradients rounded to BF16 where they enter a tensor-core product;
FP32 elsewhere), accumulated in double, with the exact FP32 biases (the
kernels add each bias inside the tensor core as three BF16 terms whose sum is
within about 2^-24 of it).  Used by tests/ to check the GPU training kernel's
loss and gradient."""
import numpy as np

OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 512, 544, 1568, 1600, 1632


def bf16(x):
    """Round float32 to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(w):
    w = np.asarray(w, np.float32)
    return (w[OFF_W1:OFF_B1].reshape(32, 16), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(32, 32),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3], w[OFF_B3])


def forward(w, x):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X = bf16(x).astype(np.float64)
    h1 = np.maximum(X @ bf16(W1).astype(np.float64).T + b1, 0).astype(np.float32)
    h2 = np.maximum(bf16(h1).astype(np.float64) @ bf16(W2).astype(np.float64).T + b2, 0).astype(np.float32)
    y = (bf16(h2).astype(np.float64) @ bf16(W3).astype(np.float64) + float(b3)).astype(np.float32)
    return X, h1, h2, y


def loss_and_grad(w, x, target):
    """Mean squared error over the samples and its gradient (1633 floats)."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    B = x.shape[0]
    X, h1, h2, y = forward(w, x)
    err = y.astype(np.float64) - target
    loss = float(np.mean(err * err))
    dy = (2.0 * err / B).astype(np.float32).astype(np.float64)
    g = np.zeros(1633, np.float64)
    g[OFF_W3:OFF_B3] = dy @ h2.astype(np.float64)
    g[OFF_B3] = dy.sum()
    dh2 = np.where(h2 > 0, dy[:, None] * bf16(W3).astype(np.float64)[None, :], 0.0).astype(np.float32)
    g[OFF_B2:OFF_W3] = dh2.astype(np.float64).sum(0)
    g[OFF_W2:OFF_B2] = (bf16(dh2).astype(np.float64).T @ bf16(h1).astype(np.float64)).reshape(-1)
    dh1 = bf16(dh2).astype(np.float64) @ bf16(W2).astype(np.float64)
    dh1 = np.where(h1 > 0, dh1, 0.0).astype(np.float32)
    g[OFF_B1:OFF_W2] = dh1.astype(np.float64).sum(0)
    g[OFF_W1:OFF_B1] = (bf16(dh1).astype(np.float64).T @ X).reshape(-1)
    return loss, g.astype(np.float32)

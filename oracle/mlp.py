"""ORACLE -- test infrastructure only: numpy float64 restatement of the
learned terminator's 3-layer perceptron (tdscha_gb300/csrc/terminator.cu):
forward, mean-squared-error loss, backpropagated gradients and one Adam step,
used by tests/ to check the GPU kernels.  No counterpart in the reference."""
import numpy as np


def unpack(params, n_in, n_h, n_out):
    o = 0
    out = []
    for shape in ((n_in, n_h), (n_h,), (n_h, n_h), (n_h,), (n_h, n_out), (n_out,)):
        n = int(np.prod(shape))
        out.append(np.asarray(params[o:o + n], dtype=np.float64).reshape(shape))
        o += n
    return out


def forward(params, x, n_in, n_h, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, n_h, n_out)
    h1 = np.tanh(x @ W1 + b1)
    h2 = np.tanh(h1 @ W2 + b2)
    return h1, h2, h2 @ W3 + b3


def loss_grad(params, x, t, n_in, n_h, n_out):
    """Mean over all output elements of (y - t)^2 and its gradient (flat)."""
    W1, b1, W2, b2, W3, b3 = unpack(params, n_in, n_h, n_out)
    x = np.asarray(x, dtype=np.float64)
    h1, h2, y = forward(params, x, n_in, n_h, n_out)
    n = y.size
    r = y - t
    loss = float(np.sum(r * r) / n)
    dy = 2 * r / n
    gW3, gb3 = h2.T @ dy, dy.sum(0)
    d2 = (dy @ W3.T) * (1 - h2 ** 2)
    gW2, gb2 = h1.T @ d2, d2.sum(0)
    d1 = (d2 @ W2.T) * (1 - h1 ** 2)
    gW1, gb1 = x.T @ d1, d1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def adam_step(params, grad, m1, m2, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m1 = b1 * m1 + (1 - b1) * grad
    m2 = b2 * m2 + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return params - lr * (m1 / c1) / (np.sqrt(m2 / c2) + eps), m1, m2

"""The perceptron's GPU kernels (csrc/terminator.cu) against the oracle, and
a short training run."""
import numpy as np
import pytest

import oracle.mlp as om
from tdscha_gb300.terminator import MLP

pytestmark = pytest.mark.gpu


def test_forward_and_gradients_match_oracle(gpu_lib):
    rng = np.random.default_rng(1)
    n_in, n_h, n_out = 64, 256, 128
    mlp = MLP(n_in, n_h, n_out, seed=3)
    p = mlp.get_params().astype(np.float64)
    x = rng.standard_normal((200, n_in)).astype(np.float32)
    t = rng.standard_normal((200, n_out)).astype(np.float32)
    y = mlp.forward(x)
    _, _, yo = om.forward(p, x.astype(np.float64), n_in, n_h, n_out)
    assert np.abs(y - yo).max() / np.abs(yo).max() < 1e-5
    yb = mlp.forward(x, bf16=True)
    assert np.abs(yb - yo).max() / np.abs(yo).max() < 3e-2      # bfloat16 inference
    loss, g = mlp.loss_grad(x, t)
    lo, go = om.loss_grad(p, x.astype(np.float64), t.astype(np.float64), n_in, n_h, n_out)
    assert abs(loss - lo) / lo < 1e-5
    assert np.abs(g - go).max() / np.abs(go).max() < 1e-4


def test_training_reduces_loss(gpu_lib):
    import torch
    rng = np.random.default_rng(2)
    n_in, n_h, n_out = 16, 64, 8
    W = rng.standard_normal((n_in, n_out)) / 4
    x = rng.standard_normal((4096, n_in)).astype(np.float32)
    t = np.tanh(x @ W).astype(np.float32)
    mlp = MLP(n_in, n_h, n_out, seed=4)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = mlp.train_step(xd[:512].contiguous(), td[:512].contiguous(), 3e-3, 1, want_loss=True)
    for it in range(2, 400):
        s = (it * 512) % 4096
        mlp.train_step(xd[s:s + 512].contiguous(), td[s:s + 512].contiguous(), 3e-3, it)
    last = mlp.loss_grad(x[:512], t[:512])[0]
    assert last < 0.1 * first
    # one Adam step on the GPU equals the oracle's
    mlp2 = MLP(n_in, n_h, n_out, seed=5)
    p = mlp2.get_params().astype(np.float64)
    _, g = mlp2.loss_grad(x[:256], t[:256])     # the kernels' own gradient, checked above
    po, _, _ = om.adam_step(p, g.astype(np.float64), np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    mlp2.train_step(xd[:256].contiguous(), td[:256].contiguous(), 1e-3, 1)
    assert np.abs(mlp2.get_params() - po).max() < 1e-6


def test_trained_terminator_gains_over_plain(gpu_lib):
    """The committed network (tdscha_gb300/data), on ten runs it was not
    trained on, at its training shapes (M in [48, 160], N = 4000, 320 Wigner
    steps with full re-orthogonalisation): extending 100 steps to 320 is
    closer to the 320-step spectrum than the 100-step continued fraction with
    the standard terminator."""
    from tdscha_gb300.terminator import LearnedTerminator, evaluate, generate_runs
    runs = generate_runs(10, 320, seed=7)
    rep = evaluate(LearnedTerminator(), runs, 100, 320)
    assert rep["learned_err_median"] < rep["plain_terminator_err_median"]
    assert rep["learned_better_fraction"] >= 0.6

"""The learned cost model's network on the GPU against its CPU restatement
(oracle/mlp.py): forward values and every gradient of the mean squared error
(FP32 device vs FP64 host, relative to the largest gradient: 1e-4), and Adam
training driving the loss down on a smooth synthetic target."""
import numpy as np
import pytest

from oracle import mlp as oracle_mlp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("B,F,H", [(1, 3, 8), (37, 17, 128), (513, 17, 128)])
def test_forward_and_gradients_match_cpu(B, F, H, cuda):
    from tensororder_gb300 import learned

    rng = np.random.default_rng(B + F + H)
    net = learned.MLP(F, H, seed=B)
    x = rng.normal(size=(B, F)).astype(np.float32)
    t = rng.normal(size=B).astype(np.float32)
    p = net.params.cpu().numpy().astype(np.float64)
    y_cpu, _ = oracle_mlp.forward(p, F, H, x)
    y_gpu = net.forward(x)
    assert np.max(np.abs(y_gpu - y_cpu)) <= 1e-4 * max(1.0, np.max(np.abs(y_cpu)))
    loss_cpu, g_cpu = oracle_mlp.loss_grad(p, F, H, x, t)
    loss_gpu, g_gpu = net.loss_grad(x, t)
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * max(1.0, loss_cpu)
    scale = max(1e-12, np.max(np.abs(g_cpu)))
    assert np.max(np.abs(g_gpu - g_cpu)) <= 1e-4 * scale
    # with a real batch most hidden units are active somewhere, so most weights get a gradient
    if B >= 37:
        assert np.count_nonzero(g_gpu) > 0.5 * g_gpu.size


def test_adam_training_fits_a_smooth_target(cuda):
    from tensororder_gb300 import learned

    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, size=(2048, 6)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] + 0.5 * x[:, 3] ** 2).astype(np.float32)
    net = learned.MLP(6, 64, seed=3)
    losses = net.train(x, t, epochs=600, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0]
    assert losses[-1] < 0.02

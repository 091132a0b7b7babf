"""The closure network (tmc_mlp_*): tensor-core forward against a numpy
model of the same arithmetic (BF16 weights and layer inputs, FP32
accumulation, tanh-form GELU), CUDA-core forward and gradient against numpy
in FP64, the tensor-core gradient against numpy models of its BF16 roundings
and of the exact gradient, and Adam training on either that fits a smooth
target."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from mlp_model import NIN, bf16, forward_np, gelu, gelu_grad, unpack  # noqa: F401


def test_tensor_core_forward_matches_model():
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=3)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1000, NIN)).astype(np.float32)  # a partial last tile
    p = net.params
    y_tc = net.forward(x, tensor_cores=True)
    y_ref, _, _ = forward_np(p, x, round_act=True)
    # the tensor-core epilogue evaluates bias and GELU in packed BF16 arithmetic
    scale = np.max(np.abs(y_ref))
    assert np.max(np.abs(y_tc - y_ref)) < 3e-2 * scale
    assert np.sqrt(np.mean((y_tc - y_ref) ** 2)) < 1e-2 * np.sqrt(np.mean(y_ref ** 2))
    y_simt = net.forward(x, tensor_cores=False)
    y_fp, _, _ = forward_np(p, x, round_act=False)
    assert np.max(np.abs(y_simt - y_fp)) < 1e-4 * np.max(np.abs(y_fp))
    net.close()


def test_gradient_matches_numpy():
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=5)
    net.set_train_mode(False)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((256, NIN)).astype(np.float32)
    t = rng.standard_normal(256).astype(np.float32)
    g, loss = net.gradient(x, t)
    p = net.params
    y, zs, W = forward_np(p, x, round_act=False)
    e = y - t
    assert abs(loss - np.mean(e ** 2)) < 1e-4 * np.mean(e ** 2)
    dy = 2 * e / len(t)
    h = [x.astype(np.float64), gelu(zs[0]), gelu(zs[1]), gelu(zs[2])]
    ref = {"W4": dy @ h[3], "b4": np.array([dy.sum()])}
    dz = np.outer(dy, W["W4"]) * gelu_grad(zs[2])
    for layer in (3, 2, 1):
        ref[f"W{layer}"] = dz.T @ h[layer - 1]
        ref[f"b{layer}"] = dz.sum(0)
        if layer > 1:
            dz = (dz @ W[f"W{layer}"]) * gelu_grad(zs[layer - 2])
    G = unpack(g)
    for k, v in ref.items():
        assert np.max(np.abs(G[k] - v)) < 2e-3 * np.max(np.abs(v)) + 1e-7, k
    net.close()


def test_adam_training_fits_a_smooth_target():
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=7)
    net.set_train_mode(False)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((65536, NIN)).astype(np.float32)
    y = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3]).astype(np.float32)
    net.set_dataset(x, y)
    losses = net.train(steps=400, batch=8192, lr=3e-3)
    assert np.all(np.isfinite(losses))
    assert losses[-20:].mean() < 0.05 * losses[:5].mean()
    pred = net.forward(x[:4096], tensor_cores=True)
    assert np.mean((pred - y[:4096]) ** 2) < 0.1 * np.var(y)
    net.close()


def tc_gradient_model(p, x, t):
    """numpy (FP64) gradient of the tensor-core trainer's arithmetic: BF16
    inputs, weights, activations and pre-activation gradients, FP32 biases
    (layer 1's as a high and a low BF16 part), exact GELU and its derivative."""
    P = unpack(p)
    W = {k: bf16(P[k]).astype(np.float64) for k in ("W1", "W2", "W3", "W4")}
    r = lambda a: bf16(a).astype(np.float64)  # noqa: E731
    b1hi = bf16(P["b1"])
    b1 = b1hi.astype(np.float64) + bf16(P["b1"] - b1hi).astype(np.float64)
    x0 = r(x)
    z1 = x0 @ W["W1"].T + b1
    h1 = r(gelu(z1))
    z2 = h1 @ W["W2"].T + P["b2"]
    h2 = r(gelu(z2))
    z3 = h2 @ W["W3"].T + P["b3"]
    h3 = r(gelu(z3))
    y = h3 @ W["W4"] + float(P["b4"][0])
    e = y - t
    dy = 2 * e / len(t)
    dz3 = r(np.outer(dy, W["W4"]) * gelu_grad(z3))
    dz2 = r((dz3 @ W["W3"]) * gelu_grad(z2))
    dz1 = r((dz2 @ W["W2"]) * gelu_grad(z1))
    dyb = r(dy)
    g = {"W1": dz1.T @ x0, "b1": dz1.sum(0), "W2": dz2.T @ h1, "b2": dz2.sum(0), "W3": dz3.T @ h2,
         "b3": dz3.sum(0), "W4": dyb @ h3, "b4": np.array([dyb.sum()])}
    return g, float(np.mean(e ** 2))


def exact_gradient(p, x, t):
    y, zs, W = forward_np(p, x, round_act=False)
    e = y - t
    dy = 2 * e / len(t)
    h = [x.astype(np.float64), gelu(zs[0]), gelu(zs[1]), gelu(zs[2])]
    ref = {"W4": dy @ h[3], "b4": np.array([dy.sum()])}
    dz = np.outer(dy, W["W4"]) * gelu_grad(zs[2])
    for layer in (3, 2, 1):
        ref[f"W{layer}"] = dz.T @ h[layer - 1]
        ref[f"b{layer}"] = dz.sum(0)
        if layer > 1:
            dz = (dz @ W[f"W{layer}"]) * gelu_grad(zs[layer - 2])
    return ref


def test_tensor_core_gradient_matches_numpy():
    """The tensor-core backward: 320 tiles of 128 rows, so blocks sum
    several tiles in their tensor-memory accumulators; against a numpy model
    of its BF16 roundings (FP32 accumulation and tanh.approx are the
    difference), against the exact FP64 gradient, and reproducible bit for
    bit (fixed-order sum over blocks)."""
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=11)
    net.set_train_mode(True)
    rng = np.random.default_rng(4)
    rows = 320 * 128
    x = rng.standard_normal((rows, NIN)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.3 * x[:, 5]).astype(np.float32)
    g, loss = net.gradient(x, t)
    g2, loss2 = net.gradient(x, t)
    assert np.array_equal(g, g2) and loss == loss2
    p = net.params
    model, mloss = tc_gradient_model(p, x, t)
    exact = exact_gradient(p, x, t)
    assert abs(loss - mloss) < 1e-3 * mloss
    G = unpack(g)
    for k in model:
        d_model = np.linalg.norm(G[k] - model[k]) / np.linalg.norm(model[k])
        d_exact = np.linalg.norm(G[k] - exact[k]) / np.linalg.norm(exact[k])
        assert d_model < 2e-4, (k, d_model)  # measured 2e-6 .. 2e-5
        assert d_exact < 2e-3, (k, d_exact)  # measured 1.1e-4 .. 1.6e-4
    # the CUDA-core gradient of the same parameters
    net.set_train_mode(False)
    gs, _ = net.gradient(x, t)
    Gs = unpack(gs)
    for k in model:
        assert np.linalg.norm(G[k] - Gs[k]) / np.linalg.norm(Gs[k]) < 2e-3, k
    net.close()


def test_tensor_core_training_fits_a_smooth_target():
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=7)
    net.set_train_mode(True)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((65536, NIN)).astype(np.float32)
    y = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3]).astype(np.float32)
    net.set_dataset(x, y)
    losses = net.train(steps=400, batch=8192, lr=3e-3)
    assert np.all(np.isfinite(losses))
    assert losses[-20:].mean() < 0.05 * losses[:5].mean()
    pred = net.forward(x[:4096], tensor_cores=True)
    assert np.mean((pred - y[:4096]) ** 2) < 0.1 * np.var(y)
    net.close()


def apvm_exact_gradient(p, x, t, dt):
    """FP64 gradient of the APVM head's loss, mean((-softplus(y) a - t)^2)
    with a = dt (x1 x22 + x0 x23) from the raw features (y_scale 1)."""
    y, zs, W = forward_np(p, x, round_act=False)
    xd = x.astype(np.float64)
    a = dt * (xd[:, 1] * xd[:, 22] + xd[:, 0] * xd[:, 23])
    pred = -np.logaddexp(0.0, y) * a
    e = pred - t
    dy = 2 * e / len(t) * (-a / (1.0 + np.exp(-y)))
    h = [xd, gelu(zs[0]), gelu(zs[1]), gelu(zs[2])]
    ref = {"W4": dy @ h[3], "b4": np.array([dy.sum()])}
    dz = np.outer(dy, W["W4"]) * gelu_grad(zs[2])
    for layer in (3, 2, 1):
        ref[f"W{layer}"] = dz.T @ h[layer - 1]
        ref[f"b{layer}"] = dz.sum(0)
        if layer > 1:
            dz = (dz @ W[f"W{layer}"]) * gelu_grad(zs[layer - 2])
    return ref, float(np.mean(e ** 2)), pred


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_apvm_head_gradient_matches_numpy(tensor_cores):
    """The APVM output head (a non-negative learned weight on the APVM
    direction): the forward output and the gradient of its loss on the CUDA
    cores (FP32) and on the tensor cores (BF16 operands) against FP64 numpy."""
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=13)
    net.set_train_mode(tensor_cores)
    dt = 0.7
    net.set_head(1, dt)
    rng = np.random.default_rng(6)
    rows = 160 * 128
    x = rng.standard_normal((rows, NIN)).astype(np.float32)
    t = (-0.5 * dt * (x[:, 1] * x[:, 22] + x[:, 0] * x[:, 23]) * (1 + 0.3 * np.tanh(x[:, 3]))).astype(np.float32)
    g, loss = net.gradient(x, t)
    p = net.params
    ref, rloss, pred = apvm_exact_gradient(p, x, t, dt)
    assert abs(loss - rloss) < 2e-3 * rloss
    G = unpack(g)
    for k in ref:
        d = np.linalg.norm(G[k] - ref[k]) / np.linalg.norm(ref[k])
        assert d < 3e-3, (k, d)
    # the forward applies the same head
    y = net.forward(x[:4096], tensor_cores=tensor_cores)
    assert np.max(np.abs(y - pred[:4096])) < 3e-2 * np.max(np.abs(pred[:4096]))
    assert np.all(y * (x[:4096, 1] * x[:4096, 22] + x[:4096, 0] * x[:4096, 23]) <= 0.0)
    net.close()


def test_apvm_head_training_lowers_its_loss():
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=14)
    dt = 0.7
    net.set_head(1, dt)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((65536, NIN)).astype(np.float32)
    d = dt * (x[:, 1] * x[:, 22] + x[:, 0] * x[:, 23])
    w = np.log1p(np.exp(1.5 * np.tanh(x[:, 2]) - 0.5))  # a smooth non-negative weight
    t = (-w * d).astype(np.float32)
    net.set_dataset(x, t)
    losses = net.train(steps=300, batch=8192, lr=3e-3)
    assert np.all(np.isfinite(losses))
    assert losses[-20:].mean() < 0.1 * losses[:5].mean()
    net.close()

"""The warm-start network: its CPU oracle pinned by finite differences, and
the GPU kernels' gradients checked against the oracle."""
import numpy as np
import pytest

from oracle import mlp_ref


def test_oracle_gradients_match_finite_differences():
    d_in, d_in_pad, hidden, layers, d_out, d_out_pad = 5, 8, 6, 2, 3, 4
    p = mlp_ref.init_params(d_in, d_in_pad, hidden, layers, d_out, d_out_pad, seed=3)
    rng = np.random.default_rng(1)
    X = np.zeros((7, d_in_pad))
    X[:, :d_in] = rng.normal(size=(7, d_in))
    Y = np.zeros((7, d_out_pad))
    Y[:, :d_out] = rng.integers(0, 2, (7, d_out))
    loss, g = mlp_ref.forward_backward(p, X, Y, d_in_pad, hidden, layers, d_out_pad, d_out,
                                       emulate_bf16=False)
    eps = 1e-6
    num = np.zeros_like(g)
    for i in range(p.size):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp_ref.forward_backward(q, X, Y, d_in_pad, hidden, layers, d_out_pad, d_out,
                                         emulate_bf16=False)
        q[i] -= 2 * eps
        lm, _ = mlp_ref.forward_backward(q, X, Y, d_in_pad, hidden, layers, d_out_pad, d_out,
                                         emulate_bf16=False)
        num[i] = (lp - lm) / (2 * eps) / X.shape[0]  # the gradient is of the mean loss
    assert np.allclose(g, num, rtol=1e-5, atol=1e-7)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0])
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [128, 192])
def test_gpu_gradients_match_oracle(built, rows):
    """The tensor-core GEMMs (tcgen05, 128-row tiles) in the forward and both
    backward products; 192 rows leave a half tile in the batch dimension."""
    import torch
    from simplexprojects_gb300.warmstart import MLP
    d_in, hidden, layers, d_out = 100, 128, 3, 70
    net = MLP(d_in, d_out, hidden, layers, max_batch=rows, seed=5)
    p = net.get_params()
    rng = np.random.default_rng(2)
    X = np.zeros((rows, net.d_in_pad), np.float32)
    X[:, :d_in] = rng.normal(size=(rows, d_in))
    Y = np.zeros((rows, net.d_out_pad), np.float32)
    Y[:, :d_out] = rng.integers(0, 2, (rows, d_out))
    g, loss = net.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda())
    lr, gr = mlp_ref.forward_backward(p, X, Y, net.d_in_pad, hidden, layers, net.d_out_pad, d_out)
    assert abs(loss - lr) <= 1e-4 * abs(lr)
    Ws_g, bs_g = mlp_ref.unpack(g, net.d_in_pad, hidden, layers, net.d_out_pad)
    Ws_r, bs_r = mlp_ref.unpack(gr, net.d_in_pad, hidden, layers, net.d_out_pad)
    for a, b in list(zip(Ws_g, Ws_r)) + list(zip(bs_g, bs_r)):
        assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b) + 1e-9


@pytest.mark.gpu
def test_gpu_forward_matches_oracle(built):
    """Logits of 320 rows (two full 128-row tiles and a half one) against the
    oracle's forward pass with the same BF16 roundings."""
    import torch
    from simplexprojects_gb300.warmstart import MLP
    d_in, hidden, layers, d_out, rows = 300, 512, 3, 316, 320
    net = MLP(d_in, d_out, hidden, layers, max_batch=rows, seed=9)
    p = net.get_params()
    rng = np.random.default_rng(4)
    X = np.zeros((rows, net.d_in_pad), np.float32)
    X[:, :d_in] = rng.normal(size=(rows, d_in))
    out = torch.zeros((rows, net.d_out_pad), dtype=torch.float32, device="cuda")
    net.predict(torch.from_numpy(X).cuda(), out)
    torch.cuda.synchronize()
    z = mlp_ref.forward(p, X, net.d_in_pad, hidden, layers, net.d_out_pad)
    got = out.cpu().numpy()
    assert np.linalg.norm(got - z) <= 2e-3 * np.linalg.norm(z)
    assert np.abs(got - z).max() <= 2e-2 * np.abs(z).max()


@pytest.mark.gpu
def test_gpu_training_reduces_loss_and_topm(built):
    import torch
    from simplexprojects_gb300 import _native as N
    from simplexprojects_gb300.warmstart import MLP
    import ctypes as C
    net = MLP(64, 60, 128, 2, max_batch=256, seed=1)
    rng = np.random.default_rng(0)
    X = np.zeros((256, net.d_in_pad), np.float32)
    X[:, :64] = rng.normal(size=(256, 64))
    Y = np.zeros((256, net.d_out_pad), np.float32)
    Y[:, :60] = (X[:, :60] > 0).astype(np.float32)  # learnable
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    losses = [net.train_step(Xd, Yd, 3e-3) for _ in range(200)]
    assert losses[-1] < 0.3 * losses[0]
    # top-m: the m highest scores in decreasing order, ties by lower column
    scores = torch.from_numpy(rng.normal(size=(3, net.d_out_pad)).astype(np.float32)).cuda()
    scores[1, 5] = scores[1, 9] = 50.0
    m = torch.tensor([4, 4, 4], dtype=torch.int32, device="cuda")
    n = torch.tensor([56, 56, 56], dtype=torch.int32, device="cuda")
    off = torch.tensor([0, 4, 8], dtype=torch.int64, device="cuda")
    hint = torch.zeros(12, dtype=torch.int32, device="cuda")
    vp = lambda t: C.c_void_p(t.data_ptr())
    N.check(N.lib().blpg_topm_hint(vp(scores), net.d_out_pad, 3, vp(m), vp(n), 60, vp(off),
                                   vp(hint), None), "topm")
    torch.cuda.synchronize()
    s = scores.cpu().numpy()[:, :60]
    want = np.concatenate([np.lexsort((np.arange(60), -s[k]))[:4] for k in range(3)])
    assert hint.cpu().numpy().tolist() == want.tolist()

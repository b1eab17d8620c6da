"""The early-exit network's hand-written CUDA training kernels against the
FP64 NumPy oracle (oracle/mlp_oracle.py).  Tolerance: FP32 kernels vs FP64,
|g - g_ref| <= 2e-4 * max|g_ref| + 1e-6 per parameter, loss to 1e-5 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 5)).astype(np.float32)
    y = (x[:, 0] - 0.5 * x[:, 3] + 0.3 * rng.standard_normal(n) > 0).astype(np.float32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return x, y, w


@pytest.mark.parametrize("n", [1, 31, 33, 4096])
def test_gradient_matches_fp64_oracle(song, n):
    from oracle import mlp_oracle as M
    x, y, w = _data(n, n)
    p = song.mlp_init(seed=n)
    for weights in (None, w):
        g, loss = song.mlp_grad(x, y, p, weights)
        l_ref, g_ref = M.loss_and_grad(x, y, p, weights)
        assert abs(loss - l_ref) <= 1e-5 * max(1.0, abs(l_ref))
        tol = 2e-4 * np.abs(g_ref).max() + 1e-6
        assert np.abs(g - g_ref).max() <= tol


def test_forward_matches_fp64_oracle(song):
    from oracle import mlp_oracle as M
    x, _, _ = _data(1000, 7)
    p = song.mlp_init(seed=3)
    z = song.mlp_forward(x, p)
    z_ref, _ = M.forward(x, p)
    assert np.abs(z - z_ref).max() <= 1e-4 * np.abs(z_ref).max() + 1e-5


def test_training_reduces_loss_and_learns(song):
    import torch
    from oracle import mlp_oracle as M
    x, y, _ = _data(50_000, 11)
    p0 = song.mlp_init(seed=0)
    l0, _ = M.loss_and_grad(x, y, p0)
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y).cuda()
    dp = torch.from_numpy(p0.copy()).cuda()
    dl = torch.zeros(5, dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(0)
    perm = torch.cat([torch.randperm(x.shape[0], device="cuda", generator=g) for _ in range(5)]).to(torch.int32)
    song.mlp_train_device(dx.data_ptr(), dy.data_ptr(), 0, x.shape[0], perm.data_ptr(), 5, 1024, 3e-3,
                          dp.data_ptr(), dl.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    p = dp.cpu().numpy()
    l1, _ = M.loss_and_grad(x, y, p)
    assert l1 < 0.5 * l0
    z, _ = M.forward(x, p)
    acc = ((z > 0) == (y > 0.5)).mean()
    assert acc > 0.9
    losses = dl.cpu().numpy()
    assert losses[-1] < losses[0]

"""GPU checks of the surrogate network's hand-written tensor-core kernels:
tcgen05 inference and tcgen05 training GEMMs (forward, backward, split-K
weight gradients) against the FP64 CPU reference (oracle/mlp_ref.py), which is
itself checked by finite differences."""
import numpy as np
import pytest

from oracle import mlp_ref


def test_reference_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.15, 28976)
    x = rng.normal(0, 1, (32, 48))
    t = rng.normal(0, 1, (32, 48))
    _, g = mlp_ref.loss_and_grads(p, x, t, round_bf16=False)
    idx = rng.choice(len(p), 40, replace=False)
    fd = mlp_ref.finite_difference(p, x, t, idx)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-5, atol=1e-9)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    return torch


@pytest.mark.gpu
def test_tcgen05_inference_matches_reference(torch_cuda):
    torch = torch_cuda
    from lqt1_gb300.surrogate import Mlp
    m = Mlp(seed=3)
    p = m.params()
    rng = np.random.default_rng(1)
    n = 128 * 37 + 5                      # partial last tile
    x = rng.normal(0, 1, (n, 48)).astype(np.float32)
    ref = mlp_ref.forward(p, x)["y"]
    xd = torch.from_numpy(x).cuda().to(torch.bfloat16)
    scale = np.abs(ref).max()
    errs = {}
    for layout in (0, 1):
        m.set_layout(layout)
        y = torch.zeros((n, 48), dtype=torch.float32, device="cuda")
        m.infer(xd, y)
        errs[layout] = float(np.abs(y.cpu().numpy() - ref).max() / scale)
    print("relative max error by descriptor layout", errs)
    assert errs[0] < 2e-2, errs


@pytest.mark.gpu
@pytest.mark.parametrize("B", [512, 8192 + 48])
def test_training_gradients_match_reference(torch_cuda, B):
    """Batch 512 (two K slices per weight gradient) and the training batch
    plus a partial row tile (33 K slices of 256 rows; a 48-row tail)."""
    torch = torch_cuda
    from lqt1_gb300.surrogate import Mlp
    m = Mlp(seed=4)
    p = m.params()
    rng = np.random.default_rng(2)
    x = rng.normal(0, 1, (B, 48)).astype(np.float32)
    t = rng.normal(0, 1, (B, 48)).astype(np.float32)
    loss = m.gradients(torch.from_numpy(x).cuda().to(torch.bfloat16), torch.from_numpy(t).cuda())
    g = m.grads()
    lref, gref = mlp_ref.loss_and_grads(p.astype(np.float64), x, t)
    assert abs(loss - lref) / lref < 1e-3
    rel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    assert rel < 1e-2, rel
    np.testing.assert_allclose(g, gref, rtol=5e-2, atol=2e-3 * np.abs(gref).max())


@pytest.mark.gpu
def test_training_reduces_loss(torch_cuda):
    torch = torch_cuda
    from lqt1_gb300.surrogate import Mlp
    rng = np.random.default_rng(5)
    B = 2048
    x = rng.normal(0, 1, (B, 48)).astype(np.float32)
    w = rng.normal(0, 0.3, (48, 48))
    t = np.tanh(x @ w).astype(np.float32)
    xd = torch.from_numpy(x).cuda().to(torch.bfloat16)
    td = torch.from_numpy(t).cuda()
    m = Mlp(seed=6)
    l0 = m.gradients(xd, td)
    for _ in range(300):
        last = m.train_step(xd, td, lr=2e-3)
    assert last < 0.1 * l0, (l0, last)


@pytest.mark.gpu
def test_training_recipe_is_reproducible(torch_cuda):
    """The recipe gives the same bits on every run: the pair generator writes
    each cell's pairs at rows fixed by a counting pass (cell order, not thread
    timing), and the weight gradients add their split-K slices in slice order
    instead of with float atomics."""
    torch = torch_cuda
    from lqt1_gb300 import surrogate as S
    runs = []
    for _ in range(2):
        X, D = S.generate(ncells=2048, cap=60_000, prob=0.02, seed=11, beats_warm=0, beats_record=2,
                          bcl=(400.0, 700.0), nsub=10)
        im, isc, osc = S.fit_norm(X, D, nsample=20_000)
        m = S.Mlp(seed=3)
        m.set_norm(im, isc, osc)
        S.train(m, X, D, epochs=1, batch=2048, seed=5, log=lambda *a: None)
        runs.append((X.cpu().numpy(), D.cpu().numpy(), m.params()))
        m.close()
    (x0, d0, p0), (x1, d1, p1) = runs
    assert len(x0) > 10_000
    np.testing.assert_array_equal(x0, x1)
    np.testing.assert_array_equal(d0, d1)
    np.testing.assert_array_equal(p0, p1)

"""Warm-start MLP kernels: FP64 numpy reference checked by finite differences
(CPU), GPU forward and gradients checked against it (BF16 operands with FP32
accumulation: relative L2 error per parameter block <= 3e-2), and Adam
training reduces the loss."""
import numpy as np
import pytest

from oracle import mlp_oracle


def data(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 16)) * np.linspace(0.5, 2.0, 16) + np.linspace(-1, 1, 16)
    W = rng.normal(size=(16, 3)) / 4.0
    t = np.tanh(x @ W) * np.array([0.01, 0.02, 0.005])
    return x, t


def norm_of(x, t):
    return x.mean(0), x.std(0) + 1e-6, np.abs(t).std(0) + 1e-9


def test_reference_gradient_by_finite_differences():
    rng = np.random.default_rng(1)
    p = rng.normal(size=mlp_oracle.n_params()) * 0.1
    x, t = data(7)
    mean, std, scale = norm_of(x, t)
    _, g = mlp_oracle.loss_grad(p, x, t, mean, std, scale)
    for k in rng.choice(len(p), 40, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        lp, _ = mlp_oracle.loss_grad(p + e, x, t, mean, std, scale)
        lm, _ = mlp_oracle.loss_grad(p - e, x, t, mean, std, scale)
        assert abs((lp - lm) / 2e-6 - g[k]) <= 1e-6 * max(1.0, abs(g[k]))


def blocks():
    out, off = [], 0
    for fi, fo in mlp_oracle.SIZES:
        out.append(slice(off, off + fi * fo))
        off += fi * fo
        out.append(slice(off, off + fo))
        off += fo
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"])
@pytest.mark.parametrize("n", [4096, 1003, 77])
def test_gpu_forward_and_gradients_match_fp64(capi_mod, engine, n):
    """Both GEMM engines; 4096 rows take the 16-byte operand loads and split
    K, 1003 and 77 rows (not a multiple of 8) the element-wise loads and
    ragged tiles."""
    m = capi_mod.Mlp(seed=3)
    m.set_gemm(engine)
    x, t = data(n, seed=2)
    mean, std, scale = norm_of(x, t)
    m.set_normalization(mean, std, scale)
    p = m.params().astype(np.float64)
    y = m.forward(x)
    y_ref = mlp_oracle.forward(p, x, mean, std, scale)
    assert np.linalg.norm(y - y_ref) <= 3e-2 * np.linalg.norm(y_ref)
    loss, g = m.loss_grad(x, t)
    loss_ref, g_ref = mlp_oracle.loss_grad(p, x, t, mean, std, scale)
    assert loss == pytest.approx(loss_ref, rel=3e-2)
    for sl in blocks():
        assert np.linalg.norm(g[sl] - g_ref[sl]) <= 3e-2 * np.linalg.norm(g_ref[sl]) + 1e-12


@pytest.mark.gpu
def test_gpu_gradients_with_empty_split_k_slices(capi_mod):
    """70,001 rows: 136 split-K slices of 576 rows, the last 14 of them
    empty (they contribute zero partial products), and a row count that is
    not a multiple of 8, so every transposed operand takes the element-wise
    loads.  Gradients against the FP64 network."""
    m = capi_mod.Mlp(seed=21)
    x, t = data(70001, seed=22)
    mean, std, scale = norm_of(x, t)
    m.set_normalization(mean, std, scale)
    p = m.params().astype(np.float64)
    loss, g = m.loss_grad(x, t)
    loss_ref, g_ref = mlp_oracle.loss_grad(p, x, t, mean, std, scale)
    assert loss == pytest.approx(loss_ref, rel=3e-2)
    for sl in blocks():
        assert np.linalg.norm(g[sl] - g_ref[sl]) <= 3e-2 * np.linalg.norm(g_ref[sl]) + 1e-12


@pytest.mark.gpu
def test_gpu_gemm_engines_agree(capi_mod):
    """The tcgen05 and mma.sync engines read the same BF16 operands and
    accumulate in FP32 in different orders: gradients agree to 5e-3 per
    parameter block (a BF16 activation may round the other way)."""
    x, t = data(20000, seed=12)
    mean, std, scale = norm_of(x, t)
    grads = []
    for engine in (0, 1):
        m = capi_mod.Mlp(seed=13)
        m.set_gemm(engine)
        m.set_normalization(mean, std, scale)
        grads.append(m.loss_grad(x, t)[1].astype(np.float64))
        m.close()
    for sl in blocks():
        assert np.linalg.norm(grads[0][sl] - grads[1][sl]) <= 5e-3 * np.linalg.norm(grads[1][sl]) + 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 127, 128, 129, 4096, 300001])
def test_tcgen05_inference_matches_fp64_and_gemm_path(capi_mod, n):
    """The fused tcgen05 kernel (path 0) against the FP64 network and the
    per-layer mma.sync path (path 1): same BF16 rounding points, so the two
    GPU paths agree to FP32 accumulation-order noise; ragged last tiles."""
    m = capi_mod.Mlp(seed=9)
    x, t = data(n, seed=11)
    mean, std, scale = norm_of(x, t) if n > 1 else (np.zeros(16), np.ones(16), np.ones(3))
    m.set_normalization(mean, std, scale)
    p = m.params().astype(np.float64)
    y_tc = m.forward(x, path=0)
    y_layers = m.forward(x, path=1)       # per-layer tcgen05 GEMMs
    m.set_gemm(m.GEMM_MMA_SYNC)
    y_mm = m.forward(x, path=1)
    assert np.isfinite(y_tc).all()
    k = min(n, 4096)
    y_ref = mlp_oracle.forward(p, x[:k], mean, std, scale)
    assert np.linalg.norm(y_tc[:k] - y_ref) <= 3e-2 * np.linalg.norm(y_ref) + 1e-6
    assert np.abs(y_tc - y_mm).max() <= 2e-2 * np.abs(y_mm).max() + 1e-6
    assert np.abs(y_layers - y_mm).max() <= 2e-2 * np.abs(y_mm).max() + 1e-6


@pytest.mark.gpu
def test_gpu_adam_training_reduces_loss(capi_mod):
    m = capi_mod.Mlp(seed=4)
    x, t = data(50000, seed=5)
    mean, std, scale = norm_of(x, t)
    m.set_normalization(mean, std, scale)
    m.set_dataset(x, t)
    l0, _ = m.loss_grad(x[:8192], t[:8192])
    m.train(400, 8192, 1e-3, seed=1)
    l1, _ = m.loss_grad(x[:8192], t[:8192])
    assert l1 < 0.2 * l0


@pytest.mark.gpu
def test_gpu_adam_steps_against_fp64_adam(capi_mod):
    """Three Adam steps of the GPU's training against the FP64 restatement
    of Adam (mlp_oracle.adam_update) driven by the same gradients.  The
    dataset is one row repeated, so every random batch is that row and a
    training step's gradient is that row's gradient, which sbs_mlp_loss_grad
    returns from the same kernels (the gradients themselves are checked
    against FP64 above).  Moves of parameters whose gradient is below 1e-6
    depend on Adam's epsilon and on rounding; they stay within Adam's bound
    on a step, lr (1 - b1) / sqrt(1 - b2)."""
    from oracle import mlp_oracle
    m = capi_mod.Mlp(seed=9)
    x1, t1 = data(1, seed=10)
    xs, ts = data(4096, seed=11)
    m.set_normalization(*norm_of(xs, ts))
    m.set_dataset(np.repeat(x1, 4096, axis=0), np.repeat(t1, 4096, axis=0))
    lr = 1e-3
    p = m.params().astype(np.float64)
    mom1 = np.zeros_like(p)
    mom2 = np.zeros_like(p)
    for k in range(1, 4):
        _, g = m.loss_grad(x1, t1)
        g = g.astype(np.float64)
        m.train(1, 1024, lr, seed=k)
        ref, mom1, mom2 = mlp_oracle.adam_update(p, g, mom1, mom2, k, lr)
        got = m.params().astype(np.float64)
        big = np.abs(g) > 1e-6
        assert big.sum() > 10000
        assert np.abs((got - p)[big] - (ref - p)[big]).max() <= 2e-3 * lr
        assert np.abs(got - p).max() <= 3.2 * lr    # Adam's step bound, lr (1 - b1) / sqrt(1 - b2)
        p = got


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"])
def test_gpu_training_is_reproducible(capi_mod, engine):
    """Two trainings from the same seeds end with identical parameters: the
    split-K weight gradients add their K slices in a fixed order."""
    x, t = data(40000, seed=6)
    mean, std, scale = norm_of(x, t)
    out = []
    for _ in range(2):
        m = capi_mod.Mlp(seed=7)
        m.set_gemm(engine)
        m.set_normalization(mean, std, scale)
        m.set_dataset(x, t)
        m.train(50, 32768, 1e-3, seed=3)    # batches large enough to split K
        out.append(m.params())
        m.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
def test_gemm_engine_argument(capi_mod):
    m = capi_mod.Mlp(seed=1)
    with pytest.raises(capi_mod.SbsError):
        m.set_gemm(2)
    with pytest.raises(capi_mod.SbsError):
        m.set_gemm(-1)
    m.set_gemm(m.GEMM_MMA_SYNC)
    m.set_gemm(m.GEMM_TC)
    m.close()

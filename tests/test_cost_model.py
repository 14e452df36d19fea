"""Learned cost model: BF16 packing (CPU), and on the GPU the forward pass and the
gradients of the library's own kernels against a float64 NumPy restatement,
training, and what the model gains over the plain bound."""
import numpy as np
import pytest

from bsbolt_gb300 import cost_model as cm
from bsbolt_gb300 import synth

F, H = cm.F, cm.H


def test_bf16_rounding_matches_definition():
    x = np.array([1.0, 1.00390625, 1.0078125, -3.3, 1e-3, 65504.0], np.float32)
    bits = cm.bf16_bits(x)
    back = cm.bf16_value(bits)
    assert np.all(np.abs(back - x) <= np.abs(x) * 2.0 ** -8)
    assert cm.bf16_bits(np.array([1.00390625], np.float32))[0] == 0x3F80   # tie rounds to even


def np_reference(params_bf, b, feat, target):
    """float64 forward/backward with the BF16-rounded weights the kernels use."""
    w1 = params_bf[: H * F].reshape(H, F).astype(np.float64)
    w2 = params_bf[H * F: H * F + H * H].reshape(H, H).astype(np.float64)
    w3 = params_bf[H * F + H * H:].astype(np.float64)
    b1, b2, b3 = b[:H].astype(np.float64), b[H:2 * H].astype(np.float64), float(b[2 * H])
    x = feat.astype(np.float64)
    a1 = x @ w1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ w2.T + b2
    h2 = np.maximum(a2, 0)
    y = h2 @ w3 + b3
    n = len(x)
    r = y - target
    dy = 2 * r / n
    g_w3 = h2.T @ dy
    d2 = (dy[:, None] * w3[None, :]) * (a2 > 0)
    g_w2 = d2.T @ h1
    g_b2 = d2.sum(0)
    d1 = (d2 @ w2) * (a1 > 0)
    g_w1 = d1.T @ x
    g_b1 = d1.sum(0)
    g_b3 = dy.sum()
    grad = np.concatenate([g_w1.ravel(), g_w2.ravel(), g_w3, g_b1, g_b2, [g_b3]])
    return y, grad, float(np.mean(r * r))


@pytest.mark.gpu
def test_forward_and_gradients_match_float64(gpu_ctx):
    torch = pytest.importorskip("torch")
    model = cm.CostModel(gpu_ctx, seed=3)
    rng = np.random.Generator(np.random.PCG64(9))
    feat = rng.uniform(0, 1, (3000, F)).astype(np.float32)
    target = rng.uniform(4, 10, 3000).astype(np.float32)
    df, dt = torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda()
    wb, fb = model.weights_bits()
    y_ref, g_ref, loss_ref = np_reference(cm.bf16_value(wb), fb, feat, target)
    y = model.forward(df).cpu().numpy()
    assert np.allclose(y, y_ref, rtol=1e-5, atol=1e-4)
    g = model.backward(df, dt).cpu().numpy()
    assert np.allclose(g[: cm.N_PARAMS], g_ref, rtol=1e-3, atol=1e-6), \
        np.max(np.abs(g[: cm.N_PARAMS] - g_ref))
    assert abs(g[cm.N_PARAMS] - loss_ref) <= 1e-4 * max(1.0, loss_ref)
    # deterministic: the same batch gives the same gradient bits
    g2 = model.backward(df, dt).cpu().numpy()
    assert np.array_equal(g, g2)


@pytest.mark.gpu
def test_model_learns_cells_better_than_bound(gpu_ctx):
    """Trained on logged cells of one job set, ranked on another: beats the plain bound."""
    torch = pytest.importorskip("torch")
    from bsbolt_gb300 import extend
    mat = synth.fill_scmat(1, 4)
    sets = []
    for seed in (101, 102):
        jobs, seq = synth.ksw_jobs(120000, seed=seed)
        _, cells = extend.ksw_extend2_batch(gpu_ctx, jobs, seq, mat, 6, 1, 6, 1, 100, want_cells=True)
        dj = torch.from_numpy(jobs.view(np.uint8).reshape(-1).copy()).cuda()
        ds = torch.from_numpy(seq).cuda()
        sets.append((jobs, seq, cells, dj, ds))
    model = cm.CostModel(gpu_ctx, seed=5)
    jobs, seq, cells, dj, ds = sets[0]
    feat = model.features(dj, len(jobs), ds, len(seq))
    target = torch.from_numpy(np.log1p(cells).astype(np.float32)).cuda()
    losses = model.train(feat, target, epochs=6)
    assert losses[-1] < losses[0]
    jobs, seq, cells, dj, ds = sets[1]
    pred = model.forward(model.features(dj, len(jobs), ds, len(seq))).cpu().numpy()
    bound = synth.cells_upper_bound(jobs).astype(np.float64)
    rho_model = cm.spearman(pred, cells)
    rho_bound = cm.spearman(bound, cells)
    assert rho_model > rho_bound, (rho_model, rho_bound)
    assert cm.mape(np.expm1(pred), cells) < cm.mape(cm.calibrated_bound(bound, cells), cells)

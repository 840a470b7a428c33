"""GPU checks of the conflict predictor's hand-written kernels against the float64 oracle
(oracle/mlp_oracle.py): forward probabilities, the gradient of the mean binary cross-entropy,
the Adam update, and that training learns a separable labelling.

Tolerances (fp32 accumulation of bf16 weights against float64 on the same bf16 weights):
probabilities 2e-5 absolute for 0/1 features (2e-4 for dense features, where a layer-1
activation may round to the neighbouring bf16 value); gradients 1e-4 relative to the
gradient's max-norm, per entry."""
import numpy as np
import pytest

import csmv_gb300 as cg
import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.cuda()


def _features(rng, n, dense=False):
    if dense:  # arbitrary bf16 values exercise the datapath beyond 0/1 indicators
        x = mo.bf16_round(rng.normal(0, 1, (n, mo.IN)).astype(np.float32))
    else:
        x = (rng.random((n, mo.IN)) < 0.25).astype(np.float32)
    return x, mo.bf16_bits(x).view(np.int16)


@pytest.mark.parametrize("n,dense", [(1, False), (63, True), (1000, False), (70000, True)])
def test_forward_and_gradient_match_oracle(n, dense):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    x, xb = _features(rng, n, dense)
    y = (rng.random(n) < 0.4).astype(np.float32)
    with cg.Mlp(seed=7) as m:
        params = m.params()
        params[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.1, mo.HID)  # nonzero biases too
        params[mo.OFF_B3] = 0.3
        m.set_params(params)
        dx, dy = _dev(torch, xb), _dev(torch, y)
        dp = torch.zeros(n, dtype=torch.float32, device="cuda")
        m.forward(n, dx.data_ptr(), dp.data_ptr())
        p_gpu = dp.cpu().numpy()
        loss = m.grad(n, dx.data_ptr(), dy.data_ptr())
        g_gpu = m.grads().astype(np.float64)
    p_ref, _ = mo.forward(params, x)
    # binary features (the scheduler's) give exactly representable layer-1 sums; with dense
    # inputs an fp32 sum can land on the other side of a bf16 rounding boundary than the float64
    # one, moving one activation by one bf16 step (2^-8 relative) and p by up to ~1e-4
    np.testing.assert_allclose(p_gpu, p_ref, rtol=0, atol=2e-4 if dense else 2e-5)
    if dense:
        assert np.mean(np.abs(p_gpu - p_ref) > 2e-5) < 1e-3
    loss_ref, g_ref = mo.loss_and_grads(params, x, y)
    assert abs(loss - loss_ref) < 1e-4 * max(1.0, abs(loss_ref))
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g_gpu, g_ref, rtol=0, atol=1e-4 * scale)


def test_adam_step_matches_oracle():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    x, xb = _features(rng, 512)
    y = (rng.random(512) < 0.5).astype(np.float32)
    with cg.Mlp(seed=9) as m:
        p0 = m.params().astype(np.float64)
        dx, dy = _dev(torch, xb), _dev(torch, y)
        mm = np.zeros_like(p0)
        vv = np.zeros_like(p0)
        for step in (1, 2):
            m.grad(512, dx.data_ptr(), dy.data_ptr())
            g = m.grads().astype(np.float64)
            m.adam_step(1e-3)
            p0, mm, vv = mo.adam(p0, g, mm, vv, step, 1e-3)
            np.testing.assert_allclose(m.params(), p0, rtol=0, atol=1e-6)
            assert not m.grads().any()  # the step clears the accumulator


def test_training_learns_a_separable_labelling():
    """y = x[3] or (x[10] and x[40]): a few hundred Adam steps drive the loss down and the
    predictions to > 97 % accuracy on fresh samples."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)

    def batch(n):
        x, xb = _features(rng, n)
        y = ((x[:, 3] > 0) | ((x[:, 10] > 0) & (x[:, 40] > 0))).astype(np.float32)
        return x, xb, y

    with cg.Mlp(seed=1) as m:
        first = None
        for it in range(300):
            _, xb, y = batch(4096)
            dx, dy = _dev(torch, xb), _dev(torch, y)
            loss = m.grad(4096, dx.data_ptr(), dy.data_ptr())
            first = loss if first is None else first
            m.adam_step(3e-3)
        _, xb, y = batch(20000)
        dx = _dev(torch, xb)
        dp = torch.zeros(20000, dtype=torch.float32, device="cuda")
        m.forward(20000, dx.data_ptr(), dp.data_ptr())
        acc = float(((dp.cpu().numpy() > 0.5) == (y > 0.5)).mean())
    assert loss < 0.25 * first and acc > 0.97, (first, loss, acc)

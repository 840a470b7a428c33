"""CPU checks of the network oracle: bf16 rounding and the analytic gradient against finite
differences (float64)."""
import numpy as np

import mlp_oracle as mo


def test_bf16_rounding_known_values():
    a = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5, 3.140625, 1e-40], np.float32)
    r = mo.bf16_round(a)
    # 1 + 2^-8 is a tie -> even (1.0); 1 + 3*2^-9 rounds up to 1 + 2^-7
    assert list(r[:4]) == [1.0, 1.0, 1.0078125, 1.0078125]
    assert r[4] == -2.5 and r[5] == 3.140625
    assert mo.bf16_bits(np.array([1.0], np.float32))[0] == 0x3F80


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = np.zeros(mo.N_PARAMS, np.float64)
    p[mo.OFF_W1:mo.OFF_B1] = rng.normal(0, 0.2, mo.IN * mo.HID)
    p[mo.OFF_W2:mo.OFF_B2] = rng.normal(0, 0.1, mo.HID * mo.HID)
    p[mo.OFF_W3:mo.OFF_B3] = rng.normal(0, 0.1, mo.HID)
    p[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.1, mo.HID)
    x = (rng.random((16, mo.IN)) < 0.3).astype(np.float64)
    y = (rng.random(16) < 0.5).astype(np.float64)

    # differentiate the float64 function (no bf16 rounding) by central differences
    def loss64(q):
        w1 = q[mo.OFF_W1:mo.OFF_B1].reshape(mo.IN, mo.HID)
        w2 = q[mo.OFF_W2:mo.OFF_B2].reshape(mo.HID, mo.HID)
        h1 = np.maximum(x @ w1 + q[mo.OFF_B1:mo.OFF_W2], 0)
        h2 = np.maximum(h1 @ w2 + q[mo.OFF_B2:mo.OFF_W3], 0)
        z = h2 @ q[mo.OFF_W3:mo.OFF_B3] + q[mo.OFF_B3]
        return np.mean(np.maximum(z, 0) - y * z + np.log1p(np.exp(-np.abs(z))))

    # the oracle with bf16-exact weights equals the float64 function
    p = mo.bf16_round(p.astype(np.float32)).astype(np.float64)
    _, g = mo.loss_and_grads(p.astype(np.float32), x, y, round_act=False)
    idx = np.concatenate([rng.integers(mo.OFF_W1, mo.OFF_B1, 20), rng.integers(mo.OFF_W2, mo.OFF_B2, 20),
                          np.arange(mo.OFF_W3, mo.OFF_W3 + 5), [mo.OFF_B3], [mo.OFF_B1 + 3]])
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (loss64(p + e) - loss64(p - e)) / 2e-6
        assert abs(fd - g[i]) < 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])

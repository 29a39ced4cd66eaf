"""CPU checks of the learned-start-value network's restatement
(oracle/mlp.py): its analytic gradient against central differences of its
own loss, the bfloat16 rounding, and Adam's first step."""
import numpy as np

from oracle import mlp


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, 0.3, mlp.N_PARAMS)
    p[mlp.OFF_MEAN:mlp.OFF_MEAN + 5] = rng.normal(0, 0.2, 5)
    p[mlp.OFF_INVSTD:mlp.OFF_INVSTD + 5] = rng.uniform(0.5, 1.5, 5)
    return p


def test_gradient_matches_central_differences():
    rng = np.random.default_rng(1)
    p = _params()
    feat = rng.normal(0, 1, (32, 5)).astype(np.float32)
    lab = rng.normal(0, 1, 32)
    loss, g = mlp.loss_and_grad(p, feat, lab)
    idx = np.concatenate([rng.choice(np.arange(mlp.OFF_W1, mlp.N_PARAMS), 60, replace=False),
                          [mlp.OFF_B3, mlp.OFF_W1, mlp.OFF_B2 + 3]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.loss_and_grad(pp, feat, lab)[0] - mlp.loss_and_grad(pm, feat, lab)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    assert np.all(g[:mlp.OFF_W1] == 0.0)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -8, -3.0e-3, 65504.0, 0.0],
                 dtype=np.float32)
    r = mlp.bf16(x)
    # ties to even: 1 + 2^-8 -> 1; 1 + 2^-7 + 2^-8 -> 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert abs(r[3] / -3.0e-3 - 1) < 2 ** -8
    assert r[4] == 65536.0 and r[5] == 0.0


def test_adam_first_step_is_signed_learning_rate():
    p = _params(2)
    g = np.linspace(-1, 1, mlp.N_PARAMS) + 1e-3
    q, m1, m2 = mlp.adam_step(p, g, np.zeros_like(g), np.zeros_like(g), 1, 1e-3)
    d = (p - q)[mlp.OFF_W1:]
    np.testing.assert_allclose(d, 1e-3 * np.sign(g[mlp.OFF_W1:]), rtol=1e-4)
    assert np.all(q[:mlp.OFF_W1] == p[:mlp.OFF_W1])


def test_bf16_operands_stay_close_to_float64():
    rng = np.random.default_rng(3)
    p = _params(4)
    feat = rng.normal(0, 1, (256, 5)).astype(np.float32)
    y64 = mlp.forward(p, feat)
    y16 = mlp.forward(p, feat, bf16_operands=True)
    assert np.max(np.abs(y64 - y16)) < 0.05 * np.max(np.abs(y64))

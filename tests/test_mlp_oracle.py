"""CPU checks of the surrogate's oracle (oracle/mlp_oracle.py): its exact
backward pass against central finite differences, its bf16-rounded pass
against the exact one (plain and energy-weighted loss), the bf16 rounding
itself, the energy weight and the feature rotation."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _params(seed, scale3=1.0):
    rng = np.random.default_rng(seed)
    w = np.zeros(mo.NPARAM, np.float32)
    w[mo.OFF_W1:mo.OFF_B1] = rng.standard_normal(mo.OFF_B1 - mo.OFF_W1) * np.sqrt(2.0 / 1341)
    w[mo.OFF_B1:mo.OFF_W2] = 0.01 * rng.standard_normal(mo.HID)
    w[mo.OFF_W2:mo.OFF_B2] = rng.standard_normal(mo.HID * mo.HID) * np.sqrt(2.0 / mo.HID)
    w[mo.OFF_W3:mo.OFF_B3] = scale3 * rng.standard_normal(mo.FPAD * mo.HID) * np.sqrt(1.0 / mo.HID)
    return w


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, mo.FPAD), np.float32)
    X[:, :1341] = rng.standard_normal((n, 1341))
    T = np.zeros((n, mo.FPAD), np.float32)
    T[:, :1332] = 0.3 * rng.standard_normal((n, 1332))
    return X, T


@pytest.mark.parametrize("weighted", [False, True])
def test_exact_gradient_vs_finite_differences(weighted):
    w = _params(0).astype(np.float64)
    X, T = _batch(8, 1)
    _, g = mo.loss_and_grad_exact(w, X, T, 1332, weighted)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.integers(a, b, 4) for a, b in ((mo.OFF_W1, mo.OFF_B1), (mo.OFF_B1, mo.OFF_W2),
                                                             (mo.OFF_W2, mo.OFF_B2), (mo.OFF_B2, mo.OFF_W3),
                                                             (mo.OFF_W3, mo.OFF_B3), (mo.OFF_B3, mo.OFF_B3 + 1332))])

    def loss(v):
        return mo.loss_and_grad_exact(v, X, T, 1332, weighted)[0]

    h = 1e-4
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (loss(wp) - loss(wm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


@pytest.mark.parametrize("weighted", [False, True])
def test_rounded_gradient_close_to_exact(weighted):
    w = _params(3, scale3=10.0)
    X, T = _batch(64, 4)
    l1, g1 = mo.loss_and_grad(w, X, T, 1332, weighted)
    l2, g2 = mo.loss_and_grad_exact(w, mo.bf16(X), mo.bf16(T), 1332, weighted)
    assert abs(l1 - l2) < 2e-2 * l2
    assert np.linalg.norm(g1 - g2) < 5e-2 * np.linalg.norm(g2)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-39, 65504.0], np.float32)
    b = mo.bf16(x)
    assert b[0] == 1.0 and b[1] == 1.0  # tie to even
    assert b[2] == np.float32(1.0078125)
    assert b[3] == -2.5
    assert (mo.bf16_bits(np.float32(1.0)) == 0x3F80).all()


def test_feature_rotation():
    pm, om = 36, 37
    th = (np.arange(1, pm + 1) - 0.5 * (pm + 1)) * (2 * np.pi / pm)
    dth = 2 * np.pi / pm
    e = np.zeros((1, pm, om), np.float32)
    e[0, 7, 3] = 1.0  # energy at direction 7, frequency 3
    X, s = mo.features(e, np.array([th[7]]), np.array([10.0]), np.array([0.3]), np.array([100.0]), 30.0,
                       np.array([0.0]), np.array([0.0]), np.array([1.2e-3]), np.array([0.0]), th, dth)
    assert s[0] == 7
    # the wind-aligned bin (p' = 0) of frequency 3 holds the energy
    k = 3 * pm + 0
    assert abs(X[0, k] - (np.log(1.0 + 1e-15) + 15.0) / 8.0) < 1e-6
    assert abs(X[0, 1332 + 1]) < 1e-6  # wind exactly on a bin: no offset


def test_energy_weight_ramp():
    # input features of bins at e = 1e-12, 1e-9, 1e-7, 1e-5, 1
    e = np.array([1e-12, 1e-9, 1e-7, 1e-5, 1.0])
    x = (np.log(e + mo.EPS) - mo.LN_C0) / mo.LN_C1
    w = mo.energy_weight(x)
    assert w[0] == np.float32(mo.WMIN) and abs(w[1] - mo.WMIN) < 1e-5
    assert abs(w[2] - 0.5) < 1e-4 and w[3] == pytest.approx(1.0, abs=1e-5) and w[4] == 1.0

"""CPU checks of the numpy restatement of the learned smoother's network
(the gradient oracle the GPU kernels are compared with)."""
import numpy as np

from oracle import mlp_oracle as mo


def _params(seed=0):
    rng = np.random.default_rng(seed)
    P = np.zeros(mo.N_PARAMS)
    W1, b1, W2, b2, W3, b3 = [a for a in mo.unpack(P)]
    P[mo.OFF_W1:mo.OFF_B1] = (rng.uniform(-1, 1, (mo.N_H, mo.N_IN_PAD)) / np.sqrt(mo.N_IN)).ravel()
    P[mo.OFF_W1:mo.OFF_B1].reshape(mo.N_H, mo.N_IN_PAD)[:, mo.N_IN:] = 0
    P[mo.OFF_B1:mo.OFF_W2] = rng.uniform(-0.1, 0.1, mo.N_H)
    P[mo.OFF_W2:mo.OFF_B2] = rng.uniform(-1, 1, mo.N_H * mo.N_H) / 16.0
    P[mo.OFF_B2:mo.OFF_W3] = rng.uniform(-0.1, 0.1, mo.N_H)
    W3v = rng.uniform(-1, 1, (mo.N_OUT_PAD, mo.N_H)) / 16.0
    W3v[mo.N_OUT:] = 0
    P[mo.OFF_W3:mo.OFF_B3] = W3v.ravel()
    P[mo.OFF_B3:mo.OFF_B3 + mo.N_OUT] = rng.uniform(-0.1, 0.1, mo.N_OUT)
    return P


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 0.0], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[3] == -2.5 and r[4] == 0.0
    assert r[1] == 1.0            # tie to even
    assert r[2] == 1.0 + 2 ** -7  # rounds up


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    P = _params(1)
    X = rng.standard_normal((6, mo.N_IN))
    T = rng.standard_normal((6, mo.N_OUT))
    loss, G = mo.loss_grad(P, X, T, round_bf16=False)
    assert abs(loss - mo.loss_only_fp64(P, X, T)) < 1e-12
    idx = [mo.OFF_W1 + 5, mo.OFF_W1 + 400 * 7 + 123, mo.OFF_B1 + 3, mo.OFF_W2 + 999,
           mo.OFF_B2 + 17, mo.OFF_W3 + 256 * 4 + 9, mo.OFF_B3 + 84]
    for i in idx:
        h = 1e-6
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (mo.loss_only_fp64(Pp, X, T) - mo.loss_only_fp64(Pm, X, T)) / (2 * h)
        assert abs(fd - G[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, G[i])
    # padding gets no gradient
    assert np.all(G[mo.OFF_W1:mo.OFF_B1].reshape(mo.N_H, mo.N_IN_PAD)[:, mo.N_IN:] == 0)
    assert np.all(G[mo.OFF_B3 + mo.N_OUT:] == 0)

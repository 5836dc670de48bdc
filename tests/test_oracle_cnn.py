"""CPU checks of the network / flexible-PCG oracle (oracle/cnn_ref.py)."""
import numpy as np
import pytest

from oracle import cnn_ref


def _rand_c(g, *shape):
    return g.standard_normal(shape) + 1j * g.standard_normal(shape)


def test_gradient_matches_finite_differences():
    ch = (2, 4, 3, 2)
    g = np.random.Generator(np.random.PCG64(3))
    theta = cnn_ref.init_params(7, ch).astype(np.float64)
    theta[-1] = 0.3
    r = _rand_c(g, 2, 9, 7)
    e = _rand_c(g, 2, 9, 7)
    L, grad = cnn_ref.loss_and_grad(theta, r, e, 1, ch)
    idx = np.concatenate([g.choice(len(theta) - 1, 25, replace=False), [len(theta) - 1]])
    for i in idx:
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (cnn_ref.loss_and_grad(tp, r, e, 1, ch)[0] - cnn_ref.loss_and_grad(tm, r, e, 1, ch)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_positive_homogeneity():
    # bias-free ReLU network with input normalisation: net(c r) = c net(r) for c > 0
    g = np.random.Generator(np.random.PCG64(4))
    theta = cnn_ref.init_params(1)
    r = _rand_c(g, 1, 12, 10)
    z1 = cnn_ref.forward(theta, r)
    z2 = cnn_ref.forward(theta, 3.5 * r)
    np.testing.assert_allclose(z2, 3.5 * z1, rtol=1e-10, atol=1e-12)
    assert np.all(cnn_ref.forward(theta, np.zeros_like(r)) == 0)


def test_fcg_identity_is_cg():
    g = np.random.Generator(np.random.PCG64(5))
    n = 40
    Q = _rand_c(g, n, n)
    H = Q.conj().T @ Q + 0.5 * np.eye(n)
    b = _rand_c(g, n)
    xs = np.linalg.solve(H + 0.1 * np.eye(n), b)
    x, res, err = cnn_ref.fcg_ref(lambda v: H @ v, b, lambda r: r, 60, lam=0.1, gtruth=xs)
    assert err[-1] < 1e-8
    # an exact preconditioner converges in one step
    Hi = np.linalg.inv(H + 0.1 * np.eye(n))
    x1, _, err1 = cnn_ref.fcg_ref(lambda v: H @ v, b, lambda r: Hi @ r, 1, lam=0.1, gtruth=xs)
    assert err1[-1] < 1e-10


def test_adam_step_matches_closed_form_first_step():
    th = np.array([1.0, -2.0, 0.5])
    gr = np.array([0.1, -0.3, 0.0])
    t2, m, v = cnn_ref.adam_step(th, gr, np.zeros(3), np.zeros(3), 1, 0.01)
    # first step moves each nonzero-gradient weight by lr * sign(g)
    np.testing.assert_allclose(t2[:2], th[:2] - 0.01 * np.sign(gr[:2]), rtol=1e-6)
    assert t2[2] == th[2]


def test_cosine_loss_gradient_and_scale_invariance():
    ch = (2, 4, 3, 2)
    g = np.random.Generator(np.random.PCG64(8))
    theta = cnn_ref.init_params(9, ch).astype(np.float64)
    theta[-1] = 0.2
    r = _rand_c(g, 2, 9, 8)
    e = _rand_c(g, 2, 9, 8)
    L, grad = cnn_ref.loss_and_grad(theta, r, e, 1, ch, kind="cos")
    assert 0.0 <= L <= 1.0
    for i in list(g.choice(len(theta) - 1, 20, replace=False)) + [len(theta) - 1]:
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (cnn_ref.loss_and_grad(tp, r, e, 1, ch, kind="cos")[0]
              - cnn_ref.loss_and_grad(tm, r, e, 1, ch, kind="cos")[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])
    # a complex rescaling of the target leaves the loss unchanged
    L2, _ = cnn_ref.loss_and_grad(theta, r, (2 - 3j) * e, 1, ch, kind="cos")
    assert abs(L2 - L) < 1e-12


def test_extended_forward_equals_layered_forward_in_the_interior():
    # away from the border (farther than the receptive-field radius) the two agree
    ch = (2, 4, 4, 2)
    g = np.random.Generator(np.random.PCG64(12))
    theta = cnn_ref.init_params(13, ch)
    r = _rand_c(g, 1, 16, 14)
    a = cnn_ref.forward(theta, r, ch, linear=True)
    b = cnn_ref.forward_extended(theta, r, ch, linear=True)
    L = len(ch) - 1
    np.testing.assert_allclose(a[:, L:-L, L:-L], b[:, L:-L, L:-L], rtol=1e-10, atol=1e-12)
    assert np.abs(a - b).max() > 1e-6     # and differ next to it

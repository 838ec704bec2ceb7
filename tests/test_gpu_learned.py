"""Learned quadrature of near-singular pairs: the network's GPU gradients
against a float64 numpy restatement, training, what the trained network gains
over the reference adaptive rule on held-out random pairs, and a mesh assembled
with the learned rules against the FP64 oracle."""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, BemRegion, qlearn as Q

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------- numpy MLP
def _unpack(w):
    H, o = 64, 0
    out = []
    for fi, fo in ((Q.NF, H), (H, H), (H, H), (H, Q.NC)):
        W = w[o:o + fo * fi].reshape(fo, fi)
        o += fo * fi
        b = w[o:o + fo]
        o += fo
        out.append((W, b))
    assert o == w.size
    return out


def _np_loss_grad(w, X, Y, V):
    """Mean over valid samples and outputs of (f(x) - y)^2 and its gradient, float64."""
    w = w.astype(np.float64)
    layers = _unpack(w)
    acts = [X.astype(np.float64)]
    for W, b in layers[:-1]:
        acts.append(np.tanh(acts[-1] @ W.T + b))
    W4, b4 = layers[-1]
    out = acts[-1] @ W4.T + b4
    e = (out - Y) * V[:, None]
    cnt = X.shape[0] * Q.NC
    loss = (e ** 2).sum() / cnt
    d = 2.0 * e / cnt
    grads = []
    for li in range(3, -1, -1):
        W, b = layers[li]
        grads.append((d.T @ acts[li], d.sum(0)))
        if li > 0:
            d = (d @ W) * (1.0 - acts[li] ** 2)
    g = []
    for gw, gb in reversed(grads):
        g += [gw.ravel(), gb]
    return loss, np.concatenate(g)


def test_mlp_gradient_matches_cpu():
    rng = np.random.default_rng(3)
    w = Q.init_weights(5)
    w += rng.normal(scale=0.05, size=w.size).astype(np.float32)
    n = 300
    X = rng.normal(size=(n, Q.NF)).astype(np.float32)
    Y = rng.normal(scale=3.0, size=(n, Q.NC)).astype(np.float32)
    V = (rng.uniform(size=n) < 0.8).astype(np.int32)
    loss, g = Q.loss_grad(w, X, Y, V)
    lref, gref = _np_loss_grad(w, X, Y, V)
    assert abs(loss - lref) / lref < 1e-5
    assert np.abs(g - gref).max() / np.abs(gref).max() < 1e-4
    out = Q.forward(w, X)
    layers = _unpack(w.astype(np.float64))
    a = X.astype(np.float64)
    for W, b in layers[:-1]:
        a = np.tanh(a @ W.T + b)
    assert np.abs(out - (a @ layers[-1][0].T + layers[-1][1])).max() < 1e-4


@pytest.fixture(scope="module")
def trained():
    e, p, k, kc = Q.random_pairs(7500, seed=11, kernel=0)
    F, Y, C, V = Q.label_pairs(e, p, k, kc)
    w = Q.init_weights(1)
    hist = Q.train(w, F[:6000], Y[:6000], V[:6000], steps=3000, batch=2048, lr=2e-3, seed=4)
    return w, hist, (F[6000:], Y[6000:], C[6000:], V[6000:])


def test_training_reduces_loss(trained):
    w, hist, _ = trained
    assert np.all(np.isfinite(hist))
    assert hist[-100:].mean() < 0.02 * hist[:10].mean()


def test_learned_rule_gains_over_reference_rule(trained):
    """Held-out pairs, against the converged integral: at the reference rule's
    default tolerance (1e-6) the learned choice meets 1e-6 far more often at
    about the same number of points, and it reaches the reliability of the
    reference rule at 1e-8 with fewer points."""
    w, _, (F, Y, C, V) = trained
    P = Q.forward(w, F)
    m = (V == 1) & (C[:, :Q.NT].min(1) > 0)
    ar = np.arange(len(F))
    ref6, ref8 = Q.REF_DEFAULT, Q.REF_DEFAULT + 2
    rel_ref6, pts_ref6 = (Y[m, ref6] <= -6).mean(), C[m, ref6].mean()
    rel_ref8, pts_ref8 = (Y[m, ref8] <= -6).mean(), C[m, ref8].mean()
    c = Q.choose(P, C, -6.5)
    rel_l, pts_l = (Y[ar, c][m] <= -6).mean(), C[ar, c][m].mean()
    assert rel_l > rel_ref6 + 0.08 and pts_l < 1.15 * pts_ref6, (rel_l, pts_l, rel_ref6, pts_ref6)
    c = Q.choose(P, C, -7.5)
    rel_l, pts_l = (Y[ar, c][m] <= -6).mean(), C[ar, c][m].mean()
    assert rel_l > rel_ref8 - 0.01 and pts_l < 0.92 * pts_ref8, (rel_l, pts_l, rel_ref8, pts_ref8)


def test_learned_quadrature_on_a_mesh(trained, oracle):
    """Slab with near-singular pairs across its thickness: the learned rules
    replace most adaptive pairs' rules; against the converged assembly
    (qsi_relative_error 1e-10) and its solution, the learned assembly is as
    accurate as the reference rule's (which is the oracle's), and restoring the
    reference rule gives the reference assembly back exactly."""
    w, _, _ = trained
    d = M.slab(4, 1)
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.02)
    om = float(M.omega_from_a0([0.5], mat)[0])
    Rc = BemRegion(d, qsi_relative_error=1e-10)
    Ac, bc = Rc.build_lse_harela(mat, om)
    Rc.close()
    R = BemRegion(d)
    A0, b0 = R.build_lse_harela(mat, om)
    nl = R.set_learned_quadrature(w, log10_tol=-7.0)
    assert nl > 0.5 * R.stats()["pairs_adaptive"]
    A1, b1 = R.build_lse_harela(mat, om)
    scale = np.abs(Ac).max()
    e0, e1 = np.abs(A0 - Ac).max() / scale, np.abs(A1 - Ac).max() / scale
    assert 0 < np.abs(A1 - A0).max() and e1 < 2.0 * e0 + 1e-9, (e0, e1)
    # solutions: the learned rules' error against the converged solution is no
    # worse than the reference rule's (the slab's condition number, 2.8e4,
    # amplifies both quadrature errors alike)
    from multifebe_gb300 import solve_lse

    def sol(A, b):
        x, _ = solve_lse(A.copy(order="F"), b.copy())
        return x.ravel()
    xc, x0, x1 = sol(Ac, bc), sol(A0, b0), sol(A1, b1)
    s0 = np.abs(x0 - xc).max() / np.abs(xc).max()
    s1 = np.abs(x1 - xc).max() / np.abs(xc).max()
    assert s1 < 2.0 * s0 + 1e-9, (s0, s1)
    # the reference-rule assembly is the oracle's
    P = oracle.Problem(d)
    Ao, bo = P.assemble_harela(mat, om)
    assert np.abs(A0 - Ao).max() / np.abs(Ao).max() < 1e-11
    R.set_learned_quadrature(None)
    A2, b2 = R.build_lse_harela(mat, om)
    assert np.abs(A2 - A0).max() == 0.0
    R.close()

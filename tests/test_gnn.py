"""The learned ordering: the numpy FP64 reference network (CPU), the GPU
forward / backward kernels against it (gradient check), training on DP
labels, and what the trained network gains over branching without it."""
import numpy as np
import pytest

from gisbdw_gb300 import gnn
from gisbdw_gb300 import graphs as G
from gisbdw_gb300.validate import check_tree


def _toy_batch(seed=0):
    rng = np.random.default_rng(seed)
    gs = [G.gnp_connected(n, 0.35, s) for n, s in ((7, 1), (9, 2), (6, 3))] + [G.path(5), G.star(6)]
    roots = [(rng.random(g.n) < 0.3).astype(np.float32) for g in gs]
    return gs, gnn.make_batch(gs, roots=roots, tds=[3, 4, 3, 3, 2])


def test_reference_gradient_matches_finite_differences():
    _, b = _toy_batch()
    shape = (gnn.IN_FEATURES, 8, 2)
    npar = shape[0] * 8 + 8 + 2 * (2 * 64 + 8) + 2 * 8 + 2
    rng = np.random.default_rng(1)
    # parameters exactly representable in BF16, so rounding does not move them
    p = gnn.bf16_round((rng.standard_normal(npar) * 0.3).astype(np.float32)).astype(np.float32)
    loss, grad = gnn.reference_loss(p, b, shape)
    for i in rng.choice(npar, 25, replace=False):
        e = np.zeros(npar)
        e[i] = 2.0 ** -6
        lp = gnn.reference_loss((p + e).astype(np.float32), b, shape, want_grad=True)[0]
        lm = gnn.reference_loss((p - e).astype(np.float32), b, shape, want_grad=True)[0]
        assert abs((lp - lm) / (2 * e[i]) - grad[i]) < 2e-3 + 0.02 * abs(grad[i]), i


def test_features_shape_and_values():
    g = G.star(5)
    f = gnn.features(g)
    assert f.shape == (5, gnn.IN_FEATURES)
    assert f[0, 0] == 1.0 and f[1, 0] == 0.25  # degree / 4
    assert f[1, 4] == 1.0 and f[0, 4] == 0.0   # pendant flag


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_reference(handle):
    _, b = _toy_batch(3)
    net = gnn.GNN(handle, seed=7)
    p = net.params()
    logits, td = net.forward(b)
    rl, rtd = gnn.reference_loss(p, b, want_grad=False)
    np.testing.assert_allclose(logits, rl, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(td, rtd, rtol=1e-4, atol=1e-4)
    grad, loss = net.gradients(b)
    rloss, rgrad = gnn.reference_loss(p, b)
    assert abs(loss - rloss) < 1e-4 * max(1.0, abs(rloss))
    # FP32 accumulation in a different order than the FP64 reference
    np.testing.assert_allclose(grad, rgrad, rtol=2e-3, atol=2e-5)


@pytest.mark.gpu
def test_training_on_dp_labels_learns_roots(handle):
    base = G.config3_graphs(count=60, seed=21)
    samples = gnn.label_samples(handle, base, per_graph=20, seed=1)
    assert len(samples) > 600
    train_s, test_s = samples[: len(samples) * 4 // 5], samples[len(samples) * 4 // 5:]
    net = gnn.GNN(handle, seed=3)
    before = gnn.root_accuracy(net, test_s)
    losses = gnn.train(net, train_s, epochs=6, batch_graphs=128, lr=3e-3)
    after = gnn.root_accuracy(net, test_s)
    assert np.mean(losses[-5:]) < np.mean(losses[:5])
    assert after["top1_root"] > after["uniform_root"] + 0.05
    assert after["top1_root"] >= before["top1_root"]


@pytest.mark.gpu
def test_learned_order_keeps_treedepth_and_cuts_search(handle):
    base = G.config3_graphs(count=80, seed=22)
    samples = gnn.label_samples(handle, base, per_graph=15, seed=2)
    net = gnn.GNN(handle, seed=5)
    gnn.train(net, samples, epochs=6, batch_graphs=128, lr=3e-3)
    gs = [g for g in G.config5_graphs(count=40, seed=9) if g.n <= 36][:16]
    plain = handle.bnb_solve_batch(gs, deadline_ns=20 * 10**9)
    orders, seeds = gnn.orders_and_seeds(net, gs)
    learned = handle.bnb_solve_batch(gs, orders=orders, seeds=seeds, deadline_ns=20 * 10**9)
    both = (plain["status"] == 0) & (learned["status"] == 0)
    print("solved plain", int((plain["status"] == 0).sum()), "learned", int((learned["status"] == 0).sum()),
          "both", int(both.sum()), "of", len(gs))
    assert both.sum() >= len(gs) // 3
    assert np.array_equal(plain["td"][both], learned["td"][both])
    for g, t, par in zip(gs, learned["td"], learned["parents"]):
        assert check_tree(g, t, par), g.name
    assert learned["nodes"][both].sum() <= plain["nodes"][both].sum()

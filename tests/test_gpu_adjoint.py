"""GPU differentiable trajectory (nd_adj_*) against the forward-mode FP64
oracle (oracle/naiveadj.c, itself pinned against central differences in
test_adjoint_oracle.py).

The GPU program computes pair forces in FP32 and keeps state in FP64; the
oracle runs the same discrete program in FP64 dual numbers.  Stated bars:
  * loss: relative difference <= 1e-5; histogram: max |dh| / max h <= 1e-5;
    final positions within 1e-6 (absolute);
  * dL/dsigma, dL/deps and the directional derivative along a random
    (dx0, dv0): relative difference <= 1e-4 (the FP32 force rounding of ~1e-7
    per step is carried through the Hessian products of every reverse step);
  * checkpointing is exact: any checkpoint interval (a multiple of the
    re-sort interval) gives bit-identical gradients, and a repeated forward +
    backward reproduces every bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHO = 0.83
LOSS_TOL = 1e-5
GRAD_TOL = 1e-4


def _case(nd, oracle, n, steps, charges=False, seed=0x4E440005, checkpoint_every=50, skin=0.3):
    side = (n / RHO) ** (1.0 / 3.0)
    x, v, q = nd.synth.lj_system(seed, n, side, 0.8, charges)
    k = 1.0 if charges else 0.0
    spec = oracle.adj_spec(steps)
    pt = oracle.md_params(sigma=1.05, epsilon=0.9, coulomb_k=k, cutoff=2.5, box_hi=(side,) * 3,
                          dt=1e-3)
    target = oracle.adj_dual(pt, spec, x, v, q=q)["hist"]
    mp = nd.md_params(sigma=1.0, epsilon=1.0, coulomb_k=k, cutoff=2.5, skin=skin, dt=1e-3,
                      box_hi=(side,) * 3, atomsperleaf=4, rebuild_every=10)
    adj = nd.Adjoint(mp, nd.adj_spec(steps, checkpoint_every=checkpoint_every), x, v, q=q)
    adj.set_target(target)
    return adj, dict(x=x, v=v, q=q, side=side, k=k, spec=spec, target=target)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-30)


@pytest.mark.parametrize("n,steps,charges", [(256, 100, False), (256, 100, True), (4096, 100, False),
                                              (1000, 50, True)])
def test_gradients_match_dual_oracle(nd, oracle, n, steps, charges):
    adj, c = _case(nd, oracle, n, steps, charges)
    rng = np.random.default_rng(11)
    dx = rng.normal(size=c["x"].shape)
    dv = rng.normal(size=c["x"].shape)
    p = oracle.md_params(coulomb_k=c["k"], cutoff=2.5, box_hi=(c["side"],) * 3, dt=1e-3)
    ref = oracle.adj_dual(p, c["spec"], c["x"], c["v"], q=c["q"], dx0=dx, dv0=dv,
                          target=c["target"])
    loss, hist = adj.forward()
    xk = adj.final_positions()
    g = adj.backward()
    adj.close()
    ddir = float((g["x0"] * dx).sum() + (g["v0"] * dv).sum())
    print(f"N={n} K={steps} coulomb={charges}: loss {_rel(loss, ref['loss']):.2e}, "
          f"hist {np.abs(hist - ref['hist']).max() / np.abs(ref['hist']).max():.2e}, "
          f"x_K {np.abs(xk - ref['x']).max():.2e}, dsigma {_rel(g['sigma'], ref['dloss'][0]):.2e}, "
          f"deps {_rel(g['epsilon'], ref['dloss'][1]):.2e}, dir {_rel(ddir, ref['dloss'][2]):.2e}")
    assert _rel(loss, ref["loss"]) <= LOSS_TOL
    assert np.abs(hist - ref["hist"]).max() <= LOSS_TOL * np.abs(ref["hist"]).max()
    assert np.abs(xk - ref["x"]).max() <= 1e-6
    assert _rel(g["sigma"], ref["dloss"][0]) <= GRAD_TOL
    assert _rel(g["epsilon"], ref["dloss"][1]) <= GRAD_TOL
    assert _rel(ddir, ref["dloss"][2]) <= GRAD_TOL


def test_checkpoint_interval_is_exact(nd, oracle):
    grads = []
    for every in (50, 100, 200):
        adj, _ = _case(nd, oracle, 1024, 200, checkpoint_every=every)
        adj.forward()
        grads.append(adj.backward())
        adj.close()
    for g in grads[1:]:
        assert np.array_equal(g["x0"], grads[0]["x0"])
        assert np.array_equal(g["v0"], grads[0]["v0"])
        assert g["sigma"] == grads[0]["sigma"] and g["epsilon"] == grads[0]["epsilon"]


def test_repeat_is_bit_identical(nd, oracle):
    adj, _ = _case(nd, oracle, 512, 100)
    l1, h1 = adj.forward()
    g1 = adj.backward()
    l2, h2 = adj.forward()
    g2 = adj.backward()
    adj.close()
    assert l1 == l2 and np.array_equal(h1, h2)
    assert np.array_equal(g1["x0"], g2["x0"]) and g1["sigma"] == g2["sigma"]


def test_set_params_matches_fresh_engine(nd, oracle):
    adj, c = _case(nd, oracle, 256, 50)
    adj.set_params(1.02, 0.97)
    l1, _ = adj.forward()
    g1 = adj.backward()
    adj.close()
    mp = nd.md_params(sigma=1.02, epsilon=0.97, cutoff=2.5, skin=0.3, dt=1e-3,
                      box_hi=(c["side"],) * 3, atomsperleaf=4, rebuild_every=10)
    fresh = nd.Adjoint(mp, nd.adj_spec(50), c["x"], c["v"])
    fresh.set_target(c["target"])
    l2, _ = fresh.forward()
    g2 = fresh.backward()
    fresh.close()
    assert l1 == l2 and g1["sigma"] == g2["sigma"] and np.array_equal(g1["x0"], g2["x0"])


def test_backward_needs_forward(nd, oracle):
    adj, _ = _case(nd, oracle, 256, 50)
    with pytest.raises(nd.NDError) as e:
        adj.backward()
    assert e.value.status == -1
    adj.forward()
    adj.backward()
    with pytest.raises(nd.NDError):
        adj.backward()  # the backward pass consumed the forward pass's lists
    adj.close()


def test_skin_violation_is_reported(nd, oracle):
    # no skin: every step moves atoms past skin/2 = 0, so every check refits,
    # but the last step's positions (where the loss is evaluated) are never
    # checked against their list: the forward pass reports the invalid list
    adj, _ = _case(nd, oracle, 256, 50, skin=0.0)
    with pytest.raises(nd.NDError) as e:
        adj.forward()
    assert e.value.status == -8
    adj.close()


def test_spec_checks(nd, oracle):
    side = (256 / RHO) ** (1.0 / 3.0)
    x, v, _ = nd.synth.lj_system(0x4E440005, 256, side, 0.8)
    mp = nd.md_params(cutoff=2.5, skin=0.3, dt=1e-3, box_hi=(side,) * 3, rebuild_every=10)
    for spec in (nd.adj_spec(105, checkpoint_every=50),    # steps not a multiple of C
                 nd.adj_spec(100, checkpoint_every=25),    # C not a multiple of the
                                                           # re-sort interval (5 windows)
                 nd.adj_spec(100, r_max=3.0)):             # histogram beyond the cutoff
        with pytest.raises(nd.NDError):
            nd.Adjoint(mp, spec, x, v)


def test_torch_autograd_function(nd, oracle):
    torch = pytest.importorskip("torch")
    adj, _ = _case(nd, oracle, 256, 50)
    fn = nd.histogram_loss_function()
    s = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    e = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    loss = fn.apply(adj, s, e)
    (2.0 * loss).backward()
    g = adj.last_grad
    adj.close()
    assert float(s.grad) == 2.0 * g["sigma"] and float(e.grad) == 2.0 * g["epsilon"]

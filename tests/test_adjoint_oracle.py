"""The forward-mode (dual-number) oracle of the differentiable trajectory,
pinned against FP64 central differences of its own loss.

The loss is piecewise smooth: the force cutoff and the wall clamps are
branches, and a finite difference whose +h and -h runs take different
branches measures a jump, not a derivative.  The oracle reports a signature
of every branch taken (pairs inside the cutoff per step, wall clamps per
step); a central difference is compared with the dual-number derivative only
where both runs took the same branches as the base run.  The step h starts at
1e-3 (the differencing step of the contract) and is divided by 10 until that
holds for h and h/2; the two quotients are combined by Richardson
extrapolation (truncation error O(h^4)) and the dual derivative must then
agree to 1e-6 relative.
"""
import numpy as np
import pytest

N = 128
RHO = 0.83


def _system(nd, n=N, seed=0x4E440005, charges=False):
    side = (n / RHO) ** (1.0 / 3.0)
    x, v, q = nd.synth.lj_system(seed, n, side, 0.8, charges)
    return x, v, q, side


def _params(oracle, side, sigma=1.0, epsilon=1.0, k=0.0):
    return oracle.md_params(sigma=sigma, epsilon=epsilon, coulomb_k=k, cutoff=2.5,
                            box_hi=(side,) * 3, dt=1e-3)


def _matched_fd(f, base_events, h0=1e-3, hmin=1e-8):
    """Richardson-extrapolated central difference at the largest h <= h0
    (decades) whose +h, -h, +h/2 and -h/2 runs took the base run's branches."""
    h = h0
    while h >= hmin:
        runs = [f(h), f(-h), f(h / 2), f(-h / 2)]
        if all(r["events"] == base_events for r in runs):
            d1 = (runs[0]["loss"] - runs[1]["loss"]) / (2 * h)
            d2 = (runs[2]["loss"] - runs[3]["loss"]) / h
            return (4.0 * d2 - d1) / 3.0, h
        h /= 10.0
    pytest.fail("no differencing step kept the branches")


@pytest.mark.parametrize("charges", [False, True])
def test_dual_matches_central_differences(nd, oracle, charges):
    x, v, q, side = _system(nd, charges=charges)
    k = 1.0 if charges else 0.0
    spec = oracle.adj_spec(40)
    target = oracle.adj_dual(_params(oracle, side, 1.05, 0.9, k), spec, x, v, q=q)["hist"]
    rng = np.random.default_rng(7)
    dx = rng.normal(size=x.shape)
    dv = rng.normal(size=x.shape)
    base = oracle.adj_dual(_params(oracle, side, k=k), spec, x, v, q=q, dx0=dx, dv0=dv,
                           target=target)
    ev = base["events"]
    fd_s, hs = _matched_fd(lambda h: oracle.adj_dual(_params(oracle, side, 1.0 + h, 1.0, k), spec,
                                                     x, v, q=q, target=target), ev)
    fd_e, he = _matched_fd(lambda h: oracle.adj_dual(_params(oracle, side, 1.0, 1.0 + h, k), spec,
                                                     x, v, q=q, target=target), ev)
    fd_d, hd = _matched_fd(lambda h: oracle.adj_dual(_params(oracle, side, k=k), spec, x + h * dx,
                                                     v + h * dv, q=q, target=target), ev)
    print(f"dL/dsigma dual {base['dloss'][0]:.9e} fd {fd_s:.9e} (h={hs:g}); "
          f"dL/deps dual {base['dloss'][1]:.9e} fd {fd_e:.9e} (h={he:g}); "
          f"directional dual {base['dloss'][2]:.9e} fd {fd_d:.9e} (h={hd:g})")
    for dual, fd in ((base["dloss"][0], fd_s), (base["dloss"][1], fd_e), (base["dloss"][2], fd_d)):
        assert abs(dual - fd) <= 1e-6 * max(abs(dual), 1e-12) + 1e-10


def test_dual_value_matches_plain_trajectory(nd, oracle):
    # the value part of the dual program is the FP64 integrator of ref_md_run
    x, v, _, side = _system(nd)
    p = _params(oracle, side)
    r = oracle.adj_dual(p, oracle.adj_spec(30), x, v)
    xr, _, _ = oracle.md_run(p, x, v, steps=30)
    assert np.abs(r["x"] - xr).max() < 1e-12


def test_histogram_counts_pairs(nd, oracle):
    # with a tiny width the smoothed histogram integrates to the pair count
    # below r_switch: sum_b h_b * sqrt(2 pi) w / bw -> pairs / N
    x, v, _, side = _system(nd)
    spec = oracle.adj_spec(1, bins=250, r_max=2.5, width=0.002, r_switch=2.4)
    p = _params(oracle, side)
    r = oracle.adj_dual(p, spec, x, v)
    bw = 2.5 / 250
    total = r["hist"].sum() * bw / (np.sqrt(2 * np.pi) * 0.002) * N
    xs = r["x"]
    d = np.linalg.norm(xs[:, None, :] - xs[None, :, :], axis=-1)
    iu = np.triu_indices(N, 1)
    inner = int(np.sum(d[iu] < 2.4 - 0.01))
    outer = int(np.sum(d[iu] < 2.5))
    assert inner - 1 <= total <= outer + 1


def test_spec_errors(nd, oracle):
    x, v, _, side = _system(nd, n=16)
    bad = oracle.adj_spec(1, r_switch=3.0)
    with pytest.raises(oracle.OracleError):
        oracle.adj_dual(_params(oracle, side), bad, x, v)

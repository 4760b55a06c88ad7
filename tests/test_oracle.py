"""The CPU oracle against the reference's own known answers and golden vectors.

These run without a GPU.  They pin the oracle before it is trusted as the
checker of the CUDA path:
  * test/BVHTraverse.jl:165-220 -- the 8-point hand fixture and its invariants;
  * test/BVHTraverse.jl:222-287 -- BVH pair list == brute-force pair list over
    the reference's r / atomsperleaf / N families (seeded stand-ins for the
    missing data/positions.jld2);
  * tests/golden/bvh_golden.json -- vectors from an independent pure-Python
    restatement (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import canon
from helpers import golden_cases, uniform

POSITION8 = np.array([[0.1, 0.1, 0.1], [0.2, 0.2, 0.2], [0.346, 0.98, 0.12], [0.01, 0.76, 0.99],
                      [0.1111, 0.4, 0.31], [0.234, 0.29, 0.2], [0.11346, 0.918, 0.1276],
                      [0.061, 0.76, 0.989]], np.float32)


def test_position8_traversability(oracle):
    # test/BVHTraverse.jl:170-211: neighbor_distance=10, atomsperleaf=1, TreeData
    t = oracle.tree(POSITION8, 10.0, 1, boxes=oracle.REF_BOX_ATOM)
    keys = t["keys"]
    assert keys[7]["skip"] == 0                      # keys[8].skip == 0
    assert all(keys[k]["skip"] != 0 for k in range(7))  # keys[1:7].skip != 0
    pi, pj, pd = oracle.build_traverse_bvh(POSITION8, 10.0, 1)
    paired = np.zeros(9, bool)
    paired[pi] = True
    paired[pj] = True
    assert paired[1:].all()                          # every atom paired
    bi, bj, bd = oracle.brute_pairs(POSITION8, 10.0, criterion=1)
    assert len(bi) == 28
    assert np.array_equal(canon(pi, pj, pd), canon(bi, bj, bd))


def test_position8_root_contains_scene(oracle):
    # test/BVHTraverse.jl:213-220 (root box overwritten to [0,1]^3)
    t = oracle.tree(POSITION8, 10.0, 1, boxes=oracle.REF_BOX_ATOM)
    root = t["keys"][8]
    assert np.all(root["min"] < POSITION8) and np.all(POSITION8 < root["max"])


def _self_consistent_tree(keys, nl):
    # is_traversable (test/BVHTraverse.jl:87-116): no self ropes, every node reached
    for k in range(2 * nl - 1):
        assert keys[k]["left"] != k + 1 and keys[k]["skip"] != k + 1
    seen = np.zeros(2 * nl, bool)
    t = keys[nl]["left"]
    seen[nl + 1] = True
    steps = 0
    while t != 0:
        seen[t] = True
        steps += 1
        assert steps <= 4 * nl
        t = keys[t - 1]["left"] if keys[t - 1]["left"] != 0 else keys[t - 1]["skip"]
    assert seen[1:].all()


@pytest.mark.parametrize("boxes", [0, 1])
def test_tree_fully_traversable(oracle, boxes):
    x = uniform(11, 400)
    for apl in (2, 4, 5):
        t = oracle.tree(x, 0.1, apl, boxes=boxes)
        _self_consistent_tree(t["keys"], t["leaves"])


@pytest.mark.parametrize("r", [1e-4, 1e-3, 1e-2, 1e-1, 1.0])
def test_family_neighbor_distance(oracle, r):
    # test/BVHTraverse.jl:225-243 (pos5000 -> 2000 seeded points; r up to 1.0)
    n = 5000 if r < 1.0 else 1500
    x = uniform(5000, n)
    bi, bj, bd = oracle.brute_pairs(x, r, criterion=0)
    for order in (0, 1):
        li, lj, ld = oracle.leafbuild_traverse_bvh(x, r, 4, order=order)
        assert np.array_equal(canon(li, lj, ld), canon(bi, bj, bd))
        ai, aj, ad = oracle.build_traverse_bvh(x, r, 4, order=order)
        assert np.array_equal(canon(ai, aj, ad), canon(bi, bj, bd))


@pytest.mark.parametrize("apl", [2, 4, 5, 10, 20, 1000])
def test_family_atomsperleaf(oracle, apl):
    # test/BVHTraverse.jl:246-265 (apl = 1 is only valid on the TreeData path)
    x = uniform(5001, 5000)
    bi, bj, bd = oracle.brute_pairs(x, 0.1, criterion=0)
    li, lj, ld = oracle.leafbuild_traverse_bvh(x, 0.1, apl)
    assert np.array_equal(canon(li, lj, ld), canon(bi, bj, bd))
    ai, aj, ad = oracle.build_traverse_bvh(x, 0.1, apl)
    assert np.array_equal(canon(ai, aj, ad), canon(bi, bj, bd))


def test_family_atomsperleaf_one_per_atom_path(oracle):
    x = uniform(5002, 2000)
    bi, bj, bd = oracle.brute_pairs(x, 0.1, criterion=0)
    ai, aj, ad = oracle.build_traverse_bvh(x, 0.1, 1)
    assert np.array_equal(canon(ai, aj, ad), canon(bi, bj, bd))
    with pytest.raises(oracle.OracleError):
        oracle.tree(x, 0.1, 1, boxes=oracle.REF_BOX_LEAF)


@pytest.mark.parametrize("n", [10, 100, 1000, 2000, 3000, 20000])
def test_family_positions(oracle, n):
    # test/BVHTraverse.jl:268-287, atomsperleaf = 5, r = 0.1
    x = uniform(n, n)
    bi, bj, bd = oracle.brute_pairs(x, 0.1, criterion=0)
    li, lj, ld = oracle.leafbuild_traverse_bvh(x, 0.1, 5)
    assert np.array_equal(canon(li, lj, ld), canon(bi, bj, bd))


def test_sqrt_criterion_disagreement_is_boundary_only(oracle):
    # Leaf path uses d^2 < r^2, AllToAll / SIMD use sqrt(d^2) < r: any pair where
    # they differ must sit within a few ulps of the cutoff.
    x = uniform(77, 3000)
    a0 = canon(*oracle.brute_pairs(x, 0.1, 0))
    a1 = canon(*oracle.brute_pairs(x, 0.1, 1))
    s0 = {tuple(r) for r in a0}
    s1 = {tuple(r) for r in a1}
    for row in s0 ^ s1:
        d = np.array([row[2]], np.int32).view(np.float32)[0]
        assert abs(d - np.float32(0.1)) <= 4 * np.spacing(np.float32(0.1))


# Two points whose Float32 squared distance is exactly 0.01f: inside r = 0.1
# by d^2 < r^2 (fl(0.1f * 0.1f) = 0.010000001f) but not by sqrt(d^2) < r
# (sqrtf(0.01f) rounds to 0.1f); the rest lie far from them.
BOUNDARY_PAIR = np.array([[0.0, 0.0, 0.0], [0.060000002, 0.08, 0.0]], np.float32)


def boundary_positions():
    rest = np.random.default_rng(11).uniform(0.5, 1.0, (62, 3)).astype(np.float32)
    return np.concatenate([BOUNDARY_PAIR, rest])


def test_simd_traversal(oracle):
    # simdneighbor_traverse: the leaf traversal with sqrt(d^2) < r -- its set
    # equals brute force with that criterion; on the boundary pair it drops
    # what leafneighbor_traverse keeps
    x = uniform(91, 4096)
    for r in (0.05, 0.1, 0.0731):
        t = oracle.tree(x, r, 4)
        assert np.array_equal(canon(*oracle.simd_leaf_traverse(t, r, 4)),
                              canon(*oracle.brute_pairs(x, r, 1)))
    xb = boundary_positions()
    d2 = np.float32(np.float32(xb[1, 0] * xb[1, 0]) + np.float32(xb[1, 1] * xb[1, 1]))
    assert d2 == np.float32(0.01) and d2 < np.float32(0.1) * np.float32(0.1)
    assert not (np.sqrt(d2) < np.float32(0.1))
    t = oracle.tree(xb, 0.1, 4)
    s0 = {tuple(r) for r in canon(*oracle.leaf_traverse(t, 0.1, 4))}
    s1 = {tuple(r) for r in canon(*oracle.simd_leaf_traverse(t, 0.1, 4))}
    assert len(s0 - s1) == 1 and not (s1 - s0)
    (i, j, _), = s0 - s1
    assert {i, j} == {1, 2}


def test_compat_forces_oracle(oracle):
    # force_coulomb! at HEAD: force[i] .+= q_i q_j / d^2, then force[j] .-=
    # force[i] (the running total) -- by hand for a three-pair list
    f32 = np.float32
    i = np.array([1, 1, 2], np.int32)
    j = np.array([2, 3, 3], np.int32)
    d = np.array([0.5, 0.25, 0.75], np.float32)
    q = np.array([1.0, -1.0, 2.0], np.float32)
    F = np.zeros(3, np.float32)
    for a, b, dd in zip(i - 1, j - 1, d):
        F[a] = f32(F[a] + f32(f32(q[a] * q[b]) / f32(dd * dd)))
        F[b] = f32(F[b] - F[a])
    out = oracle.compat_forces("coulomb", 3, (i, j, d), q)
    assert np.array_equal(out, np.repeat(F[:, None], 3, axis=1))
    # force_lennardjones! at HEAD: only force[i] receives the pair term, the
    # same on all three components, and it does not depend on the positions
    lj = oracle.compat_forces("lj", 3, (i, j, d))
    assert np.all(lj[2] == 0) and np.all(lj[:, 0] == lj[:, 1]) and np.all(lj[:, 1] == lj[:, 2])
    # each atom's additions in list order: swapping pairs of different atoms
    # changes nothing
    lj2 = oracle.compat_forces("lj", 3, (i[[2, 0, 1]], j[[2, 0, 1]], d[[2, 0, 1]]))
    assert np.array_equal(lj, lj2)
    # magnitude check of one term against float64 math (the power by squaring
    # is within an ulp of the exact power)
    t = (np.float64(f32(f32(24.0) * f32(-1e10)) / f32(0.5))
         * ((2e-4 / 0.5) ** 12 - (1e-4 / 0.5) ** 6))
    one = oracle.compat_forces("lj", 2, (np.array([1], np.int32), np.array([2], np.int32),
                                         np.array([0.5], np.float32)))
    assert one[0, 0] == np.float32(t) and np.all(one[1] == 0)


def test_compat_simulate_oracle(oracle):
    # simulate! as written, checked against by-hand cases of its formulas
    box = dict(min_dim=(0.0, 0.0, 0.0), max_dim=(1.0, 1.0, 1.0))
    # two neutral atoms far apart (no LJ pair below 0.01, no charge): the
    # all-pairs LJ term (added to force[i] only) is ~1e-11 at d = 0.7, so the
    # motion is x += v to 1e-6; a wall crossing clamps x and flips v exactly
    x = np.array([[0.2, 0.5, 0.5], [0.9, 0.5, 0.5]], np.float32)
    v = np.array([[0.1, 0.0, 0.0], [0.05, 0.0, 0.0]], np.float32)
    xs, vs, fs, log, st = oracle.compat_simulate(
        x, v, np.zeros((2, 3)), np.ones(2), np.zeros(2), temperature=0.0, objectnumber=2,
        stepwidth=1, duration=3, vdamp=0.0, **box)
    assert st == 0
    xe = np.array([[0.3, 0.5, 0.5], [0.95, 0.5, 0.5]], np.float32)
    assert np.allclose(log[1], xe, atol=1e-6) and np.allclose(log[3][0], [0.5, 0.5, 0.5], atol=1e-6)
    assert log[3][1][0] == 1.0 and vs[1][0] == np.float32(-0.05)
    assert np.all(fs[1] == 0) and np.all(fs[0] > 0) and fs[0][0] == fs[0][1] == fs[0][2]
    assert np.array_equal(log[0], xs)
    # a negative rescale_velocity! radicand at step 10 is Julia's DomainError
    rng = np.random.default_rng(3)
    x = rng.uniform(0.1, 0.9, (8, 3)).astype(np.float32)
    v = rng.uniform(-1e-3, 1e-3, (8, 3)).astype(np.float32)
    *_, st = oracle.compat_simulate(x, v, np.zeros((8, 3)), np.ones(8), np.zeros(8),
                                    temperature=1e-9, objectnumber=8, stepwidth=1,
                                    duration=12, vdamp=3.0, log=False, **box)
    assert st == 1
    # gamma = 0 leaves beta = 1; gamma = 1 scales the velocities by
    # sqrt(Tf / Ti), Ti = 2 / (3 N) sum |v_i| m_i / 2 (linear in |v|, as written)
    run = lambda g: oracle.compat_simulate(x, v, np.zeros((8, 3)), np.ones(8), np.zeros(8),
                                           temperature=0.5, objectnumber=8, stepwidth=1,
                                           duration=10, vdamp=g, log=False, **box)[1]
    v0, v1 = run(0.0), run(1.0)
    Ti = np.sum(2 / (3 * 8) * np.linalg.norm(v0.astype(np.float64), axis=1) / 2)
    assert np.allclose(v1, v0 * np.sqrt(0.5 / Ti), rtol=1e-6, atol=0)


def test_collect_objects_oracle(oracle):
    # ranges, the velocity formulas and unique_pairs_prune's rule, by hand
    box = ((0.0, 0.0, 0.0), (1.0, 2.0, 3.0))
    x, v, m, q, cnt = oracle.collect_objects(5, 3000, box[0], box[1], 0.01, False, 1.0, 5.0,
                                             0.02, -1e-9, 1e-9)
    fin = np.isfinite(x).all(axis=1)
    assert cnt == int((~fin).sum()) > 0 and fin[-1] and fin[-2]
    assert np.all((m >= 1) & (m < 5)) and np.all((q >= -1e-9) & (q < 1e-9))
    assert np.all(x[fin] >= 0) and np.all(x[fin] < np.array([1, 2, 3], np.float32))
    T, N = np.float32(0.01), np.float32(3000)
    assert np.array_equal(v, np.repeat(((T / N * np.float32(3) * N) * np.float32(1) / m)[:, None],
                                       3, axis=1))
    # pruned exactly when a later atom other than the last lies within 0.02
    _, _, _, _, c0 = oracle.collect_objects(5, 3000, box[0], box[1], 0.01, False, 1.0, 5.0, 0.0,
                                            -1e-9, 1e-9)
    x0 = oracle.collect_objects(5, 3000, box[0], box[1], 0.01, False, 1.0, 5.0, 0.0, -1e-9,
                                1e-9)[0]
    assert c0 == 0 and np.array_equal(x0[fin], x[fin])
    d = x0[:, None, :] - x0[None, :, :]
    dist = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
    close = (dist < np.float32(0.02)) & np.triu(np.ones((3000, 3000), bool), 1)
    close[:, -1] = False
    assert np.array_equal(close.any(axis=1), ~fin)
    # random split: each component's v m / (3 N T) sums to 1
    _, vr, mr, _, _ = oracle.collect_objects(6, 1000, box[0], box[1], 0.5, True, 1.0, 5.0, 0.0,
                                             0.0, 0.0)
    share = (vr.astype(np.float64) * mr[:, None]) / (3 * 1000 * 0.5)
    assert np.allclose(share.sum(axis=0), 1.0, atol=1e-5)


def test_golden_vectors(oracle):
    for c in golden_cases():
        x = np.array(c["position"], np.float32)
        boxes = oracle.REF_BOX_LEAF if c["boxes"] == "leaf" else oracle.REF_BOX_ATOM
        t = oracle.tree(x, c["r"], c["apl"], boxes=boxes)
        nl = t["leaves"]
        assert list(oracle.morton_reference(x)) == c["codes"], c["name"]
        assert list(t["perm"] + 1) == c["perm"], c["name"]
        assert list(t["index"]) == c["index"], c["name"]
        assert list(t["code"]) == c["code_sorted"], c["name"]
        for k, g in zip(t["keys"][: 2 * nl - 1], c["keys"]):
            assert [float(v) for v in k["min"]] == g[0]
            assert [float(v) for v in k["max"]] == g[1]
            assert (int(k["left"]), int(k["skip"])) == (g[2], g[3]), c["name"]
        if c["boxes"] == "leaf":
            pi, pj, pd = oracle.leaf_traverse(t, c["r"], c["apl"])
        else:
            pi, pj, pd = oracle.atom_traverse(t, c["r"], c["apl"])
        got = [[int(a), int(b), float(d)] for a, b, d in zip(pi, pj, pd)]
        assert got == c["pairs"], c["name"]


def test_morton_errors(oracle):
    x = uniform(1, 8)
    x[3, 1] = np.nan
    with pytest.raises(oracle.OracleError):
        oracle.morton_reference(x)
    x = uniform(1, 8)
    x[2, 0] = 3.0e6  # 3e6 * 1023 > 2^31: InexactError in round(Int32, ...)
    with pytest.raises(oracle.OracleError):
        oracle.morton_reference(x)
    x[2, 0] = -2.0e6  # -2.046e9 >= -2^31: still representable
    oracle.morton_reference(x)


def test_hilbert_curve_is_continuous(oracle):
    # On the coarse 8^3 grid (cells at multiples of 128 of the 1024 grid) the
    # top 9 index bits order the cells along a Hilbert curve: consecutive cells
    # are face neighbours and every cell appears once.
    cells = [(a << 7, b << 7, c << 7) for a in range(8) for b in range(8) for c in range(8)]
    idx = [oracle.hilbert3(*p) >> 21 for p in cells]
    assert sorted(idx) == list(range(512))
    order = [p for _, p in sorted(zip(idx, cells))]
    for p, q in zip(order, order[1:]):
        assert sum(abs(a - b) for a, b in zip(p, q)) == 128
    # and at full resolution along a random walk of neighbouring cells the
    # indices are distinct
    rng = np.random.default_rng(5)
    pts = {tuple(rng.integers(0, 1024, 3)) for _ in range(2000)}
    assert len({oracle.hilbert3(*p) for p in pts}) == len(pts)


def test_spec_checks(oracle):
    with pytest.raises(oracle.OracleError):
        oracle.spec(10, 4)          # 4 does not divide 10
    with pytest.raises(oracle.OracleError):
        oracle.spec(4, 4)           # a single leaf
    assert oracle.spec(12, 4) == (3, 2)


def test_hash_order_free(oracle):
    x = uniform(3, 500)
    pi, pj, pd = oracle.leafbuild_traverse_bvh(x, 0.2, 4)
    h = oracle.pair_hash(pi, pj, pd)
    p = np.random.default_rng(0).permutation(len(pi))
    assert oracle.pair_hash(pj[p], pi[p], pd[p]) == h
    t = oracle.tree(x, 0.2, 4)
    assert oracle.leaf_traverse_hash(t, 0.2, 4) == (len(pi), h)


# ------------------------------------------------------------ physics oracle

def _lj_box(n=216, side=7.0, seed=3):
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(6)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    x = (g + 0.5) * (side / 6) + rng.normal(0, 0.08, (n, 3))
    return x


def test_forces_are_minus_gradient(oracle):
    x = _lj_box()
    q = np.where(np.arange(len(x)) % 2 == 0, 1.0, -1.0)
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(7, 7, 7))
    f, _, _ = oracle.forces(p, x, q)
    h = 1e-6
    for (i, d) in [(0, 0), (17, 1), (100, 2), (215, 0)]:
        xp, xm = x.copy(), x.copy()
        xp[i, d] += h
        xm[i, d] -= h
        up = oracle.forces(p, xp, q)[1]
        um = oracle.forces(p, xm, q)[1]
        assert abs(-(up - um) / (2 * h) - f[i, d]) < 1e-5 * max(1.0, abs(f[i, d]))


def test_forces_newton_third_law_and_cells(oracle):
    x = _lj_box()
    p = oracle.md_params(cutoff=2.5, box_hi=(7, 7, 7))
    f, u, npairs = oracle.forces(p, x)
    assert np.abs(f.sum(0)).max() < 1e-9 * np.abs(f).max()
    # brute force reference of the same sum
    d = x[:, None, :] - x[None, :, :]
    r2 = (d ** 2).sum(-1)
    iu = np.triu_indices(len(x), 1)
    m = r2[iu] < 2.5 ** 2
    s6 = (1.0 / r2[iu][m]) ** 3
    assert npairs == int(m.sum())
    assert abs(u - np.sum(4 * (s6 * s6 - s6))) < 1e-9 * abs(u)


def test_md_energy_conservation(oracle):
    # Velocity Verlet is second order: the energy error over a fixed time
    # shrinks 4x per halving of dt.  The cutoff covers every pair, so the
    # truncated (unshifted) potential has no jumps.
    x = _lj_box()
    v = np.random.default_rng(1).normal(0, 0.5, x.shape)
    errs = []
    for dt in (1e-3, 5e-4):
        p = oracle.md_params(cutoff=30.0, box_lo=(-50, -50, -50), box_hi=(50, 50, 50), dt=dt)
        u0 = oracle.forces(p, x)[1]
        e0 = u0 + 0.5 * (v ** 2).sum()
        x1, v1, _ = oracle.md_run(p, x, v, steps=int(round(0.2 / dt)))
        e1 = oracle.forces(p, x1)[1] + 0.5 * (v1 ** 2).sum()
        errs.append(abs(e1 - e0) / abs(e0))
    assert errs[0] < 5e-4
    assert 3.5 < errs[0] / errs[1] < 4.5


def test_md_walls_reflect(oracle):
    x = np.array([[0.5, 0.5, 0.5], [5.0, 5.0, 5.0]])
    v = np.array([[-100.0, 0.0, 0.0], [0.0, 0.0, 300.0]])
    p = oracle.md_params(cutoff=2.5, box_lo=(0, 0, 0), box_hi=(6, 6, 6), dt=1e-2)
    x1, v1, _ = oracle.md_run(p, x, v, steps=1)
    assert x1[0, 0] == 0.0 and v1[0, 0] == 100.0
    assert x1[1, 2] == 6.0 and v1[1, 2] == -300.0


def test_cpu_baseline_matches_fp64_step(oracle):
    # ref_md_run_bvh (the timed CPU baseline) equals ref_md_run while the list holds.
    x = _lj_box()
    v = np.random.default_rng(2).normal(0, 0.5, x.shape)
    p = oracle.md_params(cutoff=2.5, box_lo=(-50, -50, -50), box_hi=(50, 50, 50))
    xa, va, fa = oracle.md_run(p, x, v, steps=20)
    xb, vb, fb, _ = oracle.md_run_bvh(p, x, v, steps=20, rebuild=10, skin=0.3, apl=4)
    assert np.abs(xa - xb).max() < 1e-11
    assert np.abs(va - vb).max() < 1e-9


def test_tree_kept_order(oracle):
    # The kept-order tree (gpubvh_neighborlist!'s refit): on the same
    # positions it is the full build; on moved positions its leaf traversal
    # gives the brute-force pair set.
    x = uniform(0x4E440052, 2000, 1.0)
    t = oracle.tree(x, 0.08, 4)
    k = oracle.tree_kept(x, 0.08, 4, t["index"], t["code"])
    assert np.array_equal(k["keys"].view(np.int32), t["keys"].view(np.int32))
    y = (x + np.random.default_rng(3).normal(0.0, 0.01, x.shape)).astype(np.float32)
    k = oracle.tree_kept(y, 0.08, 4, t["index"], t["code"])
    assert np.array_equal(canon(*oracle.leaf_traverse(k, 0.08, 4)),
                          canon(*oracle.brute_pairs(y, 0.08, 0)))

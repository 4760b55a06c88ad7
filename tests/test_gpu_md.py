"""GPU forces and dynamics against the FP64 oracle.

Tolerances (stated per result, as the contract requires):
  * forces: relative L2 error |F32 - F64|_2 / |F64|_2 <= 1e-5, and the per-atom
    error max_i |dF_i| / max(|F64_i|, 1e-3 rms|F64|) <= 1e-5 (pairs closer than
    1.3 sigma are evaluated in two-float arithmetic, the rest in plain single
    precision);
  * energies: relative error <= 1e-6;
  * dynamics over 100 steps (dt = 1e-3, rebuild every 10): positions within
    1e-5 (absolute, box side 17) of the FP64 trajectory -- an FP32 force error
    of ~5e-7 relative acts for t = 0.1 and the LJ dynamics amplify it (measured
    1.8e-6 on GB300).
"""
import numpy as np
import pytest

from conftest import canon
from helpers import force_errors

pytestmark = pytest.mark.gpu

F_L2_TOL = 1e-5
F_ATOM_TOL = 1e-5


def _config1(nd, charges=False, n=4096, side=17.0, seed=0x4E440001):
    return nd.synth.lj_system(seed, n, side, 0.8, charges)


def test_forces_lj_vs_fp64(nd, oracle):
    x, _, _ = _config1(nd)
    f32, u32 = nd.forces(x, None, nd.ForceField(1.0, 1.0, 0.0, 2.5))
    p = oracle.md_params(cutoff=2.5, box_hi=(17, 17, 17))
    f64, u64, _ = oracle.forces(p, x)
    per_atom, l2 = force_errors(f32, f64)
    print(f"LJ force error: per-atom {per_atom:.3e}  L2 {l2:.3e}  energy {abs(u32-u64)/abs(u64):.3e}")
    assert l2 <= F_L2_TOL
    assert per_atom <= F_ATOM_TOL
    assert abs(u32 - u64) <= 1e-6 * abs(u64)


def test_forces_lj_coulomb_vs_fp64(nd, oracle):
    x, _, q = _config1(nd, charges=True)
    f32, u32 = nd.forces(x, q, nd.ForceField(1.0, 1.0, 1.0, 2.5))
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(17, 17, 17))
    f64, u64, _ = oracle.forces(p, x, q)
    per_atom, l2 = force_errors(f32, f64)
    print(f"LJ+C force error: per-atom {per_atom:.3e}  L2 {l2:.3e}  energy {abs(u32-u64)/abs(u64):.3e}")
    assert l2 <= F_L2_TOL
    assert per_atom <= F_ATOM_TOL
    assert abs(u32 - u64) <= 1e-6 * abs(u64)


def test_force_calls_with_pair_list(nd, oracle):
    # force_lennardjones!(force, pairslist, position) + force_coulomb! + sum_forces!
    x, _, q = _config1(nd, charges=True, n=2048, side=13.5)
    spec = nd.SpheresBVHSpecs(2.5, len(x), 4)
    pairs = nd.leafbuild_traverse_bvh(x.astype(np.float32), spec)
    flj = np.zeros((len(x), 3), np.float32)
    fc = np.zeros((len(x), 3), np.float32)
    ulj = nd.force_lennardjones_(flj, pairs, x)
    uc = nd.force_coulomb_(fc, pairs, q, x)
    f = nd.sum_forces_(np.zeros_like(flj), flj, fc)
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(14, 14, 14))
    f64, u64, _ = oracle.forces(p, x, q)
    per_atom, l2 = force_errors(f, f64)
    assert l2 <= F_L2_TOL
    assert abs((ulj + uc) - u64) <= 1e-6 * abs(u64)


def _params(nd, side, coulomb=0.0, rebuild=10, order=1, skin=0.3, atomsperleaf=4, **kw):
    return nd.md_params(sigma=1.0, epsilon=1.0, coulomb_k=coulomb, cutoff=2.5, skin=skin, dt=1e-3,
                        box_lo=(0, 0, 0), box_hi=(side, side, side), atomsperleaf=atomsperleaf,
                        rebuild_every=rebuild, order=order, **kw)


def test_md_trajectory_vs_fp64(nd, oracle):
    # plain LJ, 4096 atoms, side 17, 100 steps, rebuild every 10
    x0, v0, _ = _config1(nd)
    eng = nd.MDEngine(_params(nd, 17.0), x0, v0)
    pe0, ke0 = eng.energy()
    eng.run(100)
    eng.sync()
    x, v, f = eng.get()
    pe1, ke1 = eng.energy()
    p = oracle.md_params(cutoff=2.5, box_hi=(17, 17, 17), dt=1e-3)
    xr, vr, fr = oracle.md_run(p, x0, v0, steps=100)
    dx = np.abs(x - xr).max()
    dv = np.abs(v - vr).max()
    print(f"100-step trajectory: max|dx| {dx:.3e}  max|dv| {dv:.3e}")
    assert dx < 1e-5
    assert dv < 1e-3
    # forces at the GPU's final positions vs FP64 forces there
    f64, u64, _ = oracle.forces(p, x)
    per_atom, l2 = force_errors(f, f64)
    print(f"forces after 100 steps: per-atom {per_atom:.3e}  L2 {l2:.3e}")
    assert l2 <= F_L2_TOL
    assert per_atom <= F_ATOM_TOL
    e0, e1 = pe0 + ke0, pe1 + ke1
    print(f"energy: {e0:.6f} -> {e1:.6f} (rel drift {abs(e1-e0)/abs(e0):.2e})")
    u0 = oracle.forces(p, x0)[1]
    assert abs(pe0 - u0) <= 1e-6 * abs(u0)
    assert abs(ke0 - 0.5 * (v0 ** 2).sum()) <= 1e-12 * ke0
    st = eng.stats()
    assert st["steps"] == 100 and st["rebuilds"] == 10
    assert eng.diagnostics()["skin_violations"] == 0


@pytest.mark.parametrize("check_every,vscale", [(1, 15.0), (3, 5.0)])
def test_md_early_refit_keeps_lists_valid(nd, oracle, check_every, vscale):
    # A hot start (velocities N(0, vscale^2)) moves atoms more than skin/4
    # inside a rebuild window: early refits must keep every atom within skin/2
    # of its list-build position (no skin violation), the trajectory must
    # follow the FP64 one, and eager (partial-window) runs must refit at the
    # same steps as the captured windows -- with a check after every step, and
    # after every third step of a window (for atoms slow enough that three
    # steps stay well inside skin/2).
    x0, v0, _ = _config1(nd, n=2048, side=13.5)
    v0 = v0 * vscale
    a = nd.MDEngine(_params(nd, 13.5, refit_check_every=check_every), x0, v0)
    a.run(60)
    a.sync()
    xa, va, fa = a.get()
    d = a.diagnostics()
    print(f"early refits {d['early_refits']} ({d['refit_kernels']} kernels each), "
          f"skin violations {d['skin_violations']}")
    assert d["early_refits"] > 0
    assert d["skin_violations"] == 0
    p = oracle.md_params(cutoff=2.5, box_hi=(13.5, 13.5, 13.5), dt=1e-3)
    xr, vr, _ = oracle.md_run(p, x0, v0, steps=60)
    assert np.abs(xa - xr).max() < 1e-5
    f64, _, _ = oracle.forces(p, xa)
    assert force_errors(fa, f64)[1] <= F_L2_TOL
    b = nd.MDEngine(_params(nd, 13.5, refit_check_every=check_every), x0, v0)
    for k in (7, 3, 11, 9, 10, 20):
        b.run(k)
    xb, vb, _ = b.get()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    assert b.diagnostics()["early_refits"] == d["early_refits"]


def test_md_refit_windows_match_resorting(nd):
    # Re-sorting at every rebuild and refitting the kept tree in between give
    # the same dynamics up to force summation order.
    x0, v0, q = _config1(nd, charges=True, n=2048, side=13.5)
    out = []
    for rs in (1, 5):
        eng = nd.MDEngine(_params(nd, 13.5, coulomb=1.0, resort_every=rs), x0, v0, q)
        eng.run(60)
        out.append(eng.get())
        assert eng.diagnostics()["skin_violations"] == 0
    assert np.abs(out[0][0] - out[1][0]).max() < 2e-6
    assert force_errors(out[1][2], np.asarray(out[0][2], np.float64))[1] < 1e-5


@pytest.mark.parametrize("apl", [1, 4, 8])
def test_md_union_searches_agree(nd, apl):
    # The block-box search and the tree walk find the same sorted union, so
    # lists, summation order and every bit of the trajectory agree, through
    # re-sorts, refits and (at a small skin) early refits.
    x0, v0, q = _config1(nd, charges=True, n=4096, side=17.0)
    out = []
    for us in (nd.ND_UNION_BLOCKS, nd.ND_UNION_TREE):
        eng = nd.MDEngine(_params(nd, 17.0, coulomb=1.0, skin=0.05, resort_every=3,
                                  union_search=us, atomsperleaf=apl), x0, v0, q)
        eng.run(70)
        out.append((eng.get(), eng.stats()["list_pairs"], eng.diagnostics()))
        eng.close()
    (xa, va, fa), la, da = out[0]
    (xb, vb, fb), lb, db = out[1]
    assert da["early_refits"] > 0 and da["resorts"] > 0 and da["refits"] > 0
    assert la == lb and da["early_refits"] == db["early_refits"]
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)


@pytest.mark.parametrize("n,side", [(1500, 12.1), (78852, 45.6)])
def test_md_partial_last_block(nd, oracle, n, side):
    # atom counts that are not a multiple of the 256-atom block: the last
    # block is partly empty (1,500: four threads per atom in the step kernel;
    # 78,852: 309 blocks, one thread per atom) -- 30 steps against FP64
    x0, v0, q = nd.synth.lj_system(0x4E440021, n, side, 0.8, charges=True)
    eng = nd.MDEngine(_params(nd, side, coulomb=1.0, refit_check_every=3), x0, v0, q)
    eng.run(30)
    xg, vg, fg = eng.get()
    d = eng.diagnostics()
    eng.close()
    assert d["skin_violations"] == 0
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(side,) * 3, dt=1e-3)
    xr, vr, _ = oracle.md_run(p, x0, v0, q, steps=30)
    assert np.abs(xg - xr).max() < 1e-5
    f64, _, _ = oracle.forces(p, xg, q)
    assert force_errors(fg, f64)[1] <= F_L2_TOL


def test_compat_force_calls(nd, oracle):
    # force_lennardjones! / force_coulomb! as the reference computes them at
    # HEAD, over the reference-order pair list of 4,096 points in the unit
    # cube: bit for bit against the oracle's restatement (the Coulomb
    # recurrence in list order, the LJ terms per atom in list order)
    x = nd.synth.uniform_positions(0x4E440031, 4096, 1.0)
    spec = nd.SpheresBVHSpecs(0.05, len(x), 4)
    pairs = nd.leafbuild_traverse_bvh(x, spec)
    q = np.where(np.arange(len(x)) % 2 == 0, 1.0, -1.0).astype(np.float32)
    lst = (pairs["i"], pairs["j"], pairs["d"])
    flj = nd.force_lennardjones_compat_(np.zeros((len(x), 3), np.float32), pairs, x)
    fc = nd.force_coulomb_compat_(np.zeros((len(x), 3), np.float32), pairs, q)
    assert np.array_equal(flj.view(np.int32), oracle.compat_forces("lj", len(x), lst).view(np.int32))
    assert np.array_equal(fc.view(np.int32),
                          oracle.compat_forces("coulomb", len(x), lst, q).view(np.int32))
    assert np.abs(flj).max() > 0 and np.abs(fc).max() > 0
    f = nd.sum_forces_(np.zeros_like(flj), flj, fc)
    assert np.array_equal(f, flj + fc)
    with pytest.raises(nd.NDError):
        bad = (pairs["i"].copy(), pairs["j"], pairs["d"])
        bad[0][0] = len(x) + 1
        nd.force_coulomb_compat_(np.zeros((len(x), 3), np.float32), bad, q)


def _dist2_ref(xf, i, j):
    """Float32 sum((a - b).^2), left to right, as the list build computes it."""
    d = xf[i] - xf[j]
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]


def _check_engine_lists(eng, oracle, x, r_list, sigma=1.0):
    """The engine's lists at its last build, as a set, against every pair with
    d^2 < r_list^2 on the same Float32 positions, and the near segment against
    d^2 < (1.3 sigma + 0.1)^2.  Up to 20,000 atoms the oracle is brute force
    (AllToAll); above, the directed lists must be symmetric and their half
    (i < j) must match the oracle's leaf-BVH traversal in count and 128-bit
    order-free hash of (i, j, bits(d))."""
    xf = np.asarray(x, np.float64).astype(np.float32)
    n = len(xf)
    pi, pj, near = eng.list_pairs()
    d2 = _dist2_ref(xf, pi - 1, pj - 1)
    rnb2 = np.float32((1.3 * sigma + 0.1) ** 2)
    assert np.array_equal(near.astype(bool), d2 < rnb2)
    got = np.sort(pi.astype(np.int64) * (n + 1) + pj)
    if n <= 20000:
        bi, bj, _ = oracle.brute_pairs(xf, np.float32(r_list), 0)
        exp = np.sort(np.concatenate([bi.astype(np.int64) * (n + 1) + bj,
                                      bj.astype(np.int64) * (n + 1) + bi]))
        assert got.shape == exp.shape, (got.shape, exp.shape)
        assert np.array_equal(got, exp)
        npairs = len(bi)
    else:
        assert np.array_equal(got, np.sort(pj.astype(np.int64) * (n + 1) + pi))
        h = pi < pj
        d = np.sqrt(d2[h])
        t = oracle.tree(xf, np.float32(r_list), 4, order=oracle.REF_ORDER_SPATIAL)
        cnt, hash_ref = oracle.leaf_traverse_hash(t, np.float32(r_list), 4)
        assert int(h.sum()) == cnt
        assert oracle.pair_hash(pi[h], pj[h], d) == hash_ref
        npairs = cnt
    return npairs, int(near.sum()) // 2


def test_md_neighbor_list_pair_set(nd, oracle):
    # The engine's own lists (the ones the dynamics use), at the first build
    # and at the rebuild after one window, equal as sets every pair with
    # d^2 < r_list^2 on the Float32 positions of that build (each pair in both
    # atoms' lists), near segments included; plain 4,096-atom LJ.
    x0, v0, _ = _config1(nd)
    eng = nd.MDEngine(_params(nd, 17.0), x0, v0)
    npairs, nnear = _check_engine_lists(eng, oracle, x0, np.float32(2.5 + 0.3))
    assert eng.stats()["list_pairs"] == 2 * npairs
    eng.run(10)
    eng.run(1)    # the rebuild at step 10, then one step
    eng2 = nd.MDEngine(_params(nd, 17.0), x0, v0)
    eng2.run(10)
    x10, _, _ = eng2.get()
    assert eng.diagnostics()["early_refits"] == 0
    npairs10, _ = _check_engine_lists(eng, oracle, x10, np.float32(2.5 + 0.3))
    print(f"engine lists: {npairs} pairs ({nnear} near) at step 0, {npairs10} at step 10")
    # reference-order pair list on the same Float32 positions, bit-exact
    xf = x10.astype(np.float32)
    b = oracle.brute_pairs(xf, np.float32(2.8), 0)
    spec = nd.SpheresBVHSpecs(2.8, len(xf), 4)
    p = nd.leafbuild_traverse_bvh(xf, spec)
    t = oracle.tree(xf, 2.8, 4)
    ri, rj, rd = oracle.leaf_traverse(t, 2.8, 4)
    assert np.array_equal(p["i"], ri) and np.array_equal(p["j"], rj)
    assert np.array_equal(p["d"].view(np.int32), rd.view(np.int32))
    assert np.array_equal(canon(p["i"], p["j"], p["d"]), canon(*b))


def test_config2_engine_vs_fp64(nd, oracle):
    # The benchmarked system: 262,144 atoms, side 68, charges +/-1, LJ +
    # Coulomb, r_c = 2.5, with the bench's engine settings (skin 0.4, eight
    # atoms per leaf).  Forces and energy at step 0 and after two rebuild
    # windows against FP64, the 20-step trajectory against the FP64
    # integrator, and the lists at the first build as a set.
    n, side = 262144, 68.0
    x0, v0, q = nd.synth.lj_system(0x4E440002, n, side, 0.8, charges=True)
    eng = nd.MDEngine(_params(nd, side, coulomb=1.0, skin=0.4, atomsperleaf=8), x0, v0, q)
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(side,) * 3, dt=1e-3)
    npairs, nnear = _check_engine_lists(eng, oracle, x0, np.float32(2.5 + 0.4))
    print(f"262k lists: {npairs} pairs, {nnear} near")
    _, _, f0 = eng.get()
    pe0, _ = eng.energy()
    f64, u64, _ = oracle.forces(p, x0, q)
    per_atom, l2 = force_errors(f0, f64)
    print(f"262k step 0: per-atom {per_atom:.3e}  L2 {l2:.3e}  energy {abs(pe0-u64)/abs(u64):.2e}")
    assert per_atom <= F_ATOM_TOL and l2 <= F_L2_TOL
    assert abs(pe0 - u64) <= 1e-6 * abs(u64)
    eng.run(20)
    xg, vg, fg = eng.get()
    pe1, _ = eng.energy()
    xr, vr, _ = oracle.md_run(p, x0, v0, q, steps=20)
    dx = np.abs(xg - xr).max()
    f64b, u64b, _ = oracle.forces(p, xg, q)
    per_atom_b, l2_b = force_errors(fg, f64b)
    print(f"262k step 20: max|dx| {dx:.2e}  per-atom {per_atom_b:.3e}  L2 {l2_b:.3e}")
    assert dx < 1e-5
    assert per_atom_b <= F_ATOM_TOL and l2_b <= F_L2_TOL
    assert abs(pe1 - u64b) <= 1e-6 * abs(u64b)
    assert eng.diagnostics()["skin_violations"] == 0


def test_md_graph_equals_eager_and_deterministic(nd):
    x0, v0, q = _config1(nd, charges=True, n=2048, side=13.5)
    a = nd.MDEngine(_params(nd, 13.5, coulomb=1.0), x0, v0, q)
    a.run(40)
    xa, va, fa = a.get()
    b = nd.MDEngine(_params(nd, 13.5, coulomb=1.0), x0, v0, q)
    for k in (7, 3, 11, 9, 10):
        b.run(k)
    xb, vb, fb = b.get()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    c = nd.MDEngine(_params(nd, 13.5, coulomb=1.0), x0, v0, q)
    c.run(40)
    xc, vc, _ = c.get()
    assert np.array_equal(xa, xc) and np.array_equal(va, vc)


@pytest.mark.parametrize("split", [2, 4])
def test_md_cta_split_same_bits(nd, split):
    """Four threads per atom with each block of 256 atoms spread over 2 or 4
    thread blocks: every atom sums the same slices in the same order, so
    positions, velocities and forces equal the unsplit engine's bit for bit
    (through rebuild windows, graphs and the measure pass)."""
    x0, v0, q = _config1(nd, charges=True, n=4096, side=17.0)
    a = nd.MDEngine(_params(nd, 17.0, coulomb=1.0, threads_per_atom=4, cta_split=1), x0, v0, q)
    a.run(35)
    xa, va, fa = a.get()
    pa, ka = a.energy()
    b = nd.MDEngine(_params(nd, 17.0, coulomb=1.0, threads_per_atom=4, cta_split=split),
                    x0, v0, q)
    b.run(35)
    xb, vb, fb = b.get()
    pb, kb = b.energy()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    # energies are summed with atomics (any order): equal to rounding
    assert abs(pa - pb) <= 1e-12 * abs(pa) and abs(ka - kb) <= 1e-12 * abs(ka)


def test_md_reference_order_matches_spatial(nd):
    # The order mode changes only the atom order, not the physics.
    x0, v0, _ = _config1(nd, n=2048, side=13.5)
    a = nd.MDEngine(_params(nd, 13.5, order=0), x0, v0)
    b = nd.MDEngine(_params(nd, 13.5, order=1), x0, v0)
    a.run(20)
    b.run(20)
    xa, _, _ = a.get()
    xb, _, _ = b.get()
    assert np.abs(xa - xb).max() < 1e-6


def test_md_walls(nd, oracle):
    # Eight atoms far apart (no interactions) fly into the walls of a box of
    # side 30: boundary_reflect! clamps the coordinate and flips the velocity.
    x0 = np.array([[5.0 + 3.2 * k, 4.0 * (k % 4) + 3.0, 6.0 * (k // 4) + 5.0] for k in range(8)])
    v0 = np.zeros((8, 3))
    v0[:, 0] = [-900.0, 700.0, -500.0, 300.0, 950.0, -650.0, 400.0, -800.0]
    p = _params(nd, 30.0, skin=50.0)
    eng = nd.MDEngine(p, x0, v0)
    eng.run(60)
    x, v, _ = eng.get()
    po = oracle.md_params(cutoff=2.5, box_hi=(30, 30, 30), dt=1e-3)
    xr, vr, _ = oracle.md_run(po, x0, v0, steps=60)
    assert x.min() >= 0.0 and x.max() <= 30.0
    assert np.array_equal(np.abs(v), np.abs(v0))
    assert np.array_equal(np.sign(v), np.sign(vr))
    assert np.abs(x - xr).max() < 1e-9


def test_md_skin_violations_counted(nd):
    # Atoms moving up to ~0.2 per step cross skin/2 = 0.15 in one step.  With
    # a check after every step each such step is followed by a refit (no step
    # runs on a stale list); with a check after every third step the steps in
    # between run on lists some atoms have left, and those are counted.
    x0, v0, _ = _config1(nd, n=512, side=8.5)
    d = {}
    for ce in (1, 3):
        eng = nd.MDEngine(_params(nd, 8.5, refit_check_every=ce), x0, v0 * 50.0)
        eng.run(10)
        eng.sync()
        d[ce] = eng.diagnostics()
        eng.close()
    assert d[1]["skin_violations"] == 0 and d[1]["early_refits"] > 0
    assert d[3]["skin_violations"] > 0
    # simulate! reports them to its caller (nd_simulate_diagnostics), and
    # stays silent with a check after every step
    import warnings
    for ce, expect in ((3, True), (1, False)):
        sys_ = nd.GenericObjectCollection(position=x0.copy(), velocity=v0 * 50.0)
        clct = nd.GenericRandomCollector(512, (0, 0, 0), (8.5, 8.5, 8.5))
        with warnings.catch_warnings(record=True) as w:
            warnings.simplefilter("always")
            nd.simulate_(sys_, nd.SimSpec(duration=10, stepwidth=1e-3), clct,
                         nd.ForceField(1.0, 1.0, 0.0, 2.5), refit_check_every=ce)
        hits = [x for x in w if issubclass(x.category, RuntimeWarning) and "skin/2" in str(x.message)]
        assert bool(hits) == expect, (ce, [str(x.message) for x in w])


def test_simulate_drop_in(nd, oracle):
    x0, v0, q = _config1(nd, charges=True, n=1024, side=10.7)
    sys_ = nd.GenericObjectCollection(position=x0, velocity=v0, charge=q)
    clct = nd.GenericRandomCollector(1024, (0, 0, 0), (10.7, 10.7, 10.7))
    nd.simulate_(sys_, nd.SimSpec(duration=30, stepwidth=1e-3), clct,
                 nd.ForceField(1.0, 1.0, 1.0, 2.5))
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(10.7, 10.7, 10.7), dt=1e-3)
    xr, vr, fr = oracle.md_run(p, x0, v0, q, steps=30)
    assert np.abs(sys_.position - xr).max() < 1e-6
    assert force_errors(sys_.force, fr)[1] <= F_L2_TOL


def test_md_masses(nd, oracle):
    x0, v0, _ = _config1(nd, n=1024, side=10.7)
    m = 1.0 + np.arange(1024) % 3
    eng = nd.MDEngine(_params(nd, 10.7), x0, v0, m=m)
    eng.run(20)
    x, v, _ = eng.get()
    p = oracle.md_params(cutoff=2.5, box_hi=(10.7, 10.7, 10.7), dt=1e-3)
    xr, vr, _ = oracle.md_run(p, x0, v0, m=m, steps=20)
    assert np.abs(x - xr).max() < 1e-6


def test_md_overflow_reported(nd):
    x0, v0, _ = _config1(nd, n=1024, side=10.7)
    with pytest.raises(nd.NDError) as e:
        eng = nd.MDEngine(_params(nd, 10.7, max_neighbors=8), x0, v0)
        eng.run(10)
        eng.sync()
    assert e.value.status == -8
    # a fresh engine on the same context still works
    eng = nd.MDEngine(_params(nd, 10.7), x0, v0)
    eng.run(10)
    eng.sync()

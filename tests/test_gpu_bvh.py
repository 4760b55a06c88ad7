"""GPU neighbour search (libnaivegpu through the C ABI) against the oracle.

Bit-exact: Morton codes, sort order, tree keys (boxes, left/skip ropes), and
the pair list (i, j, bits(d)) -- in the reference's serial emission order for
ND_PAIRS_ORDERED, as a multiset for ND_PAIRS_UNORDERED and the spatial order.
Cases follow test/BVHTraverse.jl's families plus edge cases.
"""
import numpy as np
import pytest

from conftest import canon
from helpers import golden_cases, uniform

pytestmark = pytest.mark.gpu


def _pairs_arr(p):
    return np.ascontiguousarray(p["i"]), np.ascontiguousarray(p["j"]), np.ascontiguousarray(p["d"])


def _exact(p, ref):
    pi, pj, pd = _pairs_arr(p)
    ri, rj, rd = ref
    assert len(pi) == len(ri)
    assert np.array_equal(pi, ri) and np.array_equal(pj, rj)
    assert np.array_equal(pd.view(np.int32), rd.view(np.int32))


def test_golden_vectors(nd):
    for c in golden_cases():
        x = np.array(c["position"], np.float32)
        spec = nd.SpheresBVHSpecs(c["r"], len(x), c["apl"])
        if c["boxes"] == "leaf":
            keys, pos, perm, _ = nd.leafTreeData(x, spec)
            pairs = nd.leafbuild_traverse_bvh(x, spec)
        else:
            keys, pos, perm, _ = nd.TreeData(x, spec)
            pairs = nd.build_traverse_bvh(x, spec)
        nl = spec.leaves_count
        assert list(perm) == c["perm"], c["name"]
        assert list(pos.index) == c["index"], c["name"]
        assert list(pos.morton_code) == c["code_sorted"], c["name"]
        for k, g in zip(keys[: 2 * nl - 1], c["keys"]):
            assert [float(v) for v in k["min"]] == g[0], c["name"]
            assert [float(v) for v in k["max"]] == g[1], c["name"]
            assert (int(k["left"]), int(k["skip"])) == (g[2], g[3]), c["name"]
        got = [[int(a), int(b), float(d)] for a, b, d in zip(pairs["i"], pairs["j"], pairs["d"])]
        assert got == c["pairs"], c["name"]


def _check_tree(nd, oracle, x, r, apl, order, boxes):
    spec = nd.SpheresBVHSpecs(r, len(x), apl)
    f = nd.leafTreeData if boxes == 0 else nd.TreeData
    keys, pos, perm, _ = f(x, spec, order=order)
    t = oracle.tree(x, r, apl, order=order, boxes=boxes)
    assert np.array_equal(perm, t["perm"] + 1)
    assert np.array_equal(pos.index, t["index"])
    assert np.array_equal(pos.morton_code, t["code"])
    assert np.array_equal(pos.position.view(np.int32), t["position"].view(np.int32))
    n = len(keys)
    assert np.array_equal(keys.view(np.int32).reshape(n, 8), t["keys"][:n].view(np.int32).reshape(n, 8))
    return spec, t


@pytest.mark.parametrize("r", [1e-4, 1e-3, 1e-2, 1e-1, 1.0])
def test_family_neighbor_distance(nd, oracle, r):
    # test/BVHTraverse.jl:225-243
    n = 5000 if r < 1.0 else 2000
    x = uniform(5000, n)
    for order in (0, 1):
        spec, t = _check_tree(nd, oracle, x, r, 4, order, 0)
        _exact(nd.leafbuild_traverse_bvh(x, spec, order=order), oracle.leaf_traverse(t, r, 4))
        un = nd.leafbuild_traverse_bvh(x, spec, order=order, mode=nd.ND_PAIRS_UNORDERED)
        assert np.array_equal(canon(*_pairs_arr(un)), canon(*oracle.leaf_traverse(t, r, 4)))
        spec, ta = _check_tree(nd, oracle, x, r, 4, order, 1)
        _exact(nd.build_traverse_bvh(x, spec, order=order), oracle.atom_traverse(ta, r, 4))


@pytest.mark.parametrize("apl", [1, 2, 4, 5, 10, 20, 1000])
def test_family_atomsperleaf(nd, oracle, apl):
    # test/BVHTraverse.jl:246-265
    x = uniform(5001, 5000)
    spec, ta = _check_tree(nd, oracle, x, 0.1, apl, 0, 1)
    _exact(nd.build_traverse_bvh(x, spec), oracle.atom_traverse(ta, 0.1, apl))
    if apl == 1:
        with pytest.raises(nd.SpecError):
            nd.leafbuild_traverse_bvh(x, spec)
        return
    spec, t = _check_tree(nd, oracle, x, 0.1, apl, 0, 0)
    _exact(nd.leafbuild_traverse_bvh(x, spec), oracle.leaf_traverse(t, 0.1, apl))


@pytest.mark.parametrize("n", [10, 100, 1000, 2000, 3000, 20000])
def test_family_positions(nd, oracle, n):
    # test/BVHTraverse.jl:268-287 (atomsperleaf = 5, r = 0.1)
    x = uniform(n, n)
    spec, t = _check_tree(nd, oracle, x, 0.1, 5, 0, 0)
    pairs = nd.leafbuild_traverse_bvh(x, spec)
    _exact(pairs, oracle.leaf_traverse(t, 0.1, 5))
    b = oracle.brute_pairs(x, 0.1, 0)
    assert np.array_equal(canon(*_pairs_arr(pairs)), canon(*b))


def test_position8_fixture(nd, oracle):
    # test/BVHTraverse.jl:165-220: TreeData of the eight hand-placed points at
    # r = 10, one atom per leaf; the skip ropes, the root box, every atom
    # paired, and (:205-209) the per-atom traversal's list sorted by (i, j)
    # equal to threshold_pairs(unique_pairs(position8), 10) -- indices and the
    # Float32 distances sqrt(sum((a - b).^2)) of AllToAll.jl -- on the GPU
    # and on the oracle.
    x = np.array([[0.1, 0.1, 0.1], [0.2, 0.2, 0.2], [0.346, 0.98, 0.12], [0.01, 0.76, 0.99],
                  [0.1111, 0.4, 0.31], [0.234, 0.29, 0.2], [0.11346, 0.918, 0.1276],
                  [0.061, 0.76, 0.989]], np.float32)
    spec = nd.SpheresBVHSpecs(10.0, 8, 1)
    keys, pos, perm, _ = nd.TreeData(x, spec)
    assert keys[7]["skip"] == 0 and all(keys[k]["skip"] != 0 for k in range(7))
    assert np.all(keys[8]["min"] < x) and np.all(x < keys[8]["max"])
    naive = oracle.brute_pairs(x, 10.0, criterion=1)  # unique_pairs + threshold_pairs (d < 10)
    assert len(naive[0]) == 28
    t = oracle.tree(x, 10.0, 1, boxes=oracle.REF_BOX_ATOM)
    for lst in (_pairs_arr(nd.build_traverse_bvh(x, spec)), oracle.atom_traverse(t, 10.0, 1)):
        i, j, d = (np.asarray(a) for a in lst)
        paired = np.zeros(9, bool)
        paired[i] = True
        paired[j] = True
        assert paired[1:].all()
        a, b = np.minimum(i, j), np.maximum(i, j)
        o = np.lexsort((b, a))  # sort!(list, by=x->x[2]); sort!(list, by=x->x[1])
        assert np.array_equal(a[o], naive[0]) and np.array_equal(b[o], naive[1])
        assert np.array_equal(d[o].view(np.int32), naive[2].view(np.int32))
    res = nd.gpubvh_neighborlist(None, x, nd.SpheresBVHSpecs(10.0, 8, 2))
    assert len(res.pairlist) == 28


@pytest.mark.parametrize("order", [0, 1])
def test_gpubvh_neighborlist_refresh(nd, oracle, order):
    # gpubvh_neighborlist!(neighborlist, treedata, spec, backend): the list of
    # moved positions from the kept tree (same order and codes, new boxes);
    # ordered emission bit-exact against the oracle's leaf traversal over the
    # kept-order tree, the tree and positions written back into treedata, and
    # the pair set equal to a fresh build's.
    x = uniform(0x4E440051, 4096, 1.0)
    spec = nd.SpheresBVHSpecs(0.05, len(x), 4)
    res = nd.gpubvh_neighborlist(None, x, spec, order=order)
    keys, mpos, perm, _ = res.treedata
    code0 = mpos.morton_code.copy()
    rng = np.random.default_rng(7)
    y = (x + rng.normal(0.0, 0.004, x.shape)).astype(np.float32)
    lst = res.pairlist
    out = nd.gpubvh_neighborlist_(lst, res.treedata, spec, None, position=y)
    assert out.pairlist is lst  # filled in place
    t = oracle.tree_kept(y, 0.05, 4, mpos.index, code0)
    _exact(out.pairlist, oracle.leaf_traverse(t, 0.05, 4))
    n = len(keys)
    assert np.array_equal(out.treedata[0].view(np.int32).reshape(n, 8),
                          t["keys"][:n].view(np.int32).reshape(n, 8))
    assert np.array_equal(out.treedata[1].position, t["position"])
    fresh = oracle.leafbuild_traverse_bvh(y, 0.05, 4)
    assert np.array_equal(canon(*_pairs_arr(out.pairlist)), canon(*fresh))
    # positions written into treedata by the caller (the in-place form)
    z = (y + rng.normal(0.0, 0.004, y.shape)).astype(np.float32)
    out.treedata[1].position[...] = z[out.treedata[1].index - 1]
    again = nd.gpubvh_neighborlist_(None, out.treedata, spec, None)
    t2 = oracle.tree_kept(z, 0.05, 4, mpos.index, code0)
    _exact(again.pairlist, oracle.leaf_traverse(t2, 0.05, 4))
    un = nd.gpubvh_neighborlist_(None, again.treedata, spec, None, position=z,
                                 mode=nd.ND_PAIRS_UNORDERED)
    assert np.array_equal(canon(*_pairs_arr(un.pairlist)), canon(*oracle.leaf_traverse(t2, 0.05, 4)))
    # a kept order that is not a permutation is refused
    bad = (keys, nd.APointPrimitive(mpos.index.copy(), code0, mpos.position), perm, None)
    bad[1].index[0] = bad[1].index[1]
    with pytest.raises(nd.NDError):
        nd.gpubvh_neighborlist_(None, bad, spec, None, position=z)


def test_degenerate_inputs(nd, oracle):
    # all atoms on one point: every code equal, exptdelta falls back to the
    # leaf-index tie-break (BVHTraverse.jl:693); every pair at distance 0.
    x = np.full((64, 3), 0.25, np.float32)
    spec, t = _check_tree(nd, oracle, x, 0.1, 4, 0, 0)
    p = nd.leafbuild_traverse_bvh(x, spec)
    assert len(p) == 64 * 63 // 2
    _exact(p, oracle.leaf_traverse(t, 0.1, 4))
    # duplicated blocks, negative coordinates, r = 0 (no pair)
    y = np.concatenate([uniform(2, 32), uniform(2, 32)]) - 0.5
    spec, t = _check_tree(nd, oracle, y, 0.3, 4, 0, 0)
    _exact(nd.leafbuild_traverse_bvh(y, spec), oracle.leaf_traverse(t, 0.3, 4))
    assert len(nd.leafbuild_traverse_bvh(y, nd.SpheresBVHSpecs(0.0, 64, 4))) == 0


def test_simdbuild_traverse_bvh(nd, oracle):
    # simdbuild_traverse_bvh: the leafbuild tree and order with sqrt(d^2) < r,
    # bit for bit against the oracle (radii whose sqrt threshold lies one ulp
    # under fl(r * r) and one where they coincide), and on the boundary pair
    from test_oracle import boundary_positions
    x = uniform(92, 8192)
    for r in (0.05, 0.1, 0.3, 0.0731):
        spec = nd.SpheresBVHSpecs(r, len(x), 4)
        p = nd.simdbuild_traverse_bvh(x, spec)
        t = oracle.tree(x, r, 4)
        ri, rj, rd = oracle.simd_leaf_traverse(t, r, 4)
        assert np.array_equal(p["i"], ri) and np.array_equal(p["j"], rj)
        assert np.array_equal(p["d"].view(np.int32), rd.view(np.int32))
        pu = nd.simdbuild_traverse_bvh(x, spec, mode=nd.ND_PAIRS_UNORDERED)
        assert np.array_equal(canon(pu["i"], pu["j"], pu["d"]), canon(ri, rj, rd))
    xb = boundary_positions()
    spec = nd.SpheresBVHSpecs(0.1, len(xb), 4)
    s0 = {tuple(r) for r in canon(*(nd.leafbuild_traverse_bvh(xb, spec)[k] for k in "ijd"))}
    s1 = {tuple(r) for r in canon(*(nd.simdbuild_traverse_bvh(xb, spec)[k] for k in "ijd"))}
    assert len(s0 - s1) == 1 and not (s1 - s0)
    with pytest.raises(nd.SpecError):
        nd.simdbuild_traverse_bvh(x, nd.SpheresBVHSpecs(0.05, len(x), 2))


def test_errors(nd):
    x = uniform(1, 64)
    spec = nd.SpheresBVHSpecs(0.1, 64, 4)
    x[5, 2] = np.nan
    with pytest.raises(nd.InexactError):
        nd.leafbuild_traverse_bvh(x, spec)
    x = uniform(1, 64)
    x[7, 0] = 3.0e6
    with pytest.raises(nd.InexactError):
        nd.leafTreeData(x, spec)
    # the context stays usable after a reported error
    assert len(nd.leafbuild_traverse_bvh(uniform(1, 64), spec)) >= 0


def test_capacity_protocol(nd, oracle):
    import ctypes
    from naivedynamics import _lib
    x = uniform(9, 2000)
    spec = nd.SpheresBVHSpecs(0.1, 2000, 4)
    ctx = nd.default_context()
    cs = spec.c_spec()
    cnt = ctypes.c_int64()
    st = _lib.lib().nd_leaf_pairs(ctx.handle, x.ctypes.data, ctypes.byref(cs), 0, 0, None, None,
                                  None, 0, ctypes.byref(cnt))
    assert st == _lib.ND_NEED_REALLOC
    assert cnt.value == len(oracle.brute_pairs(x, 0.1, 0)[0])
    small = cnt.value - 1
    pi = np.full(small, -7, np.int32)
    st = _lib.lib().nd_leaf_pairs(ctx.handle, x.ctypes.data, ctypes.byref(cs), 0, 0,
                                  pi.ctypes.data, np.empty(small, np.int32).ctypes.data,
                                  np.empty(small, np.float32).ctypes.data, small,
                                  ctypes.byref(cnt))
    assert st == _lib.ND_NEED_REALLOC and (pi == -7).all()


def test_device_pointer_api(nd, oracle):
    import torch
    x = uniform(21, 4096, 17.0)
    xt = torch.from_numpy(x).cuda()
    codes = torch.empty(4096, dtype=torch.int32, device="cuda")
    from naivedynamics import _lib
    ctx = nd.default_context()
    ctx.check(_lib.lib().nd_morton_codes_dev(ctx.handle, xt.data_ptr(), 4096, 0, codes.data_ptr()))
    ref = oracle.morton_reference(x)
    assert np.array_equal(codes.cpu().numpy(), ref)
    perm = torch.empty(4096, dtype=torch.int32, device="cuda")
    ctx.check(_lib.lib().nd_sortperm_dev(ctx.handle, codes.data_ptr(), 4096, perm.data_ptr()))
    assert np.array_equal(perm.cpu().numpy(), oracle.sortperm(ref))
    assert np.array_equal(codes.cpu().numpy(), np.sort(ref, kind="stable"))
    spec = nd.SpheresBVHSpecs(2.8, 4096, 4)
    t = oracle.tree(x, 2.8, 4, order=1)
    cnt_ref, h_ref = oracle.leaf_traverse_hash(t, 2.8, 4)
    cap = cnt_ref + 10
    pi = torch.empty(cap, dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    pd = torch.empty(cap, dtype=torch.float32, device="cuda")
    st, cnt = nd.neighbor_pairs_dev(xt, spec, pi, pj, pd, cap, order=1)
    assert st == 0 and cnt == cnt_ref
    assert nd.pair_hash_dev(pi, pj, pd, cnt) == h_ref


def test_config1_reference_order_exact(nd, oracle):
    # 4096 atoms in a cube of side 17 at the list radius 2.8: reference order,
    # bit-exact list in the reference's serial emission order.
    x = uniform(0x4E440001, 4096, 17.0)
    spec, t = _check_tree(nd, oracle, x, 2.8, 4, 0, 0)
    _exact(nd.leafbuild_traverse_bvh(x, spec), oracle.leaf_traverse(t, 2.8, 4))


def test_config2_positions_hash(nd, oracle):
    # 262,144 atoms in a cube of side 68 at r = 2.8, spatial order: count and
    # order-free hash equal the oracle's (reference-order traversal at this size
    # visits nearly every leaf, see the leaf-extent note in the design notes).
    import torch
    n = 262144
    x = nd.synth.uniform_positions(0x4E440002, n, 68.0)
    t = oracle.tree(x, 2.8, 4, order=1)
    cnt_ref, h_ref = oracle.leaf_traverse_hash(t, 2.8, 4)
    spec = nd.SpheresBVHSpecs(2.8, n, 4)
    xt = torch.from_numpy(x).cuda()
    pi = torch.empty(cnt_ref, dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    pd = torch.empty(cnt_ref, dtype=torch.float32, device="cuda")
    for mode in (nd.ND_PAIRS_UNORDERED, nd.ND_PAIRS_ORDERED):
        st, cnt = nd.neighbor_pairs_dev(xt, spec, pi, pj, pd, cnt_ref, order=1, mode=mode)
        assert st == 0 and cnt == cnt_ref
        assert nd.pair_hash_dev(pi, pj, pd, cnt) == h_ref


def test_ns_stress_reduced(nd, oracle):
    # The neighbour-search stress shape (64 Gaussian clusters, centres in a cube
    # of side 400, sigma in [2, 10], r = 2.5) at 1/16 of the points.
    import torch
    n = 64 * 4096
    x = nd.synth.cluster_positions(0x4E440003, n, 64, 400.0, 2.0, 10.0)
    t = oracle.tree(x, 2.5, 4, order=1)
    cnt_ref, h_ref = oracle.leaf_traverse_hash(t, 2.5, 4)
    spec = nd.SpheresBVHSpecs(2.5, n, 4)
    xt = torch.from_numpy(x).cuda()
    pi = torch.empty(cnt_ref, dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    pd = torch.empty(cnt_ref, dtype=torch.float32, device="cuda")
    st, cnt = nd.neighbor_pairs_dev(xt, spec, pi, pj, pd, cnt_ref, order=1)
    assert st == 0 and cnt == cnt_ref
    assert nd.pair_hash_dev(pi, pj, pd, cnt) == h_ref
    # full materialised compare on a random subset of query atoms
    a = pi[:cnt].cpu().numpy()
    b = pj[:cnt].cpu().numpy()
    d = pd[:cnt].cpu().numpy()
    sel = np.random.default_rng(0).choice(n, 200, replace=False) + 1
    m = np.isin(np.minimum(a, b), sel)
    tl = oracle.leaf_traverse(t, 2.5, 4)
    mr = np.isin(np.minimum(tl[0], tl[1]), sel)
    assert np.array_equal(canon(a[m], b[m], d[m]), canon(tl[0][mr], tl[1][mr], tl[2][mr]))


def test_ns_stress_full(nd, oracle):
    # The neighbour-search stress configuration at full size: 4,194,304 points
    # (64 clusters x 65,536), r = 2.5, ~2.6e9 half pairs written to device
    # memory (31 GB); exact pair count and order-free 128-bit hash of every
    # canonical (min, max, bits(d)) triple against the oracle's traversal.
    import torch
    n = 64 * 65536
    x = nd.synth.cluster_positions(0x4E440003, n, 64, 400.0, 2.0, 10.0)
    t = oracle.tree(x, 2.5, 4, order=1)
    cnt_ref, h_ref = oracle.leaf_traverse_hash(t, 2.5, 4)
    del t
    spec = nd.SpheresBVHSpecs(2.5, n, 4)
    xt = torch.from_numpy(x).cuda()
    st, cnt = nd.neighbor_pairs_dev(xt, spec, None, None, None, 0, order=1)
    assert st == nd._lib.ND_NEED_REALLOC and cnt == cnt_ref
    pi = torch.empty(cnt, dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    pd = torch.empty(cnt, dtype=torch.float32, device="cuda")
    st, cnt2 = nd.neighbor_pairs_dev(xt, spec, pi, pj, pd, cnt, order=1)
    assert st == 0 and cnt2 == cnt_ref
    assert nd.pair_hash_dev(pi, pj, pd, cnt2) == h_ref
    del pi, pj, pd
    torch.cuda.empty_cache()

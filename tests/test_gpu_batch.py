"""Batched ensembles (nd_batch_create) against the FP64 oracle, system by system.

Systems of uneven sizes, densities, sigma and epsilon are advanced by one
engine; each system must behave exactly as if it were alone:
  * forces: per system relative L2 error <= 1e-5 against the FP64 oracle run on
    that system alone (so no pair crosses systems and every system uses its
    own sigma/epsilon), per-atom error <= 1e-5 with the 1e-3 rms floor;
  * energies: per-system potential within 1e-6 (relative) of the oracle's,
    kinetic energy exact to 1e-12;
  * dynamics: 60 steps (dt = 1e-3, rebuild every 10, walls per system) within
    1e-5 of each system's FP64 trajectory;
  * the batched run agrees with the same systems run one by one through the
    plain engine (differences only from force summation order).
"""
import numpy as np
import pytest

from helpers import force_errors

pytestmark = pytest.mark.gpu

F_L2_TOL = 1e-5
F_ATOM_TOL = 1e-5


def _ensemble(nd, nsys=24, nmin=256, nmax=2048, seed=0x4E440004):
    return nd.synth.ensemble(seed, nsys=nsys, nmin=nmin, nmax=nmax)


def _params(nd, **kw):
    a = dict(cutoff=2.5, skin=0.3, dt=1e-3, atomsperleaf=4, rebuild_every=10)
    a.update(kw)
    return nd.md_params(**a)


def _table(nd, e):
    return nd.systems_table(e["n_atoms"], e["sigma"], e["epsilon"], e["box_lo"], e["box_hi"])


def _slices(e):
    off = np.concatenate([[0], np.cumsum(e["n_atoms"])])
    return [slice(int(off[k]), int(off[k + 1])) for k in range(len(e["n_atoms"]))]


def _oracle_params(oracle, e, k, dt=1e-3):
    return oracle.md_params(sigma=float(e["sigma"][k]), epsilon=float(e["epsilon"][k]),
                            cutoff=2.5, box_lo=tuple(e["box_lo"][k]),
                            box_hi=tuple(e["box_hi"][k]), dt=dt)


def test_batch_forces_and_energies_per_system(nd, oracle):
    e = _ensemble(nd)
    eng = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    _, _, f = eng.get()
    pe, ke = eng.energies()
    worst = 0.0
    for k, sl in enumerate(_slices(e)):
        f64, u64, _ = oracle.forces(_oracle_params(oracle, e, k), e["x"][sl])
        per_atom, l2 = force_errors(f[sl], f64)
        worst = max(worst, l2)
        assert l2 <= F_L2_TOL, (k, l2)
        assert per_atom <= F_ATOM_TOL, (k, per_atom)
        assert abs(pe[k] - u64) <= 1e-6 * abs(u64), (k, pe[k], u64)
        kk = 0.5 * (e["v"][sl] ** 2).sum()
        assert abs(ke[k] - kk) <= 1e-12 * kk
    tot_pe, tot_ke = eng.energy()
    assert abs(tot_pe - pe.sum()) <= 1e-9 * abs(pe.sum())
    assert abs(tot_ke - ke.sum()) <= 1e-9 * ke.sum()
    print(f"worst per-system force L2 error {worst:.2e} over {len(pe)} systems")


def slot_offset(e, k, r_list):
    """Translation of system k into the ensemble's tree frame: slots of side
    (largest extent + 2 r_list + 1) on a G x G x G grid (G the smallest power
    of two with G^3 >= systems), system k in slot (k mod G, k / G mod G,
    k / G^2) with half the gap below it."""
    ns = len(e["n_atoms"])
    side_max = float(np.max(e["box_hi"] - e["box_lo"]))
    gap = 2.0 * r_list + 1.0
    slot = side_max + gap
    g = 1
    while g * g * g < ns:
        g *= 2
    cell = (k % g, (k // g) % g, k // (g * g))
    return np.array([cell[d] * slot + 0.5 * gap - float(e["box_lo"][k][d]) for d in range(3)])


def test_full_ensemble_vs_fp64(nd, oracle):
    # The benchmarked ensemble: 512 systems of 256-16,384 atoms (log-uniform),
    # density 0.6-0.9, sigma 0.9-1.1, eps 0.8-1.2.  Every system's forces and
    # potential energy against the FP64 oracle run on that system alone, at
    # step 0 and after 20 steps (two rebuilds); the lists of the systems of up
    # to 4,096 atoms at the first build as sets.
    e = nd.synth.ensemble()
    assert len(e["n_atoms"]) == 512
    eng = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    sl = _slices(e)
    pi, pj, near = eng.list_pairs()
    off = np.concatenate([[0], np.cumsum(e["n_atoms"])])
    sys_of = np.searchsorted(off, pi - 1, side="right") - 1
    assert np.array_equal(sys_of, np.searchsorted(off, pj - 1, side="right") - 1)
    rl = np.float32(2.5 + 0.3)
    xt = None
    worst = [0.0, 0.0, 0.0]
    for t in (0, 20):
        if t:
            eng.run(t)
        x, _, f = eng.get()
        pe, _ = eng.energies()
        for k, s_ in enumerate(sl):
            p = _oracle_params(oracle, e, k)
            f64, u64, _ = oracle.forces(p, x[s_])
            per_atom, l2 = force_errors(f[s_], f64)
            worst = [max(worst[0], per_atom), max(worst[1], l2),
                     max(worst[2], abs(pe[k] - u64) / abs(u64))]
            assert per_atom <= F_ATOM_TOL and l2 <= F_L2_TOL, (t, k, per_atom, l2)
            assert abs(pe[k] - u64) <= 1e-6 * abs(u64), (t, k)
            if t == 0 and e["n_atoms"][k] <= 4096:
                # this system's lists: every pair within r_list of its
                # Float32 positions in the ensemble's tree frame (the system
                # translated into its slot, then rounded), near entries below
                # (1.3 sigma + 0.1); brute force on the systems of up to 4,096
                # atoms
                m = sys_of == k
                xf = (e["x"][s_] + slot_offset(e, k, 2.5 + 0.3)).astype(np.float32)
                bi, bj, _ = oracle.brute_pairs(xf, rl, 0)
                n = len(xf)
                a, b = pi[m] - 1 - off[k], pj[m] - 1 - off[k]
                got = np.sort(a.astype(np.int64) * (n + 1) + b)
                exp = np.sort(np.concatenate([(bi - 1).astype(np.int64) * (n + 1) + bj - 1,
                                              (bj - 1).astype(np.int64) * (n + 1) + bi - 1]))
                assert np.array_equal(got, exp), k
                d = xf[a] - xf[b]
                d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
                rnb2 = np.float32((1.3 * float(e["sigma"][k]) + 0.1) ** 2)
                assert np.array_equal(near[m].astype(bool), d2 < rnb2), k
    print(f"512-system ensemble vs FP64: worst per-atom {worst[0]:.3e}  L2 {worst[1]:.3e}  "
          f"energy {worst[2]:.2e}")
    assert eng.diagnostics()["skin_violations"] == 0


def test_batch_trajectory_per_system(nd, oracle):
    e = _ensemble(nd, nsys=12, nmax=1024)
    eng = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    eng.run(60)
    eng.sync()
    x, v, _ = eng.get()
    worst = 0.0
    for k, sl in enumerate(_slices(e)):
        xr, vr, _ = oracle.md_run(_oracle_params(oracle, e, k), e["x"][sl], e["v"][sl], steps=60)
        dx = float(np.abs(x[sl] - xr).max())
        worst = max(worst, dx)
        assert dx < 1e-5, (k, dx)
        # walls hold per system
        assert (x[sl] >= e["box_lo"][k] - 1e-12).all() and (x[sl] <= e["box_hi"][k] + 1e-12).all()
    assert eng.diagnostics()["skin_violations"] == 0
    st = eng.stats()
    assert st["steps"] == 60 and st["rebuilds"] == 6
    print(f"60-step batched trajectory: worst max|dx| {worst:.2e}")


def test_batch_matches_plain_engines(nd):
    e = _ensemble(nd, nsys=8, nmax=1024, seed=0x4E440014)
    b = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    b.run(30)
    xb, vb, fb = b.get()
    for k, sl in enumerate(_slices(e)):
        side = float(e["box_hi"][k][0])
        p = _params(nd, sigma=float(e["sigma"][k]), epsilon=float(e["epsilon"][k]),
                    box_lo=(0, 0, 0), box_hi=(side, side, side))
        a = nd.MDEngine(p, e["x"][sl], e["v"][sl])
        a.run(30)
        xa, va, fa = a.get()
        assert np.abs(xa - xb[sl]).max() < 2e-6
        assert np.abs(va - vb[sl]).max() < 1e-4
        a.close()


def test_batch_deterministic_and_graph_equals_eager(nd):
    e = _ensemble(nd, nsys=10, nmax=1024, seed=0x4E440024)
    a = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    a.run(50)
    xa, va, _ = a.get()
    b = nd.Ensemble(_params(nd), _table(nd, e), e["x"], e["v"])
    for k in (3, 17, 10, 20):
        b.run(k)
    xb, vb, _ = b.get()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_batch_resort_schedules_agree(nd):
    e = _ensemble(nd, nsys=6, nmax=1024, seed=0x4E440034)
    out = []
    for rs in (1, 5):
        eng = nd.Ensemble(_params(nd, resort_every=rs), _table(nd, e), e["x"], e["v"])
        eng.run(40)
        out.append(eng.get()[0])
    assert np.abs(out[0] - out[1]).max() < 2e-6


def test_batch_union_searches_agree(nd):
    # blocks of 256 atoms straddle systems here; both union searches must
    # still find the same leaves
    e = _ensemble(nd, nsys=20, nmax=1500, seed=0x4E440044)
    out = []
    for us in (nd.ND_UNION_BLOCKS, nd.ND_UNION_TREE):
        eng = nd.Ensemble(_params(nd, union_search=us, resort_every=2), _table(nd, e), e["x"],
                          e["v"])
        eng.run(40)
        out.append(eng.get())
        eng.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_batch_errors(nd):
    e = _ensemble(nd, nsys=4, nmax=512)
    t = _table(nd, e)
    t[1].n_atoms = t[1].n_atoms - 2  # not a whole number of leaves
    x = e["x"][: int(sum(r.n_atoms for r in t))]
    v = e["v"][: len(x)]
    with pytest.raises(nd.SpecError):
        nd.Ensemble(_params(nd), t, x, v)
    t = _table(nd, e)
    t[2].box_hi[0] = t[2].box_lo[0]  # empty box
    with pytest.raises(nd.NDError):
        nd.Ensemble(_params(nd), t, e["x"], e["v"])


def test_autotune_plain_and_batch(nd, tmp_path, monkeypatch):
    monkeypatch.setenv("ND_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    x0, v0, _ = nd.synth.lj_system(0x4E440001, 4096, 17.0, 0.8)
    p = _params(nd, box_lo=(0, 0, 0), box_hi=(17, 17, 17))
    best, sps = nd.autotune(p, x0, v0, trial_steps=20)
    assert not nd.autotune.last_cached
    assert best.threads_per_atom in (1, 2, 4)
    # the second call reads the cache: same settings, nothing timed
    again, sps2 = nd.autotune(p, x0, v0, trial_steps=20)
    assert nd.autotune.last_cached and sps2 == sps
    assert all(getattr(again, k) == getattr(best, k) for k in nd.TUNED_FIELDS)
    assert again.cutoff == p.cutoff and list(again.box_hi) == list(p.box_hi)
    # another density is another key
    x1, v1, _ = nd.synth.lj_system(0x4E440001, 4096, 18.0, 0.8)
    nd.autotune(_params(nd, box_lo=(0, 0, 0), box_hi=(18, 18, 18)), x1, v1, trial_steps=20)
    assert not nd.autotune.last_cached
    assert best.atomsperleaf in (2, 4, 8) and best.resort_every in (1, 5, 10)
    assert best.stage_policy in (0, 1) and best.union_search in (0, 1) and sps > 0
    # skin candidates: the given one -0.2 .. +0.2 in steps of 0.1, not below 0.1
    assert abs(best.skin - p.skin) < 0.25 and best.skin >= max(0.1, p.skin - 0.2) - 1e-9
    assert best.cutoff == p.cutoff and best.rebuild_every == p.rebuild_every
    e = _ensemble(nd, nsys=16, nmax=1024)
    t = _table(nd, e)
    best, sps = nd.autotune(_params(nd), e["x"], e["v"], systems=t, trial_steps=20)
    assert best.atomsperleaf in (2, 4) and sps > 0
    eng = nd.Ensemble(best, t, e["x"], e["v"])
    eng.run(20)
    eng.sync()

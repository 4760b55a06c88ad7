"""simulate! as written (Simulator.jl:154-256) on the GPU against the oracle.

The device form runs the all-pairs list with a row-per-atom Lennard-Jones
pass and the Coulomb recurrence as levels of the list; the oracle runs the
reference's loops literally (threshold_pairs compaction, every force call
twice, one pair at a time).  Results are compared bit for bit: positions,
velocities, forces and every logged frame (NaN compared as NaN: the
reference's own dynamics can produce them once two atoms are clamped into
the same wall corner).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX = ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))


def _bits(a):
    a = np.array(a, np.float32, copy=True)
    a[np.isnan(a)] = np.nan
    return a.view(np.int32)


def _collect(seed, n, temperature, qmax, randomvelocity):
    """Initial conditions shaped like collect_objects (MDInput.jl:305-369):
    uniform masses in [1, 5), charges in [-qmax, qmax), positions in the unit
    box, velocities T / N * 3N / m per component (or a normalised random
    split of that budget)."""
    rng = np.random.default_rng(seed)
    m = rng.uniform(1.0, 5.0, n).astype(np.float32)
    q = rng.uniform(-qmax, qmax, n).astype(np.float32)
    x = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    T = np.float32(temperature)
    if randomvelocity:
        v = np.empty((n, 3), np.float32)
        for k in range(3):
            vd = rng.random(n, dtype=np.float32)
            vd = vd / vd.sum(dtype=np.float32)
            v[:, k] = T * vd * np.float32(3 * n) / m
    else:
        v = np.repeat((T / np.float32(n) * np.float32(3 * n) / m)[:, None], 3, axis=1)
    return x, v, m, q


def _run_both(nd, oracle, n, seed, dt, duration, vdamp, temperature, qmax, randomvelocity):
    x, v, m, q = _collect(seed, n, temperature, qmax, randomvelocity)
    sys = nd.GenericObjectCollection(x, v, mass=m, charge=q)
    spec = nd.SimSpec(duration=duration, stepwidth=dt, vDamp=vdamp)
    clct = nd.GenericRandomCollector(objectnumber=n, minDim=BOX[0], maxDim=BOX[1],
                                     temperature=temperature)
    err = None
    try:
        log = nd.simulate_compat_(sys, spec, clct)
    except nd.NDError as e:
        err, log = e, None
    ref = oracle.compat_simulate(x, v, np.zeros((n, 3)), m, q, BOX[0], BOX[1], temperature, n,
                                 dt, duration, vdamp)
    return sys, log, err, ref


CASES = [
    # n, seed, stepwidth, duration, vDamp, temperature, |q| max, random velocities
    (1, 11, 1, 5, 1.0, 0.01, 1e-9, False),
    (2, 12, 1, 12, 1.0, 0.01, 1e-9, False),
    (300, 13, 1, 25, 1.0, 0.01, 1e-9, False),   # the reference scripts' collector
    (517, 14, 2, 21, 0.5, 0.02, 1.0, True),     # unit charges: Coulomb dominates
    (1100, 15, 1, 11, 1.0, 0.05, 0.1, True),    # > 1024 atoms: several pairs per level
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"n{c[0]}")
def test_compat_simulate_bit_exact(nd, oracle, case):
    n, seed, dt, duration, vdamp, T, qmax, rv = case
    sys, log, err, (xo, vo, fo, logo, st) = _run_both(nd, oracle, n, seed, dt, duration, vdamp,
                                                     T, qmax, rv)
    assert err is None and st == 0
    assert np.array_equal(_bits(sys.position), _bits(xo))
    assert np.array_equal(_bits(sys.velocity), _bits(vo))
    assert np.array_equal(_bits(sys.force), _bits(fo))
    assert np.array_equal(_bits(log), _bits(logo))
    # the run moved and the first frames are finite
    assert np.all(np.isfinite(log[1])) and not np.array_equal(log[1], log[duration])
    if n > 1:
        assert np.any(sys.force != 0)


def test_compat_simulate_offset_box(nd, oracle):
    # walls at negative and unequal coordinates, stepwidth 3 (dt^2 = 9)
    lo, hi = (-2.0, -0.5, 1.0), (-1.0, 0.75, 1.5)
    rng = np.random.default_rng(77)
    n = 333
    x = (np.array(lo) + rng.random((n, 3)) * (np.array(hi) - np.array(lo))).astype(np.float32)
    v = rng.uniform(-0.01, 0.01, (n, 3)).astype(np.float32)
    m = rng.uniform(1.0, 5.0, n).astype(np.float32)
    q = rng.uniform(-0.1, 0.1, n).astype(np.float32)
    sys = nd.GenericObjectCollection(x, v, mass=m, charge=q)
    clct = nd.GenericRandomCollector(objectnumber=n, minDim=lo, maxDim=hi, temperature=0.02)
    log = nd.simulate_compat_(sys, nd.SimSpec(duration=13, stepwidth=3, vDamp=0.7), clct)
    xo, vo, fo, logo, st = oracle.compat_simulate(x, v, np.zeros((n, 3)), m, q, lo, hi, 0.02, n,
                                                  3, 13, 0.7)
    assert st == 0
    assert np.array_equal(_bits(log), _bits(logo))
    assert np.array_equal(_bits(sys.velocity), _bits(vo))
    assert np.array_equal(_bits(sys.force), _bits(fo))


def test_compat_simulate_domain_error(nd, oracle):
    # gamma = 3 with Tf far below Ti: 1 + 3 (Tf / Ti - 1) < 0 at step 10
    sys, log, err, (xo, vo, fo, logo, st) = _run_both(nd, oracle, 64, 21, 1, 30, 3.0, 1e-9,
                                                     1e-9, False)
    assert st == 1 and err is not None
    assert np.array_equal(_bits(sys.position), _bits(xo))
    assert np.array_equal(_bits(sys.velocity), _bits(vo))
    assert np.array_equal(_bits(sys.force), _bits(fo))


def test_compat_simulate_global_form_and_log_chunks(nd, oracle, monkeypatch):
    # the Coulomb levels with accumulators in global memory (the form for
    # more than about 20,000 atoms) and a device log flushed every 4 frames
    monkeypatch.setenv("NAIVEGPU_COMPAT_GLOBAL", "1")
    monkeypatch.setenv("NAIVEGPU_COMPAT_LOG_CHUNK", "4")
    sys, log, err, (xo, vo, fo, logo, st) = _run_both(nd, oracle, 300, 31, 1, 14, 1.0, 0.01,
                                                     0.5, True)
    assert err is None and st == 0
    assert np.array_equal(_bits(sys.position), _bits(xo))
    assert np.array_equal(_bits(sys.velocity), _bits(vo))
    assert np.array_equal(_bits(log), _bits(logo))


def test_compat_simulate_rejects(nd):
    x, v, m, q = _collect(1, 8, 0.01, 1e-9, False)
    sys = nd.GenericObjectCollection(x, v, mass=m, charge=q)
    clct = nd.GenericRandomCollector(objectnumber=8, minDim=BOX[0], maxDim=BOX[1],
                                     temperature=0.01)
    with pytest.raises(ValueError):
        nd.simulate_compat_(sys, nd.SimSpec(duration=3, stepwidth=0.5), clct)
    with pytest.raises(nd.NDError):
        nd.simulate_compat_(sys, nd.SimSpec(duration=-1, stepwidth=1), clct)


COLLECT = [
    # objectnumber, seed, temperature, random velocities, minimumdistance
    (1, 41, 0.01, False, 0.0001),
    (2, 42, 0.01, True, 0.0001),
    (1000, 43, 0.01, False, 0.0001),   # the reference scripts' collector
    (5000, 44, 0.05, True, 0.02),      # a few hundred atoms pruned
    (20000, 45, 0.5, True, 0.005),     # 79 velocity chunks
    (256, 46, 0.1, True, 0.05),        # one full velocity chunk
    (257, 47, 0.1, True, 0.05),        # a second chunk of one atom
]


@pytest.mark.parametrize("case", COLLECT, ids=lambda c: f"n{c[0]}")
def test_collect_objects_bit_exact(nd, oracle, case):
    n, seed, T, rv, dmin = case
    clct = nd.GenericRandomCollector(objectnumber=n, minDim=(0.0, -1.0, 0.0),
                                     maxDim=(1.0, 1.0, 2.0), temperature=T, minimumdistance=dmin,
                                     randomvelocity=rv, minmass=1.0, maxmass=5.0,
                                     mincharge=-1e-9, maxcharge=1e-9)
    sys = nd.collect_objects(clct, seed=seed)
    x, v, m, q, cnt = oracle.collect_objects(seed, n, (0.0, -1.0, 0.0), (1.0, 1.0, 2.0), T, rv,
                                             1.0, 5.0, dmin, -1e-9, 1e-9)
    assert np.array_equal(_bits(sys.position), _bits(x))
    assert np.array_equal(_bits(sys.velocity), _bits(v))
    assert np.array_equal(_bits(sys.mass), _bits(m))
    assert np.array_equal(_bits(sys.charge), _bits(q))
    assert sys.pruned == cnt
    if n == 5000:
        assert cnt > 100


def test_collect_objects_rejects(nd):
    for n in (0, (1 << 20) + 1):
        clct = nd.GenericRandomCollector(objectnumber=n, minDim=BOX[0], maxDim=BOX[1])
        with pytest.raises(nd.NDError):
            nd.collect_objects(clct)


def test_collect_then_simulate_compat(nd, oracle):
    # a legacy script end to end: collect_objects, then simulate! as written
    clct = nd.GenericRandomCollector(objectnumber=400, minDim=(0.0, 0.0, 0.0),
                                     maxDim=(1.0, 1.0, 1.0), temperature=0.01,
                                     minimumdistance=0.0001, minmass=1.0, maxmass=5.0,
                                     mincharge=-1e-9, maxcharge=1e-9)
    sys = nd.collect_objects(clct, seed=7)
    x0, v0 = sys.position.astype(np.float32), sys.velocity.astype(np.float32)
    log = nd.simulate_compat_(sys, nd.SimSpec(duration=12, stepwidth=1, vDamp=1.0), clct)
    ref = oracle.compat_simulate(x0, v0, np.zeros((400, 3)), sys.mass, sys.charge, BOX[0], BOX[1],
                                 0.01, 400, 1, 12, 1.0)
    assert np.array_equal(_bits(log), _bits(ref[3]))

"""C-ABI boundary and host logic, without a GPU.

* libnaivegpu.so loads and exports every function include/naivegpu.h declares,
  and the Python binding declares a signature for each of them;
* the product path never links or imports the oracle;
* host-side argument checks mirror the reference's errors;
* the seeded generators are deterministic and have the stated properties.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG, REPO, gpu_available

HEADER = os.path.join(REPO, "include", "naivegpu.h")


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:nd_status|const char\*|void\*|int64_t)\s+(nd_\w+)\(",
                                 text, re.M)))


def test_header_symbols_exported(nd):
    from naivedynamics import _lib
    lib = _lib.lib()
    names = header_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"no ctypes signature for {name}"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (nd_\w+)", out))
    assert set(names) <= exported


def test_product_does_not_use_oracle(nd):
    from naivedynamics import _lib
    out = subprocess.run(["nm", "-D", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "ref_" not in " ".join(re.findall(r" [TU] (\w+)", out)).replace("pref_", "")
    ldd = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "naiveref" not in ldd
    pkg = os.path.join(PKG, "naivedynamics")
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            src = open(os.path.join(pkg, f)).read()
            assert "oracle" not in src.replace("no CPU fallback", ""), f


def test_library_missing_fails_loudly(tmp_path):
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import naivedynamics\n") % PKG
    env = dict(os.environ, NAIVEGPU_LIB=str(tmp_path / "missing.so"))
    r = subprocess.run(["python", "-c", code], capture_output=True, text=True, env=env)
    assert r.returncode != 0
    assert "libnaivegpu.so not found" in r.stderr


def test_spec_errors_match_reference(nd):
    # SpheresBVHSpecs (BVHTraverse.jl:74-80)
    with pytest.raises(nd.SpecError):
        nd.SpheresBVHSpecs(0.1, 10, 4)
    with pytest.raises(nd.SpecError):
        nd.SpheresBVHSpecs(0.1, 5, 5)
    with pytest.raises(nd.SpecError):
        nd.SpheresBVHSpecs(0.1, 8, 4, floattype=np.float64)
    s = nd.SpheresBVHSpecs(0.1, 8000, 4)
    assert (s.leaves_count, s.branches_count) == (2000, 1999)
    from naivedynamics import _lib
    cs = s.c_spec()
    assert (cs.atom_count, cs.leaves_count, cs.branches_count, cs.atomsperleaf) == (8000, 2000, 1999, 4)
    assert cs.neighbor_distance == np.float32(0.1)


def test_status_strings(nd):
    from naivedynamics import _lib
    for st in (0, 1, -1, -2, -3, -4, -5, -6, -7, -8, -9):
        assert _lib.status_string(st) != "unknown status"


def test_null_arguments_rejected(nd):
    from naivedynamics import _lib
    L = _lib.lib()
    assert L.nd_ctx_create(None, 0) == _lib.ND_ERR_ARG
    assert L.nd_bvh_spec_init(None, 0.1, 8, 4) == _lib.ND_ERR_ARG
    assert L.nd_tree(None, None, None, 0, 0, None, 0, None, None, None, None) == _lib.ND_ERR_ARG
    assert L.nd_md_run(None, 1) == _lib.ND_ERR_ARG
    assert L.nd_synth_uniform(1, 4, 0.0, 1.0, None) == _lib.ND_ERR_ARG


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_no_device_status(nd):
    with pytest.raises(nd.NDError) as e:
        nd.Context(0)
    assert e.value.status == -9


def test_synth_deterministic(nd):
    a = nd.synth.uniform_positions(7, 1000, 17.0)
    b = nd.synth.uniform_positions(7, 1000, 17.0)
    assert np.array_equal(a, b)
    assert a.dtype == np.float32 and a.min() >= 0 and a.max() < 17.0
    assert not np.array_equal(a, nd.synth.uniform_positions(8, 1000, 17.0))


def test_synth_mindist(nd):
    x = nd.synth.uniform_positions_mindist(3, 2000, 13.5, 0.8)
    d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    d[np.arange(len(x)), np.arange(len(x))] = 99
    assert d.min() >= 0.8
    assert x.min() >= 0 and x.max() < 13.5


def test_synth_charges_and_normal(nd):
    q = nd.synth.charges_pm1(5, 1000)
    assert (q == 1).sum() == 500 and (q == -1).sum() == 500
    v = nd.synth.normal(9, (20000, 3))
    assert abs(v.mean()) < 0.03 and abs(v.std() - 1) < 0.03


def test_synth_clusters(nd):
    x = nd.synth.cluster_positions(1, 64 * 100, 64, 400.0, 2.0, 10.0)
    assert x.shape == (6400, 3) and np.isfinite(x).all()
    c = x.reshape(64, 100, 3)
    spread = c.std(1).mean(1)
    assert spread.min() > 1.0 and spread.max() < 14.0


def test_pair_array_conversion(nd):
    from naivedynamics.dynamics import _pair_arrays
    pl = np.zeros(3, nd.PAIR_DTYPE)
    pl["i"], pl["j"], pl["d"] = [1, 2, 3], [4, 5, 6], [0.1, 0.2, 0.3]
    i, j = _pair_arrays(pl)
    assert list(i) == [1, 2, 3] and list(j) == [4, 5, 6]
    i, j = _pair_arrays([(1, 2, 0.5), (3, 4, 0.25)])
    assert list(i) == [1, 3] and list(j) == [2, 4]


def test_oracle_generators_match_library(nd, oracle):
    # The CPU baseline draws its inputs from the oracle's own generators (it
    # never loads the GPU library); they must be the GPU arm's inputs bit for
    # bit: the 262,144-atom workload's stream at a smaller size, and the plain
    # LJ box.
    for seed, n, side, ch in [(0x4E440002, 20000, 28.8, True), (0x4E440001, 4096, 17.0, False)]:
        a = oracle.synth_lj_system(seed, n, side, 0.8, ch)
        b = nd.synth.lj_system(seed, n, side, 0.8, ch)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert (a[2] is None and b[2] is None) or np.array_equal(a[2], b[2])
    assert np.array_equal(oracle.synth_uniform(7, 1000, 3.0), nd.synth.uniform_positions(7, 1000, 3.0))


def test_oracle_session_equals_run(oracle):
    # The steady-state session (create, then steps) follows the same
    # trajectory as the one-call CPU baseline loop.
    x, v, q = oracle.synth_lj_system(0x4E440002, 2048, 13.6, 0.8, True)
    p = oracle.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(13.6,) * 3, dt=1e-3)
    xa, va, fa, na = oracle.md_run_bvh(p, x, v, q, steps=25, rebuild=10, skin=0.3, apl=4)
    s = oracle.MDSession(p, x, v, q, rebuild=10, skin=0.3, apl=4)
    s.steps(10)
    nb = s.steps(15)
    xb, vb, fb = s.get()
    s.close()
    assert na == nb
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)


def test_autotune_cache_key_names_the_tuner(nd):
    """The tuned-settings cache key holds the tuner's version, the device and
    the untuned parameters, so a result from another candidate set or another
    cutoff is not reused."""
    import json

    from naivedynamics import dynamics as dyn

    class FakeCtx:
        def device_name(self):
            return "GB300-test"

    p = nd.md_params(cutoff=2.5, skin=0.3, box_hi=(17, 17, 17))
    key = json.loads(dyn._tune_key(FakeCtx(), p, 4096, None, False, False))
    assert key["tuner"] == dyn.TUNER_VERSION and key["device"] == "GB300-test"
    assert key["shape"]["n"] == 4096 and key["fixed"]["cutoff"] == 2.5
    assert "skin" not in key["fixed"]
    q = nd.md_params(cutoff=3.0, skin=0.3, box_hi=(17, 17, 17))
    assert dyn._tune_key(FakeCtx(), q, 4096, None, False, False) != json.dumps(key, sort_keys=True)

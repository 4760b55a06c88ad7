"""ctypes wrapper of the CPU oracle ``libnaiveref`` (test infrastructure only).

The oracle restates the NaiveDynamics.jl hot path in plain C (see naiveref.c for
the reference file:line of every function).  It is the checker for the GPU
library: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  The product path never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnaiveref.so")

REF_ORDER_REFERENCE = 0
REF_ORDER_SPATIAL = 1
REF_BOX_LEAF = 0
REF_BOX_ATOM = 1

KEY_DTYPE = np.dtype([("min", np.float32, 3), ("max", np.float32, 3),
                      ("left", np.int32), ("skip", np.int32)])


class OracleError(RuntimeError):
    pass


class RefAdjSpec(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int32), ("bins", ctypes.c_int32),
                ("r_max", ctypes.c_double), ("width", ctypes.c_double),
                ("r_switch", ctypes.c_double)]


class RefCompatSim(ctypes.Structure):
    _fields_ = [("min_dim", ctypes.c_float * 3), ("max_dim", ctypes.c_float * 3),
                ("temperature", ctypes.c_float), ("objectnumber", ctypes.c_int64),
                ("stepwidth", ctypes.c_int64), ("duration", ctypes.c_int64),
                ("velocity_dampening", ctypes.c_float)]


class RefCollector(ctypes.Structure):
    _fields_ = [("objectnumber", ctypes.c_int64), ("min_dim", ctypes.c_float * 3),
                ("max_dim", ctypes.c_float * 3), ("temperature", ctypes.c_float),
                ("randomvelocity", ctypes.c_int32), ("minmass", ctypes.c_float),
                ("maxmass", ctypes.c_float), ("minimumdistance", ctypes.c_float),
                ("mincharge", ctypes.c_float), ("maxcharge", ctypes.c_float)]


class RefMDParams(ctypes.Structure):
    _fields_ = [("sigma", ctypes.c_double), ("epsilon", ctypes.c_double),
                ("coulomb_k", ctypes.c_double), ("cutoff", ctypes.c_double),
                ("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3),
                ("dt", ctypes.c_double)]


_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no fast-math, no FMA contraction)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t)) if a is not None else None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            i32p = ctypes.POINTER(ctypes.c_int32)
            f32p = ctypes.POINTER(ctypes.c_float)
            f64p = ctypes.POINTER(ctypes.c_double)
            u64p = ctypes.POINTER(ctypes.c_uint64)
            L.ref_spec.argtypes = [ctypes.c_int64, ctypes.c_int64, i32p, i32p]
            L.ref_spec.restype = ctypes.c_int
            L.ref_morton_reference.argtypes = [f32p, ctypes.c_int64, i32p]
            L.ref_morton_reference.restype = ctypes.c_int
            L.ref_morton_spatial.argtypes = [f32p, ctypes.c_int64, i32p]
            L.ref_morton_spatial.restype = ctypes.c_int
            L.ref_hilbert3.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
            L.ref_hilbert3.restype = ctypes.c_uint32
            L.ref_sortperm.argtypes = [i32p, ctypes.c_int64, i32p]
            L.ref_sortperm.restype = ctypes.c_int
            L.ref_delta.argtypes = [ctypes.c_int32, i32p, ctypes.c_int32, ctypes.c_int32]
            L.ref_delta.restype = ctypes.c_int32
            L.ref_tree.argtypes = [f32p, ctypes.c_int32, ctypes.c_float, ctypes.c_int32,
                                   ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.c_int64, i32p, i32p, f32p, i32p]
            L.ref_tree.restype = ctypes.c_int
            L.ref_tree_kept.argtypes = [f32p, ctypes.c_int32, ctypes.c_float, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, i32p, i32p,
                                        f32p]
            L.ref_tree_kept.restype = ctypes.c_int
            for name in ("ref_leaf_traverse", "ref_atom_traverse"):
                fn = getattr(L, name)
                fn.argtypes = [ctypes.c_void_p, i32p, f32p, ctypes.c_int32, ctypes.c_int32,
                               ctypes.c_float, i32p, i32p, f32p, ctypes.c_int64]
                fn.restype = ctypes.c_int64
            L.ref_leaf_traverse_crit.argtypes = [ctypes.c_void_p, i32p, f32p, ctypes.c_int32,
                                                 ctypes.c_int32, ctypes.c_float, ctypes.c_int32,
                                                 i32p, i32p, f32p, ctypes.c_int64]
            L.ref_leaf_traverse_crit.restype = ctypes.c_int64
            L.ref_leaf_traverse_hash.argtypes = [ctypes.c_void_p, i32p, f32p, ctypes.c_int32,
                                                 ctypes.c_int32, ctypes.c_float, u64p]
            L.ref_leaf_traverse_hash.restype = ctypes.c_int64
            L.ref_compat_force_lj.argtypes = [ctypes.c_int32, i32p, i32p, f32p, ctypes.c_int64,
                                              f32p]
            L.ref_compat_force_lj.restype = None
            L.ref_compat_force_coulomb.argtypes = [ctypes.c_int32, i32p, i32p, f32p,
                                                   ctypes.c_int64, f32p, f32p]
            L.ref_compat_force_coulomb.restype = None
            L.ref_compat_simulate.argtypes = [ctypes.POINTER(RefCompatSim), ctypes.c_int32, f32p,
                                              f32p, f32p, f32p, f32p, f32p]
            L.ref_compat_simulate.restype = ctypes.c_int
            L.ref_collect_objects.argtypes = [ctypes.POINTER(RefCollector), ctypes.c_uint64, f32p,
                                              f32p, f32p, f32p]
            L.ref_collect_objects.restype = ctypes.c_int64
            L.ref_brute_pairs.argtypes = [f32p, ctypes.c_int32, ctypes.c_float, ctypes.c_int32,
                                          i32p, i32p, f32p, ctypes.c_int64]
            L.ref_brute_pairs.restype = ctypes.c_int64
            L.ref_pair_hash.argtypes = [i32p, i32p, f32p, ctypes.c_int64, u64p]
            L.ref_pair_hash.restype = None
            L.ref_forces.argtypes = [ctypes.POINTER(RefMDParams), ctypes.c_int32, f64p, f64p,
                                     f64p, f64p]
            L.ref_forces.restype = ctypes.c_int64
            L.ref_md_run.argtypes = [ctypes.POINTER(RefMDParams), ctypes.c_int32, f64p, f64p,
                                     f64p, f64p, f64p, ctypes.c_int64]
            L.ref_md_run.restype = ctypes.c_int
            L.ref_md_run_observed.argtypes = [ctypes.POINTER(RefMDParams), ctypes.c_int32, f64p,
                                              f64p, f64p, f64p, f64p, ctypes.c_int64,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                              ctypes.c_int32, f64p]
            L.ref_md_run_observed.restype = ctypes.c_int
            L.ref_md_run_bvh.argtypes = [ctypes.POINTER(RefMDParams), ctypes.c_int32, f64p,
                                         f64p, f64p, f64p, f64p, ctypes.c_int64, ctypes.c_int32,
                                         ctypes.c_double, ctypes.c_int32, ctypes.c_int32]
            L.ref_md_run_bvh.restype = ctypes.c_int64
            L.ref_adj_dual.argtypes = [ctypes.POINTER(RefMDParams), ctypes.POINTER(RefAdjSpec),
                                       ctypes.c_int32, f64p, f64p, f64p, f64p, f64p, f64p, f64p,
                                       f64p, f64p, f64p, f64p, f64p, u64p]
            L.ref_adj_dual.restype = ctypes.c_int
            L.ref_num_threads.argtypes = []
            L.ref_num_threads.restype = ctypes.c_int
            L.ref_md_bvh_create.argtypes = [ctypes.POINTER(RefMDParams), ctypes.c_int32, f64p,
                                            f64p, f64p, f64p, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_int32, ctypes.c_int32]
            L.ref_md_bvh_create.restype = ctypes.c_void_p
            L.ref_md_bvh_steps.argtypes = [ctypes.c_void_p, ctypes.c_int64]
            L.ref_md_bvh_steps.restype = ctypes.c_int64
            L.ref_md_bvh_get.argtypes = [ctypes.c_void_p, f64p, f64p, f64p]
            L.ref_md_bvh_get.restype = None
            L.ref_md_bvh_destroy.argtypes = [ctypes.c_void_p]
            L.ref_md_bvh_destroy.restype = None
            L.ref_synth_uniform.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_double, f32p]
            L.ref_synth_uniform.restype = ctypes.c_int
            L.ref_synth_uniform_mindist.argtypes = [ctypes.c_uint64, ctypes.c_int32,
                                                    ctypes.c_double, ctypes.c_double, f64p]
            L.ref_synth_uniform_mindist.restype = ctypes.c_int
            L.ref_synth_normal.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_double, f64p]
            L.ref_synth_normal.restype = ctypes.c_int
            L.ref_synth_charges.argtypes = [ctypes.c_uint64, ctypes.c_int32, f64p]
            L.ref_synth_charges.restype = ctypes.c_int
            _lib = L
    return _lib


def _check(st):
    if st != 0:
        raise OracleError(f"oracle status {st}")


def _xyz(xyz):
    a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float32).reshape(-1, 3))
    return a


def spec(n, apl):
    """SpheresBVHSpecs checks; returns (leaves, branches)."""
    nl = ctypes.c_int32()
    nb = ctypes.c_int32()
    _check(lib().ref_spec(n, apl, ctypes.byref(nl), ctypes.byref(nb)))
    return nl.value, nb.value


def morton_reference(xyz):
    a = _xyz(xyz)
    out = np.empty(a.shape[0], np.int32)
    _check(lib().ref_morton_reference(_p(a, ctypes.c_float), a.shape[0], _p(out, ctypes.c_int32)))
    return out


def morton_spatial(xyz):
    a = _xyz(xyz)
    out = np.empty(a.shape[0], np.int32)
    _check(lib().ref_morton_spatial(_p(a, ctypes.c_float), a.shape[0], _p(out, ctypes.c_int32)))
    return out


def hilbert3(x, y, z):
    """3-D Hilbert index of grid cell (x, y, z), each in [0, 1024)."""
    return int(lib().ref_hilbert3(x, y, z))


def sortperm(codes):
    c = np.ascontiguousarray(codes, dtype=np.int32)
    out = np.empty(c.shape[0], np.int32)
    _check(lib().ref_sortperm(_p(c, ctypes.c_int32), c.shape[0], _p(out, ctypes.c_int32)))
    return out


def tree(xyz, r, apl, order=REF_ORDER_REFERENCE, boxes=REF_BOX_LEAF, overwrite_root=True):
    """leafTreeData / TreeData.  Returns dict(keys, index, code, position, perm)."""
    a = _xyz(xyz)
    n = a.shape[0]
    nl, _ = spec(n, apl)
    nkeys = (n - 1) if boxes == REF_BOX_LEAF else (2 * nl - 1)
    nkeys = max(nkeys, 2 * nl - 1)
    keys = np.zeros(nkeys, KEY_DTYPE)
    idx = np.empty(n, np.int32)
    code = np.empty(n, np.int32)
    pos = np.empty((n, 3), np.float32)
    perm = np.empty(n, np.int32)
    _check(lib().ref_tree(_p(a, ctypes.c_float), n, np.float32(r), apl, order, boxes,
                          1 if overwrite_root else 0, keys.ctypes.data, nkeys,
                          _p(idx, ctypes.c_int32), _p(code, ctypes.c_int32),
                          _p(pos, ctypes.c_float), _p(perm, ctypes.c_int32)))
    if boxes == REF_BOX_LEAF:
        keys = keys[: n - 1]
    return dict(keys=keys, index=idx, code=code, position=pos, perm=perm, leaves=nl)


def tree_kept(xyz, r, apl, index, code, overwrite_root=True):
    """leafTreeData of new positions in a kept order (index: 1-based original
    index per sorted slot, code: the sorted codes of an earlier tree()): the
    same topology with the new boxes.  Returns the dict of tree()."""
    a = _xyz(xyz)
    n = a.shape[0]
    nl, _ = spec(n, apl)
    nkeys = max(n - 1, 2 * nl - 1)
    keys = np.zeros(nkeys, KEY_DTYPE)
    idx = np.ascontiguousarray(index, np.int32)
    cd = np.ascontiguousarray(code, np.int32)
    pos = np.empty((n, 3), np.float32)
    _check(lib().ref_tree_kept(_p(a, ctypes.c_float), n, np.float32(r), apl,
                               1 if overwrite_root else 0, keys.ctypes.data, nkeys,
                               _p(idx, ctypes.c_int32), _p(cd, ctypes.c_int32),
                               _p(pos, ctypes.c_float)))
    return dict(keys=keys[: n - 1], index=idx.copy(), code=cd.copy(), position=pos,
                perm=idx - 1, leaves=nl)


def _pairs_call(fn, *args, cap_hint=1024):
    cap = cap_hint
    while True:
        pi = np.empty(cap, np.int32)
        pj = np.empty(cap, np.int32)
        pd = np.empty(cap, np.float32)
        cnt = fn(*args, _p(pi, ctypes.c_int32), _p(pj, ctypes.c_int32), _p(pd, ctypes.c_float), cap)
        if cnt < 0:
            raise OracleError(f"oracle status {cnt}")
        if cnt <= cap:
            return pi[:cnt].copy(), pj[:cnt].copy(), pd[:cnt].copy()
        cap = int(cnt)


def leaf_traverse(t, r, apl):
    """leafneighbor_traverse in serial order over a tree from tree(..., boxes=LEAF)."""
    keys = np.ascontiguousarray(t["keys"])
    return _pairs_call(lib().ref_leaf_traverse, keys.ctypes.data, _p(t["index"], ctypes.c_int32),
                       _p(t["position"], ctypes.c_float), t["leaves"], apl, np.float32(r))


def compat_forces(kind, n, pairs, q=None):
    """The reference's force_lennardjones! (kind 'lj') or force_coulomb!
    (kind 'coulomb') as it computes them at HEAD (Forces.jl:6-66), over the
    pair list (i, j, d) in order.  Returns N x 3 Float32."""
    i = np.ascontiguousarray(pairs[0], np.int32)
    j = np.ascontiguousarray(pairs[1], np.int32)
    d = np.ascontiguousarray(pairs[2], np.float32)
    out = np.zeros((n, 3), np.float32)
    if kind == "lj":
        lib().ref_compat_force_lj(n, _p(i, ctypes.c_int32), _p(j, ctypes.c_int32),
                                  _p(d, ctypes.c_float), len(i), _p(out, ctypes.c_float))
    else:
        qq = np.ascontiguousarray(q, np.float32)
        lib().ref_compat_force_coulomb(n, _p(i, ctypes.c_int32), _p(j, ctypes.c_int32),
                                       _p(d, ctypes.c_float), len(i), _p(qq, ctypes.c_float),
                                       _p(out, ctypes.c_float))
    return out


def compat_simulate(x, v, force, mass, charge, min_dim, max_dim, temperature, objectnumber,
                    stepwidth, duration, vdamp, log=True):
    """simulate! as written (Simulator.jl:154-256) for Float32 state and an
    Int64 stepwidth.  Returns (x, v, force, poslog or None, status): status 1
    is rescale_velocity!'s DomainError."""
    x = np.array(x, np.float32, order="C").reshape(-1, 3)
    v = np.array(v, np.float32, order="C").reshape(-1, 3)
    f = np.array(force, np.float32, order="C").reshape(-1, 3)
    m = np.ascontiguousarray(mass, np.float32)
    q = np.ascontiguousarray(charge, np.float32)
    n = len(x)
    spec = RefCompatSim((ctypes.c_float * 3)(*min_dim), (ctypes.c_float * 3)(*max_dim),
                        temperature, objectnumber, stepwidth, duration, vdamp)
    log_arr = np.zeros((duration + 1, n, 3), np.float32) if log else None
    st = lib().ref_compat_simulate(ctypes.byref(spec), n, _p(x, ctypes.c_float),
                                   _p(v, ctypes.c_float), _p(f, ctypes.c_float),
                                   _p(m, ctypes.c_float), _p(q, ctypes.c_float),
                                   _p(log_arr, ctypes.c_float) if log else None)
    return x, v, f, log_arr, st


def collect_objects(seed, objectnumber, min_dim, max_dim, temperature, randomvelocity, minmass,
                    maxmass, minimumdistance, mincharge, maxcharge):
    """collect_objects (MDInput.jl:305-369) with the library's seeded stream:
    (x, v, mass, charge, number of atoms filled with Inf)."""
    n = int(objectnumber)
    cl = RefCollector(n, (ctypes.c_float * 3)(*min_dim), (ctypes.c_float * 3)(*max_dim),
                      temperature, int(bool(randomvelocity)), minmass, maxmass, minimumdistance,
                      mincharge, maxcharge)
    x = np.zeros((n, 3), np.float32)
    v = np.zeros((n, 3), np.float32)
    m = np.zeros(n, np.float32)
    q = np.zeros(n, np.float32)
    cnt = lib().ref_collect_objects(ctypes.byref(cl), ctypes.c_uint64(seed), _p(x, ctypes.c_float),
                                    _p(v, ctypes.c_float), _p(m, ctypes.c_float),
                                    _p(q, ctypes.c_float))
    return x, v, m, q, cnt


def simd_leaf_traverse(t, r, apl):
    """simdneighbor_traverse (ext/NaiveSIMD.jl:610-704) on one thread: the
    leafneighbor_traverse order with the criterion sqrt(d^2) < r."""
    keys = np.ascontiguousarray(t["keys"])
    return _pairs_call(lib().ref_leaf_traverse_crit, keys.ctypes.data,
                       _p(t["index"], ctypes.c_int32), _p(t["position"], ctypes.c_float),
                       t["leaves"], apl, np.float32(r), 1)


def leaf_traverse_hash(t, r, apl):
    keys = np.ascontiguousarray(t["keys"])
    h = np.zeros(2, np.uint64)
    cnt = lib().ref_leaf_traverse_hash(keys.ctypes.data, _p(t["index"], ctypes.c_int32),
                                       _p(t["position"], ctypes.c_float), t["leaves"], apl,
                                       np.float32(r), _p(h, ctypes.c_uint64))
    return int(cnt), (int(h[0]), int(h[1]))


def atom_traverse(t, r, apl):
    keys = np.ascontiguousarray(t["keys"])
    n = t["index"].shape[0]
    return _pairs_call(lib().ref_atom_traverse, keys.ctypes.data, _p(t["index"], ctypes.c_int32),
                       _p(t["position"], ctypes.c_float), n, apl, np.float32(r))


def leafbuild_traverse_bvh(xyz, r, apl, order=REF_ORDER_REFERENCE):
    t = tree(xyz, r, apl, order=order, boxes=REF_BOX_LEAF)
    return leaf_traverse(t, r, apl)


def build_traverse_bvh(xyz, r, apl, order=REF_ORDER_REFERENCE):
    t = tree(xyz, r, apl, order=order, boxes=REF_BOX_ATOM)
    return atom_traverse(t, r, apl)


def brute_pairs(xyz, r, criterion=0):
    a = _xyz(xyz)
    return _pairs_call(lib().ref_brute_pairs, _p(a, ctypes.c_float), a.shape[0], np.float32(r),
                       criterion)


def pair_hash(pi, pj, pd):
    pi = np.ascontiguousarray(pi, np.int32)
    pj = np.ascontiguousarray(pj, np.int32)
    pd = np.ascontiguousarray(pd, np.float32)
    h = np.zeros(2, np.uint64)
    lib().ref_pair_hash(_p(pi, ctypes.c_int32), _p(pj, ctypes.c_int32), _p(pd, ctypes.c_float),
                        pi.shape[0], _p(h, ctypes.c_uint64))
    return int(h[0]), int(h[1])


def md_params(sigma=1.0, epsilon=1.0, coulomb_k=0.0, cutoff=2.5, box_lo=(0, 0, 0),
              box_hi=(1, 1, 1), dt=1e-3):
    p = RefMDParams()
    p.sigma, p.epsilon, p.coulomb_k, p.cutoff, p.dt = sigma, epsilon, coulomb_k, cutoff, dt
    for d in range(3):
        p.box_lo[d] = box_lo[d]
        p.box_hi[d] = box_hi[d]
    return p


def forces(p, x, q=None):
    """FP64 LJ + Coulomb forces and energy (cell list).  Returns (f, energy, npairs)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
    qq = None if q is None else np.ascontiguousarray(q, np.float64)
    f = np.empty_like(x)
    e = ctypes.c_double()
    n = lib().ref_forces(ctypes.byref(p), x.shape[0], _p(x, ctypes.c_double),
                         _p(qq, ctypes.c_double), _p(f, ctypes.c_double), ctypes.byref(e))
    if n < 0:
        raise OracleError(f"oracle status {n}")
    return f, e.value, int(n)


def md_run(p, x, v, q=None, m=None, steps=1):
    """FP64 kick-drift-kick run from (x, v); returns (x, v, f)."""
    x = np.array(x, np.float64).reshape(-1, 3)
    v = np.array(v, np.float64).reshape(-1, 3)
    qq = None if q is None else np.ascontiguousarray(q, np.float64)
    mm = None if m is None else np.ascontiguousarray(m, np.float64)
    f, _, _ = forces(p, x, qq)
    _check(lib().ref_md_run(ctypes.byref(p), x.shape[0], _p(x, ctypes.c_double),
                            _p(v, ctypes.c_double), _p(f, ctypes.c_double),
                            _p(qq, ctypes.c_double), _p(mm, ctypes.c_double), steps))
    return x, v, f


def md_run_observed(p, x, v, q=None, m=None, steps=1, thermo=None, log_every=0):
    """FP64 KDK run with simulate!'s observers: thermo = (T, gamma, every) for
    rescale_velocity!, log_every for the position log.  Returns (x, v, f, poslog)."""
    x = np.array(x, np.float64).reshape(-1, 3)
    v = np.array(v, np.float64).reshape(-1, 3)
    qq = None if q is None else np.ascontiguousarray(q, np.float64)
    mm = None if m is None else np.ascontiguousarray(m, np.float64)
    f, _, _ = forces(p, x, qq)
    T, g, every = thermo if thermo else (0.0, 0.0, 0)
    nf = steps // log_every if log_every > 0 else 0
    log = np.zeros((max(nf, 1), x.shape[0], 3), np.float64)
    _check(lib().ref_md_run_observed(ctypes.byref(p), x.shape[0], _p(x, ctypes.c_double),
                                     _p(v, ctypes.c_double), _p(f, ctypes.c_double),
                                     _p(qq, ctypes.c_double), _p(mm, ctypes.c_double), steps,
                                     T, g, every, log_every, _p(log, ctypes.c_double)))
    return x, v, f, log[:nf]


def md_run_bvh(p, x, v, q=None, m=None, steps=1, rebuild=10, skin=0.3, apl=4,
               order=REF_ORDER_REFERENCE):
    """CPU baseline run (leaf BVH + FP64 forces, OpenMP).  Returns (x, v, f, npairs)."""
    x = np.array(x, np.float64).reshape(-1, 3)
    v = np.array(v, np.float64).reshape(-1, 3)
    f = np.zeros_like(x)
    qq = None if q is None else np.ascontiguousarray(q, np.float64)
    mm = None if m is None else np.ascontiguousarray(m, np.float64)
    n = lib().ref_md_run_bvh(ctypes.byref(p), x.shape[0], _p(x, ctypes.c_double),
                             _p(v, ctypes.c_double), _p(f, ctypes.c_double),
                             _p(qq, ctypes.c_double), _p(mm, ctypes.c_double), steps, rebuild,
                             skin, apl, order)
    if n < 0:
        raise OracleError(f"oracle status {n}")
    return x, v, f, int(n)


def num_threads():
    return int(lib().ref_num_threads())


def adj_spec(steps, bins=64, r_max=2.5, width=None, r_switch=None):
    """Histogram-loss specification: width defaults to the bin width, the pair
    weight switch starts at r_max - 0.25 (r_max - 4 widths at most)."""
    s = RefAdjSpec()
    s.steps, s.bins, s.r_max = steps, bins, r_max
    s.width = r_max / bins if width is None else width
    s.r_switch = (r_max - 0.25) if r_switch is None else r_switch
    return s


def adj_dual(p, s, x0, v0, q=None, m=None, dx0=None, dv0=None, target=None):
    """Forward-mode FP64 loss of a trajectory (dual numbers).  Returns dict with
    loss, dloss = (dL/dsigma, dL/depsilon, directional derivative along
    (dx0, dv0)), hist, x, v (final state) and events (branch signature)."""
    x0 = np.ascontiguousarray(x0, np.float64).reshape(-1, 3)
    v0 = np.ascontiguousarray(v0, np.float64).reshape(-1, 3)
    n = x0.shape[0]
    c = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
    q, m, dx0, dv0, target = c(q), c(m), c(dx0), c(dv0), c(target)
    hist = np.empty(s.bins, np.float64)
    loss = ctypes.c_double()
    dl = np.empty(3, np.float64)
    xo = np.empty_like(x0)
    vo = np.empty_like(v0)
    ev = np.zeros(2, np.uint64)
    f64 = ctypes.c_double
    _check(lib().ref_adj_dual(ctypes.byref(p), ctypes.byref(s), n, _p(x0, f64), _p(v0, f64),
                              _p(q, f64), _p(m, f64), _p(dx0, f64), _p(dv0, f64),
                              _p(target, f64), _p(hist, f64), ctypes.byref(loss), _p(dl, f64),
                              _p(xo, f64), _p(vo, f64), _p(ev, ctypes.c_uint64)))
    return dict(loss=loss.value, dloss=dl, hist=hist, x=xo, v=vo,
                events=(int(ev[0]), int(ev[1])))


class MDSession:
    """ref_md_bvh_*: the CPU-baseline loop as a session (first list and forces
    at creation, then steady-state steps with a rebuild every `rebuild`)."""

    def __init__(self, p, x, v, q=None, m=None, rebuild=10, skin=0.3, apl=4,
                 order=REF_ORDER_REFERENCE):
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(v, np.float64).reshape(-1, 3)
        qq = None if q is None else np.ascontiguousarray(q, np.float64)
        mm = None if m is None else np.ascontiguousarray(m, np.float64)
        self.n = x.shape[0]
        self.h = lib().ref_md_bvh_create(ctypes.byref(p), self.n, _p(x, ctypes.c_double),
                                         _p(v, ctypes.c_double), _p(qq, ctypes.c_double),
                                         _p(mm, ctypes.c_double), rebuild, skin, apl, order)
        if not self.h:
            raise OracleError("ref_md_bvh_create failed")

    def steps(self, k):
        st = lib().ref_md_bvh_steps(self.h, int(k))
        if st < 0:
            raise OracleError(f"oracle status {st}")
        return int(st)

    def get(self):
        x = np.empty((self.n, 3))
        v = np.empty((self.n, 3))
        f = np.empty((self.n, 3))
        lib().ref_md_bvh_get(self.h, _p(x, ctypes.c_double), _p(v, ctypes.c_double),
                             _p(f, ctypes.c_double))
        return x, v, f

    def close(self):
        if self.h:
            lib().ref_md_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def synth_uniform(seed, n, side, lo=0.0):
    out = np.empty((n, 3), np.float32)
    _check(lib().ref_synth_uniform(seed, n, lo, side, _p(out, ctypes.c_float)))
    return out


def synth_uniform_mindist(seed, n, side, dmin):
    out = np.empty((n, 3), np.float64)
    _check(lib().ref_synth_uniform_mindist(seed, n, side, dmin, _p(out, ctypes.c_double)))
    return out


def synth_normal(seed, shape, s=1.0):
    out = np.empty(shape, np.float64)
    _check(lib().ref_synth_normal(seed, out.size, s, _p(out, ctypes.c_double)))
    return out


def synth_charges(seed, n):
    out = np.empty(n, np.float64)
    _check(lib().ref_synth_charges(seed, n, _p(out, ctypes.c_double)))
    return out


def synth_lj_system(seed, n, side, dmin=0.8, charges=False):
    """The benchmark's LJ box inputs (x, v, q) from the oracle's own generators:
    the same seeds and streams as the GPU library's nd_synth_* generators."""
    x = synth_uniform_mindist(seed, n, side, dmin)
    v = synth_normal(seed ^ 0x5EED0001, (n, 3), 1.0)
    q = synth_charges(seed ^ 0x5EED0002, n) if charges else None
    return x, v, q

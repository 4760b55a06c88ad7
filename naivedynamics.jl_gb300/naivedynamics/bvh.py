"""Neighbour search: the GPU mirror of src/Neighbors/BVHTraverse.jl.

Names, argument meaning and results follow the reference:
  SpheresBVHSpecs          BVHTraverse.jl:63-94
  leafTreeData / TreeData  BVHTraverse.jl:544-597 / :500-543
  leafbuild_traverse_bvh   BVHTraverse.jl:1423-1428
  build_traverse_bvh       BVHTraverse.jl:1416-1421
  gpubvh_neighborlist      ext/NaiveKA.jl:470-558
  gpubvh_neighborlist!     ext/NaiveKA.jl:597-636 (gpubvh_neighborlist_)
Pair lists are structured arrays of (i, j, d) = Tuple{Int32,Int32,Float32}
with 1-based original indices, every unordered pair once.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import NamedTuple

import numpy as np

from . import _lib
from ._lib import (GRIDKEY_DTYPE, ND_BOX_ATOM, ND_BOX_LEAF, ND_NEED_REALLOC, ND_OK,
                   ND_ORDER_REFERENCE, ND_ORDER_SPATIAL, ND_PAIRS_ORDERED, ND_PAIRS_UNORDERED,
                   PAIR_DTYPE, SpecError, default_context, ptr)

__all__ = ["SpheresBVHSpecs", "APointPrimitive", "leafTreeData", "TreeData",
           "leafbuild_traverse_bvh", "simdbuild_traverse_bvh", "build_traverse_bvh",
           "gpubvh_neighborlist", "gpubvh_neighborlist_", "neighbor_pairs_dev", "pair_hash_dev", "GRIDKEY_DTYPE",
           "PAIR_DTYPE", "ND_ORDER_REFERENCE", "ND_ORDER_SPATIAL", "ND_PAIRS_ORDERED",
           "ND_PAIRS_UNORDERED"]


@dataclass(frozen=True)
class SpheresBVHSpecs:
    """SpheresBVHSpecs{Float32,Int32} (BVHTraverse.jl:63-94).

    Raises SpecError when atomsperleaf does not divide atom_count or when fewer
    than two leaves result, as the reference's constructor does.
    """
    neighbor_distance: float
    atom_count: int
    atomsperleaf: int
    floattype: type = np.float32

    def __post_init__(self):
        if self.floattype not in (np.float32, "Float32"):
            raise SpecError(_lib.ND_ERR_SPEC, "only Float32 specifications are implemented "
                            "(mortoncodes! errors for K != Int32, BVHTraverse.jl:285-287)")
        s = self.c_spec()
        del s

    @property
    def leaves_count(self) -> int:
        return self.atom_count // self.atomsperleaf

    @property
    def branches_count(self) -> int:
        return self.leaves_count - 1

    def c_spec(self) -> _lib.BVHSpec:
        s = _lib.BVHSpec()
        st = _lib.lib().nd_bvh_spec_init(ctypes.byref(s), np.float32(self.neighbor_distance),
                                         int(self.atom_count), int(self.atomsperleaf))
        if st != ND_OK:
            _lib.raise_for(st, None, "SpheresBVHSpecs: atomsperleaf must divide atom_count "
                                     "into at least two leaves")
        return s


class APointPrimitive(NamedTuple):
    """APointPrimitive (BVHTraverse.jl:142-146) in Morton order."""
    index: np.ndarray        # Int32, 1-based original index
    morton_code: np.ndarray  # Int32
    position: np.ndarray     # (N, 3) Float32


def _positions(position) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(position, dtype=np.float32).reshape(-1, 3))
    return a


def _tree(position, spec: SpheresBVHSpecs, boxes: int, order: int, ctx=None):
    ctx = ctx or default_context()
    x = _positions(position)
    if x.shape[0] != spec.atom_count:
        raise ValueError("position length differs from spec.atom_count")
    n, nl = spec.atom_count, spec.leaves_count
    nkeys = (n - 1) if boxes == ND_BOX_LEAF else (2 * nl - 1)
    keys = np.zeros(max(nkeys, 1), GRIDKEY_DTYPE)
    idx = np.empty(n, np.int32)
    code = np.empty(n, np.int32)
    pos = np.empty((n, 3), np.float32)
    perm = np.empty(n, np.int32)
    cs = spec.c_spec()
    st = _lib.lib().nd_tree(ctx.handle, ptr(x), ctypes.byref(cs), order, boxes, ptr(keys),
                            nkeys, ptr(idx), ptr(code), ptr(pos), ptr(perm))
    ctx.check(st, "tree")
    return keys[:nkeys], APointPrimitive(idx, code, pos), perm


def leafTreeData(position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE, ctx=None):
    """leafTreeData (BVHTraverse.jl:544-597) -> (keys, pos, mortsort, store).

    keys has N-1 GridKeys (leaves 1..nL, internal nodes nL+1..2nL-1, zeros after);
    leaf boxes are p -/+ r/2.  `store` (the CAS scratch, whose final contents
    depend on thread scheduling) is not returned (None).
    """
    keys, pos, perm = _tree(position, spec, ND_BOX_LEAF, order, ctx)
    return keys, pos, perm, None


def TreeData(position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE, ctx=None):
    """TreeData (BVHTraverse.jl:500-543): 2nL-1 keys, leaf boxes p -/+ r."""
    keys, pos, perm = _tree(position, spec, ND_BOX_ATOM, order, ctx)
    return keys, pos, perm, None


def _pairs(fn, ctx, *args, capacity_hint=None):
    cap = int(capacity_hint) if capacity_hint else 0
    count = ctypes.c_int64()
    while True:
        out = np.empty(max(cap, 1), PAIR_DTYPE)
        pi = np.empty(max(cap, 1), np.int32)
        pj = np.empty(max(cap, 1), np.int32)
        pd = np.empty(max(cap, 1), np.float32)
        st = fn(ctx.handle, *args, ptr(pi), ptr(pj), ptr(pd), cap, ctypes.byref(count))
        if st == ND_NEED_REALLOC:
            cap = int(count.value)
            continue
        ctx.check(st, "pairs")
        k = int(count.value)
        out = np.empty(k, PAIR_DTYPE)
        out["i"], out["j"], out["d"] = pi[:k], pj[:k], pd[:k]
        return out


def leafbuild_traverse_bvh(position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE,
                           mode: int = ND_PAIRS_ORDERED, ctx=None, capacity_hint=None):
    """leafbuild_traverse_bvh (BVHTraverse.jl:1423-1428): the half pair list.

    With mode=ND_PAIRS_ORDERED the list is in the order the reference emits it
    when run on one thread; ND_PAIRS_UNORDERED returns the same multiset in the
    order the GPU produced it.
    """
    ctx = ctx or default_context()
    x = _positions(position)
    cs = spec.c_spec()
    fn = lambda h, *a: _lib.lib().nd_leaf_pairs(h, ptr(x), ctypes.byref(cs), order, mode, *a)
    return _pairs(fn, ctx, capacity_hint=capacity_hint)


def simdbuild_traverse_bvh(position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE,
                           mode: int = ND_PAIRS_ORDERED, ctx=None, capacity_hint=None):
    """simdbuild_traverse_bvh (ext/NaiveSIMD.jl:706-710): the SIMD twin of
    leafbuild_traverse_bvh -- the same tree and traversal (atomsperleaf must be
    4), pairs kept when sqrt(d^2) < r (:529,589) rather than d^2 < r^2.  The
    reference runs its query leaves on several threads; ND_PAIRS_ORDERED gives
    its order on one thread.
    """
    ctx = ctx or default_context()
    x = _positions(position)
    cs = spec.c_spec()
    fn = lambda h, *a: _lib.lib().nd_simd_leaf_pairs(h, ptr(x), ctypes.byref(cs), order, mode, *a)
    return _pairs(fn, ctx, capacity_hint=capacity_hint)


def build_traverse_bvh(position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE,
                       ctx=None, capacity_hint=None):
    """build_traverse_bvh (BVHTraverse.jl:1416-1421): per-atom traversal over TreeData."""
    ctx = ctx or default_context()
    x = _positions(position)
    cs = spec.c_spec()
    fn = lambda h, *a: _lib.lib().nd_atom_pairs(h, ptr(x), ctypes.byref(cs), order, *a)
    return _pairs(fn, ctx, capacity_hint=capacity_hint)


class GPUNeighborList(NamedTuple):
    pairlist: np.ndarray
    treedata: tuple


def gpubvh_neighborlist(backend, position, spec: SpheresBVHSpecs, order: int = ND_ORDER_REFERENCE):
    """gpubvh_neighborlist(backend, position, spec) (ext/NaiveKA.jl:470-558).

    `backend` is a Context (or a device index, or None for device 0).  Returns
    (pairlist, treedata=(tree, mortonpositions, mortsort, store)).
    """
    if backend is None or isinstance(backend, int):
        ctx = default_context(backend or 0)
    else:
        ctx = backend
    keys, pos, perm, store = leafTreeData(position, spec, order=order, ctx=ctx)
    pairs = leafbuild_traverse_bvh(position, spec, order=order, ctx=ctx)
    return GPUNeighborList(pairs, (keys, pos, perm, store))


def gpubvh_neighborlist_(neighborlist, treedata, spec: SpheresBVHSpecs, backend, position=None,
                         mode: int = ND_PAIRS_ORDERED):
    """gpubvh_neighborlist!(neighborlist, treedata, spec, backend)
    (ext/NaiveKA.jl:597-636): the pair list of new positions from a kept tree.

    treedata is what gpubvh_neighborlist (or leafTreeData) returned: (tree,
    mortonpositions, mortsort, store).  The new positions are `position`
    (caller order), or, when it is None, the ones the caller wrote into
    treedata's mortonpositions.position (kept order, rows labelled by
    mortonpositions.index).  The kept order and sorted codes are reused -- the
    same topology, boxes of the new positions -- and treedata's tree and
    positions are updated in place; neighborlist (a PAIR_DTYPE array that owns
    its memory) is resized and filled in place.  Returns (pairlist, treedata)
    like gpubvh_neighborlist.  The reference's body reads an undefined
    `position` at HEAD; here the new positions come as described.
    """
    if backend is None or isinstance(backend, int):
        ctx = default_context(backend or 0)
    else:
        ctx = backend
    keys, mpos, perm, store = treedata
    n = spec.atom_count
    index = np.ascontiguousarray(mpos.index, np.int32)
    code = np.ascontiguousarray(mpos.morton_code, np.int32)
    if position is None:
        x = np.empty((n, 3), np.float32)
        x[index - 1] = mpos.position
    else:
        x = _positions(position)
    if x.shape[0] != n or index.shape[0] != n:
        raise ValueError("position length differs from spec.atom_count")
    cs = spec.c_spec()
    newpos = np.empty((n, 3), np.float32)
    count = ctypes.c_int64()
    cap = 0
    while True:
        pi = np.empty(max(cap, 1), np.int32)
        pj = np.empty(max(cap, 1), np.int32)
        pd = np.empty(max(cap, 1), np.float32)
        st = _lib.lib().nd_leaf_pairs_refresh(ctx.handle, ptr(x), ctypes.byref(cs), ptr(index),
                                              ptr(code), mode, ptr(keys), int(keys.shape[0]),
                                              ptr(newpos), ptr(pi), ptr(pj), ptr(pd), cap,
                                              ctypes.byref(count))
        if st == ND_NEED_REALLOC:
            cap = int(count.value)
            continue
        ctx.check(st, "gpubvh_neighborlist!")
        break
    k = int(count.value)
    mpos.position[...] = newpos
    out = neighborlist
    if out is None or out.dtype != PAIR_DTYPE:
        out = np.empty(k, PAIR_DTYPE)
    else:
        out.resize(k, refcheck=False)
    out["i"], out["j"], out["d"] = pi[:k], pj[:k], pd[:k]
    return GPUNeighborList(out, (keys, mpos, perm, store))


def neighbor_pairs_dev(xyz_dev, spec: SpheresBVHSpecs, pi_dev, pj_dev, pd_dev, capacity: int,
                       order: int = ND_ORDER_SPATIAL, mode: int = ND_PAIRS_UNORDERED, ctx=None):
    """Device-resident pair list (positions and outputs in device memory).

    Returns (status, count); status ND_NEED_REALLOC means capacity < count.
    """
    ctx = ctx or default_context()
    cs = spec.c_spec()
    count = ctypes.c_int64()
    st = _lib.lib().nd_leaf_pairs_dev(ctx.handle, ptr(xyz_dev), ctypes.byref(cs), order, mode,
                                      ptr(pi_dev), ptr(pj_dev), ptr(pd_dev), int(capacity),
                                      ctypes.byref(count))
    if st not in (ND_OK, ND_NEED_REALLOC):
        ctx.check(st, "nd_leaf_pairs_dev")
    return st, int(count.value)


def pair_hash_dev(pi_dev, pj_dev, pd_dev, npairs: int, ctx=None):
    """Order-free 128-bit hash of a device pair list."""
    ctx = ctx or default_context()
    h = (ctypes.c_uint64 * 2)()
    st = _lib.lib().nd_pair_hash_dev(ctx.handle, ptr(pi_dev), ptr(pj_dev), ptr(pd_dev),
                                     int(npairs), h)
    ctx.check(st, "pair hash")
    return int(h[0]), int(h[1])

"""Forces and dynamics: the GPU mirror of src/Forces.jl and src/Simulator.jl.

  force_lennardjones_  force_lennardjones!(force, pairslist, position)  Forces.jl:15-45
  force_coulomb_       force_coulomb!(force, pairslist, charge)          Forces.jl:56-66
  sum_forces_          sum_forces!(force, f1, f2)                        Forces.jl:68-75
  SimSpec              SimSpec(; duration, stepwidth, ...)               Simulator.jl:30-49
  simulate_            simulate!(sys, spec, clct)                        Simulator.jl:154-256
  MDEngine             device-resident form of the simulate! step loop

Julia's `f!` (mutates its first argument) is spelled `f_` here.  The physics
is the intended one (truncated Lennard-Jones + cutoff Coulomb with direction,
Newton's third law, kick-drift-kick velocity Verlet, reflecting walls), not the
reference's scalar broadcast; sigma, epsilon, k and the cutoff are keywords
instead of the constants hard-coded at Forces.jl:17-19,57.
"""
from __future__ import annotations

import ctypes
import os
import json
import hashlib
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (MDParams, ND_ORDER_SPATIAL, ND_UNION_BLOCKS, ND_UNION_TREE,
                   default_context, ptr)

__all__ = ["ForceField", "md_params", "force_lennardjones_", "force_coulomb_", "sum_forces_",
           "force_lennardjones_compat_", "force_coulomb_compat_",
           "forces", "SimSpec", "GenericObjectCollection", "GenericRandomCollector", "simulate_",
           "MDEngine", "Ensemble", "systems_table", "autotune"]


@dataclass
class ForceField:
    sigma: float = 1.0
    epsilon: float = 1.0
    coulomb_k: float = 1.0
    cutoff: float = 2.5


def md_params(sigma=1.0, epsilon=1.0, coulomb_k=0.0, cutoff=2.5, skin=0.3, dt=1e-3,
              box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0), atomsperleaf=4, rebuild_every=10,
              order=ND_ORDER_SPATIAL, max_neighbors=0, resort_every=0,
              stage_policy=0, union_search=ND_UNION_BLOCKS, refit_check_every=1,
              threads_per_atom=0, cta_split=0) -> MDParams:
    p = MDParams()
    p.sigma, p.epsilon, p.coulomb_k, p.cutoff, p.skin, p.dt = (float(sigma), float(epsilon),
                                                               float(coulomb_k), float(cutoff),
                                                               float(skin), float(dt))
    for d in range(3):
        p.box_lo[d] = float(box_lo[d])
        p.box_hi[d] = float(box_hi[d])
    p.atomsperleaf, p.rebuild_every, p.order, p.max_neighbors = (int(atomsperleaf),
                                                                 int(rebuild_every), int(order),
                                                                 int(max_neighbors))
    p.resort_every, p.stage_policy = int(resort_every), int(stage_policy)
    p.union_search, p.refit_check_every = int(union_search), int(refit_check_every)
    p.threads_per_atom, p.cta_split = int(threads_per_atom), int(cta_split)
    return p


def _f64(a, shape=None):
    x = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return x.reshape(shape) if shape is not None else x


def _pair_arrays(pairslist):
    if isinstance(pairslist, np.ndarray) and pairslist.dtype.names:
        return (np.ascontiguousarray(pairslist["i"], np.int32),
                np.ascontiguousarray(pairslist["j"], np.int32))
    arr = np.asarray([(p[0], p[1]) for p in pairslist], dtype=np.int32).reshape(-1, 2)
    return np.ascontiguousarray(arr[:, 0]), np.ascontiguousarray(arr[:, 1])


def _pair_forces(force, pairslist, position, charge, p, ctx):
    ctx = ctx or default_context()
    x = _f64(position, (-1, 3))
    n = x.shape[0]
    pi, pj = _pair_arrays(pairslist)
    q = None if charge is None else _f64(charge)
    f = np.empty((n, 3), np.float32)
    e = ctypes.c_double()
    st = _lib.lib().nd_forces_pairs(ctx.handle, ctypes.byref(p), n, ptr(x), ptr(q), ptr(pi),
                                    ptr(pj), pi.shape[0], ptr(f), ctypes.byref(e))
    ctx.check(st, "nd_forces_pairs")
    if force is not None:
        np.copyto(np.asarray(force).reshape(n, 3), f, casting="unsafe")
    return f, e.value


def force_lennardjones_(force, pairslist, position, sigma=1.0, epsilon=1.0, cutoff=2.5,
                        ctx=None):
    """force_lennardjones!(force, pairslist, position): force is overwritten.

    F_ij = 24 eps / r^2 (2 (sigma/r)^12 - (sigma/r)^6) r_ij for listed pairs with
    r < cutoff; returns the LJ potential energy."""
    p = md_params(sigma=sigma, epsilon=epsilon, coulomb_k=0.0, cutoff=cutoff)
    return _pair_forces(force, pairslist, position, None, p, ctx)[1]


def force_coulomb_(force, pairslist, charge, position, k=1.0, cutoff=2.5, ctx=None):
    """force_coulomb!(force, pairslist, charge): force is overwritten.

    F_ij = k q_i q_j r_ij / r^3 for listed pairs with r < cutoff.  Unlike the
    reference signature it needs the positions for the direction."""
    p = md_params(sigma=1.0, epsilon=0.0, coulomb_k=k, cutoff=cutoff)
    return _pair_forces(force, pairslist, position, charge, p, ctx)[1]


def _compat_pairs(pairslist):
    if isinstance(pairslist, np.ndarray) and pairslist.dtype.names:
        i, j, d = pairslist["i"], pairslist["j"], pairslist["d"]
    elif isinstance(pairslist, dict):
        i, j, d = pairslist["i"], pairslist["j"], pairslist["d"]
    else:
        i, j, d = pairslist
    return (np.ascontiguousarray(i, np.int32), np.ascontiguousarray(j, np.int32),
            np.ascontiguousarray(d, np.float32))


def force_lennardjones_compat_(force, pairslist, position=None, ctx=None):
    """force_lennardjones! as the reference computes it (Forces.jl:6-45):
    force[i] .+= (24 eps / d) ((2 sigma / d)^12 - (sigma / d)^6) for every pair
    in list order with its hard-coded eps = -1f10, sigma = 0.0001, the same
    scalar on all three components and nothing on force[j].  force (N x 3
    Float32) is overwritten; position is not used (as in the reference)."""
    ctx = ctx or default_context()
    i, j, d = _compat_pairs(pairslist)
    out = np.zeros((np.asarray(force).shape[0], 3), np.float32)
    ctx.check(_lib.lib().nd_compat_force_lennardjones(ctx.handle, out.shape[0], ptr(i), ptr(j),
                                                      ptr(d), len(i), ptr(out)),
              "nd_compat_force_lennardjones")
    force[...] = out
    return force


def force_coulomb_compat_(force, pairslist, charge, ctx=None):
    """force_coulomb! as the reference computes it (Forces.jl:46-66): for
    every pair in list order force[i] .+= q_i q_j / d^2, then force[j] .-=
    force[i] (its running total).  force (N x 3 Float32) is overwritten."""
    ctx = ctx or default_context()
    i, j, d = _compat_pairs(pairslist)
    q = np.ascontiguousarray(charge, np.float32)
    out = np.zeros((np.asarray(force).shape[0], 3), np.float32)
    ctx.check(_lib.lib().nd_compat_force_coulomb(ctx.handle, out.shape[0], ptr(i), ptr(j),
                                                 ptr(d), len(i), ptr(q), ptr(out)),
              "nd_compat_force_coulomb")
    force[...] = out
    return force


def sum_forces_(force, force1, force2):
    """sum_forces!(force, f1, f2) (Forces.jl:68-75)."""
    np.add(force1, force2, out=force)
    return force


def forces(position, charge=None, ff: ForceField | None = None, ctx=None):
    """Fused LJ + Coulomb forces and energy with the library's own neighbour search."""
    ff = ff or ForceField()
    ctx = ctx or default_context()
    x = _f64(position, (-1, 3))
    n = x.shape[0]
    q = None if charge is None else _f64(charge)
    lo, hi = x.min(0), x.max(0)
    p = md_params(sigma=ff.sigma, epsilon=ff.epsilon, coulomb_k=ff.coulomb_k if q is not None else 0.0,
                  cutoff=ff.cutoff, skin=0.0, box_lo=lo, box_hi=hi)
    f = np.empty((n, 3), np.float32)
    e = ctypes.c_double()
    st = _lib.lib().nd_forces(ctx.handle, ctypes.byref(p), n, ptr(x), ptr(q), ptr(f), ctypes.byref(e))
    ctx.check(st, "nd_forces")
    return f, e.value


@dataclass
class SimSpec:
    """SimSpec (Simulator.jl:30-49): duration (steps) and stepwidth (dt)."""
    duration: int
    stepwidth: float
    currentstep: int = 1
    logLength: int = 10
    vDamp: float = 0.0
    threshold: float = 0.0


@dataclass
class GenericRandomCollector:
    """GenericRandomCollector (MDInput.jl:67-84): the box and temperature the
    step loop uses, and the ranges collect_objects draws from."""
    objectnumber: int
    minDim: tuple
    maxDim: tuple
    temperature: float = 0.0
    minimumdistance: float = 0.0
    randomvelocity: bool = False
    minmass: float = 1.0
    maxmass: float = 1.0
    mincharge: float = 0.0
    maxcharge: float = 0.0


@dataclass
class GenericObjectCollection:
    """GenericObjectCollection (MDInput.jl:33-46), struct-of-arrays per atom."""
    position: np.ndarray
    velocity: np.ndarray
    force: np.ndarray | None = None
    mass: np.ndarray | None = None
    charge: np.ndarray | None = None
    index: np.ndarray | None = field(default=None)

    def __post_init__(self):
        self.position = _f64(self.position, (-1, 3)).copy()
        self.velocity = _f64(self.velocity, (-1, 3)).copy()
        n = self.position.shape[0]
        if self.force is None:
            self.force = np.zeros((n, 3), np.float32)
        if self.index is None:
            self.index = np.arange(1, n + 1, dtype=np.int64)


def collect_objects(clct: GenericRandomCollector, seed: int = 0, ctx=None):
    """collect_objects(clct) (MDInput.jl:305-369) on the GPU: masses, charges
    and positions uniform in the collector's ranges, velocities from its
    temperature (randomvelocity: a random split per component), and the
    reference's pruning as written -- atoms closer than clct.minimumdistance to
    a later atom (the last atom excepted) get Inf positions, their number in
    the result's `pruned`.  The draws come from a counter-based stream of
    `seed`, not Julia's RNG: same distributions, different values.  Returns a
    GenericObjectCollection (Float32 values)."""
    ctx = ctx or default_context()
    n = int(clct.objectnumber)
    cl = _lib.Collector(n, (ctypes.c_float * 3)(*clct.minDim), (ctypes.c_float * 3)(*clct.maxDim),
                        clct.temperature, int(bool(clct.randomvelocity)), clct.minmass,
                        clct.maxmass, clct.minimumdistance, clct.mincharge, clct.maxcharge)
    x = np.empty((n, 3), np.float32)
    v = np.empty((n, 3), np.float32)
    m = np.empty(n, np.float32)
    q = np.empty(n, np.float32)
    pruned = ctypes.c_int64(0)
    ctx.check(_lib.lib().nd_collect_objects(ctx.handle, ctypes.byref(cl), int(seed), ptr(x),
                                            ptr(v), ptr(m), ptr(q), ctypes.byref(pruned)),
              "nd_collect_objects")
    sys = GenericObjectCollection(x, v, mass=m, charge=q)
    sys.pruned = int(pruned.value)
    return sys


def _warn_skin(violations: int):
    if violations > 0:
        warnings.warn(f"{violations} atom-steps ran on neighbour lists that an atom had left by "
                      "more than skin/2 (pairs may have been missed): raise the skin or check "
                      "for early refits after every step (refit_check_every=1)",
                      RuntimeWarning, stacklevel=3)


def simulate_(sys: GenericObjectCollection, spec: SimSpec, clct: GenericRandomCollector,
              ff: ForceField | None = None, skin=0.3, atomsperleaf=4, rebuild_every=10,
              order=ND_ORDER_SPATIAL, log_every: int | None = None, refit_check_every=1,
              ctx=None):
    """simulate!(sys, spec, clct) (Simulator.jl:154-256) on the GPU.

    Advances sys.position / sys.velocity in place by spec.duration steps of
    kick-drift-kick velocity Verlet with reflecting walls at clct.minDim /
    clct.maxDim, and stores the final forces in sys.force.  As in the
    reference step loop, a non-zero spec.vDamp applies rescale_velocity!
    towards clct.temperature every 10 steps (Simulator.jl:241-243).  With
    log_every, the positions after every log_every-th step are logged on the
    device and returned, the initial positions first -- the poslog that
    simulate! returns (log_every = 1); otherwise sys is returned.  A
    RuntimeWarning reports atom-steps that ran on a list an atom had left by
    more than skin/2 (possible with refit_check_every > 1 on fast atoms)."""
    ff = ff or ForceField()
    ctx = ctx or default_context()
    n = sys.position.shape[0]
    q = None if sys.charge is None else _f64(sys.charge)
    m = None if sys.mass is None else _f64(sys.mass)
    p = md_params(sigma=ff.sigma, epsilon=ff.epsilon,
                  coulomb_k=ff.coulomb_k if q is not None else 0.0, cutoff=ff.cutoff, skin=skin,
                  dt=spec.stepwidth, box_lo=clct.minDim, box_hi=clct.maxDim,
                  atomsperleaf=atomsperleaf, rebuild_every=rebuild_every, order=order,
                  refit_check_every=refit_check_every)
    if not log_every and not spec.vDamp:
        f = np.empty((n, 3), np.float32)
        st = _lib.lib().nd_simulate(ctx.handle, ctypes.byref(p), n, ptr(sys.position),
                                    ptr(sys.velocity), ptr(f), ptr(q), ptr(m),
                                    int(spec.duration))
        ctx.check(st, "nd_simulate")
        sys.force = f
        d = _lib.MDDiag()
        ctx.check(_lib.lib().nd_simulate_diagnostics(ctx.handle, ctypes.byref(d)),
                  "nd_simulate_diagnostics")
        _warn_skin(d.skin_violations)
        return sys
    x0 = sys.position.copy()
    eng = MDEngine(p, sys.position, sys.velocity, q, m, ctx=ctx)
    try:
        if spec.vDamp:
            eng.set_thermostat(clct.temperature, spec.vDamp, 10)
        frames = int(spec.duration) // log_every if log_every else 0
        if frames:
            eng.set_log(log_every, frames)
        eng.run(int(spec.duration))
        x, v, f = eng.get()
        poslog = eng.log_read(0, frames) if frames else None
        _warn_skin(eng.diagnostics()["skin_violations"])
    finally:
        eng.close()
    sys.position[...] = x
    sys.velocity[...] = v
    sys.force = f
    if log_every:
        return np.concatenate([x0[None], poslog]) if frames else x0[None]
    return sys


def simulate_compat_(sys: GenericObjectCollection, spec: SimSpec, clct: GenericRandomCollector,
                     log: bool = True, ctx=None):
    """simulate!(sys, spec, clct) as the reference computes it
    (Simulator.jl:154-256): the all-pairs list of unique_pairs, the
    bug-compatible force calls (force_lennardjones! on the pairs closer than
    0.01, then on all pairs; force_coulomb! on all pairs), x += v dt +
    a(t) dt^2 / 2, v += (a(t) + a(t - dt)) dt / 2, boundary_reflect!, and
    rescale_velocity! every 10 steps towards clct.temperature with gamma =
    spec.vDamp -- in Float32 with an integer spec.stepwidth, as the
    reference's SimSpec{Int64, Float32} holds it.

    Updates sys.position / sys.velocity / sys.force (Float64 arrays holding
    Float32 values) and returns the poslog, (duration + 1) x N x 3 Float32:
    element 0 is the final positions (the reference's poslog[1] is
    sys.position itself), element k the positions after step k.  Raises
    NDError where the reference raises DomainError (a negative
    rescale_velocity! radicand); sys then holds the state at that point."""
    ctx = ctx or default_context()
    if int(spec.stepwidth) != spec.stepwidth:
        raise ValueError("SimSpec{Int64, Float32} holds an integer stepwidth")
    n = sys.position.shape[0]
    x = np.ascontiguousarray(sys.position, np.float32).copy()
    v = np.ascontiguousarray(sys.velocity, np.float32).copy()
    f = np.ascontiguousarray(sys.force, np.float32).reshape(n, 3).copy()
    m = np.ones(n, np.float32) if sys.mass is None else np.ascontiguousarray(sys.mass, np.float32)
    q = (np.zeros(n, np.float32) if sys.charge is None
         else np.ascontiguousarray(sys.charge, np.float32))
    cs = _lib.CompatSim((ctypes.c_float * 3)(*clct.minDim), (ctypes.c_float * 3)(*clct.maxDim),
                        clct.temperature, int(clct.objectnumber), int(spec.stepwidth),
                        int(spec.duration), spec.vDamp)
    poslog = np.zeros((int(spec.duration) + 1, n, 3), np.float32) if log else None
    st = _lib.lib().nd_compat_simulate(ctx.handle, ctypes.byref(cs), n, ptr(x), ptr(v), ptr(f),
                                       ptr(m), ptr(q), ptr(poslog))
    sys.position[...] = x
    sys.velocity[...] = v
    sys.force = f
    ctx.check(st, "nd_compat_simulate")
    return poslog


class MDEngine:
    """Device-resident simulation state (nd_md_*).

    Host arrays (numpy) are copied once; with device=True, x/v/q/m are device
    pointers (torch tensors or ints) and nothing crosses the host boundary."""

    def __init__(self, params: MDParams, x, v, q=None, m=None, device=False, ctx=None):
        self.ctx = ctx or default_context()
        self.params = params
        h = ctypes.c_void_p()
        if device:
            n = int(x.shape[0]) if hasattr(x, "shape") else None
            st = _lib.lib().nd_md_create_dev(self.ctx.handle, ctypes.byref(params), n, ptr(x),
                                             ptr(v), ptr(q), ptr(m), ctypes.byref(h))
        else:
            x = _f64(x, (-1, 3))
            v = _f64(v, (-1, 3))
            n = x.shape[0]
            qq = None if q is None else _f64(q)
            mm = None if m is None else _f64(m)
            st = _lib.lib().nd_md_create(self.ctx.handle, ctypes.byref(params), n, ptr(x), ptr(v),
                                         ptr(qq), ptr(mm), ctypes.byref(h))
        self.ctx.check(st, "nd_md_create")
        self.handle = h.value
        self.n = n

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().nd_md_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, steps: int):
        self.ctx.check(_lib.lib().nd_md_run(self.handle, int(steps)), "nd_md_run")

    def sync(self):
        self.ctx.check(_lib.lib().nd_md_sync(self.handle), "nd_md_sync")

    def get(self):
        x = np.empty((self.n, 3), np.float64)
        v = np.empty((self.n, 3), np.float64)
        f = np.empty((self.n, 3), np.float32)
        self.ctx.check(_lib.lib().nd_md_get(self.handle, ptr(x), ptr(v), ptr(f)), "nd_md_get")
        return x, v, f

    def get_dev(self, x=None, v=None, f=None):
        self.ctx.check(_lib.lib().nd_md_get_dev(self.handle, ptr(x), ptr(v), ptr(f)),
                       "nd_md_get_dev")

    def energy(self):
        pe, ke = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(_lib.lib().nd_md_energy(self.handle, ctypes.byref(pe), ctypes.byref(ke)),
                       "nd_md_energy")
        return pe.value, ke.value

    def set_thermostat(self, temperature: float, gamma: float, every: int = 10):
        """rescale_velocity! (Simulator.jl:119-144) after every `every`-th step;
        every = 0 switches it off."""
        self.ctx.check(_lib.lib().nd_md_set_thermostat(self.handle, float(temperature),
                                                       float(gamma), int(every)),
                       "nd_md_set_thermostat")

    def set_log(self, every: int, frames: int):
        """Position log (simulate!'s poslog) after every `every`-th step into a
        device ring of `frames` frames; every = 0 switches it off."""
        self.ctx.check(_lib.lib().nd_md_set_log(self.handle, int(every), int(frames)),
                       "nd_md_set_log")

    def log_count(self) -> int:
        c = ctypes.c_int64()
        self.ctx.check(_lib.lib().nd_md_log_count(self.handle, ctypes.byref(c)), "nd_md_log_count")
        return c.value

    def log_read(self, first: int, nframes: int) -> np.ndarray:
        out = np.empty((nframes, self.n, 3), np.float64)
        self.ctx.check(_lib.lib().nd_md_log_read(self.handle, int(first), int(nframes), ptr(out)),
                       "nd_md_log_read")
        return out

    def stats(self):
        s, r, p = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        cap = ctypes.c_int32()
        self.ctx.check(_lib.lib().nd_md_stats(self.handle, ctypes.byref(s), ctypes.byref(r),
                                              ctypes.byref(p), ctypes.byref(cap)), "nd_md_stats")
        return dict(steps=s.value, rebuilds=r.value, list_pairs=p.value, capacity=cap.value)

    def diagnostics(self):
        d = _lib.MDDiag()
        self.ctx.check(_lib.lib().nd_md_diagnostics(self.handle, ctypes.byref(d)),
                       "nd_md_diagnostics")
        return {name: getattr(d, name) for name, _ in d._fields_ if name != "reserved"}

    def list_pairs(self):
        """The engine's current neighbour lists: (i, j, near) arrays of directed
        entries (1-based caller indices; each unordered pair once from each
        side), near = 1 for the near segment."""
        n = ctypes.c_int64()
        st = _lib.lib().nd_md_list_pairs(self.handle, None, None, None, 0, ctypes.byref(n))
        if st not in (0, 1):
            self.ctx.check(st, "nd_md_list_pairs")
        cap = n.value
        pi = np.empty(cap, np.int32)
        pj = np.empty(cap, np.int32)
        near = np.empty(cap, np.uint8)
        self.ctx.check(_lib.lib().nd_md_list_pairs(self.handle, ptr(pi), ptr(pj), ptr(near), cap,
                                                   ctypes.byref(n)), "nd_md_list_pairs")
        return pi, pj, near

    def step_times(self, steps: int):
        """Advance `steps` steps eagerly, timing each step kernel with CUDA
        events on the context stream; returns the durations in ms."""
        ms = np.empty(int(steps), np.float32)
        self.ctx.check(_lib.lib().nd_md_step_times(self.handle, int(steps), ptr(ms)),
                       "nd_md_step_times")
        return ms

    def launches_per_run(self, steps: int) -> int:
        return int(_lib.lib().nd_md_launches_per_run(self.handle, int(steps)))


def systems_table(n_atoms, sigma, epsilon, box_lo, box_hi):
    """ctypes array of nd_system rows from per-system sequences (box_lo/box_hi:
    nsys x 3)."""
    n_atoms = np.asarray(n_atoms)
    ns = len(n_atoms)
    arr = (_lib.System * ns)()
    lo = np.asarray(box_lo, np.float64).reshape(ns, 3)
    hi = np.asarray(box_hi, np.float64).reshape(ns, 3)
    for k in range(ns):
        r = arr[k]
        r.n_atoms = int(n_atoms[k])
        r.sigma = float(sigma[k])
        r.epsilon = float(epsilon[k])
        for d in range(3):
            r.box_lo[d] = float(lo[k, d])
            r.box_hi[d] = float(hi[k, d])
    return arr


class Ensemble(MDEngine):
    """Batched ensemble (nd_batch_create): independent systems of uneven sizes
    advanced together, one launch per step over all of them.  x, v are the
    systems' (N_s x 3) arrays concatenated in order; `systems` is the table from
    systems_table().  run/get/energy/diagnostics behave as for MDEngine
    (energy() sums the systems); energies() gives per-system values."""

    def __init__(self, params: MDParams, systems, x, v, q=None, m=None, device=False, ctx=None):
        self.ctx = ctx or default_context()
        self.params = params
        self.systems = systems
        self.nsys = len(systems)
        self.offsets = np.concatenate([[0], np.cumsum([r.n_atoms for r in systems])])
        h = ctypes.c_void_p()
        if device:
            st = _lib.lib().nd_batch_create_dev(self.ctx.handle, ctypes.byref(params), self.nsys,
                                                systems, ptr(x), ptr(v), ptr(q), ptr(m),
                                                ctypes.byref(h))
        else:
            x = _f64(x, (-1, 3))
            v = _f64(v, (-1, 3))
            qq = None if q is None else _f64(q)
            mm = None if m is None else _f64(m)
            st = _lib.lib().nd_batch_create(self.ctx.handle, ctypes.byref(params), self.nsys,
                                            systems, ptr(x), ptr(v), ptr(qq), ptr(mm),
                                            ctypes.byref(h))
        self.ctx.check(st, "nd_batch_create")
        self.handle = h.value
        self.n = int(self.offsets[-1])

    def energies(self):
        pe = np.empty(self.nsys, np.float64)
        ke = np.empty(self.nsys, np.float64)
        self.ctx.check(_lib.lib().nd_batch_energies(self.handle, ptr(pe), ptr(ke)),
                       "nd_batch_energies")
        return pe, ke


TUNED_FIELDS = ("skin", "atomsperleaf", "resort_every", "stage_policy", "union_search",
                "refit_check_every", "threads_per_atom", "cta_split")


def autotune_cache_path() -> str:
    """The tuned-settings cache: $ND_AUTOTUNE_CACHE, else
    ~/.cache/naivedynamics/autotune.json."""
    return os.environ.get("ND_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "naivedynamics", "autotune.json")


# the tuner's candidate set: a cached result from another set is not reused
TUNER_VERSION = 3


def _tune_key(ctx, params: MDParams, n: int, systems, has_q: bool, has_m: bool) -> str:
    """Cache key: the device, the atom count, the density (1e-3 relative),
    everything of params the tuner does not change (cutoff, walls, dt, ...)
    and the tuner's version; for an ensemble the systems' sizes, sigmas,
    epsilons and walls."""
    fixed = {name: (list(getattr(params, name)) if name in ("box_lo", "box_hi")
                    else getattr(params, name))
             for name, _ in params._fields_ if name not in TUNED_FIELDS}
    if systems is None:
        vol = float(np.prod(np.asarray(params.box_hi) - np.asarray(params.box_lo)))
        shape = {"n": n, "density": float(f"{n / vol:.4g}")}
    else:
        h = hashlib.sha256()
        for r in systems:
            h.update(np.array([r.n_atoms, r.sigma, r.epsilon, *r.box_lo, *r.box_hi],
                              np.float64).tobytes())
        shape = {"n": n, "systems": len(systems), "table": h.hexdigest()[:16]}
    return json.dumps({"device": ctx.device_name(), "shape": shape, "fixed": fixed,
                       "q": has_q, "m": has_m, "tuner": TUNER_VERSION}, sort_keys=True)


def autotune(params: MDParams, x, v, q=None, m=None, systems=None, trial_steps=20, ctx=None,
             use_cache=True):
    """nd_md_autotune: the fastest (skin, atomsperleaf, resort_every,
    stage_policy, union_search, refit_check_every, threads_per_atom, cta_split) for this
    state, as a new MDParams, and its time per MD step in seconds.
    systems=None tunes a plain engine.  With use_cache, the result is kept in
    a JSON file (autotune_cache_path()) keyed by device, atom count, density
    and the untuned parameters, and a later call with the same key returns it
    without timing anything; autotune.last_cached tells which happened."""
    ctx = ctx or default_context()
    x = _f64(x, (-1, 3))
    v = _f64(v, (-1, 3))
    qq = None if q is None else _f64(q)
    mm = None if m is None else _f64(m)
    key = path = None
    if use_cache:
        key = _tune_key(ctx, params, x.shape[0], systems, q is not None, m is not None)
        path = autotune_cache_path()
        try:
            with open(path) as f:
                hit = json.load(f).get(key)
        except (OSError, ValueError):
            hit = None
        if hit:
            best = MDParams()
            ctypes.memmove(ctypes.byref(best), ctypes.byref(params), ctypes.sizeof(MDParams))
            for name in TUNED_FIELDS:
                setattr(best, name, hit["params"][name])
            autotune.last_cached = True
            return best, float(hit["seconds_per_step"])
    best = MDParams()
    sps = ctypes.c_double()
    ns = 0 if systems is None else len(systems)
    st = _lib.lib().nd_md_autotune(ctx.handle, ctypes.byref(params), x.shape[0], ns, systems,
                                   ptr(x), ptr(v), ptr(qq), ptr(mm), int(trial_steps),
                                   ctypes.byref(best), ctypes.byref(sps))
    ctx.check(st, "nd_md_autotune")
    autotune.last_cached = False
    if use_cache:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            try:
                with open(path) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
            table[key] = {"params": {name: getattr(best, name) for name in TUNED_FIELDS},
                          "seconds_per_step": sps.value}
            tmp = f"{path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass  # a read-only home: tuned, not cached
    return best, sps.value


autotune.last_cached = False

"""naivedynamics (GB300): Python host mirror of NaiveDynamics.jl's hot path.

The compute path is libnaivegpu (CUDA, sm_103a) behind the C ABI declared in
include/naivegpu.h; this package only marshals arguments.  Importing it loads
the library and fails loudly if it has not been built.
"""
from . import _lib
from ._lib import (Context, NDError, SpecError, InexactError, default_context,
                   ND_ORDER_REFERENCE, ND_ORDER_SPATIAL, ND_PAIRS_ORDERED, ND_PAIRS_UNORDERED,
                   ND_CRIT_SQUARED, ND_CRIT_SQRT, ND_UNION_BLOCKS, ND_UNION_TREE,
                   GRIDKEY_DTYPE, PAIR_DTYPE)
from .bvh import (SpheresBVHSpecs, APointPrimitive, leafTreeData, TreeData,
                  leafbuild_traverse_bvh, simdbuild_traverse_bvh, build_traverse_bvh,
                  gpubvh_neighborlist, gpubvh_neighborlist_, neighbor_pairs_dev,
                  pair_hash_dev)
from .dynamics import (ForceField, md_params, force_lennardjones_, force_coulomb_, sum_forces_,
                       force_lennardjones_compat_, force_coulomb_compat_,
                       forces, SimSpec, GenericObjectCollection, GenericRandomCollector,
                       simulate_, simulate_compat_, collect_objects, MDEngine, Ensemble,
                       systems_table, autotune, autotune_cache_path, TUNED_FIELDS)
from .adjoint import Adjoint, adj_spec, histogram_loss_function
from . import synth

_lib.lib()  # load now: no CPU fallback exists

__all__ = [n for n in dir() if not n.startswith("_")]

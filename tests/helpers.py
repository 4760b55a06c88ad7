"""Helpers shared by the test modules."""
import json
import os

import numpy as np

from conftest import canon  # noqa: F401

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bvh_golden.json")


def golden_cases():
    with open(GOLDEN) as f:
        return json.load(f)


def uniform(seed, n, side=1.0):
    """Seeded uniform Float32 positions in [0, side)^3 (reference test families)."""
    rng = np.random.default_rng(seed)
    return (rng.random((n, 3)) * side).astype(np.float32)


def force_errors(f32, f64):
    """(max_i |dF_i| / max(|F64_i|, 1e-3 rms), |dF|_2 / |F64|_2)."""
    f32 = np.asarray(f32, np.float64)
    df = np.linalg.norm(f32 - f64, axis=1)
    nf = np.linalg.norm(f64, axis=1)
    rms = np.sqrt(np.mean(nf ** 2))
    floor = 1e-3 * rms
    per_atom = float(np.max(df / np.maximum(nf, floor)))
    l2 = float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))
    return per_atom, l2

"""Shared helpers of the test suite: fixtures as systems, GPU handles, error metrics."""

from __future__ import annotations

import ast
import os

import numpy as np

from biospring_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

ARRAY_KEYS = ("xyz", "vel", "mass", "charge", "radius", "epsilon", "hydrophobicity", "sasa", "transfer",
              "is_static")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def system_from_golden(g: dict, prefix: str = "in_", name: str = "golden") -> W.System:
    cfg = ast.literal_eval(str(g[prefix + "config"][0]))
    kw = {k: g[prefix + k] for k in ARRAY_KEYS if prefix + k in g and k != "xyz"}
    return W.System(name, g[prefix + "xyz"], g[prefix + "ij"], g[prefix + "r0"], g[prefix + "k"], cfg, **kw)


def gpu_network(system: W.System, config=None):
    from biospring_gb300 import SpringNetwork
    net = SpringNetwork()
    net.addParticles(**{k: v for k, v in system.arrays().items() if v is not None})
    if system.ij.shape[0]:
        net.addSprings(system.ij, system.r0, system.k)
    if system.bodies and system.config.get("rigidbody_enable"):
        net.setRigidBodies(system.bodies)
    net.setup(system.bs_config() if config is None else config)
    return net


def rel_l2(a: np.ndarray, b: np.ndarray, mask=None) -> float:
    """||a - b||_2 / ||b||_2 over the (masked) rows, in float64."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def rel_scalar(a: float, b: float, floor: float = 1e-30) -> float:
    return abs(a - b) / max(abs(b), floor)


def dynamic_mask(system: W.System) -> np.ndarray:
    if system.is_static is None:
        return np.ones(system.n, bool)
    return np.asarray(system.is_static) == 0

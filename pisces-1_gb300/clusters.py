"""Seeded synthetic water clusters for the eigensolve workloads.

Rigid monomers with the model's own geometry (OH 0.9572 A, HOH 104.52 deg;
the reference model frame, src/ttm_data.h:8-9, so the rigid-body projection in
the site producer is near-identity).  Oxygen sites are drawn uniformly in a
sphere with a minimum O-O distance by rejection, orientations uniformly on
SO(3) through uniform unit quaternions; all randomness comes from
numpy.random.Generator(PCG64(seed)).  Coordinates are Angstrom, one row of
nine numbers (O, H1, H2) per water -- the reference's water input layout
(src/GetInput.cpp:256).
"""
from __future__ import annotations

import numpy as np

ROH = 0.9572
HOH_DEG = 104.52
ANGS2BOHR = 1.0 / 0.52917720859


def _monomer_body():
    half = np.deg2rad(HOH_DEG) / 2.0
    o = np.zeros(3)
    h1 = np.array([0.0, ROH * np.sin(half), ROH * np.cos(half)])
    h2 = np.array([0.0, -ROH * np.sin(half), ROH * np.cos(half)])
    return np.stack([o, h1, h2])


def _quat_to_rot(q):
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
    ])


def random_rotation(rng):
    q = rng.normal(size=4)
    return _quat_to_rot(q / np.linalg.norm(q))


def _uniform_in_sphere(rng, radius):
    while True:
        p = rng.uniform(-radius, radius, size=3)
        if p @ p <= radius * radius:
            return p


def water_cluster(n_waters: int, radius: float, seed: int, min_oo: float = 2.6, max_tries: int = 200000):
    """(n_waters, 9) Angstrom coordinates of a seeded rigid-water cluster."""
    rng = np.random.Generator(np.random.PCG64(seed))
    oxy = []
    tries = 0
    while len(oxy) < n_waters:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"cannot place {n_waters} waters in a {radius} A sphere with O-O >= {min_oo} A")
        p = _uniform_in_sphere(rng, radius)
        if all(np.linalg.norm(p - o) >= min_oo for o in oxy):
            oxy.append(p)
    body = _monomer_body()
    out = np.empty((n_waters, 9))
    for i, o in enumerate(oxy):
        R = random_rotation(rng)
        out[i] = (body @ R.T + o).reshape(-1)
    return out


def place_ions(waters: np.ndarray, radius: float, seed: int, charges=(1.0, -1.0), min_dist: float = 2.8,
               max_tries: int = 200000):
    """Ion sites (x, y, z, q) in Angstrom, uniformly in the sphere and at least
    min_dist from every oxygen and from each other."""
    rng = np.random.Generator(np.random.PCG64(seed))
    oxy = np.asarray(waters).reshape(-1, 9)[:, :3]
    ions = []
    tries = 0
    for q in charges:
        while True:
            tries += 1
            if tries > max_tries:
                raise RuntimeError("cannot place ions")
            p = _uniform_in_sphere(rng, radius)
            if np.all(np.linalg.norm(oxy - p, axis=1) >= min_dist) and all(
                    np.linalg.norm(p - np.asarray(i[:3])) >= min_dist for i in ions):
                ions.append([p[0], p[1], p[2], q])
                break
    return np.asarray(ions)


def jitter(waters: np.ndarray, rng, sigma: float = 0.1, rot_deg: float = 5.0):
    """Per-request perturbation of a base cluster: every monomer is shifted by
    a Gaussian displacement (sigma Angstrom per component) and turned about a
    random axis through its oxygen by rot_deg degrees."""
    w = np.asarray(waters, dtype=np.float64).reshape(-1, 3, 3).copy()
    for m in w:
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = np.deg2rad(rot_deg)
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * (K @ K)
        o = m[0].copy()
        m[:] = (m - o) @ R.T + o + rng.normal(scale=sigma, size=3)
    return w.reshape(-1, 9)

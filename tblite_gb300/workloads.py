"""Seeded synthetic molecules for the benchmark configurations.

All positions are returned in Bohr (one fixed Angstrom->Bohr constant shared
by every engine).  The constructions follow the benchmark definitions:

* water clusters: O on a cubic lattice with 3.0 A spacing, each O jittered by
  U(-0.2, 0.2) A per axis, rigid H2O (O-H 0.96 A, H-O-H 104.5 deg) with a
  uniformly random orientation (Haar-random unit quaternion);
* linear alkanes CnH2n+2: zig-zag backbone with C-C 1.53 A, C-C-C 112 deg,
  dihedrals 180 deg (p = 0.7) or +-65 deg (p = 0.15 each), C-H 1.09 A with
  tetrahedral placement.
"""
from __future__ import annotations

import math

import numpy as np

AA2BOHR = 1.0 / 0.52917721092


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def water_cluster(shape, seed, spacing=3.0, jitter=0.2):
    """(H2O)_k with O on an (nx, ny, nz) lattice.  Returns (numbers, positions/Bohr)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    half = math.radians(104.5) / 2
    tmpl = np.array([[0.0, 0.0, 0.0],
                     [0.96 * math.sin(half), 0.0, 0.96 * math.cos(half)],
                     [-0.96 * math.sin(half), 0.0, 0.96 * math.cos(half)]])
    nums, pos = [], []
    for ix in range(nx):
        for iy in range(ny):
            for iz in range(nz):
                o = np.array([ix, iy, iz], dtype=float) * spacing
                o += rng.uniform(-jitter, jitter, 3)
                rot = _random_rotation(rng)
                for k, z in enumerate((8, 1, 1)):
                    nums.append(z)
                    pos.append(o + rot @ tmpl[k])
    return np.array(nums, dtype=np.int32), np.array(pos) * AA2BOHR


def water_cluster_k(k, seed):
    """k waters on the smallest enclosing near-cubic lattice (first k sites)."""
    m = 1
    while m ** 3 < k:
        m += 1
    nums, pos = water_cluster((m, m, m), seed)
    return nums[: 3 * k], pos[: 3 * k]


def _place(a, b, c, bond, angle, dihedral):
    """Position of d given a-b-c, |cd|, angle bcd and dihedral abcd (NeRF)."""
    bc = c - b
    bc /= np.linalg.norm(bc)
    n = np.cross(b - a, bc)
    n /= np.linalg.norm(n)
    m = np.cross(n, bc)
    d2 = np.array([-bond * math.cos(angle), bond * math.sin(angle) * math.cos(dihedral),
                   bond * math.sin(angle) * math.sin(dihedral)])
    return c + d2[0] * bc + d2[1] * m + d2[2] * n


def alkane(nc, seed):
    """CnH2n+2 (n >= 1).  Returns (numbers, positions/Bohr)."""
    rng = np.random.default_rng(seed)
    cc, ch = 1.53, 1.09
    ccc = math.radians(112.0)
    carbons = [np.zeros(3)]  # noqa: E501
    if nc >= 2:
        carbons.append(np.array([cc, 0.0, 0.0]))
    if nc >= 3:
        carbons.append(carbons[1] + cc * np.array([-math.cos(ccc), math.sin(ccc), 0.0]))
    for i in range(3, nc):
        u = rng.random()
        dih = math.pi if u < 0.7 else (math.radians(65.0) if u < 0.85 else math.radians(-65.0))
        # a long random chain can fold back onto itself: keep carbons that are four or
        # more bonds apart at least 3.9 A apart, trying the other dihedrals if needed
        for cand in (dih, math.pi, math.radians(65.0), math.radians(-65.0)):
            new = _place(carbons[i - 3], carbons[i - 2], carbons[i - 1], cc, ccc, cand)
            if i < 4 or min(np.linalg.norm(new - carbons[j]) for j in range(i - 3)) > 3.9:
                break
        carbons.append(new)
    carbons = np.array(carbons)
    hs = []
    tet = math.radians(109.4712206)
    for i in range(nc):
        c = carbons[i]
        nb = [carbons[j] for j in (i - 1, i + 1) if 0 <= j < nc]
        if len(nb) == 0:  # methane
            for v in ([1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]):
                hs.append(c + ch * np.array(v) / math.sqrt(3.0))
        elif len(nb) == 1:  # CH3
            a = nb[0]
            v = c - a
            v /= np.linalg.norm(v)
            ref = carbons[i - 2] if i >= 2 else (carbons[i + 2] if i + 2 < nc else None)
            t = np.array([0.0, 0.0, 1.0]) if ref is None else ref - a
            e1 = t - (t @ v) * v
            if np.linalg.norm(e1) < 1e-8:
                e1 = np.cross(v, [1.0, 0.0, 0.0])
            e1 /= np.linalg.norm(e1)
            e2 = np.cross(v, e1)
            for k in range(3):
                phi = math.pi + 2 * math.pi * k / 3  # staggered
                d = math.cos(math.pi - tet) * v + math.sin(math.pi - tet) * (
                    math.cos(phi) * e1 + math.sin(phi) * e2)
                hs.append(c + ch * d)
        else:  # CH2
            a, b = nb
            u1 = (a - c) / np.linalg.norm(a - c)
            u2 = (b - c) / np.linalg.norm(b - c)
            bis = -(u1 + u2)
            bis /= np.linalg.norm(bis)
            w = np.cross(u1, u2)
            w /= np.linalg.norm(w)
            half = tet / 2
            for sgn in (1.0, -1.0):
                hs.append(c + ch * (math.cos(half) * bis + sgn * math.sin(half) * w))
    nums = np.array([6] * nc + [1] * len(hs), dtype=np.int32)
    pos = np.vstack([carbons, np.array(hs)]) * AA2BOHR
    return nums, pos


def config(name):
    """Named benchmark workloads: returns (numbers, positions/Bohr)."""
    if name == "h2o32":
        return water_cluster((4, 4, 2), seed=0)
    if name == "c200h402":
        return alkane(200, seed=1)
    if name == "c100h202":  # half-size chain (602 AOs): small case for kernel captures
        return alkane(100, seed=1)
    if name == "h2o1000":
        return water_cluster((10, 10, 10), seed=2)
    raise KeyError(name)


def alkane_batch(count=256, seed=3, nmin=4, nmax=40):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count)
    return [alkane(int(n), seed=seed * 100003 + i) for i, n in enumerate(sizes)]


def mixed_ensemble(count=4096, seed=4):
    """50 % water clusters k ~ log-uniform[1, 64], 50 % alkanes n ~ log-uniform[1, 60]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        if i % 2 == 0:
            k = int(math.floor(math.exp(rng.uniform(0.0, math.log(65.0)))))
            out.append(water_cluster_k(max(1, min(k, 64)), seed=seed * 1000003 + i))
        else:
            n = int(math.floor(math.exp(rng.uniform(0.0, math.log(61.0)))))
            out.append(alkane(max(1, min(n, 60)), seed=seed * 1000003 + i))
    return out

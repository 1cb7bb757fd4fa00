"""Seeded synthetic docking inputs with the shapes of the scan workloads.

The reference ships no benchmark set for its FFT scan; the workloads are
seeded synthetic pairs:

* a molecule of ``n`` heavy atoms is a random-walk chain with 3.8 A steps
  folded into a sphere of radius ``(3 n / (4 pi 0.05))^(1/3)`` (density
  0.05 atoms/A^3): a step that would leave the sphere is redrawn;
* elements are C 62 %, N 17 %, O 20 %, S 1 %; each atom also gets an
  ACE-style type in ``0..n_types-1`` from the same seed;
* rotations are Shoemake uniform quaternions turned into row-major 3x3
  matrices;
* the 18x18 desolvation matrix is symmetric, uniform in [-1, 1].

The receptor is centred at its bounding-box centre and the ligand at the
midpoint of its two most distant atoms (its diameter centre), the frames the
reference moves the pair into before the scan
(``include/PRODDL/docking_molstruct.hpp:199-245``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

ELEMENTS = ("C", "N", "O", "S")
ELEMENT_P = (0.62, 0.17, 0.20, 0.01)
STEP = 3.8
DENSITY = 0.05


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def globule(n, rng, density=DENSITY, step=STEP):
    """Random-walk chain of ``n`` atoms inside a sphere of matching density."""
    radius = (3.0 * n / (4.0 * math.pi * density)) ** (1.0 / 3.0)
    pts = np.zeros((n, 3))
    cur = np.zeros(3)
    for i in range(1, n):
        for _ in range(1000):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            nxt = cur + step * d
            if nxt @ nxt <= radius * radius:
                break
        else:
            nxt = cur * 0.9
        cur = nxt
        pts[i] = cur
    return pts


def box_centre(xyz):
    return 0.5 * (xyz.min(axis=0) + xyz.max(axis=0))


def diameter_centre(xyz):
    """Midpoint of the two most distant atoms (exact, blocked O(n^2))."""
    best = -1.0
    pair = (0, 0)
    n = xyz.shape[0]
    blk = 512
    for i0 in range(0, n, blk):
        a = xyz[i0:i0 + blk]
        d2 = ((a[:, None, :] - xyz[None, :, :]) ** 2).sum(-1)
        j = int(np.argmax(d2))
        r, c = divmod(j, n)
        if d2[r, c] > best:
            best = float(d2[r, c])
            pair = (i0 + r, c)
    return 0.5 * (xyz[pair[0]] + xyz[pair[1]])


@dataclass
class Molecule:
    xyz: np.ndarray        # (n, 3) float64
    element: np.ndarray    # (n,) int8 index into ELEMENTS
    ace_type: np.ndarray   # (n,) int32 in 0..n_types-1


def molecule(n, seed, n_types=18):
    rng = _rng(seed)
    xyz = globule(n, rng)
    element = rng.choice(len(ELEMENTS), size=n, p=ELEMENT_P).astype(np.int8)
    ace_type = rng.integers(0, n_types, size=n).astype(np.int32)
    return Molecule(xyz, element, ace_type)


def quaternion_rotations(n, seed):
    """Shoemake uniform random rotations as (n, 3, 3) row-major matrices."""
    rng = _rng(seed)
    u = rng.random((n, 3))
    s1 = np.sqrt(1.0 - u[:, 0])
    s2 = np.sqrt(u[:, 0])
    a1 = 2.0 * math.pi * u[:, 1]
    a2 = 2.0 * math.pi * u[:, 2]
    x, y = s1 * np.sin(a1), s1 * np.cos(a1)
    z, w = s2 * np.sin(a2), s2 * np.cos(a2)
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z)
    r[:, 0, 1] = 2 * (x * y - z * w)
    r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w)
    r[:, 1, 1] = 1 - 2 * (x * x + z * z)
    r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w)
    r[:, 2, 1] = 2 * (y * z + x * w)
    r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def ace_matrix(n_types, seed):
    rng = _rng(seed)
    m = rng.uniform(-1.0, 1.0, size=(n_types, n_types))
    return np.triu(m) + np.triu(m, 1).T


@dataclass
class Pair:
    receptor: Molecule
    ligand: Molecule
    rotations: np.ndarray
    ace: np.ndarray


def make_pair(n_rec, n_lig, n_rot, seed, n_types=18):
    """A receptor/ligand pair in scan frames plus a rotation set."""
    rec = molecule(n_rec, seed * 4 + 1, n_types)
    lig = molecule(n_lig, seed * 4 + 2, n_types)
    rec.xyz = rec.xyz - box_centre(rec.xyz)
    lig.xyz = lig.xyz - diameter_centre(lig.xyz)
    rots = quaternion_rotations(n_rot, seed * 4 + 3)
    return Pair(rec, lig, rots, ace_matrix(n_types, seed * 4 + 4))


def lj_params(n, seed, alpha=0.4):
    """Per-atom (sigma, eps, alpha) for the LJ potentials: sigma uniform in
    [3.0, 3.9] A, eps in [0.05, 0.6], alpha constant (the reference's option
    generator uses alpha 0.4)."""
    rng = _rng(seed)
    return rng.uniform(3.0, 3.9, n), rng.uniform(0.05, 0.6, n), np.full(n, float(alpha))


def uneven_pairs(n_pairs, seed, rec_range=(800, 6000), lig_range=(300, 2000), n_types=18):
    """Pairs with log-uniform receptor and ligand sizes (the batched-workload
    generator): a list of (receptor, ligand) molecules in scan frames."""
    rng = _rng(seed)
    out = []
    for i in range(n_pairs):
        nr = int(round(math.exp(rng.uniform(math.log(rec_range[0]), math.log(rec_range[1])))))
        nl = int(round(math.exp(rng.uniform(math.log(lig_range[0]), math.log(lig_range[1])))))
        rec = molecule(nr, seed * 100003 + 2 * i + 1, n_types)
        lig = molecule(nl, seed * 100003 + 2 * i + 2, n_types)
        rec.xyz = rec.xyz - box_centre(rec.xyz)
        lig.xyz = lig.xyz - diameter_centre(lig.xyz)
        out.append((rec, lig))
    return out


# Workloads quoted by the scan benchmarks: name -> (n_rec, n_lig, N, h, terms, n_rot, batch, peaks)
WORKLOADS = {
    "shape64": dict(n_rec=1800, n_lig=450, grid_n=64, grid_step=1.2, term_set="shape",
                    n_rot=2000, rot_batch=64, peaks=4, top=100),
    "shape_ace128": dict(n_rec=4000, n_lig=1500, grid_n=128, grid_step=1.2, term_set="shape_ace",
                         n_rot=9000, rot_batch=64, peaks=4, top=100),
    # the reference's default potential (ljComp, K = 2) at the same size
    "ljcomp128": dict(n_rec=4000, n_lig=1500, grid_n=128, grid_step=1.2, term_set="lj_comp",
                      n_rot=9000, rot_batch=64, peaks=4, top=100),
    # precision study: the 64^3 workload's molecules at 128^3, FP32 vs BF16-stored
    # receptor spectra, every rotation's 16 best cells rescored in FP64
    "precision128": dict(n_rec=1800, n_lig=450, grid_n=128, grid_step=1.2, term_set="shape",
                         n_rot=20000, rot_batch=64, peaks=16, top=100),
    # many uneven pairs: receptors 800-6000 / ligands 300-2000 atoms (log-uniform),
    # grid edge per pair from pair_grid (48-144), shape + 18 desolvation terms
    "pairs256": dict(n_pairs=256, grid_step=1.2, term_set="shape_ace", n_rot=3000, rot_batch=64, peaks=4),
}

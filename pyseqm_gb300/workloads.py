"""Seeded synthetic molecules with the shapes of the benchmark workloads.

* n-alkanes C_nH_{2n+2}: ideal staggered zig-zag chain, C-C 1.54 A, C-H 1.09 A,
  tetrahedral angles, every atom displaced by N(0, sigma).
* water clusters (H2O)_k: O-H 0.957 A, H-O-H 104.5 deg, uniformly random
  orientation, O centres on a jittered cubic lattice.

Atoms of every molecule are ordered by descending atomic number (heavy atoms
first, hydrogens last), which is the order the seqm API requires.
"""

import math

import numpy as np

TETRA = math.acos(-1.0 / 3.0)
CC, CH = 1.54, 1.09
OH, HOH = 0.957, math.radians(104.5)


def _unit(v):
    return v / np.linalg.norm(v)


def _perp_pair(a):
    t = np.array([0.0, 0.0, 1.0]) if abs(a[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    e1 = _unit(np.cross(a, t))
    e2 = np.cross(a, e1)
    return e1, e2


def alkane(n, rng=None, sigma=0.0):
    """(species, coords[A]) of C_nH_{2n+2}; heavy atoms first."""
    half = TETRA / 2.0
    cpos = np.array([[k * CC * math.sin(half), (k % 2) * CC * math.cos(half), 0.0] for k in range(n)])
    hpos = []
    if n == 1:
        dirs = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float) / math.sqrt(3.0)
        hpos = [cpos[0] + CH * d for d in dirs]
    else:
        for k in range(n):
            nbrs = [cpos[j] - cpos[k] for j in (k - 1, k + 1) if 0 <= j < n]
            if len(nbrs) == 2:
                a, b = _unit(nbrs[0]), _unit(nbrs[1])
                d = -_unit(a + b)
                nrm = _unit(np.cross(a, b))
                ang = TETRA / 2.0
                for s in (1.0, -1.0):
                    hpos.append(cpos[k] + CH * (d * math.cos(ang) + s * nrm * math.sin(ang)))
            else:
                a = _unit(nbrs[0])
                e1, e2 = _perp_pair(a)
                # put one hydrogen in the chain plane, anti to the C-C bond direction pattern
                inplane = _unit(np.cross(np.array([0.0, 0.0, 1.0]), a))
                if np.dot(inplane, e1) < 0:
                    inplane = -inplane
                e1 = inplane
                e2 = np.cross(a, e1)
                for i in range(3):
                    phi = 2.0 * math.pi * i / 3.0
                    dvec = -a / 3.0 + math.sqrt(8.0 / 9.0) * (math.cos(phi) * e1 + math.sin(phi) * e2)
                    hpos.append(cpos[k] + CH * dvec)
    coords = np.vstack([cpos, np.array(hpos)])
    species = np.array([6] * n + [1] * (2 * n + 2), dtype=np.int64)
    if rng is not None and sigma > 0:
        coords = coords + rng.normal(0.0, sigma, size=coords.shape)
    return species, coords


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster(k, rng, spacing=2.9, jitter=0.2, side=None):
    """(species, coords[A]) of (H2O)_k; O centres on the first k sites of a cubic lattice."""
    side = side or int(math.ceil(round(k ** (1.0 / 3.0), 9)))
    sites = np.array([[i, j, l] for i in range(side) for j in range(side) for l in range(side)], dtype=float)
    sites = sites[:k] * spacing + rng.uniform(-jitter, jitter, size=(k, 3))
    h1 = np.array([OH, 0.0, 0.0])
    h2 = np.array([OH * math.cos(HOH), OH * math.sin(HOH), 0.0])
    o_pos, h_pos = [], []
    for c in sites:
        R = _random_rotation(rng)
        o_pos.append(c)
        h_pos.append(c + R @ h1)
        h_pos.append(c + R @ h2)
    coords = np.vstack([np.array(o_pos), np.array(h_pos)])
    species = np.array([8] * k + [1] * (2 * k), dtype=np.int64)
    return species, coords


def pad_batch(mols):
    """List of (species, coords) -> padded (species[nmol, molsize], coords[nmol, molsize, 3])."""
    molsize = max(s.size for s, _ in mols)
    species = np.zeros((len(mols), molsize), dtype=np.int64)
    coords = np.zeros((len(mols), molsize, 3))
    for i, (s, c) in enumerate(mols):
        species[i, : s.size] = s
        coords[i, : s.size] = c
    return species, coords


def butane_batch(nmol=16, seed=0, sigma=0.03):
    """16 perturbed n-butanes (PM3 plain-path workload)."""
    rng = np.random.default_rng(seed)
    return [alkane(4, rng, sigma) for _ in range(nmol)]


def mixed_batch(nmol=4096, seed=0, sigma=0.03, alkane_range=(1, 16), water_range=(2, 24)):
    """50/50 alkanes C_n (n uniform in alkane_range) and (H2O)_k (k uniform in water_range)."""
    rng = np.random.default_rng(seed)
    mols = []
    for i in range(nmol):
        if i % 2 == 0:
            mols.append(alkane(int(rng.integers(alkane_range[0], alkane_range[1] + 1)), rng, sigma))
        else:
            mols.append(water_cluster(int(rng.integers(water_range[0], water_range[1] + 1)), rng))
    return mols


def big_water(seed=0, n_side=10, spacing=3.1, jitter=0.25):
    """(H2O)_{n_side^3} on a jittered n_side^3 lattice."""
    rng = np.random.default_rng(seed)
    return water_cluster(n_side**3, rng, spacing=spacing, jitter=jitter, side=n_side)


def request_molecules(n, seed=0, atoms=(3, 600), force_frac=0.1, sigma=0.03):
    """Molecules of a request stream: size log-uniform in `atoms` (number of atoms), drawn 50/50
    from the alkane generator (C_kH_{2k+2}, 3k + 2 atoms) and the water-cluster generator
    ((H2O)_k, 3k atoms) at the nearest size; a fraction `force_frac` also asks for forces.
    Returns [(species, coords, forces)]."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(atoms[0]), math.log(atoms[1])
    out = []
    for _ in range(n):
        na = math.exp(rng.uniform(lo, hi))
        if rng.random() < 0.5:
            sp, xyz = alkane(max(1, int(round((na - 2.0) / 3.0))), rng, sigma)
        else:
            sp, xyz = water_cluster(max(1, int(round(na / 3.0))), rng)
        out.append((sp, xyz, bool(rng.random() < force_frac)))
    return out


def poisson_arrivals(n, rate, seed=0):
    """Arrival times (s) of a Poisson process of the given rate (requests/s)."""
    rng = np.random.default_rng(seed + 7919)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))

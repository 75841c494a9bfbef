"""XYZ files in and out, as the reference's helpers read and write them (read_xyz,
read_xyz_trajectory, save_xyz).

``read_xyz`` follows seqm/seqm_functions/read_xyz.py:17-48 (one molecule per file, element
symbols or atomic numbers in the first column, atoms ordered by decreasing atomic number with a
stable sort, zero padding to the largest molecule); ``save_xyz`` follows
seqm/seqm_functions/save_xyz.py:4-45 (one ``<name>.<i>.xyz`` file per molecule with the total
energy in the comment line, coordinates and optionally forces in 15.5f columns, element symbols
from ``Constants.label``).
"""

import numpy as np
import torch

# element symbols H..Xe and their atomic numbers (the elements read_xyz accepts by symbol)
_SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se "
            "Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe").split()
ELEMENT_NUMBER = {sym: z for z, sym in enumerate(_SYMBOLS, start=1)}


def read_xyz(files, sort=True):
    """species (M, K) int and coordinates (M, K, 3) float of M xyz files, K the largest atom
    count, zero padded; sort: atoms by decreasing atomic number (stable)."""
    mols = []
    for fn in files:
        with open(fn) as f:
            lines = f.readlines()
        n = int(lines[0])
        rows = [ln.split() for ln in lines[2: 2 + n]]
        numeric = rows[0][0].isdigit()
        z = np.array([int(r[0]) if numeric else ELEMENT_NUMBER[r[0]] for r in rows], dtype=np.int64)
        xyz = np.array([[float(v) for v in r[1:4]] for r in rows], dtype=np.float64)
        if sort:
            order = np.argsort(-z, kind="stable")
            z, xyz = z[order], xyz[order]
        mols.append((z, xyz))
    K = max(z.size for z, _ in mols)
    species = np.zeros((len(mols), K), dtype=int)
    coords = np.zeros((len(mols), K, 3), dtype=float)
    for i, (z, xyz) in enumerate(mols):
        species[i, : z.size] = z
        coords[i, : z.size] = xyz
    return species, coords


def _frames(path):
    """(atom count, comment, atom lines) per frame of a concatenated xyz file."""
    with open(path) as f:
        lines = f.read().splitlines()
    out, i = [], 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i])
        block = lines[i + 2: i + 2 + n]
        if len(block) < n:
            raise ValueError("Truncated frame.")
        out.append((n, block))
        i += 2 + n
    return out


def _velocities(path, nframes, n):
    """Per frame of NEXMD's velocity.out: a comment, $VELOC, n lines vx vy vz, $ENDVELOC."""
    with open(path) as f:
        lines = f.read().splitlines()
    vel, i = [], 0
    for _ in range(nframes):
        if i + n + 3 > len(lines) or lines[i + 1].strip().upper() != "$VELOC":
            raise ValueError("Bad velocity.out ($VELOC).")
        v = np.array([[float(x) for x in ln.split()] for ln in lines[i + 2: i + 2 + n]], dtype=float)
        if v.shape != (n, 3):
            raise ValueError("Bad velocity.out (vector count).")
        if lines[i + 2 + n].strip().upper() != "$ENDVELOC":
            raise ValueError("Bad velocity.out ($ENDVELOC).")
        vel.append(v)
        i += n + 3
    return vel


def read_xyz_trajectory(file, start=0, stop=None, step=1, num=None, sort=True, vel_file=None, return_vel=False,
                        indices=None):
    """Frames of a concatenated xyz trajectory (NEXMD's coords.xyz; read_xyz.py:51-296):
    species (M, K) and coordinates (M, K, 3), with return_vel also the velocities of
    velocity.out (next to the file unless vel_file).  Frames: `indices` (in that order,
    duplicates kept, negative from the end), else start / stop / step, or `num` frames evenly
    between start and stop inclusive (rounded, unique).  The atom count must not change; the
    species and their order come from the first frame read, sorted by decreasing atomic number
    with equal ones in reverse file order (the reference's reversed stable argsort).  With stop
    None the frames run to the end of the file (the reference returns none there)."""
    import os

    if indices is not None and num is not None:
        raise ValueError("Use either indices or num, not both.")
    if indices is not None and step != 1:
        raise ValueError("When using indices, step must be 1.")
    if num is not None and step != 1:
        raise ValueError("Provide either step or num, not both.")
    if return_vel:
        vel_file = vel_file or os.path.join(os.path.dirname(file), "velocity.out")
        if not os.path.exists(vel_file):
            raise FileNotFoundError("velocity.out not found (or vel_file not provided).")
    frames = _frames(file)
    total = len(frames)
    if indices is not None:
        sel = [int(i) + total if int(i) < 0 else int(i) for i in indices]
    else:
        start = start + total if start < 0 else start
        if stop is not None and stop < 0:
            stop += total
        if num is None:
            sel = list(range(start, total if stop is None else stop, step))
        else:
            stop = total - 1 if stop is None else stop
            sel = np.unique(np.rint(np.linspace(start, stop, num=num)).astype(int)).tolist()
    sel = [i for i in sel if 0 <= i < total] if indices is None else sel
    empty = (np.zeros((0, 0), int), np.zeros((0, 0, 3), float))
    if not sel or total == 0:
        return empty + (empty[1].copy(),) if return_vel else empty
    K = frames[0][0]
    if any(n != K for n, _ in frames):
        raise ValueError("Variable atom count not supported in fast path.")
    first = frames[sel[0]][1]
    numeric = first[0].split()[0].isdigit()
    z = np.array([int(ln.split()[0]) if numeric else ELEMENT_NUMBER[ln.split()[0]] for ln in first], dtype=int)
    order = z.argsort(kind="stable")[::-1] if sort else np.arange(K)
    vel = _velocities(vel_file, total, K) if return_vel else None
    species = np.empty((len(sel), K), dtype=int)
    coords = np.empty((len(sel), K, 3), dtype=float)
    vels = np.empty((len(sel), K, 3), dtype=float) if return_vel else None
    for j, fr in enumerate(sel):
        xyz = np.array([[float(x) for x in ln.split()[1:4]] for ln in frames[fr][1]], dtype=float)
        species[j] = z[order]
        coords[j] = xyz[order]
        if return_vel:
            vels[j] = vel[fr][order]
    return (species, coords, vels) if return_vel else (species, coords)


def save_xyz(molecules, name, Forces=False):
    """One ``name.<i>.xyz`` per molecule of ``molecules`` (a Molecule after a calculation): atom
    count, ``Etot = <12.6f>`` (an empty comment line if the molecule has no energy), then per
    atom the symbol and the coordinates (and forces with Forces=True) in 15.5f columns."""
    species = molecules.species.detach().cpu()
    coords = molecules.coordinates.detach().cpu()
    force = molecules.force.detach().cpu() if Forces else None
    etot = molecules.Etot.detach().cpu() if torch.is_tensor(getattr(molecules, "Etot", None)) else None
    label = molecules.const.label
    for i in range(coords.shape[0]):
        with open(f"{name}.{i}.xyz", "w+") as f:
            n = int((species[i] > 0).sum())
            if etot is not None:
                f.write("{}\nEtot = {:12.6f} \n".format(n, float(etot[i])))
            else:
                f.write("{}\n\n".format(n))
            for a in range(coords.shape[1]):
                z = int(species[i, a])
                if z <= 0:
                    continue
                cols = [float(v) for v in coords[i, a]]
                if Forces:
                    cols += [float(v) for v in force[i, a]]
                f.write(label[z] + "".join(" {:15.5f}".format(v) for v in cols) + (" \n" if Forces else "\n"))

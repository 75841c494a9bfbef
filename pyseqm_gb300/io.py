"""XYZ files in and out, as the reference's helpers read and write them.

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

"""Functional entry point: one batched single point from host arrays.

``single_point`` is the call a user (or a C caller through the same ABI) makes
with HOST buffers: padded species/coordinates in, per-molecule energies out.
It builds the ragged layout on the host, uploads it, runs hcore + SCF + final
energies on the GPU and copies the results back.
"""

import numpy as np
import torch

from . import tables
from .layout import Layout
from .scf import BatchSCF


def single_point(species, coordinates, method="AM1", scf_eps=1.0e-8, scf_converger=(1,), sp2=(False,), charges=None,
                 device="cuda", learned=None, return_solver=False):
    """Energies (eV) of a batch of closed-shell molecules.

    species: (nmol, molsize) int, each row sorted by descending Z, 0 = padding.
    coordinates: (nmol, molsize, 3) Angstrom.
    Returns a dict of host numpy arrays: Etot, Eelec, Enuc, Eiso, Hf, iterations,
    notconverged (and the device solver if return_solver).
    """
    L = Layout.from_padded(species, coordinates, method, charges, learned).to_device(device)
    s = BatchSCF(L)
    s.hcore()
    nc = s.scf(scf_eps, tuple(scf_converger), tuple(sp2))
    Eelec, Enuc = s.final(want_vectors=False)
    host = torch.stack([Eelec, Enuc]).cpu().numpy()
    el = tables.elements()
    iso = _isolated_atom_energy(L)
    Eiso = np.bincount(L.atom_mol, weights=iso, minlength=L.nmol)
    eheat = np.bincount(L.atom_mol, weights=el["eheat_ev"][L.Z], minlength=L.nmol)
    Etot = host[0] + host[1]
    out = dict(Etot=Etot, Eelec=host[0], Enuc=host[1], Eiso=Eiso, Hf=Etot - Eiso + eheat,
               iterations=s.iters[: L.nmol].cpu().numpy(), notconverged=nc, launches=s.launches)
    if return_solver:
        out["solver"] = s
    return out


def _isolated_atom_energy(L):
    """Isolated-atom electronic energy per atom (seqm/seqm_functions/energy.py:8-23)."""
    el = tables.elements()
    from .native import PAR

    terms = (("U_ss", "ussc"), ("U_pp", "uppc"), ("g_ss", "gssc"), ("g_pp", "gppc"), ("g_sp", "gspc"),
             ("g_p2", "gp2c"), ("h_sp", "hspc"))
    Z = L.Z
    if not any(PAR[f] in L.learned for f, _ in terms):  # per element, then one gather
        tab = L.par_table
        per_el = sum(tab[PAR[f], : len(el[c])] * el[c] for f, c in terms)
        return per_el[Z]
    return sum(L.par_row(f) * el[c][Z] for f, c in terms)

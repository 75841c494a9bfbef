"""Geometry optimisation through the third-party geomeTRIC optimiser (optional dependency).

Follows seqm/optimization/geometry.py:21-107: a geomeTRIC engine whose energy and gradient come
from this package's Electronic_Structure (continuing the previous step's density, P0 = dm),
one frame per step appended to an xyz trajectory (``Step k, E = <Etot> eV``), Q-Chem-like
convergence criteria, and the last geometry written to ``optimized.xyz``.  One molecule at a
time, as in the reference.
"""

import os
import tempfile
import uuid

import torch


def _write_trajectory(path, step, molecule):
    """Append one frame: atom count, ``Step <k>, E = <Etot:.8f> eV``, symbol and 15.5f coordinates."""
    with open(path, "a") as out:
        out.write(f"{molecule.species.shape[1]}\nStep {step}, E = {float(molecule.Etot[0]):.8f} eV\n")
        coords = molecule.coordinates.detach().cpu()
        for a in range(coords.shape[1]):
            z = int(molecule.species[0, a])
            x = [float(v) for v in coords[0, a]]
            out.write(f"{molecule.const.label[z]} {x[0]:15.5f} {x[1]:15.5f} {x[2]:15.5f}\n")


def geomeTRIC_optimization(molecule, traj_file="geom_opt_traj.xyz", **run_kwargs):
    """Optimise the geometry of one molecule with geomeTRIC; run_kwargs go to its
    run_optimizer (maxsteps, ...)."""
    try:
        from geometric.engine import Engine
        from geometric.molecule import Elements
        from geometric.molecule import Molecule as GeomMolecule
        from geometric.nifty import bohr2ang, ev2au
        from geometric.optimize import run_optimizer
    except ImportError as e:
        raise ImportError("To use geometry-optimization with geomeTRIC, install the optional dependency "
                          "geomeTRIC (pip install geometric).") from e
    from .basics import Electronic_Structure

    if molecule.species.shape[0] != 1:
        raise ValueError("Geometry optimization with geomeTRIC does not work in batch mode, i.e., with inputs of "
                         "more than one molecule. Please input only one molecule")

    class _Engine(Engine):
        def __init__(self, mol, path):
            g = GeomMolecule()
            g.elem = [Elements[int(z)] for z in mol.species.detach().cpu().numpy()[0]]
            g.xyzs = [mol.coordinates.detach().cpu().numpy()[0].copy()]
            super().__init__(g)
            self.molecule, self.path, self.step = mol, path, 0
            self.driver = Electronic_Structure(mol.seqm_parameters)

        def calc_new(self, coords, dirname=None):
            m = self.molecule
            xyz = torch.tensor(coords.reshape(-1, 3) * bohr2ang, device=m.coordinates.device,
                               dtype=m.coordinates.dtype).unsqueeze(0)
            with torch.no_grad():
                m.coordinates = torch.nn.Parameter(xyz)
            self.driver(m, P0=m.dm, dm_prop="SCF")
            grad = (-m.force.detach().cpu().numpy()[0] * ev2au * bohr2ang).reshape(-1)  # eV/A -> Ha/bohr
            self.step += 1
            _write_trajectory(self.path, self.step, m)
            return {"energy": float(m.Etot[0]) * ev2au, "gradient": grad}

    engine = _Engine(molecule, traj_file)
    with tempfile.TemporaryDirectory() as tmp:
        result = run_optimizer(customengine=engine, input=os.path.join(tmp, str(uuid.uuid4())), qccnv=True,
                               **run_kwargs)
    with open("optimized.xyz", "w") as f:
        f.write("\n".join(result.write_xyz(selection=[-1])))
    return result


geometric_optimization = geomeTRIC_optimization

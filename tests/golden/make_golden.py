"""Generate the golden fixtures in this folder by running the PYSEQM reference.

This script is the only place that executes the reference.  It needs a PYSEQM
checkout, whose path is the one required argument, and runs on the CPU in float64.  ``h5py`` is
only needed by the reference's MD module, so a stub stands in for it.

Each fixture records the inputs (species, coordinates, seqm settings) and the
reference's outputs: Etot/Eelec/Enuc/Hf/Eiso, autograd forces, the converged
density (packed per molecule, hydrogen p-slots removed), orbital energies, the
SCF loop count (calls of ``fock_restricted`` minus the one before and the one
after the loop), per-molecule loop counts (each molecule run alone), and for the
"stages" fixtures the hcore blocks and two-electron integrals.

Usage:  python tests/golden/make_golden.py /path/to/PYSEQM
"""

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if len(sys.argv) != 2:
    sys.exit("usage: python make_golden.py <path to the PYSEQM source tree>")
REF = sys.argv[1]
# GOLDEN_ONLY=name1,name2 regenerates only those fixtures
ONLY = set(filter(None, os.environ.get("GOLDEN_ONLY", "").split(",")))

sys.path.insert(0, REPO)
sys.path.insert(0, REF)
h5 = types.ModuleType("h5py")
h5.Group = h5.File = h5.Dataset = type("Stub", (), {})
sys.modules.setdefault("h5py", h5)

import torch  # noqa: E402

torch.set_default_dtype(torch.float64)

import seqm.seqm_functions.scf_loop as scf_loop_mod  # noqa: E402
from seqm.basics import Energy  # noqa: E402
from seqm.ElectronicStructure import Electronic_Structure  # noqa: E402
from seqm.Molecule import Molecule  # noqa: E402
from seqm.seqm_functions.constants import Constants  # noqa: E402
from seqm.seqm_functions.hcore import hcore as ref_hcore  # noqa: E402
from seqm.seqm_functions.read_xyz import read_xyz  # noqa: E402

from pyseqm_gb300 import workloads  # noqa: E402

_calls = [0]
_orig_fock = scf_loop_mod.fock_restricted


def _counting_fock(*a, **k):
    _calls[0] += 1
    return _orig_fock(*a, **k)


scf_loop_mod.fock_restricted = _counting_fock
_orig_fock_u = scf_loop_mod.fock_u_batch


def _counting_fock_u(*a, **k):
    _calls[0] += 1
    return _orig_fock_u(*a, **k)


scf_loop_mod.fock_u_batch = _counting_fock_u


def packed_P(P, species):
    """Per molecule the density without the hydrogen p slots; (alpha, beta) pairs for UHF."""
    out = []
    for m in range(species.shape[0]):
        nh = int(np.sum(species[m] > 1))
        ny = int(np.sum(species[m] == 1))
        idx = np.concatenate([np.arange(4 * nh), 4 * nh + 4 * np.arange(ny)])
        if P.ndim == 4:
            out.append([P[m, s][np.ix_(idx, idx)].tolist() for s in range(2)])
        else:
            out.append(P[m][np.ix_(idx, idx)].tolist())
    return out


def run_es(species, coords, settings, learned=None, charges=None, mult=None):
    const = Constants()
    sp = dict(settings)
    sp["learned"] = list(learned.keys()) if learned else []
    sp.pop("elements", None)
    species_t = torch.as_tensor(species, dtype=torch.int64)
    coords_t = torch.as_tensor(coords, dtype=torch.float64)
    kw = {}
    if charges is not None:
        kw["charges"] = torch.as_tensor(charges, dtype=torch.float64)
    if mult is not None:
        kw["mult"] = torch.as_tensor(mult, dtype=torch.float64)
    mol = Molecule(const, sp, coords_t, species_t, **kw)
    mol.verbose = False
    _calls[0] = 0
    if learned:
        Z = mol.Z
        lp = {k: torch.as_tensor(np.asarray(v(Z.numpy())), dtype=torch.float64).requires_grad_(True)
              for k, v in learned.items()}
        mol.coordinates.requires_grad_(True)
        out = Energy(sp)(mol, learned_parameters=lp, all_terms=True)
        Hf, Etot, Eelec, Enuc, Eiso, EnucAB, e_gap, e, P, charge, nc = out
        Etot.sum().backward()
        grads = {k: mol.parameters[k].grad.detach().numpy().tolist() for k in learned}
        res = dict(Hf=Hf.detach().numpy().tolist(), Etot=Etot.detach().numpy().tolist(),
                   Eelec=Eelec.detach().numpy().tolist(), Enuc=Enuc.detach().numpy().tolist(),
                   Eiso=Eiso.detach().numpy().tolist(), e=e.detach().numpy().tolist(),
                   P=packed_P(P.detach().numpy(), species), notconverged=nc.numpy().tolist(),
                   dEtot_dR=mol.coordinates.grad.detach().numpy().tolist(), param_grads=grads,
                   loop_count=_calls[0] - 2, Z=Z.numpy().tolist())
        return res
    es = Electronic_Structure(sp)
    es(mol)
    return dict(Hf=mol.Hf.detach().numpy().tolist(), Etot=mol.Etot.detach().numpy().tolist(),
                Eelec=mol.Eelec.detach().numpy().tolist(), Enuc=mol.Enuc.detach().numpy().tolist(),
                Eiso=mol.Eiso.detach().numpy().tolist(), force=mol.force.detach().numpy().tolist(),
                e=mol.e_mo.detach().numpy().tolist(), P=packed_P(mol.dm.numpy(), species),
                notconverged=es.notconverged.numpy().tolist(), loop_count=_calls[0] - 2,
                q=mol.q.detach().numpy().tolist())


def stages(species, coords, method):
    const = Constants()
    sp = {"method": method, "scf_eps": 1e-6, "scf_converger": [1]}
    mol = Molecule(const, sp, torch.as_tensor(coords), torch.as_tensor(species, dtype=torch.int64))
    M, w, *_ = ref_hcore(mol)
    M = M.detach().numpy()
    return dict(M_diag=M[mol.maskd.numpy()].tolist(), M_pair=M[mol.mask.numpy()].tolist(),
                w=w.detach().numpy().tolist(), idxi=mol.idxi.numpy().tolist(), idxj=mol.idxj.numpy().tolist())


def write(name, species, coords, settings, per_molecule=False, learned=None, with_stages=False, ref_json=None,
          alone=False, charges=None, mult=None, extra=None):
    """alone: also record every molecule's energies, density and loop count from a run of that
    molecule by itself (for convergers whose state the reference shares across the batch)."""
    if ONLY and name not in ONLY:
        return
    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist())
    if charges is not None:
        rec["charges"] = list(charges)
    if mult is not None:
        rec["mult"] = list(mult)
    if extra:
        rec.update(extra)
    rec["ref"] = run_es(species, coords, settings, learned, charges, mult)
    if per_molecule:
        counts = []
        for m in range(species.shape[0]):
            n = int(np.sum(species[m] > 0))
            counts.append(run_es(species[m:m + 1, :n], coords[m:m + 1, :n], settings)["loop_count"])
        rec["ref"]["loop_count_per_molecule"] = counts
    if alone:
        runs = []
        for m in range(species.shape[0]):
            n = int(np.sum(species[m] > 0))
            r = run_es(species[m:m + 1, :n], coords[m:m + 1, :n], settings)
            runs.append(dict(Etot=r["Etot"][0], Eelec=r["Eelec"][0], P=r["P"][0], loop_count=r["loop_count"],
                             notconverged=r["notconverged"][0]))
        rec["ref"]["alone"] = runs
    if with_stages:
        rec["stages"] = stages(species, coords, settings["method"])
    if ref_json:
        with open(os.path.join(REF, "tests", "reference", ref_json)) as f:
            rec["reference_test_json"] = json.load(f)
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "loop_count", rec["ref"]["loop_count"])


def write_md(name, species, coords, settings, steps, timestep, seed, damp=None):
    """A short NVE (or Temp 0 Langevin) trajectory through the reference's own MD driver: its
    initialize() (momentum removal, first forces) and one_step() (velocity Verlet, P0 = the
    previous density), from seeded initial velocities (Angstrom / fs)."""
    if ONLY and name not in ONLY:
        return
    from seqm.MolecularDynamics import Molecular_Dynamics_Basic, Molecular_Dynamics_Langevin

    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    v0 = np.random.default_rng(seed).normal(size=coords.shape) * 0.01 * (species[..., None] > 0)
    sp = dict(settings)
    # a copy: the Molecule's coordinates share memory with the array given, and the MD moves them
    mol = Molecule(Constants(), sp, torch.as_tensor(coords.copy()), torch.as_tensor(species, dtype=torch.int64))
    mol.verbose = False
    mol.velocities = torch.as_tensor(v0.copy())
    out = {"molid": [0], "print every": 0, "checkpoint every": 0, "h5": {}}
    if damp is None:
        md = Molecular_Dynamics_Basic(sp, timestep=timestep, Temp=0.0, output=out)
    else:
        md = Molecular_Dynamics_Langevin(damp=damp, seqm_parameters=sp, timestep=timestep, Temp=0.0, output=out)
    _calls[0] = 0
    md.initialize(mol)
    traj = []

    def record(loops):
        with torch.no_grad():
            Ek = md._kinetic_energy(mol)
            traj.append(dict(coordinates=mol.coordinates.detach().numpy().tolist(),
                             velocities=mol.velocities.detach().numpy().tolist(),
                             force=mol.force.detach().numpy().tolist(), Etot=mol.Etot.detach().numpy().tolist(),
                             Ek=Ek.numpy().tolist(), T=md._calc_temperature(Ek).numpy().tolist(), loops=loops))

    record(_calls[0] - 2)
    for _ in range(steps):
        _calls[0] = 0
        md.one_step(mol)
        record(_calls[0] - 2)
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(),
               velocities0=v0.tolist(), timestep=timestep, steps=steps, damp=damp, ref={"trajectory": traj})
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "loops per step", [t["loops"] for t in traj])


def write_excited(name, species, coords, settings):
    """CIS / RPA excitation energies and amplitudes of the ground state through the reference's
    Electronic_Structure (basics.py:977-1029: rcis_batch for a batch of one species, the ragged
    rcis_any_batch otherwise, rpa)."""
    if ONLY and name not in ONLY:
        return
    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    sp = dict(settings)
    sp["excited_states"] = dict(settings["excited_states"])
    mol = Molecule(Constants(), sp, torch.as_tensor(coords.copy()), torch.as_tensor(species, dtype=torch.int64))
    mol.verbose = False
    Electronic_Structure(sp)(mol)
    amps = mol.cis_amplitudes.detach().numpy()
    # transition densities C_occ X C_virt^T in the packed AO basis (independent of the MO signs);
    # for RPA of X and of Y
    C = mol.molecular_orbitals.detach().numpy()
    nocc, norb = mol.nocc.numpy(), mol.norb.numpy()
    window = settings["excited_states"].get("orbital_window")
    if window is not None:  # occupied nocc-n .. nocc-1, virtual nocc .. nocc+m-1
        no_max, nv_max = int(window[0]), int(window[1])
    else:
        no_max, nv_max = int(nocc.max()), int((norb - nocc).max())
    sets = [amps[0], amps[1]] if amps.ndim == 4 else [amps]
    tdm = []
    for a in sets:
        per = []
        for m in range(species.shape[0]):
            n, no = int(norb[m]), int(nocc[m])
            lo, nw, mw = (no - no_max, no_max, nv_max) if window is not None else (0, no, n - no)
            X = a[m].reshape(a.shape[1], no_max, nv_max)[:, :nw, :mw]
            per.append(np.einsum("mi,ria,na->rmn", C[m, :n, lo:no], X, C[m, :n, no:no + mw]).tolist())
        tdm.append(per)
    # transition dipoles and oscillator strengths by the reference's own functions
    # (rcis_batch.py:679-710 for a batch of one species and RPA, rcis_new.py:547-585 otherwise)
    from seqm.seqm_functions.dipole import calc_dipole_matrix
    from seqm.seqm_functions.rcis_batch import calc_transition_dipoles
    from seqm.seqm_functions.rcis_new import calc_transition_dipoles_any_batch

    E = mol.cis_energies.detach()
    amp_t = mol.cis_amplitudes.detach()
    rpa = amps.ndim == 4
    amp_arg = (amp_t[0], amp_t[1]) if rpa else amp_t
    with torch.no_grad():
        if len(set(map(int, norb))) == 1 and len(set(map(int, nocc))) == 1:
            mu, f = calc_transition_dipoles(mol, amp_arg, E, E.shape[1], calc_dipole_matrix(mol), rpa,
                                            orbital_window=window)
        else:
            mu, f = calc_transition_dipoles_any_batch(mol, amp_arg, E, torch.full((species.shape[0],), E.shape[1]),
                                                      calc_dipole_matrix(mol), rpa)
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(),
               ref=dict(Etot=mol.Etot.detach().numpy().tolist(), cis_energies=mol.cis_energies.numpy().tolist(),
                        transition_dipole=mu.numpy().tolist(), oscillator_strength=f.numpy().tolist(),
                        cis_amplitudes=amps.tolist(), transition_densities=tdm,
                        e=mol.e_mo.detach().numpy().tolist(), nocc=nocc.tolist(), norb=norb.tolist()))
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "excitation energies", np.round(mol.cis_energies.numpy(), 4).tolist())


def write_reference_excited(name, xyz_names, settings, ref_json):
    """Inputs and values of one of the reference's own excited-state tests
    (tests/unit/test_excited_states.py): the molecules of its xyz files, its settings and its
    committed tests/reference/<ref_json>.json (excitation energies, oscillator strengths, and the
    forces of the first excited state, which its tests run as the active state)."""
    if ONLY and name not in ONLY:
        return
    data = os.path.join(REF, "tests", "data")
    species, coords = read_xyz([os.path.join(data, x) for x in xyz_names])
    with open(os.path.join(REF, "tests", "reference", ref_json)) as f:
        rj = json.load(f)
    rec = dict(name=name, settings=settings, species=np.asarray(species).tolist(),
               coords=np.asarray(coords, dtype=np.float64).tolist(),
               reference_test_json={k: rj[k] for k in ("cis_energies", "oscillator_strength", "force")})
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "reference energies", rj["cis_energies"])


def write_reference_md(name, xyz_names, driver, kwargs, steps, ref_json, tol, extra_settings=None):
    """Inputs, driver settings and committed values of one of the reference's own MD tests
    (tests/unit/test_md_suite.py: seed 0, Temp 300 K, timestep 0.5 fs, AM1, scf_eps 1e-7; its
    excited-state runs add CIS settings and active_state 1): per molecule the total energy per
    step, the drift and slope bounds it asserts."""
    if ONLY and name not in ONLY:
        return
    data = os.path.join(REF, "tests", "data")
    species, coords = read_xyz([os.path.join(data, x) for x in xyz_names])
    rec = dict(name=name, driver=driver, kwargs=kwargs, steps=steps, tol=tol,
               settings=dict({"method": "AM1", "scf_eps": 1.0e-7, "scf_converger": [1]}, **(extra_settings or {})),
               species=np.asarray(species).tolist(), coords=np.asarray(coords, dtype=np.float64).tolist())
    if ref_json:
        with open(os.path.join(REF, "tests", "reference", ref_json)) as f:
            rj = json.load(f)
        rec["reference_test_json"] = rj if isinstance(rj, list) else [rj]
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "written")


def write_nac(name, xyz_names, settings):
    """CIS nonadiabatic couplings through the reference's Electronic_Structure with
    seqm_parameters['nonadiabatic'] (basics.py:1042-1058, calc_nac nac.py:118-189): per state
    pair (0-based keys) the (nmol, molsize, 3) vectors, with the excitation energies."""
    if ONLY and name not in ONLY:
        return
    data = os.path.join(REF, "tests", "data")
    species, coords = read_xyz([os.path.join(data, x) for x in xyz_names])
    species, coords = np.asarray(species), np.asarray(coords, dtype=np.float64)
    sp = dict(settings)
    sp["excited_states"] = dict(settings["excited_states"])
    mol = Molecule(Constants(), sp, torch.as_tensor(coords.copy()), torch.as_tensor(species, dtype=torch.int64))
    mol.verbose = False
    Electronic_Structure(sp)(mol)
    nac = [[int(k[0]), int(k[1]), v.detach().numpy().tolist()] for k, v in mol.nac.items()]
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(),
               ref=dict(nac=nac, cis_energies=mol.cis_energies.detach().numpy().tolist()))
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "pairs", [(a, b) for a, b, _ in nac])


def write_param_dir(name, species, coords, method, src_dir, file_method):
    """A single point of the reference with seqm_parameters['parameter_file_dir'] (Pack_Parameters,
    basics.py:420-448): the parameters_<file_method>_MOPAC.csv and PWCCT files of src_dir, under
    the names `method` reads, in a scratch directory.  The fixture keeps the header and the rows of
    the batch's elements of each file, so a test can rebuild the directory."""
    if ONLY and name not in ONLY:
        return
    import tempfile

    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    zs = {int(z) for z in np.unique(species) if z > 0}
    files = {}
    with open(os.path.join(src_dir, f"parameters_{file_method}_MOPAC.csv")) as f:
        lines = f.read().splitlines()
    files[f"parameters_{method}_MOPAC.csv"] = "\n".join(
        [lines[0]] + [ln for ln in lines[1:] if ln.split(",")[0].strip().isdigit() and int(ln.split(",")[0]) in zs])
    pw = os.path.join(src_dir, f"PWCCT_{file_method}_MOPAC.csv")
    if method in ("PM6", "PM6_SP") and os.path.exists(pw):
        with open(pw) as f:
            files[f"PWCCT_{method}_MOPAC.csv"] = "\n".join(
                ln for ln in f.read().splitlines() if ln.strip() and {int(x) for x in ln.split(",")[:2]} <= zs)
    settings = {"method": method, "scf_eps": 1e-8, "scf_converger": [1]}
    with tempfile.TemporaryDirectory() as d:
        for fn, text in files.items():
            with open(os.path.join(d, fn), "w") as f:
                f.write(text + "\n")
        ref = run_es(species, coords, dict(settings, parameter_file_dir=d + "/"))
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(), param_files=files,
               ref=ref)
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "loop_count", ref["loop_count"])


def write_all_forces(name, xyz_names, settings):
    """do_all_forces through the reference's Electronic_Structure (basics.py:1124-1158): the
    ground and every excited state's forces and the states' relaxed / unrelaxed dipoles."""
    if ONLY and name not in ONLY:
        return
    data = os.path.join(REF, "tests", "data")
    species, coords = read_xyz([os.path.join(data, x) for x in xyz_names])
    species, coords = np.asarray(species), np.asarray(coords, dtype=np.float64)
    sp = dict(settings)
    sp["excited_states"] = dict(settings["excited_states"])
    mol = Molecule(Constants(), sp, torch.as_tensor(coords.copy()), torch.as_tensor(species, dtype=torch.int64))
    mol.verbose = False
    Electronic_Structure(sp)(mol)
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(),
               ref=dict(all_forces=mol.all_forces.detach().numpy().tolist(),
                        relaxed=mol.all_cis_relaxed_diploles.detach().numpy().tolist(),
                        unrelaxed=mol.all_cis_unrelaxed_diploles.detach().numpy().tolist(),
                        dipole=mol.dipole.detach().numpy().tolist(), cis_energies=mol.cis_energies.numpy().tolist()))
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "all_forces", np.asarray(rec["ref"]["all_forces"]).shape)


def write_xyz_io(name):
    """The reference's xyz helpers (read_xyz.py:17-48, save_xyz.py:4-45) on its test molecules:
    the xyz texts, read_xyz's arrays, and the files save_xyz writes (with and without forces)
    for an AM1 run of methane and benzene, with the energies and forces they print."""
    if ONLY and name not in ONLY:
        return
    import tempfile

    from seqm.seqm_functions.save_xyz import save_xyz as ref_save_xyz

    data = os.path.join(REF, "tests", "data")
    names = ["methane.xyz", "benzene.xyz", "methanal.1.xyz"]
    texts = {}
    for n in names:
        with open(os.path.join(data, n)) as f:
            texts[n] = f.read()
    reads = {}
    for group in (names[:2], names[2:], names):
        sp, c = read_xyz([os.path.join(data, n) for n in group])
        reads["+".join(group)] = dict(species=np.asarray(sp).tolist(), coords=np.asarray(c).tolist())
    sp, c = read_xyz([os.path.join(data, n) for n in names[:2]])
    settings = {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1]}
    mol = Molecule(Constants(), settings, torch.as_tensor(np.asarray(c, dtype=np.float64)),
                   torch.as_tensor(np.asarray(sp), dtype=torch.int64))
    mol.verbose = False
    Electronic_Structure(settings)(mol)
    saved = {}
    with tempfile.TemporaryDirectory() as d:
        for forces in (False, True):
            ref_save_xyz(mol, os.path.join(d, "out"), Forces=forces)
            for i in range(sp.shape[0]):
                with open(os.path.join(d, f"out.{i}.xyz")) as f:
                    saved[f"{int(forces)}.{i}"] = f.read()
    rec = dict(name=name, xyz=texts, read=reads, species=np.asarray(sp).tolist(),
               coords=np.asarray(c, dtype=np.float64).tolist(), Etot=mol.Etot.detach().numpy().tolist(),
               force=mol.force.detach().numpy().tolist(), saved=saved)
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "files", sorted(saved))


def write_traj_io(name):
    """The reference's read_xyz_trajectory (read_xyz.py:51-296) on a seeded 6-frame trajectory
    (element symbols, and atomic numbers) with its velocity.out, for several frame selections."""
    if ONLY and name not in ONLY:
        return
    import tempfile

    from seqm.seqm_functions.read_xyz import read_xyz_trajectory

    rng = np.random.default_rng(21)
    sym, num = ["C", "H", "O", "H", "H"], [6, 1, 8, 1, 1]
    xyz_s, xyz_n, vel = [], [], []
    for fr in range(6):
        xyz_s.append(f"5\nframe {fr}")
        xyz_n.append(f"5\nframe {fr}")
        vel.append(f"frame {fr}\n$VELOC")
        for a in range(5):
            x = rng.normal(size=3)
            u = rng.normal(size=3)
            xyz_s.append(f"{sym[a]} {x[0]:.6f} {x[1]:.6f} {x[2]:.6f}")
            xyz_n.append(f"{num[a]} {x[0]:.6f} {x[1]:.6f} {x[2]:.6f}")
            vel.append(f"{u[0]:.6f} {u[1]:.6f} {u[2]:.6f}")
        vel.append("$ENDVELOC")
    texts = {"coords.xyz": "\n".join(xyz_s) + "\n", "numeric.xyz": "\n".join(xyz_n) + "\n",
             "velocity.out": "\n".join(vel) + "\n"}
    cases = [dict(stop=6), dict(start=1, stop=6, step=2), dict(num=3, stop=5), dict(indices=[4, -1, 0, 4]),
             dict(start=-3, stop=6), dict(stop=6, return_vel=True), dict(indices=[2, 5], return_vel=True),
             dict(stop=3, sort=False)]
    out = []
    with tempfile.TemporaryDirectory() as d:
        for fn, t in texts.items():
            with open(os.path.join(d, fn), "w") as f:
                f.write(t)
        for file in ("coords.xyz", "numeric.xyz"):
            for kw in cases:
                r = read_xyz_trajectory(os.path.join(d, file), **kw)
                out.append(dict(file=file, kwargs=kw, result=[np.asarray(a).tolist() for a in r]))
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(dict(name=name, texts=texts, cases=out), f)
    print(name, len(out), "cases")


def write_xlbomd(name, species, coords, settings, steps, timestep, seed, k, krylov=None):
    """A short XL-BOMD trajectory (no thermostat, no Krylov kernel) through the reference's XL_BOMD
    driver: the first step's SCF, then the auxiliary density propagated with the k-th order
    dissipative coefficients and one diagonalisation of F(P) per step (MolecularDynamics.py:
    1380-1600, dynamics/xlbomd.py:58-505)."""
    if ONLY and name not in ONLY:
        return
    from seqm.MolecularDynamics import KSA_XL_BOMD, XL_BOMD

    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    v0 = np.random.default_rng(seed).normal(size=coords.shape) * 0.01 * (species[..., None] > 0)
    sp = dict(settings)
    mol = Molecule(Constants(), sp, torch.as_tensor(coords.copy()), torch.as_tensor(species, dtype=torch.int64))
    mol.verbose = False
    mol.velocities = torch.as_tensor(v0.copy())
    out = {"molid": [0], "print every": 0, "checkpoint every": 0, "h5": {}}
    params = dict({"k": k}, **(krylov or {}))
    cls = KSA_XL_BOMD if krylov else XL_BOMD
    md = cls(xl_bomd_params=params, seqm_parameters=sp, timestep=timestep, Temp=0.0, output=out)
    md.initialize(mol)
    traj = []

    def record():
        with torch.no_grad():
            Ek = md._kinetic_energy(mol)
            traj.append(dict(coordinates=mol.coordinates.detach().numpy().tolist(),
                             velocities=mol.velocities.detach().numpy().tolist(),
                             force=mol.force.detach().numpy().tolist(), Etot=mol.Etot.detach().numpy().tolist(),
                             Ek=Ek.numpy().tolist(), e_gap=mol.e_gap.detach().numpy().reshape(-1).tolist(),
                             entropy=mol.Electronic_entropy.detach().numpy().reshape(-1).tolist()))

    record()
    for i in range(steps):
        md._do_integrator_step(i, mol, {})
        record()
    rec = dict(name=name, settings=settings, species=species.tolist(), coords=coords.tolist(),
               velocities0=v0.tolist(), timestep=timestep, steps=steps, k=k, krylov=krylov,
               ref={"trajectory": traj})
    with open(os.path.join(HERE, f"{name}.json"), "w") as f:
        json.dump(rec, f)
    print(name, "Etot", [round(t["Etot"][0], 6) for t in traj])


def _open_shells():
    """CH3 (planar, doublet), OH (doublet), NO (doublet), CH2 (bent, triplet), O2 (triplet),
    H2O (singlet, run unrestricted)."""
    ang = np.radians(np.arange(3) * 120.0)
    ch3 = (np.array([6, 1, 1, 1]), np.vstack([[0.0, 0.0, 0.0], np.c_[1.08 * np.cos(ang), 1.08 * np.sin(ang),
                                                                     np.zeros(3)]]))
    oh = (np.array([8, 1]), np.array([[0.0, 0.0, 0.0], [0.98, 0.0, 0.0]]))
    no = (np.array([8, 7]), np.array([[0.0, 0.0, 0.0], [1.15, 0.0, 0.0]]))
    half = np.radians(134.0) / 2.0
    ch2 = (np.array([6, 1, 1]), np.array([[0.0, 0.0, 0.0], [1.08 * np.sin(half), 1.08 * np.cos(half), 0.0],
                                          [-1.08 * np.sin(half), 1.08 * np.cos(half), 0.0]]))
    o2 = (np.array([8, 8]), np.array([[0.0, 0.0, 0.0], [1.21, 0.0, 0.0]]))
    h2o = (np.array([8, 1, 1]), np.array([[0.0, 0.0, 0.0], [0.957, 0.0, 0.0], [-0.24, 0.927, 0.0]]))
    return [ch3, oh, no, ch2, o2, h2o], [2, 2, 2, 3, 3, 1]


# OH and NO put one electron of a spin into one of two exactly degenerate pi orbitals of the
# symmetric guess; which one is the eigensolver's arbitrary choice, so their densities are
# compared up to that choice (energies and orbital energies are unique)
OPEN_SHELL_DENSITY_AMBIGUOUS = [1, 2]


def _ions():
    """NH4+ (tetrahedral, N-H 1.02 A), OH- (0.97 A), H3O+ (pyramidal, O-H 0.98 A), H2O."""
    t = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float) / np.sqrt(3.0)
    nh4 = (np.array([7, 1, 1, 1, 1]), np.vstack([[0.0, 0.0, 0.0], 1.02 * t]))
    oh = (np.array([8, 1]), np.array([[0.0, 0.0, 0.0], [0.97, 0.0, 0.0]]))
    ang = np.radians(np.arange(3) * 120.0)
    h3o = (np.array([8, 1, 1, 1]), np.vstack([[0.0, 0.0, 0.0],
                                             np.c_[0.92 * np.cos(ang), 0.92 * np.sin(ang), np.full(3, 0.32)]]))
    h2o = (np.array([8, 1, 1]), np.array([[0.0, 0.0, 0.0], [0.957, 0.0, 0.0], [-0.24, 0.927, 0.0]]))
    return [nh4, oh, h3o, h2o]


def _sorted_mol(species, coords):
    """Atoms ordered by descending Z (the order the API requires)."""
    species = np.asarray(species)
    order = np.argsort(-species, kind="stable")
    return species[order], np.asarray(coords, dtype=np.float64)[order]


def _hetero():
    """Small molecules with Si, S, Cl, F and N: H3SiOH (the Si-O core-core exception), CH3SH,
    CH3Cl, CH3F, CH3NH2 and NH2OH; idealised bond lengths and angles."""
    tet = np.radians(109.47)

    def fan(center, bond, theta, phis):
        ph = np.radians(np.asarray(phis, dtype=float))
        return np.asarray(center) + bond * np.c_[np.sin(theta) * np.cos(ph), np.sin(theta) * np.sin(ph),
                                                 np.full(ph.size, np.cos(theta))]

    def ch3x(z, d):
        return _sorted_mol([6, z, 1, 1, 1], np.vstack([[0.0, 0.0, 0.0], [0.0, 0.0, d], fan([0, 0, 0], 1.09, tet,
                                                                                           [0, 120, 240])]))
    silanol = _sorted_mol([14, 8, 1, 1, 1, 1], np.vstack([
        [0.0, 0.0, 0.0], [0.0, 0.0, 1.64], fan([0, 0, 0], 1.48, tet, [0, 120, 240]),
        fan([0, 0, 1.64], 0.96, np.radians(60.0), [60])]))
    thiol = _sorted_mol([16, 6, 1, 1, 1, 1], np.vstack([
        [0.0, 0.0, 1.815], [0.0, 0.0, 0.0], fan([0, 0, 0], 1.09, tet, [60, 180, 300]),
        fan([0, 0, 1.815], 1.335, np.radians(84.0), [0])]))
    amine = _sorted_mol([7, 6, 1, 1, 1, 1, 1], np.vstack([
        [0.0, 0.0, 1.47], [0.0, 0.0, 0.0], fan([0, 0, 0], 1.09, tet, [60, 180, 300]),
        fan([0, 0, 1.47], 1.01, np.radians(70.5), [0, 120])]))
    hydroxylamine = _sorted_mol([8, 7, 1, 1, 1], np.vstack([
        [0.0, 0.0, 0.0], [0.0, 0.0, 1.45], fan([0, 0, 0], 0.96, np.radians(105.0), [0]),
        fan([0, 0, 1.45], 1.01, np.radians(70.5), [120, 240])]))
    return [silanol, thiol, ch3x(17, 1.78), ch3x(9, 1.39), amine, hydroxylamine]


def main():
    data = os.path.join(REF, "tests", "data")
    sp_m, c_m = read_xyz([os.path.join(data, "methane.xyz")])
    for method in ("MNDO", "AM1", "PM3"):
        write(f"smoke_{method}", sp_m, c_m, {"method": method, "scf_eps": 1e-6, "scf_converger": [1]},
              ref_json=f"smoke_single_point_{method}.json", with_stages=(method == "AM1"))
    write("force_methane_am1", sp_m, c_m, {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1]},
          ref_json="ground_force_methane.json")
    # the reference's UHF known answer: planar CH3 doublet (test_uhf.py:11-57)
    write("uhf_ch3_ref_am1", np.array([[6, 1, 1, 1]]),
          np.array([[[0.0, 0.0, 0.0], [1.1, 0.0, 0.0], [-0.5, 0.9, 0.0], [-0.5, -0.9, 0.0]]]),
          {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1], "UHF": True}, mult=[2],
          ref_json="uhf_ch3_am1.json")
    sp_b, c_b = read_xyz([os.path.join(data, "methane.xyz"), os.path.join(data, "benzene.xyz")])
    write("batch_am1", sp_b, c_b, {"method": "AM1", "scf_eps": 1e-6, "scf_converger": [1]},
          ref_json="batch_single_point_am1.json")
    write("force_mixed_am1", sp_b, c_b, {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1]},
          ref_json="ground_force_batch_mixed.json")
    sp_f, c_f = read_xyz([os.path.join(data, f"methanal.{i}.xyz") for i in (1, 2, 3)])
    write("force_methanal_am1", sp_f, c_f, {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1]},
          ref_json="ground_force_batch_methanal.json")

    sp, c = workloads.pad_batch(workloads.butane_batch(4, seed=1))
    write("butane_pm3_linear", sp, c, {"method": "PM3", "scf_eps": 1e-8, "scf_converger": [0, 0.1]},
          per_molecule=True, with_stages=True)
    mols = workloads.mixed_batch(8, seed=2, alkane_range=(1, 6), water_range=(2, 6))
    sp, c = workloads.pad_batch(mols)
    write("mixed_am1", sp, c, {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1]}, per_molecule=True,
          with_stages=True)
    write("mixed_am1_sp2", sp, c, {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1], "sp2": [True, 1e-7]})
    mols = workloads.mixed_batch(6, seed=3, alkane_range=(2, 8), water_range=(3, 9))
    sp, c = workloads.pad_batch(mols)
    write("mixed_pm3_linear", sp, c, {"method": "PM3", "scf_eps": 1e-8, "scf_converger": [0, 0.1]},
          per_molecule=True)
    write("mixed_mndo", sp, c, {"method": "MNDO", "scf_eps": 1e-8, "scf_converger": [1]})
    # Pulay DIIS (scf_converger [2]); the reference shares the DIIS history counter and its
    # resets across the batch, so each molecule is also run alone
    mols = workloads.mixed_batch(8, seed=2, alkane_range=(1, 6), water_range=(2, 6))
    sp, c = workloads.pad_batch(mols)
    write("mixed_am1_diis", sp, c, {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [2]}, alone=True)
    mols = workloads.mixed_batch(6, seed=3, alkane_range=(2, 8), water_range=(3, 9))
    sp, c = workloads.pad_batch(mols)
    write("mixed_pm3_diis", sp, c, {"method": "PM3", "scf_eps": 1e-7, "scf_converger": [2]}, alone=True)

    # unrestricted Hartree-Fock (UHF) for doublets, triplets and a singlet
    mols, mult = _open_shells()
    for method in ("MNDO", "AM1", "PM3"):
        write(f"uhf_{method.lower()}", *workloads.pad_batch(mols),
              {"method": method, "scf_eps": 1e-8, "scf_converger": [1], "UHF": True}, mult=mult,
              extra={"density_ambiguous": OPEN_SHELL_DENSITY_AMBIGUOUS})
    # charged closed shells (tot_charge): NH4+, OH-, H3O+ next to neutral water
    write("ions_am1", *workloads.pad_batch(_ions()), {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1]},
          charges=[1, -1, 1, 0])
    write("ions_pm3", *workloads.pad_batch(_ions()), {"method": "PM3", "scf_eps": 1e-8, "scf_converger": [1]},
          charges=[1, -1, 1, 0])

    # parameter_file_dir: the reference's STAR parameter set of PM6_SP, read as method PM6_SP and
    # as PM6_SP_STAR (which has no diatomic core-core parameters)
    mols = workloads.mixed_batch(6, seed=2, alkane_range=(1, 6), water_range=(2, 6))
    star = os.path.join(REF, "seqm", "params", "STAR")
    write_param_dir("pdir_pm6sp_star_params", *workloads.pad_batch(mols), "PM6_SP", star, "PM6_SP")
    write_param_dir("pdir_pm6sp_star", *workloads.pad_batch(mols), "PM6_SP_STAR", star, "PM6_SP")

    # AM1-FS1 dispersion correction (seqm_parameters['dispersion'])
    mols = workloads.mixed_batch(6, seed=3, alkane_range=(2, 8), water_range=(3, 9))
    write("disp_am1_fs1", *workloads.pad_batch(mols),
          {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1], "dispersion": True})

    # the parser's pair_outer_cutoff: pairs at or beyond 3 A are dropped from every term
    mols = workloads.mixed_batch(6, seed=3, alkane_range=(2, 8), water_range=(3, 9))
    write("mixed_am1_cutoff", *workloads.pad_batch(mols),
          {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1], "pair_outer_cutoff": 3.0}, per_molecule=True)

    # PM6 parameters on the sp basis (method PM6_SP): alkanes and water clusters (C-C, C-H, O-H
    # core-core exceptions), ions (N-H), and molecules with Si (Si-O), S, Cl, F, N; the
    # hetero-atom set also under AM1 and PM3
    mols = workloads.mixed_batch(8, seed=2, alkane_range=(1, 6), water_range=(2, 6))
    write("mixed_pm6sp", *workloads.pad_batch(mols), {"method": "PM6_SP", "scf_eps": 1e-8, "scf_converger": [1]},
          per_molecule=True, with_stages=True)
    write("ions_pm6sp", *workloads.pad_batch(_ions()), {"method": "PM6_SP", "scf_eps": 1e-8,
                                                        "scf_converger": [1]}, charges=[1, -1, 1, 0])
    for method in ("PM6_SP", "AM1", "PM3"):
        write(f"hetero_{method.lower().replace('_', '')}", *workloads.pad_batch(_hetero()),
              {"method": method, "scf_eps": 1e-8, "scf_converger": [1]}, per_molecule=True)

    # excited states: CIS on a ragged batch, CIS and RPA on a batch of one species
    rng = np.random.default_rng(8)
    mols = [workloads.alkane(2, rng, 0.03), workloads.water_cluster(2, rng), workloads.alkane(3, rng, 0.03),
            workloads.water_cluster(3, rng)]
    write_excited("cis_am1_mixed", *workloads.pad_batch(mols),
                  {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1],
                   "excited_states": {"method": "cis", "n_states": 4, "tolerance": 1e-7}})
    rng = np.random.default_rng(9)
    same = [workloads.alkane(3, rng, 0.05) for _ in range(3)]
    for method, es in (("PM3", "cis"), ("AM1", "rpa")):
        write_excited(f"{es}_{method.lower()}_same", *workloads.pad_batch(same),
                      {"method": method, "scf_eps": 1e-8, "scf_converger": [1],
                       "excited_states": {"method": es, "n_states": 5, "tolerance": 1e-7}})
    # CIS in an orbital window: the 3 highest occupied and 4 lowest virtual orbitals
    write_excited("cis_pm3_window", *workloads.pad_batch(same),
                  {"method": "PM3", "scf_eps": 1e-8, "scf_converger": [1],
                   "excited_states": {"method": "cis", "n_states": 4, "tolerance": 1e-7, "orbital_window": [3, 4]}})

    # the reference's own excited-state known answers (its tests run with active_state 1 for the
    # excited-state forces, which do not change the energies and oscillator strengths compared here)
    for method in ("cis", "rpa"):
        write_reference_excited(f"cis_ref_{method}_am1_methane", ["methane.xyz"],
                                {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1],
                                 "excited_states": {"n_states": 4, "method": method}},
                                f"excited_{method}_am1_methane.json")
    for method, ref_json in (("cis", "cis_batch_same_molecule_coords.json"),
                             ("rpa", "rpa_batch_same_molecule_coords.json")):
        write_reference_excited(f"cis_ref_{method}_am1_methanal", [f"methanal.{i}.xyz" for i in (1, 2, 3)],
                                {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1],
                                 "excited_states": {"n_states": 4, "method": method}}, ref_json)
    write_reference_excited("cis_ref_cis_am1_mixed", ["methanal.1.xyz", "methane.xyz", "benzene.xyz"],
                            {"method": "AM1", "scf_eps": 1e-7, "scf_converger": [1],
                             "excited_states": {"n_states": 4, "method": "cis"}},
                            "cis_batch_different_molecules.json")

    # the reference's own MD suite: its inputs, drivers and committed energies (test_md_suite.py)
    methane, mixed = ["methane.xyz"], ["methane.xyz", "benzene.xyz"]
    basic_tol, xl_tol = {"drift": 1e-2, "slope": 1e-3}, {"drift": 5e-2, "slope": 5e-3}
    ksa = {"max_rank": 3, "err_threshold": 0.0, "T_el": 1500}
    for name, xyz, driver, kw, steps, ref_json, tol in (
            ("md_ref_basic_methane", methane, "basic", {}, 30, "md_basic_methane.json", basic_tol),
            ("md_ref_basic_mixed", mixed, "basic", {}, 30, "md_basic_batch_mixed.json", basic_tol),
            ("md_ref_langevin_methane", methane, "langevin", {"damp": 10.0}, 50, None, None),
            ("md_ref_langevin_mixed", mixed, "langevin", {"damp": 10.0}, 50, None, None),
            ("md_ref_xl_bomd_methane", methane, "xl_bomd", {"xl_bomd_params": {"k": 6}}, 30,
             "md_xl_bomd_methane.json", xl_tol),
            ("md_ref_xl_bomd_methane_k4", methane, "xl_bomd", {"xl_bomd_params": {"k": 4}}, 30,
             "md_xl_bomd_methane_k4.json", xl_tol),
            ("md_ref_ksa_xl_bomd_methane", methane, "ksa_xl_bomd", {"xl_bomd_params": dict(ksa, k=6)}, 30,
             "md_ksa_xl_bomd_methane.json", xl_tol),
            ("md_ref_ksa_xl_bomd_methane_k4", methane, "ksa_xl_bomd", {"xl_bomd_params": dict(ksa, k=4)}, 30,
             "md_ksa_xl_bomd_methane_k4.json", xl_tol),
            ("md_ref_ksa_xl_bomd_mixed", mixed, "ksa_xl_bomd", {"xl_bomd_params": dict(ksa, k=6)}, 30,
             "md_ksa_xl_bomd_batch_mixed.json", xl_tol)):
        write_reference_md(name, xyz, driver, kw, steps, ref_json, tol)
    methanal = [f"methanal.{i}.xyz" for i in (1, 2, 3)]
    excited = {"excited_states": {"n_states": 4, "method": "cis"}, "active_state": 1}
    write_reference_md("md_ref_excited_basic_methanal", methanal, "basic", {}, 30,
                       "md_excited_basic_batch_methanal.json", {"drift": 5e-2, "slope": 5e-2}, excited)
    write_reference_md("md_ref_excited_langevin_methanal", methanal, "langevin", {"damp": 10.0}, 80, None, None,
                       excited)

    # the xyz helpers
    write_xyz_io("io_xyz")
    write_traj_io("io_traj")

    # forces of the ground and all excited states (do_all_forces), CIS and RPA
    for es in ("cis", "rpa"):
        write_all_forces(f"cis_allforces_{es}_am1_methanal", [f"methanal.{i}.xyz" for i in (1, 2, 3)],
                         {"method": "AM1", "scf_eps": 1e-9, "scf_converger": [1],
                          "excited_states": {"n_states": 3, "method": es, "tolerance": 1e-8},
                          "analytical_gradient": [True], "do_all_forces": True})

    # CIS nonadiabatic couplings of a batch of one species (the reference's calc_nac needs one)
    write_nac("cis_nac_am1_methanal", [f"methanal.{i}.xyz" for i in (1, 2, 3)],
              {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1],
               "excited_states": {"n_states": 3, "method": "cis", "tolerance": 1e-7},
               "nonadiabatic": {"compute_nac": True}})

    # molecular dynamics: velocity Verlet and Temp 0 Langevin (friction only) from seeded velocities
    rng = np.random.default_rng(5)
    mols = [workloads.alkane(2, rng, 0.03), workloads.water_cluster(3, rng), workloads.alkane(4, rng, 0.03)]
    sp, c = workloads.pad_batch(mols)
    write_md("md_am1_verlet", sp, c, {"method": "AM1", "scf_eps": 1e-8, "scf_converger": [1]}, steps=8,
             timestep=0.5, seed=6)
    write_md("md_pm3_langevin", sp, c, {"method": "PM3", "scf_eps": 1e-8, "scf_converger": [1]}, steps=8,
             timestep=0.5, seed=7, damp=5.0)

    rng = np.random.default_rng(10)
    mols = [workloads.alkane(2, rng, 0.03), workloads.water_cluster(3, rng)]
    write_xlbomd("md_am1_xlbomd", *workloads.pad_batch(mols), {"method": "AM1", "scf_eps": 1e-8,
                 "scf_converger": [1]}, steps=10, timestep=0.5, seed=11, k=6)
    write_xlbomd("md_pm3_ksa_xlbomd", *workloads.pad_batch(mols), {"method": "PM3", "scf_eps": 1e-8,
                 "scf_converger": [1]}, steps=8, timestep=0.5, seed=12, k=6,
                 krylov={"max_rank": 3, "err_threshold": 0.0, "T_el": 1500})

    rng = np.random.default_rng(4)
    mols = [workloads.alkane(8, rng, 0.05), workloads.water_cluster(4, rng)]
    sp, c = workloads.pad_batch(mols)
    import json as _json
    with open(os.path.join(REPO, "pyseqm_gb300", "data", "params_MNDO.json")) as f:
        tab = _json.load(f)
    rows = np.asarray(tab["rows"])
    fld = tab["fields"]
    learned = {k: (lambda Z, k=k: rows[Z, fld.index(k)]) for k in ("U_ss", "U_pp", "beta_s", "beta_p")}
    write("mndo_param_grads", sp, c, {"method": "MNDO", "scf_eps": 1e-8, "scf_converger": [1]}, learned=learned)


if __name__ == "__main__":
    main()

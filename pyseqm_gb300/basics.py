"""Drop-in replacements for PYSEQM's seqm API on the SCF path.

Mirrors seqm.Molecule.Molecule (Molecule.py:11-186), seqm.basics.Parser
(basics.py:199-403), Pack_Parameters (:406-448), Hamiltonian (:451-533),
Energy (:536-1244), Force (:1247-1365), seqm.ElectronicStructure.Electronic_Structure
(ElectronicStructure.py:10-127) and seqm.seqm_functions.constants.Constants
(constants.py:26-224): same constructors, same seqm_parameters keys, same return
tuples, results in the same padded layout.  The computation runs in the CUDA
library; autograd reaches the coordinates and the per-atom U_ss, U_pp, beta_s,
beta_p through ``SCFEnergyFunction``, whose backward is the adjoint kernel
(seqm_energy_grad) evaluated at the converged density, which is what the
reference's SCF0 boundary implies (scf_loop.py:1996-2031).

Supported: MNDO/AM1/PM3/PM6_SP (and PM6_SP_STAR from parameter files), closed shell
(scf_converger [0, alpha], [1] and [2] (DIIS), sp2) and unrestricted open shell (``UHF``: True
with the Molecule's ``mult``; scf_converger [0, alpha] and [1], as the reference has neither
open-shell DIIS nor SP2), learned parameters (values for any parameter; gradients for U_ss,
U_pp, beta_s, beta_p), ``parameter_file_dir``, ``pair_outer_cutoff``, AM1-FS1 ``dispersion``,
and the CIS / RPA excited states (``excited_states``: excitation energies, amplitudes,
transition dipoles, oscillator strengths, orbital windows; with active_state > 0 the state's
energy and relaxed forces; ``nonadiabatic`` couplings; ``do_all_forces``).  PM6 with d orbitals,
scf_backward >= 1 and 2nd_grad raise NotImplementedError.
"""

import copy
import math
import time

import numpy as np
import torch

from . import native, tables
from .layout import Layout
from .scf import BatchSCF, BatchUHF

TO_DEBYE = 1.60217733e-19 * 1e-10 * 2.99792458e8 / 1e-21  # seqm/seqm_functions/constants.py:13-15
DEBYE_TO_AU = 0.393456
GRAD_PARAMS = ("U_ss", "U_pp", "beta_s", "beta_p")


def _f64(x, device):
    return torch.as_tensor(np.asarray(x), dtype=torch.float64, device=device)


# ------------------------------------------------------------------ constants
class Constants(torch.nn.Module):
    """Element tables (constants.py:26-224) as non-trainable parameters, float64."""

    def __init__(self, do_timing=False, length_conversion_factor=(1.0 / tables.A0), energy_conversion_factor=1.0):
        super().__init__()
        el = tables.elements()
        self.length_conversion_factor = length_conversion_factor
        self.energy_conversion_factor = energy_conversion_factor
        for name in ("tore", "qn", "ussc", "uppc", "gssc", "gspc", "hspc", "gp2c", "gppc", "mass"):
            setattr(self, name, torch.nn.Parameter(torch.as_tensor(el[name], dtype=torch.float64),
                                                   requires_grad=False))
        self.qn_int = torch.nn.Parameter(self.qn.data.to(torch.int64), requires_grad=False)
        self.eheat = torch.nn.Parameter(torch.as_tensor(el["eheat_ev"], dtype=torch.float64), requires_grad=False)
        self.atomic_num = torch.nn.Parameter(torch.as_tensor(el["atomic_num"], dtype=torch.float64),
                                             requires_grad=False)
        self.label = list(el["label"])  # element symbols, spelled as the reference's table (save_xyz)
        self.iso = torch.nn.Parameter(torch.as_tensor(el["iso"], dtype=torch.float64), requires_grad=False)
        self.qnD_int = torch.nn.Parameter(torch.as_tensor(el["qnD_int"], dtype=torch.float64).to(torch.int64),
                                          requires_grad=False)
        self.do_timing = do_timing
        if do_timing:
            self.timing = {"Hcore + STO Integrals": [], "SCF": [], "Force": [], "MD": [], "D*": [], "CIS/RPA": []}

    def forward(self):
        pass


# --------------------------------------------------------------------- parser
def _check_options(seqm_parameters):
    if seqm_parameters.get("method") not in tables.METHOD_FIELDS:
        raise NotImplementedError(f"method {seqm_parameters.get('method')!r}: supported are {tables.SUPPORTED}")
    if seqm_parameters.get("UHF", False):
        if seqm_parameters.get("sp2", [False])[0]:
            raise NotImplementedError("SP2 has no open-shell form (the reference's SP2.py raises for UHF)")
        if seqm_parameters.get("scf_converger", [1])[0] == 2:
            raise NotImplementedError("DIIS has no open-shell form in the reference (scf_converger [0, alpha] or "
                                      "[1] with UHF)")
    exc = seqm_parameters.get("excited_states")
    if exc:
        if not isinstance(exc, dict):
            raise Exception("Invalid format for excited_states. Expected input like "
                            "'excited_states': {'method': 'rpa', 'n_states': 3, 'tolerance': 1e-6}")
        if "n_states" not in exc:
            raise ValueError("Specify the number of excited states to calculate")
        if str(exc.get("method", "cis")).lower() not in ("cis", "tda", "rpa"):
            raise Exception("Excited state method has to be CIS or RPA")
        if seqm_parameters.get("UHF", False):
            raise NotImplementedError("Unrestricted excited state methods (CIS and RPA) not available")
        if not seqm_parameters.get("eig", True):
            raise NotImplementedError("excited states need the orbitals (eig=True)")
    if seqm_parameters.get("scf_backward", 0) != 0:
        raise NotImplementedError("scf_backward >= 1 (backpropagation through the SCF) is not supported")
    conv = seqm_parameters.get("scf_converger", [1])
    if conv[0] not in (0, 1, 2):
        raise NotImplementedError("scf_converger must be [0, alpha], [1] or [2]")


class Parser(torch.nn.Module):
    """Pair list and counts in the reference's order and dtypes (basics.py:199-403)."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.outercutoff = seqm_parameters.get("pair_outer_cutoff", 1e10)
        if seqm_parameters.get("elements") is None:
            raise RuntimeError("Please instantiate a Molecule object before instantiating an object of "
                               "Electronic_structure or Molecular_Dynamics class.Alternately, provide a list called "
                               "of unique elements in the input molecules under the 'elements' key in seqm_parameters")
        self.elements = seqm_parameters["elements"]
        self.uhf = seqm_parameters.get("UHF", False)
        self.hipnn_automatic_doublet = seqm_parameters.get("HIPNN_automatic_doublet", False)

    def forward(self, molecule, themethod, return_mask_l=False, do_large_tensors=True, *args, **kwargs):
        species = molecule.species
        dev = molecule.coordinates.device
        sp = species.detach().cpu().numpy()
        nmol, molsize = sp.shape
        el = tables.elements()
        real = sp > 0
        real_atoms = np.nonzero(real.reshape(-1))[0]
        Z = sp.reshape(-1)[real_atoms]
        nheavy = (sp > 1).sum(1)
        nhyd = (sp == 1).sum(1)
        nsh = ((sp >= 13) & (sp <= 17)).sum(1)  # super-heavy of the sp elements (basics.py:258-270)
        nel = el["tore"][sp].sum(1).astype(np.int64)
        if torch.is_tensor(molecule.tot_charge):
            nel = nel - molecule.tot_charge.detach().cpu().numpy().reshape(-1).astype(np.int64)
        if self.uhf:
            # alpha / beta occupations from the multiplicity (basics.py:279-294)
            s2 = np.asarray(torch.as_tensor(molecule.mult).detach().cpu(), dtype=np.float64).reshape(-1) - 1.0
            na, nb = nel / 2.0 + s2 / 2.0, nel / 2.0 - s2 / 2.0
            odd = (na % 1 != 0) | (nb % 1 != 0)
            if odd.any():
                if not self.hipnn_automatic_doublet:
                    raise ValueError("Invalid charge/multiplicity combination!")
                na[odd] += 0.5
                nb[odd] -= 0.5
            nocc = np.stack((na, nb), axis=1).astype(np.int64)
        else:
            if np.any(nel % 2 == 1):
                raise ValueError("RHF setting requires closed shell systems (even number of electrons)")
            nocc = nel // 2
        maskd = ((np.arange(molsize) * (molsize + 1))[None, :] + (np.arange(nmol) * molsize**2)[:, None]).reshape(-1)
        maskd = maskd[real_atoms]
        atom_molid = np.repeat(np.arange(nmol), molsize)[real_atoms]
        inv = np.zeros(nmol * molsize, dtype=np.int64)
        inv[real_atoms] = np.arange(real_atoms.size)
        ii, jj = np.triu_indices(molsize, 1)
        m_all = np.repeat(np.arange(nmol), ii.size)
        i_all, j_all = np.tile(ii, nmol), np.tile(jj, nmol)
        keep = real[m_all, i_all] & real[m_all, j_all]
        if self.outercutoff < 1e10:  # pairs closer than pair_outer_cutoff (basics.py:324-328)
            c = molecule.coordinates.detach().cpu().numpy()
            dd = c[m_all, j_all] - c[m_all, i_all]
            keep &= np.sum(dd * dd, axis=1) < self.outercutoff ** 2
        mp, ip, jp = m_all[keep], i_all[keep], j_all[keep]
        t = lambda a: torch.as_tensor(a, dtype=torch.int64, device=dev)  # noqa: E731
        idxi, idxj = inv[mp * molsize + ip], inv[mp * molsize + jp]
        coords = molecule.coordinates.detach()
        d = coords[t(mp), t(jp)] - coords[t(mp), t(ip)]
        dist = torch.linalg.norm(d, dim=1)
        out = [nmol, molsize, t(nsh), t(nheavy), t(nhyd), t(nocc), t(Z), t(maskd), t(atom_molid),
               t(mp * molsize**2 + ip * molsize + jp)]
        if return_mask_l:
            out.append(t(mp * molsize**2 + jp * molsize + ip))
        out += [t(mp), t(Z[idxi]), t(Z[idxj]), t(idxi), t(idxj), d / dist.unsqueeze(1),
                dist * molecule.const.length_conversion_factor]
        return tuple(out)


class Pack_Parameters(torch.nn.Module):
    """Per-atom parameters from the method's table plus learned ones (basics.py:406-448)."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.elements = seqm_parameters["elements"]
        self.learned_list = seqm_parameters.get("learned", [])
        self.method = seqm_parameters["method"]
        self.parameters = list(tables.METHOD_FIELDS[self.method])
        self.required_list = [p for p in self.parameters if p not in self.learned_list]
        param_dir = seqm_parameters.get("parameter_file_dir")
        fields, rows = tables.method_table(self.method, param_dir)
        if rows.shape[0] <= max(self.elements):
            rows = np.vstack([rows, np.zeros((max(self.elements) + 1 - rows.shape[0], rows.shape[1]))])
        self.p = torch.nn.Parameter(torch.as_tensor(rows[:, [fields.index(f) for f in self.required_list]]),
                                    requires_grad=False)
        # diatomic core-core parameters (PWCCT, parameters.py:49-87): entries of the listed
        # elements, zero otherwise and for methods without them
        m = max(self.elements)
        alp, chi = np.zeros((m + 1, m + 1)), np.zeros((m + 1, m + 1))
        t = tables.pair_table(self.method, param_dir)
        if t is not None:
            el = [z for z in self.elements if z < t[0].shape[0]]
            ix = np.ix_(el, el)
            alp[ix], chi[ix] = t[0][ix], t[1][ix]
        self.alpha = torch.nn.Parameter(torch.as_tensor(alp), requires_grad=False)
        self.chi = torch.nn.Parameter(torch.as_tensor(chi), requires_grad=False)

    def forward(self, Z, learned_params=dict()):
        learned_params = dict(learned_params)
        for i, name in enumerate(self.required_list):
            learned_params[name] = self.p[Z, i]
        return learned_params, self.alpha, self.chi


# ------------------------------------------------------------------ molecule
class Molecule(torch.nn.Module):
    """Batch of molecules (Molecule.py:11-186): same constructor and attributes."""

    def __init__(self, const, seqm_parameters, coordinates, species, charges=0, mult=1, learned_parameters=dict(),
                 do_large_tensors=True, *args, **kwargs):
        super().__init__()
        self.const = const
        _check_species(species)
        self.species = species
        self.coordinates = torch.nn.Parameter(coordinates)
        self.coordinates.requires_grad_(do_large_tensors)
        if not torch.is_tensor(charges):
            charges = charges * torch.ones(coordinates.shape[0], device=coordinates.device)
        self.tot_charge = charges
        if not torch.is_tensor(mult):
            mult = mult * torch.ones(coordinates.shape[0], device=coordinates.device)
        self.mult = mult
        if seqm_parameters.get("elements") is None:
            seqm_parameters["elements"] = [0] + sorted(set(species.reshape(-1).tolist()))
        self.seqm_parameters = seqm_parameters
        self.method = seqm_parameters["method"]
        _check_options(seqm_parameters)
        self.parser = Parser(seqm_parameters)
        self.packpar = Pack_Parameters(seqm_parameters).to(coordinates.device)
        (self.nmol, self.molsize, self.nSuperHeavy, self.nHeavy, self.nHydro, self.nocc, self.Z, self.maskd,
         self.atom_molid, self.mask, self.mask_l, self.pair_molid, self.ni, self.nj, self.idxi, self.idxj, self.xij,
         self.rij) = self.parser(self, self.method, return_mask_l=True)
        if callable(learned_parameters):
            learned_parameters = learned_parameters(self.species, self.coordinates)
        self.parameters, self.alp, self.chi = copy.deepcopy(self.packpar(self.Z, learned_params=learned_parameters))
        _complete_parameters(self.parameters)
        self.norb = self.nHydro + 4 * self.nHeavy
        non_zero = self.species != 0
        self.num_atoms = torch.sum(non_zero, dim=1).to(coordinates.dtype)
        self.mass = self.const.mass[self.species].unsqueeze(2)
        self.mass_inverse = torch.zeros_like(self.mass)
        self.mass_inverse[non_zero] = 1.0 / self.mass[non_zero]
        for name in ("force", "velocities", "acc", "dm", "q", "w", "Hf", "Etot", "Eelec", "Enuc", "Eiso", "e_mo",
                     "e_gap", "molecular_orbitals", "charge", "dipole", "analytical_gradient", "cis_amplitudes",
                     "transition_dipole", "oscillator_strength", "cis_energies", "transition_density_matrices",
                     "cis_state_relaxed_dipole", "cis_state_unrelaxed_dipole", "all_forces", "all_cis_relaxed_diploles",
                     "all_cis_unrelaxed_diploles", "Electronic_entropy", "Fermi_occ", "dP2dt2", "Krylov_Error", "nac",
                     "nac_dot", "old_mos"):
            setattr(self, name, None)
        self.verbose = True
        self.active_state = seqm_parameters.get("active_state", 0)


def _check_species(species):
    ok = species[:, :-1] >= species[:, 1:]
    row_ok = ok.all(dim=1)
    if not row_ok.all():
        bad = (~row_ok).nonzero(as_tuple=False).squeeze(1).tolist()
        word, verb = ("row", "is") if len(bad) == 1 else ("rows", "are")
        raise ValueError(f"species must be non-increasing along each row, but {word} "
                         f"{', '.join(map(str, bad))} {verb} not sorted.")


def _complete_parameters(params):
    if "beta_s" in params and "beta_p" in params:
        params["beta"] = torch.cat((params["beta_s"].unsqueeze(1), params["beta_p"].unsqueeze(1)), dim=1)
    z = torch.zeros_like(params["zeta_s"])
    for k in ("zeta_d", "s_orb_exp_tail", "p_orb_exp_tail", "d_orb_exp_tail", "U_dd", "F0SD", "G2SD", "rho_core"):
        params[k] = z
    params["Kbeta"] = params.get("Kbeta", None)


# -------------------------------------------------------------- the SCF core
class _Solve:
    """One batched SCF solve on the GPU for a Molecule (layout, solver, options)."""

    def __init__(self, molecule, seqm_parameters, P0=None):
        _check_options(seqm_parameters)
        self.dev = molecule.coordinates.device if molecule.coordinates.is_cuda else torch.device("cuda")
        sp = molecule.species.detach().cpu().numpy()
        xyz = molecule.coordinates.detach().cpu().numpy()
        learned = {k: v.detach().cpu().numpy() for k, v in molecule.parameters.items()
                   if k in native.PAR and torch.is_tensor(v)}
        charges = molecule.tot_charge.detach().cpu().numpy() if torch.is_tensor(molecule.tot_charge) else None
        self.uhf = bool(seqm_parameters.get("UHF", False))
        mult = None
        if self.uhf:
            nocc = getattr(molecule, "nocc", None)
            if torch.is_tensor(nocc) and nocc.dim() == 2:  # the parser's alpha / beta counts
                nocc = nocc.detach().cpu().numpy()
                mult = nocc[:, 0] - nocc[:, 1] + 1
            else:
                mult = np.asarray(torch.as_tensor(molecule.mult).detach().cpu(), dtype=np.float64).reshape(-1)
        cutoff = seqm_parameters.get("pair_outer_cutoff", 1e10)
        self.L = Layout.from_padded(sp, xyz, molecule.method, charges, learned, mult=mult,
                                    pair_cutoff=cutoff if cutoff < 1e10 else None,
                                    param_dir=seqm_parameters.get("parameter_file_dir")).to_device(self.dev)
        self.s = BatchUHF(self.L) if self.uhf else BatchSCF(self.L)
        self.opts = seqm_parameters
        self.P0 = P0
        self.timing = {}
        self._species = molecule.species.detach().cpu().clone()
        self._key = (molecule.method, None if charges is None else charges.tobytes(),
                     None if mult is None else np.asarray(mult).tobytes())

    def run(self, const=None):
        o = self.opts
        t0 = time.time()
        self.s.hcore()
        if const is not None and const.do_timing:
            torch.cuda.synchronize()
            const.timing["Hcore + STO Integrals"].append(time.time() - t0)
        t0 = time.time()
        P0 = None
        if self.P0 is not None:
            P0 = self.P0.detach().to(self.dev, torch.float64)
            if self.uhf:  # (nmol, 2, N, N) spin densities
                P0 = (self.L.padded_to_packed(P0[:, 0]), self.L.padded_to_packed(P0[:, 1]))
            else:
                P0 = self.L.padded_to_packed(P0)
        eps = float(o["scf_eps"]) if not torch.is_tensor(o["scf_eps"]) else float(o["scf_eps"].item())
        self.notconverged = self.s.scf(eps, tuple(o.get("scf_converger", [1])), tuple(o.get("sp2", [False])), P0)
        self.Eelec, self.Enuc = self.s.final(want_vectors=o.get("eig", True))
        if const is not None and const.do_timing:
            torch.cuda.synchronize()
            const.timing["SCF"].append(time.time() - t0)
        return self

    def matches(self, molecule, seqm_parameters):
        """Same molecules (species, charges, multiplicities) and options as this solve."""
        if seqm_parameters is not self.opts or molecule.species.shape != self._species.shape:
            return False
        charges = molecule.tot_charge.detach().cpu().numpy() if torch.is_tensor(molecule.tot_charge) else None
        return (torch.equal(molecule.species.detach().cpu(), self._species) and self._key[0] == molecule.method
                and self._key[1] == (None if charges is None else charges.tobytes()))

    def rerun(self, molecule, const=None):
        """The same molecules at the molecule's current coordinates, starting from this solve's
        converged density with its eigenvectors as the Jacobi warm start, everything on the
        device (BatchSCF.resume; the reference's MD passes P0 = the previous density,
        MolecularDynamics.py:815-825)."""
        o = self.opts
        t0 = time.time()
        real = torch.as_tensor(self.L.real_index, device=molecule.coordinates.device)
        xyz = molecule.coordinates.detach().reshape(-1, 3)[real].cpu().numpy()
        eps = float(o["scf_eps"]) if not torch.is_tensor(o["scf_eps"]) else float(o["scf_eps"].item())
        self.P0 = None
        self.notconverged = self.s.resume(xyz, eps, tuple(o.get("scf_converger", [1])), tuple(o.get("sp2", [False])))
        self.Eelec, self.Enuc = self.s.final(want_vectors=o.get("eig", True))
        if const is not None and const.do_timing:
            torch.cuda.synchronize()
            const.timing["SCF"].append(time.time() - t0)
        return self

    def grad(self, gE, gN):
        L = self.L
        dR = torch.empty(3 * max(1, L.natoms), dtype=torch.float64, device=self.dev)
        dpar = torch.empty(4 * max(1, L.natoms), dtype=torch.float64, device=self.dev)
        work = torch.empty(7 * max(1, L.npairs), dtype=torch.float64, device=self.dev)
        lib = native.load()
        self.s.launches += 2
        Pb = native.ptr(self.s.Pb) if self.uhf else None
        native.check(lib.seqm_energy_grad(L.struct, native.ptr(self.s.P), Pb, native.ptr(gE.contiguous()),
                                          native.ptr(gN.contiguous()), native.ptr(dR), native.ptr(dpar),
                                          native.ptr(work), self.s._s()), "seqm_energy_grad")
        return dR[: 3 * L.natoms].view(L.natoms, 3), dpar[: 4 * L.natoms].view(4, L.natoms)

    def grad_excited(self, gE, D, R):
        """d(excitation energy)/dR per real atom for the molecules weighted by gE: the excited-state
        gradient of D (relaxed difference density) and R (transition density), both ragged, minus
        the ground-state terms of the same weights (rcis_grad_batch.py:10-259)."""
        L = self.L
        n3 = 3 * max(1, L.natoms)
        dR = torch.empty(n3, dtype=torch.float64, device=self.dev)
        dR0 = torch.empty(n3, dtype=torch.float64, device=self.dev)
        work = torch.empty(7 * max(1, L.npairs), dtype=torch.float64, device=self.dev)
        gN = torch.zeros_like(gE)
        lib = native.load()
        self.s.launches += 4
        gE = gE.contiguous()
        native.check(lib.seqm_energy_grad_excited(L.struct, native.ptr(self.s.P), native.ptr(D), native.ptr(R),
                                                  native.ptr(gE), native.ptr(gN), native.ptr(dR), native.ptr(work),
                                                  self.s._s()), "seqm_energy_grad_excited")
        native.check(lib.seqm_energy_grad(L.struct, native.ptr(self.s.P), None, native.ptr(gE), native.ptr(gN),
                                          native.ptr(dR0), None, native.ptr(work), self.s._s()), "seqm_energy_grad")
        return (dR - dR0)[: 3 * L.natoms].view(L.natoms, 3)

    # ------------------------------------------------------- padded outputs
    def padded(self, flat, flat_b=None):
        """Padded (nmol, N, N) matrices; with a beta-spin array, (nmol, 2, N, N) as the reference's
        unrestricted outputs."""
        if flat_b is None:
            return self.L.packed_to_padded(flat)
        return torch.stack((self.L.packed_to_padded(flat), self.L.packed_to_padded(flat_b)), dim=1)

    def _eigen_one(self, evals, evecs):
        L = self.L
        n4 = 4 * L.molsize
        nmax = int(L.norb.max())
        e = torch.zeros(L.nmol, n4, dtype=torch.float64, device=self.dev)
        v = torch.zeros(L.nmol, nmax, nmax, dtype=torch.float64, device=self.dev)
        for m in range(L.nmol):
            n = int(L.norb[m])
            e[m, :n] = evals[int(L.row_off[m]): int(L.row_off[m]) + n]
            v[m, :n, :n] = L.block(evecs, m).t()
            if n < nmax:
                v[m, n:, n:] = torch.eye(nmax - n, dtype=torch.float64, device=self.dev)
        return e, v

    def eigen_padded(self):
        """e (nmol, 4*molsize) zero-padded and v (nmol, nmax, nmax) with eigenvectors as columns;
        unrestricted: e (nmol, 2, 4*molsize) and v (nmol, 2, nmax, nmax) (diag.py:205-208)."""
        e, v = self._eigen_one(self.s.evals, self.s.evecs)
        if not self.uhf:
            return e, v
        eb, vb = self._eigen_one(self.s.evals_b, self.s.evecs_b)
        return torch.stack((e, eb), dim=1), torch.stack((v, vb), dim=1)

    def w_reference_order(self):
        """w of the kept pairs, (nref, 10, 10) in the reference's pair order."""
        L = self.L
        ref = L.reference_pair_index()
        w = torch.zeros(L.nref + 1, 10, 10, dtype=torch.float64, device=self.dev)
        pos = torch.as_tensor(np.where(ref >= 0, ref, L.nref), device=self.dev)  # skipped -> spare row
        if L.nxx:
            w[pos[: L.nxx]] = self.s.w_xx[: 100 * L.nxx].view(-1, 10, 10)
        if L.nxh:
            w[pos[L.nxx: L.nxx + L.nxh], :, 0] = self.s.w_xh[: 10 * L.nxh].view(-1, 10)
        if L.nhh:
            w[pos[L.nxx + L.nxh:], 0, 0] = self.s.w_hh[: L.nhh]
        return w[: L.nref]

    def pair_values_reference_order(self, v):
        ref = self.L.reference_pair_index()
        keep = torch.as_tensor(ref >= 0, device=self.dev)
        pos = torch.as_tensor(ref, device=self.dev)
        out = torch.empty(self.L.nref, dtype=v.dtype, device=self.dev)
        out[pos[keep]] = v[: self.L.npairs][keep]
        return out


class SCFEnergyFunction(torch.autograd.Function):
    """(coordinates of real atoms, U_ss, U_pp, beta_s, beta_p) -> (Eelec, Enuc) per molecule.

    forward runs the SCF; backward is the adjoint kernel at the converged density
    (no backpropagation through the SCF iterations, as with the reference's SCF0)."""

    @staticmethod
    def forward(ctx, xyz, uss, upp, bs, bp, solve):
        ctx.solve = solve
        return solve.Eelec.clone(), solve.Enuc.clone()

    @staticmethod
    def backward(ctx, gE, gN):
        solve = ctx.solve
        nm = solve.L.nmol
        gE = torch.zeros(nm, dtype=torch.float64, device=solve.dev) if gE is None else gE.to(solve.dev, torch.float64)
        gN = torch.zeros(nm, dtype=torch.float64, device=solve.dev) if gN is None else gN.to(solve.dev, torch.float64)
        dR, dpar = solve.grad(gE, gN)
        return dR, dpar[0], dpar[1], dpar[2], dpar[3], None


def _phase_align(new_amp, ref_amp, rpa=False):
    """Signs of the roots chosen so that each has a non-negative overlap with the previous call's
    amplitudes of the same root (_phase_align_cis, basics.py:567-593): continuous phases
    along a trajectory."""
    if not (torch.is_tensor(new_amp) and torch.is_tensor(ref_amp)):
        return new_amp
    amp = new_amp[0] if rpa else new_amp
    ref = (ref_amp[0] if rpa else ref_amp).to(amp.device)
    if amp.ndim < 3 or ref.ndim < 3 or ref.shape[0] != amp.shape[0] or ref.shape[2] != amp.shape[2]:
        return new_amp
    n = min(amp.shape[1], ref.shape[1])
    if n == 0:
        return new_amp
    sign = torch.ones(amp.shape[:2], dtype=amp.dtype, device=amp.device)
    sign[:, :n] = torch.where((ref[:, :n] * amp[:, :n]).sum(-1) >= 0, 1.0, -1.0)
    return new_amp * (sign[None, :, :, None] if rpa else sign[:, :, None])


def nac_pairs(seqm_parameters, nroots):
    """1-based state pairs of the nonadiabatic couplings asked for (resolve_nac_config), or None
    when they are not enabled."""
    cfg = resolve_nac_config(seqm_parameters, nroots=nroots)
    return cfg.pairs if cfg.enabled else None


class ExcitedEnergyFunction(torch.autograd.Function):
    """(coordinates of real atoms) -> excitation energy of each molecule's active state (0 for
    molecules in the ground state).  backward: the relaxed excited-state gradient (Z-vector
    response, rcis_grad_batch.py:10-259) minus the ground-state part, which SCFEnergyFunction
    carries."""

    @staticmethod
    def forward(ctx, xyz, solve, ex, X, Y, E_state, mask, tol):
        ctx.args = (solve, ex, X, Y, mask, tol)
        return E_state.clone()

    @staticmethod
    def backward(ctx, gE):
        solve, ex, X, Y, mask, tol = ctx.args
        gE = (gE.to(solve.dev, torch.float64) * mask).contiguous()
        with torch.no_grad():
            R, _, D = ex.state_densities(X, Y, tol)
            dR = solve.grad_excited(gE, ex.to_ragged(D), ex.to_ragged(R))
        return dR, None, None, None, None, None, None, None


def _active_states(molecule, nmol, device):
    """Active state per molecule (0 ground, k > 0 the k-th excited state): an int or a tensor
    (active_state_tensor, dynamics/active_state.py:4-15)."""
    a = molecule.active_state
    if torch.is_tensor(a):
        t = a.to(device).long()
        return t.expand(nmol) if t.dim() == 0 else t
    return torch.full((nmol,), int(a or 0), dtype=torch.long, device=device)


FS1_SR, FS1_D = 1.1058892, 1000.0  # AM1-FS1 damping constants (dispersion_am1_fs1.py:9-10)
FS1_D_TOL = 12.0 * math.log(10.0)  # the damping is clipped to 0 / 1 past this argument
EV_PER_J_PER_MOL = 1.036426966e-5


def _dispersion_am1_fs1(L, xyz):
    """AM1-FS1 dispersion energy per molecule in eV (dispersion_am1_fs1.py:16-113; Foster and
    Sohlberg, J. Chem. Theory Comput. 6, 2153 (2010)): over the kept pairs,
    -sqrt(C6_i C6_j) / R^6 f(R), f = 1 / (1 + exp(-d (R / (S_R (R0_i + R0_j)) - 1))) set to 1 / 0
    where the argument is beyond +-12 ln 10, with Grimme's 2006 C6 (J nm^6 / mol) and R0 (A).
    Differentiable in xyz (real atoms, Angstrom), so the forces follow by autograd."""
    dev = xyz.device
    if getattr(L, "_fs1", None) is None or L._fs1[0].device != dev:
        c6, r0 = tables.grimme_c6_r0()
        keep = np.ones(L.npairs, dtype=bool) if L.pair_skip is None else ~L.pair_skip
        pi, pj = L.pair_i[keep], L.pair_j[keep]
        zi, zj = L.Z[pi], L.Z[pj]
        c6z = lambda z: np.where(z < c6.size, c6[np.minimum(z, c6.size - 1)], 0.0)  # noqa: E731
        r0z = lambda z: np.where(z < r0.size, r0[np.minimum(z, r0.size - 1)], 0.0)  # noqa: E731
        t = lambda a, dt=torch.float64: torch.as_tensor(a, dtype=dt, device=dev)  # noqa: E731
        L._fs1 = (t(pi, torch.int64), t(pj, torch.int64), t(np.sqrt(c6z(zi) * c6z(zj))), t(r0z(zi) + r0z(zj)),
                  t(L.atom_mol[pi], torch.int64))
    pi, pj, c6ij, rv, mol = L._fs1
    R = torch.linalg.norm(xyz[pj] - xyz[pi], dim=1)
    arg = FS1_D * (R / (FS1_SR * rv) - 1.0)
    f = torch.sigmoid(arg)
    f = torch.where(arg > FS1_D_TOL, torch.ones_like(f), f)
    f = torch.where(arg < -FS1_D_TOL, torch.zeros_like(f), f)
    e = -c6ij * R.pow(-6.0) * f
    return torch.zeros(L.nmol, dtype=e.dtype, device=dev).index_add(0, mol, e) * (EV_PER_J_PER_MOL * 1.0e6)


def _isolated_atom_energy(const, Z, p):
    """energy.py:8-23 (differentiable in the parameters)."""
    return (p["U_ss"] * const.ussc[Z] + p["U_pp"] * const.uppc[Z] + p["g_ss"] * const.gssc[Z]
            + p["g_pp"] * const.gppc[Z] + p["g_sp"] * const.gspc[Z] + p["g_p2"] * const.gp2c[Z]
            + p["h_sp"] * const.hspc[Z])


def _dipole(molecule, solve):
    """Ground-state dipole from the diagonal density blocks (dipole.py:85-107), on the device."""
    L = solve.L
    dev = solve.dev
    P = solve.s.P + solve.s.Pb if solve.uhf else solve.s.P  # open shell: both spins (dipole.py:91-94)
    xyz = torch.as_tensor(L.xyz, device=dev)
    Z = L.Z
    el = tables.elements()
    par = L.dev["par"].view(native.NPAR, -1)
    dd = par[native.PAR["_dd"]] * tables.A0
    elec = torch.zeros(L.nmol, 3, dtype=torch.float64, device=dev)
    atom_off = L.atom_off
    for m in range(L.nmol):
        blk = L.block(P, m)
        nh = int(L.nheavy[m])
        a0, a1 = int(atom_off[m]), int(atom_off[m + 1])
        d = torch.diagonal(blk)
        idx = np.arange(a0, a1)
        heavy = idx[: nh]
        hyd = idx[nh:]
        if nh:
            occ = d[: 4 * nh].view(nh, 4).sum(1)
            sp = torch.stack([blk[4 * k, 4 * k + 1: 4 * k + 4] for k in range(nh)])
            elec[m] += -(occ[:, None] * xyz[heavy]).sum(0) - 2.0 * (dd[heavy][:, None] * sp).sum(0)
        if hyd.size:
            elec[m] += -(d[4 * nh:][:, None] * xyz[hyd]).sum(0)
    nuc = (molecule.const.tore[molecule.species].unsqueeze(-1) * molecule.coordinates.detach()).sum(dim=1)
    return ((elec.to(nuc.device) + nuc) * TO_DEBYE * DEBYE_TO_AU)


def _orbital_charges(molecule, solve, v):
    """Per-orbital atomic charges as the reference forms them (scf_loop.py:2333-2388); open
    shell: the mean of the two spins' values (scf_loop.py:2344-2371)."""
    if v.dim() == 4:
        return 0.5 * (_orbital_charges(molecule, solve, v[:, 0]) + _orbital_charges(molecule, solve, v[:, 1]))
    L = solve.L
    nmol, molsize = L.nmol, L.molsize
    charge = torch.zeros(nmol, molsize * 4, molsize, device=v.device, dtype=v.dtype)
    v2 = v**2
    for i in range(nmol):
        n, nh, ny = int(L.norb[i]), int(L.nheavy[i]), int(L.nhyd[i])
        if nh:
            charge[i, :n, :nh] = v2[i][:n, : 4 * nh].reshape(n, 4, nh).sum(dim=1)
        charge[i, :n, nh: nh + ny] = v2[i][:n, 4 * nh: 4 * nh + ny]
    return charge


# ---------------------------------------------------------------- modules
class Hamiltonian(torch.nn.Module):
    """SCF driver module (basics.py:451-533); returns the reference's 12-tuple."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.eps = torch.nn.Parameter(torch.as_tensor(seqm_parameters["scf_eps"]), requires_grad=False)
        self.sp2 = seqm_parameters.get("sp2", [False])
        self.scf_converger = seqm_parameters["scf_converger"]
        self.eig = seqm_parameters.get("eig", True)
        self.seqm_parameters = seqm_parameters

    def solve(self, molecule, P0=None, reuse=False):
        """reuse: P0 is the density this module's previous solve of the same molecules handed out
        (molecule.dm, as an MD step passes it): that solve continues on the device from its own
        state at the new coordinates instead of a new layout and a packed P0."""
        prev = getattr(molecule, "_solve", None)
        if (reuse and prev is not None and P0 is not None and P0 is getattr(molecule, "_solve_dm", None)
                and prev.matches(molecule, self.seqm_parameters)):
            return prev.rerun(molecule, molecule.const)
        return _Solve(molecule, self.seqm_parameters, P0).run(molecule.const)

    def forward(self, molecule, themethod, P0=None):
        s = self.solve(molecule, P0)
        return _hamiltonian_outputs(molecule, s, self.eig)


def _hamiltonian_outputs(molecule, s, eig=True):
    F = s.padded(s.s.F, s.s.Fb if s.uhf else None)
    P = s.padded(s.s.P, s.s.Pb if s.uhf else None)
    H = s.padded(s.s.H)
    w = s.w_reference_order()
    nc = torch.as_tensor(s.notconverged, device=F.device)
    if eig:
        e, v = s.eigen_padded()
        charge = _orbital_charges(molecule, s, v)
    else:
        e = v = charge = None
    par = s.L.dev["par"].view(native.NPAR, -1)
    ref_i, ref_j = s.L.reference_pair_atoms()
    rho0 = par[native.PAR["_rho0"]]
    rho0xi = rho0[torch.as_tensor(ref_i, device=F.device)]
    rho0xj = rho0[torch.as_tensor(ref_j, device=F.device)]
    return F, e, P, H, w, charge, rho0xi, rho0xj, None, None, nc, v


class Energy(torch.nn.Module):
    """Energy terms (basics.py:536-1244, ground state)."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.seqm_parameters = seqm_parameters
        self.method = seqm_parameters["method"]
        self.parser = Parser(seqm_parameters) if seqm_parameters.get("elements") is not None else None
        self.packpar = Pack_Parameters(seqm_parameters) if seqm_parameters.get("elements") is not None else None
        self.hamiltonian = Hamiltonian(seqm_parameters)
        self.Hf_flag = seqm_parameters.get("Hf_flag", True)
        self.eig = seqm_parameters.get("eig", True)
        _check_options(seqm_parameters)
        # excited states (basics.py:465-478): defaults, and the SCF at least 10x tighter than
        # the excited-state tolerance (the dict is updated in place, as the reference does)
        self.excited_states = seqm_parameters.get("excited_states")
        if self.excited_states:
            self.excited_states["tolerance"] = self.excited_states.get("tolerance", 1e-6)
            self.excited_states["method"] = self.excited_states.get("method", "cis").lower()
            if seqm_parameters["scf_eps"] > 1e-1 * self.excited_states["tolerance"]:
                seqm_parameters["scf_eps"] = 1e-1 * self.excited_states["tolerance"]

    def _excited(self, molecule, solve):
        """CIS / RPA excitation energies and amplitudes of the ground state (basics.py:977-1029):
        molecule.cis_energies (nmol, nroots), molecule.cis_amplitudes (nmol, nroots, nocc*nvirt),
        for RPA (2, nmol, nroots, nocc*nvirt) with X and Y; occupied / virtual padded to the
        batch's largest."""
        from .excited import ExcitedStates

        es = self.excited_states
        t0 = time.time()
        # orbital_window: CIS of a batch of one species (rcis_batch); the reference's ragged CIS
        # and its RPA run without it (basics.py:983-1026)
        L = solve.L
        window = es.get("orbital_window")
        uniform = bool(np.all(L.norb == L.norb[0]) and np.all(L.nocc == L.nocc[0]))
        ex = ExcitedStates(solve.s, window if (window is not None and es["method"] in ("cis", "tda") and uniform)
                           else None)
        with torch.no_grad():
            E, amp = ex.solve(int(es["n_states"]), float(es["tolerance"]), rpa=es["method"] == "rpa",
                              max_iter=es.get("max_iter"))
        if not ex.converged.all():
            raise Exception("Maximum iterations reached but roots have not converged")
        amp = _phase_align(amp, getattr(molecule, "cis_amplitudes", None), es["method"] == "rpa")
        dev = molecule.coordinates.device
        molecule.cis_energies = E.to(dev)
        molecule.cis_amplitudes = amp.to(dev)
        # transition dipoles and oscillator strengths (rcis_analysis, rcis_batch.py:650-676;
        # the reference computes them when the molecule is verbose, its default, or has an
        # active excited state)
        with torch.no_grad():
            mu, f = ex.transition_properties(E, amp, rpa=es["method"] == "rpa")
        molecule.transition_dipole = mu.to(dev)
        molecule.oscillator_strength = f.to(dev)
        if es.get("save_tdm", False):  # transition densities per root (rcis_batch.py:697-699)
            with torch.no_grad():
                molecule.transition_density_matrices = ex.transition_densities(amp, es["method"] == "rpa").to(dev)
        molecule._excited = ex
        # nonadiabatic couplings between CIS states (basics.py:1042-1058, calc_nac nac.py:118-189)
        pairs = nac_pairs(self.seqm_parameters, int(es["n_states"]))
        molecule.nac, molecule.nac_dot = None, None
        if pairs is not None:
            if es["method"] == "rpa":
                raise NotImplementedError("Nonadiabatic coupling vecotrs not yet implemented for RPA. Use CIS instead.")
            if ex.window is not None:
                raise NotImplementedError("nonadiabatic couplings with an orbital_window are not supported")
            molecule.nac = self._nac(molecule, solve, ex, E, amp, pairs)
        if molecule.const.do_timing:
            torch.cuda.synchronize()
            molecule.const.timing["CIS/RPA"].append(time.time() - t0)

    @staticmethod
    def _nac(molecule, solve, ex, E, amp, pairs):
        """{(s1 - 1, s2 - 1): (nmol, molsize, 3)}: d_ij = sum B_ij dF(P)/dR / (E_j - E_i), the
        unrelaxed CIS derivative couplings, with the excited-state derivative kernel (B_ij in the
        place of the relaxed density, no transition-density terms)."""
        L = solve.L
        dev = molecule.coordinates.device
        out = {}
        with torch.no_grad():
            zero = torch.zeros(ex.T, dtype=torch.float64, device=solve.dev)
            ones = torch.ones(L.nmol, dtype=torch.float64, device=solve.dev)
            real = torch.as_tensor(L.real_index, device=solve.dev)
            for (a, b), B in zip(pairs, ex.nac_densities(amp, [(a - 1, b - 1) for a, b in pairs])):
                g = solve.grad_excited(ones, ex.to_ragged(B), zero)
                full = torch.zeros(L.nmol * L.molsize, 3, dtype=torch.float64, device=solve.dev)
                full[real] = g
                d = (E[:, b - 1] - E[:, a - 1]).to(solve.dev)
                out[(a - 1, b - 1)] = (full.view(L.nmol, L.molsize, 3) / d[:, None, None]).to(dev)
        return out

    def _all_forces(self, molecule, solve, xyz):
        """do_all_forces (basics.py:1124-1158): molecule.all_forces (nmol, nroots + 1, molsize, 3),
        the ground state's forces and those of every excited state, and each state's relaxed and
        unrelaxed dipoles (make_cis_state_dipole, rcis_grad_batch.py:266-288; Debye)."""
        if not self.seqm_parameters.get("analytical_gradient", [False])[0]:
            raise Exception("when asking for calculating all gradients of excited states ask for analytical gradients")
        if not self.excited_states:
            raise Exception("do_all_forces needs excited_states")
        ex = molecule._excited
        if ex.window is not None:
            raise NotImplementedError("excited-state forces with an orbital_window are not supported")
        L = solve.L
        dev = molecule.coordinates.device
        rpa = self.excited_states["method"] == "rpa"
        amp = molecule.cis_amplitudes.to(solve.dev)
        nroots = int(self.excited_states["n_states"])
        real = torch.as_tensor(L.real_index, device=solve.dev)
        ones = torch.ones(L.nmol, dtype=torch.float64, device=solve.dev)
        tol = float(self.excited_states["tolerance"])

        def padded(g):
            full = torch.zeros(L.nmol * L.molsize, 3, dtype=torch.float64, device=solve.dev)
            full[real] = g
            return full.view(L.nmol, L.molsize, 3)

        with torch.no_grad():
            ground, _ = solve.grad(ones, ones)
        if self.seqm_parameters.get("dispersion", False) and self.method == "AM1":
            x = xyz.detach().clone().requires_grad_(True)
            with torch.enable_grad():
                gd, = torch.autograd.grad(_dispersion_am1_fs1(L, x).sum(), x)
            ground = ground + gd.to(solve.dev)
        forces = torch.empty(L.nmol, nroots + 1, L.molsize, 3, dtype=torch.float64, device=solve.dev)
        forces[:, 0] = -padded(ground)
        relaxed = torch.empty(L.nmol, nroots, 3, dtype=torch.float64, device=solve.dev)
        unrelaxed = torch.empty_like(relaxed)
        dip0 = molecule.dipole.to(solve.dev)
        with torch.no_grad():
            for k in range(nroots):
                X, Y = (amp[0, :, k], amp[1, :, k]) if rpa else (amp[:, k], None)
                R, B, D = ex.state_densities(X, Y, tol)
                forces[:, k + 1] = -padded(ground + solve.grad_excited(ones, ex.to_ragged(D), ex.to_ragged(R)))
                mu = ex.dipole_contract(torch.stack((B, D), dim=1)) * (TO_DEBYE * DEBYE_TO_AU)
                unrelaxed[:, k], relaxed[:, k] = mu[:, 0] + dip0, mu[:, 1] + dip0
        molecule.all_forces = forces.to(dev)
        molecule.all_cis_relaxed_diploles = relaxed.to(dev)
        molecule.all_cis_unrelaxed_diploles = unrelaxed.to(dev)

    def _active_energy(self, molecule, solve, act, xyz):
        """Excitation energy of each molecule's active state as a differentiable function of the
        coordinates (its gradient from ExcitedEnergyFunction)."""
        ex = molecule._excited
        if ex.window is not None:
            raise NotImplementedError("excited-state forces with an orbital_window are not supported")
        rpa = self.excited_states["method"] == "rpa"
        E = molecule.cis_energies.to(solve.dev)
        k = E.shape[1]
        if bool((act > k).any()) or bool((act < 0).any()):
            raise ValueError(f"active_state must be between 0 and the number of excited states ({k})")
        exc = (act > 0).to(solve.dev)
        idx = (act.to(solve.dev) - 1).clamp(min=0)
        amp = molecule.cis_amplitudes.to(solve.dev)
        rows = torch.arange(E.shape[0], device=solve.dev)
        if rpa:
            X, Y = amp[0, rows, idx], amp[1, rows, idx]
        else:
            X, Y = amp[rows, idx], None
        X = X * exc[:, None]
        Y = Y * exc[:, None] if Y is not None else None
        E_state = E[rows, idx] * exc
        tol = float(self.excited_states["tolerance"])
        return ExcitedEnergyFunction.apply(xyz, solve, ex, X, Y, E_state, exc.double(), tol).to(
            molecule.coordinates.device)

    @staticmethod
    def _refresh_geometry(molecule):
        with torch.no_grad():
            real = torch.nonzero(molecule.species.reshape(-1) > 0, as_tuple=False).squeeze(1)
            xyz = molecule.coordinates.reshape(-1, 3)[real]
            d = xyz[molecule.idxj] - xyz[molecule.idxi]
            r = torch.linalg.norm(d, dim=1)
            molecule.xij = d / r.unsqueeze(1)
            molecule.rij = r * molecule.const.length_conversion_factor

    def _prepare(self, molecule, learned_parameters):
        if self.parser is None:
            self.parser = Parser(self.seqm_parameters)
            self.packpar = Pack_Parameters(self.seqm_parameters).to(molecule.coordinates.device)
        (molecule.nmol, molecule.molsize, molecule.nSuperHeavy, molecule.nHeavy, molecule.nHydro, molecule.nocc,
         molecule.Z, molecule.maskd, molecule.atom_molid, molecule.mask, molecule.pair_molid, molecule.ni,
         molecule.nj, molecule.idxi, molecule.idxj, molecule.xij, molecule.rij) = self.parser(molecule, self.method)
        if callable(learned_parameters):
            learned_parameters = learned_parameters(molecule.species, molecule.coordinates)
        self.packpar = self.packpar.to(molecule.coordinates.device)
        molecule.parameters, molecule.alp, molecule.chi = copy.deepcopy(
            self.packpar(molecule.Z, learned_params=learned_parameters))
        _complete_parameters(molecule.parameters)
        for k, v in molecule.parameters.items():
            if torch.is_tensor(v) and v.requires_grad and k not in GRAD_PARAMS and k not in ("beta",):
                raise NotImplementedError(f"gradients with respect to {k} are not supported "
                                          f"(supported: {', '.join(GRAD_PARAMS)})")

    def forward(self, molecule, learned_parameters=dict(), all_terms=False, P0=None, cis_amp=None, *args, **kwargs):
        static = not callable(learned_parameters) and not learned_parameters
        prev = getattr(molecule, "_solve", None)
        if (static and prev is not None and P0 is not None and P0 is getattr(molecule, "_solve_dm", None)
                and torch.is_tensor(getattr(molecule, "idxi", None)) and self.parser is not None):
            self._refresh_geometry(molecule)  # same molecules, new coordinates (basics.py:733-746)
        else:
            self._prepare(molecule, learned_parameters)
        s = self.hamiltonian.solve(molecule, P0, reuse=static)
        dev = molecule.coordinates.device
        L = s.L
        real = torch.as_tensor(L.real_index, device=dev)
        xyz = molecule.coordinates.reshape(-1, 3)[real]
        p = molecule.parameters
        Eelec, Enuc = SCFEnergyFunction.apply(xyz, p["U_ss"], p["U_pp"], p["beta_s"], p["beta_p"], s)
        Eelec, Enuc = Eelec.to(dev), Enuc.to(dev)
        F, e, P, H, w, charge, rho0xi, rho0xj, _, _, nc, v = _hamiltonian_outputs(molecule, s, self.eig)
        molecule.w = w.to(dev)
        if self.eig:
            if s.uhf:  # per-spin gaps; none when a spin has no occupied orbital (basics.py:829-840)
                nocc = molecule.nocc.to(e.device)
                if bool((nocc == 0).any()):
                    e_gap = torch.tensor([])
                else:
                    la, lb = nocc[:, 0].unsqueeze(0).T, nocc[:, 1].unsqueeze(0).T
                    ga = e[:, 0].gather(1, la) - e[:, 0].gather(1, la - 1)
                    gb = e[:, 1].gather(1, lb) - e[:, 1].gather(1, lb - 1)
                    e_gap = torch.stack((ga.reshape(-1), gb.reshape(-1)), dim=1)
                e_gap = e_gap.to(dev)
            else:
                lumo = molecule.nocc.unsqueeze(0).T.to(e.device)
                e_gap = (e.gather(1, lumo) - e.gather(1, lumo - 1)).reshape(-1).to(dev)
            molecule.molecular_orbitals = v.to(dev)
            e = e.to(dev)
        else:
            e_gap = None
        EnucAB = s.pair_values_reference_order(s.s.enuc_pair).to(dev)
        molecule._gam = w[..., 0, 0].to(dev)
        with torch.no_grad():
            molecule.dipole = _dipole(molecule, s).to(dev)
        P = P.to(dev)
        nc = nc.to(dev)
        charge = charge.to(dev) if charge is not None else None
        molecule._solve = s
        if self.excited_states:
            self._excited(molecule, s)
        if self.seqm_parameters.get("do_all_forces", False):
            self._all_forces(molecule, s, xyz)
        act = _active_states(molecule, L.nmol, dev)
        Eexc = None
        if bool((act > 0).any()):
            # excited-state energy and forces of the active state (basics.py:1044-1105)
            if not self.excited_states:
                raise Exception("You have requested for excited state dynamics but have not given input parameters "
                                "for excited states (like n_states) in seqm_parameters")
            Eexc = self._active_energy(molecule, s, act, xyz)
        if all_terms:
            Etot = Eelec + Enuc if Eexc is None else Eelec + Enuc + Eexc
            if self.seqm_parameters.get("dispersion", False) and self.method == "AM1":  # basics.py:1233-1234
                Etot = Etot + _dispersion_am1_fs1(L, xyz).to(dev)
            Eiso = _isolated_atom_energy(molecule.const, molecule.Z, p)
            Eiso_sum = torch.zeros_like(Etot).index_add(0, molecule.atom_molid, Eiso)
            if self.Hf_flag:
                eheat = torch.zeros_like(Etot).index_add(0, molecule.atom_molid, molecule.const.eheat[molecule.Z])
                Hf = Etot - Eiso_sum + eheat
            else:
                Hf = Etot - Eiso_sum
            return Hf, Etot, Eelec, Enuc, Eiso_sum, EnucAB, e_gap, e, P, charge, nc
        return Eelec, EnucAB, P, nc


class Force(torch.nn.Module):
    """Forces -dHf/dR (basics.py:1247-1365)."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.energy = Energy(seqm_parameters)
        self.create_graph = seqm_parameters.get("2nd_grad", False)
        self.eig = seqm_parameters.get("eig", True)
        self.seqm_parameters = seqm_parameters
        if self.create_graph:
            raise NotImplementedError("second derivatives (2nd_grad) are not supported")

    def forward(self, molecule, learned_parameters=dict(), P0=None, cis_amp=None, do_force=True, *args, **kwargs):
        molecule.coordinates.requires_grad_(do_force)
        Hf, Etot, Eelec, Enuc, Eiso, _, e_gap, e, D, charge, nc = self.energy(
            molecule, learned_parameters=learned_parameters, all_terms=True, P0=P0)
        if self.eig and e is not None:
            e, e_gap = e.detach(), e_gap.detach()
        if do_force:
            t0 = time.time()
            Hf.sum().backward()
            force = -molecule.coordinates.grad.detach()
            molecule.coordinates.grad.zero_()
            if molecule.const.do_timing:
                torch.cuda.synchronize()
                molecule.const.timing["Force"].append(time.time() - t0)
            if self.seqm_parameters.get("analytical_gradient", [False])[0]:
                molecule.analytical_gradient = -force
        else:
            force = torch.tensor([])
        return (force.detach(), D.detach(), Hf.detach(), Etot.detach(), Eelec.detach(), Enuc.detach(), Eiso.detach(),
                e, e_gap, charge, nc)


def _xl_bomd_force(molecule, P, seqm_parameters, xl_params=None):
    """XL-BOMD energy and forces from the auxiliary density P (the extended-Lagrangian shadow
    potential, dynamics/xlbomd.py:58-505 without the Krylov kernel): F = F(P) (one Fock build),
    D = 2 C_occ C_occ^T of F (one eigensolve, no SCF), Eelec = tr(D F) - 1/2 tr((F - H) P)
    (energy.py:76-88), forces -d(Eelec + Enuc)/dR at fixed D and P.

    The shadow energy is tr(D H) + B(D, P) - 1/2 B(P, P) with B(X, Y) = tr(X G(Y)) symmetric and
    bilinear; the adjoint kernel gives g(X) = d/dR [tr(X H) + 1/2 B(X, X)] for any symmetric X,
    so the gradient is 3/2 g(D + P) - 1/2 g(-(D + P)) - g(D) - 2 g(P) (polarisation) plus the
    nuclear term.  The layout, integrals buffers and the eigensolver's warm start stay on the
    device between steps (the solve of the first SCF step is continued).  With max_rank in
    xl_params (KSA-XL-BOMD, xlbomd.py:200-341): D is the Fermi-Dirac density at T_el, the
    entropy term -2 T_el S is returned as Electronic_entropy and the rank-m Krylov kernel gives
    molecule.dP2dt2 for the propagation."""
    xl_params = xl_params or {}
    krylov = "max_rank" in xl_params
    if P is None:
        raise ValueError("XL-BOMD needs the auxiliary density P0")
    if bool((_active_states(molecule, int(molecule.species.shape[0]), P.device) > 0).any()):
        raise NotImplementedError("excited-state XL-BOMD (XL-ESMD) is not supported")
    if seqm_parameters.get("UHF", False):
        raise NotImplementedError("XL-BOMD is implemented for closed shells")
    sv = getattr(molecule, "_solve", None)
    if sv is None or not sv.matches(molecule, seqm_parameters):
        sv = _Solve(molecule, seqm_parameters)
        molecule._solve = sv
    L, s, dev = sv.L, sv.s, sv.dev
    lib = native.load()
    with torch.no_grad():
        real = torch.as_tensor(L.real_index, device=molecule.coordinates.device)
        L.set_coordinates(molecule.coordinates.detach().reshape(-1, 3)[real].cpu().numpy())
        s.hcore()
        Pk = L.padded_to_packed(P.detach().to(dev, torch.float64))
        s.P.copy_(Pk)
        s.fock()  # F(P)
        sp2 = tuple(seqm_parameters.get("sp2", [False]))
        use_sp2 = bool(sp2[0]) and not krylov
        if use_sp2:
            # D by SP2 purification (the reference's sp2 branch of EnergyXL, dynamics/xlbomd.py:
            # 349-357; that branch stops at its own orbital-energy line with an AttributeError,
            # the density it intends is this one, with zero orbital energies and gaps)
            s.density(s.Pnew, sp2, active=None, evecs=None, density_only=0)
        else:
            evecs = torch.empty_like(s.work)
            s.density(s.Pnew, (False,), active=None, evecs=evecs, density_only=0)
            s.evecs = evecs
        D = s.Pnew
        if krylov:
            from .xl_krylov import PaddedBasis, fermi_density, krylov_kernel

            if getattr(L, "_padded_basis", None) is None:
                L._padded_basis = PaddedBasis(L)
            basis = L._padded_basis
            T_el = float(xl_params["T_el"])
            Q = basis.to_padded(evecs).transpose(1, 2)
            e = basis.vector_to_padded(s.evals)
            Dp, S_ent, fe, mu = fermi_density(e, Q, L.nocc, basis.mask, T_el)
            d2, kerr = krylov_kernel(s, basis, Dp, basis.to_padded(Pk), Q, e, mu, T_el, int(xl_params["max_rank"]),
                                     float(xl_params["err_threshold"]))
            D = basis.to_ragged(Dp)
        if getattr(L, "_elem_mol", None) is None:
            L._elem_mol = torch.repeat_interleave(torch.arange(L.nmol, device=dev),
                                                  torch.as_tensor(L.norb * L.norb, device=dev))
        T = int(L.mat_off[-1])
        t = D[:T] * s.F[:T] - 0.5 * (s.F[:T] - s.H[:T]) * Pk[:T]
        Eelec = torch.zeros(L.nmol, dtype=torch.float64, device=dev).index_add_(0, L._elem_mol, t)
        Enuc = s.Enuc[: L.nmol].clone()
        # forces by polarisation of the adjoint kernel's quadratic form
        ones = torch.ones(max(1, L.nmol), dtype=torch.float64, device=dev)
        zeros = torch.zeros_like(ones)
        dR = torch.zeros(3 * max(1, L.natoms), dtype=torch.float64, device=dev)
        dpar = torch.empty(4 * max(1, L.natoms), dtype=torch.float64, device=dev)
        work = torch.empty(7 * max(1, L.npairs), dtype=torch.float64, device=dev)
        Dp = D[:T] + Pk[:T]
        grad = torch.zeros(3 * L.natoms, dtype=torch.float64, device=dev)
        for X, c, gE, gN in ((Dp, 1.5, ones, zeros), (-Dp, -0.5, ones, zeros), (D[:T], -1.0, ones, zeros),
                             (Pk[:T], -2.0, ones, zeros), (Pk[:T], 1.0, zeros, ones)):
            X = X.contiguous()
            s.launches += 2
            native.check(lib.seqm_energy_grad(L.struct, native.ptr(X), None, native.ptr(gE), native.ptr(gN),
                                              native.ptr(dR), native.ptr(dpar), native.ptr(work), s._s()),
                         "seqm_energy_grad")
            grad += c * dR[: 3 * L.natoms]
        cdev = molecule.coordinates.device
        force = torch.zeros(L.nmol * L.molsize, 3, dtype=torch.float64, device=cdev)
        force[real] = -grad.view(L.natoms, 3).to(cdev)
        molecule.force = force.view(L.nmol, L.molsize, 3)
        molecule.dm = L.packed_to_padded(D).to(cdev)
        Etot = (Eelec + Enuc).to(cdev)
        p = molecule.parameters
        Eiso = _isolated_atom_energy(molecule.const, molecule.Z, p)
        Eiso_sum = torch.zeros_like(Etot).index_add(0, molecule.atom_molid, Eiso.detach())
        eheat = torch.zeros_like(Etot).index_add(0, molecule.atom_molid, molecule.const.eheat[molecule.Z])
        molecule.Etot, molecule.Eelec, molecule.Enuc, molecule.Eiso = Etot, Eelec.to(cdev), Enuc.to(cdev), Eiso_sum
        molecule.Hf = Etot - Eiso_sum + eheat if seqm_parameters.get("Hf_flag", True) else Etot - Eiso_sum
        if use_sp2:  # no orbitals from SP2 (xlbomd.py:355-356)
            molecule.e_mo = torch.zeros(L.nmol, int(L.nocc.max()), dtype=torch.float64, device=cdev)
            molecule.e_gap = torch.zeros(L.nmol, 1, dtype=torch.float64, device=cdev)
        else:
            e, v = sv.eigen_padded()
            lumo = molecule.nocc.unsqueeze(0).T.to(e.device)
            molecule.e_mo = e.to(cdev)
            molecule.e_gap = (e.gather(1, lumo) - e.gather(1, lumo - 1)).reshape(-1).to(cdev)
            molecule.molecular_orbitals = v.to(cdev)
        if krylov:
            molecule.Electronic_entropy = (-2.0 * T_el * S_ent).to(cdev)
            molecule.dP2dt2 = L.packed_to_padded(basis.to_ragged(d2)).to(cdev)
            molecule.Krylov_Error = kerr.to(cdev)
            molecule.Fermi_occ = fe.to(cdev)
        else:
            molecule.Electronic_entropy = torch.zeros(L.nmol, dtype=torch.float64, device=cdev)
            molecule.dP2dt2 = None
            molecule.Krylov_Error = None
            molecule.Fermi_occ = None


class EnergyXL(torch.nn.Module):
    """XL-BOMD shadow energy terms from the auxiliary density P (EnergyXL, dynamics/xlbomd.py:
    58-508): one Fock build of F(P), D from it (eigensolve, SP2 or the Fermi-Dirac density of
    KSA-XL-BOMD with xl_bomd_params' max_rank / err_threshold / T_el).  With all_terms:
    (Hf, Etot, Eelec, EEnt, Enuc, Eiso, EnucAB, D, dP2dt2, Error, e_gap, e, Fe_occ); otherwise
    (Eelec, EnucAB, D, e_gap, e).  The forces are computed along (molecule.force)."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.seqm_parameters = seqm_parameters

    def forward(self, molecule, P, cis_amp=None, learned_parameters=dict(), xl_bomd_params=dict(), all_terms=False,
                *args, **kwargs):
        if cis_amp is not None:
            raise NotImplementedError("excited-state XL-BOMD (XL-ESMD) is not supported")
        if callable(learned_parameters) or learned_parameters:
            raise NotImplementedError("XL-BOMD with learned parameters is not supported")
        _xl_bomd_force(molecule, P, self.seqm_parameters, xl_bomd_params or {})
        m = molecule
        sv = m._solve
        EnucAB = sv.pair_values_reference_order(sv.s.enuc_pair).to(m.coordinates.device)
        if all_terms:
            return (m.Hf, m.Etot, m.Eelec, m.Electronic_entropy, m.Enuc, m.Eiso, EnucAB, m.dm, m.dP2dt2,
                    getattr(m, "Krylov_Error", None), m.e_gap, m.e_mo, getattr(m, "Fermi_occ", None))
        return m.Eelec, EnucAB, m.dm, m.e_gap, m.e_mo


class ForceXL(torch.nn.Module):
    """XL-BOMD forces (ForceXL, dynamics/xlbomd.py:511-570): (force, D, Hf, Etot, Eelec, Enuc,
    Eiso, e, e_gap, EEnt, dP2dt2, Error, Fe_occ), the forces from the adjoint kernel's
    polarisation at fixed D and P."""

    def __init__(self, seqm_parameters):
        super().__init__()
        self.energy = EnergyXL(seqm_parameters)
        self.seqm_parameters = seqm_parameters

    def forward(self, molecule, P, cis_amp=None, learned_parameters=dict(), xl_bomd_params=dict(), *args, **kwargs):
        Hf, Etot, Eelec, EEnt, Enuc, Eiso, _, D, dP2dt2, Error, e_gap, e, Fe_occ = self.energy(
            molecule, P, cis_amp, learned_parameters, xl_bomd_params, all_terms=True)
        return (molecule.force.detach(), D.detach(), Hf, Etot.detach(), Eelec.detach(), Enuc.detach(), Eiso.detach(),
                e, e_gap, EEnt, dP2dt2, Error, Fe_occ)


class NACConfig:
    """Resolved nonadiabatic-coupling settings (NACConfig, dynamics/nac_utils.py:5-8)."""

    def __init__(self, enabled, pairs):
        self.enabled, self.pairs = bool(enabled), list(pairs)

    def __repr__(self):
        return f"NACConfig(enabled={self.enabled}, pairs={self.pairs})"


def resolve_nac_config(seqm_parameters, *, nroots=None, default_enabled=False):
    """seqm_parameters['nonadiabatic'] -> NACConfig (resolve_nac_config, nac_utils.py:29-63):
    'compute_nac' on / off; 'states' gives all their pairs; 'pairs' explicit ones; all pairs of
    the nroots states when enabled without either; pairs sorted, deduplicated, diagonal and
    (given nroots) out-of-range ones dropped."""
    cfg = dict(seqm_parameters.get("nonadiabatic", {}))
    enabled = bool(cfg.get("compute_nac", default_enabled))
    pairs = []
    u = sorted({int(x) for x in cfg.get("states") or [] if isinstance(x, (int, float))})
    pairs += [(u[a], u[b]) for a in range(len(u)) for b in range(a + 1, len(u))]
    pairs += [(int(p[0]), int(p[1])) for p in cfg.get("pairs") or [] if isinstance(p, (list, tuple)) and len(p) == 2]
    if enabled and not pairs and nroots:
        pairs = [(a, b) for a in range(1, nroots + 1) for b in range(a + 1, nroots + 1)]
    out = []
    for s1, s2 in pairs:
        a, b = sorted((int(s1), int(s2)))
        if s1 == s2 or (nroots is not None and not (1 <= a <= nroots and 1 <= b <= nroots)) or (a, b) in out:
            continue
        out.append((a, b))
    return NACConfig(enabled, out)


def active_state_tensor(active_state, nmol, device):
    """active_state (int or tensor, 1-based excited states, 0 ground) as a (nmol,) long tensor
    (dynamics/active_state.py:4-15)."""
    from types import SimpleNamespace

    return _active_states(SimpleNamespace(active_state=active_state), int(nmol), device)


class Electronic_Structure(torch.nn.Module):
    """Single-point driver (ElectronicStructure.py:10-127): sets force, dm, energies, charges."""

    def __init__(self, seqm_parameters, *args, **kwargs):
        super().__init__()
        self.seqm_parameters = seqm_parameters
        self.conservative_force = Force(seqm_parameters)

    @staticmethod
    def atomic_charges(P, n_orbital=4):
        n_molecule = P.shape[0]
        n_atom = P.shape[1] // n_orbital
        return P.diagonal(dim1=1, dim2=2).reshape(n_molecule, n_atom, n_orbital).sum(axis=2)

    def forward(self, molecule, learned_parameters=dict(), xl_bomd_params=dict(), P0=None, err_threshold=None,
                max_rank=None, T_el=None, dm_prop="SCF", *args, **kwargs):
        if dm_prop == "XL-BOMD":
            if callable(learned_parameters) or learned_parameters:
                raise NotImplementedError("XL-BOMD with learned parameters is not supported")
            _xl_bomd_force(molecule, P0, self.seqm_parameters, xl_bomd_params or {})
        elif dm_prop != "SCF":
            raise NotImplementedError("dm_prop must be 'SCF' or 'XL-BOMD'")
        else:
            self._scf(molecule, P0, learned_parameters)
        with torch.no_grad():
            if molecule.dm.dim() == 4:  # open shell: both spins (ElectronicStructure.py:106-117)
                molecule.q = (molecule.const.tore[molecule.species] - self.atomic_charges(molecule.dm[:, 0])
                              - self.atomic_charges(molecule.dm[:, 1]))
            else:
                molecule.q = molecule.const.tore[molecule.species] - self.atomic_charges(molecule.dm)

    def _scf(self, molecule, P0, learned_parameters):
        (molecule.force, P, molecule.Hf, molecule.Etot, molecule.Eelec, molecule.Enuc, molecule.Eiso, molecule.e_mo,
         molecule.e_gap, self.charge, self.notconverged) = self.conservative_force(
            molecule, P0=P0, learned_parameters=learned_parameters)
        molecule.dm = P.detach()
        molecule._solve_dm = molecule.dm  # the density handed out; an MD step passes it back as P0

    def get_force(self):
        return self.force

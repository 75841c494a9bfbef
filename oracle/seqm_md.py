"""NumPy restatement of PYSEQM's molecular dynamics integrators (seqm/MolecularDynamics.py).

TEST INFRASTRUCTURE ONLY: the CPU oracle for the MD drivers, used by ``tests/``.  Nothing in
the product package imports it.  Forces come from ``seqm_oracle.single_point`` (fixed-density
central differences at the converged SCF density).

Restated: the unit conversions of PhysicalConstants (MolecularDynamics.py:21-31), momentum
removal _zero_com (:746-782), kinetic energy and temperature (:784-793), velocity Verlet
one_step (:815-842), the Langevin integrator's friction / noise factors (:1391-1407) and
its thermostat half steps (:1311-1344).  Only Temp 0 Langevin (friction, no noise) is
deterministic and restated here.
"""

import numpy as np

from . import seqm_oracle as O

ACC_SCALE = 0.009648532800137615  # eV/A / (g/mol) -> A/fs^2, MolecularDynamics.py:25
VEL_SCALE = 0.9118367323190634e-3  # sqrt(K/amu) -> A/fs, :26
KINETIC_ENERGY_SCALE = 1.0364270099032438e2  # amu (A/fs)^2 -> eV, :27
TEMPERATURE_SCALE = 1.160451812e4  # K/eV, :28


def masses(species):
    """(nmol, molsize, 1) atomic masses, 0 for padding (Molecule.py:120-125)."""
    m = O.load_elements()["mass"][np.asarray(species)]
    return m[..., None]


def kinetic_energy(mass, v):
    """MolecularDynamics.py:784-789 (eV per molecule)."""
    return np.sum(0.5 * mass * v ** 2, axis=(1, 2)) * KINETIC_ENERGY_SCALE


def temperature(ek, n_dof):
    """MolecularDynamics.py:791-793."""
    return ek * TEMPERATURE_SCALE / (0.5 * n_dof)


def zero_com(mass, r, v, remove_angular=True, restore_kinetic_energy=True):
    """Remove the centre-of-mass velocity and (optionally) the rigid rotation, returning new
    velocities (MolecularDynamics.py:746-782; pseudo-inverse of the inertia tensor with an
    absolute cutoff of 1e-10)."""
    M = np.sum(mass, axis=1, keepdims=True)
    ek0 = kinetic_energy(mass, v)
    r_rel = r - np.sum(mass * r, axis=1, keepdims=True) / M
    v = v - np.sum(mass * v, axis=1, keepdims=True) / M
    if remove_angular:
        L = np.sum(mass * np.cross(r_rel, v), axis=1)
        rr = np.sum(r_rel * r_rel, axis=2, keepdims=True)
        inertia = (np.sum(mass * rr, axis=1)[:, :, None] * np.eye(3)[None]
                   - np.sum(mass[..., None] * r_rel[..., :, None] * r_rel[..., None, :], axis=1))
        omega = np.stack([pinv_hermitian(inertia[m], 1e-10) @ L[m] for m in range(r.shape[0])])
        v = v - np.cross(np.broadcast_to(omega[:, None, :], r_rel.shape), r_rel)
    ek1 = kinetic_energy(mass, v)
    if np.any(ek1 < 1e-12):
        raise RuntimeError("Zero kinetic energy after removing COM momentum")
    if restore_kinetic_energy:
        v = v * np.sqrt(ek0 / ek1)[:, None, None]
    return v


def pinv_hermitian(a, atol):
    """Pseudo-inverse of a symmetric matrix from its eigen-decomposition, dropping eigenvalues
    with |w| <= atol (torch.linalg.pinv(hermitian=True, atol=...))."""
    w, u = np.linalg.eigh(a)
    keep = np.abs(w) > atol
    return (u[:, keep] / w[keep]) @ u[:, keep].T


def trajectory(method, species, coords, v0, steps, dt, eps, converger=(1,), damp=None, fd_step=1.0e-5):
    """Velocity Verlet (MolecularDynamics.py:815-842; with damp, the Temp 0 Langevin
    integrator's friction half steps around it, :1311-1344) from initial velocities v0; the
    initial velocities lose their centre-of-mass and rotational momentum without kinetic-energy
    restoration (initialize_velocity, :717-727).  Returns per step coordinates, velocities,
    forces, Etot and kinetic energy."""
    species = np.asarray(species)
    r = np.array(coords, dtype=np.float64)
    mass = masses(species)
    minv = np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1.0), 0.0)
    v = zero_com(mass, r, np.array(v0, dtype=np.float64), remove_angular=True, restore_kinetic_energy=False)
    c1 = 1.0 if damp is None else float(np.exp(-0.5 * dt / damp))

    def forces(r):
        out = O.single_point(method, species, r, eps, converger, forces=True, fd_step=fd_step)
        return out["force"], out["Etot"]

    f, etot = forces(r)
    a = f * minv * ACC_SCALE
    traj = [dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=etot, Ek=kinetic_energy(mass, v))]
    for _ in range(steps):
        v = v * c1
        v = v + 0.5 * a * dt
        r = r + v * dt
        f, etot = forces(r)
        a = f * minv * ACC_SCALE
        v = v + 0.5 * a * dt
        v = v * c1
        traj.append(dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=etot, Ek=kinetic_energy(mass, v)))
    return traj


# dissipative extended-Lagrangian coefficients [kappa, alpha, c0..ck] (Niklasson et al., J. Chem.
# Phys. 130, 214109 (2009); MolecularDynamics.py:1367-1376)
XL_COEFFS = {
    3: [1.69, 150e-3, -2.0, 3.0, 0.0, -1.0],
    4: [1.75, 57e-3, -3.0, 6.0, -2.0, -2.0, 1.0],
    5: [1.82, 18e-3, -6.0, 14.0, -8.0, -3.0, 4.0, -1.0],
    6: [1.84, 5.5e-3, -14.0, 36.0, -27.0, -2.0, 12.0, -6.0, 1.0],
    7: [1.86, 1.6e-3, -36.0, 99.0, -88.0, 11.0, 32.0, -25.0, 8.0, -1.0],
    8: [1.88, 0.44e-3, -99.0, 286.0, -286.0, 78.0, 78.0, -90.0, 42.0, -10.0, 1.0],
    9: [1.89, 0.12e-3, -286.0, 858.0, -936.0, 364.0, 168.0, -300.0, 184.0, -63.0, 12.0, -1.0],
}


def xl_energy(method, species, coords, P, D=None, sp2_eps=None):
    """Shadow energy of XL-BOMD (dynamics/xlbomd.py:58-505 without the Krylov kernel): F = F(P),
    D from the eigensolve of F (or SP2 purification to sp2_eps, xlbomd.py:349-357) unless given,
    Eelec = tr(D F) - 1/2 tr((F - H) P) (energy.py:76-88); returns Hf, Etot per molecule and D."""
    el = O.load_elements()
    mol = O.parse(species, coords)
    p = O.atom_params(method, mol["Z"])
    ints = O.integrals(mol, p, el)
    M = O.hcore(mol, p, ints)
    nmol, ms = mol["nmol"], mol["molsize"]
    H = O.symmetrize_upper(O.blocks_to_full(M, nmol, ms))
    F = O.fock(mol, p, ints, M, P)
    if D is None and sp2_eps is not None:
        D = O.density_sp2(F, mol["nheavy"], mol["nhyd"], mol["nocc"], sp2_eps)
    elif D is None:
        D, _, _ = O.density_eigh(F, mol["nheavy"], mol["nhyd"], mol["nocc"])
    Eelec = np.sum(D * F - 0.5 * (F - H) * P, axis=(1, 2))
    EnucAB = O.pair_nuclear_energy(method, mol, p, ints["w"][:, 0, 0], el, ints["rho0"])
    Enuc = np.zeros(nmol)
    np.add.at(Enuc, mol["pair_molid"], EnucAB)
    Eiso = np.zeros(nmol)
    np.add.at(Eiso, mol["atom_molid"], O.isolated_atom_energy(mol["Z"], p, el))
    eheat = np.zeros(nmol)
    np.add.at(eheat, mol["atom_molid"], el["eheat_ev"][mol["Z"]])
    Etot = Eelec + Enuc
    return dict(Etot=Etot, Hf=Etot - Eiso + eheat, D=D)


def xl_trajectory(method, species, coords, v0, steps, dt, eps, k, converger=(1,), h=1.0e-5, sp2_eps=None):
    """XL-BOMD without thermostat (MolecularDynamics.py:1434-1600): the first forces and density
    from the SCF, then the auxiliary density propagated with the k-th order coefficients and the
    shadow-potential forces by central differences at fixed D and P.  sp2_eps: the SCF and the
    shadow density use SP2 purification (the seqm sp2 option)."""
    species = np.asarray(species)
    r = np.array(coords, dtype=np.float64)
    mass = masses(species)
    minv = np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1.0), 0.0)
    v = zero_com(mass, r, np.array(v0, dtype=np.float64), remove_angular=True, restore_kinetic_energy=False)
    sp2_opt = (True, sp2_eps) if sp2_eps is not None else (False,)
    out = O.single_point(method, species, r, eps, converger, sp2_opt=sp2_opt, forces=True)
    f, dm = out["force"], out["P"]
    a = f * minv * ACC_SCALE
    traj = [dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=out["Etot"], Ek=kinetic_energy(mass, v))]
    m = k + 1
    kappa, alpha = XL_COEFFS[k][0], XL_COEFFS[k][1]
    coeff = np.array(XL_COEFFS[k][2:]) * alpha
    coeff[0] += 2.0 - kappa
    coeff[1] -= 1.0
    coeff = np.tile(coeff, 2)
    P = dm.copy()
    Pt = np.repeat(dm[None], m, axis=0)
    for step in range(steps):
        v = v + 0.5 * a * dt
        r = r + v * dt
        c = step % m
        P = kappa * (0.95 * dm + 0.05 * P) + np.tensordot(coeff[c: c + m], Pt, axes=1)
        Pt[m - 1 - c] = P
        e0 = xl_energy(method, species, r, P, sp2_eps=sp2_eps)
        dm = e0["D"]
        f = np.zeros_like(r)
        for mi in range(r.shape[0]):
            for at in range(r.shape[1]):
                if species[mi, at] == 0:
                    continue
                for x in range(3):
                    vals = []
                    for sgn in (1.0, -1.0):
                        rr = r.copy()
                        rr[mi, at, x] += sgn * h
                        vals.append(xl_energy(method, species, rr, P, dm)["Hf"][mi])
                    f[mi, at, x] = -(vals[0] - vals[1]) / (2.0 * h)
        a = f * minv * ACC_SCALE
        v = v + 0.5 * a * dt
        traj.append(dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=e0["Etot"],
                         Ek=kinetic_energy(mass, v)))
    return traj


KB_EV = 8.61739e-5  # eV/K, dynamics/xlbomd.py:206
CANON_DM_PRT_ITER = 10  # dynamics/xlbomd.py:55


def fermi_density(f, nocc, T):
    """Fermi-Dirac density of one packed Fock matrix (fermi_q.py:8-72): eigenpairs, mu by
    Newton iterations on sum_i f_i = nocc (64 at most, tolerance 1e-9), D = 2 Q f Q^T and the
    entropy S = -kB sum [f ln f + (1 - f) ln (1 - f)] over 1e-14 < f < 1 - 1e-14."""
    e, Q = np.linalg.eigh(f, UPLO="U")
    beta = 1.0 / (KB_EV * T)
    mu = 0.5 * (e[nocc - 1] + e[nocc])
    for _ in range(64):
        fe = 1.0 / (1.0 + np.exp(beta * (e - mu)))
        occ = fe.sum()
        if abs(nocc - occ) <= 1e-9:
            break
        mu += (nocc - occ) / max((beta * fe * (1.0 - fe)).sum(), 1e-30)
    D = 2.0 * (Q * fe) @ Q.T
    ok = (fe > 1e-14) & (1.0 - fe > 1e-14)
    p = np.where(ok, fe, 0.5)
    S = np.sum(np.where(ok, -KB_EV * (p * np.log(p) + (1.0 - p) * np.log(1.0 - p)), 0.0))
    return D, S, Q, e, mu


def canon_dm_prt(F1, T, Q, e, mu0, m=CANON_DM_PRT_ITER):
    """First-order density response to F1 by canonical density-matrix perturbation theory
    (canon_dm_prt.py:6-39; Alg. 2 of J. Chem. Theory Comput. 16, 3628 (2020))."""
    beta = 1.0 / (KB_EV * T)
    cnst = 2.0 ** (-2 - m) * beta
    p0 = (0.5 - cnst * (e - mu0))[:, None]
    P1 = -cnst * (Q.T @ F1 @ Q)
    for _ in range(m):
        p02 = p0 * p0
        dX1 = p0 * P1 + P1 * p0.T
        iD0 = 1.0 / (2.0 * (p02 - p0) + 1.0)
        p0 = iD0 * p02
        P1 = iD0 * (dX1 + 2.0 * (P1 - dX1) * p0.T)
    dpdmu = beta * p0 * (1.0 - p0)
    dmu1 = -np.trace(P1) / dpdmu.sum()
    P1 = P1 + np.diag(dpdmu[:, 0]) * dmu1
    return Q @ P1 @ Q.T


def krylov_xl(method, species, coords, P, T, rank, err_threshold=0.0):
    """Fermi density D of F(P), entropy, and the rank-m Krylov approximation of the kernel
    dP2dt2 = -V alpha (dynamics/xlbomd.py:200-341) for one molecule (packed basis)."""
    el = O.load_elements()
    mol = O.parse(species, coords)
    p = O.atom_params(method, mol["Z"])
    ints = O.integrals(mol, p, el)
    M = O.hcore(mol, p, ints)
    F = O.fock(mol, p, ints, M, P)
    idx = O.packed_index(mol["nheavy"][0], mol["nhyd"][0])
    nocc = int(mol["nocc"][0])
    D, S, Q, e, mu = fermi_density(F[0][np.ix_(idx, idx)], nocc, T)
    n4 = F.shape[-1]
    Dfull = np.zeros_like(F)
    Dfull[0][np.ix_(idx, idx)] = D
    dDS = Dfull - P
    nrm = np.linalg.norm(dDS)
    V, W = [], []
    dW = dDS
    err = 10.0
    k = -1
    zeros = np.zeros((mol["nmol"] * mol["molsize"] ** 2, 4, 4))
    while k < rank - 1 and err > err_threshold:
        k += 1
        v = dW.copy()
        for vj in V:
            v = v - np.sum(v[0].T * vj[0]) * vj
        v = v / np.linalg.norm(v)
        V.append(v)
        G = O.fock(mol, p, ints, zeros, v)
        P1 = np.zeros((1, n4, n4))
        P1[0][np.ix_(idx, idx)] = canon_dm_prt(G[0][np.ix_(idx, idx)], T, Q, e, mu)
        w = P1 - v
        W.append(w)
        dW = w
        Wm = np.stack([x[0] for x in W], axis=-1)
        Ov = np.einsum("jir,ijq->rq", Wm, Wm)
        rhs = np.einsum("jir,ij->r", Wm, dDS[0])
        alpha = np.linalg.solve(Ov, rhs)
        err = np.linalg.norm(np.einsum("ijr,r->ij", Wm, alpha) - dDS[0]) / nrm
    Vm = np.stack([x[0] for x in V], axis=-1)
    return Dfull, S, -np.einsum("ijr,r->ij", Vm, alpha)[None]


def ksa_trajectory(method, species, coords, v0, steps, dt, eps, k, T, rank, converger=(1,), h=1.0e-5):
    """KSA-XL-BOMD without thermostat (MolecularDynamics.py:1602-1616): as xl_trajectory with
    Fermi-Dirac densities at T and P propagated with the Krylov kernel's dP2dt2; per molecule,
    so that err_threshold 0 (every molecule at the full rank) decouples the batch."""
    species = np.asarray(species)
    r = np.array(coords, dtype=np.float64)
    mass = masses(species)
    minv = np.where(mass > 0, 1.0 / np.where(mass > 0, mass, 1.0), 0.0)
    v = zero_com(mass, r, np.array(v0, dtype=np.float64), remove_angular=True, restore_kinetic_energy=False)
    out = O.single_point(method, species, r, eps, converger, forces=True)
    f, dm = out["force"], out["P"]
    a = f * minv * ACC_SCALE
    traj = [dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=out["Etot"], Ek=kinetic_energy(mass, v))]
    m = k + 1
    kappa, alpha = XL_COEFFS[k][0], XL_COEFFS[k][1]
    coeff = np.array(XL_COEFFS[k][2:]) * alpha
    coeff[0] += 2.0 - kappa
    coeff[1] -= 1.0
    coeff = np.tile(coeff, 2)
    P = dm.copy()
    Pt = np.repeat(dm[None], m, axis=0)
    d2 = np.zeros_like(dm)
    nmol = species.shape[0]
    for step in range(steps):
        v = v + 0.5 * a * dt
        r = r + v * dt
        c = step % m
        P = kappa * (d2 + P) + np.tensordot(coeff[c: c + m], Pt, axes=1)
        Pt[m - 1 - c] = P
        D = np.zeros_like(P)
        S = np.zeros(nmol)
        for mi in range(nmol):
            na = int(np.sum(species[mi] > 0))
            n4 = 4 * na
            Dm, S[mi], d2m = krylov_xl(method, species[mi: mi + 1, :na], r[mi: mi + 1, :na],
                                       P[mi: mi + 1, :n4, :n4], T, rank)
            D[mi, :n4, :n4] = Dm[0]
            d2[mi] = 0.0
            d2[mi, :n4, :n4] = d2m[0]
        e0 = xl_energy(method, species, r, P, D)
        f = np.zeros_like(r)
        for mi in range(nmol):
            for at in range(r.shape[1]):
                if species[mi, at] == 0:
                    continue
                for x in range(3):
                    vals = []
                    for sgn in (1.0, -1.0):
                        rr = r.copy()
                        rr[mi, at, x] += sgn * h
                        vals.append(xl_energy(method, species, rr, P, D)["Hf"][mi])
                    f[mi, at, x] = -(vals[0] - vals[1]) / (2.0 * h)
        a = f * minv * ACC_SCALE
        v = v + 0.5 * a * dt
        traj.append(dict(coordinates=r.copy(), velocities=v.copy(), force=f, Etot=e0["Etot"],
                         Ek=kinetic_energy(mass, v), entropy=-2.0 * T * S))
    return traj

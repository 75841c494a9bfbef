"""NumPy restatement of PYSEQM's CIS and RPA excited states of the ground-state SCF.

TEST INFRASTRUCTURE ONLY: the CPU oracle for the excited-state solver, used by ``tests/``.
Nothing in the product package imports it.

The reference solves for the lowest roots with Davidson iterations (rcis_batch.py:13-247,
rcis_new.py:19-200, rpa.py:12-210) on the matrix-vector products of
matrix_vector_product_batched (rcis_batch.py:250-293):

    (A V)_ia = (e_a - e_i) V_ia + 2 (C_occ^T G(C_occ V C_virt^T) C_virt)_ia
    (B V)_ia = 2 (C_occ^T G(C_occ V C_virt^T)^T C_virt)_ia

with G the two-electron part of the Fock build for a (not symmetric) AO transition density
(makeA_pi_batched, :296-388, and makeA_pi_symm_batch, :390-507).  The oracle builds A (and B)
column by column for each molecule alone and diagonalises them exactly: CIS roots are the
lowest eigenvalues of A; RPA roots w solve (A - B)^1/2 (A + B) (A - B)^1/2 z = w^2 z, with
X + Y = (A - B)^1/2 z, X - Y = (A + B)(X + Y) / w, normalised to X.X - Y.Y = 1 (rpa.py:213-278).
"""

import numpy as np

from . import seqm_oracle as O


def g_transition(mol, p, ints, P):
    """Two-electron part G(P) of the Fock build for a general (not symmetric) AO density P
    (nmol, 4 ms, 4 ms): the symmetric part as the Fock build (Coulomb, exchange, one-centre);
    the antisymmetric part through exchange and the one-centre (s,p) and (p,p') terms only
    (rcis_batch.py:315-368)."""
    nmol, ms = mol["nmol"], mol["molsize"]
    Ps = 0.5 * (P + np.transpose(P, (0, 2, 1)))
    Pa = 0.5 * (P - np.transpose(P, (0, 2, 1)))
    Gs = O.fock(mol, p, ints, np.zeros((nmol * ms * ms, 4, 4)), Ps)
    Pab = O.full_to_blocks(Pa, nmol, ms)
    Ga = np.zeros_like(Pab)
    mask, maskd = mol["mask"], mol["maskd"]
    rem = mask % (ms * ms)
    mask_l = (mask - rem) + (rem % ms) * ms + rem // ms
    w = ints["w"]
    wk = w[:, O.KIND[:, :, None, None], O.KIND[None, None, :, :]]
    K = np.einsum("nalbs,nls->nab", wk, -0.5 * Pab[mask])
    np.add.at(Ga, mask, K)
    np.add.at(Ga, mask_l, -np.transpose(K, (0, 2, 1)))
    Pd = Pab[maskd]
    t = np.zeros_like(Pd)
    for i in (1, 2, 3):
        t[:, 0, i] = Pd[:, 0, i] * (0.5 * p["h_sp"] - 0.5 * p["g_sp"])
    for i, j in ((1, 2), (1, 3), (2, 3)):
        t[:, i, j] = Pd[:, i, j] * (0.25 * p["g_pp"] - 0.75 * p["g_p2"])
    Ga[maskd] += t - np.transpose(t, (0, 2, 1))
    return Gs + O.blocks_to_full(Ga, nmol, ms)


def transition_properties(mol, p, el, C, nocc, E, X, Y=None):
    """Transition dipoles (au) and oscillator strengths of the roots of one molecule
    (calc_transition_dipoles, rcis_batch.py:679-710): R = C_occ X C_virt^T (+ C_virt Y^T C_occ^T
    for RPA), the one-centre dipole integrals of calc_dipole_matrix (dipole.py:7-82: -R_A on
    each AO of atom A, -dd_A in Angstrom between s and p_d of heavy atoms), mu = sqrt(2)/a0 sum
    R.D, f = 2/3 (E / 27.2113962) |mu|^2."""
    nh, ny = int(mol["nheavy"][0]), int(mol["nhyd"][0])
    n = 4 * nh + ny
    dd = O.multipole_params(mol["Z"], p, el)[0] * O.A0
    xyz = np.asarray(mol["coords"][0], dtype=np.float64)[: nh + ny]
    D = np.zeros((3, n, n))
    for a in range(nh):
        o = 4 * a
        for d in range(3):
            D[d, o: o + 4, o: o + 4] -= np.eye(4) * xyz[a, d]
            D[d, o, o + 1 + d] = D[d, o + 1 + d, o] = -dd[a]
    for h in range(ny):
        D[:, 4 * nh + h, 4 * nh + h] = -xyz[nh + h]
    Co, Cv = C[:, :nocc], C[:, nocc:n]
    R = np.einsum("mi,ria,na->rmn", Co, X, Cv)
    if Y is not None:
        R = R + np.einsum("ma,ria,ni->rmn", Cv, Y, Co)
    mu = np.einsum("rmn,dmn->rd", R, D) * np.sqrt(2.0) / O.A0
    return mu, 2.0 / 3.0 * np.asarray(E) / 27.2113962 * np.sum(mu * mu, axis=1)


def ab_matrices(method, species, coords, eps, converger=(1,), with_b=False, window=None):
    """Per molecule of the batch: orbital energies, C, nocc and the CIS matrix A (and B), each
    molecule run alone (its SCF, integrals and orbitals).  window (n, m): only the n highest
    occupied and m lowest virtual orbitals (orbital_window, rcis_batch.py:900-925)."""
    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    el = O.load_elements()
    res = []
    for m in range(species.shape[0]):
        na = int(np.sum(species[m] > 0))
        sp, xyz = species[m:m + 1, :na], coords[m:m + 1, :na]
        out = O.single_point(method, sp, xyz, eps, converger)
        mol, p = out["mol"], out["params"]
        ints = O.integrals(mol, p, el)
        _, e, vecs = O.density_eigh(out["F"], mol["nheavy"], mol["nhyd"], mol["nocc"])
        C = vecs[0]
        idx = O.packed_index(mol["nheavy"][0], mol["nhyd"][0])
        n, nocc = idx.size, int(mol["nocc"][0])
        ev = e[0, :n]
        if window is not None:  # the window as a molecule of its own
            nb, ma = window
            C = C[:, nocc - nb: nocc + ma]
            ev = ev[nocc - nb: nocc + ma]
            nocc = nb
        nv = C.shape[1] - nocc
        Co, Cv = C[:, :nocc], C[:, nocc:]
        A = np.zeros((nocc * nv, nocc * nv))
        B = np.zeros_like(A) if with_b else None
        n4 = 4 * mol["molsize"]
        for col in range(nocc * nv):
            i, a = divmod(col, nv)
            Pt = np.zeros((1, n4, n4))
            Pt[0][np.ix_(idx, idx)] = np.outer(Co[:, i], Cv[:, a])
            G = g_transition(mol, p, ints, Pt)[0][np.ix_(idx, idx)]
            A[:, col] = 2.0 * (Co.T @ G @ Cv).reshape(-1)
            A[col, col] += ev[nocc + a] - ev[i]
            if with_b:
                B[:, col] = 2.0 * (Co.T @ G.T @ Cv).reshape(-1)
        res.append(dict(A=A, B=B, e=ev, nocc=nocc, nvirt=nv, Etot=out["Etot"][0], C=C, mol=mol, params=p,
                        el=el))
    return res


def cis(method, species, coords, eps, nroots, converger=(1,), window=None):
    """Lowest nroots CIS excitation energies and amplitudes (occ x virt, per molecule)."""
    out = []
    for r in ab_matrices(method, species, coords, eps, converger, window=window):
        w, v = np.linalg.eigh(r["A"])
        amp = v[:, :nroots].T.reshape(nroots, r["nocc"], r["nvirt"])
        mu, f = transition_properties(r["mol"], r["params"], r["el"], r["C"], r["nocc"], w[:nroots], amp)
        out.append(dict(energies=w[:nroots], amplitudes=amp, nocc=r["nocc"], nvirt=r["nvirt"],
                        transition_density=transition_density(r["C"], r["nocc"], amp),
                        transition_dipole=mu, oscillator_strength=f))
    return out


def rpa(method, species, coords, eps, nroots, converger=(1,)):
    """Lowest nroots RPA (TDHF) excitation energies and X, Y amplitudes per molecule."""
    out = []
    for r in ab_matrices(method, species, coords, eps, converger, with_b=True):
        A, B = r["A"], r["B"]
        wm, um = np.linalg.eigh(A - B)
        sq = (um * np.sqrt(wm)) @ um.T
        w2, z = np.linalg.eigh(sq @ (A + B) @ sq)
        w = np.sqrt(w2[:nroots])
        XpY = sq @ z[:, :nroots]
        XmY = (A + B) @ XpY / w
        X, Y = XpY + XmY, XpY - XmY
        nrm = np.sqrt((X ** 2).sum(0) - (Y ** 2).sum(0))
        X, Y = X / nrm, Y / nrm
        shape = (nroots, r["nocc"], r["nvirt"])
        Xs, Ys = X.T.reshape(shape), Y.T.reshape(shape)
        mu, f = transition_properties(r["mol"], r["params"], r["el"], r["C"], r["nocc"], w, Xs, Ys)
        out.append(dict(energies=w, X=Xs, Y=Ys, nocc=r["nocc"], nvirt=r["nvirt"],
                        transition_dipole=mu, oscillator_strength=f,
                        transition_density=transition_density(r["C"], r["nocc"], Xs),
                        transition_density_y=transition_density(r["C"], r["nocc"], Ys)))
    return out


def transition_density(C, nocc, amplitudes):
    """C_occ X C_virt^T per state in the packed AO basis (independent of the orbitals' signs)."""
    return np.einsum("mi,ria,na->rmn", C[:, :nocc], amplitudes, C[:, nocc:])


def state_energy(method, species, coords, eps, state, rpa=False):
    """Total energy of one molecule in excited state `state` (1-based): the ground-state Etot
    plus the state's CIS (or RPA) excitation energy (basics.py:1044-1060 adds it to Etot)."""
    r = ab_matrices(method, species, coords, eps, with_b=rpa)[0]
    A = r["A"]
    if rpa:
        B = r["B"]
        wm, um = np.linalg.eigh(A - B)
        sq = (um * np.sqrt(wm)) @ um.T
        w = np.sqrt(np.linalg.eigvalsh(sq @ (A + B) @ sq))
    else:
        w = np.linalg.eigvalsh(A)
    return r["Etot"] + w[state - 1]


def excited_forces_fd(method, species, coords, eps, state, rpa=False, h=1.0e-4):
    """Forces -dE/dR (eV/Angstrom) of excited state `state` of each molecule by central
    differences of state_energy with steps h and h/2, Richardson-extrapolated (error O(h^4);
    some components have third derivatives large enough that a plain central difference at
    h = 1e-4 A is off by 1e-5): the oracle for the relaxed (Z-vector) analytic gradient of
    rcis_grad_batch (rcis_grad_batch.py:10-259).  Each molecule is run alone."""
    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    f = np.zeros_like(coords)

    def central(sp, xyz, a, x, step):
        e = []
        for sgn in (1.0, -1.0):
            c = xyz.copy()
            c[0, a, x] += sgn * step
            e.append(state_energy(method, sp, c, eps, state, rpa))
        return -(e[0] - e[1]) / (2.0 * step)

    for m in range(species.shape[0]):
        na = int(np.sum(species[m] > 0))
        sp, xyz = species[m:m + 1, :na], coords[m:m + 1, :na]
        for a in range(na):
            for x in range(3):
                f[m, a, x] = (4.0 * central(sp, xyz, a, x, 0.5 * h) - central(sp, xyz, a, x, h)) / 3.0
    return f


def nac_fd(method, species, coords, eps, nroots, pairs, h=1.0e-4):
    """Unrelaxed CIS derivative couplings d_ij = d/dR [sum B_ij F(R; P)] / (E_j - E_i)
    (calc_nac, nac.py:118-189) with B_ij = sym(V_i V_j^T - O_i O_j^T), V = C_virt X^T,
    O = C_occ X, the ground-state density P and B_ij held fixed and the Fock matrix rebuilt at
    displaced geometries (Richardson-extrapolated central differences).  Per molecule (run
    alone): {(i, j): (natoms, 3)} for 1-based pairs.  Signs follow the amplitudes' signs."""
    species = np.asarray(species)
    coords = np.asarray(coords, dtype=np.float64)
    el = O.load_elements()
    out = []
    for m in range(species.shape[0]):
        na = int(np.sum(species[m] > 0))
        sp, xyz = species[m:m + 1, :na], coords[m:m + 1, :na]
        sol = O.single_point(method, sp, xyz, eps)
        P = sol["P"]
        c = cis(method, sp, xyz, eps, nroots)[0]
        mol = sol["mol"]
        idx = O.packed_index(mol["nheavy"][0], mol["nhyd"][0])
        n4 = 4 * mol["molsize"]
        C = ab_matrices(method, sp, xyz, eps)[0]["C"]
        no = c["nocc"]
        Co, Cv = C[:, :no], C[:, no:]

        def fock_at(cc):
            mol2 = O.parse(sp, cc)
            p2 = O.atom_params(method, mol2["Z"])
            ints = O.integrals(mol2, p2, el)
            return O.fock(mol2, p2, ints, O.hcore(mol2, p2, ints), P)[0]

        res = {}
        for i, j in pairs:
            Xi, Xj = c["amplitudes"][i - 1], c["amplitudes"][j - 1]
            B = (Cv @ Xi.T) @ (Cv @ Xj.T).T - (Co @ Xi) @ (Co @ Xj).T
            Bf = np.zeros((n4, n4))
            Bf[np.ix_(idx, idx)] = 0.5 * (B + B.T)
            g = np.zeros((na, 3))
            for a in range(na):
                for x in range(3):
                    def central(step):
                        v = []
                        for sgn in (1.0, -1.0):
                            cc = xyz.copy()
                            cc[0, a, x] += sgn * step
                            v.append(np.sum(Bf * fock_at(cc)))
                        return (v[0] - v[1]) / (2.0 * step)
                    g[a, x] = (4.0 * central(0.5 * h) - central(h)) / 3.0
            res[(i, j)] = g / (c["energies"][j - 1] - c["energies"][i - 1])
        out.append(res)
    return out

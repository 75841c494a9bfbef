"""NumPy restatement of PYSEQM's MNDO/AM1/PM3/PM6_SP single-point SCF path.

TEST INFRASTRUCTURE ONLY.  This module is the CPU oracle used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.  Nothing in
the product package imports it.

Every function states the reference file:line it restates (paths are relative
to the PYSEQM project root).  The layout deliberately follows the reference:
per-atom 4x4 blocks inside padded ``(nmol, 4*molsize, 4*molsize)`` matrices,
hydrogen p-slots zero, atoms of each molecule sorted by descending Z.

The oracle is pinned against outputs of the reference itself
(``tests/golden/*.json``, made by ``tests/golden/make_golden.py``).  Besides the closed-shell
path it restates the unrestricted SCF, Pulay DIIS, the PM6_SP core-core term, the pair cutoff,
the AM1-FS1 dispersion term and the SCF convergence normaliser with super-heavy atoms; the MD and
excited-state oracles live in ``seqm_md.py`` and ``seqm_excited.py``.

Known, deliberate difference: the adaptive mixer's diagonal renormalisation
(seqm/seqm_functions/scf_loop.py:396-415) loops until *every* molecule of the
padded batch is renormalised, which couples molecules.  Here each molecule
stops on its own test, so a molecule's result does not depend on its batch
mates.  The two agree whenever no molecule needs a second renormalisation pass.
"""

import json
import math
import os

import numpy as np

EV = 27.21  # seqm/seqm_functions/constants.py:4
A0 = 0.529167  # seqm/seqm_functions/constants.py:9
EV_KCALPMOL = 23.061  # seqm/seqm_functions/constants.py:10
OVERLAP_CUTOFF = 40.0  # bohr, seqm/seqm_functions/constants.py:23
MAX_ITER = 1000  # seqm/seqm_functions/scf_loop.py:29
DM_ERR_FACTOR = 2.0  # scf_loop.py:50
DM_ELEM_FACTOR = 15.0  # scf_loop.py:51

_DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pyseqm_gb300", "data")

# packed index (k) of the 10 unique products of s,px,py,pz on one atom and the
# (row, col) of the upper-triangle entry it lives in (fock.py:7-18, 74-79)
K10_ROW = np.array([0, 0, 1, 0, 1, 2, 0, 1, 2, 3])
K10_COL = np.array([0, 1, 1, 2, 2, 2, 3, 3, 3, 3])
K10_WEIGHT = np.array([1.0, 2.0, 1.0, 2.0, 2.0, 1.0, 2.0, 2.0, 2.0, 1.0])
KIND = np.array([[0, 1, 3, 6], [1, 2, 4, 7], [3, 4, 5, 8], [6, 7, 8, 9]])  # fock.py:74-79


# --------------------------------------------------------------------------- tables
def load_elements():
    with open(os.path.join(_DATA, "elements.json")) as f:
        d = json.load(f)
    return {k: np.asarray(v, dtype=np.float64) for k, v in d.items() if k != "label"}


def load_params(method):
    # PM6_SP_STAR has PM6_SP's fields; its values come from parameter files (learned overrides)
    method = "PM6_SP" if method == "PM6_SP_STAR" else method
    with open(os.path.join(_DATA, f"params_{method}.json")) as f:
        d = json.load(f)
    return d["fields"], np.asarray(d["rows"], dtype=np.float64)


def load_pair_params(method, zmax):
    """PM6 diatomic core-core parameters alp[Z1, Z2], chi[Z1, Z2] (parameters.py:49-87: the third
    and fourth columns of PWCCT_<method>_MOPAC.csv, for the listed (Z1, Z2) order)."""
    alp, chi = np.zeros((zmax + 1, zmax + 1)), np.zeros((zmax + 1, zmax + 1))
    if method == "PM6_SP_STAR":  # PWCCT reads no file for it (parameters.py:77)
        return alp, chi
    with open(os.path.join(_DATA, f"pwcct_{method}.json")) as f:
        d = json.load(f)
    for z1, z2, a, c in d["entries"]:
        if z1 <= zmax and z2 <= zmax:
            alp[z1, z2], chi[z1, z2] = a, c
    return alp, chi


# --------------------------------------------------------------------------- parser
def parse(species, coords, charges=None, mult=None, cutoff=None):
    """Pair list and counts; restates seqm/basics.py:219-403 (Parser.forward).  cutoff
    (Angstrom, pair_outer_cutoff): only pairs closer than it are kept (basics.py:324-328).

    species: (nmol, molsize) int, rows sorted descending, 0 = padding.
    coords:  (nmol, molsize, 3) Angstrom.
    mult: spin multiplicities for unrestricted HF (basics.py:278-295); nocc is then
    (nmol, 2) = (alpha, beta) occupations.
    """
    el = load_elements()
    species = np.asarray(species, dtype=np.int64)
    coords = np.asarray(coords, dtype=np.float64)
    nmol, molsize = species.shape
    if not np.all(species[:, :-1] >= species[:, 1:]):  # Molecule.py:188-206
        raise ValueError("species must be non-increasing along each row")
    nonblank = species > 0
    flat = species.reshape(-1)
    real_atoms = np.nonzero(flat > 0)[0]
    Z = flat[real_atoms]
    nheavy = np.sum(species > 1, axis=1)
    nhyd = np.sum(species == 1, axis=1)
    # super-heavy count (basics.py:258-270; of the sp elements, 13 <= Z <= 17), which only the
    # SCF convergence test reads: ||dP||/(9 nSuperHeavy + 4 nHeavy + 4 nHydro), scf_loop.py:245
    nsuper = np.sum((species >= 13) & (species <= 17), axis=1)
    n_charge = np.sum(el["tore"][species], axis=1).astype(np.int64)
    if charges is not None:
        n_charge = n_charge - np.asarray(charges, dtype=np.int64).reshape(-1)
    if mult is not None:
        s2 = np.asarray(mult, dtype=np.float64).reshape(-1) - 1.0
        na, nb = n_charge / 2.0 + s2 / 2.0, n_charge / 2.0 - s2 / 2.0
        if np.any(na % 1 != 0) or np.any(nb % 1 != 0):
            raise ValueError("Invalid charge/multiplicity combination!")
        nocc = np.stack([na, nb], axis=1).astype(np.int64)
    else:
        if np.any(n_charge % 2 == 1):  # basics.py:297-299
            raise ValueError("RHF setting requires closed shell systems (even number of electrons)")
        nocc = n_charge // 2
    maskd = (np.arange(molsize) * (molsize + 1))[None, :] + (np.arange(nmol) * molsize**2)[:, None]
    maskd = maskd.reshape(-1)[real_atoms]
    atom_molid = np.repeat(np.arange(nmol), molsize)[real_atoms]
    inv = np.zeros(nmol * molsize, dtype=np.int64)
    inv[real_atoms] = np.arange(real_atoms.size)
    # pairs (i<j) within each molecule, row-major (basics.py:313-343)
    ii, jj = np.triu_indices(molsize, 1)
    m_all = np.repeat(np.arange(nmol), ii.size)
    i_all = np.tile(ii, nmol)
    j_all = np.tile(jj, nmol)
    keep = nonblank[m_all, i_all] & nonblank[m_all, j_all]
    if cutoff is not None:
        dd = coords[m_all, j_all] - coords[m_all, i_all]
        keep &= np.sum(dd * dd, axis=1) < cutoff**2
    m_p, i_p, j_p = m_all[keep], i_all[keep], j_all[keep]
    d = coords[m_p, j_p] - coords[m_p, i_p]
    dist = np.sqrt(np.sum(d * d, axis=1))
    gi = m_p * molsize + i_p
    gj = m_p * molsize + j_p
    return dict(
        nmol=nmol, molsize=molsize, Z=Z, nheavy=nheavy, nhyd=nhyd, nsuper=nsuper, nocc=nocc, maskd=maskd,
        atom_molid=atom_molid, idxi=inv[gi], idxj=inv[gj], ni=Z[inv[gi]], nj=Z[inv[gj]],
        xij=d / dist[:, None], rij=dist / A0, mask=m_p * molsize**2 + i_p * molsize + j_p,
        pair_molid=m_p, species=species, coords=coords, uhf=mult is not None,
    )


def atom_params(method, Z, learned=None):
    """Per-atom parameter gather (basics.py:406-448, parameters.py:4-46)."""
    fields, rows = load_params(method)
    p = {f: rows[Z, k].copy() for k, f in enumerate(fields)}
    if learned:
        for k, v in learned.items():
            p[k] = np.asarray(v, dtype=np.float64).copy()
    return p


# ------------------------------------------------------------ multipole parameters
def multipole_params(Z, p, el):
    """dd, qq, rho0, rho1, rho2 per atom.

    seqm/seqm_functions/cal_par.py:11-28 (dd_qq), :106-189 (rho1 secant),
    :192-280 (rho2 secant); assembled as in two_elec_two_center_int.py:118-245.
    """
    qn = el["qn"][Z]
    isX = Z > 2
    dd = np.zeros(Z.size)
    qq = np.zeros(Z.size)
    zs, zp = p["zeta_s"][isX], p["zeta_p"][isX]
    q = qn[isX]
    dd[isX] = (2.0 * q + 1.0) * (4.0 * zs * zp) ** (q + 0.5) / (zs + zp) ** (2.0 * q + 2.0) / np.sqrt(3.0)
    qq[isX] = np.sqrt((4.0 * q**2 + 6.0 * q + 2.0) / 20.0) / zp
    hpp = np.maximum(0.5 * (p["g_pp"] - p["g_p2"]), 0.1)
    with np.errstate(divide="ignore"):
        rho0 = 0.5 * EV / p["g_ss"]
    rho1 = np.zeros(Z.size)
    rho2 = np.zeros(Z.size)
    if np.any(isX):
        rho1[isX] = _rho1(p["h_sp"][isX], dd[isX])
        rho2[isX] = _rho2(hpp[isX], qq[isX])
    return dd, qq, rho0, rho1, rho2


def _rho1(hsp_ev, D1):
    """cal_par.py:122-172: five secant steps on hsp(d) = d/2 - 1/(2 sqrt(4 D1^2 + 1/d^2))."""
    hsp = hsp_ev / EV
    d1 = (np.abs(hsp) / D1**2) ** (1.0 / 3.0)
    d1 = np.where(hsp < 0.0, -d1, d1)
    d2 = d1 + 0.04
    for _ in range(5):
        h1 = 0.5 * d1 - 0.5 / np.sqrt(4.0 * D1**2 + 1.0 / d1**2)
        h2 = 0.5 * d2 - 0.5 / np.sqrt(4.0 * D1**2 + 1.0 / d2**2)
        with np.errstate(divide="ignore", invalid="ignore"):
            d3 = np.where(np.abs(h2 - h1) > 1.0e-16, d1 + (d2 - d1) * (hsp - h1) / (h2 - h1), d2)
        d1, d2 = d2, d3
    return 0.5 / d2


def _rho2(hpp_ev, D2):
    """cal_par.py:207-245: five secant steps on hpp(q)."""
    hpp = hpp_ev / EV
    q1 = (np.abs(hpp) / 3.0 / D2**4) ** 0.2
    q1 = np.where(hpp < 0.0, -q1, q1)
    q2 = q1 + 0.04

    def f(q):
        return 0.25 * q - 0.5 / np.sqrt(4.0 * D2**2 + 1.0 / q**2) + 0.25 / np.sqrt(8.0 * D2**2 + 1.0 / q**2)

    for _ in range(5):
        h1, h2 = f(q1), f(q2)
        with np.errstate(divide="ignore", invalid="ignore"):
            q3 = np.where(np.abs(h2 - h1) > 1.0e-16, q1 + (q2 - q1) * (hpp - h1) / (h2 - h1), q2)
        q1, q2 = q2, q3
    return 0.5 / q2


# ------------------------------------------------------------ local-frame integrals
def local_integrals(r, da, db, qa0, qb0, rho0a, rho0b, rho1a, rho1b, rho2a, rho2b, kind):
    """Multipole two-centre integrals in the local (pair-axis) frame.

    Restates seqm/seqm_functions/two_elec_two_center_int_local_frame.py:18-293
    (MOPAC repp).  kind: "HH" -> (n,1); "XH" -> (n,4); "XX" -> (n,22).
    """
    ev1, ev2, ev3, ev4 = EV / 2.0, EV / 4.0, EV / 8.0, EV / 16.0
    s = np.sqrt
    if kind == "HH":
        return (EV / s(r**2 + (rho0a + rho0b) ** 2))[:, None]
    if kind == "XH":
        aee = (rho0a + rho0b) ** 2
        qa = qa0 * 2.0
        ade = (rho1a + rho0b) ** 2
        aqe = (rho2a + rho0b) ** 2
        e6 = ev1 / s(r**2 + aqe)
        ee = EV / s(r**2 + aee)
        ri = np.empty((r.size, 4))
        ri[:, 0] = ee
        ri[:, 1] = ev1 / s((r + da) ** 2 + ade) - ev1 / s((r - da) ** 2 + ade)
        ri[:, 2] = ee + ev2 / s((r + qa) ** 2 + aqe) + ev2 / s((r - qa) ** 2 + aqe) - e6
        ri[:, 3] = ee + ev1 / s(r**2 + qa**2 + aqe) - e6
        return ri
    qa, qb = qa0 * 2.0, qb0 * 2.0
    qa1, qb1 = qa0, qb0
    aee = (rho0a + rho0b) ** 2
    ade = (rho1a + rho0b) ** 2
    aqe = (rho2a + rho0b) ** 2
    aed = (rho0a + rho1b) ** 2
    aeq = (rho0a + rho2b) ** 2
    axx = (rho1a + rho1b) ** 2
    adq = (rho1a + rho2b) ** 2
    aqd = (rho2a + rho1b) ** 2
    aqq = (rho2a + rho2b) ** 2
    ee = EV / s(r**2 + aee)
    dze = -ev1 / s((r + da) ** 2 + ade) + ev1 / s((r - da) ** 2 + ade)
    e6 = ev1 / s(r**2 + aqe)
    qzze = ev2 / s((r - qa) ** 2 + aqe) + ev2 / s((r + qa) ** 2 + aqe) - e6
    qxxe = ev1 / s(r**2 + qa**2 + aqe) - e6
    edz = -ev1 / s((r - db) ** 2 + aed) + ev1 / s((r + db) ** 2 + aed)
    e12 = ev1 / s(r**2 + aeq)
    eqzz = ev2 / s((r - qb) ** 2 + aeq) + ev2 / s((r + qb) ** 2 + aeq) - e12
    eqxx = ev1 / s(r**2 + qb**2 + aeq) - e12
    e20 = ev2 / s((r + da) ** 2 + adq)
    e22 = ev2 / s((r - da) ** 2 + adq)
    e24 = ev2 / s((r - db) ** 2 + aqd)
    e26 = ev2 / s((r + db) ** 2 + aqd)
    e36 = ev2 / s(r**2 + aqq)
    e39 = ev2 / s(r**2 + qa**2 + aqq)
    e40 = ev2 / s(r**2 + qb**2 + aqq)
    e42 = ev3 / s((r - qb) ** 2 + aqq)
    e44 = ev3 / s((r + qb) ** 2 + aqq)
    e46 = ev3 / s((r + qa) ** 2 + aqq)
    e48 = ev3 / s((r - qa) ** 2 + aqq)
    ri = np.empty((r.size, 22))
    ri[:, 0] = ee
    ri[:, 1] = -dze
    ri[:, 2] = ee + qzze
    ri[:, 3] = ee + qxxe
    ri[:, 4] = -edz
    ri[:, 5] = (ev2 / s((r + da - db) ** 2 + axx) + ev2 / s((r - da + db) ** 2 + axx)
                - ev2 / s((r - da - db) ** 2 + axx) - ev2 / s((r + da + db) ** 2 + axx))
    ri[:, 6] = ev1 / s(r**2 + (da - db) ** 2 + axx) - ev1 / s(r**2 + (da + db) ** 2 + axx)
    ri[:, 7] = (-edz + ev3 / s((r + qa - db) ** 2 + aqd) - ev3 / s((r + qa + db) ** 2 + aqd)
                + ev3 / s((r - qa - db) ** 2 + aqd) - ev3 / s((r - qa + db) ** 2 + aqd) - e24 + e26)
    ri[:, 8] = (-edz - e24 + ev2 / s((r - db) ** 2 + qa**2 + aqd) + e26
                - ev2 / s((r + db) ** 2 + qa**2 + aqd))
    ri[:, 9] = (ev2 / s((qa1 - db) ** 2 + (r + qa1) ** 2 + aqd) - ev2 / s((qa1 - db) ** 2 + (r - qa1) ** 2 + aqd)
                - ev2 / s((qa1 + db) ** 2 + (r + qa1) ** 2 + aqd)
                + ev2 / s((qa1 + db) ** 2 + (r - qa1) ** 2 + aqd))
    ri[:, 10] = ee + eqzz
    ri[:, 11] = ee + eqxx
    ri[:, 12] = (-dze + ev3 / s((r + da - qb) ** 2 + adq) - ev3 / s((r - da - qb) ** 2 + adq)
                 + ev3 / s((r + da + qb) ** 2 + adq) - ev3 / s((r - da + qb) ** 2 + adq) + e22 - e20)
    ri[:, 13] = (-dze - e20 + ev2 / s((r + da) ** 2 + qb**2 + adq) + e22
                 - ev2 / s((r - da) ** 2 + qb**2 + adq))
    ri[:, 14] = (ev2 / s((da - qb1) ** 2 + (r - qb1) ** 2 + adq) - ev2 / s((da - qb1) ** 2 + (r + qb1) ** 2 + adq)
                 - ev2 / s((da + qb1) ** 2 + (r - qb1) ** 2 + adq)
                 + ev2 / s((da + qb1) ** 2 + (r + qb1) ** 2 + adq))
    ri[:, 15] = (ee + eqzz + qzze + ev4 / s((r + qa - qb) ** 2 + aqq) + ev4 / s((r + qa + qb) ** 2 + aqq)
                 + ev4 / s((r - qa - qb) ** 2 + aqq) + ev4 / s((r - qa + qb) ** 2 + aqq)
                 - e48 - e46 - e42 - e44 + e36)
    ri[:, 16] = (ee + eqzz + qxxe + ev3 / s((r - qb) ** 2 + qa**2 + aqq) + ev3 / s((r + qb) ** 2 + qa**2 + aqq)
                 - e42 - e44 - e39 + e36)
    ri[:, 17] = (ee + eqxx + qzze + ev3 / s((r + qa) ** 2 + qb**2 + aqq) + ev3 / s((r - qa) ** 2 + qb**2 + aqq)
                 - e46 - e48 - e40 + e36)
    qxxqxx = ev3 / s(r**2 + (qa - qb) ** 2 + aqq) + ev3 / s(r**2 + (qa + qb) ** 2 + aqq) - e39 - e40 + e36
    ri[:, 18] = ee + eqxx + qxxe + qxxqxx
    ri[:, 19] = (ev3 / s((r + qa1 - qb1) ** 2 + (qa1 - qb1) ** 2 + aqq)
                 - ev3 / s((r + qa1 + qb1) ** 2 + (qa1 - qb1) ** 2 + aqq)
                 - ev3 / s((r - qa1 - qb1) ** 2 + (qa1 - qb1) ** 2 + aqq)
                 + ev3 / s((r - qa1 + qb1) ** 2 + (qa1 - qb1) ** 2 + aqq)
                 - ev3 / s((r + qa1 - qb1) ** 2 + (qa1 + qb1) ** 2 + aqq)
                 + ev3 / s((r + qa1 + qb1) ** 2 + (qa1 + qb1) ** 2 + aqq)
                 + ev3 / s((r - qa1 - qb1) ** 2 + (qa1 + qb1) ** 2 + aqq)
                 - ev3 / s((r - qa1 + qb1) ** 2 + (qa1 + qb1) ** 2 + aqq))
    qxxqyy = ev2 / s(r**2 + qa**2 + qb**2 + aqq) - e39 - e40 + e36
    ri[:, 20] = ee + eqxx + qxxe + qxxqyy
    ri[:, 21] = 0.5 * (qxxqxx - qxxqyy)
    return ri


# ------------------------------------------------------------------- rotation
def quat_rotation(v):
    """3x3 rotation taking unit vector v onto +x, via a quaternion.

    Restates two_elec_two_center_int.py:1576-1631 (antipodal case |1+v_x|<1e-7
    uses a 180-degree turn about z).
    """
    n = v.shape[0]
    q = np.zeros((n, 4))
    q[:, 1] = v[:, 2]
    q[:, 2] = -v[:, 1]
    q[:, 3] = 1.0 + v[:, 0]
    anti = np.abs(q[:, 3]) < 1.0e-7
    q[anti] = np.array([0.0, 0.0, 1.0, 0.0])
    q = q / np.linalg.norm(q, axis=1, keepdims=True)
    qy, qz, qw = q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz)
    R[:, 0, 1] = -2 * (qz * qw)
    R[:, 0, 2] = 2 * (qy * qw)
    R[:, 1, 0] = 2 * (qz * qw)
    R[:, 1, 1] = 1 - 2 * (qz * qz)
    R[:, 1, 2] = 2 * (qy * qz)
    R[:, 2, 0] = -2 * (qy * qw)
    R[:, 2, 1] = 2 * (qy * qz)
    R[:, 2, 2] = 1 - 2 * (qy * qy)
    return R


def rotate_w(xij, riHH, riXH, riXX, cls):
    """Molecular-frame (10,10) integral blocks per pair.

    Restates two_elec_two_center_int.py:1384-1500 (w_withquaternion) and the
    assembly :1301-1306 (HH -> [0,0], XH -> [:,0], XX -> all).
    """
    npairs = xij.shape[0]
    w = np.zeros((npairs, 10, 10))
    R = quat_rotation(-xij)
    hh, xh, xx = cls == 0, cls == 1, cls == 2
    w[hh, 0, 0] = riHH[:, 0]
    # index (kk,ll) of the 10-list -> (orbital k, orbital l), 0 = s, 1..3 = p
    combos = [(k, l) for k in range(4) for l in range(k + 1)]
    if np.any(xh):
        rx = R[xh]
        for a, (kk, ll) in enumerate(combos):
            if kk == 0:
                val = riXH[:, 0]
            elif ll == 0:
                val = riXH[:, 1] * rx[:, 0, kk - 1]
            else:
                k, l = kk - 1, ll - 1
                val = riXH[:, 2] * rx[:, 0, k] * rx[:, 0, l] + riXH[:, 3] * (
                    rx[:, 1, k] * rx[:, 1, l] + rx[:, 2, k] * rx[:, 2, l])
            w[np.nonzero(xh)[0], a, 0] = val
    if np.any(xx):
        r = R[xx]
        ri = riXX
        r0, r1, r2 = r[:, 0], r[:, 1], r[:, 2]
        blk = np.zeros((r.shape[0], 10, 10))
        for a, (kk, ll) in enumerate(combos):
            for b, (mm, nn) in enumerate(combos):
                k, l, m, n = kk - 1, ll - 1, mm - 1, nn - 1
                if kk == 0:
                    if mm == 0:
                        val = ri[:, 0]
                    elif nn == 0:
                        val = ri[:, 4] * r0[:, m]
                    else:
                        val = ri[:, 10] * (r0[:, m] * r0[:, n]) + ri[:, 11] * (
                            r1[:, m] * r1[:, n] + r2[:, m] * r2[:, n])
                elif ll == 0:
                    if mm == 0:
                        val = ri[:, 1] * r0[:, k]
                    elif nn == 0:
                        val = ri[:, 5] * (r0[:, k] * r0[:, m]) + ri[:, 6] * (
                            r1[:, k] * r1[:, m] + r2[:, k] * r2[:, m])
                    else:
                        t0 = r0[:, k] * r0[:, m] * r0[:, n]
                        t1 = (r1[:, m] * r1[:, n] + r2[:, m] * r2[:, n]) * r0[:, k]
                        mix = (r1[:, k] * (r1[:, n] * r0[:, m] + r1[:, m] * r0[:, n])
                               + r2[:, k] * (r2[:, m] * r0[:, n] + r2[:, n] * r0[:, m]))
                        val = ri[:, 12] * t0 + ri[:, 13] * t1 + ri[:, 14] * mix
                else:
                    if mm == 0:
                        val = ri[:, 2] * (r0[:, k] * r0[:, l]) + ri[:, 3] * (
                            r1[:, k] * r1[:, l] + r2[:, k] * r2[:, l])
                    elif nn == 0:
                        t0 = r0[:, k] * r0[:, l] * r0[:, m]
                        t1 = (r1[:, k] * r1[:, l] + r2[:, k] * r2[:, l]) * r0[:, m]
                        t2 = r1[:, l] * r1[:, m] + r2[:, l] * r2[:, m]
                        val = ri[:, 7] * t0 + ri[:, 8] * t1 + ri[:, 9] * (
                            r0[:, k] * t2 + r0[:, l] * (r1[:, k] * r1[:, m] + r2[:, k] * r2[:, m]))
                    else:
                        val = ri[:, 15] * (r0[:, k] * r0[:, l] * r0[:, m] * r0[:, n])
                        val = val + ri[:, 16] * ((r1[:, k] * r1[:, l] + r2[:, k] * r2[:, l]) * r0[:, m] * r0[:, n])
                        val = val + ri[:, 17] * ((r1[:, m] * r1[:, n] + r2[:, m] * r2[:, n]) * (r0[:, k] * r0[:, l]))
                        val = val + ri[:, 18] * (r1[:, k] * r1[:, l] * r1[:, m] * r1[:, n]
                                                 + r2[:, k] * r2[:, l] * r2[:, m] * r2[:, n])
                        mix1 = r0[:, m] * (r1[:, l] * r1[:, n] + r2[:, l] * r2[:, n])
                        mix2 = r0[:, n] * (r1[:, l] * r1[:, m] + r2[:, l] * r2[:, m])
                        val5 = r0[:, k] * (mix1 + mix2) + r0[:, l] * (
                            r0[:, m] * (r1[:, k] * r1[:, n] + r2[:, k] * r2[:, n])
                            + r0[:, n] * (r1[:, k] * r1[:, m] + r2[:, k] * r2[:, m]))
                        val = val + ri[:, 19] * val5
                        val = val + ri[:, 20] * (r1[:, k] * r1[:, l] * r2[:, m] * r2[:, n]
                                                 + r2[:, k] * r2[:, l] * r1[:, m] * r1[:, n])
                        val = val + ri[:, 21] * ((r1[:, k] * r2[:, l] + r2[:, k] * r1[:, l])
                                                 * (r1[:, m] * r2[:, n] + r2[:, m] * r1[:, n]))
                blk[:, a, b] = val
        w[xx] = blk
    return w


# -------------------------------------------------------------------- overlap
def _aint(x, kmax=7):
    """A_k auxiliary integrals (diat_overlap_PM6_SP.py:464-519)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        xs = np.where(x != 0, x, np.inf)
        a = np.empty((x.size, kmax))
        a[:, 0] = np.exp(-xs) / xs
        a[:, 1] = a[:, 0] + a[:, 0] / xs
        for k in range(2, kmax):
            a[:, k] = a[:, 0] + k * a[:, k - 1] / xs
    return a


def _bint(x, kmax=7):
    """B_k auxiliary integrals (diat_overlap_PM6_SP.py:522-670)."""
    b = np.zeros((x.size, kmax))
    for k in range(0, kmax, 2):
        b[:, k] = 2.0 / (k + 1)
    ax = np.abs(x)
    c1 = ax > 0.5
    if np.any(c1):
        xc = x[c1]
        tx = np.exp(xc) / xc
        tmx = -np.exp(-xc) / xc
        bb = np.empty((xc.size, kmax))
        bb[:, 0] = tx + tmx
        for k in range(1, kmax):
            sgn = -1.0 if k % 2 == 1 else 1.0
            bb[:, k] = sgn * tx + tmx + k * bb[:, k - 1] / xc
        b[c1] = bb
    c2 = (ax <= 0.5) & (ax > 1.0e-6)
    if np.any(c2):
        xc = x[c2]
        # even k: sum_{m=0,2,4,6} x^m 2/(m!(m+k+1)); odd k: -sum_{m=1,3,5} x^m 2/(m!(m+k+1))
        even = {0: (2.0, 3.0, 60.0, 2520.0), 2: (2.0 / 3.0, 5.0, 84.0, 3240.0), 4: (2.0 / 5.0, 7.0, 108.0, 3960.0),
                6: (2.0 / 7.0, 9.0, 132.0, 4680.0)}
        odd = {1: (2.0 / 3.0, 15.0, 420.0), 3: (2.0 / 5.0, 21.0, 540.0), 5: (2.0 / 7.0, 27.0, 660.0)}
        bb = b[c2].copy()
        for k, (c0, d2, d4, d6) in even.items():
            if k < kmax:
                bb[:, k] = c0 + xc**2 / d2 + xc**4 / d4 + xc**6 / d6
        for k, (c1_, d3, d5) in odd.items():
            if k < kmax:
                bb[:, k] = -c1_ * xc - xc**3 / d3 - xc**5 / d5
        b[c2] = bb
    return b


def _set(r, za, zb):
    return _aint(0.5 * r * (za + zb)), _bint(0.5 * r * (za - zb))


def overlap_local(qni, qnj, r, zsa, zpa, zsb, zpb):
    """Local-frame overlaps S111, S211, S121, S221, S222 per pair.

    Restates diat_overlap_PM6_SP.py:56-312 (jcall classes 2,3,4,431,5,6).
    """
    n = r.size
    S = {k: np.zeros(n) for k in ("111", "211", "121", "221", "222")}
    jc = np.zeros(n, dtype=np.int64)
    jc[(qni == 1) & (qnj == 1)] = 2
    jc[(qni == 2) & (qnj == 1)] = 3
    jc[(qni == 2) & (qnj == 2)] = 4
    jc[(qni == 3) & (qnj == 1)] = 431
    jc[(qni == 3) & (qnj == 2)] = 5
    jc[(qni == 3) & (qnj == 3)] = 6
    if np.any(jc == 0):
        raise ValueError("overlap: element pair not supported (principal quantum number > 3)")
    A1, B1 = _set(r, zsa, zsb)
    A21, B21 = _set(r, zpa, zsb)
    A12, B12 = _set(r, zsa, zpb)
    A22, B22 = _set(r, zpa, zpb)
    s3, s10, s30 = np.sqrt(3.0), np.sqrt(10.0), np.sqrt(30.0)

    m = jc == 2
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = (zsa[m] * zsb[m] * r[m] ** 2) ** 1.5 * (A[:, 2] * B[:, 0] - B[:, 2] * A[:, 0]) / 4.0
    m = jc == 3
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = (zsb[m] ** 1.5 * zsa[m] ** 2.5 * r[m] ** 4
                       * (A[:, 3] * B[:, 0] - B[:, 3] * A[:, 0] + A[:, 2] * B[:, 1] - B[:, 2] * A[:, 1]) / (s3 * 8.0))
        A, B = A21[m], B21[m]
        S["211"][m] = (zsb[m] ** 1.5 * zpa[m] ** 2.5 * r[m] ** 4
                       * (A[:, 2] * B[:, 0] - B[:, 2] * A[:, 0] + A[:, 3] * B[:, 1] - B[:, 3] * A[:, 1]) / 8.0)
    m = jc == 4
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = ((zsb[m] * zsa[m]) ** 2.5 * r[m] ** 5
                       * (A[:, 4] * B[:, 0] + B[:, 4] * A[:, 0] - 2.0 * A[:, 2] * B[:, 2]) / 48.0)
        A, B = A21[m], B21[m]
        S["211"][m] = ((zsb[m] * zpa[m]) ** 2.5 * r[m] ** 5
                       * (A[:, 3] * (B[:, 0] - B[:, 2]) - A[:, 1] * (B[:, 2] - B[:, 4])
                          + B[:, 3] * (A[:, 0] - A[:, 2]) - B[:, 1] * (A[:, 2] - A[:, 4])) / (16.0 * s3))
        A, B = A12[m], B12[m]
        S["121"][m] = ((zpb[m] * zsa[m]) ** 2.5 * r[m] ** 5
                       * (A[:, 3] * (B[:, 0] - B[:, 2]) - A[:, 1] * (B[:, 2] - B[:, 4])
                          - B[:, 3] * (A[:, 0] - A[:, 2]) + B[:, 1] * (A[:, 2] - A[:, 4])) / (16.0 * s3))
        A, B = A22[m], B22[m]
        w = (zpb[m] * zpa[m]) ** 2.5 * r[m] ** 5 / 16.0
        S["221"][m] = -w * (B[:, 2] * (A[:, 4] + A[:, 0]) - A[:, 2] * (B[:, 4] + B[:, 0]))
        S["222"][m] = 0.5 * w * (A[:, 4] * (B[:, 0] - B[:, 2]) - B[:, 4] * (A[:, 0] - A[:, 2])
                                 - A[:, 2] * B[:, 0] + B[:, 2] * A[:, 0])
    m = jc == 431
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = (zsb[m] ** 1.5 * zsa[m] ** 3.5 * r[m] ** 5
                       * (A[:, 4] * B[:, 0] + 2 * B[:, 1] * A[:, 3] - 2.0 * A[:, 1] * B[:, 3] - B[:, 4] * A[:, 0])
                       / (s10 * 24.0))
        A, B = A21[m], B21[m]
        S["211"][m] = (zsb[m] ** 1.5 * zpa[m] ** 3.5 * r[m] ** 5
                       * (A[:, 3] * (B[:, 0] + B[:, 2]) - A[:, 1] * (B[:, 4] + B[:, 2])
                          + B[:, 1] * (A[:, 2] + A[:, 4]) - B[:, 3] * (A[:, 2] + A[:, 0])) / (8.0 * s30))
    m = jc == 5
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = (zsb[m] ** 2.5 * zsa[m] ** 3.5 * r[m] ** 6
                       * (A[:, 5] * B[:, 0] + B[:, 1] * A[:, 4] - 2 * B[:, 2] * A[:, 3] - 2.0 * A[:, 2] * B[:, 3]
                          + B[:, 4] * A[:, 1] + B[:, 5] * A[:, 0]) / (s30 * 48.0))
        A, B = A21[m], B21[m]
        S["211"][m] = (zsb[m] ** 2.5 * zpa[m] ** 3.5 * r[m] ** 6
                       * (A[:, 4] * B[:, 0] + B[:, 1] * A[:, 5] - 2.0 * B[:, 3] * A[:, 3] - 2.0 * A[:, 2] * B[:, 2]
                          + A[:, 1] * B[:, 5] + A[:, 0] * B[:, 4]) / (48.0 * s10))
        A, B = A12[m], B12[m]
        S["121"][m] = (zpb[m] ** 2.5 * zsa[m] ** 3.5 * r[m] ** 6
                       * ((A[:, 4] * B[:, 0] - A[:, 5] * B[:, 1]) + 2.0 * (A[:, 3] * B[:, 1] - A[:, 4] * B[:, 2])
                          - 2.0 * (A[:, 1] * B[:, 3] - A[:, 2] * B[:, 4]) - (A[:, 0] * B[:, 4] - A[:, 1] * B[:, 5]))
                       / (48.0 * s10))
        A, B = A22[m], B22[m]
        S["221"][m] = (zpb[m] ** 2.5 * zpa[m] ** 3.5 * r[m] ** 6
                       * ((A[:, 3] * B[:, 0] - A[:, 5] * B[:, 2]) + (A[:, 2] * B[:, 1] - A[:, 4] * B[:, 3])
                          - (A[:, 1] * B[:, 2] - A[:, 3] * B[:, 4]) - (A[:, 0] * B[:, 3] - A[:, 2] * B[:, 5]))
                       / (16.0 * s30))
        S["222"][m] = (zpb[m] ** 2.5 * zpa[m] ** 3.5 * r[m] ** 6
                       * ((A[:, 5] - A[:, 3]) * (B[:, 0] - B[:, 2]) + (A[:, 4] - A[:, 2]) * (B[:, 1] - B[:, 3])
                          - (A[:, 3] - A[:, 1]) * (B[:, 2] - B[:, 4]) - (A[:, 2] - A[:, 0]) * (B[:, 3] - B[:, 5]))
                       / (32.0 * s30))
    m = jc == 6
    if np.any(m):
        A, B = A1[m], B1[m]
        S["111"][m] = ((zsb[m] * zsa[m]) ** 3.5 * r[m] ** 7
                       * (A[:, 6] * B[:, 0] - 3.0 * B[:, 2] * A[:, 4] + 3.0 * A[:, 2] * B[:, 4] - A[:, 0] * B[:, 6])
                       / 1440.0)
        A, B = A21[m], B21[m]
        S["211"][m] = ((zsb[m] * zpa[m]) ** 3.5 * r[m] ** 7
                       * ((A[:, 5] * B[:, 0] + A[:, 6] * B[:, 1]) + (-A[:, 4] * B[:, 1] - A[:, 5] * B[:, 2])
                          - 2.0 * (A[:, 3] * B[:, 2] + A[:, 4] * B[:, 3]) - 2.0 * (-A[:, 2] * B[:, 3] - A[:, 3] * B[:, 4])
                          + (A[:, 1] * B[:, 4] + A[:, 2] * B[:, 5]) + (-A[:, 0] * B[:, 5] - A[:, 1] * B[:, 6]))
                       / (480.0 * s3))
        A, B = A12[m], B12[m]
        S["121"][m] = ((zpb[m] * zsa[m]) ** 3.5 * r[m] ** 7
                       * ((A[:, 5] * B[:, 0] - A[:, 6] * B[:, 1]) + (A[:, 4] * B[:, 1] - A[:, 5] * B[:, 2])
                          - 2.0 * (A[:, 3] * B[:, 2] - A[:, 4] * B[:, 3]) - 2.0 * (A[:, 2] * B[:, 3] - A[:, 3] * B[:, 4])
                          + (A[:, 1] * B[:, 4] - A[:, 2] * B[:, 5]) + (A[:, 0] * B[:, 5] - A[:, 1] * B[:, 6]))
                       / (480.0 * s3))
        A, B = A22[m], B22[m]
        S["221"][m] = (zpb[m] ** 3.5 * zpa[m] ** 3.5 * r[m] ** 7
                       * ((A[:, 4] * B[:, 0] - A[:, 6] * B[:, 2]) - 2.0 * (A[:, 2] * B[:, 2] - A[:, 4] * B[:, 4])
                          + (A[:, 0] * B[:, 4] - A[:, 2] * B[:, 6])) / 480.0)
        S["222"][m] = (zpb[m] ** 3.5 * zpa[m] ** 3.5 * r[m] ** 7
                       * ((A[:, 6] - A[:, 4]) * (B[:, 0] - B[:, 2]) - 2.0 * (A[:, 4] - A[:, 2]) * (B[:, 2] - B[:, 4])
                          + (A[:, 2] - A[:, 0]) * (B[:, 4] - B[:, 6])) / 960.0)
    return S


def overlap(xij, S):
    """4x4 molecular-frame overlap (diat_overlap_PM6_SP.py:376-392)."""
    n = xij.shape[0]
    R = np.transpose(quat_rotation(xij), (0, 2, 1))
    di = np.zeros((n, 4, 4))
    di[:, 0, 0] = S["111"]
    c0 = R[:, :, 0]
    di[:, 1:, 0] = S["211"][:, None] * c0
    di[:, 0, 1:] = -S["121"][:, None] * c0
    Mv = np.stack([-S["221"], S["222"], S["222"]], axis=1)
    di[:, 1:, 1:] = np.einsum("nij,nj,nkj->nik", R, Mv, R)
    return di


# ---------------------------------------------------------------------- hcore
def integrals(mol, p, el):
    """w (npairs,10,10), e1b/e2a (npairs,4,4) and overlap di; two_elec_two_center_int.py:98-283."""
    Z, ni, nj, idxi, idxj = mol["Z"], mol["ni"], mol["nj"], mol["idxi"], mol["idxj"]
    r, xij = mol["rij"], mol["xij"]
    dd, qq, rho0, rho1, rho2 = multipole_params(Z, p, el)
    cls = np.where(nj > 1, 2, np.where(ni > 1, 1, 0))  # 0 HH, 1 XH, 2 XX (pairs are heavy-first)
    hh, xh, xx = cls == 0, cls == 1, cls == 2
    riHH = local_integrals(r[hh], None, None, None, None, rho0[idxi[hh]], rho0[idxj[hh]], None, None, None, None, "HH")
    riXH = local_integrals(r[xh], dd[idxi[xh]], None, qq[idxi[xh]], None, rho0[idxi[xh]], rho0[idxj[xh]],
                           rho1[idxi[xh]], None, rho2[idxi[xh]], None, "XH")
    a, b = idxi[xx], idxj[xx]
    riXX = local_integrals(r[xx], dd[a], dd[b], qq[a], qq[b], rho0[a], rho0[b], rho1[a], rho1[b], rho2[a], rho2[b],
                           "XX")
    w = rotate_w(xij, riHH, riXH, riXX, cls)
    tore = el["tore"]
    e1b = np.zeros((r.size, 4, 4))
    e2a = np.zeros((r.size, 4, 4))
    # two_elec_two_center_int.py:1535-1572: core attraction from w's first column / row
    for k in range(10):
        e1b[:, K10_ROW[k], K10_COL[k]] = -tore[nj] * w[:, k, 0]
    e2a[:, 0, 0] = -tore[ni] * w[:, 0, 0]
    for k in range(1, 10):
        e2a[xx, K10_ROW[k], K10_COL[k]] = -tore[ni[xx]] * w[xx, 0, k]
    # overlap, only within the cutoff (hcore.py:80-92)
    qn = el["qn"].astype(np.int64)
    di = np.zeros((r.size, 4, 4))
    near = r <= OVERLAP_CUTOFF
    if np.any(near):
        S = overlap_local(qn[ni[near]], qn[nj[near]], r[near], p["zeta_s"][idxi[near]], p["zeta_p"][idxi[near]],
                          p["zeta_s"][idxj[near]], p["zeta_p"][idxj[near]])
        di[near] = overlap(xij[near], S)
    return dict(w=w, e1b=e1b, e2a=e2a, di=di, rho0=rho0, cls=cls)


def hcore(mol, p, ints):
    """Block-packed M (nmol*molsize^2, 4, 4), upper triangle only; hcore.py:127-179."""
    nblk = mol["nmol"] * mol["molsize"] ** 2
    M = np.zeros((nblk, 4, 4))
    maskd = mol["maskd"]
    M[maskd, 0, 0] = p["U_ss"]
    for k in (1, 2, 3):
        M[maskd, k, k] = p["U_pp"]
    np.add.at(M, maskd[mol["idxi"]], ints["e1b"])
    np.add.at(M, maskd[mol["idxj"]], ints["e2a"])
    beta = np.stack([p["beta_s"], p["beta_p"], p["beta_p"], p["beta_p"]], axis=1)
    bsum = 0.5 * (beta[mol["idxi"]][:, :, None] + beta[mol["idxj"]][:, None, :])
    M[mol["mask"]] = ints["di"] * bsum
    return M


def blocks_to_full(M, nmol, molsize):
    """(nmol*ms^2,4,4) blocks -> (nmol,4ms,4ms); scf_loop.py:150-160."""
    return M.reshape(nmol, molsize, molsize, 4, 4).transpose(0, 1, 3, 2, 4).reshape(nmol, 4 * molsize, 4 * molsize)


def full_to_blocks(P, nmol, molsize):
    return P.reshape(nmol, molsize, 4, molsize, 4).transpose(0, 1, 3, 2, 4).reshape(-1, 4, 4)


def symmetrize_upper(H):
    """h = triu(H) + triu(H,1)^T  (energy.py:39-40)."""
    return np.triu(H) + np.transpose(np.triu(H, 1), (0, 2, 1))


# ----------------------------------------------------------------------- fock
def fock(mol, p, ints, M, P):
    """Restricted Fock matrix, fock.py:132-181 (_one_center :187-231, _two_center :259-347)."""
    nmol, ms = mol["nmol"], mol["molsize"]
    Pb = full_to_blocks(P, nmol, ms)
    F = M.copy()
    maskd = mol["maskd"]
    Pd = Pb[maskd]
    Pss = Pd[:, 0, 0]
    Ppt = Pd[:, 1, 1] + Pd[:, 2, 2] + Pd[:, 3, 3]
    gss, gsp, gpp, gp2, hsp = p["g_ss"], p["g_sp"], p["g_pp"], p["g_p2"], p["h_sp"]
    f1 = gsp - 0.5 * hsp
    f2 = 1.5 * hsp - 0.5 * gsp
    f3 = 1.25 * gp2 - 0.25 * gpp
    f4 = 0.75 * gpp - 1.25 * gp2
    t = np.zeros_like(Pd)
    t[:, 0, 0] = 0.5 * Pss * gss + Ppt * f1
    for i in (1, 2, 3):
        t[:, i, i] = Pss * f1 + 0.5 * Pd[:, i, i] * gpp + (Ppt - Pd[:, i, i]) * f3
        t[:, 0, i] = Pd[:, 0, i] * f2
    for i, j in ((1, 2), (1, 3), (2, 3)):
        t[:, i, j] = Pd[:, i, j] * f4
    F[maskd] += t
    w = ints["w"]
    idxi, idxj, mask = mol["idxi"], mol["idxj"], mol["mask"]
    PA = Pb[maskd[idxi]][:, K10_COL, K10_ROW] * K10_WEIGHT
    PB = Pb[maskd[idxj]][:, K10_COL, K10_ROW] * K10_WEIGHT
    JA = np.einsum("nk,nkl->nl", PA, w)  # goes to atom j
    JB = np.einsum("nkl,nl->nk", w, PB)  # goes to atom i
    sumA = np.zeros((w.shape[0], 4, 4))
    sumB = np.zeros((w.shape[0], 4, 4))
    sumA[:, K10_ROW, K10_COL] = JA
    sumB[:, K10_ROW, K10_COL] = JB
    np.add.at(F, maskd[idxi], sumB)
    np.add.at(F, maskd[idxj], sumA)
    Pp = -0.5 * Pb[mask]
    # K[mu,nu] = sum_{lam,sig} w[kind(mu,lam), kind(nu,sig)] * Pp[lam,sig]
    wk = w[:, KIND[:, :, None, None], KIND[None, None, :, :]]  # (n, mu, lam, nu, sig)
    K = np.einsum("nalbs,nls->nab", wk, Pp)
    np.add.at(F, mask, K)
    Ff = blocks_to_full(F, nmol, ms)
    return Ff + np.transpose(np.triu(Ff, 1), (0, 2, 1))


def fock_u(mol, p, ints, M, P2):
    """Unrestricted Fock matrices F[:, s] of the spin densities P2[:, s] (fock_u_batch.py:18-100):
    Coulomb from the total density, exchange from the spin density, one-centre terms
    spin-resolved (_one_center_u, :103-146)."""
    nmol, ms = mol["nmol"], mol["molsize"]
    Pt = full_to_blocks(P2[:, 0] + P2[:, 1], nmol, ms)
    Ps = [full_to_blocks(P2[:, s], nmol, ms) for s in range(2)]
    maskd = mol["maskd"]
    gss, gsp, gpp, gp2, hsp = p["g_ss"], p["g_sp"], p["g_pp"], p["g_p2"], p["h_sp"]
    Td = Pt[maskd]
    Ptp = Td[:, 1, 1] + Td[:, 2, 2] + Td[:, 3, 3]
    Fs = []
    for s in range(2):
        Sd, Od = Ps[s][maskd], Ps[1 - s][maskd]
        Spt = Sd[:, 1, 1] + Sd[:, 2, 2] + Sd[:, 3, 3]
        t = np.zeros_like(Td)
        t[:, 0, 0] = Od[:, 0, 0] * gss + Ptp * gsp - Spt * hsp
        for i in (1, 2, 3):
            t[:, i, i] = (Td[:, 0, 0] * gsp - Sd[:, 0, 0] * hsp + Od[:, i, i] * gpp + (Ptp - Td[:, i, i]) * gp2
                          - 0.5 * (Spt - Sd[:, i, i]) * (gpp - gp2))
            t[:, 0, i] = 2.0 * Td[:, 0, i] * hsp - Sd[:, 0, i] * (hsp + gsp)
        for i, j in ((1, 2), (1, 3), (2, 3)):
            t[:, i, j] = Td[:, i, j] * (gpp - gp2) - 0.5 * Sd[:, i, j] * (gpp + gp2)
        F = M.copy()
        F[maskd] += t
        Fs.append(F)
    w = ints["w"]
    idxi, idxj, mask = mol["idxi"], mol["idxj"], mol["mask"]
    PA = Pt[maskd[idxi]][:, K10_COL, K10_ROW] * K10_WEIGHT
    PB = Pt[maskd[idxj]][:, K10_COL, K10_ROW] * K10_WEIGHT
    sumA = np.zeros((w.shape[0], 4, 4))
    sumB = np.zeros((w.shape[0], 4, 4))
    sumA[:, K10_ROW, K10_COL] = np.einsum("nk,nkl->nl", PA, w)
    sumB[:, K10_ROW, K10_COL] = np.einsum("nkl,nl->nk", w, PB)
    wk = w[:, KIND[:, :, None, None], KIND[None, None, :, :]]
    out = np.zeros((nmol, 2, 4 * ms, 4 * ms))
    for s in range(2):
        F = Fs[s]
        np.add.at(F, maskd[idxi], sumB)
        np.add.at(F, maskd[idxj], sumA)
        np.add.at(F, mask, np.einsum("nalbs,nls->nab", wk, -Ps[s][mask]))
        Ff = blocks_to_full(F, nmol, ms)
        out[:, s] = Ff + np.transpose(np.triu(Ff, 1), (0, 2, 1))
    return out


def elec_energy(P, F, Hsym):
    """Eelec = 1/2 sum P*(H+F)  (energy.py:26-49); unrestricted (P, F of shape (nmol, 2, n, n)):
    1/2 sum [(Pa + Pb) H + Pa Fa + Pb Fb] (energy.py:44-45)."""
    if P.ndim == 4:
        return 0.5 * np.sum((P[:, 0] + P[:, 1]) * Hsym + P[:, 0] * F[:, 0] + P[:, 1] * F[:, 1], axis=(1, 2))
    return 0.5 * np.sum(P * (Hsym + F), axis=(1, 2))


# --------------------------------------------------------------- density step
def packed_index(nheavy, nhyd):
    """AO indices of the packed (no H p-slots) basis inside the padded basis (pack.py:8-17)."""
    nho = 4 * nheavy
    return np.concatenate([np.arange(nho), nho + 4 * np.arange(nhyd)]).astype(np.int64)


def density_eigh(F, nheavy, nhyd, nocc):
    """P = 2 C_occ C_occ^T per molecule after eigh of the packed F (diag.py:110-241)."""
    nmol, n4, _ = F.shape
    P = np.zeros_like(F)
    e = np.zeros((nmol, n4))
    vecs = []
    for m in range(nmol):
        idx = packed_index(nheavy[m], nhyd[m])
        f = F[m][np.ix_(idx, idx)]
        ev, C = np.linalg.eigh(f, UPLO="U")
        c = C[:, : nocc[m]]
        P[m][np.ix_(idx, idx)] = 2.0 * (c @ c.T)
        e[m, : idx.size] = ev
        vecs.append(C)
    return P, e, vecs


def sp2(f, nocc, eps, factor=2.0):
    """SP2 purification of one packed Fock matrix (SP2.py:9-85, float64 branch)."""
    eps = min(max(eps, 1.0e-7), 1.0e-3)
    n = f.shape[0]
    aii = np.diag(f)
    ri = np.sum(np.abs(f), axis=1) - np.abs(aii)
    h1 = np.min(aii - ri)
    hN = np.max(aii + ri)
    a0 = (np.eye(n) * hN - f) / (hN - h1)
    err0 = abs(np.trace(a0) - nocc)
    err1 = err0
    while True:
        a2 = a0 @ a0
        tr2 = np.trace(a2)
        if abs(tr2 - nocc) < abs(2.0 * np.trace(a0) - tr2 - nocc):
            a0 = a2
        else:
            a0 = 2.0 * a0 - a2
        err1, err0 = err0, abs(np.trace(a0) - nocc)
        if err0 < eps and err1 < eps:
            break
    return factor * a0


def density_sp2(F, nheavy, nhyd, nocc, eps):
    nmol = F.shape[0]
    P = np.zeros_like(F)
    for m in range(nmol):
        idx = packed_index(nheavy[m], nhyd[m])
        P[m][np.ix_(idx, idx)] = sp2(F[m][np.ix_(idx, idx)], nocc[m], eps)
    return P


# --------------------------------------------------------------------- mixing
def adaptive_mix(k, Pprev, Pcur, old2_diag, occ=2.0):
    """MOPAC-style mixing for one molecule (scf_loop.py:360-420, 350-358); occ is the orbital
    occupation (2 restricted, 1 per spin unrestricted)."""
    dprev = np.diag(Pprev).copy()
    dcur = np.diag(Pcur).copy()
    damp = 0.05 if k > 4 else 1.0e10
    if k % 3 == 0:
        d1 = dcur - dprev
        d2 = dcur - 2.0 * dprev + old2_diag
        num, den = np.sum(d1 * d1), np.sum(d2 * d2)
        fac = math.sqrt(num / den) if (den > 0 and num < 100.0 * den) else 0.0
        Pmix = (1.0 + fac) * Pcur - fac * Pprev
    else:
        fac = 0.0
        Pmix = Pcur.copy()
    delta = dcur - dprev
    cap = np.abs(delta) > damp
    di = np.where(cap, dprev + np.sign(delta) * damp, dcur + fac * delta)
    di = np.clip(di, 0.0, occ)
    sum0 = np.sum(dcur)
    for _ in range(20):
        sum2 = np.sum(di)
        sum3 = sum0 / sum2 if sum2 > 1.0e-3 else 0.0
        if sum2 <= 1.0e-3 or abs(sum3 - 1.0) <= 1.0e-5:
            break
        scaled = np.maximum(di * sum3, 0.0)
        full = scaled > occ
        di = np.where(full, occ, scaled)
        sum0 = sum0 - np.sum(full) * occ
    np.fill_diagonal(Pmix, di)
    return Pmix, dprev


# ------------------------------------------------------------------------ SCF
def initial_density(mol, el):
    """Diagonal guess: tore/4 on heavy-atom s,p; 1 on H s (scf_loop.py:2066-2081)."""
    nmol, ms = mol["nmol"], mol["molsize"]
    P0 = np.zeros((nmol * ms * ms, 4, 4))
    Z, maskd = mol["Z"], mol["maskd"]
    heavy = Z > 1
    for k in range(4):
        P0[maskd[heavy], k, k] = el["tore"][Z[heavy]] / 4.0
    P0[maskd[Z == 1], 0, 0] = 1.0
    return blocks_to_full(P0, nmol, ms)


def scf(mol, p, ints, M, eps, converger=(1,), sp2_opt=(False,), P0=None, el=None):
    """SCF driver: scf_forward0 (linear mixing, scf_loop.py:150-347) or
    scf_forward1 (adaptive mixing, :424-635), with get_error (:106-147)."""
    el = el or load_elements()
    if mol.get("uhf"):
        return _scf_uhf(mol, p, ints, M, eps, converger, P0, el)
    nmol, ms = mol["nmol"], mol["molsize"]
    Hsym = symmetrize_upper(blocks_to_full(M, nmol, ms))
    P = initial_density(mol, el) if P0 is None else np.array(P0, dtype=np.float64)
    nheavy, nhyd, nocc = mol["nheavy"], mol["nhyd"], mol["nocc"]
    natoms4 = 9.0 * mol["nsuper"] + 4.0 * (nheavy + nhyd)

    def density(F, sel):
        if sp2_opt[0]:
            return density_sp2(F[sel], nheavy[sel], nhyd[sel], nocc[sel], sp2_opt[1])
        return density_eigh(F[sel], nheavy[sel], nhyd[sel], nocc[sel])[0]

    F = fock(mol, p, ints, M, P)
    E = elec_energy(P, F, Hsym)
    Enew = np.zeros(nmol)
    err = np.ones(nmol)
    dm_err = np.ones(nmol)
    dm_el = np.ones(nmol)
    nc = np.ones(nmol, dtype=bool)
    iters = np.zeros(nmol, dtype=np.int64)
    old2 = np.zeros((nmol, 4 * ms))
    Pold = np.zeros_like(P)
    if converger[0] == 2:
        return _scf_diis(mol, p, ints, M, eps, P, F, E, Hsym, density, natoms4)
    linear = converger[0] == 0
    alpha = converger[1] if linear else None
    kstart = 0 if linear else 1
    for k in range(kstart, MAX_ITER + 1):
        sel = np.nonzero(nc)[0]
        Pnew = density(F, sel)
        for a, m in enumerate(sel):
            Pold[m] = P[m]
            if linear:
                P[m] = alpha * P[m] + (1.0 - alpha) * Pnew[a]
            else:
                P[m], old2[m] = adaptive_mix(k, Pold[m], Pnew[a], old2[m])
        iters[sel] += 1
        F = fock(mol, p, ints, M, P)
        Enew[sel] = elec_energy(P[sel], F[sel], Hsym[sel])
        err[sel] = Enew[sel] - E[sel]
        bad = np.abs(err) > eps
        dmm = nc & ~bad
        if np.any(dmm):
            dP = P[dmm] - Pold[dmm]
            dm_err[dmm] = np.sqrt(np.sum(dP * dP, axis=(1, 2))) / natoms4[dmm]
            dm_el[dmm] = np.max(np.abs(dP), axis=(1, 2))
        nc = bad | (dm_err > eps * DM_ERR_FACTOR) | (dm_el > eps * DM_ELEM_FACTOR)
        E[nc] = Enew[nc]
        if not np.any(nc):
            break
    return P, nc, iters


def _scf_uhf(mol, p, ints, M, eps, converger, P0, el):
    """Unrestricted SCF (scf_forward0 / scf_forward1 with unrestricted=True): each spin density
    starts at half the restricted guess (scf_loop.py:2083-2085), comes from its own eigenproblem
    with occupation 1 (Pnew / 2, :259-260 and :515-516) and is mixed on its own (occupation 1,
    :361-420); F from fock_u, the energy of both spins, and the error test on the spin-summed
    density change (:136-140)."""
    nmol, ms = mol["nmol"], mol["molsize"]
    Hsym = symmetrize_upper(blocks_to_full(M, nmol, ms))
    if P0 is None:
        g = initial_density(mol, el)
        P = np.stack([0.5 * g, 0.5 * g], axis=1)
    else:
        P = np.array(P0, dtype=np.float64)
    nheavy, nhyd, nocc = mol["nheavy"], mol["nhyd"], mol["nocc"]
    natoms4 = 9.0 * mol["nsuper"] + 4.0 * (nheavy + nhyd)
    F = fock_u(mol, p, ints, M, P)
    E = elec_energy(P, F, Hsym)
    Enew = np.zeros(nmol)
    err = np.ones(nmol)
    dm_err = np.ones(nmol)
    dm_el = np.ones(nmol)
    nc = np.ones(nmol, dtype=bool)
    iters = np.zeros(nmol, dtype=np.int64)
    old2 = np.zeros((nmol, 2, 4 * ms))
    Pold = np.zeros_like(P)
    linear = converger[0] == 0
    if converger[0] not in (0, 1):
        raise NotImplementedError("unrestricted SCF supports scf_converger [0, alpha] and [1]")
    alpha = converger[1] if linear else None
    kstart = 0 if linear else 1
    for k in range(kstart, MAX_ITER + 1):
        sel = np.nonzero(nc)[0]
        Pnew = np.stack([0.5 * density_eigh(F[sel, s], nheavy[sel], nhyd[sel], nocc[sel, s])[0] for s in range(2)],
                        axis=1)
        for a, m in enumerate(sel):
            Pold[m] = P[m]
            for s_ in range(2):
                if linear:
                    P[m, s_] = alpha * P[m, s_] + (1.0 - alpha) * Pnew[a, s_]
                else:
                    P[m, s_], old2[m, s_] = adaptive_mix(k, Pold[m, s_], Pnew[a, s_], old2[m, s_], occ=1.0)
        iters[sel] += 1
        F = fock_u(mol, p, ints, M, P)
        Enew[sel] = elec_energy(P[sel], F[sel], Hsym[sel])
        err[sel] = Enew[sel] - E[sel]
        bad = np.abs(err) > eps
        dmm = nc & ~bad
        if np.any(dmm):
            dP = (P[dmm] - Pold[dmm]).sum(axis=1)
            dm_err[dmm] = np.sqrt(np.sum(dP * dP, axis=(1, 2))) / natoms4[dmm]
            dm_el[dmm] = np.max(np.abs(dP), axis=(1, 2))
        nc = bad | (dm_err > eps * DM_ERR_FACTOR) | (dm_el > eps * DM_ELEM_FACTOR)
        E[nc] = Enew[nc]
        if not np.any(nc):
            break
    return P, nc, iters


DIIS_DEPTH = 10  # nFock, scf_loop.py:893
DIIS_FACTOR = 50.0  # CONVERGENCE_DIIS_FACTOR, scf_loop.py:52


def _diis_fresh(nb):
    """EMAT after a (re)start: the lower triangle of (I - 1) (scf_loop.py:916-921)."""
    return np.tril(np.eye(DIIS_DEPTH + 1) - 1.0)


def _scf_diis(mol, p, ints, M, eps, P, F, E, Hsym, density, natoms4):
    """scf_forward2 with its default schedule (no direct or adaptive steps), scf_loop.py:639-1132:
    Pulay DIIS over the last 10 Fock matrices with the commutators F P - P F as residuals.
    EMAT gets one row per iteration and is read through its lower triangle (as eigh does there,
    so entries written before the ring wrapped stay in use); the pseudo-inverse keeps
    eigenvalues above 1e-13; a condition number above 1e7 resets the history after the
    iteration.  The history and its reset are kept per molecule (the reference shares the ring
    counter and resets the whole batch)."""
    nmol, nb = P.shape[0], P.shape[1]
    tri = np.triu_indices(nb)
    counter = np.full(nmol, -1)
    cfock = np.zeros(nmol, dtype=np.int64)
    emat = np.stack([_diis_fresh(nb) for _ in range(nmol)])
    fock_h = np.zeros((nmol, DIIS_DEPTH, nb, nb))
    fppf = np.zeros((nmol, DIIS_DEPTH, tri[0].size))
    diis_err = np.full(nmol, np.finfo(np.float64).max)
    nc = np.ones(nmol, dtype=bool)
    iters = np.zeros(nmol, dtype=np.int64)
    Enew = np.zeros(nmol)
    err = np.ones(nmol)
    dm_err = np.ones(nmol)
    dm_el = np.ones(nmol)
    Pold = np.zeros_like(P)
    for _k in range(0, MAX_ITER + 1):
        sel = np.nonzero(nc)[0]
        if sel.size == 0:
            break
        Fx = F.copy()
        reset = np.zeros(nmol, dtype=bool)
        for m in sel:
            cfock[m] = min(cfock[m] + 1, DIIS_DEPTH)
            counter[m] = (counter[m] + 1) % DIIS_DEPTH
            c, cf = counter[m], cfock[m]
            fock_h[m, c] = F[m]
            C = F[m] @ P[m] - P[m] @ F[m]
            fppf[m, c] = C[tri]
            diis_err[m] = np.max(np.abs(fppf[m, c]))
            emat[m, c, :cf] = fppf[m, :cf] @ fppf[m, c]
            if cf >= 2:
                evec = emat[m, : cf + 1, : cf + 1].copy()
                evec[:cf, :cf] /= max(evec[c, c], 1.0e-15)
                L, Q = np.linalg.eigh(evec, UPLO="L")
                a = np.abs(L)
                reset[m] = a.max() / a.min() > 1.0e7 if a.min() > 0 else True
                inv = np.where(a > 1.0e-13, 1.0 / np.where(a > 1.0e-13, L, 1.0), 0.0)
                coeff = -(Q[:cf, :] * inv[None, :]) @ Q[-1, :]
                Fx[m] = np.tensordot(coeff, fock_h[m, :cf], axes=1)
        Pnew = density(Fx, sel)
        for a_, m in enumerate(sel):
            Pold[m] = P[m]
            P[m] = 0.5 * P[m] + 0.5 * Pnew[a_] if cfock[m] < 2 else Pnew[a_]
        iters[sel] += 1
        F = fock(mol, p, ints, M, P)
        Enew[sel] = elec_energy(P[sel], F[sel], Hsym[sel])
        err[sel] = Enew[sel] - E[sel]
        bad = (np.abs(err) > eps) | (diis_err > DIIS_FACTOR * eps)
        dmm = nc & ~bad
        if np.any(dmm):
            dP = P[dmm] - Pold[dmm]
            dm_err[dmm] = np.sqrt(np.sum(dP * dP, axis=(1, 2))) / natoms4[dmm]
            dm_el[dmm] = np.max(np.abs(dP), axis=(1, 2))
        nc = bad | (dm_err > eps * DM_ERR_FACTOR) | (dm_el > eps * DM_ELEM_FACTOR)
        E[nc] = Enew[nc]
        for m in np.nonzero(reset)[0]:
            counter[m], cfock[m] = -1, 0
            emat[m] = _diis_fresh(nb)
            fock_h[m] = 0.0
            fppf[m] = 0.0
    return P, nc, iters


# ------------------------------------------------------------------- energies
def _gaussians(p, mol, rija, tore, ng):
    """Gaussian corrections Z_i Z_j / R (t5 + t6) (energy.py:128-131)."""
    ni, nj, idxi, idxj = mol["ni"], mol["nj"], mol["idxi"], mol["idxj"]
    K = np.stack([p[f"Gaussian{g}_K"] for g in range(1, ng + 1)], axis=1)
    L = np.stack([p[f"Gaussian{g}_L"] for g in range(1, ng + 1)], axis=1)
    Mm = np.stack([p[f"Gaussian{g}_M"] for g in range(1, ng + 1)], axis=1)
    t4 = tore[ni] * tore[nj] / rija
    t5 = np.sum(K[idxi] * np.exp(-L[idxi] * (rija[:, None] - Mm[idxi]) ** 2), axis=1)
    t6 = np.sum(K[idxj] * np.exp(-L[idxj] * (rija[:, None] - Mm[idxj]) ** 2), axis=1)
    return t4 * (t5 + t6)


def pm6_nuclear_energy(method, mol, p, rho0, el):
    """PM6 core-core repulsion per pair (energy.py:135-171): unpolarisable core
    1e-8 ((Z_i^1/3 + Z_j^1/3)/R)^12, the diatomic alp/chi factor on Z_i Z_j ev/sqrt(r^2 +
    (rho_i + rho_j)^2) with rho = rho_core where nonzero else rho0 (two_elec_two_center_int.py:
    274-283), the C-H/N-H/O-H, C-C and Si-O exceptions, and the Gaussians."""
    ni, nj, idxi, idxj = mol["ni"], mol["nj"], mol["idxi"], mol["idxj"]
    r = mol["rij"]
    rija = r * A0
    tore = el["tore"]
    an = el["atomic_num"]
    alp_t, chi_t = load_pair_params(method, int(max(ni.max(initial=0), nj.max(initial=0))))
    alp, chi = alp_t[ni, nj], chi_t[ni, nj]
    rc = p["rho_core"]
    rho = np.where(rc != 0.0, rc, rho0)
    rsum = rho[idxi] + rho[idxj]
    unpol = 1.0e-8 * ((an[ni] ** (1.0 / 3.0) + an[nj] ** (1.0 / 3.0)) / rija) ** 12
    gcore = tore[ni] * tore[nj] * EV / np.sqrt(r * r + rsum**2)
    xh = np.isin(ni, (6, 7, 8)) & (nj == 1)
    arg = np.where(xh, rija**2, rija + 0.0003 * rija**6)
    e = unpol + gcore * (1.0 + 2.0 * chi * np.exp(-alp * arg))
    cc = (ni == 6) & (nj == 6)
    e = e + np.where(cc, gcore * 9.28 * np.exp(-rija * 5.98), 0.0)
    sio = (ni == 14) & (nj == 8)
    e = e - np.where(sio, gcore * 0.0007 * np.exp(-((r - 2.9) ** 2)), 0.0)
    return e + _gaussians(p, mol, rija, tore, 4)


def pair_nuclear_energy(method, mol, p, gam, el, rho0=None):
    """Core-core repulsion per pair (energy.py:91-171); PM6_SP needs the atoms' rho0."""
    if method in ("PM6_SP", "PM6_SP_STAR"):
        return pm6_nuclear_energy(method, mol, p, rho0, el)
    ni, nj, idxi, idxj = mol["ni"], mol["nj"], mol["idxi"], mol["idxj"]
    rija = mol["rij"] * A0
    tore = el["tore"]
    alpha = p["alpha"]
    t1 = tore[ni] * tore[nj] * gam
    xh = ((ni == 7) | (ni == 8)) & (nj == 1)
    tmp = np.exp(-alpha[idxi] * rija)
    t2 = np.where(xh, tmp * rija, tmp)
    t3 = np.exp(-alpha[idxj] * rija)
    e = t1 * (1.0 + t2 + t3)
    if method in ("AM1", "PM3"):
        e = e + _gaussians(p, mol, rija, tore, 4 if method == "AM1" else 2)
    return e


def dispersion_am1_fs1(mol):
    """AM1-FS1 dispersion energy per molecule, eV (dispersion_am1_fs1.py:16-113): over the
    pairs, -sqrt(C6_i C6_j) (a0 r)^-6 f, f = sigmoid(1000 (a0 r / (1.1058892 (R0_i + R0_j)) - 1))
    clipped to 1 / 0 beyond +-12 ln 10; Grimme 2006 C6 (J nm^6 / mol), R0 (A)."""
    with open(os.path.join(_DATA, "grimme_2006_b97d.json")) as f:
        rows = np.asarray(json.load(f)["rows"], dtype=np.float64)
    c6 = np.zeros(120)
    r0 = np.zeros(120)
    c6[: rows.shape[0]], r0[: rows.shape[0]] = rows[:, 0], rows[:, 1]
    ni, nj = mol["ni"], mol["nj"]
    R = mol["rij"] * A0
    arg = 1000.0 * (R / (1.1058892 * (r0[ni] + r0[nj])) - 1.0)
    f = 1.0 / (1.0 + np.exp(-np.clip(arg, -700.0, 700.0)))
    tol = 12.0 * math.log(10.0)
    f = np.where(arg > tol, 1.0, np.where(arg < -tol, 0.0, f))
    e = -np.sqrt(c6[ni] * c6[nj]) * R**-6.0 * f
    out = np.zeros(mol["nmol"])
    np.add.at(out, mol["pair_molid"], e)
    return out * 1.036426966e-5 * 1.0e6


def isolated_atom_energy(Z, p, el):
    """energy.py:8-23."""
    return (p["U_ss"] * el["ussc"][Z] + p["U_pp"] * el["uppc"][Z] + p["g_ss"] * el["gssc"][Z]
            + p["g_pp"] * el["gppc"][Z] + p["g_sp"] * el["gspc"][Z] + p["g_p2"] * el["gp2c"][Z]
            + p["h_sp"] * el["hspc"][Z])


def energy_at(method, mol, p, P, el=None, dispersion=False):
    """All energy terms for a given density P (no SCF): integrals -> hcore -> fock -> E;
    dispersion: AM1-FS1 added to Etot and Hf (basics.py:1233-1234)."""
    el = el or load_elements()
    ints = integrals(mol, p, el)
    M = hcore(mol, p, ints)
    nmol, ms = mol["nmol"], mol["molsize"]
    Hsym = symmetrize_upper(blocks_to_full(M, nmol, ms))
    F = fock_u(mol, p, ints, M, P) if P.ndim == 4 else fock(mol, p, ints, M, P)
    Eelec = elec_energy(P, F, Hsym)
    EnucAB = pair_nuclear_energy(method, mol, p, ints["w"][:, 0, 0], el, ints["rho0"])
    Enuc = np.zeros(nmol)
    np.add.at(Enuc, mol["pair_molid"], EnucAB)
    Eiso = isolated_atom_energy(mol["Z"], p, el)
    Eiso_sum = np.zeros(nmol)
    np.add.at(Eiso_sum, mol["atom_molid"], Eiso)
    eheat = np.zeros(nmol)
    np.add.at(eheat, mol["atom_molid"], el["eheat_ev"][mol["Z"]])
    Etot = Eelec + Enuc
    if dispersion and method == "AM1":
        Etot = Etot + dispersion_am1_fs1(mol)
    return dict(Eelec=Eelec, Enuc=Enuc, Etot=Etot, Eiso=Eiso_sum, Hf=Etot - Eiso_sum + eheat, F=F, M=M, ints=ints)


def single_point(method, species, coords, eps, converger=(1,), sp2_opt=(False,), charges=None, learned=None,
                 forces=False, fd_step=1.0e-5, mult=None, cutoff=None, dispersion=False):
    """Full single point: parse -> hcore -> SCF -> energies (+ fixed-density forces).

    Forces are -dHf/dR at the converged density, by central finite differences of
    the fixed-density energy (the reference gets the same quantity by autograd with
    the SCF treated as constant, scf_loop.py:1996-2031, basics.py:1315-1336).
    """
    el = load_elements()
    mol = parse(species, coords, charges, mult, cutoff)
    p = atom_params(method, mol["Z"], learned)
    ints = integrals(mol, p, el)
    M = hcore(mol, p, ints)
    P, nc, iters = scf(mol, p, ints, M, eps, converger, sp2_opt, el=el)
    out = energy_at(method, mol, p, P, el, dispersion)
    if mol["uhf"]:  # orbital energies per spin, (nmol, 2, n)
        e = np.stack([density_eigh(out["F"][:, s], mol["nheavy"], mol["nhyd"], mol["nocc"][:, s])[1]
                      for s in range(2)], axis=1)
    else:
        _, e, vecs = density_eigh(out["F"], mol["nheavy"], mol["nhyd"], mol["nocc"])
    out.update(P=P, notconverged=nc, iters=iters, e=e, mol=mol, params=p)
    if forces:
        out["force"] = fd_forces(method, species, coords, P, charges, learned, fd_step, mult, cutoff, dispersion)
    return out


def fd_forces(method, species, coords, P, charges=None, learned=None, h=1.0e-5, mult=None, cutoff=None,
              dispersion=False):
    """-dHf/dR (eV/Angstrom) at fixed density by central differences."""
    coords = np.asarray(coords, dtype=np.float64)
    species = np.asarray(species)
    f = np.zeros_like(coords)
    el = load_elements()
    for m in range(coords.shape[0]):
        for a in range(coords.shape[1]):
            if species[m, a] == 0:
                continue
            for x in range(3):
                vals = []
                for sgn in (1.0, -1.0):
                    c = coords.copy()
                    c[m, a, x] += sgn * h
                    mol = parse(species, c, charges, mult, cutoff)
                    p = atom_params(method, mol["Z"], learned)
                    vals.append(energy_at(method, mol, p, P, el, dispersion)["Hf"][m])
                f[m, a, x] = -(vals[0] - vals[1]) / (2.0 * h)
    return f

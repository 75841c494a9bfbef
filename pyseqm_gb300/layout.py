"""Ragged, unpadded batch layout of molecules -> atoms -> atom pairs.

``Layout.from_padded`` takes the seqm API's padded input (species sorted by
descending Z per row, zero padding) and builds, on the host with NumPy:

* per molecule: atom / pair-class / dense-matrix / basis-row offsets, norb, nocc;
* per atom: Z, owning molecule, coordinates, parameters (structure of arrays);
* per pair: the two atom indices, in three class segments (heavy-heavy, heavy-H,
  H-H) each enumerated row-major inside its molecule (the index arithmetic the
  kernels use to find an atom's pairs).

``to_device`` uploads it once; ``struct`` returns the ``seqm_batch`` C struct
pointing at the device copies.  ``packed_to_padded`` / ``padded_to_packed``
convert per-molecule matrices to and from the reference's padded
``(nmol, 4*molsize, 4*molsize)`` layout (seqm/seqm_functions/pack.py:8-96).
"""

import ctypes

import numpy as np
import torch

from . import native, tables


def _group_fill(dest, off, counts, key_arrays, maker):
    """Fill dest[off[m] + k] for molecule groups sharing the same key (sizes)."""
    keys = np.stack(key_arrays, axis=1) if len(key_arrays) > 1 else key_arrays[0][:, None]
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    for g, key in enumerate(uniq):
        ms = np.nonzero(inv.reshape(-1) == g)[0]
        loc = maker(*key)  # tuple of arrays, each (L,)
        L = loc[0].size
        if L == 0:
            continue
        idx = off[ms][:, None] + np.arange(L)[None, :]
        for d, v in zip(dest, loc):
            d[0][idx] = d[1][ms][:, None] + v[None, :]


def set_size_classes(struct, norb_sorted):
    """Size classes of the scheduling order (molecules by descending norb) for per-molecule
    kernels: class c holds the molecules above the next bound of native.CLASS_BOUNDS; empty
    classes are dropped.  norb_sorted: the molecules' norb in scheduling order."""
    norb_sorted = np.asarray(norb_sorted)
    ends, caps = [], []
    start = 0
    for bound in native.CLASS_BOUNDS + (-1,):
        end = int(np.sum(norb_sorted > bound))
        if end > start:
            ends.append(end)
            caps.append(int(norb_sorted[start]))
        start = max(start, end)
    struct.nclass = len(ends)
    for c in range(native.MAX_CLASSES):
        struct.class_end[c] = ends[c] if c < len(ends) else 0
        struct.class_norb[c] = caps[c] if c < len(caps) else 0


class Layout:
    def __init__(self):
        self.dev = None
        self.pair_par = None

    # ------------------------------------------------------------------ build
    @classmethod
    def from_padded(cls, species, coords, method, charges=None, learned=None, mult=None, pair_cutoff=None,
                    param_dir=None):
        """mult: spin multiplicities for an unrestricted solve (nocc_a / nocc_b = alpha / beta
        occupations, basics.py:278-295); None: closed shells.  pair_cutoff (Angstrom): pairs at
        or beyond it are left out of every term, as the reference's parser drops them
        (basics.py:324-328); the set is fixed at these coordinates.  param_dir: the directory of
        MOPAC-format parameter files to read instead of the packaged tables."""
        species = np.ascontiguousarray(np.asarray(species, dtype=np.int64))
        coords = np.asarray(coords, dtype=np.float64)
        if species.ndim != 2 or coords.shape != species.shape + (3,):
            raise ValueError("species must be (nmol, molsize) and coordinates (nmol, molsize, 3)")
        if not np.all(species[:, :-1] >= species[:, 1:]):
            bad = np.nonzero(~np.all(species[:, :-1] >= species[:, 1:], axis=1))[0].tolist()
            raise ValueError(f"species must be non-increasing along each row, but rows {bad} are not sorted.")
        if method not in tables.METHOD_FIELDS:
            raise ValueError(f"unsupported method {method!r}; supported: {tables.SUPPORTED}")
        el = tables.elements()
        L = cls()
        L.method = method
        L.nmol, L.molsize = species.shape
        real = species > 0
        L.natoms_m = real.sum(1).astype(np.int64)
        L.nheavy = (species > 1).sum(1).astype(np.int64)
        L.nhyd = (species == 1).sum(1).astype(np.int64)
        L.norb = 4 * L.nheavy + L.nhyd
        # atoms the reference's parser also counts as super-heavy (basics.py:258-270); only its
        # SCF convergence test reads them (scf_loop.py:245)
        L.nsuper = ((species >= 13) & (species <= 17)).sum(1).astype(np.int64)
        nel = el["tore"][species].sum(1).astype(np.int64)
        if charges is not None:
            nel = nel - np.asarray(charges, dtype=np.float64).reshape(-1).astype(np.int64)
        L.uhf = mult is not None
        if L.uhf:
            s2 = np.asarray(mult, dtype=np.float64).reshape(-1) - 1.0
            na, nb = nel / 2.0 + s2 / 2.0, nel / 2.0 - s2 / 2.0
            if np.any(na % 1 != 0) or np.any(nb % 1 != 0) or np.any(nb < 0):
                raise ValueError("Invalid charge/multiplicity combination!")
            L.nocc_a, L.nocc_b = na.astype(np.int64), nb.astype(np.int64)
            L.nocc = L.nocc_a
        else:
            if np.any(nel % 2 == 1):
                raise ValueError("RHF setting requires closed shell systems (even number of electrons)")
            L.nocc = nel // 2
        L.atom_off = np.concatenate([[0], np.cumsum(L.natoms_m)])
        L.natoms = int(L.atom_off[-1])
        L.real_index = np.nonzero(real.reshape(-1))[0]  # flat padded index of every real atom
        L.Z = species.reshape(-1)[L.real_index]
        if np.any(el["qn"][L.Z] > 3) or np.any(L.Z == 2):
            raise ValueError("Error from diat.py, overlap matrix\nSome elements are not supported yet")
        pp = tables.pair_par(method, param_dir)
        if pp is not None and np.any(L.Z > pp[1]):
            raise ValueError(f"{method}: no diatomic core-core parameters for elements {sorted(set(L.Z[L.Z > pp[1]]))}")
        L.pair_par = pp
        L.xyz = coords.reshape(-1, 3)[L.real_index]
        L.atom_mol = np.repeat(np.arange(L.nmol), L.natoms_m)
        L.mat_off = np.concatenate([[0], np.cumsum(L.norb * L.norb)]).astype(np.int64)
        L.row_off = np.concatenate([[0], np.cumsum(L.norb)]).astype(np.int64)
        nh, ny = L.nheavy, L.nhyd
        L.nxx_m, L.nxh_m, L.nhh_m = nh * (nh - 1) // 2, nh * ny, ny * (ny - 1) // 2
        L.xx_off = np.concatenate([[0], np.cumsum(L.nxx_m)])
        L.xh_off = np.concatenate([[0], np.cumsum(L.nxh_m)])
        L.hh_off = np.concatenate([[0], np.cumsum(L.nhh_m)])
        L.nxx, L.nxh, L.nhh = int(L.xx_off[-1]), int(L.xh_off[-1]), int(L.hh_off[-1])
        L.npairs = L.nxx + L.nxh + L.nhh
        L._pairs = None  # host pair list, built on first use (to_device builds a CUDA batch's on the GPU)
        L.pair_skip = None
        if pair_cutoff is not None and L.npairs:
            pi, pj = L.pair_i, L.pair_j
            d = L.xyz[pj] - L.xyz[pi]
            skip = np.sum(d * d, axis=1) >= float(pair_cutoff) ** 2
            if skip.any():
                L.pair_skip = skip
        L.order = np.argsort(-L.norb, kind="stable")
        L.max_norb = int(L.norb.max()) if L.nmol else 0
        # per-atom parameters, structure of arrays: a per-element table (parameter slots x
        # elements, small) whose column Z is each atom's, gathered where the parameters are used
        # (on the device for a GPU batch, so the per-atom array is neither built on the host nor
        # copied), and the learned per-atom overrides
        fields, rows = tables.method_table(method, param_dir)
        ne = max(rows.shape[0], len(el["tore"]), int(L.Z.max(initial=0)) + 1)  # past the file's rows: zeros
        tab = np.zeros((native.NPAR, ne))
        for k, f in enumerate(fields):
            tab[native.PAR[f], : rows.shape[0]] = rows[:, k]
        tab[native.PAR["_tore"], : len(el["tore"])] = el["tore"]
        tab[native.PAR["_qn"], : len(el["qn"])] = el["qn"]
        # the reference's Energy sets rho_core to zero for every method but PM6 with d orbitals
        # (basics.py:796-809), so the core-core term always takes rho0 here
        tab[native.PAR["rho_core"]] = 0.0
        L.par_table = tab
        L.learned = {native.PAR[k]: np.asarray(v, dtype=np.float64).reshape(-1) for k, v in (learned or {}).items()}
        L._par = None
        return L

    @property
    def par(self):
        """Per-atom parameters (NPAR x natoms), gathered on the host on first use."""
        if self._par is None:
            par = np.take(self.par_table, self.Z, axis=1)
            for slot, v in self.learned.items():
                par[slot] = v
            self._par = par
        return self._par

    def par_row(self, name):
        """One parameter of every atom (natoms,), without the full per-atom array."""
        slot = native.PAR[name]
        return self.learned[slot] if slot in self.learned else self.par_table[slot][self.Z]

    # ------------------------------------------------------------------- pairs
    def _host_pairs(self):
        """Global atom indices of every pair in the class-segment order (what seqm_build_pairs
        writes on the device): heavy-heavy and H-H row-major i < j, heavy-H by heavy atom then H."""
        if self._pairs is None:
            nh, ny = self.nheavy, self.nhyd
            pi = np.empty(self.npairs, dtype=np.int64)
            pj = np.empty(self.npairs, dtype=np.int64)
            a0 = self.atom_off[:-1]
            nxx, nxh = self.nxx, self.nxh
            _group_fill([(pi[:nxx], a0), (pj[:nxx], a0)], self.xx_off, None, [nh], lambda n: np.triu_indices(n, 1))
            _group_fill([(pi[nxx: nxx + nxh], a0), (pj[nxx: nxx + nxh], a0 + nh)], self.xh_off, None, [nh, ny],
                        lambda a, b: (np.repeat(np.arange(a), b), np.tile(np.arange(b), a)))
            _group_fill([(pi[nxx + nxh:], a0 + nh), (pj[nxx + nxh:], a0 + nh)], self.hh_off, None, [ny],
                        lambda n: np.triu_indices(n, 1))
            self._pairs = (pi, pj)
        return self._pairs

    @property
    def pair_i(self):
        return self._host_pairs()[0]

    @property
    def pair_j(self):
        return self._host_pairs()[1]

    # ----------------------------------------------------------------- device
    def to_device(self, device="cuda"):
        i32 = lambda a: torch.as_tensor(np.asarray(a, dtype=np.int32), device=device)  # noqa: E731
        i64 = lambda a: torch.as_tensor(np.asarray(a, dtype=np.int64), device=device)  # noqa: E731
        f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device)  # noqa: E731
        d = {
            "atom_off": i32(self.atom_off), "nheavy": i32(self.nheavy), "norb": i32(self.norb),
            "nocc": i32(self.nocc), "mat_off": i64(self.mat_off), "row_off": i64(self.row_off),
            "xx_off": i32(self.xx_off), "xh_off": i32(self.xh_off), "hh_off": i32(self.hh_off),
            "order": i32(self.order), "Z": i32(self.Z), "atom_mol": i32(self.atom_mol),
            "xyz": f64(self.xyz.reshape(-1)),
        }
        # per-atom parameters gathered on the device from the element table (+ learned overrides)
        tab = f64(self.par_table)
        par = tab[:, d["Z"].long()]
        for slot, v in self.learned.items():
            par[slot] = f64(v)
        d["par"] = par.reshape(-1).contiguous()
        copied = int(tab.numel() * 8) + sum(int(v.size * 8) for v in self.learned.values())
        # a CUDA batch whose host pair list was not needed builds it on the GPU (seqm_build_pairs)
        on_gpu = torch.device(device).type == "cuda" and self._pairs is None
        if on_gpu:
            d["pair_i"] = torch.empty(max(1, self.npairs), dtype=torch.int32, device=device)
            d["pair_j"] = torch.empty(max(1, self.npairs), dtype=torch.int32, device=device)
        else:
            d["pair_i"], d["pair_j"] = i32(self.pair_i), i32(self.pair_j)
        if self.uhf:
            d["nocc_a"], d["nocc_b"] = i32(self.nocc_a), i32(self.nocc_b)
        if self.pair_par is not None:
            d["pair_par"] = f64(self.pair_par[0])
        if np.any(self.nsuper):
            d["nsuper"] = i32(self.nsuper)
        if self.pair_skip is not None:
            d["pair_skip"] = torch.as_tensor(self.pair_skip.astype(np.uint8), device=device)
        self.dev = d
        self.device = torch.device(device)
        self._struct = native.SeqmBatch(
            nmol=self.nmol, natoms=self.natoms, nxx=self.nxx, nxh=self.nxh, nhh=self.nhh,
            method=native.METHODS[self.method], max_norb=self.max_norb, pad_=0,
            mol_atom_off=d["atom_off"].data_ptr(), mol_nheavy=d["nheavy"].data_ptr(), mol_norb=d["norb"].data_ptr(),
            mol_nocc=d["nocc"].data_ptr(), mol_mat_off=d["mat_off"].data_ptr(), mol_xx_off=d["xx_off"].data_ptr(),
            mol_xh_off=d["xh_off"].data_ptr(), mol_hh_off=d["hh_off"].data_ptr(), mol_order=d["order"].data_ptr(),
            atom_Z=d["Z"].data_ptr(), atom_mol=d["atom_mol"].data_ptr(), atom_xyz=d["xyz"].data_ptr(),
            atom_par=d["par"].data_ptr(), pair_i=d["pair_i"].data_ptr(), pair_j=d["pair_j"].data_ptr(),
            pair_par=d["pair_par"].data_ptr() if self.pair_par is not None else None,
            pair_zmax=self.pair_par[1] if self.pair_par is not None else -1, pad3_=0,
            mol_nsuper=d["nsuper"].data_ptr() if "nsuper" in d else None,
            pair_skip=d["pair_skip"].data_ptr() if "pair_skip" in d else None,
            mat_total=int(self.mat_off[-1]),
        )
        set_size_classes(self._struct, self.norb[self.order] if self.nmol else np.zeros(0, np.int64))
        # bytes copied from the host (the pair list built on the GPU and the parameters gathered there
        # are not among them; the element table and learned overrides are)
        self.h2d_bytes = copied + sum(int(t.numel() * t.element_size()) for k, t in d.items()
                                      if k != "par" and not (on_gpu and k in ("pair_i", "pair_j")))
        if on_gpu and self.npairs:
            stream = torch.cuda.current_stream(self.device).cuda_stream
            native.check(native.load().seqm_build_pairs(self._struct, native.ptr(d["pair_i"]), native.ptr(d["pair_j"]),
                                                        ctypes.c_void_p(stream)), "seqm_build_pairs")
        return self

    def set_coordinates(self, xyz_real):
        """Replace the coordinates (natoms, 3), host copy and device array in place (same molecules,
        new geometry)."""
        self.xyz = np.array(xyz_real, dtype=np.float64).reshape(-1, 3)
        self.dev["xyz"].copy_(torch.as_tensor(self.xyz).reshape(-1))

    @property
    def struct(self):
        return self._struct

    # ------------------------------------------------------------ conversions
    def packed_index(self):
        """For each molecule, flat indices (inside the padded 4ms x 4ms matrix) of its packed basis."""
        out = []
        for m in range(self.nmol):
            nh, ny = int(self.nheavy[m]), int(self.nhyd[m])
            out.append(np.concatenate([np.arange(4 * nh), 4 * nh + 4 * np.arange(ny)]))
        return out

    def _scatter_maps(self):
        if getattr(self, "_maps", None) is None:
            n4 = 4 * self.molsize
            src, dst = [], []
            for m, idx in enumerate(self.packed_index()):
                n = idx.size
                src.append(self.mat_off[m] + np.arange(n * n))
                dst.append(m * n4 * n4 + (idx[:, None] * n4 + idx[None, :]).reshape(-1))
            dev = self.device if self.dev is not None else "cpu"
            self._maps = (torch.as_tensor(np.concatenate(src) if src else np.zeros(0, np.int64), device=dev),
                          torch.as_tensor(np.concatenate(dst) if dst else np.zeros(0, np.int64), device=dev))
        return self._maps

    def packed_to_padded(self, flat):
        """Concatenated per-molecule norb x norb blocks -> (nmol, 4ms, 4ms), zeros elsewhere."""
        src, dst = self._scatter_maps()
        n4 = 4 * self.molsize
        out = torch.zeros(self.nmol * n4 * n4, dtype=flat.dtype, device=flat.device)
        out[dst] = flat[src]
        return out.view(self.nmol, n4, n4)

    def padded_to_packed(self, full):
        src, dst = self._scatter_maps()
        out = torch.empty(int(self.mat_off[-1]), dtype=full.dtype, device=full.device)
        out[src] = full.reshape(-1)[dst]
        return out

    def reference_pair_index(self):
        """Position of each of our pairs (class order) in the reference's (molecule, i<j) row-major
        order of its kept pairs, -1 for a pair beyond the pair cutoff; self.nref kept pairs."""
        if getattr(self, "_refpos", None) is None:
            nat = self.natoms_m
            ref_off = np.concatenate([[0], np.cumsum(nat * (nat - 1) // 2)])
            m = self.atom_mol[self.pair_i]
            i = self.pair_i - self.atom_off[m]
            j = self.pair_j - self.atom_off[m]
            n = nat[m]
            pos = ref_off[m] + i * n - (i * (i + 1)) // 2 + (j - i - 1)
            if self.pair_skip is not None:
                kept = np.zeros(self.npairs, dtype=bool)
                kept[pos] = ~self.pair_skip
                rank = np.cumsum(kept) - 1
                pos = np.where(self.pair_skip, -1, rank[pos])
            self._refpos = pos
            self.nref = int(self.npairs if self.pair_skip is None else np.sum(~self.pair_skip))
        return self._refpos

    def reference_pair_atoms(self):
        """(idxi, idxj) global atom indices of the kept pairs in the reference's order."""
        pos = self.reference_pair_index()
        keep = pos >= 0
        ri = np.empty(self.nref, dtype=np.int64)
        rj = np.empty(self.nref, dtype=np.int64)
        ri[pos[keep]] = self.pair_i[keep]
        rj[pos[keep]] = self.pair_j[keep]
        return ri, rj

    def block(self, flat, m):
        """Molecule m's dense norb x norb matrix view from a concatenated flat array."""
        n = int(self.norb[m])
        return flat[int(self.mat_off[m]): int(self.mat_off[m]) + n * n].view(n, n)

"""ctypes binding of the C ABI declared in include/pyseqm_gb300.h.

The library must have been built (``python -m pyseqm_gb300.build`` or
``__graft_entry__.build()``).  There is no fallback: if it is missing or a call
fails, an exception is raised.
"""

import ctypes
import os

from . import build as _build

SEQM_OK = 0
SEQM_E_ARG = -1
SEQM_E_CUDA = -2
SEQM_E_UNSUPPORTED = -3
SEQM_E_TOO_LARGE = -4
METHODS = {"MNDO": 0, "AM1": 1, "PM3": 2, "PM6_SP": 3, "PM6_SP_STAR": 3}

# per-atom parameter slots (enum in the header)
PAR_NAMES = ["U_ss", "U_pp", "zeta_s", "zeta_p", "beta_s", "beta_p", "g_ss", "g_sp", "g_pp", "g_p2", "h_sp", "alpha",
             "Gaussian1_K", "Gaussian2_K", "Gaussian3_K", "Gaussian4_K",
             "Gaussian1_L", "Gaussian2_L", "Gaussian3_L", "Gaussian4_L",
             "Gaussian1_M", "Gaussian2_M", "Gaussian3_M", "Gaussian4_M", "rho_core",
             "_dd", "_qq", "_rho0", "_rho1", "_rho2", "_tore", "_qn"]
NPAR = len(PAR_NAMES)
PAR = {n: i for i, n in enumerate(PAR_NAMES)}

EXPORTS = ["seqm_hcore", "seqm_fock", "seqm_density_jacobi", "seqm_density_jacobi_noalloc", "seqm_density_sp2",
           "seqm_density_sp2_tc", "seqm_mix", "seqm_energy_error",
           "seqm_initial_density", "seqm_pair_sum", "seqm_energy_grad", "seqm_sp2_tc_work_bytes", "seqm_diis_init",
           "seqm_diis_extrapolate", "seqm_diis_mix", "seqm_fock_u", "seqm_energy_error_u", "seqm_fock_general", "seqm_energy_grad_excited", "seqm_scf_step", "seqm_build_pairs", "seqm_version"]
DIIS_STATE = 124  # SEQM_DIIS_STATE

_P = ctypes.c_void_p


MAX_CLASSES = 4  # SEQM_MAX_CLASSES
CLASS_BOUNDS = (114, 96, 64)  # size classes of per-molecule kernels: norb > 114, 97-114, 65-96, <= 64


class SeqmBatch(ctypes.Structure):
    _fields_ = [
        ("nmol", ctypes.c_int32), ("natoms", ctypes.c_int32), ("nxx", ctypes.c_int32), ("nxh", ctypes.c_int32),
        ("nhh", ctypes.c_int32), ("method", ctypes.c_int32), ("max_norb", ctypes.c_int32), ("pad_", ctypes.c_int32),
        ("mol_atom_off", _P), ("mol_nheavy", _P), ("mol_norb", _P), ("mol_nocc", _P), ("mol_mat_off", _P),
        ("mol_xx_off", _P), ("mol_xh_off", _P), ("mol_hh_off", _P), ("mol_order", _P), ("atom_Z", _P),
        ("atom_mol", _P), ("atom_xyz", _P), ("atom_par", _P), ("pair_i", _P), ("pair_j", _P),
        ("nclass", ctypes.c_int32), ("pad2_", ctypes.c_int32), ("class_end", ctypes.c_int32 * MAX_CLASSES),
        ("class_norb", ctypes.c_int32 * MAX_CLASSES),
        ("pair_par", _P), ("pair_zmax", ctypes.c_int32), ("pad3_", ctypes.c_int32), ("mol_nsuper", _P),
        ("pair_skip", _P), ("mat_total", ctypes.c_int64),
    ]


class ScfState(ctypes.Structure):
    """seqm_scf_state: device pointers and settings of one SCF iteration after the density step."""
    _fields_ = [(n, _P) for n in ("P", "Pnew", "Pold", "old2", "H", "F", "w_xx", "w_xh", "w_hh", "Eelec", "Eout",
                                  "err", "dm_err", "dm_el", "mol_row_off", "iters", "active", "diis_err",
                                  "nactive")] + [
        ("mixing", ctypes.c_int32), ("pad_", ctypes.c_int32), ("alpha", ctypes.c_double),
        ("occupation", ctypes.c_double), ("eps", ctypes.c_double), ("scratch", _P)]


def scf_scratch_doubles(nmol, natoms, npairs, sum_norb):
    """SEQM_SCF_SCRATCH_DOUBLES: scratch of the fused seqm_scf_step."""
    return 5 * nmol + natoms + npairs + 4 * sum_norb


_lib = None


class NativeError(RuntimeError):
    pass


def lib_path():
    return _build.LIB


def load(path=None):
    """Load (once) and return the ctypes library handle; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or lib_path()
    if not os.path.exists(path):
        raise NativeError(f"pyseqm_gb300 native library not built ({path}); run pyseqm_gb300.build.build()")
    lib = ctypes.CDLL(path)
    B = ctypes.POINTER(SeqmBatch)
    i32, f64 = ctypes.c_int, ctypes.c_double
    sig = {
        "seqm_hcore": [B, _P, _P, _P, _P, _P, _P],
        "seqm_fock": [B, _P, _P, _P, _P, _P, _P, _P, _P],
        "seqm_density_jacobi": [B, _P, _P, _P, _P, _P, _P, _P, _P, i32, _P, i32, i32, _P],
        "seqm_density_jacobi_noalloc": [B, _P, _P, _P, _P, _P, _P, _P, i32, _P],
        "seqm_density_sp2": [B, _P, _P, _P, f64, _P, _P, i32, _P],
        "seqm_density_sp2_tc": [B, _P, _P, _P, f64, _P, _P, i32, i32, _P],
        "seqm_mix": [B, _P, _P, _P, _P, _P, _P, i32, f64, f64, _P, _P],
        "seqm_energy_error": [B, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, f64, _P, _P],
        "seqm_diis_init": [B, _P, _P, _P],
        "seqm_diis_extrapolate": [B, _P, _P, _P, _P, _P, _P, _P, _P],
        "seqm_diis_mix": [B, _P, _P, _P, _P, _P, _P],
        "seqm_initial_density": [B, _P, _P],
        "seqm_pair_sum": [B, _P, _P, _P],
        "seqm_energy_grad": [B, _P, _P, _P, _P, _P, _P, _P, _P],
        "seqm_fock_u": [B, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
        "seqm_energy_error_u": [B, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, f64, _P],
        "seqm_fock_general": [B, i32, _P, _P, _P, _P, _P, ctypes.c_int64, _P, _P],
        "seqm_energy_grad_excited": [B, _P, _P, _P, _P, _P, _P, _P, _P],
        "seqm_scf_step": [B, ctypes.POINTER(ScfState), _P],
        "seqm_build_pairs": [B, _P, _P, _P],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.seqm_sp2_tc_work_bytes.argtypes = [ctypes.c_int64, i32, i32]
    lib.seqm_sp2_tc_work_bytes.restype = ctypes.c_size_t
    lib.seqm_version.argtypes = []
    lib.seqm_version.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(rc, what):
    if rc == SEQM_OK:
        return
    names = {SEQM_E_ARG: "bad argument", SEQM_E_CUDA: "CUDA error", SEQM_E_UNSUPPORTED: "unsupported element/method",
             SEQM_E_TOO_LARGE: "molecule too large for this kernel"}
    if rc == SEQM_E_UNSUPPORTED:
        raise ValueError(f"{what}: some elements are not supported (overlap needs principal quantum number <= 3)")
    raise NativeError(f"{what} failed: {names.get(rc, rc)}")


def ptr(t):
    """Device (or host) address of a tensor, or NULL for None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())

"""ctypes view of libsffg's C ABI (include/sff.h and include/sffg.h).

The Python names follow the reference's C API (src/sff/sff.h:118-211):
``mm_options``, ``mme_init_sff``, ``mme``, ``md``, ``conjgrad``, ``rdparm``,
``free_prm``, ``getxv``, ``putxv`` -- same arguments, same meaning, same
fail-stop error behaviour -- plus the batched ``sffg_*`` entry points.
Arrays are numpy float64/int32 and are passed by pointer, never copied into
Python objects on the hot path.
"""
import ctypes as C
import os

import numpy as np

from . import _build

REAL_P = C.POINTER(C.c_double)
INT_P = C.POINTER(C.c_int)
NAME_T = C.c_char * 6


class PARMSTRUCT_T(C.Structure):
    """Same field order and types as the reference's struct parm
    (src/sff/sff.h:40-62)."""

    _fields_ = (
        [("ititl", C.c_char * 81)]
        + [(n, C.c_int) for n in (
            "IfBox Nmxrs IfCap Natom Ntypes Nbonh Mbona Ntheth Mtheta Nphih Mphia "
            "Nhparm Nparm Nnb Nres Nbona Ntheta Nphia Numbnd Numang Nptra Natyp Nphb "
            "Nat3 Ntype2d Nttyp Nspm Iptres Nspsol Ipatm Natcap Numextra").split()]
        + [(n, C.POINTER(NAME_T)) for n in ("AtomNames", "ResNames", "AtomType", "AtomTree")]
        + [(n, REAL_P) for n in (
            "Charges Masses Rk Req Tk Teq Pk Pn Phase Solty Cn1 Cn2 HB12 HB10 Rborn Fs").split()]
        + [("Box", C.c_double * 4)]
        + [(n, C.c_double) for n in ("Cutcap", "Xcap", "Ycap", "Zcap", "Fsmax")]
        + [(n, INT_P) for n in (
            "Iac Iblo Cno Ipres ExclAt TreeJoin AtomRes BondHAt1 BondHAt2 BondHNum BondAt1 "
            "BondAt2 BondNum AngleHAt1 AngleHAt2 AngleHAt3 AngleHNum AngleAt1 AngleAt2 AngleAt3 "
            "AngleNum DihHAt1 DihHAt2 DihHAt3 DihHAt4 DihHNum DihAt1 DihAt2 DihAt3 DihAt4 "
            "DihNum Boundary AtomicNum").split()]
        + [(n, INT_P) for n in ("N14pairs", "N14pairlist")]
        + [(n, REAL_P) for n in ("Gvdw", "Scee", "Scnb", "N14sceelist", "N14scnblist")]
        + [(n, C.c_int) for n in ("Nstrand", "Ncomplex")]
        + [(n, INT_P) for n in ("Ipstrand", "Ipcomplex")]
    )


PRM_P = C.POINTER(PARMSTRUCT_T)
FUNC_T = C.CFUNCTYPE(C.c_double, REAL_P, REAL_P, INT_P)


class XMIN_OPT_T(C.Structure):
    """Same field order and types as the reference's struct xmin_opt
    (src/sff/sff.h:64-84)."""

    _fields_ = [
        ("mol_struct_opt", C.c_int), ("maxiter", C.c_int), ("grms_tol", C.c_double),
        ("method", C.c_int), ("numdiff", C.c_int), ("m_lbfgs", C.c_int), ("iter", C.c_int),
        ("xmin_time", C.c_double), ("ls_method", C.c_int), ("ls_maxiter", C.c_int),
        ("ls_maxatmov", C.c_double), ("beta_armijo", C.c_double), ("c_armijo", C.c_double),
        ("mu_armijo", C.c_double), ("ftol_wolfe", C.c_double), ("gtol_wolfe", C.c_double),
        ("ls_iter", C.c_int), ("print_level", C.c_int), ("error_flag", C.c_int),
    ]



class LMOD_OPT_T(C.Structure):
    """Same field order and types as the reference's struct lmod_opt
    (src/sff/sff.h:86-113)."""

    _fields_ = [
        ("niter", C.c_int), ("nmod", C.c_int), ("kmod", C.c_int), ("nrotran_dof", C.c_int),
        ("nconf", C.c_int), ("minim_grms", C.c_double), ("energy_window", C.c_double),
        ("conf_separation_rms", C.c_double), ("eig_recalc", C.c_int), ("ndim_arnoldi", C.c_int),
        ("lmod_restart", C.c_int), ("n_best_struct", C.c_int), ("mc_option", C.c_int),
        ("rtemp", C.c_double), ("lmod_step_size_min", C.c_double), ("lmod_step_size_max", C.c_double),
        ("nof_lmod_steps", C.c_int), ("lmod_relax_grms", C.c_double), ("nlig", C.c_int),
        ("apply_rigdock", C.c_int), ("nof_poses_to_try", C.c_int), ("random_seed", C.c_int),
        ("print_level", C.c_int), ("lmod_time", C.c_double), ("aux_time", C.c_double),
        ("error_flag", C.c_int),
    ]

_lib = None


def lib():
    """Load libsffg.so (built in-tree by nabc_gb300._build).  Raises if the
    CUDA library is missing: there is no CPU fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"libsffg.so not found at {path}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path, mode=C.RTLD_GLOBAL)
    L.mm_options.argtypes = [C.c_char_p]
    L.mm_options.restype = C.c_int
    L.rdparm.argtypes = [C.c_char_p]
    L.rdparm.restype = PRM_P
    L.wrparm.argtypes = [PRM_P, C.c_char_p]
    L.wrparm.restype = C.c_int
    L.free_prm.argtypes = [PRM_P]
    L.free_prm.restype = C.c_int
    L.getxv.argtypes = [C.c_char_p, C.c_int, C.c_double, REAL_P, REAL_P]
    L.getxv.restype = C.c_int
    L.putxv.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_double, REAL_P, REAL_P]
    L.putxv.restype = C.c_int
    L.sffg_synth_molecule.argtypes = [C.c_int, C.c_ulonglong, REAL_P, REAL_P]
    L.sffg_synth_molecule.restype = PRM_P
    L.xmin_opt_init.argtypes = [C.POINTER(XMIN_OPT_T)]
    L.xmin_opt_init.restype = C.c_int
    L.xmin.argtypes = [C.c_void_p, INT_P, REAL_P, REAL_P, REAL_P, REAL_P, C.POINTER(XMIN_OPT_T)]
    L.xmin.restype = C.c_double
    L.xminC.argtypes = [INT_P, INT_P, INT_P, REAL_P, INT_P, INT_P, INT_P, REAL_P, REAL_P, REAL_P,
                        REAL_P, INT_P, REAL_P, INT_P, INT_P, INT_P, INT_P, REAL_P, REAL_P, REAL_P,
                        REAL_P, REAL_P, REAL_P, INT_P, INT_P]
    L.xminC.restype = C.c_double
    L.lmod_opt_init.argtypes = [C.POINTER(LMOD_OPT_T), C.POINTER(XMIN_OPT_T)]
    L.lmod_opt_init.restype = C.c_int
    lmod_args = [INT_P, REAL_P, REAL_P, REAL_P, REAL_P, REAL_P, INT_P, INT_P, INT_P, REAL_P, REAL_P,
                 REAL_P, REAL_P, C.POINTER(XMIN_OPT_T), C.POINTER(LMOD_OPT_T)]
    L.lmod.argtypes = lmod_args
    L.lmod.restype = C.c_double
    L.sffg_lmod_func.argtypes = [C.c_void_p] + lmod_args
    L.sffg_lmod_func.restype = C.c_double
    L.lmodC.restype = C.c_double  # 38 pointer arguments, passed as given
    L.sffg_low_modes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_void_p, REAL_P,
                                 REAL_P]
    L.sffg_low_modes.restype = C.c_int
    if hasattr(L, "mme_init_sff"):
        L.mme_init_sff.argtypes = [PRM_P, INT_P, INT_P, REAL_P, C.c_char_p]
        L.mme_init_sff.restype = C.c_int
        L.mme.argtypes = [REAL_P, REAL_P, INT_P]
        L.mme_rattle.restype = C.c_double
        L.mme_rattle.argtypes = [REAL_P, REAL_P, INT_P]
        L.mme.restype = C.c_double
        L.md.argtypes = [C.c_int, C.c_int, REAL_P, REAL_P, REAL_P, C.c_void_p]
        L.md.restype = C.c_int
        L.conjgrad.argtypes = [REAL_P, INT_P, REAL_P, C.c_void_p, REAL_P, REAL_P, INT_P]
        L.conjgrad.restype = C.c_int
        L.mme_timer.argtypes = []
        L.mme_timer.restype = C.c_int
        L.sffg_options_reset.argtypes = []
        L.sffg_options_reset.restype = None
        L.sffg_last_error.argtypes = []
        L.sffg_last_error.restype = C.c_char_p
        vp = C.c_void_p
        L.sffg_batch_create.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.sffg_batch_add_system.argtypes = [vp, PRM_P, INT_P, REAL_P, INT_P]
        L.sffg_batch_finalize.argtypes = [vp]
        L.sffg_batch_set_restraints.argtypes = [vp, C.c_int, INT_P, REAL_P]
        L.sffg_batch_num_systems.argtypes = [vp]
        L.sffg_batch_num_atoms.argtypes = [vp, C.c_int]
        for name in ("set_coords", "get_coords", "get_grad", "get_reff", "set_velocities",
                     "get_velocities"):
            getattr(L, "sffg_batch_" + name).argtypes = [vp, C.c_int, REAL_P, vp]
        L.sffg_batch_eval.argtypes = [vp, C.c_int, vp]
        L.sffg_batch_get_energy.argtypes = [vp, C.c_int, REAL_P, vp]
        L.sffg_batch_num_pairs.argtypes = [vp, C.c_int]
        L.sffg_batch_num_pairs.restype = C.c_longlong
        L.sffg_batch_md.argtypes = [vp, C.c_int, vp]
        L.sffg_batch_cg.argtypes = [vp, C.c_int, C.c_double, C.c_double, INT_P, REAL_P, vp]
        L.sffg_batch_xmin.argtypes = [vp, C.POINTER(XMIN_OPT_T), INT_P, INT_P, REAL_P, vp]
        L.sffg_batch_lmod.argtypes = [vp, C.POINTER(LMOD_OPT_T), C.POINTER(XMIN_OPT_T), INT_P, REAL_P, INT_P,
                                      REAL_P, vp]
        L.sffg_batch_status.argtypes = [vp, INT_P, vp]
        L.sffg_checked_code.argtypes = []
        L.sffg_checked_code.restype = C.c_int
        L.sffg_list_overflows.argtypes = []
        L.sffg_list_overflows.restype = C.c_longlong
        L.sffg_batch_save.argtypes = [vp, C.c_char_p, vp]
        L.sffg_batch_load.argtypes = [vp, C.c_char_p, vp]
        L.mm_set_checkpoint.argtypes = [C.POINTER(C.c_char_p)]
        L.mm_set_checkpoint.restype = None
        L.sffg_batch_md_begin.argtypes = [vp, vp]
        L.sffg_batch_md_steps.argtypes = [vp, C.c_int, C.c_int, vp]
        L.sffg_batch_launch_count.argtypes = [vp]
        L.sffg_batch_launch_count.restype = C.c_longlong
        L.sffg_batch_set_profiling.argtypes = [vp, C.c_int]
        L.sffg_batch_kernel_times.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
        L.sffg_batch_tuned_split.argtypes = [vp, C.c_int, INT_P, INT_P]
        L.sffg_batch_device_bytes.argtypes = [vp]
        L.sffg_batch_device_bytes.restype = C.c_size_t
        L.sffg_batch_destroy.argtypes = [vp]
    _lib = L
    return L


def set_output(path):
    """Point the library's nabout stream (the reference's global output
    FILE*) at a file; returns the previous FILE* value."""
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    fp = libc.fopen(os.fsencode(path), b"a")
    var = C.c_void_p.in_dll(lib(), "nabout")
    old = var.value
    var.value = fp
    return old


def restore_output(previous):
    """Close the file set_output opened and point nabout back at previous."""
    libc = C.CDLL(None)
    libc.fclose.argtypes = [C.c_void_p]
    var = C.c_void_p.in_dll(lib(), "nabout")
    fp = var.value
    var.value = previous
    if fp and fp != previous:
        libc.fclose(fp)


def flush_output():
    libc = C.CDLL(None)
    libc.fflush.argtypes = [C.c_void_p]
    libc.fflush(C.c_void_p.in_dll(lib(), "nabout"))


def dptr(a):
    return a.ctypes.data_as(REAL_P)


def iptr(a):
    return a.ctypes.data_as(INT_P)


def natom(prm):
    return prm.contents.Natom


def rdparm(path):
    return lib().rdparm(os.fsencode(path))


def free_prm(prm):
    lib().free_prm(prm)


def getxv(path, n):
    x = np.zeros(3 * n)
    v = np.zeros(3 * n)
    lib().getxv(os.fsencode(path), n, 0.0, dptr(x), dptr(v))
    return x, v


def mm_options(opts):
    return lib().mm_options(opts.encode())


def synth_molecule(natom_, seed):
    """(prm, x, radius) for the synthetic chain molecule."""
    x = np.zeros(3 * natom_)
    r = C.c_double(0.0)
    prm = lib().sffg_synth_molecule(natom_, seed, dptr(x), C.byref(r))
    if not prm:
        raise ValueError("synthetic molecule generation failed")
    return prm, x, r.value


def read_pdb_coords(path, n):
    """Coordinates from columns 31-54 of ATOM/HETATM records, in file order
    (the order NAB's getpdb gives the test molecules)."""
    xs = []
    with open(path) as f:
        for line in f:
            if line.startswith("ATOM") or line.startswith("HETATM"):
                xs.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    a = np.array(xs[:n], dtype=np.float64).reshape(-1)
    if a.size != 3 * n:
        raise ValueError(f"{path}: expected {n} atoms")
    return a


class Session:
    """The legacy single-system session: mm_options + mme_init_sff + mme.

    Like the reference's mme_init_sff, the library borrows the frozen and
    constrained arrays for the life of the session: keep this object alive
    while the session is in use."""

    def __init__(self, prm, opts, frozen=None, reset=True):
        L = lib()
        n = natom(prm)
        self.prm = prm
        self.n = n
        if reset:
            L.sffg_options_reset()
        L.mm_options(opts.encode())
        self.frozen = np.zeros(n, np.int32) if frozen is None else np.asarray(frozen, np.int32)
        self.constrained = np.zeros(n, np.int32)
        L.mme_init_sff(prm, iptr(self.frozen), iptr(self.constrained), None, None)

    def mme(self, x, it=-2):
        g = np.zeros(3 * self.n)
        i = C.c_int(it)
        e = lib().mme(dptr(x), dptr(g), C.byref(i))
        return e, g

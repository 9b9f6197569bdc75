"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle
(oracle/sffo.c).  Used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker; never by the product path."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsffo.so")

REAL_P = C.POINTER(C.c_double)
INT_P = C.POINTER(C.c_int)


class Opts(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("cut", "rgbmax", "kappa", "epsext", "dielc")] + \
               [(n, C.c_int) for n in ("gb", "nsnb", "ntpr")] + \
               [(n, C.c_double) for n in ("dt", "temp0", "tempi", "gamma_ln", "tautp", "vlimit")] + \
               [(n, C.c_int) for n in ("zerov", "ntpr_md")] + \
               [("wcons", C.c_double), ("nscm", C.c_int)]


_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.sffo_default_opts.argtypes = [C.POINTER(Opts)]
        L.sffo_create.argtypes = [C.c_void_p, C.POINTER(Opts), INT_P]
        L.sffo_create.restype = C.c_void_p
        L.sffo_destroy.argtypes = [C.c_void_p]
        L.sffo_mme.argtypes = [C.c_void_p, REAL_P, REAL_P, REAL_P, REAL_P, C.c_int]
        L.sffo_mme.restype = C.c_double
        L.sffo_npairs.argtypes = [C.c_void_p]
        L.sffo_npairs.restype = C.c_long
        L.sffo_md.argtypes = [C.c_void_p, C.c_int, REAL_P, REAL_P, REAL_P, INT_P, REAL_P]
        L.sffo_conjgrad.argtypes = [C.c_void_p, REAL_P, REAL_P, C.c_double, C.c_double, C.c_int,
                                    REAL_P, INT_P]
        L.sffo_gauss_stream.argtypes = [INT_P, C.c_int, C.c_double, REAL_P, REAL_P]
        L.sffo_set_restraints.argtypes = [C.c_void_p, INT_P, REAL_P]
        L.sffo_set_threads.argtypes = [C.c_int]
        L.sffo_set_threads.restype = C.c_int
        L.sffo_synth_molecule.argtypes = [C.c_int, C.c_ulonglong, REAL_P, REAL_P]
        L.sffo_synth_molecule.restype = C.c_void_p
        L.sffo_synth_free.argtypes = [C.c_void_p]
        L.sffo_prm_natom.argtypes = [C.c_void_p]
        L.sffo_prm_natom.restype = C.c_int
        L.sffo_prm_fsmax.argtypes = [C.c_void_p]
        L.sffo_prm_fsmax.restype = C.c_double
        _lib = L
    return _lib


def xmin_functions():
    """The minimiser test functions of oracle/xmin_funcs.c (extended
    Rosenbrock and a bead chain), built without floating-point contraction:
    the same compiled code the reference's XMIN ran on to make the golden
    traces."""
    path = os.path.join(HERE, "_build", "libxminf.so")
    if not os.path.exists(path):
        build()
    F = C.CDLL(path)
    for name in ("xf_rosenbrock", "xf_chain"):
        getattr(F, name).restype = C.c_double
        getattr(F, name).argtypes = [REAL_P, REAL_P, INT_P]
    return F


def _p(a):
    return a.ctypes.data_as(REAL_P)


def parse_opts(text):
    """The subset of the mm_options grammar the oracle needs."""
    o = Opts()
    lib().sffo_default_opts(C.byref(o))
    items = text.replace(",", " ").replace("=", " = ").split()
    i = 0
    while i < len(items):
        key = items[i]
        if i + 2 < len(items) and items[i + 1] == "=":
            val = items[i + 2]
            i += 3
        else:
            val = items[i + 1]
            i += 2
        if key == "diel":
            continue
        if key in ("gb", "nsnb", "ntpr", "zerov", "ntpr_md", "nscm"):
            setattr(o, key, int(val))
        elif key in dict(Opts._fields_):
            setattr(o, key, float(val))
    return o


class SynthMolecule:
    """A synthetic molecule made by oracle/synth.c, the C restatement of the
    library's generator (sffg_synth_molecule): the same coordinates and
    topology, made without loading the library.  .ptr is its PARMSTRUCT_T
    (only the fields the oracle reads are filled)."""

    def __init__(self, natom, seed):
        self.x = np.zeros(3 * natom)
        r = C.c_double(0.0)
        self.ptr = lib().sffo_synth_molecule(natom, seed, _p(self.x), C.byref(r))
        if not self.ptr:
            raise ValueError("synthetic molecule generation failed")
        self.radius = r.value
        self.natom = lib().sffo_prm_natom(self.ptr)
        self.fsmax = lib().sffo_prm_fsmax(self.ptr)

    def close(self):
        if self.ptr:
            lib().sffo_synth_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()


class Oracle:
    """One FP64 oracle session on a PARMSTRUCT_T pointer (ctypes) or a
    SynthMolecule."""

    def __init__(self, prm, opts, frozen=None):
        self.o = parse_opts(opts) if isinstance(opts, str) else opts
        if isinstance(prm, SynthMolecule):
            self.n, ptr = prm.natom, C.c_void_p(prm.ptr)
        else:
            self.n, ptr = prm.contents.Natom, C.cast(prm, C.c_void_p)
        self.frozen = None if frozen is None else np.ascontiguousarray(frozen, np.int32)
        self.h = lib().sffo_create(ptr, C.byref(self.o),
                                   None if self.frozen is None else self.frozen.ctypes.data_as(INT_P))

    def close(self):
        if self.h:
            lib().sffo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def mme(self, x, rebuild=True):
        """(total energy, ene[13], gradient[3N], reff[N])."""
        x = np.ascontiguousarray(x, np.float64)
        g = np.zeros(3 * self.n)
        ene = np.zeros(13)
        reff = np.zeros(self.n)
        e = lib().sffo_mme(self.h, _p(x), _p(g), _p(ene), _p(reff), int(rebuild))
        return e, ene, g, reff

    def npairs(self):
        return lib().sffo_npairs(self.h)

    def set_restraints(self, constrained, x0):
        c = np.ascontiguousarray(constrained, np.int32)
        x0 = np.ascontiguousarray(x0, np.float64)
        lib().sffo_set_restraints(self.h, c.ctypes.data_as(INT_P), _p(x0))

    def conjgrad(self, x, rmsgrad, dfpred, maxiter):
        x = np.array(x, np.float64)
        f = C.c_double(0.0)
        etrace = np.zeros(maxiter + 2)
        nev = C.c_int(0)
        ret = lib().sffo_conjgrad(self.h, _p(x), C.byref(f), rmsgrad, dfpred, maxiter,
                                  _p(etrace), C.byref(nev))
        return ret, f.value, x, etrace[:nev.value]

    def md(self, x, v, nsteps, seed=-1):
        x = np.array(x, np.float64)
        v = np.array(v, np.float64)
        f = np.zeros(3 * self.n)
        s = C.c_int(seed)
        trace = np.zeros(2 * nsteps)
        lib().sffo_md(self.h, nsteps, _p(x), _p(f), _p(v), C.byref(s), _p(trace))
        return x, v, trace.reshape(-1, 2)


def set_threads(n):
    """Threads of the oracle's OpenMP loops (n > 0 sets it); the count in
    effect."""
    return lib().sffo_set_threads(int(n))


def gauss_stream(n, sd, seed=-1):
    sd = np.ascontiguousarray(np.broadcast_to(np.asarray(sd, np.float64), (n,)))
    out = np.zeros(n)
    s = C.c_int(seed)
    lib().sffo_gauss_stream(C.byref(s), n, 0.0, _p(sd), _p(out))
    return out, s.value

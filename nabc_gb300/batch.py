"""Python handle for the batched C API (include/sffg.h)."""
import ctypes as C
import os

import numpy as np

from . import sff


class SffgError(RuntimeError):
    pass


def _check(rc, what):
    if rc != 0:
        msg = sff.lib().sffg_last_error()
        raise SffgError(f"{what}: status {rc}: {msg.decode() if msg else ''}")


class Batch:
    """Many independent systems resident on the GPU, evaluated together."""

    def __init__(self, opts):
        L = sff.lib()
        self.h = C.c_void_p()
        _check(L.sffg_batch_create(opts.encode(), C.byref(self.h)), "sffg_batch_create")
        self.natoms = []

    def add(self, prm, x, frozen=None, constrained=None, x0=None):
        """Adds a system; constrained/x0 hold atoms to reference positions
        with the option wcons."""
        L = sff.lib()
        idx = C.c_int(-1)
        fz = None if frozen is None else sff.iptr(np.ascontiguousarray(frozen, np.int32))
        x = np.ascontiguousarray(x, np.float64)
        _check(L.sffg_batch_add_system(self.h, prm, fz, sff.dptr(x), C.byref(idx)), "add_system")
        if constrained is not None:
            c = np.ascontiguousarray(constrained, np.int32)
            r = np.ascontiguousarray(x0, np.float64)
            _check(L.sffg_batch_set_restraints(self.h, idx.value, sff.iptr(c), sff.dptr(r)), "set_restraints")
        self.natoms.append(prm.contents.Natom)
        return idx.value

    def finalize(self):
        _check(sff.lib().sffg_batch_finalize(self.h), "finalize")
        return self

    def set_coords(self, s, x, stream=None):
        x = np.ascontiguousarray(x, np.float64)
        _check(sff.lib().sffg_batch_set_coords(self.h, s, sff.dptr(x), stream), "set_coords")

    def coords(self, s):
        x = np.zeros(3 * self.natoms[s])
        _check(sff.lib().sffg_batch_get_coords(self.h, s, sff.dptr(x), None), "get_coords")
        return x

    def eval(self, rebuild=False, stream=None):
        _check(sff.lib().sffg_batch_eval(self.h, int(rebuild), stream), "eval")

    def energy(self, s):
        e = np.zeros(13)
        _check(sff.lib().sffg_batch_get_energy(self.h, s, sff.dptr(e), None), "get_energy")
        return e

    def grad(self, s):
        g = np.zeros(3 * self.natoms[s])
        _check(sff.lib().sffg_batch_get_grad(self.h, s, sff.dptr(g), None), "get_grad")
        return g

    def reff(self, s):
        r = np.zeros(self.natoms[s])
        _check(sff.lib().sffg_batch_get_reff(self.h, s, sff.dptr(r), None), "get_reff")
        return r

    def velocities(self, s):
        v = np.zeros(3 * self.natoms[s])
        _check(sff.lib().sffg_batch_get_velocities(self.h, s, sff.dptr(v), None), "get_velocities")
        return v

    def set_velocities(self, s, v):
        v = np.ascontiguousarray(v, np.float64)
        _check(sff.lib().sffg_batch_set_velocities(self.h, s, sff.dptr(v), None), "set_velocities")

    def num_pairs(self, s):
        return sff.lib().sffg_batch_num_pairs(self.h, s)

    def md(self, nsteps, stream=None):
        _check(sff.lib().sffg_batch_md(self.h, nsteps, stream), "md")

    def cg(self, maxiter, rmsgrad, dfpred=1.0, stream=None):
        n = len(self.natoms)
        st = np.zeros(n, np.int32)
        en = np.zeros(n)
        _check(sff.lib().sffg_batch_cg(self.h, maxiter, rmsgrad, dfpred, sff.iptr(st), sff.dptr(en), stream),
               "cg")
        return st, en

    def save(self, path, stream=None):
        """Write every system's md state (sffg_batch_save)."""
        _check(sff.lib().sffg_batch_save(self.h, os.fsencode(path), stream), "save")

    def load(self, path, stream=None):
        """Read a saved md state into this batch (sffg_batch_load)."""
        _check(sff.lib().sffg_batch_load(self.h, os.fsencode(path), stream), "load")

    def status(self, stream=None):
        """Per system: 0, or sffg's SFFG_ENONFINITE (-5) once an evaluation
        met a non-finite coordinate of that system."""
        st = np.zeros(len(self.natoms), np.int32)
        _check(sff.lib().sffg_batch_status(self.h, sff.iptr(st), stream), "status")
        return st

    def xmin(self, stream=None, **opts):
        """The reference's XMIN on every system (sffg_batch_xmin); opts set
        fields of XMIN_OPT_T over xmin_opt_init's defaults (method, maxiter,
        grms_tol, ls_maxatmov, ...).  Returns (status, iterations, energy)
        per system; the minimised coordinates stay in the batch."""
        L = sff.lib()
        xo = sff.XMIN_OPT_T()
        L.xmin_opt_init(C.byref(xo))
        for k, v in opts.items():
            setattr(xo, k, v)
        n = len(self.natoms)
        st = np.zeros(n, np.int32)
        it = np.zeros(n, np.int32)
        en = np.zeros(n)
        _check(L.sffg_batch_xmin(self.h, C.byref(xo), sff.iptr(st), sff.iptr(it), sff.dptr(en), stream), "xmin")
        return st, it, en

    def lmod(self, xmin_opts=None, stream=None, **opts):
        """LMOD searches on every system (sffg_batch_lmod); opts set fields
        of LMOD_OPT_T over lmod_opt_init's defaults (niter, nmod, kmod,
        mc_option, random_seed, ...), xmin_opts fields of the XMIN_OPT_T the
        minimisations use.  Returns (status, lowest energy, number of
        structures, conflib) per system, conflib[s] an (nconf, natom, 3)
        array; the lowest structures stay in the batch."""
        L = sff.lib()
        lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
        L.lmod_opt_init(C.byref(lo), C.byref(xo))
        for k, v in opts.items():
            setattr(lo, k, v)
        for k, v in (xmin_opts or {}).items():
            setattr(xo, k, v)
        n = len(self.natoms)
        st = np.zeros(n, np.int32)
        gm = np.zeros(n)
        nc = np.zeros(n, np.int32)
        flat = np.zeros(3 * int(np.sum(self.natoms)) * lo.nconf)
        _check(L.sffg_batch_lmod(self.h, C.byref(lo), C.byref(xo), sff.iptr(st), sff.dptr(gm), sff.iptr(nc),
                                 sff.dptr(flat), stream), "lmod")
        out, off = [], 0
        for s, na in enumerate(self.natoms):
            blk = flat[3 * off * lo.nconf:3 * (off + na) * lo.nconf].reshape(lo.nconf, na, 3)
            out.append(blk[:nc[s]].copy())
            off += na
        return st, gm, nc, out

    def md_begin(self, stream=None):
        _check(sff.lib().sffg_batch_md_begin(self.h, stream), "md_begin")

    def md_steps(self, step0, nsteps, stream=None):
        _check(sff.lib().sffg_batch_md_steps(self.h, step0, nsteps, stream), "md_steps")

    def launches(self):
        return sff.lib().sffg_batch_launch_count(self.h)

    def set_profiling(self, on=True):
        _check(sff.lib().sffg_batch_set_profiling(self.h, int(on)), "set_profiling")

    def kernel_times(self):
        ms = (C.c_double * 3)()
        n = C.c_longlong(0)
        _check(sff.lib().sffg_batch_kernel_times(self.h, ms, C.byref(n)), "kernel_times")
        return list(ms), n.value

    def device_bytes(self):
        return sff.lib().sffg_batch_device_bytes(self.h)

    def tuned_split(self):
        """(claim, blocks) of the three pair passes."""
        out = []
        for p in range(3):
            c, b = C.c_int(0), C.c_int(0)
            _check(sff.lib().sffg_batch_tuned_split(self.h, p, C.byref(c), C.byref(b)), "tuned_split")
            out.append((c.value, b.value))
        return out

    def close(self):
        if self.h:
            sff.lib().sffg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

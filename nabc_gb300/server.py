"""Python handle for the serving API (include/sffg.h, sffg_server_*):
continuous batching of minimisation and md requests on one GPU."""
import ctypes as C

import numpy as np

from . import sff

KINDS = {"minimize": 0, "md": 1}


class ServerError(RuntimeError):
    pass


def _proto(L):
    if getattr(L, "_sffg_server_proto", False):
        return L
    vp = C.c_void_p
    L.sffg_server_create.argtypes = [C.c_char_p, C.c_double, C.c_int, C.POINTER(vp)]
    L.sffg_server_submit.argtypes = [vp, sff.PRM_P, sff.REAL_P, C.c_int, C.c_int, C.c_double,
                                     C.POINTER(C.c_longlong)]
    L.sffg_server_pump.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.sffg_server_result.argtypes = [vp, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_double), sff.REAL_P,
                                     C.POINTER(C.c_double)]
    L.sffg_server_device_bytes.argtypes = [vp]
    L.sffg_server_device_bytes.restype = C.c_size_t
    L.sffg_server_counts.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_double)]
    L.sffg_server_error.argtypes = [vp]
    L.sffg_server_error.restype = C.c_char_p
    L.sffg_server_destroy.argtypes = [vp]
    L._sffg_server_proto = True
    return L


class Server:
    """Requests wait in arrival order; every pump() admits those that fit
    the memory budget -- a minimisation into the running minimisation group
    (joining that batch at its next list-rebuild turn) or a new group, md
    requests as a new group -- launches `turns` evaluations or md
    steps of every group whose earlier turns have finished (the groups'
    work overlaps on the GPU), waits until one group's turns finish and
    takes the results of systems that ended."""

    def __init__(self, opts, memory_budget_gb=150.0, max_groups=8):
        self.L = _proto(sff.lib())
        self.h = C.c_void_p()
        rc = self.L.sffg_server_create(opts.encode(), memory_budget_gb, max_groups, C.byref(self.h))
        if rc != 0:
            raise ServerError(f"sffg_server_create: status {rc}")
        self.natoms = {}

    def _check(self, rc, what):
        if rc != 0:
            raise ServerError(f"{what}: status {rc}: {self.L.sffg_server_error(self.h).decode()}")

    def submit(self, prm, x, kind="minimize", nsteps=2000, rmsgrad=0.01):
        rid = C.c_longlong(0)
        x = np.ascontiguousarray(x, np.float64)
        self._check(self.L.sffg_server_submit(self.h, prm, sff.dptr(x), KINDS[kind], nsteps, rmsgrad,
                                              C.byref(rid)), "submit")
        self.natoms[rid.value] = sff.natom(prm)
        return rid.value

    def pump(self, turns=16):
        nr, npend = C.c_int(0), C.c_int(0)
        self._check(self.L.sffg_server_pump(self.h, turns, C.byref(nr), C.byref(npend)), "pump")
        return nr.value, npend.value

    def result(self, rid):
        """None while the request waits or runs; else a dict with its
        return code, energy, coordinates and latency in ms."""
        st, en, lat = C.c_int(0), C.c_double(0.0), C.c_double(0.0)
        x = np.zeros(3 * self.natoms[rid])
        rc = self.L.sffg_server_result(self.h, rid, C.byref(st), C.byref(en), sff.dptr(x), C.byref(lat))
        if rc == -4:
            return None
        self._check(rc, "result")
        return {"status": st.value, "energy": en.value, "x": x, "latency_ms": lat.value}

    def device_bytes(self):
        return self.L.sffg_server_device_bytes(self.h)

    def counts(self):
        """Groups started, joins, requests that joined a running group, and
        the host milliseconds spent forming batches."""
        v = [C.c_longlong(0) for _ in range(3)]
        ms = C.c_double(0.0)
        self._check(self.L.sffg_server_counts(self.h, *[C.byref(a) for a in v], C.byref(ms)), "counts")
        return {"groups_started": v[0].value, "joins": v[1].value, "joined_requests": v[2].value,
                "form_ms": ms.value}

    def run(self, turns=16):
        """Pumps until no request runs or waits."""
        while True:
            nr, npend = self.pump(turns)
            if nr == 0 and npend == 0:
                return

    def close(self):
        if self.h:
            self.L.sffg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

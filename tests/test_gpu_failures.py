"""GPU: failure isolation without any GPU fault.  A system whose
coordinates turn non-finite is reported and ends alone; every other system
of its batch, server group or batched minimisation gets the same bits it
gets without it.  The failure is made on the host (a NaN written into one
request's coordinates)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPTS = "gb=5, cut=999.0, rgbmax=20.0, nsnb=5, dt=0.001, gamma_ln=5.0, temp0=300.0"
ENONFINITE = -5


def molecules():
    from nabc_gb300 import sff
    return [sff.synth_molecule(n, 900 + k)[:2] for k, n in enumerate((400, 700, 300))]


def test_batch_status_isolates_nonfinite_system(lib):
    from nabc_gb300.batch import Batch
    mols = molecules()
    runs = []
    for poison in (False, True):
        b = Batch(OPTS)
        for k, (prm, x) in enumerate(mols):
            x = x.copy()
            if poison and k == 1:
                x[7] = np.nan
            b.add(prm, x)
        b.finalize()
        b.eval()
        runs.append((b.status(), [b.energy(s) for s in range(3)], [b.grad(s) for s in range(3)]))
        if poison:  # finite coordinates again (and fresh lists) clear the flag
            b.set_coords(1, mols[1][1])
            b.eval(rebuild=True)
            assert list(b.status()) == [0, 0, 0]
            # the poisoned system's atoms were ordered into tiles with the NaN
            # present, so its FP32 sums group differently: equal to 1e-7
            # (measured 2e-8; the parity bar against FP64 is 1e-6)
            e = b.energy(1)
            assert abs(e[0] - runs[0][1][1][0]) <= 1e-7 * abs(e[0])
        b.close()
    (st0, e0, g0), (st1, e1, g1) = runs
    assert list(st0) == [0, 0, 0]
    assert list(st1) == [0, ENONFINITE, 0]
    for s in (0, 2):
        assert np.array_equal(e0[s], e1[s]) and np.array_equal(g0[s], g1[s])


def test_server_ends_nonfinite_request_alone(lib):
    from nabc_gb300.server import Server
    mols = molecules()
    results = []
    for poison in (False, True):
        srv = Server(OPTS, memory_budget_gb=20.0, max_groups=2)
        ids = []
        for k, (prm, x) in enumerate(mols):
            x = x.copy()
            if poison and k == 1:
                x[7] = np.nan
            ids.append(srv.submit(prm, x, "minimize" if k != 2 else "md", 30, 0.05))
        srv.run(turns=5)
        results.append([srv.result(i) for i in ids])
        assert srv.device_bytes() == 0
        srv.close()
    clean, poisoned = results
    assert poisoned[1]["status"] == ENONFINITE
    for k in (0, 2):
        assert poisoned[k]["status"] == clean[k]["status"]
        assert poisoned[k]["energy"] == clean[k]["energy"]
        assert np.array_equal(poisoned[k]["x"], clean[k]["x"])


def test_batch_xmin_ends_nonfinite_system_alone(lib):
    from nabc_gb300.batch import Batch
    mols = molecules()
    b = Batch(OPTS)
    for k, (prm, x) in enumerate(mols):
        x = x.copy()
        if k == 1:
            x[4] = np.inf
        b.add(prm, x)
    b.finalize()
    st, it, en = b.xmin(method=2, maxiter=20, grms_tol=1e-3)
    b.close()
    assert st[1] == -7 and en[1] == 0.0
    assert st[0] == 0 and st[2] == 0 and it[0] == 20 and it[2] == 20


def test_mme_checkpoint_files(lib, tmp_path):
    """mm_set_checkpoint: mme() writes the coordinates every nchk iterations
    in the reference's Cartesian format, the name's %d replaced by the
    iteration number (or the number appended)."""
    import os
    from nabc_gb300 import sff
    prm, x = molecules()[0]
    n = prm.contents.Natom
    L = sff.lib()
    for tmpl, want in (("ck_%d.xyz", ["ck_2.xyz", "ck_4.xyz"]), ("ck_", ["ck_2", "ck_4"])):
        d = tmp_path / tmpl.replace("%d", "T")
        os.makedirs(d, exist_ok=True)
        session = sff.Session(prm, "gb=5, cut=999.0, rgbmax=20.0, nchk=2, ntpr=1000")
        name = C.c_char_p(str(d / tmpl).encode())
        L.mm_set_checkpoint(C.byref(name))
        g = np.zeros(3 * n)
        for k in range(1, 5):
            it = C.c_int(k)
            L.mme(sff.dptr(x), sff.dptr(g), C.byref(it))
        empty = C.c_char_p(b"")
        L.mm_set_checkpoint(C.byref(empty))
        del session
        assert sorted(os.listdir(d)) == want
        lines = open(d / want[0]).read().splitlines()
        assert int(lines[0]) == n and len(lines) == n + 1
        xyz = np.array([[float(line[20 * c:20 * (c + 1)]) for c in range(3)] for line in lines[1:]])
        np.testing.assert_allclose(xyz.ravel(), x, atol=1e-14)


def test_md_checkpoint_resume_bit_identical(lib, tmp_path):
    """Batched Langevin md saved after step 10 (a list-rebuild step,
    nsnb 5) and resumed in a new batch built from the same inputs repeats
    the uninterrupted run's coordinates and velocities bit for bit at step
    20; a state file of another batch is refused."""
    from nabc_gb300.batch import Batch
    from nabc_gb300 import sff
    mols = molecules()[:2]
    opts = "gb=5, cut=12.0, rgbmax=10.0, nsnb=5, dt=0.002, gamma_ln=5.0, temp0=300.0"

    def make():
        b = Batch(opts)
        for prm, x in mols:
            b.add(prm, x)
        b.finalize()
        return b

    b = make()
    b.md_begin()
    b.md_steps(0, 20)
    want = [(b.coords(s), b.velocities(s)) for s in range(2)]
    b.close()
    path = str(tmp_path / "md.state")
    b = make()
    b.md_begin()
    b.md_steps(0, 10)
    b.save(path)
    b.close()
    b = make()
    b.load(path)
    b.md_steps(10, 10)
    got = [(b.coords(s), b.velocities(s)) for s in range(2)]
    b.close()
    for (x1, v1), (x2, v2) in zip(want, got):
        assert np.array_equal(x1, x2) and np.array_equal(v1, v2)
    other = Batch(opts)
    prm, x = mols[0]
    other.add(prm, x)
    other.finalize()
    from nabc_gb300.batch import SffgError
    with pytest.raises(SffgError):
        other.load(path)
    other.close()

"""LMOD (nabc_gb300/csrc/lmod.cpp) against the reference's own search
(src/sff/lmodC.c compiled from source into oracle/_ref/lmodref) on the bead
chain of oracle/xmin_funcs.c.  Both call the same compiled chain function
and both take their low modes from the same Lanczos solver (the reference
through ref_shim/arpack_standin.cpp, as its Fortran ARPACK cannot be built
here), so everything else -- the random draws, ZIG-ZAG moves, barrier test,
Monte Carlo choice, archive pruning, restarts, ligand moves, the xmin()
minimisations -- must leave the same structures, conflib, trajectory,
conflib.dat and printout bit for bit.  The Lanczos solver itself is checked
against numpy's dense eigensolver.  No GPU is used."""
import ctypes as C

import numpy as np
import pytest

from nabc_gb300 import sff


@pytest.fixture(scope="module")
def funcs(oracle_mod):
    return oracle_mod.xmin_functions()


def lmod_cases(checks):
    return checks["lmod_chain"]["cases"]


def run_lmod(L, F, args, refrun, k, log_path):
    (n, frozen, niter, nmod, kmod, mc, nsteps, recalc, narn, restart, nbest, window, sep, nlig, ls, le, lc, pl,
     seed) = args
    C.c_int.in_dll(F, "xf_natom").value = n
    fr = (C.c_int * 64).in_dll(F, "xf_frozen")
    for i in range(64):
        fr[i] = 0
    if frozen >= 0:
        fr[frozen] = 1
    lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
    L.lmod_opt_init(C.byref(lo), C.byref(xo))
    lo.niter, lo.nmod, lo.kmod, lo.mc_option = niter, nmod, kmod, mc
    lo.nof_lmod_steps, lo.eig_recalc, lo.ndim_arnoldi = nsteps, recalc, narn
    lo.lmod_restart, lo.n_best_struct = restart, nbest
    lo.energy_window, lo.conf_separation_rms = window, sep
    lo.nlig, lo.print_level, lo.random_seed = nlig, pl, seed
    lo.apply_rigdock, lo.nof_poses_to_try = 2, 3
    xo.ls_maxatmov = 0.15
    x = refrun[f"lmod{k}_start"].copy()
    g = np.zeros_like(x)
    conflib = np.zeros(3 * n * lo.nconf)
    ntraj = niter + 1
    if pl == 5:
        ntraj = (4 * (nsteps or 20) + 3) * (niter * kmod + nmod + 2)
    traj = np.zeros(3 * n * ntraj)
    fn = C.cast(F.xf_chain, C.c_void_p)
    raw = sff.FUNC_T(fn.value)
    it = C.c_int(0)
    e = C.c_double(raw(sff.dptr(x), sff.dptr(g), C.byref(it)))
    ints = [C.c_int(v) for v in (n, ls, le, lc)]
    dbl = [C.c_double(v) for v in (0.5, 1.5, 10.0, 60.0)]
    previous = sff.set_output(str(log_path))
    try:
        ret = L.sffg_lmod_func(fn, C.byref(ints[0]), sff.dptr(x), sff.dptr(g), C.byref(e), sff.dptr(conflib),
                               sff.dptr(traj), C.byref(ints[1]), C.byref(ints[2]), C.byref(ints[3]),
                               C.byref(dbl[0]), C.byref(dbl[1]), C.byref(dbl[2]), C.byref(dbl[3]), C.byref(xo),
                               C.byref(lo))
    finally:
        sff.flush_output()
        sff.restore_output(previous)
    return ret, e.value, x, conflib[:3 * n * lo.nconf], traj, lo


@pytest.mark.parametrize("k", range(8))
def test_lmod_matches_reference_bitwise(lib, funcs, checks, refrun, k, tmp_path, monkeypatch):
    cases = lmod_cases(checks)
    if k >= len(cases):
        pytest.skip("no such golden case")
    case = cases[k]
    monkeypatch.chdir(tmp_path)
    for r in range(case["runs"]):  # a second run starts from the first one's conflib.dat
        ret, e, x, conflib, traj, lo = run_lmod(lib, funcs, case["args"], refrun, k, tmp_path / f"log{r}.txt")
    assert lo.error_flag == case["error_flag"] == 0
    assert lo.nconf == case["nconf"]
    assert lo.ndim_arnoldi == case["ndim_arnoldi"]
    ref_ret, ref_e = refrun[f"lmod{k}_scalars"]
    assert ret == ref_ret and e == ref_e
    np.testing.assert_array_equal(x, refrun[f"lmod{k}_x"])
    np.testing.assert_array_equal(conflib, refrun[f"lmod{k}_conflib"])
    np.testing.assert_array_equal(traj, refrun[f"lmod{k}_traj"])
    dat = np.frombuffer((tmp_path / "conflib.dat").read_bytes(), np.uint8)
    np.testing.assert_array_equal(dat, refrun[f"lmod{k}_conflib_dat"])
    log = (tmp_path / f"log{case['runs'] - 1}.txt").read_text()
    assert log == case["log"]


def test_lmod_parameter_errors(lib, funcs, tmp_path, monkeypatch, capfd):
    """The reference's parameter checks (lmodC.c:1733-1955): an invalid set
    returns 0 with error_flag -1 before any evaluation."""
    monkeypatch.chdir(tmp_path)
    calls = []

    @sff.FUNC_T
    def f(xp, gp, it):
        calls.append(1)
        return 0.0

    for field, value in (("kmod", 9), ("mc_option", 4), ("rtemp", 0.0), ("nconf", 0), ("print_level", 6)):
        lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
        lib.lmod_opt_init(C.byref(lo), C.byref(xo))
        setattr(lo, field, value)
        n = C.c_int(4)
        x = np.arange(12, dtype=np.float64)
        g = np.ones(12)
        conflib = np.zeros(12 * lo.nconf if lo.nconf > 0 else 12)
        traj = np.zeros(12 * (lo.niter + 1))
        e = C.c_double(0.0)
        z = C.c_int(0)
        d = C.c_double(0.0)
        ret = lib.sffg_lmod_func(C.cast(f, C.c_void_p), C.byref(n), sff.dptr(x), sff.dptr(g), C.byref(e),
                                 sff.dptr(conflib), sff.dptr(traj), C.byref(z), C.byref(z), C.byref(z), C.byref(d),
                                 C.byref(d), C.byref(d), C.byref(d), C.byref(xo), C.byref(lo))
        assert ret == 0.0 and lo.error_flag == -1, field
    assert not calls
    assert "ERROR in lmod()" in capfd.readouterr().err
    assert not (tmp_path / "conflib.dat").exists()


@pytest.mark.parametrize("n,nev,ncv", [(30, 5, 30), (30, 5, 12), (90, 11, 30), (120, 11, 120), (3, 1, 3)])
def test_low_modes_against_dense_eigensolver(lib, n, nev, ncv):
    """The Lanczos solver that replaces ARPACK (sffg_low_modes) against
    numpy.linalg.eigh: the nev eigenvalues of smallest magnitude, ascending,
    with orthonormal eigenvectors whose residual meets the relative bound
    tol (ARPACK's criterion), with (ncv < n) and without thick restarts.
    The operator has a cluster of small eigenvalues of both signs and
    near-zero ones, as a Hessian with its rotations and translations."""
    rng = np.random.default_rng(n * 100 + ncv)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    small = np.concatenate([[-0.3, 1e-7, -2e-7], np.linspace(0.02, 0.4, max(nev - 3, 0))])[:nev]
    w = np.concatenate([small, np.linspace(2.0, 60.0, n - nev)])
    A = (q * w) @ q.T
    A = 0.5 * (A + A.T)
    products = []

    @C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)
    def matvec(xp, yp, ctx):
        x = np.ctypeslib.as_array(xp, (n,))
        y = np.ctypeslib.as_array(yp, (n,))
        y[:] = A @ x
        products.append(1)

    tol = 1e-6
    vals = np.zeros(nev)
    vecs = np.zeros(nev * n)
    nconv = lib.sffg_low_modes(n, nev, ncv, tol, 100000, matvec, None, sff.dptr(vals), sff.dptr(vecs))
    assert nconv == nev
    ev = np.linalg.eigh(A)[0]
    want = np.sort(ev[np.argsort(np.abs(ev), kind="stable")[:nev]])
    assert np.all(np.diff(vals) >= 0)
    np.testing.assert_allclose(vals, want, rtol=0, atol=1e-6 * np.abs(ev).max())
    V = vecs.reshape(nev, n)
    np.testing.assert_allclose(V @ V.T, np.eye(nev), atol=1e-10)
    for lam, v in zip(vals, V):
        assert np.linalg.norm(A @ v - lam * v) <= 2 * tol * max(abs(lam), 2.31e-11) + 1e-12 * np.abs(ev).max()
    if ncv == n:
        assert len(products) == n  # one sweep spans the space


def test_lmodC_reverse_communication(lib, funcs, checks, refrun, tmp_path, monkeypatch):
    """lmodC() driven directly, with the reference's lmod() driver loop
    (lmodC.c:3366-3462) written out here over the chain function and this
    library's xmin(): the first golden search again, bit for bit, and the
    reference's labels (2-7 while running, 0 at the end)."""
    monkeypatch.chdir(tmp_path)
    case = checks["lmod_chain"]["cases"][0]
    (n, frozen, niter, nmod, kmod, mc, nsteps, recalc, narn, restart, nbest, window, sep, nlig, ls, le, lc, pl,
     seed) = case["args"]
    F = funcs
    C.c_int.in_dll(F, "xf_natom").value = n
    fr = (C.c_int * 64).in_dll(F, "xf_frozen")
    for i in range(64):
        fr[i] = 0
    lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
    lib.lmod_opt_init(C.byref(lo), C.byref(xo))
    lo.niter, lo.nmod, lo.kmod, lo.mc_option = niter, nmod, kmod, mc
    lo.nof_lmod_steps, lo.eig_recalc, lo.ndim_arnoldi = nsteps, recalc, narn
    lo.lmod_restart, lo.n_best_struct = restart, nbest
    lo.energy_window, lo.conf_separation_rms = window, sep
    lo.random_seed = seed
    lo.apply_rigdock, lo.nof_poses_to_try = 2, 3
    xo.ls_maxatmov = 0.15
    fn = C.cast(F.xf_chain, C.c_void_p)
    raw = sff.FUNC_T(fn.value)
    x = refrun["lmod0_start"].copy()
    g = np.zeros_like(x)
    conflib = np.zeros(3 * n * lo.nconf)
    traj = np.zeros(3 * n * (niter + 1))
    it = C.c_int(0)
    e = C.c_double(raw(sff.dptr(x), sff.dptr(g), C.byref(it)))
    nn = C.c_int(n)
    zi = C.c_int(0)
    zd = C.c_double(0.0)
    rf, label = C.c_int(0), C.c_int(0)
    grms = C.c_double(0.0)
    labels = set()
    for _ in range(100000):
        ret = lib.lmodC(C.byref(lo, type(lo).niter.offset), C.byref(lo, type(lo).nmod.offset),
                        C.byref(lo, type(lo).kmod.offset), C.byref(lo, type(lo).nrotran_dof.offset), C.byref(nn),
                        sff.dptr(x), C.byref(e), sff.dptr(g), C.byref(lo, type(lo).nconf.offset),
                        C.byref(lo, type(lo).energy_window.offset), C.byref(lo, type(lo).conf_separation_rms.offset),
                        sff.dptr(conflib), sff.dptr(traj), C.byref(lo, type(lo).eig_recalc.offset),
                        C.byref(lo, type(lo).ndim_arnoldi.offset), C.byref(lo, type(lo).lmod_restart.offset),
                        C.byref(lo, type(lo).n_best_struct.offset), C.byref(lo, type(lo).mc_option.offset),
                        C.byref(lo, type(lo).rtemp.offset), C.byref(lo, type(lo).lmod_step_size_min.offset),
                        C.byref(lo, type(lo).lmod_step_size_max.offset), C.byref(lo, type(lo).nof_lmod_steps.offset),
                        C.byref(lo, type(lo).nlig.offset), C.byref(zi), C.byref(zi),
                        C.byref(lo, type(lo).apply_rigdock.offset), C.byref(lo, type(lo).nof_poses_to_try.offset),
                        C.byref(zd), C.byref(zd), C.byref(zi), C.byref(zd), C.byref(zd),
                        C.byref(lo, type(lo).random_seed.offset), C.byref(lo, type(lo).print_level.offset),
                        C.byref(lo, type(lo).lmod_time.offset), C.byref(lo, type(lo).aux_time.offset), C.byref(rf),
                        C.byref(label))
        if rf.value == 0:
            break
        labels.add(label.value)
        if rf.value in (1, 2, 3, 4):
            it.value = -4 if rf.value <= 2 else -2
            e.value = raw(sff.dptr(x), sff.dptr(g), C.byref(it))
        else:
            if rf.value == 5:
                xo.grms_tol = lo.minim_grms
            elif rf.value == 6:
                xo.grms_tol = lo.lmod_relax_grms
            ev = np.array([e.value])
            e.value = lib.xmin(fn, C.byref(nn), sff.dptr(x), sff.dptr(g), sff.dptr(ev), C.byref(grms), C.byref(xo))
    assert label.value == 0 and rf.value == 0
    assert labels == {2, 3, 4, 5, 6}  # 7: the ligand minimisations, not used here
    assert ret == refrun["lmod0_scalars"][0]
    np.testing.assert_array_equal(x, refrun["lmod0_x"])
    np.testing.assert_array_equal(conflib[:3 * n * lo.nconf], refrun["lmod0_conflib"])
    np.testing.assert_array_equal(traj, refrun["lmod0_traj"])


def test_low_modes_rejects_inconsistent_sizes(lib):
    """nev < ncv <= n is required (ARPACK's dsaupd rule); anything else
    returns -1 without calling the operator."""
    calls = []

    @C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)
    def matvec(xp, yp, ctx):
        calls.append(1)

    vals, vecs = np.zeros(8), np.zeros(64)
    for n, nev, ncv in ((8, 4, 4), (8, 0, 4), (8, 4, 9), (0, 1, 2)):
        assert lib.sffg_low_modes(n, nev, ncv, 1e-4, 10, matvec, None, sff.dptr(vals), sff.dptr(vecs)) == -1
    assert not calls

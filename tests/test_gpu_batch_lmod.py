"""Batched LMOD (sffg_batch_lmod): every system of a batch runs the
reference's low-mode search, its evaluations and minimisations batched on
the GPU.

A one-system batch takes the legacy lmod()'s path bit for bit (same random
stream, same evaluations, same pair-list rebuild points): lowest energy,
conflib and final structure compared with ==.  Several systems together
are deterministic (two runs agree bit for bit), and each system's result is
checked against the energy function: its lowest energy is the energy of the
structure it returns, and every structure of its conflib is no lower."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

OPTS = "gb=1, cut=99.0, rgbmax=99.0, ntpr=100000"
LMOD = dict(niter=3, nmod=4, kmod=2, mc_option=2, nof_lmod_steps=3, conf_separation_rms=0.5, random_seed=7)
XMIN = dict(grms_tol=1e-3, maxiter=500, ls_maxatmov=0.15)
MOLECULES = [{"prmtop": "asp.top", "coords": "asp.pdb"}, {"prmtop": "NMA_scee+scnb.prmtop", "coords": "NMA.pdb"}]


def solo_lmod(prm, x, seed):
    from nabc_gb300 import sff
    L = sff.lib()
    session = sff.Session(prm, OPTS)
    n = prm.contents.Natom
    g = np.zeros(3 * n)
    it = C.c_int(-1)
    e = C.c_double(L.mme(sff.dptr(x), sff.dptr(g), C.byref(it)))
    lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
    L.lmod_opt_init(C.byref(lo), C.byref(xo))
    for k, v in LMOD.items():
        setattr(lo, k, v)
    lo.random_seed = seed
    for k, v in XMIN.items():
        setattr(xo, k, v)
    conflib = np.zeros(3 * n * lo.nconf)
    traj = np.zeros(3 * n * (lo.niter + 1))
    zi, zd, nn = C.c_int(0), C.c_double(0.0), C.c_int(n)
    ret = L.lmod(C.byref(nn), sff.dptr(x), sff.dptr(g), C.byref(e), sff.dptr(conflib), sff.dptr(traj),
                 C.byref(zi), C.byref(zi), C.byref(zi), C.byref(zd), C.byref(zd), C.byref(zd), C.byref(zd),
                 C.byref(xo), C.byref(lo))
    del session
    return ret, x, conflib[:3 * n * lo.nconf].reshape(lo.nconf, n, 3), lo.error_flag


def test_single_system_batch_equals_solo(lib, tmp_path, monkeypatch):
    from nabc_gb300.batch import Batch
    monkeypatch.chdir(tmp_path)  # the legacy search writes conflib.dat
    for mol in MOLECULES:
        prm, x = load_case(mol)
        b = Batch(OPTS)
        b.add(prm, x)
        b.finalize()
        st, gm, nc, conf = b.lmod(xmin_opts=XMIN, **LMOD)
        xb = b.coords(0)
        b.close()
        (tmp_path / "conflib.dat").unlink(missing_ok=True)
        ret, xs, cs, err = solo_lmod(prm, x.copy(), LMOD["random_seed"])
        assert st[0] == err == 0
        assert gm[0] == ret
        assert nc[0] == len(cs)
        assert np.array_equal(conf[0], cs)
        assert np.array_equal(xb, xs)


def test_batch_deterministic_and_consistent(lib):
    from nabc_gb300.batch import Batch
    mols = [load_case(m) for m in MOLECULES] + [load_case(MOLECULES[0])]  # asp twice: seeds 7 and 9
    runs = []
    for rep in range(2):
        b = Batch(OPTS)
        for prm, x in mols:
            b.add(prm, x)
        b.finalize()
        st, gm, nc, conf = b.lmod(xmin_opts=XMIN, **LMOD)
        xb = [b.coords(s) for s in range(len(mols))]
        # the energy function at each returned structure
        energies = []
        for s, (prm, _) in enumerate(mols):
            es = []
            for c in conf[s]:
                b.set_coords(s, c.ravel())
                b.eval(rebuild=True)
                es.append(b.energy(s)[0])
            energies.append(es)
        b.close()
        runs.append((st, gm, nc, conf, xb, energies))
    (st, gm, nc, conf, xb, energies), (st2, gm2, nc2, conf2, xb2, _) = runs
    assert np.array_equal(st, st2) and np.array_equal(gm, gm2) and np.array_equal(nc, nc2)
    assert all(np.array_equal(a, c) for a, c in zip(conf, conf2))
    assert all(np.array_equal(a, c) for a, c in zip(xb, xb2))
    for s in range(len(mols)):
        assert st[s] == 0 and nc[s] >= 1
        assert np.array_equal(xb[s], conf[s][0].ravel())
        # the lowest energy is the energy at the returned structure (1e-6
        # relative: a rebuilt list regroups the FP32 sums), and no conflib
        # structure is lower
        assert abs(energies[s][0] - gm[s]) <= 1e-6 * abs(gm[s])
        assert min(energies[s]) >= gm[s] - 1e-6 * abs(gm[s])


def test_nonfinite_system_ends_alone(lib):
    """A system whose energy is not finite (a NaN coordinate) ends with
    status -8 before its search starts; the others search as usual and
    give the same results as without it in the batch only up to rounding,
    so they are checked for status and consistency."""
    from nabc_gb300.batch import Batch
    prm_a, xa = load_case(MOLECULES[0])
    prm_n, xn = load_case(MOLECULES[1])
    bad = xn.copy()
    bad[4] = np.nan
    b = Batch(OPTS)
    b.add(prm_a, xa)
    b.add(prm_n, bad)
    b.finalize()
    st, gm, nc, conf = b.lmod(xmin_opts=XMIN, **LMOD)
    assert st[1] == -8 and nc[1] == 0
    assert st[0] == 0 and nc[0] >= 1 and np.isfinite(gm[0])
    np.testing.assert_array_equal(b.coords(0), conf[0][0].ravel())
    b.close()

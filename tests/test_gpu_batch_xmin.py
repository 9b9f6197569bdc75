"""Batched XMIN (sffg_batch_xmin): every system of a batch runs the
reference's minimiser with its evaluations batched on the GPU.

A one-system batch ends bit for bit where the legacy xmin() over mme() ends
(same evaluations, same pair-list rebuild points), compared with ==.  In a
batch of several systems, a list rebuild that one system's minimiser asks
for regroups every system's pair lists, which changes FP32 rounding in the
others: their runs stay deterministic (two runs agree bit for bit) and end
within the tolerance written below of their lone runs."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

OPTS = "gb=5, cut=999.0, rgbmax=15.0, ntpr=100000"


def solo_xmin(prm, x, frozen, **opts):
    from nabc_gb300 import sff
    L = sff.lib()
    session = sff.Session(prm, OPTS, frozen=frozen)
    n = prm.contents.Natom
    g = np.zeros(3 * n)
    it = C.c_int(-2)
    e = np.array([L.mme(sff.dptr(x), sff.dptr(g), C.byref(it))])
    xo = sff.XMIN_OPT_T()
    L.xmin_opt_init(C.byref(xo))
    for k, v in opts.items():
        setattr(xo, k, v)
    grms = np.zeros(1)
    nn = C.c_int(n)
    ret = L.xmin(C.cast(L.mme, C.c_void_p), C.byref(nn), sff.dptr(x), sff.dptr(g), sff.dptr(e), sff.dptr(grms),
                 C.byref(xo))
    del session
    return ret, x, xo.iter, xo.error_flag


def systems(checks):
    from nabc_gb300 import sff
    out = []
    for name in ("xfin", "gbrna"):
        prm, x = load_case(checks[name])
        out.append((prm, x, None))
    prm, x, _ = sff.synth_molecule(300, 5)
    frozen = np.zeros(300, np.int32)
    frozen[::7] = 1
    out.append((prm, x, frozen))
    return out


CASES = [dict(method=2, maxiter=40, grms_tol=1e-4, ls_maxatmov=0.15),
         dict(method=3, maxiter=8, grms_tol=1e-4),
         dict(method=1, maxiter=25, grms_tol=1e-4, ls_method=1)]


@pytest.mark.parametrize("opts", CASES)
def test_single_system_batch_equals_solo(lib, checks, opts):
    from nabc_gb300.batch import Batch
    for prm, x, frozen in systems(checks):
        b = Batch(OPTS)
        b.add(prm, x, frozen=frozen)
        b.finalize()
        st, it, en = b.xmin(**opts)
        xb = b.coords(0)
        b.close()
        ret, xs, iters, err = solo_xmin(prm, x.copy(), frozen, **opts)
        assert st[0] == err == 0
        assert it[0] == iters
        assert en[0] == ret
        assert np.array_equal(xb, xs)
        if frozen is not None:  # frozen atoms never move
            f = np.repeat(frozen.astype(bool), 3)
            assert np.array_equal(xb[f], x[f])


@pytest.mark.parametrize("opts", CASES)
def test_mixed_batch_deterministic_and_close_to_solo(lib, checks, opts):
    """Three systems together: two runs give the same bits; each system's
    final energy is within 1e-5 relative of its lone run for L-BFGS
    (measured: about 1e-6 after 40 iterations, the growth of FP32 rounding
    along a minimisation).  PRCG's conjugate directions carry a rounding
    difference further: its runs are required to end within 5e-4 (measured:
    1.0e-4 apart after 25 iterations; run on to a gradient of 0.1 the two
    paths ended in different nearby minima of xfin, 7e-5 apart).  TNCG's truncated CG amplifies any
    rounding difference into another path (its Hessian products are finite
    differences of gradients), so for it the runs are only required to end
    within 3% of each other, both far below the start (measured: 1.1%, the
    batched run lower)."""
    from nabc_gb300.batch import Batch
    sysl = systems(checks)
    runs = []
    for rep in range(2):
        b = Batch(OPTS)
        for prm, x, frozen in sysl:
            b.add(prm, x, frozen=frozen)
        b.finalize()
        st, it, en = b.xmin(**opts)
        runs.append((st, it, en, [b.coords(s) for s in range(len(sysl))]))
        b.close()
    (st, it, en, xb), (st2, it2, en2, xb2) = runs
    assert np.array_equal(st, st2) and np.array_equal(it, it2) and np.array_equal(en, en2)
    assert all(np.array_equal(a, c) for a, c in zip(xb, xb2))
    for s, (prm, x, frozen) in enumerate(sysl):
        ret, xs, iters, err = solo_xmin(prm, x.copy(), frozen, **opts)
        assert st[s] == err == 0
        tol = {1: 5e-4, 2: 1e-5, 3: 3e-2}[opts["method"]]
        assert abs(en[s] - ret) <= tol * abs(ret)


def test_reactivated_systems_get_their_lists(lib):
    """A system switched off by a batched minimiser while the pair list was
    rebuilt gets a fresh list before its next evaluation: after a batched
    minimisation with a finite cutoff in which one system ended first, a
    plain evaluation equals a rebuilt one for every system."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    opts = "gb=5, cut=12.0, rgbmax=10.0"
    prms = []
    small, xs, _ = sff.synth_molecule(200, 1)
    big, xb, _ = sff.synth_molecule(1500, 2)
    prms += [small, big]
    # the small molecule first minimised alone, so it ends at once below
    b = Batch(opts)
    b.add(small, xs)
    b.finalize()
    st, it, en = b.xmin(method=2, maxiter=3000, grms_tol=0.05)
    xs = b.coords(0)
    tol = 2.0 * np.sqrt((b.grad(0) ** 2).mean())  # above the small one's end, far below the big one's start
    b.close()
    b = Batch(opts)
    b.add(small, xs)
    b.add(big, xb)
    b.finalize()
    st, it, en = b.xmin(method=2, maxiter=30, grms_tol=tol)
    assert it[0] < it[1]  # one system ended while the other went on
    b.eval(rebuild=False)
    e0 = [b.energy(s) for s in range(2)]
    b.eval(rebuild=True)
    e1 = [b.energy(s) for s in range(2)]
    b.close()
    for a, c in zip(e0, e1):
        assert np.array_equal(a, c)
    for p in prms:
        sff.free_prm(p)

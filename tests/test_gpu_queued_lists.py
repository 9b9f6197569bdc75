"""Pair-list rebuilds without host round trips.

Inside mme() and device-resident md, a list rebuild launches all its stages
at once, with the list stores sized from the previous build's counts plus
50% headroom; the stages check the stores' capacities on the device, and a
store that proves too small empties the lists and raises a flag.  mme()
then evaluates again with the stores sized exactly; md replays the steps
taken since that rebuild from a snapshot of the state the rebuild step
started from.  These tests make a store too small on purpose -- the atoms
are moved 30% closer together between two rebuilds, which nearly triples
the pairs within the cutoff -- and check that the results are bit for bit
those of a run whose stores were sized for the moved atoms."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPTS = "gb=5, cut=12.0, rgbmax=10.0, nsnb=10, ntpr=100000"


def test_mme_redoes_an_overflowed_rebuild(lib):
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(3000, 61)
    xc = 0.7 * x
    s = sff.Session(prm, OPTS)
    s.mme(x.copy(), it=0)  # the first build, sized for x
    n0 = lib.sffg_list_overflows()
    e1, g1 = s.mme(xc.copy(), it=10)  # a rebuild at the moved atoms
    assert lib.sffg_list_overflows() > n0  # the stores sized for x were too small
    del s
    s = sff.Session(prm, OPTS)
    e2, g2 = s.mme(xc.copy(), it=0)  # a fresh session: sized for xc from the start
    del s
    assert e1 == e2
    assert np.array_equal(g1, g2)
    sff.free_prm(prm)


def test_md_replays_steps_after_an_overflowed_rebuild(lib):
    """Steps 1-9, then the atoms moved, then steps 10-13 (step 10 rebuilds
    the lists): once with the stores still sized for the old positions
    (the rebuild overflows and the steps are replayed) and once after an
    evaluation with a rebuild has sized them for the new ones."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    opts = OPTS + ", dt=0.001, gamma_ln=5.0, temp0=300.0"
    prm, x, _ = sff.synth_molecule(3000, 62)
    xc = 0.7 * x
    runs = []
    for sized in (False, True):
        b = Batch(opts)
        b.add(prm, x)
        b.finalize()
        b.md_begin()
        b.md_steps(0, 9)
        b.set_coords(0, xc)
        if sized:
            b.eval(rebuild=True)
        n0 = lib.sffg_list_overflows()
        b.md_steps(9, 4)
        xs, vs, es = b.coords(0), b.velocities(0), b.energy(0)
        runs.append((xs, vs, es, lib.sffg_list_overflows() - n0))
        b.close()
    (xa, va, ea, oa), (xb, vb, eb, ob) = runs
    assert oa >= 1 and ob == 0
    assert np.all(np.isfinite(xa))
    assert np.array_equal(xa, xb)
    assert np.array_equal(va, vb)
    assert np.array_equal(ea, eb)
    sff.free_prm(prm)

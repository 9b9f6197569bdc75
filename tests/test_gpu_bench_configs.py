"""GPU parity at the sizes the benchmark runs, against the FP64 oracle.

FP32 pair arithmetic loses accuracy as molecules grow (larger coordinates,
more terms per sum), so the 1e-6 relative energy and 1e-5 kcal/mol/A RMS
gradient bars are checked at the benchmark's own configurations:

  * a 25,000-atom molecule, gb=5 (OBC II), rgbmax 15, cut 25 -- the single
    large system, including evaluations on a list made at other coordinates
    (the md case between list rebuilds);
  * GBneck2 (gb=8), rgbmax 25, cut 30 -- the uneven batch's settings -- at
    200, 2,000 and 20,000 atoms (the ends and middle of its size range);
  * a 3,000-atom molecule and a perturbed conformer of it (sigma 0.3 A),
    gb=5, cut 999 -- the conformer batch;
  * a 50,000-atom molecule, gb=5, cut 999 -- the largest request size of
    the serving workload (1.25e9 pairs).

Every case also asserts the pair count of the reference's list.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_close, gpu_eval

pytestmark = pytest.mark.gpu


def check(oracle_mod, prm, x, opts):
    ene, g, reff, npairs = gpu_eval(prm, x, opts)
    o = oracle_mod.Oracle(prm, opts)
    e0, ene0, g0, reff0 = o.mme(x)
    assert npairs == o.npairs()
    assert_close(ene, g, reff, ene0, g0, reff0)
    return ene, ene0


def test_single_large_system_25k(lib, oracle_mod):
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(25000, 2025)
    check(oracle_mod, prm, x, "gb=5, rgbmax=15.0, cut=25.0, nsnb=10")
    sff.free_prm(prm)


def test_25k_between_list_builds(lib, oracle_mod):
    """The pair list made at x_a, evaluated at x_b = x_a + N(0, 0.2^2) per
    coordinate (atoms move ~0.35 A, past the distance that remakes the
    Born-radius lists of a tile): the reference keeps its list from x_a too
    (mme with iter % nsnb != 0), so both sides use the same pair set."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    opts = "gb=5, rgbmax=15.0, cut=25.0, nsnb=10"
    prm, xa, _ = sff.synth_molecule(25000, 2026)
    xb = xa + np.random.default_rng(7).normal(0.0, 0.2, xa.shape)
    b = Batch(opts)
    b.add(prm, xa)
    b.finalize()
    b.eval(rebuild=True)
    b.set_coords(0, xb)
    b.eval(rebuild=False)
    ene, g, reff = b.energy(0), b.grad(0), b.reff(0)
    b.close()
    o = oracle_mod.Oracle(prm, opts)
    o.mme(xa, rebuild=True)
    e0, ene0, g0, reff0 = o.mme(xb, rebuild=False)
    assert_close(ene, g, reff, ene0, g0, reff0)
    sff.free_prm(prm)


@pytest.mark.parametrize("natom", [200, 2000, 20000])
def test_uneven_batch_settings(lib, oracle_mod, natom):
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(natom, 9000 + natom)
    check(oracle_mod, prm, x, "gb=8, rgbmax=25.0, cut=30.0")
    sff.free_prm(prm)


def test_conformers_3k(lib, oracle_mod):
    from nabc_gb300 import sff
    prm, x0, _ = sff.synth_molecule(3000, 777)
    opts = "gb=5, cut=999.0"
    check(oracle_mod, prm, x0, opts)
    xc = x0 + np.random.default_rng(778).normal(0.0, 0.3, x0.shape)
    check(oracle_mod, prm, xc, opts)
    sff.free_prm(prm)


def test_largest_request_50k(lib, oracle_mod):
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(50000, 12000)
    check(oracle_mod, prm, x, "gb=5, cut=999.0")
    sff.free_prm(prm)

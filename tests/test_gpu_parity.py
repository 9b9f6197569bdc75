"""GPU parity: the sm_103a kernels against the FP64 oracle on the
reference's own test systems and on synthetic molecules.

Tolerances (the accuracy bar of this path): total energy within 1e-6 relative, every
component within 1e-6 of the total energy's magnitude (Coulomb and
Lennard-Jones totals are small differences of large terms, so their FP32
error scales with the system, not with the component), RMS gradient
difference within 1e-5 kcal/mol/A, effective Born radii within 2e-6
relative.  The arithmetic is FP32 per pair with 64-bit fixed-point sums, so
results are deterministic but not bitwise equal to FP64.
"""
import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

E_REL = 1e-6
G_RMS = 1e-5
REFF_REL = 2e-6

CASES = ["gbrna", "gbtrx", "gb5trx", "gb7trx", "gb8trx", "xfin", "s300_gb1", "s300_gb2", "s300_gb5",
         "s300_gb7", "s300_gb8", "s1000_gb5_cut", "s1000_gb8_cut", "s1000_gb1_kappa"]


def gpu_eval(prm, x, opts):
    from nabc_gb300.batch import Batch
    b = Batch(opts)
    b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True)
    out = b.energy(0), b.grad(0), b.reff(0), b.num_pairs(0)
    b.close()
    return out


def assert_close(ene, g, reff, ene0, g0, reff0, g_rms=G_RMS):
    assert abs(ene[0] - ene0[0]) <= E_REL * abs(ene0[0]), (ene[0], ene0[0])
    for k in (1, 2, 3, 4, 5, 7, 8, 10):
        assert abs(ene[k] - ene0[k]) <= E_REL * max(abs(ene0[k]), abs(ene0[0])), (k, ene[k], ene0[k])
    rms = np.sqrt(((g - g0) ** 2).mean())
    assert rms <= g_rms, rms
    if reff is not None:
        assert np.max(np.abs(reff / reff0 - 1.0)) <= REFF_REL


@pytest.mark.parametrize("name", CASES)
def test_energy_gradient_radii(lib, oracle_mod, checks, name):
    c = checks[name]
    prm, x = load_case(c)
    ene, g, reff, npairs = gpu_eval(prm, x, c["options"])
    o = oracle_mod.Oracle(prm, c["options"])
    e0, ene0, g0, reff0 = o.mme(x)
    assert npairs == o.npairs()
    assert_close(ene, g, reff, ene0, g0, reff0)


def test_gb8_radii_known_answer(lib, checks):
    """Per-atom GBneck2 radii of test/nab/aspgb8.out (7 significant digits)."""
    c = checks["aspgb8"]
    prm, x = load_case(c)
    ene, g, reff, _ = gpu_eval(prm, x, c["options"])
    assert np.abs(reff - np.array(c["reff"])).max() < 2e-6
    assert ene[10] == pytest.approx(c["sp"]["egb"], rel=1e-6)


@pytest.mark.parametrize("natom,opts", [
    (33, "gb=5, cut=999.0, rgbmax=15.0"),          # one full tile + one atom
    (64, "gb=1, cut=999.0, rgbmax=15.0"),          # exactly two tiles
    (97, "gb=8, cut=999.0, rgbmax=25.0"),
    (2000, "gb=1, cut=999.0, rgbmax=15.0"),        # the 2,000-atom all-pairs workload
    (3000, "gb=5, cut=25.0, rgbmax=15.0"),         # cutoff list with partial tile pairs
    # rgbmax below 2 max(s) / 0.3: rgbmax tails with q > 0.3 take the
    # logarithmic form instead of the polynomial one
    (520, "gb=5, cut=20.0, rgbmax=6.0"),
    (520, "gb=1, cut=20.0, rgbmax=6.0"),
    (520, "gb=8, cut=20.0, rgbmax=6.0"),
])
def test_sizes_and_lists(lib, oracle_mod, natom, opts):
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(natom, 100 + natom)
    ene, g, reff, npairs = gpu_eval(prm, x, opts)
    o = oracle_mod.Oracle(prm, opts)
    e0, ene0, g0, reff0 = o.mme(x)
    assert npairs == o.npairs()
    assert_close(ene, g, reff, ene0, g0, reff0)
    sff.free_prm(prm)


def test_frozen_atoms(lib, oracle_mod):
    """Frozen atoms: no pairs between two frozen atoms, no diagonal or chain
    row for them, zero gradient (eff.c:1884, 2203, 2826-2834)."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    prm, x, _ = sff.synth_molecule(400, 5)
    frozen = np.zeros(400, np.int32)
    frozen[::3] = 1
    opts = "gb=5, cut=16.0, rgbmax=12.0"
    b = Batch(opts)
    b.add(prm, x, frozen=frozen)
    b.finalize()
    b.eval(rebuild=True)
    ene, g, reff = b.energy(0), b.grad(0), b.reff(0)
    o = oracle_mod.Oracle(prm, opts, frozen=frozen)
    e0, ene0, g0, reff0 = o.mme(x)
    assert b.num_pairs(0) == o.npairs()
    assert_close(ene, g, reff, ene0, g0, reff0)
    assert np.all(g.reshape(-1, 3)[frozen == 1] == 0.0)
    b.close()


def test_deterministic(lib, checks):
    """Fixed-point accumulation: repeated evaluations are bit-identical."""
    c = checks["gb5trx"]
    prm, x = load_case(c)
    from nabc_gb300.batch import Batch
    b = Batch(c["options"])
    b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True)
    e1, g1 = b.energy(0), b.grad(0)
    for _ in range(3):
        b.eval(rebuild=True)
        assert np.array_equal(b.energy(0), e1)
        assert np.array_equal(b.grad(0), g1)
    b.close()


@pytest.mark.parametrize("gbk", [1, 5, 8])
def test_single_ion(lib, oracle_mod, checks, gbk):
    """One atom (Na+): a tile holding a single atom, no pairs at all; the
    Born self-energy of the compiled reference and the oracle, zero
    gradient."""
    c = checks[f"na_gb{gbk}"]
    prm, x = load_case(c)
    ene, g, reff, npairs = gpu_eval(prm, x, c["options"])
    assert npairs == 0
    assert ene[0] == pytest.approx(c["sp"]["Total"], rel=E_REL)
    assert ene[10] == pytest.approx(c["sp"]["egb"], rel=E_REL)
    assert np.all(g == 0.0)
    o = oracle_mod.Oracle(prm, c["options"])
    e0, ene0, g0, reff0 = o.mme(x)
    assert_close(ene, g, reff, ene0, g0, reff0)


@pytest.mark.parametrize("natom", [4, 5, 8, 12, 31, 32])
def test_tiny_molecules(lib, oracle_mod, natom):
    """Tiny synthetic molecules (one partial or exactly full tile, most
    pairs excluded as 1-2/1-3 neighbours) for each GB model, against the
    oracle.  These compact chains have steep repulsive contacts (gradients
    up to 67 kcal/mol/A for 12 atoms), where FP32 rounding of the r^-12 term
    is ~5e-7 of the component, so the gradient bar here is the larger of
    1e-5 kcal/mol/A and 1e-6 of the gradient's RMS (measured worst: 1.0e-5
    against an RMS gradient of 21)."""
    from nabc_gb300 import sff
    prm, x, _ = sff.synth_molecule(natom, 40 + natom)
    for opts in ("gb=1, cut=999.0, rgbmax=15.0", "gb=5, cut=999.0, rgbmax=15.0, kappa=0.1",
                 "gb=8, cut=999.0, rgbmax=25.0"):
        ene, g, reff, npairs = gpu_eval(prm, x, opts)
        o = oracle_mod.Oracle(prm, opts)
        e0, ene0, g0, reff0 = o.mme(x)
        assert npairs == o.npairs()
        assert_close(ene, g, reff, ene0, g0, reff0, g_rms=max(G_RMS, 1e-6 * np.sqrt((g0 ** 2).mean())))
    sff.free_prm(prm)

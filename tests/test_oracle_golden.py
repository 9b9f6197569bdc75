"""The CPU oracle (oracle/sffo.c) against the reference's own outputs:
its shipped .check files and runs of the reference library compiled from
source (tests/golden/refrun.npz).  These pin the oracle that every GPU
parity test uses."""
import numpy as np
import pytest

from conftest import load_case

REF_CG = ["gbrna", "gbtrx", "gb5trx", "gb7trx", "gb8trx"]
SYNTH = ["s300_gb1", "s300_gb2", "s300_gb5", "s300_gb7", "s300_gb8", "s1000_gb5_cut", "s1000_gb8_cut",
         "s1000_gb1_kappa"]
KEYS = {"bond": 3, "angle": 4, "dihedral": 5, "enb14": 7, "eel14": 8, "enb": 1, "eel": 2, "egb": 10,
        "Total": 0}


@pytest.mark.parametrize("name", REF_CG)
def test_conjgrad_trace_matches_check_file(lib, oracle_mod, checks, name):
    """11 conjgrad evaluations reproduce the reference's ff: totals."""
    c = checks[name]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    n = prm.contents.Natom
    ret, f, xo, etrace = o.conjgrad(x, 3 * n * 0.0001, 10.0, 10)
    assert ret == c["conjgrad_returns"]
    want = [row[1] for row in c["ff"]]
    assert len(etrace) == len(want)
    assert [round(e, 2) for e in etrace] == pytest.approx(want, abs=0.006)


@pytest.mark.parametrize("name", REF_CG + SYNTH + ["xfin"])
def test_single_point_matches_reference(lib, oracle_mod, checks, refrun, name):
    c = checks[name]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    e, ene, g, reff = o.mme(x)
    for k, idx in KEYS.items():
        assert ene[idx] == pytest.approx(c["sp"][k], abs=2e-9 + 1e-12 * abs(c["sp"][k])), k
    frms = np.sqrt((g * g).mean())
    assert frms == pytest.approx(c["sp"]["frms"], abs=2e-9)
    if f"{name}_g" in refrun:
        gref = refrun[f"{name}_g"]
        assert np.sqrt(((g - gref) ** 2).mean()) < 1e-10 * max(1.0, np.sqrt((gref ** 2).mean()))


def test_gb8_born_radii(lib, oracle_mod, checks):
    c = checks["aspgb8"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    e, ene, g, reff = o.mme(x)
    assert np.round(reff, 7) == pytest.approx(np.array(c["reff"]), abs=1.01e-7)
    assert ene[10] == pytest.approx(c["sp"]["egb"], abs=2e-9)


def test_synthetic_conjgrad(lib, oracle_mod, checks, refrun):
    c = checks["s300_cg"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    ret, f, xo, etrace = o.conjgrad(x, c["rmsgrad"], c["dfpred"], c["maxiter"])
    assert ret == c["conjgrad_returns"]
    assert f == pytest.approx(c["energy"], rel=1e-12)
    assert np.abs(xo - refrun["s300_cg_x"]).max() < 1e-9


def test_synthetic_langevin_md(lib, oracle_mod, checks, refrun):
    """20 Langevin steps with the reference's serial noise stream."""
    c = checks["s300_md"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    xo, vo, trace = o.md(x, np.zeros_like(x), c["nsteps"], seed=-1)
    assert np.abs(xo - refrun["s300_md_x"]).max() < 1e-9
    assert np.abs(vo - refrun["s300_md_v"]).max() < 1e-9
    md = np.array(c["md"])
    assert trace[:, 0] == pytest.approx(md[:, 2], abs=0.006)   # ekin column (%10.2f)
    assert trace[:, 1] == pytest.approx(md[:, 3], abs=0.006)   # epot column


def test_planted_error_is_detected(lib, oracle_mod, checks, refrun):
    """A deliberately wrong oracle configuration (rgbmax off by 1%) must fail
    the comparison that the GPU parity tests rely on."""
    c = checks["s300_gb5"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"].replace("rgbmax=15.0", "rgbmax=15.15"))
    e, ene, g, reff = o.mme(x)
    assert abs(ene[10] - c["sp"]["egb"]) / abs(c["sp"]["egb"]) > 1e-6


@pytest.mark.parametrize("name", ["s300_md_nscm", "s300_md_nscm_vw"])
def test_md_centre_of_mass_removal(lib, oracle_mod, checks, refrun, name):
    """md with nscm: the reference removes the centre-of-mass translation
    (Langevin) and also its velocity and rotation (Berendsen, tempi start)."""
    c = checks[name]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    xo, vo, trace = o.md(x, np.zeros_like(x), c["nsteps"], seed=-1)
    assert np.abs(xo - refrun[f"{name}_x"]).max() < 1e-9
    assert np.abs(vo - refrun[f"{name}_v"]).max() < 1e-9
    md = np.array(c["md"])
    assert trace[:, 0] == pytest.approx(md[:, 2], abs=0.006)


def restraint_inputs(c, x):
    n = len(x) // 3
    constrained = np.zeros(n, np.int32)
    constrained[::c["every"]] = 1
    x0 = x + c["shift"] * (np.arange(3 * n) % 5 - 2)
    return constrained, x0


def test_positional_restraints(lib, oracle_mod, checks, refrun):
    """econs: the restraint energy and gradient of the reference (eff.c:17)."""
    c = checks["s300_cons"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    o.set_restraints(*restraint_inputs(c, x))
    e, ene, g, _ = o.mme(x)
    assert ene[9] == pytest.approx(c["sp"]["econs"], abs=1e-9)
    assert e == pytest.approx(c["energy"], rel=1e-12)
    assert np.abs(g - refrun["s300_cons_g"]).max() < 1e-8

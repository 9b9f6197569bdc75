"""GPU: batches, the legacy drop-in entry points (mme / conjgrad / md) and
the minimiser and integrator against the oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_path, load_case

pytestmark = pytest.mark.gpu


def test_batch_equals_individual(lib):
    """A system's result is bit-identical alone and inside a mixed batch."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    opts = "gb=5, cut=30.0, rgbmax=25.0"
    mols = [sff.synth_molecule(n, 40 + n) for n in (150, 700, 1234, 64)]
    alone = []
    for prm, x, _ in mols:
        b = Batch(opts)
        b.add(prm, x)
        b.finalize()
        b.eval(rebuild=True)
        alone.append((b.energy(0), b.grad(0)))
        b.close()
    b = Batch(opts)
    for prm, x, _ in mols:
        b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True)
    for s, (e, g) in enumerate(alone):
        assert np.array_equal(b.energy(s), e)
        assert np.array_equal(b.grad(s), g)
    b.close()


def test_batch_mixed_screens_equals_individual(lib, oracle_mod):
    """Systems with different screened radii in one batch.  Each system's
    rgbmax + Fsmax cutoff (eff.c:1520), its list-B radius and the form of
    its rgbmax tails follow its own atoms, so a system's result is
    bit-identical alone and batched with a system of larger screens, and
    each matches the FP64 oracle.  With rgbmax 10 the plain molecule's
    largest screened radius (1.28 A) lets every tail take the polynomial
    form; the scaled one's (1.79 A) does not."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    from test_gpu_parity import assert_close
    opts = "gb=5, cut=30.0, rgbmax=10.0"
    mols = [sff.synth_molecule(n, 900 + n) for n in (300, 520)]
    prm1 = mols[1][0]
    n1 = prm1.contents.Natom
    fs = np.ctypeslib.as_array(prm1.contents.Fs, shape=(n1,))
    rb = np.ctypeslib.as_array(prm1.contents.Rborn, shape=(n1,))
    fs *= 1.4
    prm1.contents.Fsmax = float(np.max(fs * (rb - 0.09)))
    assert prm1.contents.Fsmax > mols[0][0].contents.Fsmax + 0.4
    alone = []
    for prm, x, _ in mols:
        b = Batch(opts)
        b.add(prm, x)
        b.finalize()
        b.eval(rebuild=True)
        alone.append((b.energy(0), b.grad(0)))
        b.close()
        o = oracle_mod.Oracle(prm, opts)
        e0, ene0, g0, reff0 = o.mme(x)
        assert_close(alone[-1][0], alone[-1][1], None, ene0, g0, reff0)
    for order in ((0, 1), (1, 0)):
        b = Batch(opts)
        for k in order:
            b.add(mols[k][0], mols[k][1])
        b.finalize()
        b.eval(rebuild=True)
        for s, k in enumerate(order):
            assert np.array_equal(b.energy(s), alone[k][0])
            assert np.array_equal(b.grad(s), alone[k][1])
        b.close()
    for prm, _, _ in mols:
        sff.free_prm(prm)


def test_legacy_mme_matches_oracle(lib, oracle_mod, checks):
    """mm_options + mme_init_sff + mme(iter=-1), the reference's drop-in path."""
    from nabc_gb300 import sff
    c = checks["gb8trx"]
    prm, x = load_case(c)
    s = sff.Session(prm, c["options"])
    e, g = s.mme(x, it=-1)
    prm2, _ = load_case(c)
    o = oracle_mod.Oracle(prm2, c["options"])
    e0, ene0, g0, _ = o.mme(x)
    assert abs(e - e0) <= 1e-6 * abs(e0)
    assert np.sqrt(((g - g0) ** 2).mean()) <= 1e-5


@pytest.mark.parametrize("name", ["gbrna", "gb5trx", "gb8trx"])
def test_legacy_conjgrad_matches_check(lib, checks, name):
    """conjgrad(..., mme, ...) reproduces the reference's 11 ff: totals
    (printed with two decimals) and return code."""
    from nabc_gb300 import sff
    c = checks[name]
    prm, x = load_case(c)
    session = sff.Session(prm, c["options"])  # keeps the borrowed frozen/constrained arrays alive
    L = sff.lib()
    n = C.c_int(3 * prm.contents.Natom)
    f = C.c_double(0.0)
    rms = C.c_double(3 * prm.contents.Natom * 0.0001)
    dfp = C.c_double(10.0)
    maxit = C.c_int(10)
    ret = L.conjgrad(sff.dptr(x), C.byref(n), C.byref(f), C.cast(L.mme, C.c_void_p), C.byref(rms),
                     C.byref(dfp), C.byref(maxit))
    assert ret == c["conjgrad_returns"]
    assert f.value == pytest.approx(c["ff"][-1][1], abs=0.011)
    del session


def test_batched_conjgrad_matches_oracle(lib, oracle_mod, checks, refrun):
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    c = checks["s300_cg"]
    prm, x = load_case(c)
    b = Batch(c["options"])
    b.add(prm, x)
    b.add(prm, x + 0.01)
    b.finalize()
    st, en = b.cg(c["maxiter"], c["rmsgrad"], c["dfpred"])
    assert st[0] == c["conjgrad_returns"]
    assert en[0] == pytest.approx(c["energy"], rel=1e-6)
    o = oracle_mod.Oracle(prm, c["options"])
    ret, f1, x1, _ = o.conjgrad(x + 0.01, c["rmsgrad"], c["dfpred"], c["maxiter"])
    assert st[1] == ret
    assert en[1] == pytest.approx(f1, rel=1e-6)
    b.close()


def test_legacy_md_reference_noise(lib, oracle_mod, checks, refrun):
    """md(..., mme) on the device with the reference's noise stream tracks
    the reference trajectory (20 Langevin steps)."""
    from nabc_gb300 import sff
    c = checks["s300_md"]
    prm, x = load_case(c)
    session = sff.Session(prm, c["options"])
    L = sff.lib()
    seed = C.c_int(-1)
    L.setseed(C.byref(seed))
    n = 3 * prm.contents.Natom
    v = np.zeros(n)
    f = np.zeros(n)
    L.md(n, c["nsteps"], sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
    assert np.abs(x - refrun["s300_md_x"]).max() < 1e-5
    assert np.abs(v - refrun["s300_md_v"]).max() < 1e-4
    del session


def test_graph_replay_bit_identical(lib):
    """md steps and evaluations replayed from captured CUDA graphs give the
    same bits as direct launches (list rebuilds, list-B remakes and the
    Philox step counter included)."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    prm, x, _ = sff.synth_molecule(3000, 77)
    out = []
    for graph in (0, 1):
        b = Batch(f"gb=5, cut=20.0, rgbmax=12.0, nsnb=5, dt=0.002, gamma_ln=5.0, temp0=300.0, sffg_graph={graph}")
        b.add(prm, x)
        b.finalize()
        b.md_begin()
        for step in range(23):
            b.md_steps(step, 1)
        b.eval()
        out.append((b.coords(0), b.velocities(0), b.energy(0), b.grad(0)))
        b.close()
    for u, v in zip(out[0], out[1]):
        assert np.array_equal(u, v)
    sff.free_prm(prm)


def test_lj_table_shared_and_global_bit_identical(lib, checks):
    """Pass 2 reads the Lennard-Jones table from shared memory when it is
    small (sffg_lj_shared=1) and from global memory otherwise; both give the
    same bits, on a batch of the reference's test systems with kappa and
    without."""
    from nabc_gb300.batch import Batch
    out = []
    for kappa in (0.0, 0.10395):
        for ljs in (1, 0):
            b = Batch(f"gb=5, cut=99.0, rgbmax=15.0, kappa={kappa}, sffg_lj_shared={ljs}")
            prms = []
            for name in ("gbrna", "gbtrx", "xfin"):
                prm, x = load_case(checks[name])
                prms.append(prm)
                b.add(prm, x)
            b.finalize()
            b.eval()
            out.append([(b.energy(s), b.grad(s)) for s in range(3)])
            b.close()
    for a, c in ((out[0], out[1]), (out[2], out[3])):
        for (e1, g1), (e2, g2) in zip(a, c):
            assert np.array_equal(e1, e2) and np.array_equal(g1, g2)


def test_autotuned_split_bit_identical(lib):
    """The autotuner picks the work split of each pass by timing; the
    results are the same bits with or without it."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    prm, x, _ = sff.synth_molecule(22000, 31)
    res = []
    for tune in (0, 1):
        b = Batch(f"gb=5, cut=20.0, rgbmax=15.0, sffg_tune={tune}")
        b.add(prm, x)
        b.finalize()
        b.eval(rebuild=True)
        b.eval()
        res.append((b.energy(0), b.grad(0), b.tuned_split()))
        b.close()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    for claim, blocks in res[1][2]:
        assert claim in (1, 2, 4, 8) and blocks > 0
    sff.free_prm(prm)


def test_positional_restraints(lib, oracle_mod, checks, refrun):
    """econs on the device, through the batch API and through mme_init_sff's
    constrained/x0 arguments, against the reference's run."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    from test_oracle_golden import restraint_inputs
    c = checks["s300_cons"]
    prm, x = load_case(c)
    cons, x0 = restraint_inputs(c, x)
    b = Batch(c["options"])
    b.add(prm, x, constrained=cons, x0=x0)
    b.finalize()
    b.eval(rebuild=True)
    ene, g = b.energy(0), b.grad(0)
    b.close()
    assert ene[9] == pytest.approx(c["sp"]["econs"], abs=1e-8)
    assert abs(ene[0] - c["energy"]) <= 1e-6 * abs(c["energy"])
    assert np.sqrt(((g - refrun["s300_cons_g"]) ** 2).mean()) <= 1e-5
    L = sff.lib()
    L.sffg_options_reset()
    L.mm_options(c["options"].encode())
    frozen = np.zeros(len(cons), np.int32)
    L.mme_init_sff(prm, sff.iptr(frozen), sff.iptr(cons), sff.dptr(x0), None)
    gl = np.zeros_like(x)
    it = C.c_int(-1)
    e = L.mme(sff.dptr(x), sff.dptr(gl), C.byref(it))
    assert abs(e - c["energy"]) <= 1e-6 * abs(c["energy"])
    assert np.sqrt(((gl - refrun["s300_cons_g"]) ** 2).mean()) <= 1e-5


@pytest.mark.parametrize("name", ["s300_md_nscm", "s300_md_nscm_vw"])
def test_legacy_md_centre_of_mass_removal(lib, checks, refrun, name):
    """md(..., mme) with nscm on the device tracks the reference trajectory
    (translation removal under Langevin; translation, velocity and rotation
    under Berendsen from tempi velocities)."""
    from nabc_gb300 import sff
    c = checks[name]
    prm, x = load_case(c)
    session = sff.Session(prm, c["options"])
    L = sff.lib()
    seed = C.c_int(-1)
    L.setseed(C.byref(seed))
    n = 3 * prm.contents.Natom
    v = np.zeros(n)
    f = np.zeros(n)
    L.md(n, c["nsteps"], sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
    assert np.abs(x - refrun[f"{name}_x"]).max() < 1e-5
    assert np.abs(v - refrun[f"{name}_v"]).max() < 1e-4
    del session


@pytest.mark.parametrize("name", ["s300_md_rattle2", "s300_md_rattle1"])
def test_legacy_md_rattle(lib, checks, refrun, name):
    """md with RATTLE bond constraints (rattle=2: bonds to hydrogen, rattle=1:
    all bonds) at dt = 2 fs tracks the reference's trajectory."""
    from nabc_gb300 import sff
    c = checks[name]
    prm, x = load_case(c)
    session = sff.Session(prm, c["options"])
    L = sff.lib()
    seed = C.c_int(-1)
    L.setseed(C.byref(seed))
    n = 3 * prm.contents.Natom
    v = np.zeros(n)
    f = np.zeros(n)
    L.md(n, c["nsteps"], sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
    assert np.abs(x - refrun[f"{name}_x"]).max() < 1e-5
    assert np.abs(v - refrun[f"{name}_v"]).max() < 1e-4
    del session


def test_mme_rattle(lib, checks, refrun):
    """mme_rattle restores the bond lengths, then projects the gradient onto
    the constraints, as the reference does."""
    from nabc_gb300 import sff
    c = checks["s300_rattle_sp"]
    prm, x = load_case(c)
    x = x + c["shift"] * (np.arange(len(x)) % 3 - 1)
    session = sff.Session(prm, c["options"])
    L = sff.lib()
    g = np.zeros_like(x)
    it = C.c_int(-1)
    e = L.mme_rattle(sff.dptr(x), sff.dptr(g), C.byref(it))
    assert np.abs(x - refrun["s300_rattle_sp_x"]).max() < 1e-12
    assert abs(e - c["energy"]) <= 1e-6 * abs(c["energy"])
    assert np.sqrt(((g - refrun["s300_rattle_sp_g"]) ** 2).mean()) <= 1e-5
    del session


def test_tmd_check_file(lib, checks, tmp_path):
    """The reference's md test (test/tmd.c: xfin.md1.rst7, gb=1, cut 20,
    Langevin at 300 K with the reference's noise stream, rattle=1, 500 steps)
    against its shipped tmd.out.check: every ff: and md: line (steps 0, 1,
    100, ..., 500) to the printed digits (0.01), which the FP32 pair
    arithmetic holds over the whole run."""
    import os
    from nabc_gb300 import sff
    c = checks["tmd"]
    prm, x = load_case(c)
    n = prm.contents.Natom
    _, v = sff.getxv(golden_path(c["coords"]), n)
    session = sff.Session(prm, c["options"])
    L = sff.lib()
    seed = C.c_int(-1)
    L.setseed(C.byref(seed))
    out = str(tmp_path / "tmd.out")
    sff.set_output(out)
    try:
        f = np.zeros(3 * n)
        L.md(3 * n, c["nsteps"], sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
        sff.flush_output()
    finally:
        sff.set_output(os.devnull)
    del session
    text = open(out).read()
    ff = [[float(t) for t in line.split()[1:]] for line in text.splitlines() if line.startswith("ff:")]
    md = [[float(t) for t in line.split()[1:]] for line in text.splitlines() if line.startswith("md:")]
    print("ff", ff)
    print("md", md)
    assert len(md) == len(c["md"]) and len(ff) == len(c["ff"])
    for got, want in zip(ff, c["ff"]):
        assert got[:7] == pytest.approx(want[:7], abs=0.011)
        assert got[7] == pytest.approx(want[7], rel=0.01)  # frms, printed with 3 digits
    for got, want in zip(md, c["md"]):
        assert got == pytest.approx(want, abs=0.011)


def test_md_trajectory_device_path(lib, tmp_path):
    """md() through the device-resident path writes its Amber NetCDF frames
    from device state: every ntwx steps, the last frame equal to the final
    structure in single precision, and a frame that falls on an nscm step
    taken before the centre-of-mass removal (sff.c:2341-2351)."""
    from scipy.io import netcdf_file
    from nabc_gb300 import sff
    prm = sff.rdparm(golden_path("xfin.parm7"))
    n = prm.contents.Natom
    x, _ = sff.getxv(golden_path("xfin.rst7"), n)
    L = sff.lib()
    for nscm, nsteps in ((0, 20), (10, 20)):
        L.sffg_options_reset()
        L.mm_options(f"gb=1, cut=99.0, rgbmax=15.0, ntwx=5, ntpr_md=5, nscm={nscm}, gamma_ln=5.0, "
                     "temp0=300.0, zerov=1, dt=0.001".encode())
        frozen = np.zeros(n, np.int32)
        cons = np.zeros(n, np.int32)
        path = str(tmp_path / f"md{nscm}.nc")
        L.mme_init_sff(prm, sff.iptr(frozen), sff.iptr(cons), None, path.encode())
        xx = x.copy()
        v = np.zeros(3 * n)
        f = np.zeros(3 * n)
        L.md(3 * n, nsteps, sff.dptr(xx), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
        nc = netcdf_file(path, "r", mmap=False)
        coords = nc.variables["coordinates"][:].astype(np.float64)
        times = nc.variables["time"][:].copy()
        nc.close()
        assert coords.shape == (nsteps // 5, n, 3)
        np.testing.assert_allclose(times, 0.005 * np.arange(1, nsteps // 5 + 1), rtol=1e-6)
        if nscm == 0:
            np.testing.assert_array_equal(coords[-1].ravel(), xx.astype(np.float32).astype(np.float64))
        else:
            shift = coords[-1] - xx.reshape(n, 3)
            assert np.abs(shift - shift.mean(0)).max() < 1e-4
            assert np.abs(shift.mean(0)).max() > 1e-6


def run_legacy_md(c, tmp_path, ncname=None):
    """md() through the legacy API on the case's structure with the
    reference's noise stream from its default seed; returns the printed ff:
    and md: rows."""
    import os
    from nabc_gb300 import sff
    prm, x = load_case(c)
    n = prm.contents.Natom
    L = sff.lib()
    L.sffg_options_reset()
    L.mm_options(c["options"].encode())
    frozen = np.zeros(n, np.int32)
    cons = np.zeros(n, np.int32)
    L.mme_init_sff(prm, sff.iptr(frozen), sff.iptr(cons), None, ncname.encode() if ncname else None)
    seed = C.c_int(-1)
    L.setseed(C.byref(seed))
    out = str(tmp_path / "md.out")
    sff.set_output(out)
    try:
        v = np.zeros(3 * n)
        f = np.zeros(3 * n)
        L.md(3 * n, c["nsteps"], sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(L.mme, C.c_void_p))
        sff.flush_output()
    finally:
        sff.set_output(os.devnull)
    text = open(out).read()
    ff = [[float(t) for t in line.split()[1:]] for line in text.splitlines() if line.startswith("ff:")]
    md = [[float(t) for t in line.split()[1:]] for line in text.splitlines() if line.startswith("md:")]
    return ff, md


@pytest.mark.parametrize("name", ["nab_rattle_md", "nab_gbnetcdf"])
def test_nab_md_check_files(lib, checks, tmp_path, name):
    """The reference's test/nab/rattle_md.nab (gbrna, gb=1 with kappa,
    velocities drawn at tempi 300 K, rattle=1, 20 steps) and gbnetcdf.nab
    (the same for 100 steps with rgbmax 25 and a NetCDF frame every 10
    steps) against their shipped .out.check: every ff: and md: line to the
    printed digits; the trajectory holds the 10 frames."""
    from scipy.io import netcdf_file
    c = checks[name]
    nc = str(tmp_path / "gbtrj.nc") if name == "nab_gbnetcdf" else None
    ff, md = run_legacy_md(c, tmp_path, nc)
    assert len(ff) == len(c["ff"]) and len(md) == len(c["md"])
    for got, want in zip(ff, c["ff"]):
        assert got[:7] == pytest.approx(want[:7], abs=0.011)
        assert got[7] == pytest.approx(want[7], rel=0.01)
    for got, want in zip(md, c["md"]):
        assert got == pytest.approx(want, abs=0.011)
    if nc:
        f = netcdf_file(nc, "r", mmap=False)
        assert f.variables["coordinates"].shape[0] == 10
        np.testing.assert_allclose(f.variables["time"][:], 0.01 * np.arange(1, 11), rtol=1e-6)
        f.close()


def test_variable_14_scaling(lib, checks):
    """The reference's test/nab/variable_14scale.nab: N-methylacetamide
    whose prmtop carries per-dihedral SCEE/SCNB 1-4 scale factors, gb=1:
    every energy component of the compiled reference within 1e-6 of the
    total's magnitude, and the shipped ff: line."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    c = checks["variable_14"]
    prm, x = load_case(c)
    bt = Batch(c["options"])
    bt.add(prm, x)
    bt.finalize()
    bt.eval()
    b = bt.energy(0)
    bt.close()
    session = sff.Session(prm, c["options"])
    g = np.zeros(3 * prm.contents.Natom)
    it = C.c_int(-2)
    e = sff.lib().mme(sff.dptr(x), sff.dptr(g), C.byref(it))
    del session
    tot = abs(c["sp"]["Total"])
    for k, idx in (("bond", 3), ("angle", 4), ("dihedral", 5), ("enb14", 7), ("eel14", 8), ("enb", 1), ("eel", 2),
                   ("egb", 10)):
        assert b[idx] == pytest.approx(c["sp"][k], abs=1e-6 * tot), k
    assert e == pytest.approx(c["sp"]["Total"], abs=1e-6 * tot)
    assert round(e, 2) == c["ff"][0][1]


@pytest.mark.parametrize("rattle", [1, 2])
def test_batched_md_rattle(lib, rattle):
    """Batched md with RATTLE on the device (rattle=1: all bonds, 2: bonds to
    hydrogen).  After the run every constrained bond has the length the
    position sweeps hold it to (|req^2 - r^2| within the reference's
    tolerance, 1e-7 A^2, at the last sweep), the bonds left free do not,
    every system ends with status OK, and each system's trajectory is
    bit-identical alone and batched (Berendsen coupling, no noise: a
    batch's default noise key is the system's index)."""
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    opts = f"gb=1, cut=999.0, rgbmax=15.0, dt=0.002, gamma_ln=0.0, temp0=300.0, tempi=0.0, rattle={rattle}"
    mols = [sff.synth_molecule(n, 60 + n) for n in (150, 420)]
    nsteps = 30

    def run(idx):
        b = Batch(opts)
        for k in idx:
            b.add(mols[k][0], mols[k][1])
        b.finalize()
        b.md(nsteps)
        out = [(b.coords(s), b.velocities(s)) for s in range(len(idx))]
        assert list(b.status()) == [0] * len(idx)
        b.close()
        return out

    alone = [run([k])[0] for k in range(len(mols))]
    both = run([0, 1])
    for (x, v), (xa, va) in zip(both, alone):
        assert np.array_equal(x, xa) and np.array_equal(v, va)
    for (prm, x0, _), (x, _) in zip(mols, both):
        p = prm.contents
        nh, na = p.Nbonh, p.Mbona
        bonds = [(p.BondHAt1[i] // 3, p.BondHAt2[i] // 3, p.Req[p.BondHNum[i] - 1]) for i in range(nh)]
        heavy = [(p.BondAt1[i] // 3, p.BondAt2[i] // 3, p.Req[p.BondNum[i] - 1]) for i in range(na)]
        held = bonds + (heavy if rattle == 1 else [])
        xr = x.reshape(-1, 3)
        dev = [abs(req * req - ((xr[a] - xr[b]) ** 2).sum()) for a, b, req in held]
        assert max(dev) < 2e-7, max(dev)
        if rattle == 2 and heavy:
            free = [abs(req * req - ((xr[a] - xr[b]) ** 2).sum()) for a, b, req in heavy]
            assert max(free) > 1e-4

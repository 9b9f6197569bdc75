"""Host-side logic of the library, without a GPU: the parm7 reader and
writer, coordinate files, the mm_options grammar, status codes of the
batched API, and the synthetic molecule generator."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_path

INT_ARRAYS = ["Iac", "Iblo", "Cno", "Ipres", "ExclAt", "BondHAt1", "BondHAt2", "BondHNum", "BondAt1", "BondAt2",
              "BondNum", "AngleHAt1", "AngleHAt2", "AngleHAt3", "AngleHNum", "AngleAt1", "AngleAt2", "AngleAt3",
              "AngleNum", "DihHAt1", "DihHAt2", "DihHAt3", "DihHAt4", "DihHNum", "DihAt1", "DihAt2", "DihAt3",
              "DihAt4", "DihNum"]


def int_len(p, name):
    n = {"Iac": p.Natom, "Iblo": p.Natom, "Cno": p.Ntype2d, "Ipres": p.Nres + 1, "ExclAt": p.Nnb}
    if name in n:
        return n[name]
    if name.startswith("BondH"):
        return p.Nbonh
    if name.startswith("Bond"):
        return p.Mbona
    if name.startswith("AngleH"):
        return p.Ntheth
    if name.startswith("Angle"):
        return p.Mtheta
    if name.startswith("DihH"):
        return p.Nphih
    return p.Mphia


def arrays(prm):
    p = prm.contents
    out = {}
    for name in ("Charges", "Masses", "Rborn", "Fs"):
        out[name] = np.ctypeslib.as_array(getattr(p, name), (p.Natom,)).copy()
    for name, n in (("Rk", p.Numbnd), ("Req", p.Numbnd), ("Tk", p.Numang), ("Teq", p.Numang), ("Pk", p.Nptra),
                    ("Pn", p.Nptra), ("Phase", p.Nptra), ("Cn1", p.Nttyp), ("Cn2", p.Nttyp)):
        out[name] = np.ctypeslib.as_array(getattr(p, name), (n,)).copy() if n else np.zeros(0)
    for name in INT_ARRAYS:
        n = int_len(p, name)
        out[name] = np.ctypeslib.as_array(getattr(p, name), (n,)).copy() if n else np.zeros(0, np.int32)
    return out


@pytest.mark.parametrize("name", ["xfin.parm7", "prmtop.gb2", "gbrna.prmtop", "n300_s11.parm7"])
def test_parm7_write_read_round_trip(lib, tmp_path, name):
    from nabc_gb300 import sff
    prm = sff.rdparm(golden_path(name))
    assert prm
    out = str(tmp_path / "copy.parm7")
    assert lib.wrparm(prm, out.encode()) == 0
    prm2 = sff.rdparm(out)
    a, b = arrays(prm), arrays(prm2)
    for k in a:
        # the format writes %16.8E reals: 9 significant digits
        if a[k].dtype.kind == "f":
            assert np.allclose(a[k], b[k], rtol=2e-8, atol=0), k
        else:
            assert np.array_equal(a[k], b[k]), k
    assert prm.contents.Natom == prm2.contents.Natom and prm.contents.Nres == prm2.contents.Nres
    sff.free_prm(prm)
    sff.free_prm(prm2)


def test_rst7_round_trip(lib, tmp_path):
    from nabc_gb300 import sff
    n = 300
    x, v = sff.getxv(golden_path("n300_s11.rst7"), n)
    path = str(tmp_path / "out.rst7")
    assert lib.putxv(path.encode(), b"round trip", n, 0.0, sff.dptr(x), sff.dptr(v)) == 0
    x2, v2 = sff.getxv(path, n)
    assert np.allclose(x, x2, atol=5e-8) and np.allclose(v, v2, atol=5e-8)


def run_py(code):
    env = dict(os.environ, PYTHONPATH=ROOT)
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)


def test_mm_options_echo_and_fail_stop():
    """Accepted items are echoed to nabout; an unknown key prints an error
    and exits the process, as the reference's option scanner does."""
    r = run_py("from nabc_gb300 import sff\n"
               "sff.mm_options('cut=12.5, gb=5  rgbmax = 10.0\\tntpr=5')\n"
               "sff.flush_output()\n"
               "sff.mm_options('bogus=1')\n"
               "print('not reached')")
    assert r.returncode == 1
    assert "mm_options:  cut=12.5" in r.stdout and "mm_options:  gb=5" in r.stdout
    assert "rgbmax = 10.0" in r.stdout or "rgbmax=10.0" in r.stdout
    assert "not reached" not in r.stdout
    assert "bogus=1" in r.stderr


def test_mm_options_rejects_value_outside_the_key_set():
    r = run_py("from nabc_gb300 import sff\nsff.mm_options('gb=4')\nprint('not reached')")
    assert r.returncode == 1 and "not reached" not in r.stdout


def test_batch_api_status_codes(lib):
    h = C.c_void_p()
    assert lib.sffg_batch_create(b"gb=5, nosuchkey=1", C.byref(h)) == -1
    assert b"nosuchkey" in lib.sffg_last_error()
    assert lib.sffg_batch_create(b"gb=0", C.byref(h)) == -1
    assert lib.sffg_batch_create(b"gb=5, cut=10.0, rgbmax=25.0", C.byref(h)) == -1  # rgbmax > cut
    assert lib.sffg_batch_create(b"gb=5, cut=30.0, rgbmax=25.0", C.byref(h)) == 0
    assert lib.sffg_batch_finalize(h) == -1  # no systems
    assert lib.sffg_batch_num_systems(h) == 0
    assert lib.sffg_batch_destroy(h) == 0
    assert lib.sffg_batch_finalize(None) == -1


def test_synthetic_molecule_properties(lib):
    """Compact self-avoiding chain: neutral, bonded neighbours 1.53 A apart,
    no two non-bonded atoms closer than 2.5 A, seeded and reproducible."""
    from nabc_gb300 import sff
    from scipy.spatial import cKDTree
    n = 2000
    prm, x, radius = sff.synth_molecule(n, 42)
    prm2, x2, radius2 = sff.synth_molecule(n, 42)
    assert np.array_equal(x, x2) and radius == radius2
    p = prm.contents
    assert p.Natom == n
    q = np.ctypeslib.as_array(p.Charges, (n,))
    assert abs(q.sum()) < 1e-9 * 18.2223 * n
    X = x.reshape(-1, 3)
    d = np.linalg.norm(X[1:] - X[:-1], axis=1)
    assert np.allclose(d, 1.53, atol=1e-6)
    pairs = cKDTree(X).query_pairs(2.5 - 1e-6, output_type="ndarray")
    # only chain neighbours (1-2 at 1.53 A, and 1-3 via the 111-degree
    # angle at 2.52 A is outside) may be this close
    assert np.all(np.abs(pairs[:, 0] - pairs[:, 1]) <= 2)
    assert np.linalg.norm(X, axis=1).max() <= radius + 1e-6  # confining sphere about the origin
    sff.free_prm(prm)
    sff.free_prm(prm2)


def test_mm_options_ntpr_zero_is_refused():
    """ntpr takes [1-9][0-9]* in the reference's grammar (mm_options.l:32)."""
    r = run_py("from nabc_gb300 import sff\nsff.mm_options('ntpr=0')\nprint('not reached')")
    assert r.returncode == 1 and "ntpr=0" in r.stderr


@pytest.mark.parametrize("natom,seed", [(4, 1), (37, 5), (600, 7), (3000, 777), (25000, 2025)])
def test_oracle_generator_matches_library(lib, oracle_mod, natom, seed):
    """oracle/synth.c, which the CPU baseline and the reference arm of
    bench.py make their inputs with (without loading libsffg), gives the
    library generator's molecule bit for bit: coordinates, radius, and
    every topology array the oracle reads."""
    from nabc_gb300 import sff
    prm, x, radius = sff.synth_molecule(natom, seed)
    m = oracle_mod.SynthMolecule(natom, seed)
    assert np.array_equal(m.x, x)
    assert m.radius == radius and m.natom == natom and m.fsmax == prm.contents.Fsmax
    P = C.POINTER(sff.PARMSTRUCT_T)
    q = C.cast(C.c_void_p(m.ptr), P).contents
    p = prm.contents
    for name in ("Natom", "Ntypes", "Nbonh", "Mbona", "Ntheth", "Mtheta", "Ntheta", "Nphih", "Mphia", "Nnb"):
        assert getattr(q, name) == getattr(p, name), name
    ln = {"Charges": natom, "Masses": natom, "Rborn": natom, "Fs": natom, "Cn1": 10, "Cn2": 10,
          "Rk": 1, "Req": 1, "Tk": 1, "Teq": 1, "Pk": 1, "Pn": 1, "Phase": 1}
    for name, n in ln.items():
        assert np.array_equal(np.ctypeslib.as_array(getattr(q, name), (n,)),
                              np.ctypeslib.as_array(getattr(p, name), (n,))), name
    for name in INT_ARRAYS + ["AtomicNum"]:
        if name == "Ipres":
            continue
        n = natom if name == "AtomicNum" else int_len(p, name)
        if n:
            assert np.array_equal(np.ctypeslib.as_array(getattr(q, name), (n,)),
                                  np.ctypeslib.as_array(getattr(p, name), (n,))), name
    n14 = int(np.ctypeslib.as_array(p.N14pairs, (natom,)).sum())
    assert np.array_equal(np.ctypeslib.as_array(q.N14pairs, (natom,)), np.ctypeslib.as_array(p.N14pairs, (natom,)))
    for name in ("N14pairlist", "N14sceelist", "N14scnblist"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(q, name), (n14,)),
                              np.ctypeslib.as_array(getattr(p, name), (n14,))), name
    # the oracle gives the same energy on both (to the rounding of its
    # OpenMP reduction, whose order varies from run to run)
    o1 = oracle_mod.Oracle(prm, "gb=5, cut=12.0")
    o2 = oracle_mod.Oracle(m, "gb=5, cut=12.0")
    if natom <= 3000:
        assert o1.mme(x)[0] == pytest.approx(o2.mme(m.x)[0], rel=1e-12)
    m.close()
    sff.free_prm(prm)

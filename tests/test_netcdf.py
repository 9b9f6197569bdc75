"""md()'s Amber NetCDF trajectory (nabc_gb300/csrc/netcdf.cpp): the file
mme_init_sff creates when given a name, with a frame every ntwx steps, read
back with an independent NetCDF reader (scipy.io.netcdf_file).  The layout
is the reference's (src/sff/AmberNetcdf.c:595-740): 64-bit-offset classic
format, AMBER conventions, float coordinates(frame, atom, spatial).  These
run md() on the host loop with a harmonic test potential, so no GPU is
needed; tests/test_gpu_drivers.py covers the device-resident md path."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_path

netcdf = pytest.importorskip("scipy.io")


def run_md(lib, tmp_path, opts, nsteps):
    from nabc_gb300 import sff
    prm = sff.rdparm(golden_path("xfin.parm7"))
    n = prm.contents.Natom
    x, v = sff.getxv(golden_path("xfin.rst7"), n)
    lib.sffg_options_reset()
    lib.mm_options(opts.encode())
    frozen = np.zeros(n, np.int32)
    cons = np.zeros(n, np.int32)
    path = str(tmp_path / "md.nc")
    lib.mme_init_sff(prm, sff.iptr(frozen), sff.iptr(cons), None, path.encode())
    x0 = x.copy()

    @sff.FUNC_T
    def harmonic(xp, gp, it):
        xa = np.ctypeslib.as_array(xp, (3 * n,))
        ga = np.ctypeslib.as_array(gp, (3 * n,))
        d = xa - x0 - 0.3
        ga[:] = 2.0 * d
        return float((d * d).sum())

    f = np.zeros(3 * n)
    lib.md(3 * n, nsteps, sff.dptr(x), sff.dptr(f), sff.dptr(v), C.cast(harmonic, C.c_void_p))
    masses = np.array([prm.contents.Masses[i] for i in range(n)])
    return path, x, masses, n


def test_amber_layout(lib, tmp_path):
    path, x, masses, n = run_md(lib, tmp_path, "gb=1, cut=99.0, rgbmax=15.0, ntwx=5, ntpr_md=5, zerov=1, "
                                               "gamma_ln=0.0, dt=0.001", 20)
    from scipy.io import netcdf_file
    nc = netcdf_file(path, "r", mmap=False)
    assert nc.version_byte == 2  # 64-bit offsets
    assert nc.dimensions == {"frame": None, "spatial": 3, "atom": n, "cell_spatial": 3, "label": 5,
                             "cell_angular": 3}
    want = {"time": (("frame",), "f"), "spatial": (("spatial",), "c"),
            "coordinates": (("frame", "atom", "spatial"), "f"), "cell_spatial": (("cell_spatial",), "c"),
            "cell_angular": (("cell_angular", "label"), "c")}
    assert {k: (v.dimensions, v.typecode()) for k, v in nc.variables.items()} == want
    assert nc._attributes == {"title": b"AmberNetcdf trajectory", "application": b"AMBER",
                              "program": b"AmberNetcdf", "programVersion": b"1.0", "Conventions": b"AMBER",
                              "ConventionVersion": b"1.0"}
    assert nc.variables["coordinates"].units == b"angstrom"
    assert nc.variables["time"].units == b"picosecond"
    assert b"".join(nc.variables["spatial"][:]) == b"xyz"
    assert b"".join(nc.variables["cell_spatial"][:]) == b"abc"
    assert b"".join(nc.variables["cell_angular"][:].ravel()) == b"alphabeta gamma"
    coords = nc.variables["coordinates"][:].copy()
    assert coords.shape == (4, n, 3)
    np.testing.assert_allclose(nc.variables["time"][:], [0.005, 0.010, 0.015, 0.020], rtol=1e-6)
    # the last frame is the final structure in single precision
    np.testing.assert_array_equal(coords[-1].ravel(), x.astype(np.float32))
    assert not np.array_equal(coords[0], coords[1])
    nc.close()


def test_frame_precedes_com_removal(lib, tmp_path):
    """With nscm dividing the frame step, the frame holds the structure
    before the centre of mass is moved to the origin (sff.c:2341-2351)."""
    path, x, masses, n = run_md(lib, tmp_path, "gb=1, cut=99.0, rgbmax=15.0, ntwx=10, ntpr_md=10, nscm=10, "
                                               "zerov=1, gamma_ln=0.0, dt=0.001", 20)
    from scipy.io import netcdf_file
    nc = netcdf_file(path, "r", mmap=False)
    last = nc.variables["coordinates"][-1].astype(np.float64)
    nc.close()
    xr = x.reshape(n, 3)
    com = (masses[:, None] * xr).sum(0) / masses.sum()
    assert np.abs(com).max() < 1e-9  # final structure: centre of mass at the origin
    shift = last - xr
    assert np.abs(shift - shift.mean(0)).max() < 1e-4  # frame = final + one translation
    assert np.abs(shift.mean(0)).max() > 0.01


def test_no_frames_without_ntwx(lib, tmp_path):
    """ntwx = 0 (the default) creates the file at mme_init_sff but writes no
    frame, as the reference."""
    path, x, masses, n = run_md(lib, tmp_path, "gb=1, cut=99.0, rgbmax=15.0, zerov=1, gamma_ln=0.0", 10)
    from scipy.io import netcdf_file
    nc = netcdf_file(path, "r", mmap=False)
    assert nc.variables["coordinates"].shape == (0, n, 3)
    nc.close()

"""sffg_born_radii_static, the allocation-free Born-radius entry point, called
twice in a row through the C ABI: against the FP64 oracle's radii (every
pair listed, cut 999) and against the batch path's radii, and with the
device's free memory unchanged across the calls.  Collected last so that it
also runs after every other test in one process."""
import ctypes as C

import numpy as np
import pytest

REFF_REL = 2e-6  # the bar of the batch-path parity tests


def static_fn(L):
    from nabc_gb300 import sff
    f = L.sffg_born_radii_static
    f.restype = C.c_int
    f.argtypes = [C.c_int, sff.REAL_P, sff.REAL_P, sff.REAL_P, C.c_int, C.c_double, sff.REAL_P, C.c_void_p]
    return f


def topology_arrays(prm, natom):
    rb = np.ctypeslib.as_array(prm.contents.Rborn, shape=(natom,)).copy()
    fs = np.ctypeslib.as_array(prm.contents.Fs, shape=(natom,)).copy()
    return rb, fs


@pytest.mark.gpu
@pytest.mark.parametrize("natom,gb,rgbmax", [(3000, 5, 15.0), (777, 1, 12.0), (8192, 2, 25.0)])
def test_static_radii_match_oracle_and_batch(lib, oracle_mod, natom, gb, rgbmax):
    import torch
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    prm, x, _ = sff.synth_molecule(natom, 900 + natom)
    opts = f"gb={gb}, cut=999.0, rgbmax={rgbmax}"
    b = Batch(opts)
    b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True)
    ref = b.reff(0)
    b.close()
    _, _, _, reff0 = oracle_mod.Oracle(prm, opts).mme(x)
    rb, fs = topology_arrays(prm, natom)
    f = static_fn(lib)
    warm = np.zeros(natom)
    # warm-up: the first call on the device may load the library's device code
    assert f(natom, sff.dptr(x), sff.dptr(rb), sff.dptr(fs), gb, rgbmax, sff.dptr(warm), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    outs = []
    for _ in range(2):
        out = np.zeros(natom)
        assert f(natom, sff.dptr(x), sff.dptr(rb), sff.dptr(fs), gb, rgbmax, sff.dptr(out), None) == 0
        assert np.max(np.abs(out / reff0 - 1.0)) <= REFF_REL
        assert np.max(np.abs(out / ref - 1.0)) <= REFF_REL
        outs.append(out)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0  # the calls allocated no device memory
    assert np.array_equal(outs[0], outs[1])  # fixed-point sums: bit-identical repeats
    assert np.array_equal(outs[0], warm)
    sff.free_prm(prm)


@pytest.mark.gpu
def test_static_refuses_capturing_stream(lib):
    """A call on a stream under capture is refused and the capture survives."""
    import torch
    from nabc_gb300 import sff
    f = static_fn(lib)
    n = 64
    prm, x, _ = sff.synth_molecule(n, 5)
    rb, fs = topology_arrays(prm, n)
    out = np.zeros(n)
    assert f(n, sff.dptr(x), sff.dptr(rb), sff.dptr(fs), 5, 15.0, sff.dptr(out), None) == 0
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    buf = torch.zeros(4, device="cuda")
    with torch.cuda.graph(g, stream=s):
        buf.add_(1.0)
        rc = f(n, sff.dptr(x), sff.dptr(rb), sff.dptr(fs), 5, 15.0, sff.dptr(out),
               C.c_void_p(s.cuda_stream))
    assert rc == -1  # SFFG_EINVAL
    g.replay()
    torch.cuda.synchronize()
    assert float(buf[0]) == 1.0
    sff.free_prm(prm)


def test_static_rejects_without_device_work(lib):
    """Sizes past the static scratch and bad arguments are refused before
    any CUDA call (runs without a GPU)."""
    from nabc_gb300 import sff
    f = static_fn(lib)
    n = 8193
    x, rb, fs, out = np.zeros(3 * n), np.full(n, 1.5), np.full(n, 0.8), np.zeros(n)
    args = (sff.dptr(x), sff.dptr(rb), sff.dptr(fs))
    assert f(n, *args, 5, 15.0, sff.dptr(out), None) == -2        # SFFG_ENOMEM: does not fit
    assert f(100, *args, 7, 15.0, sff.dptr(out), None) == -1      # SFFG_EINVAL: GBneck not offered
    assert f(0, *args, 5, 15.0, sff.dptr(out), None) == -1        # SFFG_EINVAL: empty molecule
    assert f(100, *args, 5, 0.0, sff.dptr(out), None) == -1       # SFFG_EINVAL: rgbmax
    assert f(100, None, args[1], args[2], 5, 15.0, sff.dptr(out), None) == -1

"""XMIN (nabc_gb300/csrc/xmin.cpp) against the reference's own minimiser
(src/sff/xminC.c compiled from source into oracle/_ref/xminref) on the
deterministic test functions of oracle/xmin_funcs.c.  Both minimisers call
the same compiled function, so every requested function value, the final
point, the iteration counts and the error status must agree bit for bit:
PRCG, L-BFGS and TNCG, Armijo and More-Thuente line searches, forward and
central Hessian products, frozen atoms, capped steps, maxiter 0 and the
reference's y.s = 0 error exit.  No GPU is used: the minimiser is host code
and the functions are plain C."""
import ctypes as C

import numpy as np
import pytest

from nabc_gb300 import sff

FUNC_RAW = C.CFUNCTYPE(C.c_double, sff.REAL_P, sff.REAL_P, sff.INT_P)


@pytest.fixture(scope="module")
def funcs(oracle_mod):
    return oracle_mod.xmin_functions()


def setup_case(L, F, case, k, refrun):
    xo = sff.XMIN_OPT_T()
    L.xmin_opt_init(C.byref(xo))
    xo.method, xo.ls_method, xo.numdiff = case["method"], case["ls_method"], case["numdiff"]
    xo.m_lbfgs, xo.maxiter = case["m_lbfgs"], case["maxiter"]
    xo.grms_tol, xo.ls_maxatmov = case["grms_tol"], case["ls_maxatmov"]
    if case["function"] == "rosen":
        f = F.xf_rosenbrock
        xo.mol_struct_opt = 0
        C.c_int.in_dll(F, "xf_dim").value = case["ndim"]
        n = case["ndim"]
    else:
        f = F.xf_chain
        xo.mol_struct_opt = 1
        n = case["ndim"] // 3
        C.c_int.in_dll(F, "xf_natom").value = n
        frozen = (C.c_int * 64).in_dll(F, "xf_frozen")
        for i in range(64):
            frozen[i] = 0
        frozen[4] = 1
    raw = FUNC_RAW(C.cast(f, C.c_void_p).value)
    x = refrun[f"xmin{k}_start"].copy()
    return xo, raw, x, n


def run_xmin(L, raw, x, n, xo):
    """xmin() through a recording wrapper; returns (value, x, g, e, grms, trace)."""
    trace = []

    @sff.FUNC_T
    def rec(xp, gp, it):
        v = raw(xp, gp, it)
        trace.append(v)
        return v

    g = np.zeros_like(x)
    it = C.c_int(0)
    raw(sff.dptr(x), sff.dptr(g), C.byref(it))  # the gradient on entry marks frozen atoms
    e = np.zeros(1)
    grms = np.zeros(1)
    nn = C.c_int(n)
    ret = L.xmin(C.cast(rec, C.c_void_p), C.byref(nn), sff.dptr(x), sff.dptr(g), sff.dptr(e), sff.dptr(grms),
                 C.byref(xo))
    return ret, x, g, e[0], grms[0], np.array(trace)


def ncases(checks):
    return len(checks["xmin_functions"]["cases"])


@pytest.mark.parametrize("k", range(15))
def test_xmin_matches_reference_bitwise(lib, funcs, checks, refrun, k):
    cases = checks["xmin_functions"]["cases"]
    if k >= len(cases):
        pytest.skip("no such golden case")
    case = cases[k]
    xo, raw, x, n = setup_case(lib, funcs, case, k, refrun)
    ret, x, g, e, grms, trace = run_xmin(lib, raw, x, n, xo)
    want = refrun[f"xmin{k}_trace"]
    assert len(trace) == len(want)
    assert np.array_equal(trace, want), "function values requested differ"
    assert np.array_equal(x, refrun[f"xmin{k}_x"])
    assert np.array_equal(g, refrun[f"xmin{k}_g"])
    r_ret, r_e, r_grms = refrun[f"xmin{k}_scalars"]
    assert ret == r_ret and e == r_e
    assert (xo.iter, xo.ls_iter, xo.error_flag) == (case["iter"], case["ls_iter"], case["error_flag"])
    if case["error_flag"] == 0:
        assert grms == r_grms
    if case["function"] == "chain":  # the frozen atom never moves
        np.testing.assert_array_equal(x[12:15], refrun[f"xmin{k}_start"][12:15])


def test_reverse_communication_equals_xmin(lib, funcs, checks, refrun):
    """xminC() driven by the caller gives xmin()'s iterates exactly."""
    k = 7  # L-BFGS on the chain
    case = checks["xmin_functions"]["cases"][k]
    xo, raw, x, n = setup_case(lib, funcs, case, k, refrun)
    g = np.zeros_like(x)
    it = C.c_int(0)
    raw(sff.dptr(x), sff.dptr(g), C.byref(it))
    ints = {name: C.c_int(getattr(xo, name)) for name in
            ("mol_struct_opt", "method", "maxiter", "m_lbfgs", "numdiff", "print_level", "ls_method", "ls_maxiter")}
    dbls = {name: C.c_double(getattr(xo, name)) for name in
            ("grms_tol", "ls_maxatmov", "beta_armijo", "c_armijo", "mu_armijo", "ftol_wolfe", "gtol_wolfe")}
    natm, enrg, grms, iters, ttime, lsit = C.c_int(n), C.c_double(0.0), C.c_double(0.0), C.c_int(0), \
        C.c_double(0.0), C.c_int(0)
    flag, label = C.c_int(0), C.c_int(0)
    trace = []
    while True:
        lib.xminC(C.byref(ints["mol_struct_opt"]), C.byref(ints["method"]), C.byref(ints["maxiter"]),
                  C.byref(dbls["grms_tol"]), C.byref(natm), C.byref(ints["m_lbfgs"]), C.byref(ints["numdiff"]),
                  sff.dptr(x), C.byref(enrg), sff.dptr(g), C.byref(grms), C.byref(iters), C.byref(ttime),
                  C.byref(ints["print_level"]), C.byref(ints["ls_method"]), C.byref(ints["ls_maxiter"]),
                  C.byref(lsit), C.byref(dbls["ls_maxatmov"]), C.byref(dbls["beta_armijo"]),
                  C.byref(dbls["c_armijo"]), C.byref(dbls["mu_armijo"]), C.byref(dbls["ftol_wolfe"]),
                  C.byref(dbls["gtol_wolfe"]), C.byref(flag), C.byref(label))
        if label.value != 1:
            break
        assert flag.value in (6, 8, 9)
        enrg.value = raw(sff.dptr(x), sff.dptr(g), C.byref(it))
        trace.append(enrg.value)
    assert label.value == 0 and flag.value == 0
    assert np.array_equal(np.array(trace), refrun[f"xmin{k}_trace"])
    assert np.array_equal(x, refrun[f"xmin{k}_x"])
    assert (iters.value, lsit.value) == (case["iter"], case["ls_iter"])


def test_defaults(lib):
    xo = sff.XMIN_OPT_T()
    lib.xmin_opt_init(C.byref(xo))
    assert (xo.mol_struct_opt, xo.maxiter, xo.method, xo.numdiff, xo.m_lbfgs, xo.ls_method, xo.ls_maxiter,
            xo.print_level) == (1, 1000, 3, 1, 5, 2, 20, 0)
    assert (xo.grms_tol, xo.ls_maxatmov, xo.beta_armijo, xo.c_armijo, xo.mu_armijo, xo.ftol_wolfe,
            xo.gtol_wolfe) == (0.05, 0.5, 0.5, 0.4, 1.0, 0.0001, 0.9)


@pytest.mark.parametrize("field,value", [("maxiter", -1), ("grms_tol", -1.0), ("m_lbfgs", -2), ("ls_maxiter", 0),
                                         ("ls_maxatmov", 0.0), ("beta_armijo", 1.0), ("c_armijo", 0.5),
                                         ("mu_armijo", 2.0), ("method", 7), ("ls_method", 3), ("numdiff", 0)])
def test_parameter_errors(lib, funcs, checks, refrun, field, value):
    """Out-of-range options end with error_flag -1 before any evaluation,
    the coordinates untouched, as the reference's xminC checks them."""
    case = checks["xmin_functions"]["cases"][7]
    xo, raw, x, n = setup_case(lib, funcs, case, 7, refrun)
    setattr(xo, field, value)
    x0 = x.copy()
    ret, x, g, e, grms, trace = run_xmin(lib, raw, x, n, xo)
    assert ret == 0.0 and xo.error_flag == -1 and len(trace) == 0
    np.testing.assert_array_equal(x, x0)


def test_too_few_moving_atoms(lib, funcs, checks, refrun):
    case = checks["xmin_functions"]["cases"][7]
    xo, raw, x, n = setup_case(lib, funcs, case, 7, refrun)
    frozen = (C.c_int * 64).in_dll(funcs, "xf_frozen")
    for i in range(n - 1):
        frozen[i] = 1
    try:
        ret, x, g, e, grms, trace = run_xmin(lib, raw, x, n, xo)
    finally:
        for i in range(64):
            frozen[i] = 0
    assert xo.error_flag == -1 and len(trace) == 0


def test_lbfgs_needs_memory(lib, funcs, checks, refrun):
    """L-BFGS with m_lbfgs = 0 is the reference's MINIMZ_ERROR (-5)."""
    case = checks["xmin_functions"]["cases"][7]
    xo, raw, x, n = setup_case(lib, funcs, case, 7, refrun)
    xo.m_lbfgs = 0
    ret, x, g, e, grms, trace = run_xmin(lib, raw, x, n, xo)
    assert ret == 0.0 and xo.error_flag == -5


def test_gradient_check_mode(lib, funcs, checks, refrun, capfd):
    """method 4 compares analytic and central-difference derivatives of
    every coordinate and leaves the coordinates where they were."""
    case = checks["xmin_functions"]["cases"][0]
    xo, raw, x, n = setup_case(lib, funcs, case, 0, refrun)
    xo.method = 4
    x0 = x.copy()
    ret, x, g, e, grms, trace = run_xmin(lib, raw, x, n, xo)
    assert xo.error_flag == 0 and len(trace) == 1 + 3 * n
    np.testing.assert_array_equal(x, x0)
    err = capfd.readouterr().err
    rows = [line.split() for line in err.splitlines() if line.strip()[:1].isdigit() or line.strip()[:1] == "*"]
    assert len(rows) == n
    for row in rows:  # analytic vs numerical derivative
        anal, num = float(row[-4]), float(row[-3])
        assert anal == pytest.approx(num, rel=1e-5, abs=1e-3)


def test_nab_txmin_through_oracle(lib, oracle_mod, checks, tmp_path):
    """The reference's own test/nab/txmin.nab (gbrna, gb=1 with kappa 0.10395,
    the default TNCG, 5 iterations, print_level 1) run by this library's
    XMIN over the FP64 oracle energy: every MIN line of the shipped
    txmin.out.check (iteration, evaluations so far, energy to the printed 5
    decimals, RMS gradient to the printed 8 digits) and the END line."""
    import os
    import re
    from conftest import load_case
    c = checks["nab_txmin"]
    prm, x = load_case(c)
    o = oracle_mod.Oracle(prm, c["options"])
    n = prm.contents.Natom

    @sff.FUNC_T
    def energy(xp, gp, it):
        e, ene, g, reff = o.mme(np.ctypeslib.as_array(xp, (3 * n,)).copy())
        np.ctypeslib.as_array(gp, (3 * n,))[:] = g
        return e

    g = np.zeros(3 * n)
    it = C.c_int(0)
    e = np.array([energy(sff.dptr(x), sff.dptr(g), C.byref(it))])
    xo = sff.XMIN_OPT_T()
    lib.xmin_opt_init(C.byref(xo))
    xo.maxiter, xo.grms_tol, xo.ls_maxatmov, xo.print_level = c["maxiter"], c["grms_tol"], c["ls_maxatmov"], 1
    out = str(tmp_path / "txmin.out")
    sff.set_output(out)
    try:
        grms = np.zeros(1)
        nn = C.c_int(n)
        lib.xmin(C.cast(energy, C.c_void_p), C.byref(nn), sff.dptr(x), sff.dptr(g), sff.dptr(e), sff.dptr(grms),
                 C.byref(xo))
        sff.flush_output()
    finally:
        sff.set_output(os.devnull)
    text = open(out).read()
    rows = [[int(m.group(1)), int(m.group(2)), float(m.group(3)), float(m.group(4))]
            for m in re.finditer(r" MIN: Iter =\s*(\d+)\s+NFunc =\s*(\d+)\s+E =\s*(\S+)\s+RMSG =\s*(\S+)", text)]
    assert "Starting TNCG minimisation" in text
    assert len(rows) == len(c["min_lines"])
    for got, want in zip(rows, c["min_lines"]):
        assert got[:2] == want[:2]
        assert got[2] == pytest.approx(want[2], abs=1.1e-5)
        assert got[3] == pytest.approx(want[3], rel=1e-7)
    end = re.search(r"END:\s+:-\)\s+E =\s*(\S+)\s+RMSG =\s*(\S+)", text)
    assert float(end.group(1)) == pytest.approx(c["end"][0], abs=1.1e-5)
    assert float(end.group(2)) == pytest.approx(c["end"][1], abs=1.1e-7)

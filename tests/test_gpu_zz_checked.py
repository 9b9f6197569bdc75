"""GPU: the checked build.  compute-sanitizer is closed on this machine, so a
build with -DSFFG_CHECKED tests every indirect index of the kernels (list
entry slots, tiles, Lennard-Jones rows, neck-table cells, atoms of bonded
terms) against its array's extent, records a code on a failure and reads
element 0 instead, never trapping.  The checked library is built into a
temporary directory and drives evaluations, cutoff lists, md, conjgrad,
XMIN and a batch of the reference's test systems with every GB model; no
check may fail.  (Collected last: it compiles a second library.)"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOAD = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
from conftest import load_case
import json
from nabc_gb300 import sff
from nabc_gb300.batch import Batch
L = sff.lib()
assert L.sffg_checked_code() == 0, "not the checked build"
checks = json.load(open(sys.argv[1] + "/tests/golden/checks.json"))
for opts in ("gb=1, cut=99.0, rgbmax=99.0, kappa=0.1", "gb=5, cut=14.0, rgbmax=12.0, nsnb=4",
             "gb=8, cut=99.0, rgbmax=25.0", "gb=7, cut=16.0, rgbmax=15.0"):
    b = Batch(opts + ", dt=0.001, gamma_ln=5.0, temp0=300.0")
    # GBneck (gb 7, 8) takes radii of 1-2 A only: the trx topology
    for name in (("gb5trx",) if "gb=7" in opts or "gb=8" in opts else ("gbrna", "gb5trx", "xfin")):
        prm, x = load_case(checks[name])
        b.add(prm, x)
    for n, seed in ((33, 1), (1000, 2)):
        prm, x, _ = sff.synth_molecule(n, seed)
        b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True)
    b.md_begin()
    b.md_steps(0, 12)
    b.cg(8, 1e-3)
    b.xmin(method=2, maxiter=4, grms_tol=1e-3)
    b.close()
print("CODE", L.sffg_checked_code())
"""


def test_checked_build_runs_clean(tmp_path):
    libdir = str(tmp_path / "checked")
    env = dict(os.environ, SFFG_BUILD_DIR=libdir, SFFG_NVCC_EXTRA="-DSFFG_CHECKED")
    subprocess.run([sys.executable, "-c", "import nabc_gb300._build as b; b.build()"], cwd=ROOT, env=env,
                   check=True, timeout=900)
    env = dict(os.environ, SFFG_LIBRARY=os.path.join(libdir, "libsffg.so"))
    out = subprocess.run([sys.executable, "-c", WORKLOAD, ROOT], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    codes = [line.split()[1] for line in out.stdout.splitlines() if line.startswith("CODE")]
    assert codes == ["0"], out.stdout[-2000:]

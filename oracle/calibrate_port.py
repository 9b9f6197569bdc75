"""TEST INFRASTRUCTURE ONLY: times the FP64 restatement (oracle/sffo.c, the
CPU baseline of bench.py) against the reference itself compiled from its
sources (oracle/_ref/sffref, `make -C oracle ref`) on the same molecule, the
same options and the same number of threads, where both can run (the
reference's source tree is not on the GPU host, so the baseline there is
the restatement; this ratio says how it stands against the reference).

Each side evaluates mme() n times at the normal cadence (the pair list
rebuilt on the first and every nsnb-th evaluation, the reference with its
k-d tree, the restatement with a brute-force search).  Usage:

    python oracle/calibrate_port.py [natom] [threads] [n]
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
# the repository root, in place of this script's own directory
sys.path[0] = os.path.dirname(HERE)

OPTS = "gb=5, rgbmax=15.0, cut=25.0, nsnb=10, ntpr=100000"


def main():
    natom = int(sys.argv[1]) if len(sys.argv) > 1 else 25000
    threads = int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 1)
    n = int(sys.argv[3]) if len(sys.argv) > 3 else 20
    sffref = os.path.join(HERE, "_ref", "sffref")
    if not os.path.exists(sffref):
        raise SystemExit("build the reference first: make -C oracle ref")
    from nabc_gb300 import sff
    from oracle import oracle
    sff.lib()
    sff.set_output(os.devnull)
    prm, x, _ = sff.synth_molecule(natom, 2025)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    with tempfile.TemporaryDirectory() as d:
        top, crd = os.path.join(d, "mol.parm7"), os.path.join(d, "mol.rst7")
        sff.lib().wrparm(prm, top.encode())
        sff.lib().putxv(crd.encode(), b"synthetic", natom, 0.0, sff.dptr(x), sff.dptr(x))
        out = subprocess.run([sffref, top, crd, "timei", OPTS, str(n)], env=env, capture_output=True, text=True,
                             check=True).stdout
    line = [l for l in out.splitlines() if l.startswith("oracle_time:")][-1]
    t_ref = float(line.split()[3])
    m = oracle.SynthMolecule(natom, 2025)
    o = oracle.Oracle(m, OPTS)
    oracle.set_threads(threads)
    o.mme(m.x)  # the untimed first call, as the driver makes one
    t0 = time.perf_counter()
    for k in range(n):
        o.mme(m.x, rebuild=(k % 10 == 0))
    t_port = time.perf_counter() - t0
    print(f"natom {natom}, {threads} threads, {n} evaluations: reference {t_ref:.3f} s "
          f"({n / t_ref:.2f} evals/s), restatement {t_port:.3f} s ({n / t_port:.2f} evals/s), "
          f"restatement / reference speed {t_ref / t_port:.2f}")


if __name__ == "__main__":
    main()

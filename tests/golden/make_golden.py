"""Regenerate the golden fixtures under tests/golden/.

Run where the reference's source tree is at hand (by default the directory
"reference" beside this repository):

    make -C oracle ref [REFROOT=<reference tree>]
    python tests/golden/make_golden.py [<reference tree>]

It produces
  ref/          the reference's own test inputs for the GB path (prmtops,
                PDB/restart coordinates), copied unchanged;
  checks.json   the reference's expected outputs parsed from its shipped
                .check files (test/nab/{gbrna,gbtrx,gb5trx,gb7trx,gb8trx},
                test/nab/aspgb8.out);
  synth/        small synthetic molecules (parm7 + rst7) from the
                benchmark generator;
  refrun.npz    outputs of the reference library itself (oracle/_ref/sffref,
                compiled from the reference sources) on those inputs:
                energy components, full gradients, conjgrad traces, short
                Langevin trajectories, XMIN minimisations of xfin (the
                reference's test/txmin.c) and of the test functions of
                oracle/xmin_funcs.c (oracle/_ref/xminref), each with every
                function value XMIN asked for, and LMOD searches on the
                bead chain of oracle/xmin_funcs.c (oracle/_ref/lmodref: the
                reference's lmodC.c with the ARPACK stand-in) -- final
                structure, conflib, trajectory, conflib.dat and printout.
"""
import json
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SFFREF = os.path.join(ROOT, "oracle", "_ref", "sffref")
XMINREF = os.path.join(ROOT, "oracle", "_ref", "xminref")
LMODREF = os.path.join(ROOT, "oracle", "_ref", "lmodref")

# LMOD on the bead chain (oracle/xmin_funcs.c), the lmodref arguments
# (ref_shim/lmod_driver.c): natom, frozen atom (-1: none), niter, nmod, kmod,
# mc_option, nof_lmod_steps, eig_recalc, ndim_arnoldi, lmod_restart,
# n_best_struct, energy_window, conf_separation_rms, nlig, lig_start,
# lig_end, lig_cent, print_level, random_seed
LMOD_CASES = [
    ("metropolis", [14, -1, 6, 5, 3, 1, 0, 5, 0, 10, 10, 50.0, 2.0, 0, 0, 0, 0, 2, 314159]),
    ("total_quench_restarted_krylov", [14, -1, 8, 5, 3, 2, 3, 2, 6, 3, 3, 50.0, 0.5, 0, 0, 0, 0, 2, 99]),
    ("quick_quench_frozen", [14, 4, 8, 4, 2, 3, 0, 1, 0, 4, 2, 5.0, 0.5, 0, 0, 0, 0, 1, 7]),
    ("docking_centroid", [14, -1, 6, 5, 3, 1, 0, 3, 0, 10, 10, 50.0, 0.5, 1, 11, 14, 0, 2, 314159]),
    ("docking_atom_centre", [14, -1, 6, 5, 3, 2, 2, 3, 0, 10, 10, 50.0, 0.5, 1, 11, 14, 12, 2, 5]),
    ("zigzag_movie", [14, -1, 2, 4, 2, 1, 2, 1, 0, 10, 10, 50.0, 0.5, 0, 0, 0, 0, 5, 11]),
    ("quiet_long", [14, -1, 12, 5, 3, 1, 0, 5, 8, 4, 3, 20.0, 0.7, 0, 0, 0, 0, 0, 271]),
]
# run twice in one directory: the second search starts from conflib.dat
LMOD_RESTART_CASE = ("conflib_restart", [14, -1, 4, 5, 3, 1, 0, 2, 0, 10, 10, 50.0, 0.5, 0, 0, 0, 0, 2, 42])

# XMIN on the test functions of oracle/xmin_funcs.c: (function, method,
# ls_method, numdiff, m_lbfgs, maxiter, grms_tol, ls_maxatmov)
XMIN_CASES = [
    ("rosen", 2, 2, 1, 5, 200, 1e-8, 0.5),
    ("rosen", 1, 2, 1, 5, 200, 1e-8, 0.5),
    ("rosen", 2, 1, 1, 5, 200, 1e-8, 0.5),
    ("rosen", 3, 2, 1, 5, 100, 1e-8, 0.5),   # TNCG ends on y.s = 0 (error -4)
    ("rosen", 3, 1, 2, 5, 100, 1e-8, 0.5),   # the same with Armijo, central differences
    ("rosen", 3, 2, 1, 3, 100, 1e-8, 0.5),
    ("rosen", 3, 2, 2, 0, 100, 1e-8, 0.5),   # TNCG without preconditioning
    ("chain", 2, 2, 1, 5, 200, 1e-6, 0.5),
    ("chain", 2, 1, 1, 7, 60, 1e-6, 0.05),   # steps capped by ls_maxatmov
    ("chain", 2, 2, 1, 3, 0, 1e-6, 0.5),     # maxiter 0
    ("chain", 1, 1, 1, 5, 200, 1e-6, 0.5),
    ("chain", 1, 2, 1, 5, 200, 1e-6, 0.5),
    ("chain", 3, 2, 1, 5, 100, 1e-6, 0.3),
    ("chain", 3, 2, 2, 5, 100, 1e-6, 0.5),
    ("chain", 3, 1, 1, 0, 100, 1e-6, 0.5),
]

# (name, prmtop, coordinates, options, conjgrad args) for the reference's
# GB regression tests (test/nab/*.nab, test/txmin.c)
REF_CASES = [
    ("gbrna", "nab/gbrna.prmtop", "nab/gbrna.pdb",
     "ntpr=1, gb=1, kappa=0.10395, rgbmax=99., cut=99.0, diel=C", "gbrna.out.check"),
    ("gbtrx", "nab/prmtop.gb2", "nab/trxox.2.4ns.pdb",
     "ntpr=1, gb=2, kappa=0.14701, rgbmax=99.0, cut=99.0, diel=C", "gbtrx.out.check"),
    ("gb5trx", "nab/prmtop.gb2", "nab/trxox.2.4ns.pdb",
     "ntpr=1, gb=5, kappa=0.14701, rgbmax=99.0, cut=99.0, diel=C", "gb5trx.out.check"),
    ("gb7trx", "nab/prmtop.gb2", "nab/trxox.2.4ns.pdb",
     "ntpr=1, gb=7, rgbmax=15.0, cut=99.0, diel=C, e_debug=0", "gb7trx.out.check"),
    ("gb8trx", "nab/prmtop.gb2", "nab/trxox.2.4ns.pdb",
     "ntpr=1, gb=8, rgbmax=15.0, cut=99.0, diel=C, e_debug=0", "gb8trx.out.check"),
]
EXTRA_INPUTS = ["nab/asp.top", "nab/asp.pdb", "xfin.parm7", "xfin.rst7", "xfin.md1.rst7", "nab/NMA.pdb",
                "nab/NMA_scee+scnb.prmtop", "nab/Na+.parm7", "nab/Na+.pdb"]

BREAKDOWN = ["bond", "angle", "dihedral", "enb14", "eel14", "enb", "eel", "egb", "econs", "esurf", "Total",
             "frms"]

# synthetic cases: (name, natom, seed, options)
SYNTH = [
    ("s300_gb1", 300, 11, "gb=1, cut=999.0, rgbmax=15.0"),
    ("s300_gb2", 300, 11, "gb=2, cut=999.0, rgbmax=15.0"),
    ("s300_gb5", 300, 11, "gb=5, cut=999.0, rgbmax=15.0"),
    ("s300_gb7", 300, 11, "gb=7, cut=999.0, rgbmax=15.0"),
    ("s300_gb8", 300, 11, "gb=8, cut=999.0, rgbmax=25.0"),
    ("s1000_gb5_cut", 1000, 12, "gb=5, cut=12.0, rgbmax=10.0, nsnb=10"),
    ("s1000_gb8_cut", 1000, 12, "gb=8, cut=14.0, rgbmax=12.0, nsnb=10"),
    ("s1000_gb1_kappa", 1000, 13, "gb=1, cut=999.0, rgbmax=15.0, kappa=0.10395"),
]


def run(args, cwd=None):
    r = subprocess.run(args, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"{args}: {r.stderr}")
    return r.stdout


def parse_ff(text):
    rows = []
    for line in text.splitlines():
        if line.startswith("ff:"):
            f = line.split()
            rows.append([int(f[1])] + [float(v) for v in f[2:]])
    return rows


def parse_breakdown(text):
    out = {}
    for line in text.splitlines():
        m = re.match(r"\s*(\w+):\s+([-+0-9.eE]+)\s*$", line)
        if m and m.group(1) in BREAKDOWN and m.group(1) not in out:
            out[m.group(1)] = float(m.group(2))
    return out


def parse_min_lines(text):
    """[iteration, energy, gradient RMS] of every " MIN:" progress line."""
    rows = []
    for line in text.splitlines():
        m = re.match(r" MIN:\s+Iter =\s*(\d+).*\sE =\s*(\S+)\s+RMSG =\s*(\S+)", line)
        if m:
            rows.append([float(m.group(1)), float(m.group(2)), float(m.group(3))])
    return rows


def read_dump(path):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(4), np.int32)[0])
        e = float(np.frombuffer(f.read(8), np.float64)[0])
        x = np.frombuffer(f.read(24 * n), np.float64).copy()
        g = np.frombuffer(f.read(24 * n), np.float64).copy()
    return n, e, x, g


def main():
    repo = os.path.dirname(os.path.dirname(HERE))
    refroot = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(repo), "reference")
    test = os.path.join(refroot, "test")
    if not os.path.exists(SFFREF):
        raise SystemExit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "ref"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "synth"), exist_ok=True)
    files = sorted({c[1] for c in REF_CASES} | {c[2] for c in REF_CASES} | set(EXTRA_INPUTS))
    for rel in files:
        shutil.copyfile(os.path.join(test, rel), os.path.join(HERE, "ref", os.path.basename(rel)))
    checks = {}
    arrays = {}
    tmp = os.path.join(HERE, "_tmp.bin")
    # reference regression tests: shipped .check outputs and our runs of the reference
    for name, prm, crd, opts, check in REF_CASES:
        text = open(os.path.join(test, "nab", check)).read()
        checks[name] = {"prmtop": os.path.basename(prm), "coords": os.path.basename(crd), "options": opts,
                        "ff": parse_ff(text),
                        "conjgrad_returns": int(re.search(r"conjgrad returns (-?\d+)", text).group(1))}
        out = run([SFFREF, os.path.join(HERE, "ref", os.path.basename(prm)),
                   os.path.join(HERE, "ref", os.path.basename(crd)), "sp", opts, tmp])
        n, e, x, g = read_dump(tmp)
        checks[name]["sp"] = parse_breakdown(out)
        arrays[f"{name}_x"] = x
        arrays[f"{name}_g"] = g
    # xfin (418 atoms, gb=1, kappa, all pairs) through the reference library
    opts = "ntpr=1, gb=1, kappa=0.10395, rgbmax=99., cut=99.0, diel=C"
    out = run([SFFREF, os.path.join(HERE, "ref", "xfin.parm7"), os.path.join(HERE, "ref", "xfin.rst7"), "sp",
               opts, tmp])
    n, e, x, g = read_dump(tmp)
    checks["xfin"] = {"prmtop": "xfin.parm7", "coords": "xfin.rst7", "options": opts, "sp": parse_breakdown(out)}
    arrays["xfin_x"] = x
    arrays["xfin_g"] = g
    # aspgb8: per-atom Born radii and breakdown (test/nab/aspgb8.out, which
    # the current reference reproduces; the .check file is stale)
    text = open(os.path.join(test, "nab", "aspgb8.out")).read()
    radii = {}
    for line in text.splitlines():
        m = re.match(r"(\d+)\t\s*([0-9.]+)\t\s*([0-9.]+)$", line)
        if m:
            radii[int(m.group(1))] = float(m.group(3))
    checks["aspgb8"] = {"prmtop": "asp.top", "coords": "asp.pdb",
                        "options": "rgbmax=100., cut=100.0, nsnb=999, gb=8, diel=C",
                        "reff": [radii[i + 1] for i in range(len(radii))], "sp": parse_breakdown(text)}
    # synthetic molecules through the reference library
    from nabc_gb300 import sff
    L = sff.lib()
    for name, natom, seed, opts in SYNTH:
        prm, x, radius = sff.synth_molecule(natom, seed)
        base = os.path.join(HERE, "synth", f"n{natom}_s{seed}")
        if not os.path.exists(base + ".parm7"):
            L.wrparm(prm, (base + ".parm7").encode())
            L.putxv((base + ".rst7").encode(), b"synthetic", natom, 0.0, sff.dptr(x), None)
        sff.free_prm(prm)
        out = run([SFFREF, base + ".parm7", base + ".rst7", "sp", opts, tmp])
        n, e, xr, g = read_dump(tmp)
        checks[name] = {"prmtop": os.path.basename(base) + ".parm7", "coords": os.path.basename(base) + ".rst7",
                        "options": opts, "sp": parse_breakdown(out), "natom": natom}
        arrays[f"{name}_x"] = xr
        arrays[f"{name}_g"] = g
    # conjgrad and Langevin dynamics of one synthetic molecule
    base = os.path.join(HERE, "synth", "n300_s11")
    opts = "gb=5, cut=999.0, rgbmax=15.0, ntpr=1"
    out = run([SFFREF, base + ".parm7", base + ".rst7", "cg", opts, "20", "1.0", "0.01", tmp])
    n, e, x, g = read_dump(tmp)
    checks["s300_cg"] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                         "ff": parse_ff(out), "maxiter": 20, "dfpred": 1.0, "rmsgrad": 0.01,
                         "conjgrad_returns": int(re.search(r"conjgrad returns (-?\d+)", out).group(1)),
                         "energy": e}
    arrays["s300_cg_x"] = x
    opts = "gb=5, cut=999.0, rgbmax=15.0, ntpr=10, gamma_ln=5.0, temp0=300.0, dt=0.001, ntpr_md=1, zerov=1"
    out = run([SFFREF, base + ".parm7", base + ".rst7", "md", opts, "20", tmp])
    n, e, x, v = read_dump(tmp)
    md_lines = [[float(t) for t in line.split()[1:]] for line in out.splitlines() if line.startswith("md:")]
    checks["s300_md"] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                         "nsteps": 20, "md": md_lines}
    arrays["s300_md_x"] = x
    arrays["s300_md_v"] = v
    # md with centre-of-mass removal: Langevin (translation only) and
    # Berendsen from tempi velocities (translation, velocity and rotation)
    for name, opts in (("s300_md_nscm", "gb=5, cut=999.0, rgbmax=15.0, ntpr=10, gamma_ln=5.0, temp0=300.0, "
                                        "dt=0.001, ntpr_md=1, zerov=1, nscm=4"),
                       ("s300_md_nscm_vw", "gb=5, cut=999.0, rgbmax=15.0, ntpr=10, gamma_ln=0.0, temp0=300.0, "
                                           "tempi=300.0, tautp=0.2, dt=0.001, ntpr_md=1, nscm=3")):
        out = run([SFFREF, base + ".parm7", base + ".rst7", "md", opts, "20", tmp])
        n, e, x, v = read_dump(tmp)
        md_lines = [[float(t) for t in line.split()[1:]] for line in out.splitlines() if line.startswith("md:")]
        checks[name] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                        "nsteps": 20, "md": md_lines}
        arrays[f"{name}_x"] = x
        arrays[f"{name}_v"] = v
    # RATTLE: md with bonds to hydrogen (rattle=2) and all bonds (rattle=1)
    # constrained, and mme_rattle on a structure with perturbed bonds
    for name, opts in (("s300_md_rattle2", "gb=5, cut=999.0, rgbmax=15.0, ntpr=10, gamma_ln=5.0, temp0=300.0, "
                                           "dt=0.002, ntpr_md=1, zerov=1, rattle=2"),
                       ("s300_md_rattle1", "gb=5, cut=999.0, rgbmax=15.0, ntpr=10, gamma_ln=5.0, temp0=300.0, "
                                           "dt=0.002, ntpr_md=1, zerov=1, rattle=1")):
        out = run([SFFREF, base + ".parm7", base + ".rst7", "md", opts, "20", tmp])
        n, e, x, v = read_dump(tmp)
        md_lines = [[float(t) for t in line.split()[1:]] for line in out.splitlines() if line.startswith("md:")]
        checks[name] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                        "nsteps": 20, "md": md_lines}
        arrays[f"{name}_x"] = x
        arrays[f"{name}_v"] = v
    opts = "gb=5, cut=999.0, rgbmax=15.0, ntpr=1, rattle=2"
    out = run([SFFREF, base + ".parm7", base + ".rst7", "spr", opts, tmp])
    n, e, x, g = read_dump(tmp)
    checks["s300_rattle_sp"] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                                "shift": 0.02, "energy": e,
                                "frms": float(re.search(r"frms:\s+([0-9.eE+-]+) \(corrected", out).group(1))}
    arrays["s300_rattle_sp_x"] = x
    arrays["s300_rattle_sp_g"] = g
    # positional restraints (econs): every 7th atom held to shifted positions
    opts = "gb=5, cut=999.0, rgbmax=15.0, ntpr=1, wcons=2.5"
    out = run([SFFREF, base + ".parm7", base + ".rst7", "spc", opts, "7", tmp])
    n, e, x, g = read_dump(tmp)
    checks["s300_cons"] = {"prmtop": "n300_s11.parm7", "coords": "n300_s11.rst7", "options": opts,
                           "every": 7, "shift": 0.05, "sp": parse_breakdown(out), "energy": e}
    arrays["s300_cons_g"] = g
    # the reference's md test (test/tmd.c on xfin.md1.rst7: gb=1, cut 20,
    # Langevin 300 K, rattle=1, 500 steps of 1 fs): its shipped .check lines,
    # which the compiled reference reproduces digit for digit
    text = open(os.path.join(test, "tmd.out.check")).read()
    checks["tmd"] = {"prmtop": "xfin.parm7", "coords": "xfin.md1.rst7",
                     "options": "cut=20.0, rgbmax=20.0, ntpr=500, nsnb=10, gb=1, diel=C, gamma_ln=5.0, "
                                "temp0=300.0, ntpr_md=100, rattle=1",
                     "nsteps": 500, "ff": parse_ff(text),
                     "md": [[float(t) for t in line.split()[1:]] for line in text.splitlines()
                            if line.startswith("md:")]}
    # NAB tests on the GB path with shipped outputs: variable 1-4 scaling
    # (per-dihedral SCEE/SCNB factors), TNCG through mme on gbrna, md with
    # RATTLE from tempi velocities (Berendsen with tautp 99999), and md with
    # RATTLE writing a NetCDF trajectory every 10 steps
    nab = os.path.join(test, "nab")
    text = open(os.path.join(nab, "variable_14scale.out.check")).read()
    opts = "ntpr=1, gb=1, cut=99.0, diel=C, e_debug=0"
    out = run([SFFREF, os.path.join(HERE, "ref", "NMA_scee+scnb.prmtop"), os.path.join(HERE, "ref", "NMA.pdb"), "sp",
               opts, tmp])
    checks["variable_14"] = {"prmtop": "NMA_scee+scnb.prmtop", "coords": "NMA.pdb", "options": opts,
                             "ff": parse_ff(text), "sp": parse_breakdown(out)}
    # a single ion: the Born self-energy alone (one atom, no pairs)
    for gbk in (1, 5, 8):
        opts = f"gb={gbk}, cut=999.0, rgbmax=15.0"
        out = run([SFFREF, os.path.join(HERE, "ref", "Na+.parm7"), os.path.join(HERE, "ref", "Na+.pdb"), "sp", opts,
                   tmp])
        checks[f"na_gb{gbk}"] = {"prmtop": "Na+.parm7", "coords": "Na+.pdb", "options": opts,
                                 "sp": parse_breakdown(out)}
    text = open(os.path.join(nab, "txmin.out.check")).read()
    checks["nab_txmin"] = {"prmtop": "gbrna.prmtop", "coords": "gbrna.pdb",
                           "options": "ntpr=1, gb=1, kappa=0.10395, rgbmax=99., cut=99.0, diel=C",
                           "maxiter": 5, "grms_tol": 0.001, "ls_maxatmov": 0.15, "ff": parse_ff(text),
                           "min_lines": [[int(m.group(1)), int(m.group(2)), float(m.group(3)), float(m.group(4))]
                                         for m in re.finditer(r" MIN: Iter =\s*(\d+)\s+NFunc =\s*(\d+)\s+E =\s*(\S+)"
                                                              r"\s+RMSG =\s*(\S+)", text)],
                           "end": [float(t) for t in re.search(r"END:.*E =\s*(\S+)\s+RMSG =\s*(\S+)", text).groups()]}
    for name, check, opts, nsteps in (
            ("nab_rattle_md", "rattle_md.out.check",
             "ntpr=5, gb=1, kappa=0.10395, rgbmax=99., cut=99.0, diel=C, tempi=300., tautp=99999.,rattle=1", 20),
            ("nab_gbnetcdf", "gbnetcdf.out.check",
             "ntpr=10, ntwx=10, ntpr_md=50, gb=1, kappa=0.10395, cut=99.0, diel=C, tempi=300., rattle=1", 100)):
        text = open(os.path.join(nab, check)).read()
        checks[name] = {"prmtop": "gbrna.prmtop", "coords": "gbrna.pdb", "options": opts, "nsteps": nsteps,
                        "ff": parse_ff(text),
                        "md": [[float(t) for t in line.split()[1:]] for line in text.splitlines()
                               if line.startswith("md:")]}
    # XMIN on xfin as the reference's test/txmin.c runs it (L-BFGS through
    # mme_rattle, 50 iterations), the same through mme, and TNCG
    opts = "ntpr=1, gb=1, kappa=0.10395, rgbmax=99., cut=99.0, diel=C"
    tr = os.path.join(HERE, "_trace.bin")
    for name, method, maxiter, gtol, atmov, rattle in (("xfin_xmin", 2, 50, 0.0005, 0.15, 1),
                                                       ("xfin_xmin_mme", 2, 50, 0.0005, 0.15, 0),
                                                       ("xfin_tncg", 3, 10, 0.0005, 0.15, 0)):
        out = run([SFFREF, os.path.join(HERE, "ref", "xfin.parm7"), os.path.join(HERE, "ref", "xfin.rst7"), "xmin",
                   opts, str(method), str(maxiter), str(gtol), str(atmov), str(rattle), tmp, tr])
        n, e, x, g = read_dump(tmp)
        m = re.search(r"xmin returns (\S+) iter (-?\d+) ls_iter (-?\d+) error (-?\d+) grms (\S+)", out)
        mins = parse_min_lines(out)
        checks[name] = {"prmtop": "xfin.parm7", "coords": "xfin.rst7", "options": opts, "method": method,
                        "maxiter": maxiter, "grms_tol": gtol, "ls_maxatmov": atmov, "rattle": rattle,
                        "returns": float(m.group(1)), "iter": int(m.group(2)), "ls_iter": int(m.group(3)),
                        "error_flag": int(m.group(4)), "grms": float(m.group(5)), "min_lines": mins,
                        "final": parse_breakdown(out.split("xmin returns")[1]), "energy": e}
        arrays[f"{name}_x"] = x
        arrays[f"{name}_trace"] = np.fromfile(tr, np.float64)
    os.remove(tr)
    text = open(os.path.join(test, "txmin.out.check")).read()
    checks["xfin_xmin"]["check_file"] = {
        "min_lines": parse_min_lines(text),
        "initial": parse_breakdown(text.split("setting print")[0]),
        "final": parse_breakdown(text.split(" END:")[1])}
    # XMIN on the test functions (bit-for-bit cases)
    xcases = []
    for k, (fn, method, lsm, nd, mlb, maxiter, gtol, atmov) in enumerate(XMIN_CASES):
        out = run([XMINREF, fn, str(method), str(lsm), str(nd), str(mlb), str(maxiter), repr(gtol), repr(atmov),
                   tmp])
        with open(tmp, "rb") as f:
            ndim, ncalls, it, lsit, err = np.frombuffer(f.read(20), np.int32)
            ret, e, grms = np.frombuffer(f.read(24), np.float64)
            rest = np.frombuffer(f.read(), np.float64)
        xcases.append({"function": fn, "method": method, "ls_method": lsm, "numdiff": nd, "m_lbfgs": mlb,
                       "maxiter": maxiter, "grms_tol": gtol, "ls_maxatmov": atmov, "ndim": int(ndim),
                       "iter": int(it), "ls_iter": int(lsit), "error_flag": int(err)})
        arrays[f"xmin{k}_scalars"] = np.array([ret, e, grms])
        arrays[f"xmin{k}_start"] = rest[:ndim]
        arrays[f"xmin{k}_x"] = rest[ndim:2 * ndim]
        arrays[f"xmin{k}_g"] = rest[2 * ndim:3 * ndim]
        arrays[f"xmin{k}_trace"] = rest[3 * ndim:3 * ndim + ncalls]
    checks["xmin_functions"] = {"frozen_chain_atom": 4, "cases": xcases}
    # LMOD on the bead chain (bit-for-bit cases)
    lcases = []
    for name, largs in LMOD_CASES + [LMOD_RESTART_CASE]:
        work = os.path.join(HERE, "_lmod_tmp")
        shutil.rmtree(work, ignore_errors=True)
        os.makedirs(work)
        runs = 2 if name == LMOD_RESTART_CASE[0] else 1
        for _ in range(runs):
            out = run([LMODREF] + [repr(a) if isinstance(a, float) else str(a) for a in largs] + ["out.bin"], cwd=work)
        with open(os.path.join(work, "out.bin"), "rb") as f:
            n, nconf, err, narn = np.frombuffer(f.read(16), np.int32)
            ret, e = np.frombuffer(f.read(16), np.float64)
            rest = np.frombuffer(f.read(), np.float64)
        k = len(lcases)
        d = 3 * int(n)
        arrays[f"lmod{k}_scalars"] = np.array([ret, e])
        arrays[f"lmod{k}_start"] = rest[:d]
        arrays[f"lmod{k}_x"] = rest[d:2 * d]
        arrays[f"lmod{k}_conflib"] = rest[2 * d:2 * d + d * int(nconf)]
        arrays[f"lmod{k}_traj"] = rest[2 * d + d * int(nconf):]
        with open(os.path.join(work, "conflib.dat"), "rb") as f:
            arrays[f"lmod{k}_conflib_dat"] = np.frombuffer(f.read(), np.uint8)
        lcases.append({"name": name, "args": largs, "runs": runs, "nconf": int(nconf), "error_flag": int(err),
                       "ndim_arnoldi": int(narn), "log": out.split("lmod returns")[0]})
        shutil.rmtree(work)
    checks["lmod_chain"] = {"cases": lcases}
    # LMOD through the reference's mme() on asp (GB 1): the test/tlmod.c
    # driver with GB in place of its distance-dependent dielectric
    work = os.path.join(HERE, "_lmod_tmp")
    shutil.rmtree(work, ignore_errors=True)
    os.makedirs(work)
    opts = "ntpr=99999, gb=1, cut=99.0, rgbmax=99.0, nsnb=9999"
    largs = [3, 5, 3, 2, 5, 99, 1e-4, 2000]
    out = run([SFFREF, os.path.join(HERE, "ref", "asp.top"), os.path.join(HERE, "ref", "asp.pdb"), "lmod", opts] +
              [str(a) for a in largs] + ["out.bin"], cwd=work)
    m = re.search(r"lmod returns (\S+) error (-?\d+) nconf (\d+)", out)
    iters = [float(v) for v in re.findall(r"^ +\d+ +E = +(-?[0-9.]+) \(", out, re.M)]
    checks["lmod_asp"] = {"prmtop": "asp.top", "coords": "asp.pdb", "options": opts,
                          "niter": 3, "nmod": 5, "kmod": 3, "mc_option": 2, "nof_lmod_steps": 5, "seed": 99,
                          "grms_tol": 1e-4, "maxiter": 2000, "glob_min": float(m.group(1)),
                          "error_flag": int(m.group(2)), "nconf": int(m.group(3)), "iteration_energies": iters,
                          # the log names the topology file: kept relative to the repository
                          "log": out.split("lmod returns")[0].replace(os.path.dirname(ROOT) + os.sep, "")}
    shutil.rmtree(work)
    os.remove(tmp)
    with open(os.path.join(HERE, "checks.json"), "w") as f:
        json.dump(checks, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "refrun.npz"), **arrays)
    print("wrote", len(checks), "cases")


if __name__ == "__main__":
    main()

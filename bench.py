"""Benchmark of the generalized-Born energy/gradient path on one GB300.

Workload (the single-large-system configuration): one synthetic 25,000-atom
chain molecule, gb=5 (OBC II), rgbmax = 15 A, GB/nonbonded cutoff 25 A
with the GPU-built tile pair list (rebuilt every nsnb = 10 steps), Langevin
dynamics at dt = 2 fs, gamma = 5/ps, 300 K.  One step = one energy+gradient
evaluation plus the integrator update, device-resident.

  value   device-resident evaluations per second (MD steps/s), each step
          timed with CUDA events on the launching stream, L2 flushed
          (256 MiB write) between steps outside the timed events
  e2e     evaluations per second through the reference-facing C ABI
          (mme(x, f, &iter) with pinned host buffers: coordinates copied in
          and gradient copied out inside every timed call; the atoms take an
          md-sized random step between calls, so pair-list remakes happen at
          the md rate)
  reference arm (--impl reference): the same workload on the host CPU
          cores through the FP64 CPU restatement of the reference's egb()/
          mme() (oracle/sffo.c), with its input made by oracle/synth.c, the
          restatement of the library's generator: that process loads no
          library of the product (the reference itself cannot be built on
          the GPU host, which has no copy of its source tree)

Both arms print the same "config": the workload, its options, the
generator's realised radius and density and the pair counts.

Further keys of the same line (--no-batched skips the batched and serving
sections; --only serving|batched|uneven runs one section alone):
  md_long   --md-long steps (10,000) of the workload back to back: ns/day
  small_md  the 2,000-atom all-pairs case (gb=1, cut 999, 1,000 Langevin
            steps at dt 1 fs) on the GPU and through the CPU restatement
  batched   the uneven-size batch (2,048 molecules of 200-20,000 atoms,
            gb=8), 512 conformers of a 3,000-atom molecule (evaluations,
            conjgrad, XMIN L-BFGS) and batched LMOD searches, each against
            the same systems one at a time
  serving   a Poisson stream of minimisation requests (500-50,000 atoms,
            conjgrad to RMS 0.01 or 2,000 evaluations) at 10, 100, 1,000 and
            2,000 requests/s through the server, against one at a time

Multi-GPU (--gpus N under torchrun): independent replicas (the path has
no data exchange between systems), value = total evaluations/s; scaling
weak.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GB energy+force evals/s & pairs/s, batched vs plain at fixed err; p50/p99 ms"
WORKLOAD = "single {natom:,}-atom synthetic molecule, gb=5 (OBC II), rgbmax 15, cut 25, Langevin MD dt 2 fs"
OPTS = "gb=5, rgbmax=15.0, cut=25.0, nsnb=10, dt=0.002, gamma_ln=5.0, temp0=300.0, kappa=0.0"
# Algorithmic work per unordered in-list pair (FP32 flops counted FADD/FMUL
# = 1, FFMA = 2) for the three passes, from the reference formulas at
# kappa = 0 with the far-field Born branch.
FLOPS_PASS = (36.0, 60.0, 62.0)
# MUFU (special-function unit) operations per unordered in-list pair of each
# pass (reciprocal square roots and the exponential of the GB kernel).
MUFU_PASS = (1.0, 4.0, 1.0)
# DRAM bytes (read + write) per launch of each pass on this workload, from
# one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum): the inputs
# (~1.6 MB of per-atom data, the lists) stay in L2, so traffic is far below
# what the FP32 work would allow.
TRAFFIC_PASS = (6.61e6, 21.71e6, 7.12e6)
PASS_NAMES = ("k_born (pass 1, Born radii)", "k_gbpair (pass 2, GB+Coulomb+LJ)", "k_chain (pass 3, chain rule)")
# Per SM and clock: FP32 lanes (an FFMA counts 2 flops) and MUFU results.
FP32_LANES_PER_SM, MUFU_PER_SM = 128, 16
CUT, RGBMAX, NSNB = 25.0, 15.0, 10


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def aggregate(total_ms, e2e_s, steps, e2e_steps, world, dist, device):
    """Whole-job rates of independent replicas: each rank's timed region is
    reduced with MAX over ranks (the job lasts as long as its slowest
    replica) and the units of all ranks are counted."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([total_ms, e2e_s], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_s = float(t[0]), float(t[1])
    return world * steps / (total_ms * 1e-3), world * e2e_steps / e2e_s, total_ms


UNEVEN_OPTS = "gb=8, rgbmax=25.0, cut=30.0"   # GBneck2, the uneven-size batch
CONFORMER_OPTS = "gb=5, cut=999.0"           # OBC II, all pairs, the conformer batch


def make_molecules(sizes, seed0):
    """Synthetic molecules of the given atom counts (seeds seed0 + k),
    generated on all host cores."""
    from concurrent.futures import ThreadPoolExecutor
    from nabc_gb300 import sff
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        return list(ex.map(lambda k: sff.synth_molecule(int(sizes[k]), seed0 + k), range(len(sizes))))


def timed(fn, reps, stream, flush):
    """Device milliseconds of reps calls of fn, each bracketed by CUDA
    events on stream, with L2 flushed between calls (outside the events)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for k in range(reps):
        flush.zero_()
        ev[k][0].record(stream)
        fn()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(c) for a, c in ev]


def uneven_sizes(n):
    """Atom counts of the uneven-size batch: log-uniform 200..20,000."""
    rng = np.random.default_rng(4242)
    return np.floor(np.exp(rng.uniform(np.log(200), np.log(20000), n))).astype(int)


def bench_uneven_alone(args, stream, sp, flush):
    """The uneven-size batch's evaluations alone (no plain loop, no oracle):
    for profiling the batched GBneck evaluation by itself."""
    import torch
    from nabc_gb300.batch import Batch
    sizes = uneven_sizes(args.uneven)
    mols = make_molecules(sizes, 9000)
    b = Batch(UNEVEN_OPTS + (", sffg_tune=0" if args.no_tune else ""))
    for prm, x, _ in mols:
        b.add(prm, x)
    b.finalize()
    b.eval(rebuild=True, stream=sp)
    b.eval(stream=sp)
    torch.cuda.synchronize()
    t = timed(lambda: b.eval(stream=sp), max(1, args.steps), stream, flush)
    res = {"systems": len(sizes), "atoms": int(sizes.sum()), "options": UNEVEN_OPTS, "evals": len(t),
           "ms_per_eval_of_all": float(np.median(t)), "tuned_split_claim_blocks": b.tuned_split()}
    if args.uneven_md > 0:
        # md steps of every molecule at once (the integrator's kernels at
        # millions of atoms)
        b.md_begin(stream=sp)
        steps = [0]

        def one():
            b.md_steps(steps[0], 1, stream=sp)
            steps[0] += 1
        tm = timed(one, args.uneven_md, stream, flush)
        res["md_steps"] = len(tm)
        res["ms_per_md_step_of_all"] = float(np.median(tm))
    b.close()
    return res


def bench_batched(args, stream, sp, flush):
    """Batched versus plain evaluation on the GPU: many systems in one
    flattened work queue (one Batch) against one Batch per system evaluated
    one after another, same systems, same stream."""
    import torch
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    from oracle import oracle
    out = {}

    def compare(opts, systems, reps, label):
        b = Batch(opts)
        for prm, x in systems:
            b.add(prm, x)
        b.finalize()
        b.eval(rebuild=True, stream=sp)
        b.eval(stream=sp)  # the first evaluation without a rebuild tunes the work split
        plain = []
        for prm, x in systems:
            p = Batch(opts)
            p.add(prm, x)
            p.finalize()
            p.eval(rebuild=True, stream=sp)
            p.eval(stream=sp)
            plain.append(p)
        torch.cuda.synchronize()
        t_b = timed(lambda: b.eval(stream=sp), reps, stream, flush)
        t_p = timed(lambda: [p.eval(stream=sp) for p in plain], reps, stream, flush)
        n = len(systems)
        ident = all(np.array_equal(b.energy(k), plain[k].energy(0)) for k in range(n))
        res = {"systems": n, "atoms": int(sum(sff.natom(prm) for prm, _ in systems)), "options": opts,
               "batched_evals_per_s": n * reps / (sum(t_b) * 1e-3),
               "plain_evals_per_s": n * reps / (sum(t_p) * 1e-3),
               "batched_ms_per_eval_of_all": float(np.median(t_b)), "plain_ms_per_loop_of_all": float(np.median(t_p)),
               "same_bits_alone_and_batched": bool(ident)}
        res["speedup"] = res["batched_evals_per_s"] / res["plain_evals_per_s"]
        return b, plain, res

    # uneven-size batch: log-uniform 200..20,000 atoms, each its own topology
    sizes = uneven_sizes(args.uneven)
    mols = make_molecules(sizes, 9000)
    b, plain, res = compare(UNEVEN_OPTS, [(prm, x) for prm, x, _ in mols], 3, "uneven")
    # accuracy of the smallest, the median and the largest molecule against
    # the FP64 oracle
    errs = []
    order = np.argsort(sizes)
    checked = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
    for k in checked:
        prm, x, _ = mols[k]
        o = oracle.Oracle(prm, UNEVEN_OPTS)
        e0, _, g0, _ = o.mme(x)
        errs.append((abs(b.energy(int(k))[0] - e0) / abs(e0), float(np.sqrt(((b.grad(int(k)) - g0) ** 2).mean()))))
    res["energy_rel_max"] = max(e for e, _ in errs)
    res["force_rms_max"] = max(f for _, f in errs)
    res["checked_vs_fp64"] = {"atoms": [int(sizes[k]) for k in checked],
                              "which": "smallest, median and largest molecule of the batch"}
    res["pairs_in_cut"] = int(sum(b.num_pairs(k) for k in range(len(sizes))))
    res["batched_pairs_per_s"] = res["pairs_in_cut"] * res["batched_evals_per_s"] / len(sizes)
    res["plain_pairs_per_s"] = res["pairs_in_cut"] * res["plain_evals_per_s"] / len(sizes)
    b.close()
    for p in plain:
        p.close()
    out["uneven"] = res

    # conformers: one 3,000-atom topology, base + N(0, 0.3^2) per coordinate
    prm, x0, _ = sff.synth_molecule(3000, 777)
    rng = np.random.default_rng(778)
    confs = [(prm, x0 + rng.normal(0.0, 0.3, x0.shape)) for _ in range(args.conformers)]
    b, plain, res = compare(CONFORMER_OPTS, confs, 3, "conformers")
    for p in plain:
        p.close()
    t0 = time.perf_counter()
    st, en = b.cg(args.cg_steps, 0.01, 1.0, stream=sp)
    torch.cuda.synchronize()
    res["cg_steps"] = args.cg_steps
    res["cg_ms_per_step"] = (time.perf_counter() - t0) * 1e3 / args.cg_steps
    res["cg_conformer_steps_per_s"] = args.conformers * args.cg_steps / (time.perf_counter() - t0)
    b.close()
    # the same conformers through batched XMIN (L-BFGS, the reference's
    # minimiser per conformer, evaluations batched)
    from nabc_gb300.batch import Batch
    bx = Batch(CONFORMER_OPTS)
    for prm_c, x_c in confs:
        bx.add(prm_c, x_c)
    bx.finalize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, it, en = bx.xmin(method=2, maxiter=args.xmin_iters, grms_tol=0.01)
    xs = time.perf_counter() - t0
    bx.close()
    res["xmin_lbfgs_iterations"] = args.xmin_iters
    res["xmin_conformer_iterations_per_s"] = float(np.sum(it)) / xs
    res["xmin_seconds"] = xs
    # per-conformer outcome: XMIN's status (0 ended normally: converged or
    # the iteration limit; negative: an error such as y.s = 0)
    codes, counts = np.unique(np.asarray(st), return_counts=True)
    res["xmin_status_counts"] = {str(int(c)): int(k) for c, k in zip(codes, counts)}
    res["xmin_converged"] = int(np.sum((np.asarray(st) == 0) & (np.asarray(it) < args.xmin_iters)))
    res["xmin_at_iteration_limit"] = int(np.sum((np.asarray(st) == 0) & (np.asarray(it) >= args.xmin_iters)))
    res["xmin_errored"] = int(np.sum(np.asarray(st) != 0))
    out["conformers"] = res

    # LMOD searches: small molecules, each searched by the reference's
    # low-mode algorithm; batched (sffg_batch_lmod) against lmod() one
    # molecule after another (timed on a sample, per search)
    if args.lmod_systems > 0:
        import tempfile
        sizes = np.full(args.lmod_systems, 60)
        lm_mols = make_molecules(sizes, 31000)
        lopts = dict(niter=2, nmod=3, kmod=2, mc_option=2, nof_lmod_steps=2, random_seed=11)
        xopts = dict(grms_tol=0.05, maxiter=200, ls_maxatmov=0.15)
        bl = Batch(CONFORMER_OPTS)
        for prm_l, x_l, _ in lm_mols:
            bl.add(prm_l, x_l)
        bl.finalize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, gm, nc, _ = bl.lmod(xmin_opts=xopts, **lopts)
        tb = time.perf_counter() - t0
        bl.close()
        L = sff.lib()
        nplain = min(2, len(lm_mols))
        t_plain = 0.0
        with tempfile.TemporaryDirectory() as d:
            cwd = os.getcwd()
            os.chdir(d)
            try:
                for prm_l, x_l, _ in lm_mols[:nplain]:
                    session = sff.Session(prm_l, CONFORMER_OPTS)
                    na = sff.natom(prm_l)
                    xl = x_l.copy()
                    gl = np.zeros(3 * na)
                    it = C.c_int(-1)
                    t1 = time.perf_counter()
                    e = C.c_double(L.mme(sff.dptr(xl), sff.dptr(gl), C.byref(it)))
                    lo, xo = sff.LMOD_OPT_T(), sff.XMIN_OPT_T()
                    L.lmod_opt_init(C.byref(lo), C.byref(xo))
                    for k, v in lopts.items():
                        setattr(lo, k, v)
                    for k, v in xopts.items():
                        setattr(xo, k, v)
                    conf = np.zeros(3 * na * lo.nconf)
                    traj = np.zeros(3 * na * (lo.niter + 1))
                    zi, zd, nn = C.c_int(0), C.c_double(0.0), C.c_int(na)
                    L.lmod(C.byref(nn), sff.dptr(xl), sff.dptr(gl), C.byref(e), sff.dptr(conf), sff.dptr(traj),
                           C.byref(zi), C.byref(zi), C.byref(zi), C.byref(zd), C.byref(zd), C.byref(zd),
                           C.byref(zd), C.byref(xo), C.byref(lo))
                    t_plain += time.perf_counter() - t1
                    os.remove("conflib.dat")
                    del session
            finally:
                os.chdir(cwd)
        out["lmod"] = {"systems": len(lm_mols), "atoms_each": 60, "options": CONFORMER_OPTS,
                       "lmod_options": lopts, "xmin_options": xopts,
                       "all_ok": bool(np.all(st == 0)),
                       "batched_searches_per_s": len(lm_mols) / tb, "batched_seconds": tb,
                       "plain_searches_per_s": nplain / t_plain, "plain_sample": nplain,
                       "speedup": (len(lm_mols) / tb) / (nplain / t_plain)}
    return out


SERVE_OPTS = "gb=5, cut=999.0"


def bench_serving(args):
    """Poisson stream of minimisation requests (conjgrad to RMS gradient
    0.01 or maxiter evaluations) served with continuous batching, against
    the plain path: the same requests one at a time, each its own batch."""
    from nabc_gb300.batch import Batch
    from nabc_gb300.server import Server
    rng = np.random.default_rng(5150)
    n = args.serve_requests
    sizes = np.floor(np.exp(rng.uniform(np.log(500), np.log(args.serve_max_atoms), n))).astype(int)
    mols = make_molecules(sizes, 12000)
    out = {"requests": n, "atoms_log_uniform": [500, args.serve_max_atoms], "options": SERVE_OPTS,
           "groups": "one per size class" if args.serve_classes else "one minimisation group",
           "rmsgrad": 0.01, "maxiter": args.serve_maxiter, "memory_budget_gb": 150.0}
    # plain: one request at a time
    t0 = time.perf_counter()
    plain_ms = []
    for prm, x, _ in mols:
        t1 = time.perf_counter()
        b = Batch(SERVE_OPTS)
        b.add(prm, x)
        b.finalize()
        b.cg(args.serve_maxiter, 0.01)
        b.close()
        plain_ms.append(round((time.perf_counter() - t1) * 1e3, 1))
    plain_s = time.perf_counter() - t0
    out["plain_requests_per_s"] = n / plain_s
    out["plain_ms_per_request"] = plain_ms
    rates = []
    for rate in args.serve_rates:
        arrive = np.cumsum(rng.exponential(1.0 / rate, n))
        s = Server(SERVE_OPTS + (", sffg_serve_classes=1" if args.serve_classes else ""), memory_budget_gb=150.0,
                   max_groups=16)
        ids = [None] * n
        t0 = time.perf_counter()
        k = 0
        while True:
            now = time.perf_counter() - t0
            while k < n and arrive[k] <= now:
                prm, x, _ = mols[k]
                ids[k] = s.submit(prm, x, "minimize", args.serve_maxiter, 0.01)
                k += 1
            nr, npend = s.pump(16)
            if k == n and nr == 0 and npend == 0:
                break
            if nr == 0 and npend == 0 and k < n:
                time.sleep(max(0.0, min(arrive[k] - (time.perf_counter() - t0), 0.01)))
        span = time.perf_counter() - t0
        res = [s.result(i) for i in ids]
        lat = np.array([r["latency_ms"] for r in res])
        adm = s.counts()
        s.close()
        codes, counts = np.unique([r["status"] for r in res], return_counts=True)
        rates.append({"arrival_per_s": rate, "throughput_requests_per_s": n / span,
                      "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                      "conjgrad_returns": {str(int(c)): int(k) for c, k in zip(codes, counts)},
                      "admission": adm,
                      "per_request": [{"atoms": int(sizes[i]), "status": int(res[i]["status"]),
                                       "latency_ms": round(float(res[i]["latency_ms"]), 1)} for i in range(n)]})
    out["served"] = rates
    out["atoms"] = [int(v) for v in sizes]
    return out


def count_pairs(x, cut, rcut_gb):
    """Unordered pairs within cut and within rgbmax + Fsmax (k-d tree)."""
    from scipy.spatial import cKDTree
    t = cKDTree(x.reshape(-1, 3))
    return int(t.count_neighbors(t, cut) - len(x) // 3) // 2, int(t.count_neighbors(t, rcut_gb) - len(x) // 3) // 2


def cpu_model():
    """The host CPU's model name."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def workload(natom, seed, world):
    """(config, molecule): the workload's description, the same in both
    arms, from oracle/synth.c's molecule (the library generator's molecule
    bit for bit, made without loading the library)."""
    from oracle import oracle
    oracle.build()
    m = oracle.SynthMolecule(natom, seed)
    npairs, npairs_gb = count_pairs(m.x, CUT, RGBMAX + m.fsmax)
    cfg = {"workload": WORKLOAD.format(natom=natom), "natom": natom, "seed": seed, "options": OPTS,
           "generator": "compact self-avoiding chain (bond 1.53 A, angle 111 deg, no non-bonded atom within "
                        "2.5 A), C/N/O/H 0.32/0.09/0.09/0.50, charges N(0, 0.4^2) neutralised",
           "specified_density_per_A3": 0.09,
           "realised_radius_A": m.radius,
           "realised_density_per_A3": natom / (4.0 / 3.0 * math.pi * m.radius ** 3),
           "pairs_in_cut": npairs, "pairs_in_rgbmax_fsmax": npairs_gb,
           "l2": "inputs (~1.6 MB per-atom data + lists) fit L2; a 256 MiB buffer is written between timed "
                 "GPU steps (outside the timed events)",
           "parallelism": f"{world} independent replica(s), one per GPU"}
    return cfg, m


def time_oracle(o, x, n):
    """Seconds for n oracle evaluations at the nsnb cadence (the pair list
    rebuilt on the first and every tenth)."""
    t0 = time.perf_counter()
    for k in range(n):
        o.mme(x, rebuild=(k % NSNB == 0))
    return time.perf_counter() - t0


def cpu_baseline(m, cores, n_all, n_warm=1):
    """The FP64 restatement of the reference's egb()/mme34() on this host:
    n_all evaluations on all threads, and the 1-thread rate from one
    evaluation with a list rebuild and two without, weighted to the
    cadence of one rebuild per nsnb evaluations."""
    from oracle import oracle
    o = oracle.Oracle(m, OPTS)
    oracle.set_threads(cores)
    for _ in range(n_warm):
        o.mme(m.x)
    dt_all = time_oracle(o, m.x, n_all)
    oracle.set_threads(1)
    t0 = time.perf_counter()
    o.mme(m.x, rebuild=True)
    t_rebuild = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.mme(m.x, rebuild=False)
    o.mme(m.x, rebuild=False)
    t_eval = (time.perf_counter() - t0) / 2
    oracle.set_threads(cores)
    o.close()
    return {"value": n_all / dt_all, "unit": "evals/s", "cores": cores, "kind": "port",
            "sample": f"{n_all} mme() evaluations of the workload, pair list rebuilt every {NSNB} "
                      "(FP64 CPU restatement of the reference egb()/mme34() in oracle/sffo.c, OpenMP, "
                      "brute-force pair list)",
            "cpu_model": cpu_model(), "nproc": os.cpu_count(),
            "one_thread_value": NSNB / (t_rebuild + (NSNB - 1) * t_eval),
            "one_thread_sample": "1 thread: one evaluation with a list rebuild and two without, weighted "
                                 f"1:{NSNB - 1}"}


C1_OPTS = "gb=1, cut=999.0, rgbmax=15.0, dt=0.001, gamma_ln=5.0, temp0=300.0, tempi=0.0"


def bench_small_md(args, stream, sp, cores):
    """The small all-pairs case: 2,000 atoms, gb=1 (HCT), cut 999, one
    mme() then 1,000 Langevin md() steps at dt 1 fs, 300 K, gamma 5/ps, from
    zero velocities; on the GPU (device-resident batch md, CUDA events) and
    through the FP64 restatement on all host cores (the full run)."""
    import torch
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    from oracle import oracle
    n, seed, nsteps = 2000, 2000, args.c1_steps
    prm, x, _ = sff.synth_molecule(n, seed)
    b = Batch(C1_OPTS)
    b.add(prm, x)
    b.finalize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    e0.record(stream)
    b.eval(rebuild=True, stream=sp)
    e1.record(stream)
    b.md_begin(stream=sp)
    b.md_steps(0, nsteps, stream=sp)
    e2.record(stream)
    torch.cuda.synchronize()
    sp_ms, md_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)
    b.close()
    sff.free_prm(prm)
    m = oracle.SynthMolecule(n, seed)
    o = oracle.Oracle(m, C1_OPTS + ", ntpr_md=1000000")
    oracle.set_threads(cores)
    t0 = time.perf_counter()
    o.mme(m.x)
    cpu_sp = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.md(m.x, np.zeros_like(m.x), nsteps)
    cpu_md = time.perf_counter() - t0
    o.close()
    return {"natom": n, "options": C1_OPTS, "md_steps": nsteps,
            "gpu_single_point_ms": sp_ms, "gpu_md_ms": md_ms, "gpu_md_steps_per_s": nsteps / (md_ms * 1e-3),
            "gpu_ns_per_day": nsteps * 0.001e-3 / (md_ms * 1e-3) * 86400,
            "cpu_single_point_ms": cpu_sp * 1e3, "cpu_md_s": cpu_md, "cpu_md_steps_per_s": nsteps / cpu_md,
            "cpu_cores": cores, "cpu_kind": "port (FP64 restatement, OpenMP)",
            "gpu_over_cpu_md": (nsteps / (md_ms * 1e-3)) / (nsteps / cpu_md)}


def reference_arm(args, cores):
    """--impl reference: the workload through the FP64 CPU restatement on
    all host cores, with its 1-thread rate; rank 0 only."""
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    cfg, m = workload(args.natom, args.seed, args.gpus)
    cb = cpu_baseline(m, cores, steps, n_warm=warmup)
    rate = cb["value"]
    line = {"metric": METRIC, "value": rate, "unit": "evals/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": warmup, "ms_per_step": 1e3 / rate, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "config": cfg, "cpu_baseline": cb,
            "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--natom", type=int, default=25000)
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--cpu-sample", type=int, default=10, help="evaluations in the CPU-baseline sample")
    ap.add_argument("--md-long", type=int, default=10000, help="steps of the long md run (ns/day)")
    ap.add_argument("--c1-steps", type=int, default=1000, help="md steps of the 2,000-atom all-pairs case")
    ap.add_argument("--uneven", type=int, default=2048, help="molecules in the uneven-size batch")
    ap.add_argument("--conformers", type=int, default=512, help="conformers in the conformer batch")
    ap.add_argument("--cg-steps", type=int, default=200, help="batched conjgrad steps on the conformers")
    ap.add_argument("--xmin-iters", type=int, default=50, help="batched L-BFGS iterations on the conformers")
    ap.add_argument("--lmod-systems", type=int, default=32, help="molecules in the batched LMOD search (0: skip)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-versus-plain measurements")
    ap.add_argument("--no-tune", action="store_true",
                    help="default work split instead of the autotuned one (for profiler runs, whose timing the "
                         "tuner would otherwise follow)")
    ap.add_argument("--serve-requests", type=int, default=12, help="requests per arrival-rate run")
    ap.add_argument("--serve-max-atoms", type=int, default=50000, help="requests log-uniform in 500 .. this")
    ap.add_argument("--serve-maxiter", type=int, default=2000, help="conjgrad evaluation limit per request")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[10.0, 100.0, 1000.0, 2000.0])
    ap.add_argument("--serve-classes", action="store_true",
                    help="serving: one minimisation group per size class (option sffg_serve_classes=1)")
    ap.add_argument("--uneven-md", type=int, default=0, help="with --only uneven: md steps of the whole batch")
    ap.add_argument("--only", choices=["serving", "batched", "uneven"],
                    help="run only this section and print its JSON (for profiling it alone)")
    args = ap.parse_args()
    rank, world, local = rank_info()
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, cores)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from nabc_gb300 import sff
    from nabc_gb300.batch import Batch
    sff.lib()
    sff.set_output(os.devnull)
    if args.only:
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        if args.only == "serving":
            out = bench_serving(args)
        elif args.only == "uneven":
            out = bench_uneven_alone(args, stream, C.c_void_p(stream.cuda_stream), flush)
        else:
            out = bench_batched(args, stream, C.c_void_p(stream.cuda_stream), flush)
        print(json.dumps({args.only: out}))
        return
    seed = args.seed + rank  # each replica its own molecule
    cfg, mol = workload(args.natom, seed, world)
    prm, x, _ = sff.synth_molecule(args.natom, seed)
    assert np.array_equal(x, mol.x), "library and oracle generators disagree"
    n = args.natom
    npairs, npairs_gb = cfg["pairs_in_cut"], cfg["pairs_in_rgbmax_fsmax"]
    props = torch.cuda.get_device_properties(local)
    nsm = props.multi_processor_count

    opts = OPTS + (", sffg_tune=0" if args.no_tune else "")
    b = Batch(opts)
    b.add(prm, x)
    b.finalize()
    # one explicit stream carries the flush, the timing events and every
    # kernel of the library
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = C.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # accuracy at the start point against the FP64 oracle (rank 0)
    err = None
    if rank == 0:
        from oracle import oracle
        b.eval(rebuild=True, stream=sp)
        torch.cuda.synchronize()
        e_gpu, g_gpu = b.energy(0), b.grad(0)
        o = oracle.Oracle(mol, OPTS)
        e0, ene0, g0, _ = o.mme(x)
        o.close()
        err = {"energy_rel": abs(e_gpu[0] - e0) / abs(e0), "force_rms": float(np.sqrt(((g_gpu - g0) ** 2).mean())),
               "oracle": "FP64 CPU restatement of egb()/mme34()"}

    b.md_begin(stream=sp)
    step = 0
    for _ in range(max(3, args.warmup)):
        b.md_steps(step, 1, stream=sp)
        step += 1
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = b.launches()
    overflows0 = sff.lib().sffg_list_overflows()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            b.md_steps(step, 1, stream=sp)
            ev[k][1].record(stream)
            step += 1
        torch.cuda.synchronize()
    launches = b.launches() - launches0
    overflows = sff.lib().sffg_list_overflows() - overflows0
    split = b.tuned_split()
    step_ms = [a.elapsed_time(c) for a, c in ev]
    total_ms = sum(step_ms)

    # device time of each pair pass: events around the passes of a separate
    # run of the same steps (event timing replaces graph replay there)
    b.set_profiling(True)
    b.kernel_times()
    for k in range(max(10, min(args.steps, 50))):
        flush.zero_()
        b.md_steps(step, 1, stream=sp)
        step += 1
    torch.cuda.synchronize()
    pass_ms, nev = b.kernel_times()
    b.set_profiling(False)

    # the long md run: md_long steps back to back (one call), ns/day
    md_long = None
    if args.md_long > 0:
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(stream)
        b.md_steps(step, args.md_long, stream=sp)
        a1.record(stream)
        torch.cuda.synchronize()
        step += args.md_long
        long_ms = a0.elapsed_time(a1)
        md_long = {"steps": args.md_long, "dt_fs": 2.0, "seconds": long_ms * 1e-3,
                   "steps_per_s": args.md_long / (long_ms * 1e-3),
                   "ns_per_day": args.md_long * 2e-6 / (long_ms * 1e-3) * 86400}

    # e2e through the reference-facing C ABI with pinned host buffers
    L = sff.lib()
    L.sffg_options_reset()
    L.mm_options(OPTS.encode())
    frozen = np.zeros(n, np.int32)
    constrained = np.zeros(n, np.int32)
    L.mme_init_sff(prm, sff.iptr(frozen), sff.iptr(constrained), None, None)
    xh = torch.empty(3 * n, dtype=torch.float64, pin_memory=True).numpy()
    fh = torch.empty(3 * n, dtype=torch.float64, pin_memory=True).numpy()
    xh[:] = x
    it = C.c_int(0)
    L.mme(sff.dptr(xh), sff.dptr(fh), C.byref(it))
    it.value = 1
    L.mme(sff.dptr(xh), sff.dptr(fh), C.byref(it))  # untimed: tunes the work split
    e2e_steps = max(10, args.steps // 4)
    e2e_s = 0.0
    # the atoms move between calls as in md (a random walk of 0.02 A per
    # coordinate and call, about a 2 fs step at 300 K), so the timed calls
    # remake pair lists at the md rate; the move is made outside the timing
    walk = np.random.default_rng(args.seed + 1)
    for k in range(e2e_steps):
        xh += walk.normal(0.0, 0.02, xh.shape)
        flush.zero_()
        torch.cuda.synchronize()
        it.value = k + 2
        t0 = time.perf_counter()
        L.mme(sff.dptr(xh), sff.dptr(fh), C.byref(it))
        e2e_s += time.perf_counter() - t0
    value, e2e, total_ms = aggregate(total_ms, e2e_s, args.steps, e2e_steps, world, dist, "cuda")

    if rank != 0:
        dist.barrier() if dist else None
        return

    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 2070.0
    fp32_peak = nsm * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    mufu_peak = nsm * MUFU_PER_SM * sm_mhz * 1e6 / 1e12
    pass_avg = [m_ / max(nev, 1) for m_ in pass_ms]
    pairs_pass = (npairs_gb, npairs, npairs_gb)
    passes = []
    for k in range(3):
        fl = FLOPS_PASS[k] * pairs_pass[k] / (pass_avg[k] * 1e-3) / 1e12
        mu = MUFU_PASS[k] * pairs_pass[k] / (pass_avg[k] * 1e-3) / 1e12
        passes.append({"kernel": PASS_NAMES[k], "avg_launch_ms": pass_avg[k], "pairs": pairs_pass[k],
                       "flops_per_pair": FLOPS_PASS[k], "mufu_per_pair": MUFU_PASS[k],
                       "fp32_tflops": fl, "fp32_frac": fl / fp32_peak,
                       "mufu_tops": mu, "mufu_frac": mu / mufu_peak,
                       "pairs_per_s": pairs_pass[k] / (pass_avg[k] * 1e-3)})
    dom = int(np.argmax(pass_avg))
    flops_dom = FLOPS_PASS[dom] * pairs_pass[dom]

    c1 = None if args.c1_steps <= 0 else bench_small_md(args, stream, sp, cores)
    batched = None if args.no_batched else bench_batched(args, stream, sp, flush)
    serving = None if args.no_batched else bench_serving(args)

    # CPU baseline: the oracle port on the host cores, bounded sample
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cb = cpu_baseline(mol, cores, args.cpu_sample)

    ms_sorted = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair arithmetic, 64-bit fixed-point sums, f64 state",
        "data": "synthetic",
        "config": cfg,
        "pairs_per_s": npairs * value,
        "ns_per_day": value * 0.002 * 86400 * 1e-3 / world,
        "latency_ms": {"p50": ms_sorted[len(ms_sorted) // 2],
                       "p99": ms_sorted[min(len(ms_sorted) - 1, int(0.99 * len(ms_sorted)))]},
        "accuracy_vs_fp64": err,
        "step_ms": [round(v, 4) for v in step_ms],
        "list_store_overflows_in_timed_steps": int(overflows),
        "tuned_split_claim_blocks": split,
        "md_long": md_long,
        "roofline": {"bound": "fp32", "kernel": PASS_NAMES[dom], "achieved": passes[dom]["fp32_tflops"],
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": passes[dom]["fp32_frac"],
                     "traffic": TRAFFIC_PASS[dom],
                     "peak_source": f"nominal FP32 rate ({nsm} SMs x {FP32_LANES_PER_SM} lanes x 2 flops) at the "
                                    f"sampled median SM clock {sm_mhz:.0f} MHz; MUFU peak {nsm} SMs x "
                                    f"{MUFU_PER_SM}/clock; no tensor core or HBM bound applies to the pair passes",
                     "algorithmic_flops_per_launch": flops_dom, "avg_launch_ms": pass_avg[dom],
                     "mufu_peak_tops": mufu_peak, "passes": passes},
        "cpu_baseline": cb,
        "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": 3 * n * 8,
                "d2h_bytes_per_step": 3 * n * 8 + 8 * 8,
                "path": "mme(x, f, &iter) of the C ABI, pinned host buffers"},
        "gpu_launches": launches,
        "clocks": clocks,
        "small_md": c1,
        "batched": batched,
        "serving": serving,
    }
    print(json.dumps(line))
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()

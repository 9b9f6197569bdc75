/*
 * sffg.h -- the batched and serving API of libsffg (no counterpart in the
 * reference, which evaluates one process-global system at a time).
 *
 * A batch holds many independent systems (conformers or molecules of any
 * size) resident on one GPU.  One evaluation computes every system's
 * generalized-Born energy and gradient in a single flattened work queue.
 * The model options (gb, cut, rgbmax, kappa, epsext, dielc, nsnb) use the
 * mm_options() grammar and are shared by all systems of a batch.
 *
 * Every call returns SFFG_OK (0) or a negative status and never exits the
 * process; sffg_last_error() describes the most recent failure on the
 * calling thread.  Streams are passed as void* (a cudaStream_t; NULL is the
 * legacy default stream).  A handle must not be used from two threads at
 * once.
 */
#ifndef SFFG_SFFG_H
#define SFFG_SFFG_H

#include <stddef.h>

#include "sff.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SFFG_OK 0
#define SFFG_EINVAL (-1)    /* bad argument or option */
#define SFFG_ENOMEM (-2)    /* device or host allocation failed, or budget exceeded */
#define SFFG_ECUDA (-3)     /* a CUDA call failed */
#define SFFG_ESTATE (-4)    /* call not valid in the handle's current state */
#define SFFG_ENONFINITE (-5) /* non-finite coordinates or energy in a system */
#define SFFG_ENODEV (-6)    /* no usable CUDA device */
#define SFFG_ECONSTRAINT (-7) /* RATTLE's sweeps reached their limit in md (the reference stops there) */

/* Energy components of one system, in the reference's ene[] layout
 * (src/sff/eff.c:2864-2874): 0 total, 1 vdW, 2 elec, 3 bond, 4 angle,
 * 5 dihedral, 7 1-4 vdW, 8 1-4 elec, 10 generalized Born. */
#define SFFG_NENE 13

const char *sffg_last_error(void);

/* Restores every mm_options() setting to the reference's defaults
 * (src/sff/sff.c:68-199).  mm_options() settings are cumulative, as in the
 * reference; this gives test harnesses and long-lived services a clean
 * start. */
void sffg_options_reset(void);

/* ---- synthetic molecules (benchmarks and tests) ------------------------ */

/* A compact self-avoiding chain molecule of natom atoms generated from seed
 * (see the README of the package for the recipe).  Writes 3*natom
 * coordinates into x and the realised confining radius into *radius.
 * Release the topology with free_prm(). */
PARMSTRUCT_T *sffg_synth_molecule(int natom, unsigned long long seed, double *x,
                                  double *radius);

/* ---- batches ------------------------------------------------------------ */

typedef struct sffg_batch sffg_batch;

int sffg_batch_create(const char *opts, sffg_batch **out);
/* Adds a system (topology borrowed only during the call; coordinates x,
 * 3*Natom doubles; frozen may be NULL).  Returns the system index. */
int sffg_batch_add_system(sffg_batch *b, PARMSTRUCT_T *prm, const int *frozen, const double *x,
                          int *sys_index);
/* Harmonic positional restraints of one system (the reference's
 * constrained/x0 arguments of mme_init_sff with the option wcons,
 * src/sff/eff.c:17-80): atoms with constrained[i] != 0 are held to x0
 * (3*Natom).  Before finalize; the arrays are copied. */
int sffg_batch_set_restraints(sffg_batch *b, int sys, const int *constrained, const double *x0);
/* Uploads topologies and allocates device state; no systems may be added
 * afterwards. */
int sffg_batch_finalize(sffg_batch *b);
int sffg_batch_num_systems(const sffg_batch *b);
int sffg_batch_num_atoms(const sffg_batch *b, int sys);

/* Copies coordinates of one system host->device (stream-ordered). */
int sffg_batch_set_coords(sffg_batch *b, int sys, const double *x, void *stream);
int sffg_batch_get_coords(sffg_batch *b, int sys, double *x, void *stream);
/* Energy and gradient of every system.  The pair lists are rebuilt when
 * rebuild != 0 and on the first evaluation. */
int sffg_batch_eval(sffg_batch *b, int rebuild, void *stream);
int sffg_batch_get_energy(sffg_batch *b, int sys, double *ene, void *stream);
int sffg_batch_get_grad(sffg_batch *b, int sys, double *g, void *stream);
/* Effective Born radii of the last evaluation, in atom order. */
int sffg_batch_get_reff(sffg_batch *b, int sys, double *reff, void *stream);
/* Per-system status: status[s] is SFFG_OK; SFFG_ENONFINITE once an
 * evaluation met a non-finite coordinate of system s (its results are then
 * meaningless; the other systems' results are unaffected; setting the
 * system's coordinates again clears it); or SFFG_ECONSTRAINT once RATTLE's
 * sweeps (md with the option rattle = 1 or 2) reached their limit of 1,000
 * for system s, where the reference stops with "ERROR in RATTLE".
 * Synchronises the stream. */
int sffg_batch_status(sffg_batch *b, int *status, void *stream);

/* Number of unordered pairs on the current pair lists of one system. */
long long sffg_batch_num_pairs(sffg_batch *b, int sys);

/* Langevin md() on every system with device Philox noise (the reference's
 * integrator, src/sff/sff.c:2223-2354, options dt/temp0/gamma_ln/...).
 * Velocities start at zero unless set with sffg_batch_set_velocities.  With
 * the option rattle = 1 (all bonds) or 2 (bonds to hydrogen) every system's
 * bond lengths are held by RATTLE (src/sff/rattle.c) on the device, with the
 * reference's sweep order and arithmetic. */
int sffg_batch_md(sffg_batch *b, int nsteps, void *stream);
/* The same integrator split for callers that drive it step by step: md_begin
 * evaluates the first force and initial accelerations; md_steps advances
 * nsteps steps numbered step0+1 .. step0+nsteps. */
int sffg_batch_md_begin(sffg_batch *b, void *stream);
int sffg_batch_md_steps(sffg_batch *b, int step0, int nsteps, void *stream);
int sffg_batch_set_velocities(sffg_batch *b, int sys, const double *v, void *stream);
int sffg_batch_get_velocities(sffg_batch *b, int sys, double *v, void *stream);

/* Checkpoint and resume of batched md (no counterpart in the reference,
 * whose md() cannot resume: its noise generator's state is not saved,
 * src/sff/rand2.c:22-25).  save writes every system's coordinates,
 * velocities, accelerations and Berendsen factors; load reads them into a
 * batch of the same systems and evaluates there with fresh pair lists.
 * Continued with sffg_batch_md_steps from the saved step number (the noise
 * is counter-based), a run repeats the original bit for bit when the batch
 * was built from the same topologies and initial coordinates and the state
 * was saved right after a step whose number is a multiple of nsnb (where md
 * rebuilds its lists) and not of nscm.  SFFG_EINVAL for a file of another
 * batch. */
int sffg_batch_save(sffg_batch *b, const char *path, void *stream);
int sffg_batch_load(sffg_batch *b, const char *path, void *stream);

/* Batched conjgrad() (src/sff/conjgrad.c:34): each system runs its own
 * copy of the reference's state machine; at most maxiter evaluations.
 * status[sys] receives the reference's return code (>0 converged after that
 * many evaluations, -1..-4 as the reference) and energy[sys] the final
 * energy; either may be NULL. */
int sffg_batch_cg(sffg_batch *b, int maxiter, double rmsgrad, double dfpred, int *status,
                  double *energy, void *stream);

/* XMIN on every system at once (no counterpart in the reference, whose
 * xmin(), src/sff/xminC.c:2997, minimises one system): each system runs its
 * own copy of the reference's minimiser with the options xo
 * (mol_struct_opt must be 1; print_level is ignored), and their energy
 * evaluations are batched on the GPU.  The pair lists are rebuilt for the
 * whole batch whenever any system's minimiser asks for a rebuild; that
 * regroups the other systems' lists (and, with a finite cutoff, may change
 * their pair sets), so a system of a mixed batch follows its lone run only
 * to FP32 rounding, while a one-system batch ends bit for bit where xmin()
 * over mme() ends.  Runs are deterministic.  status[s] receives the
 * system's error_flag (0, the reference's negative code -1..-6, or -7 when
 * the system's energy turned non-finite, which ends that system alone),
 * iters[s] its iteration count and energy[s] its final energy (0 on an
 * error); any may be NULL.  The minimised coordinates stay in the batch
 * (sffg_batch_get_coords). */
int sffg_batch_xmin(sffg_batch *b, const XMIN_OPT_T *xo, int *status, int *iters, double *energy, void *stream);

/* LMOD searches on every system of the batch at once: each system runs the
 * reference's search (lmod(), include/sff.h) with the options lo -- its
 * minimisations by XMIN with xo, the tolerances set as lmod() sets them --
 * and its own random stream seeded lo->random_seed + s; ligand moves
 * (nlig), printout and conflib.dat are not used.  All systems' evaluations
 * of a turn run as one pass over the batch.  status[s]: 0, a negative LMOD
 * status, or -8 if the system's energy turned non-finite; glob_min[s] its
 * lowest energy; nconf[s] the structures returned.  conflib (may be NULL)
 * receives system s's structures, lowest first, at offset
 * lo->nconf * 3 * (atom offset of s), room for lo->nconf * 3 * natom(s)
 * doubles each.  Each system's lowest structure is left in the batch
 * (sffg_batch_get_coords).  A one-system batch takes lmod()'s path bit for
 * bit; in a larger batch pair-list rebuilds one search asks for change the
 * others' FP32 rounding.  No reference counterpart. */
int sffg_batch_lmod(sffg_batch *b, const LMOD_OPT_T *lo, const XMIN_OPT_T *xo, int *status, double *glob_min,
                    int *nconf, double *conflib, void *stream);

/* LMOD over any energy function: the reference's lmod() driver
 * (src/sff/lmodC.c:3108-3462, which hard-wires mme()) with func in mme()'s
 * place, for its energies and for the xmin() minimisations.  Arguments and
 * result as lmod() (include/sff.h).  No reference counterpart. */
REAL_T sffg_lmod_func(REAL_T (*func)(REAL_T *, REAL_T *, INT_T *), INT_T *natm, REAL_T *xyz, REAL_T *grad,
                      REAL_T *energy, REAL_T *conflib, REAL_T *lmod_trajectory, INT_T *lig_start, INT_T *lig_end,
                      INT_T *lig_cent, REAL_T *tr_min, REAL_T *tr_max, REAL_T *rot_min, REAL_T *rot_max,
                      XMIN_OPT_T *xo, LMOD_OPT_T *lo);

/* The nev eigenpairs of smallest magnitude of a symmetric n x n operator
 * (thick-restart Lanczos, the solver LMOD takes its low modes from, in place
 * of the reference's ARPACK dsaupd/dseupd with which = "SM"): matvec(x, y,
 * ctx) stores y = A x; nev < ncv <= n basis vectors, relative residual bound
 * tol, at most max_restarts restarts.  values[nev] receives the converged
 * eigenvalues in ascending order, vectors[nev * n] the eigenvectors one
 * after another.  Returns the number converged, or -1. */
int sffg_low_modes(int n, int nev, int ncv, double tol, int max_restarts,
                   void (*matvec)(const double *x, double *y, void *ctx), void *ctx, double *values,
                   double *vectors);

/* Kernel launches issued by this batch since it was created. */
long long sffg_batch_launch_count(const sffg_batch *b);
/* With profiling on, the three pair passes of every evaluation are
 * bracketed by CUDA events on the launching stream; kernel_times returns
 * the accumulated device milliseconds of pass 1 (Born radii), pass 2 (GB +
 * Coulomb + LJ) and pass 3 (chain rule) and the number of evaluations
 * timed, then clears the accumulators. */
int sffg_batch_set_profiling(sffg_batch *b, int on);
int sffg_batch_kernel_times(sffg_batch *b, double *ms3, long long *nevals);

/* The work split of pair pass `pass` (0: Born radii, 1: GB + Coulomb + LJ,
 * 2: chain rule): work items a warp claims per grab of the queue and
 * persistent blocks.  With the option sffg_tune=1 (default) batches of
 * 20,000 atoms or more choose it by timing candidates at their first
 * evaluation without a list rebuild; results do not depend on it. */
int sffg_batch_tuned_split(const sffg_batch *b, int pass, int *claim, int *blocks);

/* Device memory the batch holds, in bytes. */
size_t sffg_batch_device_bytes(const sffg_batch *b);
int sffg_batch_destroy(sffg_batch *b);

/* ---- serving ------------------------------------------------------------ */

/* A request loop with continuous batching (no counterpart in the
 * reference).  Requests -- a minimisation (the reference's conjgrad() to
 * rmsgrad or nsteps evaluations) or nsteps of Langevin md with the batch
 * integrator -- are admitted in arrival order while they fit the
 * device-memory budget.  Requests run in groups, one batch on its own
 * stream each.  A minimisation joins the running minimisation group: it
 * enters that batch's flattened work queue at the group's next turn that is
 * a multiple of nsnb, where the running systems move into a new batch with
 * the newcomers.  With no such group, or for md, it starts a new group.
 * (Option sffg_serve_classes=1: one minimisation group per size class --
 * under 4,096 atoms, then one class per doubling.)
 * Every sffg_server_pump launches the next `turns` evaluations or steps of
 * every group whose earlier turns have finished, waits until some group's
 * turns finish, and takes the result of every system that ended.  A result
 * is the same whether the request ran alone or among others, and whether
 * it joined or started a group.  All requests of a server share its model
 * options.  Not thread-safe: one thread drives a server. */
#define SFFG_REQ_MINIMIZE 0
#define SFFG_REQ_MD 1

typedef struct sffg_server sffg_server;

/* memory_budget_gb: device memory the running groups may hold (an estimate
 * per request at admission, the measured size once admitted); max_groups:
 * groups running at once. */
int sffg_server_create(const char *opts, double memory_budget_gb, int max_groups, sffg_server **out);
/* Copies the topology and coordinates (3*Natom) of one request; *id
 * identifies it.  SFFG_ENOMEM when the request alone exceeds the budget. */
int sffg_server_submit(sffg_server *s, PARMSTRUCT_T *prm, const double *x, int kind, int nsteps, double rmsgrad,
                       long long *id);
/* Admit, launch, wait for one group, collect; reports the groups running
 * and the requests waiting. */
int sffg_server_pump(sffg_server *s, int turns, int *nrunning, int *npending);
/* The result of a finished request: the driver's return code (conjgrad's,
 * or the steps run for md; SFFG_ENONFINITE when its coordinates turned
 * non-finite; another negative SFFG status, with a NaN energy, when the
 * batch it was to run in could not be formed), final energy, coordinates
 * (3*Natom, may be NULL) and the time from submission to the end, in ms.
 * SFFG_ESTATE while it runs or waits. */
int sffg_server_result(sffg_server *s, long long id, int *status, double *energy, double *x, double *latency_ms);
/* Device memory the running groups hold (bytes). */
size_t sffg_server_device_bytes(const sffg_server *s);
/* Counts since creation (any pointer may be NULL): groups started, joins
 * (a running group's batch formed again with newcomers), requests that
 * entered a running group by a join, and the host milliseconds spent
 * forming batches (starts and joins). */
int sffg_server_counts(const sffg_server *s, long long *groups_started, long long *joins, long long *joined,
                       double *form_ms);
/* The most recent failure of this server. */
const char *sffg_server_error(const sffg_server *s);
int sffg_server_destroy(sffg_server *s);

/* ---- Born radii without allocation ------------------------------------- */

/* Largest molecule sffg_born_radii_static accepts: its scratch is one fixed
 * device array of SFFG_STATIC_MAX_ATOMS x 104 bytes (about 0.85 MB). */
#define SFFG_STATIC_MAX_ATOMS 8192

/* Effective Born radii of one molecule, every pair listed (pass 1 of the
 * reference's egb() and its HCT/OBC radius formula, src/sff/eff.c:1566-1733,
 * as when cut exceeds the molecule's extent).  No counterpart in the
 * reference, which keeps the radii internal to egb().
 *
 * It allocates nothing: no cudaMalloc/cudaFree and no other allocating
 * routine.  It is meant for callers that cannot allocate -- a host whose
 * device memory is all owned by its own pool or budget, where one more
 * cudaMalloc can fail or fragment it, or a loop that must not stall, which
 * cudaFree would do by synchronising the device.  Every working buffer
 * lives in one statically sized device array.
 *
 * x: 3*natom coordinates; rborn, fs: the topology's RADII and SCREEN values
 * (PARMSTRUCT_T Rborn and Fs); gb: 1 (HCT), 2 (OBC I) or 5 (OBC II), with
 * the reference's offset 0.09; reff: natom radii out.  All four are host
 * arrays.  The call is ordered on stream (NULL: the legacy default stream)
 * and returns once reff is written.
 *
 * Every call looks up the static array's device address for the device
 * current at the call (cudaGetSymbolAddress, which allocates nothing); the
 * first call on a device also loads this library's device code there.
 * The call copies through pageable host memory and waits for its stream,
 * so it must not be made on a stream that is being captured: it returns
 * SFFG_EINVAL there and leaves the capture intact.
 *
 * All calls on one device share the one array: calls whose GPU work
 * overlaps (different streams or threads) race and corrupt each other's
 * results, so serialise them.
 *
 * Returns SFFG_OK; SFFG_ENOMEM when natom > SFFG_STATIC_MAX_ATOMS (the
 * molecule does not fit the static scratch); SFFG_EINVAL for natom < 1, a
 * NULL array, another gb, rgbmax <= 0 or a capturing stream; SFFG_ENODEV /
 * SFFG_ECUDA when no device is current or a CUDA call fails (after waiting
 * for any of its work already queued).  On entry it clears the CUDA
 * runtime's last-error state, so an earlier unrelated launch failure is not
 * reported as its own.  It does not update
 * sffg_last_error(), which would need a host allocation. */
int sffg_born_radii_static(int natom, const double *x, const double *rborn, const double *fs, int gb,
                           double rgbmax, double *reff, void *stream);

/* ---- pair-list builds ---------------------------------------------------- */

/* Pair-list rebuilds inside device-resident md (sffg_batch_md,
 * sffg_batch_md_steps, md requests of the server) and inside mme() launch
 * all their stages without reading counts back to the host: the list
 * stores keep 50% headroom over the last build's counts and the stages
 * check the stores' capacities on the device.  When a store proves too
 * small (the pairs grew by more than the headroom between two rebuilds),
 * mme() redoes its evaluation with the stores sized exactly, and md
 * replays the steps since that rebuild from a snapshot of the state it
 * started from, before any result is read; the results are the ones an
 * exactly sized build gives.  Returns how many rebuilds of this process
 * were redone that way. */
long long sffg_list_overflows(void);

/* ---- checked build ------------------------------------------------------ */

/* A library built with -DSFFG_CHECKED (for example SFFG_NVCC_EXTRA=
 * -DSFFG_CHECKED SFFG_BUILD_DIR=<dir> python -m nabc_gb300._build) tests
 * every indirect index of its kernels against the array's extent and, on a
 * failure, records a code (1 list entry slot, 2 tile, 3 Lennard-Jones row,
 * 4 neck table, 5 bonded-term atom) and reads element 0 instead, without
 * trapping.  Returns the first code recorded, 0 when every check passed,
 * -1 in the normal build. */
int sffg_checked_code(void);

#ifdef __cplusplus
}
#endif

#endif /* SFFG_SFFG_H */

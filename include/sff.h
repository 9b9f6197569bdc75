/*
 * sff.h -- the C ABI of the generalized-Born energy/gradient path, as a
 * drop-in replacement for the SFF library of dacase/nabc.
 *
 * Every declaration here mirrors one in the reference's src/sff/sff.h; the
 * comment on each gives the reference line it replaces.  The topology struct
 * keeps the reference's exact field order and types (src/sff/sff.h:40-62) so
 * that a driver compiled against the reference header (for example
 * test/tmd.c) links against libsffg.so unchanged.
 *
 * Semantics that callers rely on (src/sff/eff.c:2432-2439, sff.c:858-1846):
 *  - coordinates x and gradients f are double[3*Natom], xyz interleaved;
 *    f is the gradient dE/dx (md() integrates -f);
 *  - units are kcal/mol, Angstrom, charges pre-multiplied by 18.2223;
 *  - mme_init_sff borrows prm, frozen and constrained for the life of the
 *    session and modifies prm in place (charges scaled by 1/sqrt(dielc),
 *    screening factors overwritten for gb=7/8);
 *  - the iter argument of mme: >=0 normal call (pair list rebuilt on the
 *    first call and whenever iter%nsnb==0, "ff:" line every ntpr),
 *    -1 verbose energy breakdown, -3 release per-session state,
 *    -4 force a pair-list rebuild, other negatives quiet with no rebuild;
 *  - errors in these legacy entry points are fail-stop (message, exit(1)),
 *    as in the reference; the batched API in sffg.h returns status codes.
 *
 * The library is one GPU-resident session: these entry points are not
 * re-entrant, like the reference's process-global state.
 */
#ifndef SFFG_SFF_H
#define SFFG_SFF_H

#include <stdio.h>
#include <stddef.h>

#ifndef FALSE
#define FALSE 0
#endif
#ifndef TRUE
#define TRUE 1
#endif

typedef int INT_T;
typedef size_t SIZE_T;
#define REAL_T double
typedef char STRING_T;
typedef FILE FILE_T;

#define NAMESIZE 6
typedef char NAME_T[NAMESIZE];

/* Topology read from a parm7 file (src/sff/sff.h:40-62, same layout). */
typedef struct parm {
  char ititl[81];
  INT_T IfBox, Nmxrs, IfCap,
      Natom, Ntypes, Nbonh, Mbona, Ntheth, Mtheta,
      Nphih, Mphia, Nhparm, Nparm, Nnb, Nres,
      Nbona, Ntheta, Nphia, Numbnd, Numang, Nptra,
      Natyp, Nphb, Nat3, Ntype2d, Nttyp, Nspm, Iptres, Nspsol,
      Ipatm, Natcap, Numextra;
  NAME_T *AtomNames, *ResNames, *AtomType, *AtomTree;
  REAL_T *Charges, *Masses, *Rk, *Req, *Tk, *Teq, *Pk, *Pn, *Phase,
      *Solty, *Cn1, *Cn2, *HB12, *HB10, *Rborn, *Fs;
  REAL_T Box[4], Cutcap, Xcap, Ycap, Zcap, Fsmax;
  INT_T *Iac, *Iblo, *Cno, *Ipres, *ExclAt, *TreeJoin,
      *AtomRes, *BondHAt1, *BondHAt2, *BondHNum, *BondAt1, *BondAt2,
      *BondNum, *AngleHAt1, *AngleHAt2, *AngleHAt3, *AngleHNum,
      *AngleAt1, *AngleAt2, *AngleAt3, *AngleNum, *DihHAt1,
      *DihHAt2, *DihHAt3, *DihHAt4, *DihHNum, *DihAt1, *DihAt2,
      *DihAt3, *DihAt4, *DihNum, *Boundary, *AtomicNum;
  INT_T *N14pairs, *N14pairlist;
  REAL_T *Gvdw, *Scee, *Scnb, *N14sceelist, *N14scnblist;
  INT_T Nstrand, Ncomplex;
  INT_T *Ipstrand, *Ipcomplex;
} PARMSTRUCT_T;

#ifdef __cplusplus
extern "C" {
#endif

/* Output stream for every printed line; defined by the caller, as in the
 * reference (src/sff/sff.h:116, test/tmd.c:18). */
extern FILE *nabout;

/* Option string "key=value, ..." with the reference's grammar
 * (src/sff/sff.h:139, src/sff/mm_options.l:18-97). Keys prefixed "sffg_"
 * are this library's own additions. */
INT_T mm_options(STRING_T *opts);

/* Start a session on prm (src/sff/sff.h:148, src/sff/sff.c:858). */
INT_T mme_init_sff(PARMSTRUCT_T *prm, INT_T *frozen, INT_T *constrained,
                   REAL_T *x0, STRING_T *ncname);

/* Energy and gradient; returns the total energy (src/sff/sff.h:141,
 * src/sff/sff.c:1854 -> eff.c:2442). */
REAL_T mme(REAL_T *x, REAL_T *f, INT_T *iter);

/* Velocity-Verlet Langevin/Berendsen dynamics driven by func
 * (src/sff/sff.h:136, src/sff/sff.c:2071). */
INT_T md(INT_T n, INT_T maxstep, REAL_T *x, REAL_T *f, REAL_T *v,
         REAL_T (*func)(REAL_T *, REAL_T *, INT_T *));

/* Conjugate-gradient minimisation driven by func (src/sff/sff.h:124,
 * src/sff/conjgrad.c:34). */
INT_T conjgrad(REAL_T *x, INT_T *n, REAL_T *f,
               REAL_T (*func)(REAL_T *, REAL_T *, INT_T *),
               REAL_T *rmsgrad, REAL_T *dfpred, INT_T *maxiter);

/* Name the checkpoint files mme() writes every nchk iterations (option
 * nchk, default 10000): the coordinates in the reference's Cartesian
 * format, the name's leftmost "%d" replaced by the iteration number or the
 * number appended (src/sff/sff.h:140, sff.c:789-830, 2056; eff.c:2536). */
void mm_set_checkpoint(STRING_T **fname);

/* Print the timing summary (src/sff/sff.h:149, src/sff/timer.c:71). */
INT_T mme_timer(void);

/* mme() of a structure whose bond lengths RATTLE first restores (rattle=1:
 * all bonds, rattle=2: bonds to hydrogen), with the gradient projected onto
 * the constraints (src/sff/sff.h:147, sff.c:1882-2010).  md() applies the
 * same constraints after each drift and kick when the rattle option is
 * set (sff.c:2251-2280). */
REAL_T mme_rattle(REAL_T *x, REAL_T *f, INT_T *iter);

/* Options of the XMIN minimiser, the reference's layout and meaning
 * (src/sff/sff.h:64-84): method 1 PRCG, 2 L-BFGS, 3 L-BFGS-preconditioned
 * TNCG, 4 gradient check; ls_method 1 Armijo, 2 More-Thuente (Wolfe);
 * numdiff 1 forward, 2 central differences for TNCG's Hessian products;
 * print_level 0 quiet, 1 every iteration, 2 with line-search details, n > 2
 * every n-th iteration.  iter, ls_iter, xmin_time and error_flag are
 * outputs. */
typedef struct xmin_opt {
  INT_T mol_struct_opt;
  INT_T maxiter;
  REAL_T grms_tol;
  INT_T method;
  INT_T numdiff;
  INT_T m_lbfgs;
  INT_T iter;
  REAL_T xmin_time;
  INT_T ls_method;
  INT_T ls_maxiter;
  REAL_T ls_maxatmov;
  REAL_T beta_armijo;
  REAL_T c_armijo;
  REAL_T mu_armijo;
  REAL_T ftol_wolfe;
  REAL_T gtol_wolfe;
  INT_T ls_iter;
  INT_T print_level;
  INT_T error_flag;
} XMIN_OPT_T;

/* Defaults of the XMIN options (src/sff/sff.h:168, xminC.c:2976). */
INT_T xmin_opt_init(struct xmin_opt *xo);

/* Minimise func from xyz with XMIN (src/sff/sff.h:169-170,
 * xminC.c:2997): natm atoms (mol_struct_opt=1; atoms whose gradient in
 * grad is exactly zero on entry stay fixed) or natm dimensions
 * (mol_struct_opt=0).  func gets -4 (rebuild the pair list), -2 (keep it)
 * or the iteration count as its third argument, as mme() reads it.  On
 * return xyz, grad, energy and grms hold the minimum; the return value is
 * the energy, or 0 with xo->error_flag < 0 on an error. */
REAL_T xmin(REAL_T (*func)(REAL_T *, REAL_T *, INT_T *), INT_T *natm,
            REAL_T *xyz, REAL_T *grad, REAL_T *energy, REAL_T *grms,
            struct xmin_opt *xo);

/* XMIN's reverse-communication form (src/sff/sff.h:171-176,
 * xminC.c:2491): call with *label = 0; while it returns *label = 1,
 * evaluate energy and gradient at xyz_ext (pair-list policy in
 * *return_flag: 4-6 rebuild, 7-9 keep) and call again; *label = 0 and
 * *return_flag = 0 mean done, *label < 0 an error. */
REAL_T xminC(INT_T *xyz_min, INT_T *minim_method, INT_T *maxiter,
             REAL_T *grms_tol, INT_T *natm_ext, INT_T *m_lbfgs,
             INT_T *numdiff, REAL_T *xyz_ext, REAL_T *enrg,
             REAL_T *grad_ext, REAL_T *grms, INT_T *iter,
             REAL_T *total_time, INT_T *print_level, INT_T *ls_method,
             INT_T *ls_maxiter, INT_T *ls_iter, REAL_T *ls_maxatmov,
             REAL_T *beta_armijo, REAL_T *c_armijo, REAL_T *mu_armijo,
             REAL_T *ftol_wolfe, REAL_T *gtol_wolfe, INT_T *return_flag,
             INT_T *label);

/* Options of the LMOD low-mode search (src/sff/sff.h:86-113, the
 * reference's layout and meaning): niter iterations over nmod low modes,
 * kmod of them explored per iteration after the first nrotran_dof; nconf
 * structures kept within energy_window of the lowest and
 * conf_separation_rms apart; modes recomputed every eig_recalc iterations
 * in a Krylov basis of ndim_arnoldi (+ nrotran_dof) vectors (0: all);
 * restart from one of the n_best_struct best every lmod_restart
 * iterations; mc_option 1 Metropolis at rtemp, 2 total, 3 quick quenching;
 * steps between lmod_step_size_min and _max, nof_lmod_steps zig-zag steps
 * (0: up to 20, stopping at a barrier), relaxed to lmod_relax_grms and
 * minimised to minim_grms; nlig ligands moved every apply_rigdock
 * iterations in nof_poses_to_try tries; random_seed (0: from the clock);
 * print_level 0-5.  lmod_time, aux_time and error_flag are outputs. */
typedef struct lmod_opt {
  INT_T niter;
  INT_T nmod;
  INT_T kmod;
  INT_T nrotran_dof;
  INT_T nconf;
  REAL_T minim_grms;
  REAL_T energy_window;
  REAL_T conf_separation_rms;
  INT_T eig_recalc;
  INT_T ndim_arnoldi;
  INT_T lmod_restart;
  INT_T n_best_struct;
  INT_T mc_option;
  REAL_T rtemp;
  REAL_T lmod_step_size_min;
  REAL_T lmod_step_size_max;
  INT_T nof_lmod_steps;
  REAL_T lmod_relax_grms;
  INT_T nlig;
  INT_T apply_rigdock;
  INT_T nof_poses_to_try;
  INT_T random_seed;
  INT_T print_level;
  REAL_T lmod_time;
  REAL_T aux_time;
  INT_T error_flag;
} LMOD_OPT_T;

/* Defaults of the LMOD and its minimiser's options (src/sff/sff.h:135,
 * lmodC.c:3064). */
INT_T lmod_opt_init(struct lmod_opt *lo, struct xmin_opt *xo);

/* LMOD search driving mme() and xmin() (src/sff/sff.h:130-134,
 * lmodC.c:3108): natm atoms from xyz (atoms whose gradient in grad is
 * exactly zero stay fixed); conflib receives up to lo->nconf structures
 * (3 natm each, lowest energy first), lmod_trajectory the niter + 1
 * structures visited; lig_* / tr_* / rot_* describe the ligands (1-based
 * atom numbers, translation in A, rotation in degrees).  Writes
 * conflib.dat in the working directory and reads one left there.  Returns
 * the lowest energy found, its structure in xyz; 0 with lo->error_flag < 0
 * on an error. */
REAL_T lmod(INT_T *natm, REAL_T *xyz, REAL_T *grad, REAL_T *energy,
            REAL_T *conflib, REAL_T *lmod_trajectory, INT_T *lig_start,
            INT_T *lig_end, INT_T *lig_cent, REAL_T *tr_min, REAL_T *tr_max,
            REAL_T *rot_min, REAL_T *rot_max, struct xmin_opt *xo,
            struct lmod_opt *lo);

/* LMOD's reverse-communication form (lmodC.c:1686): call with *label = 0;
 * while it returns *return_flag > 0, act on the request -- 1/2 energy and
 * gradient with a new pair list, 3/4 with the old one, 5 minimise, 6 relax,
 * 7 minimise the start structure, each at xyz_ext -- and call again with
 * the *label it returned; *return_flag = 0 means done (*label < 0: an
 * error). */
REAL_T lmodC(INT_T *nlmodit, INT_T *nmod, INT_T *kmod, INT_T *rotran,
             INT_T *natm_ext, REAL_T *xyz_ext, REAL_T *enrg, REAL_T *grad_ext,
             INT_T *nconf, REAL_T *enrg_win, REAL_T *separ_rms,
             REAL_T *conflib, REAL_T *trajectory, INT_T *arpk_recalc,
             INT_T *arpk_dim, INT_T *lmod_restart, INT_T *topten,
             INT_T *mc_option, REAL_T *rtemp, REAL_T *lmod_step_min,
             REAL_T *lmod_step_max, INT_T *nof_lmod_step, INT_T *nligs,
             INT_T *lig_start, INT_T *lig_end, INT_T *try_now, INT_T *ntry,
             REAL_T *trmin, REAL_T *trmax, INT_T *lig_rot_cent,
             REAL_T *angmin, REAL_T *angmax, INT_T *seed,
             INT_T *print_level, REAL_T *lmod_time, REAL_T *extn_time,
             INT_T *return_flag, INT_T *label);

/* parm7 reader, writer and release (src/sff/sff.h:178-180, prm.c:584,
 * prm.c:1997, prm.c:2810). */
PARMSTRUCT_T *rdparm(STRING_T *name);
INT_T wrparm(PARMSTRUCT_T *prm, STRING_T *name);
INT_T free_prm(PARMSTRUCT_T *prm);

/* Amber ASCII restart read/write (src/sff/sff.h:128,163; sff.c:651,733). */
INT_T getxv(STRING_T *fname, INT_T natom, REAL_T start_time, REAL_T *x,
            REAL_T *v);
INT_T putxv(STRING_T *fname, STRING_T *title, INT_T natom, REAL_T start_time,
            REAL_T *x, REAL_T *v);

/* The serial uniform/Gaussian stream md() draws its Langevin noise from
 * (src/sff/sff.h:162,165; rand2.c:119-140; gauss2 is rand2.c:125). */
REAL_T rand2(void);
REAL_T gauss2(REAL_T *mean, REAL_T *sd);
INT_T setseed(INT_T *seed);

#ifdef __cplusplus
}
#endif

#endif /* SFFG_SFF_H */

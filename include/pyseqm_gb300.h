/*
 * pyseqm_gb300 — C ABI of the GB300 (sm_103a) batched semi-empirical SCF library.
 *
 * Every pointer argument is DEVICE memory unless the name ends in _host.  Every
 * entry point returns 0 on success or a negative SEQM_E* code, launches its work
 * on the given CUDA stream (a cudaStream_t passed as void*; NULL = legacy default
 * stream) and does not synchronise unless it says so.
 *
 * Data layout (ragged, unpadded):
 *   molecules m = 0..nmol-1; atoms of molecule m are atom_off[m] .. atom_off[m+1]-1,
 *   heavy atoms (Z>1) first, then hydrogens (the seqm API's descending-Z order);
 *   the molecule's packed AO basis has norb = 4*nheavy + nhyd functions
 *   (s,px,py,pz per heavy atom, then one s per hydrogen; the order of
 *   seqm/seqm_functions/pack.py:8-17);
 *   every per-molecule square matrix (F, P, Hcore, eigenvectors) is a dense
 *   row-major norb x norb FP64 block starting at mat_off[m] of one flat array;
 *   atom pairs (i<j inside a molecule) are split in three class segments:
 *   heavy-heavy [0,nxx), heavy-H [nxx,nxx+nxh), H-H [nxx+nxh, npairs); the
 *   two-electron integrals of pair p are w_xx[100*p] (10x10, row = atom i's
 *   orbital product, col = atom j's, product order ss,pxs,pxpx,pys,pypx,pypy,
 *   pzs,pzpx,pzpy,pzpz), w_xh[10*(p-nxx)] (column 0 only) and w_hh[p-nxx-nxh].
 */
#ifndef PYSEQM_GB300_H
#define PYSEQM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEQM_OK 0
#define SEQM_E_ARG (-1)       /* bad argument or size */
#define SEQM_E_CUDA (-2)      /* a CUDA launch or API call failed */
#define SEQM_E_UNSUPPORTED (-3) /* element / method not supported (ValueError in the reference) */
#define SEQM_E_TOO_LARGE (-4) /* molecule larger than the density kernel's limit */

/* methods */
#define SEQM_MNDO 0
#define SEQM_AM1 1
#define SEQM_PM3 2
#define SEQM_PM6_SP 3 /* PM6 parameters on the sp basis (method "PM6_SP", seqm/basics.py:132-162) */

/* per-atom parameter slots of seqm_batch.atom_par (structure of arrays, natoms each) */
enum {
  SEQM_P_USS = 0, SEQM_P_UPP, SEQM_P_ZS, SEQM_P_ZP, SEQM_P_BS, SEQM_P_BP, SEQM_P_GSS, SEQM_P_GSP,
  SEQM_P_GPP, SEQM_P_GP2, SEQM_P_HSP, SEQM_P_ALPHA,
  SEQM_P_K1, SEQM_P_K2, SEQM_P_K3, SEQM_P_K4, SEQM_P_L1, SEQM_P_L2, SEQM_P_L3, SEQM_P_L4,
  SEQM_P_M1, SEQM_P_M2, SEQM_P_M3, SEQM_P_M4,
  SEQM_P_RHOCORE, /* PM6_SP: core radius replacing rho0 in the core-core term when nonzero */
  /* derived by seqm_hcore: multipole separations and additive terms, valence charge, n */
  SEQM_P_DD, SEQM_P_QQ, SEQM_P_RHO0, SEQM_P_RHO1, SEQM_P_RHO2, SEQM_P_TORE, SEQM_P_QN,
  SEQM_NPAR
};

#define SEQM_MAX_CLASSES 4

typedef struct seqm_batch {
  int32_t nmol, natoms, nxx, nxh, nhh, method, max_norb, pad_;
  const int32_t *mol_atom_off;  /* [nmol+1] */
  const int32_t *mol_nheavy;    /* [nmol] */
  const int32_t *mol_norb;      /* [nmol] */
  const int32_t *mol_nocc;      /* [nmol] */
  const int64_t *mol_mat_off;   /* [nmol+1] element offsets of the dense per-molecule matrices */
  const int32_t *mol_xx_off;    /* [nmol+1] pair offsets inside the heavy-heavy segment */
  const int32_t *mol_xh_off;    /* [nmol+1] ... heavy-H segment (relative to nxx) */
  const int32_t *mol_hh_off;    /* [nmol+1] ... H-H segment (relative to nxx+nxh) */
  const int32_t *mol_order;     /* [nmol] molecules by descending norb (scheduling order of per-molecule kernels) */
  const int32_t *atom_Z;        /* [natoms] */
  const int32_t *atom_mol;      /* [natoms] */
  const double *atom_xyz;       /* [natoms*3] Angstrom */
  double *atom_par;             /* [SEQM_NPAR*natoms] parameters (SoA), derived slots written by seqm_hcore */
  const int32_t *pair_i;        /* [npairs] global index of the first (heavier or equal) atom */
  const int32_t *pair_j;        /* [npairs] global index of the second atom */
  /* optional size classes of mol_order (host values; nclass 0 = one class of max_norb):
   * molecules mol_order[class_end[c-1] .. class_end[c]) (class_end[-1] = 0, class_end[nclass-1]
   * = nmol) have norb <= class_norb[c].  Per-molecule kernels launch once per class with
   * resources sized for it. */
  int32_t nclass, pad2_;
  int32_t class_end[SEQM_MAX_CLASSES];
  int32_t class_norb[SEQM_MAX_CLASSES];
  /* PM6_SP diatomic core-core parameters (NULL for the other methods), (pair_zmax+1)^2 x 3
   * doubles at [Z1*(pair_zmax+1) + Z2]: alp, chi and cbrt(atomic_num Z1) + cbrt(atomic_num Z2),
   * Z1 the pair's first atom (parameters.py:49-87, energy.py:135-171) */
  const double *pair_par;
  int32_t pair_zmax, pad3_;
  /* [nmol] atoms with 13 <= Z <= 17 per molecule (NULL: none).  The SCF convergence test divides
   * ||dP||_F by 9 nSuperHeavy + 4 nHeavy + 4 nHydro (scf_loop.py:245, :501, :728), and the
   * reference's parser counts these elements as super-heavy for every method (basics.py:258-270),
   * on top of their count as heavy atoms. */
  const int32_t *mol_nsuper;
  /* [npairs] nonzero: the pair lies beyond the parser's pair_outer_cutoff and is left out of
   * every term (integrals, Hcore block, core-core, gradients), as the reference drops it from its
   * pair list (basics.py:324-328); NULL: all pairs kept. */
  const uint8_t *pair_skip;
  /* host value: mol_mat_off[nmol], the number of dense matrix elements of the batch (sum of
   * norb^2), or 0 if the caller does not know it; entry points that size their scratch from it
   * then read it back from the device and wait for that read. */
  int64_t mat_total;
} seqm_batch;

/* Pair list of the batch on the device: pair_i[p], pair_j[p] (global atom indices, the
 * layout's class segments, each row-major i < j inside its molecule) from the batch's atom and
 * segment offsets and heavy-atom counts alone (b->pair_i / pair_j are not read).  Replaces the
 * pair enumeration of Parser.forward (seqm/basics.py:313-342) for the unpadded layout; the
 * caller then points b->pair_i / pair_j at the outputs. */
int seqm_build_pairs(const seqm_batch *b, int32_t *pair_i, int32_t *pair_j, void *stream);

/* Integrals + core Hamiltonian.  Replaces hcore(molecule) (seqm/seqm_functions/hcore.py:9-179),
 * which calls two_elec_two_center_int (two_elec_two_center_int.py:98-283) and
 * diatom_overlap_matrix_PM6_SP (diat_overlap_PM6_SP.py:6-444).  Writes the derived
 * per-atom slots, w_xx/w_xh/w_hh, the full symmetric Hcore (H, dense per molecule) and
 * the core-core repulsion of every pair (enuc_pair, energy.py:91-171: MNDO/AM1/PM3 from w[0,0],
 * PM6_SP from the pair table; an element pair outside the table gives SEQM_E_ARG). */
int seqm_hcore(const seqm_batch *b, double *w_xx, double *w_xh, double *w_hh, double *H, double *enuc_pair,
               void *stream);

/* Fock matrix F = H + G(P) for the molecules with active[m] != 0 (all if active == NULL).
 * Replaces fock(...) (seqm/seqm_functions/fock.py:132-181).  F is full and symmetric. */
int seqm_fock(const seqm_batch *b, const double *P, const double *H, const double *w_xx, const double *w_xh,
              const double *w_hh, double *F, const uint8_t *active, void *stream);

/* Batched symmetric eigensolver (cyclic Jacobi, FP64, one CTA per molecule, norb <= 160) and
 * closed-shell density P = 2 C_occ C_occ^T.  Replaces sym_eig_trunc(F, nHeavy, nHydro, nocc)
 * (seqm/seqm_functions/diag.py:110-241).  evals[mol_row_off[m]..] receives the ascending
 * eigenvalues (mol_row_off = prefix sum of norb), evecs (NULL: skip) the eigenvectors as
 * ROWS of the molecule's norb x norb block (row k <-> evals k), P the density (NULL: skip).
 * work: scratch of mat_off[nmol] doubles (unsorted eigenvector rows).
 * warm (NULL: cold start for all): molecules with warm[m] != 0 start from the orthonormal
 * rows already in `work` (the previous call's eigenvectors) and rotate A = V F V^T, which
 * converges in fewer sweeps when F changed little (successive SCF iterations); needs P.  The
 * call then sets warm[m] = 1 for every molecule it solves (its rows in `work` are valid).
 * mixed_threshold > 0 (needs P): molecules starting cold, or whose previous call (status[m]
 * on entry) took >= mixed_threshold sweeps, first sweep in FP32 (A and the rotation product
 * in shared memory), then lift the vectors to FP64 (one Newton-Schulz re-orthonormalisation)
 * and finish with FP64 sweeps; 0 = FP64 sweeps only.  The result is FP64-accurate either way.
 * density_only != 0 (an SCF iteration: needs P, evecs NULL): once A = V F V^T is nearly
 * diagonal (largest occupied-virtual element over the HOMO-LUMO gap of its diagonal <= 1e-5,
 * directly from a warm start, after one FP32 rotation of a warm start whose ratio is <= 1e-3,
 * or after the FP32 sweeps), P is formed from the first-order
 * occupied-virtual rotation of the smaller set, re-orthonormalised (Loewdin), instead of
 * further FP64 sweeps; error second order in that ratio (<= ~1e-10 in P); evals are then the
 * diagonal of A.  density_only == 2 (evecs NULL: eigenvalues only, as the reference's final
 * eig_only call; P's block is scratch and no density is written): A = V F V^T brought nearly
 * diagonal (FP32 sweeps, re-orthonormalised vectors, FP64 rotation), and the eigenvalues are
 * a_kk + sum_j a_kj^2 / (a_kk - a_jj) when every coupling is below 3e-3 of its diagonal
 * splitting (error third order); otherwise FP64 sweeps.  0 = always sweep to the FP64
 * tolerance (eigenpairs for output).
 * status[m]: sweeps taken (FP32 + FP64), or -1 if the FP64 sweep cap was hit, or -2 for an
 * active molecule with norb > 160, which is left untouched (give it to an SP2 entry point), or
 * -3 if b's size classes put the molecule in a class of smaller class_norb (left untouched).
 * With size classes (b->nclass > 0) the molecules are processed by one launch per class. */
int seqm_density_jacobi(const seqm_batch *b, const double *F, double *P, double *evals, double *evecs,
                        double *work, const int64_t *mol_row_off, const uint8_t *active, int32_t *status,
                        int max_sweeps, uint8_t *warm, int mixed_threshold, int density_only,
                        void *stream);

/* Allocation-free seqm_density_jacobi.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (a host that owns a fixed device-memory pool,
 * or one that must not stall the GPU with cudaMalloc/cudaFree mid-pipeline).  Same inputs
 * and outputs as seqm_density_jacobi, minus `work`: the eigenvector scratch is a fixed
 * 16 MiB device array inside the library (held by every GPU that loads it, until exit).
 * Limit: sum of norb^2 over the batch <= SEQM_NOALLOC_JACOBI_DOUBLES, else SEQM_E_TOO_LARGE
 * and no launch.  A batch whose b->max_norb is above 160 is rejected the same way, as a whole
 * (seqm_density_jacobi instead skips such molecules with status -2 and solves the rest).
 * The size check takes b->mat_total; when that is 0 the call reads mat_off[nmol] back and waits
 * for that read (it synchronises `stream` once, which a stream capture cannot hold).
 * The first call on a device resolves the array's device address (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture.  Later calls with
 * b->mat_total set can be captured.
 * All calls share the array: calls that overlap on the GPU race. */
#define SEQM_NOALLOC_JACOBI_DOUBLES (1 << 21)
int seqm_density_jacobi_noalloc(const seqm_batch *b, const double *F, double *P, double *evals, double *evecs,
                                const int64_t *mol_row_off, const uint8_t *active, int32_t *status, int max_sweeps,
                                void *stream);

/* SP2 purification (FP64), replaces SP2(a, nocc, eps) (seqm/seqm_functions/SP2.py:9-85)
 * applied per molecule to its packed Fock matrix (eps clamped to [1e-7, 1e-3] as there).
 * work: SEQM_SP2_WORK_DOUBLES(T, nmol, max_norb) doubles with T = mat_off[nmol].
 * P = 2 X at convergence.  status[m]: SP2 steps taken, or -1 if max_iter was hit.
 * Called on a stream that is not being captured, it synchronises the stream every 4 SP2 steps
 * to test convergence.  Called while the stream is being captured into a CUDA graph, it adds
 * the step loop to the graph as a conditional WHILE node whose last kernel ends the loop on the
 * device once no molecule runs (at most max_iter trips), with no host synchronisation; give b
 * its mat_total then, since a read-back of mol_mat_off cannot be captured. */
#define SEQM_SP2_STATE 11
#define SEQM_SP2_WORK_DOUBLES(T, nmol, maxn) \
  (2 * (size_t)(T) + (SEQM_SP2_STATE + 2 * (size_t)(maxn)) * (size_t)(nmol) + 2)
int seqm_density_sp2(const seqm_batch *b, const double *F, double *P, double *work, double eps,
                     const uint8_t *active, int32_t *status, int max_iter, void *stream);

/* SP2 with the squarings on the tensor cores (tcgen05, FP16 hi+lo split products, FP32
 * accumulation in tensor memory; operands as pre-split tiles moved by bulk asynchronous
 * copies, the SP2 update fused into the product's epilogue), then one FP32 McWeeny step
 * X <- 3X^2 - 2X^3 of X = P/2 and mcweeny_steps FP64-accurate ones (X <- X + D (I - 2X),
 * D = X^2 - X, with X^2 FP64-accurate from FP32 pairs and the small correction product on the
 * tensor cores, D scaled per molecule into FP16's range): idempotency ~1e-11 after one, FP64
 * level after two.  Molecules with active[m] == 2 (an SCF iteration that may keep the FP32-level
 * density, see seqm_scf_step) take the FP32 McWeeny step only.  Same purification and branch test as
 * SP2.py:9-85 (the trace of X^2 for the test is ||X||_F^2 in FP64); a molecule stops when
 * the trace error is below eps, or below 1e-2 and no longer improving (SP2.py:76-80).  No
 * counterpart of the mixed-precision form in the reference.  work: 256-byte aligned,
 * seqm_sp2_tc_work_bytes(mat_off[nmol], nmol, max_norb) bytes.  At most 65535 molecules.
 * status[m] = SP2 steps, -1 at the step cap, SEQM_E_CUDA if the product kernel gave up
 * waiting on one of its barriers (it then releases its resources and returns; the call's return
 * value says so too when the stream is not being captured).  On a stream that is not being captured it
 * synchronises the stream every 4 SP2 steps; under CUDA graph capture the step loop becomes a
 * conditional WHILE node ended on the device (two SP2 steps per trip, at most max_iter + 1
 * steps), as seqm_density_sp2 describes. */
size_t seqm_sp2_tc_work_bytes(int64_t total_matrix_elements, int nmol, int max_norb);
int seqm_density_sp2_tc(const seqm_batch *b, const double *F, double *P, void *work, double eps,
                        const uint8_t *active, int32_t *status, int max_iter, int mcweeny_steps, void *stream);

/* One mixing step for active molecules.  Replaces the P update of scf_forward0 (linear,
 * scf_loop.py:258-267: P <- alpha P + (1-alpha) Pnew) and scf_forward1 (adaptive,
 * adaptive_mix, scf_loop.py:360-420).  iters[m] counts the molecule's density steps and is
 * incremented here (the adaptive mixer keys on the 1-based count), old2 = diagonal of P
 * from two steps before (at mol_row_off[m]).  Pold receives P before the update.
 * occupation: 2 for a restricted density, 1 for one spin of an unrestricted one (the clamp and
 * the renormalisation of the adaptive mixer, scf_loop.py:371-413). */
int seqm_mix(const seqm_batch *b, double *P, const double *Pnew, double *Pold, double *old2,
             const int64_t *mol_row_off, int32_t *iters, int linear, double alpha, double occupation,
             const uint8_t *active, void *stream);

/* Electronic energy 1/2 sum P(H+F) per molecule (energy.py:26-49) for active molecules, and
 * the SCF convergence test of get_error (scf_loop.py:106-147): updates err, dm_err, dm_el,
 * Eelec (the previous energy), clears active[m] for molecules that converged, and writes
 * Eout[m] = the new energy.  When Pold == NULL only the energy is computed.  diis_err (NULL
 * unless the DIIS converger runs): max |F P - P F| per molecule; the test then also fails
 * while it exceeds 50 eps (scf_loop.py:130-132). */
int seqm_energy_error(const seqm_batch *b, const double *P, const double *Pold, const double *H,
                      const double *F, double *Eelec, double *Eout, double *err, double *dm_err,
                      double *dm_el, uint8_t *active, double eps, const double *diis_err, void *stream);

/* The rest of one SCF iteration after the density step, for the active molecules: mixing,
 * Fock build of the mixed density, energy and convergence test, retirement of the molecules
 * that pass it, and a count of those still active.  Replaces the body of the reference's
 * iteration loop after its density step (scf_forward0 scf_loop.py:258-300, scf_forward1
 * :505-598): P <- mix(P, Pnew) (seqm_mix), F <- F(P) (seqm_fock), Eelec and the test of
 * get_error (seqm_energy_error), where the reference ends each iteration with a host read of
 * the not-converged count (scf_loop.py:598, Nnot = int(notconverged.sum())); here the count goes
 * to *nactive on the device (NULL: not counted) and no call synchronises the stream, so
 * iterations can be queued ahead or captured in a CUDA graph.
 * mixing: 0 linear (alpha), 1 adaptive, -1 none (P already mixed, e.g. by seqm_diis_mix; pass
 * diis_err then).  Every pointer is device memory; the struct itself is read on the host.
 * active[m]: 0 retired, 1 active, 2 active with a density from seqm_density_sp2_tc that skipped
 * the FP64-accurate McWeeny step.  A molecule at 2 is never retired on that density: the test
 * keeps it active and moves it to 1 (refined densities from then on) once |dE| < 1 eV or after
 * 8 iterations (iters).  A caller that starts molecules at 2 saves that step's cost, about three
 * times the rest of an iteration at thousands of basis functions, on the early iterations. */
typedef struct seqm_scf_state {
  double *P;                /* [T] in: density; out: the mixed density */
  const double *Pnew;       /* [T] the density step's output */
  double *Pold;             /* [T] out: P before the mixing (unfused step; the fused one leaves it) */
  double *old2;             /* [sum norb] adaptive mixer's diagonal history (seqm_mix) */
  const double *H;          /* [T] core Hamiltonian */
  double *F;                /* [T] out: F(P) */
  const double *w_xx, *w_xh, *w_hh;               /* integrals of seqm_hcore */
  double *Eelec, *Eout, *err, *dm_err, *dm_el;    /* [nmol] as seqm_energy_error */
  const int64_t *mol_row_off;                     /* [nmol+1] prefix sum of norb */
  int32_t *iters;           /* [nmol] density steps per molecule (seqm_mix) */
  uint8_t *active;          /* [nmol] in/out: 0, 1 or 2 (above) */
  const double *diis_err;   /* [nmol] or NULL */
  int32_t *nactive;         /* [1] out, or NULL */
  int32_t mixing, pad_;
  double alpha, occupation, eps;
  double *scratch;          /* SEQM_SCF_SCRATCH_DOUBLES, or NULL (below) */
} seqm_scf_state;
/* With scratch != NULL and mixing >= 0 the step is fused: the mixer takes ||dP|| itself and leaves
 * Pold untouched, the Fock build adds up P (H + F) per atom and per pair as it writes F, and one
 * small kernel forms each molecule's energy from those sums in a fixed order and runs the test.
 * No separate energy pass reads P, Pold, H and F again; the results equal the unfused step's to
 * rounding.  Needs max_norb <= 12800.  Its size in doubles: */
#define SEQM_SCF_SCRATCH_DOUBLES(nmol, natoms, npairs, sum_norb) \
  (5 * (size_t)(nmol) + (size_t)(natoms) + (size_t)(npairs) + 4 * (size_t)(sum_norb))
int seqm_scf_step(const seqm_batch *b, const seqm_scf_state *st, void *stream);

/* Pulay DIIS converger (scf_converger [2]; scf_forward2, scf_loop.py:639-1132), per molecule.
 * state: SEQM_DIIS_STATE doubles per molecule (ring counter, stored count, reset flag, the
 * 11 x 11 EMAT); hist: SEQM_DIIS_HIST_DOUBLES(T) doubles (10 Fock matrices, 10 commutators
 * F P - P F, one F P product) with T = mat_off[nmol].  seqm_diis_init before the loop;
 * per iteration: seqm_diis_extrapolate (stores F and its commutator, counts the iteration in
 * iters, replaces F by the DIIS extrapolation once 2 are stored), the density step on that
 * F, seqm_diis_mix (P <- (P + Pnew)/2 while fewer than 2 are stored, else Pnew), the Fock
 * build and seqm_energy_error with diis_err.  The history resets (per molecule; the reference
 * resets the whole batch) when the DIIS matrix's condition number exceeds 1e7.
 * seqm_diis_extrapolate reads mat_off[nmol] back (one stream synchronisation). */
#define SEQM_DIIS_STATE 124
#define SEQM_DIIS_HIST_DOUBLES(T) (21 * (size_t)(T))
int seqm_diis_init(const seqm_batch *b, double *state, double *diis_err, void *stream);
int seqm_diis_extrapolate(const seqm_batch *b, double *F, const double *P, double *hist, double *state,
                          double *diis_err, const uint8_t *active, int32_t *iters, void *stream);
int seqm_diis_mix(const seqm_batch *b, double *P, const double *Pnew, double *Pold, const double *state,
                  const uint8_t *active, void *stream);

/* Diagonal initial density (scf_loop.py:2066-2081): tore/4 on heavy-atom s,p; 1 on H s. */
int seqm_initial_density(const seqm_batch *b, double *P, void *stream);

/* Per-molecule sums of per-pair core-core energies: Enuc[m] (energy.py:177-192). */
int seqm_pair_sum(const seqm_batch *b, const double *pair_val, double *mol_sum, void *stream);

/* Gradient of sum_m gE[m]*Eelec[m] + gN[m]*Enuc[m] at fixed densities P, i.e. what the
 * reference's autograd gives with the SCF as a constant (SCF0, scf_loop.py:1996-2031;
 * Force.forward, basics.py:1260-1365): dR[natoms*3] = dE/dR (eV/Angstrom; force = -dR) and
 * dpar[4*natoms] = dE/d(U_ss, U_pp, beta_s, beta_p) per atom (NULL: skip).  Integrals,
 * overlaps and core-core terms are recomputed with forward-mode derivatives, not stored.
 * work: scratch of 7*npairs doubles.  Pbeta (NULL: restricted, P the total density): P and
 * Pbeta are the alpha and beta densities of an unrestricted solve. */
int seqm_energy_grad(const seqm_batch *b, const double *P, const double *Pbeta, const double *gE, const double *gN,
                     double *dR, double *dpar, double *work, void *stream);

/* Gradient of a CIS / RPA excited-state energy (ground state included).  Replaces
 * rcis_grad_batch(..., include_ground_state=True) (seqm/seqm_functions/rcis_grad_batch.py:10-259):
 * the ground-state terms of seqm_energy_grad for the closed-shell density P, plus the relaxed
 * difference density D (symmetric: the unrelaxed difference density and the Z-vector
 * response, make_cis_densities rcis_batch.py:971-1059) in the Coulomb, core-attraction,
 * exchange and resonance terms, and the transition density R (C_occ X C_virt^T, + C_virt Y^T
 * C_occ^T for RPA) in its Coulomb (symmetric part) and exchange (symmetric and antisymmetric
 * parts) terms.  All three are ragged dense per-molecule matrices; gE, gN, dR, work as
 * seqm_energy_grad (no parameter gradients). */
int seqm_energy_grad_excited(const seqm_batch *b, const double *P, const double *D, const double *R,
                             const double *gE, const double *gN, double *dR, double *work, void *stream);

/* Unrestricted Fock matrices (fock_u_batch, seqm/seqm_functions/fock_u_batch.py:18-100):
 * Fa, Fb of the spin densities Pa, Pb (Coulomb of Pa + Pb, exchange of the spin density,
 * spin-resolved one-centre terms), for active molecules. */
int seqm_fock_u(const seqm_batch *b, const double *Pa, const double *Pb, const double *H, const double *w_xx,
                const double *w_xh, const double *w_hh, double *Fa, double *Fb, const uint8_t *active,
                void *stream);

/* Unrestricted energy 1/2 sum [(Pa + Pb) H + Pa Fa + Pb Fb] (energy.py:44-45) and, with
 * Pa_old/Pb_old, the get_error test (scf_loop.py:106-147) on the spin-summed density change;
 * same outputs as seqm_energy_error. */
int seqm_energy_error_u(const seqm_batch *b, const double *Pa, const double *Pb, const double *Pa_old,
                        const double *Pb_old, const double *H, const double *Fa, const double *Fb, double *Eelec,
                        double *Eout, double *err, double *dm_err, double *dm_el, uint8_t *active, double eps,
                        void *stream);

/* Two-electron part G(P) of the Fock build for nvec sets of general (not symmetric) AO
 * densities: the matrix-vector product of the CIS / RPA solvers.  Replaces makeA_pi_batched
 * and makeA_pi_symm_batch (seqm/seqm_functions/rcis_batch.py:296-507): Coulomb from the
 * symmetric part of the partners' diagonal blocks, one-centre terms of the symmetric and the
 * antisymmetric part, exchange of each off-diagonal block from its own block of P (no Hcore).
 * Set v lives at P + v * stride (each set a full ragged batch, stride >= mol_mat_off[nmol]);
 * G has the same layout; nvec <= 65535.  Molecules with active[m] == 0 are skipped. */
int seqm_fock_general(const seqm_batch *b, int nvec, const double *P, const double *w_xx, const double *w_xh,
                      const double *w_hh, double *G, int64_t stride, const uint8_t *active, void *stream);

/* Library build string (host memory; no GPU needed). */
const char *seqm_version(void);

#ifdef __cplusplus
}
#endif

#endif

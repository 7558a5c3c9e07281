/*
 * pnfam_gpu.h -- C ABI of the GB300 pnFAM solver library (libpnfam_gb300.so).
 *
 * The reference runs the finite-amplitude-method (FAM) iteration of one
 * (operator, K, omega) point per pnfam_main.x process on the CPU
 * (pnfam_solver.f90:32-221).  This library keeps the ground state and the
 * operator resident on one GPU and solves a batch of omega points at once.
 *
 * Conventions
 *  - All arrays are caller-owned host memory, copied in/out; float64.
 *  - Block matrices: "one non-zero block per block row" layout of the
 *    reference blockmatrix type (pnfam_type_blockmatrix.f90:22-26): blocks in
 *    increasing block-row order, each block column-major (Fortran order).
 *  - The basis is the doubled (explicit time-reversed) basis of
 *    hfbtho_solution.f90:164-353, spin-up states first inside every block.
 *  - Return value 0 = success; otherwise one of PNFAM_E* below, with a
 *    message available from pnfam_gpu_last_error().  Contexts are not
 *    thread-safe: one context per host thread.
 */
#ifndef PNFAM_GPU_H
#define PNFAM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PNFAM_OK = 0,
  PNFAM_EINVAL = 1,      /* bad shape / argument */
  PNFAM_ENOMEM = 2,      /* device allocation failed */
  PNFAM_ECUDA = 3,       /* CUDA runtime error, or no usable GPU */
  PNFAM_ENONFINITE = 4,  /* non-finite value produced by the iteration */
  PNFAM_ESTATE = 5       /* call out of order (e.g. solve before set_operator) */
};

typedef struct pnfam_ctx pnfam_ctx_t;

/* Basis description (doubled basis). */
typedef struct {
  int nb;                 /* number of blocks (even; block i+nb/2 is the TR partner of i) */
  const int* db;          /* [nb] block sizes */
  const int* num_spin_up; /* [nb] spin-up states at the start of each block */
  const int* ns;          /* [dqp] 2*spin projection, +1 / -1 */
  int nghl;               /* mesh points */
} pnfam_basis_t;

/* Residual-interaction couplings (pnfam_interaction.f90:246-258). */
typedef struct {
  const double* crho;     /* [nghl] C^rho(r)  */
  const double* cs;       /* [nghl] C^s(r)    */
  const double* cpair;    /* [nghl] C^pair(r) */
  const double* cspair;   /* [nghl] C^spair(r)*/
  double scalars[12];     /* cdrho, ctau, ctj0, ctj1, ctj2, crdj, cds, ct, cj, cgs, cf, csdj */
} pnfam_coupl_t;

/* Solver options (namelist &solver, pnfam_setup.f90:102-103; mixing factor
 * of pnfam_broyden.f90:20). */
typedef struct {
  int max_iter;               /* iterations before giving up (iter_conv = -1) */
  int broyden_history_size;   /* M; 0 = linear mixing; <0 = no mixing */
  double convergence_epsilon;
  double alpha_mix;           /* 0.7 in the reference */
  double quench_residual_int; /* scales the residual interaction; 0 skips it */
  int precision;              /* 0 = FP64 everywhere (the drop-in form);
                                 1 = mixed form (defect correction): the residual interaction
                                 (block GEMMs, densities, fields) is evaluated in FP32 on the
                                 increment X - X_a from an anchor X_a whose image g(X_a) is
                                 held in FP64.  While max|X - X_a| <= 1000*epsilon the FP32
                                 error is far below epsilon and convergence (si < epsilon) is
                                 accepted on an increment evaluation; farther out a point
                                 takes an FP64 anchor evaluation when si < 10^-reserved[1]
                                 (default 100*epsilon) or si stops falling at the FP32 noise
                                 floor (si <= 1e-3 max|X - X_a|), and convergence
                                 is accepted only on that anchor.  Every evaluation counts
                                 against max_iter.  Broyden, Green's function and strength
                                 are FP64 in both modes. */
  int reserved[7];            /* [0]: per-stage event timing on/off; [1]: see precision;
                                 [2]: live timing of the FP32 density and field-projection
                                 launches (an event pair around each launch on its own
                                 stream, read after the engine's wait; no serialisation);
                                 [3] = n > 0: convergence also asks every strength value
                                 (Re and Im of the strength and each cross term) to have
                                 settled, |S - S_previous| <= 10^-n |S| + 1e-13 max|S|, for
                                 at most 20 iterations beyond si < epsilon (0: the
                                 reference's test si < epsilon alone);
                                 [4] = n > 0: the mixed form's "near its anchor" bound is
                                 10^n epsilon instead of 1000 epsilon;
                                 [5] != 0: mixed form, asynchronous anchors: an FP64 anchor
                                 evaluation that meets FP32 increments in one launch runs on
                                 the context's second stream and its points wait (parked)
                                 while the engine keeps stepping the others (same arithmetic
                                 per point; 0: the anchor and the increments of a launch end
                                 together) */
} pnfam_solver_opts_t;

/*
 * Create a context on the current CUDA device and upload the ground state.
 * Replaces the reference's per-process set-up of the HFB solution
 * (pnfam_setup.f90:285-382 setup_hfb_solution) and of the residual
 * interaction (pnfam_setup.f90:389-400 setup_hamiltonian).
 *   Ep, En        [dqp] quasiparticle energies (zero above the pairing window)
 *   Up, Un        block diagonal, block i: db[i] x db[i]
 *   Vp, Vn        block i: db[i] x db[partner(i)] (rows of block i)
 *   phi           [5][dqp][nghl]: wf, d/dr wf, y*nl*wf, d/dz wf, Laplacian
 *                 (hfbtho_solution.f90:114-121 wf, wfdr, wfdp, wfdz, wfd2_all)
 *   wdcori        [nghl] inverse quadrature weights
 */
int pnfam_gpu_init(const pnfam_basis_t* basis,
                   const double* Ep, const double* En,
                   const double* Up, const double* Vp,
                   const double* Un, const double* Vn,
                   const double* phi, const double* wdcori,
                   const pnfam_coupl_t* coupl,
                   pnfam_ctx_t** out);

/*
 * Set the external field (operator O_K) and its cross terms.
 * Replaces the operator half of init_pnfam_solver (pnfam_solver.f90:226-381:
 * Fqp = W^T Fsp W and the block structures that follow from F).
 *   beta_minus    1 for beta-, 0 for beta+
 *   fcols         [nb] block column of F for each block row, -1 if empty
 *                 (init_fam_mapping, pnfam_extfield.f90:763-841)
 *   Fsp           F_sp elements in the fcols structure
 *   n_xterms, Gsp cross-term operators with the same structure (may be 0/NULL)
 */
int pnfam_gpu_set_operator(pnfam_ctx_t* ctx, int beta_minus, const int* fcols,
                           const double* Fsp, int n_xterms, const double* const* Gsp);

/*
 * Statistical FAM: quasiparticle occupations of a finite-temperature or an
 * EFA-blocked ground state (setup_hfb_solution, pnfam_setup.f90:324-381; the
 * use_diagonal_blocks branch of init_pnfam_solver, pnfam_solver.f90:248-254,
 * 425-458).  With occupations the QP state carries the quadrants P and Q besides
 * X and Y, the Green's function of P/Q is -1/(E1 - E2 -/+ w) and the response is
 * weighted by 1 - f1 - f2 (X, Y) and f2 - f1 (P, Q); the Broyden vector doubles.
 *   fp, fn   [dqp] proton / neutron occupations in [0, 1] (the doubled basis),
 *            both NULL to return to the zero-temperature form
 * Call before pnfam_gpu_set_operator (it clears the operator).  Solved in either
 * form (precision 0 or 1).
 */
int pnfam_gpu_set_occupations(pnfam_ctx_t* ctx, const double* fp, const double* fn);

/*
 * Solve npts omega points (ifam, pnfam_solver.f90:93-221) as one batch.
 *   re_w, im_w    [npts] complex energies
 *   re_S, im_S    [npts*(1+n_xterms)] strength and cross terms (-1/pi contraction)
 *   iters         [npts] iteration at convergence, -1 if max_iter was reached
 *   si_out        [npts] final Broyden residual si
 *   hist          optional, NULL or [npts*(max_iter+1)*3]: per iteration
 *                 (si, Re S, Im S) as printed in the reference's iteration table
 */
int pnfam_gpu_solve(pnfam_ctx_t* ctx, int npts, const double* re_w, const double* im_w,
                    const pnfam_solver_opts_t* opts,
                    double* re_S, double* im_S, int* iters, double* si_out, double* hist);

/*
 * pnfam_gpu_solve with the restart storage of pnfam_solve (pnfam_solver.f90:63-81,
 * pnfam_storage.f90:62-137): x0 (or NULL) holds a start vector per point, the
 * Broyden vector of the reference (qrpa_broin: Re X | Re Y | Im X | Im Y, and
 * Re P | Re Q | Im P | Im Q after them in the statistical FAM, each quadrant in
 * block-matrix order), npts x pnfam_gpu_state_size(ctx) doubles; the first
 * iteration then evaluates the field of that state (an FP64 anchor in the mixed
 * form) and the Broyden history starts empty, as in the reference.  x_out (or
 * NULL) receives the final vectors in the same layout (what the reference writes
 * to <fam_output_filename>.bin).
 */
int pnfam_gpu_solve_state(pnfam_ctx_t* ctx, int npts, const double* re_w, const double* im_w,
                          const pnfam_solver_opts_t* opts, const double* x0,
                          double* re_S, double* im_S, int* iters, double* si_out, double* hist,
                          double* x_out);

/* Length of one point's state vector: 4 nxy, or 8 nxy in the statistical FAM. */
long long pnfam_gpu_state_size(const pnfam_ctx_t* ctx);

/*
 * Continuous batching.  No counterpart in the reference, which runs one point
 * per process (pynfam's task farm): an engine keeps `slots` omega points of
 * one (nucleus, operator) context on the device, each slot iterating on its
 * own counter exactly as pnfam_gpu_solve iterates a point, and a slot whose
 * point has converged (or reached max_iter) takes the next point while the
 * others keep iterating.  Engines of different contexts run on their own
 * streams and overlap on the GPU.  One engine per context at a time; the
 * context's solve buffers belong to the engine until pnfam_gpu_engine_free.
 *
 *   create   slots and solver options (as for pnfam_gpu_solve)
 *   admit    up to n points into free slots; returns the number admitted
 *            (>= 0), or minus an error code; tags identify the points in the
 *            results
 *   launch   enqueue one iteration of every active slot (returns at once)
 *   finish   wait for it, advance the slots, and copy out up to maxout
 *            finished points: tag, strength [nops] per point, iters (-1: not
 *            converged), si; *nout = number copied (the rest stay queued)
 *   active   number of slots holding a point that is still iterating
 */
typedef struct pnfam_engine pnfam_engine_t;
int pnfam_gpu_engine_create(pnfam_ctx_t* ctx, int slots, const pnfam_solver_opts_t* opts,
                            pnfam_engine_t** engine);
int pnfam_gpu_engine_admit(pnfam_engine_t* engine, int n, const double* re_w, const double* im_w,
                           const long long* tags);
int pnfam_gpu_engine_launch(pnfam_engine_t* engine);
int pnfam_gpu_engine_finish(pnfam_engine_t* engine, int maxout, long long* tags, double* re_S,
                            double* im_S, int* iters, double* si, int* nout);
int pnfam_gpu_engine_active(const pnfam_engine_t* engine);
/* 1 when pnfam_gpu_engine_finish would not wait (no evaluation in flight, or the
 * one in flight has completed), 0 while it runs, minus an error code */
int pnfam_gpu_engine_ready(const pnfam_engine_t* engine);
void pnfam_gpu_engine_free(pnfam_engine_t* engine);

/*
 * The reference's in-process plugin seam: calc_hamiltonian
 * (pnfam_setup.f90:74-89 calc_dHsp_interface; pnfam_hamiltonian_blas.f90:51-74).
 * Given the perturbed single-particle densities (rho_pn in the F structure,
 * kappa(+) in the transpose of the X structure, rho_np in the F structure,
 * kappa(-) in the transpose of the Y structure; each as Re and Im arrays of
 * nxy elements) return the perturbed fields h_pn (F), Delta(+) (X),
 * h_np (F), Delta(-) (Y).  Requires pnfam_gpu_set_operator.
 */
int pnfam_gpu_calc_hamiltonian(pnfam_ctx_t* ctx,
                               const double* re_rho_pn, const double* im_rho_pn,
                               const double* re_kp, const double* im_kp,
                               const double* re_rho_np, const double* im_rho_np,
                               const double* re_km, const double* im_km,
                               double* re_h_pn, double* im_h_pn,
                               double* re_dp, double* im_dp,
                               double* re_h_np, double* im_h_np,
                               double* re_dm, double* im_dm);

/*
 * The same field evaluation in the arithmetic of the mixed form's increment
 * evaluations: densities and fields in FP32, the field projection on the
 * tensor cores as 3xTF32 products (about FP32 accuracy).  No counterpart in
 * the reference.  Inputs and outputs as for pnfam_gpu_calc_hamiltonian.
 */
int pnfam_gpu_calc_hamiltonian_mixed(pnfam_ctx_t* ctx,
                                     const double* re_rho_pn, const double* im_rho_pn,
                                     const double* re_kp, const double* im_kp,
                                     const double* re_rho_np, const double* im_rho_np,
                                     const double* re_km, const double* im_km,
                                     double* re_h_pn, double* im_h_pn,
                                     double* re_dp, double* im_dp,
                                     double* re_h_np, double* im_h_np,
                                     double* re_dm, double* im_dm);

/*
 * Allocation-free field evaluation.  No counterpart in the reference: the
 * reference evaluates the field only inside its own process.
 *
 * For callers that cannot allocate device memory themselves through CUDA (a
 * host program that owns every device buffer through its own memory pool or
 * through mapped host memory, or code running where device allocation is not
 * allowed): the same computation as pnfam_gpu_calc_hamiltonian, with every
 * input and output given as a DEVICE pointer by the caller and all
 * intermediates kept in one fixed device array inside the library (about
 * 12.5 MB, held on every GPU that loads the library until the process exits).
 * This entry point calls no cudaMalloc/cudaFree and no allocating library
 * routine.
 *
 *   basis         host struct with host arrays (as for pnfam_gpu_init)
 *   d_phi         device [5][dqp][nghl] basis functions
 *   d_wdcori      device [nghl]
 *   d_coupl       couplings: the four arrays are DEVICE pointers [nghl]
 *   fcols         host [nb] block map of the operator (as for set_operator)
 *   d_in[8]       device: Re/Im rho_pn, Re/Im kappa(+), Re/Im rho_np, Re/Im kappa(-)
 *   d_out[8]      device: Re/Im h_pn, Re/Im Delta(+), Re/Im h_np, Re/Im Delta(-)
 *                 (structures as for pnfam_gpu_calc_hamiltonian)
 *   stream        cudaStream_t to run on (NULL: the default stream); the call
 *                 returns after the stream has finished the work
 * Limits: nxy <= 32768, nghl <= 1600, dqp <= 1024, nb <= 64 (every operator
 * up to N_sh = 12 on a 40 x 40 mesh); larger sizes return PNFAM_EINVAL.
 * The first call on a device looks up the array's device address and sets a
 * kernel attribute.  No call can be captured into a CUDA graph: each copies
 * host tables to the device and synchronises the stream before returning.  All
 * calls share the array: calls that overlap on the GPU (from several threads
 * or streams) race and must be serialised by the caller.
 */
int pnfam_gpu_calc_hamiltonian_noalloc(const pnfam_basis_t* basis, const double* d_phi,
                                       const double* d_wdcori, const pnfam_coupl_t* d_coupl,
                                       const int* fcols, const double* const* d_in,
                                       double* const* d_out, void* stream);

/*
 * Host-only introspection, no device needed: the block-GEMM task tables that
 * pnfam_gpu_set_operator builds for the QP <-> SP transforms of a basis and an
 * operator structure (the triprod_bbm products of pnfam_solver.f90:144-166), for
 * verification against a CPU restatement.
 *   stage       0/1: dR_sp = W1 dR_qp W2^T (T = op(B) op(C), then out = sum a op(A) T);
 *               2/3: dH_qp = W1^T dH_sp W2 (same two steps)
 *   out         [cap][PNFAM_TASK_RECORD] per task: M, N, K, nterm, cbuf, coff, ldc,
 *               then per term (PNFAM_TASK_TERMS): abuf, aoff, lda, tA, bbuf, boff,
 *               ldb, tB, alpha_re, alpha_im  (buffer ids: 0 UP, 1 VP, 2 UN, 3 VN,
 *               4 QP state, 5 scratch, 6 dR_sp, 7 dH_sp, 8 dH_qp; offsets within a
 *               Re or Im plane; the state and dH_qp hold X, Y[, P, Q] nxy apart, the
 *               SP buffers rho_pn, kappa+, kappa-, rho_np)
 *   ntask       number of tasks (all of them, even beyond cap)
 *   nxy, scratch elements per QP quadrant and per scratch plane
 */
#define PNFAM_TASK_TERMS 4
#define PNFAM_TASK_RECORD (7 + 10 * PNFAM_TASK_TERMS)
int pnfam_gpu_task_tables(int nb, const int* db, const int* num_spin_up, int beta_minus,
                          const int* fcols, int statistical, int stage, double* out, int cap,
                          int* ntask, long long* nxy, long long* scratch);

/* Number of non-trivial FAM matrix elements nxy (valid after set_operator). */
long long pnfam_gpu_nxy(const pnfam_ctx_t* ctx);

/* Timing of the last solve: per stage accumulated device ms (order:
 * k1_blockgemm, density, meanfield, field_projection, k2_blockgemm, green,
 * broyden, strength; filled only when opts.reserved[0] != 0), then, if
 * nstage > 8, the whole solve's device time (CUDA events on the solver's
 * stream), if nstage > 10 the FP64 and FP32 point-iterations of the solve,
 * then (entries 11-15) the first five stages of the FP32 evaluations of the
 * mixed form (entries 0-4 then hold the FP64 evaluations only), then (entries
 * 16-19, with opts.reserved[2] != 0) the number and total device ms of the FP32
 * density launches and of the FP32 field-projection launches, then (entries
 * 20-22) the autotuner's choices for the context's operator: the point count from
 * which FP32 evaluations take the pair-tensor GEMMs (2^30: never), the K chunks per
 * density task of those GEMMs, and the autotuner's host time in ms (0: not run; it
 * runs once per operator when the first mixed-form engine or solve sets up its FP32
 * buffers, unless PNFAM_GB300_AUTOTUNE=0), and the number of kernel launches.  An
 * engine's figures accumulate from its creation. */
int pnfam_gpu_last_profile(const pnfam_ctx_t* ctx, double* stage_ms, int nstage,
                           long long* launches);

void pnfam_gpu_free(pnfam_ctx_t* ctx);

/*
 * Finite-range two-body-current field: the contraction of the Yukawa part of
 * the axial two-body current with the ground-state density matrices, computed on
 * the GPU.  Replaces effective_2bc_extfield (pnfam_extfield_2bc.f90:26-915, the
 * production branch :128-465 and the final basis reorder :901-913), which the
 * reference calls from setup_extfield (pnfam_solver.f90:620-633) when no .tbc
 * file exists; its output is what write_tbc stores (pnfam_storage.f90:488-560).
 *
 *   ntx, nbx        basis states and blocks of HFBTHO (Omega > 0 half)
 *   block_size      [nbx] states per block
 *   nz, nr, nl, ns  [ntx] oscillator quantum numbers in HFBTHO's order
 *   bz, bp          oscillator lengths (fm)
 *   rk_n, rk_p      HFBTHO's density matrices rk (twice rho) per block,
 *                   column-major [size x size], blocks concatenated
 *   K               projection of the operator's angular momentum (-1, 0, 1)
 *   beta_minus      1 for beta-, 0 for beta+
 *   use_p           1: add the pion-pole (momentum-dependent) pieces
 *   op_cols         [2 nbx] block column (0-based, -1 empty) of each block row of
 *                   the operator on the time-reversal-doubled basis
 *   op_offsets      [2 nbx] start of each block row's block in the flat storage
 *   nxy             elements of the operator's flat storage
 * Output: pieces [6][nxy] (host) = c3 direct, c3 exchange, c4 direct, c4
 * exchange, pion-pole direct, pion-pole exchange, in the operator's flat layout
 * on the spin-sorted basis, with the LECs stripped (c3 = 1, c4 + 1/4 = 1): the
 * field for given LECs is c3 (c3d + c3e) + (c4 + 1/4) (c4d + c4e) + cpd + cpe.
 * stats (may be NULL) [6]: host set-up ms, stage-1 ms, stage-2 ms (CUDA events),
 * radial terms, radial groups, (z_b, z_d) pairs.
 */
typedef struct {
  int ntx, nbx;
  const int* block_size;
  const int *nz, *nr, *nl, *ns;
  double bz, bp;
  const double* rk_n;
  const double* rk_p;
  int K, beta_minus, use_p;
  const int* op_cols;
  const long long* op_offsets;
  long long nxy;
} pnfam_2bc_input_t;

int pnfam_gpu_2bc_field(const pnfam_2bc_input_t* in, double* pieces, double* stats);

/*
 * HFB reconstruction on the GPU (the arithmetic of rebuilding an HFBTHO ground
 * state from its .hel fields; the particle-number loop stays with the caller).
 * Host arrays in and out; mesh index ih + il*ngh; states in HFBTHO order.
 *
 * pnfam_gpu_hfb_basis: oscillator basis functions on the mesh with the square
 *   roots of the quadrature weights (gaupol, hfbtho_solver.f90:3463-3671):
 *   out [4][nt][ngh*ngl] = function, d/dr, d/dz, (r, z) Laplacian part.
 * pnfam_gpu_hfb_matrices: the HFB matrices h and Delta of every block and isospin
 *   from the fields (gamdel, hfbtho_solver.f90:5190-5302).  fields [2][11][nghl]:
 *   per isospin (n, p) v, vhb, vr, vz, vd, vs, vSFIZ, vSZFI, vSFIR, vSRFI, dv;
 *   y [nghl] = 1/r; xlam, xlap [nb] = Omega -/+ 1/2 of the block; out: per block,
 *   per isospin, h then Delta, nd x nd row-major.
 * pnfam_gpu_sym_eigen: eigenvalues (ascending) and eigenvectors (columns) of a
 *   batch of real symmetric matrices (sizes 1..512, concatenated row-major), by
 *   cyclic Jacobi on the GPU (one CTA per matrix); replaces hfbdiag's DSYEVR.
 *   v0 (may be NULL): starting orthogonal matrices, same layout (the eigenvectors
 *   of nearby matrices, e.g. the previous step of the particle-number loop): the
 *   rotations then start from v0^T a v0.  sweeps (may be NULL) [nmat]: Jacobi
 *   sweeps used.
 * pnfam_gpu_hfb_densities: sums of DENSIT (hfbtho_solver.f90:4318-4734) over the
 *   quasiparticles of each block: W [per block nd x nd row-major] the V matrix with
 *   the columns of quasiparticles outside the pairing window zero; at finite
 *   temperature also U (same layout) and f [nt] (thermal occupation per column);
 *   out [3][nghl] = rho, tau, Laplacian-rho sums before normalisation.
 */
int pnfam_gpu_hfb_basis(int ngh, int ngl, const double* xh, const double* wh, const double* xl,
                        const double* wl, double bz, double bp, int nt, const int* nr, const int* nz,
                        const int* nl, double* out);
int pnfam_gpu_hfb_matrices(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                           const double* y, const double* xlam, const double* xlap, const double* fields,
                           double* out);
int pnfam_gpu_sym_eigen(int nmat, const int* dims, const double* a, const double* v0, double* w, double* v,
                        int* sweeps);
int pnfam_gpu_hfb_densities(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                            const double* y, const double* xlam, const double* xlap, const double* W,
                            const double* U, const double* f, double* out);

/* Message of the last failing call on this thread ("" if none). */
const char* pnfam_gpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PNFAM_GPU_H */

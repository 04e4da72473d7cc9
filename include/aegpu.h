/*
 * aegpu.h -- thin C ABI of the GB300 statevector engine.
 *
 * The drop-in layer (stateAnsatzManager and the AnsatzSynthInterface functions,
 * include/AnsatzSynthInterface.h) calls CUDA only through these entry points.
 * Plain pointers and sizes only; all arrays are host memory unless a name ends in
 * _dev, in which case they are device pointers and `stream` is a cudaStream_t.
 * Every call returns AEGPU_OK (0) or a positive status and never traps; the text
 * of the last failure is available from aegpu_last_error().
 *
 * Conventions (the reference's internal ones: operatorpool.cpp:198-199, 221-230):
 *  - spin orbital k < N is beta (low bits), k >= N is alpha (high bits);
 *  - excitations are 4 signed 0-based orbital indices, -1 = absent, op-major;
 *  - the sector basis is the ascending list of bitstrings in the sector; vectors
 *    are "compressed" (one entry per sector determinant; complex mode interleaves
 *    re, im);
 *  - angles are per operator, in the order the operators were given;
 *  - H is applied as y = H x with rows = output determinants.
 * An engine is not thread-safe: one thread at a time per engine (the reference-
 * compatible layer serialises its calls per context with a mutex); different
 * engines may be used from different threads.
 */
#ifndef AEGPU_H
#define AEGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AEGPU_OK 0
#define AEGPU_ERR_ARG 1          /* invalid argument (null pointer, size, index) */
#define AEGPU_ERR_STATE 2        /* call out of order (no problem / Hamiltonian set) */
#define AEGPU_ERR_CUDA 3         /* CUDA runtime failure (message in aegpu_last_error) */
#define AEGPU_ERR_NOMEM 4        /* device allocation failed */
#define AEGPU_ERR_UNSUPPORTED 5  /* input outside what the engine implements */
#define AEGPU_ERR_TOO_LARGE 6    /* input larger than a fixed-size buffer allows */

#define AEGPU_BASIS_FULL 0
#define AEGPU_BASIS_NUMBER 1
#define AEGPU_BASIS_SZ 2

#define AEGPU_HAM_AUTO 0         /* stored ELL rows if they fit in HBM, else on the fly */
#define AEGPU_HAM_STORED 1       /* fixed-width (ELL) rows built on the GPU from the integrals */
#define AEGPU_HAM_ON_THE_FLY 2   /* rows regenerated from h_pq / (pq|rs) on every apply */

typedef struct aegpu_engine aegpu_engine;

/* Context lifetime.  One engine = one problem on the current CUDA device. */
int aegpu_create(aegpu_engine **out);
void aegpu_destroy(aegpu_engine *e);
const char *aegpu_last_error(const aegpu_engine *e);

/* Problem definition: sector basis + excitation list (replaces the setup of
 * FusedEvolve::updateExc / regenCache, fusedevolve.cpp:2085-2095, 1797-1967). */
int aegpu_set_problem(aegpu_engine *e, int nq, int basis_kind, int n_elec, int n_alpha, int n_beta,
                      int complex_mode, int nops, const int *ops);
int64_t aegpu_dim(const aegpu_engine *e);
/* doubles per amplitude: 1 real, 2 complex (re, im interleaved) */
int aegpu_amplitude_width(const aegpu_engine *e);
int aegpu_basis_states(const aegpu_engine *e, uint32_t *out);
int aegpu_num_blocks(const aegpu_engine *e);
/* Operator application order (the reference's m_excPerm) and the size of every pass. */
int aegpu_block_layout(const aegpu_engine *e, int *perm, int *block_sizes);

/* Initial state in the sector (D doubles, 2D in complex mode). */
int aegpu_set_initial(aegpu_engine *e, const double *amps);

/* Hamiltonian as a sector CSR matrix (row = output determinant); duplicates must
 * already be summed.  Replaces HamiltonianMatrix(value, i, j, comp),
 * hamiltonianmatrix.cpp:628-659. */
int aegpu_set_ham_csr(aegpu_engine *e, int64_t nnz, const int64_t *rowptr, const int32_t *col, const double *val);
/* Hamiltonian from molecular-orbital integrals h[p*N+q], g[((p*N+q)*N+r)*N+s] = (pq|rs)
 * (the layout of <prefix>_oneEInts.bin / _twoEInts.bin, hamiltonianmatrix.cpp:402-554).
 * Needs the Sz sector. */
int aegpu_set_ham_integrals(aegpu_engine *e, const double *h1, const double *g2, int mode);

/* Batches (no counterpart in the reference, which evaluates one angle vector per
 * call).  After aegpu_set_batch(e, nb) every evaluation below works on nb instances
 * of the problem at once: angles[nb][nops], energy[nb], grad[nb][nops],
 * state / x / y [nb][D*(1+complex)].  All instances start from the same initial
 * state.  A Hamiltonian set by aegpu_set_ham_csr / aegpu_set_ham_integrals is shared
 * by all instances; aegpu_set_ham_integrals_batch gives instance b its own integrals
 * h1s[b][N*N], g2s[b][N^4] (set the batch size first: changing it drops them).
 * nb is 1..65535; the Hessian needs nb = 1. */
int aegpu_set_batch(aegpu_engine *e, int nb);
/* Launch-shape knobs (picked by the autotuner, ansatzevolve_gb300/autotune.py):
 * excitations fused per pass (1..6; before aegpu_set_problem), CTAs per SM of the
 * pass kernels (1..64; before aegpu_set_problem), threads per CTA of the on-the-fly
 * H kernel (64..1024, multiple of 32; before the Hamiltonian; unset, 512, or as many as
 * fit in equal beta chunks of up to 1024 when the string tables leave room for only one
 * CTA per SM), threads per row of the
 * stored-H product (1, 2, 4, 8; 0 = chosen by size; before the first evaluation),
 * programmatic dependent launch of the pass kernels (0 off, 1 on, -1 by size, the
 * default: on up to 2^19 amplitudes per launch; each pass's CTAs are scheduled while
 * the previous pass drains and wait on the device for its results; any time, it
 * rebuilds the captured graphs), reuse of H psi between an energy and a gradient at the
 * same angles (1, the default, or 0: the gradient recomputes H psi as the reference's
 * evolveDerivative does, fusedevolve.cpp:2292; the environment variable
 * AEGPU_REUSE_HPSI=0 sets 0 for engines created afterwards, e.g. the one behind the
 * reference-compatible C ABI), and the spin-flip half product of the energy's H psi
 * (1, the default, or 0; AEGPU_FLIP=0 in the environment sets 0 for engines created
 * afterwards): with as many alpha as beta electrons and an integral Hamiltonian (coded
 * stored rows or on the fly), a state with psi(a,b) = psi(b,a) for every pair of alpha
 * and beta strings, which the device tests before every such product (relative norm
 * of the difference <= 1e-12), has H psi of the same symmetry, so only the rows with
 * a <= b are computed and mirrored; and the spin-flip half passes (1, the default, or
 * 0; AEGPU_HALF=0 in the environment sets 0 for engines created afterwards): where
 * every pass holds the mirror of each of its excitations (alpha and beta orbitals
 * exchanged) with the same sign rule, the start state has psi(a,b) = psi(b,a) and, at
 * each evaluation, every excitation's angle equals its mirror's (a device test per
 * instance), the evolution keeps that symmetry, so the forward and adjoint passes
 * visit one orbit of every mirror pair, only the amplitudes with a <= b are kept
 * current during the sweeps (the evolved state is completed by copying them to their
 * mirrors), and each gradient is the sum over the visited orbits for the excitation
 * and its mirror.  Projected gradients always run the full passes; Hessians run the
 * full passes on one tangent of every mirror pair where the same symmetry holds (and
 * on every tangent otherwise).
 * A sweep launch whose CTAs are all resident at once hands its warp tasks out
 * warp-major (warp w of CTA c starts at task w * CTAs + c, so that the tasks left over
 * once every warp has one spread over every SM); AEGPU_TASK_ORDER=0 in the
 * environment keeps the CTA-major order of larger launches everywhere, for engines
 * created afterwards (a diagnostic switch; both orders give results equal to rounding).
 * No counterpart in the reference. */
enum { AEGPU_TUNE_PASS_OPS = 1, AEGPU_TUNE_CTAS_PER_SM = 2, AEGPU_TUNE_OTF_THREADS = 3, AEGPU_TUNE_SPMV_TPR = 4,
       AEGPU_TUNE_PDL = 5, AEGPU_TUNE_REUSE_HPSI = 6, AEGPU_TUNE_FLIP = 7, AEGPU_TUNE_HALF = 8 };
int aegpu_set_tuning(aegpu_engine *e, int knob, int value);
int aegpu_get_tuning(const aegpu_engine *e, int knob);
/* used[b] = 1 where the last energy evaluation's H psi of instance b took the spin-flip
 * half product, 0 where it took the full one (or did not test; masked instances keep
 * their earlier value).  Synchronises the engine's stream. */
int aegpu_flip_status(aegpu_engine *e, int *used);
/* used[b] = 1 where the last evaluation of instance b ran the spin-flip half passes
 * (AEGPU_TUNE_HALF).  info[4]: whether the problem allows them, amplitudes touched per
 * sweep over all passes with them, FP64 instructions of their forward and adjoint
 * passes per evaluation (as aegpu_fp64_work counts the full ones).  No counterpart in
 * the reference. */
int aegpu_half_status(aegpu_engine *e, int *used);
int aegpu_half_info(const aegpu_engine *e, int64_t *info);
int aegpu_batch_size(const aegpu_engine *e);
/* Instance mask of batched evaluations: active[b] = 0 skips instance b (its results are
 * left as they were); NULL makes every instance active.  The Hessian and the H*x
 * calls ignore the mask. */
int aegpu_set_active(aegpu_engine *e, const int *active);
int aegpu_set_ham_integrals_batch(aegpu_engine *e, const double *h1s, const double *g2s, int mode);
/* Which representation is in use: 1 CSR, 2 stored ELL, 3 on the fly; and its stored entries. */
int aegpu_ham_info(const aegpu_engine *e, int *kind, int64_t *stored_entries);

/* Evaluations (FusedEvolve::evolve / getEnergy / evolveDerivative / evolveHessian,
 * fusedevolve.cpp:2105-2159, 2782-2795, 2263-2346, 2437-2780).  Energies exclude
 * any nuclear constant.  state may be NULL. */
int aegpu_evolve(aegpu_engine *e, const double *angles, double *state);
int aegpu_energy(aegpu_engine *e, const double *angles, double *energy);
int aegpu_gradient(aegpu_engine *e, const double *angles, double *energy, double *grad_ops);
/* Hessian in the compressed parameters: theta_op = scale[op] * x[param[op]]. */
int aegpu_hessian(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                  double *energy, double *grad_comp, double *hess_comp);
int aegpu_apply_h(aegpu_engine *e, const double *x, double *y);
/* Projected Hessian (FusedEvolve::evolveHessianProj, fusedevolve.cpp:2882-3183):
 * d^2 <proj|psi> / dx_i dx_j in the compressed parameters, with the gradient
 * d<proj|psi>/dx and overlap <proj|psi>; proj[D*(1+complex)], batch of 1. */
int aegpu_hessian_proj(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                       const double *proj, double *overlap, double *grad_comp, double *hess_comp);
/* aegpu_hessian plus the metric g = Re(T_C^dagger T_C) of the compressed tangents
 * T_C mu = d psi / d x_mu (nparams x nparams; tupsquantities.cpp:386-389). */
int aegpu_hessian_metric(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                         double *energy, double *grad_comp, double *hess_comp, double *metric);

/* Properties (TUPSQuantities::writeProperties, tupsquantities.cpp:185-568;
 * doSubspaceDiagonalisation, :1600-1769).  Batch of 1.
 *
 * aegpu_lowest_eigenpair: the lowest eigenvalue of H in the determinant sector and its
 * eigenvector, kept on the device until H is replaced.  Lanczos from the initial state
 * with full reorthogonalisation, restarted from the Ritz vector after `basis` products,
 * until the residual estimate is below tol / 2 or max_products H products are spent;
 * eigenvalue is the Rayleigh quotient of the unit eigenvector, residual its true
 * ||H v - lambda v||, products the H products used.  Its sign makes <start|v> >= 0.
 * (The reference iterates v <- H v / |H v| from the same start, which converges to the
 * eigenvector of largest |lambda|: the same vector whenever the lowest eigenvalue is
 * also the largest in magnitude.)  Not converging within max_products is not an error:
 * compare the residual with tol. */
int aegpu_lowest_eigenpair(aegpu_engine *e, double tol, int basis, int max_products, double *eigenvalue,
                           double *residual, int *products);
/* The nstates lowest eigenpairs (eigenvalues ascending; residuals nullable), for the
 * overlaps with several eigenstates that writeProperties reports
 * (TUPSQuantitiesOptions::numberOfOverlapsToCompute, tupsquantities.cpp:229-276, where the
 * reference takes every eigenvector of a dense H below 5,000 rows).  The same Lanczos
 * iteration as aegpu_lowest_eigenpair, but started from a seeded pseudo-random real vector so
 * that eigenstates of every spin symmetry of the sector appear in their order, restarted
 * from the sum of the Ritz vectors, converged when every one of the nstates residual
 * estimates is below tol / 2.  The eigenvectors replace the one of aegpu_lowest_eigenpair
 * on the device (state 0 is then the lowest of all symmetries).  Signs: <start|v> > 0, or
 * the largest-magnitude entry positive where that overlap vanishes. */
int aegpu_lowest_eigenpairs(aegpu_engine *e, int nstates, double tol, int basis, int max_products, double *eigenvalues,
                            double *residuals, int *products);
/* <psi(angles)|v_i> for the first nstates eigenvectors held: overlaps[2 i] real part,
 * overlaps[2 i + 1] imaginary part. */
int aegpu_ground_overlaps(aegpu_engine *e, const double *angles, int nstates, double *overlaps);
/* The eigenvector, D*(1+complex) doubles in sector order. */
int aegpu_ground_state(aegpu_engine *e, double *state);
/* <psi(angles)|v>: overlap[0] real part, overlap[1] imaginary part. */
int aegpu_ground_overlap(aegpu_engine *e, const double *angles, double *overlap);
/* <r|H|r> / <r|r> for the real part r of psi(angles) (tupsquantities.cpp:418-423; the
 * energy itself for real states). */
int aegpu_real_energy(aegpu_engine *e, const double *angles, double *real_energy);
/* For nsets angle vectors (angles[nsets][nops]): H_ij = <psi_i|H|psi_j> and
 * S_ij = <psi_i|psi_j>, row-major nsets x nsets; the imaginary parts (h_im, s_im, may
 * be NULL) are 0 for real states. */
int aegpu_subspace_matrices(aegpu_engine *e, int nsets, const double *angles, double *h_re, double *h_im, double *s_re,
                            double *s_im);

/* One path's row of the reference's properties table (printOutputLine calls,
 * tupsquantities.cpp:538-566), at per-operator angles with the compressed parameters
 * (param, scale): row[AEGPU_PROPERTY_ROWS], NaN where not computed.  flags:
 * AEGPU_PROP_HESSIAN adds the Hessian / metric counts (eigenvalues and diagonal entries
 * below -1e-10, within 1e-10, above 1e-10; :466-533) and fills hessian / metric
 * (nparams^2 each, nullable); AEGPU_PROP_OVERLAP adds <psi|v> with the eigenvector of
 * aegpu_lowest_eigenpair.  Energies exclude nuclear_energy except the third row. */
#define AEGPU_PROP_HESSIAN 1
#define AEGPU_PROP_OVERLAP 2
#define AEGPU_PROP_HF_PATH 4  /* writeProperties: the first path is the zero-angle ("HF") one */
#define AEGPU_PROP_ELEC_ENERGY 0
#define AEGPU_PROP_REAL_ELEC_ENERGY 1
#define AEGPU_PROP_ELEC_NUC_ENERGY 2
#define AEGPU_PROP_NEG_HESSIAN_EVALUES 3
#define AEGPU_PROP_NEAR_ZERO_HESSIAN_EVALUES 4
#define AEGPU_PROP_POS_HESSIAN_EVALUES 5
#define AEGPU_PROP_NEG_HESSIAN_DIAG 6
#define AEGPU_PROP_NEAR_ZERO_HESSIAN_DIAG 7
#define AEGPU_PROP_POS_HESSIAN_DIAG 8
#define AEGPU_PROP_POS_METRIC_EVALUES 9
#define AEGPU_PROP_ZERO_METRIC_EVALUES 10
#define AEGPU_PROP_ZERO_METRIC_DIAG 11
#define AEGPU_PROP_NORM_OF_GRAD 12
#define AEGPU_PROP_OVERLAP_RE 13
#define AEGPU_PROP_OVERLAP_IM 14
#define AEGPU_PROP_OVERLAP_MAG 15
#define AEGPU_PROPERTY_ROWS 16
int aegpu_path_properties(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                          double nuclear_energy, int flags, double *row, double *hessian, double *metric);
/* Subspace diagonalisation of nsets states (doSubspaceDiagonalisation,
 * tupsquantities.cpp:1600-1700): the eigenvalues (ascending, nsets) of S^-1/2 H S^-1/2,
 * with S's eigenvalues below 1e-14 treated as its null space (whose directions give
 * eigenvalue 0, as in the reference), and that null space's dimension. */
int aegpu_subspace_eigenvalues(aegpu_engine *e, int nsets, const double *angles, double *eigenvalues, int *null_rank);

/* Projected sweep (FusedEvolve::evolveDerivativeProj, fusedevolve.cpp:2814-2880):
 * overlap[b] = <proj_b|psi_b(theta_b)> and grad[b][op] = d overlap / d theta_op for a
 * fixed bra proj[nb][D*(1+complex)] (no factor 2, unlike the energy gradient). */
int aegpu_gradient_proj(aegpu_engine *e, const double *angles, const double *proj, double *overlap, double *grad_ops);

/* Device-resident variants (inputs already in HBM): angles_dev[nb][nops],
 * energy_dev[nb], grad_dev[nb][nops].  Enqueued on `stream`; nothing is synchronised. */
int aegpu_gradient_dev(aegpu_engine *e, const double *angles_dev, double *energy_dev, double *grad_dev, void *stream);
int aegpu_energy_dev(aegpu_engine *e, const double *angles_dev, double *energy_dev, void *stream);
/* aegpu_gradient_dev replays one captured CUDA graph of the whole evaluation
 * (default; phase timing uses the stream path instead).  enable = 0 disables it. */
int aegpu_use_graphs(aegpu_engine *e, int enable);
/* The engine's own device buffers that its captured evaluation graph reads (angles
 * [nb][nops]) and writes (energies [nb], gradients [nb][nops]).  Valid until the
 * batch size or the problem changes. */
int aegpu_io_dev(aegpu_engine *e, double **angles_dev, double **energy_dev, double **grad_dev);
/* Copies between host arrays and those buffers, enqueued on `stream` (NULL: the
 * engine's own stream); aegpu_io_get_results synchronises the stream. */
int aegpu_io_put_angles(aegpu_engine *e, const double *angles, void *stream);
int aegpu_io_get_results(aegpu_engine *e, double *energy, double *grad, void *stream);
/* Energy + gradient of every instance at the angles in the io buffer, written to
 * the io result buffers: one replay of the captured graph on `stream`. */
int aegpu_launch_io(aegpu_engine *e, void *stream);
/* A group evaluates several engines (e.g. batches of different determinant-space
 * sizes) with ONE graph launch: each member's captured energy + gradient graph is a
 * child node with no dependencies, reading and writing the member's aegpu_io_dev
 * buffers.  Launching fails with AEGPU_ERR_STATE once a member's batch size or
 * Hamiltonian has changed.  No counterpart in the reference. */
typedef struct aegpu_group aegpu_group;
int aegpu_group_create(aegpu_group **out, aegpu_engine *const *engines, int n);
/* stream NULL: the group's own stream.  aegpu_group_sync waits for the latest launch. */
int aegpu_group_launch(aegpu_group *g, void *stream);
int aegpu_group_sync(aegpu_group *g);
int64_t aegpu_group_launch_count(const aegpu_group *g);
void aegpu_group_destroy(aegpu_group *g);
/* Optimisers.  Compressed parameters x[P]: theta_op = scale[op] * x[param[op]].
 * aegpu_optimise_newton: the reference's Newton method (TUPSQuantities::OptimiseTups,
 * tupsquantities.cpp:1940-2011) for a batch of 1, with the analytic Hessian; x is the
 * start on entry and the optimum on return.
 * aegpu_optimise_batch: all nb instances (x[nb][P]) by lockstep BFGS, one batched
 * energy + gradient evaluation per round, until |g| < gtol for every instance or
 * max_rounds rounds; max_step bounds each trial step's length (<= 0: 1.0).  hinv
 * (nullable, [nb][P][P]): each instance's initial inverse Hessian on entry (else a
 * scaled identity), its final BFGS approximation on return.
 * No counterpart in the reference for the batched optimiser. */
int aegpu_optimise_newton(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x, double gtol,
                          double *energy, double *gnorm, int64_t *hessian_evals, int64_t *energy_evals);
int aegpu_optimise_batch(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x, double gtol,
                         int max_rounds, double max_step, double *hinv, double *energy, double *gnorm, int *iters,
                         int64_t *rounds);
/* The reference's projected iteration (TUPSQuantities::iterativeTups with
 * runNewtonMethodProjected, tupsquantities.cpp:2044-2145, 1238-1465) on a batch-of-1
 * engine: freeze psiH = H psi, minimise <psiH|psi(x)> by projected Newton steps, renew
 * psiH; stop when the projected gradient is below gtol (the reference uses 1e-5) or
 * after max_outer renewals.  x: start on entry, result on return. */
int aegpu_optimise_projected(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x,
                             double gtol, int max_outer, double *energy, double *gnorm, int64_t *hessian_evals,
                             int64_t *energy_evals, int *outer_iters);
/* The same with DIIS over the renewals (the reference's iterativeTups with doDIIS,
 * tupsquantities.cpp:2101-2122; diis.h:16-209): the compressed angles are extrapolated
 * from the last diis_size iterations with the state changes as error vectors; ediis
 * selects EDIIS (non-negative coefficients, the reference's choice, size 15) over
 * Pulay DIIS.  diis_size 0 is aegpu_optimise_projected. */
int aegpu_optimise_projected_diis(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x,
                                  double gtol, int max_outer, int diis_size, int ediis, double *energy, double *gnorm,
                                  int64_t *hessian_evals, int64_t *energy_evals, int *outer_iters);
/* Host-only: the DIIS coefficients for an n x n matrix of error inner products. */
int aegpu_host_diis_coefficients(int n, const double *B, int ediis, double *c);
/* Learned warm start (no counterpart in the reference): an MLP
 * n_in -> n_hidden -> n_hidden -> n_out with GELU activations, BF16 weights in every
 * product, FP32 accumulation, FP32 master weights trained by Adam on the mean squared
 * error of standardised targets.  Inputs are standardised with (x - in_mean) /
 * in_scale and outputs returned as y * out_scale + out_mean (identity by default).
 * Parameters (aegpu_mlp_get_params / set_params / loss_grad gradients), FP32:
 * W1[H][n_in], b1[H], W2[H][H], b2[H], W3[n_out][H], b3[n_out]. */
typedef struct aegpu_mlp aegpu_mlp;
int aegpu_mlp_create(aegpu_mlp **out, int n_in, int n_hidden, int n_out, uint64_t seed);
void aegpu_mlp_destroy(aegpu_mlp *m);
const char *aegpu_mlp_last_error(const aegpu_mlp *m);
int64_t aegpu_mlp_num_params(const aegpu_mlp *m);
int aegpu_mlp_set_scaling(aegpu_mlp *m, const float *in_mean, const float *in_scale, const float *out_mean,
                          const float *out_scale);
int aegpu_mlp_get_params(aegpu_mlp *m, float *params);
int aegpu_mlp_set_params(aegpu_mlp *m, const float *params);
int aegpu_mlp_train(aegpu_mlp *m, const float *X, const float *T, int n, int epochs, int batch, float lr,
                    uint64_t seed, float *epoch_loss);
int aegpu_mlp_loss_grad(aegpu_mlp *m, const float *X, const float *T, int n, float *loss, float *grads);
int aegpu_mlp_predict(aegpu_mlp *m, const float *X, int n, float *Y);
int aegpu_mlp_predict_dev(aegpu_mlp *m, const float *X_dev, int n, float *Y_dev, void *stream);
/* y_dev = H x_dev on device vectors (one per instance of the batch, one launch);
 * energy_dev (nullable) receives <x|H x>.  Flip-invariant inputs take the spin-flip half
 * product (AEGPU_TUNE_FLIP). */
int aegpu_apply_dev(aegpu_engine *e, const double *x_dev, double *y_dev, double *energy_dev, void *stream);
/* CUDA-event timing of the phases of aegpu_gradient_dev (evolve, H*psi + energy,
 * adjoint sweep): enable, then read the accumulated milliseconds (and the number of
 * evaluations) -- reading resets the accumulators. */
int aegpu_phase_timing(aegpu_engine *e, int enable);
int aegpu_phase_times(aegpu_engine *e, double *ms3, int64_t *count);
/* info[8]: D, operators, fused blocks, Hamiltonian kind, stored H entries, stored row
 * width (padded), amplitudes touched per sweep over all blocks, nonzeros of H. */
int aegpu_problem_info(const aegpu_engine *e, int64_t *info);
/* Device pointers of the current state and of H*state (D or 2D doubles). */
int aegpu_state_dev(aegpu_engine *e, const double **psi, const double **hpsi);

/* Host-only (no GPU): the lowest eigenpair of a symmetric tridiagonal matrix
 * (diagonal a[k], off-diagonal b[k-1]) as aegpu_lowest_eigenpair's Lanczos step solves it. */
int aegpu_host_tridiag_lowest(int k, const double *a, const double *b, double *v, double *theta);
/* Host-only: the nev lowest eigenpairs of the same matrix as aegpu_lowest_eigenpairs solves
 * it: theta[nev] ascending, V[j * k + i] the unit eigenvectors. */
int aegpu_host_tridiag_lowest_k(int k, int nev, const double *a, const double *b, double *theta, double *V);
/* Host-only: the eigen-analysis of aegpu_subspace_eigenvalues on given matrices
 * (row-major nsets x nsets real / imaginary parts; the imaginary parts may be NULL). */
int aegpu_host_subspace_eigenvalues(int nsets, const double *h_re, const double *h_im, const double *s_re,
                                    const double *s_im, double *eigenvalues, int *null_rank);
/* Host-only inspection of the setup (no GPU needed): the operator application order
 * and block sizes (negative = diagonal block) that aegpu_set_problem would use, and
 * the orbit tables of one block of excitations.  For tests of the setup logic.
 * aegpu_host_orbits: n_idx / n_groups / n_tiles are in/out capacities -> sizes;
 * groups are 4 uint32 (idx_off, n_orbits, k, mask) each, tiles 4 uint32 each. */
int aegpu_host_block_layout(int nq, int nops, const int *ops, int *perm, int *block_sizes, int *n_blocks);
/* Spin-flip half tables of one pass of commuting excitations (Sz basis, nA_elec alpha
 * and as many beta electrons; host setup, no GPU; no counterpart in the reference):
 * idx / bits are the entries (canonical ranks; bit 31 of a bitstring marks a member of a
 * self-mirror orbit that does not write), tasks 4 uint32 each (group with bit 31 for a
 * self-mirror task, elem_off, n, mask); n_idx / n_tasks are capacities -> sizes.
 * AEGPU_ERR_UNSUPPORTED where an excitation has no mirror in the pass or a sign differs
 * from its mirror's. */
int aegpu_host_half_orbits(int nq, int nA_elec, int nops, const int *ops, uint32_t *idx, uint32_t *bits,
                           int64_t *n_idx, uint32_t *tasks, int64_t *n_tasks);
/* The engine's passes for an operator list (host setup, no GPU; no counterpart in the
 * reference): the grouping of aegpu_host_block_layout cut into passes of <= max_pass
 * paired operators (1..6), runs of diagonal blocks merged into passes of <= 12; with
 * mirror_split, commuting blocks merged and cut between spin-flip mirror pairs, as for
 * the half passes (AEGPU_ERR_UNSUPPORTED, with the plain cut, where an operator has no
 * mirror).  pass_sizes[p] = operators of pass p (negative for a diagonal pass),
 * pass_ops the operators pass by pass; n_passes is the capacity in, the count out. */
int aegpu_host_pass_layout(int nq, int nops, const int *ops, int max_pass, int mirror_split, int *pass_ops,
                           int *pass_sizes, int *n_passes);
int aegpu_host_orbits(int nq, int basis_kind, int n_elec, int n_alpha, int n_beta, int nops, const int *ops,
                      uint32_t *idx, int64_t *n_idx, uint32_t *groups, int64_t *n_groups, uint32_t *tiles, int64_t *n_tiles);

/* The excitation rule itself, for bit-exact checks against the reference's
 * applyExcToBasisState_ (fusedevolve.cpp:27-145): for every operator o (ops[4 o ..],
 * 0-based spin orbitals, -1 absent) and determinant bitstring states[i],
 * partner[o * n + i] and sign[o * n + i] in the reference's convention -- a paired
 * determinant gives its partner and +1 / -1, an inactive one itself and -1, an active
 * phase operator itself and +1 (0 would mean the pass kernels' sign form disagrees).
 * aegpu_exc_rule_dev runs the device code the pass kernels use (device pointers,
 * enqueued on `stream`); aegpu_host_exc_rule the host code the orbit tables are
 * built with. */
int aegpu_exc_rule_dev(int nops, const int *ops, const uint32_t *states_dev, int64_t n, uint32_t *partner_dev,
                       int8_t *sign_dev, void *stream);
int aegpu_host_exc_rule(int nops, const int *ops, const uint32_t *states, int64_t n, uint32_t *partner, int8_t *sign);

/* The Hessian's Gram contraction on caller-held device columns (a test and timing
 * hook; the engine calls the same kernels): the upper triangle (i <= j < V) of
 * C = alpha * A^H B, column-major with leading dimension ldc, for V columns of nrows
 * rows of W doubles (W = 2: complex, re / im interleaved; Cim receives the imaginary
 * part).  Column c of A starts at A + c * lda (lda >= nrows * W).  Entries below the
 * diagonal are left untouched.  Enqueued on `stream`; its scratch comes from the
 * stream-ordered allocator. */
int aegpu_gram_upper_dev(const double *A, int64_t lda, const double *B, int64_t ldb, int64_t nrows, int W, int V,
                         double alpha, double *Cre, double *Cim, int ldc, void *stream);

/* Allocation-free H * x (no counterpart in the reference).
 * For callers that cannot allocate device memory at all -- code running inside a
 * CUDA memory-pool or allocator callback, a library whose device memory is owned and
 * budgeted by a host framework, or a context with no free memory left -- this entry
 * point computes y = H x and <x|H x> for a sector CSR matrix that the caller already
 * holds in device memory (rowptr[D+1], col[nnz], val[nnz]; row = output), without any
 * cudaMalloc, cudaFree or allocating library call.  Its only scratch (one partial sum
 * per 256 rows) lives in a fixed 128 KiB device array that every GPU loading this
 * library keeps until the process exits, so D is limited to 4,194,304 rows; larger
 * inputs return AEGPU_ERR_TOO_LARGE (and print why) without launching anything.
 * The first call on a device looks up that array's device address with the device
 * current; make that first call before any stream capture.  All calls share the one
 * array: calls that overlap on the GPU (different streams, or host threads, without
 * ordering between them) race and give wrong sums; calls ordered on one stream are
 * safe.  Nothing needs clearing between calls -- each call writes every partial sum
 * it reads.  x, y, energy are device pointers that must not overlap (the product is
 * not in place: x == y, or energy on x or y, returns AEGPU_ERR_ARG); stream is a
 * cudaStream_t (NULL = the default stream).  The work is enqueued, not synchronised.
 * The array's device address is looked up once per device and kept until the process
 * exits: it belongs to the device context current at that first call, so after a
 * cudaDeviceReset (or another library resetting the primary context) this entry point
 * must not be called again in that process. */
int aegpu_csr_energy_noalloc(int64_t D, const int64_t *rowptr_dev, const int32_t *col_dev, const double *val_dev,
                             const double *x_dev, double *y_dev, double *energy_dev, void *stream);

/* Bytes of HBM held by the engine, and kernel launches issued since creation. */
int64_t aegpu_device_bytes(const aegpu_engine *e);
/* Fault injection for tests: the next n engine allocations succeed and every later one
 * fails as out of memory (AEGPU_ERR_NOMEM is returned, nothing traps); n < 0 turns it
 * off.  Process-wide. */
void aegpu_debug_fail_alloc_after(int64_t n);
/* FP64 instructions of one energy + gradient evaluation per instance: work[0] H psi
 * (one DFMA per matrix element + the energy FMA), work[1] forward passes, work[2]
 * adjoint passes (complex mode counts each real part), work[3] H psi by the spin-flip
 * half product (its rows, the energy FMAs and the invariance test; 0 where the engine
 * cannot take it).  work holds 4 entries. */
int aegpu_fp64_work(const aegpu_engine *e, int64_t *work);
/* Measured DFMA throughput of the current device, TFLOP/s (FMA = 2 flops). */
int aegpu_fp64_peak(double *tflops);
int64_t aegpu_launch_count(const aegpu_engine *e);

#ifdef __cplusplus
}
#endif
#endif

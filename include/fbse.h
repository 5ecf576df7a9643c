/*
 * fbse.h -- C ABI of libfbse_gpu, the GB300 (sm_103a) implementation of
 * FilterBSE's filter-diagonalization hot path.
 *
 * Plain C: pointers, sizes and POD descriptors only.  Every entry point
 * returns FBSE_OK (0) or a negative FBSE_ERR_* code; the message of the last
 * failure is available from fbse_last_error().  Callers that mirror the
 * reference's error behaviour print that message to stderr and
 * exit(EXIT_FAILURE) (as filter_mpi/norm.c:150-159 and read.c:875 do).
 *
 * Memory: a context owns all of its device scratch.  State arrays passed to
 * the compute entry points are DEVICE pointers (allocate them with
 * fbse_alloc or any CUDA allocator on the context's device); the host-side
 * helpers at the end of this header work on host memory.  All work is
 * ordered on the context's stream; entry points that return host values
 * synchronise that stream.
 *
 * State layouts (the reference's, filter_mpi/fd.h:333-337):
 *   "zomplex state": nspin blocks of ngrid complex values (spin-up first),
 *     grid index jxyz = nx*(ny*jz + jy) + jx, interleaved (re, im), in the
 *     context's working precision (double for FBSE_FP64, float for
 *     FBSE_MIXED).  Used by fbse_hpsi / fbse_hnorm.
 *   "psitot state": stlen = complex_idx * nspin * ngrid doubles, i.e. one
 *     double per point for real jobs and (re, im) pairs for complex jobs --
 *     the layout of psi_rank / psitot / psi.dat.  Always FP64.
 */
#ifndef FBSE_H
#define FBSE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ABI version: fbse_version() returns the value the library was built with */
#define FBSE_ABI_VERSION 1

#define FBSE_OK 0
#define FBSE_ERR_ARG (-1)         /* invalid argument or size */
#define FBSE_ERR_CUDA (-2)        /* CUDA runtime error (message has details) */
#define FBSE_ERR_OOM (-3)         /* device allocation failed */
#define FBSE_ERR_NAN (-4)         /* zero or NaN norm (filter_mpi/norm.c:150-159) */
#define FBSE_ERR_STATE (-5)       /* call out of order / missing setup */
#define FBSE_ERR_UNSUPPORTED (-6) /* configuration not supported by this library */
#define FBSE_ERR_NOCONV (-7)      /* an iterative solver hit its iteration limit */

enum { FBSE_FP64 = 0, FBSE_MIXED = 1 };

typedef struct fbse_ctx fbse_ctx;

/* Grid and job switches: the fields of grid_st / index_st / flag_st that the
 * hot path reads (filter_mpi/fd.h:30-91, 96-163, 257-299). */
typedef struct fbse_grid_desc {
  long nx, ny, nz;   /* grid points per axis (any sizes) */
  double dx, dy, dz; /* spacing, bohr */
  double ke_max;     /* KEmax, Ha: kinetic cap (filter_mpi/init.c:338-349) */
  int nspin;         /* 1, or 2 for spinors */
  int is_complex;    /* flag->isComplex (complex_idx - 1) */
  int so;            /* flag->SO: spin-orbit projectors */
  int nl;            /* flag->NL: nonlocal projectors */
  double dkx, dky, dkz; /* reciprocal spacings; 0 = derived as init_grid_params does
                           (2 pi / (n d) for even n, 2 pi / ((n - 1) d) for odd n,
                           filter_mpi/init.c:65-80); set them to reproduce runs of
                           older versions that used 2 pi / (n d) for every n */
} fbse_grid_desc;

/* Projector table: a structure-of-arrays copy of the reference's nlc_st
 * array (filter_mpi/fd.h:382-398) as built by init_NL_projectors
 * (filter_mpi/init.c, body lines 508-589).  Row stride npts = n_NL_gridpts. */
typedef struct fbse_proj_desc {
  long n_atoms;          /* n_NL_atoms (ligands excluded, filter_mpi/read.c:1102) */
  long npts;             /* n_NL_gridpts: row stride */
  int nproj;             /* ist->nproj (5) */
  const long *nl;        /* [n_atoms] points used per atom */
  const int *jxyz;       /* [n_atoms*npts] grid index of each point */
  const double *y1;      /* [n_atoms*npts][3][2] Y_1m, m = 0..2, (re, im) */
  const double *so_proj; /* [n_atoms*npts][nproj] SO radial (x sqrt(SO_par)) */
  const double *nl_proj; /* [n_atoms*npts][nproj] NL radial */
  const int *nl_sign;    /* [n_atoms][nproj] sign of each NL channel */
  const double *LS;      /* [6][6][2] L.S, LS[(j'*6 + j)] (re, im); NULL: built as def_LS does */
} fbse_proj_desc;

/* ---- context ------------------------------------------------------------ */

/* Replaces the setup of mod_mem_alloc / mod_pseudopot (filter_mpi/mod_mem.c:3,
 * filter_mpi/mod_pseudopot.c:3): uploads the local potential (ngrid doubles;
 * the reference stores it twice, filter_mpi/init.c:666 -- pass one copy) and
 * the projector table, and plans the FFTs.  proj may be NULL when so = nl = 0.
 * precision: FBSE_FP64 (plain) or FBSE_MIXED (FP32 recursion and FFTs). */
int fbse_create(fbse_ctx **out, const fbse_grid_desc *grid, const double *pot_local,
                const fbse_proj_desc *proj, int precision);
void fbse_destroy(fbse_ctx *ctx);
const char *fbse_last_error(const fbse_ctx *ctx);
int fbse_version(void);
/* Number of CUDA kernels this library has launched since it was loaded
 * (all contexts), for launch accounting around a timed region. */
long fbse_launch_count(void);

/* ---- device memory helpers --------------------------------------------- */
int fbse_alloc(fbse_ctx *ctx, void **dptr, size_t bytes);
int fbse_free(fbse_ctx *ctx, void *dptr);
int fbse_upload(fbse_ctx *ctx, void *dst_dev, const void *src_host, size_t bytes);
int fbse_download(fbse_ctx *ctx, void *dst_host, const void *src_dev, size_t bytes);
int fbse_sync(fbse_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t) so callers can order their own
 * work and events with the context's kernels. */
void *fbse_stream(fbse_ctx *ctx);

/* ---- kernel choices and the autotuner (no counterpart in the reference) ----
 * The launch shapes and kernel variants a context uses.  A field left 0 is
 * chosen by the context: the autotuner fields are timed on the first call that
 * needs them (on the context's stream, on that call's own data, all
 * candidates giving bit-identical results) and the fastest is kept for the
 * context's life; fbse_tuning_report lists every choice with its timings.  A
 * nonzero field fixes the choice.  Set it before the first compute call; the
 * first call of each batch size should come before any stream capture. */
typedef struct fbse_tuning {
  int fft_kernels;         /* 0: register-resident kernels for 64/128/256-point axes where they fit,
                              mixed-radix elsewhere; 1: mixed-radix kernels on every axis; 2: mixed-radix
                              x lines and y/z columns (no plane kernel).  Results differ in rounding only */
  int fft_plane_cluster;   /* 0: one CTA per 128 x 128 FP32 plane; 1: two-CTA clusters (same results) */
  long fft_chunk_blocks;   /* 3D blocks (state x spin) per FFT launch sequence; 0: autotuned */
  int scatter_states;      /* projector scatter: 1/2/4/8 states per thread (a thread per point), or
                              18/20: a CTA per chunk of points with 2/4 states per group; 0: autotuned */
  int gather_points;       /* points per lane per projector-gather iteration, 1/2/4; 0: autotuned */
  int newton_ring;         /* Newton ring slots, 8..128 (the FP32 block sums depend on it); 0: 128 */
  int bse_simt;            /* 1: the mixed path's BSE contraction on the FP32 SIMT kernel instead of
                              the tensor cores */
  double tc_image_bytes;   /* tensor-core operand images per K chunk, bytes; 0: 24e9 */
  double ritz_cut;         /* overlap eigenvalues kept by fbse_ortho_diag_sigma, relative to the largest
                              (the role of SVDEPS, filter_mpi/fd.h); 0: 1e-12 (FP64), the mixed path's own
                              default otherwise */
  int ritz_hpsi;           /* H psi of the mixed path's Rayleigh-Ritz step: 0 default (FP32), 1 FP32,
                              2 FP64 (the FP64 operator's tables are held by every context) */
  int hpsi_fused;          /* 1: FP32 H psi on 128 x 128 x nz grids with the projector gather and scatter
                              fused into the xy plane passes (slower than the separate projector
                              kernels on the measured workloads); 0: separate projector kernels.
                              Results differ in rounding only */
  int hpsi_streams;        /* parts of an H psi batch with projectors, each on its own stream of the
                              context (when input and output do not overlap), so that one part's
                              projector kernels and tail waves overlap the others' kernels: 0 = 2,
                              1 = the whole batch on the context's stream, 2..4.  Same results */
} fbse_tuning;
int fbse_get_tuning(fbse_ctx *ctx, fbse_tuning *t);
int fbse_set_tuning(fbse_ctx *ctx, const fbse_tuning *t);
/* JSON text of the autotuner's decisions so far (kernel, problem, candidates
 * with their times in microseconds, choice); returns the length needed
 * (excluding the terminating 0), writes at most n bytes including it. */
long fbse_tuning_report(fbse_ctx *ctx, char *buf, long n);

/* ---- H psi ------------------------------------------------------------------
 * fbse_hpsi and fbse_hnorm only enqueue kernels on the context's stream (no
 * host synchronisation); the first call sizes their scratch and sets kernel
 * attributes.  The composite calls below (filter, energy range, orthogonal-
 * isation / diagonalisation / sigma, the BSE stages) synchronise with the host
 * between phases (eigensolver sweeps, convergence checks, small host-side
 * steps) and return with their results on the host or complete on the device.
 * Capturing fbse_hpsi into a CUDA graph is not exercised by the tests.
 *
 * Replaces p_hamiltonian (filter_mpi/phamiltonian.c:10-60) for a batch:
 * psi_out[s] = H psi_in[s] for nstates zomplex states.  For real jobs the two
 * channels are two independent real states (H is real), so a real state in
 * .re with .im = 0 gives the reference's real-path result in .re. */
int fbse_hpsi(fbse_ctx *ctx, const void *psi_in, void *psi_out, long nstates);

/* Replaces p_hnorm (filter_mpi/filter.c:375-410): psi_out = (4/dE)(H psi_in)
 * - (2 + zn + 4 Vmin/dE) psi_in, for nstates zomplex states. */
int fbse_hnorm(fbse_ctx *ctx, const void *psi_in, void *psi_out, long nstates, double vmin, double de, double zn);

/* ---- Newton filter -------------------------------------------------------
 * Replaces filter_cycle (filter_mpi/filter.c:187-371) for nstart random starts
 * at once.  zn: ncheby sample points (host); an: [m][ncheby] complex Newton
 * coefficients (host, interleaved; imaginary parts must be 0, which
 * gen_newton_coeff always produces); psi0: [nstart] psitot states (device);
 * filtered: [nstart][m] psitot states (device) -- the psi_rank layout
 * (ns_block = jns*m*stlen, filter_mpi/filter.c:253). */
int fbse_newton_filter(fbse_ctx *ctx, const double *zn, const double *an, long ncheby, long m, double vmin,
                       double de, const double *psi0, long nstart, double *filtered);

/* ---- spectrum range ------------------------------------------------------
 * Replaces the iterative branch of get_energy_range (filter_mpi/energy.c:
 * 169-379): imaginary-time descent (tau = 0.05) for Emin and power iteration
 * for Emax from random states drawn with the reference's generator starting
 * at `seed` (the reference uses -874917403), stopping at a relative change
 * below 1e-6 or max_iter iterations.  Returns the raw Emin / Emax; the
 * range inflation is applied by fbse_inflate_range. */
int fbse_energy_range(fbse_ctx *ctx, long seed, long max_iter, double *emin, double *emax, long *iters);

/* ---- normalisation and energies ------------------------------------------
 * normalize_all (filter_mpi/norm.c:82-179) and energy_all
 * (filter_mpi/energy.c:61-165) over n psitot states (device).  norms / ene
 * are host arrays of n doubles (may be NULL for norms).  A zero or NaN norm
 * returns FBSE_ERR_NAN. */
int fbse_normalize_all(fbse_ctx *ctx, double *psitot, long n, double *norms);
int fbse_energy_all(fbse_ctx *ctx, const double *psitot, long n, double *ene);

/* calc_sigma_E (filter_mpi/energy.c:383-539) over n psitot states (device):
 * eval_i = dv Re<psi_i|H psi_i> and sigma_i = sqrt|dv <H psi_i|H psi_i> -
 * eval_i^2| (host arrays of n doubles).  The reference forms <psi|H (H psi)>,
 * equal for Hermitian H; the states are not normalised here (the reference
 * expects normalised states, as after diag_H or restart_from_sigma). */
int fbse_sigma_e(fbse_ctx *ctx, const double *psitot, long n, double *eval, double *sigma);

/* fbse_normalize_all without any allocation (no counterpart in the reference):
 * for callers that must not allocate device memory mid-run.  Its scratch is a
 * file-scope device array of about 1.06 MB, at most 1024 states per call
 * (more returns FBSE_ERR_ARG).  The first call in each CUDA context (the
 * device's primary context for runtime-API callers; a device reset makes a new
 * one) looks the array's address up (cudaGetSymbolAddress, with that device
 * current) and should come before any stream capture.  The array is shared by
 * all fbse contexts on a device: calls that overlap in time race.  norms may
 * be NULL; on a zero or NaN norm it holds the norms up to and including the
 * first failing state, as fbse_normalize_all leaves it, and the states are
 * left unscaled. */
int fbse_normalize_all_noalloc(fbse_ctx *ctx, double *psitot, long n, double *norms);

/* ---- orthogonalisation, subspace diagonalisation, sigma_E ----------------
 * Replaces mod_ortho + mod_diag + mod_sigma (filter_mpi/mod_ortho.c:3-94,
 * mod_diag.c:324-449, mod_sigma.c:6-63) for n psitot states (device, in
 * place): the span is orthonormalised (overlap eigen-decomposition, rank
 * cutoff s_i/s_0 < 1e-10 as SVDEPS in filter_mpi/fd.h), H is diagonalised in
 * it in FP64 on the GPU, the first n_kept states are overwritten with the
 * eigenvectors (ascending eigenvalue, normalised), and eval / sigma (host,
 * n doubles each) receive E_i = <psi_i|H|psi_i> and
 * sigma_i = ||(H - E_i) psi_i||, which equals the reference's
 * sqrt|<H^2> - <H>^2| for normalised states. */
int fbse_ortho_diag_sigma(fbse_ctx *ctx, double *psitot, long n, long *n_kept, double *eval, double *sigma);

/* ---- spin and angular-momentum statistics of the filter's states ---------
 * Replaces calc_angular_exp (filter_mpi/angular.c:4-165), the
 * calcSpinAngStat output of mod_optional_output (mod_optional_output.c:51-62),
 * for n complex spinor states (psitot layout, device, FP64; the context must
 * have nspin = 2 and is_complex = 1, else FBSE_ERR_UNSUPPORTED).  Each state
 * passes the reference's k-space low-pass (low_pass_filter, angular.c:403-455)
 * and is normalised; J = L + S is applied with L = r x p, p = -i grad by FFT
 * on the context's grid (apply_L_op, angular.c:218-400; coordinates gx, gy,
 * gz on the host as grid->x / y / z, distribution centre at the origin as in
 * the reference) and S = sigma / 2 (apply_J_op, angular.c:169-216).  stats
 * (host, 8 n doubles) receives per state the columns of angular.dat:
 * <Jx>, <Jx^2>, <Jy>, <Jy^2>, <Jz>, <Jz^2>, <J^2>, norm.  Every state is
 * read from its own slot (angular.c:63 reads the spin-up imaginary part of
 * state i > 0 from offset i * nspinngrid instead of 2 i * nspinngrid).
 * Returns FBSE_ERR_NAN for a state whose low-passed norm is zero or NaN. */
int fbse_angular_stats(fbse_ctx *ctx, const double *psitot, long n, const double *gx, const double *gy,
                       const double *gz, double *stats);

/* ---- slab products (FP64) ---------------------------------------------------
 * The two dense products of the Rayleigh-Ritz step restricted to a slab of
 * each state's values [off, off + len) (complex values for complex states, as
 * psitot holds them; off = 0, len = nspin * ngrid for whole states): the
 * dv-weighted overlap of diag_H / the SVD of ortho (filter_mpi/Hmat.c:115-170,
 * ortho.c:150), and the rotation Psi C of diag_H (Hmat.c:230-281).  With the
 * points of every state split into slabs over processes, the all-reduced sum of
 * the slab Grams is the Gram of the whole states, and each process rotates its
 * own slab.
 *   fbse_gram:   out[i][j] = dv sum_l conj(A_i[l]) B_j[l], na x nb complex
 *                (host, row-major, (re, im) pairs); A, B device psitot rows.
 *   fbse_rotate: out_j[l] = sum_i coef[i][j] A_i[l] for j < k, l in the slab;
 *                coef host na x k complex, row-major; out device psitot rows
 *                (values outside the slab untouched), not aliasing A. */
int fbse_gram(fbse_ctx *ctx, const double *A, long na, const double *B, long nb, long off, long len, double *out);
int fbse_rotate(fbse_ctx *ctx, const double *A, long na, const double *coef, long k, long off, long len, double *out);

/* ---- whole filter stage with host buffers ----------------------------------
 * run_filter_cycles + mod_ortho + mod_diag + mod_sigma + mod_output's state
 * selection (filter_mpi/filter.c:5-183, mod_ortho.c:3-94, mod_diag.c:324-449,
 * mod_sigma.c:6-63, mod_output.c:5-162) in one call on HOST buffers:
 * psi0_host [nstart] psitot states in; eval_host / sigma_host (nstart*m
 * doubles each) and psi_host ([nstart*m] psitot states, may be NULL) out, in
 * ascending eigenvalue order.  sigma_cut <= 0 keeps every state
 * (getAllStates = 1); otherwise only states with sigma_E <= sigma_cut are
 * returned (getAllStates = 0).  *n_out receives the number returned. */
int fbse_filter_job(fbse_ctx *ctx, const double *zn, const double *an, long ncheby, long m, double vmin, double de,
                    const double *psi0_host, long nstart, double sigma_cut, long *n_out, double *eval_host,
                    double *sigma_host, double *psi_host);

/* ---- multi-dot filter in one CUDA graph (no counterpart in the reference) ----
 * Independent dots of uneven size (each its own context: grid, potential,
 * projector table) filtered by one graph launch instead of their kernels
 * one by one.  fbse_batch_create validates every dot, uploads its Newton
 * coefficients, runs each dot's filter once through fbse_newton_filter
 * (buffers sized, launch shapes autotuned; filtered receives the result) and
 * captures the filters of all dots into one graph, each dot an independent
 * branch on its context's stream.  fbse_batch_run replays it (results
 * bit-identical to the sequential path); fbse_batch_run_sequential runs
 * fbse_newton_filter dot after dot, for comparison.  The dots' device
 * buffers (psi0, filtered) must stay valid while the batch exists.  The
 * reference's parallel dimension is the random starts of one dot, one MPI
 * rank each (filter_mpi/filter.c:100-104, mod_filter.c:155-159). */
typedef struct fbse_batch_dot {
  fbse_ctx *ctx;          /* one context per dot */
  const double *zn;       /* host [ncheby] */
  const double *an;       /* host [m][ncheby] complex */
  long ncheby, m;
  double vmin, de;
  const double *psi0;     /* device psitot [nstart] */
  long nstart;
  double *filtered;       /* device psitot [nstart * m] */
} fbse_batch_dot;
typedef struct fbse_batch fbse_batch;
int fbse_batch_create(fbse_batch **out, const fbse_batch_dot *dots, int ndots);
int fbse_batch_run(fbse_batch *b);
int fbse_batch_run_sequential(fbse_batch *b);
long fbse_batch_graph_nodes(const fbse_batch *b);
const char *fbse_batch_last_error(const fbse_batch *b);
void fbse_batch_destroy(fbse_batch *b);

/* ---- learned residual preconditioner and refinement ------------------------
 * No counterpart in the reference: its only remedy for unconverged states is
 * to filter again with more starts and terms (retryFilter,
 * filter_mpi/mod_output.c:131-147).  A small 3D convolutional network maps
 * the residual r = (H - E) psi of a Ritz pair to a correction of psi.  Each
 * real field of r (real and imaginary part of each spin block) is one input,
 * normalised by its RMS; the network sees it with the local potential as
 * [r^, r^ (V - E) / 1 Ha] (2 channels), runs four 3x3x3 convolutions with
 * 16 channels (tanh after the first three, no biases, so the correction is
 * odd in r) and returns one channel y, scaled back by the RMS and added to the
 * input: P(r) = r + y rms (a residual connection, so a network whose last
 * layer is zero is the plain residual refinement).  Weights are FP32
 * (FBSE_PRECOND_NWEIGHTS floats: layer l's [c_out][c_in][27] blocks in order),
 * activations BF16, arithmetic FP32.  Training (Adam, mean squared error
 * against target corrections) and inference run on the GPU in the library's
 * own forward and backward kernels. */
typedef struct fbse_precond fbse_precond;
#define FBSE_PRECOND_NWEIGHTS 15120
/* weights NULL: seeded random initialisation (scaled uniform; the last layer
 * at a tenth of its scale, so P starts close to the identity) */
int fbse_precond_create(fbse_ctx *ctx, fbse_precond **out, const float *weights_host, long seed);
/* May come before or after fbse_destroy of its context (it touches only its
 * own memory); every other fbse_precond_* call needs the context alive. */
void fbse_precond_destroy(fbse_precond *p);
int fbse_precond_get_weights(fbse_precond *p, float *weights_host);
int fbse_precond_set_weights(fbse_precond *p, const float *weights_host);
/* forward on n psitot states (device): out[i] = P(resid[i]; V - ene[i]),
 * ene host.  out must not alias resid. */
int fbse_precond_apply(fbse_precond *p, const double *resid, const double *ene, long n, double *out);
/* loss and weight gradient (host, FBSE_PRECOND_NWEIGHTS floats, may be NULL)
 * of the mean squared error between P(resid[i]) / rms and corr[i] / rms over
 * the n states (device psitot, ene host) without changing the weights */
int fbse_precond_grad(fbse_precond *p, const double *resid, const double *corr, const double *ene, long n,
                      double *loss, float *grad_host);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) with learning rate lr on the same
 * loss; *loss receives the loss before the step */
int fbse_precond_train_step(fbse_precond *p, const double *resid, const double *corr, const double *ene, long n,
                            double lr, double *loss);
/* Residual refinement of n Ritz pairs (psitot rows 0..n-1 on the device,
 * normalised, with eval / sigma on the host as fbse_ortho_diag_sigma returns
 * them).  Each of `steps` rounds forms r = (H - E) psi for the pairs with
 * sigma > tol, appends P(r) (p NULL: r itself) as new rows (each
 * normalised) and runs fbse_ortho_diag_sigma on the enlarged set.  psitot
 * must hold cap rows; a round appends at most cap - n rows (pairs in
 * increasing row order while they fit).  eval / sigma need cap doubles; *n_out
 * receives the final number of Ritz pairs. */
int fbse_refine(fbse_ctx *ctx, fbse_precond *p, double *psitot, long n, long cap, int steps, double tol,
                long *n_out, double *eval, double *sigma);
/* out[i] = H psi_i - ene[i] psi_i for n psitot states (device; ene host; H psi
 * in the context's precision, the difference in FP64); out must not alias
 * psitot.  The residual of calc_sigma_E (filter_mpi/energy.c:383-539). */
int fbse_residual(fbse_ctx *ctx, const double *psitot, long n, const double *ene, double *out);

/* ---- Bethe-Salpeter stage (bse_cplx/) --------------------------------------
 * States: psi_qp holds the quasiparticle basis as complex spinor states
 * (nspin*ngrid complex doubles each, device): holes at indices 0..n_h-1, the
 * electrons at lumo_idx..lumo_idx+n_e-1 (get_qp_basis, bse_cplx/basis.c:258).
 * Pair index ibs = (a - lumo_idx) * n_h + i; n_xton = n_h * n_e. */

/* init_elec_hole_kernel (bse_cplx/init.c:8-268): bare v(k) and screened W(k)
 * on the context's grid (ngrid complex doubles each, device), including the
 * 1/N of the FFT.  gx/gy/gz: grid coordinates (host); xmin..zmin: grid origin;
 * eps_*: the dielectric constants (epsX/epsY/epsZ of bse input.par). */
int fbse_bse_potentials(fbse_ctx *ctx, const double *gx, const double *gy, const double *gz, double xmin, double ymin,
                        double zmin, double eps_x, double eps_y, double eps_z, double *pot_bare,
                        double *pot_screened);

/* calc_eh_kernel_cplx (bse_cplx/coulomb.c:20-738): direct and exchange kernels,
 * n_xton x n_xton complex (device), lower triangle ibs >= jbs filled as the
 * reference fills it (the rest is zero). */
int fbse_bse_kernel(fbse_ctx *ctx, const double *psi_qp, long n_h, long n_e, long lumo_idx, const double *pot_bare,
                    const double *pot_screened, double *direct, double *exchange);

/* build_h0_mat + build_BSE_mat + bethe_salpeter (bse_cplx/mod_bse.c:54-148,
 * bethe-salpeter.c:7-350): H = diag(e_a - e_i) - (K^d + K^x), FP64 Hermitian
 * eigensolve on the GPU.  eval_qp_host: n_qp quasiparticle energies (host).
 * direct/exchange (device) are completed to full Hermitian matrices; xton_ene
 * (host, n_xton) ascending; coeff (device, n_xton x n_xton complex, row-major,
 * column j = exciton j); h/d/x/h0_exp (host, may be NULL): <H>, <K^d>, <K^x>,
 * <h0> per exciton -- the columns of exciton.dat. */
int fbse_bse_solve(fbse_ctx *ctx, const double *eval_qp_host, long n_qp, long n_h, long n_e, long lumo_idx,
                   double *direct, double *exchange, double *xton_ene, double *coeff, double *h_exp, double *d_exp,
                   double *x_exp, double *h0_exp);

/* calc_elec_dipole (bse_cplx/dipole.c:7-158): mu[(i * n_e + a)][3] complex
 * (host) = dv sum_{r,sigma} conj(psi_i) r psi_a. */
int fbse_bse_dipoles(fbse_ctx *ctx, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                     long n_h, long n_e, long lumo_idx, double *mu_host);

/* calc_eh_kernel_cplx of the real-valued BSE (bse_real/coulomb.c:20-705):
 * psi_qp holds real one-component states (ngrid doubles each, device; the
 * context has nspin = 1), direct / exchange are n_xton x n_xton doubles
 * (device), lower triangles as fbse_bse_kernel; K^d uses the real part of the
 * convolution (bse_real/hartree.c:31) and K^x the singlet factor 2
 * (exchange = -2 dv sum, bse_real/coulomb.c:568). */
int fbse_bse_kernel_real(fbse_ctx *ctx, const double *psi_qp, long n_h, long n_e, long lumo_idx,
                         const double *pot_bare, const double *pot_screened, double *direct, double *exchange);

/* calc_mag_dipole (bse_cplx/dipole.c:160-331): magnetic transition dipoles
 * m_ia = -(1/2) <i|L|a>, L = r x p with p = -i grad by FFT (l_operator,
 * p_operator, bse_cplx/ang_mom_operators.c:6-170), for the same basis and
 * coordinates as fbse_bse_dipoles.  m_host: [n_h][n_e][3] complex (host,
 * interleaved), pair index i * n_e + (a - lumo_idx). */
int fbse_bse_mag_dipoles(fbse_ctx *ctx, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                         long n_h, long n_e, long lumo_idx, double *m_host);

/* calc_qp_spin_mtrx + calc_qp_ang_mom_mtrx (bse_cplx/angular.c:7-690) for
 * complex spinor states, with the reference's conventions per block: holes
 * i, j < n_h at pair index i * n_h + j, electrons a, b at n_h^2 + (a - lumo)
 * * n_e + (b - lumo).  s_mom, l_mom: [n_h^2 + n_e^2][3] complex; l2_mom
 * (<L^2>) and ldots (<L.S>): [n_h^2 + n_e^2] complex (host, interleaved).
 * L is l_operator's -(r x p) with p by FFT (as fbse_bse_mag_dipoles), L^2 is
 * sum_d L_d L_d; the L quantities are computed for j >= i and the rest filled
 * by Hermitian conjugation, as the reference does. */
int fbse_bse_qp_ang_mom(fbse_ctx *ctx, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                        long n_h, long n_e, long lumo_idx, double *s_mom, double *l_mom, double *l2_mom,
                        double *ldots);

/* calc_optical_exc (bse_cplx/optical.c:6-99), electric part: exciton transition
 * dipoles mu_j = sum_ibs coeff[ibs][j] mu_(i(ibs), a(ibs)).  coeff: device, as
 * fbse_bse_solve returns it; mu_pairs_host: fbse_bse_dipoles' output;
 * mu_xton_host: [n_xton][3] complex (host); the same sum of the magnetic pair
 * dipoles (fbse_bse_mag_dipoles) gives M.dat.  OS.dat's columns follow from it:
 * |mu_j|, E_j, (2/3) E_j |mu_j|^2. */
int fbse_bse_optical(fbse_ctx *ctx, const double *coeff, const double *mu_pairs_host, long n_h, long n_e,
                     double *mu_xton_host);

/* ---- setup on the GPU -----------------------------------------------------
 * build_local_pot (filter_mpi/init.c:481-703) for short-ranged tables
 * (no strain, no cubic/ortho interpolation, no LSD, no long range):
 * pot[jxyz] = sum_a v_{atype[a]}(|r - R_a|) with interpolate()'s linear rule
 * (filter_mpi/interpolate.c:5-49).  gx/gy/gz: grid coordinates (host, nx/ny/nz
 * each); coords: [natoms][3] (host); tables: type t occupies rows
 * [tab_off[t], tab_off[t] + tab_len[t]) of tab_r / tab_v (host).  pot: host,
 * ngrid doubles.  Uses the current CUDA device; no context needed. */
int fbse_build_local_pot(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz,
                         long natoms, const double *coords, const int *atype, int ntypes, const double *tab_r,
                         const double *tab_v, const long *tab_off, const long *tab_len, double *pot);

/* init_NL_projectors (filter_mpi/init.c:848-1135, body 508-589): for each of
 * nat projector atoms (xyz [nat][3], host) the grid points with
 * r^2 < rcut2 in jz, jy, jx order, with Y_1m under the reference's EPSDX
 * shifts (init.c:1002-1040) and the radial projectors interpolated at r
 * (interpolate(), linear): so_tab [nproj][1024] (PROJ_LEN) scaled per atom
 * by sqrt(so_par[a]), nl_tab [nat][nproj][1024] (either may be NULL: zeros).
 * Computed on the current CUDA device (one CTA per atom, no fused multiply-add,
 * so the table is bit-identical to the plain IEEE evaluation); returns host
 * arrays allocated with malloc (the caller frees them): nl[nat], and with
 * row stride *npts (the largest count) jxyz[nat*npts], y1[nat*npts][6]
 * (Y_1m, m = 0..2, re/im), so_p and nl_p [nat*npts][nproj] -- the arrays of
 * fbse_proj_desc.  No context needed. */
int fbse_build_nlc(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz, long nat,
                   const double *xyz, const double *so_par, const double *so_tab, const double *nl_tab, int nproj,
                   double rcut2, long *npts, long **nl, int **jxyz, double **y1, double **so_p, double **nl_p);

/* ---- host-side helpers (no device work) --------------------------------- */

/* samp_points_ashkenazy on [-2, 2] (filter_mpi/coeff.c:227-293): writes
 * ncheby Leja-type nodes to zn (host) and returns the capacity estimate. */
double fbse_samp_points(long ncheby, double *zn);

/* gen_newton_coeff (filter_mpi/coeff.c:8-118): an is [m][ncheby] complex
 * (host, interleaved); dt = (ncheby / (2.5 dE))^2 as filter_mpi/mod_filter.c:114. */
int fbse_newton_coeff(long ncheby, long m, const double *zn, const double *targets, double vmin, double de,
                      double dt, double *an);

/* ran_nrc (filter_mpi/rand.c:22-62): the reference's generator with its
 * process-wide state.  Returns one U(0,1) draw and advances *seed. */
double fbse_ran(long *seed);

/* init_filter_states (filter_mpi/init.c:1138-1255) without file output:
 * n_filters random starts into psitot states (host, nspin*ngrid*complex_idx
 * doubles each), each spin block drawn and normalised on its own.  Returns the
 * advanced seed; seeds_out (may be NULL) receives the n_filters*nspin seeds the
 * reference prints to seed-<rank>.dat. */
long fbse_init_filter_states(double *psitot, long n_filters, long ngrid, int nspin, int is_complex, double dv,
                             long seed, long *seeds_out);

#ifdef __cplusplus
}
#endif
#endif /* FBSE_H */

/*
 * lqg.h - C ABI of the GB300 per-chunk QMLE engine (lyspeq's hot path).
 *
 * lyspeq has no C ABI of its own: the per-chunk path is the C++ API
 *   Chunk::Chunk(const qio::QSOFile&, int i1, int i2)       core/chunk_estimate.cpp:141-167
 *   Chunk::oneQSOiteration(ps, dbt_sum, fisher_sum)           core/chunk_estimate.cpp:837-914
 *   OneQSOEstimate::oneQSOiteration(...)                      core/one_qso_estimate.cpp:176-197
 *   OneDQuadraticPowerEstimate::iterate()                     core/quadratic_estimate.cpp:398-546
 *   OneDQuadraticPowerEstimate::invertTotalFisherMatrix()     core/quadratic_estimate.cpp:261-288
 *   OneDQuadraticPowerEstimate::computePowerSpectrumEstimates() :290-318
 * The entry points below are what a binding of that API binds: plain
 * pointers and sizes, integer status codes, no C++ or torch types.  The C++
 * facade in include/lyspeq_api.hpp keeps the reference's class
 * names on top of them.
 *
 * Conventions
 *  - All arrays are row-major IEEE double unless noted.
 *  - Every function returns LQG_OK (0) or a negative LQG_ERR_* code; the
 *    message of the last error of a context is lqg_last_error(ctx).
 *  - A chunk that the reference would reject or skip gets a positive
 *    LQG_CHUNK_* status and contributes nothing, as the reference logs and
 *    drops it (core/one_qso_estimate.cpp:117-124, chunk_estimate.cpp:905-913).
 *  - One context per host thread.  Work is enqueued on the context's CUDA
 *    stream; functions that return host data synchronise that stream.
 */
#ifndef LQG_H
#define LQG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3: the tuning table entries of lqg_tuning_get / lqg_tuning_set carry
 * LQG_TUNING_FIELDS (5) ints */
#define LQG_ABI_VERSION 3

/* status codes */
#define LQG_OK 0
#define LQG_ERR_ARG -1          /* invalid argument */
#define LQG_ERR_CUDA -2         /* CUDA runtime error */
#define LQG_ERR_NOMEM -3        /* device or host allocation failed */
#define LQG_ERR_STATE -4        /* call out of order (e.g. no batch) */
#define LQG_ERR_TIMEOUT -5      /* a bounded device wait gave up */
#define LQG_ERR_UNSUPPORTED -6  /* option not implemented on this path */
#define LQG_ERR_SINGULAR -7     /* global Fisher matrix could not be inverted */
#define LQG_ERR_TOO_LARGE -8    /* size beyond a fixed limit of the entry point */

/* per-chunk status */
#define LQG_CHUNK_OK 0
#define LQG_CHUNK_SHORT 1       /* Chunk::_copyQSOFile short chunk, chunk_estimate.cpp:173-187 */
#define LQG_CHUNK_NO_TABLE 2    /* no (R, dv) table, chunk_estimate.cpp:197-206 */
#define LQG_CHUNK_EMPTY 3       /* all pixels masked (QSOFile::_cutMaskedBoundary) */
#define LQG_CHUNK_OUT_OF_RANGE 4 /* no redshift bin touched */
#define LQG_CHUNK_NOT_SPD 5     /* covariance not positive definite ("not invertable") */
#define LQG_CHUNK_BAD_INPUT 6   /* non-finite pixel values */
#define LQG_CHUNK_TOO_LARGE 7   /* more pixels than the engine's maximum */
#define LQG_CHUNK_TIMEOUT 8     /* a bounded device wait gave up; results dropped */
#define LQG_CHUNK_INDEX_CHECK 9 /* self-checking build only: an index would have left
                                   its buffer; the chunk was skipped */

/* arithmetic of the per-chunk products */
#define LQG_PRECISION_FP64 0    /* everything in IEEE binary64 */
#define LQG_PRECISION_MIXED 1   /* df64 factorisation to W = P L^-1 D (C^-1 = W^T W, P the
                                   continuum projector); B_k = W Q_k W^T on tensor cores as
                                   fp16 hi/lo split products (3 terms, fp32 accumulation),
                                   traces F_ij = <B_i, B_j> over B's upper triangle, fp64
                                   reduction of partial sums */
#define LQG_PRECISION_MIXED_AUTO 3 /* mixed, with the form (whitened or direct), the products'
                                   drain interval and the Gram's K split chosen per padded
                                   chunk size by the context's table (lqg_autotune,
                                   lqg_tuning_set); MIXED's choices where it has none */
#define LQG_PRECISION_MIXED_DIRECT 2 /* as MIXED but with the direct products A_k = C^-1 Q_k
                                   and F_ij = <A_i^T, A_j>: cheaper with continuum
                                   marginalisation, less accurate at high signal to noise
                                   (its errors grow with the ratio of signal to noise
                                   power at low k) */

typedef struct lqg_ctx lqg_ctx;

/* k and z binning: bins::setUpBins, core/global_numbers.cpp:209-251 */
typedef struct {
    int nk;                     /* NUMBER_OF_K_BANDS */
    int nz;                     /* NUMBER_OF_Z_BINS */
    const double *k_edges;      /* KBAND_EDGES [nk + 1] */
    const double *z_centers;    /* ZBIN_CENTERS [nz] */
    double z_bin_width;         /* Z_BIN_WIDTH */
    int triangular;             /* 1: RedshiftBinningMethod 1, 0: top hat */
} lqg_bins;

/* S/Q lookup tables: SQLookupTable, core/sq_table.cpp:148-175, 325-368.
 * All tables share the v grid [0, v_length] with nv points and the z grid
 * [z_c0 - dz, z_c0 - dz + dz (nz + 1)] with nzp points. */
typedef struct {
    int n_tables;               /* number of (R, dv) pairs (FileNameRList) */
    const int *r_fwhm;          /* [n_tables] spectrograph resolution R */
    const double *dv;           /* [n_tables] pixel width, km/s */
    int nv;                     /* NumberVPoints */
    double v_length;            /* VelocityLength */
    int nzp;                    /* NumberZPoints */
    const double *deriv;        /* [n_tables][nk][nv]   Q_k(v) */
    const double *signal;       /* [n_tables][nv][nzp]  S(z, v), z fastest; NULL if
                                   turn_off_sfid */
} lqg_tables;

typedef struct {
    double max_forest_length;   /* MaximumForestLength (already divided by the
                                   DynamicChunkNumber, i.e. MAX_FOREST_LENGTH_V) */
    double max_mean_pixel_size; /* MaximumMeanPixelSize */
    int cont_logl_order;        /* ContinuumLogLambdaMargOrder */
    int cont_l_order;           /* ContinuumLambdaMargOrder */
    int turn_off_sfid;          /* TurnOffBaseline > 0 */
    int skip_fisher;            /* PrecomputedFisher given: Fisher not computed */
    size_t workspace_bytes;     /* device workspace cap; 0 = 60% of free memory */
    int smooth_noise_weights;   /* SmoothNoiseWeights: < 0 off; 0 the mean noise;
                                   > 0 Gaussian sigma in pixels.  C is built with the
                                   smoothed ivar (Chunk::setInvertCovarianceMatrix,
                                   core/chunk_estimate.cpp:685-691), N of the bias
                                   traces keeps the raw ivar (:767-786) */
    int redshift_growth_on;     /* RedshiftGrowthOn > 0: Q_k scaled by
                                   ((1 + z_ij) / (1 + z_m))^B
                                   (_scaleDerivativesWithRedshiftGrowth, :539-573) */
    double fid_redshift_power;  /* B of the fiducial PD13 (FiducialRedshiftPower) */
} lqg_opts;

/* Create a context on CUDA device `device`; bins and tables are copied.
 * Replaces SQLookupTable::readTables + glmemory::allocMemory. */
int lqg_ctx_create(lqg_ctx **ctx, const lqg_bins *bins, const lqg_tables *tables,
                   const lqg_opts *opts, int device);
int lqg_ctx_destroy(lqg_ctx *ctx);
const char *lqg_last_error(const lqg_ctx *ctx);
int lqg_abi_version(void);

/* Add chunks, each given as the pixel range of one spectrum after lyspeq's
 * reading and cleaning (qio::QSOFile after cutBoundary / maskOutliers and
 * OneQSOEstimate::decideIndices).  lambda is the observed wavelength in
 * Angstrom, ivar the inverse variance (0 = masked).  For each chunk this does
 * what Chunk::Chunk does (core/chunk_estimate.cpp:141-257): trims masked
 * edges, takes the median dv, applies the short-chunk rule, finds the table,
 * KBIN_UPP, the redshift bins, N_Q_MATRICES and fisher_index_start.
 * status_out[n_chunks] receives LQG_CHUNK_* per chunk; rejected chunks are
 * kept out of the batch.  Pixel data are copied to the device. */
int lqg_batch_add(lqg_ctx *ctx, int n_chunks, const int64_t *offsets,
                  const double *lambda, const double *delta, const double *ivar,
                  const int *r_fwhm, int *status_out);
/* Add chunks that carry a resolution matrix (UseResoMatrix): lyspeq then
 * evaluates S and the band derivatives Q_k on the matrix's grid and uses
 * R S R^T and R Q_k R^T (Chunk::_setFiducialSignalMatrix, _setQiMatrix,
 * core/chunk_estimate.cpp:400-480, with Resolution::sandwich,
 * mathtools/matrix_helper.cpp:815-821, 877-903).  Q_k is the analytic band
 * (dk / pi) cos(k_c v) sinc(dk v / 2) (:444-454), S comes from table 0
 * (RES_INDEX = 0, :189-193); the redshift weights apply after the sandwich.
 * lambda, delta, ivar and offsets are as for lqg_batch_add.  resomat holds
 * nelem doubles per pixel, aligned with lambda:
 *  - oversampling > 0: the pixel's row of the oversampled matrix
 *    (Resolution::oversample, mathtools/matrix_helper.cpp:1008-1073, i.e. the
 *    output of lqg_resomat_oversample), nelem = 2 (ndiags / 2) oversampling + 1;
 *    the row's weights sit at grid points i * oversampling + a of the grid
 *    lambda_0 / LYA + (p - nelem / 2) dlambda / LYA / oversampling, dlambda the
 *    chunk's median pixel width (core/chunk_estimate.cpp:927-938);
 *  - oversampling <= 0: the diagonal matrix, the pixel's column on each of the
 *    nelem = ndiags diagonals (entry d is DiaMatrix values[d][pixel], diagonal
 *    d holding offset ndiags / 2 - d); S and Q_k stay on the pixel grid.
 * Limits of the engine's tiles: nelem <= 48 and 31 * max(oversampling, 1) +
 * nelem <= 128 (else LQG_ERR_UNSUPPORTED).  No table lookup by (R, dv) is
 * made; every other rule of lqg_batch_add applies. */
int lqg_batch_add_reso(lqg_ctx *ctx, int n_chunks, const int64_t *offsets,
                       const double *lambda, const double *delta, const double *ivar,
                       int oversampling, int nelem, const double *resomat, int *status_out);
/* Resolution-matrix preprocessing of one spectrum (before chunking, as
 * OneQSOEstimate::_readQsoFile does, core/one_qso_estimate.cpp:75-89).
 * values: DiaMatrix layout values[ndiags][n] (diagonal d holds offset
 * ndiags / 2 - d, its entry of column c at [d][c]; rows at the spectrum's
 * edges mirror their missing entries, DiaMatrix::_getRowIndices).
 * lqg_resomat_deconvolve: DiaMatrix::deconvolve(m) in place
 *   (mathtools/matrix_helper.cpp:653-682, real_field.cpp:95-110).
 * lqg_resomat_oversample: Resolution::oversample(osamp, dlambda)
 *   (mathtools/matrix_helper.cpp:1008-1073); rows[n][2 (ndiags / 2) osamp + 1].
 * Host only: neither touches the device nor needs a context. */
int lqg_resomat_deconvolve(int n, int ndiags, double *values, double m);
int lqg_resomat_oversample(int n, int ndiags, const double *values, int osamp, double dlambda,
                           double *rows);
/* Smoother::smoothIvar (mathtools/smoother.cpp:170-218) for one chunk's ivar
 * of n pixels: sigmapix = SmoothNoiseWeights (0: the mean ivar, > 0: Gaussian
 * filter of 51 taps with that sigma on the noise variance), masked and
 * high-noise pixels keep their ivar.  The reference's padding is kept as it
 * is: its right-hand pad lands on the last 25 pixels and leaves the 25 pad
 * cells beyond them at 0, so unless the last pixel is masked the last 25
 * pixels come out with ivar 0.  Host only; out may not alias ivar. */
int lqg_smooth_ivar(int n, const double *ivar, int sigmapix, double *out);
/* Smoother::smooth1D (mathtools/smoother.cpp:144-168) on each of the ndiags
 * diagonals of a DiaMatrix values[ndiags][n], in place: what
 * OneQSOEstimate::_readQsoFile does before deconvolution when
 * SmoothResolutionMatrix > 0 and SmoothNoiseWeights >= 0
 * (core/one_qso_estimate.cpp:79-81).  sigmapix = SmoothNoiseWeights; the
 * padding is the one lqg_smooth_ivar describes.  Host only. */
int lqg_resomat_smooth(int n, int ndiags, double *values, int sigmapix);
/* SQ lookup tables on the GPU: SQLookupTable::computeTables
 * (core/sq_table.cpp:201-323, CreateSQLookUpTable), for n_tables (R, dv)
 * pairs on the grids lqg_tables describes (nv points over [0, v_length], nzp
 * redshift points over [z_c0 - dz, z_c0 - dz + dz (nz + 1)]).
 *   deriv  [n_tables][nk][nv]: Q_k(v) = (1/pi) int_{k1}^{k2} W^2(k) cos(k v) dk,
 *          W(k) = sinc(k dv / 2) exp(-k^2 R^2 / 2), R = c / R_fwhm / 2.35482
 *          (q_matrix_integrand, core/fiducial_cosmology.cpp:305-331), by
 *          composite 8-point Gauss-Legendre quadrature on panels of width
 *          <= 3 / v_length (the reference integrates with GSL QAWO);
 *   signal [n_tables][nv][nzp] (z fastest), if with_signal: the reference's
 *          own discretisation, the real inverse FFT of W^2 P_fid(k, z) on the
 *          grid of RealField(2^(ceil(log2(4 nv)) + 1), dv_table / 2) sampled at
 *          every second point (core/sq_table.cpp:222-228, 286-310).
 * fid: the six PD13 parameters A, n, alpha, B, beta, lambda
 * (core/fiducial_cosmology.cpp:268-282).  FP64; synchronous; allocates and
 * frees its own device memory on `device`; host arrays in and out. */
int lqg_tables_generate(const lqg_bins *bins, int n_tables, const int *r_fwhm, const double *dv,
                        int nv, double v_length, int nzp, const double *fid, int with_signal,
                        double *deriv, double *signal, int device);
int lqg_batch_clear(lqg_ctx *ctx);
int lqg_batch_size(const lqg_ctx *ctx);

/* Metadata of batch chunk i (in insertion order of accepted chunks):
 * info[0..7] = n, fisher_index_start, n_q_matrices, kbin_upp, res_index,
 * zbin_low, zbin_upp, input index (position in the lqg_batch_add call). */
int lqg_chunk_info(const lqg_ctx *ctx, int i, int *info);

/* What lqg_batch_add (resomat NULL) or lqg_batch_add_reso (resomat, with its
 * oversampling and nelem; r_fwhm may then be NULL) would make of each chunk,
 * without a context or a GPU: Chunk::Chunk's checks and numbers
 * (core/chunk_estimate.cpp:141-257) for the same arguments, from the same
 * code.  status_out[n_chunks] gets LQG_CHUNK_* and
 * info_out[8 * n_chunks] the lqg_chunk_info fields of each accepted chunk
 * (input index = its position in this call; zeros for a rejected one).  Of
 * tables only n_tables, r_fwhm and dv are read (deriv and signal may be
 * NULL).  A driver that shards chunks over contexts or processes can cost
 * them first, as OneQSOEstimate::getComputeTimeEst does for lyspeq's load
 * balancing (core/one_qso_estimate.cpp:132-174): n pixels and
 * (n_q_matrices / NUMBER_OF_K_BANDS) * kbin_upp stored matrices. */
int lqg_chunk_plan(const lqg_bins *bins, const lqg_tables *tables, const lqg_opts *opts, int n_chunks,
                   const int64_t *offsets, const double *lambda, const double *delta, const double *ivar,
                   const int *r_fwhm, int oversampling, int nelem, const double *resomat, int *status_out,
                   int *info_out);

/* One Newton-Raphson iteration over the whole batch: for every chunk build
 * S and Q_k from the tables, C = S + sum theta_k Q_k + N, invert, continuum
 * marginalisation, then d_k, b_k, t_k and the chunk Fisher matrix, summed
 * into the global accumulators exactly as Chunk::oneQSOiteration does
 * (core/chunk_estimate.cpp:837-914): F upper triangle, NOT halved.
 * theta: TOTAL_KZ_BINS values (powerspectra_fits) or NULL for zeros.
 * Runs on the context stream and returns when the iteration has finished;
 * results stay on the device. */
int lqg_nr_iteration(lqg_ctx *ctx, const double *theta, int precision);

/* The same iteration, asynchronous: ordered after the work already enqueued
 * on `stream` (a cudaStream_t; NULL: no ordering), and work enqueued on
 * `stream` afterwards waits for it; returns once the launches are enqueued
 * (planning, workspace allocation and the batch upload happen on the host
 * before that, and the first iteration of a batch may wait for them).  theta
 * is copied before the call returns.  lqg_sync, lqg_download,
 * lqg_chunk_result, the bootstraps and the next iteration complete it (the
 * chunk statuses, the index checks of the self-checking build and the phase
 * timings are read then).  Replaces the per-chunk loop of
 * OneDQuadraticPowerEstimate::iterate (core/quadratic_estimate.cpp:438-475),
 * with a stream argument the reference does not have. */
int lqg_nr_iteration_async(lqg_ctx *ctx, const double *theta, int precision, void *stream);
/* Waits for the iteration lqg_nr_iteration_async enqueued; returns its status. */
int lqg_sync(lqg_ctx *ctx);

/* Autotuner of the mixed path's launch plan (no counterpart in the reference,
 * whose only scheduling input is its cost model, core/chunk_estimate.cpp:
 * 297-382).  For every padded chunk size (ld, a multiple of 64) in the
 * current batch it runs the FP64 path on up to 4 chunks of that size and the
 * mixed path on the same chunks with each candidate plan: whitened or direct
 * form (flags & 1), hi*hi drain interval of the products 4, 8 or 16 K blocks
 * (flags & 2); a candidate is kept when every per-chunk d, b, t (normwise)
 * and Fisher element (normalised by sqrt(F_ii F_jj)) of the sample is within
 * 0.8 max_rel_err of the FP64 results (room for the chunks not sampled).
 * The kept candidates are timed on up to max_chunks chunks of that size
 * (device time of an iteration over them) and the fastest is stored; then the
 * Gram's K elements per split, 16384, 32768 or 65536 (flags & 4), by time;
 * with flags & 8 before that, the products on CTA pairs (tcgen05 cta_group::2,
 * 256 x 128 tiles), kept when within the bound and faster.
 * LQG_PRECISION_MIXED_AUTO iterations use the table; the results of the
 * batch's last iteration are invalidated.  flags = 0 means all (15);
 * max_rel_err <= 0 means 1e-5; max_chunks <= 0 means 48. */
int lqg_autotune(lqg_ctx *ctx, double max_rel_err, int max_chunks, int flags);
/* The table, one entry of LQG_TUNING_FIELDS ints per padded size: ld, form
 * (1 whitened, 0 direct), drain interval, Gram K per split, CTA-pair products
 * (1) or single-CTA (0).  lqg_tuning_get returns the number of entries
 * (writing at most n); lqg_tuning_set replaces the table. */
#define LQG_TUNING_FIELDS 5
int lqg_tuning_get(const lqg_ctx *ctx, int *entries, int n);
int lqg_tuning_set(lqg_ctx *ctx, const int *entries, int n);

/* Copy the accumulated results of the last iteration to host memory (any
 * pointer may be NULL): d, b, t [nkz] and fisher [nkz * nkz] (upper, not
 * halved) and chunk_status [batch size].  Synchronises the stream. */
int lqg_download(lqg_ctx *ctx, double *d, double *b, double *t, double *fisher,
                 int *chunk_status);

/* Per-chunk results of the last iteration for batch chunk i: d, b, t
 * [n_q_matrices] and fisher [n_q * n_q] (upper triangle filled), the
 * Chunk::dbt_estimate_before_fisher_vector / fisher_matrix members. */
int lqg_chunk_result(lqg_ctx *ctx, int i, double *d, double *b, double *t, double *fisher);

/* Global Newton-Raphson update, OneDQuadraticPowerEstimate::iterate tail
 * (core/quadratic_estimate.cpp:456-457, 261-318, mathtools/matrix_helper.cpp:330-358):
 * F <- F/2 symmetrised; zero-diagonal bins are set to 1 for the inversion;
 * if the singular values of F show a jump > 8 the damped solver
 * (F^2 + s I)^-1 F is used; theta = 1/2 F_solver (d - b - t).
 * In: fisher_sum [nkz^2] (upper, unhalved), dbt [3][nkz].
 * Out (any may be NULL): fisher [nkz^2] halved and symmetric, solver and
 * inverse [nkz^2], weighted [3][nkz] (0.5 F_solver d, b, t), theta [nkz],
 * damped (0/1), dof, damp.  FP64, O(nkz^3), on the host CPU. */
int lqg_fisher_solve(lqg_ctx *ctx, const double *fisher_sum, const double *dbt,
                     double *fisher, double *solver, double *inverse, double *weighted,
                     double *theta, int *damped, int *dof, double *damp);

/* lqg_fisher_solve without a context, for nkz (k, z) bins: the same update
 * for a caller that holds only the sums (the rank that reduced the other
 * processes' sums).  Host only: needs no GPU. */
int lqg_fisher_solve_n(int nkz, const double *fisher_sum, const double *dbt, double *fisher,
                       double *solver, double *inverse, double *weighted, double *theta,
                       int *damped, int *dof, double *damp);

/* Device time (ms) of the phases of the last iteration, CUDA events on the
 * context stream, summed over the size-bucketed waves: [0] S and C build,
 * [1] FP64 factorisation, inverse and marginalisation, [2] Q_k build,
 * [3] C^-1 Q_k products, [4] Fisher / bias traces, [5] per-chunk reduction,
 * [6] global accumulation, [7] whole iteration.  Returns the number written. */
int lqg_last_timings(const lqg_ctx *ctx, double *ms, int n);

/* Poisson bootstrap over spectra after an iteration, lyspeq's FastBootstrap
 * (PoissonBootstrapper::_fastBootstrap and _meanBootstrap, core/bootstrapper.hpp,
 * with OneQSOEstimate::collapseBootstrap, core/one_qso_estimate.cpp:200-238).
 * The spectra are consecutive ranges of the batch's chunks: spectrum q owns
 * batch chunks [qso_offsets[q], qso_offsets[q+1]) (ranges may be empty, for a
 * spectrum all of whose chunks were rejected; it still takes its draws).
 * theta_q = sum of its chunks' d - b - t from the last lqg_nr_iteration;
 * realization x_b = sum_q p_qb theta_q with p_qb ~ Poisson(1) drawn on the host
 * by std::mt19937_64 seeded with `seed` (the reference seeds with the MPI rank)
 * and std::poisson_distribution, nboots draws per spectrum in order.
 * Out (any may be NULL): mean [nkz] of the realizations (not normalised, as
 * the reference writes it), fisher_cov [nkz^2] = covariance / 4, cov [nkz^2] =
 * F^-1 (covariance / 4) F^-T with F^-1 = solver_invfisher (the solver matrix of
 * lqg_fisher_solve; required for cov), realizations [nboots][nkz].  FP64 on
 * the device; synchronous. */
int lqg_bootstrap(lqg_ctx *ctx, int n_qso, const int *qso_offsets, int nboots, unsigned long long seed,
                  const double *solver_invfisher, double *mean, double *cov, double *fisher_cov,
                  double *realizations);
/* The complete bootstrap (FastBootstrap 0, PoissonBootstrapper::_oneBoot and
 * _meanBootstrap, core/bootstrapper.hpp:126-135, 217-257, 291-345): realization
 * b draws one coefficient per spectrum (spectra in order, realizations in
 * order) and solves F_b x_b = r_b with F_b = sum_q p_bq F_q and r_b = sum_q
 * p_bq theta_q, F_q the upper sum of the spectrum's chunk Fisher matrices
 * (collapseBootstrap, core/one_qso_estimate.cpp:225-235), by Cholesky with
 * zero-diagonal bins held out (LAPACKE_safeSolveCho,
 * mathtools/matrix_helper.cpp:385-396).  Realizations whose F_b is not
 * positive definite are dropped; the valid ones fill the slots of
 * realizations [nboots][nkz] in order (a failed last realization leaves its
 * unsolved sum in the next slot, zeros after it, as the reference's buffer
 * holds them), *n_valid receives their number, mean [nkz] = sum of all slots /
 * n_valid and cov [nkz^2] = sum over all slots of (x - mean)(x - mean)^T /
 * (n_valid - 1).  nkz <= 1023.  FP64 on the device; synchronous;
 * LQG_ERR_STATE when fewer than two realizations are valid. */
int lqg_bootstrap_complete(lqg_ctx *ctx, int n_qso, const int *qso_offsets, int nboots,
                           unsigned long long seed, double *mean, double *cov, double *realizations,
                           int *n_valid);
/* The Poisson coefficients either bootstrap draws, p[q * nboots + b]: host
 * only (per_realization = 0: FastBootstrap's order, 1: the complete
 * bootstrap's). */
int lqg_bootstrap_coefficients(int n_qso, int nboots, unsigned long long seed, int per_realization,
                               unsigned char *p);
/* Number of kernel launches the last lqg_nr_iteration enqueued. */
int lqg_last_launch_count(const lqg_ctx *ctx);
/* Number of size-bucketed waves of the last iteration: each phase-B kernel
 * (Q build, products, traces, reduction) is launched once per wave. */
int lqg_last_wave_count(const lqg_ctx *ctx);
/* Bytes the last iteration copied from host to device: the batch's pixel
 * arrays and chunk metadata when the batch changed since the previous
 * iteration, theta, and the launch plan's descriptors. */
int lqg_last_h2d_bytes(const lqg_ctx *ctx, int64_t *bytes);

/* Limit of every wait inside the tensor-core kernels of later iterations
 * (seconds, at most 60; 0 restores the default of 2 s).  A wait that runs out
 * makes its CTA stop, drain its own copies and MMAs, free its tensor memory
 * and mark its chunks LQG_CHUNK_TIMEOUT; the iteration returns and the context
 * stays usable.  No counterpart in the reference (its loops have no device
 * waits); tests use a tiny limit to exercise that path without a fault. */
int lqg_set_wait_limit(lqg_ctx *ctx, double seconds);

/* on = 1: the results of later iterations are those of lyspeq built with
 * FISHER_OPTIMIZATION (./configure --enable-fisher-optimization): of each
 * chunk's Fisher matrix only the pairs of local kz indices i <= j with
 * j - i <= 5 or |j - i - NUMBER_OF_K_BANDS| <= 2 are kept, the others are 0
 * (Chunk::oneQSOiteration, core/chunk_estimate.cpp:823-827), in the per-chunk
 * results, the global sum and the bootstraps alike.  on = 0 (the default):
 * full matrices.  LQG_ERR_ARG for any other value. */
int lqg_set_fisher_optimization(lqg_ctx *ctx, int on);

/* Measured FP64 (DFMA) throughput of device `device` in TFLOP/s: independent
 * FMA chains on every SM, best of five timed launches.  The denominator of the
 * FP64 kernels' rooflines; no counterpart in the reference. */
int lqg_probe_fp64_rate(int device, double *tflops);

/* Factorisation of one chunk's covariance without allocating: no counterpart
 * in the reference (there it is part of Chunk::setInvertCovarianceMatrix,
 * _addMarginalizations and computePSbeforeFvector, core/chunk_estimate.cpp:
 * 668-719, 576-665, 746-750, which use the glmemory pool).  For callers that
 * cannot let a library call cudaMalloc/cudaFree (which may synchronise the
 * device) or allocate from their memory pool: all buffers are the caller's
 * device memory, and the only scratch is a fixed 2 MiB static device array per
 * device.  Enqueued on `stream` (a cudaStream_t; NULL = legacy default stream);
 * nothing is copied from or to the host and nothing is synchronised.
 *   n, ld       pixels and leading dimension: ld % 64 == 0, n <= ld <= 4096
 *               (larger: LQG_ERR_TOO_LARGE, checked before any device work)
 *   cov         in: C = S + sum theta_k Q_k, symmetric n x n in an ld x ld
 *               row-major buffer (padding ignored); out: C^-1 (ld x ld, zero
 *               padding; masked pixels give zero rows and columns)
 *   wave        lambda / lambda_Lya per pixel (the marginalisation templates)
 *   delta, ivar flux contrast and inverse variance per pixel
 *   cont_*      ContinuumLogLambdaMargOrder / ContinuumLambdaMargOrder
 *               (at most 4 template vectors, else LQG_ERR_UNSUPPORTED)
 *   y           out: C^-1 delta, ld values
 *   status      device int, out: LQG_CHUNK_OK or LQG_CHUNK_NOT_SPD (and, in the
 *               self-checking build, LQG_CHUNK_INDEX_CHECK).  The call sets it to
 *               LQG_CHUNK_OK first: nothing needs to start at zero.
 * The static scratch is shared by every call on a device: two calls in flight
 * at the same time (other streams, other host threads) race on it and give
 * wrong results; order them (one stream, or events).  Every call looks up
 * the scratch address on the current device (no allocation); the first call
 * on each device also sets a kernel attribute, so make it before any stream
 * capture.  That attribute is kept for the life of the process: resetting a
 * device (cudaDeviceReset) while this library is loaded is not supported. */
int lqg_factor_noalloc(int n, int ld, double *cov, const double *wave, const double *delta,
                       const double *ivar, int cont_logl_order, int cont_l_order, double *y,
                       int *status, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* LQG_H */

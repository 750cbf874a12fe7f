/*
 * cravagpu.h -- C-ABI of the GB300 (sm_103a) FFT-domain Bayesian AVO
 * inversion library (libcravagpu.so).
 *
 * Every entry point takes plain pointers and sizes, returns CG_OK (0) or a
 * negative status (cg_last_error() gives the text) and never exits the
 * process.  Buffers follow the reference FFTGrid in-place layout
 * (src/fftgrid.cpp:40-70): a padded cube of nxp*nyp*nzp cells is stored as
 * rnxp*nyp*nzp floats with rnxp = 2*(nxp/2+1), x fastest; after a forward
 * transform the same memory holds cnxp*nyp*nzp interleaved complex floats
 * (cnxp = nxp/2+1), bin (i,j,k) at i + cnxp*j + cnxp*nyp*k.
 *
 * Unless an entry point's name ends in _host, pointers are device pointers
 * and work is queued on `stream` (a cudaStream_t, NULL = legacy default
 * stream) without synchronising.  _host variants take host memory, copy it to
 * the device, run, copy the results back and synchronise.
 *
 * Paths in comments are relative to the CRAVA source tree.
 */
#ifndef CRAVAGPU_H
#define CRAVAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define CG_OK 0
#define CG_ERR_ARG (-1)         /* bad argument (size, pointer, type) */
#define CG_ERR_CUDA (-2)        /* CUDA runtime error */
#define CG_ERR_UNSUPPORTED (-3) /* valid input the library does not handle */
#define CG_ERR_STATE (-4)       /* call out of order (e.g. handle not set up) */

/* ---- cube types: the values of FFTGrid::gridTypes (src/fftgrid.h:199) -- */
#define CG_CTMISSING 0
#define CG_DATA 1
#define CG_PARAMETER 2
#define CG_COVARIANCE 3
#define CG_VELOCITY 4
#define CG_OPERATOR 5

/* ---- precision modes of the fused per-bin posterior ------------------- */
#define CG_PREC_FP32 0  /* all FP32 */
#define CG_PREC_MIXED 1 /* FP32 bulk, FP64 Cholesky/solves + 1 refinement step on flagged bins */
#define CG_PREC_FP64 2  /* all FP64 (accuracy reference on the GPU) */

/* Text of the last error raised on the calling thread. */
const char *cg_last_error(void);
/* Library version, e.g. 100 = 0.1.0. */
int cg_version(void);
/* How many memory allocations (device, pinned host, memory pools) the
 * library has made in this process: a diagnostic for callers that must know
 * whether a call allocated (no reference counterpart). */
long cg_alloc_calls(void);
/* Largest transform length supported along one axis. */
int cg_fft_max_length(void);

/* Launch tracing (the GPU counterpart of the reference's Timings phase timers,
 * src/timings.h:11-30).  When enabled, every library launch records CUDA
 * events on its own stream and its algorithmic HBM bytes (the bytes the
 * kernel must move at minimum).  cg_trace_collect synchronises and returns
 * the number of distinct kernels; cg_trace_entry reads one aggregate. */
int cg_trace_enable(int on);
int cg_trace_collect(void);
int cg_trace_entry(int index, char *name, int name_len, long *launches, double *ms_total, double *bytes_total);

/* Device fault word of the current device: kernels that wait on an mbarrier
 * (the TMA-fed column pass) give up after a bounded number of polls, set this
 * word and return instead of hanging.  Copies it to *flag (0 = no wait gave
 * up) and clears it; synchronises with the device. */
int cg_device_faults(int *flag);

/* Launch-variant tuning table.  Keys: CG_TUNE_COLS_MINB (resident CTAs the
 * column-pass build targets, 2, 3 or 4 (4: lengths up to 256, register-
 * direct and four-step kernels), per axis length n), CG_TUNE_COLS_PIPE
 * (column-pass kernel per n: 0 shared-memory staged, 1 persistent
 * double-buffered, 2 first and last stages in registers, 3 four-step, 4
 * persistent register prefetch, 5 persistent four-step fed by tensor-memory-
 * accelerator loads (n = 256 along y or z; 2 elsewhere)),
 * CG_TUNE_BIN_MINB (fused bin kernel: resident 128-thread CTAs the build
 * targets, 4, 5 or 6 (128, 96 or 85 registers), 1 = no target; the FP32
 * mode takes 4 where 6 is set; per stack count n), CG_TUNE_ROWS_KERNEL (x-row pass kernel per
 * half length n = nxp/2, or n = nxp for odd nxp: 0 shared-memory staged or
 * generic, 1 four-step),
 * CG_TUNE_FUSED_Y (cg_invert_cubes_fused per y length n: 0 three-pass
 * transforms around the bin kernel, 1 y pass fused with the bin loop, 2 the
 * y transform of the means split in two 16-point stages, the first in the x
 * row kernels, the second in the bin kernel (nxp = nyp = 256), an even c >= 4:
 * forward y pass, bins and inverse y pass run per chunk of c z-planes so that
 * the chunk's spectra stay in L2), CG_TUNE_BIN_FORM (fused bin solve per
 * stack count n: 0 Cholesky of the n x n data covariance, 1 information form:
 * a 3 x 3 Cholesky per bin from per-k eigen-decompositions of the error
 * covariance, for models whose every in-band error diagonal is positive;
 * the default), CG_TUNE_XY_PLANE (x and y passes of a 3D transform per x
 * length n = nxp: 0 two launches, 1 one launch of plane kernels, one z-plane
 * per two-CTA cluster with the plane's intermediate spectrum in distributed
 * shared memory; nxp = nyp = 256), CG_TUNE_COLS_SHAPE (four-step column
 * tile per axis length n: bit 0 swaps the two factors N1 x N2 of n (N1 the
 * largest divisor not above sqrt(n) instead of the smallest not below it),
 * bit 1 takes the other tile width (16 <-> 32 columns); 0 = default),
 * CG_TUNE_BIN_RUNS (fused bin kernels per stack count n: 256-bin runs each
 * CTA solves with one staged per-k table, 1..8, or 0 = about four waves of
 * CTAs, the default).  n = 0 sets the value for every n.  Built-in defaults were
 * measured on GB300; crava_gb300.autotune measures the candidates and stores
 * its choices. */
#define CG_TUNE_COLS_MINB 0
#define CG_TUNE_COLS_PIPE 1
#define CG_TUNE_BIN_MINB 2
#define CG_TUNE_ROWS_KERNEL 3
#define CG_TUNE_FUSED_Y 4
#define CG_TUNE_BIN_FORM 5
#define CG_TUNE_XY_PLANE 6
#define CG_TUNE_COLS_SHAPE 7
#define CG_TUNE_BIN_RUNS 8
int cg_tune_set(int key, int n, int value);
int cg_tune_get(int key, int n);
int cg_tune_clear(void);

/* ========================================================================
 * 3D real<->complex transforms of padded cubes.
 * ======================================================================== */

/* Replaces FFTGrid::fftInPlace (src/fftgrid.cpp:1783-1809): scale by
 * 1/sqrt(nxp*nyp*nzp) unless cubetype is CG_COVARIANCE or CG_OPERATOR, then an
 * unnormalised forward (sign -1) R2C transform in place, as
 * rfftwnd_one_real_to_complex (libs/fft/rfftw/rfftwnd.c:558). */
int cg_fft3d_r2c(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* Replaces FFTGrid::invFFTInPlace (src/fftgrid.cpp:1811-1842): unnormalised
 * backward (sign +1) C2R transform in place -- complex dimensions first, then
 * x, keeping only the real part of the x=0 and (even nxp) x=nxp/2 bins as
 * rfftwnd_one_complex_to_real does (libs/fft/rfftw/rfftwnd.c:564) -- then
 * scale by 1/N (CG_COVARIANCE, CG_OPERATOR) or 1/sqrt(N) (others). */
int cg_fft3d_c2r(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* The same two transforms on `count` equally sized cubes in one launch per
 * pass (bufs: host array of device pointers). */
int cg_fft3d_r2c_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, void *stream);
int cg_fft3d_c2r_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* FP64 variants (double buffers, same layout); the GPU accuracy reference. */
int cg_fft3d_r2c_f64(double *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);
int cg_fft3d_c2r_f64(double *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* The same transforms without any device allocation, for callers that cannot
 * let a library call cudaMalloc (an application capturing a CUDA graph with
 * allocation forbidden, or a host whose device memory belongs to its own
 * allocator).  No counterpart in the reference.  cg_fft3d_r2c/c2r allocate
 * their twiddle tables the first time a length is used; these keep them in
 * one 128 KiB array in the library's static device memory instead, which
 * every GPU that loads the library holds until exit.  Limits: even nxp with
 * nxp/2 in {32,40,48,50,60,64,80,96,100,120,128,160,192,200,240,256}, nyp
 * and nzp equal to 1 or in {64,80,96,100,120,128,160,192,200,240,256,320,
 * 384,400,480,512}, nxp+nyp+nzp <= 16384; anything else is rejected with
 * CG_ERR_ARG or CG_ERR_UNSUPPORTED before the buffer is touched.  Every call
 * rewrites the shared array, so calls that overlap on the GPU race.  The
 * first call on a device looks the array up for that device; make it before
 * any stream capture.  The column passes here always use register-direct or
 * four-step kernels, whatever the tuning table selects (the TMA-fed pass
 * allocates a fault word on first use), and the launch tracer records
 * nothing for these calls (it would create CUDA events). */
int cg_fft3d_r2c_noalloc(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);
int cg_fft3d_c2r_noalloc(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* Host-memory variants of cg_fft3d_r2c / cg_fft3d_c2r (synchronous). */
int cg_fft3d_r2c_host(float *hbuf, int nxp, int nyp, int nzp, int cubetype);
int cg_fft3d_c2r_host(float *hbuf, int nxp, int nyp, int nzp, int cubetype);

/* ========================================================================
 * Model set-up helpers.
 * ======================================================================== */

/* Per-k operator tables of Crava::fillErrMultVectors (src/crava.cpp:1337-1361,
 * constant-thickness branch) from the resampled wavelets (HOST arrays):
 * wavelets [ntheta][nzp] real samples in FFT order (Wavelet::resample,
 * src/wavelet.cpp:416-463), A [ntheta][3] reflection coefficients.  Outputs
 * (HOST): K [nzp][ntheta][3], em1/em2/em3 [nzp][ntheta] interleaved complex,
 * band [nzp] (lowCut*minRelThick < f_k < highCut, src/crava.cpp:1104-1105). */
int cg_operator_tables(int ntheta, int nz, int nzp, const float *wavelets, const float *A, float dt_ms,
                       float min_rel_thick, float low_cut, float high_cut, float *K, float *em1, float *em2,
                       float *em3, unsigned char *band);

/* FFTGrid::findClosestFactorableNumber (src/fftgrid.cpp:2857-2885). */
int cg_find_closest_factorable(int n);

/* FFTGrid::fillInParamCorr (src/fftgrid.cpp:1072-1119) times `scalar` into a
 * padded real cube (device): corr_xy [nyp][nxp], circ_corr_t [nzp]. */
int cg_fill_param_corr(float *buf, int nxp, int nyp, int nzp, const float *corr_xy, const float *circ_corr_t,
                       float grad_i, float grad_j, float scalar, void *stream);

/* FFTGrid::fillInErrCorr (src/fftgrid.cpp:1018-1070) into a padded real cube
 * (device). */
int cg_fill_err_corr(float *buf, int nxp, int nyp, int nzp, const float *corr_xy, float grad_i, float grad_j,
                     void *stream);

/* FFTGrid::multiplyByScalar (src/fftgrid.cpp:1985-1996) over n floats
 * (device, 16-byte aligned). */
int cg_scale(float *buf, long n, float scalar, void *stream);

/* FFTGrid::add (src/fftgrid.cpp:1870-1891): y += x over n floats (device,
 * 16-byte aligned). */
int cg_add(float *y, const float *x, long n, void *stream);

/* ========================================================================
 * Data ingest before the inversion
 * ======================================================================== */

/* FFTGrid::fillInData (src/fftgrid.cpp:138-370), the per-trace numerical
 * core, for every column c = i + rnxp*j (i < rnxp, j < nyp) of the padded real
 * cube buf (device, rnxp*nyp*nzp floats, written).  traces (device,
 * [rnxp*nyp][n_data]) hold one trace per column, found by the caller's
 * geometry lookup (getFillNumber, Simbox::getCoord, the nearest SegY or STORM
 * trace); state[c] != 0 marks a dead or outside trace (its column is set to
 * 0); z0_data[c] is the time of the trace's first sample, z0_grid[c] and
 * dz_grid[c] the column's simbox top and cell thickness, dz_data the sample
 * interval.  DATA cubes get the guard-zone taper over smooth_length; other
 * cube types the end extrapolation and trend removal/restoration.  Traces are
 * resampled through transforms of length findClosestFactorableNumber(n_data)
 * and 4x that, then interpolated onto the cells.  extrap_out (host, may be
 * NULL; the call then waits for the stream) receives the largest leading and
 * trailing extrapolation. */
int cg_fill_in_data(float *buf, int nxp, int nyp, int nzp, int nz, int cubetype, const float *traces, int n_data,
                    const unsigned char *state, const float *z0_data, const float *z0_grid, const float *dz_grid,
                    float dz_data, float smooth_length, int *extrap_out, void *stream);

/* ========================================================================
 * Non-constant simbox thickness (the relative thickness varies laterally).
 * ======================================================================== */

/* fillErrMultVectors tables with the thickness branch chosen: constant_thickness
 * != 0 is cg_operator_tables; 0 the non-constant branch (src/crava.cpp:1362-1385):
 * K = kD*A, errMult1 = 1/||w||, errMult2 = kD3/||e3||, errMult3 =
 * fillInverseAbskWRobust (:1493-1519).  min_rel_thick: smallest relative
 * thickness of the simbox (the band's lower edge is lowCut*min_rel_thick). */
int cg_operator_tables_ex(int ntheta, int nz, int nzp, const float *wavelets, const float *A, float dt_ms,
                          float min_rel_thick, float low_cut, float high_cut, int constant_thickness, float *K,
                          float *em1, float *em2, float *em3, unsigned char *band);

/* Floats per angle of the scale-wavelet tables (a multiple of 4). */
int cg_scale_wavelet_table_size(int nzp);

/* Per-angle tables of Crava::computeAdjustmentFactor (src/crava.cpp:807-903),
 * HOST arrays: wavelets [ntheta][nzp] (time samples in FFT order), A
 * [ntheta][3], prior_var0 [3][3] (Crava::priorVar0_), circ_corr_t [nzp] (cyclic
 * prior temporal correlation, 1 at lag 0; filtered to lags < nz as
 * getPriorCorrTFiltered), err_theta_cov [ntheta][ntheta].  dz_ms: the
 * wavelet's sample interval, lz_ms: the simbox's time thickness.  tables:
 * [ntheta][cg_scale_wavelet_table_size(nzp)] floats. */
int cg_scale_wavelet_tables(int ntheta, int nz, int nzp, const float *wavelets, const float *A,
                            const double *prior_var0, const float *circ_corr_t, const double *err_theta_cov,
                            float dz_ms, float lz_ms, float low_cut, float high_cut, float wnc, float *tables);

/* Crava::divideDataByScaleWavelet (src/crava.cpp:678-804) on ntheta real
 * padded DATA cubes (device, in place; ntheta <= 16), followed per cube by
 * FFTGrid::interpolateSeismic with energy_threshold (skipped when negative).
 * tables: device copy of cg_scale_wavelet_tables; rel_thick: [nyp][nxp]
 * (device) Simbox::getRelThick at every padded trace (must be positive);
 * shift, gain: [ntheta][ny][nx] (device) local wavelet time shift (ms) and
 * gain surfaces, or NULL for none; gain as Wavelet::setGainGrid leaves it
 * (src/wavelet.cpp:704-737: divided by its geometric mean, which multiplies
 * the wavelet the tables are built from).  n_bad (host, ntheta ints, may be NULL):
 * traces at or below the energy limit.  The slack floats of each row (x >=
 * nxp) are overwritten.  Waits for the stream when interpolating. */
int cg_divide_by_scale_wavelet(float *const *data, int ntheta, int nx, int ny, int nz, int nxp, int nyp, int nzp,
                               const float *tables, const float *rel_thick, const float *shift, const float *gain,
                               float dz_ms, float lz_ms, float low_cut, float high_cut, float energy_threshold,
                               int *n_bad, void *stream);

/* The product of Crava::multiplyDataByScaleWaveletAndWriteToFile (src/crava.cpp:
 * 906-968) on ncubes real padded cubes (device, in place): every simbox trace
 * (i < nx, j < ny) times the conjugate of its stretched local wavelet
 * spectrum; cube l uses angle l of the tables. */
int cg_multiply_by_scale_wavelet(float *const *data, int ncubes, int nx, int ny, int nxp, int nyp, int nzp,
                                 const float *tables, const float *rel_thick, const float *shift, const float *gain,
                                 float dz_ms, void *stream);

/* FFTGrid::interpolateSeismic + extrapolateSeismic (src/fftgrid.cpp:2576-2738)
 * on one real padded DATA cube (device, in place).  n_bad (host, may be NULL):
 * traces at or below the energy limit.  Synchronous. */
int cg_interpolate_seismic(float *data, int nx, int ny, int nz, int nxp, int nyp, int nzp, float energy_threshold,
                           int *n_bad, void *stream);

/* ========================================================================
 * Local noise (the error variance scales laterally, per angle).
 * ======================================================================== */

/* Crava::correctAlphaBetaRho (src/crava.cpp:2471-2569) with
 * newPosteriorCovPointwise (:2345-2451): every simbox cell of the 3 real padded
 * posterior-mean cubes post (device, in place) becomes mean + sigmanew (post -
 * mean), mean the 3 prior-mean cubes; sigmanew per trace = Delta^1/2
 * (Sm - Spost)^-1/2 with Delta = Sm G^T (G Sm G^T + D Se D)^+ G Sm, D =
 * diag(sqrt(scale_l / min scale_l)).  HOST inputs: G [ntheta][3] from
 * Crava::computeG (:2261-2343; its eigenvector signs are the caller's LAPACK
 * choice and the result depends on them), err_theta_cov [ntheta][ntheta],
 * prior_var0 and post_var0 [3][3] (Crava::priorVar0_, postVar0_).  Device:
 * noise_scale [ntheta][ny][nx] doubles (the local noise scale grids; each is
 * divided by its minimum over values other than RMISSING; a trace whose scale
 * is RMISSING counts as the minimum, where the reference computes NaN); sigmamd (may be
 * NULL) [ny][nx][9] doubles receives Crava::sigmamdnew_ (sqrt of the local
 * posterior covariance times postVar0^-1/2) for simulation. */
int cg_correct_alpha_beta_rho(float *const *post, const float *const *mean, int nx, int ny, int nz, int nxp, int nyp,
                              int nzp, int ntheta, const double *G, const double *err_theta_cov,
                              const double *prior_var0, const double *post_var0, const double *noise_scale,
                              double *sigmamd, void *stream);

/* The local-noise step of Crava::simulate (src/crava.cpp:1686-1704) on 3 real
 * padded simulated fields (device, in place): simbox cells x -> M x with the
 * trace's matrix M (mats [ny][nx][9] doubles, from cg_correct_alpha_beta_rho's
 * sigmamd), then, when mean is not NULL, every cell plus the posterior mean
 * (FFTGrid::add). */
int cg_apply_trace_matrices(float *const *fields, const float *const *mean, const double *mats, int nx, int ny,
                            int nz, int nxp, int nyp, int nzp, void *stream);

/* ========================================================================
 * File formats either side of the path (host memory, synchronous)
 * ======================================================================== */

/* FFTGrid::writeCravaFile / readCravaFile (src/fftgrid.cpp:2410-2493): the
 * padded real cube rvalue (rnxp*nyp*nzp floats) with its simbox geometry.
 * geom[11] = x0 y0 dx dy IL0 XL0 ILStepX ILStepY XLStepX XLStepY angle,
 * nxny[2] = nx ny.  Reading fails (CG_ERR_ARG) when the file's padded size
 * differs from rnxp x nyp x nzp, as the reference does; geom and nxny may be
 * NULL when reading. */
int cg_crava_file_write(const char *path, const float *rvalue, int rnxp, int nyp, int nzp, const double *geom,
                        const int *nxny);
int cg_crava_file_read(const char *path, float *rvalue, int rnxp, int nyp, int nzp, double *geom, int *nxny);

/* STORM binary grids (NRLib StormContGrid, libs/nrlib/stormgrid/
 * stormcontgrid.cpp:72-200): values are ni*nj*nk floats, i fastest.  Each of
 * the four surfaces (top, bottom, erosion top, erosion bottom) is a constant
 * or a STORM binary surface file (NRLib Volume::WriteVolumeToFile /
 * ReadVolumeFromFile, libs/nrlib/volume/volume.cpp:338-440): a non-empty
 * *_file field is written into the header in place of the constant, and a
 * header token that is not a number is returned there (the file name as the
 * header holds it; the reference resolves it against the grid file's
 * directory).  ASCII grids and grids with barriers give CG_ERR_UNSUPPORTED. */
typedef struct {
  int zone_number;
  char model_file[256];
  float missing_code;
  char variable[256];
  double x_min, lx, y_min, ly;
  double z_top, z_bot, erosion_top, erosion_bot;  /* constant surfaces */
  double lz, angle_deg;
  char z_top_file[256], z_bot_file[256], erosion_top_file[256], erosion_bot_file[256];
} cg_storm_header;

int cg_storm_write(const char *path, const float *values, int ni, int nj, int nk, const cg_storm_header *header);
int cg_storm_read_header(const char *path, cg_storm_header *header, int *ni, int *nj, int *nk);
int cg_storm_read(const char *path, float *values, long n);

/* STORM binary surfaces (NRLib WriteStormBinarySurf / ReadStormBinarySurf,
 * libs/nrlib/surface/surfaceio.hpp:101-147,439-464): an ni x nj regular grid
 * of big-endian doubles (i fastest) over [x_min, x_min + lx] x [y_min,
 * y_min + ly], nodes at spacing lx/(ni-1), ly/(nj-1); -999 marks a missing
 * node.  ni, nj >= 2.  read_header checks dx = lx/(ni-1) and dy = ly/(nj-1)
 * as the reference does.  The reference's other surface formats (Irap
 * classic ASCII, SGRI) are refused with CG_ERR_ARG.  The grid header's lz is
 * written as given (the reference samples max(bottom - top) on a 100 x 100
 * grid over the volume, Volume::RecalculateLZ, volume.cpp:494-515). */
int cg_storm_surface_write(const char *path, const double *z, int ni, int nj, double x_min, double y_min,
                           double lx, double ly);
int cg_storm_surface_read_header(const char *path, int *ni, int *nj, double *x_min, double *y_min, double *lx,
                                 double *ly);
int cg_storm_surface_read(const char *path, double *z, long n);

/* ========================================================================
 * Output grids after the bin loop
 * ======================================================================== */

/* FFTGrid::expTransf / logTransf (src/fftgrid.cpp:1726-1763) over n floats
 * (device, 16-byte aligned).  exp keeps RMISSING (-99999) values; log maps
 * RMISSING and values <= 0 to 0. */
int cg_exp_transform(float *buf, long n, void *stream);
int cg_log_transform(float *buf, long n, void *stream);

/* invFFTInPlace of count cubes followed by expTransf, the exp fused into the
 * transform's last pass (ParameterOutput::writeParameters,
 * src/parameteroutput.cpp:87-108, on the log-domain posterior means). */
int cg_fft3d_c2r_exp_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, void *stream);

/* SeismicParametersHolder::updatePriorVar + createPostCov00
 * (src/seismicparametersholder.cpp:771-807) on the real-domain posterior
 * covariance grids cov_real[6] (order 00 11 22 01 02 12, after the
 * COVARIANCE inverse transforms of invFFTCovGrids): post_var0 receives the
 * symmetric 3x3 lag-0 matrix (row-major), post_cov00 (may be NULL) the
 * values (0,0,k), k < nz, of the alpha, beta and rho grids ([3][nz]).
 * Synchronous. */
int cg_cov_origin(const float *const *cov_real, int nxp, int nyp, int nzp, int nz, double *post_var0,
                  float *post_cov00, void *stream);

/* Page-lock a caller's host buffer (e.g. an FFTGrid's fftw_malloc block) so
 * the _host entry points copy it at full link speed; undo with
 * cg_host_unregister. */
int cg_host_register(void *ptr, size_t bytes);
int cg_host_unregister(void *ptr);

/* No reference counterpart (a building block of the host-buffer entry
 * points).  Copy bytes with a kernel between any two addresses the device
 * can reach: device memory, page-locked host memory (the GPU reads and writes
 * it over the coherent NVLink-C2C link), or pageable host memory when the
 * device reports pageable access (cg_host_access bit 1).  Pointers and size
 * 16-byte aligned.  CG_ERR_UNSUPPORTED when a pointer is out of the device's
 * reach. */
int cg_copy(void *dst, const void *src, size_t bytes, void *stream);

/* How this device reaches host memory, as bits: 1 pageable memory access,
 * 2 through the host's page tables, 4 registered memory at its host
 * address. */
int cg_host_access(void);

/* ========================================================================
 * Per-frequency-bin posterior (Crava::computePostMeanResidAndFFTCov bin loop,
 * src/crava.cpp:1084-1247).
 * ======================================================================== */

/* Device-side state of one inversion model: per-k operator tables, the
 * separable prior spectra, and the mixed-precision fix-up queue. */
typedef struct cg_workspace_s *cg_workspace;

/* Model description; every pointer is HOST memory, read during
 * cg_workspace_set_model only.  Complex arrays are interleaved (re, im) float
 * pairs in the reference's per-k loop order. */
typedef struct cg_model {
  int ntheta;                  /* angle stacks, 1..8 */
  float wnc;                   /* white-noise component (Crava::wnc_) */
  int is4d;                    /* 4D branch of findParameterVariances
                                  (src/seismicparametersholder.cpp:366-373) */
  const float *K;              /* [nzp][ntheta][3] complex: kD(k) conj(W_l(k)) A[l][p]
                                  (Crava::fillErrMultVectors, src/crava.cpp:1337-1361) */
  const float *em1;            /* [nzp][ntheta] complex errMult1 */
  const float *em2;            /* [nzp][ntheta] complex errMult2 */
  const float *em3;            /* [nzp][ntheta] complex errMult3 */
  const unsigned char *band;   /* [nzp] 1 = invert this k (src/crava.cpp:1104-1105) */
  const double *err_theta_cov; /* [ntheta][ntheta] Crava::errThetaCov_ */
  const double *sigma0;        /* [3][3] prior covariance (priorVar0) */
  double cond_threshold;       /* CG_PREC_MIXED: redo a bin in FP64 when the squared
                                  ratio of largest to smallest Cholesky pivot exceeds
                                  this; <= 0 selects 1e3 */
} cg_model;

/* Allocate the device workspace for nxp x nyp x nzp cubes and ntheta stacks
 * (on the current device).  Allocation happens here only. */
int cg_workspace_create(cg_workspace *ws, int nxp, int nyp, int nzp, int ntheta);
void cg_workspace_destroy(cg_workspace ws);

/* Upload the model and build the per-k tables: the per-model work the
 * reference repeats inside computePostMeanResidAndFFTCov for every k before
 * its bins (Crava::fillErrMultVectors products and the getNextErrorVariance
 * factors, src/crava.cpp:1108-1120).  cg_workspace_set_model is synchronous.
 * cg_workspace_set_model_async copies the model into the workspace's pinned
 * staging buffer (waiting only for the previous model's copy to have left
 * it), then queues one host-to-device copy and the table kernel on `stream`;
 * inversions on other streams must be ordered after it by the caller. */
int cg_workspace_set_model(cg_workspace ws, const cg_model *model);
int cg_workspace_set_model_async(cg_workspace ws, const cg_model *model, void *stream);

/* Counters: bins queued for FP64 by the last mixed-precision inversion, and,
 * since the last reset, bins whose Cholesky failed (they keep the prior, like
 * lib_matrCholCpx failures in the reference, src/crava.cpp:1421-1423) and
 * queue overflows.  Synchronises. */
int cg_workspace_stats(cg_workspace ws, int *flagged, int *failed, int *overflow);
int cg_workspace_reset_stats(cg_workspace ws, void *stream);

/* Reference dataflow, FP32.  data[ntheta]: data spectra in, residual spectra
 * out; mean[3]: prior-mean spectra in, posterior-mean spectra out; cov[6]
 * (order covAlpha, covBeta, covRho, crCovAlphaBeta, crCovAlphaRho,
 * crCovBetaRho): prior covariance spectra (unnormalised COVARIANCE transforms
 * of fillInParamCorr cubes) in, posterior covariance spectra out; errcorr: the
 * error-correlation spectrum (fillInErrCorr + COVARIANCE transform). */
int cg_invert_bins_plain(cg_workspace ws, float *const *data, float *const *mean, float *const *cov,
                         const float *errcorr, void *stream);

/* Rebuild the separable prior spectra from the lateral correlation surface
 * corr_xy (device, nyp rows of nxp floats, ModelGeneral::findCorrXYGrid) and
 * the cyclic temporal correlation circ_corr_t (device, nzp floats,
 * SeismicParametersHolder::computeCircCorrT).  Replaces FFTCovGrids and the
 * errCorr transform of the reference when the correlation gradients are 0.
 * precision CG_PREC_FP64 also builds the FP64 tables. */
int cg_prior_spectra(cg_workspace ws, const float *corr_xy, const float *circ_corr_t, int precision,
                     void *stream);

/* The prior of the fused forms for any correlation gradients (corrGradI/J,
 * ModelGeneral::getCorrGradIJ, src/modelgeneral.cpp:2400-2414).  Zero
 * gradients: cg_prior_spectra.  Otherwise the correlation is no longer
 * separable, so the parameter-correlation cube (FFTGrid::fillInParamCorr,
 * src/fftgrid.cpp:1072-1119) and the error-correlation cube
 * (FFTGrid::fillInErrCorr, src/fftgrid.cpp:1018-1070) are filled and
 * transformed as FFTCovGrids transforms them, and every bin's prior scale
 * |Re P| and error eigenvalue |Re E| are kept in a per-bin table (8 bytes per
 * bin, 16 more for CG_PREC_FP64) that the fused bin kernels read in place of
 * the separable factors.  The table stays in use until the next
 * cg_prior_spectra / cg_prior_spectra_grad call. */
int cg_prior_spectra_grad(cg_workspace ws, const float *corr_xy, const float *circ_corr_t, float grad_i,
                          float grad_j, int precision, void *stream);

/* Fused posterior: same data/mean in-out convention as the plain form; cov[6]
 * is output only.  precision CG_PREC_FP32 or CG_PREC_MIXED.  Needs
 * cg_prior_spectra first. */
int cg_invert_bins_fused(cg_workspace ws, float *const *data, float *const *mean, float *const *cov,
                         int precision, void *stream);

/* The whole fused inversion from real-domain cubes (the transforms and bin
 * loop of Crava::computePostMeanResidAndFFTCov, src/crava.cpp:177-184 and
 * :975-1285): data[ntheta] real DATA cubes in, residual spectra out; mean[3]
 * real prior-mean cubes in, real posterior means out; cov[6] posterior
 * covariance spectra out.  For y lengths 128, 200 and 256 the forward
 * transform runs its axes as x, z, y and the y pass is fused with the bin
 * loop and the inverse y pass of the means (one HBM round trip fewer for
 * every cube); other sizes run the three-pass transforms around
 * cg_invert_bins_fused.  Needs cg_prior_spectra first. */
int cg_invert_cubes_fused(cg_workspace ws, float *const *data, float *const *mean, float *const *cov,
                          int precision, void *stream);

/* Condition estimates of the current model's in-band bins, for choosing the
 * CG_PREC_MIXED threshold (no reference counterpart: the reference runs
 * every bin in FP32).  Needs cg_prior_spectra.  hist_chol[b] counts the bins
 * whose FP64 Cholesky of the data covariance Sd has a squared pivot ratio in
 * [10^b, 10^(b+1)) (the Cholesky form's guard estimate), hist_info[b] the
 * same for the 3 x 3 information-form matrix in FP32 as the default kernel's
 * guard computes it (all zero when the model has no information-form
 * tables); b = 0 also takes ratios below 1, b = nbuckets-2 everything above,
 * and b = nbuckets-1 counts failed factorisations.  Host arrays of nbuckets
 * (2..32) entries; synchronises `stream`. */
int cg_condition_histogram(cg_workspace ws, unsigned long long *hist_chol, unsigned long long *hist_info,
                           int nbuckets, void *stream);

/* Fused posterior on FP64 spectra (needs cg_prior_spectra with CG_PREC_FP64). */
int cg_invert_bins_fused_f64(cg_workspace ws, double *const *data, double *const *mean, double *const *cov,
                             void *stream);

/* One vintage of the 4D time-lapse inversion (src/doinversion.cpp:96-135,
 * src/crava.cpp:1028-1040) in one pass over the bins: State4D::merge,
 * the bin loop with the 4D branch of findParameterVariances
 * (src/seismicparametersholder.cpp:366-373) and State4D::split
 * (src/state4d.cpp:140-580) for each bin, replacing cg_state4d_merge,
 * cg_invert_bins_plain and cg_state4d_split.  The workspace's model must have
 * is4d = 1.  State spectra (mu_s[3], mu_d[3], ss[6], sd[9], dd[6], the
 * cg_state4d_* orders) are updated in place; data[ntheta]: data spectra in,
 * residual spectra out; post_mean[3]: the current state's posterior mean
 * out (the vintage's output before its inverse transform).  CG_PREC_FP32 is
 * bit for bit the three separate passes; CG_PREC_MIXED redoes the bins whose
 * data-covariance Cholesky fails or whose pivot-ratio estimate exceeds the
 * model's cond_threshold in FP64 (merge, solve and split).  *nsplit_dev
 * (device int, may be NULL) counts bins whose split kept the prior. */
int cg_vintage4d(cg_workspace ws, float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd,
                 float *const *dd, float *const *data, const float *errcorr, float *const *post_mean, int precision,
                 int *nsplit_dev, void *stream);

/* ========================================================================
 * Whole inversion from host buffers: the entry point a replacement of
 * Crava::computePostMeanResidAndFFTCov (src/crava.cpp:975-1285) calls with
 * its FFTGrids' host memory.  The context owns the device cubes, the model
 * tables and a stream.
 * ======================================================================== */
typedef struct cg_inversion_s *cg_inversion;

typedef struct cg_inversion_model {
  int ntheta;
  const float *wavelets;        /* [ntheta][nzp] resampled wavelets, FFT order */
  const float *A;               /* [ntheta][3] reflection coefficients */
  const double *err_theta_cov;  /* [ntheta][ntheta] */
  const double *sigma0;         /* [3][3] priorVar0 */
  const float *corr_xy;         /* [nyp][nxp] lateral correlation (findCorrXYGrid) */
  const float *circ_corr_t;     /* [nzp] cyclic temporal correlation (computeCircCorrT) */
  float wnc, low_cut, high_cut, dt_ms, min_rel_thick;
  double cond_threshold;        /* CG_PREC_MIXED guard, <= 0 for the default */
  float corr_grad_i, corr_grad_j; /* correlation gradients (ModelGeneral::getCorrGradIJ), 0 for none */
} cg_inversion_model;

int cg_inversion_create(cg_inversion *inv, int nx, int ny, int nz, int nxp, int nyp, int nzp,
                        const cg_inversion_model *model);
void cg_inversion_destroy(cg_inversion inv);

/* One inversion.  seis_data[ntheta]: host rsize-float buffers, real data in,
 * residual spectra out; mean[3]: prior-mean real cubes in, posterior-mean real
 * cubes out; post_cov[6]: posterior covariance spectra out.  form 0 = plain
 * (then prior_cov_real[6] and err_corr_real are the real-domain
 * fillInParamCorr / fillInErrCorr cubes), 1 = fused FP32, 2 = fused mixed.
 * Synchronous. */
int cg_inversion_run_host(cg_inversion inv, float *const *seis_data, float *const *mean, float *const *post_cov,
                          const float *const *prior_cov_real, const float *err_corr_real, int form);

/* No reference counterpart: cg_inversion_run_host split in two so that a
 * caller with a sequence of inversions (several cubes, vintages or
 * realisations of the inputs) can keep the link busy in both directions.
 * submit queues the whole inversion on the context's streams and returns at
 * once; wait blocks until its outputs are in host memory.  Inputs are read
 * from seis_data / mean and outputs written to resid_out / mean_out, which may
 * be the same buffers (the reference's in-place semantics).  Host buffers must
 * stay untouched until wait returns.  Two contexts used in turn overlap one
 * inversion's output copies with the next one's input copies and compute;
 * submits on one context run in order. */
int cg_inversion_submit_host(cg_inversion inv, const float *const *seis_data, const float *const *mean,
                             float *const *resid_out, float *const *mean_out, float *const *post_cov,
                             const float *const *prior_cov_real, const float *err_corr_real, int form);
int cg_inversion_wait(cg_inversion inv);

/* Counters of the last runs (see cg_workspace_stats). */
int cg_inversion_stats(cg_inversion inv, int *flagged, int *failed, int *overflow);

/* ========================================================================
 * Batches of independent inversions of uneven size: each cube's whole
 * computePostMeanResidAndFFTCov (fused form) queued on one of several streams
 * forked from the caller's stream, optionally captured once into a CUDA graph
 * and replayed.  (The reference inverts one cube per run of the program.)
 * ======================================================================== */
typedef struct cg_batch_s *cg_batch;

typedef struct cg_batch_cube {
  int nx, ny, nz, nxp, nyp, nzp;
  cg_inversion_model model;     /* host arrays, read during cg_batch_create only */
} cg_batch_cube;

/* Allocates every cube's device grids, pristine input copies and model.
 * nstreams: concurrent cube streams; on GB300 two or three were fastest for
 * 64 uneven cubes (13.3 ms against 14.9 ms with eight and 14.8 ms with one). */
int cg_batch_create(cg_batch *batch, const cg_batch_cube *cubes, int ncubes, int nstreams);
void cg_batch_destroy(cg_batch batch);
/* Upload cube i's real-domain inputs (host, rsize floats each) as its pristine copy. */
int cg_batch_load(cg_batch batch, int i, const float *const *seis_data, const float *const *mean);
/* Working grids <- pristine inputs, queued on `stream`. */
int cg_batch_reset(cg_batch batch, void *stream);
/* One inversion of every cube, ordered after earlier work on `stream` and
 * before later work on it.  form 1 = fused FP32, 2 = fused mixed.  use_graph:
 * the first call runs once uncaptured (creating transform tables), captures
 * the batch into a CUDA graph and launches it; later calls launch the graph. */
int cg_batch_run(cg_batch batch, int form, int use_graph, void *stream);
/* Copy cube i's results to host buffers (any may be NULL); synchronises. */
int cg_batch_read(cg_batch batch, int i, float *const *post_mean, float *const *resid, float *const *post_cov);
/* Total frequency bins of the batch (sum of cnxp*nyp*nzp). */
long cg_batch_bins(cg_batch batch);
/* Posterior simulation inside the batch (Crava::simulate, src/crava.cpp:1551-1734, per cube): every later
 * cg_batch_run draws nreal realisations of cube i right after its inversion, on the cube's stream -- the
 * per-bin posterior factor (cg_posterior_cholesky), seeded counter-based noise keyed by (seed, realisation),
 * three inverse transforms and the posterior-mean add (cg_simulate_fields).  Allocates the cube's factor and
 * 3*nreal field cubes now, never during a run; nreal = 0 removes the simulation.  A captured graph is
 * recaptured on the next graph run.  Cubes may have different realisation counts. */
int cg_batch_set_simulation(cg_batch batch, int i, int nreal, unsigned long long seed);
/* Realisation r of cube i: 3 real padded cubes (host, rnxp*nyp*nzp floats each: alpha, beta, rho); synchronises. */
int cg_batch_read_fields(cg_batch batch, int i, int r, float *const *fields);

/* ========================================================================
 * Posterior simulation (Crava::simulate, src/crava.cpp:1551-1734).
 * ======================================================================== */

/* Cholesky factor (lib_matrCholCpx semantics, libs/lib/lib_matr.c:78-168) of
 * every bin's 3x3 posterior covariance post_cov[6] (device spectra, order as
 * cg_invert_bins_plain's cov) into `chol`: 9 planes of cnxp*nyp*nzp floats
 * (L00 L11 L22 Re L10 Im L10 Re L20 Im L20 Re L21 Im L21).  A bin whose
 * factorisation fails gets a zero factor, i.e. zero noise, as in the
 * reference (src/crava.cpp:1644-1651); nfail_dev (device int, may be NULL)
 * counts them.  Compute once per posterior, reuse for every realisation. */
int cg_posterior_cholesky(float *const *post_cov, float *chol, int nxp, int nyp, int nzp, int *nfail_dev,
                          void *stream);

/* Realisations real0 .. real0+nreal-1 of the posterior: fields[3*r + p] (r <
 * nreal, p = Vp, Vs, rho) are padded cubes that receive
 *   C2R(L xi) (PARAMETER scaling) + post_mean[p]
 * where xi is the injected noise[3] (complex spectra, nreal must be 1), or, if
 * noise is NULL, complex Gaussian noise drawn in the kernel from a
 * Philox4x32-10 stream keyed by (seed, realisation) with the Hermitian
 * structure of FFTGrid::fillInComplexNoise (src/fftgrid.cpp:1191-1241).
 * post_mean[3] are real posterior-mean cubes (device), or NULL to skip the
 * add. */
int cg_simulate_fields(const float *chol, const float *const *noise, float *const *fields, int nreal, int real0,
                       uint64_t seed, int nxp, int nyp, int nzp, const float *const *post_mean, void *stream);

/* ========================================================================
 * 4D time-lapse state (State4D, src/state4d.cpp:140-580).  All grids are
 * device spectra.  6x6 prior layout: ss[6] static-static (0,0)(0,1)(0,2)
 * (1,1)(1,2)(2,2); sd[9] static-dynamic (0,3)(0,4)(0,5)(1,3)(1,4)(1,5)(2,3)
 * (2,4)(2,5); dd[6] dynamic-dynamic (3,3)(3,4)(3,5)(4,4)(4,5)(5,5).
 * Current-state covariance order cov_cur[6]: 00 01 02 11 12 22.
 * ======================================================================== */

/* State4D::merge / mergeCov (src/state4d.cpp:140-299): mu_cur = mu_s + mu_d,
 * cov_cur = S_ss + S_dd + S_sd + S_ds folded to 3x3. */
int cg_state4d_merge(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd, float *const *dd,
                     float *const *mu_cur, float *const *cov_cur, int nxp, int nyp, int nzp, void *stream);

/* State4D::split (src/state4d.cpp:301-580): conditional update of the
 * 6-parameter state (updated in place) from the current-state posterior
 * mu_post[3] / cov_post[6].  Bins whose 3x3 prior factorisation fails keep
 * their prior (counted in nfail_dev, may be NULL). */
int cg_state4d_split(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd, float *const *dd,
                     float *const *mu_post, float *const *cov_post, int nxp, int nyp, int nzp, int *nfail_dev,
                     void *stream);

/* State4D::evolve (src/state4d.cpp:800-996), the step between two vintages
 * (ModelGeneral::advanceTime, src/modelgeneral.cpp:4852-4870), on the state
 * spectra in place: per bin mu <- E mu (+ c sqrt(nxp*nyp*nzp) at bin
 * (0,0,0), a constant in the real domain) and Sig <- E Sig E^T +
 * C Re(lambda), with E = evolution[36], c = mean_correction[6], C =
 * cov_correction[36] (row-major 6x6, parameter order Vp, Vs, rho static then
 * dynamic: TimeEvolution::getEvolutionMatrix / getMeanCorrectionTerm /
 * getCovarianceCorrectionTerm) and lambda_spec the transformed correlation of
 * the increment (cg_fill_genexp_corr + COVARIANCE transform; NULL for none).
 * The reference forms the products in FP64 and stores FP32; they are formed
 * in FP32 here (FP64 runs at a small fraction of the FP32 rate on GB300). */
int cg_state4d_evolve(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd, float *const *dd,
                      const float *lambda_spec, const double *evolution, const double *mean_correction,
                      const double *cov_correction, int nxp, int nyp, int nzp, void *stream);

/* FFTGrid::fillInGenExpCorr (src/fftgrid.cpp:1144-1187): the real padded
 * cube exp(-3 sqrt((i/Rx)^2 + (j/Ry)^2 + (k'/Rz)^2)) with cyclic lags and k'
 * the k lag shifted by the gradients, RMISSING in the row padding.  State4D::
 * evolve fills it with Rx = nx/3, Ry = ny/3, Rz = 20 and no gradients. */
int cg_fill_genexp_corr(float *buf, int nxp, int nyp, int nzp, double range_x, double range_y, double range_z,
                        float grad_i, float grad_j, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CRAVAGPU_H */

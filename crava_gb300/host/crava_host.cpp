// C++ host layer: FFTGrid / Crava mirror over the C-ABI, plus the
// host-buffer inversion entry point (cg_inversion_*) that a drop-in
// replacement of Crava::computePostMeanResidAndFFTCov calls.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cravagpu.h"
#include "cravagpu_host.hpp"
#include "../csrc/trace.cuh"
#include "../csrc/fused_entry.h"

namespace cg {
cudaError_t dev_malloc(void **p, size_t bytes);  // cudaMalloc, counted (cg_alloc_calls)
void set_error(const char *fmt, ...);
}

namespace cravagpu {

void check(int status, const char *what)
{
  if (status != CG_OK) throw Error(status, std::string(what) + ": " + cg_last_error());
}

static void cuda_check(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw Error(CG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

// ---------------------------------------------------------------------------
// FFTGrid
// ---------------------------------------------------------------------------
FFTGrid::FFTGrid(int nx, int ny, int nz, int nxp, int nyp, int nzp)
    : nx_(nx), ny_(ny), nz_(nz), nxp_(nxp), nyp_(nyp), nzp_(nzp)
{
  if (nxp < 1 || nyp < 1 || nzp < 1) throw Error(CG_ERR_ARG, "FFTGrid: bad padded size");
  cuda_check(cg::dev_malloc((void **)&d_, sizeof(float) * (size_t)getrsize()), "FFTGrid allocation");
  cuda_check(cudaMemset(d_, 0, sizeof(float) * (size_t)getrsize()), "FFTGrid clear");
}

FFTGrid::~FFTGrid()
{
  if (d_) cudaFree(d_);
}

void FFTGrid::fftInPlace(void *stream)
{
  if (istransformed_) throw Error(CG_ERR_STATE, "fftInPlace on a transformed grid");
  if (cubetype_ == CTMISSING) throw Error(CG_ERR_STATE, "fftInPlace on a grid without a cube type");
  check(cg_fft3d_r2c(d_, nxp_, nyp_, nzp_, cubetype_, stream), "fftInPlace");
  istransformed_ = true;
}

void FFTGrid::invFFTInPlace(void *stream)
{
  if (!istransformed_) throw Error(CG_ERR_STATE, "invFFTInPlace on a real grid");
  if (cubetype_ == CTMISSING) throw Error(CG_ERR_STATE, "invFFTInPlace on a grid without a cube type");
  check(cg_fft3d_c2r(d_, nxp_, nyp_, nzp_, cubetype_, stream), "invFFTInPlace");
  istransformed_ = false;
}

void FFTGrid::fillInFromArray(const float *host)
{
  cuda_check(cudaMemcpy(d_, host, sizeof(float) * (size_t)getrsize(), cudaMemcpyHostToDevice), "fillInFromArray");
}

void FFTGrid::copyToArray(float *host) const
{
  cuda_check(cudaMemcpy(host, d_, sizeof(float) * (size_t)getrsize(), cudaMemcpyDeviceToHost), "copyToArray");
}

// FFTGrid::getComplexValue / setComplexValue (src/fftgrid.cpp:1526-1556,
// :1667-1684): outside the (extended) simbox the getter returns RMISSING and
// the setter returns 1.
static const float kRMissing = -99999.0f;

Complex FFTGrid::getComplexValue(int i, int j, int k, bool ext) const
{
  if (!istransformed_) throw Error(CG_ERR_STATE, "getComplexValue on a real grid");
  const bool in = ext ? (i < getCNxp() && j < nyp_ && k < nzp_) : (i < nx_ && j < ny_ && k < nz_);
  if (!in || i < 0 || j < 0 || k < 0) return Complex{kRMissing, kRMissing};
  Complex v;
  const long idx = i + (long)j * getCNxp() + (long)k * getCNxp() * nyp_;
  cuda_check(cudaMemcpy(&v, d_ + 2 * idx, sizeof(v), cudaMemcpyDeviceToHost), "getComplexValue");
  return v;
}

int FFTGrid::setComplexValue(int i, int j, int k, Complex value, bool ext)
{
  if (!istransformed_) throw Error(CG_ERR_STATE, "setComplexValue on a real grid");
  const bool in = ext ? (i < getCNxp() && j < nyp_ && k < nzp_) : (i < nx_ && j < ny_ && k < nz_);
  if (!in || i < 0 || j < 0 || k < 0) return 1;
  const long idx = i + (long)j * getCNxp() + (long)k * getCNxp() * nyp_;
  cuda_check(cudaMemcpy(d_ + 2 * idx, &value, sizeof(value), cudaMemcpyHostToDevice), "setComplexValue");
  return 0;
}

float FFTGrid::getRealValue(int i, int j, int k, bool ext) const
{
  if (istransformed_) throw Error(CG_ERR_STATE, "getRealValue on a transformed grid");
  const bool in = ext ? (i < nxp_ && j < nyp_ && k < nzp_) : (i < nx_ && j < ny_ && k < nz_);
  if (!in || i < 0 || j < 0 || k < 0) return kRMissing;
  float v;
  const long idx = i + (long)j * getRNxp() + (long)k * getRNxp() * nyp_;
  cuda_check(cudaMemcpy(&v, d_ + idx, sizeof(v), cudaMemcpyDeviceToHost), "getRealValue");
  return v;
}

int FFTGrid::setRealValue(int i, int j, int k, float value, bool ext)
{
  if (istransformed_) throw Error(CG_ERR_STATE, "setRealValue on a transformed grid");
  const bool in = ext ? (i < nxp_ && j < nyp_ && k < nzp_) : (i < nx_ && j < ny_ && k < nz_);
  if (!in || i < 0 || j < 0 || k < 0) return 1;
  const long idx = i + (long)j * getRNxp() + (long)k * getRNxp() * nyp_;
  cuda_check(cudaMemcpy(d_ + idx, &value, sizeof(value), cudaMemcpyHostToDevice), "setRealValue");
  return 0;
}

void FFTGrid::multiplyByScalar(float s, void *stream)
{
  check(cg_scale(d_, getrsize(), s, stream), "multiplyByScalar");
}

void FFTGrid::add(const FFTGrid *o, void *stream)
{
  if (!o || o->nxp_ != nxp_ || o->nyp_ != nyp_ || o->nzp_ != nzp_) throw Error(CG_ERR_ARG, "add: size mismatch");
  check(cg_add(d_, o->d_, getrsize(), stream), "add");
}

void FFTGrid::fillInParamCorr(const float *corr_xy, const float *circ_t, float gradI, float gradJ, void *stream)
{
  if (istransformed_) throw Error(CG_ERR_STATE, "fillInParamCorr on a transformed grid");
  check(cg_fill_param_corr(d_, nxp_, nyp_, nzp_, corr_xy, circ_t, gradI, gradJ, 1.0f, stream), "fillInParamCorr");
}

void FFTGrid::fillInErrCorr(const float *corr_xy, float gradI, float gradJ, void *stream)
{
  if (istransformed_) throw Error(CG_ERR_STATE, "fillInErrCorr on a transformed grid");
  check(cg_fill_err_corr(d_, nxp_, nyp_, nzp_, corr_xy, gradI, gradJ, stream), "fillInErrCorr");
}

// ---------------------------------------------------------------------------
// Crava
// ---------------------------------------------------------------------------
Crava::Crava(int nx, int ny, int nz, int nxp, int nyp, int nzp, const InversionModel &model)
    : nx_(nx), ny_(ny), nz_(nz), nxp_(nxp), nyp_(nyp), nzp_(nzp), m_(model)
{
  const int n = m_.ntheta;
  if (n < 1 || (int)m_.wavelets.size() != n * nzp || (int)m_.A.size() != 3 * n ||
      (int)m_.errThetaCov.size() != n * n || m_.sigma0.size() != 9 || (long)m_.corrXY.size() != (long)nxp * nyp ||
      (int)m_.circCorrT.size() != nzp)
    throw Error(CG_ERR_ARG, "Crava: model arrays do not match the grid sizes");
  std::vector<float> K((size_t)nzp * n * 6), e1((size_t)nzp * n * 2), e2((size_t)nzp * n * 2), e3((size_t)nzp * n * 2);
  band_.assign(nzp, 0);
  check(cg_operator_tables(n, nz, nzp, m_.wavelets.data(), m_.A.data(), m_.dt_ms, m_.minRelThick, m_.lowCut,
                           m_.highCut, K.data(), e1.data(), e2.data(), e3.data(), band_.data()),
        "operator tables");
  check(cg_workspace_create(&ws_, nxp, nyp, nzp, n), "workspace");
  cg_model cm;
  memset(&cm, 0, sizeof(cm));
  cm.ntheta = n;
  cm.wnc = m_.wnc;
  cm.is4d = 0;
  cm.K = K.data();
  cm.em1 = e1.data();
  cm.em2 = e2.data();
  cm.em3 = e3.data();
  cm.band = band_.data();
  cm.err_theta_cov = m_.errThetaCov.data();
  cm.sigma0 = m_.sigma0.data();
  cm.cond_threshold = m_.condThreshold;
  check(cg_workspace_set_model(ws_, &cm), "set model");
  cuda_check(cg::dev_malloc((void **)&d_corr_xy_, sizeof(float) * m_.corrXY.size()), "corrXY");
  cuda_check(cg::dev_malloc((void **)&d_circ_t_, sizeof(float) * m_.circCorrT.size()), "circCorrT");
  cuda_check(cudaMemcpy(d_corr_xy_, m_.corrXY.data(), sizeof(float) * m_.corrXY.size(), cudaMemcpyHostToDevice),
             "corrXY upload");
  cuda_check(cudaMemcpy(d_circ_t_, m_.circCorrT.data(), sizeof(float) * m_.circCorrT.size(), cudaMemcpyHostToDevice),
             "circCorrT upload");
}

Crava::~Crava()
{
  if (ws_) cg_workspace_destroy(ws_);
  if (d_corr_xy_) cudaFree(d_corr_xy_);
  if (d_circ_t_) cudaFree(d_circ_t_);
  if (d_chol_) cudaFree(d_chol_);
}

int Crava::computePostMeanResidAndFFTCov(FFTGrid **seisData, FFTGrid *&postAlpha, FFTGrid *&postBeta,
                                         FFTGrid *&postRho, FFTGrid **postCov, FFTGrid *errCorr, Form form,
                                         void *stream, void *binsDone)
{
  const int n = m_.ntheta;
  FFTGrid *mean[3] = {postAlpha, postBeta, postRho};
  std::vector<float *> fwd;
  for (int l = 0; l < n; l++) {
    if (seisData[l]->getIsTransformed()) throw Error(CG_ERR_STATE, "seismic data already transformed");
    fwd.push_back(seisData[l]->devicePtr());
  }
  for (int p = 0; p < 3; p++) {
    if (mean[p]->getIsTransformed()) throw Error(CG_ERR_STATE, "prior mean already transformed");
    fwd.push_back(mean[p]->devicePtr());
  }
  float *d[8], *mu[3], *cv[6];
  for (int l = 0; l < n; l++) { d[l] = seisData[l]->devicePtr(); seisData[l]->setTransformedStatus(true); }
  for (int p = 0; p < 3; p++) { mu[p] = mean[p]->devicePtr(); mean[p]->setTransformedStatus(true); }
  for (int t = 0; t < 6; t++) cv[t] = postCov[t]->devicePtr();
  if (form == PLAIN) {
    // DATA and PARAMETER share the 1/sqrt(N) scaling: one batched transform
    check(cg_fft3d_r2c_batch(fwd.data(), (int)fwd.size(), nxp_, nyp_, nzp_, CG_DATA, stream), "forward transforms");
    if (!errCorr) throw Error(CG_ERR_ARG, "the plain form needs the error-correlation cube");
    std::vector<float *> covs(cv, cv + 6);
    covs.push_back(errCorr->devicePtr());
    check(cg_fft3d_r2c_batch(covs.data(), 7, nxp_, nyp_, nzp_, CG_COVARIANCE, stream), "FFTCovGrids");
    errCorr->setTransformedStatus(true);
    check(cg_invert_bins_plain(ws_, d, mu, cv, errCorr->devicePtr(), stream), "bin loop (plain)");
  } else {
    // separable prior tables, or the per-bin table when the correlation gradients are nonzero
    check(cg_prior_spectra_grad(ws_, d_corr_xy_, d_circ_t_, m_.corrGradI, m_.corrGradJ, CG_PREC_FP32, stream),
          "prior spectra");
    // transforms, bin loop and inverse transforms of the means in one call (the y passes fused with the bins)
    check(cg::invert_cubes_fused(ws_, d, mu, cv, form == FUSED_MIXED ? CG_PREC_MIXED : CG_PREC_FP32, stream,
                                 (cudaEvent_t)binsDone),
          "fused inversion");
    for (int t = 0; t < 6; t++) { postCov[t]->setType(FFTGrid::COVARIANCE); postCov[t]->setTransformedStatus(true); }
    for (int p = 0; p < 3; p++) mean[p]->setTransformedStatus(false);
    return 0;
  }
  for (int t = 0; t < 6; t++) { postCov[t]->setType(FFTGrid::COVARIANCE); postCov[t]->setTransformedStatus(true); }
  if (binsDone) cuda_check(cudaEventRecord((cudaEvent_t)binsDone, (cudaStream_t)stream), "bins-done event");
  check(cg_fft3d_c2r_batch(mu, 3, nxp_, nyp_, nzp_, CG_PARAMETER, stream), "posterior-mean inverse transforms");
  for (int p = 0; p < 3; p++) mean[p]->setTransformedStatus(false);
  return 0;
}

int Crava::simulate(FFTGrid **postCov, FFTGrid *const *postMean, int nSim, unsigned long long seed, FFTGrid **fields,
                    void *stream)
{
  if (nSim < 1) return 0;
  if (!d_chol_)
    cuda_check(cg::dev_malloc((void **)&d_chol_, sizeof(float) * 9 * (size_t)postCov[0]->getcsize()), "factor planes");
  float *cv[6];
  for (int t = 0; t < 6; t++) cv[t] = postCov[t]->devicePtr();
  check(cg_posterior_cholesky(cv, d_chol_, nxp_, nyp_, nzp_, nullptr, stream), "posterior factor");
  const float *mean[3] = {postMean[0]->devicePtr(), postMean[1]->devicePtr(), postMean[2]->devicePtr()};
  std::vector<float *> f(3 * (size_t)nSim);
  for (int t = 0; t < 3 * nSim; t++) { f[t] = fields[t]->devicePtr(); fields[t]->setType(FFTGrid::PARAMETER); }
  check(cg_simulate_fields(d_chol_, nullptr, f.data(), nSim, 0, seed, nxp_, nyp_, nzp_, mean, stream), "simulate");
  for (int t = 0; t < 3 * nSim; t++) fields[t]->setTransformedStatus(false);
  return 0;
}

}  // namespace cravagpu

// ---------------------------------------------------------------------------
// host-buffer inversion context (C-ABI)
// ---------------------------------------------------------------------------
using namespace cravagpu;

struct cg_inversion_s {
  int nx, ny, nz, nxp, nyp, nzp, ntheta;
  Crava *crava = nullptr;
  std::vector<FFTGrid *> data, mean, cov;
  FFTGrid *errcorr = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t out_stream = nullptr;  // residual and covariance copies, beside the mean inverse transforms
  cudaEvent_t bins_done = nullptr;
  cudaEvent_t out_done = nullptr;     // the last submit's output copies have read the device cubes
  bool out_pending = false;
};

#define CG_TRY(...)                                    \
  try {                                                \
    __VA_ARGS__                                        \
  } catch (const Error &e) {                           \
    cg::set_error("%s", e.what());                     \
    return e.status;                                   \
  } catch (const std::exception &e) {                  \
    cg::set_error("%s", e.what());                     \
    return CG_ERR_STATE;                               \
  }

extern "C" int cg_inversion_create(cg_inversion *out, int nx, int ny, int nz, int nxp, int nyp, int nzp,
                                   const cg_inversion_model *m)
{
  if (!out || !m) { cg::set_error("null argument"); return CG_ERR_ARG; }
  *out = nullptr;
  CG_TRY({
    InversionModel im;
    im.ntheta = m->ntheta;
    if (m->ntheta < 1 || m->ntheta > 8) throw Error(CG_ERR_ARG, "ntheta outside 1..8");
    if (!m->wavelets || !m->A || !m->err_theta_cov || !m->sigma0 || !m->corr_xy || !m->circ_corr_t)
      throw Error(CG_ERR_ARG, "null model array");
    im.wavelets.assign(m->wavelets, m->wavelets + (size_t)m->ntheta * nzp);
    im.A.assign(m->A, m->A + 3 * m->ntheta);
    im.errThetaCov.assign(m->err_theta_cov, m->err_theta_cov + m->ntheta * m->ntheta);
    im.sigma0.assign(m->sigma0, m->sigma0 + 9);
    im.corrXY.assign(m->corr_xy, m->corr_xy + (size_t)nxp * nyp);
    im.circCorrT.assign(m->circ_corr_t, m->circ_corr_t + nzp);
    im.wnc = m->wnc;
    im.lowCut = m->low_cut;
    im.highCut = m->high_cut;
    im.dt_ms = m->dt_ms;
    im.minRelThick = m->min_rel_thick > 0 ? m->min_rel_thick : 1.0f;
    im.condThreshold = m->cond_threshold;
    im.corrGradI = m->corr_grad_i;
    im.corrGradJ = m->corr_grad_j;
    cg_inversion_s *h = new cg_inversion_s();
    h->nx = nx; h->ny = ny; h->nz = nz; h->nxp = nxp; h->nyp = nyp; h->nzp = nzp; h->ntheta = m->ntheta;
    try {
      h->crava = new Crava(nx, ny, nz, nxp, nyp, nzp, im);
      for (int l = 0; l < m->ntheta; l++) { h->data.push_back(new FFTGrid(nx, ny, nz, nxp, nyp, nzp)); h->data.back()->setType(FFTGrid::DATA); }
      for (int p = 0; p < 3; p++) { h->mean.push_back(new FFTGrid(nx, ny, nz, nxp, nyp, nzp)); h->mean.back()->setType(FFTGrid::PARAMETER); }
      for (int t = 0; t < 6; t++) { h->cov.push_back(new FFTGrid(nx, ny, nz, nxp, nyp, nzp)); h->cov.back()->setType(FFTGrid::COVARIANCE); }
      cuda_check(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
      cuda_check(cudaStreamCreateWithFlags(&h->out_stream, cudaStreamNonBlocking), "stream");
      cuda_check(cudaEventCreateWithFlags(&h->bins_done, cudaEventDisableTiming), "event");
      cuda_check(cudaEventCreateWithFlags(&h->out_done, cudaEventDisableTiming), "event");
    } catch (...) {
      cg_inversion_destroy(h);
      throw;
    }
    *out = h;
    return CG_OK;
  })
}

extern "C" void cg_inversion_destroy(cg_inversion h)
{
  if (!h) return;
  for (auto *g : h->data) delete g;
  for (auto *g : h->mean) delete g;
  for (auto *g : h->cov) delete g;
  delete h->errcorr;
  delete h->crava;
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->out_stream) cudaStreamDestroy(h->out_stream);
  if (h->bins_done) cudaEventDestroy(h->bins_done);
  if (h->out_done) cudaEventDestroy(h->out_done);
  delete h;
}

static void submit_host(cg_inversion h, const float *const *seis_data, const float *const *mean,
                        float *const *resid_out, float *const *mean_out, float *const *post_cov,
                        const float *const *prior_cov_real, const float *err_corr_real, int form)
{
  const size_t bytes = sizeof(float) * (size_t)h->data[0]->getrsize();
  cudaStream_t st = h->stream, os = h->out_stream;
  // the previous submit's output copies (on the output stream) read the same device cubes
  if (h->out_pending) cuda_check(cudaStreamWaitEvent(st, h->out_done, 0), "wait previous outputs");
  {
    cg::TraceScope ts("copy_h2d", st, (double)bytes * (h->ntheta + 3));
    for (int l = 0; l < h->ntheta; l++) {
      cuda_check(cudaMemcpyAsync(h->data[l]->devicePtr(), seis_data[l], bytes, cudaMemcpyHostToDevice, st), "H2D data");
      h->data[l]->setTransformedStatus(false);
    }
    for (int p = 0; p < 3; p++) {
      cuda_check(cudaMemcpyAsync(h->mean[p]->devicePtr(), mean[p], bytes, cudaMemcpyHostToDevice, st), "H2D mean");
      h->mean[p]->setTransformedStatus(false);
    }
  }
  Crava::Form f = form == 0 ? Crava::PLAIN : form == 1 ? Crava::FUSED_FP32 : Crava::FUSED_MIXED;
  if (f == Crava::PLAIN) {
    if (!prior_cov_real || !err_corr_real) throw Error(CG_ERR_ARG, "the plain form needs the real prior covariance cubes");
    if (!h->errcorr) { h->errcorr = new FFTGrid(h->nx, h->ny, h->nz, h->nxp, h->nyp, h->nzp); h->errcorr->setType(FFTGrid::COVARIANCE); }
    for (int t = 0; t < 6; t++) {
      cuda_check(cudaMemcpyAsync(h->cov[t]->devicePtr(), prior_cov_real[t], bytes, cudaMemcpyHostToDevice, st), "H2D cov");
      h->cov[t]->setTransformedStatus(false);
    }
    cuda_check(cudaMemcpyAsync(h->errcorr->devicePtr(), err_corr_real, bytes, cudaMemcpyHostToDevice, st), "H2D errCorr");
    h->errcorr->setTransformedStatus(false);
  }
  FFTGrid *a = h->mean[0], *b = h->mean[1], *c = h->mean[2];
  h->crava->computePostMeanResidAndFFTCov(h->data.data(), a, b, c, h->cov.data(), h->errcorr, f, st, h->bins_done);
  // residual and covariance spectra leave while the posterior means are transformed back
  cuda_check(cudaStreamWaitEvent(os, h->bins_done, 0), "wait bins");
  {
    cg::TraceScope ts("copy_d2h_resid_cov", os, (double)bytes * (h->ntheta + 6));
    for (int l = 0; l < h->ntheta; l++)
      cuda_check(cudaMemcpyAsync(resid_out[l], h->data[l]->devicePtr(), bytes, cudaMemcpyDeviceToHost, os), "D2H residual");
    for (int t = 0; t < 6; t++)
      cuda_check(cudaMemcpyAsync(post_cov[t], h->cov[t]->devicePtr(), bytes, cudaMemcpyDeviceToHost, os), "D2H cov");
  }
  {
    cg::TraceScope ts("copy_d2h_mean", st, (double)bytes * 3);
    for (int p = 0; p < 3; p++)
      cuda_check(cudaMemcpyAsync(mean_out[p], h->mean[p]->devicePtr(), bytes, cudaMemcpyDeviceToHost, st), "D2H mean");
  }
  cuda_check(cudaEventRecord(h->out_done, os), "outputs-done event");
  h->out_pending = true;
}

static void check_host_args(cg_inversion h, const void *a, const void *b, const void *c, const void *d, const void *e)
{
  if (!h || !a || !b || !c || !d || !e) throw Error(CG_ERR_ARG, "null argument");
}

extern "C" int cg_inversion_run_host(cg_inversion h, float *const *seis_data, float *const *mean, float *const *post_cov,
                                     const float *const *prior_cov_real, const float *err_corr_real, int form)
{
  CG_TRY({
    check_host_args(h, seis_data, mean, post_cov, seis_data, mean);
    submit_host(h, seis_data, mean, seis_data, mean, post_cov, prior_cov_real, err_corr_real, form);
    const cudaError_t e1 = cudaStreamSynchronize(h->stream), e2 = cudaStreamSynchronize(h->out_stream);
    cuda_check(e1 != cudaSuccess ? e1 : e2, "inversion");
    return CG_OK;
  })
}

extern "C" int cg_inversion_submit_host(cg_inversion h, const float *const *seis_data, const float *const *mean,
                                        float *const *resid_out, float *const *mean_out, float *const *post_cov,
                                        const float *const *prior_cov_real, const float *err_corr_real, int form)
{
  CG_TRY({
    check_host_args(h, seis_data, mean, resid_out, mean_out, post_cov);
    submit_host(h, seis_data, mean, resid_out, mean_out, post_cov, prior_cov_real, err_corr_real, form);
    return CG_OK;
  })
}

extern "C" int cg_inversion_wait(cg_inversion h)
{
  if (!h) { cg::set_error("null argument"); return CG_ERR_ARG; }
  CG_TRY({
    const cudaError_t e1 = cudaStreamSynchronize(h->stream), e2 = cudaStreamSynchronize(h->out_stream);
    cuda_check(e1 != cudaSuccess ? e1 : e2, "inversion");
    return CG_OK;
  })
}

extern "C" int cg_inversion_stats(cg_inversion h, int *flagged, int *failed, int *overflow)
{
  if (!h) { cg::set_error("null argument"); return CG_ERR_ARG; }
  return cg_workspace_stats(h->crava->workspace(), flagged, failed, overflow);
}

extern "C" int cg_host_register(void *ptr, size_t bytes)
{
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterPortable | cudaHostRegisterMapped);
  if (e != cudaSuccess) { (void)cudaGetLastError(); cg::set_error("cudaHostRegister: %s", cudaGetErrorString(e)); return CG_ERR_CUDA; }
  return CG_OK;
}

extern "C" int cg_host_unregister(void *ptr)
{
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) { (void)cudaGetLastError(); cg::set_error("cudaHostUnregister: %s", cudaGetErrorString(e)); return CG_ERR_CUDA; }
  return CG_OK;
}

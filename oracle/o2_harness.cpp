// In-process harness around the reference's own compiled classes -- TEST
// INFRASTRUCTURE ONLY (it generates golden fixtures; nothing in the product
// links it).  Built by oracle/Makefile.o2 from the unmodified reference
// sources; runs only where the reference checkout is (x86 build container).
//
//   crava_o2 inversion  <dir>   Ricker wavelets (Wavelet1D + Wavelet::resample),
//                               prior covariance cubes (SeismicParametersHolder::
//                               initializeCorrelations: computeCircCorrT +
//                               FFTGrid::fillInParamCorr), error correlation
//                               (FFTGrid::fillInErrCorr; both with the correlation
//                               gradients grad_i / grad_j, 0 when absent), the data and prior-mean
//                               transforms (FFTGrid::fftInPlace), then
//                               Crava::computePostMeanResidAndFFTCov itself
//                               (src/crava.cpp:975-1285); afterwards the per-k
//                               tables of Crava::fillErrMultVectors for both
//                               thickness branches (src/crava.cpp:1337-1386).
//   crava_o2 state4d    <dir>   State4D::merge and State4D::split
//                               (src/state4d.cpp:140-580) on given spectra.
//   crava_o2 state4d_evolve <dir>
//                               State4D::evolve (src/state4d.cpp:800-996) for given
//                               evolution and correction terms.
//   crava_o2 adjust     <dir>   Crava::computeAdjustmentFactor (src/crava.cpp:807-903)
//                               for given local shifts, gains and stretches.
//   crava_o2 localnoise <dir>   Crava::computeG and Crava::correctAlphaBetaRho
//                               (src/crava.cpp:2261-2569) on given cubes and scales.
//   crava_o2 fillindata <dir>   FFTGrid::fillInData from a STORM grid onto a simbox.
//   crava_o2 interpolate <dir>  FFTGrid::interpolateSeismic on a DATA cube.
//   crava_o2 divide     <dir>   Crava::divideDataByScaleWavelet on a simbox of non-constant thickness,
//                               then Crava::multiplyDataByScaleWaveletAndWriteToFile on the result.
//   crava_o2 crava_write / crava_read <dir>
//                               FFTGrid::writeCravaFile / readCravaFile.
//   crava_o2 storm_write / storm_read <dir>
//                               NRLib::StormContGrid::WriteToFile / ReadFromFile
//                               (constant surfaces).
//   crava_o2 storm_write_surf / storm_read_surf <dir>
//                               the same with regular top and bottom surfaces
//                               written to / read from files beside the grid.
//   crava_o2 factorable <dir>   FFTGrid::findClosestFactorableNumber.
//
// <dir> holds params.txt ("key value" lines) and raw little-endian arrays
// named in this file; outputs are written to the same directory.  A minimal
// Crava / ModelGeneral is set up by writing the few members the called
// methods read (seisData_, ntheta_, nzp_; do4DInversion_), which is why the
// reference headers are included with their access specifiers opened.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <csignal>
#include <execinfo.h>
#include <unistd.h>
#include <fstream>
#include <iostream>
#include <list>
#include <new>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#define private public
#define protected public
#include "src/crava.h"
#include "src/definitions.h"
#include "src/fftgrid.h"
#include "src/modelavodynamic.h"
#include "src/modelgeneral.h"
#include "src/modelsettings.h"
#include "src/seismicparametersholder.h"
#include "src/simbox.h"
#include "src/state4d.h"
#include "src/timeevolution.h"
#include "src/wavelet1D.h"
#include "nrlib/stormgrid/stormcontgrid.hpp"
#include "nrlib/surface/surface.hpp"
#include "nrlib/surface/regularsurface.hpp"
#undef private
#undef protected

namespace {

std::string g_dir;

std::map<std::string, double> read_params()
{
  std::map<std::string, double> p;
  std::ifstream f((g_dir + "/params.txt").c_str());
  std::string k;
  double v;
  while (f >> k >> v) p[k] = v;
  return p;
}

template <typename T>
std::vector<T> read_arr(const std::string &name, size_t n)
{
  std::vector<T> v(n);
  FILE *f = fopen((g_dir + "/" + name).c_str(), "rb");
  if (!f || fread(&v[0], sizeof(T), n, f) != n) {
    fprintf(stderr, "cannot read %s (%zu values)\n", name.c_str(), n);
    exit(2);
  }
  fclose(f);
  return v;
}

void write_raw(const std::string &name, const void *p, size_t bytes)
{
  FILE *f = fopen((g_dir + "/" + name).c_str(), "wb");
  if (!f || fwrite(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "cannot write %s\n", name.c_str());
    exit(2);
  }
  fclose(f);
}

// a grid holding `vals` (rsize floats, the FFTGrid in-place layout) in the given domain
FFTGrid *make_grid(int nx, int ny, int nz, int nxp, int nyp, int nzp, int cubetype, const float *vals, bool transformed)
{
  FFTGrid *g = new FFTGrid(nx, ny, nz, nxp, nyp, nzp);
  g->createRealGrid(false);
  g->setType(cubetype);
  if (vals) memcpy(g->rvalue_, vals, sizeof(float) * (size_t)g->rsize_);
  g->istransformed_ = transformed;
  return g;
}

void dump_grid(const std::string &name, FFTGrid *g)
{
  write_raw(name, g->rvalue_, sizeof(float) * (size_t)g->rsize_);
}

int cmd_inversion()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"], n = (int)p["ntheta"];
  const int ncorrt = (int)p["ncorrt"], min_int_fq = (int)p["min_int_fq"];
  const float dt = (float)p["dt"], fpeak = (float)p["fpeak"], low_cut = (float)p["low_cut"];
  const float high_cut = (float)p["high_cut"], wnc = (float)p["wnc"];
  const float grad_i = (float)p["grad_i"], grad_j = (float)p["grad_j"];  // correlation gradients (0 if absent)
  const int cnxp = nxp / 2 + 1, rnxp = 2 * cnxp;
  const size_t rsize = (size_t)rnxp * nyp * nzp;

  std::vector<float> theta = read_arr<float>("theta.f32", n);
  std::vector<float> A = read_arr<float>("A.f32", (size_t)n * 3);
  std::vector<double> etc = read_arr<double>("etc.f64", (size_t)n * n);
  std::vector<float> s0 = read_arr<float>("sigma0.f32", 9);
  std::vector<double> cxy = read_arr<double>("corrxy.f64", (size_t)nxp * nyp);
  std::vector<float> corrT = read_arr<float>("corrt.f32", ncorrt);
  std::vector<float> data = read_arr<float>("data.f32", rsize * n);
  std::vector<float> mean = read_arr<float>("mean.f32", rsize * 3);

  // wavelets: the reference's Ricker (239 taps at 1 ms), resampled onto the grid in FFT order; one set
  // for the inversion (which transforms them) and one for the table extraction afterwards
  // (given_wavelets = 1: the resampled samples are replaced by wavelets_in.f32, n x nzp in FFT order, and
  // the norm recomputed from them as Wavelet::resample computes it, src/wavelet.cpp:442-446)
  ModelSettings ms;
  Wavelet **wav = new Wavelet *[n], **wav2 = new Wavelet *[n];
  std::vector<float> wav_out((size_t)n * nzp), wav_norm(n), given;
  if (p["given_wavelets"] != 0.0) given = read_arr<float>("wavelets_in.f32", (size_t)n * nzp);
  for (int set = 0; set < 2; set++)
    for (int l = 0; l < n; l++) {
      int err = 0;
      Wavelet1D *w = new Wavelet1D(&ms, &A[3 * l], theta[l], fpeak, err);
      if (err) { fprintf(stderr, "wavelet %d: error %d\n", l, err); return 3; }
      w->resample(dt, nz, nzp);
      if (!given.empty()) {
        double norm2 = 0.0;
        for (int k = 0; k < nzp; k++) {
          w->rAmp_[k] = given[(size_t)l * nzp + k];
          norm2 += static_cast<double>(w->rAmp_[k] * w->rAmp_[k]);
        }
        w->norm_ = static_cast<float>(sqrt(norm2));
      }
      if (set == 0) {
        for (int k = 0; k < nzp; k++) wav_out[(size_t)l * nzp + k] = w->rAmp_[k];
        wav_norm[l] = w->norm_;
        wav[l] = w;
      } else {
        wav2[l] = w;
      }
    }
  write_raw("wavelets.f32", &wav_out[0], sizeof(float) * wav_out.size());
  write_raw("wavelet_norms.f32", &wav_norm[0], sizeof(float) * n);

  // lateral correlation surface (ModelGeneral::findCorrXYGrid's output), nxp x nyp
  Surface corr_xy(0.0, 0.0, 25.0 * nxp, 25.0 * nyp, nxp, nyp, 0.0);
  for (int j = 0; j < nyp; j++)
    for (int i = 0; i < nxp; i++) corr_xy(i + nxp * j) = cxy[(size_t)j * nxp + i];

  // prior covariance cubes: computeCircCorrT + fillInParamCorr x priorVar0
  SeismicParametersHolder sp;
  sp.priorVar0_.resize(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) sp.priorVar0_(a, b) = static_cast<double>(s0[3 * a + b]);
  sp.createCorrGrids(nx, ny, nz, nxp, nyp, nzp, false);
  sp.initializeCorrelations(&corr_xy, corrT, grad_i, grad_j, min_int_fq, nzp);
  fftw_real *circ = sp.computeCircCorrT(corrT, min_int_fq, nzp);
  write_raw("circcorrt.f32", circ, sizeof(float) * nzp);
  fftw_free(circ);
  FFTGrid *covs[6] = {sp.covAlpha_, sp.covBeta_, sp.covRho_, sp.crCovAlphaBeta_, sp.crCovAlphaRho_, sp.crCovBetaRho_};
  {
    std::vector<float> prior_cov(rsize * 6);
    for (int t = 0; t < 6; t++) memcpy(&prior_cov[rsize * t], covs[t]->rvalue_, sizeof(float) * rsize);
    write_raw("prior_cov_real.f32", &prior_cov[0], sizeof(float) * prior_cov.size());
  }

  FFTGrid *errcorr = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::COVARIANCE, NULL, false);
  errcorr->fillInErrCorr(&corr_xy, grad_i, grad_j);
  dump_grid("errcorr_real.f32", errcorr);

  // data and prior means, transformed by the reference's own fftInPlace (src/crava.cpp:177-184)
  FFTGrid **seis = new FFTGrid *[n];
  for (int l = 0; l < n; l++) {
    seis[l] = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::DATA, &data[rsize * l], false);
    seis[l]->fftInPlace();
  }
  FFTGrid *mu[3];
  for (int q = 0; q < 3; q++) {
    mu[q] = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::PARAMETER, &mean[rsize * q], false);
    mu[q]->fftInPlace();
  }
  {
    std::vector<float> spec(rsize * (n + 3));
    for (int l = 0; l < n; l++) memcpy(&spec[rsize * l], seis[l]->rvalue_, sizeof(float) * rsize);
    for (int q = 0; q < 3; q++) memcpy(&spec[rsize * (n + q)], mu[q]->rvalue_, sizeof(float) * rsize);
    write_raw("input_spectra.f32", &spec[0], sizeof(float) * spec.size());
  }

  // the minimal Crava / ModelGeneral / Simbox the inversion reads
  Crava *crava = static_cast<Crava *>(operator new(sizeof(Crava)));
  memset((void *)crava, 0, sizeof(Crava));
  crava->seisData_ = seis;
  crava->ntheta_ = n;
  crava->nzp_ = nzp;
  crava->nz_ = nz;
  ModelGeneral *mg = static_cast<ModelGeneral *>(operator new(sizeof(ModelGeneral)));
  memset((void *)mg, 0, sizeof(ModelGeneral));
  mg->do4DInversion_ = false;
  Simbox simbox;
  simbox.lz_ = (double)nz * dt;
  simbox.constThick_ = true;
  simbox.minRelThick_ = 1.0;

  double **etcp = new double *[n];
  float **Ap = new float *[n];
  for (int l = 0; l < n; l++) { etcp[l] = &etc[(size_t)n * l]; Ap[l] = &A[3 * l]; }

  crava->computePostMeanResidAndFFTCov(mg, &simbox, sp, mu[0], mu[1], mu[2], errcorr, seis, wav, etcp, Ap, &theta[0], n,
                                       low_cut, high_cut, wnc, nz, nzp, nyp, nxp, 1, false);

  {
    std::vector<float> out(rsize * (3 + n + 6));
    for (int q = 0; q < 3; q++) memcpy(&out[rsize * q], mu[q]->rvalue_, sizeof(float) * rsize);
    for (int l = 0; l < n; l++) memcpy(&out[rsize * (3 + l)], seis[l]->rvalue_, sizeof(float) * rsize);
    for (int t = 0; t < 6; t++) memcpy(&out[rsize * (3 + n + t)], covs[t]->rvalue_, sizeof(float) * rsize);
    write_raw("output.f32", &out[0], sizeof(float) * out.size());
    dump_grid("errcorr_spec.f32", errcorr);
  }

  // the per-k tables both thickness branches hand to the bin solve, built from the second wavelet set in
  // the order computePostMeanResidAndFFTCov builds them (src/crava.cpp:1002-1049)
  Wavelet1D *d1 = new Wavelet1D(Wavelet::FIRSTORDERFORWARDDIFF, nz, nzp);
  Wavelet1D *d2 = new Wavelet1D(d1, Wavelet::FIRSTORDERBACKWARDDIFF);
  Wavelet1D *d3 = new Wavelet1D(d2, Wavelet::FIRSTORDERCENTRALDIFF);
  d1->fft1DInPlace();
  d3->fft1DInPlace();
  Wavelet1D **es = new Wavelet1D *[n], **es3 = new Wavelet1D *[n], **wnorm = new Wavelet1D *[n];
  crava->makeErrorSmooth(es, es3, seis, wav2, &theta[0], n);
  for (int l = 0; l < n; l++) {
    wnorm[l] = wav2[l]->createWavelet1DForErrorNorm();
    wnorm[l]->fft1DInPlace();
  }
  for (int branch = 1; branch >= 0; branch--) {  // the non-constant branch reads the wavelets untransformed
    const bool constant = branch == 0;
    if (constant)
      for (int l = 0; l < n; l++) wav2[l]->fft1DInPlace();
    std::vector<float> K((size_t)nzp * n * 3 * 2), e1((size_t)nzp * n * 2), e2(e1.size()), e3(e1.size());
    std::vector<unsigned char> band(nzp);
    fftw_complex *m1 = new fftw_complex[n], *m2 = new fftw_complex[n], *m3 = new fftw_complex[n];
    fftw_complex **Kk = crava->allocateFFTComplex(n, 3);
    for (int k = 0; k < nzp; k++) {
      const float f = static_cast<float>((nz * 1000.0f) / (simbox.getlz() * nzp) * std::min(k, nzp - k));
      band[k] = (f > low_cut * simbox.getMinRelThick() && f < high_cut) ? 1 : 0;
      crava->fillErrMultVectors(m1, m2, m3, Kk, d1->getCAmp(k), d3->getCAmp(k), wav2, wnorm, es3, Ap, constant, n, k);
      for (int l = 0; l < n; l++) {
        for (int q = 0; q < 3; q++) {
          K[(((size_t)k * n + l) * 3 + q) * 2] = Kk[l][q].re;
          K[(((size_t)k * n + l) * 3 + q) * 2 + 1] = Kk[l][q].im;
        }
        e1[((size_t)k * n + l) * 2] = m1[l].re; e1[((size_t)k * n + l) * 2 + 1] = m1[l].im;
        e2[((size_t)k * n + l) * 2] = m2[l].re; e2[((size_t)k * n + l) * 2 + 1] = m2[l].im;
        e3[((size_t)k * n + l) * 2] = m3[l].re; e3[((size_t)k * n + l) * 2 + 1] = m3[l].im;
      }
    }
    const std::string sfx = constant ? "" : "_nct";
    write_raw("K" + sfx + ".f32", &K[0], sizeof(float) * K.size());
    write_raw("em1" + sfx + ".f32", &e1[0], sizeof(float) * e1.size());
    write_raw("em2" + sfx + ".f32", &e2[0], sizeof(float) * e2.size());
    write_raw("em3" + sfx + ".f32", &e3[0], sizeof(float) * e3.size());
    write_raw("band" + sfx + ".u8", &band[0], band.size());
  }
  return 0;
}

int cmd_state4d()
{
  std::map<std::string, double> p = read_params();
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"];
  const int cnxp = nxp / 2 + 1, rnxp = 2 * cnxp;
  const size_t rsize = (size_t)rnxp * nyp * nzp;
  // state spectra in: mu_s(3) mu_d(3) ss(6) sd(9) dd(6); posterior of the current state: mu(3) cov(6)
  std::vector<float> st = read_arr<float>("state.f32", rsize * 27);
  std::vector<float> post = read_arr<float>("post.f32", rsize * 9);
  std::vector<FFTGrid *> g(27);
  for (int t = 0; t < 27; t++)
    g[t] = make_grid(nxp, nyp, nzp, nxp, nyp, nzp, t < 6 ? FFTGrid::PARAMETER : FFTGrid::COVARIANCE, &st[rsize * t], true);
  State4D s4;
  s4.setStaticMu(g[0], g[1], g[2]);
  s4.setDynamicMu(g[3], g[4], g[5]);
  s4.setStaticSigma(g[6], g[7], g[8], g[9], g[10], g[11]);
  s4.setStaticDynamicSigma(g[12], g[13], g[14], g[15], g[16], g[17], g[18], g[19], g[20]);
  s4.setDynamicSigma(g[21], g[22], g[23], g[24], g[25], g[26]);

  // merge: the current state's prior (means and covariance spectra)
  SeismicParametersHolder cur;
  cur.muAlpha_ = make_grid(nxp, nyp, nzp, nxp, nyp, nzp, FFTGrid::PARAMETER, NULL, true);
  cur.muBeta_ = make_grid(nxp, nyp, nzp, nxp, nyp, nzp, FFTGrid::PARAMETER, NULL, true);
  cur.muRho_ = make_grid(nxp, nyp, nzp, nxp, nyp, nzp, FFTGrid::PARAMETER, NULL, true);
  FFTGrid **cg[6] = {&cur.covAlpha_, &cur.crCovAlphaBeta_, &cur.crCovAlphaRho_, &cur.covBeta_, &cur.crCovBetaRho_,
                     &cur.covRho_};
  for (int t = 0; t < 6; t++) *cg[t] = make_grid(nxp, nyp, nzp, nxp, nyp, nzp, FFTGrid::COVARIANCE, NULL, true);
  s4.merge(cur);
  {
    std::vector<float> out(rsize * 9);
    FFTGrid *m[3] = {cur.muAlpha_, cur.muBeta_, cur.muRho_};
    for (int q = 0; q < 3; q++) memcpy(&out[rsize * q], m[q]->rvalue_, sizeof(float) * rsize);
    for (int t = 0; t < 6; t++) memcpy(&out[rsize * (3 + t)], (*cg[t])->rvalue_, sizeof(float) * rsize);
    write_raw("merged.f32", &out[0], sizeof(float) * out.size());
  }
  // split with the given posterior of the current state (order: mu 3, then 00 01 02 11 12 22)
  FFTGrid *m[3] = {cur.muAlpha_, cur.muBeta_, cur.muRho_};
  for (int q = 0; q < 3; q++) memcpy(m[q]->rvalue_, &post[rsize * q], sizeof(float) * rsize);
  for (int t = 0; t < 6; t++) memcpy((*cg[t])->rvalue_, &post[rsize * (3 + t)], sizeof(float) * rsize);
  s4.split(cur);
  {
    std::vector<float> out(rsize * 27);
    for (int t = 0; t < 27; t++) memcpy(&out[rsize * t], g[t]->rvalue_, sizeof(float) * rsize);
    write_raw("split.f32", &out[0], sizeof(float) * out.size());
  }
  return 0;
}

// State4D::evolve (src/state4d.cpp:800-996) with one time step of a TimeEvolution whose evolution matrix,
// mean and covariance correction terms are E.f64, c.f64, C.f64, on the 27 state spectra of state.f32 (grids
// of logical size nx x ny x nz, which set the increment's correlation ranges); also the increment's
// correlation cube as evolve builds it (FFTGrid::fillInGenExpCorr) before and after its transform
int cmd_state4d_evolve()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"];
  const size_t rsize = (size_t)2 * (nxp / 2 + 1) * nyp * nzp;
  std::vector<float> st = read_arr<float>("state.f32", rsize * 27);
  std::vector<double> E = read_arr<double>("E.f64", 36), c = read_arr<double>("c.f64", 6),
                      C = read_arr<double>("C.f64", 36);
  std::vector<FFTGrid *> g(27);
  for (int t = 0; t < 27; t++)
    g[t] = make_grid(nx, ny, nz, nxp, nyp, nzp, t < 6 ? FFTGrid::PARAMETER : FFTGrid::COVARIANCE, &st[rsize * t], true);
  State4D s4;
  s4.setStaticMu(g[0], g[1], g[2]);
  s4.setDynamicMu(g[3], g[4], g[5]);
  s4.setStaticSigma(g[6], g[7], g[8], g[9], g[10], g[11]);
  s4.setStaticDynamicSigma(g[12], g[13], g[14], g[15], g[16], g[17], g[18], g[19], g[20]);
  s4.setDynamicSigma(g[21], g[22], g[23], g[24], g[25], g[26]);
  TimeEvolution te;
  NRLib::Matrix Em(6, 6), Cm(6, 6);
  NRLib::Vector cv(6);
  for (int a = 0; a < 6; a++) {
    cv(a) = c[a];
    for (int b = 0; b < 6; b++) { Em(a, b) = E[6 * a + b]; Cm(a, b) = C[6 * a + b]; }
  }
  te.evolution_matrix_.push_back(Em);
  te.mean_correction_term_.push_back(cv);
  te.cov_correction_term_.push_back(Cm);
  s4.evolve(0, te);
  {
    std::vector<float> out(rsize * 27);
    for (int t = 0; t < 27; t++) memcpy(&out[rsize * t], g[t]->rvalue_, sizeof(float) * rsize);
    write_raw("evolved.f32", &out[0], sizeof(float) * out.size());
  }
  FFTGrid lam(nx, ny, nz, nxp, nyp, nzp);
  lam.createGrid();
  lam.fillInGenExpCorr(float(nx) / 3.0, float(ny) / 3.0, 20.0, 0.0f, 0.0f);
  dump_grid("genexp_real.f32", &lam);
  lam.fftInPlace();
  dump_grid("genexp_spec.f32", &lam);
  return 0;
}

// Crava::computeAdjustmentFactor (src/crava.cpp:807-903) for a list of (time shift, gain, stretch) cases:
// the local wavelet is the global Ricker copied and shifted / scaled as createLocalWavelet1D does
int cmd_adjust()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"], nc = (int)p["ncases"];
  const int ncorrt = (int)p["ncorrt"], min_int_fq = (int)p["min_int_fq"];
  const float dt = (float)p["dt"], fpeak = (float)p["fpeak"], theta = (float)p["theta"];
  const float error_var = (float)p["error_var"];
  std::vector<float> A = read_arr<float>("A.f32", 3);
  std::vector<float> s0 = read_arr<float>("sigma0.f32", 9);
  std::vector<double> cxy = read_arr<double>("corrxy.f64", (size_t)nxp * nyp);
  std::vector<float> corrT = read_arr<float>("corrt.f32", ncorrt);
  std::vector<float> cases = read_arr<float>("cases.f32", (size_t)nc * 3);

  ModelSettings ms;
  int err = 0;
  Wavelet1D *wglob = new Wavelet1D(&ms, &A[0], theta, fpeak, err);
  if (err) { fprintf(stderr, "wavelet: error %d\n", err); return 3; }
  wglob->resample(dt, nz, nzp);
  write_raw("wavelet.f32", wglob->rAmp_, sizeof(float) * nzp);

  Surface corr_xy(0.0, 0.0, 25.0 * nxp, 25.0 * nyp, nxp, nyp, 0.0);
  for (int j = 0; j < nyp; j++)
    for (int i = 0; i < nxp; i++) corr_xy(i + nxp * j) = cxy[(size_t)j * nxp + i];
  SeismicParametersHolder sp;
  sp.priorVar0_.resize(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) sp.priorVar0_(a, b) = static_cast<double>(s0[3 * a + b]);
  sp.createCorrGrids(nx, ny, nz, nxp, nyp, nzp, false);
  sp.initializeCorrelations(&corr_xy, corrT, 0.0f, 0.0f, min_int_fq, nzp);
  float *filtered = sp.getPriorCorrTFiltered(nz, nzp);
  write_raw("corrt_filtered.f32", filtered, sizeof(float) * nzp);
  delete[] filtered;

  Simbox simbox;
  simbox.lz_ = (double)nz * dt;
  Crava *crava = static_cast<Crava *>(operator new(sizeof(Crava)));
  memset((void *)crava, 0, sizeof(Crava));
  crava->nz_ = nz;
  crava->nzp_ = nzp;
  crava->lowCut_ = (float)p["low_cut"];
  crava->highCut_ = (float)p["high_cut"];
  crava->wnc_ = (float)p["wnc"];
  crava->simbox_ = &simbox;
  new (&crava->priorVar0_) NRLib::Matrix(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) crava->priorVar0_(a, b) = static_cast<double>(s0[3 * a + b]);

  const int cnzp = nzp / 2 + 1;
  std::vector<float> out((size_t)nc * cnzp * 2);
  fftw_complex *adj = new fftw_complex[cnzp];
  for (int c = 0; c < nc; c++) {
    Wavelet1D *loc = new Wavelet1D(wglob);
    loc->shiftAndScale(cases[3 * c], cases[3 * c + 1]);
    crava->computeAdjustmentFactor(adj, loc, (double)cases[3 * c + 2], wglob, sp, &A[0], error_var);
    for (int k = 0; k < cnzp; k++) {
      out[((size_t)c * cnzp + k) * 2] = adj[k].re;
      out[((size_t)c * cnzp + k) * 2 + 1] = adj[k].im;
    }
    delete loc;
  }
  write_raw("adjust.f32", &out[0], sizeof(float) * out.size());
  return 0;
}

// Crava::computeG and Crava::correctAlphaBetaRho (src/crava.cpp:2261-2343, :2471-2569) on the posterior and
// prior-mean cubes post.f32 / mean.f32 (real domain, 3 cubes each), the local noise scales scale.f64 (ntheta x
// ny x nx, the ModelAVODynamic grids), errThetaCov and the prior / posterior variances at the origin.  Writes G
// (ntheta x 3) and the corrected posterior cubes.
int cmd_localnoise()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"], n = (int)p["ntheta"];
  const size_t rsize = (size_t)2 * (nxp / 2 + 1) * nyp * nzp;
  std::vector<double> etc = read_arr<double>("etc.f64", (size_t)n * n);
  std::vector<double> pv0 = read_arr<double>("priorvar0.f64", 9);
  std::vector<double> qv0 = read_arr<double>("postvar0.f64", 9);
  std::vector<double> scale = read_arr<double>("scale.f64", (size_t)n * nx * ny);
  std::vector<float> post = read_arr<float>("post.f32", rsize * 3);
  std::vector<float> mean = read_arr<float>("mean.f32", rsize * 3);

  Crava *crava = static_cast<Crava *>(operator new(sizeof(Crava)));
  memset((void *)crava, 0, sizeof(Crava));
  crava->nx_ = nx;
  crava->ny_ = ny;
  crava->nz_ = nz;
  crava->ntheta_ = n;
  crava->errThetaCov_ = new double *[n];
  for (int l = 0; l < n; l++) {
    crava->errThetaCov_[l] = new double[n];
    for (int m = 0; m < n; m++) crava->errThetaCov_[l][m] = etc[(size_t)l * n + m];
  }
  new (&crava->priorVar0_) NRLib::Matrix(3, 3);
  new (&crava->postVar0_) NRLib::Matrix(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      crava->priorVar0_(a, b) = pv0[3 * a + b];
      crava->postVar0_(a, b) = qv0[3 * a + b];
    }
  FFTGrid **pg[3] = {&crava->postAlpha_, &crava->postBeta_, &crava->postRho_};
  FFTGrid **mg[3] = {&crava->meanAlpha_, &crava->meanBeta_, &crava->meanRho_};
  for (int q = 0; q < 3; q++) {
    *pg[q] = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::PARAMETER, &post[rsize * q], false);
    *mg[q] = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::PARAMETER, &mean[rsize * q], false);
  }
  // the ModelAVODynamic members correctAlphaBetaRho reads: the angles (their count) and the noise-scale grids
  ModelAVODynamic *mad = static_cast<ModelAVODynamic *>(operator new(sizeof(ModelAVODynamic)));
  memset((void *)mad, 0, sizeof(ModelAVODynamic));
  new (&mad->angle_) std::vector<float>(n, 0.0f);
  new (&mad->localNoiseScale_) std::vector<Grid2D *>(n, (Grid2D *)NULL);
  for (int l = 0; l < n; l++) {
    Grid2D *g = new Grid2D(nx, ny, 0.0);
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) (*g)(i, j) = scale[((size_t)l * ny + j) * nx + i];
    mad->localNoiseScale_[l] = g;
  }
  crava->modelAVOdynamic_ = mad;

  NRLib::Matrix G(n, 3);
  crava->computeG(G);
  std::vector<double> gout((size_t)n * 3);
  for (int l = 0; l < n; l++)
    for (int q = 0; q < 3; q++) gout[(size_t)l * 3 + q] = G(l, q);
  write_raw("G.f64", &gout[0], sizeof(double) * gout.size());

  ModelSettings ms;
  ms.nSimulations_ = 0;
  crava->correctAlphaBetaRho(&ms);
  dump_grid("post_alpha.f32", crava->postAlpha_);
  dump_grid("post_beta.f32", crava->postBeta_);
  dump_grid("post_rho.f32", crava->postRho_);
  return 0;
}

// FFTGrid::fillInData (src/fftgrid.cpp:138-370) from a STORM grid (grid.f32, gnk x gny x gnx, a box from
// (gx0, gy0, gz0) of size glx x gly x glz) into a cube on a constant-thickness simbox (x0, y0, top z0, lx x ly x lz,
// rotation rot, cells dx x dy x dz).  Writes the filled cube and, per column c = i + rnxp*j, what the reference's
// own geometry code hands the per-trace core: the trace (makeTraceFromStormGrid), its first-sample time and
// interval, the column's simbox top and cell thickness (getFillNumber, Simbox::getCoord, getdz) and whether the
// column is outside the grid or its trace missing.
int cmd_fillindata()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"];
  const int gnx = (int)p["gnx"], gny = (int)p["gny"], gnk = (int)p["gnk"], cubetype = (int)p["cubetype"];
  const float smooth = (float)p["smooth_length"];
  std::vector<float> vals = read_arr<float>("grid.f32", (size_t)gnx * gny * gnk);
  Surface top(p["x0"], p["y0"], p["lx"], p["ly"], 2, 2, p["z0"]);
  Simbox sb(p["x0"], p["y0"], top, p["lx"], p["ly"], p["lz"], p["rot"], p["dx"], p["dy"], p["dz"]);
  NRLib::Volume vol(p["gx0"], p["gy0"], p["gz0"], p["glx"], p["gly"], p["glz"], p["rot"]);
  StormContGrid grid(vol, gnx, gny, gnk);
  for (int k = 0; k < gnk; k++)
    for (int j = 0; j < gny; j++)
      for (int i = 0; i < gnx; i++) grid(i, j, k) = vals[((size_t)k * gny + j) * gnx + i];

  FFTGrid *fg = new FFTGrid(nx, ny, nz, nxp, nyp, nzp);
  fg->setType(cubetype);
  const int rnxp = 2 * (nxp / 2 + 1), ncol = rnxp * nyp;
  std::vector<float> traces((size_t)ncol * gnk, 0.0f), z0d(ncol, 0.0f), dzd(ncol, 0.0f), z0g(ncol), dzg(ncol);
  std::vector<int> state(ncol, 1);
  for (int j = 0; j < nyp; j++)
    for (int i = 0; i < rnxp; i++) {
      const int c = i + rnxp * j;
      const int refi = fg->getFillNumber(i, nx, nxp), refj = fg->getFillNumber(j, ny, nyp);
      double x, y, z0;
      sb.getCoord(refi, refj, 0, x, y, z0);
      z0g[c] = static_cast<float>(z0);
      dzg[c] = static_cast<float>(sb.getdz(refi, refj));
      const float xf = static_cast<float>(x), yf = static_cast<float>(y);
      if (!grid.IsInside(xf, yf)) continue;
      std::vector<float> tr;
      bool missing = true;
      float z0_data = RMISSING, dz_data = RMISSING, dz_min = RMISSING;
      fg->makeTraceFromStormGrid(&grid, tr, missing, z0_data, dz_data, dz_min, xf, yf);
      if (missing) continue;
      state[c] = 0;
      z0d[c] = z0_data;
      dzd[c] = dz_data;
      for (int k = 0; k < gnk && k < (int)tr.size(); k++) traces[(size_t)c * gnk + k] = tr[k];
    }
  int m1 = 0, m2 = 0, m3 = 0;
  std::string err;
  fg->fillInData(&sb, &grid, NULL, smooth, 1, m1, m2, m3, std::string("data"), err, false, false);
  dump_grid("cube.f32", fg);
  write_raw("traces.f32", &traces[0], sizeof(float) * traces.size());
  write_raw("state.i32", &state[0], sizeof(int) * state.size());
  write_raw("z0_data.f32", &z0d[0], sizeof(float) * ncol);
  write_raw("dz_data.f32", &dzd[0], sizeof(float) * ncol);
  write_raw("z0_grid.f32", &z0g[0], sizeof(float) * ncol);
  write_raw("dz_grid.f32", &dzg[0], sizeof(float) * ncol);
  const int counts[3] = {m1, m2, m3};
  write_raw("counts.i32", counts, sizeof(counts));
  return 0;
}

// Crava::divideDataByScaleWavelet (src/crava.cpp:678-804) on ntheta DATA cubes (data.f32, real domain) over a
// simbox of non-constant thickness: a flat top at z0 and a bottom z0 + lz r(x, y), r given at ni x nj nodes over
// the simbox area (thick.f64, max 1), local wavelet shift and gain grids (shift.f32, gain.f32, ntheta x ny x nx),
// Ricker wavelets built and resampled by the reference (Wavelet1D), the prior temporal correlation of corrt.f32.
// Writes the divided cubes, the simbox's relative thickness at every padded trace, its lz, the wavelets and gain
// grids as Wavelet::setGainGrid leaves them (grid divided by its geometric mean, wavelet multiplied by it) and the
// filtered temporal correlation the adjustment factor used.
int cmd_divide()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"], n = (int)p["ntheta"];
  const int ncorrt = (int)p["ncorrt"], min_int_fq = (int)p["min_int_fq"], ni = (int)p["ni"], nj = (int)p["nj"];
  const float dt = (float)p["dt"], fpeak = (float)p["fpeak"];
  const double dx = p["dx"], dy = p["dy"], z0 = p["z0"];
  const size_t rsize = (size_t)2 * (nxp / 2 + 1) * nyp * nzp;
  std::vector<float> theta = read_arr<float>("theta.f32", n);
  std::vector<float> A = read_arr<float>("A.f32", (size_t)n * 3);
  std::vector<double> etc = read_arr<double>("etc.f64", (size_t)n * n);
  std::vector<float> s0 = read_arr<float>("sigma0.f32", 9);
  std::vector<double> cxy = read_arr<double>("corrxy.f64", (size_t)nxp * nyp);
  std::vector<float> corrT = read_arr<float>("corrt.f32", ncorrt);
  std::vector<float> data = read_arr<float>("data.f32", rsize * n);
  std::vector<double> thick = read_arr<double>("thick.f64", (size_t)ni * nj);
  std::vector<float> shift = read_arr<float>("shift.f32", (size_t)n * nx * ny);
  std::vector<float> gain = read_arr<float>("gain.f32", (size_t)n * nx * ny);

  ModelSettings ms;
  Surface corr_xy(0.0, 0.0, 25.0 * nxp, 25.0 * nyp, nxp, nyp, 0.0);
  for (int j = 0; j < nyp; j++)
    for (int i = 0; i < nxp; i++) corr_xy(i + nxp * j) = cxy[(size_t)j * nxp + i];
  SeismicParametersHolder sp;
  sp.priorVar0_.resize(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) sp.priorVar0_(a, b) = static_cast<double>(s0[3 * a + b]);
  sp.createCorrGrids(nx, ny, nz, nxp, nyp, nzp, false);
  sp.initializeCorrelations(&corr_xy, corrT, 0.0f, 0.0f, min_int_fq, nzp);
  float *filtered = sp.getPriorCorrTFiltered(nz, nzp);
  write_raw("corrt_filtered.f32", filtered, sizeof(float) * nzp);
  delete[] filtered;

  const double lx = dx * nx, ly = dy * ny, lz = (double)nz * dt;
  Surface top(0.0, 0.0, lx, ly, ni, nj, z0);
  Surface bot(0.0, 0.0, lx, ly, ni, nj, z0);
  for (int j = 0; j < nj; j++)
    for (int i = 0; i < ni; i++) bot(i + ni * j) = z0 + lz * thick[(size_t)j * ni + i];
  Simbox sb(0.0, 0.0, top, lx, ly, lz, 0.0, dx, dy, (double)dt);
  sb.setDepth(top, bot, nz);
  std::vector<double> rel((size_t)nxp * nyp);
  for (int j = 0; j < nyp; j++)
    for (int i = 0; i < nxp; i++) rel[(size_t)j * nxp + i] = sb.getRelThick(i, j);
  write_raw("relthick.f64", &rel[0], sizeof(double) * rel.size());
  const double lz_box = sb.getlz();
  write_raw("lz.f64", &lz_box, sizeof(double));

  Crava *crava = static_cast<Crava *>(operator new(sizeof(Crava)));
  memset((void *)crava, 0, sizeof(Crava));
  crava->nx_ = nx;
  crava->ny_ = ny;
  crava->nz_ = nz;
  crava->nxp_ = nxp;
  crava->nyp_ = nyp;
  crava->nzp_ = nzp;
  crava->ntheta_ = n;
  crava->lowCut_ = (float)p["low_cut"];
  crava->highCut_ = (float)p["high_cut"];
  crava->wnc_ = (float)p["wnc"];
  crava->energyTreshold_ = (float)p["energy_threshold"];
  crava->simbox_ = &sb;
  new (&crava->priorVar0_) NRLib::Matrix(3, 3);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) crava->priorVar0_(a, b) = static_cast<double>(s0[3 * a + b]);
  crava->thetaDeg_ = new float[n];
  crava->A_ = new float *[n];
  crava->errThetaCov_ = new double *[n];
  crava->seisWavelet_ = new Wavelet *[n];
  crava->seisData_ = new FFTGrid *[n];
  std::vector<float> wavs((size_t)n * nzp);
  for (int l = 0; l < n; l++) {
    crava->thetaDeg_[l] = theta[l];
    crava->A_[l] = new float[3];
    for (int q = 0; q < 3; q++) crava->A_[l][q] = A[(size_t)l * 3 + q];
    crava->errThetaCov_[l] = new double[n];
    for (int m = 0; m < n; m++) crava->errThetaCov_[l][m] = etc[(size_t)l * n + m];
    int err = 0;
    Wavelet1D *w = new Wavelet1D(&ms, crava->A_[l], theta[l], fpeak, err);
    if (err) { fprintf(stderr, "wavelet: error %d\n", err); return 3; }
    w->resample(dt, nz, nzp);
    Grid2D *gs = new Grid2D(nx, ny, 0.0), *gg = new Grid2D(nx, ny, 1.0);
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        (*gs)(i, j) = shift[((size_t)l * ny + j) * nx + i];
        (*gg)(i, j) = gain[((size_t)l * ny + j) * nx + i];
      }
    w->setShiftGrid(gs);
    w->setGainGrid(gg);  // divides the grid by its geometric mean and multiplies the wavelet by it
    // the wavelet (time domain) and the gain grid as the division sees them
    Wavelet1D wt(w);
    if (!wt.isReal_) wt.invFFT1DInPlace();
    for (int k = 0; k < nzp; k++) wavs[(size_t)l * nzp + k] = wt.rAmp_[k];
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) gain[((size_t)l * ny + j) * nx + i] = (float)(*gg)(i, j);
    crava->seisWavelet_[l] = w;
    crava->seisData_[l] = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::DATA, &data[rsize * l], false);
  }
  write_raw("wavelets.f32", &wavs[0], sizeof(float) * wavs.size());
  write_raw("gain_normalised.f32", &gain[0], sizeof(float) * gain.size());
  crava->divideDataByScaleWavelet(sp);
  for (int l = 0; l < n; l++) dump_grid("out" + NRLib::ToString(l) + ".f32", crava->seisData_[l]);
  // the inverse step, as it runs on the residuals before they are written: the divided cubes are
  // transformed (the state the bin loop leaves them in) and handed to
  // Crava::multiplyDataByScaleWaveletAndWriteToFile (src/crava.cpp:906-968); with no output format set
  // (FFTGrid::formatFlag_ = 0) its writeFile writes nothing
  for (int l = 0; l < n; l++) {
    crava->seisData_[l]->setAccessMode(FFTGrid::RANDOMACCESS);
    crava->seisData_[l]->fftInPlace();
    crava->seisData_[l]->endAccess();
  }
  FFTGrid::formatFlag_ = 0;
  crava->multiplyDataByScaleWaveletAndWriteToFile("residuals");
  for (int l = 0; l < n; l++) dump_grid("mult" + NRLib::ToString(l) + ".f32", crava->seisData_[l]);
  return 0;
}

// FFTGrid::interpolateSeismic (src/fftgrid.cpp:2576-2738) on the DATA cube cube.f32 (real domain) with the
// energy threshold of params.txt; writes the result
int cmd_interpolate()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nz = (int)p["nz"];
  const int nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"];
  const size_t rsize = (size_t)2 * (nxp / 2 + 1) * nyp * nzp;
  std::vector<float> cube = read_arr<float>("cube.f32", rsize);
  FFTGrid *g = make_grid(nx, ny, nz, nxp, nyp, nzp, FFTGrid::DATA, &cube[0], false);
  g->interpolateSeismic((float)p["threshold"]);
  dump_grid("out.f32", g);
  return 0;
}

// FFTGrid::writeCravaFile (src/fftgrid.cpp:2410-2441) of the cube cube.f32 with the geometry of params.txt
int cmd_crava_write()
{
  std::map<std::string, double> p = read_params();
  const int nx = (int)p["nx"], ny = (int)p["ny"], nxp = (int)p["nxp"], nyp = (int)p["nyp"], nzp = (int)p["nzp"];
  FFTGrid *g = make_grid(nx, ny, nzp, nxp, nyp, nzp, FFTGrid::PARAMETER, NULL, false);
  std::vector<float> v = read_arr<float>("cube.f32", (size_t)g->rsize_);
  memcpy(g->rvalue_, &v[0], sizeof(float) * v.size());
  Simbox sb;
  sb.x_min_ = p["x0"];
  sb.y_min_ = p["y0"];
  sb.dx_ = p["dx"];
  sb.dy_ = p["dy"];
  sb.nx_ = nx;
  sb.ny_ = ny;
  sb.inLine0_ = p["il0"];
  sb.crossLine0_ = p["xl0"];
  sb.ilStepX_ = p["ilstepx"];
  sb.ilStepY_ = p["ilstepy"];
  sb.xlStepX_ = p["xlstepx"];
  sb.xlStepY_ = p["xlstepy"];
  sb.angle_ = p["angle"];
  g->writeCravaFile(g_dir + "/out", &sb);
  return 0;
}

// FFTGrid::readCravaFile (src/fftgrid.cpp:2445-2493) of in.crava into a grid of the params.txt size
int cmd_crava_read()
{
  std::map<std::string, double> p = read_params();
  FFTGrid *g = new FFTGrid((int)p["nxp"], (int)p["nyp"], (int)p["nzp"], (int)p["nxp"], (int)p["nyp"], (int)p["nzp"]);
  std::string err;
  g->readCravaFile(g_dir + "/in.crava", err, false);
  if (!err.empty()) {
    std::ofstream f((g_dir + "/error.txt").c_str());
    f << err;
    return 0;
  }
  dump_grid("cube_read.f32", g);
  return 0;
}

// NRLib::StormContGrid::WriteToFile (libs/nrlib/stormgrid/stormcontgrid.cpp:169-205) of values.f32 with
// constant surfaces
int cmd_storm_write()
{
  std::map<std::string, double> p = read_params();
  const size_t ni = (size_t)p["ni"], nj = (size_t)p["nj"], nk = (size_t)p["nk"];
  std::vector<float> v = read_arr<float>("values.f32", ni * nj * nk);
  NRLib::StormContGrid g(ni, nj, nk);
  g.SetDimensions(p["x_min"], p["y_min"], p["lx"], p["ly"]);
  g.SetAngle(p["angle_deg"] * NRLib::Pi / 180.0);
  g.SetSurfaces(NRLib::ConstantSurface<double>(p["z_top"]), NRLib::ConstantSurface<double>(p["z_bot"]),
                NRLib::ConstantSurface<double>(p["erosion_top"]), NRLib::ConstantSurface<double>(p["erosion_bot"]));
  g.SetZoneNumber((int)p["zone"]);
  g.SetModelFileName("ModelFile");
  g.SetMissingCode((float)p["missing"]);
  g.SetVariableName("Vp");
  std::copy(v.begin(), v.end(), g.begin());
  g.WriteToFile(g_dir + "/out.storm");
  return 0;
}

// NRLib::StormContGrid::ReadFromFile (libs/nrlib/stormgrid/stormcontgrid.cpp:72-165) of in.storm
int cmd_storm_read()
{
  NRLib::StormContGrid g;
  g.ReadFromFile(g_dir + "/in.storm");
  std::vector<float> v(g.begin(), g.end());
  write_raw("values_read.f32", &v[0], sizeof(float) * v.size());
  std::ofstream f((g_dir + "/header.txt").c_str());
  f.precision(17);
  f << "ni " << g.GetNI() << "\nnj " << g.GetNJ() << "\nnk " << g.GetNK() << "\nzone " << g.GetZoneNumber()
    << "\nmissing " << g.GetMissingCode() << "\nx_min " << g.GetXMin() << "\ny_min " << g.GetYMin()
    << "\nlx " << g.GetLX() << "\nly " << g.GetLY() << "\nlz " << g.GetLZ() << "\nangle " << g.GetAngle()
    << "\nz_top " << g.GetTopSurface().GetZ(0.0, 0.0) << "\nz_bot " << g.GetBotSurface().GetZ(0.0, 0.0) << "\n";
  return 0;
}

// StormContGrid::WriteToFile of values.f32 whose top and bottom surfaces are regular surfaces (top.f64,
// bot.f64: surf_ni x surf_nj nodes over [sx_min, sx_min + slx] x [sy_min, sy_min + sly]) and whose erosion
// surfaces are constants: out.storm plus the surface files the writer puts beside it (out.storm_top,
// out.storm_bot, WriteStormBinarySurf)
int cmd_storm_write_surf()
{
  std::map<std::string, double> p = read_params();
  const size_t ni = (size_t)p["ni"], nj = (size_t)p["nj"], nk = (size_t)p["nk"];
  const size_t sni = (size_t)p["surf_ni"], snj = (size_t)p["surf_nj"];
  std::vector<float> v = read_arr<float>("values.f32", ni * nj * nk);
  std::vector<double> top = read_arr<double>("top.f64", sni * snj), bot = read_arr<double>("bot.f64", sni * snj);
  NRLib::RegularSurface<double> st(p["sx_min"], p["sy_min"], p["slx"], p["sly"], sni, snj, 0.0);
  NRLib::RegularSurface<double> sb(p["sx_min"], p["sy_min"], p["slx"], p["sly"], sni, snj, 0.0);
  std::copy(top.begin(), top.end(), st.begin());
  std::copy(bot.begin(), bot.end(), sb.begin());
  NRLib::StormContGrid g(ni, nj, nk);
  g.SetDimensions(p["x_min"], p["y_min"], p["lx"], p["ly"]);
  g.SetAngle(p["angle_deg"] * NRLib::Pi / 180.0);
  g.SetSurfaces(st, sb, NRLib::ConstantSurface<double>(p["erosion_top"]),
                NRLib::ConstantSurface<double>(p["erosion_bot"]));
  g.SetZoneNumber((int)p["zone"]);
  g.SetModelFileName("ModelFile");
  g.SetMissingCode((float)p["missing"]);
  g.SetVariableName("Vp");
  std::copy(v.begin(), v.end(), g.begin());
  g.WriteToFile(g_dir + "/out.storm");
  return 0;
}

// StormContGrid::ReadFromFile of in.storm, whose top and bottom surfaces are files beside it: the values,
// and the two surfaces as the reader loaded them (nodes and geometry)
int cmd_storm_read_surf()
{
  NRLib::StormContGrid g;
  g.ReadFromFile(g_dir + "/in.storm");
  std::vector<float> v(g.begin(), g.end());
  write_raw("values_read.f32", &v[0], sizeof(float) * v.size());
  const NRLib::Surface<double> *surf[2] = {&g.GetTopSurface(), &g.GetBotSurface()};
  const char *name[2] = {"top", "bot"};
  for (int q = 0; q < 2; q++) {
    const NRLib::RegularSurface<double> *rs = dynamic_cast<const NRLib::RegularSurface<double> *>(surf[q]);
    if (!rs) { fprintf(stderr, "%s surface is not a regular surface\n", name[q]); return 3; }
    std::vector<double> z(rs->begin(), rs->end());
    write_raw(std::string(name[q]) + "_read.f64", &z[0], sizeof(double) * z.size());
    const double geom[6] = {(double)rs->GetNI(), (double)rs->GetNJ(), rs->GetXMin(), rs->GetYMin(),
                            rs->GetXMax() - rs->GetXMin(), rs->GetYMax() - rs->GetYMin()};
    write_raw(std::string(name[q]) + "_geom.f64", geom, sizeof(geom));
  }
  return 0;
}

int cmd_factorable()
{
  std::map<std::string, double> p = read_params();
  const int n = (int)p["count"];
  std::vector<int> in = read_arr<int>("n.i32", n), out(n);
  for (int i = 0; i < n; i++) out[i] = FFTGrid::findClosestFactorableNumber(in[i]);
  write_raw("factorable.i32", &out[0], sizeof(int) * n);
  return 0;
}

}  // namespace

// a reference code path that reaches a left-out routine stops with a backtrace instead of silently
void on_fault(int sig)
{
  void *frames[64];
  const int n = backtrace(frames, 64);
  fprintf(stderr, "crava_o2: signal %d\n", sig);
  backtrace_symbols_fd(frames, n, 2);
  _exit(128 + sig);
}

int main(int argc, char **argv)
{
  signal(SIGSEGV, on_fault);
  signal(SIGABRT, on_fault);
  if (argc != 3) {
    fprintf(stderr, "usage: crava_o2 {inversion|state4d|adjust|localnoise|fillindata|interpolate|divide|crava_write|crava_read|storm_write|storm_read|"
                    "factorable} <dir>\n");
    return 1;
  }
  g_dir = argv[2];
  const std::string c = argv[1];
  if (c == "inversion") return cmd_inversion();
  if (c == "state4d") return cmd_state4d();
  if (c == "factorable") return cmd_factorable();
  if (c == "adjust") return cmd_adjust();
  if (c == "localnoise") return cmd_localnoise();
  if (c == "fillindata") return cmd_fillindata();
  if (c == "interpolate") return cmd_interpolate();
  if (c == "divide") return cmd_divide();
  if (c == "storm_write_surf") return cmd_storm_write_surf();
  if (c == "state4d_evolve") return cmd_state4d_evolve();
  if (c == "storm_read_surf") return cmd_storm_read_surf();
  if (c == "crava_write") return cmd_crava_write();
  if (c == "crava_read") return cmd_crava_read();
  if (c == "storm_write") return cmd_storm_write();
  if (c == "storm_read") return cmd_storm_read();
  fprintf(stderr, "unknown command %s\n", c.c_str());
  return 1;
}

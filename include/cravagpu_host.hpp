// cravagpu_host.hpp -- C++ host layer over the cravagpu C-ABI, mirroring the
// reference's FFTGrid / Crava calling surface for the inversion path.
//
//   cravagpu::FFTGrid  -- a padded cube resident in GPU memory with the
//                         reference FFTGrid's layout, cube types, in-place
//                         fftInPlace / invFFTInPlace (src/fftgrid.h:160-161),
//                         get/setComplexValue, multiplyByScalar, add,
//                         fillInParamCorr / fillInErrCorr.
//   cravagpu::Crava    -- computePostMeanResidAndFFTCov (src/crava.h:43-64)
//                         and simulate (src/crava.h:154) on FFTGrids, with the
//                         model objects (Simbox, SeismicParametersHolder,
//                         Wavelet) replaced by the plain arrays they hold.
//
// Errors are reported as exceptions (cravagpu::Error) carrying the C-ABI
// status and text; nothing calls exit().
#ifndef CRAVAGPU_HOST_HPP
#define CRAVAGPU_HOST_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "cravagpu.h"

namespace cravagpu {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &what) : std::runtime_error(what), status(s) {}
};

void check(int status, const char *what);

struct Complex {
  float re, im;
};

class FFTGrid {
 public:
  enum gridTypes { CTMISSING, DATA, PARAMETER, COVARIANCE, VELOCITY, OPERATOR };

  FFTGrid(int nx, int ny, int nz, int nxp, int nyp, int nzp);
  ~FFTGrid();
  FFTGrid(const FFTGrid &) = delete;
  FFTGrid &operator=(const FFTGrid &) = delete;

  void setType(int cubetype) { cubetype_ = cubetype; }
  int getType() const { return cubetype_; }
  bool getIsTransformed() const { return istransformed_; }
  void setTransformedStatus(bool s) { istransformed_ = s; }

  int getNx() const { return nx_; }
  int getNy() const { return ny_; }
  int getNz() const { return nz_; }
  int getNxp() const { return nxp_; }
  int getNyp() const { return nyp_; }
  int getNzp() const { return nzp_; }
  int getCNxp() const { return nxp_ / 2 + 1; }
  int getRNxp() const { return 2 * (nxp_ / 2 + 1); }
  long getcsize() const { return (long)getCNxp() * nyp_ * nzp_; }
  long getrsize() const { return (long)getRNxp() * nyp_ * nzp_; }

  void fftInPlace(void *stream = nullptr);
  void invFFTInPlace(void *stream = nullptr);

  // bulk host <-> device transfers of the whole padded buffer (rsize floats)
  void fillInFromArray(const float *host_rsize);
  void copyToArray(float *host_rsize) const;

  Complex getComplexValue(int i, int j, int k, bool extSimbox = false) const;
  int setComplexValue(int i, int j, int k, Complex value, bool extSimbox = false);
  float getRealValue(int i, int j, int k, bool extSimbox = false) const;
  int setRealValue(int i, int j, int k, float value, bool extSimbox = false);

  void multiplyByScalar(float scalar, void *stream = nullptr);
  void add(const FFTGrid *other, void *stream = nullptr);
  void fillInParamCorr(const float *corr_xy_dev, const float *circ_corr_t_dev, float gradI, float gradJ,
                       void *stream = nullptr);
  void fillInErrCorr(const float *corr_xy_dev, float gradI, float gradJ, void *stream = nullptr);

  float *devicePtr() { return d_; }
  const float *devicePtr() const { return d_; }

 private:
  int nx_, ny_, nz_, nxp_, nyp_, nzp_;
  int cubetype_ = CTMISSING;
  bool istransformed_ = false;
  float *d_ = nullptr;
};

// The model pieces computePostMeanResidAndFFTCov reads from ModelGeneral,
// Simbox, SeismicParametersHolder and the Wavelet objects.
struct InversionModel {
  int ntheta = 0;
  std::vector<float> wavelets;       // ntheta * nzp, resampled, FFT order
  std::vector<float> A;              // ntheta * 3
  std::vector<double> errThetaCov;   // ntheta * ntheta
  std::vector<double> sigma0;        // 9 (priorVar0)
  std::vector<float> corrXY;         // nyp * nxp (ModelGeneral::findCorrXYGrid)
  std::vector<float> circCorrT;      // nzp (computeCircCorrT)
  float corrGradI = 0, corrGradJ = 0;
  float wnc = 0.1f, lowCut = 5.0f, highCut = 55.0f;
  float dt_ms = 4.0f, minRelThick = 1.0f;
  double condThreshold = 0;          // CG_PREC_MIXED guard (0 = default)
};

class Crava {
 public:
  enum Form { PLAIN = 0, FUSED_FP32 = 1, FUSED_MIXED = 2 };

  Crava(int nx, int ny, int nz, int nxp, int nyp, int nzp, const InversionModel &model);
  ~Crava();

  // The bin loop and the transforms around it, as Crava::computePostMeanResidAndFFTCov
  // (src/crava.cpp:975-1285): seisData (ntheta real DATA cubes) become the
  // residual spectra, postAlpha/Beta/Rho (real prior-mean cubes) the
  // real-domain posterior means, postCov[6] the posterior covariance spectra.
  // The plain form also needs the 6 prior covariance cubes and errCorr in the
  // real domain (it transforms them, as FFTCovGrids does).  binsDone, when
  // given (a cudaEvent_t), is recorded on the stream once the residual and
  // covariance spectra are final, before the posterior-mean inverse
  // transforms: a caller can start copying those cubes out from then on.
  int computePostMeanResidAndFFTCov(FFTGrid **seisData, FFTGrid *&postAlpha, FFTGrid *&postBeta,
                                    FFTGrid *&postRho, FFTGrid **postCov, FFTGrid *errCorr, Form form,
                                    void *stream = nullptr, void *binsDone = nullptr);

  // Crava::simulate (src/crava.cpp:1551-1734) for nSim realisations, written
  // to fields[3*r + p]; the posterior covariance spectra are factored once.
  int simulate(FFTGrid **postCov, FFTGrid *const *postMean, int nSim, unsigned long long seed, FFTGrid **fields,
               void *stream = nullptr);

  cg_workspace workspace() { return ws_; }
  const std::vector<unsigned char> &band() const { return band_; }

 private:
  int nx_, ny_, nz_, nxp_, nyp_, nzp_;
  InversionModel m_;
  cg_workspace ws_ = nullptr;
  float *d_corr_xy_ = nullptr, *d_circ_t_ = nullptr, *d_chol_ = nullptr;
  std::vector<unsigned char> band_;
};

}  // namespace cravagpu

#endif

// Per-frequency-bin posterior: tables and device math shared by the kernels.
#pragma once

#include "common.cuh"

namespace cg {

constexpr int kMaxTheta = 8;
constexpr int kTri = kMaxTheta * (kMaxTheta + 1) / 2;
constexpr double kCholTol = 1e-20;  // lib_matr.c:19, applied to the pivots scaled by A00
constexpr int kCondBucketsMax = 32;  // buckets of cg_condition_histogram

__host__ __device__ constexpr int tri(int l, int m) { return l * (l + 1) / 2 + m; }  // l >= m

// Per temporal-frequency tables.  For one k (constant-thickness branch of
// Crava::fillErrMultVectors, src/crava.cpp:1337-1361, and getNextErrorVariance,
// src/crava.cpp:1442-1469), with S0 the 3x3 prior and lam the per-(i,j)
// error-correlation eigenvalue:
//   K      forward operator kD(k) conj(W_l(k)) A_l            (ntheta x 3)
//   KS0    K S0                                               (ntheta x 3)
//   M      K S0 K^H                                           (lower, packed)
//   E      0.5 (1-wnc) errThetaCov (e1 e1^H + e2 e2^H)        (lower, packed)
//   D      wnc errThetaCov_ll |Re e3_l|^2                     (diagonal)
// so that for a bin with prior scale s and error eigenvalue lam the data
// covariance is  Sd = s M + lam E + diag(D).
template <typename T>
struct KTab {
  C2<T> K[kMaxTheta][3];
  C2<T> KS0[kMaxTheta][3];
  C2<T> M[kTri];
  C2<T> E[kTri];
  T D[kMaxTheta];
  int band;
  int pad_[3];
};

// Per-k tables of the information form of the fused bin solve (FP32).  With
// D^-1/2 E D^-1/2 = U diag(mu) U^H and v_m = D^-1/2 u_m, g_m = K^H v_m:
//   (lam E + D)^-1 = sum_m v_m v_m^H / (lam mu_m + 1),
//   S+ = (Sigma0^-1 / s + sum_m g_m g_m^H / (lam mu_m + 1))^-1,
//   mu+ = mu + S+ sum_m g_m (v_m^H (d - K mu)) / (lam mu_m + 1).
struct ITab {
  float2 K[kMaxTheta][3];
  float2 V[kMaxTheta][kMaxTheta];  // V[l][m]: component l of v_m
  float2 G[kMaxTheta][3];          // G[m][p] = (K^H v_m)[p]
  float P[kMaxTheta][9];           // g_m g_m^H: 00 11 22, then 01 02 12 as (re, im)
  float mu[kMaxTheta];
  int band;
  int pad_[3];
};

// Arguments of the per-model set-up kernel (prep.cu): the uploaded
// reference-order tables in, the per-k tables out.
struct PrepArgs {
  int nt;
  int nzp;
  int sym;  // the tables of plane nzp-k are the conjugates of plane k's: compute k <= nzp/2 only
  float wnc;
  int is4d;
  const float2 *K, *em1, *em2, *em3;
  const unsigned char *band;
  const double *etc;
  double s0[9];  // float(priorVar0) widened, row-major
  KTab<float> *tf;
  KTab<double> *td;
  ITab *ti;
};
// queues the set-up kernel over nplanes planes (prep.cu)
int launch_prep_model(const PrepArgs &p, int nplanes, cudaStream_t st);

// Opaque workspace behind cg_workspace (device buffers of one model).
struct Workspace {
  int device;
  int nxp, nyp, nzp, ntheta;
  float wnc;
  int is4d;
  double sigma0[9];
  float sigma0f[9];
  double etc_host[kMaxTheta * kMaxTheta];  // errThetaCov, host copy (per-launch constants)
  double cond_threshold;
  // per-model tables (device)
  KTab<float> *ktab_f;
  KTab<double> *ktab_d;
  // uploaded model tables: one device block and its pinned host staging copy
  // (one host-to-device copy per model; the event marks when the staging
  // copy may be rewritten)
  void *model_dev;
  void *model_host;
  size_t model_bytes;
  cudaEvent_t model_copied;
  float2 *K;        // nzp*ntheta*3 (reference-order tables for the plain path)
  float2 *em1, *em2, *em3;
  unsigned char *band;
  double *etc;      // ntheta*ntheta
  // separable prior spectra (device), rebuilt by every fused inversion
  float *cxy_f;     // real staging rnxp*nyp -> complex cnxp*nyp
  float *ct_f;      // real staging 2*(nzp/2+1) -> complex nzp/2+1
  double *cxy_d;
  double *ct_d;
  // per-bin (|Re P|, |Re E|) table of a prior with correlation gradients
  // (cg_prior_spectra_grad), allocated on first use; used while sl_on
  float2 *sl_f;
  double2 *sl_d;
  bool sl_on, sl_d_on;
  // mixed-precision fix-up queue and counters (device)
  int *queue;
  int queue_cap;
  int *counters;    // [0] flagged, [1] failed cholesky, [2] queue overflow
  long inband_bins;  // bins whose k is inside the inversion band
  // information-form tables (valid when every in-band D > 0 and the model is 3D)
  ITab *itab;
  bool info_ok;
  float sig0inv[6];  // Sigma0^-1 in bin order 00 11 22 01 02 12
  bool model_set;
};

}  // namespace cg

// the C-ABI handle is the workspace itself
struct cg_workspace_s : public cg::Workspace {};

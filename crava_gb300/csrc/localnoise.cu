// Local-noise correction of the posterior means (Crava::correctAlphaBetaRho,
// src/crava.cpp:2471-2569, with newPosteriorCovPointwise, :2345-2451) and the
// local-noise step of simulation (Crava::simulate, :1686-1700).
//
// With local noise the error covariance of trace (i, j) is D Σe D, D =
// diag(sqrt(scale_l(i, j) / min scale_l)).  Per trace, in double:
//   H        = G Σm Gᵀ + D Σe D                     (ntheta × ntheta)
//   Δ        = Σm Gᵀ H⁺ G Σm,  H⁺ = Σ_{λ > 1e-8} v vᵀ / λ
//   sigmanew = Δ^½ (Σm − Σpost)^-½   (the latter robust: λ > 1e-7)
//   sigmamd  = (Σm − Δ)^½ Σpost^-½   (optional, for simulation)
// and every simbox cell becomes μ + sigmanew (post − μ) (μ: prior mean).  G
// (ntheta × 3, Crava::computeG) is an input: it is built from eigenvectors of
// a 3×3 matrix whose signs are the LAPACK routine's choice, and the
// correction depends on them, so the caller supplies the G its eigen solver
// gives.  Everything else here is invariant to eigenvector signs (only
// V f(Λ) Vᵀ products are formed), so a Jacobi solver gives the reference's
// matrices to rounding.  One thread per trace for the matrices (FP64), one per
// cell for the update.
#include <cmath>

#include "common.cuh"
#include "posterior.cuh"
#include "trace.cuh"

namespace cg {
namespace {

constexpr int kLnMax = kMaxTheta;

struct CubeSet3 {
  float *p[3];
};

struct LnArgs {
  double gsg[kLnMax * kLnMax];  // G Σm Gᵀ
  double sgt[3 * kLnMax];       // Σm Gᵀ (row-major 3 × n)
  double etc[kLnMax * kLnMax];  // Σe
  double sdinv[9];              // (Σm − Σpost)^-½, robust
  double pvinv[9];              // Σpost^-½
  double sm[9];                 // Σm
  int n;
};

// Cyclic Jacobi eigen-decomposition of a symmetric n × n matrix (row-major,
// destroyed): eigenvalues on the diagonal of a, eigenvectors in the columns
// of v.  Rotation angle from the standard stable form t = sgn(θ)/(|θ| +
// sqrt(θ² + 1)), θ = (a_qq − a_pp) / (2 a_pq).
__host__ __device__ inline void jacobi_eig(double *a, double *v, int n)
{
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) v[i * n + j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < n; p++) {
      diag += a[p * n + p] * a[p * n + p];
      for (int q = p + 1; q < n; q++) off += a[p * n + q] * a[p * n + q];
    }
    if (off <= 1e-32 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = a[p * n + q];
        if (apq == 0.0) continue;
        const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {  // columns p, q
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {  // rows p, q
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
}

// out = V f(Λ) Vᵀ for a symmetric 3 × 3 matrix; mode 0: f = sqrt on λ > 0,
// mode 1: f = 1/sqrt on λ > thr
__host__ __device__ inline void sym3_fun(const double *m, double *out, int mode, double thr)
{
  double a[9], v[9];
  for (int i = 0; i < 9; i++) a[i] = m[i];
  jacobi_eig(a, v, 3);
  double f[3];
  for (int i = 0; i < 3; i++) {
    const double l = a[i * 3 + i];
    f[i] = mode == 0 ? (l > 0.0 ? sqrt(l) : 0.0) : (l > thr ? 1.0 / sqrt(l) : 0.0);
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += v[r * 3 + k] * f[k] * v[c * 3 + k];
      out[r * 3 + c] = s;
    }
}

__host__ __device__ inline void mul3(const double *a, const double *b, double *out)
{
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += a[r * 3 + k] * b[k * 3 + c];
      out[r * 3 + c] = s;
    }
}

// Grid2D::FindMin(RMISSING) of each angle's scale grid (one block per angle)
__global__ void k_ln_min(const double *__restrict__ scale, int nxy, double *__restrict__ mins)
{
  const int l = blockIdx.x;
  const double *g = scale + (long)l * nxy;
  const double miss = (double)kRMissing;
  double m = INFINITY;
  for (int t = threadIdx.x; t < nxy; t += blockDim.x)
    if (g[t] != miss && g[t] < m) m = g[t];
  __shared__ double red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && red[threadIdx.x + s] < red[threadIdx.x]) red[threadIdx.x] = red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) mins[l] = red[0] == INFINITY ? miss : red[0];
}

__global__ void __launch_bounds__(128) k_ln_matrices(LnArgs a, const double *__restrict__ scale,
                                                     const double *__restrict__ mins, int nx, int ny,
                                                     double *__restrict__ sigmanew, double *__restrict__ sigmamd)
{
  const long ntr = (long)nx * ny;
  const int n = a.n;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ntr; t += (long)gridDim.x * blockDim.x) {
    double d[kLnMax], h[kLnMax * kLnMax], v[kLnMax * kLnMax];
    // a missing scale (RMISSING; the reference's result is NaN there) counts as the minimum
    for (int l = 0; l < n; l++) {
      const double sv = scale[(long)l * ntr + t];
      d[l] = sv == (double)kRMissing ? 1.0 : sqrt(sv / mins[l]);
    }
    for (int l = 0; l < n; l++)
      for (int m = 0; m < n; m++) h[l * n + m] = a.gsg[l * n + m] + (d[l] * a.etc[l * n + m]) * d[m];
    jacobi_eig(h, v, n);
    // Δ = Σm Gᵀ H⁺ G Σm = Σ_{λ > 1e-8} (Σm Gᵀ v)(Σm Gᵀ v)ᵀ / λ
    double delta[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = 0; e < n; e++) {
      const double lam = h[e * n + e];
      if (!(lam > 1e-8)) continue;
      double w[3];
      for (int r = 0; r < 3; r++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += a.sgt[r * n + k] * v[k * n + e];
        w[r] = s;
      }
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) delta[r * 3 + c] += w[r] * w[c] / lam;
    }
    double dsq[9], out[9];
    sym3_fun(delta, dsq, 0, 0.0);
    mul3(dsq, a.sdinv, out);
    for (int i = 0; i < 9; i++) sigmanew[t * 9 + i] = out[i];
    if (sigmamd) {
      double post[9], psq[9];
      for (int i = 0; i < 9; i++) post[i] = a.sm[i] - delta[i];
      sym3_fun(post, psq, 0, 0.0);
      mul3(psq, a.pvinv, out);
      for (int i = 0; i < 9; i++) sigmamd[t * 9 + i] = out[i];
    }
  }
}

// y = mean + M (x − mean) on simbox cells (correctAlphaBetaRho's trace loop, :2538-2550)
__global__ void k_ln_correct(CubeSet3 post, CubeSet3 mean, const double *__restrict__ mats, int nx, int ny, int nz,
                             int nxp, int nyp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long total = (long)nx * ny * nz;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % nx);
    const long r = idx / nx;
    const int j = (int)(r % ny), k = (int)(r / ny);
    const long o = ((long)k * nyp + j) * rnxp + i;
    const double *m = mats + ((long)j * nx + i) * 9;
    const float ma = mean.p[0][o], mb = mean.p[1][o], mc = mean.p[2][o];
    const float da = post.p[0][o] - ma, db = post.p[1][o] - mb, dc = post.p[2][o] - mc;
    post.p[0][o] = (float)((double)ma + m[0] * da + m[1] * db + m[2] * dc);
    post.p[1][o] = (float)((double)mb + m[3] * da + m[4] * db + m[5] * dc);
    post.p[2][o] = (float)((double)mc + m[6] * da + m[7] * db + m[8] * dc);
  }
}

// simulation with local noise: simbox cells x -> M x, then every cell + mean
__global__ void k_ln_fields(CubeSet3 f, CubeSet3 mean, int has_mean, const double *__restrict__ mats, int nx, int ny,
                            int nz, int nxp, int nyp, int nzp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long total = (long)nxp * nyp * nzp;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % nxp);
    const long r = idx / nxp;
    const int j = (int)(r % nyp), k = (int)(r / nyp);
    const long o = ((long)k * nyp + j) * rnxp + i;
    float a = f.p[0][o], b = f.p[1][o], c = f.p[2][o];
    if (i < nx && j < ny && k < nz) {
      const double *m = mats + ((long)j * nx + i) * 9;
      const float na = (float)(m[0] * a + m[1] * b + m[2] * c);
      const float nb = (float)(m[3] * a + m[4] * b + m[5] * c);
      const float nc = (float)(m[6] * a + m[7] * b + m[8] * c);
      a = na; b = nb; c = nc;
    }
    if (has_mean) {
      a += mean.p[0][o];
      b += mean.p[1][o];
      c += mean.p[2][o];
    }
    f.p[0][o] = a;
    f.p[1][o] = b;
    f.p[2][o] = c;
  }
}

int grid_ln(long n)
{
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    nsm = 152;
  const long want = (n + 255) / 256;
  return (int)(want < 16L * nsm ? (want > 0 ? want : 1) : 16L * nsm);
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" int cg_correct_alpha_beta_rho(float *const *post, const float *const *mean, int nx, int ny, int nz, int nxp,
                                         int nyp, int nzp, int ntheta, const double *G, const double *err_theta_cov,
                                         const double *prior_var0, const double *post_var0,
                                         const double *noise_scale, double *sigmamd, void *stream)
{
  if (!post || !mean || !G || !err_theta_cov || !prior_var0 || !post_var0 || !noise_scale || ntheta < 1 ||
      ntheta > kLnMax || nx < 1 || ny < 1 || nz < 1 || nx > nxp || ny > nyp || nz > nzp) {
    set_error("cg_correct_alpha_beta_rho: bad argument");
    return CG_ERR_ARG;
  }
  CubeSet3 P, M;
  for (int p = 0; p < 3; p++) {
    if (!post[p] || !mean[p]) { set_error("cg_correct_alpha_beta_rho: null cube %d", p); return CG_ERR_ARG; }
    P.p[p] = post[p];
    M.p[p] = const_cast<float *>(mean[p]);
  }
  // per-model matrices (host, double)
  const int n = ntheta;
  LnArgs a;
  a.n = n;
  for (int i = 0; i < 9; i++) a.sm[i] = prior_var0[i];
  for (int r = 0; r < 3; r++)
    for (int l = 0; l < n; l++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += prior_var0[r * 3 + k] * G[l * 3 + k];
      a.sgt[r * n + l] = s;
    }
  for (int l = 0; l < n; l++)
    for (int m = 0; m < n; m++) {
      double s = 0.0;
      for (int r = 0; r < 3; r++) s += G[l * 3 + r] * a.sgt[r * n + m];
      a.gsg[l * n + m] = s;
      a.etc[l * n + m] = err_theta_cov[l * n + m];
    }
  double sdelta[9];
  for (int i = 0; i < 9; i++) sdelta[i] = prior_var0[i] - post_var0[i];
  sym3_fun(sdelta, a.sdinv, 1, 1e-7);
  sym3_fun(post_var0, a.pvinv, 1, 0.0);
  cudaStream_t st = (cudaStream_t)stream;
  const long ntr = (long)nx * ny;
  double *mins = nullptr, *mats = nullptr;
  CG_CUDA(scratch_alloc((void **)&mins, sizeof(double) * n, st));
  cudaError_t e = scratch_alloc((void **)&mats, sizeof(double) * 9 * ntr, st);
  if (e == cudaSuccess) {
    k_ln_min<<<n, 256, 0, st>>>(noise_scale, (int)ntr, mins);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    TraceScope ts("k_ln_matrices", st, 0.0);
    k_ln_matrices<<<grid_ln(ntr), 128, 0, st>>>(a, noise_scale, mins, nx, ny, mats, sigmamd);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    TraceScope ts("k_ln_correct", st, 36.0 * (double)nx * ny * nz);
    k_ln_correct<<<grid_ln((long)nx * ny * nz), 256, 0, st>>>(P, M, mats, nx, ny, nz, nxp, nyp);
    e = cudaGetLastError();
  }
  if (mats) cudaFreeAsync(mats, st);
  cudaFreeAsync(mins, st);
  if (e != cudaSuccess) return cuda_status(e, "cg_correct_alpha_beta_rho");
  return CG_OK;
}

extern "C" int cg_apply_trace_matrices(float *const *fields, const float *const *mean, const double *mats, int nx,
                                       int ny, int nz, int nxp, int nyp, int nzp, void *stream)
{
  if (!fields || !mats || nx < 1 || ny < 1 || nz < 1 || nx > nxp || ny > nyp || nz > nzp) {
    set_error("cg_apply_trace_matrices: bad argument");
    return CG_ERR_ARG;
  }
  CubeSet3 F, M;
  for (int p = 0; p < 3; p++) {
    if (!fields[p] || (mean && !mean[p])) { set_error("cg_apply_trace_matrices: null cube %d", p); return CG_ERR_ARG; }
    F.p[p] = fields[p];
    M.p[p] = mean ? const_cast<float *>(mean[p]) : nullptr;
  }
  cudaStream_t st = (cudaStream_t)stream;
  TraceScope ts("k_ln_fields", st, (mean ? 36.0 : 24.0) * (double)nxp * nyp * nzp);
  k_ln_fields<<<grid_ln((long)nxp * nyp * nzp), 256, 0, st>>>(F, M, mean ? 1 : 0, mats, nx, ny, nz, nxp, nyp, nzp);
  CG_CHECK_LAUNCH("k_ln_fields");
  return CG_OK;
}

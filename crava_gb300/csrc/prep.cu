// Per-model set-up of the fused bin kernels: for every temporal frequency k,
// the operator and error tables of the Cholesky form (KTab, FP64 and FP32)
// and the information-form tables (ITab).  This is the GPU counterpart of
// the per-k work the reference does inside its bin loop before the bins of a
// plane (Crava::fillErrMultVectors products and getNextErrorVariance's
// per-k factors, src/crava.cpp:1108-1120, :1337-1386, :1442-1469).
//
// One warp per k.  The tables of plane nzp-k are the conjugates of plane k's
// when the uploaded model is conjugate-symmetric in k, as the reference's
// tables are (Wavelet::getCAmp reflects k >= nzp/2+1); the host checks that
// and then launches planes 0..nzp/2 only, each writing its mirror plane too.
// The lanes build the table entries in parallel (an entry
// per lane), and the information form's Hermitian eigen-decomposition is a
// parallel Jacobi: in each step the lanes compute the rotations of up to four
// disjoint index pairs at once (round-robin pairing), then apply them to the
// columns, the eigenvectors and the rows with one matrix element per lane.
// The FP64 rate of this GPU is low, so the work is spread over one warp per
// plane on all SMs instead of one thread per plane, the Jacobi sweeps run in
// FP32 first and finish in FP64 from there (see below), and the FP64
// rotation's square roots and reciprocal are hardware approximations refined
// by Newton-Raphson steps.
#include "posterior.cuh"

namespace cg {

namespace {

constexpr int kPrepSweeps = 40;

// packed lower-triangle index t -> (l, m), l >= m
__device__ __forceinline__ void tri_lm(int t, int &l, int &m)
{
  l = 0;
  while ((l + 1) * (l + 2) / 2 <= t) l++;
  m = t - l * (l + 1) / 2;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// x^(-1/2) for normal x > 0: the hardware approximation refined by two Newton-Raphson steps for
// f(y) = 1/y^2 - x, y <- y (3 - x y^2) / 2 (each step squares the relative error)
__device__ __forceinline__ double rsqrt_nr(double x)
{
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(x));
  y = y * (1.5 - 0.5 * x * y * y);
  return y * (1.5 - 0.5 * x * y * y);
}

// 1/x for normal x > 0: the hardware approximation refined by two Newton-Raphson steps for
// f(y) = 1/y - x, y <- y (2 - x y)
__device__ __forceinline__ double rcp_nr(double x)
{
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  y = y * (2.0 - x * y);
  return y * (2.0 - x * y);
}

// conjugates n complex values in shared memory (lanes in parallel)
template <typename C>
__device__ __forceinline__ void conj_all(C *v, int n, int lane)
{
  for (int i = lane; i < n; i += 32) v[i].y = -v[i].y;
}

// 1/sqrt(x) and 1/x per element type: FP64 as above, FP32 from the hardware's own instructions
__device__ __forceinline__ double jrsqrt(double x) { return rsqrt_nr(x); }
__device__ __forceinline__ double jrcp(double x) { return rcp_nr(x); }
__device__ __forceinline__ float jrsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ float jrcp(float x) { return __frcp_rn(x); }

template <typename T>
struct JacobiScratch {
  int rp[kMaxTheta / 2], rq[kMaxTheta / 2];
  T rc[kMaxTheta / 2], rsn[kMaxTheta / 2];
  C2<T> rph[kMaxTheta / 2];
};

// Parallel cyclic Jacobi sweeps on the Hermitian nt x nt matrix a (shared memory), accumulating the
// rotations into v, until the squared off-diagonal Frobenius norm falls to tol times the squared diagonal
// (or max_sweeps).  Over an even number of indices (index nt is a dummy when nt is odd: its pairs are
// skipped); the lanes compute the rotations of up to four disjoint pairs at once (round-robin pairing), then
// apply them to the columns of a and v and the rows of a with one matrix element per lane.
template <typename T>
__device__ void jacobi_sweeps(C2<T> (*a)[kMaxTheta], C2<T> (*v)[kMaxTheta], JacobiScratch<T> &js, int nt,
                              int max_sweeps, T tol, T tiny, T small_rel, int lane)
{
  const int ne = nt + (nt & 1), np = ne / 2;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      if (l == m) diag += (double)a[l][l].x * a[l][l].x;
      else if (m > l) off += (double)a[l][m].x * a[l][m].x + (double)a[l][m].y * a[l][m].y;
    }
    off = warp_sum(off);
    diag = warp_sum(diag);
    if (off <= (double)tol * diag || off == 0.0) break;
    for (int r = 0; r < ne - 1; r++) {
      if (lane < np) {
        int i0, i1;
        if (lane == 0) { i0 = ne - 1; i1 = r; }
        else { i0 = (r + lane) % (ne - 1); i1 = (r - lane + ne - 1) % (ne - 1); }
        const int pp = min(i0, i1), qq = max(i0, i1);
        T c = 1, s = 0;
        C2<T> e = mk<T>(1, 0);
        if (qq < nt) {
          const C2<T> apq = a[pp][qq];
          const T mag2 = apq.x * apq.x + apq.y * apq.y;
          // an element far under the stopping criterion is left (the approximations need normal operands)
          if (mag2 > tiny && mag2 > small_rel * (a[pp][pp].x * a[pp][pp].x + a[qq][qq].x * a[qq][qq].x)) {
            const T ri = jrsqrt(mag2);
            e = mk<T>(apq.x * ri, -apq.y * ri);  // e^{-i arg a_pq}
            const T th = (a[qq][qq].x - a[pp][pp].x) * ((T)0.5 * ri);
            const T q = th * th + (T)1;
            const T tt = (th >= (T)0 ? (T)1 : (T)-1) * jrcp(fabs(th) + q * jrsqrt(q));
            c = jrsqrt(tt * tt + (T)1);
            s = tt * c;
          }
        }
        js.rp[lane] = pp; js.rq[lane] = qq; js.rc[lane] = c; js.rsn[lane] = s; js.rph[lane] = e;
      }
      __syncwarp();
      // columns of a and v: a <- a J, v <- v J
      for (int i = lane; i < 2 * np * nt; i += 32) {
        const int which = i / (np * nt), j = (i / nt) % np, row = i % nt;
        const int pp = js.rp[j], qq = js.rq[j];
        if (qq >= nt) continue;
        C2<T> (*x)[kMaxTheta] = which ? v : a;
        const T c = js.rc[j], s = js.rsn[j];
        const C2<T> xp = x[row][pp], xq = cmul<T>(js.rph[j], x[row][qq]);
        x[row][pp] = mk<T>(c * xp.x - s * xq.x, c * xp.y - s * xq.y);
        x[row][qq] = mk<T>(s * xp.x + c * xq.x, s * xp.y + c * xq.y);
      }
      __syncwarp();
      // rows of a: a <- J^H a
      for (int i = lane; i < np * nt; i += 32) {
        const int j = i / nt, col = i % nt;
        const int pp = js.rp[j], qq = js.rq[j];
        if (qq >= nt) continue;
        const T c = js.rc[j], s = js.rsn[j];
        const C2<T> xp = a[pp][col], xq = cmul<T>(cconj<T>(js.rph[j]), a[qq][col]);
        a[pp][col] = mk<T>(c * xp.x - s * xq.x, c * xp.y - s * xq.y);
        a[qq][col] = mk<T>(s * xp.x + c * xq.x, s * xp.y + c * xq.y);
      }
      __syncwarp();
    }
  }
}

}  // namespace

template <int NT>
__global__ void __launch_bounds__(32) k_prep_model(const __grid_constant__ PrepArgs p)
{
  const int k = blockIdx.x;
  const int lane = threadIdx.x;
  constexpr int nt = NT;
  // with symmetric tables this CTA also writes plane nzp - k, the conjugate of plane k
  const int km = (p.sym && k > 0 && 2 * k != p.nzp) ? p.nzp - k : -1;
  __shared__ KTab<double> t;
  __shared__ KTab<float> f;
  __shared__ ITab o;
  __shared__ double2 a[kMaxTheta][kMaxTheta], v[kMaxTheta][kMaxTheta], g[kMaxTheta][3];
  __shared__ double2 a0[kMaxTheta][kMaxTheta];
  __shared__ float2 af[kMaxTheta][kMaxTheta], vf[kMaxTheta][kMaxTheta];
  __shared__ double dm[kMaxTheta];
  __shared__ JacobiScratch<double> jsd;
  __shared__ JacobiScratch<float> jsf;

  for (int i = lane; i < (int)(sizeof(KTab<double>) / sizeof(double)); i += 32) ((double *)&t)[i] = 0.0;
  for (int i = lane; i < (int)(sizeof(KTab<float>) / sizeof(float)); i += 32) ((float *)&f)[i] = 0.0f;
  for (int i = lane; i < (int)(sizeof(ITab) / sizeof(float)); i += 32) ((float *)&o)[i] = 0.0f;
  __syncwarp();

  // K (ntheta x 3) and K S0
  for (int i = lane; i < nt * 3; i += 32) {
    const float2 kv = p.K[((long)k * nt) * 3 + i];
    t.K[i / 3][i % 3] = make_double2(kv.x, kv.y);
  }
  __syncwarp();
  for (int i = lane; i < nt * 3; i += 32) {
    const int l = i / 3, c = i % 3;
    double2 acc = make_double2(0, 0);
    for (int q = 0; q < 3; q++) {
      acc.x += t.K[l][q].x * p.s0[q * 3 + c];
      acc.y += t.K[l][q].y * p.s0[q * 3 + c];
    }
    t.KS0[l][c] = acc;
  }
  __syncwarp();
  // M = K S0 K^H and E = 0.5 (1 - wnc) errThetaCov (e1 e1^H + e2 e2^H), lower triangles
  const double c0 = 0.5 * (1.0 - (double)p.wnc);
  for (int i = lane; i < nt * (nt + 1) / 2; i += 32) {
    int l, m;
    tri_lm(i, l, m);
    double2 acc = make_double2(0, 0);
    for (int c = 0; c < 3; c++) acc = cadd<double>(acc, cmulc<double>(t.KS0[l][c], t.K[m][c]));
    t.M[i] = acc;
    const float2 e1l = p.em1[(long)k * nt + l], e2l = p.em2[(long)k * nt + l];
    const float2 e1m = p.em1[(long)k * nt + m], e2m = p.em2[(long)k * nt + m];
    const double re = (double)e1l.x * e1m.x + (double)e1l.y * e1m.y + (double)e2l.x * e2m.x + (double)e2l.y * e2m.y;
    const double im = (-(double)e1l.x * e1m.y + (double)e1l.y * e1m.x) + (-(double)e2l.x * e2m.y + (double)e2l.y * e2m.x);
    const double fc = c0 * p.etc[l * nt + m];
    t.E[i] = l == m ? make_double2(fc * re, 0.0) : make_double2(fc * re, fc * im);
  }
  // D = wnc errThetaCov_ll |Re e3_l|^2
  for (int l = lane; l < nt; l += 32) {
    const float2 e3 = p.em3[(long)k * nt + l];
    t.D[l] = (double)p.wnc * p.etc[l * nt + l] * (double)e3.x * (double)e3.x;
  }
  if (lane == 0) t.band = p.band[k];
  __syncwarp();

  // FP32 copy of the tables
  for (int i = lane; i < kMaxTheta * 3; i += 32) {
    const int l = i / 3, c = i % 3;
    f.K[l][c] = make_float2((float)t.K[l][c].x, (float)t.K[l][c].y);
    f.KS0[l][c] = make_float2((float)t.KS0[l][c].x, (float)t.KS0[l][c].y);
  }
  for (int i = lane; i < kTri; i += 32) {
    f.M[i] = make_float2((float)t.M[i].x, (float)t.M[i].y);
    f.E[i] = make_float2((float)t.E[i].x, (float)t.E[i].y);
  }
  for (int l = lane; l < kMaxTheta; l += 32) f.D[l] = (float)t.D[l];
  if (lane == 0) f.band = t.band;
  __syncwarp();
  {
    const double *src = (const double *)&t;
    double *dst = (double *)&p.td[k];
    for (int i = lane; i < (int)(sizeof(KTab<double>) / sizeof(double)); i += 32) dst[i] = src[i];
    const float *fs = (const float *)&f;
    float *fd = (float *)&p.tf[k];
    for (int i = lane; i < (int)(sizeof(KTab<float>) / sizeof(float)); i += 32) fd[i] = fs[i];
  }
  if (km >= 0) {
    // plane nzp - k: K, KS0, M, E conjugated, D and the band as they are (the information form below
    // reads only K, E and D of t: it runs before t is conjugated)
    __shared__ KTab<float> fm;
    {
      const float *fs = (const float *)&f;
      float *fmw = (float *)&fm;
      for (int i = lane; i < (int)(sizeof(KTab<float>) / sizeof(float)); i += 32) fmw[i] = fs[i];
    }
    __syncwarp();
    conj_all(&fm.K[0][0], kMaxTheta * 3, lane);
    conj_all(&fm.KS0[0][0], kMaxTheta * 3, lane);
    conj_all(fm.M, kTri, lane);
    conj_all(fm.E, kTri, lane);
    __syncwarp();
    const float *fs = (const float *)&fm;
    float *fd = (float *)&p.tf[km];
    for (int i = lane; i < (int)(sizeof(KTab<float>) / sizeof(float)); i += 32) fd[i] = fs[i];
    const double *src = (const double *)&t;
    double *dst = (double *)&p.td[km];
    for (int i = lane; i < (int)(sizeof(KTab<double>) / sizeof(double)); i += 32) {
      // the complex arrays K, KS0, M, E come first (double2 each): odd words are imaginary parts
      const int nc = 2 * (2 * kMaxTheta * 3 + 2 * kTri);
      dst[i] = (i < nc && (i & 1)) ? -src[i] : src[i];
    }
  }
  if (p.is4d) return;

  // information form: D^-1/2 E D^-1/2 = U diag(mu) U^H, v_m = D^-1/2 u_m, g_m = K^H v_m
  for (int i = lane; i < nt * 3; i += 32) o.K[i / 3][i % 3] = f.K[i / 3][i % 3];
  if (lane == 0) o.band = t.band;
  bool ok = true;
  for (int l = 0; l < nt; l++) ok = ok && t.D[l] > 0.0;
  __syncwarp();
  if (ok) {
    for (int l = lane; l < nt; l += 32) dm[l] = 1.0 / sqrt(t.D[l]);
    __syncwarp();
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      const double2 e = l >= m ? t.E[tri(l, m)] : make_double2(t.E[tri(m, l)].x, -t.E[tri(m, l)].y);
      a[l][m] = make_double2(dm[l] * e.x * dm[m], dm[l] * e.y * dm[m]);
      v[l][m] = make_double2(l == m ? 1.0 : 0.0, 0.0);
    }
    __syncwarp();
    // The eigen-decomposition in two precisions: cyclic Jacobi sweeps in FP32 down to FP32's resolution
    // (a handful of sweeps at the FP32 rate), the accumulated rotations re-orthonormalised in FP64
    // (modified Gram-Schmidt), the matrix brought to that basis in FP64 (a similarity transform, so the
    // eigenvalues are the original's), and FP64 sweeps from there: from FP32 accuracy they converge in one
    // or two sweeps (quadratic convergence) instead of the whole run in FP64, the slow unit of this GPU.
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      a0[l][m] = a[l][m];
      af[l][m] = make_float2((float)a[l][m].x, (float)a[l][m].y);
      vf[l][m] = make_float2(l == m ? 1.0f : 0.0f, 0.0f);
    }
    __syncwarp();
    jacobi_sweeps<float>(af, vf, jsf, nt, 10, 1e-12f, 1e-36f, 1e-14f, lane);
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      v[l][m] = make_double2((double)vf[l][m].x, (double)vf[l][m].y);
    }
    __syncwarp();
    for (int j = 0; j < nt; j++) {
      for (int q = 0; q < j; q++) {
        // v_j -= (v_q^H v_j) v_q
        double2 d = make_double2(0.0, 0.0);
        if (lane < nt) d = cmulc<double>(v[lane][j], v[lane][q]);
        d.x = warp_sum(d.x);
        d.y = warp_sum(d.y);
        if (lane < nt) v[lane][j] = csub<double>(v[lane][j], cmul<double>(d, v[lane][q]));
        __syncwarp();
      }
      double n2 = lane < nt ? v[lane][j].x * v[lane][j].x + v[lane][j].y * v[lane][j].y : 0.0;
      n2 = warp_sum(n2);
      const double rn = rsqrt_nr(n2);
      if (lane < nt) v[lane][j] = make_double2(v[lane][j].x * rn, v[lane][j].y * rn);
      __syncwarp();
    }
    // a = v^H a0 v (through a: first a0 v, then v^H of it)
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      double2 acc = make_double2(0.0, 0.0);
      for (int k2 = 0; k2 < nt; k2++) acc = cadd<double>(acc, cmul<double>(a0[l][k2], v[k2][m]));
      a[l][m] = acc;
    }
    __syncwarp();
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      double2 acc = make_double2(0.0, 0.0);
      for (int k2 = 0; k2 < nt; k2++) acc = cadd<double>(acc, cmul<double>(cconj<double>(v[k2][l]), a[k2][m]));
      a0[l][m] = acc;
    }
    __syncwarp();
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      // Hermitian by construction: take the upper triangle's value for both
      a[l][m] = l <= m ? a0[l][m] : cconj<double>(a0[m][l]);
      if (l == m) a[l][m].y = 0.0;
    }
    __syncwarp();
    jacobi_sweeps<double>(a, v, jsd, nt, kPrepSweeps, 1e-30, 1e-300, 1e-40, lane);
    for (int m = lane; m < nt; m += 32) o.mu[m] = (float)(a[m][m].x > 0.0 ? a[m][m].x : 0.0);
    for (int i = lane; i < nt * nt; i += 32) {
      const int l = i / nt, m = i % nt;
      const double2 vl = make_double2(dm[l] * v[l][m].x, dm[l] * v[l][m].y);
      v[l][m] = vl;
      o.V[l][m] = make_float2((float)vl.x, (float)vl.y);
    }
    __syncwarp();
    for (int i = lane; i < nt * 3; i += 32) {
      const int m = i / 3, c = i % 3;
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < nt; l++) acc = cadd<double>(acc, cmul<double>(cconj<double>(t.K[l][c]), v[l][m]));
      g[m][c] = acc;
      o.G[m][c] = make_float2((float)acc.x, (float)acc.y);
    }
    __syncwarp();
    // g g^H: entry (p, q) = g_p conj(g_q); 00 11 22, then 01 02 12 as (re, im)
    for (int m = lane; m < nt; m += 32) {
      for (int c = 0; c < 3; c++) o.P[m][c] = (float)(g[m][c].x * g[m][c].x + g[m][c].y * g[m][c].y);
      const double2 x01 = cmulc<double>(g[m][0], g[m][1]), x02 = cmulc<double>(g[m][0], g[m][2]);
      const double2 x12 = cmulc<double>(g[m][1], g[m][2]);
      o.P[m][3] = (float)x01.x; o.P[m][4] = (float)x01.y;
      o.P[m][5] = (float)x02.x; o.P[m][6] = (float)x02.y;
      o.P[m][7] = (float)x12.x; o.P[m][8] = (float)x12.y;
    }
  }
  __syncwarp();
  const float *os = (const float *)&o;
  float *od = (float *)&p.ti[k];
  for (int i = lane; i < (int)(sizeof(ITab) / sizeof(float)); i += 32) od[i] = os[i];
  if (km >= 0) {
    // plane nzp - k: the conjugate matrix has the conjugate eigenvectors and the same eigenvalues, so
    // K, V, G and the off-diagonal entries of g g^H are conjugated
    __syncwarp();
    conj_all(&o.K[0][0], kMaxTheta * 3, lane);
    conj_all(&o.V[0][0], kMaxTheta * kMaxTheta, lane);
    conj_all(&o.G[0][0], kMaxTheta * 3, lane);
    for (int m = lane; m < kMaxTheta; m += 32) {
      o.P[m][4] = -o.P[m][4];
      o.P[m][6] = -o.P[m][6];
      o.P[m][8] = -o.P[m][8];
    }
    __syncwarp();
    float *odm = (float *)&p.ti[km];
    for (int i = lane; i < (int)(sizeof(ITab) / sizeof(float)); i += 32) odm[i] = os[i];
  }
}

// one instantiation per stack count: every index below is then a compile-time expression
int launch_prep_model(const PrepArgs &p, int nplanes, cudaStream_t st)
{
  switch (p.nt) {
    case 1: k_prep_model<1><<<nplanes, 32, 0, st>>>(p); break;
    case 2: k_prep_model<2><<<nplanes, 32, 0, st>>>(p); break;
    case 3: k_prep_model<3><<<nplanes, 32, 0, st>>>(p); break;
    case 4: k_prep_model<4><<<nplanes, 32, 0, st>>>(p); break;
    case 5: k_prep_model<5><<<nplanes, 32, 0, st>>>(p); break;
    case 6: k_prep_model<6><<<nplanes, 32, 0, st>>>(p); break;
    case 7: k_prep_model<7><<<nplanes, 32, 0, st>>>(p); break;
    case 8: k_prep_model<8><<<nplanes, 32, 0, st>>>(p); break;
    default: set_error("ntheta %d outside 1..%d", p.nt, kMaxTheta); return CG_ERR_ARG;
  }
  return CG_OK;
}

}  // namespace cg

// Batched inversions of many independent cubes of uneven size, angle count,
// model and realisation count, as one unit of GPU work.
//
// Every cube has its own model (operator tables, workspace) and device cubes.
// A batch run queues each cube's whole inversion (prior spectra, forward
// transforms, fused bin kernel, inverse transforms) and, where set, its
// posterior simulation (factor, noise, inverse transforms, mean add) on one of several streams
// forked from the caller's stream and joins them back, so small cubes run
// side by side on the GPU.  With use_graph, the first run is captured into a
// CUDA graph (after a warm-up run that creates every twiddle table and kernel
// attribute the capture must not create) and every later run replays it: one
// graph launch for the whole batch instead of ~20 launches per cube.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "cravagpu.h"
#include "cravagpu_host.hpp"

namespace cg {
cudaError_t dev_malloc(void **p, size_t bytes);  // cudaMalloc, counted (cg_alloc_calls)
void set_error(const char *fmt, ...);
}

using namespace cravagpu;

namespace {

void cuda_check(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw Error(CG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

struct BatchCube {
  int nx, ny, nz, nxp, nyp, nzp, ntheta;
  Crava *crava = nullptr;
  std::vector<FFTGrid *> data, mean, cov;
  std::vector<float *> data_in, mean_in;  // pristine real-domain inputs (device)
  // posterior simulation after the inversion (cg_batch_set_simulation): factor planes, 3*nreal fields
  int nreal = 0;
  unsigned long long seed = 0;
  float *chol = nullptr;
  std::vector<float *> fields;
  long rsize() const { return 2L * (nxp / 2 + 1) * nyp * nzp; }
  long bins() const { return (long)(nxp / 2 + 1) * nyp * nzp; }
};

}  // namespace

struct cg_batch_s {
  std::vector<BatchCube> cubes;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  // graphs are captured on and launched from this stream, ordered after and
  // before the caller's stream by the two events (the caller's stream may be
  // the legacy default stream, which cannot be captured)
  cudaStream_t cap = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_form = -1;
  bool warm = false;
};

#define CG_TRY(...)                  \
  try {                              \
    __VA_ARGS__                      \
  } catch (const Error &e) {         \
    cg::set_error("%s", e.what());   \
    return e.status;                 \
  } catch (const std::exception &e) { \
    cg::set_error("%s", e.what());   \
    return CG_ERR_STATE;             \
  }

extern "C" void cg_batch_destroy(cg_batch b)
{
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto &c : b->cubes) {
    for (auto *g : c.data) delete g;
    for (auto *g : c.mean) delete g;
    for (auto *g : c.cov) delete g;
    for (auto *p : c.data_in) cudaFree(p);
    for (auto *p : c.mean_in) cudaFree(p);
    if (c.chol) cudaFree(c.chol);
    for (auto *p : c.fields) cudaFree(p);
    delete c.crava;
  }
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev_out) cudaEventDestroy(b->ev_out);
  delete b;
}

extern "C" int cg_batch_create(cg_batch *out, const cg_batch_cube *cubes, int ncubes, int nstreams)
{
  if (!out || !cubes || ncubes < 1 || nstreams < 1) { cg::set_error("cg_batch_create: bad argument"); return CG_ERR_ARG; }
  *out = nullptr;
  cg_batch_s *b = new cg_batch_s();
  CG_TRY({
    try {
      b->cubes.resize(ncubes);
      for (int i = 0; i < ncubes; i++) {
        const cg_batch_cube &d = cubes[i];
        const cg_inversion_model *m = &d.model;
        BatchCube &c = b->cubes[i];
        c.nx = d.nx; c.ny = d.ny; c.nz = d.nz; c.nxp = d.nxp; c.nyp = d.nyp; c.nzp = d.nzp; c.ntheta = m->ntheta;
        if (m->ntheta < 1 || m->ntheta > 8 || !m->wavelets || !m->A || !m->err_theta_cov || !m->sigma0 ||
            !m->corr_xy || !m->circ_corr_t)
          throw Error(CG_ERR_ARG, "cube " + std::to_string(i) + ": bad model");
        InversionModel im;
        im.ntheta = m->ntheta;
        im.wavelets.assign(m->wavelets, m->wavelets + (size_t)m->ntheta * d.nzp);
        im.A.assign(m->A, m->A + 3 * m->ntheta);
        im.errThetaCov.assign(m->err_theta_cov, m->err_theta_cov + m->ntheta * m->ntheta);
        im.sigma0.assign(m->sigma0, m->sigma0 + 9);
        im.corrXY.assign(m->corr_xy, m->corr_xy + (size_t)d.nxp * d.nyp);
        im.circCorrT.assign(m->circ_corr_t, m->circ_corr_t + d.nzp);
        im.wnc = m->wnc;
        im.lowCut = m->low_cut;
        im.highCut = m->high_cut;
        im.dt_ms = m->dt_ms;
        im.minRelThick = m->min_rel_thick > 0 ? m->min_rel_thick : 1.0f;
        im.condThreshold = m->cond_threshold;
        c.crava = new Crava(d.nx, d.ny, d.nz, d.nxp, d.nyp, d.nzp, im);
        for (int l = 0; l < c.ntheta; l++) {
          c.data.push_back(new FFTGrid(d.nx, d.ny, d.nz, d.nxp, d.nyp, d.nzp));
          c.data.back()->setType(FFTGrid::DATA);
          float *p = nullptr;
          cuda_check(cg::dev_malloc((void **)&p, sizeof(float) * c.rsize()), "batch input");
          c.data_in.push_back(p);
        }
        for (int q = 0; q < 3; q++) {
          c.mean.push_back(new FFTGrid(d.nx, d.ny, d.nz, d.nxp, d.nyp, d.nzp));
          c.mean.back()->setType(FFTGrid::PARAMETER);
          float *p = nullptr;
          cuda_check(cg::dev_malloc((void **)&p, sizeof(float) * c.rsize()), "batch input");
          c.mean_in.push_back(p);
        }
        for (int t = 0; t < 6; t++) {
          c.cov.push_back(new FFTGrid(d.nx, d.ny, d.nz, d.nxp, d.nyp, d.nzp));
          c.cov.back()->setType(FFTGrid::COVARIANCE);
        }
      }
      for (int s = 0; s < nstreams; s++) {
        cudaStream_t st;
        cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "batch stream");
        b->streams.push_back(st);
        cudaEvent_t e;
        cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "batch event");
        b->join.push_back(e);
      }
      cuda_check(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "batch event");
      cuda_check(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking), "batch capture stream");
      cuda_check(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming), "batch event");
      cuda_check(cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming), "batch event");
    } catch (...) {
      cg_batch_destroy(b);
      throw;
    }
    *out = b;
    return CG_OK;
  })
}

extern "C" int cg_batch_load(cg_batch b, int i, const float *const *seis_data, const float *const *mean)
{
  if (!b || i < 0 || i >= (int)b->cubes.size() || !seis_data || !mean) { cg::set_error("cg_batch_load: bad argument"); return CG_ERR_ARG; }
  CG_TRY({
    BatchCube &c = b->cubes[i];
    const size_t bytes = sizeof(float) * c.rsize();
    for (int l = 0; l < c.ntheta; l++) cuda_check(cudaMemcpy(c.data_in[l], seis_data[l], bytes, cudaMemcpyHostToDevice), "batch load");
    for (int q = 0; q < 3; q++) cuda_check(cudaMemcpy(c.mean_in[q], mean[q], bytes, cudaMemcpyHostToDevice), "batch load");
    return CG_OK;
  })
}

// working cubes <- pristine inputs (what a fresh inversion starts from)
extern "C" int cg_batch_reset(cg_batch b, void *stream)
{
  if (!b) { cg::set_error("null batch"); return CG_ERR_ARG; }
  CG_TRY({
    cudaStream_t st = (cudaStream_t)stream;
    for (auto &c : b->cubes) {
      const size_t bytes = sizeof(float) * c.rsize();
      for (int l = 0; l < c.ntheta; l++) {
        cuda_check(cudaMemcpyAsync(c.data[l]->devicePtr(), c.data_in[l], bytes, cudaMemcpyDeviceToDevice, st), "reset");
        c.data[l]->setTransformedStatus(false);
      }
      for (int q = 0; q < 3; q++) {
        cuda_check(cudaMemcpyAsync(c.mean[q]->devicePtr(), c.mean_in[q], bytes, cudaMemcpyDeviceToDevice, st), "reset");
        c.mean[q]->setTransformedStatus(false);
      }
    }
    return CG_OK;
  })
}

// Cubes to streams, longest first onto the least-loaded stream (LPT): the
// streams finish close together instead of one stream ending on a run of
// large cubes.  Work is estimated as bins x (stacks + 9 output spectra + 9 per
// realisation: three fields through three inverse passes).
static std::vector<int> stream_of_cubes(const cg_batch_s *b)
{
  const size_t n = b->cubes.size(), ns = b->streams.size();
  std::vector<int> order(n), sid(n);
  for (size_t i = 0; i < n; i++) order[i] = (int)i;
  auto work = [&](int i) { return (double)b->cubes[i].bins() * (b->cubes[i].ntheta + 9 + 9 * b->cubes[i].nreal); };
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
  std::vector<double> load(ns, 0.0);
  for (int i : order) {
    size_t best = 0;
    for (size_t s = 1; s < ns; s++)
      if (load[s] < load[best]) best = s;
    sid[i] = (int)best;
    load[best] += work(i);
  }
  return sid;
}

static void queue_batch(cg_batch b, Crava::Form form, cudaStream_t st)
{
  cuda_check(cudaEventRecord(b->fork, st), "fork");
  for (auto s : b->streams) cuda_check(cudaStreamWaitEvent(s, b->fork, 0), "fork wait");
  const std::vector<int> sid = stream_of_cubes(b);
  // largest cubes first, so each stream starts on its biggest piece of work
  std::vector<int> order(b->cubes.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->cubes[x].bins() > b->cubes[y].bins(); });
  for (int i : order) {
    BatchCube &c = b->cubes[i];
    cudaStream_t cs = b->streams[sid[i]];
    for (auto *g : c.data) g->setTransformedStatus(false);
    for (auto *g : c.mean) g->setTransformedStatus(false);
    FFTGrid *a = c.mean[0], *bb = c.mean[1], *cc = c.mean[2];
    c.crava->computePostMeanResidAndFFTCov(c.data.data(), a, bb, cc, c.cov.data(), nullptr, form, cs);
    if (c.nreal > 0) {
      float *cov[6], *pm[3];
      for (int t = 0; t < 6; t++) cov[t] = c.cov[t]->devicePtr();
      for (int q = 0; q < 3; q++) pm[q] = c.mean[q]->devicePtr();
      int rc = cg_posterior_cholesky(cov, c.chol, c.nxp, c.nyp, c.nzp, nullptr, cs);
      if (rc == CG_OK)
        rc = cg_simulate_fields(c.chol, nullptr, c.fields.data(), c.nreal, 0, c.seed, c.nxp, c.nyp, c.nzp, pm, cs);
      if (rc != CG_OK) throw Error(rc, "batch simulation: " + std::string(cg_last_error()));
    }
  }
  for (size_t s = 0; s < b->streams.size(); s++) {
    cuda_check(cudaEventRecord(b->join[s], b->streams[s]), "join");
    cuda_check(cudaStreamWaitEvent(st, b->join[s], 0), "join wait");
  }
}

// One inversion of every cube (working cubes must hold real-domain inputs,
// e.g. after cg_batch_reset).  form 1 = fused FP32, 2 = fused mixed.
extern "C" int cg_batch_run(cg_batch b, int form, int use_graph, void *stream)
{
  if (!b || (form != 1 && form != 2)) { cg::set_error("cg_batch_run: bad argument (form 1 or 2)"); return CG_ERR_ARG; }
  CG_TRY({
    cudaStream_t st = (cudaStream_t)stream;
    const Crava::Form f = form == 1 ? Crava::FUSED_FP32 : Crava::FUSED_MIXED;
    if (!use_graph) {
      queue_batch(b, f, st);
      b->warm = true;
      return CG_OK;
    }
    if (!b->exec || b->graph_form != form) {
      if (!b->warm) {
        // create twiddle tables and kernel attributes outside the capture
        queue_batch(b, f, st);
        cuda_check(cudaStreamSynchronize(st), "batch warm-up");
        cg_batch_reset(b, stream);
        b->warm = true;
      }
      if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
      if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
      cuda_check(cudaStreamSynchronize(st), "batch pre-capture");
      cuda_check(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
      try {
        queue_batch(b, f, b->cap);
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(b->cap, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      cuda_check(cudaStreamEndCapture(b->cap, &b->graph), "end capture");
      cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
      b->graph_form = form;
    }
    cuda_check(cudaEventRecord(b->ev_in, st), "order in");
    cuda_check(cudaStreamWaitEvent(b->cap, b->ev_in, 0), "order in wait");
    cuda_check(cudaGraphLaunch(b->exec, b->cap), "graph launch");
    cuda_check(cudaEventRecord(b->ev_out, b->cap), "order out");
    cuda_check(cudaStreamWaitEvent(st, b->ev_out, 0), "order out wait");
    return CG_OK;
  })
}

extern "C" int cg_batch_read(cg_batch b, int i, float *const *post_mean, float *const *resid, float *const *post_cov)
{
  if (!b || i < 0 || i >= (int)b->cubes.size()) { cg::set_error("cg_batch_read: bad argument"); return CG_ERR_ARG; }
  CG_TRY({
    BatchCube &c = b->cubes[i];
    const size_t bytes = sizeof(float) * c.rsize();
    cuda_check(cudaDeviceSynchronize(), "batch read");
    if (post_mean)
      for (int q = 0; q < 3; q++) cuda_check(cudaMemcpy(post_mean[q], c.mean[q]->devicePtr(), bytes, cudaMemcpyDeviceToHost), "read");
    if (resid)
      for (int l = 0; l < c.ntheta; l++) cuda_check(cudaMemcpy(resid[l], c.data[l]->devicePtr(), bytes, cudaMemcpyDeviceToHost), "read");
    if (post_cov)
      for (int t = 0; t < 6; t++) cuda_check(cudaMemcpy(post_cov[t], c.cov[t]->devicePtr(), bytes, cudaMemcpyDeviceToHost), "read");
    return CG_OK;
  })
}

extern "C" int cg_batch_set_simulation(cg_batch b, int i, int nreal, unsigned long long seed)
{
  if (!b || i < 0 || i >= (int)b->cubes.size() || nreal < 0) { cg::set_error("cg_batch_set_simulation: bad argument"); return CG_ERR_ARG; }
  CG_TRY({
    BatchCube &c = b->cubes[i];
    cuda_check(cudaDeviceSynchronize(), "batch simulation set-up");
    if (c.chol) { cudaFree(c.chol); c.chol = nullptr; }
    for (auto *p : c.fields) cudaFree(p);
    c.fields.clear();
    c.nreal = 0;
    c.seed = seed;
    if (nreal > 0) {
      cuda_check(cg::dev_malloc((void **)&c.chol, sizeof(float) * 9 * (size_t)c.bins()), "batch factor");
      for (int t = 0; t < 3 * nreal; t++) {
        float *f = nullptr;
        cuda_check(cg::dev_malloc((void **)&f, sizeof(float) * c.rsize()), "batch field");
        c.fields.push_back(f);
      }
      c.nreal = nreal;
    }
    // the captured graph no longer matches the work: recapture on the next graph run
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    b->graph_form = -1;
    b->warm = false;
    return CG_OK;
  })
}

extern "C" int cg_batch_read_fields(cg_batch b, int i, int r, float *const *fields)
{
  if (!b || i < 0 || i >= (int)b->cubes.size() || !fields) { cg::set_error("cg_batch_read_fields: bad argument"); return CG_ERR_ARG; }
  CG_TRY({
    BatchCube &c = b->cubes[i];
    if (r < 0 || r >= c.nreal) throw Error(CG_ERR_ARG, "cube " + std::to_string(i) + " has no realisation " + std::to_string(r));
    const size_t bytes = sizeof(float) * c.rsize();
    cuda_check(cudaDeviceSynchronize(), "batch read");
    for (int q = 0; q < 3; q++)
      if (fields[q]) cuda_check(cudaMemcpy(fields[q], c.fields[3 * r + q], bytes, cudaMemcpyDeviceToHost), "read field");
    return CG_OK;
  })
}

extern "C" long cg_batch_bins(cg_batch b)
{
  if (!b) return -1;
  long n = 0;
  for (auto &c : b->cubes) n += c.bins();
  return n;
}

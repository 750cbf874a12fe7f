// RAII launch tracer (see trace.cu).
#pragma once

#include <cuda_runtime.h>

namespace cg {

bool trace_on();

// While one of these lives on a thread, launches on that thread record no
// trace events (event creation is kept off the paths that promise to
// allocate nothing).
class TraceSuppress {
 public:
  TraceSuppress();
  ~TraceSuppress();

 private:
  bool prev_;
};

class TraceScope {
 public:
  TraceScope(const char *name, cudaStream_t st, double bytes);
  ~TraceScope();

 private:
  const char *name_;
  cudaStream_t st_;
  double bytes_;
  void *a_ = nullptr;
  void *b_ = nullptr;
};

}  // namespace cg

// noalloc.h — what the allocation-free step (noalloc.cu) reads from a
// context (hc_api.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/hc/hc.h"
#include "kernels.h"

namespace hc {

struct NoallocView {
  StepArgs args;        // the context's step arguments; the caller replaces
                        // every scratch and output pointer
  int device;
  cudaStream_t stream;  // the context's stream
  int max_geom_id;
  size_t n_samples;     // ray-sample keys of all sensors
};

// Fills `v` when the context is ready to step without re-dispatching its
// pairs; otherwise returns the failing status (message set).
hc_status noalloc_view(hc_context* c, NoallocView* v);

// Sets the calling thread's hc_last_error message and returns `st`.
hc_status set_last_error(hc_status st, const char* msg);

}  // namespace hc

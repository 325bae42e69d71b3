// Shared declarations of the engine (CUDA) and host (C++) halves of libmfx.
#pragma once
#include <string>

struct mfx_engine;
struct mfx_job;

namespace mfx {
// Records `fmt` as the calling thread's last error and returns `code`.
int set_error(int code, const char *fmt, ...);
int lattice_nshift(int lattice);
// CUDA device ordinal of an engine
int engine_device(const mfx_engine *eng);
// Loads the allocation-free noise entry point's module on `dev` (current):
// its fixed scratch array and kernels become resident at engine creation
// instead of at that entry point's first call.
int noalloc_prepare(int dev);

// What the Eulerian (PPT) field pass needs of a finished job: its device,
// stream and k-space potentials (phi1, phi2: N x N x (N/2+1) complex of double
// or float, stored as scale x the unscaled potential), the growth
// coefficients, the amplitude table (host copy) and the velocity unit.
struct JobFields {
  int device, N, order;
  bool fp64, has_potentials;
  void *stream;  // cudaStream_t
  const void *phi1, *phi2;
  double scale1, scale2, g1, g2, vfac1, boxlen, vunit;
  const double *amp;
  size_t amp_len;
};
int job_fields(const mfx_job *job, JobFields *out);
}  // namespace mfx

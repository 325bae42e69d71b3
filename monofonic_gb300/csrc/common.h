// Shared declarations of the engine (CUDA) and host (C++) halves of libmfx.
#pragma once
#include <string>

struct mfx_engine;

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
}  // namespace mfx

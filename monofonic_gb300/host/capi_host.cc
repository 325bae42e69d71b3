// C ABI of the host-side plugin logic (include/mfx.h, "host-side plugin
// logic" section): NGenIC seed table, cosmology calculator, amplitude table.
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <thread>
#include <vector>

#include "../../include/mfx.h"
#include "../csrc/common.h"
#include "../csrc/ranlxd.cuh"
#include "cosmology.h"

using namespace mfx;

struct mfx_cosmology {
  config_file cf;
  std::unique_ptr<calculator> calc;
};

#define HOST_GUARD_BEGIN try {
#define HOST_GUARD_END                                          \
  }                                                             \
  catch (const std::bad_alloc &) {                              \
    return set_error(MFX_ENOMEM, "host allocation failed");     \
  }                                                             \
  catch (const std::exception &ex) {                            \
    return set_error(MFX_EINVAL, "%s", ex.what());              \
  }                                                             \
  catch (...) {                                                 \
    return set_error(MFX_EINVAL, "unknown C++ exception");      \
  }

namespace mfx {

// RNG_ngenic constructor (random_ngenic.cc:39-75): one ranlxd1 stream seeded
// with `seed` fills the table in the plugin's spiral order, each entry being
// floor(0x7fffffff * u).
void ngenic_seed_table(long seed, size_t n, uint32_t *t) {
  Ranlxd1 r;
  ranlxd1_seed_any(r, (unsigned long)seed);
  std::memset(t, 0, n * n * sizeof(uint32_t));
  const double m = double(0x7fffffff);
  auto draw = [&]() { return uint32_t(m * r.uniform()); };
  for (size_t i = 0; i < n / 2; ++i) {
    for (size_t j = 0; j < i; j++) t[i * n + j] = draw();
    for (size_t j = 0; j < i + 1; j++) t[j * n + i] = draw();
    for (size_t j = 0; j < i; j++) t[(n - 1 - i) * n + j] = draw();
    for (size_t j = 0; j < i + 1; j++) t[(n - 1 - j) * n + i] = draw();
    for (size_t j = 0; j < i; j++) t[i * n + (n - 1 - j)] = draw();
    for (size_t j = 0; j < i + 1; j++) t[j * n + (n - 1 - i)] = draw();
    for (size_t j = 0; j < i; j++) t[(n - 1 - i) * n + (n - 1 - j)] = draw();
    for (size_t j = 0; j < i + 1; j++) t[(n - 1 - j) * n + (n - 1 - i)] = draw();
  }
}

// amp[n] = get_amplitude(k)/k^2 at k = kf sqrt(n), the factor that turns the
// normalised noise into -phi(1) (ic_generator.cc:509-516); amp[0] = 0.
void fill_amp_table(const calculator &c, uint32_t ngrid, double boxlen, double *table, size_t len) {
  const double kf = 2.0 * M_PI / boxlen;
  (void)ngrid;
  unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (len < 4096) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    th.emplace_back([&, t]() {
      for (size_t n = t; n < len; n += nt) {
        if (n == 0) {
          table[0] = 0.0;
          continue;
        }
        const double k = kf * std::sqrt(double(n));
        table[n] = c.get_amplitude(k, delta_matter) / (k * k);
      }
    });
  }
  for (auto &x : th) x.join();
}

}  // namespace mfx

extern "C" {

int mfx_ngenic_seed_table(long seed, size_t ngrid, uint32_t *table) {
  HOST_GUARD_BEGIN
  if (!table || ngrid == 0) return set_error(MFX_EINVAL, "bad arguments");
  ngenic_seed_table(seed, ngrid, table);
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_create(const char *ini_text, mfx_cosmology **out) {
  HOST_GUARD_BEGIN
  if (!ini_text || !out) return set_error(MFX_EINVAL, "null argument");
  auto c = std::make_unique<mfx_cosmology>();
  c->cf = config_file::from_text(ini_text);
  c->calc = std::make_unique<calculator>(c->cf);
  *out = c.release();
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_destroy(mfx_cosmology *c) {
  delete c;
  return MFX_OK;
}

int mfx_cosmology_get(mfx_cosmology *c, const char *name, double *value) {
  HOST_GUARD_BEGIN
  if (!c || !name || !value) return set_error(MFX_EINVAL, "null argument");
  *value = c->calc->cosmo_param_.get(name);
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_amplitude(mfx_cosmology *c, const double *k, size_t count, double *out) {
  HOST_GUARD_BEGIN
  if (!c || !k || !out) return set_error(MFX_EINVAL, "null argument");
  for (size_t q = 0; q < count; ++q) out[q] = c->calc->get_amplitude(k[q], delta_matter);
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_transfer(mfx_cosmology *c, const double *k, size_t count, double *out) {
  HOST_GUARD_BEGIN
  if (!c || !k || !out) return set_error(MFX_EINVAL, "null argument");
  for (size_t q = 0; q < count; ++q) out[q] = c->calc->transfer_function_->compute(k[q], delta_matter);
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_growth(mfx_cosmology *c, double a, double *dplus) {
  HOST_GUARD_BEGIN
  if (!c || !dplus) return set_error(MFX_EINVAL, "null argument");
  *dplus = c->calc->get_growth_factor(a);
  return MFX_OK;
  HOST_GUARD_END
}

int mfx_cosmology_amp_table(mfx_cosmology *c, uint32_t ngrid, double boxlen, double *table, size_t len) {
  HOST_GUARD_BEGIN
  if (!c || !table) return set_error(MFX_EINVAL, "null argument");
  const size_t need = 3 * size_t(ngrid / 2) * (ngrid / 2) + 1;
  if (len < need) return set_error(MFX_EINVAL, "amp table needs %zu entries", need);
  fill_amp_table(*c->calc, ngrid, boxlen, table, len);
  return MFX_OK;
  HOST_GUARD_END
}

}  // extern "C"

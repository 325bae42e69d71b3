// A C++ host calling the engine through include/mfx.h alone, the way a C++
// driver (the reference's ic_generator::run, ic_generator.cc:92-1181) would:
// cosmology and tables from the config text, one job created, run, waited
// for and fetched into host buffers, particles written to a file.
//
// usage: abi_caller <config.ini> <ngrid> <boxlen> <zstart> <order> <lattice> <seed> <precision 0|1> <out.bin>
// out.bin: uint64 particle count, then positions (3 f64 each), velocities
// (3 f64 each), ids (u64).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "mfx.h"

static int fail(const char *what, int rc) {
  char msg[512];
  mfx_last_error(msg, sizeof msg);
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, msg);
  return 1;
}

#define CHECK(call)                     \
  do {                                  \
    const int rc_ = (call);             \
    if (rc_ != MFX_OK) return fail(#call, rc_); \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 10) {
    std::fprintf(stderr, "usage: %s config.ini ngrid boxlen zstart order lattice seed precision out.bin\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string ini = ss.str();
  const uint32_t n = uint32_t(std::atoi(argv[2]));
  const double L = std::atof(argv[3]), z = std::atof(argv[4]);
  const int order = std::atoi(argv[5]), lattice = std::atoi(argv[6]), precision = std::atoi(argv[8]);
  const long seed = std::atol(argv[7]);

  mfx_cosmology *cosmo = nullptr;
  CHECK(mfx_cosmology_create(ini.c_str(), &cosmo));
  double dplus = 0, vfac = 0;
  CHECK(mfx_cosmology_get(cosmo, "dplus_start", &dplus));
  CHECK(mfx_cosmology_get(cosmo, "vfact_start", &vfac));
  std::vector<uint32_t> seeds(size_t(n) * n);
  CHECK(mfx_ngenic_seed_table(seed, n, seeds.data()));
  std::vector<double> amp(3 * size_t(n / 2) * (n / 2) + 1);
  CHECK(mfx_cosmology_amp_table(cosmo, n, L, amp.data(), amp.size()));

  mfx_engine_opts eo{0, 0};
  mfx_engine *eng = nullptr;
  CHECK(mfx_engine_create(&eo, &eng));

  mfx_job_desc d{};
  d.ngrid = n;
  d.boxlen = L;
  d.lpt_order = order;
  d.lattice = lattice;
  d.plt = 0;
  d.precision = precision;
  d.seed_table = seeds.data();
  d.amp_table = amp.data();
  d.amp_table_len = amp.size();
  // ic_generator.cc:252-269
  d.g1 = -dplus;
  d.g2 = order > 1 ? -3.0 / 7.0 * dplus * dplus : 0.0;
  d.g3 = order > 2 ? 1.0 / 3.0 * dplus * dplus * dplus : 0.0;
  d.g3c = order > 2 ? 1.0 / 7.0 * dplus * dplus * dplus : 0.0;
  d.vfac1 = vfac;
  d.vfac2 = 2 * vfac;
  d.vfac3 = 3 * vfac;
  d.lunit = L;
  d.vunit = L / std::sqrt(1.0 / (1.0 + z));
  d.pos64 = d.vel64 = d.id64 = 1;
  d.want_particles = 1;

  mfx_job *job = nullptr;
  CHECK(mfx_job_create(eng, &d, &job));
  CHECK(mfx_job_run(job));
  CHECK(mfx_job_wait(job, -1));
  const size_t np = size_t(1) << lattice;
  const uint64_t count = np * n * n * n;
  std::vector<double> pos(3 * count), vel(3 * count);
  std::vector<uint64_t> ids(count);
  CHECK(mfx_job_fetch_particles(job, pos.data(), vel.data(), ids.data()));
  CHECK(mfx_job_destroy(job));
  CHECK(mfx_engine_destroy(eng));
  CHECK(mfx_cosmology_destroy(cosmo));

  std::FILE *f = std::fopen(argv[9], "wb");
  if (!f) return 3;
  std::fwrite(&count, sizeof count, 1, f);
  std::fwrite(pos.data(), sizeof(double), pos.size(), f);
  std::fwrite(vel.data(), sizeof(double), vel.size(), f);
  std::fwrite(ids.data(), sizeof(uint64_t), ids.size(), f);
  std::fclose(f);
  std::printf("ok %llu particles\n", (unsigned long long)count);
  return 0;
}

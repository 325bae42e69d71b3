// Whole-run driver: the in-scope part of ic_generator::run
// (ic_generator.cc:92-1181) on top of the GPU engine, and the particle
// output-plugin interface it writes through (output_plugin.hh:33-133).
//
// Config keys are the reference's ([setup] GridRes, BoxLength, zstart,
// LPTorder, ParticleLoad, DoFixing, DoInversion, DoBaryons, DoBaryonVrel;
// [random] generator, seed; [cosmology] ...; [output] format, filename).  Two reference compile-time
// switches become run-time keys: [setup] DoPLT (CMakeLists.txt:111, ENABLE_PLT)
// and [execution] Precision = double | float (CMakeLists.txt:82-93,
// CODE_PRECISION; "float" selects the FP32-compensated form).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mfx.h"
#include "../csrc/common.h"
#include "config_file.h"
#include "cosmology.h"

namespace mfx {
void ngenic_seed_table(long seed, size_t n, uint32_t *t);
void fill_amp_table(const calculator &c, uint32_t ngrid, double boxlen, double *table, size_t len);

enum class cosmo_species { dm, baryon, neutrino };

// particle::container (particle_container.hh:29-188): interleaved xyz
struct particle_container {
  std::vector<float> positions32_, velocities32_, mass32_;
  std::vector<double> positions64_, velocities64_, mass64_;
  std::vector<uint32_t> ids32_;
  std::vector<uint64_t> ids64_;
  size_t get_local_num_particles() const { return std::max(ids32_.size(), ids64_.size()); }
};

class output_plugin {
 public:
  output_plugin(const config_file &cf, const calculator &cc) : cf_(cf), cc_(cc) {
    fname_ = cf.get_value<std::string>("output", "filename");
  }
  virtual ~output_plugin() {}
  virtual void write_particle_data(const particle_container &pc, const cosmo_species &s, double Omega) = 0;
  virtual bool has_64bit_reals() const = 0;
  virtual bool has_64bit_ids() const = 0;
  virtual double position_unit() const = 0;
  virtual double velocity_unit() const = 0;

 protected:
  const config_file &cf_;
  const calculator &cc_;
  std::string fname_;
};

using output_creator = std::unique_ptr<output_plugin> (*)(const config_file &, const calculator &);
std::map<std::string, output_creator> &get_output_plugin_map() {
  static std::map<std::string, output_creator> m;
  return m;
}

// "binary": one flat little-endian file, positions in Mpc/h and velocities in
// the Gadget convention (units as output_gadget_hdf5.cc:83-85)
class binary_output_plugin : public output_plugin {
 public:
  binary_output_plugin(const config_file &cf, const calculator &cc) : output_plugin(cf, cc) {
    const double astart = 1.0 / (1.0 + cf.get_value<double>("setup", "zstart"));
    lunit_ = cf.get_value<double>("setup", "BoxLength");
    vunit_ = lunit_ / std::sqrt(astart);
    b64reals_ = cf.get_value_safe<bool>("output", "UseDoublePrecision", true);
    b64ids_ = cf.get_value_safe<bool>("output", "UseLongids", true);
  }
  // one file per species: the dark matter (or CDM) particles in `filename`,
  // the baryons of a two-species run in `filename.baryon`; files of
  // particles with individual masses carry them after the ids (format 002)
  void write_particle_data(const particle_container &pc, const cosmo_species &s, double Omega) override {
    const std::string fn = s == cosmo_species::baryon ? fname_ + ".baryon" : fname_;
    FILE *f = std::fopen(fn.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot open output file '" + fn + "'");
    const bool masses = !pc.mass64_.empty() || !pc.mass32_.empty();
    const char magic[8] = {'M', 'F', 'X', 'I', 'C', '0', '0', masses ? '2' : '1'};
    const uint64_t np = pc.get_local_num_particles();
    const uint32_t rs = b64reals_ ? 8 : 4, is = b64ids_ ? 8 : 4;
    const double hdr[3] = {lunit_, Omega, cc_.cosmo_param_["h"]};
    bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(&np, 8, 1, f) == 1 && std::fwrite(&rs, 4, 1, f) == 1 &&
              std::fwrite(&is, 4, 1, f) == 1 && std::fwrite(hdr, 8, 3, f) == 3;
    if (b64reals_) {
      ok = ok && std::fwrite(pc.positions64_.data(), 8, 3 * np, f) == 3 * np;
      ok = ok && std::fwrite(pc.velocities64_.data(), 8, 3 * np, f) == 3 * np;
    } else {
      ok = ok && std::fwrite(pc.positions32_.data(), 4, 3 * np, f) == 3 * np;
      ok = ok && std::fwrite(pc.velocities32_.data(), 4, 3 * np, f) == 3 * np;
    }
    if (b64ids_) ok = ok && std::fwrite(pc.ids64_.data(), 8, np, f) == np;
    else ok = ok && std::fwrite(pc.ids32_.data(), 4, np, f) == np;
    if (masses) {
      if (b64reals_) ok = ok && std::fwrite(pc.mass64_.data(), 8, np, f) == np;
      else ok = ok && std::fwrite(pc.mass32_.data(), 4, np, f) == np;
    }
    std::fclose(f);
    if (!ok) throw std::runtime_error("short write to '" + fn + "'");
  }
  bool has_64bit_reals() const override { return b64reals_; }
  bool has_64bit_ids() const override { return b64ids_; }
  double position_unit() const override { return lunit_; }
  double velocity_unit() const override { return vunit_; }

 private:
  double lunit_, vunit_;
  bool b64reals_, b64ids_;
};

namespace {
// MUSIC1's white-noise file (grafic records, random_music_wnoise_generator.cc:
// 68-282): a header record (nx ny nz iseed as 32-bit ints) and nz records of
// nx*ny floats or doubles, each record framed by its byte count (32- or
// 64-bit markers); value (x, y) of record z, x fastest, goes to cell
// [x][y][z], negated unless grafic_sign.  The result is [x][y][z], z fastest.
std::vector<double> read_grafic_noise(const std::string &path, unsigned res, bool grafic_sign) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("Could not open random number file '" + path + "'!");
  auto rd = [&](void *p, size_t n) {
    f.read(reinterpret_cast<char *>(p), std::streamsize(n));
    if (!f) throw std::runtime_error("corrupt random number file");
  };
  uint32_t b32 = 0, nx = 0, ny = 0, nz = 0;
  int32_t iseed = 0;
  rd(&b32, 4);
  rd(&nx, 4);
  int mw = 4;  // marker width
  if (b32 != 16 || nx != res) {
    f.seekg(0);
    uint64_t b64 = 0;
    rd(&b64, 8);
    rd(&nx, 4);
    if (b64 != 16 || nx != res) throw std::runtime_error("corrupt random number file");
    mw = 8;
  }
  f.seekg(0);
  auto marker = [&]() -> uint64_t {
    uint64_t m = 0;
    if (mw == 4) {
      uint32_t m32 = 0;
      rd(&m32, 4);
      m = m32;
    } else {
      rd(&m, 8);
    }
    return m;
  };
  marker();
  rd(&nx, 4);
  rd(&ny, 4);
  rd(&nz, 4);
  rd(&iseed, 4);
  marker();
  if (nx != res || ny != res || nz != res)
    throw std::runtime_error("White noise file dimensions do not match level dimensions");
  const size_t plane = size_t(nx) * ny;
  std::vector<double> out(plane * nz);
  std::vector<float> buf4;
  std::vector<double> buf8;
  const double sign = grafic_sign ? 1.0 : -1.0;
  for (uint32_t z = 0; z < nz; ++z) {
    const uint64_t m = marker();
    if (m == plane * 4) {
      buf4.resize(plane);
      rd(buf4.data(), plane * 4);
      for (size_t q = 0; q < plane; ++q) out[((q % nx) * ny + q / nx) * nz + z] = sign * double(buf4[q]);
    } else if (m == plane * 8) {
      buf8.resize(plane);
      rd(buf8.data(), plane * 8);
      for (size_t q = 0; q < plane; ++q) out[((q % nx) * ny + q / nx) * nz + z] = sign * buf8[q];
    } else {
      throw std::runtime_error("corrupt random number file");
    }
    if (marker() != m) throw std::runtime_error("corrupt random number file");
  }
  return out;
}

std::unique_ptr<output_plugin> make_binary(const config_file &cf, const calculator &cc) {
  return std::make_unique<binary_output_plugin>(cf, cc);
}
struct register_binary {
  register_binary() { get_output_plugin_map()["binary"] = &make_binary; }
} s_register_binary;

struct Cleanup {
  mfx_job *job = nullptr;
  ~Cleanup() {
    if (job) mfx_job_destroy(job);
  }
};
}  // namespace

int run_config(mfx_engine *eng, const std::string &text) {
  const config_file cf = config_file::from_text(text);
  const uint32_t ngrid = cf.get_value<uint32_t>("setup", "GridRes");
  const double boxlen = cf.get_value<double>("setup", "BoxLength");
  const double zstart = cf.get_value<double>("setup", "zstart");
  int order = int(cf.get_value_safe<double>("setup", "LPTorder", 100));
  order = std::max(1, std::min(3, order));
  if (ngrid % 2 != 0 && order > 1) throw std::runtime_error("Orszag convolver for LPTorder>1 requires even grid size!");
  const std::string load = cf.get_value_safe<std::string>("setup", "ParticleLoad", "sc");
  int lattice;
  if (load == "sc") lattice = MFX_LATTICE_SC;
  else if (load == "bcc") lattice = MFX_LATTICE_BCC;
  else if (load == "fcc") lattice = MFX_LATTICE_FCC;
  else throw std::runtime_error("ParticleLoad '" + load + "' is not supported by this engine (sc, bcc, fcc)");
  // [random] generator (random_plugin.cc:62-81): NGENIC with its seed, or
  // MUSIC1 with seed[level] keys (random_music.cc:75, 160-283)
  const std::string gen = cf.get_value<std::string>("random", "generator");
  long seed = 0;
  int64_t music_seeds[12] = {};
  std::vector<double> noise_file;  // MUSIC1 noise read from a file
  unsigned noise_file_res = 0;     // its cells per axis below GridRes: the refinement chain's start
  int noise_gen = MFX_NOISE_NGENIC;
  unsigned cubesize = 0;
  if (gen == "NGENIC") {
    seed = cf.get_value<long>("random", "seed");
  } else if (gen == "MUSIC1") {
    // seed[l] for every level up to log2(GridRes) (random_music.cc:160-215);
    // the coarsest seeded level is refined up to the grid's
    int lmin = 0;
    while ((1u << lmin) < ngrid) ++lmin;
    if ((1u << lmin) != ngrid) throw std::runtime_error("MUSIC1 white noise needs GridRes a power of two");
    bool any = false;
    for (int l = 0; l <= 100; ++l) {
      const std::string key = "seed[" + std::to_string(l) + "]";
      if (!cf.contains_key("random", key)) continue;
      const std::string val = cf.get_value<std::string>("random", key);
      const bool number = !val.empty() && val.find_first_not_of("-0123456789") == std::string::npos;
      if (!number) {
        // a white-noise file in place of the seed (random_music.cc:186-193).
        // Used at the coarsest level given (levelmin_seed): at the grid's
        // level as the noise itself, below it as the start of the refinement
        // chain; a file above a coarser seed or file is ignored, as the
        // reference does (random_music.cc:231-234)
        if (any) {
          std::fprintf(stderr, "MUSIC1 %s: a noise file above the coarsest level given is ignored\n", key.c_str());
          continue;
        }
        if (l > lmin)
          throw std::runtime_error("MUSIC1 " + key + ": a noise file finer than log2(GridRes) = " +
                                   std::to_string(lmin) + " is not supported");
        noise_file = read_grafic_noise(val, 1u << l, cf.get_value_safe<bool>("random", "grafic_sign", false));
        noise_file_res = l < lmin ? (1u << l) : 0;
        any = true;
        continue;
      }
      if (l > lmin + 3 || l >= 12)
        throw std::runtime_error("MUSIC1 " + key + ": seeds more than three levels finer than log2(GridRes) = " +
                                 std::to_string(lmin) + " are not supported");
      const long v = cf.get_value<long>("random", key);
      if (v <= 0) throw std::runtime_error("Seed values need to be >0");
      music_seeds[l] = v;
      any = true;
    }
    if (!any) throw std::runtime_error("No seed specified for MUSIC1 RNG plugin!");
    if (!noise_file.empty() && noise_file_res == 0)
      for (int l = 0; l < 12; ++l)
        if (music_seeds[l] > 0)
          throw std::runtime_error("MUSIC1: a noise file at log2(GridRes) together with seed[" + std::to_string(l) +
                                   "] is not supported");
    seed = music_seeds[lmin];
    cubesize = cf.get_value_safe<unsigned>("random", "cubesize", 32);
    noise_gen = (noise_file.empty() || noise_file_res) ? MFX_NOISE_MUSIC1 : MFX_NOISE_FIELD;
  } else {
    throw std::runtime_error("random generator '" + gen + "' is not supported (NGENIC, MUSIC1)");
  }
  const std::string prec = cf.get_value_safe<std::string>("execution", "Precision", "double");

  calculator cc(cf);
  const double astart = 1.0 / (1.0 + zstart);
  const double Dplus0 = cc.get_growth_factor(astart), vfac = cc.get_vfact_start();
  const std::string fmt = cf.get_value<std::string>("output", "format");
  auto &om = get_output_plugin_map();
  if (!om.count(fmt)) throw std::runtime_error("Output plug-in '" + fmt + "' not found");
  auto out = om[fmt](cf, cc);

  std::vector<uint32_t> seeds;
  if (noise_gen == MFX_NOISE_NGENIC) {
    seeds.resize(size_t(ngrid) * ngrid);
    ngenic_seed_table(seed, ngrid, seeds.data());
  }
  const size_t alen = 3 * size_t(ngrid / 2) * (ngrid / 2) + 1;
  std::vector<double> amp(alen);
  fill_amp_table(cc, ngrid, boxlen, amp.data(), alen);
  std::vector<double> plt;
  const bool do_plt = cf.get_value_safe<bool>("setup", "DoPLT", false);
  if (do_plt) {
    plt.resize(MFX_PLT_TABLE_DOUBLES);
    int rc = mfx_plt_table_build(eng, lattice, plt.data());
    if (rc != MFX_OK) return rc;
  }
  mfx_job_desc d{};
  d.ngrid = ngrid;
  d.boxlen = boxlen;
  d.lpt_order = order;
  d.lattice = lattice;
  d.plt = do_plt;
  d.precision = (prec == "float") ? MFX_FP32C : MFX_FP64;
  d.fixing = cf.get_value_safe<bool>("setup", "DoFixing", false);
  d.inversion = cf.get_value_safe<bool>("setup", "DoInversion", false);
  d.seed_table = seeds.empty() ? nullptr : seeds.data();
  d.noise_generator = noise_gen;
  d.music_seed = noise_gen == MFX_NOISE_MUSIC1 ? seed : 0;
  d.music_cubesize = cubesize;
  std::memcpy(d.music_seeds, music_seeds, sizeof(music_seeds));
  d.noise_field = noise_file.empty() ? nullptr : noise_file.data();
  d.noise_field_res = noise_file_res;
  d.amp_table = amp.data();
  d.amp_table_len = alen;
  d.plt_table = do_plt ? plt.data() : nullptr;
  d.g1 = -Dplus0;
  d.g2 = order > 1 ? -3.0 / 7.0 * Dplus0 * Dplus0 : 0.0;
  d.g3 = order > 2 ? 1.0 / 3.0 * Dplus0 * Dplus0 * Dplus0 : 0.0;
  d.g3c = order > 2 ? 1.0 / 7.0 * Dplus0 * Dplus0 * Dplus0 : 0.0;
  d.vfac1 = vfac;
  d.vfac2 = 2 * vfac;
  d.vfac3 = 3 * vfac;
  d.lunit = out->position_unit();
  d.vunit = out->velocity_unit();
  d.pos64 = out->has_64bit_reals();
  d.vel64 = out->has_64bit_reals();
  d.id64 = out->has_64bit_ids();
  d.id_offset = 0;
  d.want_particles = 1;
  Cleanup cl;
  int rc = mfx_job_create(eng, &d, &cl.job);
  if (rc != MFX_OK) return rc;
  if ((rc = mfx_job_run(cl.job)) != MFX_OK) return rc;
  if ((rc = mfx_job_wait(cl.job, -1)) != MFX_OK) return rc;
  particle_container pc;
  const size_t np = size_t(1 << lattice) * ngrid * ngrid * ngrid;
  void *pp, *vp, *ip;
  if (d.pos64) {
    pc.positions64_.resize(3 * np);
    pc.velocities64_.resize(3 * np);
    pp = pc.positions64_.data();
    vp = pc.velocities64_.data();
  } else {
    pc.positions32_.resize(3 * np);
    pc.velocities32_.resize(3 * np);
    pp = pc.positions32_.data();
    vp = pc.velocities32_.data();
  }
  if (d.id64) {
    pc.ids64_.resize(np);
    ip = pc.ids64_.data();
  } else {
    pc.ids32_.resize(np);
    ip = pc.ids32_.data();
  }
  const bool baryons = cf.get_value_safe<bool>("setup", "DoBaryons", false);
  if (!baryons) {
    if ((rc = mfx_job_fetch_particles(cl.job, pp, vp, ip)) != MFX_OK) return rc;
    out->write_particle_data(pc, cosmo_species::dm, cc.cosmo_param_["Omega_m"]);
    return MFX_OK;
  }
  // baryon + CDM: both species from the potentials of the run above
  // (ic_generator.cc:151-166, 706-780, 1016-1020), masses per particle
  const bool vrel = cf.get_value_safe<bool>("setup", "DoBaryonVrel", false);
  const double Om = cc.cosmo_param_["Omega_m"], Ob = cc.cosmo_param_["Omega_b"];
  const double fb = Ob / Om;
  std::vector<double> dbc(alen, 0.0), tbc(alen, 0.0);
  for (size_t n = 1; n < alen; ++n) {
    const double k = 2.0 * M_PI / boxlen * std::sqrt(double(n));
    dbc[n] = cc.get_amplitude_delta_bc(k, vrel);
    tbc[n] = cc.get_amplitude_theta_bc(k, vrel);
  }
  if (d.pos64) pc.mass64_.resize(np);
  else pc.mass32_.resize(np);
  void *mp = d.pos64 ? static_cast<void *>(pc.mass64_.data()) : static_cast<void *>(pc.mass32_.data());
  const double munit = 1.0;  // the binary plugin's mass unit (masses in units of the critical density x box volume)
  for (const cosmo_species sp : {cosmo_species::dm, cosmo_species::baryon}) {
    const bool bar = sp == cosmo_species::baryon;
    const double omega = bar ? Ob : Om - Ob;
    mfx_species_desc s{};
    s.secondary_lattice = bar;
    s.id_offset = bar ? 1 : 0;
    s.c_species = bar ? 1.0 - fb : -fb;
    s.mass_factor = omega * munit;
    s.amp_dbc = dbc.data();
    s.amp_tbc = vrel ? tbc.data() : nullptr;
    s.amp_len = alen;
    s.want_masses = 1;
    if ((rc = mfx_job_set_species(cl.job, &s)) != MFX_OK) return rc;
    if ((rc = mfx_job_assemble(cl.job, 7)) != MFX_OK) return rc;
    if ((rc = mfx_job_fetch_particles(cl.job, pp, vp, ip)) != MFX_OK) return rc;
    if ((rc = mfx_job_fetch_masses(cl.job, 0, np, mp)) != MFX_OK) return rc;
    out->write_particle_data(pc, sp, omega);
  }
  return MFX_OK;
}

}  // namespace mfx

extern "C" int mfx_run_config(mfx_engine *eng, const char *ini_text) {
  try {
    if (!eng || !ini_text) return mfx::set_error(MFX_EINVAL, "null argument");
    return mfx::run_config(eng, ini_text);
  } catch (const std::bad_alloc &) {
    return mfx::set_error(MFX_ENOMEM, "host allocation failed");
  } catch (const std::exception &ex) {
    return mfx::set_error(MFX_EINVAL, "%s", ex.what());
  }
}

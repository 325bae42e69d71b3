// GB300 engine for monofonIC's IC hot path: job arena, cuFFT plans, the stage
// pipeline and the C ABI declared in include/mfx.h.
//
// Pipeline of one job (reference: ic_generator.cc:288-1060):
//   noise -> phi1                               k_noise_phi1
//   phi1 Hessians (6, padded M^3)              k_pad_hessian + 6 c2r
//   phi2 source -> r2c -> unpad/invLap         k_src2, r2c, k_unpad_invlap
//   phi3a: 5 pairwise products, each           k_mul, r2c, k_trunc_repad, c2r, k_acc3a
//   phi2 Hessians (6)                          k_pad_hessian + 6 c2r
//   phi3b + A3 sources                          k_src3
//   4 x (r2c -> unpad/invLap)                   phi3, A3x, A3y, A3z
//   assembly of all sub-lattices in k-space    k_assemble
//   per sub-lattice: 6 c2r + particle read-out k_particles
// Sums of convolve2 results that the reference unpads one by one are summed
// in real space before a single forward transform (linearity of unpad); this
// changes only rounding.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>
#include <time.h>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/mfx.h"
#include "common.h"
#include "kernels.cuh"
#include "fused_launch.cuh"
#include "music.cuh"

namespace mfx {

thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

const char *cufft_name(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    default: return "CUFFT_ERROR";
  }
}

#define CU(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return set_error(e_ == cudaErrorMemoryAllocation ? MFX_ENOMEM : MFX_ECUDA, "%s: %s (%s:%d)", \
                       #call, cudaGetErrorString(e_), __FILE__, __LINE__);                        \
  } while (0)
#define CF(call)                                                                                        \
  do {                                                                                                  \
    cufftResult r_ = (call);                                                                            \
    if (r_ != CUFFT_SUCCESS)                                                                            \
      return set_error(r_ == CUFFT_ALLOC_FAILED ? MFX_ENOMEM : MFX_ECUDA, "%s: %s (%s:%d)", #call,        \
                       cufft_name(r_), __FILE__, __LINE__);                                             \
  } while (0)
#define TRY(x)                 \
  do {                         \
    int rc_ = (x);             \
    if (rc_ != MFX_OK) return rc_; \
  } while (0)

static size_t align_up(size_t v, size_t a = 256) { return (v + a - 1) / a * a; }

int lattice_nshift(int lattice) { return 1 << lattice; }

// particle_generator.hh:47-54
static const double kShifts[3][4][3] = {
    {{0, 0, 0}},
    {{0, 0, 0}, {0.5, 0.5, 0.5}},
    {{0, 0, 0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}},
};

}  // namespace mfx

using namespace mfx;

struct Plan {
  cufftHandle h = 0;
  size_t work = 0;
  bool valid = false;
  int n = 0;
  bool fp64 = false, r2c = false;
  int batch = 1;            // transforms per execution
  long long dist_bytes = 0; // distance between consecutive transforms' buffers
};

struct mfx_engine {
  int device = 0;
  size_t budget = 0;
  std::mutex mu;
  size_t in_use = 0;
  // jobs and servers alive on this engine; mfx_engine_destroy with some still
  // alive only marks the engine closing, and the last of them releases it
  int holders = 0;
  bool closing = false;
  // cuFFT plans returned by finished jobs, reused by later jobs of the same
  // size class (plan creation is the slowest part of admitting a job)
  std::vector<Plan> plan_pool;
  // autotuned pencil-tile shapes of the fused transforms per grid size:
  // N -> (pencils per CTA of the x/y passes, rows per CTA of the z passes)
  struct FFTiles {
    int pxy, pz, pz2;
    int pk[6];
  };
  std::map<int, FFTiles> ff_tuned;  // per grid size: x/y tile, ZSRC3 and ZSRC2 shapes
};

struct mfx_job {
  mfx_engine *eng = nullptr;
  mfx_job_desc d{};
  int N = 0, M = 0, nh = 0, nk = 0, mk = 0, ns = 0, group = 0;
  bool fp64 = true;
  bool fused = false;          // padded convolutions through fused.cuh
  int ff_pxy = 8, ff_pz = 1, ff_pz2 = 1;  // pencils per CTA (x/y passes), ZSRC3 / ZSRC2 shapes (1, 2 rows; 3 wide; 4 warp)
  // x/y tile per pass kind (Y3, X6, XF, YF unpad, YF truncate, XI), tuned
  // one by one; 0: ff_pxy
  int ff_pk[6] = {};
  int xy_tile(int kind) const { return ff_pk[kind] ? ff_pk[kind] : ff_pxy; }
  void *ffB[3] = {};           // B-space [N][M][N/2] complex
  void *ffC[17] = {};          // C-space [M][M][N/2] complex
  float2 *ff_tw = nullptr;     // W_M^t, t < M
  float2 *ff_twn = nullptr;    // W_N^t, t < N (fused assembly)
  int *dstatus = nullptr;      // device status word: nonzero when a kernel's bounded wait ran out
  size_t rsize = 8;
  cudaStream_t stream = nullptr;
  cudaStream_t xfer[4] = {};  // particle downloads, split across copy streams
  // pipelined output (mfx_job_set_output_ring): one or two particle sets
  // outside the arena; a run writes set ring_next while the downloads of the
  // earlier runs' particles (enqueued on xfer[0] by the asynchronous fetch)
  // may still run -- with two sets the whole run overlaps them, with one set
  // everything before the run's assembly does
  char *ring = nullptr;
  size_t ring_set_bytes = 0;
  int ring_sets = 0;
  int ring_next = 0;
  cudaEvent_t ring_free[2] = {};  // the last download from set s is done
  cudaEvent_t fetched = nullptr;  // the last asynchronous download is done
  cudaEvent_t ev[6] = {};
  bool timed = false;
  // arena
  char *arena = nullptr;
  size_t arena_bytes = 0;
  size_t n_field_bytes = 0, m_field_bytes = 0;
  // device pointers
  uint32_t *seeds = nullptr;
  double *amp = nullptr;
  double *plt = nullptr;
  float4 *plt4 = nullptr;  // FP32 form: the PLT tables interleaved per mode
  double2 *phase = nullptr;
  float2 *phase32 = nullptr;  // the phase tables rounded to float (FP32 form)
  double *qtab = nullptr;  // [shift][axis][N] unperturbed coordinates times lunit
  void *nf[6] = {};       // phi1, phi2, phi3, A3x, A3y, A3z
  char *region = nullptr; // M-region / assembly union
  size_t region_bytes = 0;
  void *mslot[18] = {};
  void *asmbuf[24] = {};
  void *pos = nullptr, *vel = nullptr, *ids = nullptr;
  std::vector<std::thread> id_fill;  // host threads writing the ids / positions of a fetch
  // host-side positions (mfx_job_set_host_positions): the device keeps float
  // displacements, a fetch copies them to page-locked staging and host threads
  // form q + Psi in FP64 from the lattice coordinates qhost ([shift][axis][N])
  bool host_q = false;
  float *psi_host = nullptr;
  // the fused read-out writes no device ids (every host destination gets them
  // from host threads); a device destination gets them from k_fill_ids, and
  // mfx_job_particles_device from this array, filled on request
  void *ids_dev = nullptr;
  std::vector<double> qhost;
  std::vector<cudaEvent_t> psi_ev;  // one per staging chunk of a fetch
  void *work = nullptr;
  size_t work_bytes = 0;
  Plan m_r2c, m_c2r, n_c2r;
  Plan n_r2c;  // N-grid forward transform of the MUSIC1 cube noise
  // MUSIC1 from coarser seeded levels: the levels' forward transforms
  // (level music_l0 + q at music_plans[q]) and two coarse k-space buffers
  std::vector<Plan> music_plans;
  int music_l0 = 0, music_lmin = 0, music_lfile = -1;
  void *music_buf[2] = {nullptr, nullptr};
  // CUDA graph of the whole pipeline (mfx_job_capture)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // accounting
  int own_launches = 0, fft_execs = 0;
  bool has_run = false, noise_only = false;
  size_t npart = 0;
  double scale1 = 1, scale2 = 1, scale3 = 1;  // per-field scales of the FP32 form
  // baryon + CDM species of the next assembly (mfx_job_set_species)
  std::vector<double> amp_host;    // the amplitude table, for the species' ratio tables
  uint64_t base_id_offset = 0;     // the descriptor's IDoffset
  double lat_off[3] = {0, 0, 0};   // secondary-lattice shift (particle_generator.hh:56-63)
  double c_species = 0, mass_factor = 0;
  bool want_masses = false, has_masses = false;
  char *sp_mem = nullptr;          // one allocation: tables, mass field, masses, FFT work
  size_t sp_bytes = 0, sp_len = 0;
  double *qvbc = nullptr, *rho_ratio = nullptr;
  float *qvbc32 = nullptr;
  void *rho = nullptr, *mass = nullptr, *rho_work = nullptr;
  Plan rho_c2r;
  // per-launch profiling (events on the job stream + algorithmic bytes)
  struct ProfRec {
    const char *name;
    double bytes;
    cudaEvent_t a, b;
  };
  bool prof = false;
  std::vector<ProfRec> prof_recs;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_next = 0;
  cudaEvent_t pend = nullptr;
  cudaEvent_t next_event() {
    if (ev_next == ev_pool.size()) {
      cudaEvent_t e = nullptr;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_next++];
  }
};

int mfx::engine_device(const mfx_engine *eng) { return eng ? eng->device : 0; }

int mfx::job_fields(const mfx_job *j, JobFields *o) {
  if (!j || !o) return set_error(MFX_EINVAL, "null argument");
  o->device = j->eng->device;
  o->N = j->N;
  o->order = j->d.lpt_order;
  o->fp64 = j->fp64;
  o->has_potentials = j->has_run && !j->noise_only;
  o->stream = j->stream;
  o->phi1 = j->nf[0];
  o->phi2 = j->d.lpt_order > 1 ? j->nf[1] : nullptr;
  o->scale1 = j->scale1;
  o->scale2 = j->scale2;
  o->g1 = j->d.g1;
  o->g2 = j->d.g2;
  o->vfac1 = j->d.vfac1;
  o->boxlen = j->d.boxlen;
  o->vunit = j->d.vunit;
  o->amp = j->amp_host.data();
  o->amp_len = j->amp_host.size();
  return MFX_OK;
}

// ---------------------------------------------------------------------------
// sizes
// ---------------------------------------------------------------------------
struct Layout {
  size_t seeds, amp, plt, phase, nfields, region, work_est, total;
  size_t n_field, m_field, asm_bytes, part_bytes, mregion, music;
  int nslots, group;
  size_t ff_b, ff_d, ff_tw, status;
  int ff_nc;
};

static size_t n_field_bytes(int N, size_t rs) { return size_t(N) * N * (N / 2 + 1) * 2 * rs; }

// MUSIC1 levels of a descriptor: the grid's level lmin, the coarsest seeded
// level l0 <= lmin and the effective seed of every level l0..lmin (a given
// seed[l], music_seed at lmin, else the level's dummy seed)
// (l0 > lmin: seeds only at finer levels; the coarsest of them is filled and
// restricted down to lmin, random_music.cc:247-272)
struct MusicLevels {
  int l0 = 0, lmin = 0;
  int lfile = -1;  // the level a noise field gives (the chain's coarsest), else -1
  int64_t seed[12] = {};
};
static MusicLevels music_levels(const mfx_job_desc *d) {
  MusicLevels m;
  while ((1u << m.lmin) < d->ngrid && m.lmin < 11) ++m.lmin;
  m.l0 = -1;
  if (d->noise_generator == MFX_NOISE_MUSIC1 && d->noise_field && d->noise_field_res > 1) {
    m.lfile = 0;
    while ((1u << m.lfile) < d->noise_field_res && m.lfile < 11) ++m.lfile;
    m.l0 = m.lfile;
  }
  for (int l = 0; l < 12 && m.l0 < 0; ++l)
    if (d->music_seeds[l] > 0 || (l == m.lmin && d->music_seed > 0)) m.l0 = l;
  if (m.l0 < 0) m.l0 = m.lmin;
  if (m.l0 > m.lmin) {
    m.seed[m.l0] = d->music_seeds[m.l0];
    return m;
  }
  for (int l = m.l0; l <= m.lmin; ++l) {
    int64_t s = d->music_seeds[l];
    if (s <= 0 && l == m.lmin && d->music_seed > 0) s = d->music_seed;
    m.seed[l] = s > 0 ? s : music::dummy_seed(l);
  }
  return m;
}

static int check_desc(const mfx_job_desc *d) {
  if (!d) return set_error(MFX_EINVAL, "null job descriptor");
  if (d->ngrid < 8 || (d->ngrid % 4) != 0)
    return set_error(MFX_EINVAL, "ngrid must be a multiple of 4 and >= 8 (got %u)", d->ngrid);
  if (d->ngrid > 2048) return set_error(MFX_EINVAL, "ngrid %u above the supported maximum 2048", d->ngrid);
  if (!(d->boxlen > 0)) return set_error(MFX_EINVAL, "boxlen must be positive");
  if (d->lpt_order < 1 || d->lpt_order > 3) return set_error(MFX_EINVAL, "lpt_order must be 1, 2 or 3");
  if (d->lattice < 0 || d->lattice > 2) return set_error(MFX_EINVAL, "lattice must be SC, BCC or FCC");
  if (d->precision != MFX_FP64 && d->precision != MFX_FP32C) return set_error(MFX_EINVAL, "bad precision");
  if (d->noise_generator == MFX_NOISE_NGENIC) {
    if (!d->seed_table) return set_error(MFX_EINVAL, "seed_table is required");
  } else if (d->noise_generator == MFX_NOISE_MUSIC1) {
    // one level at the grid's own resolution: 2^levelmin cells per axis
    // (random_music.cc:75), cubes that tile it (random_music_wnoise_generator.cc:588-626)
    if (d->ngrid & (d->ngrid - 1)) return set_error(MFX_EINVAL, "MUSIC1 noise needs ngrid a power of two (got %u)", d->ngrid);
    int lmin = 0;
    while ((1u << lmin) < d->ngrid) ++lmin;
    bool any = d->music_seed > 0;
    for (int l = 0; l < 12; ++l) {
      if (d->music_seeds[l] < 0) return set_error(MFX_EINVAL, "MUSIC1 seed[%d] must be positive", l);
      if (d->music_seeds[l] > 0 && l > lmin + 3)
        return set_error(MFX_EINVAL, "MUSIC1 seed[%d] more than three levels finer than the grid's (%d)", l, lmin);
      any = any || d->music_seeds[l] > 0;
    }
    if (d->noise_field) {
      // a noise file at the chain's coarsest level (random_music.cc:216-236)
      const uint32_t r = d->noise_field_res;
      if (r < 2 || (r & (r - 1)) || r >= d->ngrid)
        return set_error(MFX_EINVAL, "MUSIC1 noise_field_res must be a power of two from 2 below ngrid (got %u)", r);
      int lf = 0;
      while ((1u << lf) < r) ++lf;
      for (int l = 0; l <= lf; ++l)
        if (d->music_seeds[l] > 0)
          return set_error(MFX_EINVAL, "MUSIC1 seed[%d] at or below the noise field's level %d", l, lf);
      any = true;
    }
    if (d->music_seed < 0 || !any) return set_error(MFX_EINVAL, "MUSIC1 noise needs a positive seed");
    const unsigned cs = d->music_cubesize ? d->music_cubesize : 32u;
    if (cs < 2 || (d->ngrid >= cs && d->ngrid % cs != 0))
      return set_error(MFX_EINVAL, "MUSIC1 cubesize %u does not tile ngrid %u", cs, d->ngrid);
    if (std::min(cs, d->ngrid) > 256u)
      return set_error(MFX_EINVAL, "MUSIC1 cubes above 256^3 cells (one sequential stream each) are not supported");
  } else if (d->noise_generator == MFX_NOISE_FIELD) {
    if (!d->noise_field) return set_error(MFX_EINVAL, "MFX_NOISE_FIELD needs noise_field");
    if (d->noise_field_res && d->noise_field_res != d->ngrid)
      return set_error(MFX_EINVAL, "MFX_NOISE_FIELD gives the grid's level: noise_field_res must be 0 or ngrid");
  } else {
    return set_error(MFX_EINVAL, "unknown noise_generator %d", d->noise_generator);
  }
  size_t need = 3 * size_t(d->ngrid / 2) * (d->ngrid / 2) + 1;
  if (!d->amp_table || d->amp_table_len < need)
    return set_error(MFX_EINVAL, "amp_table needs at least %zu entries", need);
  if (d->plt && !d->plt_table) return set_error(MFX_EINVAL, "plt requested without plt_table");
  return MFX_OK;
}

// The FP32 form runs the padded convolutions through the pruned, fused
// transforms (fused.cuh) for every padded length they are built for; the
// plain FP64 form and other sizes use cuFFT.  MFX_FUSED=0 in the environment
// sends the FP32 form through cuFFT as well (for comparisons).
static bool fused_supported(const mfx_job_desc *d) {
  if (d->precision != MFX_FP32C || d->lpt_order < 2) return false;
  // the pruned transforms take phi(1) with empty Nyquist planes (NGenIC's
  // noise); MUSIC1 noise fills them
  if (d->noise_generator != MFX_NOISE_NGENIC) return false;
  const char *env = getenv("MFX_FUSED");
  if (env && env[0] == '0') return false;
  const int N = d->ngrid, M = 3 * N / 2;
  return (N / 2) % 8 == 0 && ff::ff_length_supported(M);
}

// group_all: hold every sub-lattice's assembled components at once even where
// that grows the region beyond the padded fields (the fused assembly then
// assembles each mode once for all sub-lattices)
static Layout plan_layout(const mfx_job_desc *d, size_t work_bytes, bool group_all = false) {
  Layout L{};
  const int N = d->ngrid, M = 3 * N / 2;
  const size_t rs = d->precision == MFX_FP64 ? 8 : 4;
  const int ns = lattice_nshift(d->lattice);
  L.n_field = n_field_bytes(N, rs);
  L.m_field = size_t(M) * M * (M / 2 + 1) * 2 * rs;
  L.seeds = align_up(size_t(N) * N * 4);
  L.amp = align_up(d->amp_table_len * 8);
  L.plt = d->plt ? align_up(size_t(MFX_PLT_TABLE_DOUBLES) * 8) + align_up(size_t(MFX_PLT_TABLE_DOUBLES) * 4) : 0;
  L.phase = align_up(size_t(ns) * 3 * N * sizeof(double2)) + align_up(size_t(ns) * 3 * N * sizeof(double)) +
            align_up(size_t(ns) * 3 * N * sizeof(float2));
  const int nfield = d->lpt_order == 1 ? 1 : (d->lpt_order == 2 ? 2 : 6);
  L.nfields = nfield * align_up(L.n_field);
  L.nslots = d->lpt_order == 1 ? 0 : (d->lpt_order == 2 ? 7 : 17);
  L.mregion = size_t(L.nslots) * align_up(L.m_field);
  if (fused_supported(d)) {
    // no real-space M-grid fields: three B-space [N][M][N/2] and 7 (2LPT) or
    // 17 (3LPT) C-space [M][M][N/2] complex fields, and the twiddles
    const size_t kh = N / 2;
    L.nslots = 0;
    L.ff_b = align_up(size_t(N) * M * kh * 8);
    L.ff_d = align_up(size_t(M) * M * kh * 8);
    L.ff_nc = d->lpt_order == 3 ? 17 : 7;
    L.mregion = 3 * L.ff_b + size_t(L.ff_nc) * L.ff_d;
    // the twiddles outlive the run: not in the region the particles reuse
    L.ff_tw = align_up(size_t(M) * 8) + align_up(size_t(N) * 8);
    L.status = align_up(sizeof(int));
  }
  const size_t np = size_t(ns) * N * N * N;
  L.part_bytes = 0;
  if (d->want_particles) {
    L.part_bytes = align_up(np * 3 * (d->pos64 ? 8 : 4)) + align_up(np * 3 * (d->vel64 ? 8 : 4)) +
                   align_up(np * (d->id64 ? 8 : 4));
  }
  // all sub-lattices assembled in one pass when it fits beside the particles
  // in the region the padded fields leave behind, else one at a time
  int group = ns;
  if (d->want_particles) {
    size_t full = L.part_bytes + size_t(6 * ns) * align_up(L.n_field);
    if (L.mregion > 0 && full > L.mregion && !group_all) group = 1;
  }
  L.group = group;
  L.asm_bytes = d->want_particles ? L.part_bytes + size_t(6 * group) * align_up(L.n_field) : 0;
  L.region = std::max(L.mregion, L.asm_bytes);
  L.work_est = align_up(work_bytes);
  // MUSIC1 from coarser seeded levels: two coarse-level k-space fields
  L.music = 0;
  if (d->noise_generator == MFX_NOISE_FIELD) L.music = align_up(size_t(N) * N * N * 8);  // the field's upload
  if (d->noise_generator == MFX_NOISE_MUSIC1) {
    const MusicLevels ml = music_levels(d);
    if (ml.l0 < ml.lmin) L.music = 2 * align_up(n_field_bytes(N / 2, rs));
    // the finer seeded level and, for two steps or more, one level below it
    if (ml.l0 > ml.lmin)
      L.music = align_up(n_field_bytes(1 << ml.l0, rs)) +
                (ml.l0 - ml.lmin >= 2 ? align_up(n_field_bytes(1 << (ml.l0 - 1), rs)) : 0);
  }
  L.total = L.seeds + L.amp + L.plt + L.phase + L.ff_tw + L.status + L.nfields + L.region + L.work_est + L.music;
  return L;
}

// ---------------------------------------------------------------------------
// cuFFT plans (in-place, padded rows as in the reference's Grid_FFT)
// ---------------------------------------------------------------------------
// batch > 1: `batch` in-place transforms whose buffers lie dist_bytes apart
static int make_plan(Plan &p, int n, bool fp64, bool r2c, int batch = 1, long long dist_bytes = 0) {
  CF(cufftCreate(&p.h));
  CF(cufftSetAutoAllocation(p.h, 0));
  long long dims[3] = {n, n, n};
  long long rembed[3] = {n, n, n + 2};
  long long cembed[3] = {n, n, n / 2 + 1};
  const long long rs = fp64 ? 8 : 4;
  long long rdist = (long long)n * n * (n + 2), cdist = (long long)n * n * (n / 2 + 1);
  if (batch > 1) {
    rdist = dist_bytes / rs;
    cdist = dist_bytes / (2 * rs);
  }
  cufftType t = fp64 ? (r2c ? CUFFT_D2Z : CUFFT_Z2D) : (r2c ? CUFFT_R2C : CUFFT_C2R);
  size_t ws = 0;
  if (r2c)
    CF(cufftMakePlanMany64(p.h, 3, dims, rembed, 1, rdist, cembed, 1, cdist, t, batch, &ws));
  else
    CF(cufftMakePlanMany64(p.h, 3, dims, cembed, 1, cdist, rembed, 1, rdist, t, batch, &ws));
  p.batch = batch;
  p.dist_bytes = dist_bytes;
  p.work = ws;
  p.valid = true;
  return MFX_OK;
}

static void destroy_plan(Plan &p) {
  if (p.valid) cufftDestroy(p.h);
  p.valid = false;
}

static int acquire_plan(mfx_engine *eng, Plan &p, int n, bool fp64, bool r2c, int batch = 1,
                        long long dist_bytes = 0) {
  {
    std::lock_guard<std::mutex> lk(eng->mu);
    for (size_t q = 0; q < eng->plan_pool.size(); ++q) {
      const Plan &c = eng->plan_pool[q];
      if (c.n == n && c.fp64 == fp64 && c.r2c == r2c && c.batch == batch && c.dist_bytes == dist_bytes) {
        p = c;
        eng->plan_pool.erase(eng->plan_pool.begin() + q);
        return MFX_OK;
      }
    }
  }
  TRY(make_plan(p, n, fp64, r2c, batch, dist_bytes));
  p.n = n;
  p.fp64 = fp64;
  p.r2c = r2c;
  return MFX_OK;
}

// The engine outlives the jobs and servers made on it: each holds a reference.
static void engine_retain(mfx_engine *eng) {
  std::lock_guard<std::mutex> lk(eng->mu);
  ++eng->holders;
}

static void engine_free(mfx_engine *eng) {
  for (auto &p : eng->plan_pool) destroy_plan(p);
  delete eng;
}

static void engine_release(mfx_engine *eng) {
  bool last = false;
  {
    std::lock_guard<std::mutex> lk(eng->mu);
    last = --eng->holders == 0 && eng->closing;
  }
  if (last) engine_free(eng);
}

static void release_plan(mfx_engine *eng, Plan &p) {
  if (!p.valid) return;
  std::lock_guard<std::mutex> lk(eng->mu);
  if (eng->plan_pool.size() < 96) {
    eng->plan_pool.push_back(p);
  } else {
    cufftDestroy(p.h);
  }
  p.valid = false;
}

static void kbegin(mfx_job *j);
static void kend_prof(mfx_job *j, const char *name, double bytes);

static int exec_fft(mfx_job *j, Plan &p, void *buf, bool r2c) {
  kbegin(j);
  if (j->fp64) {
    if (r2c) CF(cufftExecD2Z(p.h, (cufftDoubleReal *)buf, (cufftDoubleComplex *)buf));
    else CF(cufftExecZ2D(p.h, (cufftDoubleComplex *)buf, (cufftDoubleReal *)buf));
  } else {
    if (r2c) CF(cufftExecR2C(p.h, (cufftReal *)buf, (cufftComplex *)buf));
    else CF(cufftExecC2R(p.h, (cufftComplex *)buf, (cufftReal *)buf));
  }
  j->fft_execs++;
  const bool m = (&p != &j->n_c2r) && (&p != &j->n_r2c);
  kend_prof(j, m ? (r2c ? "cufft_r2c_M" : "cufft_c2r_M") : (r2c ? "cufft_r2c_N" : "cufft_c2r_N"),
            2.0 * double(m ? j->m_field_bytes : j->n_field_bytes) * p.batch);
  return MFX_OK;
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
static unsigned grid_for(size_t n, int block, int num_sm) {
  size_t b = (n + block - 1) / block;
  size_t cap = size_t(num_sm) * 16;  // grid-stride beyond 16 resident blocks / SM
  return unsigned(std::max<size_t>(1, std::min(b, cap)));
}

static int g_num_sm = 0;
static int num_sm() {
  if (!g_num_sm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sm, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sm <= 0) g_num_sm = 148;
  }
  return g_num_sm;
}

// KBEGIN / KEND bracket every launch: launch-error check, launch count and,
// when profiling is on, events on the job stream plus the launch's
// algorithmic byte count (each distinct input read once, each output written once).
static void kbegin(mfx_job *j) {
  j->pend = nullptr;
  if (j->prof) {
    j->pend = j->next_event();
    cudaEventRecord(j->pend, j->stream);
  }
}
static void kend_prof(mfx_job *j, const char *name, double bytes) {
  if (j->prof && j->pend) {
    cudaEvent_t b = j->next_event();
    cudaEventRecord(b, j->stream);
    j->prof_recs.push_back({name, bytes, j->pend, b});
  }
  j->pend = nullptr;
}
#define KBEGIN(j) kbegin(j)
#define KEND(j, name, bytes)                                                                       \
  do {                                                                                             \
    cudaError_t e_ = cudaGetLastError();                                                           \
    if (e_ != cudaSuccess)                                                                         \
      return set_error(MFX_ECUDA, "kernel launch: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
    (j)->own_launches++;                                                                           \
    kend_prof((j), (name), double(bytes));                                                         \
  } while (0)

template <typename R> static int launch_noise(mfx_job *j, int mode, void *out) {
  NoiseArgs a;
  a.seeds = j->seeds;
  a.amp = j->amp;
  a.amp_len = j->d.amp_table_len;
  a.N = j->N;
  a.mode = mode;
  a.fixing = j->d.fixing;
  const double volfac = std::pow(j->d.boxlen / j->N / 2.0 / M_PI, 1.5);
  a.norm = (j->d.inversion ? -1.0 : 1.0) / volfac;
  a.out_scale = j->scale1;
  const int cols = j->N * j->N;
  KBEGIN(j);
  k_noise_phi1<R><<<(cols + 127) / 128, 128, 0, j->stream>>>(a, (typename Cplx<R>::T *)out);
  KEND(j, "noise_phi1", j->n_field_bytes + 4.0 * cols + 8.0 * j->d.amp_table_len);
  return MFX_OK;
}

// MUSIC1 noise: cube normals into the padded real field, the N-grid forward
// transform in place, then the k-space pass (music.cuh)
template <typename R> static int launch_music(mfx_job *j, int mode, void *out) {
  const int N = j->N;
  const int cs = j->d.music_cubesize ? int(j->d.music_cubesize) : 32;
  using C = typename Cplx<R>::T;
  // one level's cubes into buf (padded real), then its forward transform
  auto level = [&](int l, void *buf, Plan &plan) -> int {
    const int n = 1 << l;
    music::CubeArgs c;
    c.seed = reinterpret_cast<const long long *>(j->seeds) + l;
    c.N = n;
    c.cs = n < cs ? n : cs;
    c.nc = n / c.cs;
    c.row = 2LL * (n / 2 + 1);
    KBEGIN(j);
    music::k_music_cubes<R><<<unsigned(c.nc) * c.nc * c.nc, 32, 0, j->stream>>>(c, (R *)buf);
    KEND(j, "music_cubes", double(n) * n * n * sizeof(R));
    return exec_fft(j, plan, buf, true);
  };
  const double cells = double(N) * N * N;
  if (j->d.noise_generator == MFX_NOISE_FIELD) {
    // the given real-space field: uploaded, rounded into the padded layout,
    // transformed (pageable memory is staged before the copy call returns)
    CU(cudaMemcpyAsync(j->music_buf[0], j->d.noise_field, size_t(cells) * 8, cudaMemcpyHostToDevice, j->stream));
    KBEGIN(j);
    music::k_field_to_padded<R><<<grid_for(size_t(cells), 256, num_sm()), 256, 0, j->stream>>>(
        (const double *)j->music_buf[0], (R *)out, N);
    KEND(j, "field_to_padded", cells * (8.0 + sizeof(R)));
    TRY(exec_fft(j, j->n_r2c, out, true));
  } else if (j->music_l0 == j->music_lmin) {
    TRY(level(j->music_lmin, out, j->n_r2c));
  } else if (j->music_l0 > j->music_lmin) {
    // the finer seeded level, restricted one level at a time in k-space; the
    // reference's c2r / r2c round trip between levels keeps the Hermitian
    // part of the kz = 0 and kz = n/2 planes, which the restricted spectrum
    // need not be on its Nyquist indices
    TRY(level(j->music_l0, j->music_buf[0], j->music_plans[0]));
    void *src = j->music_buf[0];
    for (int l = j->music_l0 - 1, q = 1; l >= j->music_lmin; --l, ++q) {
      void *dst = l == j->music_lmin ? out : j->music_buf[q & 1];
      const int nc = 1 << l;
      KBEGIN(j);
      music::k_music_restrict<R><<<grid_for(size_t(nc) * nc * (nc / 2 + 1), 256, num_sm()), 256, 0, j->stream>>>(
          (const C *)src, (C *)dst, nc, 1);
      KEND(j, "music_restrict", 2.0 * n_field_bytes(nc, j->rsize));
      KBEGIN(j);
      music::k_music_hermitian_planes<R><<<grid_for(size_t(nc) * nc * 2, 256, num_sm()), 256, 0, j->stream>>>(
          (C *)dst, nc);
      KEND(j, "music_planes", 8.0 * nc * nc * (j->fp64 ? 16 : 8));
      src = dst;
    }
  } else {
    // the coarsest seeded level, then each finer one with the coarser modes
    // replaced (its real-space round trip, c2r then r2c, is the identity on
    // these Hermitian spectra and is left out)
    void *prev = j->music_buf[0];
    if (j->music_lfile >= 0) {
      // the level a noise file gives: uploaded (staged in the grid-level
      // buffer, which the chain writes last), into the padded layout,
      // transformed
      const int n0 = 1 << j->music_l0;
      const size_t c0 = size_t(n0) * n0 * n0;
      CU(cudaMemcpyAsync(out, j->d.noise_field, c0 * 8, cudaMemcpyHostToDevice, j->stream));
      KBEGIN(j);
      music::k_field_to_padded<R><<<grid_for(c0, 256, num_sm()), 256, 0, j->stream>>>((const double *)out, (R *)prev,
                                                                                     n0);
      KEND(j, "field_to_padded", double(c0) * (8.0 + sizeof(R)));
      TRY(exec_fft(j, j->music_plans[0], prev, true));
    } else {
      TRY(level(j->music_l0, prev, j->music_plans[0]));
    }
    for (int l = j->music_l0 + 1; l <= j->music_lmin; ++l) {
      void *dst = l == j->music_lmin ? out : j->music_buf[(l - j->music_l0) & 1];
      TRY(level(l, dst, l == j->music_lmin ? j->n_r2c : j->music_plans[size_t(l - j->music_l0)]));
      const int nc = 1 << (l - 1);
      KBEGIN(j);
      music::k_music_embed<R><<<grid_for(size_t(nc) * nc * (nc / 2 + 1), 256, num_sm()), 256, 0, j->stream>>>(
          (const C *)prev, (C *)dst, nc, 1 << l);
      KEND(j, "music_embed", 2.0 * n_field_bytes(nc, j->rsize));
      prev = dst;
    }
  }
  music::KArgs k;
  k.amp = j->amp;
  k.amp_len = j->d.amp_table_len;
  k.N = N;
  k.mode = mode;
  k.fixing = j->d.fixing;
  k.keep_dc = j->d.noise_generator == MFX_NOISE_FIELD || j->music_lfile >= 0;  // a file's mean is kept
  k.unit = 1.0 / std::sqrt(cells);
  const double volfac = std::pow(j->d.boxlen / N / 2.0 / M_PI, 1.5);
  k.norm = (j->d.inversion ? -1.0 : 1.0) / volfac;
  k.out_scale = j->scale1;
  const size_t modes = size_t(N) * N * (N / 2 + 1);
  KBEGIN(j);
  music::k_music_phi1<R><<<grid_for(modes, 256, num_sm()), 256, 0, j->stream>>>(k, (typename Cplx<R>::T *)out);
  KEND(j, "music_phi1", 2.0 * j->n_field_bytes + (mode == 2 ? 8.0 * j->d.amp_table_len : 0.0));
  return MFX_OK;
}

template <typename R> static int make_noise(mfx_job *j, int mode, void *out) {
  return j->d.noise_generator == MFX_NOISE_NGENIC ? launch_noise<R>(j, mode, out) : launch_music<R>(j, mode, out);
}

static const int8_t kHa[6] = {0, 1, 2, 0, 0, 1};
static const int8_t kHb[6] = {0, 1, 2, 1, 2, 2};

template <typename R> static int hessians(mfx_job *j, const void *phi, void **out) {
  PadArgs a;
  a.phi = phi;
  for (int c = 0; c < 6; ++c) {
    a.out[c] = out[c];
    a.ca[c] = kHa[c];
    a.cb[c] = kHb[c];
  }
  a.ncomp = 6;
  a.N = j->N;
  a.M = j->M;
  a.kfac = 2.0 * M_PI / j->d.boxlen;
  const double M3 = double(j->M) * j->M * j->M;
  a.fac = std::pow(1.5, 1.5) / std::sqrt(M3);
  const size_t total = size_t(j->M) * j->M * j->mk;
  KBEGIN(j);
  k_pad_hessian<R><<<grid_for(total, 256, num_sm()), 256, 0, j->stream>>>(a);
  KEND(j, "pad_hessian", j->n_field_bytes + 6.0 * j->m_field_bytes);
  for (int c = 0; c < 6; ++c) TRY(exec_fft(j, j->m_c2r, out[c], false));
  return MFX_OK;
}

template <typename R> static int unpad_invlap(mfx_job *j, void *F, void *out) {
  TRY(exec_fft(j, j->m_r2c, F, true));
  UnpadArgs a;
  a.F = F;
  a.out = out;
  a.N = j->N;
  a.M = j->M;
  a.kfac = 2.0 * M_PI / j->d.boxlen;
  const double M3 = double(j->M) * j->M * j->M, N3 = double(j->N) * j->N * j->N;
  const double rfac_u = std::sqrt(M3) / std::sqrt(N3);
  a.fac = 1.0 / std::sqrt(M3) / rfac_u;
  const size_t total = size_t(j->N) * j->N * j->nk;
  KBEGIN(j);
  k_unpad_invlap<R><<<grid_for(total, 256, num_sm()), 256, 0, j->stream>>>(a);
  KEND(j, "unpad_invlap", 2.0 * j->n_field_bytes);
  return MFX_OK;
}

// ---------------------------------------------------------------------------
// pruned, fused transforms of the FP32 form (fused.cuh)
// ---------------------------------------------------------------------------
static void tune_fused(mfx_job *j);

static ff::FArgs ff_args(mfx_job *j) {
  ff::FArgs a{};
  a.tw = j->ff_tw;
  a.status = j->dstatus;
  a.kfac = float(2.0 * M_PI / j->d.boxlen);
  return a;
}

// x/y pass kinds with a tile of their own (mfx_job::ff_pk)
enum XYKind { K_Y3 = 0, K_X6 = 1, K_XF = 2, K_YF = 3, K_YT = 4, K_XI = 5 };
static const char *const kXYNames[6] = {"ff_y3", "ff_x6", "ff_x_fwd", "ff_y_fwd", "ff_y_trunc", "ff_x_inv"};

static int ff_run(mfx_job *j, int op, int p, const ff::FArgs &a, const char *name, double bytes) {
  KBEGIN(j);
  const cudaError_t e = ff::ff_launch(j->M, op, p, a, j->stream);
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "%s (M = %d, tile %d): %s", name, j->M, p, cudaGetErrorString(e));
  KEND(j, name, bytes);
  return MFX_OK;
}

// the six padded Hessians of an N-grid field into C-space C[0..5]
static int ff_hessians(mfx_job *j, const void *phi, void *const *C) {
  const int N = j->N, M = j->M, Kh = N / 2;
  const double M3 = double(M) * M * M;
  const double bB = double(N) * M * Kh * 8, bC = double(M) * M * Kh * 8;
  ff::FArgs y = ff_args(j);
  y.src[0] = static_cast<const float2 *>(phi);
  for (int o = 0; o < 3; ++o) y.dst[o] = static_cast<float2 *>(j->ffB[o]);
  y.ncomp = 3;
  y.fac = float(std::pow(1.5, 1.5) / std::sqrt(M3));
  TRY(ff_run(j, ff::FF_Y3, j->xy_tile(K_Y3), y, "ff_y3", double(N) * N * Kh * 8 + 3 * bB));
  ff::FArgs x = ff_args(j);
  for (int o = 0; o < 3; ++o) x.src[o] = static_cast<const float2 *>(j->ffB[o]);
  for (int c = 0; c < 6; ++c) x.dst[c] = static_cast<float2 *>(C[c]);
  x.ncomp = 6;
  x.mode = 0;
  TRY(ff_run(j, ff::FF_XINV, j->xy_tile(K_X6), x, "ff_x6", 3 * bB + 6 * bC));
  return MFX_OK;
}

// forward x and y transforms of D-space outputs: unpadded and inverse
// Laplacian'd into N-grid fields (mode 0), or truncated and brought back to
// C-space (mode 1, convolve3's first pairs)
static int ff_finish(mfx_job *j, void *D, void *out, int mode) {
  const int N = j->N, M = j->M, Kh = N / 2;
  const double M3 = double(M) * M * M, N3 = double(N) * N * N;
  const double bB = double(N) * M * Kh * 8, bC = double(M) * M * Kh * 8;
  const double rfac_u = std::sqrt(M3) / std::sqrt(N3), rfac_p = std::pow(1.5, 1.5);
  ff::FArgs x = ff_args(j);
  x.src[0] = static_cast<const float2 *>(D);
  x.dst[0] = static_cast<float2 *>(j->ffB[0]);
  x.ncomp = 1;
  TRY(ff_run(j, ff::FF_XFWD, j->xy_tile(K_XF), x, "ff_x_fwd", bC + bB));
  ff::FArgs y = ff_args(j);
  y.src[0] = static_cast<const float2 *>(j->ffB[0]);
  y.ncomp = 1;
  y.mode = mode;
  if (mode == 0) {
    y.dst[0] = static_cast<float2 *>(out);
    y.fac = float(1.0 / std::sqrt(M3) / rfac_u);
    TRY(ff_run(j, ff::FF_YFWD, j->xy_tile(K_YF), y, "ff_y_fwd", bB + double(j->n_field_bytes)));
  } else {
    y.dst[0] = static_cast<float2 *>(j->ffB[0]);  // each CTA owns its tile: in place
    y.fac = float((1.0 / std::sqrt(M3) / rfac_u) * rfac_p / std::sqrt(M3));
    TRY(ff_run(j, ff::FF_YFWD, j->xy_tile(K_YT), y, "ff_y_trunc", 2 * bB));
    ff::FArgs xi = ff_args(j);
    xi.src[0] = static_cast<const float2 *>(j->ffB[0]);
    xi.dst[0] = static_cast<float2 *>(out);
    xi.ncomp = 1;
    xi.mode = 1;
    TRY(ff_run(j, ff::FF_XINV, j->xy_tile(K_XI), xi, "ff_x_inv", bB + bC));
  }
  return MFX_OK;
}

// LPT potentials phi2, phi3, A3 through the fused transforms (FP32 form).
// C-space slots: ffC[0..5] phi1 Hessians, ffC[6..11] the 2LPT source and the
// five pair products (then the phi2 Hessians), ffC[12..16] truncated pairs.
static int run_potentials_fused(mfx_job *j) {
  const int order = j->d.lpt_order, M = j->M, Kh = j->N / 2;
  const double bC = double(M) * M * Kh * 8;
  void *const *C1 = &j->ffC[0];
  void *const *D = &j->ffC[6];
  TRY(ff_hessians(j, j->nf[0], C1));
  {
    ff::FArgs z = ff_args(j);
    for (int c = 0; c < 6; ++c) z.src[c] = static_cast<const float2 *>(C1[c]);
    const int nout = order >= 3 ? 6 : 1;
    for (int o = 0; o < nout; ++o) z.dst[o] = static_cast<float2 *>(D[o]);
    z.mode = order >= 3 ? 1 : 0;
    TRY(ff_run(j, ff::FF_ZSRC2, j->ff_pz2, z, "ff_zsrc2", 6 * bC + nout * bC));
  }
  TRY(ff_finish(j, D[0], j->nf[1], 0));
  if (j->timed) CU(cudaEventRecord(j->ev[2], j->stream));
  if (order >= 3) {
    void *const *CT = &j->ffC[12];
    for (int t = 0; t < 5; ++t) TRY(ff_finish(j, D[1 + t], CT[t], 1));
    void *const *C2 = &j->ffC[6];
    TRY(ff_hessians(j, j->nf[1], C2));
    ff::FArgs z = ff_args(j);
    for (int c = 0; c < 6; ++c) {
      z.src[c] = static_cast<const float2 *>(C1[c]);
      z.src[6 + c] = static_cast<const float2 *>(C2[c]);
    }
    for (int t = 0; t < 5; ++t) z.src[12 + t] = static_cast<const float2 *>(CT[t]);
    for (int o = 0; o < 4; ++o) z.dst[o] = static_cast<float2 *>(CT[o]);  // in place, row by row
    TRY(ff_run(j, ff::FF_ZSRC3, j->ff_pz, z, "ff_zsrc3", 17 * bC + 4 * bC));
    for (int o = 0; o < 4; ++o) TRY(ff_finish(j, CT[o], j->nf[2 + o], 0));
  }
  return MFX_OK;
}

// default tile shapes: the largest x/y tile of at most 512 threads, and one
// row per step of the persistent z passes (two fit one CTA per SM only)
static void ff_default_tiles(mfx_job *j) {
  j->ff_pxy = 4;
  for (int p : {16, 8, 4})
    if (ff::ff_valid(j->M, ff::FF_XFWD, p) && p * ff::ff_maxj(j->M) <= 512) {
      j->ff_pxy = p;
      break;
    }
  j->ff_pz = 1;
}

// pencil-tile shapes chosen by mfx_job_autotune for this size class, if any
static void tune_fused(mfx_job *j) {
  std::lock_guard<std::mutex> lk(j->eng->mu);
  auto it = j->eng->ff_tuned.find(j->N);
  if (it != j->eng->ff_tuned.end()) {
    j->ff_pxy = it->second.pxy;
    j->ff_pz = it->second.pz;
    j->ff_pz2 = it->second.pz2;
    for (int k = 0; k < 6; ++k) j->ff_pk[k] = it->second.pk[k];
  }
}

// Times the fused passes for every admissible pencil-tile shape on the job's
// own buffers and keeps the fastest per size class (engine-wide cache).
static int autotune_fused(mfx_job *j) {
  const int N = j->N, M = j->M;
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  auto timed = [&](auto &&launch) -> float {
    launch();  // warm
    cudaEventRecord(e0, j->stream);
    launch();
    cudaEventRecord(e1, j->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  const bool prof = j->prof;
  j->prof = false;
  int best_xy = j->ff_pxy;
  float tbest = 1e30f;
  int rc = MFX_OK;
  // every x/y tile on the phi1 Hessian passes and one forward x/y pair of each
  // kind, each launch timed on its own (the job's profiling events); each pass
  // kind keeps its fastest tile, ff_pxy the fastest over all of them
  float tk[6], tsum_best = 1e30f;
  int pk[6] = {};
  for (int k = 0; k < 6; ++k) tk[k] = 1e30f;
  for (int p : {32, 16, 8, 4}) {
    if (rc != MFX_OK || !ff::ff_valid(M, ff::FF_XFWD, p)) continue;
    const int save = j->ff_pxy;
    int savek[6];
    for (int k = 0; k < 6; ++k) {
      savek[k] = j->ff_pk[k];
      j->ff_pk[k] = 0;
    }
    j->ff_pxy = p;
    float tp[6] = {0, 0, 0, 0, 0, 0};
    for (int rep = 0; rep < 2 && rc == MFX_OK; ++rep) {  // warm, then timed
      j->prof = true;
      j->prof_recs.clear();
      j->ev_next = 0;
      if (rc == MFX_OK) rc = ff_hessians(j, j->nf[0], &j->ffC[0]);
      if (rc == MFX_OK) rc = ff_finish(j, j->ffC[0], j->ffC[6], 1);
      if (rc == MFX_OK) rc = ff_finish(j, j->ffC[0], j->nf[1], 0);
      if (rc == MFX_OK && cudaStreamSynchronize(j->stream) != cudaSuccess) rc = set_error(MFX_ECUDA, "autotune sync");
      if (rep == 1 && rc == MFX_OK)
        for (const auto &r : j->prof_recs) {
          float e = 0;
          cudaEventElapsedTime(&e, r.a, r.b);
          for (int k = 0; k < 6; ++k)
            if (std::strcmp(r.name, kXYNames[k]) == 0) tp[k] += e;
        }
    }
    j->prof_recs.clear();
    j->ff_pxy = save;
    for (int k = 0; k < 6; ++k) j->ff_pk[k] = savek[k];
    if (rc != MFX_OK) break;
    float tsum = 0;
    for (int k = 0; k < 6; ++k) {
      tsum += tp[k];
      if (tp[k] < tk[k]) {
        tk[k] = tp[k];
        pk[k] = p;
      }
    }
    if (tsum < tsum_best) {
      tsum_best = tsum;
      best_xy = p;
    }
  }
  j->prof = false;
  // the z passes, each shape timed on the job's own fields: ZSRC2 always,
  // ZSRC3 for 3LPT jobs
  int best_z2 = j->ff_pz2, best_z3 = j->ff_pz;
  for (int op : {ff::FF_ZSRC2, ff::FF_ZSRC3}) {
    if (op == ff::FF_ZSRC3 && j->d.lpt_order < 3) continue;
    tbest = 1e30f;
    for (int p : {1, 2, 3, 4}) {
      if (rc != MFX_OK || !ff::ff_valid(M, op, p)) continue;
      const float t = timed([&] {
        ff::FArgs z = ff_args(j);
        if (op == ff::FF_ZSRC3) {
          for (int c = 0; c < 17; ++c) z.src[c] = static_cast<const float2 *>(j->ffC[c]);
          for (int o = 0; o < 4; ++o) z.dst[o] = static_cast<float2 *>(j->ffC[12 + o]);
          if (rc == MFX_OK) rc = ff_run(j, ff::FF_ZSRC3, p, z, "ff_zsrc3", 0);
        } else {
          // the 3LPT form's ZSRC2 (mode 1: the five pair products as well)
          for (int c = 0; c < 6; ++c) z.src[c] = static_cast<const float2 *>(j->ffC[c]);
          const int nout = j->d.lpt_order >= 3 ? 6 : 1;
          for (int o = 0; o < nout; ++o) z.dst[o] = static_cast<float2 *>(j->ffC[6 + o]);
          z.mode = nout > 1 ? 1 : 0;
          if (rc == MFX_OK) rc = ff_run(j, ff::FF_ZSRC2, p, z, "ff_zsrc2", 0);
        }
      });
      if (t < tbest) {
        tbest = t;
        (op == ff::FF_ZSRC3 ? best_z3 : best_z2) = p;
      }
    }
  }
  j->prof = prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(rc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "autotune: %s", cudaGetErrorString(e));
  j->ff_pxy = best_xy;
  for (int k = 0; k < 6; ++k) j->ff_pk[k] = pk[k];
  j->ff_pz = best_z3;
  j->ff_pz2 = best_z2;
  std::lock_guard<std::mutex> lk(j->eng->mu);
  j->eng->ff_tuned[N] = {best_xy, best_z3, best_z2, {pk[0], pk[1], pk[2], pk[3], pk[4], pk[5]}};
  return MFX_OK;
}

// Displacement / velocity assembly and particles (ic_generator.cc:937-1030):
// the LPT orders in `mask` (bit n-1: order n) are combined, the others left out.
// Fused assembly of the FP32 form (fused_asm.cuh): per sub-lattice, the
// assembly with the inverse x transform, the inverse y transform, and the
// inverse z transform with the particle read-out; the six components live in
// the first six assembly buffers.
static int assemble_fused(mfx_job *j, const AsmArgs &as) {
  const int N = j->N, ns = j->ns, order = j->d.lpt_order;
  const double qf = double(N) * N * (N / 2) * 8;  // one component field
  const double nfb = double(j->n_field_bytes);
  const double N3 = double(N) * N * N;
  const double pb = j->host_q ? N3 * (12.0 + 3.0 * (j->d.vel64 ? 8 : 4))
                               : N3 * (3.0 * (j->d.pos64 ? 8 : 4) + 3.0 * (j->d.vel64 ? 8 : 4) + (j->d.id64 ? 8 : 4));
  // velocity / displacement magnitude ratio of the assembly: vfac * vunit / lunit
  const double vfmax = std::max({std::fabs(as.vfac1), std::fabs(as.vfac2), std::fabs(as.vfac3)});
  const double ratio = (vfmax > 0 && as.pfac != 0) ? vfmax * std::fabs(as.vfac / as.pfac) : 1.0;
  const float vscale = float(ratio > 0 ? 1.0 / ratio : 1.0);
  // all sub-lattices from one assembly when their components fit the buffers;
  // MFX_FA_KEEP=0 in the environment assembles per sub-lattice (for comparisons)
  const char *env = getenv("MFX_FA_KEEP");
  const bool keep = !(env && env[0] == '0');
  const int nsub = (keep && ns > 1 && ff::fa_all(j->M) && j->group >= ns) ? ns : 1;
  // ASM1 in halves (tiles of 8 pencils) from N = 384 up, where the x pass's
  // 32-byte row pieces of the 4-pencil tiles lie megabytes apart (768^3 FCC:
  // 57 -> 44 ms; 256^3 BCC: 0.63 -> 0.93 ms, so not there), and wherever the
  // 4-pencil form does not fit; MFX_FA_HALVES = 0 / 1 in the environment
  // forces it off / on where both fit (for comparisons)
  const char *envh = getenv("MFX_FA_HALVES");
  const bool halves = nsub > 1 && ff::fa_halves(j->M) &&
                      (!ff::fa_keep(j->M) || (envh ? envh[0] == '1' : N >= 384));
  const bool plt = as.plt != nullptr;
  ff::FAArgs fa{};
  fa.as = as;
  fa.tw = j->ff_twn;
  fa.status = j->dstatus;
  fa.pos = j->pos;
  fa.vel = j->vel;
  fa.ids = nullptr;  // ids on request (k_fill_ids) or from the fetch's host threads
  fa.pos_disp = j->host_q ? 1 : 0;
  fa.pos64 = j->d.pos64;
  fa.vel64 = j->d.vel64;
  fa.id64 = j->d.id64;
  fa.nshift_total = ns;
  fa.id_offset = j->d.id_offset * uint64_t(ns) * uint64_t(N3);
  fa.vscale = vscale;
  fa.vunscale = 1.0 / double(vscale);
  fa.vunscale_f = float(fa.vunscale);
  fa.halves = halves ? 1 : 0;
  auto pass = [&](int op, const char *name, double bytes) -> int {
    KBEGIN(j);
    const cudaError_t e = ff::fa_launch(j->M, op, plt, fa, j->stream);
    if (e != cudaSuccess) return set_error(MFX_ECUDA, "%s (N = %d): %s", name, N, cudaGetErrorString(e));
    KEND(j, name, bytes);
    return MFX_OK;
  };
  const double in_b = (order == 1 ? 1.0 : (order == 2 ? 2.0 : 6.0)) * nfb;
  // sub-lattices with equal x-shifts (FCC: 0, 0, 1/2, 1/2) share one x pass
  // output: the x pass applies only the x factor of the phase and the y pass
  // the y and z factors; each shared output is read out of place by the other
  // sub-lattices first and in place by its own last.  MFX_FA_XONLY=0 in the
  // environment turns this off (for comparisons)
  int xrep[4] = {0, 0, 0, 0}, xvar[4] = {0, 0, 0, 0}, nxv = 0;
  for (int s = 0; s < ns; ++s) {
    int v = 0;
    while (v < nxv && kShifts[j->d.lattice][xrep[v]][0] != kShifts[j->d.lattice][s][0]) ++v;
    if (v == nxv) xrep[nxv++] = s;
    xvar[s] = v;
  }
  const char *envx = getenv("MFX_FA_XONLY");
  if (nsub == ns && nxv < ns && !(envx && envx[0] == '0')) {
    fa.shift = 0;
    fa.nsub = nxv;
    fa.xonly = 1;
    for (int v = 0; v < nxv; ++v) {
      fa.xsub[v] = xrep[v];
      for (int c = 0; c < 6; ++c) fa.qx[6 * v + c] = static_cast<float2 *>(j->asmbuf[6 * xrep[v] + c]);
    }
    TRY(pass(ff::FA_X, "fa_x", in_b + 6 * nxv * qf));
    fa.xonly = 0;
    fa.yzphase = 1;
    for (int v = 0; v < nxv; ++v)
      for (int pass_rep = 0; pass_rep < 2; ++pass_rep)
        for (int s = 0; s < ns; ++s) {
          if (xvar[s] != v || (s == xrep[v]) != (pass_rep == 1)) continue;
          fa.shift = s;
          for (int c = 0; c < 6; ++c) {
            fa.q[c] = static_cast<float2 *>(j->asmbuf[6 * s + c]);
            fa.qin[c] = s == xrep[v] ? nullptr : static_cast<const float2 *>(j->asmbuf[6 * xrep[v] + c]);
          }
          fa.qtab = j->qtab + size_t(s) * 3 * N;
          TRY(pass(ff::FA_Y, "fa_y", 12 * qf));
          TRY(pass(ff::FA_Z, "fa_z", 6 * qf + pb));
        }
    return MFX_OK;
  }
  for (int s0 = 0; s0 < ns; s0 += nsub) {
    fa.shift = s0;
    fa.nsub = nsub;
    for (int q = 0; q < 6 * nsub; ++q) fa.qx[q] = static_cast<float2 *>(j->asmbuf[q]);
    TRY(pass(ff::FA_X, "fa_x", in_b + 6 * nsub * qf));
    for (int s = 0; s < nsub; ++s) {
      fa.shift = s0 + s;
      for (int c = 0; c < 6; ++c) fa.q[c] = static_cast<float2 *>(j->asmbuf[6 * s + c]);
      fa.qtab = j->qtab + size_t(s0 + s) * 3 * N;
      TRY(pass(ff::FA_Y, "fa_y", 12 * qf));
      TRY(pass(ff::FA_Z, "fa_z", 6 * qf + pb));
    }
  }
  return MFX_OK;
}

// Particle masses of the job's species (mfx_job_set_species), per sub-lattice:
// the delta_bc field from phi1 with the sub-lattice phase, its c2r and the
// read-out (ic_generator.cc:749-780, particle_generator.hh:369-427)
static NyqSteps nyq_steps(const mfx_job *j);

template <typename R> static int mass_stage(mfx_job *j) {
  const int N = j->N, nsm = num_sm();
  const double N3 = double(N) * N * N;
  MassArgs m{};
  m.phi1 = j->nf[0];
  m.ratio = j->rho_ratio;
  m.ratio_len = j->rho_ratio ? j->sp_len : 0;
  m.phase = j->phase;
  m.field = j->rho;
  m.mass = j->mass;
  m.N = N;
  m.nshift_total = j->ns;
  m.c_species = j->c_species;
  m.norm = 1.0 / std::sqrt(N3);
  m.scale = j->mass_factor / (double(j->ns) * N3);
  m.nyq = nyq_steps(j);
  const size_t total = size_t(N) * N * j->nk;
  for (int s = 0; s < j->ns; ++s) {
    m.shift = s;
    KBEGIN(j);
    k_mass_field<R><<<grid_for(total, 256, nsm), 256, 0, j->stream>>>(m);
    KEND(j, "mass_field", 2.0 * j->n_field_bytes);
    kbegin(j);
    if (j->fp64) CF(cufftExecZ2D(j->rho_c2r.h, (cufftDoubleComplex *)j->rho, (cufftDoubleReal *)j->rho));
    else CF(cufftExecC2R(j->rho_c2r.h, (cufftComplex *)j->rho, (cufftReal *)j->rho));
    j->fft_execs++;
    kend_prof(j, "cufft_c2r_mass", 2.0 * j->n_field_bytes);
    KBEGIN(j);
    if (j->d.pos64) k_masses<R, double><<<grid_for(size_t(N3), 256, nsm), 256, 0, j->stream>>>(m);
    else k_masses<R, float><<<grid_for(size_t(N3), 256, nsm), 256, 0, j->stream>>>(m);
    KEND(j, "masses", N3 * (double(j->rsize) + (j->d.pos64 ? 8.0 : 4.0)));
  }
  j->has_masses = true;
  return MFX_OK;
}

template <typename R> static int assemble_stage(mfx_job *j, int mask) {
  const int order = j->d.lpt_order;
  const int nsm = num_sm();
  const int N = j->N;
  const double N3 = double(N) * N * N;
  AsmArgs a{};
  for (int q = 0; q < 3; ++q) {
    a.phi[q] = j->nf[q];
    a.A3[q] = j->nf[3 + q];
  }
  a.plt = j->d.plt ? j->plt : nullptr;
  a.plt4 = j->d.plt ? j->plt4 : nullptr;
  a.phase = j->phase;
  a.phase32 = j->phase32;
  a.N = N;
  a.order = order;
  a.kfac = 2.0 * M_PI / j->d.boxlen;
  a.mapratio = double(MFX_PLT_NGRID) / double(N);
  a.boxlen = j->d.boxlen;
  a.g1 = j->d.g1;
  a.g2 = j->d.g2;
  a.g3 = j->d.g3;
  a.g3c = j->d.g3c;
  a.vfac1 = j->d.vfac1;
  a.vfac2 = j->d.vfac2;
  a.vfac3 = j->d.vfac3;
  if (!(mask & 1)) a.g1 = a.vfac1 = 0.0;
  if (!(mask & 2)) a.g2 = a.vfac2 = 0.0;
  if (!(mask & 4)) a.g3 = a.g3c = a.vfac3 = 0.0;
  a.pfac = j->d.lunit / j->d.boxlen / std::sqrt(N3);
  a.vfac = j->d.vunit / j->d.boxlen / std::sqrt(N3);
  a.in_scale1 = 1.0 / j->scale1;
  a.in_scale2 = 1.0 / j->scale2;
  a.in_scale3 = 1.0 / j->scale3;
  asm_float_coefficients(a);
  if (j->qvbc && (mask & 1)) {
    a.qvbc = j->qvbc;
    a.qvbc32 = j->qvbc32;
    a.qvbc_len = j->sp_len;
  }
  a.nyq = nyq_steps(j);
  if (j->fused) {
    TRY(assemble_fused(j, a));
    return j->want_masses ? mass_stage<R>(j) : MFX_OK;
  }
  const size_t total = size_t(N) * N * j->nk;
  for (int s0 = 0; s0 < j->ns; s0 += j->group) {
    const int g = std::min(j->group, j->ns - s0);
    a.shift0 = s0;
    a.nshift = g;
    for (int q = 0; q < 6 * g; ++q) a.out[q] = j->asmbuf[q];
    KBEGIN(j);
    if (a.plt) k_assemble<R, true><<<grid_for(total, 256, nsm), 256, 0, j->stream>>>(a);
    else k_assemble<R, false><<<grid_for(total, 256, nsm), 256, 0, j->stream>>>(a);
    KEND(j, "assemble", ((order == 1 ? 1.0 : (order == 2 ? 2.0 : 6.0)) + 6.0 * g) * j->n_field_bytes);
    for (int s = 0; s < g; ++s) {
      TRY(exec_fft(j, j->n_c2r, j->asmbuf[s * 6], false));  // the six components (batched)
      PartArgs p{};
      for (int q = 0; q < 6; ++q) p.f[q] = j->asmbuf[s * 6 + q];
      p.pos = j->pos;
      p.vel = j->vel;
      p.ids = j->ids;
      p.N = N;
      p.nshift_total = j->ns;
      p.ishift = s0 + s;
      p.pos64 = j->d.pos64;
      p.vel64 = j->d.vel64;
      p.id64 = j->d.id64;
      p.sx = kShifts[j->d.lattice][s0 + s][0] + j->lat_off[0];
      p.sy = kShifts[j->d.lattice][s0 + s][1] + j->lat_off[1];
      p.sz = kShifts[j->d.lattice][s0 + s][2] + j->lat_off[2];
      p.lunit = j->d.lunit;
      p.qtab = j->qtab + size_t(s0 + s) * 3 * N;
      p.id_offset = j->d.id_offset * uint64_t(j->ns) * uint64_t(N3);
      KBEGIN(j);
      const unsigned pg = grid_for(size_t(N) * N * N / 4, 256, nsm);
      if (p.pos64 && p.vel64) k_particles<R, double, double><<<pg, 256, 0, j->stream>>>(p);
      else if (p.pos64) k_particles<R, double, float><<<pg, 256, 0, j->stream>>>(p);
      else if (p.vel64) k_particles<R, float, double><<<pg, 256, 0, j->stream>>>(p);
      else k_particles<R, float, float><<<pg, 256, 0, j->stream>>>(p);
      KEND(j, "particles", N3 * (6.0 * j->rsize + 3.0 * (p.pos64 ? 8 : 4) + 3.0 * (p.vel64 ? 8 : 4) + (p.id64 ? 8 : 4)));
    }
  }
  return j->want_masses ? mass_stage<R>(j) : MFX_OK;
}

// points the particle arrays at ring set s (pos | vel | ids)
static void ring_point(mfx_job *j, int s) {
  const size_t np = j->npart;
  char *a = j->ring + size_t(s) * j->ring_set_bytes;
  j->pos = a;
  a += align_up(np * 3 * (j->host_q ? 4 : (j->d.pos64 ? 8 : 4)));
  j->vel = a;
  a += align_up(np * 3 * (j->d.vel64 ? 8 : 4));
  j->ids = (j->host_q || j->fused) ? nullptr : a;  // the fused read-out writes no device ids
}

template <typename R> static int run_pipeline(mfx_job *j) {
  const int order = j->d.lpt_order;
  const size_t mreal = size_t(j->M) * j->M * (j->M + 2);
  const int nsm = num_sm();
  j->own_launches = 0;
  j->fft_execs = 0;
  j->prof_recs.clear();
  j->ev_next = 0;
  // an asynchronous download of the last run's particles may still read them:
  // in the arena they lie in the region this run's fields overwrite, so the
  // run waits for it; in the ring only this run's assembly waits, for the
  // download from the set it writes
  if (j->fetched && !j->ring) CU(cudaStreamWaitEvent(j->stream, j->fetched, 0));
  const int rset = j->ring_next;
  if (j->ring) ring_point(j, rset);
  if (j->timed) CU(cudaEventRecord(j->ev[0], j->stream));
  TRY(make_noise<R>(j, 2, j->nf[0]));
  if (j->timed) CU(cudaEventRecord(j->ev[1], j->stream));
  void **H1 = &j->mslot[0];
  if (j->fused) {
    TRY(run_potentials_fused(j));
  } else {
  if (order >= 2) {
    TRY(hessians<R>(j, j->nf[0], H1));
    SrcArgs s{};
    for (int c = 0; c < 6; ++c) s.h1[c] = H1[c];
    s.out[0] = j->mslot[6];
    s.count = mreal;
    KBEGIN(j);
    k_src2<R><<<grid_for(mreal, 256, nsm), 256, 0, j->stream>>>(s);
    KEND(j, "src2", 7.0 * j->m_field_bytes);
    TRY(unpad_invlap<R>(j, j->mslot[6], j->nf[1]));
  }
  if (j->timed) CU(cudaEventRecord(j->ev[2], j->stream));
  if (order >= 3) {
    // phi3a: pairwise dealiased triple products (ic_generator.cc:577-586).
    // The five first-pair products are formed in one pass, each is truncated to
    // the N-grid modes (r2c, unpad, re-pad, c2r), and one fused kernel combines
    // them with the third factors, the phi3b terms and the A3 sources.
    void **T = &j->mslot[6];
    void **H2 = &j->mslot[11];
    const double M3 = double(j->M) * j->M * j->M, N3 = double(j->N) * j->N * j->N;
    const double rfac_u = std::sqrt(M3) / std::sqrt(N3), rfac_p = std::pow(1.5, 1.5);
    {
      SrcArgs s{};
      for (int c = 0; c < 6; ++c) s.h1[c] = H1[c];
      for (int t = 0; t < 5; ++t) s.out[t] = T[t];
      s.count = mreal;
      KBEGIN(j);
      k_pairs3a<R><<<grid_for(mreal, 256, nsm), 256, 0, j->stream>>>(s);
      KEND(j, "pairs3a", 10.0 * j->m_field_bytes);
    }
    for (int t = 0; t < 5; ++t) {
      TRY(exec_fft(j, j->m_r2c, T[t], true));
      TruncArgs ta;
      ta.F = T[t];
      ta.N = j->N;
      ta.M = j->M;
      ta.fac = (1.0 / std::sqrt(M3) / rfac_u) * rfac_p / std::sqrt(M3);
      KBEGIN(j);
      k_trunc_repad<R><<<grid_for(size_t(j->M) * j->M * j->mk, 256, nsm), 256, 0, j->stream>>>(ta);
      KEND(j, "trunc_repad", 2.0 * j->m_field_bytes);
      TRY(exec_fft(j, j->m_c2r, T[t], false));
    }
    TRY(hessians<R>(j, j->nf[1], H2));
    SrcArgs s{};
    for (int c = 0; c < 6; ++c) {
      s.h1[c] = H1[c];
      s.h2[c] = H2[c];
    }
    for (int t = 0; t < 5; ++t) s.t[t] = T[t];
    for (int q = 0; q < 4; ++q) s.out[q] = T[q];  // phi3 source, A3x, A3y, A3z
    s.count = mreal;
    KBEGIN(j);
    k_src3<R><<<grid_for(mreal, 256, nsm), 256, 0, j->stream>>>(s);
    KEND(j, "src3", 21.0 * j->m_field_bytes);
    TRY(unpad_invlap<R>(j, T[0], j->nf[2]));
    for (int d = 0; d < 3; ++d) TRY(unpad_invlap<R>(j, T[1 + d], j->nf[3 + d]));
  }
  }  // cuFFT path
  if (j->timed) CU(cudaEventRecord(j->ev[3], j->stream));
  if (j->ring) CU(cudaStreamWaitEvent(j->stream, j->ring_free[rset], 0));
  if (j->d.want_particles) TRY(assemble_stage<R>(j, 7));
  if (j->timed) CU(cudaEventRecord(j->ev[4], j->stream));
  if (j->ring) j->ring_next = (rset + 1) % j->ring_sets;
  j->has_run = true;
  j->noise_only = false;
  return MFX_OK;
}

// ---------------------------------------------------------------------------
// job set-up
// ---------------------------------------------------------------------------
static int upload_tables(mfx_job *j, const mfx_job_desc *d) {
  const int N = j->N;
  j->amp_host.assign(d->amp_table, d->amp_table + d->amp_table_len);
  // the MUSIC1 base seed lives on the device like NGenIC's table, so that a
  // captured pipeline draws the noise of the seed uploaded last
  if (d->noise_generator == MFX_NOISE_NGENIC)
    CU(cudaMemcpyAsync(j->seeds, d->seed_table, size_t(N) * N * 4, cudaMemcpyHostToDevice, j->stream));
  else
  {
    // the effective seed of every level, indexed by level (pageable: staged
    // before the call returns)
    const MusicLevels ml = music_levels(d);
    CU(cudaMemcpyAsync(j->seeds, ml.seed, sizeof(ml.seed), cudaMemcpyHostToDevice, j->stream));
  }
  CU(cudaMemcpyAsync(j->amp, d->amp_table, d->amp_table_len * 8, cudaMemcpyHostToDevice, j->stream));
  if (d->plt) {
    CU(cudaMemcpyAsync(j->plt, d->plt_table, size_t(MFX_PLT_TABLE_DOUBLES) * 8, cudaMemcpyHostToDevice,
                       j->stream));
    if (!j->fp64) {
      // interleave (D_r, D_theta, D_phi, alpha^-1) per mode for the FP32 form,
      // on the device from the tables just uploaded: no copy from pageable
      // host memory (which synchronises the host and can queue behind the
      // particle downloads of a pipelined run on the copy engine)
      const size_t nm = size_t(MFX_PLT_TABLE_DOUBLES) / 4;
      k_plt_to_f4<<<int((nm + 255) / 256), 256, 0, j->stream>>>(j->plt, j->plt4, nm);
      CU(cudaGetLastError());
    }
  }
  return MFX_OK;
}

// Particle ids are a closed form of the particle's index, the lattice
// generator's rule (particle_generator.hh:229-248): particle p = shift * N^3 +
// cell carries id_offset * ns * N^3 + ns * cell + shift, the value the read-out
// kernels write on the device.  A fetch writes them into the caller's array
// with host threads beside the copies instead of moving 8 (or 4) more bytes per
// particle over the host link, which bounds a realisation end to end.
struct IdRule {
  uint64_t base, ns, n3;
  bool id64;
};
static IdRule id_rule(const mfx_job *j) {
  const uint64_t n3 = uint64_t(j->d.ngrid) * j->d.ngrid * j->d.ngrid, ns = uint64_t(j->ns);
  return {j->d.id_offset * ns * n3, ns, n3, j->d.id64 != 0};
}
template <class T>
static void write_ids(T *o, uint64_t p0, uint64_t p1, const IdRule &r) {
  while (p0 < p1) {  // one run of cells per sub-lattice shift
    const uint64_t s = p0 / r.n3, c0 = p0 % r.n3, c1 = std::min<uint64_t>(r.n3, c0 + (p1 - p0));
    const uint64_t b = r.base + s;
    for (uint64_t c = c0; c < c1; ++c) o[c - c0] = T(b + r.ns * c);
    o += c1 - c0;
    p0 += c1 - c0;
  }
}
static void write_ids(const IdRule &r, uint64_t p0, uint64_t p1, void *dst) {  // dst holds particle p0
  if (r.id64) write_ids(static_cast<uint64_t *>(dst), p0, p1, r);
  else write_ids(static_cast<uint32_t *>(dst), p0, p1, r);
}
// starts host threads writing the ids of particles [first, first + count) into
// dst; join_id_fill waits for them
static void start_id_fill(mfx_job *j, size_t first, size_t count, void *dst) {
  if (!dst || !count) return;
  const IdRule r = id_rule(j);
  const size_t hw = std::max(2u, std::thread::hardware_concurrency());
  const size_t nt = std::max<size_t>(1, std::min<size_t>({size_t(8), hw / 2, count >> 21}));
  const size_t per = (count + nt - 1) / nt, es = r.id64 ? 8 : 4;
  for (size_t t = 0; t < nt; ++t) {
    const size_t a = first + t * per, b = std::min(first + count, a + per);
    if (a >= b) break;
    void *o = static_cast<char *>(dst) + es * (a - first);
    try {
      j->id_fill.emplace_back([r, a, b, o] { write_ids(r, a, b, o); });
    } catch (const std::system_error &) {
      write_ids(r, a, b, o);  // no thread to be had: this share is written here
    }
  }
}
// true when host threads can write p (pageable, page-locked or managed memory);
// ids for a device destination are copied from the device's array instead
static bool host_writable(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return at.type != cudaMemoryTypeDevice;
}
// q + Psi in FP64 for particles [p0, p1) from the float displacements in the
// staging buffer (indexed by particle), the device's read-out sum
// (fused_asm.cuh k_fa_z) done on the host: the same doubles
static void write_positions(const mfx_job *j, size_t p0, size_t p1, double *dst) {  // dst holds particle p0
  const size_t N = size_t(j->N), n3 = N * N * N;
  const float *psi = j->psi_host;
  size_t p = p0;
  while (p < p1) {
    const size_t s = p / n3, c = p - s * n3, x = c / (N * N), y = (c / N) % N;
    const double *q = j->qhost.data() + s * 3 * N;
    const double qx = q[x], qy = q[N + y];
    const size_t zend = std::min(p1 - p, N - c % N);  // to the end of this row
    for (size_t t = 0, z = c % N; t < zend; ++t, ++z, ++p) {
      double *o = dst + 3 * (p - p0);
      const float *f = psi + 3 * p;
      o[0] = qx + double(f[0]);
      o[1] = qy + double(f[1]);
      o[2] = q[2 * N + z] + double(f[2]);
    }
  }
}

// The float displacements of particles [first, first + count) to the staging
// buffer on stream x, in chunks of 4M particles (48 MB) each followed by an
// event, and host threads that take the chunks in turn (thread t: chunks t,
// t + nt, ...), each waiting for its chunk and writing q + Psi into dst
// (joined by join_id_fill): every thread starts with the first chunks, and
// one chunk's work is left after the last copy.  At 768^3 the fetch is then
// bound by the host's memory (about 120 GB a step through DRAM: the staging
// written and read, positions, velocities and ids written).
static int start_pos_fill(mfx_job *j, size_t first, size_t count, void *dst, cudaStream_t x) {
  if (!j->psi_host) {
    CU(cudaHostAlloc(reinterpret_cast<void **>(&j->psi_host), j->npart * 3 * sizeof(float), cudaHostAllocDefault));
  }
  constexpr size_t kChunk = size_t(1) << 22;
  const size_t nch = (count + kChunk - 1) / kChunk;
  while (j->psi_ev.size() < nch) {
    cudaEvent_t e = nullptr;
    CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    j->psi_ev.push_back(e);
  }
  const float *src = static_cast<const float *>(j->pos);
  for (size_t c = 0; c < nch; ++c) {
    const size_t a = first + c * kChunk, b = std::min(first + count, a + kChunk);
    CU(cudaMemcpyAsync(j->psi_host + 3 * a, src + 3 * a, (b - a) * 3 * sizeof(float), cudaMemcpyDeviceToHost, x));
    CU(cudaEventRecord(j->psi_ev[c], x));
  }
  const size_t hw = std::max(2u, std::thread::hardware_concurrency());
  const size_t nt = std::max<size_t>(1, std::min<size_t>({size_t(16), hw, nch}));
  for (size_t t = 0; t < nt; ++t) {
    auto work = [j, t, nt, nch, first, count, dst] {
      for (size_t c = t; c < nch; c += nt) {
        const size_t a = first + c * kChunk, b = std::min(first + count, a + kChunk);
        if (cudaEventSynchronize(j->psi_ev[c]) != cudaSuccess) return;
        write_positions(j, a, b, static_cast<double *>(dst) + 3 * (a - first));
      }
    };
    try {
      j->id_fill.emplace_back(work);
    } catch (const std::system_error &) {
      work();
    }
  }
  return MFX_OK;
}

// ids [first, first + count) of the last run into device memory dst on stream st
// (ordered after the job's work; the fused read-out writes no ids itself)
static int fill_ids_device(mfx_job *j, size_t first, size_t count, void *dst, cudaStream_t st) {
  const IdRule r = id_rule(j);
  const size_t b = std::min<size_t>((count + 255) / 256, size_t(num_sm()) * 16);
  const unsigned g = unsigned(std::max<size_t>(b, 1));
  if (r.id64) k_fill_ids<uint64_t><<<g, 256, 0, st>>>(static_cast<uint64_t *>(dst), first, count, r.base, r.ns, r.n3);
  else k_fill_ids<uint32_t><<<g, 256, 0, st>>>(static_cast<uint32_t *>(dst), first, count, r.base, r.ns, r.n3);
  CU(cudaGetLastError());
  return MFX_OK;
}

static void join_id_fill(mfx_job *j) {
  for (auto &t : j->id_fill) t.join();
  j->id_fill.clear();
}

static void free_job(mfx_job *j) {
  if (!j) return;
  join_id_fill(j);
  if (j->stream) cudaStreamSynchronize(j->stream);
  if (j->gexec) cudaGraphExecDestroy(j->gexec);
  if (j->graph) cudaGraphDestroy(j->graph);
  if (j->eng) {
    release_plan(j->eng, j->m_r2c);
    release_plan(j->eng, j->m_c2r);
    release_plan(j->eng, j->n_c2r);
    release_plan(j->eng, j->n_r2c);
    for (auto &p : j->music_plans) release_plan(j->eng, p);
  } else {
    destroy_plan(j->m_r2c);
    destroy_plan(j->m_c2r);
    destroy_plan(j->n_c2r);
    destroy_plan(j->n_r2c);
    for (auto &p : j->music_plans) destroy_plan(p);
  }
  // stream-ordered free: never synchronises other jobs' streams
  if (j->arena) {
    cudaFreeAsync(j->arena, j->stream);
    cudaStreamSynchronize(j->stream);
  }
  for (auto &e : j->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : j->ev_pool)
    if (e) cudaEventDestroy(e);
  for (auto &x : j->xfer)
    if (x) {
      cudaStreamSynchronize(x);
      cudaStreamDestroy(x);
    }
  if (j->ring) {
    cudaFreeAsync(j->ring, j->stream);
    cudaStreamSynchronize(j->stream);
  }
  for (auto &e : j->ring_free)
    if (e) cudaEventDestroy(e);
  if (j->fetched) cudaEventDestroy(j->fetched);
  if (j->sp_mem) {
    cudaFreeAsync(j->sp_mem, j->stream);
    cudaStreamSynchronize(j->stream);
  }
  if (j->psi_host) cudaFreeHost(j->psi_host);
  if (j->ids_dev) {
    cudaFreeAsync(j->ids_dev, j->stream);
    cudaStreamSynchronize(j->stream);
  }
  for (auto &e : j->psi_ev)
    if (e) cudaEventDestroy(e);
  if (j->eng) release_plan(j->eng, j->rho_c2r);
  else destroy_plan(j->rho_c2r);
  if (j->stream) cudaStreamDestroy(j->stream);
  mfx_engine *eng = j->eng;
  if (eng) {
    std::lock_guard<std::mutex> lk(eng->mu);
    eng->in_use -= std::min(eng->in_use, j->arena_bytes + size_t(j->ring_sets) * j->ring_set_bytes + j->sp_bytes);
  }
  delete j;
  if (eng) engine_release(eng);
}

// phase tables exp(i s_a k_a dx) per sub-lattice and axis (grid_fft.hh:836-839)
// and the unperturbed lattice coordinates (m + s)/N * lunit, the reference's
// get_unit_r_shifted(...)[axis] * lunit (grid_fft.hh:240-250,
// particle_generator.hh:529-531); s includes the species' secondary-lattice
// shift (particle_generator.hh:388-395)
// The per-step angles at the Nyquist wavenumber of the job's sub-lattice
// shifts (NyqSteps): the secondary species' global shift first, then the
// steps between consecutive sub-lattices (particle_generator.hh:510-522).
static NyqSteps nyq_steps(const mfx_job *j) {
  NyqSteps t{};
  t.active = j->d.noise_generator != MFX_NOISE_NGENIC;
  const int N = j->N;
  const double kny = double(N / 2) * 2.0 * M_PI / j->d.boxlen, dx = j->d.boxlen / N;
  const bool second = j->lat_off[0] != 0.0 || j->lat_off[1] != 0.0 || j->lat_off[2] != 0.0;
  for (int s = 0; s < j->ns && s < 4; ++s) {
    int n = 0;
    if (second) {
      for (int ax = 0; ax < 3; ++ax) t.ang[s][n][ax] = j->lat_off[ax] * kny * dx;
      ++n;
    }
    for (int q = 1; q <= s && n < 4; ++q, ++n)
      for (int ax = 0; ax < 3; ++ax)
        t.ang[s][n][ax] = (kShifts[j->d.lattice][q][ax] - kShifts[j->d.lattice][q - 1][ax]) * kny * dx;
    t.nsteps[s] = n;
  }
  return t;
}

static int upload_shift_tables(mfx_job *j) {
  const int N = j->N;
  const mfx_job_desc *d = &j->d;
  std::vector<double2> ph(size_t(j->ns) * 3 * N);
  const double kfac = 2.0 * M_PI / d->boxlen, dx = d->boxlen / N;
  for (int s = 0; s < j->ns; ++s)
    for (int ax = 0; ax < 3; ++ax)
      for (int m = 0; m < N; ++m) {
        const double km = (double(m) - double(m > N / 2) * N) * kfac;
        const double th = (kShifts[d->lattice][s][ax] + j->lat_off[ax]) * km * dx;
        ph[(size_t(s) * 3 + ax) * N + m] = make_double2(std::cos(th), std::sin(th));
      }
  std::vector<double> qt(size_t(j->ns) * 3 * N);
  for (int s = 0; s < j->ns; ++s)
    for (int ax = 0; ax < 3; ++ax)
      for (int m = 0; m < N; ++m)
        qt[(size_t(s) * 3 + ax) * N + m] =
            (double(m) + (kShifts[d->lattice][s][ax] + j->lat_off[ax])) / double(N) * d->lunit;
  std::vector<float2> ph32(ph.size());
  for (size_t q = 0; q < ph.size(); ++q) ph32[q] = make_float2(float(ph[q].x), float(ph[q].y));
  j->qhost = qt;
  if (cudaMemcpyAsync(j->phase, ph.data(), ph.size() * sizeof(double2), cudaMemcpyHostToDevice, j->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(j->phase32, ph32.data(), ph32.size() * sizeof(float2), cudaMemcpyHostToDevice, j->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(j->qtab, qt.data(), qt.size() * sizeof(double), cudaMemcpyHostToDevice, j->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(j->stream) != cudaSuccess)
    return set_error(MFX_ECUDA, "phase table upload failed");
  return MFX_OK;
}

// priority: the CUDA stream priority of the job's stream (0: the default)
static int create_job(mfx_engine *eng, const mfx_job_desc *d, mfx_job **out, int priority = 0) {
  TRY(check_desc(d));
  CU(cudaSetDevice(eng->device));
  auto *j = new mfx_job();
  j->eng = eng;
  engine_retain(eng);
  j->d = *d;
  j->base_id_offset = d->id_offset;
  j->N = d->ngrid;
  j->M = 3 * j->N / 2;
  j->nh = j->N / 2;
  j->nk = j->nh + 1;
  j->mk = j->M / 2 + 1;
  j->ns = lattice_nshift(d->lattice);
  j->fp64 = d->precision == MFX_FP64;
  j->rsize = j->fp64 ? 8 : 4;
  // per-field scaling of the FP32 form: carry phi(1) as the growth-scaled
  // potential D+ phi so that Hessians are O(delta) and products stay far from
  // the FP32 exponent limits; phi2 / phi3 inherit the square / cube.
  if (!j->fp64) {
    const double s = std::fabs(d->g1) > 0 ? std::fabs(d->g1) : 1.0;
    j->scale1 = s;
    j->scale2 = s * s;
    j->scale3 = s * s * s;
  }
  int rc = MFX_OK;
  auto fail = [&](int code) {
    free_job(j);
    return code;
  };
  if (cudaStreamCreateWithPriority(&j->stream, cudaStreamNonBlocking, priority) != cudaSuccess)
    return fail(set_error(MFX_ECUDA, "cudaStreamCreate failed"));
  for (auto &e : j->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(set_error(MFX_ECUDA, "cudaEventCreate failed"));
  j->timed = true;
  // plans
  size_t work = 0;
  j->fused = fused_supported(d);
  if (j->fused) {
    ff_default_tiles(j);
    tune_fused(j);
  }
  if (d->lpt_order >= 2 && !j->fused) {
    if ((rc = acquire_plan(eng, j->m_r2c, j->M, j->fp64, true)) != MFX_OK) return fail(rc);
    if ((rc = acquire_plan(eng, j->m_c2r, j->M, j->fp64, false)) != MFX_OK) return fail(rc);
    work = std::max(work, std::max(j->m_r2c.work, j->m_c2r.work));
  }
  if (d->want_particles && !j->fused) {
    // the six assembled components of a sub-lattice lie one padded field apart:
    // one batched c2r per sub-lattice
    const long long nfb = (long long)align_up(n_field_bytes(j->N, j->rsize));
    if ((rc = acquire_plan(eng, j->n_c2r, j->N, j->fp64, false, 6, nfb)) != MFX_OK) return fail(rc);
    work = std::max(work, j->n_c2r.work);
  }
  if (d->noise_generator == MFX_NOISE_FIELD) {
    if ((rc = acquire_plan(eng, j->n_r2c, j->N, j->fp64, true)) != MFX_OK) return fail(rc);
    work = std::max(work, j->n_r2c.work);
  }
  if (d->noise_generator == MFX_NOISE_MUSIC1) {
    if ((rc = acquire_plan(eng, j->n_r2c, j->N, j->fp64, true)) != MFX_OK) return fail(rc);
    work = std::max(work, j->n_r2c.work);
    const MusicLevels ml = music_levels(d);
    j->music_l0 = ml.l0;
    j->music_lmin = ml.lmin;
    j->music_lfile = ml.lfile;
    // the coarser levels' forward transforms, or the one of the finer seeded level
    j->music_plans.resize(ml.l0 < ml.lmin ? size_t(ml.lmin - ml.l0) : (ml.l0 > ml.lmin ? 1 : 0));
    for (size_t q = 0; q < j->music_plans.size(); ++q) {
      Plan &p = j->music_plans[q];
      const int l = ml.l0 < ml.lmin ? ml.l0 + int(q) : ml.l0;
      if ((rc = acquire_plan(eng, p, 1 << l, j->fp64, true)) != MFX_OK) return fail(rc);
      work = std::max(work, p.work);
    }
  }
  Layout L = plan_layout(d, work);
  {
    std::lock_guard<std::mutex> lk(eng->mu);
    // the fused assembly emits all sub-lattices from one assembly of each mode
    // when their components are held together: worth the extra memory while
    // the engine budget has it
    if (j->fused && d->want_particles && L.group < j->ns && ff::fa_all(j->M)) {
      const Layout La = plan_layout(d, work, true);
      if (eng->in_use + La.total <= eng->budget) L = La;
    }
    if (eng->in_use + L.total > eng->budget)
      return fail(set_error(MFX_EADMIT, "job needs %zu bytes, engine budget has %zu of %zu free", L.total,
                            eng->budget - std::min(eng->budget, eng->in_use), eng->budget));
    eng->in_use += L.total;
  }
  j->arena_bytes = L.total;
  // stream-ordered allocation from the device's default pool (kept cached,
  // see mfx_engine_create): admitting and retiring jobs never synchronises
  // the device
  cudaError_t e = cudaMallocAsync(&j->arena, L.total, j->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->stream);
  if (e == cudaErrorMemoryAllocation) {
    // the cached pool may hold freed arenas of other shapes: hand its unused
    // memory back to the device and try once more
    cudaGetLastError();
    j->arena = nullptr;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
      cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocAsync(&j->arena, L.total, j->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(j->stream);
  }
  if (e != cudaSuccess) {
    j->arena = nullptr;
    cudaGetLastError();
    return fail(set_error(MFX_ENOMEM, "allocation of %zu bytes for the job arena failed: %s", L.total,
                          cudaGetErrorString(e)));
  }
  char *p = j->arena;
  j->seeds = (uint32_t *)p;
  p += L.seeds;
  j->amp = (double *)p;
  p += L.amp;
  j->plt = d->plt ? (double *)p : nullptr;
  j->plt4 = d->plt ? (float4 *)(p + align_up(size_t(MFX_PLT_TABLE_DOUBLES) * 8)) : nullptr;
  p += L.plt;
  j->phase = (double2 *)p;
  j->qtab = (double *)(p + align_up(size_t(j->ns) * 3 * j->N * sizeof(double2)));
  j->phase32 = (float2 *)(p + align_up(size_t(j->ns) * 3 * j->N * sizeof(double2)) +
                          align_up(size_t(j->ns) * 3 * j->N * sizeof(double)));
  p += L.phase;
  j->ff_tw = L.ff_tw ? reinterpret_cast<float2 *>(p) : nullptr;
  j->ff_twn = L.ff_tw ? reinterpret_cast<float2 *>(p + align_up(size_t(j->M) * 8)) : nullptr;
  p += L.ff_tw;
  j->dstatus = L.status ? reinterpret_cast<int *>(p) : nullptr;
  p += L.status;
  if (j->dstatus && (cudaMemsetAsync(j->dstatus, 0, sizeof(int), j->stream) != cudaSuccess))
    return fail(set_error(MFX_ECUDA, "status word reset failed"));
  const int nfield = d->lpt_order == 1 ? 1 : (d->lpt_order == 2 ? 2 : 6);
  j->n_field_bytes = L.n_field;
  j->m_field_bytes = L.m_field;
  for (int q = 0; q < nfield; ++q) {
    j->nf[q] = p;
    p += align_up(L.n_field);
  }
  j->region = p;
  j->region_bytes = L.region;
  p += L.region;
  j->work = L.work_est ? p : nullptr;
  j->work_bytes = L.work_est;
  p += L.work_est;
  if (L.music) {
    j->music_buf[0] = p;
    // the second coarse buffer of a refinement; of a restriction, the level
    // below the seeded one
    j->music_buf[1] = d->noise_generator != MFX_NOISE_MUSIC1 ? nullptr
                      : j->music_l0 < j->music_lmin
                          ? p + L.music / 2
                          : (j->music_l0 - j->music_lmin >= 2 ? p + align_up(n_field_bytes(1 << j->music_l0, j->rsize))
                                                             : nullptr);
  }
  for (int q = 0; q < L.nslots; ++q) j->mslot[q] = j->region + size_t(q) * align_up(L.m_field);
  if (j->fused) {
    char *f = j->region;
    for (int q = 0; q < 3; ++q, f += L.ff_b) j->ffB[q] = f;
    for (int q = 0; q < L.ff_nc; ++q, f += L.ff_d) j->ffC[q] = f;
    for (const int L : {j->M, j->N}) {
      std::vector<float2> tw(L);
      for (int t = 0; t < L; ++t) {
        const double a = 2.0 * M_PI * double(t) / double(L);
        tw[t] = make_float2(float(std::cos(a)), float(-std::sin(a)));
      }
      if (cudaMemcpyAsync(L == j->M ? j->ff_tw : j->ff_twn, tw.data(), tw.size() * sizeof(float2),
                          cudaMemcpyHostToDevice, j->stream) != cudaSuccess ||
          cudaStreamSynchronize(j->stream) != cudaSuccess)
        return fail(set_error(MFX_ECUDA, "twiddle upload failed"));
    }
  }
  j->group = L.group;
  if (d->want_particles) {
    char *a = j->region;
    const size_t np = size_t(j->ns) * j->N * j->N * j->N;
    j->npart = np;
    j->pos = a;
    a += align_up(np * 3 * (d->pos64 ? 8 : 4));
    j->vel = a;
    a += align_up(np * 3 * (d->vel64 ? 8 : 4));
    j->ids = j->fused ? nullptr : a;  // the fused read-out writes no device ids
    a += align_up(np * (d->id64 ? 8 : 4));
    for (int q = 0; q < 6 * j->group; ++q) {
      j->asmbuf[q] = a;
      a += align_up(L.n_field);
    }
  }
  if (j->work) {
    if (j->m_r2c.valid && cufftSetWorkArea(j->m_r2c.h, j->work) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetWorkArea failed"));
    if (j->m_c2r.valid && cufftSetWorkArea(j->m_c2r.h, j->work) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetWorkArea failed"));
    if (j->n_c2r.valid && cufftSetWorkArea(j->n_c2r.h, j->work) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetWorkArea failed"));
    if (j->n_r2c.valid && cufftSetWorkArea(j->n_r2c.h, j->work) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetWorkArea failed"));
    for (auto &p : j->music_plans)
      if (p.valid && cufftSetWorkArea(p.h, j->work) != CUFFT_SUCCESS)
        return fail(set_error(MFX_ECUDA, "cufftSetWorkArea failed"));
  }
  for (Plan *pl : {&j->m_r2c, &j->m_c2r, &j->n_c2r, &j->n_r2c})
    if (pl->valid && cufftSetStream(pl->h, j->stream) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetStream failed"));
  for (auto &p : j->music_plans)
    if (p.valid && cufftSetStream(p.h, j->stream) != CUFFT_SUCCESS)
      return fail(set_error(MFX_ECUDA, "cufftSetStream failed"));
  if ((rc = upload_shift_tables(j)) != MFX_OK) return fail(rc);
  if ((rc = upload_tables(j, d)) != MFX_OK) return fail(rc);
  if (cudaStreamSynchronize(j->stream) != cudaSuccess) return fail(set_error(MFX_ECUDA, "table upload failed"));
  *out = j;
  return MFX_OK;
}

// Records the job's whole pipeline into a CUDA graph (stream capture on the
// job stream).  Per-stage events and per-launch profiling stay out of graphs.
static int capture_pipeline(mfx_job *j, cudaGraph_t *out) {
  const bool prof = j->prof, timed = j->timed;
  j->prof = false;
  j->timed = false;
  cudaError_t e = cudaStreamBeginCapture(j->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    j->prof = prof;
    j->timed = timed;
    return set_error(MFX_ECUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
  }
  const int rc = j->fp64 ? run_pipeline<double>(j) : run_pipeline<float>(j);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(j->stream, &g);
  j->prof = prof;
  j->timed = timed;
  j->has_run = false;
  if (rc != MFX_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
  *out = g;
  return MFX_OK;
}

// An ensemble: independent jobs whose captured pipelines are the parallel
// branches (child-graph nodes) of one executable graph.
struct mfx_batch {
  mfx_engine *eng = nullptr;
  std::vector<mfx_job *> jobs;
  std::vector<cudaGraph_t> children;
  cudaGraph_t parent = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ran = false;
};

static void free_batch(mfx_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->parent) cudaGraphDestroy(b->parent);
  for (auto g : b->children)
    if (g) cudaGraphDestroy(g);
  for (auto j : b->jobs) free_job(j);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define GUARD_BEGIN try {
#define GUARD_END                                                       \
  }                                                                     \
  catch (const std::bad_alloc &) {                                      \
    return set_error(MFX_ENOMEM, "host allocation failed");             \
  }                                                                     \
  catch (const std::exception &ex) {                                    \
    return set_error(MFX_EINVAL, "%s", ex.what());                      \
  }                                                                     \
  catch (...) {                                                         \
    return set_error(MFX_EINVAL, "unknown C++ exception");              \
  }

extern "C" {

size_t mfx_last_error(char *buf, size_t len) {
  const std::string &s = g_last_error;
  if (buf && len) {
    size_t n = std::min(len - 1, s.size());
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return s.size();
}

const char *mfx_version(void) { return "mfx 0.1 (sm_103a)"; }

int mfx_engine_create(const mfx_engine_opts *opts, mfx_engine **out) {
  GUARD_BEGIN
  if (!out) return set_error(MFX_EINVAL, "null output pointer");
  int dev = opts ? opts->device : 0;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    return set_error(MFX_ECUDA, "no CUDA device available");
  if (dev < 0 || dev >= count) return set_error(MFX_EINVAL, "device %d out of range", dev);
  CU(cudaSetDevice(dev));
  TRY(noalloc_prepare(dev));
  size_t free_b = 0, total_b = 0;
  CU(cudaMemGetInfo(&free_b, &total_b));
  auto *e = new mfx_engine();
  e->device = dev;
  {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;  // keep freed job arenas cached in the process
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  e->budget = (opts && opts->hbm_budget_bytes) ? opts->hbm_budget_bytes : size_t(double(free_b) * 0.9);
  *out = e;
  return MFX_OK;
  GUARD_END
}

int mfx_engine_destroy(mfx_engine *eng) {
  if (!eng) return MFX_OK;
  {
    std::lock_guard<std::mutex> lk(eng->mu);
    eng->closing = true;
    if (eng->holders > 0) return MFX_OK;  // the last job or server releases it
  }
  engine_free(eng);
  return MFX_OK;
}

int mfx_job_footprint(mfx_engine *eng, const mfx_job_desc *desc, size_t *bytes) {
  GUARD_BEGIN
  TRY(check_desc(desc));
  if (!bytes) return set_error(MFX_EINVAL, "null output");
  // FFT work areas are bounded by the largest transform's data size: the
  // padded cuFFT transforms (plain form), the batch of six N-grid c2r
  const int M = 3 * desc->ngrid / 2;
  const size_t rs = desc->precision == MFX_FP64 ? 8 : 4;
  const bool fused = fused_supported(desc);
  size_t work = (desc->want_particles && !fused) ? 6 * n_field_bytes(desc->ngrid, rs) : 0;
  if (desc->lpt_order >= 2 && !fused) work = std::max(work, size_t(M) * M * (M / 2 + 1) * 2 * rs);
  if (desc->noise_generator == MFX_NOISE_MUSIC1) work = std::max(work, n_field_bytes(desc->ngrid, rs));
  *bytes = plan_layout(desc, work).total;
  return MFX_OK;
  GUARD_END
}

int mfx_job_create(mfx_engine *eng, const mfx_job_desc *desc, mfx_job **out) {
  GUARD_BEGIN
  if (!eng || !out) return set_error(MFX_EINVAL, "null argument");
  return create_job(eng, desc, out);
  GUARD_END
}

int mfx_job_upload(mfx_job *job, const mfx_job_desc *desc) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  TRY(check_desc(desc));
  if (desc->ngrid != job->d.ngrid || desc->amp_table_len != job->d.amp_table_len || desc->plt != job->d.plt ||
      desc->noise_generator != job->d.noise_generator || desc->music_cubesize != job->d.music_cubesize)
    return set_error(MFX_EINVAL, "upload descriptor does not match the job's sizes");
  if (desc->noise_generator == MFX_NOISE_MUSIC1 &&
      (music_levels(desc).l0 != job->music_l0 || music_levels(desc).lfile != job->music_lfile))
    return set_error(MFX_EINVAL, "upload descriptor changes the coarsest seeded MUSIC1 level or its noise file");
  job->d.seed_table = desc->seed_table;
  job->d.noise_field = desc->noise_field;
  job->d.music_seed = desc->music_seed;
  std::memcpy(job->d.music_seeds, desc->music_seeds, sizeof(desc->music_seeds));
  job->d.amp_table = desc->amp_table;
  job->d.plt_table = desc->plt_table;
  return upload_tables(job, desc);
  GUARD_END
}

int mfx_job_run(mfx_job *job) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  CU(cudaSetDevice(job->eng->device));
  if (job->gexec) {
    CU(cudaGraphLaunch(job->gexec, job->stream));
    job->has_run = true;
    job->noise_only = false;
    return MFX_OK;
  }
  return job->fp64 ? run_pipeline<double>(job) : run_pipeline<float>(job);
  GUARD_END
}

int mfx_job_assemble(mfx_job *job, int orders_mask) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (!job->has_run || job->noise_only) return set_error(MFX_ESTATE, "job has no potentials (run it first)");
  if (orders_mask < 1 || orders_mask > 7) return set_error(MFX_EINVAL, "orders_mask %d outside 1..7", orders_mask);
  CU(cudaSetDevice(job->eng->device));
  job->ev_next = 0;
  job->prof_recs.clear();
  if (job->fetched) CU(cudaStreamWaitEvent(job->stream, job->fetched, 0));  // downloads of these particles
  TRY(job->fp64 ? assemble_stage<double>(job, orders_mask) : assemble_stage<float>(job, orders_mask));
  CU(cudaStreamSynchronize(job->stream));
  return MFX_OK;
  GUARD_END
}

// drops the species' allocation and plan (the job's stream is idle)
static void release_species(mfx_job *job) {
  if (job->sp_mem) {
    cudaFreeAsync(job->sp_mem, job->stream);
    cudaStreamSynchronize(job->stream);
    std::lock_guard<std::mutex> lk(job->eng->mu);
    job->eng->in_use -= std::min(job->eng->in_use, job->sp_bytes);
  }
  release_plan(job->eng, job->rho_c2r);
  job->sp_mem = nullptr;
  job->sp_bytes = job->sp_len = 0;
  job->qvbc = job->rho_ratio = nullptr;
  job->qvbc32 = nullptr;
  job->rho = job->mass = job->rho_work = nullptr;
  job->want_masses = job->has_masses = false;
  job->c_species = job->mass_factor = 0.0;
  for (double &o : job->lat_off) o = 0.0;
  job->d.id_offset = job->base_id_offset;
}

int mfx_job_set_species(mfx_job *job, const mfx_species_desc *sp) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (job->gexec) return set_error(MFX_ESTATE, "job already captured into a graph");
  const size_t len = 3 * size_t(job->nh) * job->nh + 1;
  if (sp && (sp->amp_dbc || sp->amp_tbc) && sp->amp_len < len)
    return set_error(MFX_EINVAL, "species tables need %zu entries (got %zu)", len, sp->amp_len);
  if (sp && !(std::isfinite(sp->c_species) && std::isfinite(sp->mass_factor)))
    return set_error(MFX_EINVAL, "species factors must be finite");
  CU(cudaSetDevice(job->eng->device));
  for (auto &x : job->xfer)
    if (x) CU(cudaStreamSynchronize(x));
  CU(cudaStreamSynchronize(job->stream));
  release_species(job);
  if (sp) {
    static const double kSecond[3][3] = {{0.5, 0.5, 0.5}, {0.5, 0.5, 0.0}, {0.5, 0.5, 0.5}};
    for (int ax = 0; ax < 3; ++ax) job->lat_off[ax] = sp->secondary_lattice ? kSecond[job->d.lattice][ax] : 0.0;
    job->d.id_offset = sp->id_offset;
    job->c_species = sp->c_species;
    job->mass_factor = sp->mass_factor;
    job->want_masses = sp->want_masses != 0;
    const int N = job->N;
    const bool vbc = sp->amp_tbc != nullptr, dbc = job->want_masses && sp->amp_dbc != nullptr;
    const size_t rs = job->fp64 ? 8 : 4;
    size_t off_q = 0, off_q32 = 0, off_r = 0, off_rho = 0, off_m = 0, off_w = 0, tot = 0;
    auto take = [&](size_t &off, size_t bytes) {
      off = tot;
      tot += align_up(bytes);
    };
    if (vbc) {
      take(off_q, len * 8);
      take(off_q32, len * 4);
    }
    if (dbc) take(off_r, len * 8);
    if (job->want_masses) {
      TRY(acquire_plan(job->eng, job->rho_c2r, N, job->fp64, false));
      take(off_rho, size_t(N) * N * (N + 2) * rs);
      take(off_m, job->npart * (job->d.pos64 ? 8 : 4));
      take(off_w, std::max<size_t>(job->rho_c2r.work, 256));
    }
    if (tot) {
      {
        std::lock_guard<std::mutex> lk(job->eng->mu);
        if (job->eng->in_use + tot > job->eng->budget) {
          release_plan(job->eng, job->rho_c2r);
          return set_error(MFX_EADMIT, "species buffers need %zu bytes beyond the engine budget", tot);
        }
        job->eng->in_use += tot;
      }
      cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&job->sp_mem), tot, job->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(job->stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        job->sp_mem = nullptr;
        std::lock_guard<std::mutex> lk(job->eng->mu);
        job->eng->in_use -= std::min(job->eng->in_use, tot);
        release_plan(job->eng, job->rho_c2r);
        return set_error(MFX_ENOMEM, "species buffers of %zu bytes: %s", tot, cudaGetErrorString(e));
      }
      job->sp_bytes = tot;
    }
    job->sp_len = len;
    // host tables: with w = -phi1 / A(n) (phi1 = -A(n) w, A the amplitude table)
    const double kf = 2.0 * M_PI / job->d.boxlen, g1 = job->d.g1;
    const std::vector<double> &A = job->amp_host;
    if (vbc) {
      // velocity weight of phi1 times 1 + C A_theta_bc / (A k^2 g1)
      std::vector<double> q(len, 0.0);
      std::vector<float> q32(len, 0.f);
      for (size_t n = 1; n < len; ++n)
        if (n < A.size() && A[n] != 0.0 && g1 != 0.0)
          q[n] = sp->c_species * sp->amp_tbc[n] / (A[n] * kf * kf * double(n) * g1);
      for (size_t n = 0; n < len; ++n) q32[n] = float(q[n]);
      job->qvbc = reinterpret_cast<double *>(job->sp_mem + off_q);
      job->qvbc32 = reinterpret_cast<float *>(job->sp_mem + off_q32);
      CU(cudaMemcpyAsync(job->qvbc, q.data(), len * 8, cudaMemcpyHostToDevice, job->stream));
      CU(cudaMemcpyAsync(job->qvbc32, q32.data(), len * 4, cudaMemcpyHostToDevice, job->stream));
    }
    if (dbc) {
      // delta_bc(k) = w A_delta_bc = -(phi1 field / scale1) A_delta_bc / A
      std::vector<double> r(len, 0.0);
      for (size_t n = 1; n < len; ++n)
        if (n < A.size() && A[n] != 0.0) r[n] = -sp->amp_dbc[n] / (A[n] * job->scale1);
      job->rho_ratio = reinterpret_cast<double *>(job->sp_mem + off_r);
      CU(cudaMemcpyAsync(job->rho_ratio, r.data(), len * 8, cudaMemcpyHostToDevice, job->stream));
    }
    if (job->want_masses) {
      job->rho = job->sp_mem + off_rho;
      job->mass = job->sp_mem + off_m;
      job->rho_work = job->sp_mem + off_w;
      CF(cufftSetWorkArea(job->rho_c2r.h, job->rho_work));
      CF(cufftSetStream(job->rho_c2r.h, job->stream));
    }
    CU(cudaStreamSynchronize(job->stream));
  }
  TRY(upload_shift_tables(job));
  return MFX_OK;
  GUARD_END
}

int mfx_job_fetch_masses(mfx_job *job, size_t first, size_t count, void *out) {
  GUARD_BEGIN
  if (!job || !out) return set_error(MFX_EINVAL, "null argument");
  if (!job->has_masses || !job->mass) return set_error(MFX_ESTATE, "no masses: set a species with masses and run");
  if (first > job->npart || count > job->npart - first)
    return set_error(MFX_EINVAL, "range [%zu, %zu) outside the %zu particles", first, first + count, job->npart);
  CU(cudaSetDevice(job->eng->device));
  CU(cudaStreamSynchronize(job->stream));
  const size_t es = job->d.pos64 ? 8 : 4;
  CU(cudaMemcpy(out, static_cast<char *>(job->mass) + es * first, es * count, cudaMemcpyDefault));
  return MFX_OK;
  GUARD_END
}

int mfx_job_set_tiles(mfx_job *job, int pencils_xy, int rows_z) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->fused) return set_error(MFX_ESTATE, "job does not use the fused transforms");
  if (!ff::ff_valid(job->M, ff::FF_XFWD, pencils_xy))
    return set_error(MFX_EINVAL, "x/y tile of %d pencils not admissible for M = %d", pencils_xy, job->M);
  if (!ff::ff_valid(job->M, ff::FF_ZSRC3, rows_z) || !ff::ff_valid(job->M, ff::FF_ZSRC2, rows_z))
    return set_error(MFX_EINVAL, "z tile of %d rows not admissible for M = %d", rows_z, job->M);
  if (job->gexec) return set_error(MFX_ESTATE, "job already captured into a graph");
  job->ff_pxy = pencils_xy;
  for (int k = 0; k < 6; ++k) job->ff_pk[k] = 0;
  job->ff_pz = rows_z;
  job->ff_pz2 = rows_z;
  return MFX_OK;
  GUARD_END
}

int mfx_job_autotune(mfx_job *job, int *pencils_xy, int *rows_z) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  CU(cudaSetDevice(job->eng->device));
  if (job->fused) TRY(autotune_fused(job));
  if (pencils_xy) *pencils_xy = job->fused ? job->ff_pxy : 0;
  if (rows_z) *rows_z = job->fused ? (job->d.lpt_order >= 3 ? job->ff_pz : job->ff_pz2) : 0;
  return MFX_OK;
  GUARD_END
}

int mfx_job_capture(mfx_job *job) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  CU(cudaSetDevice(job->eng->device));
  if (job->gexec) return MFX_OK;
  if (job->ring) return set_error(MFX_ESTATE, "a job with an output ring cannot be captured");
  cudaGraph_t g = nullptr;
  TRY(capture_pipeline(job, &g));
  cudaError_t e = cudaGraphInstantiate(&job->gexec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    job->gexec = nullptr;
    return set_error(MFX_ECUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  }
  job->graph = g;
  return MFX_OK;
  GUARD_END
}

int mfx_job_run_noise(mfx_job *job, int raw) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  CU(cudaSetDevice(job->eng->device));
  job->own_launches = 0;
  int rc = job->fp64 ? make_noise<double>(job, raw ? 0 : 1, job->nf[0])
                     : make_noise<float>(job, raw ? 0 : 1, job->nf[0]);
  if (rc == MFX_OK) {
    job->noise_only = true;
    job->has_run = true;
  }
  return rc;
  GUARD_END
}

// the device status word of a finished job: a kernel whose bounded wait for
// its own asynchronous copies ran out set it and left its work undone
static int check_status(mfx_job *job) {
  if (!job->dstatus) return MFX_OK;
  int st = 0;
  CU(cudaMemcpy(&st, job->dstatus, sizeof(int), cudaMemcpyDeviceToHost));
  if (st) return set_error(MFX_ETIMEOUT, "a fused-transform kernel timed out waiting for its staged inputs");
  return MFX_OK;
}

int mfx_job_wait(mfx_job *job, int timeout_ms) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (timeout_ms < 0) {
    CU(cudaStreamSynchronize(job->stream));
    return check_status(job);
  }
  // bounded host-side poll
  for (int waited = 0;; ++waited) {
    cudaError_t e = cudaStreamQuery(job->stream);
    if (e == cudaSuccess) return check_status(job);
    if (e != cudaErrorNotReady) return set_error(MFX_ECUDA, "job stream: %s", cudaGetErrorString(e));
    if (waited >= timeout_ms) return set_error(MFX_ETIMEOUT, "job not finished after %d ms", timeout_ms);
    struct timespec ts = {0, 1000000};
    nanosleep(&ts, nullptr);
  }
  GUARD_END
}

// Downloads after the job's work: each copy is cut into pieces of at least
// 32 MB spread over four copy streams (one stream's copies do not fill the
// host link), all waiting on the job stream, and joined before returning.
struct Xfer {
  void *dst;
  const void *src;
  size_t bytes;
};
static int download(mfx_job *j, const Xfer *xs, int n) {
  for (auto &x : j->xfer)
    if (!x) CU(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  cudaEvent_t ready = nullptr;
  CU(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ready, j->stream);
  for (auto &x : j->xfer)
    if (e == cudaSuccess) e = cudaStreamWaitEvent(x, ready, 0);
  size_t total = 0;
  for (int q = 0; q < n; ++q) total += xs[q].dst ? xs[q].bytes : 0;
  const size_t piece = std::max<size_t>(size_t(32) << 20, (total + 7) / 8);
  int s = 0;
  for (int q = 0; q < n && e == cudaSuccess; ++q) {
    if (!xs[q].dst) continue;
    for (size_t off = 0; off < xs[q].bytes && e == cudaSuccess; off += piece) {
      const size_t len = std::min(piece, xs[q].bytes - off);
      e = cudaMemcpyAsync(static_cast<char *>(xs[q].dst) + off, static_cast<const char *>(xs[q].src) + off, len,
                          cudaMemcpyDefault, j->xfer[s]);
      s = (s + 1) % 4;
    }
  }
  for (auto &x : j->xfer) {
    const cudaError_t f = cudaStreamSynchronize(x);
    if (e == cudaSuccess) e = f;
  }
  cudaEventDestroy(ready);
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "particle download: %s", cudaGetErrorString(e));
  return MFX_OK;
}

int mfx_job_fetch_particles(mfx_job *job, void *pos, void *vel, void *ids) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (!job->has_run || job->noise_only) return set_error(MFX_ESTATE, "job has not produced particles");
  return mfx_job_fetch_particles_range(job, 0, job->npart, pos, vel, ids);
  GUARD_END
}

int mfx_job_fetch_particles_range(mfx_job *job, size_t first, size_t count, void *pos, void *vel, void *ids) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (!job->has_run || job->noise_only) return set_error(MFX_ESTATE, "job has not produced particles");
  if (first > job->npart || count > job->npart - first)
    return set_error(MFX_EINVAL, "range [%zu, %zu) outside the %zu particles", first, first + count, job->npart);
  CU(cudaSetDevice(job->eng->device));
  const size_t ps = job->d.pos64 ? 8 : 4, vs = job->d.vel64 ? 8 : 4, is = job->d.id64 ? 8 : 4;
  const bool host_ids = ids && host_writable(ids);
  if (job->host_q && ((pos && !host_writable(pos)) || (ids && !host_ids)))
    return set_error(MFX_ESTATE, "a job with host-side positions fetches positions and ids into host memory only");
  const bool kernel_ids = ids && !host_ids && !job->ids;  // no device array: the closed form on the device
  const Xfer xs[3] = {{job->host_q ? nullptr : pos, static_cast<char *>(job->pos) + 3 * ps * first, 3 * ps * count},
                      {vel, static_cast<char *>(job->vel) + 3 * vs * first, 3 * vs * count},
                      {(host_ids || kernel_ids) ? nullptr : ids, static_cast<char *>(job->ids) + is * first, is * count}};
  join_id_fill(job);
  if (host_ids) start_id_fill(job, first, count, ids);
  if (kernel_ids) TRY(fill_ids_device(job, first, count, ids, job->stream));
  if (job->host_q && pos) {
    if (!job->xfer[0]) CU(cudaStreamCreateWithFlags(&job->xfer[0], cudaStreamNonBlocking));
    if (!job->fetched) CU(cudaEventCreateWithFlags(&job->fetched, cudaEventDisableTiming));
    CU(cudaEventRecord(job->fetched, job->stream));
    CU(cudaStreamWaitEvent(job->xfer[0], job->fetched, 0));
    const int prc = start_pos_fill(job, first, count, pos, job->xfer[0]);
    if (prc != MFX_OK) {
      join_id_fill(job);
      return prc;
    }
  }
  const int rc = download(job, xs, 3);
  join_id_fill(job);
  return rc;
  GUARD_END
}

int mfx_job_set_host_positions(mfx_job *job, int on) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (on && !(job->fused && !job->fp64 && job->d.pos64))
    return set_error(MFX_ESTATE, "host-side positions need the FP32 form's fused route and 64-bit positions");
  if (job->ring) return set_error(MFX_ESTATE, "set host-side positions before the output ring");
  if (job->gexec) return set_error(MFX_ESTATE, "job already captured into a graph");
  if (!on == !job->host_q) return MFX_OK;
  CU(cudaSetDevice(job->eng->device));
  join_id_fill(job);
  for (auto &x : job->xfer)
    if (x) CU(cudaStreamSynchronize(x));
  CU(cudaStreamSynchronize(job->stream));
  job->host_q = on != 0;
  // the particles of the last run, in the new form
  if (job->has_run && !job->noise_only) {
    TRY(assemble_stage<float>(job, 7));
    CU(cudaStreamSynchronize(job->stream));
  }
  return MFX_OK;
  GUARD_END
}

int mfx_job_set_output_ring(mfx_job *job, int on) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (job->gexec) return set_error(MFX_ESTATE, "job already captured into a graph");
  CU(cudaSetDevice(job->eng->device));
  if (on < 0 || on > 2) return set_error(MFX_EINVAL, "output sets must be 0, 1 or 2 (got %d)", on);
  if (on == job->ring_sets) return MFX_OK;
  for (auto &x : job->xfer)
    if (x) CU(cudaStreamSynchronize(x));
  CU(cudaStreamSynchronize(job->stream));
  mfx_engine *eng = job->eng;
  if (job->ring) {
    CU(cudaFreeAsync(job->ring, job->stream));
    CU(cudaStreamSynchronize(job->stream));
    job->ring = nullptr;
    {
      std::lock_guard<std::mutex> lk(eng->mu);
      eng->in_use -= std::min(eng->in_use, size_t(job->ring_sets) * job->ring_set_bytes);
    }
    job->ring_set_bytes = 0;
    job->ring_sets = 0;
    // back to the arena's particle arrays (the last run's particles are gone)
    job->has_run = false;
    char *a = job->region;
    job->pos = a;
    a += align_up(job->npart * 3 * (job->d.pos64 ? 8 : 4));
    job->vel = a;
    a += align_up(job->npart * 3 * (job->d.vel64 ? 8 : 4));
    job->ids = job->fused ? nullptr : a;
  }
  if (!on) return MFX_OK;
  const size_t np = job->npart;
  // host-side positions: float displacements; the fused read-out: no device ids
  const bool no_ids = job->host_q || job->fused;
  const size_t set = align_up(np * 3 * (job->host_q ? 4 : (job->d.pos64 ? 8 : 4))) +
                     align_up(np * 3 * (job->d.vel64 ? 8 : 4)) + (no_ids ? 0 : align_up(np * (job->d.id64 ? 8 : 4)));
  const size_t total = size_t(on) * set;
  {
    std::lock_guard<std::mutex> lk(eng->mu);
    if (eng->in_use + total > eng->budget)
      return set_error(MFX_EADMIT, "output ring needs %zu bytes, engine budget has %zu free", total,
                       eng->budget - std::min(eng->budget, eng->in_use));
    eng->in_use += total;
  }
  char *r = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&r), total, job->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(job->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(eng->mu);
    eng->in_use -= std::min(eng->in_use, total);
    return set_error(MFX_ENOMEM, "output ring of %zu bytes: %s", total, cudaGetErrorString(e));
  }
  for (auto &ev : job->ring_free)
    if (!ev) CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  job->ring = r;
  job->ring_set_bytes = set;
  job->ring_sets = on;
  job->ring_next = 0;
  job->has_run = false;
  ring_point(job, 0);
  return MFX_OK;
  GUARD_END
}

int mfx_job_fetch_particles_range_async(mfx_job *job, size_t first, size_t count, void *pos, void *vel, void *ids) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (!job->d.want_particles) return set_error(MFX_ESTATE, "job was created without particles");
  if (!job->has_run || job->noise_only) return set_error(MFX_ESTATE, "job has not produced particles");
  if (first > job->npart || count > job->npart - first)
    return set_error(MFX_EINVAL, "range [%zu, %zu) outside the %zu particles", first, first + count, job->npart);
  CU(cudaSetDevice(job->eng->device));
  if (!job->xfer[0]) CU(cudaStreamCreateWithFlags(&job->xfer[0], cudaStreamNonBlocking));
  if (!job->fetched) CU(cudaEventCreateWithFlags(&job->fetched, cudaEventDisableTiming));
  // after the job's work enqueued so far (the run whose particles these are)
  CU(cudaEventRecord(job->fetched, job->stream));
  CU(cudaStreamWaitEvent(job->xfer[0], job->fetched, 0));
  const size_t ps = job->d.pos64 ? 8 : 4, vs = job->d.vel64 ? 8 : 4, is = job->d.id64 ? 8 : 4;
  const bool host_ids = ids && host_writable(ids);
  if (job->host_q && ((pos && !host_writable(pos)) || (ids && !host_ids)))
    return set_error(MFX_ESTATE, "a job with host-side positions fetches positions and ids into host memory only");
  const bool kernel_ids = ids && !host_ids && !job->ids;  // no device array: the closed form on the device
  const Xfer xs[3] = {{job->host_q ? nullptr : pos, static_cast<char *>(job->pos) + 3 * ps * first, 3 * ps * count},
                      {vel, static_cast<char *>(job->vel) + 3 * vs * first, 3 * vs * count},
                      {(host_ids || kernel_ids) ? nullptr : ids, static_cast<char *>(job->ids) + is * first, is * count}};
  join_id_fill(job);  // an earlier fetch's host threads (long done when fetches are a step apart)
  if (host_ids) start_id_fill(job, first, count, ids);
  if (job->host_q && pos) TRY(start_pos_fill(job, first, count, pos, job->xfer[0]));
  if (kernel_ids) TRY(fill_ids_device(job, first, count, ids, job->xfer[0]));
  // one copy stream: the host link is full with one (193 GB/s on GB300), and
  // several streams' copies beside a running job made the step times vary
  cudaStream_t x = job->xfer[0];
  for (const Xfer &q : xs)
    if (q.dst && q.bytes) CU(cudaMemcpyAsync(q.dst, q.src, q.bytes, cudaMemcpyDefault, x));
  CU(cudaEventRecord(job->fetched, x));
  // the set the last run wrote
  if (job->ring) CU(cudaEventRecord(job->ring_free[(job->ring_next + job->ring_sets - 1) % job->ring_sets], x));
  return MFX_OK;
  GUARD_END
}

int mfx_job_wait_fetch(mfx_job *job) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  join_id_fill(job);
  if (job->xfer[0]) CU(cudaStreamSynchronize(job->xfer[0]));
  return MFX_OK;
  GUARD_END
}

int mfx_job_particles_device(mfx_job *job, const void **pos, const void **vel, const void **ids, size_t *np) {
  GUARD_BEGIN
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (pos) *pos = job->pos;
  if (vel) *vel = job->vel;
  if (ids) {
    if (job->ids) {
      *ids = job->ids;
    } else {
      // the fused read-out writes no ids: fill them into an array of their own
      CU(cudaSetDevice(job->eng->device));
      if (!job->ids_dev) {
        CU(cudaMallocAsync(&job->ids_dev, job->npart * (job->d.id64 ? 8 : 4), job->stream));
      }
      TRY(fill_ids_device(job, 0, job->npart, job->ids_dev, job->stream));
      CU(cudaStreamSynchronize(job->stream));
      *ids = job->ids_dev;
    }
  }
  if (np) *np = job->npart;
  return MFX_OK;
  GUARD_END
}

int mfx_job_fetch_field(mfx_job *job, int field_id, double *out) {
  GUARD_BEGIN
  if (!job || !out) return set_error(MFX_EINVAL, "null argument");
  if (!job->has_run) return set_error(MFX_ESTATE, "job has not run");
  int slot = -1;
  double scale = 1.0;
  switch (field_id) {
    case MFX_FIELD_NOISE:
      if (!job->noise_only) return set_error(MFX_ESTATE, "noise is only kept after mfx_job_run_noise");
      slot = 0;
      break;
    case MFX_FIELD_PHI1: slot = 0; scale = 1.0 / job->scale1; break;
    case MFX_FIELD_PHI2: slot = 1; scale = 1.0 / job->scale2; break;
    case MFX_FIELD_PHI3: slot = 2; scale = 1.0 / job->scale3; break;
    case MFX_FIELD_A3X: slot = 3; scale = 1.0 / job->scale3; break;
    case MFX_FIELD_A3Y: slot = 4; scale = 1.0 / job->scale3; break;
    case MFX_FIELD_A3Z: slot = 5; scale = 1.0 / job->scale3; break;
    default: return set_error(MFX_EINVAL, "unknown field id %d", field_id);
  }
  if (field_id != MFX_FIELD_NOISE && job->noise_only) return set_error(MFX_ESTATE, "only the noise was run");
  if (!job->nf[slot]) return set_error(MFX_EINVAL, "field %d not computed at LPT order %d", field_id, job->d.lpt_order);
  const size_t nc = size_t(job->N) * job->N * job->nk;
  CU(cudaStreamSynchronize(job->stream));
  if (job->fp64) {
    CU(cudaMemcpy(out, job->nf[slot], nc * 16, cudaMemcpyDeviceToHost));
    if (scale != 1.0)
      for (size_t q = 0; q < 2 * nc; ++q) out[q] *= scale;
  } else {
    std::vector<float> tmp(2 * nc);
    CU(cudaMemcpy(tmp.data(), job->nf[slot], nc * 8, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < 2 * nc; ++q) out[q] = double(tmp[q]) * scale;
  }
  return MFX_OK;
  GUARD_END
}

int mfx_job_stage_times(mfx_job *job, double *ms, int max_stages) {
  if (!job || !ms) return set_error(MFX_EINVAL, "null argument");
  if (!job->has_run || job->noise_only) return 0;
  if (cudaStreamSynchronize(job->stream) != cudaSuccess) return set_error(MFX_ECUDA, "sync failed");
  int n = 0;
  for (int s = 0; s < 4 && n < max_stages; ++s) {
    float t = 0;
    if (cudaEventElapsedTime(&t, job->ev[s], job->ev[s + 1]) != cudaSuccess) t = 0;
    ms[n++] = t;
  }
  return n;
}

int mfx_job_algorithmic_bytes(mfx_job *job, double *bytes) {
  if (!job || !bytes) return set_error(MFX_EINVAL, "null argument");
  // ideal-fused stage model: each stage reads each distinct input once and
  // writes each output once; FFTs count only their callback inputs/outputs.
  const double s = double(job->rsize);
  const double N3 = double(job->N) * job->N * job->N, M3 = double(job->M) * job->M * job->M;
  const double F = s * N3, P = s * M3;
  double b = F;  // phi1
  if (job->d.lpt_order == 2) b += 12 * P + 7 * F;
  if (job->d.lpt_order == 3) b += 57 * P + 25 * F;
  if (job->d.want_particles) {
    const int npot = job->d.lpt_order == 1 ? 1 : (job->d.lpt_order == 2 ? 2 : 6);
    const double pos_b = job->d.pos64 ? 8 : 4, vel_b = job->d.vel64 ? 8 : 4;
    b += npot * F + job->ns * (6 * F + 3 * pos_b * N3 + 3 * vel_b * N3 + (job->d.id64 ? 8 : 4) * N3);
  }
  *bytes = b;
  return MFX_OK;
}

int mfx_job_launch_count(mfx_job *job, int *own, int *ffts) {
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (own) *own = job->own_launches;
  if (ffts) *ffts = job->fft_execs;
  return MFX_OK;
}

int mfx_job_set_profiling(mfx_job *job, int on) {
  if (!job) return set_error(MFX_EINVAL, "null job");
  job->prof = on != 0;
  return MFX_OK;
}

int mfx_job_kernel_profile(mfx_job *job, int max_entries, char *names, double *ms, double *bytes, int *launches) {
  if (!job) return set_error(MFX_EINVAL, "null job");
  if (cudaStreamSynchronize(job->stream) != cudaSuccess) return set_error(MFX_ECUDA, "sync failed");
  std::vector<std::string> keys;
  std::vector<double> t, b;
  std::vector<int> c;
  for (const auto &r : job->prof_recs) {
    float e = 0;
    if (cudaEventElapsedTime(&e, r.a, r.b) != cudaSuccess) e = 0;
    size_t q = 0;
    while (q < keys.size() && keys[q] != r.name) ++q;
    if (q == keys.size()) {
      keys.push_back(r.name);
      t.push_back(0);
      b.push_back(0);
      c.push_back(0);
    }
    t[q] += e;
    b[q] += r.bytes;
    c[q] += 1;
  }
  const int n = int(keys.size());
  for (int q = 0; q < n && q < max_entries; ++q) {
    if (names) {
      std::strncpy(names + 32 * q, keys[q].c_str(), 31);
      names[32 * q + 31] = 0;
    }
    if (ms) ms[q] = t[q];
    if (bytes) bytes[q] = b[q];
    if (launches) launches[q] = c[q];
  }
  return n;
}

int mfx_job_destroy(mfx_job *job) {
  free_job(job);
  return MFX_OK;
}

int mfx_batch_create(mfx_engine *eng, const mfx_job_desc *descs, int count, mfx_batch **out) {
  GUARD_BEGIN
  if (!eng || !descs || !out || count <= 0) return set_error(MFX_EINVAL, "bad arguments");
  CU(cudaSetDevice(eng->device));
  auto *b = new mfx_batch();
  b->eng = eng;
  auto fail = [&](int rc) {
    free_batch(b);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess)
    return fail(set_error(MFX_ECUDA, "batch stream/event creation failed"));
  if (cudaGraphCreate(&b->parent, 0) != cudaSuccess) return fail(set_error(MFX_ECUDA, "cudaGraphCreate failed"));
  for (int q = 0; q < count; ++q) {
    mfx_job *j = nullptr;
    int rc = create_job(eng, &descs[q], &j);
    if (rc != MFX_OK) return fail(rc);
    b->jobs.push_back(j);
    cudaGraph_t g = nullptr;
    if ((rc = capture_pipeline(j, &g)) != MFX_OK) return fail(rc);
    b->children.push_back(g);
    cudaGraphNode_t node;
    if (cudaGraphAddChildGraphNode(&node, b->parent, nullptr, 0, g) != cudaSuccess)
      return fail(set_error(MFX_ECUDA, "cudaGraphAddChildGraphNode failed for job %d", q));
  }
  cudaError_t e = cudaGraphInstantiate(&b->exec, b->parent, 0);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return fail(set_error(MFX_ECUDA, "cudaGraphInstantiate(batch): %s", cudaGetErrorString(e)));
  }
  *out = b;
  return MFX_OK;
  GUARD_END
}

int mfx_batch_run(mfx_batch *b) {
  GUARD_BEGIN
  if (!b) return set_error(MFX_EINVAL, "null batch");
  CU(cudaSetDevice(b->eng->device));
  CU(cudaEventRecord(b->e0, b->stream));
  CU(cudaGraphLaunch(b->exec, b->stream));
  CU(cudaEventRecord(b->e1, b->stream));
  for (auto j : b->jobs) {
    j->has_run = true;
    j->noise_only = false;
  }
  b->ran = true;
  return MFX_OK;
  GUARD_END
}

int mfx_batch_wait(mfx_batch *b, double *device_ms) {
  GUARD_BEGIN
  if (!b) return set_error(MFX_EINVAL, "null batch");
  CU(cudaStreamSynchronize(b->stream));
  if (device_ms) {
    float ms = 0;
    if (b->ran) CU(cudaEventElapsedTime(&ms, b->e0, b->e1));
    *device_ms = ms;
  }
  return MFX_OK;
  GUARD_END
}

int mfx_batch_job(mfx_batch *b, int index, mfx_job **job) {
  if (!b || !job || index < 0 || index >= int(b->jobs.size())) return set_error(MFX_EINVAL, "bad arguments");
  *job = b->jobs[index];
  return MFX_OK;
}

int mfx_batch_destroy(mfx_batch *b) {
  free_batch(b);
  return MFX_OK;
}

int mfx_debug_ranlxd1_words(mfx_engine *eng, unsigned long seed, size_t count, uint64_t *out) {
  GUARD_BEGIN
  if (!eng || !out) return set_error(MFX_EINVAL, "null argument");
  if (seed >= 0x80000000UL) return set_error(MFX_EINVAL, "device seeding takes seeds below 2^31");
  CU(cudaSetDevice(eng->device));
  uint64_t *d = nullptr;
  CU(cudaMalloc(&d, count * 8));
  k_ranlux_words<<<1, 1>>>(uint32_t(seed), count, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, d, count * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return set_error(MFX_ECUDA, "ranlux words: %s", cudaGetErrorString(e));
  return MFX_OK;
  GUARD_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Serving: a request loop with admission by HBM footprint.
//
// Requests are copied at submission and queued.  An admission thread admits
// a queued job as soon as an in-flight slot is free and the job's arena fits
// the engine's HBM budget: the oldest job that fits, scanning from the head
// (a later job may pass a head that does not fit yet), unless the head has
// waited longer than the bypass age limit, after which only the head may be
// admitted, so that large jobs are not starved.  Admitted jobs are set up --
// arena, tables, launches -- by a small pool of setup threads, so that setting
// up one job never holds back the admission of the next; the footprints of
// admitted jobs are reserved against the budget until their arenas exist.
// Each job runs on its own stream and keeps its fields and particles resident
// on the device until the client fetches and releases it.  Admitted jobs
// overlap on the GPU; arenas come from the stream-ordered pool and FFT plans
// from the plan pool, so admission and retirement never synchronise the
// device.  A job's results do not depend on what else runs: every job has its
// own arena and plans.
// ---------------------------------------------------------------------------
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <thread>

namespace {
using clk = std::chrono::steady_clock;

// the life of a request; a ticket is finished (results readable or an error
// recorded) exactly when its state is kDone or kFailed
enum TicketState { kQueued = 0, kSetup = 1, kRunning = 2, kDone = 3, kFailed = 4 };

struct Ticket {
  uint64_t id = 0;
  mfx_job_desc d{};
  std::vector<uint32_t> seeds;
  std::vector<double> amp, plt;
  size_t footprint = 0;
  clk::time_point t_submit, t_admit, t_launch, t_done;  // t_launch: set up, pipeline enqueued
  int state = 0;  // TicketState
  bool small = false;  // admitted beside the in-flight slots (mfx_server_set_small_jobs)
  int rc = MFX_OK;
  std::string err;
  mfx_job *job = nullptr;
  cudaEvent_t done = nullptr;
};
constexpr int kSetupThreads = 2;
}  // namespace

struct mfx_server {
  mfx_engine *eng = nullptr;
  int max_inflight = 8;
  bool bypass = true;
  double bypass_age_ms = 100.0;
  bool size_priority = true;  // stream priority by the job's footprint
  bool small_first = true;    // the smallest jobs on the highest priority
  bool largest_first = false; // admit the largest queued job that fits, not the oldest
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Ticket *> queue;     // waiting for admission
  std::deque<Ticket *> setup_q;   // admitted, waiting for a setup thread
  std::map<uint64_t, std::unique_ptr<Ticket>> tickets;
  std::thread worker;
  std::vector<std::thread> setup;
  bool stop = false;
  uint64_t next_id = 1;
  int inflight = 0;     // admitted and not yet finished (setting up or running)
  size_t reserved = 0;  // footprints of admitted jobs whose arenas do not exist yet
  // small jobs (footprint <= small_bytes) are admitted beside the max_inflight
  // slots, at most max_small of them at once (mfx_server_set_small_jobs)
  size_t small_bytes = 0;
  int max_small = 0, inflight_small = 0;
  bool is_small(const Ticket *t) const { return small_bytes > 0 && t->footprint <= small_bytes; }
  bool slot_free(const Ticket *t) const {
    return is_small(t) ? inflight_small < max_small : inflight < max_inflight;
  }
};

static double ms_between(clk::time_point a, clk::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// Index of the queued job to admit next, or -1 (s->mu held).
static int pick_admission(mfx_server *s, clk::time_point now) {
  if (s->queue.empty()) return -1;
  size_t in_use;
  {
    std::lock_guard<std::mutex> ek(s->eng->mu);
    in_use = s->eng->in_use;
  }
  const bool head_may_be_passed = s->bypass && ms_between(s->queue.front()->t_submit, now) <= s->bypass_age_ms;
  const size_t free_bytes = s->eng->budget - std::min(s->eng->budget, in_use + s->reserved);
  if (s->largest_first && head_may_be_passed) {
    // the largest jobs set the latency tail: admit the largest that fits
    // (the oldest among equals) while the head is young enough to be passed
    int best = -1;
    for (size_t q = 0; q < s->queue.size(); ++q)
      if (s->queue[q]->footprint <= free_bytes && s->slot_free(s->queue[q]) &&
          (best < 0 || s->queue[q]->footprint > s->queue[size_t(best)]->footprint))
        best = int(q);
    return best;
  }
  // a small job takes no in-flight slot: it may pass a head that waits only
  // for a slot (the head fits the budget) however old the head is
  const Ticket *head = s->queue.front();
  const bool head_waits_for_slot_only = !s->is_small(head) && head->footprint <= free_bytes;
  for (size_t q = 0; q < s->queue.size(); ++q) {
    const Ticket *t = s->queue[q];
    if (q > 0 && !head_may_be_passed && !(s->is_small(t) && head_waits_for_slot_only)) continue;
    if (t->footprint <= free_bytes && s->slot_free(t)) return int(q);
  }
  return -1;
}

static void server_loop(mfx_server *s) {
  cudaSetDevice(s->eng->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    // retire finished jobs (their results stay resident)
    for (auto &kv : s->tickets) {
      Ticket *t = kv.second.get();
      if (t->state != kRunning) continue;
      const cudaError_t q = cudaEventQuery(t->done);
      if (q == cudaErrorNotReady) continue;
      t->t_done = clk::now();
      t->state = (q == cudaSuccess) ? kDone : kFailed;
      if (q != cudaSuccess) {
        t->rc = MFX_ECUDA;
        t->err = cudaGetErrorString(q);
      }
      --(t->small ? s->inflight_small : s->inflight);
      s->cv.notify_all();
    }
    // admit while a slot and the HBM budget allow; the setup threads take it from here
    while (true) {
      const auto now = clk::now();
      const int q = pick_admission(s, now);
      if (q < 0) break;  // wait for running jobs to finish and results to be released
      Ticket *t = s->queue[size_t(q)];
      s->queue.erase(s->queue.begin() + q);
      t->t_admit = now;
      t->state = kSetup;
      t->small = s->is_small(t);
      s->reserved += t->footprint;
      ++(t->small ? s->inflight_small : s->inflight);
      s->setup_q.push_back(t);
      s->cv.notify_all();
    }
    s->cv.wait_for(lk, std::chrono::microseconds(s->inflight + s->inflight_small > 0 ? 50 : 2000));
  }
}

// Stream priority by footprint, one level per factor of four above 64 MB
// (up to the device's range).  small_first: the smallest jobs on the highest
// priority.  The fused kernels are persistent (a grid fills the GPU), so jobs
// on the GPU together run kernel by kernel rather than side by side, and a
// small job's forty short kernels would each wait behind a large job's long
// ones; ahead of them, the small jobs finish in about their own time and
// delay the large ones by little.  Otherwise the largest jobs go first.
static int stream_priority_for(size_t footprint, bool small_first) {
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return 0;
  int level = 0;
  for (size_t f = footprint >> 26; f >= 4; f >>= 2) ++level;  // 64 MB units, x4 per level
  return small_first ? std::min(least, greatest + level) : std::max(greatest, least - level);
}

static void setup_loop(mfx_server *s) {
  cudaSetDevice(s->eng->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv.wait(lk, [s] { return s->stop || !s->setup_q.empty(); });
    if (s->stop) return;
    Ticket *t = s->setup_q.front();
    s->setup_q.pop_front();
    lk.unlock();
    mfx_job *j = nullptr;
    int rc = create_job(s->eng, &t->d, &j, s->size_priority ? stream_priority_for(t->footprint, s->small_first) : 0);
    std::string err = rc == MFX_OK ? "" : g_last_error;
    if (rc == MFX_OK) rc = j->fp64 ? run_pipeline<double>(j) : run_pipeline<float>(j);
    if (rc == MFX_OK && cudaEventRecord(t->done, j->stream) != cudaSuccess) rc = MFX_ECUDA;
    if (rc != MFX_OK && err.empty()) err = g_last_error;
    if (rc != MFX_OK && j) {
      free_job(j);
      j = nullptr;
    }
    lk.lock();
    s->reserved -= std::min(s->reserved, t->footprint);
    if (rc != MFX_OK) {
      t->state = kFailed;
      t->rc = rc;
      t->err = err;
      t->t_done = clk::now();
      --(t->small ? s->inflight_small : s->inflight);
    } else {
      t->job = j;
      t->t_launch = clk::now();
      t->state = kRunning;
    }
    s->cv.notify_all();
  }
}

extern "C" {

int mfx_server_create(mfx_engine *eng, int max_inflight, mfx_server **out) {
  GUARD_BEGIN
  if (!eng || !out || max_inflight < 1) return set_error(MFX_EINVAL, "bad arguments");
  auto *s = new mfx_server();
  s->eng = eng;
  engine_retain(eng);
  s->max_inflight = max_inflight;
  s->worker = std::thread(server_loop, s);
  for (int q = 0; q < kSetupThreads; ++q) s->setup.emplace_back(setup_loop, s);
  *out = s;
  return MFX_OK;
  GUARD_END
}

int mfx_server_set_policy(mfx_server *s, int bypass, double bypass_age_ms) {
  if (!s || bypass_age_ms < 0) return set_error(MFX_EINVAL, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  s->bypass = bypass != 0;
  s->bypass_age_ms = bypass_age_ms;
  s->size_priority = (bypass & 2) == 0;  // bit 1: every job at the default priority
  s->largest_first = (bypass & 4) != 0;  // bit 2: largest queued job first
  s->small_first = (bypass & 8) == 0;    // bit 3: the largest jobs on the highest priority
  s->cv.notify_all();
  return MFX_OK;
}

int mfx_server_submit(mfx_server *s, const mfx_job_desc *desc, uint64_t *ticket) {
  GUARD_BEGIN
  if (!s || !ticket) return set_error(MFX_EINVAL, "null argument");
  TRY(check_desc(desc));
  auto t = std::make_unique<Ticket>();
  t->d = *desc;
  const size_t n = desc->ngrid;
  if (desc->noise_generator == MFX_NOISE_NGENIC) t->seeds.assign(desc->seed_table, desc->seed_table + n * n);
  t->amp.assign(desc->amp_table, desc->amp_table + desc->amp_table_len);
  if (desc->plt) t->plt.assign(desc->plt_table, desc->plt_table + MFX_PLT_TABLE_DOUBLES);
  t->d.seed_table = desc->noise_generator == MFX_NOISE_NGENIC ? t->seeds.data() : nullptr;
  t->d.amp_table = t->amp.data();
  t->d.plt_table = desc->plt ? t->plt.data() : nullptr;
  TRY(mfx_job_footprint(s->eng, desc, &t->footprint));
  if (t->footprint > s->eng->budget)
    return set_error(MFX_EADMIT, "job footprint %zu exceeds the engine budget %zu", t->footprint, s->eng->budget);
  CU(cudaSetDevice(s->eng->device));
  CU(cudaEventCreateWithFlags(&t->done, cudaEventDisableTiming));
  t->t_submit = clk::now();
  std::lock_guard<std::mutex> lk(s->mu);
  t->id = s->next_id++;
  *ticket = t->id;
  s->queue.push_back(t.get());
  s->tickets[t->id] = std::move(t);
  s->cv.notify_all();
  return MFX_OK;
  GUARD_END
}

int mfx_server_wait(mfx_server *s, uint64_t ticket, int timeout_ms) {
  GUARD_BEGIN
  if (!s) return set_error(MFX_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return set_error(MFX_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  Ticket *t = it->second.get();
  auto pred = [t] { return t->state >= kDone; };
  if (timeout_ms < 0) s->cv.wait(lk, pred);
  else if (!s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return set_error(MFX_ETIMEOUT, "ticket %llu not finished after %d ms", (unsigned long long)ticket, timeout_ms);
  if (t->state == kFailed) return set_error(t->rc, "ticket %llu failed: %s", (unsigned long long)ticket, t->err.c_str());
  return MFX_OK;
  GUARD_END
}

int mfx_server_ticket_times(mfx_server *s, uint64_t ticket, double *queued_ms, double *latency_ms) {
  if (!s) return set_error(MFX_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return set_error(MFX_EINVAL, "unknown ticket");
  Ticket *t = it->second.get();
  if (t->state < kDone) return set_error(MFX_ESTATE, "ticket not finished");
  if (queued_ms) *queued_ms = ms_between(t->t_submit, t->t_admit);
  if (latency_ms) *latency_ms = ms_between(t->t_submit, t->t_done);
  return MFX_OK;
}

int mfx_server_set_small_jobs(mfx_server *s, size_t footprint_bytes, int max_small) {
  if (!s || max_small < 0) return set_error(MFX_EINVAL, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  s->small_bytes = max_small > 0 ? footprint_bytes : 0;
  s->max_small = max_small;
  s->cv.notify_all();
  return MFX_OK;
}

int mfx_server_ticket_phases(mfx_server *s, uint64_t ticket, double *queued_ms, double *setup_ms, double *run_ms) {
  if (!s) return set_error(MFX_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return set_error(MFX_EINVAL, "unknown ticket");
  Ticket *t = it->second.get();
  if (t->state != kDone) return set_error(MFX_ESTATE, "ticket not finished");
  if (queued_ms) *queued_ms = ms_between(t->t_submit, t->t_admit);
  if (setup_ms) *setup_ms = ms_between(t->t_admit, t->t_launch);
  if (run_ms) *run_ms = ms_between(t->t_launch, t->t_done);
  return MFX_OK;
}

int mfx_server_job(mfx_server *s, uint64_t ticket, mfx_job **job) {
  if (!s || !job) return set_error(MFX_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return set_error(MFX_EINVAL, "unknown ticket");
  if (it->second->state != kDone) return set_error(MFX_ESTATE, "ticket not finished");
  *job = it->second->job;
  return MFX_OK;
}

int mfx_server_release(mfx_server *s, uint64_t ticket) {
  GUARD_BEGIN
  if (!s) return set_error(MFX_EINVAL, "null server");
  std::unique_ptr<Ticket> t;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return set_error(MFX_EINVAL, "unknown ticket");
    if (it->second->state < kDone) return set_error(MFX_ESTATE, "ticket still queued, being set up or running");
    t = std::move(it->second);
    s->tickets.erase(it);
  }
  if (t->job) free_job(t->job);
  if (t->done) cudaEventDestroy(t->done);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->cv.notify_all();
  }
  return MFX_OK;
  GUARD_END
}

int mfx_server_destroy(mfx_server *s) {
  if (!s) return MFX_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (auto &th : s->setup)
    if (th.joinable()) th.join();
  for (auto &kv : s->tickets) {
    if (kv.second->job) free_job(kv.second->job);
    if (kv.second->done) cudaEventDestroy(kv.second->done);
  }
  mfx_engine *eng = s->eng;
  delete s;
  engine_release(eng);
  return MFX_OK;
}

}  // extern "C"

/*
 * mfx -- GB300-native engine for monofonIC's initial-condition hot path.
 *
 * Thin C ABI over the CUDA engine (libmfx.so).  No C++ or torch types cross
 * it: plain pointers, sizes and integer status codes.  Every entry point
 * returns MFX_OK (0) or a negative status; mfx_last_error() returns the
 * message of the calling thread's last failure.  C++ exceptions never cross
 * this boundary.
 *
 * Each declaration names the reference interface it replaces
 * (file:line inside the monofonIC source tree).
 */
#ifndef MFX_H
#define MFX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MFX_OK 0
#define MFX_EINVAL (-1)    /* invalid argument                          */
#define MFX_ENOMEM (-2)    /* device or host allocation failed           */
#define MFX_ECUDA (-3)     /* CUDA / cuFFT error                         */
#define MFX_ETIMEOUT (-4)  /* wait timed out                             */
#define MFX_ECANCEL (-5)   /* job cancelled                              */
#define MFX_ESTATE (-6)    /* call not valid in the object's state       */
#define MFX_EADMIT (-7)    /* serving: job does not fit the HBM budget   */

/* ---- enums --------------------------------------------------------------- */
/* particle::lattice, particle_generator.hh:31-39 (Bravais lattices only) */
#define MFX_LATTICE_SC 0
#define MFX_LATTICE_BCC 1
#define MFX_LATTICE_FCC 2

/* arithmetic form of a job */
#define MFX_FP64 0  /* plain form: the reference's FP64 algorithm            */
#define MFX_FP32C 1 /* FP32 FFTs/products, compensated 3LPT source sums,
                       FP64 tables and FP64 q+Psi position sum              */

/* white-noise generators (the [random] generator key) */
#define MFX_NOISE_NGENIC 0
#define MFX_NOISE_MUSIC1 1
/* a white-noise field given in real space (noise_field): MUSIC1's noise read
   from a file in place of a seed (random_music_wnoise_generator.cc:68-282) */
#define MFX_NOISE_FIELD 2

/* fields fetchable with mfx_job_fetch_field (k-space, N x N x (N/2+1) complex) */
#define MFX_FIELD_NOISE 0 /* white noise as RNG_plugin::Fill_Grid leaves it   */
#define MFX_FIELD_PHI1 1  /* phi(1), unscaled, ic_generator.cc:509-516         */
#define MFX_FIELD_PHI2 2  /* phi(2), unscaled, ic_generator.cc:523-548         */
#define MFX_FIELD_PHI3 3  /* phi(3), unscaled, ic_generator.cc:571-611         */
#define MFX_FIELD_A3X 4   /* A(3) components, unscaled, ic_generator.cc:613-628 */
#define MFX_FIELD_A3Y 5
#define MFX_FIELD_A3Z 6

/* ---- objects -------------------------------------------------------------- */
typedef struct mfx_engine mfx_engine;
typedef struct mfx_job mfx_job;

typedef struct {
  int device;              /* CUDA device ordinal                               */
  size_t hbm_budget_bytes; /* 0 = 90% of free memory at creation                */
} mfx_engine_opts;

/*
 * One initial-conditions job.  Replaces the parameter set that
 * ic_generator::run reads (ic_generator.cc:100-273) plus the inputs the hot
 * path takes from the RNG / transfer-function plugins.
 */
typedef struct {
  uint32_t ngrid;    /* [setup] GridRes, even, >= 8                          */
  double boxlen;     /* [setup] BoxLength (Mpc/h)                            */
  int lpt_order;     /* 1, 2 or 3                                            */
  int lattice;       /* MFX_LATTICE_*                                        */
  int plt;           /* 1: PLT gradient + vfac_corr (needs plt_table)        */
  int precision;     /* MFX_FP64 or MFX_FP32C                                */
  int fixing;        /* [setup] DoFixing                                     */
  int inversion;     /* [setup] DoInversion                                  */
  /* NGenIC per-column seed table, N*N uint32 (random_ngenic.cc:47-74) */
  const uint32_t *seed_table;
  /* amplitude table indexed by n = i^2+j^2+k^2 over signed mode indices:
     amp_table[n] = get_amplitude(kf*sqrt(n)) / (kf^2 n), amp_table[0] = 0,
     kf = 2 pi / boxlen; length >= 3*(N/2)^2 + 1 (cosmology_calculator.hh:429-432) */
  const double *amp_table;
  size_t amp_table_len;
  /* PLT tables from mfx_plt_table_build (NULL when plt == 0) */
  const double *plt_table;
  /* LPT time coefficients, ic_generator.cc:252-269 */
  double g1, g2, g3, g3c;
  double vfac1, vfac2, vfac3;
  /* output_plugin::position_unit / velocity_unit (output_plugin.hh:86-90) */
  double lunit, vunit;
  int pos64;  /* positions as double (else float)                           */
  int vel64;  /* velocities as double (else float)                          */
  int id64;   /* IDs as uint64 (else uint32), output_plugin::has_64bit_ids    */
  uint64_t id_offset; /* lattice_generator IDoffset (particle_generator.hh:232) */
  int want_particles; /* 0: stop after the LPT potentials (fields only)     */
  /* the [random] generator plugin (random_plugin.cc:62-81): MFX_NOISE_NGENIC
     reads seed_table; MFX_NOISE_MUSIC1 (random_music.cc; ngrid a power of
     two) draws the noise on the device from its seeds and music_cubesize and
     ignores seed_table */
  int noise_generator;
  int64_t music_seed;       /* [random] seed[log2 ngrid], > 0 (or 0 with music_seeds) */
  uint32_t music_cubesize;  /* [random] cubesize, 0 = 32 (random_plugin.hh:24) */
  /* [random] seed[l] for the levels l <= log2 ngrid + 3, 0 where the config
     has no such key.  The coarsest seeded level is filled; if it is coarser
     than the grid's, each finer level up to the grid's refines the one below
     by coarse mode replacement with its own seed, or the level's dummy seed
     (random_music.cc:160-245, random_music_wnoise_generator.cc:392-547); if
     it is finer, it is restricted down to the grid's level by k-space
     averaging (random_music.cc:238-265, random_music_wnoise_generator.cc:
     288-380). */
  int64_t music_seeds[12];
  /* MFX_NOISE_FIELD: ngrid^3 doubles, [x][y][z] with z fastest, the values
     Fill_Grid copies into the grid.  MFX_NOISE_MUSIC1: NULL, or the noise of
     a level coarser than the grid's read from a file (random_music.cc:216-236,
     a noise file at the coarsest level given): noise_field_res^3 doubles, the
     start of the refinement chain, whose finer levels come from music_seeds
     (or their dummy seeds).  Read at every run of the job (host memory:
     page-locked memory must stay unchanged until the run's noise stage has
     finished) */
  const double *noise_field;
  /* cells per axis of noise_field: 0 = ngrid.  With MFX_NOISE_MUSIC1 a power
     of two, at least 2 and below ngrid, with no music_seeds at or below its
     level */
  uint32_t noise_field_res;
} mfx_job_desc;

/* ---- errors -------------------------------------------------------------- */
/* Copies the calling thread's last error message; returns its full length. */
size_t mfx_last_error(char *buf, size_t len);
const char *mfx_version(void);

/* ---- engine -------------------------------------------------------------- */
/* Replaces the process-wide FFTW/OpenMP set-up of main.cc:156-182.
   Jobs, batches and servers made on an engine keep it alive: destroying the
   engine while some remain only marks it closing, and the last of them to be
   destroyed releases it (the engine must not be used after
   mfx_engine_destroy either way). */
int mfx_engine_create(const mfx_engine_opts *opts, mfx_engine **out);
int mfx_engine_destroy(mfx_engine *eng);
/* Device bytes a job with this descriptor needs (arena + FFT work area). */
int mfx_job_footprint(mfx_engine *eng, const mfx_job_desc *desc, size_t *bytes);

/* ---- jobs ----------------------------------------------------------------- */
/* Allocates the job's device arena, creates (or reuses) its FFT plans and
   uploads the descriptor's tables.  Replaces the Grid_FFT / OrszagConvolver /
   lattice_generator allocations of ic_generator.cc:288-310, 475, 743-745. */
int mfx_job_create(mfx_engine *eng, const mfx_job_desc *desc, mfx_job **out);
/* Re-uploads the tables of `desc` (same sizes as at creation) from host
   memory, asynchronously on the job's stream. */
int mfx_job_upload(mfx_job *job, const mfx_job_desc *desc);
/* Enqueues the whole hot path on the job's stream: RNG_plugin::Fill_Grid
   (random_ngenic.cc:84-154) through the particle read-out of
   lattice_generator::set_positions / set_velocities
   (particle_generator.hh:499-687), i.e. ic_generator.cc:288-1060. */
int mfx_job_run(mfx_job *job);
/* Waits for the job's stream; timeout_ms < 0 waits forever.  MFX_ETIMEOUT
   leaves the job running and usable. */
int mfx_job_wait(mfx_job *job, int timeout_ms);
/* Copies the particle container (particle_container.hh:29-188 layout:
   interleaved xyz) into caller buffers; each pointer may be host or device
   memory or NULL to skip.  Ids for a host buffer are not copied: they are a
   closed form of the particle index (particle_generator.hh:229-248), written
   by host threads while the positions and velocities cross the host link. */
int mfx_job_fetch_particles(mfx_job *job, void *pos, void *vel, void *ids);
/* Copies particles [first, first + count) only, for output plugins that write
   a large container in chunks (the reference's plugins write the whole
   container at once, output_plugin.hh:62-68). */
int mfx_job_fetch_particles_range(mfx_job *job, size_t first, size_t count, void *pos, void *vel, void *ids);
/* Re-runs the displacement / velocity assembly and the particle stage
   (ic_generator.cc:937-1030) on the potentials of the last mfx_job_run,
   combining only the LPT orders in orders_mask (bit n-1: order n, 1..7), so
   that each order's displacement and velocity can be read on its own (the
   per-order error statement of the FP32 form).  Not capturable in a graph. */
int mfx_job_assemble(mfx_job *job, int orders_mask);
/* Baryon + CDM runs (ic_generator.cc:706-1064 with [setup] DoBaryons):
   both species share the LPT potentials of one mfx_job_run and differ in the
   assembly.  mfx_job_set_species selects the species the next run or
   mfx_job_assemble produces: its lattice (the baryons' secondary lattice is
   shifted by particle_generator.hh:56-63), its particle IDoffset
   (ic_generator.cc:738-739), the linear relative-velocity term
   -vfac1 C A_theta_bc(k) w grad / k^2 added to the velocities before
   vfac_corr (ic_generator.cc:1016-1020; amp_tbc = get_amplitude_theta_bc per
   |k|^2 index like amp_table, NULL for none) and the particle masses
   (1 + C delta_bc(x)) * mass_factor / (n_s N^3) with delta_bc(k) =
   w A_delta_bc(k) (ic_generator.cc:749-780, particle_generator.hh:369-427;
   amp_dbc = get_amplitude_delta_bc per |k|^2 index, NULL for unperturbed
   masses); c_species is the C factor of ic_generator.cc:718-726 and
   mass_factor = Omega_species * output_plugin::mass_unit.  want_masses = 0
   skips the masses.  NULL restores the single species of the descriptor. */
typedef struct {
  int secondary_lattice;
  uint64_t id_offset;
  double c_species;
  double mass_factor;
  const double *amp_dbc;
  const double *amp_tbc;
  size_t amp_len; /* length of amp_dbc / amp_tbc, >= 3*(N/2)^2 + 1 */
  int want_masses;
} mfx_species_desc;
int mfx_job_set_species(mfx_job *job, const mfx_species_desc *species);
/* Masses of particles [first, first + count) of the last run or assembly with
   masses (double when the job's positions are double, else float;
   particle_container.hh:44-74), into host or device memory. */
int mfx_job_fetch_masses(mfx_job *job, size_t first, size_t count, void *out);
/* Semiclassical (PPT) Eulerian fields of a species (ic_generator.cc:783-901,
   output_type::field_eulerian): from the potentials of the last mfx_job_run,
   the wave function psi = sqrt(1 + C delta_bc) exp(i (phi [+ phi2]) /
   (hbar D+)) with hbar = 1.01 max|grad phi| / (pi D+), one free drift step and
   (2LPT and above) a second kick, then the density contrast
   delta = |psi|^2 - 1 and the velocities v_d = D+ vfac / L * vunit *
   hbar Im(conj(psi) d_d psi) / |psi|^2 -- the fields the reference hands to
   output_plugin::write_grid_data (density, vx, vy, vz).  Computed in FP64
   for either arithmetic form, through complex FFTs on the device.
   c_species and amp_dbc (get_amplitude_delta_bc per |k|^2 index, NULL for
   none) as in mfx_species_desc; D+ = -g1 and vfac = vfac1 of the job.  Each
   output is N^3 doubles, x slowest (host or device memory, NULL to skip);
   *hbar (optional) receives hbar.  Device scratch of about 56 N^3 bytes is
   allocated for the call and freed before it returns. */
int mfx_job_ppt_fields(mfx_job *job, double c_species, const double *amp_dbc, size_t amp_len, double *delta,
                       double *vx, double *vy, double *vz, double *hbar);
/* Pipelined output (no counterpart in the reference, whose output plugins
   write a realisation after it is generated): `sets` = 1 or 2 gives the job
   that many particle sets of its own, outside the arena (charged to the
   engine budget; MFX_EADMIT / MFX_ENOMEM when they do not fit), and runs take
   them in turn, so that a run computes while the particles of earlier runs
   are still being copied to the host by mfx_job_fetch_particles_range_async.
   A run's assembly waits only for the downloads from the set it writes: with
   two sets the whole next run overlaps a download, with one set (the choice
   when two do not fit beside the fields) everything before its assembly does.
   sets = 0 returns to the arena's particle arrays.  Either way the particles
   of earlier runs are no longer fetchable.  MFX_ESTATE for a captured job
   (and capture refuses a job with the ring). */
int mfx_job_set_output_ring(mfx_job *job, int sets);
/* Host-side positions (FP32 form, fused route, 64-bit positions; no
   counterpart in the reference): the read-out keeps each particle's float
   displacement Psi on the device instead of q + Psi in FP64, and every fetch
   into host memory copies the 12 displacement bytes instead of 24 position
   bytes and forms q + Psi in FP64 with host threads from the lattice
   coordinates -- the same doubles the device would store (the FP32 form's Psi
   is a float, and both sides add it to the same q in FP64).  With the ids
   also written on the host, a particle crosses the host link in 24 bytes
   (f32 velocities) instead of 44.  Positions and ids then reach host memory
   only (MFX_ESTATE for device destinations), and mfx_job_particles_device
   returns the displacements as the position array.  Set it before
   mfx_job_set_output_ring; a job that has run is re-assembled in the new
   form.  on = 0 returns to device-side positions. */
int mfx_job_set_host_positions(mfx_job *job, int on);
/* Enqueues the download of particles [first, first + count) of the job's
   last run into host buffers (page-locked for the copies to overlap) behind
   the job's enqueued work, and returns.  Call it before the next
   mfx_job_run.  The buffers are filled when mfx_job_wait_fetch returns.
   Without the output ring the next run waits for the download before it
   starts (its fields overwrite the particles); mfx_job_assemble always waits
   for it. */
int mfx_job_fetch_particles_range_async(mfx_job *job, size_t first, size_t count, void *pos, void *vel, void *ids);
/* Waits for the job's asynchronous downloads. */
int mfx_job_wait_fetch(mfx_job *job);
/* Device pointers of the particle arrays (valid until the next run/destroy). */
int mfx_job_particles_device(mfx_job *job, const void **pos, const void **vel, const void **ids,
                             size_t *num_particles);
/* Copies one k-space field as complex128, N*N*(N/2+1) entries.  Test hook
   standing in for output_plugin::write_grid_data (output_plugin.hh:71). */
int mfx_job_fetch_field(mfx_job *job, int field_id, double *out);
/* Runs only the white-noise fill (raw = 1: as Fill_Grid leaves it;
   raw = 0: normalised, fixed / inverted, ic_generator.cc:378-383). */
int mfx_job_run_noise(mfx_job *job, int raw);
/* Per-stage device times (ms) of the last run: noise+phi1, phi2, phi3+A3,
   assembly+particles.  Returns the number of stages written. */
int mfx_job_stage_times(mfx_job *job, double *ms, int max_stages);
/* Device-side algorithmic byte count of one run (ideal-fused stage model). */
int mfx_job_algorithmic_bytes(mfx_job *job, double *bytes);
/* Number of kernels (own + cuFFT) the last run launched. */
int mfx_job_launch_count(mfx_job *job, int *own_kernels, int *fft_execs);
/* Per-launch profiling: when on, every kernel and FFT of a run is bracketed
   by CUDA events on the job's stream and tagged with its algorithmic bytes
   (the reference's equivalent is its per-stage "took" log lines,
   ic_generator.cc:506-628).  mfx_job_kernel_profile aggregates the last run
   by kernel name (32-byte name slots) and returns the number of names. */
int mfx_job_set_profiling(mfx_job *job, int on);
int mfx_job_kernel_profile(mfx_job *job, int max_entries, char *names, double *ms, double *bytes, int *launches);
int mfx_job_destroy(mfx_job *job);

/* Sets the pencil-tile shape of the fused transforms by hand (the choice
   mfx_job_autotune makes by timing): pencils per CTA of the x/y passes
   (4, 8, 16 or 32; tiles wider than 1024 butterflies run in the lean form:
   a third as many threads, in-place transforms; lean tiles whose two input
   stages do not fit beside the transform run in an in-place form, the tile
   its own stage) and the z passes' shape:
   1 or 2 rows per CTA, 3 for one row per CTA and as many pencils per
   transform as one CTA per SM holds (the wide shape of the long padded
   lengths), or 4 for one row per CTA of three warps, each pencil transformed
   by one warp (padded lengths up to 576), for both z passes (2LPT and 3LPT
   sources).  MFX_EINVAL for a shape the padded length does not admit,
   MFX_ESTATE for a job without the fused transforms. */
int mfx_job_set_tiles(mfx_job *job, int pencils_xy, int rows_z);
/* Autotuner of the FP32 form's fused transforms: times every admissible
   pencil-tile shape (pencils per CTA of the x/y passes; the z shape of the
   2LPT and, for 3LPT jobs, the 3LPT source pass, each on its own) on the
   job's own buffers and keeps the fastest for the job and, per grid size,
   for later jobs of the engine.  Call it before mfx_job_run: it overwrites
   the job's buffers.  Returns the x/y tile and the z shape of the job's last
   source pass (0, 0 when the job does not use the fused transforms).  The
   reference has no tunables: its FFTW plans use FFTW_ESTIMATE
   (general.hh:87-93). */
int mfx_job_autotune(mfx_job *job, int *pencils_xy, int *rows_z);

/* Captures the job's whole pipeline into a CUDA graph; later mfx_job_run
   calls replay it with one cudaGraphLaunch (no per-kernel launch cost).  The
   reference has no equivalent: it runs the same stages as OpenMP loops and
   FFTW calls (ic_generator.cc:288-1060).  Stage times and per-launch
   profiling are not recorded for graph replays. */
int mfx_job_capture(mfx_job *job);

/* Ensemble of independent realisations (uneven grid sizes, seeds, boxes)
   run as ONE executable CUDA graph whose parallel branches are the jobs'
   captured pipelines.  The reference runs one realisation per process
   invocation (main.cc:73-289).  mfx_batch_wait returns the device time of the
   whole graph; mfx_batch_job gives access to each job (fetch particles or
   fields); the batch owns the jobs. */
typedef struct mfx_batch mfx_batch;
int mfx_batch_create(mfx_engine *eng, const mfx_job_desc *descs, int count, mfx_batch **out);
int mfx_batch_run(mfx_batch *b);
int mfx_batch_wait(mfx_batch *b, double *device_ms);
int mfx_batch_job(mfx_batch *b, int index, mfx_job **job);
int mfx_batch_destroy(mfx_batch *b);

/* Serving: a request loop with admission by HBM footprint (no counterpart in
   the reference, which runs one job per process, main.cc:73-289).  Submitted
   jobs (their tables are copied) wait in a queue; an admission thread admits
   the oldest queued job that fits -- fewer than max_inflight jobs running and
   its arena within the engine's HBM budget -- so a later job that fits may
   start while a larger head waits, until the head has waited longer than the
   bypass age limit (default 100 ms; mfx_server_set_policy), after which only
   the head is admitted.  Two setup threads create admitted jobs and enqueue
   them on their own streams, so jobs that arrive while others are on the GPU
   overlap with them.  Results stay resident until mfx_server_release;
   mfx_server_job gives the finished job (fetch particles / fields through the
   mfx_job_* calls).  mfx_server_ticket_times: submit -> admit and
   submit -> done (ms). */
typedef struct mfx_server mfx_server;
int mfx_server_create(mfx_engine *eng, int max_inflight, mfx_server **out);
int mfx_server_submit(mfx_server *s, const mfx_job_desc *desc, uint64_t *ticket);
int mfx_server_wait(mfx_server *s, uint64_t ticket, int timeout_ms);
int mfx_server_ticket_times(mfx_server *s, uint64_t ticket, double *queued_ms, double *latency_ms);
/* the latency of a finished ticket in three phases: queued (submit ->
   admit), set-up (admit -> pipeline enqueued on the job's stream: arena,
   tables, launches) and run (-> the job's completion seen by the server) */
int mfx_server_ticket_phases(mfx_server *s, uint64_t ticket, double *queued_ms, double *setup_ms, double *run_ms);
int mfx_server_job(mfx_server *s, uint64_t ticket, mfx_job **job);
int mfx_server_release(mfx_server *s, uint64_t ticket);
int mfx_server_destroy(mfx_server *s);
/* bypass bit 0 clear: strict first-in first-out admission; set: a later job
   may pass a head that has waited at most bypass_age_ms.  Jobs run on CUDA
   streams whose priority follows their footprint (one level per factor of
   four above 64 MB), the smallest on the highest: jobs on the GPU together
   run kernel by kernel, and ahead of the large jobs' long kernels the small
   ones finish in about their own time.  bypass bit 1 set: every job at the
   default priority; bit 3 set: the largest jobs on the highest priority.
   bypass bit 2 set (with bit 0): while the head may be passed, admit the
   largest queued job that fits instead of the oldest. */
int mfx_server_set_policy(mfx_server *s, int bypass, double bypass_age_ms);
/* Jobs whose footprint is at most footprint_bytes are admitted beside the
   max_inflight slots, up to max_small of them at once (0: off, the default).
   Such a job may pass a head that waits only for a slot, at any age: it
   takes no slot, and its kernels (smallest first by stream priority) finish
   in about the job's own time. */
int mfx_server_set_small_jobs(mfx_server *s, size_t footprint_bytes, int max_small);

/* Allocation-free white-noise fill (no counterpart in the reference): writes
   the NGenIC noise of RNG_plugin::Fill_Grid -- raw (raw = 1) or normalised /
   fixed / inverted (raw = 0) -- into a k-space field the caller allocated
   (out_device, N*N*(N/2+1) complex of double for MFX_FP64 or float for
   MFX_FP32C), for callers that cannot let a library call cudaMalloc (a host
   code that owns all of HBM through its own pool, or one running under a
   device-memory cap).  It allocates nothing; the device copy of the seed table
   lives in a fixed 4 MiB __device__ array, so ngrid is limited to
   MFX_NOALLOC_MAX_NGRID and larger sizes are rejected with MFX_EINVAL.  That
   array and the call's kernels become resident on a device when
   mfx_engine_create runs there (also under CUDA's lazy module loading), so
   create the engine before reserving the rest of HBM and before any stream
   capture; they stay resident until the process exits.  Calls share the
   array: calls that overlap on the GPU race, so order them on one stream.
   The seed table is read by a copy ordered on `stream`: a page-locked
   seed_table must stay unchanged until the work on `stream` has finished
   (pageable memory is staged before the call returns).  The call leaves the
   caller's current device unchanged.  `stream` is a cudaStream_t or NULL. */
#define MFX_NOALLOC_MAX_NGRID 1024
int mfx_noise_fill_noalloc(mfx_engine *eng, uint32_t ngrid, double boxlen, const uint32_t *seed_table, int raw,
                           int fixing, int inversion, int precision, void *out_device, void *stream);

/* Debug hook: first `count` 48-bit words of the ranlxd1 stream of `seed`,
   computed on the device (bit-exactness check of the device generator). */
int mfx_debug_ranlxd1_words(mfx_engine *eng, unsigned long seed, size_t count, uint64_t *out);

/* ---- host-side plugin logic (C++ host library, same .so) ------------------ */
/* RNG_ngenic constructor: the N*N per-column seed table
   (random_ngenic.cc:39-75). */
int mfx_ngenic_seed_table(long seed, size_t ngrid, uint32_t *table);

/* PLT eigenmode tables for a lattice on the 64^3 mesh
   (particle::lattice_gradient::init_D, particle_plt.hh:68-515).
   `out` receives 4 * 64*64*33 doubles: D_r, D_theta, D_phi, alpha^{-1}
   in kelem order.  The Ewald sums run on the device of `eng`. */
#define MFX_PLT_NGRID 64
#define MFX_PLT_TABLE_DOUBLES (4 * 64 * 64 * 33)
int mfx_plt_table_build(mfx_engine *eng, int lattice, double *out);

/* cosmology::calculator (cosmology_calculator.hh:44-523) with the
   Eisenstein & Hu transfer plugin (transfer_eisenstein.cc:25-258), built
   from INI text in the reference's config_file format (config_file.hh:96-164). */
typedef struct mfx_cosmology mfx_cosmology;
int mfx_cosmology_create(const char *ini_text, mfx_cosmology **out);
int mfx_cosmology_destroy(mfx_cosmology *c);
/* named scalars: "dplus_start", "vfact_start", "pnorm", "sqrtpnorm",
   "Omega_m", "Omega_b", "Omega_DE", "Omega_r", "h", "n_s", "sigma_8", ... */
int mfx_cosmology_get(mfx_cosmology *c, const char *name, double *value);
/* get_amplitude(k, delta_matter) (cosmology_calculator.hh:429-432) for k in h/Mpc */
int mfx_cosmology_amplitude(mfx_cosmology *c, const double *k, size_t count, double *out);
/* transfer_function_->compute(k, delta_matter) */
int mfx_cosmology_transfer(mfx_cosmology *c, const double *k, size_t count, double *out);
/* D+(a) normalised to D+(1) = 1 */
int mfx_cosmology_growth(mfx_cosmology *c, double a, double *dplus);
/* Fills amp_table (length 3*(N/2)^2+1) for grid size N and box L. */
int mfx_cosmology_amp_table(mfx_cosmology *c, uint32_t ngrid, double boxlen, double *table, size_t len);

/* Whole-run driver: the equivalent of `monofonIC <config>` for the in-scope
   path (ic_generator::run, ic_generator.cc:92-1181), writing through the
   selected output plugin.  Returns MFX_OK on success. */
int mfx_run_config(mfx_engine *eng, const char *ini_text);

#ifdef __cplusplus
}
#endif
#endif /* MFX_H */

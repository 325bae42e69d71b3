"""ctypes binding of libmfx (include/mfx.h) for tests, the bench and Python callers.

The library is built in-tree by ``monofonic_gb300.build``; loading fails loudly
when it is missing -- there is no CPU fallback for any engine entry point.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

from . import build as _build

MFX_OK, MFX_EINVAL, MFX_ENOMEM, MFX_ECUDA, MFX_ETIMEOUT, MFX_ECANCEL, MFX_ESTATE, MFX_EADMIT = 0, -1, -2, -3, -4, -5, -6, -7
SC, BCC, FCC = 0, 1, 2
NOISE_NGENIC, NOISE_MUSIC1, NOISE_FIELD = 0, 1, 2
FP64, FP32C = 0, 1
FIELD_NOISE, FIELD_PHI1, FIELD_PHI2, FIELD_PHI3, FIELD_A3X, FIELD_A3Y, FIELD_A3Z = range(7)
PLT_NGRID = 64
PLT_TABLE_DOUBLES = 4 * 64 * 64 * 33

# every entry point include/mfx.h declares
EXPORTS = [
    "mfx_last_error", "mfx_version", "mfx_engine_create", "mfx_engine_destroy", "mfx_job_footprint",
    "mfx_job_create", "mfx_job_upload", "mfx_job_run", "mfx_job_wait", "mfx_job_fetch_particles",
    "mfx_job_fetch_particles_range", "mfx_job_assemble", "mfx_job_set_tiles",
    "mfx_job_particles_device", "mfx_job_fetch_field", "mfx_job_run_noise", "mfx_job_stage_times",
    "mfx_job_algorithmic_bytes", "mfx_job_launch_count", "mfx_job_set_profiling", "mfx_job_kernel_profile",
    "mfx_job_destroy", "mfx_job_autotune", "mfx_job_capture", "mfx_batch_create", "mfx_batch_run", "mfx_batch_wait",
    "mfx_batch_job", "mfx_batch_destroy", "mfx_server_create", "mfx_server_submit", "mfx_server_wait",
    "mfx_server_ticket_times", "mfx_server_ticket_phases", "mfx_server_set_small_jobs", "mfx_server_job", "mfx_server_release", "mfx_server_destroy", "mfx_server_set_policy", "mfx_job_set_species", "mfx_job_fetch_masses", "mfx_job_ppt_fields", "mfx_job_set_host_positions", "mfx_noise_fill_noalloc", "mfx_debug_ranlxd1_words",
    "mfx_ngenic_seed_table", "mfx_plt_table_build", "mfx_cosmology_create", "mfx_cosmology_destroy",
    "mfx_cosmology_get", "mfx_cosmology_amplitude", "mfx_cosmology_transfer", "mfx_cosmology_growth",
    "mfx_cosmology_amp_table", "mfx_run_config", "mfx_job_set_output_ring", "mfx_job_fetch_particles_range_async",
    "mfx_job_wait_fetch",
]


class MfxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mfx error %d: %s" % (code, msg))
        self.code = code


class EngineOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_size_t)]


class JobDesc(C.Structure):
    _fields_ = [
        ("ngrid", C.c_uint32), ("boxlen", C.c_double), ("lpt_order", C.c_int), ("lattice", C.c_int),
        ("plt", C.c_int), ("precision", C.c_int), ("fixing", C.c_int), ("inversion", C.c_int),
        ("seed_table", C.c_void_p), ("amp_table", C.c_void_p), ("amp_table_len", C.c_size_t),
        ("plt_table", C.c_void_p),
        ("g1", C.c_double), ("g2", C.c_double), ("g3", C.c_double), ("g3c", C.c_double),
        ("vfac1", C.c_double), ("vfac2", C.c_double), ("vfac3", C.c_double),
        ("lunit", C.c_double), ("vunit", C.c_double),
        ("pos64", C.c_int), ("vel64", C.c_int), ("id64", C.c_int), ("id_offset", C.c_uint64),
        ("want_particles", C.c_int),
        ("noise_generator", C.c_int), ("music_seed", C.c_int64), ("music_cubesize", C.c_uint32),
        ("music_seeds", C.c_int64 * 12),
        ("noise_field", C.c_void_p),
        ("noise_field_res", C.c_uint32),
    ]


class SpeciesDesc(C.Structure):
    _fields_ = [("secondary_lattice", C.c_int), ("id_offset", C.c_uint64), ("c_species", C.c_double),
                ("mass_factor", C.c_double), ("amp_dbc", C.c_void_p), ("amp_tbc", C.c_void_p),
                ("amp_len", C.c_size_t), ("want_masses", C.c_int)]


_lib = None


def lib_path() -> pathlib.Path:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libmfx.so (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("libmfx.so not built (%s); run monofonic_gb300.build.build()" % p)
    L = C.CDLL(str(p))
    vp, sz, i32, u32, dbl = C.c_void_p, C.c_size_t, C.c_int, C.c_uint32, C.c_double
    L.mfx_last_error.argtypes = [C.c_char_p, sz]
    L.mfx_last_error.restype = sz
    L.mfx_version.restype = C.c_char_p
    L.mfx_engine_create.argtypes = [C.POINTER(EngineOpts), C.POINTER(vp)]
    L.mfx_engine_destroy.argtypes = [vp]
    L.mfx_job_footprint.argtypes = [vp, C.POINTER(JobDesc), C.POINTER(sz)]
    L.mfx_job_create.argtypes = [vp, C.POINTER(JobDesc), C.POINTER(vp)]
    L.mfx_job_upload.argtypes = [vp, C.POINTER(JobDesc)]
    L.mfx_job_run.argtypes = [vp]
    L.mfx_job_wait.argtypes = [vp, i32]
    L.mfx_job_fetch_particles.argtypes = [vp, vp, vp, vp]
    L.mfx_job_particles_device.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(sz)]
    L.mfx_job_fetch_field.argtypes = [vp, i32, vp]
    L.mfx_job_run_noise.argtypes = [vp, i32]
    L.mfx_job_stage_times.argtypes = [vp, C.POINTER(dbl), i32]
    L.mfx_job_algorithmic_bytes.argtypes = [vp, C.POINTER(dbl)]
    L.mfx_job_launch_count.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.mfx_job_set_profiling.argtypes = [vp, i32]
    L.mfx_job_kernel_profile.argtypes = [vp, i32, vp, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i32)]
    L.mfx_job_destroy.argtypes = [vp]
    L.mfx_job_capture.argtypes = [vp]
    L.mfx_batch_create.argtypes = [vp, C.POINTER(JobDesc), i32, C.POINTER(vp)]
    L.mfx_batch_run.argtypes = [vp]
    L.mfx_batch_wait.argtypes = [vp, C.POINTER(dbl)]
    L.mfx_batch_job.argtypes = [vp, i32, C.POINTER(vp)]
    L.mfx_batch_destroy.argtypes = [vp]
    L.mfx_noise_fill_noalloc.argtypes = [vp, u32, dbl, vp, i32, i32, i32, i32, vp, vp]
    L.mfx_debug_ranlxd1_words.argtypes = [vp, C.c_ulong, sz, vp]
    L.mfx_ngenic_seed_table.argtypes = [C.c_long, sz, vp]
    L.mfx_plt_table_build.argtypes = [vp, i32, vp]
    L.mfx_cosmology_create.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.mfx_cosmology_destroy.argtypes = [vp]
    L.mfx_cosmology_get.argtypes = [vp, C.c_char_p, C.POINTER(dbl)]
    L.mfx_cosmology_amplitude.argtypes = [vp, vp, sz, vp]
    L.mfx_cosmology_transfer.argtypes = [vp, vp, sz, vp]
    L.mfx_cosmology_growth.argtypes = [vp, dbl, C.POINTER(dbl)]
    L.mfx_cosmology_amp_table.argtypes = [vp, u32, dbl, vp, sz]
    L.mfx_run_config.argtypes = [vp, C.c_char_p]
    L.mfx_job_set_output_ring.argtypes = [vp, i32]
    L.mfx_job_fetch_particles_range_async.argtypes = [vp, sz, sz, vp, vp, vp]
    L.mfx_job_wait_fetch.argtypes = [vp]
    _lib = L
    return L


def last_error() -> str:
    L = load()
    buf = C.create_string_buffer(2048)
    L.mfx_last_error(buf, 2048)
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != MFX_OK:
        raise MfxError(rc, last_error())


# ----------------------------------------------------------------------------
# host-side plugin logic
# ----------------------------------------------------------------------------
def ngenic_seed_table(seed: int, n: int) -> np.ndarray:
    t = np.zeros(n * n, dtype=np.uint32)
    check(load().mfx_ngenic_seed_table(seed, n, t.ctypes.data))
    return t


class Cosmology:
    """cosmology::calculator + transfer plugin built from INI text."""

    def __init__(self, ini_text: str):
        self._h = C.c_void_p()
        check(load().mfx_cosmology_create(ini_text.encode(), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.mfx_cosmology_destroy(self._h)
            self._h = C.c_void_p()

    def get(self, name: str) -> float:
        v = C.c_double()
        check(load().mfx_cosmology_get(self._h, name.encode(), C.byref(v)))
        return v.value

    def amplitude(self, k) -> np.ndarray:
        k = np.ascontiguousarray(k, dtype=np.float64).ravel()
        out = np.zeros_like(k)
        check(load().mfx_cosmology_amplitude(self._h, k.ctypes.data, k.size, out.ctypes.data))
        return out

    def transfer(self, k) -> np.ndarray:
        k = np.ascontiguousarray(k, dtype=np.float64).ravel()
        out = np.zeros_like(k)
        check(load().mfx_cosmology_transfer(self._h, k.ctypes.data, k.size, out.ctypes.data))
        return out

    def growth(self, a: float) -> float:
        v = C.c_double()
        check(load().mfx_cosmology_growth(self._h, a, C.byref(v)))
        return v.value

    def amp_table(self, n: int, boxlen: float) -> np.ndarray:
        ln = 3 * (n // 2) ** 2 + 1
        t = np.zeros(ln)
        check(load().mfx_cosmology_amp_table(self._h, n, boxlen, t.ctypes.data, ln))
        return t


def ini_text(ngrid, boxlen, zstart, order, seed, lattice="sc", sigma8=0.81, omega_m=0.3, omega_b=0.045,
             h0=70.0, n_s=0.965, fixing=False, plt=False, precision="double", fmt="binary", filename="ics.bin",
             generator="NGENIC", cubesize=32):
    """INI text in monofonIC's config format for the configs this engine serves.
    generator="MUSIC1" gives the seed at the grid's level, seed[log2 ngrid]."""
    if generator == "MUSIC1":
        level = int(ngrid).bit_length() - 1
        rnd = f"generator = MUSIC1\nseed[{level}] = {seed}\ncubesize = {cubesize}"
    else:
        rnd = f"generator = {generator}\nseed = {seed}"
    return f"""[setup]
GridRes = {ngrid}
BoxLength = {boxlen}
zstart = {zstart}
LPTorder = {order}
ParticleLoad = {lattice}
DoFixing = {'yes' if fixing else 'no'}
DoPLT = {'yes' if plt else 'no'}
[cosmology]
ParameterSet = none
Omega_m = {omega_m}
Omega_b = {omega_b}
H0 = {h0}
n_s = {n_s}
sigma_8 = {sigma8}
transfer = eisenstein
ZeroRadiation = true
m_nu1 = 0
[random]
{rnd}
[execution]
Precision = {precision}
[output]
format = {fmt}
filename = {filename}
"""


# ----------------------------------------------------------------------------
# engine / jobs
# ----------------------------------------------------------------------------
class Engine:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self._h = C.c_void_p()
        opts = EngineOpts(device, hbm_budget_bytes)
        check(load().mfx_engine_create(C.byref(opts), C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h and self._h.value:
            load().mfx_engine_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def plt_table(self, lattice: int) -> np.ndarray:
        out = np.zeros(PLT_TABLE_DOUBLES)
        check(load().mfx_plt_table_build(self._h, lattice, out.ctypes.data))
        return out.reshape(4, 64, 64, 33)

    def ranlxd1_words(self, seed: int, count: int) -> np.ndarray:
        out = np.zeros(count, dtype=np.uint64)
        check(load().mfx_debug_ranlxd1_words(self._h, seed, count, out.ctypes.data))
        return out

    def run_config(self, text: str):
        check(load().mfx_run_config(self._h, text.encode()))


def lpt_coefficients(dplus: float, vfac: float, order: int) -> dict:
    """ic_generator.cc:252-269, evaluated in the reference's order (left to
    right, D+ * D+ * D+ rather than a power), so that the coefficients equal
    the reference's bit for bit"""
    return dict(g1=-dplus,
                g2=(-3.0 / 7.0 * dplus * dplus) if order > 1 else 0.0,
                g3=(1.0 / 3.0 * dplus * dplus * dplus) if order > 2 else 0.0,
                g3c=(1.0 / 7.0 * dplus * dplus * dplus) if order > 2 else 0.0,
                vfac1=vfac, vfac2=2 * vfac, vfac3=3 * vfac)


def _field_res(field) -> int:
    """Cells per axis of a cubic real-space noise field (0 for none)."""
    if field is None:
        return 0
    n = field.shape[0] if field.ndim == 3 else int(round(field.size ** (1.0 / 3.0)))
    if n ** 3 != field.size:
        raise ValueError("noise field of %d values is not a cube" % field.size)
    return n


class Job:
    """One IC job on the device (mfx_job_*)."""

    def __init__(self, engine: Engine, ngrid, boxlen, order, seed_table, amp_table, coef, lattice=SC,
                 precision=FP64, plt_table=None, fixing=False, inversion=False, lunit=1.0, vunit=1.0,
                 pos64=True, vel64=True, id64=True, id_offset=0, want_particles=True,
                 noise_generator=None, music_seed=0, music_cubesize=32, music_seeds=None, noise_field=None):
        """seed_table: NGenIC's per-column seeds; None with noise_generator=
        NOISE_MUSIC1, which draws the noise from music_seed (the seed at the
        grid's level) and music_cubesize, or from music_seeds {level: seed}
        given at coarser levels as well; noise_field: a real-space white-noise
        field [x][y][z] (NOISE_FIELD), e.g. MUSIC1's noise read from a file;
        a field coarser than the grid starts MUSIC1's refinement chain at its
        level, the finer levels from music_seeds."""
        self.engine = engine
        self.n = ngrid
        self.lattice = lattice
        self.precision = precision
        self.pos64, self.vel64, self.id64 = pos64, vel64, id64
        self._field = None if noise_field is None else np.ascontiguousarray(noise_field, dtype=np.float64)
        field_res = _field_res(self._field)
        if noise_generator is None:
            noise_generator = ((NOISE_FIELD if field_res == ngrid else NOISE_MUSIC1) if self._field is not None else
                               NOISE_NGENIC if seed_table is not None else NOISE_MUSIC1)
        self._seed = None if seed_table is None else np.ascontiguousarray(seed_table, dtype=np.uint32)
        self._amp = np.ascontiguousarray(amp_table, dtype=np.float64)
        self._plt = None if plt_table is None else np.ascontiguousarray(plt_table, dtype=np.float64)
        d = JobDesc()
        d.ngrid, d.boxlen, d.lpt_order, d.lattice = ngrid, boxlen, order, lattice
        d.plt = 1 if plt_table is not None else 0
        d.precision = precision
        d.fixing, d.inversion = int(fixing), int(inversion)
        d.seed_table = self._seed.ctypes.data if self._seed is not None else None
        d.noise_generator = noise_generator
        d.music_seed = music_seed
        d.music_cubesize = music_cubesize
        for level, sd in (music_seeds or {}).items():
            d.music_seeds[level] = sd
        d.noise_field = self._field.ctypes.data if self._field is not None else None
        d.noise_field_res = field_res if noise_generator == NOISE_MUSIC1 else 0
        d.amp_table = self._amp.ctypes.data
        d.amp_table_len = self._amp.size
        d.plt_table = self._plt.ctypes.data if self._plt is not None else None
        for k in ("g1", "g2", "g3", "g3c", "vfac1", "vfac2", "vfac3"):
            setattr(d, k, coef[k])
        d.lunit, d.vunit = lunit, vunit
        d.pos64, d.vel64, d.id64 = int(pos64), int(vel64), int(id64)
        d.id_offset = id_offset
        d.want_particles = int(want_particles)
        self.desc = d
        self._h = C.c_void_p()
        check(load().mfx_job_create(engine.handle, C.byref(d), C.byref(self._h)))
        self.num_particles = (1 << lattice) * ngrid ** 3

    def close(self):
        if self._h and self._h.value:
            load().mfx_job_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def upload(self, seed_table=None, amp_table=None, plt_table=None, music_seed=None, music_seeds=None):
        if seed_table is not None:
            np.copyto(self._seed, seed_table)
        if music_seed is not None:
            self.desc.music_seed = music_seed
        if music_seeds is not None:
            for level in range(12):
                self.desc.music_seeds[level] = music_seeds.get(level, 0)
        if amp_table is not None:
            np.copyto(self._amp, amp_table)
        if plt_table is not None and self._plt is not None:
            np.copyto(self._plt, plt_table)
        check(load().mfx_job_upload(self._h, C.byref(self.desc)))

    def run(self, wait=True):
        check(load().mfx_job_run(self._h))
        if wait:
            self.wait()

    def wait(self, timeout_ms=-1):
        check(load().mfx_job_wait(self._h, timeout_ms))

    def run_noise(self, raw=True):
        check(load().mfx_job_run_noise(self._h, 1 if raw else 0))
        self.wait()

    def field(self, fid: int) -> np.ndarray:
        n = self.n
        out = np.zeros((n, n, n // 2 + 1), dtype=np.complex128)
        check(load().mfx_job_fetch_field(self._h, fid, out.ctypes.data))
        return out

    def particles(self):
        npart = self.num_particles
        pos = np.zeros((npart, 3), dtype=np.float64 if self.pos64 else np.float32)
        vel = np.zeros((npart, 3), dtype=np.float64 if self.vel64 else np.float32)
        ids = np.zeros(npart, dtype=np.uint64 if self.id64 else np.uint32)
        check(load().mfx_job_fetch_particles(self._h, pos.ctypes.data, vel.ctypes.data, ids.ctypes.data))
        return pos, vel, ids

    def fetch_particles_into(self, pos, vel, ids):
        check(load().mfx_job_fetch_particles(self._h, pos, vel, ids))

    def set_tiles(self, pencils_xy: int, rows_z: int):
        """Pencil-tile shape of the fused transforms (what autotune() picks)."""
        L = load()
        L.mfx_job_set_tiles.argtypes = [C.c_void_p, C.c_int, C.c_int]
        check(L.mfx_job_set_tiles(self._h, int(pencils_xy), int(rows_z)))

    def assemble(self, orders_mask: int):
        """Re-assemble the particles from the last run's potentials with only the
        LPT orders in orders_mask (bit n-1: order n)."""
        L = load()
        L.mfx_job_assemble.argtypes = [C.c_void_p, C.c_int]
        check(L.mfx_job_assemble(self._h, int(orders_mask)))

    def fetch_particles_range_into(self, first: int, count: int, pos, vel, ids):
        """Copies particles [first, first + count) to host (or device) addresses."""
        L = load()
        L.mfx_job_fetch_particles_range.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p,
                                                    C.c_void_p]
        check(L.mfx_job_fetch_particles_range(self._h, first, count, pos, vel, ids))

    def set_output_ring(self, on=True):
        """Pipelined output: particle sets outside the arena, so that a run
        computes while the previous run's particles are still downloading.
        on: True = two sets, False = none, or the number of sets (0, 1, 2)."""
        sets = (2 if on else 0) if isinstance(on, bool) else int(on)
        check(load().mfx_job_set_output_ring(self._h, sets))

    def set_host_positions(self, on: bool = True):
        """Positions leave the device as float displacements; fetches into host
        memory form q + Psi in FP64 on the host (mfx_job_set_host_positions)."""
        L = load()
        L.mfx_job_set_host_positions.argtypes = [C.c_void_p, C.c_int]
        check(L.mfx_job_set_host_positions(self._h, int(on)))

    def set_species(self, secondary=False, id_offset=0, c_species=0.0, mass_factor=0.0, amp_dbc=None,
                    amp_tbc=None, want_masses=True, reset=False):
        """Species of the next assembly of a baryon + CDM run (mfx_job_set_species);
        reset=True restores the descriptor's single species."""
        L = load()
        L.mfx_job_set_species.argtypes = [C.c_void_p, C.c_void_p]
        if reset:
            check(L.mfx_job_set_species(self._h, None))
            return
        dbc = None if amp_dbc is None else np.ascontiguousarray(amp_dbc, dtype=np.float64)
        tbc = None if amp_tbc is None else np.ascontiguousarray(amp_tbc, dtype=np.float64)
        ln = len(dbc) if dbc is not None else (len(tbc) if tbc is not None else 0)
        sd = SpeciesDesc(int(secondary), int(id_offset), float(c_species), float(mass_factor),
                         dbc.ctypes.data if dbc is not None else None, tbc.ctypes.data if tbc is not None else None,
                         ln, int(want_masses))
        check(L.mfx_job_set_species(self._h, C.byref(sd)))

    def ppt_fields(self, c_species=0.0, amp_dbc=None):
        """Semiclassical (PPT) Eulerian density contrast and velocities of the
        last run's potentials (mfx_job_ppt_fields): (delta, (vx, vy, vz), hbar),
        each field N x N x N."""
        L = load()
        L.mfx_job_ppt_fields.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        n = self.n
        dbc = None if amp_dbc is None else np.ascontiguousarray(amp_dbc, dtype=np.float64)
        out = [np.zeros((n, n, n)) for _ in range(4)]
        hb = C.c_double()
        check(L.mfx_job_ppt_fields(self._h, float(c_species), dbc.ctypes.data if dbc is not None else None,
                                   len(dbc) if dbc is not None else 0, *[o.ctypes.data for o in out], C.byref(hb)))
        return out[0], tuple(out[1:]), hb.value

    def masses(self, first: int = 0, count=None) -> np.ndarray:
        """Particle masses of the last assembly with masses."""
        L = load()
        L.mfx_job_fetch_masses.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]
        count = self.num_particles - first if count is None else count
        out = np.zeros(count, dtype=np.float64 if self.pos64 else np.float32)
        check(L.mfx_job_fetch_masses(self._h, first, count, out.ctypes.data))
        return out

    def fetch_particles_range_async(self, first: int, count: int, pos, vel, ids):
        """Enqueues the download of particles [first, first + count) of the last
        run to page-locked host addresses and returns; wait_fetch() completes it."""
        check(load().mfx_job_fetch_particles_range_async(self._h, first, count, pos, vel, ids))

    def wait_fetch(self):
        check(load().mfx_job_wait_fetch(self._h))

    def particles_range(self, first: int, count: int):
        """Particles [first, first + count) as numpy arrays."""
        L = load()
        L.mfx_job_fetch_particles_range.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p,
                                                    C.c_void_p]
        pos = np.zeros((count, 3), dtype=np.float64 if self.pos64 else np.float32)
        vel = np.zeros((count, 3), dtype=np.float64 if self.vel64 else np.float32)
        ids = np.zeros(count, dtype=np.uint64 if self.id64 else np.uint32)
        check(L.mfx_job_fetch_particles_range(self._h, first, count, pos.ctypes.data, vel.ctypes.data,
                                              ids.ctypes.data))
        return pos, vel, ids

    def stage_times(self):
        ms = (C.c_double * 8)()
        n = load().mfx_job_stage_times(self._h, ms, 8)
        if n < 0:
            check(n)
        return list(ms)[:n]

    def algorithmic_bytes(self) -> float:
        b = C.c_double()
        check(load().mfx_job_algorithmic_bytes(self._h, C.byref(b)))
        return b.value

    def capture(self):
        """Record the pipeline into a CUDA graph; later run() calls replay it."""
        check(load().mfx_job_capture(self._h))

    def autotune(self):
        """Pick the fused transforms' pencil-tile shape; returns (pencils_xy, rows_z)."""
        L = load()
        L.mfx_job_autotune.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        a, b = C.c_int(), C.c_int()
        check(L.mfx_job_autotune(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_profiling(self, on=True):
        check(load().mfx_job_set_profiling(self._h, 1 if on else 0))

    def kernel_profile(self):
        """{name: (ms, algorithmic bytes, launches)} of the last run."""
        mx = 64
        names = C.create_string_buffer(32 * mx)
        ms, by, cnt = (C.c_double * mx)(), (C.c_double * mx)(), (C.c_int * mx)()
        n = load().mfx_job_kernel_profile(self._h, mx, names, ms, by, cnt)
        if n < 0:
            check(n)
        out = {}
        for q in range(min(n, mx)):
            nm = names.raw[32 * q:32 * q + 32].split(b"\0")[0].decode()
            out[nm] = (ms[q], by[q], cnt[q])
        return out

    def launch_count(self):
        a, b = C.c_int(), C.c_int()
        check(load().mfx_job_launch_count(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value


class _JobView(Job):
    """A job owned by a Batch (not destroyed by this wrapper)."""

    def __init__(self, handle, num_particles, pos64, vel64, id64, n):
        self._h = handle
        self.num_particles = num_particles
        self.pos64, self.vel64, self.id64 = pos64, vel64, id64
        self.n = n

    def close(self):
        self._h = C.c_void_p()


class Batch:
    """Ensemble of independent jobs run as one CUDA graph (mfx_batch_*)."""

    def __init__(self, engine: Engine, specs):
        """specs: list of dicts with the Job() keyword arguments
        (ngrid, boxlen, order, seed_table, amp_table, coef, lattice, precision, ...)."""
        self.engine = engine
        self._keep = []
        descs = (JobDesc * len(specs))()
        self._meta = []
        for q, sp in enumerate(specs):
            seed = np.ascontiguousarray(sp["seed_table"], dtype=np.uint32)
            amp = np.ascontiguousarray(sp["amp_table"], dtype=np.float64)
            plt = sp.get("plt_table")
            plt = None if plt is None else np.ascontiguousarray(plt, dtype=np.float64)
            self._keep += [seed, amp, plt]
            d = descs[q]
            d.ngrid, d.boxlen, d.lpt_order = sp["ngrid"], sp["boxlen"], sp["order"]
            d.lattice = sp.get("lattice", SC)
            d.plt = 1 if plt is not None else 0
            d.precision = sp.get("precision", FP64)
            d.fixing, d.inversion = int(sp.get("fixing", False)), int(sp.get("inversion", False))
            d.seed_table, d.amp_table, d.amp_table_len = seed.ctypes.data, amp.ctypes.data, amp.size
            d.plt_table = plt.ctypes.data if plt is not None else None
            for k in ("g1", "g2", "g3", "g3c", "vfac1", "vfac2", "vfac3"):
                setattr(d, k, sp["coef"][k])
            d.lunit, d.vunit = sp.get("lunit", 1.0), sp.get("vunit", 1.0)
            d.pos64, d.vel64, d.id64 = int(sp.get("pos64", True)), int(sp.get("vel64", True)), int(sp.get("id64", True))
            d.id_offset = sp.get("id_offset", 0)
            d.want_particles = int(sp.get("want_particles", True))
            self._meta.append(((1 << d.lattice) * d.ngrid ** 3, bool(d.pos64), bool(d.vel64), bool(d.id64), d.ngrid))
        self._descs = descs
        self._h = C.c_void_p()
        check(load().mfx_batch_create(engine.handle, descs, len(specs), C.byref(self._h)))
        self.count = len(specs)
        self.num_particles = sum(m[0] for m in self._meta)

    def run(self):
        check(load().mfx_batch_run(self._h))

    def wait(self) -> float:
        ms = C.c_double()
        check(load().mfx_batch_wait(self._h, C.byref(ms)))
        return ms.value

    def job(self, q: int) -> Job:
        h = C.c_void_p()
        check(load().mfx_batch_job(self._h, q, C.byref(h)))
        return _JobView(h, *self._meta[q])

    def close(self):
        if self._h and self._h.value:
            load().mfx_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def desc_from_spec(sp):
    """A job descriptor from a dict of Job() keyword arguments, and the arrays
    its pointers refer to (keep them alive while the descriptor is used)."""
    seed = sp.get("seed_table")
    seed = None if seed is None else np.ascontiguousarray(seed, dtype=np.uint32)
    amp = np.ascontiguousarray(sp["amp_table"], dtype=np.float64)
    plt = sp.get("plt_table")
    plt = None if plt is None else np.ascontiguousarray(plt, dtype=np.float64)
    d = JobDesc()
    d.ngrid, d.boxlen, d.lpt_order = sp["ngrid"], sp["boxlen"], sp["order"]
    d.lattice = sp.get("lattice", SC)
    d.plt = 1 if plt is not None else 0
    d.precision = sp.get("precision", FP64)
    d.fixing, d.inversion = int(sp.get("fixing", False)), int(sp.get("inversion", False))
    d.seed_table = seed.ctypes.data if seed is not None else None
    d.amp_table, d.amp_table_len = amp.ctypes.data, amp.size
    d.plt_table = plt.ctypes.data if plt is not None else None
    for k in ("g1", "g2", "g3", "g3c", "vfac1", "vfac2", "vfac3"):
        setattr(d, k, sp["coef"][k])
    d.lunit, d.vunit = sp.get("lunit", 1.0), sp.get("vunit", 1.0)
    d.pos64, d.vel64, d.id64 = int(sp.get("pos64", True)), int(sp.get("vel64", True)), int(sp.get("id64", True))
    d.id_offset = sp.get("id_offset", 0)
    d.want_particles = int(sp.get("want_particles", True))
    field = sp.get("noise_field")
    field = None if field is None else np.ascontiguousarray(field, dtype=np.float64)
    res = _field_res(field)
    d.noise_generator = sp.get("noise_generator", (NOISE_FIELD if res == sp["ngrid"] else NOISE_MUSIC1)
                               if field is not None else NOISE_NGENIC if seed is not None else NOISE_MUSIC1)
    d.noise_field = field.ctypes.data if field is not None else None
    d.noise_field_res = res if d.noise_generator == NOISE_MUSIC1 else 0
    d.music_seed, d.music_cubesize = sp.get("music_seed", 0), sp.get("music_cubesize", 32)
    for level, sd in (sp.get("music_seeds") or {}).items():
        d.music_seeds[level] = sd
    return d, (seed, amp, plt, field)


def footprint(engine, sp) -> int:
    """The HBM bytes a job of this spec takes (mfx_job_footprint)."""
    d, _keep = desc_from_spec(sp)
    fp = C.c_size_t()
    check(load().mfx_job_footprint(engine.handle, C.byref(d), C.byref(fp)))
    return fp.value


class Server:
    """Request loop with admission by HBM footprint (mfx_server_*)."""

    def __init__(self, engine: Engine, max_inflight: int = 8):
        L = load()
        L.mfx_server_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.mfx_server_submit.argtypes = [C.c_void_p, C.POINTER(JobDesc), C.POINTER(C.c_uint64)]
        L.mfx_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int]
        L.mfx_server_ticket_times.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.mfx_server_ticket_phases.argtypes = [C.c_void_p, C.c_uint64] + [C.POINTER(C.c_double)] * 3
        L.mfx_server_job.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]
        L.mfx_server_release.argtypes = [C.c_void_p, C.c_uint64]
        L.mfx_server_destroy.argtypes = [C.c_void_p]
        self.engine = engine
        self._h = C.c_void_p()
        check(L.mfx_server_create(engine.handle, max_inflight, C.byref(self._h)))
        self._meta = {}

    def submit(self, sp) -> int:
        """sp: dict of Job() keyword arguments (see Batch)."""
        d, _keep = desc_from_spec(sp)
        t = C.c_uint64()
        check(load().mfx_server_submit(self._h, C.byref(d), C.byref(t)))
        self._meta[t.value] = ((1 << d.lattice) * d.ngrid ** 3, bool(d.pos64), bool(d.vel64), bool(d.id64), d.ngrid)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        check(load().mfx_server_wait(self._h, ticket, timeout_ms))

    def set_policy(self, bypass: bool = True, bypass_age_ms: float = 100.0, size_priority: bool = True,
                   largest_first: bool = False, small_first: bool = True):
        """Admission order: a later job that fits may pass a head that has
        waited at most bypass_age_ms (bypass), or strict first-in first-out;
        largest_first: while the head may be passed, the largest queued job
        that fits goes first; size_priority: stream priority by footprint,
        the smallest jobs highest (small_first) or the largest."""
        L = load()
        L.mfx_server_set_policy.argtypes = [C.c_void_p, C.c_int, C.c_double]
        flags = (int(bool(bypass)) | (0 if size_priority else 2) | (4 if largest_first else 0)
                 | (0 if small_first else 8))
        check(L.mfx_server_set_policy(self._h, flags, float(bypass_age_ms)))

    def times(self, ticket: int):
        q, l = C.c_double(), C.c_double()
        check(load().mfx_server_ticket_times(self._h, ticket, C.byref(q), C.byref(l)))
        return q.value, l.value

    def set_small_jobs(self, footprint_bytes: int, max_small: int = 16):
        """Admit jobs with footprint <= footprint_bytes beside the in-flight
        slots, at most max_small at once (0 turns it off)."""
        L = load()
        L.mfx_server_set_small_jobs.argtypes = [C.c_void_p, C.c_size_t, C.c_int]
        check(L.mfx_server_set_small_jobs(self._h, int(footprint_bytes), int(max_small)))

    def phases(self, ticket: int):
        """(queued, set-up, run) ms of a finished ticket."""
        q, su, r = C.c_double(), C.c_double(), C.c_double()
        check(load().mfx_server_ticket_phases(self._h, ticket, C.byref(q), C.byref(su), C.byref(r)))
        return q.value, su.value, r.value

    def job(self, ticket: int) -> Job:
        h = C.c_void_p()
        check(load().mfx_server_job(self._h, ticket, C.byref(h)))
        return _JobView(h, *self._meta[ticket])

    def release(self, ticket: int):
        check(load().mfx_server_release(self._h, ticket))
        self._meta.pop(ticket, None)

    def close(self):
        if self._h and self._h.value:
            load().mfx_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

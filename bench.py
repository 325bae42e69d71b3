"""Benchmark of the LPT initial-condition hot path on GB300.

Default workload (one GPU): 3LPT + PLT on an FCC lattice, 768^3 grid (padded
convolutions at 1152^3), 4 x 768^3 = 1.81e9 particles, box 1000 Mpc/h,
z_start = 24, amplitude-fixed NGenIC white noise (seed 1), E&H transfer
function (Omega_m 0.3, Omega_b 0.045, h 0.7, sigma_8 0.81, n_s 0.965),
FP32-compensated form.  One step = one full pass of the hot path (white noise
-> phi1/phi2/phi3/A3 -> displacements/velocities -> particles).  ``--workload
bcc256`` runs the 3LPT + PLT BCC 256^3 configuration instead.

  value  particles/s with all inputs resident in HBM (device time, CUDA events
         on the engine's stream, L2 flushed between steps)
  e2e    the same through the C ABI with host buffers: every step uploads the
         seed / amplitude / PLT tables from pinned host memory and copies the
         particles (f64 positions, f32 velocities) back to pinned host memory
         (ids written on the host)
  fp64_form  the plain FP64 form of the same workload, for the FP32/FP64 ratio,
         with its FFT throughput against GB300's FP64 rate
  roofline   the dominant own kernel against the measured HBM copy bandwidth

``--impl reference`` times the C++/OpenMP restatement of the reference's CPU
path (oracle/lpt_omp.cc: the reference's loop structure and its 99 padded
FFTs per 3LPT run, with an own FFT instead of FFTW; the reference itself
cannot be built: it needs FFTW3, GSL and HDF5) with all host cores, on a
bounded sample of the same workload's physics (a smaller grid, throughput
per particle).

Multi-GPU (torchrun): independent replicas, one realisation per rank (seed +
rank), no data-path collective; value = all ranks' particles / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (ngrid, boxlen, zstart, order, lattice, plt, seed, fixing)
    "bcc256": (256, 300.0, 24.0, 3, 1, True, 4242, False),
    "sc64": (64, 100.0, 49.0, 2, 0, False, 12345, False),
    "fcc768": (768, 1000.0, 24.0, 3, 2, True, 1, True),
    "fcc384": (384, 1000.0, 24.0, 3, 2, True, 1, True),
    # the 768^3 FCC physics at 512^3 (L scaled): the padded length 768 between 576 and 1152
    "fcc512": (512, 666.6666666666666, 24.0, 3, 2, True, 1, True),
    # the 256^3 BCC physics at 128^3 (L scaled): profiling captures of every kernel
    "bcc128": (128, 150.0, 24.0, 3, 1, True, 4242, False),
}
LATNAME = {0: "sc", 1: "bcc", 2: "fcc"}
# grid of the CPU restatement's timed sample: once in our own line's
# cpu_baseline, and per step in the reference arm (bounded so that the whole
# --steps/--warmup run stays within a few minutes)
CPU_SAMPLE = {"fcc768": 384, "fcc512": 256, "fcc384": 384, "bcc256": 256, "bcc128": 128, "sc64": 64}
REF_SAMPLE = {"fcc768": 192, "fcc512": 192, "fcc384": 192, "bcc256": 256, "bcc128": 128, "sc64": 64}
# GB300 FP64 (non-tensor) arithmetic rate, NVIDIA's published figure (FLOP/s):
# the ceiling of the plain FP64 form's cuFFT transforms
FP64_PEAK_SPEC = 1.25e12


def describe(name, prec):
    n, L, z, order, lat, plt, seed, fix = WORKLOADS[name]
    return {"workload": "%dLPT%s %s %d^3 L=%g Mpc/h z=%g seed %d %s" % (
        order, "+PLT" if plt else "", LATNAME[lat].upper(), n, L, z, seed, prec),
        "ngrid": n, "boxlen": L, "zstart": z, "lpt_order": order, "lattice": LATNAME[lat], "plt": plt,
        "seed": seed, "fixing": fix, "particles": (1 << lat) * n ** 3, "precision": prec,
        "cosmology": "Om=0.3 Ob=0.045 h=0.7 s8=0.81 ns=0.965 E&H", "l2_flush": True}


def metric_name(name, prec):
    n, L, z, order, lat, plt, seed, fix = WORKLOADS[name]
    return "%dLPT particles/s (%s form) on 1 GB300, %dLPT%s %s %d^3" % (
        order, "FP32-compensated" if prec == "fp32c" else "plain FP64", order, "+PLT" if plt else "",
        LATNAME[lat].upper(), n)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_throughput(local_ms, local_particles, device="cpu"):
    """Replicas only: every rank runs its own realisation; the job's time is the
    slowest rank's and the throughput counts every rank's particles.  Returns
    (max ms over ranks, total particles / that time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_ms, local_particles / (local_ms * 1e-3)
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(local_particles)], dtype=torch.float64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), float(n.item()) / (float(t.item()) * 1e-3)


_T0 = time.perf_counter()


def progress(msg):
    """Phase markers with elapsed seconds, on stderr (the JSON line is stdout)."""
    print("[bench %7.1f s] %s" % (time.perf_counter() - _T0, msg), file=sys.stderr, flush=True)


_CLOCK_DIR = None


def clock_csv(name):
    """Path for an nvidia-smi sample file, in a per-process temporary directory."""
    global _CLOCK_DIR
    if _CLOCK_DIR is None:
        import tempfile
        _CLOCK_DIR = tempfile.mkdtemp(prefix="mfx_bench_clocks_")
    return os.path.join(_CLOCK_DIR, name)


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self, index, path):
        self.path = path
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(mfx, name, rank=0):
    n, L, z, order, lat, plt, seed, fix = WORKLOADS[name]
    seed = seed + rank
    cosmo = mfx.Cosmology(mfx.ini_text(n, L, z, order, seed, LATNAME[lat], fixing=fix, plt=plt))
    dplus, vfac = cosmo.get("dplus_start"), cosmo.get("vfact_start")
    coef = mfx.lpt_coefficients(dplus, vfac, order)
    seeds = mfx.ngenic_seed_table(seed, n)
    amp = cosmo.amp_table(n, L)
    return dict(n=n, L=L, z=z, order=order, lat=lat, plt=plt, fix=fix, seed=seed, cosmo=cosmo, coef=coef,
                seeds=seeds, amp=amp, lunit=L, vunit=L / np.sqrt(1.0 / (1.0 + z)))


def pinned(nbytes):
    import torch
    t = torch.empty(max(1, nbytes), dtype=torch.uint8, pin_memory=True)
    return t, t.numpy()


def l2_flush(buf):
    buf.add_(1.0)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from monofonic_gb300 import mfx

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    mfx.load(build_if_missing=True)
    eng = mfx.Engine(local)
    inp = make_inputs(mfx, args.workload, rank)
    prec = mfx.FP32C if args.precision == "fp32c" else mfx.FP64
    plt_tab = eng.plt_table(inp["lat"]) if inp["plt"] else None
    # pinned host copies of the per-step inputs (uploaded every e2e step)
    hs_t, hs = pinned(inp["seeds"].nbytes)
    hs = hs[:inp["seeds"].nbytes].view(np.uint32)
    hs[:] = inp["seeds"]
    ha_t, ha = pinned(inp["amp"].nbytes)
    ha = ha[:inp["amp"].nbytes].view(np.float64)
    ha[:] = inp["amp"]
    hp = None
    if plt_tab is not None:
        hp_t, hp = pinned(plt_tab.nbytes)
        hp = hp[:plt_tab.nbytes].view(np.float64).reshape(plt_tab.shape)
        hp[:] = plt_tab
    pos64, vel64 = True, (prec == mfx.FP64)
    job = mfx.Job(eng, inp["n"], inp["L"], inp["order"], hs, ha, inp["coef"], lattice=inp["lat"], precision=prec,
                  plt_table=hp, fixing=inp["fix"], lunit=inp["lunit"], vunit=inp["vunit"], pos64=pos64,
                  vel64=vel64, id64=True)
    npart = job.num_particles
    tiles = None
    if prec == mfx.FP32C:
        if args.tiles:  # fixed pencil tiles (profiling runs), else the autotuner's (untimed)
            tiles = tuple(int(x) for x in args.tiles.split(","))
            job.set_tiles(*tiles)
        else:
            tiles = job.autotune()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    progress("job created, tiles %s; warm-up" % (tiles,))
    for _ in range(args.warmup):
        job.run()
    progress("timed device steps")
    job.set_profiling(True)
    barrier()
    clocks = Clocks(local, clock_csv("clocks_rank%d.csv" % rank)) if rank == 0 else None
    dev_ms, prof_tot = [], {}
    t0 = time.perf_counter()
    for _ in range(args.steps):
        l2_flush(flush)
        torch.cuda.synchronize()
        job.run()
        dev_ms.append(sum(job.stage_times()))
        for k, (ms, by, cnt) in job.kernel_profile().items():
            a = prof_tot.setdefault(k, [0.0, 0.0, 0])
            a[0] += ms
            a[1] += by
            a[2] += cnt
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop() if clocks else None
    own, ffts = job.launch_count()
    job.set_profiling(False)
    ms_step, value = replica_throughput(float(np.mean(dev_ms)), npart, device="cuda")

    if args.no_e2e:  # profiling runs: the device-timed steps and the kernel table only
        job.close()
        kern = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[2] / args.steps,
                    "alg_GBps": (v[1] / (v[0] * 1e-3) / 1e9) if v[0] > 0 else None, "share": None}
                for k, v in prof_tot.items()}
        return {"profiling_run": True, "workload": args.workload, "value": value, "ms_per_step": ms_step,
                "kernels": kern, "clocks": clk, "fused_tiles": list(tiles) if tiles else None}, None, inp, plt_tab
    # ---- e2e through the C ABI with host buffers ----
    # the FP32 form keeps float displacements on the device and forms q + Psi
    # in FP64 on the host (mfx_job_set_host_positions: the same doubles), so a
    # particle crosses the host link in 12 + 12 bytes instead of 24 + 12
    host_pos = False
    if prec == mfx.FP32C and args.host_positions:
        try:
            job.set_host_positions(True)
            host_pos = True
        except RuntimeError:
            host_pos = False
    # particles come back in chunks of at most 128M (a bounded pinned buffer),
    # the way an output plugin drains them
    chunk = min(npart, 1 << 27)
    pb_t, pb = pinned(chunk * 3 * 8)
    vb_t, vb = pinned(chunk * 3 * (8 if vel64 else 4))
    ib_t, ib = pinned(chunk * 8)
    h2d = hs.nbytes + ha.nbytes + (hp.nbytes if hp is not None else 0)
    # positions and velocities cross the host link; the ids (a closed form of the
    # particle index) are written into the host buffer by the fetch's host threads
    d2h = npart * (3 * (4 if host_pos else 8) + 3 * (8 if vel64 else 4))

    def fetch_all():
        for first in range(0, npart, chunk):
            job.fetch_particles_range_into(first, min(chunk, npart - first), pb.ctypes.data, vb.ctypes.data,
                                           ib.ctypes.data)

    progress("end to end, one step at a time")
    job.upload(hs, ha, hp)
    job.run()
    fetch_all()
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        l2_flush(flush)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        job.upload(hs, ha, hp)
        job.run(wait=False)
        fetch_all()
        e2e_t.append(time.perf_counter() - t1)
    barrier()
    e2e_ms, e2e_val = replica_throughput(float(np.mean(e2e_t)) * 1e3, npart, device="cuda")
    e2e_serial = {"value": e2e_val, "unit": "particles/s", "ms_per_step": e2e_ms,
                  "mode": "one step at a time: upload, run, download, next step"}
    e2e = dict(e2e_serial)
    # pipelined output (mfx_job_set_output_ring): with two particle sets on the
    # device a step computes while the previous step's particles download (the
    # host link, ~190 GB/s, then bounds the step rather than adding to it);
    # where two sets do not fit beside the fields (768^3), one set: the next
    # step's noise and potentials overlap the download and only its assembly
    # waits for it.  Every step still uploads its inputs and downloads all its
    # particles into page-locked host memory (two host sets alternating, or
    # one reused: a step's download starts after the previous one has ended);
    # no L2 flush is needed between steps: each step's inputs come from the
    # host and its HBM traffic (17 GB at 256^3) is far above the 129 MB L2.
    host_set = npart * (3 * 8 + 3 * (8 if vel64 else 4) + 8)  # f64 positions, velocities, ids
    ring = 0
    # one page-locked host set serves one or two device sets: a step's copies
    # go on the copy stream after the previous step's, and a fetch joins the
    # previous fetch's host threads before it starts its own
    for sets, host_sets in ((2, 1), (1, 1)):
        if host_sets * host_set > (100 << 30):
            continue
        try:
            job.set_output_ring(sets)
            ring = sets
            break
        except RuntimeError:
            continue
    progress("end to end, pipelined with %d device set(s)" % ring)
    modes = {}
    if ring:
        nh = host_sets
        host = [(pinned(npart * 3 * 8), pinned(npart * 3 * (8 if vel64 else 4)), pinned(npart * 8)) for _ in range(nh)]
        hsets = [tuple(x[1] for x in st) for st in host]  # numpy views; `host` keeps the tensors alive

        def step(k):
            job.upload(hs, ha, hp)
            job.run(wait=False)
            p, v, i = hsets[k % nh]
            job.fetch_particles_range_async(0, npart, p.ctypes.data, v.ctypes.data, i.ctypes.data)

        def pipelined():
            for k in range(2):
                step(k)
            job.wait()
            job.wait_fetch()
            barrier()
            t1 = time.perf_counter()
            for k in range(args.steps):
                step(k)
            job.wait()
            job.wait_fetch()
            barrier()
            return replica_throughput((time.perf_counter() - t1) * 1e3 / args.steps, npart, device="cuda")

        mode = ("pipelined: step k+1 computes while step k's particles download (output ring of two sets)"
                if ring == 2 else
                "pipelined: step k+1's noise and potentials run while step k's particles download "
                "(output ring of one set; its assembly waits for the download)")
        e2e_ms, e2e_val = pipelined()
        modes["device_positions"] = {"value": e2e_val, "ms_per_step": e2e_ms, "d2h_bytes_per_step": int(d2h),
                                     "device_sets": ring}
        e2e = {"value": e2e_val, "unit": "particles/s", "ms_per_step": e2e_ms, "mode": mode}
        # the other output form of the same public API: float displacements
        # cross the host link and the fetch's host threads form q + Psi in FP64
        # (the same doubles).  Which is faster depends on the machine's host link
        # against its host memory bandwidth; the line reports the faster.
        if prec == mfx.FP32C and not host_pos:
            try:
                job.set_output_ring(0)
                job.set_host_positions(True)
                # float displacements make a device set smaller: two may fit
                # where only one did
                ring2 = 0
                for nsets in (2, 1):
                    try:
                        job.set_output_ring(nsets)
                        ring2 = nsets
                        break
                    except RuntimeError:
                        continue
                if ring2:
                    progress("end to end, pipelined with %d device set(s), positions formed on the host" % ring2)
                    ms2, val2 = pipelined()
                    d2h2 = npart * (3 * 4 + 3 * (8 if vel64 else 4))
                    modes["host_positions"] = {"value": val2, "ms_per_step": ms2, "d2h_bytes_per_step": int(d2h2),
                                               "device_sets": ring2}
                    if val2 > e2e_val:
                        mode2 = ("pipelined: step k+1 computes while step k's particles download "
                                 "(output ring of two sets)" if ring2 == 2 else mode)
                        e2e = {"value": val2, "unit": "particles/s", "ms_per_step": ms2, "mode": mode2}
                        host_pos, d2h = True, d2h2
                job.set_output_ring(0)
                job.set_host_positions(False)
            except RuntimeError:
                pass
        job.set_output_ring(0)
    e2e.update({"h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ids": "written into the host buffers by the fetch (host threads, beside the copies)",
                "positions": ("float displacements copied, q + Psi formed in FP64 by the fetch's host threads"
                              if host_pos else "FP64 positions copied")})
    if ring:
        e2e["serial"] = e2e_serial
    if modes:
        e2e["output_forms"] = modes

    out = None
    if rank == 0:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        peak = peaks.get("hbm_gbs", 6800.0)
        peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
        steps = args.steps
        kern = {k: {"ms_per_step": v[0] / steps, "launches_per_step": v[2] / steps,
                    "alg_GBps": (v[1] / (v[0] * 1e-3) / 1e9) if v[0] > 0 else None}
                for k, v in prof_tot.items()}
        total_k = sum(v[0] for v in prof_tot.values())
        for k in kern:
            kern[k]["share"] = prof_tot[k][0] / total_k if total_k else None
        own_only = {k: v for k, v in prof_tot.items() if not k.startswith("cufft")}
        dom = max(own_only, key=lambda k: own_only[k][0])
        d = prof_tot[dom]
        achieved = d[1] / (d[0] * 1e-3) / 1e9
        traffic = None
        tfile = ROOT / "profiles" / "traffic.json"
        if tfile.exists():
            tj = json.loads(tfile.read_text())
            traffic = tj.get(args.workload + "/" + args.precision, {}).get(dom)
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else "fallback",
                "traffic": traffic, "alg_bytes_per_launch": d[1] / d[2], "launches": d[2]}
        fft = {k: v for k, v in prof_tot.items() if k.startswith("cufft")}
        fft_ms = sum(v[0] for v in fft.values())
        fft_bytes = sum(v[1] for v in fft.values())
        alg_total = job.algorithmic_bytes()
        out = {
            "metric": metric_name(args.workload, args.precision),
            "value": value, "unit": "particles/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == mfx.FP32C else "f64", "data": "synthetic (NGenIC white noise, seeded)",
            "config": describe(args.workload, args.precision),
            "e2e": e2e, "gpu_launches": int(own) * args.steps, "fft_execs_per_step": int(ffts),
            "roofline": roof,
            "fft_roofline": {"achieved": fft_bytes / (fft_ms * 1e-3) / 1e9 if fft_ms else None, "peak": peak,
                             "unit": "GB/s", "share_of_step": fft_ms / total_k if total_k else None},
            "whole_step_alg": {"bytes": alg_total, "achieved_GBps": alg_total / (ms_step * 1e-3) / 1e9,
                               "frac": alg_total / (ms_step * 1e-3) / 1e9 / peak},
            "kernels": kern, "clocks": clk, "wall_s_timed": wall,
            "fused_tiles": {"pencils_xy": tiles[0], "rows_z": tiles[1]} if tiles else None,
        }
    job.close()
    return out, eng, inp, plt_tab


def ensemble_manifest():
    """64 independent 2LPT realisations: 32 x 128^3 (seeds 1-32), 24 x 192^3
    (33-56), 8 x 256^3 (57-64); boxes U[50,500] Mpc/h and sigma_8 U[0.7,0.9]
    from numpy.random.default_rng(20261203); SC, z = 49."""
    rng = np.random.default_rng(20261203)
    boxes = rng.uniform(50.0, 500.0, size=64)
    s8 = rng.uniform(0.7, 0.9, size=64)
    sizes = [128] * 32 + [192] * 24 + [256] * 8
    return [dict(seed=q + 1, ngrid=sizes[q], boxlen=float(boxes[q]), sigma8=float(s8[q]), zstart=49.0, order=2,
                 lattice="sc") for q in range(64)]


def run_ensemble(args):
    """Config 4: the 64-realisation ensemble as one captured CUDA graph."""
    import torch
    from monofonic_gb300 import mfx
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    mfx.load(build_if_missing=True)
    eng = mfx.Engine(local)
    man = ensemble_manifest()
    prec = mfx.FP32C if args.precision == "fp32c" else mfx.FP64
    specs = []
    host_bytes = 0
    for m in man:
        c = mfx.Cosmology(mfx.ini_text(m["ngrid"], m["boxlen"], m["zstart"], m["order"], m["seed"] + 1000 * rank,
                                       m["lattice"], sigma8=m["sigma8"]))
        sp = dict(ngrid=m["ngrid"], boxlen=m["boxlen"], order=m["order"],
                  seed_table=mfx.ngenic_seed_table(m["seed"] + 1000 * rank, m["ngrid"]),
                  amp_table=c.amp_table(m["ngrid"], m["boxlen"]),
                  coef=mfx.lpt_coefficients(c.get("dplus_start"), c.get("vfact_start"), m["order"]),
                  lattice=mfx.SC, precision=prec, lunit=m["boxlen"],
                  vunit=m["boxlen"] / np.sqrt(1.0 / (1.0 + m["zstart"])), pos64=True, vel64=(prec == mfx.FP64),
                  id64=True)
        host_bytes += sp["seed_table"].nbytes + sp["amp_table"].nbytes
        specs.append(sp)
    # the autotuner picks the fused transforms' tiles once per size class (the
    # engine keeps them for every later job of that size), before the capture
    t0 = time.perf_counter()
    tuned = {}
    if prec == mfx.FP32C:
        for sp in specs:
            if sp["ngrid"] in tuned:
                continue
            j = mfx.Job(eng, sp["ngrid"], sp["boxlen"], sp["order"], sp["seed_table"], sp["amp_table"], sp["coef"],
                        lattice=sp["lattice"], precision=prec, lunit=sp["lunit"], vunit=sp["vunit"],
                        pos64=sp["pos64"], vel64=sp["vel64"], id64=sp["id64"])
            tuned[sp["ngrid"]] = list(j.autotune())
            j.close()
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = mfx.Batch(eng, specs)
    setup_s = time.perf_counter() - t0
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        batch.run()
        batch.wait()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local, clock_csv("clocks_ensemble.csv")) if rank == 0 else None
    ms = []
    for _ in range(args.steps):
        l2_flush(flush)
        torch.cuda.synchronize()
        batch.run()
        ms.append(batch.wait())
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    ms_step = float(np.mean(ms))
    npart = batch.num_particles
    # e2e: upload every job's tables from pinned host memory, run the graph,
    # copy every job's particles back to pinned host memory
    jobs = [batch.job(q) for q in range(batch.count)]
    pin = []
    for q, sp in enumerate(specs):
        tt, st = pinned(sp["seed_table"].nbytes)
        st = st[:sp["seed_table"].nbytes].view(np.uint32)
        st[:] = sp["seed_table"]
        ta, at = pinned(sp["amp_table"].nbytes)
        at = at[:sp["amp_table"].nbytes].view(np.float64)
        at[:] = sp["amp_table"]
        n = jobs[q].num_particles
        tp, pb = pinned(n * 24)
        tv, vb = pinned(n * (8 if prec == mfx.FP64 else 4) * 3)
        ti, ib = pinned(n * 8)
        d = batch._descs[q]
        d.seed_table, d.amp_table = st.ctypes.data, at.ctypes.data
        pin.append((tt, ta, tp, tv, ti, pb, vb, ib, d))
    d2h = sum(p[5].nbytes + p[6].nbytes for p in pin)  # ids are written on the host by the fetch
    e2e_t = []
    for s in range(args.steps + 1):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for q, p in enumerate(pin):
            mfx.check(mfx.load().mfx_job_upload(jobs[q].handle, mfx.C.byref(p[8])))
        torch.cuda.synchronize()
        batch.run()
        batch.wait()
        for q, p in enumerate(pin):
            jobs[q].fetch_particles_into(p[5].ctypes.data, p[6].ctypes.data, p[7].ctypes.data)
        if s > 0:
            e2e_t.append(time.perf_counter() - t1)
    e2e_s = float(np.mean(e2e_t))
    out = {
        "metric": "ensemble particles/s (64 x 2LPT SC, 128^3/192^3/256^3, one CUDA graph)",
        "value": world * npart / (ms_step * 1e-3), "unit": "particles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == mfx.FP32C else "f64",
        "data": "synthetic (NGenIC white noise, seeds 1-64; boxes and sigma_8 from default_rng(20261203))",
        "config": {"workload": "ensemble64: 32x128^3 + 24x192^3 + 8x256^3, 2LPT SC z=49, " + args.precision,
                   "realisations": 64, "particles": npart, "l2_flush": True, "graph_setup_s": setup_s,
                   "autotune_s": tune_s, "tiles_per_size": {str(k): v for k, v in tuned.items()}},
        "e2e": {"value": world * npart / e2e_s, "unit": "particles/s", "h2d_bytes_per_step": int(host_bytes),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3},
        "clocks": clk,
    }
    batch.close()
    return out


def serving_requests(count, rng_seed=7):
    """Config 5 request mix: N ~ U{64,128,192,256,384}, LPT order ~ U{1,2,3},
    lattice ~ U{SC,BCC,FCC} (PLT on for BCC/FCC), sequential seeds, drawn from
    numpy.random.default_rng(7); box scaled with N (300 Mpc/h at 256^3), z = 24."""
    rng = np.random.default_rng(rng_seed)
    out = []
    for q in range(count):
        n = int(rng.choice([64, 128, 192, 256, 384]))
        order = int(rng.integers(1, 4))
        lat = int(rng.integers(0, 3))
        out.append(dict(seed=q + 1, ngrid=n, order=order, lattice=lat, plt=lat != 0, boxlen=300.0 * n / 256,
                        zstart=24.0))
    return out


def drain(srv, tickets, parts, stop_when_all=True):
    """Client loop: polls the outstanding tickets, releases each result as soon
    as it is done (results hold HBM until released) and returns the latencies
    (ms, submit -> done as the server measured them) and completed particles."""
    lat, done_parts = [], 0
    pending = dict(tickets)
    while pending:
        for tk in list(pending):
            try:
                srv.wait(tk, 0)
            except Exception:
                continue
            lat.append(srv.times(tk)[1])
            done_parts += pending.pop(tk)
            srv.release(tk)
        time.sleep(0.0005)
    return lat, done_parts


def run_serving(args):
    """Config 5: Poisson arrivals into the serving loop at offered loads from
    0.5 to 1.1 of the batched rate (every request queued at once), >= 500
    requests per point; p50/p99 latency per point, and the highest throughput
    whose p99 meets the stated target, as a fraction of the batched
    throughput; the plain FP64 form run serially on a sample of the requests."""
    import threading
    import torch
    from monofonic_gb300 import mfx
    torch.cuda.set_device(0)
    mfx.load(build_if_missing=True)
    eng = mfx.Engine(0)
    reqs = serving_requests(args.requests)
    plt = {lat: eng.plt_table(lat) for lat in (1, 2)}
    cos, amps = {}, {}
    specs = []
    for r in reqs:
        key = (r["ngrid"], r["order"])
        if key not in cos:
            cos[key] = mfx.Cosmology(mfx.ini_text(r["ngrid"], r["boxlen"], r["zstart"], r["order"], 1))
        c = cos[key]
        if key not in amps:
            amps[key] = c.amp_table(r["ngrid"], r["boxlen"])
        specs.append(dict(ngrid=r["ngrid"], boxlen=r["boxlen"], order=r["order"],
                          seed_table=mfx.ngenic_seed_table(r["seed"], r["ngrid"]), amp_table=amps[key],
                          coef=mfx.lpt_coefficients(c.get("dplus_start"), c.get("vfact_start"), r["order"]),
                          lattice=r["lattice"], plt_table=plt.get(r["lattice"]), precision=mfx.FP32C,
                          lunit=r["boxlen"], vunit=r["boxlen"] / np.sqrt(1.0 / (1.0 + r["zstart"])),
                          pos64=True, vel64=False, id64=True))
    parts = [(1 << s["lattice"]) * s["ngrid"] ** 3 for s in specs]
    # the autotuner picks the fused transforms' tiles once per size class at
    # start-up (the engine keeps them for the jobs the server creates)
    tuned = {}
    for s in sorted(specs, key=lambda s: -s["order"]):
        if s["ngrid"] in tuned or s["order"] < 2:
            continue
        j = mfx.Job(eng, s["ngrid"], s["boxlen"], s["order"], s["seed_table"], s["amp_table"], s["coef"],
                    lattice=s["lattice"], precision=mfx.FP32C, plt_table=s["plt_table"], lunit=s["lunit"],
                    vunit=s["vunit"], pos64=True, vel64=False, id64=True)
        tuned[s["ngrid"]] = list(j.autotune())
        j.close()
    srv = mfx.Server(eng, max_inflight=args.inflight)
    srv.set_policy(bypass=True, bypass_age_ms=args.bypass_age_ms, size_priority=not args.no_priority,
                   largest_first=args.largest_first, small_first=not args.large_priority)
    if args.small_gb > 0:
        srv.set_small_jobs(int(args.small_gb * 2 ** 30), args.max_small)
    # warm the plan pool and the memory pool with one pass over the size classes
    warm = {}
    for s in specs:
        warm.setdefault((s["ngrid"], s["order"], s["lattice"]), s)
    drain(srv, {srv.submit(s): 0 for s in warm.values()}, parts)
    # each size class alone through the server (submit -> done, nothing else
    # queued or running): the latency floor of the sweep's percentiles
    alone_ms, footprint_mb = {}, {}
    for key, s in sorted(warm.items()):
        lat1, _ = drain(srv, {srv.submit(s): 0}, parts)
        name = "%d/%d/%s" % (key[0], key[1], "sc bcc fcc".split()[key[2]])
        alone_ms[name] = float(lat1[0])
        footprint_mb[name] = mfx.footprint(eng, s) / 2 ** 20

    # batched: every request queued at once
    t0 = time.perf_counter()
    tk = {srv.submit(s): parts[q] for q, s in enumerate(specs)}
    sat_lat, _ = drain(srv, tk, parts)
    sat_span = time.perf_counter() - t0
    sat_tput = sum(parts) / sat_span
    sat_rate = len(specs) / sat_span

    def offered(load, rng_seed):
        rate = load * sat_rate
        gaps = np.random.default_rng(rng_seed).exponential(1.0 / rate, size=len(specs))
        tickets = {}
        lock = threading.Lock()
        t_start = time.perf_counter()

        def producer():
            t = t_start
            for q, s in enumerate(specs):
                t += gaps[q]
                d = t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                h = srv.submit(s)
                with lock:
                    tickets[h] = q

        th = threading.Thread(target=producer)
        th.start()
        lat, qlat, got, by_size = [], [], 0, {}
        while th.is_alive() or tickets:
            with lock:
                cur = dict(tickets)
            for h in cur:
                try:
                    srv.wait(h, 0)
                except Exception:
                    continue
                qms, ms = srv.times(h)
                lat.append(ms)
                qlat.append(srv.phases(h))
                by_size.setdefault(specs[cur[h]]["ngrid"], []).append(ms)
                got += parts[cur[h]]
                srv.release(h)
                with lock:
                    tickets.pop(h)
            time.sleep(0.0005)
        th.join()
        span = time.perf_counter() - t_start
        return {"load": load, "arrival_rate_jobs_per_s": rate, "requests": len(lat), "span_s": span,
                "throughput": got / span, "throughput_vs_batched": got / span / sat_tput,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(np.max(lat)),
                # the slowest 1%: median time queued, in set-up and running
                "tail_phases_ms": [float(np.median([ph[k] for ph, l in zip(qlat, lat) if l >= np.percentile(lat, 99)]))
                                   for k in range(3)],
                "median_phases_ms": [float(np.median([ph[k] for ph in qlat])) for k in range(3)],
                "p50_ms_by_grid": {str(n): float(np.percentile(v, 50)) for n, v in sorted(by_size.items())},
                "p99_ms_by_grid": {str(n): float(np.percentile(v, 99)) for n, v in sorted(by_size.items())}}

    clocks = Clocks(0, clock_csv("clocks_serving.csv"))
    sweep = [offered(load, 11 + q) for q, load in enumerate(args.loads)]
    clk = clocks.stop()
    srv.close()
    target = args.p99_target_ms
    # the highest offered load up to which every point of the sweep met the target
    best = None
    for pt in sorted(sweep, key=lambda pt: pt["load"]):
        if pt["p99_ms"] > target:
            break
        best = pt
    # the plain FP64 form, one job at a time, on a sample of the requests
    serial_s, serial_parts = 0.0, 0
    if not args.no_fp64:
        sample = specs[:args.fp64_sample]
        t1 = time.perf_counter()
        for s in sample:
            j = mfx.Job(eng, s["ngrid"], s["boxlen"], s["order"], s["seed_table"], s["amp_table"], s["coef"],
                        lattice=s["lattice"], precision=mfx.FP64, plt_table=s["plt_table"], lunit=s["lunit"],
                        vunit=s["vunit"])
            j.run()
            j.close()
            serial_parts += (1 << s["lattice"]) * s["ngrid"] ** 3
        serial_s = time.perf_counter() - t1
    return {
        "metric": "serving: particles/s at the stated p99 job latency under Poisson arrivals (mixed sizes/orders/lattices)",
        "value": best["throughput"] if best else None, "unit": "particles/s", "n_gpus": 1, "steps": len(sweep),
        "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (NGenIC white noise, seeds 1..%d; mix from default_rng(7))" % len(specs),
        "config": {"workload": "serve: %d requests per load point, N in {64..384}, order 1-3, SC/BCC/FCC (+PLT), "
                               "FP32-compensated" % len(specs), "max_inflight": args.inflight,
                   "admission": ("largest" if args.largest_first else "oldest") + " queued job that fits; a head "
                                "older than %g ms is not passed" % args.bypass_age_ms,
                   "small_jobs": ("footprint <= %g GiB beside the slots, at most %d" % (args.small_gb, args.max_small)
                                  if args.small_gb > 0 else None),
                   "stream_priority": ("default for every job" if args.no_priority else
                                       "by footprint, " + ("largest" if args.large_priority else "smallest") + " first"),
                   "particles_per_point": sum(parts), "tiles_per_size": {str(k): v for k, v in tuned.items()}},
        "p99_target_ms": target,
        "throughput_at_target_vs_batched": best["throughput_vs_batched"] if best else None,
        "load_at_target": best["load"] if best else None,
        "target_rule": "the highest offered load up to which every load point's p99 met the target",
        "batched": {"value": sat_tput, "unit": "particles/s", "span_s": sat_span,
                    "p50_ms": float(np.percentile(sat_lat, 50)), "p99_ms": float(np.percentile(sat_lat, 99)),
                    "mode": "every request queued at once"},
        "sweep": sweep,
        "alone_ms": alone_ms,
        "footprint_mb": footprint_mb,
        "fp64_serial": ({"value": serial_parts / serial_s, "unit": "particles/s", "span_s": serial_s,
                         "requests": len(specs[:args.fp64_sample])} if serial_s else None),
        "clocks": clk,
    }


def fp64_and_error(args, eng, inp, plt_tab, out):
    """Times the plain FP64 form of the same workload and states the FP32 form's
    error against it in units of the mean interparticle spacing: for the full
    displacement and, through mfx_job_assemble, for each LPT order on its own."""
    import torch
    from monofonic_gb300 import mfx
    res = {}
    parts = {}
    order = inp["order"]
    for prec in (mfx.FP64, mfx.FP32C):
        j = mfx.Job(eng, inp["n"], inp["L"], order, inp["seeds"], inp["amp"], inp["coef"], lattice=inp["lat"],
                    precision=prec, plt_table=plt_tab, fixing=inp["fix"], lunit=inp["lunit"], vunit=inp["vunit"],
                    pos64=True, vel64=True, id64=True)
        j.run()
        if prec == mfx.FP64:
            ms = []
            j.set_profiling(True)
            fft = {}
            for _ in range(max(1, min(args.steps, 3))):
                torch.cuda.synchronize()
                j.run()
                ms.append(sum(j.stage_times()))
                for k, (kms, kby, kcnt) in j.kernel_profile().items():
                    if k.startswith("cufft"):
                        a = fft.setdefault(k, [0.0, 0.0])
                        a[0] += kms
                        a[1] += kby
            j.set_profiling(False)
            res["fp64_form"] = {"value": j.num_particles / (np.mean(ms) * 1e-3), "unit": "particles/s",
                                "ms_per_step": float(np.mean(ms)), "steps": len(ms)}
            res["fp64_form"]["fft_rate"] = fp64_fft_rate(fft, inp["n"], len(ms), float(np.mean(ms)))
        # compared particles: all of them up to 64M (16M per order), else the first ones
        count = min(j.num_particles, 1 << 26)
        count_o = min(j.num_particles, 1 << 24)
        parts[prec] = {"all": j.particles_range(0, count)[:2]}
        for n in range(1, order + 1):
            j.assemble(1 << (n - 1))
            parts[prec][n] = j.particles_range(0, count_o)[:2]
        j.close()
    spacing = inp["L"] / (inp["n"] * 2 ** (inp["lat"] / 3.0))

    def stat(key):
        (p32, v32), (p64, v64) = parts[mfx.FP32C][key], parts[mfx.FP64][key]
        d = p32 - p64
        d -= inp["L"] * np.round(d / inp["L"])  # a particle wrapped across the box edge in one form only
        e = d / spacing
        return {"psi_rms_spacing": float(np.sqrt(np.mean(e ** 2))), "psi_max_spacing": float(np.max(np.abs(e))),
                "vel_rel_l2": float(np.linalg.norm(v32 - v64) / np.linalg.norm(v64)), "particles_compared": int(len(e))}

    res["error_vs_fp64"] = dict(stat("all"), spacing_mpc_h=spacing)
    res["error_vs_fp64_per_order"] = {"psi%d" % n: stat(n) for n in range(1, order + 1)}
    res["speedup_fp32c_over_fp64"] = res["fp64_form"]["ms_per_step"] / out["ms_per_step"]
    return res


def fp64_fft_rate(fft, n, steps, ms_step):
    """FLOP rate of the plain FP64 form's cuFFT transforms: 2.5 L log2 L per
    real transform of L points (the usual split-radix count), transforms
    counted from the bytes each execution moves (2 x the padded field)."""
    m = 3 * n // 2
    out = {}
    flops = ms = 0.0
    for k, (kms, kby) in fft.items():
        length = m if k.endswith("_M") else n
        field = (length + 2) * length * length * 8.0
        count = kby / (2.0 * field) / steps
        f = count * 2.5 * length ** 3 * np.log2(float(length) ** 3)
        out[k] = {"transforms_per_step": count, "ms_per_step": kms / steps,
                  "gflops": f / (kms / steps * 1e-3) / 1e9 if kms else None}
        flops += f
        ms += kms / steps
    rate = flops / (ms * 1e-3) if ms else None
    return {"kernels": out, "fft_ms_per_step": ms, "share_of_step": ms / ms_step if ms_step else None,
            "fft_tflops": rate / 1e12 if rate else None, "fp64_peak_tflops": FP64_PEAK_SPEC / 1e12,
            "frac_of_fp64_peak": rate / FP64_PEAK_SPEC if rate else None,
            "peak_source": "GB300 FP64 published rate (spec figure, not measured)"}


def cpu_restatement(n_sample, name, plt_tab=None, seed_offset=0):
    """One pass of the C++/OpenMP restatement of the reference path
    (oracle/lpt_omp.cc) on the workload's physics at grid n_sample (box scaled
    with the grid so the modes sampled keep their spacing); inputs from the
    oracle's own cosmology.  Returns (particles/s, seconds, stage seconds)."""
    from oracle import cosmo as ocosmo, lpt
    n, L, z, order, lat, plt, seed, fix = WORKLOADS[name]
    Ls = L * n_sample / n
    c = ocosmo.Cosmology()
    a = 1.0 / (1.0 + z)
    kf = 2 * np.pi / Ls
    q = np.arange(3 * (n_sample // 2) ** 2 + 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        k = kf * np.sqrt(q)
        amp = np.where(q > 0, c.amplitude(k) / (k * k), 0.0)
    coef = lpt.lpt_coefficients(c.growth(a), c.vfact(a), order)
    seeds = lpt.ngenic_seed_table(seed + seed_offset, n_sample)
    t0 = time.perf_counter()
    res = lpt.run_lpt_omp(n_sample, Ls, seeds, amp, order, coef, lattice=lat, lunit=Ls, vunit=Ls / np.sqrt(a),
                          fixing=fix, plt_table=plt_tab if plt else None)
    dt = time.perf_counter() - t0
    return (1 << lat) * n_sample ** 3 / dt, dt, [float(x) for x in res["times"]]


def oracle_plt_tables(name):
    """PLT tables of the workload's lattice from the oracle (numpy, CPU), or None."""
    n, L, z, order, lat, plt, seed, fix = WORKLOADS[name]
    if not plt:
        return None, 0.0
    from oracle import plt as oplt
    t0 = time.perf_counter()
    tab = oplt.plt_tables(lat)
    return tab, time.perf_counter() - t0


def cpu_sample_text(n_sample, name, dt, stages, tab_s, threads):
    n, order = WORKLOADS[name][0], WORKLOADS[name][3]
    return ("one full hot-path pass (noise -> %dLPT potentials -> particles, FP64) at %d^3 of the %d^3 workload "
            "(%.1f s; stages noise/phi1/phi2/phi3/A3/particles %s s), throughput per particle extrapolated to "
            "%d^3; PLT table build (%.1f s) excluded as on the GPU; C++/OpenMP CPU restatement of the reference "
            "loops (oracle/lpt_omp.cc, %d threads; own FFT, not FFTW)"
            % (order, n_sample, n, dt, "/".join("%.2f" % x for x in stages), n, tab_s, threads))


def run_reference(args):
    """The reference arm: the C++/OpenMP restatement of the reference's CPU
    path, each step one pass on a bounded sample of the workload."""
    rank, world, local = dist_env()
    if rank != 0:
        return None
    from oracle import lpt
    lpt.build_lib()
    lpt.build_omp_lib()
    threads = int(lpt.omp_lib().mfxo_omp_threads())
    n_sample = REF_SAMPLE[args.workload]
    tab, tab_s = oracle_plt_tables(args.workload)
    vals, dts, stages = [], [], None
    for s in range(args.warmup + args.steps):
        v, dt, st = cpu_restatement(n_sample, args.workload, tab, seed_offset=s)
        progress("reference step %d: %.1f s" % (s, dt))
        if s >= args.warmup:
            vals.append(v)
            dts.append(dt)
            stages = st
    total = sum(dts)
    npart = (1 << WORKLOADS[args.workload][4]) * n_sample ** 3
    v = npart * len(dts) / total
    sample = cpu_sample_text(n_sample, args.workload, float(np.mean(dts)), stages, tab_s, threads)
    cfg = describe(args.workload, args.precision)
    cfg["timed_sample_grid"] = n_sample
    return {"metric": metric_name(args.workload, args.precision), "impl": "reference",
            "value": v, "unit": "particles/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(dts)) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (NGenIC white noise, seeded)", "config": cfg,
            "cpu_baseline": {"value": v, "unit": "particles/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fcc768", choices=sorted(WORKLOADS) + ["ensemble64", "serve"])
    ap.add_argument("--requests", type=int, default=1000, help="serve: requests per load point")
    ap.add_argument("--loads", type=lambda v: [float(x) for x in v.split(",")],
                    default=[0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1], help="serve: offered loads / batched job rate")
    ap.add_argument("--p99-target-ms", type=float, default=100.0, help="serve: stated p99 job latency target")
    ap.add_argument("--fp64-sample", type=int, default=48, help="serve: requests run serially in FP64")
    ap.add_argument("--no-priority", action="store_true", help="serve: every job at the default stream priority")
    ap.add_argument("--inflight", type=int, default=2, help="serve: max jobs in flight")
    ap.add_argument("--largest-first", action="store_true", help="serve: admit the largest queued job that fits")
    ap.add_argument("--large-priority", action="store_true", help="serve: the largest jobs on the highest priority")
    ap.add_argument("--small-gb", type=float, default=0.0, help="serve: jobs up to this footprint take no slot")
    ap.add_argument("--max-small", type=int, default=16, help="serve: small jobs in flight at most")
    ap.add_argument("--bypass-age-ms", type=float, default=100.0, help="serve: age after which the head is not passed")
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="profiling runs: skip the end-to-end pass and the report")
    ap.add_argument("--host-positions", action="store_true",
                    help="end to end: float displacements cross the link, q + Psi formed on the host")
    ap.add_argument("--tiles", default="", help="fused-transform tiles 'PXY,PZ' instead of the autotuner's")
    args = ap.parse_args()
    if args.impl == "reference":
        out = run_reference(args)
        if out:
            print(json.dumps(out))
        return
    if args.workload == "serve":
        print(json.dumps(run_serving(args)))
        return
    if args.workload == "ensemble64":
        out = run_ensemble(args)
        if dist_env()[0] == 0:
            print(json.dumps(out))
        return
    out, eng, inp, plt_tab = run_ours(args)
    rank, world, _ = dist_env()
    if out is not None and out.get("profiling_run"):  # --no-e2e
        if rank == 0:
            print(json.dumps(out))
    elif rank == 0:
        if not args.no_fp64 and args.precision == "fp32c":
            progress("plain FP64 form and the error statement")
            out.update(fp64_and_error(args, eng, inp, plt_tab, out))
        if not args.no_cpu_baseline and world == 1:
            from oracle import lpt
            lpt.build_lib()
            lpt.build_omp_lib()
            threads = int(lpt.omp_lib().mfxo_omp_threads())
            n_sample = CPU_SAMPLE[args.workload]
            progress("CPU baseline at %d^3 (%d threads)" % (n_sample, threads))
            tab, tab_s = oracle_plt_tables(args.workload)
            v, dt, st = cpu_restatement(n_sample, args.workload, tab)
            out["cpu_baseline"] = {"value": v, "unit": "particles/s", "cores": threads, "kind": "port",
                                   "sample": cpu_sample_text(n_sample, args.workload, dt, st, tab_s, threads)}
            out["config"]["cpu_baseline_timed_grid"] = n_sample
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

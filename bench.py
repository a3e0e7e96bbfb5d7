#!/usr/bin/env python
"""Benchmark: AHC k-points/s at num_wann=32 (the triclinic MDRS workload).

Workload: seeded random TB model, triclinic lattice (3-5 A, 80-100 deg), nw=32,
R in [-4,4]^3 with Wigner-Seitz replicas (MDRS, mp_grid 9 -> ~1275 R-vectors),
192^3 k-points in 24^3 FFT blocks (NKdiv=8), AHC over 1001 Fermi levels in [-2,2] eV.
One step = one batch of FFT blocks through the whole hot path (R->k fields, FP64 eigh,
U^dagger X U, fused Berry curvature + Fermi-scan histogram).  Synthetic data (no
dataset exists for this workload).  Every step's fields (GBs) exceed the 129 MB L2, so
no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W] [--precision mixed|fp64] [--impl reference]

The GPU arm prints one JSON line with value (device-resident throughput), e2e
(public-API run() with pinned host->device upload of the R-space matrices and the
result read back every step), the roofline of the dominant kernel measured live with
CUDA events, the CPU baseline (the oracle on the host cores) and SM clocks sampled
during the timed region, plus three secondary measurements: "batched" and "served"
(multi-system runs through the continuous-batching server) and "tetra" (the same AHC with
the tetrahedron method over the whole grid in one run()), and "configs" (the cubic nw=8 and
spinor nw=96 models through run(), with the oracle on one core beside them).  --impl reference times the
reference algorithm's CPU restatement (oracle) on all host cores with the same metric.
--tetra-only [--nkfft N --tetra-nkdiv D] runs the tetrahedron measurement alone.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, 'wannier-berri_gb300'))
sys.path.insert(0, REPO)

NW = 32
NKFFT = 24
NKDIV = 8
NEF = 1001
METRIC = "AHC k-points/s at nw=32 (192^3 grid in 24^3 blocks, MDRS, 1001 E_F)"
UNIT = "k-points/s"
CPU_SAMPLE_NKFFT = 12
THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def build_system(device=None):
    """The nw=32 MDRS model; device='cuda' runs the Wigner-Seitz replica search on the GPU
    (same replica set as the host search)."""
    from wbgpu import models, System_R
    d = models.config_system(2)
    s = System_R.from_dict(d)
    s.do_ws_dist(9, device=device)
    return s


# ---------------------------------------------------------------------------------------
# CPU side: the oracle on a process pool (spawned, so no CUDA state is inherited)
# ---------------------------------------------------------------------------------------
def _cpu_worker(args):
    """One FFT block of the workload through the oracle (AHC at NEF levels): (seconds, the block's
    AHC normalised by its k-points).  The AHC values are the checker of the GPU path on the same
    blocks."""
    path, dK, nkfft = args
    sys.path.insert(0, REPO)
    from oracle import wb_oracle as O
    f = np.load(path)
    XX = {'Ham': f['Ham'], 'AA': f['AA']}
    s = O.RSystem(f['real_lattice'], f['iRvec'], f['wcc'], XX)
    t = time.perf_counter()
    data = O.DataK(s, (nkfft,) * 3, dK)
    res = O.AHC(Efermi=np.linspace(-2, 2, NEF))(data)
    return time.perf_counter() - t, np.asarray(res.data)


def save_system_npz(s):
    fd, path = tempfile.mkstemp(suffix='.npz', prefix='wbbench_')
    os.close(fd)
    np.savez(path, real_lattice=s.real_lattice, iRvec=s.iRvec, wcc=s.wannier_centers_cart,
             Ham=s.get_R_mat('Ham'), AA=s.get_R_mat('AA'))
    return path


def spawn_pool(procs):
    """Spawned workers with one BLAS thread each (set in the environment they inherit, before
    they import numpy), one process per host core -- the reference's own decomposition."""
    for v in THREAD_VARS:
        os.environ[v] = "1"
    return mp.get_context('spawn').Pool(procs)


def cpu_blocks(nblocks, seed=1):
    """Shifts dK of the CPU sample's blocks (random offsets of 12^3 FFT grids)."""
    rng = np.random.default_rng(seed)
    return [rng.random(3) / CPU_SAMPLE_NKFFT for _ in range(nblocks)]


def cpu_rate(path, nblocks, procs, pool=None, seed=1):
    """k-points/s of the oracle AHC on `nblocks` 12^3 blocks of the workload spread over `procs`
    processes, the wall time, the blocks' shifts and their AHC results."""
    dKs = cpu_blocks(nblocks, seed)
    jobs = [(path, dK, CPU_SAMPLE_NKFFT) for dK in dKs]
    own = pool is None
    if own:
        pool = spawn_pool(procs)
    t = time.perf_counter()
    out = pool.map(_cpu_worker, jobs, chunksize=1)
    wall = time.perf_counter() - t
    if own:
        pool.close()
        pool.join()
    return nblocks * CPU_SAMPLE_NKFFT ** 3 / wall, wall, dKs, [o[1] for o in out]


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    procs = os.cpu_count() or 1
    s = build_system()
    path = save_system_npz(s)
    pool = spawn_pool(procs)
    try:
        cpu_rate(path, procs, procs, pool)  # start-up + warm caches
        for _ in range(max(args.warmup - 1, 0)):
            cpu_rate(path, procs, procs, pool)
        t = time.perf_counter()
        for i in range(args.steps):
            pool.map(_cpu_worker, [(path, dK, CPU_SAMPLE_NKFFT) for dK in cpu_blocks(procs, seed=100 + i)],
                     chunksize=1)
        wall = time.perf_counter() - t
    finally:
        pool.close()
        pool.join()
        os.unlink(path)
    nk = args.steps * procs * CPU_SAMPLE_NKFFT ** 3
    value = nk / wall
    sample = (f"{procs} oracle processes x one {CPU_SAMPLE_NKFFT}^3 block each per step of the nw=32 MDRS "
              f"system (AHC, {NEF} E_F)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128/f64",
            "data": "synthetic (seeded random TB model)", "config": config_dict(args), "precision": "fp64 (CPU)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def config_dict(args):
    """The workload, identical for the GPU arm and the reference arm (precision is a key of its own)."""
    return {"workload": "random TB nw=32, triclinic, R in [-4,4]^3 + MDRS(mp 9), 192^3 k in 24^3 blocks, "
                        "AHC 1001 E_F", "num_wann": NW, "NKFFT": args.nkfft, "NKdiv": NKDIV,
            "blocks_per_step": args.blocks_per_step, "k_per_step": args.blocks_per_step * args.nkfft ** 3,
            "parallelism": f"blocks sharded over {args.gpus} GPU(s)",
            "l2": "inputs larger than L2 (GB-scale fields per step)"}


def dtype_of(precision):
    if precision == 'fp64':
        return "f64 / c128 throughout"
    return ("f64 energies, gaps, scan; double-float (48-bit) H(k); fp32 eigensolver refined by one "
            "Ogita-Aishima step against the double-float H (double-float residuals; energies to ~1e-13 |H|, "
            "U c64 rounded once); double-float velocity transform (rounded to c64), other fields fp32 with "
            "R-space hi+lo residuals; 3xTF32 tensor-core rotation, fp32 accumulation")


# ---------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv', prefix='wbclk_')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = [r.split(',') for r in open(self.path).read().strip().splitlines() if r.count(',') >= 8]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == 'active'})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows)}


def probe_peak(torch, fp64):
    import ctypes
    from wbgpu import _lib
    from wbgpu.engine import _ptr, _stream
    lib = _lib.load()
    blocks, threads, iters = 152 * 8, 256, 2048 if fp64 else 16384
    out = torch.empty(blocks * threads, dtype=torch.float64 if fp64 else torch.float32, device='cuda')
    fl = ctypes.c_double(0)
    _lib.check(lib.wbg_probe_fma(int(fp64), blocks, threads, 16, _ptr(out), ctypes.byref(fl), _stream()), "probe")
    best = 0.0
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        _lib.check(lib.wbg_probe_fma(int(fp64), blocks, threads, iters, _ptr(out), ctypes.byref(fl), _stream()), "probe")
        e.record()
        e.synchronize()
        best = max(best, fl.value / (s.elapsed_time(e) * 1e-3))
    return best / 1e9  # GFLOP/s


# DRAM bytes per k-point of the mixed path's eigensolver kernels at nw = 32 (dram__bytes_read.sum +
# dram__bytes_write.sum of eigh_tridiag<float, cdf, float>, eigh_ql<float>,
# eigh_vectors<float, float, float2> and the two eigh_refine<cdf> launches) from one ncu capture of
# the 16^3 case (python bench.py --nkfft 16 --blocks-per-step 1 --steps 1 --warmup 3 --no-cpu-baseline
# --no-fp64-compare --no-serve --no-tetra --no-configs --no-graphs-tune, ncu --metrics
# dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum -k regex:eigh_ -s 15 -c 5; 4096
# matrices per launch).  Each matrix's traffic is its own (H read by the solve and the refinement,
# reflectors, d / e / tau, U written and re-read), so it scales with the matrices of a launch.
EIGH_MIXED_DRAM_BYTES_PER_K = (42.0 + 1.1 + 1.1 + 0.0 + 27.3 + 13.6 + 77.1 + 0.4) * 1e6 / 4096


def stage_roofline(stage, ms_total, n_calls, k_per_call, precision, peaks, nF_fields):
    """Roofline of one stage from its algorithmic work per launch alone:
      R->k     2 F nw^2 s bytes per k-point (each field written and read back once; s = 16 B FP64,
               8 B FP32 complex, 16 B double-float H);
      eigh     20 nw^3 flops per matrix (FP64-class: tridiagonalisation, back-transform and
               tridiagonal eigenvectors), against the pipe the arithmetic runs on -- the FP64 pipe
               (FP64 path) or the FP32 pipe (double-float, mixed path);
      rotation 16 nw^3 flops per field and k-point (two complex GEMMs; the three TF32 products of
               the split count once), 9 fields, against dense TF32 (mixed) or the FP64 pipe;
      Omega    9 nw^2 s bytes per k-point (V, A and the rotA diagonal read).
    The extra arithmetic of the precision scheme (about 8.5 FP32 flops per double-float flop; three
    tensor products per rotation product) is reported apart as `pipe_work_frac`, how busy the
    pipe is, and does not enter `frac`."""
    n = NW
    per_launch_ms = ms_total / max(n_calls, 1)
    pipe_factor = None
    if stage == 'eigh':
        work = 20.0 * n ** 3 * k_per_call
        if precision == 'fp64':
            bound, unit, peak, src = 'fp64', 'GFLOP/s', peaks['fp64'], 'wbg_probe_fma FP64 FMA rate measured in this run'
        else:  # FP32 solve (tridiagonalisation, QL, inverse iteration, back-transform) + refinement
            bound, unit, peak, src = 'fp32', 'GFLOP/s', peaks['fp32'], 'wbg_probe_fma FP32 FMA rate measured in this run' 
    elif stage == 'rotate':
        work = 16.0 * n ** 3 * 9 * k_per_call      # two complex GEMMs per field, 9 fields
        if precision == 'fp64':
            bound, unit, peak, src = 'fp64', 'GFLOP/s', peaks['fp64'], 'wbg_probe_fma FP64 FMA rate measured in this run'
        else:  # tcgen05 kind::tf32, three TF32 products per product (3xTF32)
            bound, unit, peak, src = 'tensor', 'GFLOP/s', peaks['tf32'], \
                'MEASURED_PEAKS.json bf16_tflops (burst) / 2: dense TF32 rate'
            pipe_factor = 3.0
    elif stage.startswith('r2k'):
        s = 16 if stage in ('r2k_fp64', 'r2k_df64') else 8
        work = 2.0 * nF_fields[stage] * n * n * s * k_per_call   # bytes: write + read back of each field
        bound, unit, peak, src = 'hbm', 'GB/s', peaks['hbm'], 'MEASURED_PEAKS.json hbm_gbs'
    else:  # berry_omega
        s = 16 if precision == 'fp64' else 8
        work = 9.0 * n * n * s * k_per_call
        bound, unit, peak, src = 'hbm', 'GB/s', peaks['hbm'], 'MEASURED_PEAKS.json hbm_gbs'
    achieved = work / (per_launch_ms * 1e-3) / 1e9
    out = {"kernel": stage, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
           "frac": achieved / peak if peak else None, "peak_source": src, "ms_per_launch": per_launch_ms,
           "work_per_launch": work, **_traffic(stage, precision, k_per_call)}
    if pipe_factor:
        out["pipe_work_frac"] = achieved * pipe_factor / peak
        out["pipe_work_factor"] = pipe_factor
    return out


def _traffic(stage, precision, k_per_call):
    """DRAM traffic per launch where an ncu capture of the kernels exists (scaled from the
    captured case by the k-points of a launch), else None."""
    if stage == 'eigh' and precision == 'mixed':
        return {"traffic": EIGH_MIXED_DRAM_BYTES_PER_K * k_per_call,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the five eigh launches, "
                                  "16^3 case (4096 matrices) scaled to the k-points of a launch"}
    return {"traffic": None}


def run_gpu(args):
    import torch
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', str(args.gpus)))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    s = build_system(device='cuda')
    cpu = None
    cpu_check = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        path = save_system_npz(s)
        try:
            rate, wall, cdKs, cres = cpu_rate(path, procs, procs)
        finally:
            os.unlink(path)
        cpu_check = (np.array(cdKs), np.sum(cres, axis=0) / len(cres))
        cpu = {"value": rate, "unit": UNIT, "cores": procs, "kind": "port",
               "sample": f"{procs} spawned oracle processes, one {CPU_SAMPLE_NKFFT}^3 block each of the same nw=32 "
                         f"MDRS system (AHC, {NEF} E_F), {wall:.1f} s wall; the oracle is the reference's "
                         "algorithm restated in numpy (per k-point, per band-group loops), measured 1.64x faster "
                         "per core than the reference's own run() on the same block"}
    import wbgpu
    from wbgpu import engine, _lib
    from wbgpu.calculators import AHC
    _lib.load()
    torch.cuda.init()
    grid = wbgpu.Grid(s, NKdiv=NKDIV, NKFFT=args.nkfft)
    nblocks = grid.nblocks
    shifts = grid.block_shifts()
    # contiguous shard of the division grid per rank (blocks are independent: weak scaling)
    from wbgpu.distributed import shard_blocks
    mine = shard_blocks(nblocks, rank, world)
    B = args.blocks_per_step
    nk = grid.nk_per_block
    EF = np.linspace(-2, 2, NEF)

    def step_blocks(i):
        start = (i * B) % (len(mine) - B + 1)
        return mine[start:start + B]

    dev = engine.DeviceSystem(s)
    calc = AHC(Efermi=EF)
    quantities = calc.quantities(s)
    calc.reset(dev.device)
    phases = {p: dev.grid_phases(shifts, grid.FFT, p)
              for p in sorted(set(engine.phase_precs('fp64') + engine.phase_precs('mixed')))}

    def step(i, precision, c=calc):
        blocks = step_blocks(i)
        bd = engine.band_data(dev, shifts[blocks], grid.FFT, quantities, precision, phases=phases,
                              block_start=int(blocks[0]))
        c.accumulate(bd, s)
        return bd

    def timed_loop(precision, K, W, timer=None):
        for i in range(W):
            step(i, precision)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        engine.set_timer(timer)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for i in range(W, W + K):
            bd = step(i, precision)
        t1.record()
        torch.cuda.synchronize()
        engine.set_timer(None)
        engine.check_flag(bd)
        ms = t0.elapsed_time(t1)
        if world > 1:
            tt = torch.tensor([ms], device='cuda')
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            ms = float(tt.item())
        return ms

    precision = args.precision
    clocks = ClockSampler(local)
    timer = engine.StageTimer()
    clocks.start()
    ms = timed_loop(precision, args.steps, args.warmup, timer)
    clk = clocks.stop()
    total_k = world * args.steps * B * nk
    value = total_k / (ms * 1e-3)
    stage_ms = timer.totals_ms()
    counts = timer.counts()
    # every timed step is one batch: kernels per batch of each stage (the mixed path calls the
    # eigensolver in two stages around the side-stream field transform, 3 kernels in all)
    # eigh: tridiagonalisation, QL, inverse iteration, and the refinement's two launches (mixed, 24 < nw <= 32)
    kernels_per_batch = {'r2k_fp64': 3, 'r2k_fp32': 3, 'r2k_df64': 3, 'r2k_df64c': 3,
                         'eigh': 5 if (precision == 'mixed' and 24 < NW <= 32) else 3, 'rotate': 1,
                         'berry_omega': 1}
    gpu_launches = int(args.steps * sum(kernels_per_batch[k] for k in counts))

    # plain FP64 drop-in throughput on the same blocks, and the mixed-vs-FP64 error of one step
    fp64_value = None
    fp64_timer = None
    K64 = max(1, min(args.steps, 3))
    err = None
    if precision == 'mixed' and not args.no_fp64_compare:
        fp64_timer = engine.StageTimer()
        ms64 = timed_loop('fp64', K64, 1, fp64_timer)
        fp64_value = world * K64 * B * nk / (ms64 * 1e-3)
        c1, c2 = AHC(Efermi=EF), AHC(Efermi=EF)
        c1.reset(dev.device)
        c2.reset(dev.device)
        step(0, 'mixed', c1)
        step(0, 'fp64', c2)
        a = c1.finalize(s.cell_volume, nk)
        b = c2.finalize(s.cell_volume, nk)
        err = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    # both precisions against the oracle on the CPU baseline's blocks (the same system, 12^3 FFT
    # blocks at the oracle's shifts): the checker of the benchmarked path
    err_oracle = None
    if cpu_check is not None:
        cdKs, cref = cpu_check
        nkc = CPU_SAMPLE_NKFFT ** 3
        err_oracle = {"sample": f"{len(cdKs)} blocks of {CPU_SAMPLE_NKFFT}^3 k-points (the CPU baseline's), "
                                "AHC at 1001 E_F, max over E_F and components / max |AHC|"}
        for prec in ('mixed', 'fp64'):
            c = AHC(Efermi=EF)
            c.reset(dev.device)
            bdc = engine.band_data(dev, cdKs, (CPU_SAMPLE_NKFFT,) * 3, quantities, prec)
            c.accumulate(bdc, s)
            got = c.finalize(s.cell_volume, nkc) / len(cdKs)
            err_oracle[prec] = float(np.max(np.abs(got - cref)) / np.max(np.abs(cref)))

    # end-to-end through the public API: fresh device upload of the R-space matrices from
    # pinned host memory, run() over this step's blocks, result read back to the host
    def e2e_run(prec):
        Ke = max(1, min(args.steps, 5))
        h2d = 0
        for i in range(args.warmup):  # warm-up of the e2e path
            wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision=prec, blocks=step_blocks(i))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(Ke):
            dsys = engine.DeviceSystem(s)
            r = wbgpu.run(s, grid, {'ahc': AHC(Efermi=EF)}, precision=prec, blocks=step_blocks(i), dev_system=dsys)
            h2d = dsys.h2d_bytes
            _ = r['ahc'].data  # already on the host (device->host copy inside run())
        e1.record()
        torch.cuda.synchronize()
        ems = e0.elapsed_time(e1)
        if world > 1:
            tt = torch.tensor([ems], device='cuda')
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            ems = float(tt.item())
        return {"value": world * Ke * B * nk / (ems * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": NEF * 3 * 8}

    e2e = e2e_run(precision)
    e2e64 = e2e_run('fp64') if fp64_value is not None else None

    peaks = {'fp64': probe_peak(torch, True), 'fp32': probe_peak(torch, False)}
    try:
        mp_ = json.load(open(os.path.join(REPO, 'MEASURED_PEAKS.json')))
        peaks['hbm'] = float(mp_['hbm_gbs'])
        peaks['tf32'] = float(mp_['bf16_tflops']) * 1e3 / 2.0  # GFLOP/s
    except (OSError, KeyError, ValueError):
        peaks['hbm'] = 6800.0  # fallback figures of the profiling recipe
        peaks['tf32'] = 1.9e6 / 2.0
    # fields per stage of the AHC step: FP64 path H + 9; mixed path H (double-float), V (double-float
    # transform rounded to complex64) and A, rotA (FP32)
    nF_fields = {'r2k_fp64': 10, 'r2k_df64': 1, 'r2k_df64c': 3, 'r2k_fp32': 6}
    dominant = max(stage_ms, key=stage_ms.get)
    roof = stage_roofline(dominant, stage_ms[dominant], args.steps, B * nk, precision, peaks, nF_fields)
    # every stage against its own bound (stage times from CUDA events on the stage's stream; the
    # field transform runs next to the eigensolver on a side stream, so its span is stretched)
    stages_roof = {}
    for st_name in stage_ms:
        r_ = stage_roofline(st_name, stage_ms[st_name], args.steps, B * nk, precision, peaks, nF_fields)
        stages_roof[st_name] = {k_: r_[k_] for k_ in ('bound', 'achieved', 'peak', 'unit', 'frac')}
    fp64_dropin = None
    if fp64_value is not None:
        st64 = fp64_timer.totals_ms()
        dom64 = max(st64, key=st64.get)
        fp64_dropin = {"value": fp64_value, "unit": UNIT, "steps": K64, "dtype": dtype_of('fp64'),
                       "e2e": e2e64,
                       "roofline": stage_roofline(dom64, st64[dom64], K64, B * nk, 'fp64', peaks, nF_fields),
                       "stage_ms_per_step": {k: v / K64 for k, v in st64.items()},
                       "mixed_speedup": value / fp64_value, "mixed_e2e_speedup": e2e["value"] / e2e64["value"]}
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype_of(precision), "precision": precision,
            "data": "synthetic (seeded random TB model)", "config": config_dict(args),
            "roofline": roof, "stages_roofline": stages_roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": gpu_launches, "clocks": clk,
            "stage_ms_per_step": {k: v / args.steps for k, v in stage_ms.items()},
            "fp64_dropin": fp64_dropin, "max_rel_err_vs_fp64": err, "max_rel_err_vs_oracle": err_oracle,
            "peaks_measured_gflops": {"fp64": peaks['fp64'], "fp32": peaks['fp32']}}
    if world == 1 and not args.no_serve:
        for key, fn in (("batched", bench_batched), ("served", bench_served)):
            try:
                line[key] = fn()
            except Exception as e:  # the headline line is still printed
                line[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if world == 1 and not args.no_configs:
        try:
            line["configs"] = bench_configs()
        except Exception as e:
            line["configs"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if world == 1 and not args.no_graphs_tune:
        for key, fn in (("cuda_graph", bench_graphs), ("autotune", bench_autotune)):
            try:
                line[key] = fn()
            except Exception as e:
                line[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if world == 1 and not args.no_tetra:
        try:
            line["tetra"] = bench_tetra(s, dev, args.nkfft, NKDIV)
        except Exception as e:
            line["tetra"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------------------
# Tetrahedron method: AHC with tetra=True over the whole grid in one run()
# ---------------------------------------------------------------------------------------
def bench_tetra(s, dev, nkfft, nkdiv, err_blocks=8):
    """AHC (1001 E_F) with tetra=True over the NKdiv^3 x NKFFT^3 grid through run(): k-points/s
    of the whole run (corner energies included, timed with a device synchronisation on both
    sides) against the same run() without tetra, stage times, and the mixed-vs-FP64 error of the
    tetrahedron AHC on the first `err_blocks` blocks."""
    import numpy as np
    import torch
    import wbgpu
    from wbgpu import engine
    from wbgpu.calculators import AHC
    ef = np.linspace(-2, 2, NEF)
    grid = wbgpu.Grid(s, NKdiv=nkdiv, NKFFT=nkfft)
    nk = grid.nk_per_block * grid.nblocks
    few = list(range(min(err_blocks, grid.nblocks)))
    wbgpu.run(s, grid, {'a': AHC(Efermi=ef, tetra=True)}, precision='mixed', dev_system=dev, blocks=few)
    out = {}
    for key, tetra in (("tetra", True), ("plain", False)):
        timer = engine.StageTimer()
        torch.cuda.synchronize()
        engine.set_timer(timer)
        t0 = time.perf_counter()
        wbgpu.run(s, grid, {'a': AHC(Efermi=ef, tetra=tetra)}, precision='mixed', dev_system=dev)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        engine.set_timer(None)
        out[key] = (nk / dt, {k: round(v, 2) for k, v in timer.totals_ms().items()})
    a = wbgpu.run(s, grid, {'a': AHC(Efermi=ef, tetra=True)}, precision='mixed', dev_system=dev, blocks=few)['a'].data
    b = wbgpu.run(s, grid, {'a': AHC(Efermi=ef, tetra=True)}, precision='fp64', dev_system=dev, blocks=few)['a'].data
    return {"workload": f"AHC tetra=True, {NEF} E_F, {nkdiv * nkfft}^3 grid in {nkfft}^3 blocks, one run(), mixed",
            "kpoints": nk, "kpoints_per_s": out["tetra"][0], "stage_ms": out["tetra"][1],
            "without_tetra_kpoints_per_s": out["plain"][0],
            "max_rel_err_vs_fp64": float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
            "err_sample": f"first {len(few)} blocks"}


def run_tetra_only(args):
    """--tetra-only: the tetrahedron measurement alone (profiling captures of its kernels)."""
    import torch
    from wbgpu import engine, _lib
    s = build_system(device='cuda')
    _lib.load()
    torch.cuda.init()
    print(json.dumps({"tetra": bench_tetra(s, engine.DeviceSystem(s), args.nkfft, args.tetra_nkdiv)}), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# The other single-system configurations: cubic nw=8 (AHC) and spinor nw=96 (Kubo + AHC)
# ---------------------------------------------------------------------------------------
def _timed_run(s, grid, mk, precision, dev, blocks=None):
    import torch
    import wbgpu
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = wbgpu.run(s, grid, mk(), precision=precision, dev_system=dev, blocks=blocks)
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def _oracle_rate(s, nkfft, calcs):
    """k-points/s of the oracle on one block of `s` (one host process, one BLAS thread)."""
    from oracle import wb_oracle as O
    o = O.RSystem(s.real_lattice, s.iRvec, s.wannier_centers_cart, s._XX_R)
    data = O.DataK(o, nkfft, np.array([0.31, 0.17, 0.53]) / np.array(nkfft))
    t0 = time.perf_counter()
    for c in calcs.values():
        c(data)
    return int(np.prod(nkfft)) / (time.perf_counter() - t0)


def bench_kubo_block(nkfft):
    """One NKFFT^3 block of the spinor nw = 96 model through run() (OpticalConductivity at 11 E_F x
    400 frequencies, Lorentzian 0.05 eV, + AHC), mixed precision, after one warm-up block: wall
    time and CUDA-event stage times."""
    import torch
    import wbgpu
    from wbgpu import engine, models, System_R
    from wbgpu.calculators import AHC, OpticalConductivity
    ef3, om = np.linspace(-1, 1, 11), np.linspace(0, 4, 400)
    s3 = System_R.from_dict(models.config_system(3))
    g3 = wbgpu.Grid(s3, NKdiv=6, NKFFT=nkfft)
    d3 = engine.DeviceSystem(s3)
    mk3 = lambda: {'opt': OpticalConductivity(Efermi=ef3, omega=om, smr_fixed_width=0.05), 'ahc': AHC(Efermi=ef3)}
    wbgpu.run(s3, g3, mk3(), precision='mixed', dev_system=d3, blocks=[5])
    torch.cuda.synchronize()
    timer = engine.StageTimer()
    engine.set_timer(timer)
    t0 = time.perf_counter()
    wbgpu.run(s3, g3, mk3(), precision='mixed', dev_system=d3, blocks=[0])
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    engine.set_timer(None)
    stages = {k: sum(a.elapsed_time(b) for a, b in evs) for k, evs in timer.events.items()}
    return {"nkfft": nkfft, "kpoints": nkfft ** 3, "ms": dt * 1e3, "kpoints_per_s": nkfft ** 3 / dt,
            "stage_ms": stages}


def bench_rotation_engines(nk, reps):
    """CUDA-event time of U^dagger X U at nw = 32 on `nk` synthetic k-points with the mixed AHC
    path's fields (V and A from lower triangles, V plain, A Hermitian part, rotA diagonal only) for
    each engine of the rotation (wbg_tune ROTATE_ENGINE): 1 tensor cores warp-specialised, 3
    tensor cores one tile at a time, 2 CUDA cores; and the largest difference between the engines."""
    import torch
    from wbgpu import autotune, engine
    nw = 32
    g = torch.Generator(device='cuda').manual_seed(1)
    U = (torch.randn(nk, nw, nw, dtype=torch.complex64, device='cuda', generator=g) / nw ** 0.5).contiguous()
    X = torch.randn(nk, 9, nw, nw, dtype=torch.complex64, device='cuda', generator=g)
    sel, herm = list(range(9)), [0 | 4] * 3 + [1 | 4] * 3 + [2 | 4] * 3
    out = {}
    ref = None
    for e in (3, 1, 2):
        autotune.set_value(autotune.ROTATE_ENGINE, nw, 0, e)
        Y = torch.empty((nk, 9, nw, nw), dtype=torch.complex64, device='cuda')
        for _ in range(2):
            engine.rotate(U, X, 9, sel, herm, nw, nk, 0, out=Y)
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(1, reps)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            engine.rotate(U, X, 9, sel, herm, nw, nk, 0, out=Y)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        d = torch.arange(nw, device='cuda')
        if ref is None:
            ref = Y.clone()
            diff = 0.0
        else:
            diff = max(float((Y[:, :6] - ref[:, :6]).abs().max()), float((Y[:, 6:, d, d] - ref[:, 6:, d, d]).abs().max()))
        out[{1: "tensor_warp_specialised", 2: "cuda_cores", 3: "tensor_one_tile"}[e]] = {
            "ms_median": float(np.median(ts)), "max_abs_diff_vs_one_tile": diff}
    autotune.set_value(autotune.ROTATE_ENGINE, nw, 0, 0)
    out["nk"] = nk
    out["device_flags"] = engine.device_flags()
    return out


def bench_configs():
    """run() throughput of the cubic nw = 8 model (AHC at 501 E_F, the whole 48^3 grid in 8^3
    blocks) and of the spinor nw = 96 model with SOC (R in [-5,5]^3; OpticalConductivity at 11
    E_F x 400 frequencies, Lorentzian 0.05 eV, + AHC; 2 of the 216 16^3 blocks of its 96^3
    grid), mixed precision, with the error against the FP64 path on the same blocks and the oracle
    on one host core (a small block of the same model) beside it."""
    import wbgpu
    from wbgpu import engine, models, System_R
    from wbgpu.calculators import AHC, OpticalConductivity
    from oracle import wb_oracle as O
    out = {}
    ef1 = np.linspace(-2, 2, 501)
    s1 = System_R.from_dict(models.config_system(1))
    g1 = wbgpu.Grid(s1, NKdiv=6, NKFFT=8)
    d1 = engine.DeviceSystem(s1)
    mk1 = lambda: {'ahc': AHC(Efermi=ef1)}
    _timed_run(s1, g1, mk1, 'mixed', d1, blocks=[0])
    r, dt = _timed_run(s1, g1, mk1, 'mixed', d1)
    r64, dt64 = _timed_run(s1, g1, mk1, 'fp64', d1)
    a, b = r['ahc'].data, r64['ahc'].data
    out["c1"] = {"workload": "cubic nw=8, R in [-2,2]^3, AHC at 501 E_F, 48^3 k in 8^3 blocks, one run()",
                 "kpoints_per_s": 48 ** 3 / dt, "fp64_kpoints_per_s": 48 ** 3 / dt64,
                 "max_rel_err_vs_fp64": float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
                 "cpu_kpoints_per_s_per_core": _oracle_rate(s1, (8, 8, 8), {'ahc': O.AHC(Efermi=ef1)}),
                 "cpu_sample": "oracle, one 8^3 block, one process"}
    ef3, om = np.linspace(-1, 1, 11), np.linspace(0, 4, 400)
    s3 = System_R.from_dict(models.config_system(3))
    g3 = wbgpu.Grid(s3, NKdiv=6, NKFFT=16)
    d3 = engine.DeviceSystem(s3)
    mk3 = lambda: {'opt': OpticalConductivity(Efermi=ef3, omega=om, smr_fixed_width=0.05), 'ahc': AHC(Efermi=ef3)}
    _timed_run(s3, g3, mk3, 'mixed', d3, blocks=[5])
    blocks = [0, 1]
    r, dt = _timed_run(s3, g3, mk3, 'mixed', d3, blocks=blocks)
    r64, dt64 = _timed_run(s3, g3, mk3, 'fp64', d3, blocks=blocks)
    err = {k: float(np.max(np.abs(r[k].data - r64[k].data)) / np.max(np.abs(r64[k].data))) for k in ('opt', 'ahc')}
    nk3 = len(blocks) * 16 ** 3
    ocs = {'opt': O.OpticalConductivity(Efermi=ef3, omega=om, smr_fixed_width=0.05), 'ahc': O.AHC(Efermi=ef3)}
    out["c3"] = {"workload": "spinor nw=96 with SOC, R in [-5,5]^3, OpticalConductivity 11 E_F x 400 omega "
                             "(Lorentzian 0.05 eV) + AHC, 2 blocks of 16^3 of the 96^3 grid, one run()",
                 "kpoints_per_s": nk3 / dt, "fp64_kpoints_per_s": nk3 / dt64, "max_rel_err_vs_fp64": err,
                 "cpu_kpoints_per_s_per_core": _oracle_rate(s3, (2, 2, 1), ocs),
                 "cpu_sample": "oracle, one 2x2x1 block, one process"}
    return out


# ---------------------------------------------------------------------------------------
# Batched and served workloads (scaled-down forms of the multi-system configurations)
# ---------------------------------------------------------------------------------------
def tb_pool(n, seed, nw_lo, nw_hi):
    """n seeded random TB systems, num_wann log-uniform in [nw_lo, nw_hi], R half-width 1 or 2."""
    import numpy as np
    from wbgpu import models, System_R
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nw = int(round(np.exp(rng.uniform(np.log(nw_lo), np.log(nw_hi)))))
        d = models.random_tb(nw, int(rng.integers(1, 3)), models.triclinic_lattice(rng), 1.5, seed + i,
                             centers='random', keys=('Ham', 'AA'))
        out.append(System_R.from_dict(d))
    return out


def bench_batched(nsys=32):
    """AHC + Berry-curvature dipole of `nsys` systems (num_wann 4-128) on 16^3 grids: all jobs
    through one continuous-batching server (mixed precision) against looping the plain FP64
    run() system by system."""
    import numpy as np
    import torch
    import wbgpu
    from wbgpu.calculators import AHC, BerryDipole_FermiSea
    ef = np.linspace(-1, 1, 201)
    systems = tb_pool(nsys, 4000, 4, 128)
    mk = lambda: {'ahc': AHC(Efermi=ef), 'bcd': BerryDipole_FermiSea(Efermi=ef)}
    jobs = [(s, wbgpu.Grid(s, NKdiv=1, NKFFT=16), mk()) for s in systems]
    wbgpu.run_many(jobs[:4], precision='mixed')  # build the library's lazy state
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    got = wbgpu.run_many(jobs, precision='mixed', max_active=8)
    torch.cuda.synchronize()
    t_b = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = [wbgpu.run(s, g, mk(), precision='fp64') for s, g, _ in jobs]
    torch.cuda.synchronize()
    t_p = time.perf_counter() - t0
    nk = sum(g.nk_per_block * g.nblocks for _, g, _ in jobs)
    err = {k: max(float(np.max(np.abs(a[k].data - b[k].data)) / np.max(np.abs(b[k].data))) for a, b in zip(got, ref))
           for k in ('ahc', 'bcd')}
    return {"workload": f"{nsys} systems, num_wann log-uniform 4-128 (seeded), R half-width 1-2, 16^3 k each, "
                        "AHC + BCD at 201 E_F", "kpoints": nk, "kpoints_per_s": nk / t_b,
            "plain_fp64_loop_kpoints_per_s": nk / t_p, "speedup_vs_plain_loop": t_p / t_b,
            "max_rel_err_vs_fp64": err, "nw": [s.num_wann for s in systems]}


def bench_served(nsys=16, nreq=120, load=0.7, nbase=24):
    """Poisson arrivals of AHC requests over `nsys` resident systems (num_wann log-uniform
    8-128), grids 16^3-32^3, each with 0-3 rounds of refinement around the largest Berry
    curvatures (8^3 sub-grids around the top 1% of k-points by |Omega| per round).  The offered
    rate is `load` times the server's capacity, measured first by serving the same requests all at
    once; p50 / p99 latency from submit to result at that rate, and throughput, against the plain
    FP64 path of the first `nbase` requests (same refinement) one after the other."""
    import numpy as np
    import torch
    import wbgpu
    from wbgpu import engine
    from wbgpu.calculators import AHC
    from wbgpu.run import run_refine_omega
    ef = np.linspace(-1, 1, 201)
    systems = tb_pool(nsys, 5000, 8, 128)
    rng = np.random.default_rng(5001)
    reqs = []
    for i in range(nreq):
        s = int(rng.integers(nsys))
        reqs.append((s, int(rng.choice([1, 2])), 16, int(rng.integers(0, 4))))
    grids = {}
    grid_of = lambda r: grids.setdefault(r[:3], wbgpu.Grid(systems[r[0]], NKdiv=r[1], NKFFT=r[2]))
    srv = wbgpu.Server(precision='mixed', max_active=8)
    for i, s in enumerate(systems):
        srv.add_system(i, s)
    submit = lambda r: srv.submit(r[0], grid_of(r), {'ahc': AHC(Efermi=ef)}, refine_omega=r[3])
    for r in set(q[:3] for q in reqs):  # warm the per-(system, grid) caches: R-space fields, phase tables
        srv.submit(r[0], grid_of(r), {'ahc': AHC(Efermi=ef)})
    srv.run_until_idle()
    torch.cuda.synchronize()
    # capacity: every request at once
    srv._finished.clear()
    t0 = time.perf_counter()
    cal = [submit(r) for r in reqs]
    srv.run_until_idle()
    torch.cuda.synchronize()
    capacity = nreq / (time.perf_counter() - t0)
    rate = load * capacity
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    srv._finished.clear()
    tickets = []
    with srv:
        t0 = time.perf_counter()
        for r, ta in zip(reqs, arrivals):
            dt = t0 + ta - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets.append(submit(r))
        for t in tickets:
            t.wait(600)
    st = srv.stats(tickets)
    devs = {}
    sample = [reqs[i] for i in sorted(rng.choice(nreq, size=min(nbase, nreq), replace=False))]

    def serial(precision):
        """The sample's requests one after the other through run() / run_refine_omega."""
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nkb = 0
        for s, nkdiv, nkfft, nit in sample:
            g = grid_of((s, nkdiv, nkfft))
            dev = devs.setdefault(s, engine.DeviceSystem(systems[s]))
            if nit:  # k-points as the server counts them: the grid, then per round 1% of it x (8^3 + 1)
                run_refine_omega(systems[s], g, {'ahc': AHC(Efermi=ef)}, precision, rounds=nit, dev_system=dev)
                n = g.nk_per_block * g.nblocks
                nkb += n + nit * max(1, int(round(0.01 * n))) * (8 ** 3 + 1)
            else:
                wbgpu.run(systems[s], g, {'ahc': AHC(Efermi=ef)}, precision=precision, dev_system=dev)
                nkb += g.nk_per_block * g.nblocks
        torch.cuda.synchronize()
        return nkb / (time.perf_counter() - t0)

    serial_mixed = serial('mixed')
    serial_fp64 = serial('fp64')
    err = max(float(np.max(np.abs(a.wait()['ahc'].data - b.wait()['ahc'].data)) /
                    np.max(np.abs(b.wait()['ahc'].data))) for a, b in zip(tickets[:4], cal[:4]))
    st.update({"workload": f"{nreq} AHC requests over {nsys} resident systems (num_wann log-uniform 8-128, "
                           "seeded), grids 16^3-32^3, 0-3 rounds of refinement around the top 1% |Omega| "
                           "k-points (8^3 sub-grids), 201 E_F, mixed precision",
               "capacity_requests_per_s": capacity, "offered_rate_per_s": rate, "offered_load": load,
               "plain_fp64_serial_kpoints_per_s": serial_fp64, "mixed_serial_kpoints_per_s": serial_mixed,
               "mixed_vs_fp64_serial": serial_mixed / serial_fp64,
               "serial_sample": f"{len(sample)} random requests of the stream, one after the other",
               "same_request_repeat_max_rel_diff": err})
    return st


# ---------------------------------------------------------------------------------------
# CUDA-graph replay and launch-shape autotuning
# ---------------------------------------------------------------------------------------
def bench_graphs(reps=3):
    """run() over many small batches (the cubic nw=8 model, 512 blocks of 4^3, AHC at 501 E_F)
    with plain launches and with stages 1-3 replayed from CUDA graphs (cuda_graph=True): the
    regime where per-batch host dispatch, not the GPU, sets the pace."""
    import numpy as np
    import torch
    import wbgpu
    from wbgpu import engine, models
    from wbgpu.calculators import AHC
    s = wbgpu.System_R.from_dict(models.config_system(1))
    grid = wbgpu.Grid(s, NKdiv=8, NKFFT=4)
    ef = np.linspace(-2, 2, 501)
    dev = engine.DeviceSystem(s)
    nk = grid.nblocks * grid.nk_per_block
    out = {"workload": "cubic nw=8 model, 32^3 k-points in 512 blocks of 4^3, AHC at 501 E_F, whole run()"}
    for prec in ('mixed', 'fp64'):
        for bpb in (4, 16):
            r = {}
            for g in (False, True):
                call = lambda: wbgpu.run(s, grid, {'ahc': AHC(Efermi=ef)}, precision=prec, blocks_per_batch=bpb,
                                         cuda_graph=g, dev_system=dev)
                call()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(reps):
                    call()
                torch.cuda.synchronize()
                r["graph" if g else "plain"] = nk * reps / (time.perf_counter() - t0)
            r["speedup"] = r["graph"] / r["plain"]
            out[f"{prec}_blocks_per_batch_{bpb}_kpoints_per_s"] = r
    return out


def bench_autotune(nws=(8, 32, 96)):
    """Eigensolver launch time (double-float solve, the mixed path) with the built-in shapes and
    with the autotuner's choice, per num_wann; the table is restored afterwards."""
    from wbgpu import autotune
    out = {"workload": "wbg_eigh_batched mode 3 on seeded random Hermitian matrices "
                       "(16384 x (32/nw)^3 matrices, clamped to 1024-32768)"}
    for nw in nws:
        autotune.reset([nw])
        base = autotune.time_eigh(nw, 3 | autotune.PRECISE_VECTORS)
        t0 = time.perf_counter()
        entry, _ = autotune.tune_eigh(nw, 3 | autotune.PRECISE_VECTORS)
        tune_s = time.perf_counter() - t0
        tuned = autotune.time_eigh(nw, 3 | autotune.PRECISE_VECTORS)
        autotune.reset([nw])
        out[f"nw{nw}"] = {"matrices": autotune.default_batch(nw), "builtin_ms": base, "tuned_ms": tuned,
                          "choice": entry, "tuning_s": tune_s}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=30)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gpu', choices=['gpu', 'reference'])
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--blocks-per-step', type=int, default=4)
    ap.add_argument('--nkfft', type=int, default=NKFFT, help='FFT block edge (smaller only for profiling captures)')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-fp64-compare', action='store_true')
    ap.add_argument('--no-serve', action='store_true', help='skip the batched and served measurements')
    ap.add_argument('--no-tetra', action='store_true', help='skip the tetrahedron-method measurement')
    ap.add_argument('--no-configs', action='store_true', help='skip the nw=8 and nw=96 configurations')
    ap.add_argument('--configs-only', action='store_true', help='run only the nw=8 and nw=96 configurations')
    ap.add_argument('--tetra-only', action='store_true', help='run only the tetrahedron-method measurement')
    ap.add_argument('--tetra-nkdiv', type=int, default=NKDIV, help='NKdiv of --tetra-only')
    ap.add_argument('--no-graphs-tune', action='store_true', help='skip the CUDA-graph and autotuner measurements')
    ap.add_argument('--graphs-tune-only', action='store_true', help='run only the CUDA-graph and autotuner measurements')
    ap.add_argument('--kubo-only', type=int, default=0, metavar='NKFFT',
                    help='only run the nw = 96 spinor model (OpticalConductivity at 11 E_F x 400 omega + AHC) over '
                         'one NKFFT^3 block, mixed precision, with per-stage times (profiling captures)')
    ap.add_argument('--rotation-engines', type=int, default=0, metavar='NK',
                    help='only time the nw = 32 rotation engines (tensor cores: warp-specialised and one tile at '
                         'a time; CUDA cores) on NK synthetic k-points of the AHC field set')
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)
    if args.kubo_only:
        print(json.dumps({"kubo_c3": bench_kubo_block(args.kubo_only)}), flush=True)
        return 0
    if args.rotation_engines:
        print(json.dumps({"rotation_engines": bench_rotation_engines(args.rotation_engines, args.steps)}), flush=True)
        return 0
    if args.graphs_tune_only:
        import torch
        from wbgpu import _lib
        _lib.load()
        torch.cuda.init()
        print(json.dumps({"cuda_graph": bench_graphs(), "autotune": bench_autotune()}), flush=True)
        return 0
    if args.tetra_only:
        return run_tetra_only(args)
    if args.configs_only:
        import torch
        from wbgpu import _lib
        _lib.load()
        torch.cuda.init()
        print(json.dumps({"configs": bench_configs()}), flush=True)
        return 0
    return run_gpu(args)


if __name__ == '__main__':
    sys.exit(main())

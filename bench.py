#!/usr/bin/env python
"""Throughput of the mPIE position loop on GB300: positions*iterations/s.

Workload (the configuration the headline metric is quoted on): CPM mPIE,
npsm = 4 probe modes, Np = 128, No = 512, 400 Fermat-spiral positions,
alpha = beta = 0.25, friction 0.7, feedback 0.3, random position order and the
reference's momentum draws (PtyLab/Engines/mPIE.py:96-195).  Seeded synthetic
data (Gaussian-random-field object in amplitude [0.6, 1] and phase [0, 2*pi],
Hermite-Gauss probe modes with powers 1:0.5:0.25:0.125, 1e6-photon Poisson
intensities) stand in for measured scans.

One step = one reconstruction iteration (every position once) over a batch
of G independent scans, one thread-block cluster per scan, in one kernel
launch; G is the number of clusters the GPU holds at once in the library's
throughput shape (16 rows per CTA).  `single_scan` times one scan alone in the
latency shape (8 rows per CTA).  `value` is timed
with CUDA events on the launching stream with all inputs resident in HBM; the
batch streams G x 26 MB of intensities per step, more than L2 (129 MB), so no
L2 flush is needed.  `e2e` runs the public API (ptylab_gb300.Engines.mPIE(...)
.reconstruct()) on one scan from host NumPy arrays to host NumPy arrays.

`--impl reference` times the reference algorithm's CPU implementation (the
NumPy oracle, oracle/ptyoracle.py) on all host cores: one independent scan per
process.  Under torchrun every rank reconstructs its own batch (weak scaling);
rank 0 prints one JSON line.
"""

from __future__ import annotations

import argparse
import copy
import ctypes as C
import json
import multiprocessing as mp
import os
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NP, NO, NPOS, NPSM = 128, 512, 400, 4
METRIC = "positions*iterations/s, mPIE CPM npsm=4 Np=128 No=512 400 positions (1 GB300)"
UNIT = "positions*iterations/s"
WORKLOAD = "mPIE CPM Fraunhofer, npsm=4, nosm=1, Np=128, No=512, 400 Fermat positions, random order, momentum"


def c1_spec(seed):
    from ptylab_gb300.simulate import ScanSpec

    return ScanSpec(
        Np=NP, No=NO, num_positions=NPOS, npsm=NPSM, step_fraction=0.3, probe_radius_fraction=1 / 4,
        photons=1e6, phase_max=2 * np.pi, amp_min=0.6, sigma_px=4.0, seed=seed,
    )


def make_scan(seed):
    from ptylab_gb300.simulate import cpm_problem

    d, p, rec, _, _ = cpm_problem(c1_spec(seed), engine_seed=seed)
    p.positionOrder = "random"
    return d, p, rec


def scan_orders(seed, iters, nf):
    """Per-iteration orders and momentum flags drawn as the reference draws them
    (BaseEngine.py:646-653 shuffle from the third iteration, mPIE.py:170)."""
    rs = np.random.RandomState(seed)
    orders, flags = [], []
    for it in range(iters):
        idx = np.arange(nf)
        if it >= 2:
            rs.shuffle(idx)
        orders.append(idx)
        flags.append(rs.rand(nf) > 0.95)
    return np.concatenate(orders).astype(np.int32), np.concatenate(flags).astype(np.uint8)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, device_index):
        self.proc = None
        self.path = None
        self.device_index = device_index

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(
            ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
             "-i", str(self.device_index)],
            stdout=open(self.path, "w"), stderr=subprocess.DEVNULL,
        )
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r.split(", ") for r in Path(self.path).read_text().splitlines() if r.strip()]
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(rows),
        }


# ------------------------------------------------------------------ peaks
def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return float(j["hbm_gbs"]), "measured", float(j.get("sm_max_mhz", 2070.0))
    return 6800.0, "fallback", 2070.0


def algorithmic_counts(flags_per_step, nscans):
    """Per step (one launch): bytes and FP32 flops of the algorithm, not of the code.
    Per position: object patch read + write (16*Np^2 B), intensities (4*Np^2 B);
    the probe stays on chip.  Per momentum step: object and probe read (X, buffer,
    momentum) and written (X, buffer, momentum): 48*(No^2 + npsm*Np^2) B -- three
    arrays written, not two, because objectBuffer / probeBuffer are separate
    caller-visible arrays that must hold the new object and probe (mPIE.py:196-224).
    Flops: 5*N*log2(N) per complex 2D transform of N = Np^2 points, two per mode,
    plus 60 flops per pixel per mode of elementwise work."""
    n2 = NP * NP
    per_pos_bytes = 20 * n2
    mom_bytes = 48 * (NO * NO + NPSM * n2)
    bytes_ = nscans * NPOS * per_pos_bytes + flags_per_step * mom_bytes
    per_pos_flops = NPSM * (2 * 5 * n2 * np.log2(n2) + 60 * n2)
    flops = nscans * NPOS * per_pos_flops + flags_per_step * 12 * (NO * NO + NPSM * n2)
    return float(bytes_), float(flops), float(per_pos_bytes), float(per_pos_flops)


# DRAM bytes per position of the batched launch, from one ncu capture
# (dram__bytes.sum.per_second x gpu__time_duration of a 15-scan launch / 6000
# positions; the summary is profiles/engine_kernel_mpie_c1.md)
TRAFFIC_PER_POSITION = 410_520


# ------------------------------------------------------------------ ranks
def reduce_over_ranks(seconds, units, device=None):
    """Whole-job timing under torch.distributed: the slowest rank's time and
    the units all ranks processed (weak scaling: every rank owns its scans)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ------------------------------------------------------------------ gb300 arm
def run_gb300(args, rank, world, local_rank):
    import torch

    from ptylab_gb300 import DummyMonitor, Engines, _native

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    lib = _native.require(local_rank)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def geometry(nscans, throughput):
        return _native.Geometry(Np=NP, No=NO, nosm=1, npsm=NPSM, nslice=1, num_frames=NPOS, num_scans=nscans,
                                engine=_native.ENGINES["mPIE"], propagator=0, fftshift=0, fpm=0,
                                cluster=args.cluster, throughput=throughput,
                                threads=args.threads if throughput else 0,
                                probe_in_smem=args.probe_smem if throughput else 0)

    probe_plan = C.c_void_p()
    _native.check(lib.ptyg_plan_create(C.byref(geometry(1, 1)), C.byref(probe_plan)))
    cl, th, sm, maxc = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    _native.check(lib.ptyg_plan_info(probe_plan, C.byref(cl), C.byref(th), C.byref(sm), C.byref(maxc)))
    lib.ptyg_plan_destroy(probe_plan)
    G = args.scans if args.scans > 0 else max(1, maxc.value)
    iters = args.warmup + args.steps

    def build_batch(host_scans, seed0, throughput):
        nscans = len(host_scans)
        keep, plan = [], C.c_void_p()
        _native.check(lib.ptyg_plan_create(C.byref(geometry(nscans, throughput)), C.byref(plan)))
        flag_counts = np.zeros(iters, dtype=np.int64)
        for s in range(nscans):
            seed = seed0 + s
            d, p, rec = host_scans[s]
            t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)  # noqa: E731
            obj = t(rec.object, torch.complex64)
            prb = t(rec.probe, torch.complex64)
            bufs = [obj.clone(), torch.zeros_like(obj), prb.clone(), torch.zeros_like(prb)]
            pos = t(rec.positions.astype(np.int32), torch.int32)
            data = t(d.ptychogram, torch.float32)
            order, flags = scan_orders(seed, iters, NPOS)
            flag_counts += flags.reshape(iters, NPOS).sum(axis=1).astype(np.int64)
            od, fd = t(order, torch.int32), t(flags, torch.uint8)
            b = _native.ScanBuffers(object=obj.data_ptr(), probe=prb.data_ptr(), positions=pos.data_ptr(),
                                    order=od.data_ptr(), momentum_flags=fd.data_ptr(),
                                    object_buffer=bufs[0].data_ptr(), object_momentum=bufs[1].data_ptr(),
                                    probe_buffer=bufs[2].data_ptr(), probe_momentum=bufs[3].data_ptr())
            _native.check(lib.ptyg_plan_bind_scan(plan, s, C.byref(b), data.data_ptr(), sptr))
            _native.check(lib.ptyg_plan_set_order(plan, s, od.data_ptr(), fd.data_ptr(), iters * NPOS, sptr))
            keep += [obj, prb, pos, data, od, fd, b] + bufs
        return plan, keep, flag_counts

    u = _native.UpdateParams(beta_object=0.25, beta_probe=0.25, alpha_object=0.25, alpha_probe=0.25,
                             reg_object=1.0, reg_probe=1.0, friction=0.7, feedback=0.3, probe_weight=1.0,
                             slice_beta=0.9)

    def timed(plan, nsteps, nwarm):
        for w in range(nwarm):
            _native.check(lib.ptyg_plan_run(plan, C.byref(u), w * NPOS, NPOS, 0, sptr))
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(nsteps):
            _native.check(lib.ptyg_plan_run(plan, C.byref(u), (nwarm + k) * NPOS, NPOS, 0, sptr))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / 1e3

    # G scans of host data, used by the device-resident run and the end-to-end one
    host_scans = [make_scan(1000 * rank + 1 + s) for s in range(G)]

    # batched, device-resident: the kernel view
    plan, keep, flag_counts = build_batch(host_scans, 1000 * rank + 1, 1)
    clocks = ClockSampler(local_rank)
    clocks.start()
    t = timed(plan, args.steps, args.warmup)
    clk = clocks.stop()
    lib.ptyg_plan_destroy(plan)
    del keep
    t, units = reduce_over_ranks(t, G * NPOS * args.steps, dev)
    value = units / t
    ms_per_step = t / args.steps * 1e3
    flags_timed = float(flag_counts[args.warmup:].sum()) / args.steps
    bytes_step, flops_step, per_pos_bytes, per_pos_flops = algorithmic_counts(flags_timed, G)
    hbm_peak, peak_kind, _ = measured_peaks()
    achieved_gbs = bytes_step / (t / args.steps) / 1e9
    props = torch.cuda.get_device_properties(dev)
    sm_max = (clk or {}).get("sm_max_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    achieved_tf = flops_step / (t / args.steps) / 1e12

    out = {}
    if rank == 0:
        # one scan alone: latency view of the same kernel
        plan1, keep1, _ = build_batch([make_scan(7)], 7, 0)
        t1 = timed(plan1, min(args.steps, 50), args.warmup)
        lib.ptyg_plan_destroy(plan1)
        del keep1
        single = {"value": NPOS * min(args.steps, 50) / t1, "us_per_position": t1 / (min(args.steps, 50) * NPOS) * 1e6}
        # against the roofline of the SMs one scan runs on (its cluster)
        probe1 = C.c_void_p()
        _native.check(lib.ptyg_plan_create(C.byref(geometry(1, 0)), C.byref(probe1)))
        cl1 = C.c_int()
        _native.check(lib.ptyg_plan_info(probe1, C.byref(cl1), C.byref(th), C.byref(sm), C.byref(maxc)))
        lib.ptyg_plan_destroy(probe1)
        single["cluster_ctas"] = cl1.value
        single["cluster_fp32_frac"] = single["value"] * per_pos_flops / (cl1.value * 128 * 2 * sm_max * 1e6)

        # end to end through the public API, host NumPy in and out: the same
        # G scans as engines built the PtyLab way, reconstructed together
        def engines_from(scans, n_it):
            out = []
            for d, p, rec in scans:
                e = Engines.mPIE(copy.deepcopy(rec), d, copy.deepcopy(p), DummyMonitor())
                e.alphaObject = e.alphaProbe = 0.25
                e.numIterations = n_it
                out.append(e)
            return out

        Engines.reconstruct_batch(engines_from(host_scans, args.warmup))
        engs = engines_from(host_scans, args.steps)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        Engines.reconstruct_batch(engs)
        torch.cuda.synchronize(dev)
        te = time.perf_counter() - t0
        d0, _, r0 = host_scans[0]
        per_scan_h2d = d0.ptychogram.nbytes + 3 * r0.object.nbytes + 3 * r0.probe.nbytes + NPOS * 2 * 4
        per_scan_d2h = 3 * r0.object.nbytes + 3 * r0.probe.nbytes + NPOS * NP * NP * 8  # detectorError as float64
        h2d = G * (per_scan_h2d + args.steps * NPOS * 5)
        d2h = G * (per_scan_d2h + args.steps * NPOS * 8)
        e2e = {"value": G * NPOS * args.steps / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": int(d2h / args.steps), "scans": G,
               "api": "ptylab_gb300.Engines.reconstruct_batch([Engines.mPIE(...) per scan]), NumPy in/out"}

        # one scan through Engines.mPIE(...).reconstruct(): PtyLab's own call
        n1 = min(args.steps, 50)
        d, p, rec = make_scan(99)
        eng = Engines.mPIE(rec, d, p, DummyMonitor())
        eng.numIterations = n1
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        eng.reconstruct()
        torch.cuda.synchronize(dev)
        e2e_single = {"value": NPOS * n1 / (time.perf_counter() - t0), "unit": UNIT, "steps": n1,
                      "api": "ptylab_gb300.Engines.mPIE(...).reconstruct(), NumPy in/out"}

        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (FP32 complex, the mPIE momentum step included, in the reference's complex64 rounding order; FP64 error sums)",
            "data": "synthetic: seeded Fermat scans, GRF objects, Hermite-Gauss probes, 1e6-photon Poisson",
            "config": {
                "workload": WORKLOAD, "scans_per_gpu": G, "cluster_ctas_per_scan": cl.value,
                "threads_per_cta": th.value, "smem_per_cta": sm.value, "parallelism": f"replicas x{world}",
                "l2": f"no flush: each step streams {G} x {NPOS * NP * NP * 4 / 1e6:.1f} MB of intensities (> 129 MB L2)",
                "step": "one iteration over every position of every scan, one kernel launch",
            },
            "roofline": {
                "bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": TRAFFIC_PER_POSITION * G * NPOS, "peak_kind": peak_kind,
                "traffic_note": "DRAM bytes per launch: ncu dram__bytes_read+write of one 15-scan launch "
                                "(profiles/engine_kernel_mpie_c1.md) per position, times this launch's positions",
                "algorithmic_bytes_per_position": per_pos_bytes, "bytes_per_launch": bytes_step,
            },
            "roofline_fp32": {
                "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak,
                "peak_kind": "nominal: SMs x 128 FP32 lanes x 2 x max SM clock",
                "flops_per_position": per_pos_flops,
            },
            "gpu_launches": args.steps,
            "clocks": clk,
            "single_scan": single,
            "e2e": e2e,
            "e2e_single_scan": e2e_single,
        }
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args.cpu_iters)
        if not args.no_configs:
            cfgs = {"C1": {"engine": "mPIE", "value": value, "unit": UNIT, "ms_per_step": ms_per_step,
                           "scans": G, "roofline": {"hbm_frac": achieved_gbs / hbm_peak,
                                                    "fp32_frac": achieved_tf / fp32_peak,
                                                    "frac": max(achieved_gbs / hbm_peak, achieved_tf / fp32_peak)},
                           "single_scan": single, "note": "the headline line above"}}
            for name in ("C0", "C2", "C3"):
                cfgs[name] = measure_config(name, dev, lib, with_cpu=world == 1 and not args.no_cpu_baseline)
            cfgs["C2_gradient"] = measure_c2_gradient(dev)
            out["configs"] = cfgs
    return out


# ------------------------------------------------------------------ other configurations
# The plain loop's other benchmark configurations (ptylab_gb300.simulate):
# C0 ePIE Np 64, C2 multislice e3PIE Np 256 (4 slices, 900 positions), C3 FPM
# qNewton Np 128.  Each is timed through the engine API: the set-up of
# Engines.reconstruct_batch (data and state moved to HBM once), then K timed
# iterations of every scan (host order draw and upload, one launch, error
# record, constraints), with CUDA events on the engines' stream.
CONFIG_STEPS = {"C0": (20, 3), "C2": (4, 3), "C3": (20, 3)}


def config_counts(name, rec):
    """Algorithmic FP32 flops and HBM bytes per position-iteration: 5 N log2 N
    flops per complex 2D transform of N = Np^2 points plus 60 flops per pixel
    per mode (per slice for multislice) of elementwise work; bytes = object
    patch read and written (16 B per pixel per slice) and the intensities
    (4 B per pixel).  Multislice runs 2 + 4 (S - 1) transforms per position."""
    n2 = int(rec.Np) ** 2
    lg = np.log2(n2)
    K = int(rec.nosm) * int(rec.npsm) * int(getattr(rec, "nlambda", 1))
    S = int(rec.nslice)
    if S > 1:
        flops = (2 + 4 * (S - 1)) * 5 * n2 * lg + 60 * n2 * S
        bytes_ = S * 16 * n2 + 4 * n2
    else:
        flops = K * (2 * 5 * n2 * lg + 60 * n2)
        bytes_ = 20 * n2
    return float(flops), float(bytes_)


def _config_cpu_sample(name, target_positions):
    """The oracle (complex64 NumPy, one core) on the first positions of the
    configuration's scan: positions*iterations/s."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import simulate as S

    eng, d, p, rec = S.config_problem(name)
    kw = {"C3": dict(order="NA", operationMode="FPM", probeBoundary=True)}.get(name, {})
    g = O.Geometry(Np=int(rec.Np), No=int(rec.No), dxp=float(rec.dxp), wavelength=float(rec.wavelength),
                   zo=float(rec.zo), npsm=int(rec.npsm), nslice=int(rec.nslice), dz=float(getattr(rec, "dz", 0) or 0))
    s = O.Settings(engine=eng, entrancePupilDiameter=float(d.entrancePupilDiameter or 0.0), **kw)
    nf = d.ptychogram.shape[0]
    n = min(nf, target_positions)
    iters = max(1, target_positions // nf)
    st = O.State(object=rec.object.copy(), probe=rec.probe.copy())
    oe = O.OracleEngine(s, g, st, d.ptychogram[:n], np.asarray(rec.positions)[:n], d.energyAtPos[:n])
    np.random.seed(1)
    t0 = time.perf_counter()
    oe.reconstruct(iters)
    t = time.perf_counter() - t0
    return {"value": n * iters / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{name}: oracle {eng}, {n} positions x {iters} iterations on one core"}


def measure_config(name, dev, lib, with_cpu=True):
    """Batched and single-scan throughput of one configuration, its roofline
    fractions and the one-core NumPy sample."""
    import torch

    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300 import simulate as S
    from ptylab_gb300.Engines.batch import begin_batch, finish_batch, iterate_batch

    eng_name, d, p, rec = S.config_problem(name)
    steps, warm = CONFIG_STEPS[name]
    nf = d.ptychogram.shape[0]
    stream = torch.cuda.current_stream(dev)

    def engines(n):
        out = []
        for _ in range(n):
            e = getattr(Engines, eng_name)(copy.deepcopy(rec), copy.deepcopy(d), copy.deepcopy(p), DummyMonitor())
            out.append(S.configure_engine(name, e, warm + steps))
        return out

    def timed(n, throughput):
        es = begin_batch(engines(n), throughput)
        cl, th, sm, mx = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        lib.ptyg_plan_info(es[0]._plan, C.byref(cl), C.byref(th), C.byref(sm), C.byref(mx))
        for loop in range(warm):
            iterate_batch(es, loop)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for loop in range(warm, warm + steps):
            iterate_batch(es, loop)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        t = e0.elapsed_time(e1) / 1e3
        finish_batch(es)
        return t, cl.value, mx.value

    # how many scans the throughput shape holds at once
    _, _, G = timed(1, 1)
    G = max(1, G)
    t, cl, _ = timed(G, 1)
    t1, cl1, _ = timed(1, 0)
    flops, bytes_ = config_counts(name, rec)
    hbm_peak, peak_kind, _ = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    clock = 2070.0
    fp32_sm = 128 * 2 * clock * 1e6 / 1e12  # TFLOP/s per SM
    value = G * nf * steps / t
    single = nf * steps / t1
    frac_f = value * flops / 1e12 / (props.multi_processor_count * fp32_sm)
    frac_b = value * bytes_ / 1e9 / hbm_peak
    out = {
        "engine": eng_name, "value": value, "unit": UNIT, "ms_per_step": t / steps * 1e3, "steps": steps,
        "warmup": warm, "scans": G, "cluster_ctas_per_scan": cl, "positions": nf,
        "roofline": {"bound": "fp32" if frac_f >= frac_b else "hbm", "frac": max(frac_f, frac_b),
                     "fp32_tflops": value * flops / 1e12, "fp32_frac": frac_f,
                     "hbm_gbs": value * bytes_ / 1e9, "hbm_frac": frac_b, "hbm_peak": hbm_peak,
                     "hbm_peak_kind": peak_kind, "fp32_peak": props.multi_processor_count * fp32_sm,
                     "fp32_peak_kind": "nominal: SMs x 128 FP32 lanes x 2 x 2070 MHz",
                     "flops_per_position": flops, "bytes_per_position": bytes_},
        "single_scan": {"value": single, "us_per_position": t1 / (steps * nf) * 1e6, "cluster_ctas": cl1,
                        "cluster_fp32_frac": single * flops / 1e12 / (cl1 * fp32_sm)},
        "step": "one iteration of every scan through the engine API (order draw and upload, one launch, "
                "error record, constraints); data and state resident in HBM",
    }
    if with_cpu:
        target = {"C0": 2000, "C2": 60, "C3": 1125}[name]
        out["cpu_baseline"] = _config_cpu_sample(name, target)
    return out


def measure_c2_gradient(dev, steps=4, warm=2):
    """C2's gradient engine: Engines.e3qNewton (the quasi-Newton step on the
    adjoint of the multislice model, 64 positions per step) on the C2 scan,
    one scan on the whole GPU; K timed iterations after the set-up, CUDA
    events on the engine's stream."""
    import torch

    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300 import simulate as S

    _, d, p, rec = S.config_problem("C2")
    eng = Engines.e3qNewton(rec, d, p, DummyMonitor())
    eng.numIterations = warm + steps
    nf = d.ptychogram.shape[0]
    np.random.seed(2)
    eng._begin()
    for loop in range(warm):
        eng._iterate(loop)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for loop in range(warm, warm + steps):
        eng._iterate(loop)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) / 1e3
    eng._end()
    flops, bytes_ = config_counts("C2", rec)
    hbm_peak, peak_kind, _ = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    fp32_peak = props.multi_processor_count * 128 * 2 * 2070.0 * 1e6 / 1e12
    value = nf * steps / t
    return {
        "engine": "e3qNewton", "value": value, "unit": UNIT, "ms_per_step": t / steps * 1e3, "steps": steps,
        "warmup": warm, "scans": 1, "positions": nf, "positions_per_step": int(eng.batchSize),
        "error_curve": [float(x) for x in np.asarray(rec.error)],
        "roofline": {"bound": "fp32", "frac": value * flops / 1e12 / fp32_peak, "fp32_tflops": value * flops / 1e12,
                     "fp32_frac": value * flops / 1e12 / fp32_peak,
                     "hbm_frac": value * bytes_ / 1e9 / hbm_peak, "hbm_peak": hbm_peak, "hbm_peak_kind": peak_kind,
                     "flops_per_position": flops, "bytes_per_position": bytes_},
        "step": "one iteration: order draw and upload, then per 64 positions one gradient pass (forward, amplitude "
                "residual, adjoint) and the quasi-Newton step of the 4 object slices and the probe",
    }


# ------------------------------------------------------------------ CPU legs
def _oracle_scan(seed):
    from oracle import ptyoracle as O

    d, p, rec = make_scan(seed)
    g = O.Geometry(Np=NP, No=NO, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo, npsm=NPSM)
    s = O.Settings(engine="mPIE", order="random", alphaObject=0.25, alphaProbe=0.25,
                   entrancePupilDiameter=d.entrancePupilDiameter)
    st = O.State(object=rec.object.copy(), probe=rec.probe.copy())
    return O.OracleEngine(s, g, st, d.ptychogram, rec.positions, d.energyAtPos)


def _oracle_worker(args):
    seed, warm, steps, barrier = args
    os.environ["OMP_NUM_THREADS"] = "1"
    eng = _oracle_scan(seed)
    np.random.seed(seed)
    eng.reconstruct(warm)
    if barrier is not None:
        barrier.wait()
    t0 = time.perf_counter()
    eng.reconstruct(steps)
    return time.perf_counter() - t0


def cpu_baseline(iters):
    """The oracle's mPIE on this host, one core, one C1 scan, `iters` iterations."""
    t = _oracle_worker((5, 1, iters, None))
    return {"value": NPOS * iters / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"one C1 scan, {iters} iterations x {NPOS} positions after 1 warm-up iteration"}


def run_reference(args):
    ncores = os.cpu_count() or 1
    nproc = args.ref_procs if args.ref_procs > 0 else ncores
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        barrier = m.Barrier(nproc)
        with ctx.Pool(nproc) as pool:
            times = pool.map(_oracle_worker, [(11 + i, args.warmup_ref, args.steps, barrier) for i in range(nproc)])
    t = max(times)
    value = nproc * NPOS * args.steps / t
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (NumPy complex64, as the reference)",
        "data": "synthetic: seeded Fermat scans, GRF objects, Hermite-Gauss probes, 1e6-photon Poisson",
        "config": {"workload": WORKLOAD, "scans": nproc, "parallelism": f"{nproc} processes, one scan each"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "port",
                         "sample": f"{nproc} independent C1 scans, {args.steps} iterations each, after {args.warmup_ref} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_calibration(args):
    """FPM illumination calibration (PtyLab's IlluminationCalibration with the
    example script's settings: radius calibration, translation fit) on a
    synthetic 15 x 15 LED scan of 256 x 256 frames whose LED array is shifted
    and whose NA is given 8 % low: GPU end to end (host frames in, encoder
    out), best of ``--calib-reps``, against the NumPy/SciPy oracle on one
    core, run once on the same data; "agree" says whether every integer
    decision (brightfield split, per-LED positions, fitted positions) matched."""
    import types

    import numpy as np
    import torch

    from oracle import calib_oracle as co
    from ptylab_gb300.CalibrationFPM import IlluminationCalibration
    from ptylab_gb300.simulate import FPMSpec, simulate_fpm

    spec = FPMSpec(Np=256, No=1024, grid=15, photons=1e5, amp_contrast=0.2, phase_scale=0.3 * np.pi,
                   led_shift=(6e-4, 4e-4), NA=0.092, true_NA=0.1)
    I, enc, _, _, dxp = simulate_fpm(spec)
    conv = -(1 / spec.wavelength) * dxp * spec.Np
    pos = np.round(conv * enc / np.sqrt(enc[:, 0] ** 2 + enc[:, 1] ** 2 + spec.zled**2)[..., None])
    pos = (pos + spec.No // 2 - spec.Np // 2).astype(int)

    def gpu_once():
        rec = types.SimpleNamespace(Np=spec.Np, No=spec.No, dxp=dxp, dxo=dxp, wavelength=spec.wavelength,
                                    NA=spec.NA, zled=spec.zled, positions=pos.copy())
        data = types.SimpleNamespace(ptychogram=I, encoder=enc.copy())
        ic = IlluminationCalibration(rec, data)
        ic.calibrateRadius = True
        ic.fit_mode = "Translation"
        np.random.seed(1234)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ic.runCalibration()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, ic

    gpu_once()  # library and allocator warm-up
    times, ic = [], None
    for _ in range(max(1, args.calib_reps)):
        t, ic = gpu_once()
        times.append(t)
    oracle = co.CalibrationOracle(spec.Np, spec.No, dxp, spec.wavelength, spec.NA, calibrateRadius=True,
                                  fit_mode="Translation")
    np.random.seed(1234)
    t0 = time.perf_counter()
    _, _, _, fitted = oracle.run(I.copy(), pos)
    cpu = time.perf_counter() - t0
    agree = (np.array_equal(ic.brightfieldIndices, oracle.brightfieldIndices)
             and np.array_equal(ic.calibrated_positions, oracle.calibrated_positions)
             and np.array_equal(ic.positionsFitted, fitted) and ic.apertRadiusPixel == oracle.apertRadiusPixel)
    return {
        "metric": "FPM illumination calibration time", "value": round(min(times), 4), "unit": "s",
        "higher_is_better": False, "n_gpus": 1, "steps": len(times), "warmup": 1,
        "dtype": "f32 frames, c64 transforms, f64 decisions", "data": "synthetic: shifted 15 x 15 LED array, NA 8 % low",
        "config": {"workload": "IlluminationCalibration.runCalibration, 225 LEDs, 256 x 256 frames, "
                               "calibrateRadius=True, fit_mode='Translation'",
                   "brightfield": int(np.sum(ic.brightfieldIndices)), "search_rounds": int(ic.rounds)},
        "times_s": [round(t, 4) for t in times], "agree": bool(agree),
        "cpu_baseline": {"value": round(cpu, 3), "unit": "s", "cores": 1, "kind": "port",
                         "sample": "the same calibration once (NumPy/SciPy oracle)"},
    }


def run_network(args):
    """The warm-start network's tensor-core kernels (BF16 operands, FP32
    accumulation): with --layer NAME, that layer's 3x3 convolution and its
    weight gradient on random operands; otherwise the whole forward pass and
    the whole backward pass (data and weight gradients of every layer), eager
    and as CUDA graphs.  FLOPs are 2 M N K per GEMM (M pixels, N output
    channels, K = 9 x input channels; the backward pass counts a weight
    gradient for every layer and a data gradient for every layer but the
    first).  CUDA-event times after 3 warm-up repetitions."""
    import numpy as np
    import torch

    from ptylab_gb300 import _native
    from ptylab_gb300.warmstart.network import LEVELS, WarmStartNet, layer_specs

    lib = _native.require(0)
    B, S, reps = args.net_batch, args.net_size, args.net_reps
    level = {"e1": 1, "e2": 2, "e3": 3, "ba": 4, "bb": 4, "d3": 3, "d2": 2, "d1": 1, "he": 1}

    def timed(f):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            f()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps / 1e3

    out = {"metric": "warm-start network tensor-core throughput", "unit": "TFLOP/s", "higher_is_better": True,
           "dtype": "bf16 operands, f32 accumulation", "data": "synthetic (random operands)",
           "config": {"batch": B, "size": S, "levels": list(LEVELS), "reps": reps}}
    if args.layer:
        spec = {name: (cins, co) for name, cins, co, _ in layer_specs(LEVELS)}
        if args.layer not in spec or args.layer in ("e1a", "head"):
            raise SystemExit(f"--layer: one of {[n for n in spec if n not in ('e1a', 'head')]}")
        cins, co = spec[args.layer]
        c0, c1 = cins[0], (cins[1] if len(cins) > 1 else 0)
        H = W = S >> (level[args.layer[:2]] - 1)
        bf = torch.bfloat16
        x0 = torch.randn(B * H * W, c0, device="cuda").to(bf)
        x1 = torch.randn(B * H * W, max(c1, 8), device="cuda").to(bf)
        w = torch.randn(co, 9 * (c0 + c1), device="cuda").to(bf)
        y = torch.empty(B * H * W, co, device="cuda", dtype=bf)
        bias = torch.zeros(co, device="cuda")
        dy = torch.randn(B * H * W, co, device="cuda").to(bf)
        splits = 8
        part = torch.empty(splits, co, 9 * (c0 + c1), device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        x1p = x1.data_ptr() if c1 else None
        conv = lambda: _native.check(lib.ptyg_nn_conv3(x0.data_ptr(), x1p, c0, c1, B, H, W, w.data_ptr(), co, None,  # noqa: E731
                                                       y.data_ptr(), bias.data_ptr(), 1, st.data_ptr(), None))
        wgrad = lambda: _native.check(lib.ptyg_nn_conv3_wgrad(dy.data_ptr(), co, x0.data_ptr(), x1p, c0, c1, B, H, W,  # noqa: E731
                                                              splits, part.data_ptr(), st.data_ptr(), None))
        flop = 2.0 * B * H * W * co * 9 * (c0 + c1)
        res = {}
        for name, f in (("conv3_forward", conv), ("weight_gradient", wgrad)):
            t = timed(f)
            res[name] = {"us": t * 1e6, "tflops": flop / t / 1e12, "M": B * H * W, "N": co, "K": 9 * (c0 + c1)}
        if int(st.item()) != 0:
            raise TimeoutError("a bounded tensor-core wait gave up")
        out.update(workload=f"layer {args.layer}", value=res["conv3_forward"]["tflops"], layer=res)
        return out
    fwd = bwd = 0.0
    for name, cins, co, _ in layer_specs(LEVELS):
        side = S >> (level[name[:2]] - 1)
        k = (1 if name == "head" else 9) * sum(cins)
        f = 2.0 * B * side * side * co * k
        fwd += f
        bwd += f if name == "e1a" else 2 * f
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.standard_normal((B, S, S)).astype(np.float32)).cuda()
    dy = torch.as_tensor(rng.standard_normal((B, S, S, 2)).astype(np.float32)).cuda()
    res = {}
    for mode in ("eager", "graphs"):
        net = WarmStartNet(seed=0)
        if mode == "graphs":
            net.enable_graphs()
        for name, f, flop in (("forward", lambda: net.forward(x), fwd), ("backward", lambda: net.backward(dy), bwd)):
            t = timed(f)
            res[f"{name}_{mode}"] = {"ms": t * 1e3, "gflop": flop / 1e9, "tflops": flop / t / 1e12}
        net.check_status()
    out.update(workload="whole network, forward and backward passes", value=res["forward_graphs"]["tflops"],
               passes=res)
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scans", type=int, default=0, help="independent scans per GPU (0: as many as fit at once)")
    ap.add_argument("--cluster", type=int, default=0, help="CTAs per scan (0: the library's choice)")
    ap.add_argument("--cpu-iters", type=int, default=8, help="iterations of the one-core CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the C0 / C2 / C3 lines")
    ap.add_argument("--threads", type=int, default=0, help="CTA size of the batched launch (0 = the plan's choice)")
    ap.add_argument("--probe-smem", type=int, default=0,
                    help="batched launch: 0 = plan's choice, 1 = probe rows in L2, 2 = in shared memory")
    ap.add_argument("--ref-procs", type=int, default=0)
    ap.add_argument("--warmup-ref", type=int, default=1)
    ap.add_argument("--calibration", action="store_true",
                    help="time the FPM illumination calibration instead of the reconstruction")
    ap.add_argument("--calib-reps", type=int, default=3)
    ap.add_argument("--network", action="store_true",
                    help="time the warm-start network's forward and backward passes instead")
    ap.add_argument("--layer", default="", help="with --network: time one layer (e.g. d3a) instead")
    ap.add_argument("--net-batch", type=int, default=16)
    ap.add_argument("--net-size", type=int, default=128)
    ap.add_argument("--net-reps", type=int, default=20)
    ap.add_argument("--config", default="", choices=["", "C0", "C2", "C3", "C2_gradient"],
                    help="time only this configuration's line (as in the headline line's configs)")
    args = ap.parse_args()
    if args.config:
        import torch

        torch.cuda.set_device(0)
        dev = torch.device("cuda", 0)
        if args.config == "C2_gradient":
            print(json.dumps(measure_c2_gradient(dev, steps=args.steps, warm=args.warmup)), flush=True)
        else:
            from ptylab_gb300 import _native

            CONFIG_STEPS[args.config] = (args.steps, args.warmup)
            out = measure_config(args.config, dev, _native.require(0), with_cpu=not args.no_cpu_baseline)
            print(json.dumps(out), flush=True)
        return
    if args.calibration:
        print(json.dumps(run_calibration(args)), flush=True)
        return
    if args.network:
        print(json.dumps(run_network(args)), flush=True)
        return
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            # reference CPU steps are ~1 s each: cap the sample so the run stays within minutes
            args.steps = min(args.steps, 10)
            print(json.dumps(run_reference(args)), flush=True)
        return

    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    out = run_gb300(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

"""The benchmark configurations as parity cases: engine runs on the GPU and
oracle runs (complex64 and complex128) on the host, from the same seeded
data and initial guesses (ptylab_gb300.simulate.config_problem).

The two oracle precisions run in parallel spawned processes (the inputs are
passed to them, not re-simulated), so a configuration-size case costs about
the slower of the two oracle runs.
"""

from __future__ import annotations

import copy
import multiprocessing as mp
from concurrent.futures import ProcessPoolExecutor

import numpy as np

ORACLE_KW = {
    "C0": {},
    "C1": {"order": "random", "alphaObject": 0.25, "alphaProbe": 0.25},
    "C2": {},
    "C3": {"order": "NA", "operationMode": "FPM", "probeBoundary": True},
}

_PROBLEMS: dict = {}


def problem(name, **spec_overrides):
    """(engine name, ExperimentalData, Params, Reconstruction) of configuration
    `name`, cached per process; callers get deep copies."""
    from ptylab_gb300 import simulate as S

    key = (name, tuple(sorted(spec_overrides.items())))
    if key not in _PROBLEMS:
        if spec_overrides:
            spec = S.config_spec(name)
            for k, v in spec_overrides.items():
                setattr(spec, k, v)
            if name == "C3":
                d, p, rec, _, _ = S.fpm_problem(spec)
            else:
                d, p, rec, _, _ = S.cpm_problem(spec)
            if name == "C1":
                p.positionOrder = "random"
            _PROBLEMS[key] = (S.CONFIG_ENGINES[name], d, p, rec)
        else:
            _PROBLEMS[key] = S.config_problem(name)
    eng, d, p, rec = _PROBLEMS[key]
    return eng, copy.deepcopy(d), copy.deepcopy(p), copy.deepcopy(rec)


def oracle_inputs(name, engine, d, rec, **settings):
    g = dict(Np=int(rec.Np), No=int(rec.No), dxp=float(rec.dxp), wavelength=float(rec.wavelength), zo=float(rec.zo),
             npsm=int(rec.npsm), nslice=int(rec.nslice), dz=float(getattr(rec, "dz", 0.0) or 0.0))
    s = dict(engine=engine, entrancePupilDiameter=float(d.entrancePupilDiameter or 0.0), **ORACLE_KW[name])
    s.update(settings)
    return dict(geometry=g, settings=s, object=rec.object.copy(), probe=rec.probe.copy(),
                ptychogram=d.ptychogram, positions=np.asarray(rec.positions).copy(), energyAtPos=d.energyAtPos)


def _oracle_worker(args):
    inputs, iters, seed, complex_dtype = args
    import os

    os.environ["OMP_NUM_THREADS"] = "1"
    from oracle import ptyoracle as O

    cdt = np.dtype(complex_dtype)
    fdt = np.float64 if cdt == np.complex128 else np.float32
    g = O.Geometry(**inputs["geometry"])
    s = O.Settings(**inputs["settings"])
    st = O.State(object=inputs["object"].astype(cdt), probe=inputs["probe"].astype(cdt))
    np.random.seed(seed)
    eng = O.OracleEngine(s, g, st, inputs["ptychogram"].astype(fdt), inputs["positions"], inputs["energyAtPos"])
    st = eng.reconstruct(iters)
    return {k: np.asarray(getattr(st, k)) for k in ("object", "probe", "error")}


def oracle_pair(inputs, iters, seed):
    """(complex64 run, complex128 run) of the oracle, in two spawned processes."""
    ctx = mp.get_context("spawn")
    with ProcessPoolExecutor(max_workers=2, mp_context=ctx) as ex:
        futs = [ex.submit(_oracle_worker, (inputs, iters, seed, dt)) for dt in ("complex64", "complex128")]
        return futs[0].result(), futs[1].result()


def gpu_run(engine_name, d, p, rec, iters, seed, batch=False, name=None):
    """The GB300 engine from PtyLab's surface: reconstruct() (the single-scan
    latency shape) or reconstruct_batch([engine]) (the many-scan throughput
    shape: fewer, wider CTAs per scan, probe rows in shared memory)."""
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import configure_engine

    eng = getattr(Engines, engine_name)(rec, d, p, DummyMonitor())
    if name is not None:
        configure_engine(name, eng, iters)
    else:
        eng.numIterations = iters
    np.random.seed(seed)
    if batch:
        Engines.reconstruct_batch([eng])
    else:
        eng.reconstruct()
    return {k: np.asarray(getattr(rec, k)) for k in ("object", "probe", "error")}

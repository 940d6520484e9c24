"""GB300 engines against the reference's own outputs (fixtures) and the oracle.

Parity metric: relative Frobenius error, as in the reference's GPU-vs-CPU
test (tests/regression/test_engine_regression.py:140-175).  The reference
accepts 1e-3 there (its CuPy/cuFFT path measured 1e-8 ... 2.2e-4); this suite
uses the same 1e-3 bound on the 2-5 iteration fixtures and records the
measured values in the assertion messages.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import fixture_names, load_fixture, platform_reproduces_order, rel_err
from test_host_logic import containers

pytestmark = pytest.mark.gpu
TOL_FIXTURE = 1e-3
IN_SCOPE = fixture_names("reg_") + fixture_names("scan_")


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def run_fixture_gpu(fx, engine_name=None, iters=None, attrs=None):
    from ptylab_gb300 import DummyMonitor, Engines

    m, i, d, p, rec = containers(fx)
    rec.initialGuessObject = i["init_object"].copy()
    rec.initialGuessProbe = i["init_probe"].copy()
    rec.object = i["init_object"].copy()
    rec.probe = i["init_probe"].copy()
    eng = getattr(Engines, engine_name or str(m["engine"]))(rec, d, p, DummyMonitor())
    eng.numIterations = int(m["iters"]) if iters is None else iters
    for k, v in (attrs or {}).items():
        setattr(eng, k, v)
    if "momentum_method" in m and str(m["engine"]) == "mqNewton":
        eng.momentum_method = str(m["momentum_method"])
    np.random.seed(int(m["seed"]))
    eng.reconstruct()
    run_fixture_gpu.params = p
    return rec, eng


def reference_spread(fx):
    """The reference's own FP32 noise floor on this case: how far its
    complex64 result lies from a complex128 oracle run from the same inputs,
    or from a complex64 oracle run whose initial probe differs by one part in
    1e7 (a rounding-level change), whichever is larger.  The second term
    matters only where the case amplifies rounding (a strongly mismatched
    start, e.g. the unsquared constraints after probe-power correction);
    elsewhere it is orders of magnitude below the first."""
    from oracle import ptyoracle as O

    st = O.run_fixture(fx, dtype=np.complex128)
    moved = dict(fx)
    p = fx["in_init_probe"]
    moved["in_init_probe"] = (p * (1 + 1e-7 * np.random.default_rng(0).standard_normal(p.shape))).astype(p.dtype)
    st2 = O.run_fixture(moved)
    keys = ("object", "probe", "error", "errorAtPos", "background", "intensityScaling", "reference")
    return {
        k: max(rel_err(fx[f"out_{k}"], getattr(st, k)), rel_err(fx[f"out_{k}"], getattr(st2, k)))
        for k in keys
        if f"out_{k}" in fx
    }


@pytest.mark.parametrize("name", IN_SCOPE)
def test_engine_matches_reference_fixture(torch_cuda, name):
    """GB300 result vs the reference's own result: within max(1e-3, 3 x the
    reference's complex64-vs-complex128 spread on the same case).  Where this
    platform's np.argsort orders tied 'NA' positions differently from the
    recording platform, the reference is not reproducible here and the
    comparison is against the oracle (the reference's algorithm) on this platform."""
    from oracle import ptyoracle as O

    fx = load_fixture(name)
    rec, _ = run_fixture_gpu(fx)
    if platform_reproduces_order(fx):
        target = {k: fx[f"out_{k}"] for k in ("object", "probe", "error", "errorAtPos", "objectMomentum", "probeMomentum") if f"out_{k}" in fx}
        floor = reference_spread(fx)
    else:
        st64, st128 = O.run_fixture(fx), O.run_fixture(fx, dtype=np.complex128)
        target = {k: getattr(st64, k) for k in ("object", "probe", "error", "errorAtPos", "objectMomentum", "probeMomentum") if getattr(st64, k, None) is not None}
        floor = {k: rel_err(target[k], getattr(st128, k)) for k in ("object", "probe", "error", "errorAtPos")}
    errs = {k: rel_err(getattr(rec, k), target[k]) for k in ("object", "probe", "error", "errorAtPos")}
    assert rec.object.dtype == np.complex64 and rec.probe.dtype == np.complex64
    assert rec.object.shape == fx["out_object"].shape and rec.probe.shape == fx["out_probe"].shape
    bad = {k: (errs[k], floor[k]) for k in errs if errs[k] >= max(TOL_FIXTURE, 3 * floor[k])}
    assert not bad, f"{name}: (error, reference c64-vs-c128 spread) {bad}"
    if "out_detectorError" in fx:
        assert rel_err(rec.detectorError, fx["out_detectorError"]) < TOL_FIXTURE
    if "objectMomentum" in target:
        assert rel_err(rec.objectMomentum, target["objectMomentum"]) < max(1e-2, 3 * floor["object"])
        assert rel_err(rec.probeMomentum, target["probeMomentum"]) < max(1e-2, 3 * floor["probe"])
    if "out_reference" in fx:
        # the interferometric reference field (BaseEngine.py:975-982), per mode
        assert rec.reference.shape == fx["out_reference"].shape
        assert rel_err(rec.reference, fx["out_reference"]) < max(TOL_FIXTURE, 3 * floor["reference"])
    for key in ("background", "intensityScaling"):
        if f"out_{key}" in fx and platform_reproduces_order(fx):
            got = rec.background if key == "background" else run_fixture_gpu.params.intensityScaling
            assert rel_err(got, fx[f"out_{key}"]) < max(TOL_FIXTURE, 3 * floor[key]), (key, rel_err(got, fx[f"out_{key}"]), floor[key])
    if str(fx["meta_engine"]) == "mqNewton":
        # the object buffer equals the final object; the probe buffer is the
        # probe before the last iteration's constraints; the second moments
        # are uniform arrays
        np.testing.assert_array_equal(rec.objectBuffer, rec.object)
        if "out_probeBuffer" in fx and platform_reproduces_order(fx):
            assert rel_err(rec.probeBuffer, fx["out_probeBuffer"]) < max(TOL_FIXTURE, 3 * floor["probe"])
        for key, part in (("objectMomentum_v", "object"), ("probeMomentum_v", "probe")):
            if f"out_{key}" in fx and platform_reproduces_order(fx):
                assert getattr(rec, key).shape == fx[f"out_{key}"].shape
                assert rel_err(getattr(rec, key), fx[f"out_{key}"]) < max(1e-2, 3 * floor[part]), key


@pytest.mark.parametrize("name", ["scan_epie_asp", "scan_epie_asp_denoise_background", "reg_epie_asp"])
def test_asp_table_placement_agrees(torch_cuda, name):
    """The ASP transfer function's CTA columns copied into shared memory once
    per launch by the bulk-copy engine (asp_table_in_smem = 2, the default
    where it fits) or read from global memory at every position (1): the same
    reconstruction bit for bit, and both at the reference's result."""
    fx = load_fixture(name)
    rec_g, _ = run_fixture_gpu(fx, attrs={"aspTableInSmem": 1})
    rec_s, _ = run_fixture_gpu(fx, attrs={"aspTableInSmem": 2})
    for k in ("object", "probe", "error"):
        np.testing.assert_array_equal(np.asarray(getattr(rec_g, k)), np.asarray(getattr(rec_s, k)))
    if platform_reproduces_order(fx):
        floor = reference_spread(fx)
        assert rel_err(rec_s.object, fx["out_object"]) < max(TOL_FIXTURE, 3 * floor["object"])


def test_engine_runs_are_deterministic(torch_cuda):
    """Same inputs, same launch: bitwise identical results (no atomics on data paths)."""
    fx = load_fixture("scan_qnewton_fpm")
    a, _ = run_fixture_gpu(fx)
    for _ in range(3):
        b, _ = run_fixture_gpu(fx)
        np.testing.assert_array_equal(a.object, b.object)
        np.testing.assert_array_equal(a.probe, b.probe)
        np.testing.assert_array_equal(a.error, b.error)


def test_stepwise_equals_reconstruct(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_random")
    rec_a, _ = run_fixture_gpu(fx)
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    eng = Engines.ePIE(rec, d, p, DummyMonitor())
    eng.numIterations = int(m["iters"])
    np.random.seed(int(m["seed"]))
    steps = list(eng.reconstruct_stepwise())
    assert len(steps) == int(m["iters"]) * d.numFrames
    np.testing.assert_array_equal(rec.object, rec_a.object)
    np.testing.assert_array_equal(rec.probe, rec_a.probe)
    np.testing.assert_array_equal(rec.error, rec_a.error)


def test_unsupported_switch_raises(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_asp")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    p.intensityConstraint = "interferometric"  # with ASP: not on this path
    eng = Engines.ePIE(rec, d, p, DummyMonitor())
    with pytest.raises(NotImplementedError):
        eng.reconstruct()
    p.propagatorType = "Fraunhofer"
    rec.initialGuessObject, rec.initialGuessProbe = i["init_object"].copy(), i["init_probe"].copy()
    with pytest.raises(NotImplementedError):  # with mqNewton: not on this path
        Engines.mqNewton(rec, d, p, DummyMonitor()).reconstruct()
    p.intensityConstraint = "sigmoid"  # not a constraint PtyLab knows (BaseEngine.py:963-964)
    with pytest.raises(ValueError):
        Engines.ePIE(rec, d, p, DummyMonitor()).reconstruct()


def test_asp_with_fftshift_raises_value_error(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_asp")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    p.fftshiftSwitch = True
    with pytest.raises(ValueError):
        Engines.ePIE(rec, d, p, DummyMonitor()).reconstruct()


def test_position_outside_object_raises(torch_cuda):
    from ptylab_gb300 import DummyMonitor, Engines

    fx = load_fixture("scan_epie_random")
    m, i, d, p, rec = containers(fx)
    rec.object, rec.probe = i["init_object"].copy(), i["init_probe"].copy()
    rec.encoder_corrected = rec.encoder_corrected * 100
    with pytest.raises(ValueError):
        Engines.ePIE(rec, d, p, DummyMonitor()).reconstruct()


@pytest.mark.parametrize("engine", ["ePIE", "qNewton", "mqNewton"])
def test_reconstruct_batch_equals_single_engines(torch_cuda, engine):
    """Engines.reconstruct_batch (one launch per iteration for all scans)
    gives every scan what its own reconstruct() gives (sequential order: no
    RNG between the engines).  The batch runs the many-scan kernel shape
    (fewer, wider CTAs per scan); every sum that feeds the updates is formed
    in a tree fixed by the patch size, so object, probe and detector error
    are bit-identical, and only the error metric can differ in its last
    bits: each thread sums its pixels' |I_meas - I_est| in FP32 before the
    FP64 CTA and frame sums, and the batch shape gives a thread more pixels
    (at Np = 64 the whole patch is one CTA: 16 pixels per thread)."""
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    def engines():
        out = []
        for g in range(3):
            d, p, rec, _, _ = cpm_problem(ScanSpec(Np=64, No=192, num_positions=30, seed=300 + g), engine_seed=g)
            e = getattr(Engines, engine)(rec, d, p, DummyMonitor())
            e.numIterations = 3
            out.append(e)
        return out

    single = engines()
    for e in single:
        e.reconstruct()
    batch = engines()
    Engines.reconstruct_batch(batch)
    for a, b in zip(single, batch):
        ra, rb = a.reconstruction, b.reconstruction
        assert isinstance(rb.object, np.ndarray) and rb.object.dtype == np.complex64
        np.testing.assert_array_equal(rb.object, ra.object)
        np.testing.assert_array_equal(rb.probe, ra.probe)
        np.testing.assert_array_equal(rb.detectorError, ra.detectorError)
        assert rel_err(np.asarray(rb.error), np.asarray(ra.error)) < 1e-8


def test_batched_scans_equal_single_runs(torch_cuda):
    """G independent scans in one launch (one cluster each) reproduce G single-scan launches bitwise."""
    torch = torch_cuda
    from ptylab_gb300 import _native
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    lib = _native.require(0)
    G, Np, No, nf = 3, 64, 192, 30
    scans = []
    for g in range(G):
        d, p, rec, _, _ = cpm_problem(ScanSpec(Np=Np, No=No, num_positions=nf, seed=100 + g), engine_seed=g)
        scans.append((d, rec))

    def run(scan_ids):
        geom = _native.Geometry(Np=Np, No=No, nosm=1, npsm=1, nslice=1, num_frames=nf, num_scans=len(scan_ids),
                                engine=0, propagator=0, fftshift=0, fpm=0, cluster=0)
        plan = C.c_void_p()
        _native.check(lib.ptyg_plan_create(C.byref(geom), C.byref(plan)))
        keep, outs = [], []
        for s, g in enumerate(scan_ids):
            d, rec = scans[g]
            obj = torch.from_numpy(rec.object.copy()).cuda()
            prb = torch.from_numpy(rec.probe.copy()).cuda()
            pos = torch.from_numpy(rec.positions.astype(np.int32)).cuda()
            order = torch.arange(nf, dtype=torch.int32, device="cuda")
            data = torch.from_numpy(d.ptychogram).cuda()
            b = _native.ScanBuffers(object=obj.data_ptr(), probe=prb.data_ptr(), positions=pos.data_ptr(),
                                    order=order.data_ptr())
            _native.check(lib.ptyg_plan_bind_scan(plan, s, C.byref(b), data.data_ptr(), None))
            keep += [obj, prb, pos, order, data, b]
            outs.append((obj, prb))
        u = _native.UpdateParams(beta_object=0.25, beta_probe=0.25, probe_weight=1.0)
        for _ in range(3):
            _native.check(lib.ptyg_plan_run(plan, C.byref(u), 0, nf, 0, None))
        torch.cuda.synchronize()
        lib.ptyg_plan_destroy(plan)
        return [(o.cpu().numpy(), q.cpu().numpy()) for o, q in outs]

    batched = run(list(range(G)))
    for g in range(G):
        single = run([g])[0]
        np.testing.assert_array_equal(batched[g][0], single[0])
        np.testing.assert_array_equal(batched[g][1], single[1])


@pytest.mark.parametrize("engine", ["ePIE", "mPIE"])
def test_config0_size_precision_vs_complex128(torch_cuda, engine):
    """Np=64, No=256, 100 Fermat positions, 20 iterations from the same seeded
    guesses.  Precision statement: the GB300 FP32 result is as close to a
    complex128 oracle run as the reference's own complex64 path is (within 3x:
    mPIE and qNewton amplify rounding chaotically, so two FP32 implementations
    land at random distances of the same order from the exact answer)."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    d, p, rec, _, _ = cpm_problem(ScanSpec())
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    eng = getattr(Engines, engine)(rec, d, p, DummyMonitor())
    eng.numIterations = 20
    np.random.seed(5)
    eng.reconstruct()
    g = O.Geometry(Np=64, No=256, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = O.Settings(engine=engine, entrancePupilDiameter=d.entrancePupilDiameter)

    def oracle(cdt, fdt):
        st = O.State(object=obj0.astype(cdt), probe=prb0.astype(cdt))
        np.random.seed(5)
        return O.OracleEngine(s, g, st, d.ptychogram.astype(fdt), rec.positions, d.energyAtPos).reconstruct(20)

    r64, r128 = oracle(np.complex64, np.float32), oracle(np.complex128, np.float64)
    keys = ("object", "probe", "error")
    gpu_vs_128 = {k: rel_err(getattr(rec, k), getattr(r128, k)) for k in keys}
    ref_vs_128 = {k: rel_err(getattr(r64, k), getattr(r128, k)) for k in keys}
    gpu_vs_64 = {k: rel_err(getattr(rec, k), getattr(r64, k)) for k in keys}
    msg = f"{engine}: gpu-c128 {gpu_vs_128} ref-c128 {ref_vs_128} gpu-ref {gpu_vs_64}"
    print(msg)
    # the 1e-4 parity target wherever the reference's own spread leaves room for
    # it (ePIE object and error curve), else a small multiple of that spread
    chaos = 4.0 if engine == "mPIE" else 3.0
    for k in keys:
        assert gpu_vs_128[k] <= 3 * ref_vs_128[k] + 1e-6 or gpu_vs_128[k] <= 1e-4, msg
        assert gpu_vs_64[k] <= max(1e-4, chaos * ref_vs_128[k]), msg


def test_config3_fpm_qnewton_precision_vs_complex128(torch_cuda):
    """FPM qNewton at the LED-array configuration (15 x 15 LEDs, Np = 128,
    No = 512, NA order, probeBoundary), 5 iterations: the GB300 result is as
    close to a complex128 oracle run as the reference's complex64 path."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import FPMSpec, fpm_problem

    d, p, rec, _, _ = fpm_problem(FPMSpec())
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    positions = rec.positions.copy()
    eng = Engines.qNewton(rec, d, p, DummyMonitor())
    eng.numIterations = 5
    eng.reconstruct()
    g = O.Geometry(Np=128, No=512, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = O.Settings(engine="qNewton", order="NA", operationMode="FPM", probeBoundary=True,
                   entrancePupilDiameter=d.entrancePupilDiameter)

    def oracle(cdt, fdt):
        st = O.State(object=obj0.astype(cdt), probe=prb0.astype(cdt))
        return O.OracleEngine(s, g, st, d.ptychogram.astype(fdt), positions, d.energyAtPos).reconstruct(5)

    r64, r128 = oracle(np.complex64, np.float32), oracle(np.complex128, np.float64)
    keys = ("object", "probe", "error")
    gpu_vs_128 = {k: rel_err(getattr(rec, k), getattr(r128, k)) for k in keys}
    ref_vs_128 = {k: rel_err(getattr(r64, k), getattr(r128, k)) for k in keys}
    msg = f"qNewton FPM: gpu-c128 {gpu_vs_128} ref-c128 {ref_vs_128}"
    print(msg)
    for k in keys:
        assert gpu_vs_128[k] <= 3 * ref_vs_128[k] + 5e-4, msg


@pytest.mark.parametrize("denoise", [False, True])
def test_config3_fpm_mqnewton_nadam_precision_vs_complex128(torch_cuda, denoise):
    """The FPM example's engine (mqNewton, NADAM, beta1 = beta2 = 0.5,
    exampleReconstructionFPM.py:54-75, with and without its adaptive
    denoising) at the LED-array configuration, 3 iterations: every position
    adds a momentum step over the whole 512 x 512 spectrum.  The GB300 result
    is as close to a complex128 oracle run as the reference's complex64 path."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import FPMSpec, fpm_problem

    d, p, rec, _, _ = fpm_problem(FPMSpec())
    p.adaptiveDenoisingSwitch = denoise
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    positions = rec.positions.copy()
    eng = Engines.mqNewton(rec, d, p, DummyMonitor())
    eng.momentum_method = "NADAM"
    eng.numIterations = 3
    eng.reconstruct()
    g = O.Geometry(Np=128, No=512, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo)
    s = O.Settings(engine="mqNewton", momentum_method="NADAM", order="NA", operationMode="FPM",
                   probeBoundary=True, entrancePupilDiameter=d.entrancePupilDiameter,
                   adaptiveDenoisingSwitch=denoise)

    def oracle(cdt, fdt):
        st = O.State(object=obj0.astype(cdt), probe=prb0.astype(cdt))
        return O.OracleEngine(s, g, st, d.ptychogram.astype(fdt), positions, d.energyAtPos).reconstruct(3)

    r64, r128 = oracle(np.complex64, np.float32), oracle(np.complex128, np.float64)
    keys = ("object", "probe", "error", "objectMomentum", "probeMomentum")
    gpu_vs_128 = {k: rel_err(getattr(rec, k), getattr(r128, k)) for k in keys}
    ref_vs_128 = {k: rel_err(getattr(r64, k), getattr(r128, k)) for k in keys}
    msg = f"mqNewton FPM: gpu-c128 {gpu_vs_128} ref-c128 {ref_vs_128}"
    print(msg)
    for k in keys:
        assert gpu_vs_128[k] <= 3 * ref_vs_128[k] + 5e-4, msg
    assert rel_err(rec.objectMomentum_v, r128.objectMomentum_v) <= 3 * rel_err(r64.objectMomentum_v, r128.objectMomentum_v) + 1e-4


@pytest.mark.parametrize("pad", [0, 1])
@pytest.mark.parametrize("method", ["ADAM", "NADAM", "momentum"])
def test_mqnewton_positions_match_oracle(torch_cuda, pad, method):
    """mqNewton's kernel position by position through the C ABI: the first
    eight positions of an iteration against the oracle stepping through the
    same positions.  Whole iterations of these CPM scans are chaotic (a 1-ulp
    change of the initial object moves the result by 1e-2 after three
    iterations, in the reference too), so the arithmetic is pinned here before
    rounding differences can grow.  pad=1 grows the object by one row and
    column: an odd size takes the 8-byte path of the momentum step, an even
    one the 16-byte path."""
    torch = torch_cuda
    from oracle import ptyoracle as O
    from ptylab_gb300 import _native

    fx = load_fixture("scan_mqnewton_adam")
    i = {k[3:]: fx[k] for k in fx if k.startswith("in_")}
    Np, No = int(i["Np"]), int(i["No"]) + pad
    obj0 = np.ones((1, 1, 1, 1, No, No), np.complex64)
    obj0[..., : No - pad, : No - pad] = i["init_object"]
    prb0 = i["init_probe"].astype(np.complex64)
    data = i["ptychogram"].astype(np.float32)
    positions = i["positions"].astype(np.int32)
    nf, npos = data.shape[0], 8
    order = np.arange(nf, dtype=np.int32)

    lib = _native.require(0)
    geom = _native.Geometry(Np=Np, No=No, nosm=1, npsm=1, nslice=1, num_frames=nf, num_scans=1,
                            engine=_native.ENGINES["mqNewton"], propagator=0, fftshift=0, fpm=0, cluster=0)
    plan = C.c_void_p()
    _native.check(lib.ptyg_plan_create(C.byref(geom), C.byref(plan)))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    t = dict(obj=dev(obj0), prb=dev(prb0), pos=dev(positions), order=dev(order), data=dev(data))
    t.update(omom=torch.zeros_like(t["obj"]), pbuf=t["prb"].clone(), pmom=torch.zeros_like(t["prb"]),
             m2=torch.zeros(2, dtype=torch.float32, device="cuda"))
    b = _native.ScanBuffers(object=t["obj"].data_ptr(), probe=t["prb"].data_ptr(), positions=t["pos"].data_ptr(),
                            order=t["order"].data_ptr(), object_momentum=t["omom"].data_ptr(),
                            probe_buffer=t["pbuf"].data_ptr(), probe_momentum=t["pmom"].data_ptr(),
                            second_moment=t["m2"].data_ptr())
    _native.check(lib.ptyg_plan_bind_scan(plan, 0, C.byref(b), t["data"].data_ptr(), None))
    u = _native.UpdateParams(beta_object=1, beta_probe=1, reg_object=1, reg_probe=1, friction=0.7, probe_weight=1,
                             momentum_method=_native.MOMENTUM_METHODS[method], beta1=0.5, beta2=0.5,
                             beta1_scale=0.5, beta2_scale=0.5, beta_object_m=0.25, beta_probe_m=0.25)
    _native.check(lib.ptyg_plan_run(plan, C.byref(u), 0, npos, 0, None))
    torch.cuda.synchronize()
    st_gpu = C.c_int()
    _native.check(lib.ptyg_plan_status(plan, 0, C.byref(st_gpu), None))
    lib.ptyg_plan_destroy(plan)
    assert st_gpu.value == 0
    gpu = {k: t[n].cpu().numpy() for k, n in (("object", "obj"), ("probe", "prb"), ("objectMomentum", "omom"),
                                              ("probeMomentum", "pmom"))}

    def oracle(cdt, fdt):
        g = O.Geometry(Np=Np, No=No, dxp=float(i["dxp"]), wavelength=float(i["wavelength"]), zo=float(i["zo"]))
        s = O.Settings(engine="mqNewton", momentum_method=method, entrancePupilDiameter=float(i["entrancePupilDiameter"]))
        st = O.State(object=obj0.astype(cdt), probe=prb0.astype(cdt))
        eng = O.OracleEngine(s, g, st, data.astype(fdt), positions, i["energyAtPos"])
        eng.prepare()
        if method != "momentum":
            st.objectMomentum_v = np.zeros_like(st.object)
            st.probeMomentum_v = np.zeros_like(st.probe)
        for j in order[:npos]:
            eng.position(int(j))
        return st

    r64, r128 = oracle(np.complex64, np.float32), oracle(np.complex128, np.float64)
    errs = {k: rel_err(gpu[k], getattr(r64, k)) for k in gpu}
    floor = {k: rel_err(getattr(r64, k), getattr(r128, k)) for k in gpu}
    msg = f"mqNewton {method} No={No}, {npos} positions: gpu-ref {errs} ref-c128 {floor}"
    print(msg)
    for k in gpu:
        assert errs[k] < max(1e-4, 3 * floor[k]), msg
    assert abs(float(t["m2"][0]) - float(np.real(r64.objectMomentum_v.flat[0]))) <= 1e-4 * abs(
        float(np.real(r64.objectMomentum_v.flat[0]))) if method != "momentum" else True


def _run_plan_c1(torch, cluster, nf=40, iters=3):
    """mPIE, npsm = 4, Np = 128 through the C ABI with a given cluster size."""
    from ptylab_gb300 import _native
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    lib = _native.require(0)
    d, p, rec, _, _ = cpm_problem(ScanSpec(Np=128, No=320, num_positions=nf, npsm=4, probe_radius_fraction=0.25,
                                           step_fraction=0.3, seed=3))
    geom = _native.Geometry(Np=128, No=320, nosm=1, npsm=4, nslice=1, num_frames=nf, num_scans=1,
                            engine=_native.ENGINES["mPIE"], propagator=0, fftshift=0, fpm=0, cluster=cluster)
    plan = C.c_void_p()
    _native.check(lib.ptyg_plan_create(C.byref(geom), C.byref(plan)))
    cl, th, sm, mx = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    _native.check(lib.ptyg_plan_info(plan, C.byref(cl), C.byref(th), C.byref(sm), C.byref(mx)))
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)  # noqa: E731
    obj, prb = t(rec.object, torch.complex64), t(rec.probe, torch.complex64)
    bufs = [obj.clone(), torch.zeros_like(obj), prb.clone(), torch.zeros_like(prb)]
    pos, data = t(rec.positions.astype(np.int32), torch.int32), t(d.ptychogram, torch.float32)
    rs = np.random.RandomState(0)
    order = t(np.concatenate([rs.permutation(nf) for _ in range(iters)]).astype(np.int32), torch.int32)
    flags = t((rs.rand(iters * nf) > 0.8).astype(np.uint8), torch.uint8)
    b = _native.ScanBuffers(object=obj.data_ptr(), probe=prb.data_ptr(), positions=pos.data_ptr(), order=order.data_ptr(),
                            momentum_flags=flags.data_ptr(), object_buffer=bufs[0].data_ptr(),
                            object_momentum=bufs[1].data_ptr(), probe_buffer=bufs[2].data_ptr(),
                            probe_momentum=bufs[3].data_ptr())
    _native.check(lib.ptyg_plan_bind_scan(plan, 0, C.byref(b), data.data_ptr(), None))
    _native.check(lib.ptyg_plan_set_order(plan, 0, order.data_ptr(), flags.data_ptr(), iters * nf, None))
    u = _native.UpdateParams(beta_object=0.25, beta_probe=0.25, alpha_object=0.25, alpha_probe=0.25, friction=0.7,
                             feedback=0.3, probe_weight=1.0)
    for k in range(iters):
        _native.check(lib.ptyg_plan_run(plan, C.byref(u), k * nf, nf, 0, None))
    torch.cuda.synchronize()
    lib.ptyg_plan_destroy(plan)
    return cl.value, sm.value, obj.cpu().numpy(), prb.cpu().numpy(), bufs[1].cpu().numpy()


def test_cluster_shapes_agree(torch_cuda):
    """16-CTA clusters (probe rows in shared memory) and 8-CTA clusters (probe
    rows left in global memory, for layouts that exceed a CTA's shared memory)
    compute the same reconstruction bit for bit."""
    c16 = _run_plan_c1(torch_cuda, 16)
    c8 = _run_plan_c1(torch_cuda, 8)
    assert (c16[0], c8[0]) == (16, 8)
    for a, b in zip(c16[2:], c8[2:]):
        np.testing.assert_array_equal(a, b)


def test_config2_size_e3pie_precision_vs_complex128(torch_cuda):
    """Multislice at the config-2 field size: Np = 256, four weak-phase slices
    10 um apart, 13.5 nm wavelength, 20 nm pixels; 24 positions, 3 iterations.
    The GB300 result is as close to a complex128 oracle run as the
    reference's complex64 path (within 3x)."""
    from oracle import ptyoracle as O
    from ptylab_gb300 import DummyMonitor, Engines
    from ptylab_gb300.simulate import ScanSpec, cpm_problem

    spec = ScanSpec(Np=256, No=384, num_positions=24, probe_radius_fraction=0.2, step_fraction=0.35,
                    wavelength=13.5e-9, zo=0.05, dxd=13.5e-9 * 0.05 / (256 * 20e-9), photons=1e5, phase_max=0.3, seed=9)
    d, p, rec, _, _ = cpm_problem(spec)
    rec.nslice = 4
    rec.dz = 10e-6
    rec.refrIndex = 1.0
    np.random.seed(4)
    rec.initializeObjectProbe()
    obj0, prb0 = rec.object.copy(), rec.probe.copy()
    eng = Engines.e3PIE(rec, d, p, DummyMonitor())
    eng.numIterations = 3
    eng.reconstruct()
    g = O.Geometry(Np=256, No=384, dxp=rec.dxp, wavelength=rec.wavelength, zo=rec.zo, nslice=4, dz=10e-6)
    s = O.Settings(engine="e3PIE", entrancePupilDiameter=d.entrancePupilDiameter)

    def oracle(cdt, fdt):
        st = O.State(object=obj0.astype(cdt), probe=prb0.astype(cdt))
        return O.OracleEngine(s, g, st, d.ptychogram.astype(fdt), rec.positions, d.energyAtPos).reconstruct(3)

    r64, r128 = oracle(np.complex64, np.float32), oracle(np.complex128, np.float64)
    keys = ("object", "probe", "error")
    gpu_vs_128 = {k: rel_err(getattr(rec, k), getattr(r128, k)) for k in keys}
    ref_vs_128 = {k: rel_err(getattr(r64, k), getattr(r128, k)) for k in keys}
    gpu_vs_64 = {k: rel_err(getattr(rec, k), getattr(r64, k)) for k in keys}
    msg = f"e3PIE C2 size: gpu-c128 {gpu_vs_128} ref-c128 {ref_vs_128} gpu-ref {gpu_vs_64}"
    print(msg)
    for k in keys:
        assert gpu_vs_128[k] <= 3 * ref_vs_128[k] + 1e-5, msg
    assert rec.objectProd.shape == (1, 1, 1, 384, 384)


@pytest.mark.parametrize("propagator,modes", [("polychromeASP", (2, 1, 2)), ("Fraunhofer", (3, 1, 1)),
                                              ("polychromeASP", (2, 2, 1))])
def test_several_wavelengths_follow_the_oracle_on_a_moving_scan(torch_cuda, propagator, modes):
    """ePIE over several wavelengths on the Fermat scan (the regression
    dataset's frames all sit at one position): the GPU against the oracle
    (the reference's algorithm, checked bit-exact against the reference's
    polychrome golden) from the same seeded start, 2 iterations."""
    from oracle import ptyoracle as O

    fx = dict(load_fixture("scan_epie_random"))
    nl, nos, nps = modes
    m, i, d, p, rec = containers(fx)
    rec.nlambda, rec.nosm, rec.npsm = nl, nos, nps
    rec.spectralDensity = float(np.atleast_1d(rec.wavelength)[0]) * np.linspace(0.98, 1.02, nl)
    np.random.seed(int(fx["meta_seed"]))
    rec.initializeObjectProbe()
    fx["meta_modes"] = np.array([nl, nos, nps, 1])
    fx["meta_propagator"] = np.asarray(propagator)
    fx["meta_iters"] = np.asarray(2)
    fx["in_spectralDensity"] = np.asarray(rec.spectralDensity)
    fx["in_init_object"], fx["in_init_probe"] = rec.object.copy(), rec.probe.copy()
    got, _ = run_fixture_gpu(fx)
    want, want128 = O.run_fixture(fx), O.run_fixture(fx, dtype=np.complex128)
    for key in ("object", "probe", "error"):
        e = rel_err(getattr(got, key), getattr(want, key))
        floor = rel_err(getattr(want, key), getattr(want128, key))
        assert e < max(1e-4, 3 * floor), (key, e, floor)

"""GPU parity of the tensor-core vertical pass (exact integer digit products
on bf16 operands, tcgen05): output bytes against the CPU oracle and the
reference's golden digests, with the pass forced on ("gpu:vertical" =
"tensor") wherever the layout allows it, and the statistics confirming that
it ran.  Integer output must be byte-identical."""
import ctypes as C
import hashlib

import numpy as np
import pytest

from conftest import load_workload_digests
from imageworsener_gb300 import workloads as W
from imageworsener_gb300.iwapi import Job, IMGTYPE_GRAY, IMGTYPE_RGB, CT_ALL, DITHER_ORDERED, _collect, run_job
import iwcases

pytestmark = pytest.mark.gpu

# downscale filters (family, p1, p2): every one has windows that close in order
TC_FILTERS = [("lanczos", 3, 0), ("lanczos", 2, 0), ("lanczos", 5, 0), ("hanning", 3, 0), ("blackman", 4, 0),
              ("cubic", 1 / 3, 1 / 3), ("cubic", 0, 0.5), ("hermite", 0, 0), ("boxavg", 0, 0), ("triangle", 0, 0),
              ("quadratic", 0, 0), ("gaussian", 0, 0)]


def tensor_case(seed: int) -> Job:
    """An 8-bit gray or RGB downscale with a ragged width (strips of 128 byte
    columns end part-way), a vertical factor from 1.5 to 40 and sometimes a
    crop, ordered dither or a reduced colour count."""
    rng = np.random.default_rng(seed)
    imgtype = IMGTYPE_RGB if rng.random() < 0.7 else IMGTYPE_GRAY
    w = int(rng.integers(1, 420))
    oh = int(rng.integers(1, 40))
    h = int(min(1400, max(oh + 1, round(oh * rng.uniform(1.5, 40.0)))))
    ow = int(rng.integers(1, max(2, w)))
    px, bpr = iwcases.make_pixels(rng, imgtype, 8, w, h, str(rng.choice(["mixed", "smooth", "noise"])))
    calls = [("iw_set_output_profile", int(rng.choice([iwcases.PPM, iwcases.PNG, iwcases.PAM]))),
             ("iw_set_output_canvas_size", ow, oh)]
    fam, p1, p2 = TC_FILTERS[int(rng.integers(len(TC_FILTERS)))]
    blur = 1.0 if rng.random() < 0.8 else float(rng.choice([0.7, 1.5]))
    calls += iwcases._resize_calls(fam, p1, p2, blur)
    if rng.random() < 0.2:
        calls.append(("iw_set_input_crop", int(rng.integers(0, max(1, w // 3))), int(rng.integers(0, max(1, h // 4))),
                      int(rng.integers(max(1, w // 2), w + 1)), int(rng.integers(max(2, h // 2), h + 1))))
    if rng.random() < 0.25:
        calls.append(("iw_set_dither_type", CT_ALL, DITHER_ORDERED, 0))
    if rng.random() < 0.15:
        calls.append(("iw_set_color_count", CT_ALL, int(rng.choice([16, 32, 100]))))
    return Job(imgtype, 8, w, h, px, bpr=bpr, calls=calls)


def run_with_stats(lib, job: Job, vertical: str):
    """Run the job with the given vertical-pass choice; (result, stats)."""
    from bench import Stats, make_ctx
    ctx = make_ctx(lib, job, [("iw_set_option", b"gpu:vertical", vertical.encode())])
    try:
        ok = bool(lib.iw_process_image(ctx))
        res = _collect(lib, ctx, ok, [])
        st = Stats()
        lib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
        lib.dll.iwg_get_stats(ctx, C.byref(st))
        return res, st
    finally:
        lib.iw_destroy_context(ctx)


def test_tensor_vertical_vs_oracle(gpulib, oracle):
    bad, used = [], 0
    n = 120
    for seed in range(7000, 7000 + n):
        job = tensor_case(seed)
        want = run_job(oracle, job)
        got, st = run_with_stats(gpulib, tensor_case(seed), "tensor")
        used += st.vertical_tensor
        if want.key() != got.key():
            bad.append((seed, want.error, got.error, st.vertical_tensor))
    assert not bad, f"{len(bad)} cases differ: {bad[:8]}"
    # almost every case is eligible (a few crops / tiny outputs are not)
    assert used >= n * 3 // 4, f"tensor-core pass ran on only {used} of {n} cases"


def test_tensor_vertical_same_as_cuda_path(gpulib):
    """Both vertical passes give the same bytes on the same job."""
    for seed in range(7500, 7530):
        a, sa = run_with_stats(gpulib, tensor_case(seed), "tensor")
        b, sb = run_with_stats(gpulib, tensor_case(seed), "cuda")
        assert sb.vertical_tensor == 0
        assert a.key() == b.key(), seed


def test_tensor_vertical_random_grid(gpulib, oracle):
    """The general settings grid with the tensor-core pass forced where eligible."""
    bad = []
    for seed in range(0, 400):
        job = iwcases.random_case(seed)
        a = run_job(oracle, job)
        j2 = iwcases.random_case(seed)
        j2.calls = list(j2.calls) + [("iw_set_option", b"gpu:vertical", b"tensor")]
        b = run_job(gpulib, j2)
        if a.key() != b.key() and not (not b.ok and b.error and "Floating-point input" in b.error):
            bad.append((seed, a.error, b.error))
    assert not bad, f"{len(bad)} cases differ: {bad[:8]}"


def test_tensor_vertical_full_size_downscale(gpulib):
    """8192x8192 RGB8 -> 256x256 Lanczos3 against the reference's digest, on
    the tensor-core pass, two calls in a row; it flags fewer pixels for exact
    re-evaluation than the FP32 CUDA-core pass (its bound is tighter)."""
    g = load_workload_digests()["downscale"]
    job = W.downscale()
    assert hashlib.sha256(job.pixels).hexdigest() == g["input_sha256"]
    flagged = {}
    for vertical in ("tensor", "tensor", "cuda"):
        res, st = run_with_stats(gpulib, job, vertical)
        assert res.ok, res.error
        assert res.digest() == g["output_digest"], vertical
        assert st.vertical_tensor == (1 if vertical == "tensor" else 0)
        flagged[vertical] = st.flagged
    assert flagged["tensor"] < flagged["cuda"], flagged


def _stats_after(lib, ctx):
    from bench import Stats
    st = Stats()
    lib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    lib.dll.iwg_get_stats(ctx, C.byref(st))
    return st


def test_timed_replays_run_as_cuda_graph(gpulib, oracle):
    """iwg_process_image_timed replays the fp32 form's launches as a CUDA
    graph; the output is the lone run's, and the calls after it (the FP64
    plain form on the same lane, a 16-bit output) are unaffected."""
    from bench import make_ctx
    job = W.precision(n=1024, out=250)
    want = run_job(gpulib, W.precision(n=1024, out=250))
    ctx = make_ctx(gpulib, job)
    try:
        gpulib.dll.iwg_process_image_timed.restype = C.c_int
        gpulib.dll.iwg_process_image_timed.argtypes = [C.c_void_p, C.c_int, C.c_int]
        assert gpulib.dll.iwg_process_image_timed(ctx, 1, 4)
        got = _collect(gpulib, ctx, True, [])
        st = _stats_after(gpulib, ctx)
    finally:
        gpulib.iw_destroy_context(ctx)
    assert st.graph == 1 and st.ms_device > 0
    assert got.key() == want.key()
    plain = W.precision(n=1024, out=250)
    plain.calls = list(plain.calls) + [("iw_set_option", b"gpu:precision", b"fp64")]
    assert run_job(gpulib, plain).key() == want.key()
    for seed in (3, 11, 29):   # 16-bit output: the plain form
        job = [j for j in W.batch(40, seed=seed, max_side=400) if j.bit_depth == 16][0]
        assert run_job(gpulib, job).key() == run_job(oracle, job).key()


@pytest.mark.parametrize("vertical", ["tensor", "cuda"])
def test_autotuned_bands_same_bytes(gpulib, vertical):
    """The band count chosen by the autotuner never changes the output."""
    for seed in (7700, 7701, 7702):
        a, _ = run_with_stats(gpulib, tensor_case(seed), vertical)
        job = tensor_case(seed)
        job.calls = list(job.calls) + [("iw_set_option", b"gpu:autotune", b"off")]
        b, _ = run_with_stats(gpulib, job, vertical)
        assert a.key() == b.key(), seed


def _props_job(kind: str, seed: int) -> Job:
    """Inputs whose output post-pass has to scan the whole image: opaque,
    gray-valued, 8-bit-representable 16-bit samples, or a single partial
    alpha value / coloured pixel far from the start."""
    from imageworsener_gb300.iwapi import IMGTYPE_RGBA, IMGTYPE_GRAYA
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(40, 200)), int(rng.integers(40, 200))
    g = rng.integers(0, 256, (h, w)).astype(np.uint16)
    if kind == "rgba16_opaque_gray":
        px = np.stack([g * 257, g * 257, g * 257, np.full_like(g, 65535)], -1).astype(">u2").tobytes()
        return Job(IMGTYPE_RGBA, 16, w, h, px, calls=[("iw_set_output_profile", iwcases.PNG),
                                                       ("iw_set_output_canvas_size", w, h),
                                                       ("iw_set_output_depth", 16)] + iwcases._resize_calls("null", 0, 0))
    if kind == "rgb8_late_colour":
        a = np.stack([g, g, g], -1).astype(np.uint8)
        a[h - 1, w - 1, 0] ^= 1
        return Job(IMGTYPE_RGB, 8, w, h, a.tobytes(), calls=[("iw_set_output_profile", iwcases.PNG),
                                                            ("iw_set_output_canvas_size", w, h)] + iwcases._resize_calls("null", 0, 0))
    a = np.stack([g, np.full_like(g, 255)], -1).astype(np.uint8)   # graya8, one partial alpha at the end
    a[h - 1, w - 1, 1] = 128
    return Job(IMGTYPE_GRAYA, 8, w, h, a.tobytes(), calls=[("iw_set_output_profile", iwcases.PNG),
                                                          ("iw_set_output_canvas_size", w // 2 + 1, h // 2 + 1)])


@pytest.mark.parametrize("kind", ["rgba16_opaque_gray", "rgb8_late_colour", "graya8_late_partial"])
def test_post_pass_properties_from_device(gpulib, oracle, kind):
    """The post-pass's property scan (16-bit need, transparency, colour) runs
    as a device reduction over the output; the repacked image equals the
    oracle's."""
    for seed in range(3):
        want = run_job(oracle, _props_job(kind, seed))
        got = run_job(gpulib, _props_job(kind, seed))
        assert got.key() == want.key(), (kind, seed)
    if kind == "rgba16_opaque_gray":
        assert got.imgtype == 1 and got.bit_depth == 8   # alpha stripped, gray, 8-bit

"""The fused vertical + horizontal pass of the fp32 form (one launch, the
intermediate rows kept in shared memory; option gpu:fuse=on) against the CPU
oracle and against the default two-kernel form (the intermediate image in
device memory).  16-bit RGBA downscales with
premultiplied alpha are the layout it takes; the cases vary the width (tile
planning, 16-byte alignment of the tile strips), the scale factor, the
filter, crops, dither and the output size.  Integer output: byte-identical."""
import numpy as np
import pytest

from imageworsener_gb300.iwapi import Job, RT, IMGTYPE_RGBA, CT_ALL, DITHER_ORDERED, run_job, run_job_stats
from imageworsener_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# (width, height, out w, out h, filter, p1, p2, crop (x, y, w, h) or None, dither)
CASES = [
    (1024, 1024, 250, 250, "cubic", 1 / 3, 1 / 3, None, True),
    (1000, 600, 333, 200, "lanczos", 3, 0, None, True),
    (2048, 512, 1000, 250, "lanczos", 2, 0, None, False),
    (1536, 1536, 700, 97, "cubic", 0, 0.5, None, True),
    (600, 800, 150, 400, "triangle", 0, 0, None, True),
    (2000, 300, 211, 151, "cubic", 1 / 3, 1 / 3, (13, 7, 1501, 280), True),
    (4096, 256, 1000, 64, "hermite", 0, 0, (2, 0, 4090, 256), False),
    (512, 512, 37, 41, "box", 0, 0, None, True),
    (800, 800, 799, 400, "cubic", 1 / 3, 1 / 3, None, True),
]


def make_job(case, seed):
    w, h, ow, oh, filt, p1, p2, crop, dith = case
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 65536, size=(h, w, 4), dtype=np.uint32)
    # a fully transparent block and a smooth colour channel
    img[: h // 3, : w // 4, 3] = 0
    yy, xx = np.mgrid[0:h, 0:w]
    img[..., 0] = (xx * 65535 // max(w - 1, 1) + rng.integers(0, 300, size=(h, w))) % 65536
    calls = [("iw_set_output_profile", W.PNG_PROFILE), ("iw_set_output_canvas_size", ow, oh)]
    calls += [("iw_set_resize_alg", d, RT[filt], 1.0, float(p1), float(p2)) for d in (0, 1)]
    if dith:
        calls.append(("iw_set_dither_type", CT_ALL, DITHER_ORDERED, 0))
    if crop:
        calls.append(("iw_set_input_crop",) + tuple(crop))
    return Job(IMGTYPE_RGBA, 16, w, h, img.astype(">u2").tobytes(), calls=calls)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}x{c[1]}-{c[2]}x{c[3]}-{c[4]}")
def test_fused_matches_oracle_and_unfused(gpulib, oracle, case):
    seed = 1000 + CASES.index(case)
    job = make_job(case, seed)
    want = run_job(oracle, job)
    job.calls = list(job.calls) + [("iw_set_option", b"gpu:fuse", b"on")]
    got, st = run_job_stats(gpulib, job)
    assert got.ok, got.error
    assert st["form"] == 1
    job_off = make_job(case, seed)
    off, st_off = run_job_stats(gpulib, job_off)
    assert st_off["fused"] == 0
    assert got.key() == want.key(), "fused output differs from the oracle"
    assert off.key() == want.key(), "two-kernel output differs from the oracle"


def test_precision_workload_takes_fused_pass_on_request(gpulib, oracle):
    """The precision configuration's layout takes the fused pass when asked,
    with the reference's bytes."""
    job = W.precision(n=1024, out=250)
    want = run_job(oracle, job)
    job.calls = list(job.calls) + [("iw_set_option", b"gpu:fuse", b"on")]
    res, st = run_job_stats(gpulib, job)
    assert res.ok and st["form"] == 1 and st["fused"] == 1
    assert res.key() == want.key()

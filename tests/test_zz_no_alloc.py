"""iwg_resize_u8_noalloc: the entry point that allocates nothing.

Each case runs the same image through iw_process_image() (the library's
ordinary entry point, output post-pass options off so the image keeps its
type, except the one that packs a gray result back to gray), through the CPU
oracle with the same settings, and through iwg_resize_u8_noalloc() twice in
a row, and requires identical bytes.  Integer output, so the tolerance is zero.  This file sorts
last so it also runs after every other GPU test in one session.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from imageworsener_gb300.iwapi import (Job, RT, IMGTYPE_GRAY, IMGTYPE_GRAYA, IMGTYPE_RGB, IMGTYPE_RGBA,
                                       CS_SRGB, CS_LINEAR, CS_GAMMA, CS_REC709, DIM_H, DIM_V, run_job,
                                       num_channels)
from conftest import HAS_GPU
from iwcases import PNG, make_pixels

pytestmark = pytest.mark.gpu

# (imgtype, src w, h, dst w, h, filter, p1, p2, cstype, gamma)
CASES = [
    (IMGTYPE_RGBA, 301, 207, 517, 143, "lanczos", 3, 0, CS_SRGB, 0.0),
    (IMGTYPE_RGB, 640, 480, 211, 157, "cubic", 0, 0.5, CS_SRGB, 0.0),
    (IMGTYPE_GRAYA, 123, 77, 123, 301, "hanning", 4, 0, CS_LINEAR, 0.0),
    (IMGTYPE_GRAY, 97, 310, 401, 66, "triangle", 0, 0, CS_GAMMA, 2.2),
    (IMGTYPE_RGBA, 64, 48, 48, 64, "nearest", 0, 0, CS_REC709, 0.0),
    (IMGTYPE_RGB, 20, 17, 33, 17, "auto", 0, 0, CS_SRGB, 0.0),
    (IMGTYPE_GRAYA, 40, 30, 90, 20, "null", 0, 0, CS_SRGB, 0.0),
    (IMGTYPE_RGBA, 1000, 750, 333, 250, "boxavg", 0, 0, CS_SRGB, 0.0),
]


def _bind(lib):
    f = lib.dll.iwg_resize_u8_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_longlong, C.c_void_p, C.c_int, C.c_int, C.c_longlong,
                  C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_char_p, C.c_int]
    return f


def _expected(lib, case, pixels, bpr):
    imgtype, sw, sh, dw, dh, filt, p1, p2, cst, gamma = case
    calls = [("iw_set_output_profile", PNG), ("iw_set_output_canvas_size", dw, dh),
             ("iw_set_input_colorspace", ("cs", cst, gamma)), ("iw_set_output_colorspace", ("cs", cst, gamma))]
    for d in (DIM_H, DIM_V):
        calls.append(("iw_set_resize_alg", d, RT[filt], 1.0, float(p1), float(p2)))
    # The reference resamples a gray image as RGB with three equal channels and
    # its output post-pass packs that back to gray; keep that one post-pass
    # option for gray images and turn the others off.
    gray = imgtype in (IMGTYPE_GRAY, IMGTYPE_GRAYA)
    for opt in range(2 if gray else 1, 6):
        calls.append(("iw_set_allow_opt", opt, 0))
    r = run_job(lib, Job(imgtype, 8, sw, sh, pixels, bpr=bpr, calls=calls))
    assert r.ok, r.error
    assert (r.imgtype, r.bit_depth, r.width, r.height) == (imgtype, 8, dw, dh)
    return r


@pytest.fixture(scope="module")
def torch_cuda():
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    import torch
    return torch


def _call(f, torch, case, src, src_bpr, dst, dst_bpr):
    imgtype, sw, sh, dw, dh, filt, p1, p2, cst, gamma = case
    msg = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    ok = f(src, sw, sh, src_bpr, dst, dw, dh, dst_bpr, imgtype, RT[filt], p1, p2, cst, gamma,
           C.c_void_p(stream), msg, 256)
    assert ok == 1, msg.value.decode()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]:#x}-{c[1]}x{c[2]}-{c[3]}x{c[4]}-{c[5]}")
def test_noalloc_matches_process_image(gpulib, oracle, torch_cuda, case):
    torch = torch_cuda
    f = _bind(gpulib)
    imgtype, sw, sh, dw, dh = case[:5]
    nch = num_channels(imgtype)
    rng = np.random.default_rng(sw * 7919 + sh * 31 + dw)
    pixels, bpr = make_pixels(rng, imgtype, 8, sw, sh)
    exp = _expected(gpulib, case, pixels, bpr)
    # the same job through the CPU oracle: the comparison below is then with
    # the reference's arithmetic directly, not only with this library
    assert _expected(oracle, case, pixels, bpr).pixels == exp.pixels, "iw_process_image differs from the oracle"
    src = torch.from_numpy(np.frombuffer(pixels, dtype=np.uint8).copy()).cuda()
    dst_bpr = exp.bpr
    assert dst_bpr == dw * nch
    for attempt in range(2):   # two calls in a row share the scratch array
        dst = torch.full((dst_bpr * dh,), 0xA5, dtype=torch.uint8, device="cuda")
        _call(f, torch, case, src.data_ptr(), bpr, dst.data_ptr(), dst_bpr)
        torch.cuda.synchronize()
        got = dst.cpu().numpy().tobytes()
        assert got == exp.pixels, f"call {attempt + 1}: output differs from iw_process_image"


def test_noalloc_back_to_back_cases(gpulib, torch_cuda):
    """Two different jobs queued on one stream without a host wait between."""
    torch = torch_cuda
    f = _bind(gpulib)
    jobs = []
    for case in (CASES[0], CASES[1]):
        imgtype, sw, sh, dw, dh = case[:5]
        rng = np.random.default_rng(12345 + sw)
        pixels, bpr = make_pixels(rng, imgtype, 8, sw, sh)
        exp = _expected(gpulib, case, pixels, bpr)
        src = torch.from_numpy(np.frombuffer(pixels, dtype=np.uint8).copy()).cuda()
        dst = torch.zeros((exp.bpr * dh,), dtype=torch.uint8, device="cuda")
        jobs.append((case, src, bpr, dst, exp))
    for case, src, bpr, dst, exp in jobs:
        _call(f, torch, case, src.data_ptr(), bpr, dst.data_ptr(), exp.bpr)
    torch.cuda.synchronize()
    for case, src, bpr, dst, exp in jobs:
        assert dst.cpu().numpy().tobytes() == exp.pixels


def test_noalloc_host_buffers(gpulib, torch_cuda):
    """Ordinary host memory, where the device can read pageable memory."""
    torch = torch_cuda
    info = C.create_string_buffer(256)
    gpulib.dll.iwg_device_info(info, 256)
    if b"pageable host memory access 1" not in info.value:
        pytest.skip("device cannot access pageable host memory")
    f = _bind(gpulib)
    case = CASES[0]
    imgtype, sw, sh, dw, dh = case[:5]
    rng = np.random.default_rng(99)
    pixels, bpr = make_pixels(rng, imgtype, 8, sw, sh)
    exp = _expected(gpulib, case, pixels, bpr)
    src = np.frombuffer(pixels, dtype=np.uint8).copy()
    for _ in range(2):
        dst = np.full(exp.bpr * dh, 0x5A, dtype=np.uint8)
        _call(f, torch, case, src.ctypes.data, bpr, dst.ctypes.data, exp.bpr)
        torch.cuda.synchronize()
        assert dst.tobytes() == exp.pixels


def test_noalloc_rejects_oversize_and_bad_args(gpulib, torch_cuda):
    """Jobs beyond the limits fail with a message before any launch."""
    torch = torch_cuda
    f = _bind(gpulib)
    src = torch.zeros(16, dtype=torch.uint8, device="cuda")
    dst = torch.zeros(16, dtype=torch.uint8, device="cuda")
    msg = C.create_string_buffer(256)
    # RGBA 4000 wide, 3000 output rows: a 192 MB intermediate, over the 32 MiB scratch
    ok = f(src.data_ptr(), 4000, 3000, 16000, dst.data_ptr(), 4000, 3000, 16000, IMGTYPE_RGBA, RT["cubic"],
           0.0, 0.5, CS_SRGB, 0.0, None, msg, 256)
    assert ok == 0 and b"scratch" in msg.value
    ok = f(src.data_ptr(), 4, 4, 4, dst.data_ptr(), 4, 4, 4, 0x1000, RT["cubic"], 0.0, 0.5, CS_SRGB, 0.0,
           None, msg, 256)
    assert ok == 0 and b"image type" in msg.value
    ok = f(src.data_ptr(), 20000, 1, 80000, dst.data_ptr(), 4, 4, 16, IMGTYPE_RGBA, RT["cubic"], 0.0, 0.5,
           CS_SRGB, 0.0, None, msg, 256)
    assert ok == 0 and b"dimensions" in msg.value


def test_noalloc_allocates_nothing(gpulib, torch_cuda):
    """After the first call on the device (which resolves the scratch
    array), further calls leave the device's free memory unchanged: nothing
    is allocated on the device (a cudaMalloc takes at least one 2 MiB page)."""
    torch = torch_cuda
    f = _bind(gpulib)
    case = CASES[1]
    imgtype, sw, sh, dw, dh = case[:5]
    rng = np.random.default_rng(4242)
    pixels, bpr = make_pixels(rng, imgtype, 8, sw, sh)
    nch = num_channels(imgtype)
    src = torch.from_numpy(np.frombuffer(pixels, dtype=np.uint8).copy()).cuda()
    dst = torch.zeros((dw * nch * dh,), dtype=torch.uint8, device="cuda")
    _call(f, torch, case, src.data_ptr(), bpr, dst.data_ptr(), dw * nch)
    torch.cuda.synchronize()
    first = dst.cpu().numpy().tobytes()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        _call(f, torch, case, src.data_ptr(), bpr, dst.data_ptr(), dw * nch)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes across calls"
    assert dst.cpu().numpy().tobytes() == first

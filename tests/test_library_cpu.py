"""The C-ABI library without a GPU: it builds, loads, exports every declared
entry point, and its host-side API behaves like the reference's."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT, HAS_GPU
from imageworsener_gb300.iwapi import Csdescr, Job, IMGTYPE_RGB, run_job

HEADERS = [os.path.join(ROOT, "include", h) for h in ("imagew.h", "imagew_gb300.h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        names.update(re.findall(r"IW_EXPORT\([^)]*\)\s+(\w+)\s*\(", text))
    return sorted(names)


def test_headers_declare_the_core_api():
    names = declared_symbols()
    for must in ("iw_create_context", "iw_process_image", "iw_get_output_image", "iw_set_resize_alg",
                 "iw_set_dither_type", "iwg_get_stats"):
        assert must in names


def test_library_exports_every_declared_symbol(gpulib):
    missing = [n for n in declared_symbols() if not hasattr(gpulib.dll, n)]
    assert not missing, missing


def test_oracle_exports_every_core_symbol(oracle):
    missing = [n for n in declared_symbols() if n.startswith("iw_") and not hasattr(oracle.dll, n)]
    assert not missing, missing


def _settings_probe(lib):
    """Exercise setters/getters and stateless helpers; return observations."""
    obs = []
    ctx = lib.iw_create_context(None)
    for code, val in ((11, 1), (13, 1), (15, 1), (16, 3), (17, 1), (18, 3), (45, 100), (46, 200), (53, 1)):
        lib.iw_set_value(ctx, code, val)
        obs.append(lib.iw_get_value(ctx, code))
    lib.iw_set_value_dbl(ctx, 42, 1.25)
    obs.append(lib.iw_get_value_dbl(ctx, 42))
    obs.append(lib.iw_get_value(ctx, 10))
    lib.iw_set_option(ctx, b"gpu:test", b"")
    obs.append(lib.iw_get_option(ctx, b"gpu:test"))
    lib.iw_set_value(ctx, 30, 85)   # legacy code forwarded to an option string
    obs.append(lib.iw_get_option(ctx, b"jpeg:quality"))
    lib.iw_destroy_context(ctx)
    for fmt in range(0, 14):
        obs.append(lib.iw_get_profile_by_fmt(fmt))
    obs.append(lib.iw_get_version_int())
    cs = Csdescr()
    for cstype, gamma in ((0, 0.0), (1, 0.0), (2, 2.2), (3, 0.0)):
        cs.cstype, cs.gamma = cstype, gamma
        for v in (0.0, 0.002, 0.04, 0.5, 0.9999999999, 1.0):
            obs.append(lib.iw_convert_sample_to_linear(v, C.byref(cs)))
            obs.append(lib.iw_convert_sample_from_linear(v, C.byref(cs)))
    for fn in (b"a.png", b"b.JPEG", b"c.pam", b"d", b"e.tiff"):
        obs.append(lib.dll.iw_detect_fmt_from_filename(fn))
    return obs


def test_settings_api_matches_oracle(gpulib, oracle):
    assert _settings_probe(gpulib) == _settings_probe(oracle)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU failure mode")
def test_process_without_gpu_fails_cleanly(gpulib):
    job = Job(IMGTYPE_RGB, 8, 8, 8, bytes(8 * 8 * 3),
              calls=[("iw_set_output_profile", 0x40), ("iw_set_output_canvas_size", 4, 4)])
    res = run_job(gpulib, job)
    assert not res.ok
    assert "CUDA" in (res.error or "")


def test_planning_errors_match_oracle_without_gpu(gpulib, oracle):
    """Errors raised while planning (before any device work) match."""
    px = bytes(4 * 4 * 3)
    for calls in ([], [("iw_set_output_profile", 0x40)],
                  [("iw_set_output_profile", 0x40), ("iw_set_output_canvas_size", 50000, 10)]):
        job = Job(IMGTYPE_RGB, 8, 4, 4, px, calls=calls)
        a, b = run_job(gpulib, job), run_job(oracle, job)
        assert (a.ok, a.error) == (b.ok, b.error)


@pytest.mark.parametrize("block", range(4))
def test_planning_warnings_match_oracle_on_random_grid(gpulib, oracle, block):
    """The library's planning (output type, depth, colour space, background
    and offset decisions) raises the same warnings as the oracle, in the same
    order, on the random settings grid.  Without a GPU the run stops after
    planning with a CUDA error; with one it completes."""
    import iwcases
    bad = []
    for seed in range(block * 600, block * 600 + 600):
        a = run_job(gpulib, iwcases.random_case(seed), keep_warnings=True)
        b = run_job(oracle, iwcases.random_case(seed), keep_warnings=True)
        if b.ok:
            status_ok = a.ok or "CUDA" in (a.error or "")
        else:
            status_ok = not a.ok and a.error == b.error
        if not status_ok or a.warnings != b.warnings:
            bad.append((seed, a.error, b.error, a.warnings, b.warnings))
    assert not bad, bad[:3]


def _same_refusal(a, b) -> bool:
    """The library refuses exactly what the oracle refuses, with its message;
    what the oracle processes gets past planning (to the device, or to a
    CUDA error where there is none)."""
    if not b.ok:
        return not a.ok and a.error == b.error
    return a.ok or "CUDA" in (a.error or "")


def test_crops_outside_the_image_refused_like_oracle(gpulib, oracle):
    """Crops the reference's clamp leaves with zero or negative sizes, all
    refused while planning, before any device work: the negative ones with
    the reference's message; the empty ones (which the reference resamples
    from empty buffers) with "Input crop is empty"."""
    import iwcases
    bad, refused, empty = [], 0, 0
    for i in range(1500):
        job = iwcases.crop_case(i)
        a = run_job(gpulib, job, keep_warnings=True)
        b = run_job(oracle, iwcases.crop_case(i), keep_warnings=True)
        refused += not b.ok
        _, _, cw, ch = iwcases.clamped_crop(job)
        if b.ok and min(cw, ch) == 0:
            empty += 1
            ok = not a.ok and a.error == "Input crop is empty"
        else:
            ok = _same_refusal(a, b)
        if not ok or a.warnings != b.warnings:
            bad.append((i, a.error, b.error))
    assert not bad, bad[:5]
    assert refused > 500 and empty > 20


def test_images_over_the_allocation_limit_refused_like_oracle(gpulib, oracle):
    import iwcases
    for name, job in iwcases.over_limit_cases():
        a, b = run_job(gpulib, job), run_job(oracle, job)
        assert not b.ok and b.error == "Image too large to process", name
        assert (a.ok, a.error) == (b.ok, b.error), name

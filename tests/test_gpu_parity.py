"""GPU parity: libimagew_gb300 (through its C ABI) against the CPU oracle and
against golden outputs of the reference.  Integer output must be
byte-identical; both precision forms are checked."""
import hashlib

import pytest

from conftest import load_grid, load_workload_digests
from imageworsener_gb300.iwapi import run_job
from imageworsener_gb300 import workloads as W
import iwcases

pytestmark = pytest.mark.gpu

FORMS = ["fp32", "fp64"]

def same(job, want_key, got):
    # (floating-point input in a non-linear colour space included: the host
    # linearises it with glibc, as the reference does per sample)
    return want_key == got.key()


def with_form(job, form):
    job.calls = list(job.calls) + [("iw_set_option", b"gpu:precision", form.encode())]
    return job


@pytest.mark.parametrize("form", FORMS)
def test_golden_grid(gpulib, form):
    bad = []
    for job, digest, meta in load_grid():
        res = run_job(gpulib, with_form(job, form))
        if res.digest() != digest:
            bad.append((meta["seed"], res.error))
    assert not bad, f"{len(bad)} cases differ from the reference: {bad[:8]}"


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("block", range(4))
def test_random_vs_oracle(gpulib, oracle, form, block):
    bad = []
    for seed in range(block * 500, block * 500 + 500):
        job = iwcases.random_case(seed)
        a = run_job(oracle, job, keep_warnings=True)
        b = run_job(gpulib, with_form(iwcases.random_case(seed), form), keep_warnings=True)
        if not same(job, a.key(), b) or (b.ok and a.warnings != b.warnings):
            bad.append((seed, a.error, b.error))
    assert not bad, f"{len(bad)} cases differ: {bad[:8]}"


@pytest.mark.parametrize("form", FORMS)
def test_random_large_vs_oracle(gpulib, oracle, form):
    bad = []
    for seed in range(50000, 50100):
        job = iwcases.random_case(seed, max_dim=300)
        a = run_job(oracle, job)
        b = run_job(gpulib, with_form(iwcases.random_case(seed, max_dim=300), form))
        if not same(job, a.key(), b):
            bad.append((seed, a.error, b.error))
    assert not bad, bad


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", ["small", "precision", "downscale", "downscale_fs4"])
def test_full_size_workloads(gpulib, form, name):
    """The benchmark workloads at full size against the reference's digests."""
    g = load_workload_digests()[name]
    job = {"small": W.small, "precision": W.precision, "downscale": W.downscale,
           "downscale_fs4": lambda: W.downscale(fs4=True)}[name]()
    assert hashlib.sha256(job.pixels).hexdigest() == g["input_sha256"], "workload generator drifted"
    res = run_job(gpulib, with_form(job, form))
    assert res.ok, res.error
    assert res.digest() == g["output_digest"]


@pytest.mark.parametrize("form", FORMS)
def test_batch_workload(gpulib, form):
    g = load_workload_digests()["batch24"]
    for job, want in zip(W.batch(24, max_side=1024), g):
        assert run_job(gpulib, with_form(job, form)).digest() == want["output_digest"]


def test_repeat_calls_identical(gpulib):
    """Buffers are reused between calls; results must not depend on history."""
    j1 = W.small(w=300, h=200, ow=97, oh=61)
    first = run_job(gpulib, j1).key()
    run_job(gpulib, W.precision(n=512, out=333))
    assert run_job(gpulib, W.small(w=300, h=200, ow=97, oh=61)).key() == first


def test_stats_report_form(gpulib):
    """The fp32 form runs (and flags few pixels) on the benchmark layout."""
    import ctypes as C
    from bench import Stats, make_ctx
    job = W.precision(n=1024, out=250)
    for form, want in (("fp32", 1), ("fp64", 0)):
        ctx = make_ctx(gpulib, job, [("iw_set_option", b"gpu:precision", form.encode())])
        assert gpulib.iw_process_image(ctx)
        st = Stats()
        gpulib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
        gpulib.dll.iwg_get_stats(ctx, C.byref(st))
        gpulib.iw_destroy_context(ctx)
        assert st.form == want
        if form == "fp32":
            assert st.flagged < 0.05 * 250 * 250
            assert 0 <= st.flagged_exact <= st.flagged


def test_crops_inside_and_outside_the_image(gpulib, oracle):
    """Crops drawn to land outside the image as often as inside: the ones the
    oracle processes give the oracle's bytes on the GPU; the ones the
    reference refuses (negative clamped sizes) are refused with its message,
    and crops that clamp to nothing with "Input crop is empty" -- all while
    planning, before any device work."""
    bad = []
    for i in range(400):
        job = iwcases.crop_case(i)
        a = run_job(gpulib, job, keep_warnings=True)
        b = run_job(oracle, iwcases.crop_case(i), keep_warnings=True)
        _, _, cw, ch = iwcases.clamped_crop(job)
        if b.ok and min(cw, ch) == 0:
            ok = not a.ok and a.error == "Input crop is empty"
        else:
            ok = a.key() == b.key()
        if not ok or a.warnings != b.warnings:
            bad.append((i, a.error, b.error))
    assert not bad, bad[:5]


def test_images_over_the_allocation_limit_refused(gpulib, oracle):
    for name, job in iwcases.over_limit_cases():
        a, b = run_job(gpulib, job), run_job(oracle, job)
        assert (a.ok, a.error) == (b.ok, b.error) == (False, "Image too large to process"), name

"""iwg_process_batch: many contexts in one call.

Every context of a batch must come out exactly as iw_process_image() gives it
alone (the key covers the pixels, image type, depth, palette, colour key,
background label and reduced-depth fields).  Batches mix image types, depths,
filters, sizes, settings the batched form does not take (they run alone inside
the call) and contexts that fail.
"""
import pytest

from conftest import load_workload_digests
from imageworsener_gb300.iwapi import run_batch, run_job, run_served, Job, IMGTYPE_RGB, RT
from imageworsener_gb300 import workloads as W
import iwcases

pytestmark = pytest.mark.gpu


def test_batch_workload_matches_reference_digests(gpulib):
    """The batched-config generator, 24 images, against the reference's digests."""
    g = load_workload_digests()["batch24"]
    jobs = W.batch(24, max_side=1024)
    for res, want in zip(run_batch(gpulib, jobs), g):
        assert res.digest() == want["output_digest"]


@pytest.mark.parametrize("seed", [11, 12])
def test_batch_equals_lone_runs_random_settings(gpulib, seed):
    """Random settings (dither, backgrounds, crops, offsets, float output ...):
    the batch runs what it can together and the rest alone."""
    jobs = [iwcases.random_case(1000 * seed + k) for k in range(40)]
    lone = [run_job(gpulib, j) for j in jobs]
    batched = run_batch(gpulib, jobs)
    for k, (a, b) in enumerate(zip(lone, batched)):
        assert a.key() == b.key(), f"case {k}: {jobs[k].calls}"


def test_batch_mixed_sizes_and_depths(gpulib):
    jobs = W.batch(96, seed=21, max_side=700)
    lone = [run_job(gpulib, j) for j in jobs]
    batched = run_batch(gpulib, jobs)
    for k, (a, b) in enumerate(zip(lone, batched)):
        assert a.ok and a.key() == b.key(), f"image {k}"


def test_batch_with_failing_context(gpulib):
    good = W.batch(3, seed=5, max_side=300)
    px = bytes(range(256)) * 3
    bad = Job(IMGTYPE_RGB, 8, 16, 16, px * 1, calls=[("iw_set_output_profile", 0x8040),
                                                     ("iw_set_output_canvas_size", 8, 8),
                                                     ("iw_set_resize_alg", 0, 0x7f, 1.0, 0.0, 0.0),
                                                     ("iw_set_resize_alg", 1, RT["cubic"], 1.0, 0.0, 0.5)])
    jobs = [good[0], bad, good[1], good[2]]
    lone = [run_job(gpulib, j) for j in jobs]
    batched = run_batch(gpulib, jobs)
    assert not lone[1].ok and not batched[1].ok and lone[1].error == batched[1].error
    for k in (0, 2, 3):
        assert lone[k].key() == batched[k].key()


def test_batch_repeat_is_stable(gpulib):
    jobs = W.batch(16, seed=31, max_side=512)
    a = run_batch(gpulib, jobs)
    b = run_batch(gpulib, jobs)
    assert [r.key() for r in a] == [r.key() for r in b]


@pytest.mark.parametrize("mode", ["zero", "copy", "stage", "pull"])
def test_transfer_modes_identical(gpulib, mode):
    """Zero copy, cudaMemcpy, pinned staging and the pull kernel give the same bytes, alone and batched."""
    jobs = W.batch(12, seed=41, max_side=600)
    opt = [("iw_set_option", b"gpu:upload", mode.encode())]
    ref = [run_job(gpulib, j) for j in jobs]
    for j in jobs:
        j.calls = list(j.calls) + opt
    lone = [run_job(gpulib, j) for j in jobs]
    batched = run_batch(gpulib, jobs)
    for a, b, c in zip(ref, lone, batched):
        assert a.key() == b.key() == c.key()


def test_server_mix_same_as_alone(gpulib):
    """Requests served together (continuous batching, error diffusion on the
    second lane) come out exactly as each does alone."""
    jobs = W.batch(40, seed=51, max_side=800)
    jobs += [iwcases.random_case(7000 + k) for k in range(30)]
    for k in range(0, 40, 7):   # error diffusion on some thumbnails
        jobs[k].calls = list(jobs[k].calls) + [("iw_set_dither_type", 10, 2, 0)]
    lone = [run_job(gpulib, j) for j in jobs]
    served = run_served(gpulib, jobs)
    for k, (a, b) in enumerate(zip(lone, served)):
        assert a.key() == b.key(), f"request {k}"


def test_server_small_budget(gpulib):
    """A budget smaller than one image still admits one request at a time."""
    jobs = W.batch(10, seed=61, max_side=500)
    lone = [run_job(gpulib, j) for j in jobs]
    served = run_served(gpulib, jobs, budget=1 << 20, max_batch=3)
    assert [r.key() for r in lone] == [r.key() for r in served]


"""The FP32 form's linear-light error against the FP64 form (whose values are
the reference's), read back through the library's debug option.

For every output sample the FP32 tail quantises a value v32 together with a
rigorous bound E on |v32 - v64| (the error model of the guard band); a
sample whose interval [v32 - E, v32 + E] touches a decision of the reference
is re-evaluated exactly.  These tests check that the bound holds on every
sample of several configurations (any violation could change an output byte
without a flag), that the output bytes of both forms agree, and they report
the measured max / RMS error of the intermediate image and of the final
values.  Tolerance: zero bound violations; integer output identical.
"""
import numpy as np
import pytest

from imageworsener_gb300 import workloads as W
from imageworsener_gb300.iwapi import fp_error, run_debug_values
import iwcases

pytestmark = pytest.mark.gpu


def _check(stats):
    assert stats["form"] == 1, "the fp32 form did not take the configuration"
    assert stats["identical_output"], "fp32 and fp64 output bytes differ"
    assert stats["bound_violations"] == 0, stats
    assert stats["final_max"] <= stats["final_bound_max"]
    # both forms keep the intermediate within float rounding of each other:
    # far below a quantisation step of 8-bit output
    assert stats["interm_max"] < 1e-4, stats


def test_fp_error_precision_reduced(gpulib):
    """The precision configuration's settings (16-bit RGBA, premultiplied
    Mitchell, 8x8 ordered dither) at 1024^2 -> 250^2."""
    _check(fp_error(gpulib, W.precision(n=1024, out=250)))


def test_fp_error_small(gpulib):
    _check(fp_error(gpulib, W.small()))


def test_fp_error_downscale_tensor(gpulib):
    """Wide windows (Lanczos3 at 16:1): the vertical pass on the tensor cores."""
    stats = fp_error(gpulib, W.downscale(n=2048, out=128))
    _check(stats)
    assert stats["vertical_tensor"] == 1


def test_fp_error_batch_images(gpulib):
    for job in W.batch(12, seed=4):
        stats = fp_error(gpulib, job)
        if stats["form"] != 1:   # 16-bit output: the fp64 form runs
            continue
        _check(stats)


def test_fp_error_random_grid(gpulib):
    """Seeded settings of the random grid that the fp32 form takes."""
    taken = 0
    for seed in range(300):
        job = iwcases.random_case(seed)
        if job.sampletype != 0:
            continue
        r, i32, v32, e32, st = run_debug_values(gpulib, job, "fp32")
        if not r.ok or st["form"] != 1 or v32.size == 0:
            continue
        _, i64, v64, _, _ = run_debug_values(gpulib, iwcases.random_case(seed), "fp64")
        ok = ~(np.isnan(v32) | np.isnan(v64))
        d = np.abs(v32 - v64)[ok]
        assert (d <= e32[ok]).all(), f"seed {seed}: {(d > e32[ok]).sum()} samples beyond the bound"
        taken += 1
    assert taken >= 20

"""Failure detection without a GPU fault.

* A bounded device wait that runs out: the option gpu:wait_test starves the
  bulk-copy pipeline of the vertical pass (and of the fused pass): its
  producer issues no copies, so no barrier the consumers wait on ever
  completes, and the waits are shortened to a few thousand polls.  The
  kernel must record the error and return; iw_process_image must fail with
  "A device wait ran out of time", and the library must stay usable: the
  same job afterwards gives the reference's bytes.
* A device allocation that fails (host-side injection, option
  gpu:fail_alloc): iw_process_image fails with the library's message for a
  failed device allocation, and the error is sticky like the reference's
  first error (src/imagew-api.c:106-119): a later error does not replace it.

Nothing here faults, traps or hangs a GPU: the waits are bounded and the
allocation failure is made on the host.
"""
import ctypes as C

import pytest

from imageworsener_gb300 import workloads as W
from imageworsener_gb300.iwapi import run_job, run_job_stats, _setup

pytestmark = pytest.mark.gpu


def _job(extra, fuse=True):
    job = W.precision(n=1024, out=250)
    job.calls = list(job.calls) + [("iw_set_option", b"gpu:autotune", b"off")] + list(extra)
    if fuse:
        job.calls.append(("iw_set_option", b"gpu:fuse", b"on"))
    return job


@pytest.mark.parametrize("fuse", [True, False], ids=["fused", "two-kernel"])
def test_device_wait_runs_out_and_library_recovers(gpulib, oracle, fuse):
    want = run_job(oracle, W.precision(n=1024, out=250))
    bad = run_job(gpulib, _job([("iw_set_option", b"gpu:wait_test", b"1")], fuse))
    assert not bad.ok
    assert bad.error is not None and "A device wait ran out of time" in bad.error
    good, st = run_job_stats(gpulib, _job([], fuse))
    assert good.ok and good.key() == want.key()
    assert st["fused"] == (1 if fuse else 0)


def test_injected_allocation_failure_is_sticky_first_error(gpulib):
    lib = gpulib
    ctx = lib.iw_create_context(None)
    try:
        _setup(lib, ctx, _job([("iw_set_option", b"gpu:fail_alloc", b"1")]))
        assert lib.iw_process_image(ctx) == 0
        assert lib.iw_get_errorflag(ctx)
        mb = C.create_string_buffer(256)
        assert lib.iw_get_errormsg(ctx, mb, 256).decode() == "Out of GPU memory"
        # a second error on the same context (processing twice) keeps the first message
        assert lib.iw_process_image(ctx) == 0
        assert lib.iw_get_errormsg(ctx, mb, 256).decode() == "Out of GPU memory"
    finally:
        lib.iw_destroy_context(ctx)
    # the library is usable afterwards
    r = run_job(lib, W.small(w=256, h=192, ow=128, oh=96))
    assert r.ok

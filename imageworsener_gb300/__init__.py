"""imageworsener_gb300: GPU (sm_103a) implementation of ImageWorsener's
iw_process_image() pixel pipeline behind the libimagew C ABI.

The product is the shared library ``libimagew_gb300.so`` (C ABI declared in
``include/imagew.h`` and ``include/imagew_gb300.h``).  This package builds it
(:mod:`.build`) and binds it from Python with ctypes (:mod:`.iwapi`) for tests
and benchmarks.
"""
import os

from .iwapi import IWLib, Job, Result, run_job  # noqa: F401

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libimagew_gb300.so")


def load(build_if_missing: bool = True) -> IWLib:
    """Open libimagew_gb300.so (building it first if asked and needed).

    Raises if the library is missing: there is no fallback implementation.
    """
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise FileNotFoundError(f"{LIB_PATH} not built; run python -m imageworsener_gb300.build")
        from . import build
        build.build()
    return IWLib(LIB_PATH)

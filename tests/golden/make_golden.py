"""Regenerate the golden fixtures from the reference ImageWorsener.

Run in a checkout where the reference sources exist and
``make -C oracle ref`` has built ``oracle/_ref/libimagew_ref.so`` (the
unmodified reference core compiled from its own sources):

    python tests/golden/make_golden.py

Writes
  grid.npz / grid.json   small seeded cases (tests/iwcases.py) with their full
                         inputs, API calls and the reference's outputs;
  workloads.json         SHA-256 digests of the inputs and of the reference's
                         outputs for the full-size benchmark workloads
                         (imageworsener_gb300/workloads.py), which every machine
                         regenerates bit-identically from their seeds.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from imageworsener_gb300.iwapi import IWLib, run_job  # noqa: E402
from imageworsener_gb300 import workloads as W  # noqa: E402
import iwcases  # noqa: E402

GRID_SEEDS = range(100000, 100400)


def _jsonable(calls):
    out = []
    for c in calls:
        out.append([list(a) if isinstance(a, tuple) else a for a in c])
    return out


def make_grid(ref: IWLib):
    meta, arrays = [], {}
    for n, seed in enumerate(GRID_SEEDS):
        job = iwcases.random_case(seed)
        res = run_job(ref, job)
        arrays[f"in{n}"] = np.frombuffer(job.pixels, dtype=np.uint8)
        arrays[f"out{n}"] = np.frombuffer(res.pixels, dtype=np.uint8)
        meta.append(dict(seed=seed, imgtype=job.imgtype, bit_depth=job.bit_depth, width=job.width,
                         height=job.height, bpr=job.bpr, sampletype=job.sampletype, orient=job.orient,
                         calls=_jsonable(job.calls),
                         result=dict(ok=res.ok, error=res.error, imgtype=res.imgtype, bit_depth=res.bit_depth,
                                     sampletype=res.sampletype, width=res.width, height=res.height, bpr=res.bpr,
                                     palette=res.palette, colorkey=res.colorkey, bkgdlabel=res.bkgdlabel,
                                     reduced_maxcolors=res.reduced_maxcolors, digest=res.digest())))
    np.savez_compressed(os.path.join(HERE, "grid.npz"), **arrays)
    with open(os.path.join(HERE, "grid.json"), "w") as f:
        json.dump(meta, f, indent=0)


def make_workloads(ref: IWLib):
    import hashlib
    out = {}
    specs = [("small", lambda: W.small()), ("precision", lambda: W.precision()),
             ("downscale", lambda: W.downscale()), ("downscale_fs4", lambda: W.downscale(fs4=True))]
    for name, fn in specs:
        job = fn()
        t = time.time()
        res = run_job(ref, job)
        dt = time.time() - t
        out[name] = dict(input_sha256=hashlib.sha256(job.pixels).hexdigest(), output_digest=res.digest(),
                         ok=res.ok, width=res.width, height=res.height, imgtype=res.imgtype,
                         reference_seconds=round(dt, 3))
        print(name, out[name], flush=True)
    batch = W.batch(24, max_side=1024)
    out["batch24"] = [dict(input_sha256=hashlib.sha256(j.pixels).hexdigest(), output_digest=run_job(ref, j).digest())
                      for j in batch]
    with open(os.path.join(HERE, "workloads.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    lib = IWLib(os.path.join(ROOT, "oracle", "_ref", "libimagew_ref.so"))
    if "--workloads-only" not in sys.argv:
        make_grid(lib)
    if "--grid-only" not in sys.argv:
        make_workloads(lib)

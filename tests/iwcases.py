"""Seeded parity cases for the libimagew API.

Each case is an :class:`imageworsener_gb300.iwapi.Job`: a synthetic input
image plus the API calls that configure one ``iw_process_image`` run.  The
same cases drive every parity check:

* CPU oracle vs the reference built from its own sources (tests here),
* GPU library vs CPU oracle (GPU tests),
* golden fixtures generated from the reference (tests/golden/).

The grid covers the settings the reference's own regression suite exercises
(tests/runtest:60-300 of ImageWorsener 1.3.5): every filter family and its
parameters, blur, the three edge policies, translation and channel offsets,
crop and orientation, the four colour-space families, 1/2/4/8/16-bit and float
input, 8/16-bit and float output, reduced max colour codes, colour counts,
ordered / error-diffusion / random dither, solid and checkerboard
backgrounds, background labels, grayscale conversion, negation and the output
post-pass options.
"""
from __future__ import annotations

import numpy as np

from imageworsener_gb300.iwapi import (Job, RT, PROFILE, IMGTYPE_GRAY, IMGTYPE_GRAYA, IMGTYPE_RGB,
                                       IMGTYPE_RGBA, SAMPLETYPE_FLOAT, CT_ALL, CT_NONALPHA, CT_ALPHA,
                                       CT_RED, CT_GREEN, CT_BLUE, CT_GRAY, CS_SRGB, CS_LINEAR, CS_GAMMA,
                                       CS_REC709, DITHER_ORDERED, DITHER_ERRDIFF, DITHER_RANDOM, VAL,
                                       num_channels)

P = PROFILE
PNG = (P["TRANSPARENCY"] | P["GRAYSCALE"] | P["PALETTETRNS"] | P["GRAY1"] | P["GRAY2"] | P["GRAY4"] |
       P["BPS16"] | P["BINARYTRNS"] | P["PAL1"] | P["PAL2"] | P["PAL4"] | P["PAL8"] | P["REDUCEDBITDEPTHS"] |
       P["PNG_BKGD"])
PAM = P["BPS16"] | P["REDUCEDBITDEPTHS"] | P["GRAYSCALE"] | P["GRAY1"] | P["TRANSPARENCY"]
PPM = P["BPS16"] | P["REDUCEDBITDEPTHS"]
MIFF = P["TRANSPARENCY"] | P["GRAYSCALE"] | P["ALWAYSLINEAR"] | P["HDRI"] | P["RGB16_BKGD"]
BMP = P["PAL1"] | P["PAL4"] | P["PAL8"] | P["REDUCEDBITDEPTHS"]
# A profile that lets every sample through untouched by the post-pass repacking.
RAW = P["TRANSPARENCY"] | P["BPS16"] | P["REDUCEDBITDEPTHS"]

FILTERS = [("lanczos", 3, 0), ("lanczos", 2, 0), ("lanczos", 5, 0), ("hanning", 3, 0), ("blackman", 4, 0),
           ("sinc", 3, 0), ("cubic", 1 / 3, 1 / 3), ("cubic", 0, 0.5), ("cubic", 1, 0), ("cubic", 0, 1),
           ("hermite", 0, 0), ("box", 0, 0), ("boxavg", 0, 0), ("triangle", 0, 0), ("quadratic", 0, 0),
           ("gaussian", 0, 0), ("mix", 0, 0), ("nearest", 0, 0), ("null", 0, 0), ("auto", 0, 0)]


def make_pixels(rng: np.random.Generator, imgtype: int, depth: int, w: int, h: int, kind: str = "mixed",
                sampletype: int = 0) -> tuple[bytes, int]:
    """Synthetic image: smooth gradients + noise, some flat and extreme areas,
    and (with alpha) a mix of opaque, transparent and partial pixels."""
    nch = num_channels(imgtype)
    if sampletype == SAMPLETYPE_FLOAT:
        a = rng.random((h, w, nch), dtype=np.float32) * np.float32(1.2) - np.float32(0.1)
        return a.astype("<f4").tobytes(), w * nch * 4
    maxv = (1 << depth) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    base = np.zeros((h, w, nch), dtype=np.float64)
    for c in range(nch):
        fx, fy = rng.uniform(0.5, 3.0, 2)
        ph = rng.uniform(0, 6.28)
        g = 0.5 + 0.5 * np.sin(fx * 6.28 * xx / max(w, 1) + fy * 6.28 * yy / max(h, 1) + ph)
        base[..., c] = g
    if kind in ("mixed", "noise"):
        base += rng.normal(0, 0.08 if kind == "mixed" else 0.3, base.shape)
    v = np.clip(np.rint(base * maxv), 0, maxv).astype(np.int64)
    if kind == "mixed" and h > 4 and w > 4:
        v[: h // 4, : w // 4, :] = maxv  # a saturated block
        v[-(h // 5):, -(w // 5):, :] = 0  # a black block
    if imgtype in (IMGTYPE_GRAYA, IMGTYPE_RGBA):
        a = v[..., -1]
        m = rng.random((h, w))
        a[m < 0.25] = 0
        a[(m >= 0.25) & (m < 0.55)] = maxv
        if h > 6 and w > 6:
            a[h // 3: h // 3 + max(2, h // 6), w // 3: w // 3 + max(2, w // 6)] = 0
        v[..., -1] = a
    if depth == 16:
        raw = v.astype(">u2").tobytes()
        return raw, w * nch * 2
    if depth == 8:
        return v.astype(np.uint8).tobytes(), w * nch
    # 1/2/4-bit gray, packed MSB-first, rows padded to whole bytes
    assert nch == 1
    bpr = (w * depth + 7) // 8
    out = bytearray(bpr * h)
    per = 8 // depth
    for y in range(h):
        for x in range(w):
            out[y * bpr + x // per] |= int(v[y, x, 0]) << (8 - depth * (x % per + 1))
    return bytes(out), bpr


def _resize_calls(fam, p1, p2, blur=1.0, dims=(0, 1)):
    return [("iw_set_resize_alg", d, RT[fam], blur, float(p1), float(p2)) for d in dims]


def random_case(seed: int, max_dim: int = 48) -> Job:
    """One randomly configured job; the same seed always gives the same job."""
    rng = np.random.default_rng(seed)
    r = rng.random

    # input
    kind = rng.choice(["gray", "graya", "rgb", "rgba"])
    imgtype = dict(gray=IMGTYPE_GRAY, graya=IMGTYPE_GRAYA, rgb=IMGTYPE_RGB, rgba=IMGTYPE_RGBA)[kind]
    sampletype = 0
    if imgtype == IMGTYPE_GRAY and r() < 0.2:
        depth = int(rng.choice([1, 2, 4]))
    else:
        depth = int(rng.choice([8, 8, 16]))
    if r() < 0.04 and depth == 8:
        sampletype, depth = SAMPLETYPE_FLOAT, 32
    big = r() < 0.45  # > 512 pixels: exercises the reference's lookup tables
    lo = 24 if big else 2
    w = int(rng.integers(lo, max_dim + 1))
    h = int(rng.integers(lo, max_dim + 1))
    orient = int(rng.integers(0, 8)) if rng.random() < 0.1 else 0
    # With a transposing orientation (4..7) the stored image is h wide, w tall.
    pw, ph = (h, w) if orient >= 4 else (w, h)
    px, bpr = make_pixels(rng, imgtype, depth, pw, ph, str(rng.choice(["mixed", "smooth", "noise"])), sampletype)

    calls: list[tuple] = []
    profile = int(rng.choice([PNG, PNG, PAM, PPM, RAW, RAW, MIFF, BMP, PNG & ~P["TRANSPARENCY"]]))
    if r() < 0.1:
        profile |= P["ALWAYSLINEAR"]
    calls.append(("iw_set_output_profile", profile))

    # output geometry
    ow = int(rng.integers(1, max_dim + 1)) if r() < 0.8 else w
    oh = int(rng.integers(1, max_dim + 1)) if r() < 0.8 else h
    if r() < 0.35 and big:
        ow, oh = max(24, ow), max(24, oh)  # keep output > 512 px sometimes
    calls.append(("iw_set_output_canvas_size", ow, oh))
    if r() < 0.1:
        calls.append(("iw_set_output_image_size", ow * rng.uniform(0.6, 1.0), oh * rng.uniform(0.6, 1.0)))
    if r() < 0.15:
        calls.append(("iw_set_input_crop", int(rng.integers(-2, w)), int(rng.integers(-2, h)),
                      int(rng.integers(-1, w + 2)), int(rng.integers(-1, h + 2))))

    # resampling
    for d in (0, 1):
        if d == 1 and r() < 0.6:
            calls.append(calls[-1][:1] + (1,) + calls[-1][2:])  # same filter both ways
            continue
        fam, p1, p2 = FILTERS[int(rng.integers(len(FILTERS)))]
        blur = 1.0 if r() < 0.8 else float(rng.choice([0.5, 0.8, 1.3, 2.0]))
        calls += _resize_calls(fam, p1, p2, blur, dims=(d,))
    for d, code in ((0, VAL["EDGE_POLICY_X"]), (1, VAL["EDGE_POLICY_Y"])):
        if r() < 0.35:
            calls.append(("iw_set_value", code, int(rng.choice([1, 2, 3]))))
    if r() < 0.12:
        calls.append(("iw_set_value_dbl", VAL["TRANSLATE_X"], float(rng.uniform(-3, 3))))
    if r() < 0.12:
        calls.append(("iw_set_value_dbl", VAL["TRANSLATE_Y"], float(rng.uniform(-3, 3))))
    if r() < 0.08:
        for ct in (CT_RED, CT_BLUE):
            calls.append(("iw_set_channel_offset", ct, int(rng.integers(0, 2)), float(rng.uniform(-1, 1))))

    # colour spaces and precision
    def cs():
        t = int(rng.choice([CS_SRGB, CS_SRGB, CS_LINEAR, CS_GAMMA, CS_REC709]))
        return ("cs", t, float(rng.uniform(0.4, 2.6)) if t == CS_GAMMA else 0.0)
    if r() < 0.3:
        calls.append(("iw_set_input_colorspace", cs()))
    if r() < 0.3:
        calls.append(("iw_set_output_colorspace", cs()))
    if r() < 0.05:
        calls.append(("iw_set_value", VAL["DISABLE_GAMMA"], 1))
    if r() < 0.08:
        calls.append(("iw_set_value", VAL["INT_CLAMP"], 1))
    if r() < 0.3:
        calls.append(("iw_set_output_depth", 16))
    if r() < 0.12:
        for ct in (CT_RED, CT_GREEN, CT_BLUE, CT_ALPHA, CT_GRAY):
            if r() < 0.6:
                calls.append(("iw_set_output_max_color_code", ct, int(rng.integers(1, 300))))
    if r() < 0.15:
        calls.append(("iw_set_color_count", int(rng.choice([CT_ALL, CT_NONALPHA, CT_ALPHA, CT_GRAY])),
                      int(rng.integers(1, 40))))
    if r() < 0.05 and depth == 8:
        calls.append(("iw_set_input_max_color_code", int(rng.integers(0, num_channels(imgtype))),
                      int(rng.integers(1, 255))))

    # dithering
    dr = r()
    if dr < 0.2:
        calls.append(("iw_set_dither_type", int(rng.choice([CT_ALL, CT_NONALPHA, CT_ALPHA])), DITHER_ORDERED,
                      int(rng.integers(0, 2))))
    elif dr < 0.4:
        calls.append(("iw_set_dither_type", int(rng.choice([CT_ALL, CT_NONALPHA])), DITHER_ERRDIFF,
                      int(rng.integers(0, 8))))
    elif dr < 0.48:
        calls.append(("iw_set_dither_type", CT_ALL, DITHER_RANDOM, int(rng.integers(0, 2))))
        calls.append(("iw_set_random_seed", 0, int(rng.integers(0, 1000))))

    # backgrounds, labels, grayscale, negation, post-pass options
    if r() < 0.25:
        calls.append(("iw_set_apply_bkgd_2", tuple(float(x) for x in rng.random(3)) + (
            1.0 if r() < 0.7 else float(rng.random()),)))
        if r() < 0.4:
            calls.append(("iw_set_bkgd_checkerboard_2", int(rng.integers(0, 7)),
                          tuple(float(x) for x in rng.random(3)) + (1.0 if r() < 0.7 else float(rng.random()),)))
            calls.append(("iw_set_bkgd_checkerboard_origin", int(rng.integers(0, 5)), int(rng.integers(0, 5))))
    if r() < 0.12:
        calls.append(("iw_set_input_bkgd_label", *(float(x) for x in rng.random(3))))
        if r() < 0.5:
            calls.append(("iw_set_value", VAL["USE_BKGD_LABEL"], 1))
    if r() < 0.08:
        calls.append(("iw_set_output_bkgd_label_2", tuple(float(x) for x in rng.random(3)) + (1.0,)))
    if r() < 0.15:
        calls.append(("iw_set_value", VAL["CVT_TO_GRAYSCALE"], 1))
        if r() < 0.5:
            calls.append(("iw_set_value", VAL["GRAYSCALE_FORMULA"], int(rng.integers(0, 4))))
            if r() < 0.5:
                calls.append(("iw_set_grayscale_weights", *(float(x) for x in rng.random(3))))
    if r() < 0.06:
        calls.append(("iw_set_value", VAL["NEGATE_TARGET"], 1))
    if r() < 0.2:
        for opt in range(1, 6):
            if r() < 0.5:
                calls.append(("iw_set_allow_opt", opt, 0))
    return Job(imgtype, depth, w, h, px, bpr=bpr, calls=calls, sampletype=sampletype, orient=orient)


def plain_small_case(seed: int = 1, w: int = 1024, h: int = 768, ow: int = 512, oh: int = 384) -> Job:
    """The plain small workload: 8-bit sRGB RGB, smooth gradients plus uniform
    noise in [-16, 16], Lanczos3 in linear light, 8-bit output, no dither."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.empty((h, w, 3))
    img[..., 0] = 255 * xx / (w - 1)
    img[..., 1] = 255 * yy / (h - 1)
    img[..., 2] = 255 * (xx + yy) / (w + h - 2)
    img += rng.integers(-16, 17, img.shape)
    px = np.clip(np.rint(img), 0, 255).astype(np.uint8).tobytes()
    calls = [("iw_set_output_profile", PPM), ("iw_set_output_canvas_size", ow, oh)]
    calls += _resize_calls("lanczos", 3, 0)
    return Job(IMGTYPE_RGB, 8, w, h, px, calls=calls)


def crop_case(i: int) -> Job:
    """A small image with a crop drawn to land outside it as often as inside:
    the reference's clamp then leaves zero or negative sizes (it limits the y
    origin by moving the x origin), which it refuses at its first buffer of
    that size or processes as an empty crop."""
    rng = np.random.default_rng(80_000 + i)
    w, h = int(rng.integers(1, 12)), int(rng.integers(1, 12))
    imgtype = [IMGTYPE_RGB, IMGTYPE_GRAY, IMGTYPE_RGBA][i % 3]
    calls = [("iw_set_output_profile", 0x41),
             ("iw_set_input_crop", int(rng.integers(-3, 20)), int(rng.integers(-3, 20)),
              int(rng.integers(-2, 15)), int(rng.integers(-2, 15))),
             ("iw_set_output_canvas_size", int(rng.integers(1, 15)), int(rng.integers(1, 15)))]
    fam = str(rng.choice(["auto", "null", "nearest", "mix", "cubic", "lanczos", "box"]))
    if fam != "auto":
        for d in (0, 1):
            calls.append(("iw_set_resize_alg", d, RT[fam], 1.0, 3.0 if fam == "lanczos" else 0.0, 0.5))
    if i % 5 == 0:
        calls.append(("iw_set_dither_type", CT_ALL, DITHER_ERRDIFF, 0))
    px = rng.integers(0, 256, w * h * num_channels(imgtype), dtype=np.uint8).tobytes()
    return Job(imgtype, 8, w, h, px, calls=calls)


def over_limit_cases() -> list[tuple[str, Job]]:
    """Jobs whose output or intermediate image exceeds the allocation limit
    (2e9 bytes by default, or a smaller one set by the caller)."""
    prof = ("iw_set_output_profile", 0x41)
    return [
        ("output 30000x30000 RGB", Job(IMGTYPE_RGB, 8, 1, 1, bytes(3), calls=[prof, ("iw_set_output_canvas_size", 30000, 30000)])),
        ("intermediate 23000x23000", Job(IMGTYPE_GRAY, 8, 23000, 1, bytes(23000),
                                         calls=[prof, ("iw_set_output_canvas_size", 1, 23000)])),
        ("alpha intermediate", Job(IMGTYPE_RGBA, 8, 23000, 1, bytes(92000), calls=[prof, ("iw_set_output_canvas_size", 1, 23000)])),
        ("limit 1e6", Job(IMGTYPE_GRAY, 8, 600, 1, bytes(600),
                          calls=[prof, ("iw_set_max_malloc", 1000000), ("iw_set_output_canvas_size", 1, 600)])),
    ]


def clamped_crop(job: Job) -> tuple[int, int, int, int]:
    """The crop (x, y, w, h) the reference's clamp gives an upright job
    (src/imagew-cmd.c:1311-1325 and the library's own clamp, which limits
    the y origin by moving the x origin)."""
    cx, cy, cw, ch = [c for c in job.calls if c[0] == "iw_set_input_crop"][0][1:]
    w, h = job.width, job.height
    x, y = max(cx, 0), max(cy, 0)
    if x > w - 1:
        x = w - 1
    if y > h - 1:
        x = h - 1
    cw = w - x if cw < 0 else cw
    ch = h - y if ch < 0 else ch
    cw, ch = max(cw, 1), max(ch, 1)
    cw = min(cw, w - x)
    ch = min(ch, h - y)
    return x, y, cw, ch

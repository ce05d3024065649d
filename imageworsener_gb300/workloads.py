"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Inputs are generated with integer hashing (splitmix64) and plain float64
arithmetic only -- no transcendental functions and no library random
generators -- so every machine (x86_64 or aarch64, any numpy) regenerates
byte-identical images from the same seed.  That lets golden output hashes
computed once with the reference stand in for the reference on machines where
it cannot run.

Configurations (output Mpix/s is measured on these):
  small     1024x768 RGB8 sRGB, gradients + uniform integer noise in [-16,16],
            Lanczos3 to 512x384, 8-bit output, no dither.
  precision 4096x4096 RGBA16, value-noise fields per channel, alpha uniform in
            [0,65535] with 20% of 64x64 blocks fully transparent; Mitchell
            (B=C=1/3) to 1000x1000, 8-bit output, 8x8 ordered dither on all
            channels, PNG-style output profile.
  downscale 8192x8192 RGB8, checkerboard of 1-64 px cells (one size per 256 px
            tile), random cell colours + approximately Gaussian noise (sigma 8,
            sum of four uniforms); Lanczos3 to 256x256, 8-bit output; the
            "fs4" variant adds Floyd-Steinberg dither to 4 bits/channel.
  batch     many images, width and height log-uniform in [64, 2048], gray /
            RGB / RGBA, 8 or 16 bit, fitted into a 256x256 box with a
            per-image filter from {lanczos3, mitchell, catrom, hermite, box}.
"""
from __future__ import annotations

import numpy as np

from .iwapi import (Job, RT, PROFILE, IMGTYPE_GRAY, IMGTYPE_RGB, IMGTYPE_RGBA, CT_ALL, DITHER_ORDERED,
                    DITHER_ERRDIFF, num_channels)

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """Vectorised splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M64
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int | tuple) -> np.ndarray:
    """Uniform doubles in [0,1) from (seed, stream, index)."""
    shape = (n,) if isinstance(n, int) else n
    count = int(np.prod(shape))
    base = np.uint64((seed * 1000003 + stream * 7919) & 0xFFFFFFFFFFFF) << np.uint64(16)
    idx = np.arange(count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = splitmix64((idx * np.uint64(0x100000001B3) + base) & M64)
    return ((h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)).reshape(shape)


def value_noise(seed: int, stream: int, h: int, w: int, cell: int) -> np.ndarray:
    """Smooth noise in [0,1]: random lattice values, smoothstep-interpolated."""
    gh, gw = h // cell + 2, w // cell + 2
    lat = uniform(seed, stream, (gh, gw))
    ys = np.arange(h, dtype=np.float64) / cell
    xs = np.arange(w, dtype=np.float64) / cell
    y0 = ys.astype(np.int64)
    x0 = xs.astype(np.int64)
    fy = ys - y0
    fx = xs - x0
    sy = fy * fy * (3.0 - 2.0 * fy)
    sx = fx * fx * (3.0 - 2.0 * fx)
    a = lat[y0][:, x0]
    b = lat[y0][:, x0 + 1]
    c = lat[y0 + 1][:, x0]
    d = lat[y0 + 1][:, x0 + 1]
    top = a + (b - a) * sx[None, :]
    bot = c + (d - c) * sx[None, :]
    return top + (bot - top) * sy[:, None]


PNG_PROFILE = (PROFILE["TRANSPARENCY"] | PROFILE["GRAYSCALE"] | PROFILE["PALETTETRNS"] | PROFILE["GRAY1"] |
               PROFILE["GRAY2"] | PROFILE["GRAY4"] | PROFILE["BPS16"] | PROFILE["BINARYTRNS"] | PROFILE["PAL1"] |
               PROFILE["PAL2"] | PROFILE["PAL4"] | PROFILE["PAL8"] | PROFILE["REDUCEDBITDEPTHS"] |
               PROFILE["PNG_BKGD"])
PPM_PROFILE = PROFILE["BPS16"] | PROFILE["REDUCEDBITDEPTHS"]


def _resize(fam, p1=0.0, p2=0.0):
    return [("iw_set_resize_alg", d, RT[fam], 1.0, float(p1), float(p2)) for d in (0, 1)]


def small(seed: int = 1, w: int = 1024, h: int = 768, ow: int = 512, oh: int = 384) -> Job:
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.empty((h, w, 3))
    img[..., 0] = 255.0 * xx / (w - 1)
    img[..., 1] = 255.0 * yy / (h - 1)
    img[..., 2] = 255.0 * (xx + yy) / (w + h - 2)
    noise = np.floor(uniform(seed, 1, (h, w, 3)) * 33.0) - 16.0
    px = np.clip(np.floor(img + noise + 0.5), 0, 255).astype(np.uint8).tobytes()
    calls = [("iw_set_output_profile", PPM_PROFILE), ("iw_set_output_canvas_size", ow, oh)] + _resize("lanczos", 3)
    return Job(IMGTYPE_RGB, 8, w, h, px, calls=calls)


def precision(seed: int = 2, n: int = 4096, out: int = 1000) -> Job:
    chans = []
    for c in range(3):
        f = 0.55 * value_noise(seed, 10 + c, n, n, 256) + 0.3 * value_noise(seed, 20 + c, n, n, 48) + \
            0.15 * value_noise(seed, 30 + c, n, n, 9)
        chans.append(np.clip(np.floor(f * 65535.0 + 0.5), 0, 65535))
    alpha = np.floor(uniform(seed, 40, (n, n)) * 65536.0)
    nb = n // 64
    trans = uniform(seed, 41, (nb, nb)) < 0.2
    mask = np.repeat(np.repeat(trans, 64, axis=0), 64, axis=1)
    alpha[mask[:n, :n]] = 0
    img = np.stack(chans + [alpha], axis=-1).astype(">u2")
    calls = [("iw_set_output_profile", PNG_PROFILE), ("iw_set_output_canvas_size", out, out),
             ("iw_set_dither_type", CT_ALL, DITHER_ORDERED, 0)] + _resize("cubic", 1 / 3, 1 / 3)
    return Job(IMGTYPE_RGBA, 16, n, n, img.tobytes(), calls=calls)


def downscale(seed: int = 3, n: int = 8192, out: int = 256, fs4: bool = False) -> Job:
    tiles = max(1, n // 256)
    cellsz = 1 + np.floor(uniform(seed, 50, (tiles, tiles)) * 64.0).astype(np.int64)
    xs = np.arange(n, dtype=np.int64)
    tx = np.minimum(xs // 256, tiles - 1)
    sigma_scale = 8.0 / (4.0 * 65536.0 * 65536.0 / 12.0) ** 0.5   # sum of four 16-bit uniforms -> sigma 8
    out_px = np.empty((n, n, 3), dtype=np.uint8)
    step = 256
    for y0 in range(0, n, step):
        ys = np.arange(y0, min(n, y0 + step), dtype=np.int64)
        ty = np.minimum(ys // 256, tiles - 1)
        cs = cellsz[ty][:, tx]                      # per-pixel cell size (that of its 256x256 tile)
        cy = ys[:, None] // cs
        cx = xs[None, :] // cs
        key = (cy * 1000003 + cx * 7 + ty[:, None] * 131 + tx[None, :] * 17).astype(np.uint64)
        img = np.empty((len(ys), n, 3), dtype=np.float64)
        with np.errstate(over="ignore"):
            for c in range(3):
                h = splitmix64((key * np.uint64(0x9E3779B97F4A7C15) + np.uint64(seed * 97 + c)) & M64)
                img[..., c] = (h >> np.uint64(56)).astype(np.float64)   # cell colour 0..255
            idx = ((ys[:, None, None] * n + xs[None, :, None]) * 3 + np.arange(3)[None, None, :]).astype(np.uint64)
            hn = splitmix64((idx + np.uint64((seed * 131 + 60) << 40)) & M64)
            s = np.zeros(hn.shape, dtype=np.float64)
            for q in range(4):
                s += ((hn >> np.uint64(16 * q)) & np.uint64(0xFFFF)).astype(np.float64)
        img += (s - 2.0 * 65535.0) * sigma_scale
        out_px[y0:y0 + len(ys)] = np.clip(np.floor(img + 0.5), 0, 255).astype(np.uint8)
    px = out_px.tobytes()
    calls = [("iw_set_output_profile", PPM_PROFILE), ("iw_set_output_canvas_size", out, out)] + _resize("lanczos", 3)
    if fs4:
        calls += [("iw_set_dither_type", CT_ALL, DITHER_ERRDIFF, 0)]
        calls += [("iw_set_output_max_color_code", ct, 15) for ct in (0, 1, 2)]
    return Job(IMGTYPE_RGB, 8, n, n, px, calls=calls)


# log-spaced sizes 64..2048 (integers; the list is fixed so no exp() is needed)
_LOGSIZES = [int(round(64 * 2 ** (k / 32))) for k in range(161)]
_FILTERS = [("lanczos", 3, 0), ("cubic", 1 / 3, 1 / 3), ("cubic", 0, 0.5), ("hermite", 0, 0), ("box", 0, 0)]


def bestfit(w: int, h: int, bw: int, bh: int) -> tuple[int, int]:
    """Largest size with the image's aspect ratio that fits a bw x bh box
    (the semantics of imagew's -bestfit, src/imagew-cmd.c:427-454)."""
    ow = bw
    oh = int(0.5 + (float(ow) * h) / w)
    if oh > bh:
        oh = bh
        ow = int(0.5 + (float(oh) * w) / h)
    return max(ow, 1), max(oh, 1)


def batch(count: int, seed: int = 4, box: int = 256, max_side: int = 2048) -> list[Job]:
    jobs = []
    u = uniform(seed, 70, (count, 6))
    sizes = [s for s in _LOGSIZES if s <= max_side]
    for k in range(count):
        w = sizes[int(u[k, 0] * len(sizes))]
        h = sizes[int(u[k, 1] * len(sizes))]
        imgtype = (IMGTYPE_GRAY, IMGTYPE_RGB, IMGTYPE_RGBA)[int(u[k, 2] * 3)]
        depth = 8 if u[k, 3] < 0.5 else 16
        fam, p1, p2 = _FILTERS[int(u[k, 4] * len(_FILTERS))]
        nch = num_channels(imgtype)
        maxv = (1 << depth) - 1
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
        base = (xx / max(w - 1, 1))[..., None] * np.linspace(0.2, 1.0, nch)[None, None, :] + \
            (yy / max(h - 1, 1))[..., None] * np.linspace(0.8, 0.1, nch)[None, None, :]
        noise = uniform(seed, 1000 + k, (h, w, nch)) * 0.1
        v = np.clip(np.floor((0.5 * base + noise) * maxv + 0.5), 0, maxv)
        px = v.astype(">u2" if depth == 16 else np.uint8).tobytes()
        ow, oh = bestfit(w, h, box, box)
        calls = [("iw_set_output_profile", PNG_PROFILE), ("iw_set_output_canvas_size", ow, oh),
                 ("iw_set_output_depth", depth)] + _resize(fam, p1, p2)
        jobs.append(Job(imgtype, depth, w, h, px, calls=calls))
    return jobs


# 4:3 input sizes 160x120 .. 1024x768 (log-spaced widths)
_UPWIDTHS = [int(round(160 * 2 ** (k / 16))) // 4 * 4 for k in range(43)]


def upscale_pool(count: int, seed: int = 6) -> list[Job]:
    """Serving-mix upscales: 4:3 inputs 160x120..1024x768, RGB or RGBA 8-bit,
    enlarged 2-4x with Catmull-Rom (cubic B=0, C=0.5)."""
    jobs = []
    u = uniform(seed, 80, (count, 4))
    widths = [w for w in _UPWIDTHS if w <= 1024]
    for k in range(count):
        w = widths[int(u[k, 0] * len(widths))]
        h = w * 3 // 4
        imgtype = (IMGTYPE_RGB, IMGTYPE_RGBA)[int(u[k, 1] * 2)]
        factor = 2.0 + 2.0 * u[k, 2]
        ow, oh = int(w * factor), int(h * factor)
        nch = 3 if imgtype == IMGTYPE_RGB else 4
        yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
        base = (xx / max(w - 1, 1))[..., None] * np.linspace(0.3, 0.9, nch)[None, None, :] + \
            (yy / max(h - 1, 1))[..., None] * np.linspace(0.7, 0.2, nch)[None, None, :]
        noise = uniform(seed, 2000 + k, (h, w, nch)) * 0.1
        px = np.clip(np.floor((0.5 * base + noise) * 255.0 + 0.5), 0, 255).astype(np.uint8).tobytes()
        calls = [("iw_set_output_profile", PNG_PROFILE), ("iw_set_output_canvas_size", ow, oh)] + _resize("cubic", 0.0, 0.5)
        jobs.append(Job(imgtype, 8, w, h, px, calls=calls))
    return jobs


def serving_schedule(rate: float, seconds: float, seed: int = 7) -> list[tuple[float, str, bool]]:
    """Poisson arrivals: (time s, "thumb" | "up", error diffusion?) -- 70 %
    thumbnails, 30 % upscales, 10 % of all requests with error diffusion."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            return out
        out.append((t, "thumb" if rng.random() < 0.7 else "up", bool(rng.random() < 0.1)))


def out_pixels(job: Job) -> int:
    """Output pixel count of a job (its canvas size)."""
    for c in job.calls:
        if c[0] == "iw_set_output_canvas_size":
            return int(c[1]) * int(c[2])
    return 0


def in_bytes(job: Job) -> int:
    return job.bpr * job.height

"""Input files and option sets for the command-line tool's tests: seeded PNM /
PAM images written to a directory, and the argument lists tried on them."""
from __future__ import annotations

import os

import numpy as np

KINDS = ["ppm8", "ppm16", "pgm8", "pgm1000", "pam_rgba8", "pam_rgba16", "pam_graya8", "pam_gray31", "pam_rgb8", "pbm"]


def write_input(path: str, kind: str, w: int, h: int, seed: int) -> None:
    """A seeded image of the given kind (gradient plus noise, some flat areas)."""
    rng = np.random.default_rng(seed)
    nch = {"ppm8": 3, "ppm16": 3, "pgm8": 1, "pgm1000": 1, "pam_rgba8": 4, "pam_rgba16": 4, "pam_graya8": 2,
           "pam_gray31": 1, "pam_rgb8": 3, "pbm": 1}[kind]
    maxval = {"ppm16": 65535, "pgm1000": 1000, "pam_rgba16": 65535, "pam_gray31": 31, "pbm": 1}.get(kind, 255)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    base = np.stack([(xx / max(w - 1, 1)) * (0.3 + 0.2 * c) + (yy / max(h - 1, 1)) * (0.6 - 0.1 * c)
                     for c in range(nch)], axis=-1) * 0.8
    v = np.clip(base + rng.uniform(-0.15, 0.15, base.shape), 0, 1)
    if nch in (2, 4):   # alpha: opaque, transparent and partial areas
        a = v[..., -1]
        a[(xx < w / 3)] = 1.0
        a[(yy < h / 4) & (xx >= w / 3)] = 0.0
    q = np.floor(v * maxval + 0.5).astype(np.int64)
    with open(path, "wb") as f:
        if kind == "pbm":
            bits = (q[..., 0] == 0).astype(np.uint8)   # 1 = black
            f.write(b"P4\n%d %d\n" % (w, h))
            f.write(np.packbits(bits, axis=1).tobytes())
            return
        dt = ">u2" if maxval > 255 else np.uint8
        data = q.astype(dt).tobytes()
        if kind.startswith("ppm"):
            f.write(b"P6\n%d %d\n%d\n" % (w, h, maxval))
        elif kind.startswith("pgm"):
            f.write(b"P5\n# seeded test image\n%d %d\n%d\n" % (w, h, maxval))
        else:
            tt = {1: b"GRAYSCALE", 2: b"GRAYSCALE_ALPHA", 3: b"RGB", 4: b"RGB_ALPHA"}[nch]
            f.write(b"P7\nWIDTH %d\nHEIGHT %d\nDEPTH %d\nMAXVAL %d\nTUPLTYPE %s\nENDHDR\n" % (w, h, nch, maxval, tt))
        f.write(data)


FILTERS = ["lanczos", "lanczos2", "mitchell", "catrom", "hermite", "box", "boxavg", "triangle", "gaussian", "mix",
           "nearest", "hann4", "blackman", "sinc3", "bspline", "cubic0.5,0.25", "keys0.6", "quadratic", "auto"]
DITHERS = ["f", "o", "halftone", "r", "r2", "jjn", "stucki", "burkes", "sierra", "sierra2", "sierralite",
           "atkinson", "none"]
OUTS = ["ppm", "pgm", "pam", "pnm"]


def case(seed: int) -> dict:
    """One CLI case: input kind and size, output extension, arguments."""
    rng = np.random.default_rng(10_000 + seed)
    kind = KINDS[int(rng.integers(len(KINDS)))]
    w, h = int(rng.integers(1, 160)), int(rng.integers(1, 160))
    out = OUTS[int(rng.integers(len(OUTS)))]
    args: list[str] = []
    r = rng.random
    pick = r()
    if pick < 0.3:
        args += ["-w", str(int(rng.integers(1, 220)))]
    elif pick < 0.5:
        args += ["-h", str(int(rng.integers(1, 220)))]
    elif pick < 0.75:
        args += ["-w", str(int(rng.integers(1, 220))), "-h", str(int(rng.integers(1, 220)))]
        if r() < 0.5:
            args.append("-bestfit")
    elif pick < 0.85:
        args.append("-noresize")
    if r() < 0.6:
        args += ["-filter", FILTERS[int(rng.integers(len(FILTERS)))]]
    elif r() < 0.3:
        args += ["-filterx", FILTERS[int(rng.integers(len(FILTERS)))], "-filtery", FILTERS[int(rng.integers(len(FILTERS)))]]
    if r() < 0.15:
        args += ["-blur", str(float(rng.choice([0.6, 1.5, 2.0])))]
    if r() < 0.2:
        args += ["-edge", str(rng.choice(["s", "r", "t"]))]
    if r() < 0.3:
        args += ["-depth", str(int(rng.choice([1, 2, 4, 5, 8, 12, 16])))]
    if r() < 0.2:
        args += ["-cc", str(int(rng.choice([2, 5, 16, 100])))]
    if r() < 0.35:
        args += ["-dither", DITHERS[int(rng.integers(len(DITHERS)))]]
    if r() < 0.15:
        args.append("-grayscale")
    if r() < 0.15:
        args += ["-crop", "%d,%d,%d,%d" % (int(rng.integers(-2, w)), int(rng.integers(-2, h)),
                                         int(rng.integers(-1, w + 2)), int(rng.integers(-1, h + 2)))]
    return {"seed": seed, "kind": kind, "w": w, "h": h, "out": out, "args": args}


def run_case(exe: str, c: dict, tmpdir: str) -> tuple[int, str | None]:
    """(exit code, SHA-256 of the written file or None) of one case."""
    import hashlib
    import subprocess
    inp = os.path.join(tmpdir, "in_%d.%s" % (c["seed"], "pam" if c["kind"].startswith("pam") else
                                             ("pbm" if c["kind"] == "pbm" else c["kind"][:3])))
    if not os.path.exists(inp):
        write_input(inp, c["kind"], c["w"], c["h"], c["seed"])
    out = os.path.join(tmpdir, "out_%d_%s.%s" % (c["seed"], os.path.basename(exe), c["out"]))
    if os.path.exists(out):
        os.remove(out)
    r = subprocess.run([exe, "-noinfo", "-nowarn", *c["args"], inp, out], capture_output=True, timeout=120)
    digest = None
    if os.path.exists(out):
        with open(out, "rb") as f:
            digest = hashlib.sha256(f.read()).hexdigest()
    return r.returncode, digest

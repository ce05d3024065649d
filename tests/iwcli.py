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


HEX = ["ff0000", "0f0", "12345678", "0000ffff0000", "808080", "fff", "c0ffee80", "zz"]
REORIENT = ["fliph", "flipv", "rotate90", "rotate180", "rotate270", "transpose", "transverse", "3", "6"]
CSPACES = ["linear", "gamma1.8", "gamma2.4", "srgb", "srgbp", "srgbr", "rec709"]


def _extra_options(rng) -> list[str]:
    """One of the options beyond size / filter / depth / dither / crop:
    relative and fitted sizes, interpolating blur, translation, image size,
    channel offsets, per-channel depths / colour counts / dithers, grayscale
    formulas, colour spaces, gamma and clamping switches, optimisation
    switches, random seeds, backgrounds, reorientation, PBM output."""
    i = int(rng.integers(22))
    num = lambda lo, hi: "%g" % round(float(rng.uniform(lo, hi)), 2)  # noqa: E731
    if i == 0:
        return [str(rng.choice(["-w", "-h"])), "x" + num(0.2, 2.5)]
    if i == 1:
        return [str(rng.choice(["-s", "-S"])), "%d,%d" % (int(rng.integers(1, 200)), int(rng.integers(1, 200)))]
    if i == 2:
        return [str(rng.choice(["-blur", "-blurx", "-blury"])), str(rng.choice(["x", "x" + num(0.5, 1.5)]))]
    if i == 3:
        return ["-translate", ("s" if rng.random() < 0.4 else "") + num(-3, 3) + "," + num(-3, 3)] + \
            (["-edge", "t"] if rng.random() < 0.5 else [])
    if i == 4:
        return ["-imagesize", "%s,%s" % (num(5, 120), num(5, 120)), "-edge", str(rng.choice(["s", "t"]))]
    if i == 5:
        return ["-offset" + str(rng.choice(["red", "green", "blue", "rb", "vred", "vgreen", "vblue", "vrb"])), num(-2, 2)]
    if i == 6:
        return ["-depth", ",".join(str(int(rng.integers(1, 17))) for _ in range(int(rng.integers(3, 5))))]
    if i == 7:
        return [str(rng.choice(["-depthgray", "-depthalpha"])), str(int(rng.integers(1, 16)))]
    if i == 8:
        return ["-depthcc", str(int(rng.choice([2, 3, 6, 100, 300])))]
    if i == 9:
        return ["-cc", ",".join(str(int(rng.integers(2, 40))) for _ in range(4))]
    if i == 10:
        return ["-cc" + str(rng.choice(["color", "alpha", "red", "green", "blue", "gray"])), str(int(rng.integers(2, 20)))]
    if i == 11:
        return ["-dither" + str(rng.choice(["color", "alpha", "red", "green", "blue", "gray"])),
                str(rng.choice(DITHERS)), "-cc", str(int(rng.integers(2, 12)))]
    if i == 12:
        return [str(rng.choice(["-gsf", "-grayscaleformula"])),
                str(rng.choice(["s", "c", "w0.2,0.5,0.3", "v1,0.4,0.1", "v1", "w2,1,1"]))]
    if i == 13:
        return ["-condgrayscale"]
    if i == 14:
        return [str(rng.choice(["-cs", "-inputcs"])), str(rng.choice(CSPACES))] + \
            (["-intent", str(rng.choice(["p", "r", "s", "a", "default", "none", "d"]))] if rng.random() < 0.3 else [])
    if i == 15:
        return [str(rng.choice(["-nogamma", "-intclamp", "-negate", "-nocslabel"]))]
    if i == 16:
        return ["-noopt", str(rng.choice(["all", "grayscale", "palette", "reduceto8", "stripalpha", "binarytrns"]))]
    if i == 17:
        return ["-randseed", str(int(rng.integers(1, 1000))), "-dither", str(rng.choice(["r", "r2"])),
                "-cc", str(int(rng.integers(2, 8)))]
    if i == 18:
        if rng.random() < 0.5:
            return ["-bkgd", str(rng.choice(HEX))]
        return ["-bkgd", "%s,%s" % (rng.choice(HEX[:6]), rng.choice(HEX[:6])), "-checkersize", str(int(rng.integers(1, 9))),
                "-checkerorigin", "%d,%d" % (int(rng.integers(0, 5)), int(rng.integers(0, 5)))]
    if i == 19:
        return ["-reorient", str(rng.choice(REORIENT))]
    if i == 20:
        return ["-outfmt", "pbm"] + (["-dither", str(rng.choice(["f", "o", "halftone"]))] if rng.random() < 0.5 else [])
    return ["-nobestfit", "-w", str(int(rng.integers(1, 200))), "-h", str(int(rng.integers(1, 200))), "-bestfit"]


def case_ext(seed: int) -> dict:
    """A case of case(seed)'s kind, size and output with one to three of the
    further options added."""
    c = case(seed)
    rng = np.random.default_rng(20_000 + seed)
    args = list(c["args"])
    for _ in range(int(rng.integers(1, 4))):
        args += _extra_options(rng)
    return {**c, "args": args}


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

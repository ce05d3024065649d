"""The reference's own regression suite -- tests/runtest, its srcimg/ inputs
and expected/ outputs -- replayed through a command-line tool that reads and
writes PNM/PAM files only.

* Each `$IW <in> <out> <options>` line of tests/runtest is expanded (shell
  variables and `for` loops).
* A PNG input is decoded (tests/pngread.py) the way the reference's PNG
  reader hands it to the library (src/imagew-png.c:296-401): palettes
  expanded to RGB(A), tRNS colour keys expanded to an alpha channel (low-bit
  gray to 8 bits first), sBIT applied as a shift plus maximum codes, other
  images at their own bit depth.  It is written as PGM/PPM/PAM.  For
  non-square pixel densities the size the front end would fit is computed
  here and passed as an exact size.  The four lines a PNM/PAM file cannot
  carry (per-channel sBIT in or out, the input's background label used as
  the background) run through the library API instead (api_jobs); lines
  with other formats (GIF, BMP, JPEG, WebP, TIFF, MIFF) are skipped.
* A PNG output is compared as sample values: the tool writes PAM instead (the
  PNG and PAM output profiles differ only in what the output optimizer may
  pack -- palettes, colour keys, 1/2/4-bit gray -- so the pixel values are
  the same), and both files become exact value/maxval fractions per channel
  (RGBA; colour of fully transparent pixels ignored).  PNM/PAM outputs are
  compared byte for byte as well.

Test infrastructure only.
"""
from __future__ import annotations

import os
import re
import shlex
import subprocess
from dataclasses import dataclass

import numpy as np

from pngread import read_png

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PNM_OUT = {"ppm", "pnm", "pam", "pgm", "pbm"}


def reference_tests_dir() -> str | None:
    """tests/ beside the reference's src/ (the location oracle/Makefile's
    REFSRC names, or the REFSRC environment variable); None if absent."""
    src = os.environ.get("REFSRC")
    if not src:
        with open(os.path.join(ROOT, "oracle", "Makefile")) as f:
            for line in f:
                m = re.match(r"^REFSRC\s*\?=\s*(\S+)", line)
                if m:
                    src = m.group(1)
    if not src:
        return None
    d = os.path.join(os.path.dirname(src.rstrip("/")), "tests")
    return d if os.path.isfile(os.path.join(d, "runtest")) else None


# --------------------------------------------------------------------------
# tests/runtest

def runtest_commands(path: str) -> list[list[str]]:
    """The imagew invocations of the script, as argument lists after the
    program name: [input, output, options...]."""
    with open(path) as f:
        text = f.read().replace("\\\n", " ")
    env: dict[str, str] = {}
    out: list[list[str]] = []

    def expand(s: str, loop: dict[str, str]) -> str:
        return re.sub(r"\$\{?(\w+)\}?", lambda m: loop.get(m.group(1), env.get(m.group(1), m.group(0))), s)

    lines = [ln.strip() for ln in text.splitlines()]
    i = 0
    while i < len(lines):
        ln = lines[i]
        m = re.match(r'^([A-Z][A-Z0-9]*)="([^"$]*)"$', ln)
        if m:
            env[m.group(1)] = m.group(2)
        elif ln.startswith("for "):
            var, values = re.match(r"^for (\w+) in (.*)$", ln).groups()
            body = []
            i += 1
            while lines[i] != "done":
                if lines[i] != "do":
                    body.append(lines[i])
                i += 1
            for v in values.split():
                for b in body:
                    if b.startswith("$IW "):
                        out.append(shlex.split(expand(b[4:], {var: v})))
        elif ln.startswith("$IW "):
            out.append(shlex.split(expand(ln[4:], {})))
        i += 1
    return out


# --------------------------------------------------------------------------
# files and sample values

class Unsupported(Exception):
    pass


def _write_pnm(path: str, s: np.ndarray, maxval: int) -> None:
    h, w, ch = s.shape
    data = s.astype(">u2" if maxval > 255 else np.uint8).tobytes()
    with open(path, "wb") as f:
        if ch == 1:
            f.write(b"P5\n%d %d\n%d\n" % (w, h, maxval))
        elif ch == 3:
            f.write(b"P6\n%d %d\n%d\n" % (w, h, maxval))
        else:
            tt = b"GRAYSCALE_ALPHA" if ch == 2 else b"RGB_ALPHA"
            f.write(b"P7\nWIDTH %d\nHEIGHT %d\nDEPTH %d\nMAXVAL %d\nTUPLTYPE %s\nENDHDR\n" % (w, h, ch, maxval, tt))
        f.write(data)


def png_as_read(path: str) -> tuple[np.ndarray, int, dict]:
    """(samples (h, w, ch), maxval, info) of a PNG file as the reference's
    reader passes it to the library; info: 'density' (x, y, unit) or None,
    'bkgd' True if the file has a background label."""
    g = read_png(path)
    s = g.samples.astype(np.int64)
    depth, ct = g.bit_depth, g.color_type
    info = {"density": g.phys, "bkgd": g.bkgd is not None}
    if g.gamma is not None and g.srgb_intent is None:
        raise Unsupported("gAMA input")
    if ct == 3:   # palette -> RGB or RGBA, 8 bits (src/imagew-png.c:322-325)
        idx = s[..., 0]
        rgb = g.palette[idx].astype(np.int64)
        if g.trns is not None:
            alpha = np.full(len(g.palette), 255, np.int64)
            alpha[:len(g.trns)] = np.frombuffer(g.trns, np.uint8)
            s = np.concatenate([rgb, alpha[idx][..., None]], axis=-1)
        else:
            s = rgb
        depth = 8
        if g.sbit is not None:   # shifted after the expansion; alpha counts as 8 bits
            bits = list(g.sbit[:3]) + ([8] if s.shape[-1] == 4 else [])
            if len(set(bits)) != 1:
                raise Unsupported("per-channel sBIT")
            s = s >> (8 - bits[0])
            return s, (1 << bits[0]) - 1, info
        return s, 255, info
    if g.trns is not None and ct in (0, 2):   # colour key -> alpha (src/imagew-png.c:326-332)
        if ct == 0:
            key = np.frombuffer(g.trns, ">u2")[:1]
        else:
            key = np.frombuffer(g.trns, ">u2")[:3]
        transparent = np.all(s == key.astype(np.int64), axis=-1)
        if depth < 8:   # low-bit gray is expanded to 8 bits first
            s = s * (255 // ((1 << depth) - 1))
            depth = 8
        top = (1 << depth) - 1
        s = np.concatenate([s, np.where(transparent, 0, top)[..., None]], axis=-1)
    if g.sbit is not None:
        bits = list(g.sbit[:s.shape[-1]])
        if len(set(bits)) != 1:
            raise Unsupported("per-channel sBIT")
        s = s >> (depth - bits[0])
        return s, (1 << bits[0]) - 1, info
    return s, (1 << depth) - 1, info


def read_pnm(path: str) -> tuple[np.ndarray, int]:
    """(samples (h, w, ch), maxval) of a binary PBM/PGM/PPM or PAM file."""
    with open(path, "rb") as f:
        data = f.read()
    magic = data[:2]
    pos = 2
    if magic == b"P7":
        hdr = {}
        while True:
            end = data.index(b"\n", pos)
            line = data[pos:end].strip()
            pos = end + 1
            if line == b"ENDHDR":
                break
            if line and not line.startswith(b"#"):
                k, _, v = line.partition(b" ")
                hdr[k.decode()] = v.strip().decode()
        w, h, ch, maxval = int(hdr["WIDTH"]), int(hdr["HEIGHT"]), int(hdr["DEPTH"]), int(hdr["MAXVAL"])
    else:
        nums = []
        while len(nums) < (2 if magic == b"P4" else 3):
            while data[pos:pos + 1].isspace():
                pos += 1
            if data[pos:pos + 1] == b"#":
                pos = data.index(b"\n", pos) + 1
                continue
            start = pos
            while not data[pos:pos + 1].isspace():
                pos += 1
            nums.append(int(data[start:pos]))
        pos += 1
        w, h = nums[0], nums[1]
        if magic == b"P4":
            rowbytes = (w + 7) // 8
            bits = np.unpackbits(np.frombuffer(data[pos:pos + rowbytes * h], np.uint8).reshape(h, rowbytes), axis=1)
            return (1 - bits[:, :w]).astype(np.int64)[..., None], 1
        maxval = nums[2]
        ch = 3 if magic == b"P6" else 1
    dt = ">u2" if maxval > 255 else np.uint8
    n = w * h * ch
    s = np.frombuffer(data[pos:pos + n * np.dtype(dt).itemsize], dt).astype(np.int64)
    return s.reshape(h, w, ch), maxval


def png_values(path: str) -> np.ndarray:
    """Exact sample fractions (h, w, 4) of a PNG as written by the reference:
    palette and colour key expanded, sBIT undone (src/imagew-png.c:769-778)."""
    g = read_png(path)
    s = g.samples.astype(np.int64)
    ct, depth = g.color_type, g.bit_depth
    if ct == 3:
        rgb = g.palette[s[..., 0]].astype(np.float64) / 255.0
        alpha = np.ones(s.shape[:2])
        if g.trns is not None:
            a = np.full(len(g.palette), 255, np.int64)
            a[:len(g.trns)] = np.frombuffer(g.trns, np.uint8)
            alpha = a[s[..., 0]] / 255.0
        return _rgba(np.concatenate([rgb, alpha[..., None]], axis=-1))
    maxv = np.full(s.shape[-1], (1 << depth) - 1, np.int64)
    if g.sbit is not None:
        bits = np.array(g.sbit[:s.shape[-1]], np.int64)
        s = s >> (depth - bits)
        maxv = (1 << bits) - 1
    v = s / maxv
    if g.trns is not None and ct in (0, 2):
        key = np.frombuffer(g.trns, ">u2")[:s.shape[-1]].astype(np.int64)
        transparent = np.all(g.samples.astype(np.int64) == key, axis=-1)
        v = np.concatenate([v, np.where(transparent, 0.0, 1.0)[..., None]], axis=-1)
    return _rgba(v)


def pnm_values(path: str) -> np.ndarray:
    s, maxval = read_pnm(path)
    return _rgba(s / float(maxval))


def _rgba(v: np.ndarray) -> np.ndarray:
    ch = v.shape[-1]
    if ch in (1, 2):
        v = np.concatenate([v[..., :1]] * 3 + ([v[..., 1:2]] if ch == 2 else []), axis=-1)
    if v.shape[-1] == 3:
        v = np.concatenate([v, np.ones(v.shape[:2] + (1,))], axis=-1)
    v = v.copy()
    v[v[..., 3] == 0, :3] = 0.0   # the colour of a fully transparent pixel is not compared
    return v


# --------------------------------------------------------------------------
# cases and replay

@dataclass
class Case:
    name: str             # the expected file's name
    source: str           # input, relative to the suite's folder
    options: list[str]
    skip: str | None = None

    @property
    def ext(self) -> str:
        return self.name.rsplit(".", 1)[1]


def _fits_size(opts: list[str]) -> bool:
    """Whether the front end fits the size to the input's aspect ratio (where
    non-square pixels would change it; src/imagew-cmd.c:836-840)."""
    if "-noresize" in opts:
        return False
    w = any(o in opts for o in ("-w", "-width", "-s", "-S"))
    h = any(o in opts for o in ("-h", "-height", "-s", "-S"))
    return not (w and h) or "-bestfit" in opts or "-s" in opts


def cases(tdir: str) -> list[Case]:
    out = []
    for args in runtest_commands(os.path.join(tdir, "runtest")):
        src, dst, opts = args[0], args[1], args[2:]
        c = Case(os.path.basename(dst), src.replace("actual/", "expected/"), opts)
        if c.ext not in PNM_OUT and c.ext != "png":
            c.skip = "%s output (not PNM/PAM/PNG)" % c.ext
        elif not src.endswith((".png", ".pgm", ".ppm", ".pam")):
            c.skip = "%s input (not PNM/PAM/PNG)" % src.rsplit(".", 1)[1]
        elif not os.path.exists(os.path.join(tdir, c.source)) or not os.path.exists(os.path.join(tdir, "expected", c.name)):
            c.skip = "no file"
        out.append(c)
    return out


def _density_size(opts: list[str], sw: int, sh: int, dx: float, dy: float) -> list[str]:
    """The options with the size the front end computes for an input of
    non-square pixels (src/imagew-cmd.c:805-900, do_bestfit :427-454): the
    source is stretched to square pixels before fitting.  Only -w/-width,
    -h/-height (pixels or x<factor>) and -density are expected here."""
    aw, ah = sw, sh
    if dx > dy:
        ah = int(0.5 + (dx / dy) * sh)
    else:
        aw = int(0.5 + (dy / dx) * sw)
    req = {0: -1, 1: -1}
    rest: list[str] = []
    it = iter(opts)
    for o in it:
        if o in ("-w", "-width", "-h", "-height"):
            k, v = (0 if o in ("-w", "-width") else 1), next(it)
            req[k] = max(1, int(0.5 + float(v[1:]) * (aw if k == 0 else ah))) if v.startswith("x") else int(v)
        elif o == "-density":
            rest += [o, next(it)]
        elif o.startswith("-") and o not in ("-zipcmprlevel",):
            raise Unsupported("non-square pixel density with option %s" % o)
        else:
            rest.append(o)
    w, h = req[0], req[1]
    if w == -1 and h == -1:
        w, h = aw, ah
    elif w == -1 or h == -1:   # fit the one given
        if h == -1:
            h = int(0.5 + ah * (w / aw))
        else:
            w = int(0.5 + aw * (h / ah))
    return rest + ["-S", "%d,%d" % (max(w, 1), max(h, 1))]


def prepare_input(c: Case, tdir: str, tmpdir: str) -> tuple[str, list[str]]:
    """The case's input as a file the PNM/PAM tool reads, and the options to
    give it (raises Unsupported)."""
    src = os.path.join(tdir, c.source)
    if not src.endswith(".png"):
        return src, c.options
    s, maxval, info = png_as_read(src)
    opts = c.options
    d = info["density"]
    if d is not None and d[0] != d[1] and _fits_size(c.options):
        opts = _density_size(c.options, s.shape[1], s.shape[0], float(d[0]), float(d[1]))
    if info["bkgd"] and "-usebkgdlabel" in c.options:
        raise Unsupported("input background label used as the background")
    ext = {1: "pgm", 3: "ppm"}.get(s.shape[-1], "pam")
    path = os.path.join(tmpdir, "in_" + c.name.rsplit(".", 1)[0].replace("/", "_") + "." + ext)
    _write_pnm(path, s, maxval)
    return path, opts


def expected_values(c: Case, tdir: str) -> np.ndarray:
    path = os.path.join(tdir, "expected", c.name)
    return png_values(path) if c.ext == "png" else pnm_values(path)


def run_case(exe: str, c: Case, tdir: str, tmpdir: str) -> tuple[str, str | None]:
    """('match' | 'differ' | 'failed' | 'skipped', detail) of one case run with
    the given tool."""
    if c.skip:
        return "skipped", c.skip
    try:
        inp, opts = prepare_input(c, tdir, tmpdir)
    except Unsupported as e:
        return "skipped", str(e)
    out_ext = "pam" if c.ext == "png" else c.ext
    out = os.path.join(tmpdir, "%s_%s.%s" % (os.path.basename(exe), c.name.rsplit(".", 1)[0], out_ext))
    if os.path.exists(out):
        os.remove(out)
    extra = ["-outfmt", "pam"] if c.ext == "png" else []
    r = subprocess.run([exe, "-noinfo", "-nowarn", *opts, *extra, inp, out], capture_output=True, timeout=120)
    if r.returncode or not os.path.exists(out):
        msg = r.stderr.decode(errors="replace").strip()
        if c.ext == "png" and "requires equal bit depths" in msg:
            return "skipped", "per-channel output depths (a PAM file holds one)"
        return "failed", msg
    want = expected_values(c, tdir)
    got = pnm_values(out)
    if c.ext != "png":
        with open(out, "rb") as f1, open(os.path.join(tdir, "expected", c.name), "rb") as f2:
            if f1.read() != f2.read():
                return "differ", "file bytes"
    if want.shape != got.shape:
        return "differ", "size %s vs %s" % (want.shape[:2], got.shape[:2])
    if not np.array_equal(want, got):
        n = int(np.count_nonzero(np.any(want != got, axis=-1)))
        return "differ", "%d of %d pixels" % (n, want.shape[0] * want.shape[1])
    return "match", None


# --------------------------------------------------------------------------
# lines replayed through the library API instead of the PNM/PAM tool

def result_values(r) -> np.ndarray:
    """Exact sample fractions (h, w, 4) of an output image from
    imageworsener_gb300.iwapi.run_job: palette, colour key and per-channel
    maximum codes resolved."""
    from imageworsener_gb300 import iwapi
    ch = iwapi.num_channels(r.imgtype)
    row_bytes = r.bpr
    raw = np.frombuffer(r.pixels, np.uint8).reshape(r.height, row_bytes)
    n = r.width * ch
    if r.bit_depth == 16:
        s = raw[:, :2 * n].copy().view(">u2").astype(np.int64)
    elif r.bit_depth == 8:
        s = raw[:, :n].astype(np.int64)
    else:
        bits = np.unpackbits(raw, axis=1)[:, :n * r.bit_depth].reshape(r.height, n, r.bit_depth)
        s = (bits.astype(np.int64) * (1 << np.arange(r.bit_depth - 1, -1, -1))).sum(axis=-1)
    s = s.reshape(r.height, r.width, ch)
    if r.imgtype == iwapi.IMGTYPE_PALETTE:
        pal = np.array(r.palette, np.float64) / 255.0
        return _rgba(pal[s[..., 0]])
    types = {iwapi.IMGTYPE_GRAY: [iwapi.CT_GRAY], iwapi.IMGTYPE_GRAYA: [iwapi.CT_GRAY, iwapi.CT_ALPHA],
             iwapi.IMGTYPE_RGB: [iwapi.CT_RED, iwapi.CT_GREEN, iwapi.CT_BLUE],
             iwapi.IMGTYPE_RGBA: [iwapi.CT_RED, iwapi.CT_GREEN, iwapi.CT_BLUE, iwapi.CT_ALPHA]}[r.imgtype]
    top = (1 << r.bit_depth) - 1
    maxv = np.array([r.reduced_maxcolors[t] if r.reduced_maxcolors else top for t in types], np.float64)
    v = s / maxv
    if r.colorkey is not None:
        key = np.array(r.colorkey[:ch], np.int64)
        v = np.concatenate([v, np.where(np.all(s == key, axis=-1), 0.0, 1.0)[..., None]], axis=-1)
    return _rgba(v)


def api_jobs(tdir: str, lib) -> dict:
    """The regression lines whose inputs need library calls that a PNM/PAM
    file cannot express, as iwapi jobs for ``lib``: input maximum codes per
    channel from sBIT (src/imagew-png.c:182-226), the input's background label
    used as the background (src/imagew-png.c:228-250, src/imagew-cmd.c:1302),
    and output depths per channel (src/imagew-cmd.c:984-1044).  Each follows
    the front end's order of calls for the line's options; background colours
    are given in sRGB and linearised by ``lib`` as the front end does
    (src/imagew-cmd.c:1280-1291)."""
    import ctypes as C
    from imageworsener_gb300 import iwapi
    from pngread import read_png
    png = PNG_PROFILE
    srgb = iwapi.Csdescr(iwapi.CS_SRGB, 0, 0.0)
    lin = lambda x: lib.iw_convert_sample_to_linear(float(x), C.byref(srgb))   # noqa: E731

    def rgba8(name):
        g = read_png(os.path.join(tdir, "srcimg", name))
        if g.color_type != 3:
            return g.samples.astype(np.int64), g
        rgb = g.palette[g.samples[..., 0]].astype(np.int64)
        if g.trns is None:
            return rgb, g
        a = np.full(len(g.palette), 255, np.int64)
        a[:len(g.trns)] = np.frombuffer(g.trns, np.uint8)
        return np.concatenate([rgb, a[g.samples[..., 0]][..., None]], axis=-1), g

    def job(s, calls):
        h, w, ch = s.shape
        imgtype = {3: iwapi.IMGTYPE_RGB, 4: iwapi.IMGTYPE_RGBA}[ch]
        return iwapi.Job(imgtype, 8, w, h, s.astype(np.uint8).tobytes(), calls=calls)

    jobs = {}
    s, g = rgba8("rgb8a-sbit.png")   # sBIT on RGBA8, no options
    bits = np.array(g.sbit[:4], np.int64)
    jobs["sbit1.png"] = job(s >> (8 - bits), [("iw_set_input_max_color_code", k, (1 << int(bits[k])) - 1) for k in range(4)]
                            + [("iw_set_output_profile", png), ("iw_set_output_canvas_size", g.width, g.height)])
    s, g = rgba8("p8-sbit.png")      # palette with sBIT: shifted after the expansion
    bits = np.array(g.sbit[:3], np.int64)
    jobs["sbit2.png"] = job(s >> (8 - bits), [("iw_set_input_max_color_code", k, (1 << int(bits[k])) - 1) for k in range(3)]
                            + [("iw_set_output_profile", png), ("iw_set_output_canvas_size", g.width, g.height)])
    s, g = rgba8("rgb8a.png")        # -width 24 -height 24 -depth 6,8,5,7
    jobs["sbitw.png"] = job(s, [("iw_set_output_profile", png), ("iw_set_output_depth", 8),
                                ("iw_set_output_max_color_code", 0, 63), ("iw_set_output_max_color_code", 2, 31),
                                ("iw_set_output_max_color_code", 3, 127), ("iw_set_output_canvas_size", 24, 24)])
    s, g = rgba8("p8tbg.png")        # -bkgd 080,008 -checkersize 2 -usebkgdlabel; bKGD = a palette entry
    label = g.palette[g.bkgd[0]] / 255.0
    jobs["rbkgd2.png"] = job(s, [("iw_set_input_bkgd_label", *(float(x) for x in label)),
                                 ("iw_set_output_profile", png),
                                 ("iw_set_apply_bkgd_2", (lin(0), lin(8 / 15), lin(0), 1.0)),
                                 ("iw_set_bkgd_checkerboard_2", 2, (lin(0), lin(0), lin(8 / 15), 1.0)),
                                 ("iw_set_bkgd_checkerboard_origin", 0, 0),
                                 ("iw_set_value", iwapi.VAL["USE_BKGD_LABEL"], 1),
                                 ("iw_set_output_canvas_size", g.width, g.height)])
    return jobs


# the reference's PNG output profile (src/imagew-util.c:562-567)
PNG_PROFILE = 0x0001 | 0x0002 | 0x0004 | 0x0008 | 0x0010 | 0x0020 | 0x0040 | 0x0100 | 0x0200 | 0x0400 | 0x0800 | \
    0x1000 | 0x8000 | 0x10000

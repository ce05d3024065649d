"""ctypes binding of the libimagew C ABI (include/imagew.h).

The same binding drives any shared library that exports the libimagew core
API: the GPU library built by this package (``libimagew_gb300.so``), and,
in the tests, the CPU checkers.  Each library is opened with ``RTLD_LOCAL``
so several libraries exporting the same ``iw_*`` names coexist in one process.

A processing job is described by a :class:`Job`: the input image (raw bytes
in the reference's layout: interleaved samples, 16-bit samples big-endian,
rows ``bpr`` bytes apart) plus an ordered list of API calls that configure the
context.  :func:`run_job` creates a context, applies the calls, runs
``iw_process_image`` and returns the output image exactly as
``iw_get_output_image`` describes it (reference: src/imagew.h:497-737).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Any, Sequence

# ---- constants (values fixed by the ABI; see include/imagew.h) ----
IMGTYPE_GRAY, IMGTYPE_GRAYA, IMGTYPE_RGB, IMGTYPE_RGBA, IMGTYPE_PALETTE = 0x0001, 0x0101, 0x0010, 0x0110, 0x1000
SAMPLETYPE_UINT, SAMPLETYPE_FLOAT = 0, 1
DIM_H, DIM_V = 0, 1
CT_RED, CT_GREEN, CT_BLUE, CT_ALPHA, CT_GRAY, CT_ALL, CT_NONALPHA = 0, 1, 2, 3, 4, 10, 11
CS_SRGB, CS_LINEAR, CS_GAMMA, CS_REC709 = 0, 1, 2, 3
DITHER_NONE, DITHER_ORDERED, DITHER_ERRDIFF, DITHER_RANDOM = 0, 1, 2, 3
EDGE_REPLICATE, EDGE_STANDARD, EDGE_TRANSPARENT = 1, 2, 3
RT = dict(auto=0x01, null=0x02, nearest=0x10, mix=0x11, box=0x20, triangle=0x21, quadratic=0x22,
          gaussian=0x23, hermite=0x24, cubic=0x25, boxavg=0x26, sinc=0x30, lanczos=0x31, hanning=0x32,
          blackman=0x33)
PROFILE = dict(TRANSPARENCY=0x0001, GRAYSCALE=0x0002, PALETTETRNS=0x0004, GRAY1=0x0008, GRAY2=0x0010,
               GRAY4=0x0020, BPS16=0x0040, BINARYTRNS=0x0100, PAL1=0x0200, PAL2=0x0400, PAL4=0x0800,
               PAL8=0x1000, ALWAYSLINEAR=0x2000, HDRI=0x4000, REDUCEDBITDEPTHS=0x8000, PNG_BKGD=0x10000,
               RGB8_BKGD=0x20000, RGB16_BKGD=0x40000)
FMT_PNG, FMT_PAM, FMT_PPM, FMT_PGM, FMT_MIFF, FMT_BMP = 1, 12, 11, 10, 5, 3
VAL = dict(CVT_TO_GRAYSCALE=11, DISABLE_GAMMA=13, INT_CLAMP=15, GRAYSCALE_FORMULA=16, EDGE_POLICY_X=17,
           EDGE_POLICY_Y=18, TRANSLATE_X=42, TRANSLATE_Y=43, MAX_WIDTH=45, MAX_HEIGHT=46, NO_BKGD_LABEL=48,
           NEGATE_TARGET=53, USE_BKGD_LABEL=37)
OPT_GRAYSCALE, OPT_PALETTE, OPT_16_TO_8, OPT_STRIP_ALPHA, OPT_BINARY_TRNS = 1, 2, 3, 4, 5


def num_channels(imgtype: int) -> int:
    return {IMGTYPE_RGBA: 4, IMGTYPE_RGB: 3, IMGTYPE_GRAYA: 2}.get(imgtype, 1)


class Color(C.Structure):
    _fields_ = [("c", C.c_double * 4)]


class Csdescr(C.Structure):
    _fields_ = [("cstype", C.c_int), ("srgb_intent", C.c_int), ("gamma", C.c_double)]


class Image(C.Structure):
    _fields_ = [("imgtype", C.c_int), ("bit_depth", C.c_int), ("sampletype", C.c_int),
                ("width", C.c_int), ("height", C.c_int), ("pixels", C.c_void_p), ("bpr", C.c_size_t),
                ("orient_transform", C.c_uint), ("native_grayscale", C.c_int), ("density_code", C.c_int),
                ("density_x", C.c_double), ("density_y", C.c_double), ("has_colorkey_trns", C.c_int),
                ("colorkey", C.c_uint * 3), ("reduced_maxcolors", C.c_int), ("maxcolorcode", C.c_uint * 5),
                ("has_bkgdlabel", C.c_int), ("bkgdlabel", Color), ("rendering_intent", C.c_int)]


class RGBA8(C.Structure):
    _fields_ = [("r", C.c_ubyte), ("g", C.c_ubyte), ("b", C.c_ubyte), ("a", C.c_ubyte)]


class Palette(C.Structure):
    _fields_ = [("num_entries", C.c_int), ("entry", RGBA8 * 256)]


class InitParams(C.Structure):
    _fields_ = [("api_version", C.c_int), ("userdata", C.c_void_p), ("mallocfn", C.c_void_p),
                ("freefn", C.c_void_p)]


WARNFN = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p)

_libc = C.CDLL(None)
_libc.malloc.restype = C.c_void_p
_libc.malloc.argtypes = [C.c_size_t]
_libc.free.argtypes = [C.c_void_p]

_D, _I, _V, _P, _S = C.c_double, C.c_int, None, C.c_void_p, C.c_char_p
# name -> (restype, argtypes)
_SIGS: dict[str, tuple[Any, list[Any]]] = {
    "iw_create_context": (_P, [_P]),
    "iw_destroy_context": (_V, [_P]),
    "iw_process_image": (_I, [_P]),
    "iw_reorient_image": (_V, [_P, C.c_uint]),
    "iw_get_errorflag": (_I, [_P]),
    "iw_get_errormsg": (_S, [_P, _S, _I]),
    "iw_set_warning_fn": (_V, [_P, WARNFN]),
    "iw_set_max_malloc": (_V, [_P, C.c_size_t]),
    "iw_set_output_canvas_size": (_V, [_P, _I, _I]),
    "iw_set_output_image_size": (_V, [_P, _D, _D]),
    "iw_set_input_crop": (_V, [_P, _I, _I, _I, _I]),
    "iw_set_output_profile": (_V, [_P, C.c_uint]),
    "iw_set_output_depth": (_V, [_P, _I]),
    "iw_set_output_max_color_code": (_V, [_P, _I, _I]),
    "iw_set_dither_type": (_V, [_P, _I, _I, _I]),
    "iw_set_color_count": (_V, [_P, _I, _I]),
    "iw_set_resize_alg": (_V, [_P, _I, _I, _D, _D, _D]),
    "iw_set_channel_offset": (_V, [_P, _I, _I, _D]),
    "iw_set_grayscale_weights": (_V, [_P, _D, _D, _D]),
    "iw_set_input_bkgd_label": (_V, [_P, _D, _D, _D]),
    "iw_set_input_bkgd_label_2": (_V, [_P, C.POINTER(Color)]),
    "iw_set_output_bkgd_label_2": (_V, [_P, C.POINTER(Color)]),
    "iw_set_apply_bkgd_2": (_V, [_P, C.POINTER(Color)]),
    "iw_set_bkgd_checkerboard_2": (_V, [_P, _I, C.POINTER(Color)]),
    "iw_set_bkgd_checkerboard_origin": (_V, [_P, _I, _I]),
    "iw_set_output_colorspace": (_V, [_P, C.POINTER(Csdescr)]),
    "iw_set_input_colorspace": (_V, [_P, C.POINTER(Csdescr)]),
    "iw_make_gamma_csdescr": (_V, [C.POINTER(Csdescr), _D]),
    "iw_set_random_seed": (_V, [_P, _I, _I]),
    "iw_set_allow_opt": (_V, [_P, _I, _I]),
    "iw_set_input_image": (_V, [_P, C.POINTER(Image)]),
    "iw_get_output_image": (_V, [_P, C.POINTER(Image)]),
    "iw_get_output_colorspace": (_V, [_P, C.POINTER(Csdescr)]),
    "iw_get_output_palette": (C.POINTER(Palette), [_P]),
    "iw_set_value": (_V, [_P, _I, _I]),
    "iw_get_value": (_I, [_P, _I]),
    "iw_set_value_dbl": (_V, [_P, _I, _D]),
    "iw_get_value_dbl": (_D, [_P, _I]),
    "iw_set_option": (_V, [_P, _S, _S]),
    "iw_get_option": (_S, [_P, _S]),
    "iw_set_input_max_color_code": (_V, [_P, _I, _I]),
    "iw_get_version_int": (_I, []),
    "iw_get_profile_by_fmt": (C.c_uint, [_I]),
    "iw_convert_sample_to_linear": (_D, [_D, C.POINTER(Csdescr)]),
    "iw_convert_sample_from_linear": (_D, [_D, C.POINTER(Csdescr)]),
}


class IWLib:
    """One loaded library exporting the libimagew API."""

    def __init__(self, path: str):
        self.path = os.path.abspath(path)
        self.dll = C.CDLL(self.path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
        for name, (res, args) in _SIGS.items():
            fn = getattr(self.dll, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args

    def __getattr__(self, name: str):
        return getattr(self.dll, name)


@dataclass
class Job:
    """Input image plus the configuration calls applied before processing.

    ``calls`` is a sequence of ``(api_name, *args)``.  Colour arguments may be
    given as 4-tuples (converted to ``struct iw_color``) and colour-space
    arguments as ``("cs", cstype, gamma)``.
    """
    imgtype: int
    bit_depth: int
    width: int
    height: int
    pixels: bytes
    bpr: int = 0
    calls: Sequence[tuple] = field(default_factory=list)
    sampletype: int = SAMPLETYPE_UINT
    orient: int = 0

    def __post_init__(self):
        if not self.bpr:
            self.bpr = (self.width * self.bit_depth * num_channels(self.imgtype) + 7) // 8


@dataclass
class Result:
    ok: bool
    error: str | None
    imgtype: int = 0
    bit_depth: int = 0
    sampletype: int = 0
    width: int = 0
    height: int = 0
    bpr: int = 0
    pixels: bytes = b""
    palette: list[tuple[int, int, int, int]] | None = None
    colorkey: tuple[int, int, int] | None = None
    bkgdlabel: tuple[float, float, float, float] | None = None
    reduced_maxcolors: tuple[int, ...] | None = None
    warnings: list[str] = field(default_factory=list)

    def key(self):
        """Everything that must match between two implementations."""
        return (self.ok, self.error, self.imgtype, self.bit_depth, self.sampletype, self.width, self.height,
                self.bpr, self.pixels, self.palette, self.colorkey, self.bkgdlabel, self.reduced_maxcolors)

    def digest(self) -> str:
        """SHA-256 over :meth:`key` in a canonical encoding."""
        import hashlib
        h = hashlib.sha256()
        k = self.key()
        h.update(repr(k[:8]).encode())
        h.update(k[8])
        h.update(repr(k[9:]).encode())
        return h.hexdigest()


def _convert_arg(a):
    if isinstance(a, tuple) and len(a) == 3 and a[0] == "cs":
        cs = Csdescr()
        cs.cstype, cs.srgb_intent, cs.gamma = a[1], 0, a[2]
        return C.byref(cs)
    if isinstance(a, tuple) and len(a) == 4:
        col = Color()
        for i in range(4):
            col.c[i] = float(a[i])
        return C.byref(col)
    return a


def _setup(lib: IWLib, ctx, job: Job) -> None:
    # a transposing orientation (4..7) stores the image 'height' pixels wide
    nbytes = job.bpr * (job.width if job.orient >= 4 else job.height)
    buf = _libc.malloc(max(nbytes, 1))
    if not buf:
        raise MemoryError("malloc failed")
    C.memmove(buf, job.pixels, nbytes)
    img = Image()
    img.imgtype, img.bit_depth, img.sampletype = job.imgtype, job.bit_depth, job.sampletype
    img.width, img.height, img.pixels, img.bpr = job.width, job.height, buf, job.bpr
    img.orient_transform = job.orient
    lib.iw_set_input_image(ctx, C.byref(img))  # the library now owns buf
    for call in job.calls:
        name, args = call[0], [_convert_arg(a) for a in call[1:]]
        getattr(lib, name)(ctx, *args)


def _collect(lib: IWLib, ctx, ok: bool, warnings: list[str]) -> Result:
    err = None
    if lib.iw_get_errorflag(ctx):
        mb = C.create_string_buffer(256)
        err = lib.iw_get_errormsg(ctx, mb, 256).decode("utf-8", "replace")
    if not ok:
        return Result(False, err, warnings=warnings)
    out = Image()
    lib.iw_get_output_image(ctx, C.byref(out))
    n = out.bpr * out.height
    pix = C.string_at(out.pixels, n) if (out.pixels and n) else b""
    pal = None
    p = lib.iw_get_output_palette(ctx)
    if p:
        pal = [(p.contents.entry[i].r, p.contents.entry[i].g, p.contents.entry[i].b, p.contents.entry[i].a)
               for i in range(p.contents.num_entries)]
    ck = tuple(out.colorkey) if out.has_colorkey_trns else None
    lbl = tuple(out.bkgdlabel.c) if out.has_bkgdlabel else None
    rm = tuple(out.maxcolorcode) if out.reduced_maxcolors else None
    return Result(True, err, out.imgtype, out.bit_depth, out.sampletype, out.width, out.height, out.bpr,
                  pix, pal, ck, lbl, rm, warnings)


def run_job(lib: IWLib, job: Job, keep_warnings: bool = False) -> Result:
    """Run one job through ``lib`` and collect the output image."""
    ctx = lib.iw_create_context(None)
    if not ctx:
        return Result(False, "iw_create_context failed")
    warnings: list[str] = []
    cb = None
    try:
        if keep_warnings:
            cb = WARNFN(lambda _c, msg: warnings.append(msg.decode("utf-8", "replace")))
            lib.iw_set_warning_fn(ctx, cb)
        _setup(lib, ctx, job)
        ok = bool(lib.iw_process_image(ctx))
        return _collect(lib, ctx, ok, warnings)
    finally:
        lib.iw_destroy_context(ctx)
        del cb


def run_batch(lib: IWLib, jobs: Sequence[Job]) -> list[Result]:
    """Run jobs as one ``iwg_process_batch`` call (libimagew_gb300 only)."""
    ctxs = []
    try:
        for job in jobs:
            ctx = lib.iw_create_context(None)
            if not ctx:
                raise MemoryError("iw_create_context failed")
            ctxs.append(ctx)
            _setup(lib, ctx, job)
        f = lib.dll.iwg_process_batch
        f.restype = C.c_int
        f.argtypes = [C.POINTER(C.c_void_p), C.c_int]
        arr = (C.c_void_p * len(ctxs))(*ctxs)
        f(arr, len(ctxs))
        return [_collect(lib, ctx, not lib.iw_get_errorflag(ctx), []) for ctx in ctxs]
    finally:
        for ctx in ctxs:
            lib.iw_destroy_context(ctx)


class Completion(C.Structure):
    _fields_ = [("tag", C.c_ulonglong), ("ok", C.c_int), ("latency_ms", C.c_double), ("planned_ms", C.c_double),
                ("started_ms", C.c_double), ("ran_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("in_flight", C.c_int), ("queued", C.c_int), ("batches", C.c_longlong),
                ("batched_requests", C.c_longlong), ("device_ms", C.c_double), ("slow_batches", C.c_longlong),
                ("slow_requests", C.c_longlong), ("slow_device_ms", C.c_double), ("batch_wall_ms", C.c_double),
                ("rest_wall_ms", C.c_double), ("plan_ms", C.c_double), ("batch_phase_ms", C.c_double * 10)]


def server_api(lib: IWLib):
    """ctypes signatures of the iwg_server_* entry points."""
    d = lib.dll
    d.iwg_server_create.restype = C.c_void_p
    d.iwg_server_create.argtypes = [C.c_size_t, C.c_int, C.c_int]
    d.iwg_server_submit.restype = C.c_int
    d.iwg_server_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_ulonglong]
    d.iwg_server_poll.restype = C.c_int
    d.iwg_server_poll.argtypes = [C.c_void_p, C.POINTER(Completion), C.c_int, C.c_int]
    d.iwg_server_destroy.restype = None
    d.iwg_server_destroy.argtypes = [C.c_void_p]
    d.iwg_server_info.restype = C.c_int
    d.iwg_server_info.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    return d


def run_served(lib: IWLib, jobs: Sequence[Job], budget: int = 0, max_batch: int = 0) -> list[Result]:
    """Submit every job to one iwg_server, collect the completions."""
    d = server_api(lib)
    srv = d.iwg_server_create(budget, max_batch, 0)
    ctxs = []
    try:
        for k, job in enumerate(jobs):
            ctx = lib.iw_create_context(None)
            ctxs.append(ctx)
            _setup(lib, ctx, job)
            d.iwg_server_submit(srv, ctx, k)
        got = {}
        buf = (Completion * 64)()
        while len(got) < len(jobs):
            n = d.iwg_server_poll(srv, buf, 64, 10000)
            if n == 0:
                raise TimeoutError("server returned no completion within 10 s")
            for i in range(n):
                got[buf[i].tag] = buf[i].ok
        return [_collect(lib, ctxs[k], bool(got[k]), []) for k in range(len(jobs))]
    finally:
        d.iwg_server_destroy(srv)
        for ctx in ctxs:
            lib.iw_destroy_context(ctx)



class GpuStats(C.Structure):
    """struct iwg_stats (include/imagew_gb300.h)."""
    _fields_ = [("ms_total", C.c_double), ("ms_device", C.c_double), ("ms_part", C.c_double * 4),
                ("flagged", C.c_longlong), ("form", C.c_int), ("kernels", C.c_int), ("zero_copy", C.c_int),
                ("flagged_exact", C.c_longlong), ("vertical_tensor", C.c_int), ("graph", C.c_int),
                ("fused", C.c_int), ("ms_phase", C.c_double * 6)]


def _stats_dict(lib: IWLib, ctx) -> dict:
    st = GpuStats()
    lib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(GpuStats)]
    lib.dll.iwg_get_stats(ctx, C.byref(st))
    return {"form": st.form, "flagged": st.flagged, "flagged_exact": st.flagged_exact,
            "vertical_tensor": st.vertical_tensor, "fused": st.fused, "kernels": st.kernels,
            "ms_device": st.ms_device, "ms_part": list(st.ms_part), "ms_phase": list(st.ms_phase)}


def run_job_stats(lib: IWLib, job: Job) -> tuple:
    """``run_job`` through libimagew_gb300, also returning its iwg_stats as a dict."""
    ctx = lib.iw_create_context(None)
    if not ctx:
        raise MemoryError("iw_create_context failed")
    try:
        _setup(lib, ctx, job)
        ok = bool(lib.iw_process_image(ctx))
        return _collect(lib, ctx, ok, []), _stats_dict(lib, ctx)
    finally:
        lib.iw_destroy_context(ctx)


def run_debug_values(lib: IWLib, job: Job, precision: str):
    """Runs ``job`` once in the given form ("fp32" or "fp64") with the
    library's debug readback on and returns (result, interm, value, bound,
    stats): the intermediate image [n][rows][cols], the linear-light value
    each output sample is quantised from [channel][row][col] and, for the
    fp32 form, its rigorous error bound (all float64 numpy arrays; NaN where
    the tail decided without a value)."""
    import numpy as np
    f = lib.dll.iwg_debug_values
    f.restype = C.c_longlong
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_int)]
    ctx = lib.iw_create_context(None)
    if not ctx:
        raise MemoryError("iw_create_context failed")
    try:
        _setup(lib, ctx, job)
        lib.iw_set_option(ctx, b"gpu:precision", precision.encode())
        lib.iw_set_option(ctx, b"gpu:debug_values", b"1")
        ok = bool(lib.iw_process_image(ctx))
        res = _collect(lib, ctx, ok, [])
        arrays = []
        for which in range(3):
            dims = (C.c_int * 3)()
            n = f(ctx, which, None, 0, dims)
            a = np.empty(max(n, 0), dtype=np.float64)
            if n > 0:
                f(ctx, which, a.ctypes.data, n, dims)
                a = a.reshape(tuple(dims))
            arrays.append(a)
        return res, arrays[0], arrays[1], arrays[2], _stats_dict(lib, ctx)
    finally:
        lib.iw_destroy_context(ctx)


def fp_error(lib: IWLib, job: Job) -> dict:
    """Max and RMS error of the fp32 form's linear-light values against the
    fp64 form's (which are the reference's), at the two points the reference
    stores them: the float intermediate after the vertical pass and the value
    each output sample is quantised from; plus how many samples exceed the
    fp32 form's own bound (must be 0) and the flagged-pixel fraction."""
    import numpy as np
    r32, i32, v32, e32, s32 = run_debug_values(lib, job, "fp32")
    r64, i64, v64, _, s64 = run_debug_values(lib, job, "fp64")
    out = {"form": s32["form"], "identical_output": r32.ok and r64.ok and r32.key() == r64.key()}
    if s32["form"] != 1 or i32.shape != i64.shape or v32.shape != v64.shape:
        out["note"] = "the fp32 form does not take this configuration"
        return out
    di = np.abs(i32 - i64)
    ok = ~(np.isnan(v32) | np.isnan(v64))
    dv = np.abs(v32 - v64)[ok]
    eb = e32[ok]
    npx = v32.shape[1] * v32.shape[2]
    out.update({
        "interm_max": float(di.max()) if di.size else 0.0,
        "interm_rms": float(np.sqrt(np.mean(di * di))) if di.size else 0.0,
        "final_max": float(dv.max()) if dv.size else 0.0,
        "final_rms": float(np.sqrt(np.mean(dv * dv))) if dv.size else 0.0,
        "final_bound_max": float(eb.max()) if eb.size else 0.0,
        "final_max_over_bound": float((dv / np.maximum(eb, 1e-300)).max()) if dv.size else 0.0,
        "bound_violations": int((dv > eb).sum()),
        "samples": int(dv.size), "flagged_fraction": s32["flagged"] / npx,
        "flagged_left_to_fp64": s32["flagged_exact"], "vertical_tensor": s32["vertical_tensor"],
    })
    return out

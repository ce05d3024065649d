"""The host-side utility functions of the libimagew API -- number parsing,
transfer functions, format tables, byte order, sizes -- compared on
thousands of inputs between the product library (loaded without a GPU),
the oracle and, where it is built, the reference core.  Front ends parse
their options with these (the command-line tool does), so they must agree
with the reference's src/imagew-util.c and src/imagew-api.c to the bit.
"""
import ctypes as C
import string

import numpy as np
import pytest

from imageworsener_gb300.iwapi import Csdescr

_D, _I, _U, _P, _S = C.c_double, C.c_int, C.c_uint, C.c_void_p, C.c_char_p
SIGS = {
    "iw_parse_number": (_D, [_S]),
    "iw_parse_int": (_I, [_S]),
    "iw_parse_number_list": (_I, [_S, _I, C.POINTER(_D)]),
    "iw_round_to_int": (_I, [_D]),
    "iw_max_color_to_bitdepth": (_I, [_U]),
    "iw_imgtype_num_channels": (_I, [_I]),
    "iw_calc_bytesperrow": (C.c_size_t, [_I, _I]),
    "iw_is_valid_density": (_I, [_D, _D, _I]),
    "iw_stricmp": (_I, [_S, _S]),
    "iw_get_ui16le": (_U, [_S]), "iw_get_ui16be": (_U, [_S]), "iw_get_ui32le": (_U, [_S]),
    "iw_get_ui32be": (_U, [_S]), "iw_get_i32le": (_I, [_S]),
    "iw_get_ui16_e": (_U, [_S, _I]), "iw_get_ui32_e": (_U, [_S, _I]),
    "iw_set_ui16le": (None, [_P, _U]), "iw_set_ui16be": (None, [_P, _U]),
    "iw_set_ui32le": (None, [_P, _U]), "iw_set_ui32be": (None, [_P, _U]),
    "iw_get_host_endianness": (_I, []),
    "iw_detect_fmt_from_filename": (_I, [_S]),
    "iw_get_fmt_name": (_S, [_I]),
    "iw_get_profile_by_fmt": (_U, [_I]),
    "iw_convert_sample_to_linear": (_D, [_D, C.POINTER(Csdescr)]),
    "iw_convert_sample_from_linear": (_D, [_D, C.POINTER(Csdescr)]),
    "iw_strlcpy": (None, [_P, _S, C.c_size_t]),
    "iw_create_context": (_P, [_P]),
    "iw_destroy_context": (None, [_P]),
    "iw_check_image_dimensions": (_I, [_P, _I, _I]),
    "iw_get_errormsg": (_S, [_P, _S, _I]),
    "iw_get_errorflag": (_I, [_P]),
}


def _fns(lib):
    out = {}
    for name, (res, args) in SIGS.items():
        f = getattr(lib.dll, name)
        f.restype, f.argtypes = res, args
        out[name] = f
    return out


def _number_strings() -> list[bytes]:
    fixed = ["", "0", "1", "-1", "+1", "1.5", "-1.5", ".5", "-.5", "5.", "1e3", "1E3", "1e-3", "2.5e+2", "e5",
             "1.2.3", "--1", "+-1", " 7", "7 ", "x1.5", "0x10", "007", "1,2", "1,2,3,4,5", ",1", "1,,2", "1, 2",
             "3,", "-0", "0.0000001", "123456789012", "99999999999999999999", "1.9999999999999999", "0.5",
             "2.5", "-2.5", "1.49999999", "abc", "12abc", "1e", "1e+", ".", "-", "+", "1_000", "inf", "nan",
             "4294967296", "-2147483649", "2147483647.6", "1.5,-2.5,3.5,-4.5"]
    rng = np.random.default_rng(1)
    alphabet = list(string.digits * 3 + ".,-+eE x")
    rand = ["".join(rng.choice(alphabet, int(rng.integers(1, 14)))) for _ in range(3000)]
    return [s.encode() for s in fixed + rand]


def _observe(lib) -> list:
    f = _fns(lib)
    obs = []
    nums = (_D * 4)()
    for s in _number_strings():
        obs.append(("n", s, f["iw_parse_number"](s), f["iw_parse_int"](s)))
        for k in range(4):
            nums[k] = -777.0
        c = f["iw_parse_number_list"](s, 4, nums)
        obs.append(("l", s, c, tuple(nums)))
    for x in list(np.linspace(-6, 6, 97)) + [0.5, -0.5, 1.5, -1.5, 2.5, 1e9, -1e9, 0.49999999999999994]:
        obs.append(("r", float(x), f["iw_round_to_int"](float(x))))
    obs.append(("b", tuple(f["iw_max_color_to_bitdepth"](m) for m in range(0, 70000, 7))))
    obs.append(("c", tuple(f["iw_imgtype_num_channels"](t) for t in (0, 1, 0x101, 0x10, 0x110, 0x1000, 5))))
    obs.append(("bpr", tuple(f["iw_calc_bytesperrow"](n, b) for n in (0, 1, 3, 7, 8, 9, 1001)
                             for b in (1, 2, 4, 8, 16, 24, 32, 48, 64))))
    obs.append(("dens", tuple(f["iw_is_valid_density"](x, y, code) for x in (0.0, -1.0, 1.0, 2835.0, 1e-9, 1e9)
                              for y in (0.0, 1.0, 2835.0) for code in (0, 1, 2, 3))))
    pairs = [(b"abc", b"ABC"), (b"a", b"b"), (b"B", b"a"), (b"", b""), (b"png", b"PNGx"), (b"Zz", b"zZ")]
    obs.append(("cmp", tuple(int(np.sign(f["iw_stricmp"](a, b))) for a, b in pairs)))
    rng = np.random.default_rng(2)
    for _ in range(200):
        b = bytes(rng.integers(0, 256, 4, dtype=np.uint8))
        obs.append(("ui", b, f["iw_get_ui16le"](b), f["iw_get_ui16be"](b), f["iw_get_ui32le"](b),
                    f["iw_get_ui32be"](b), f["iw_get_i32le"](b), f["iw_get_ui16_e"](b, 0), f["iw_get_ui16_e"](b, 1),
                    f["iw_get_ui32_e"](b, 0), f["iw_get_ui32_e"](b, 1)))
        v = int(rng.integers(0, 2**32))
        out = []
        for name in ("iw_set_ui16le", "iw_set_ui16be", "iw_set_ui32le", "iw_set_ui32be"):
            buf = C.create_string_buffer(4)
            f[name](buf, v)
            out.append(buf.raw)
        obs.append(("set", v, tuple(out)))
    obs.append(("endian", f["iw_get_host_endianness"]()))
    names = [b"a.png", b"b.JPEG", b"c.pam", b"d", b"e.tiff", b"f.jpg", b"g.bmp", b"h.gif", b"i.webp", b"j.miff",
             b"k.pnm", b"l.ppm", b"m.pgm", b"n.pbm", b"o.tif", b".png", b"p.PnG", b"q.png.txt", b"r.", b"dir.x/s"]
    obs.append(("fmt", tuple(f["iw_detect_fmt_from_filename"](n) for n in names)))
    obs.append(("fmtname", tuple(f["iw_get_fmt_name"](k) for k in range(0, 16))))
    obs.append(("prof", tuple(f["iw_get_profile_by_fmt"](k) for k in range(0, 16))))
    cs = Csdescr()
    xs = np.concatenate([np.linspace(0, 1, 401), rng.random(600), [1e-12, 0.0031308, 0.04045, 0.018, 0.081]])
    for cstype, gamma in ((0, 0.0), (1, 0.0), (2, 2.2), (2, 1.0 / 2.2), (2, 1.8), (3, 0.0)):
        cs.cstype, cs.srgb_intent, cs.gamma = cstype, 0, gamma
        obs.append(("lin", cstype, gamma, tuple(f["iw_convert_sample_to_linear"](float(x), C.byref(cs)) for x in xs)))
        obs.append(("unlin", cstype, gamma,
                    tuple(f["iw_convert_sample_from_linear"](float(x), C.byref(cs)) for x in xs)))
    for n in (0, 1, 2, 5, 64):
        buf = C.create_string_buffer(b"#" * 64, 64)
        f["iw_strlcpy"](buf, b"hello world", n)
        obs.append(("strlcpy", n, buf.raw))
    ctx = f["iw_create_context"](None)
    for w, h in ((1, 1), (0, 5), (5, 0), (-1, 3), (1000000, 1000000), (40000, 40000), (1, 1000000), (123, 456)):
        msg = C.create_string_buffer(200)
        obs.append(("dims", w, h, f["iw_check_image_dimensions"](ctx, w, h), f["iw_get_errorflag"](ctx),
                    f["iw_get_errormsg"](ctx, msg, 200)))
    f["iw_destroy_context"](ctx)
    return obs


def _compare(a: list, b: list) -> list:
    assert len(a) == len(b)
    # NaN compares unequal to itself: compare representations
    return [(x, y) for x, y in zip(a, b) if repr(x) != repr(y)]


def test_utilities_match_oracle(gpulib, oracle):
    bad = _compare(_observe(gpulib), _observe(oracle))
    assert not bad, bad[:5]


def test_utilities_match_reference(gpulib, reference):
    bad = _compare(_observe(gpulib), _observe(reference))
    assert not bad, bad[:5]


@pytest.mark.parametrize("s,want", [(b"1.5", 1.5), (b"-2", -2.0), (b"x", 0.0)])
def test_parse_number_examples(gpulib, s, want):
    f = _fns(gpulib)
    assert f["iw_parse_number"](s) == want

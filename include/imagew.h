/*
 * imagew.h -- public C ABI of libimagew_gb300.
 *
 * This header declares the libimagew 1.3.5 core API that libimagew_gb300.so
 * exports as a drop-in replacement.  Every name, numeric constant and struct
 * layout here must be identical to the reference's public header
 * (src/imagew.h in ImageWorsener 1.3.5) so that an application compiled
 * against that header links and runs against this library unchanged.  The
 * declarations are grouped by concern rather than in the reference's order.
 *
 * Scope: the core context / settings / processing API (src/imagew.h:497-737)
 * and the utility functions of its IW_INCLUDE_UTIL_FUNCTIONS section
 * (src/imagew.h:740-852).  The file-format codecs (iw_read_*_file,
 * iw_write_*_file, iw_read_file_by_fmt ...) are not part of this library.
 *
 * Behaviour: iw_process_image() runs its pixel work on the GPU (CUDA, sm_103a).
 * Results are byte-identical to the reference for integer output.  Errors use
 * the reference's convention: sticky first error, iw_get_errorflag() /
 * iw_get_errormsg(); CUDA failures are reported the same way.
 */
#ifndef IMAGEW_H
#define IMAGEW_H

#include <stddef.h>
#include <stdint.h>
#ifdef IW_INCLUDE_UTIL_FUNCTIONS
#include <stdarg.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#ifdef __GNUC__
#define iw_gnuc_attribute __attribute__
#else
#define iw_gnuc_attribute(x)
#endif

#define IW_EXPORT(x) x

/* Version of the API this header describes (1.3.5). src/imagew.h:40 */
#define IW_VERSION_INT 0x010305

/* ---- Value codes for iw_set_value / iw_get_value (src/imagew.h:43-149) ---- */
#define IW_VAL_API_VERSION             1
#define IW_VAL_PRECISION              10
#define IW_VAL_CVT_TO_GRAYSCALE       11
#define IW_VAL_COMPRESSION            12
#define IW_VAL_DISABLE_GAMMA          13
#define IW_VAL_NO_CSLABEL             14
#define IW_VAL_INT_CLAMP              15
#define IW_VAL_GRAYSCALE_FORMULA      16
#define IW_VAL_EDGE_POLICY_X          17
#define IW_VAL_EDGE_POLICY_Y          18
#define IW_VAL_INPUT_NATIVE_GRAYSCALE 20
#define IW_VAL_INPUT_WIDTH            21
#define IW_VAL_INPUT_HEIGHT           22
#define IW_VAL_INPUT_IMAGE_TYPE       23
#define IW_VAL_INPUT_DEPTH            24
#define IW_VAL_PREF_UNITS             26
#define IW_VAL_JPEG_QUALITY           30
#define IW_VAL_JPEG_SAMP_FACTOR_H     31
#define IW_VAL_JPEG_SAMP_FACTOR_V     32
#define IW_VAL_DEFLATE_CMPR_LEVEL     33
#define IW_VAL_OUTPUT_PALETTE_GRAYSCALE 35
#define IW_VAL_OUTPUT_INTERLACED      36
#define IW_VAL_USE_BKGD_LABEL         37
#define IW_VAL_WEBP_QUALITY           38
#define IW_VAL_PAGE_TO_READ           39
#define IW_VAL_INCLUDE_SCREEN         40
#define IW_VAL_JPEG_ARITH_CODING      41
#define IW_VAL_TRANSLATE_X            42
#define IW_VAL_TRANSLATE_Y            43
#define IW_VAL_BMP_NO_FILEHEADER      44
#define IW_VAL_MAX_WIDTH              45
#define IW_VAL_MAX_HEIGHT             46
#define IW_VAL_BMP_VERSION            47
#define IW_VAL_NO_BKGD_LABEL          48
#define IW_VAL_INTENT                 49
#define IW_VAL_OUTPUT_SAMPLE_TYPE     50
#define IW_VAL_OUTPUT_COLOR_TYPE      51
#define IW_VAL_OUTPUT_FORMAT          52
#define IW_VAL_NEGATE_TARGET          53

/* ---- File format codes (src/imagew.h:151-167) ---- */
#define IW_FORMAT_UNKNOWN  0
#define IW_FORMAT_PNG      1
#define IW_FORMAT_JPEG     2
#define IW_FORMAT_BMP      3
#define IW_FORMAT_TIFF     4
#define IW_FORMAT_MIFF     5
#define IW_FORMAT_WEBP     6
#define IW_FORMAT_GIF      7
#define IW_FORMAT_PNM      8
#define IW_FORMAT_PBM      9
#define IW_FORMAT_PGM      10
#define IW_FORMAT_PPM      11
#define IW_FORMAT_PAM      12

/* ---- Output-format capability bits (src/imagew.h:169-205) ---- */
#define IW_PROFILE_TRANSPARENCY      0x0001
#define IW_PROFILE_GRAYSCALE         0x0002
#define IW_PROFILE_PALETTETRNS       0x0004
#define IW_PROFILE_GRAY1             0x0008
#define IW_PROFILE_GRAY2             0x0010
#define IW_PROFILE_GRAY4             0x0020
#define IW_PROFILE_16BPS             0x0040
#define IW_PROFILE_ALWAYSSRGB        0x0080
#define IW_PROFILE_BINARYTRNS        0x0100
#define IW_PROFILE_PAL1              0x0200
#define IW_PROFILE_PAL2              0x0400
#define IW_PROFILE_PAL4              0x0800
#define IW_PROFILE_PAL8              0x1000
#define IW_PROFILE_ALWAYSLINEAR      0x2000
#define IW_PROFILE_HDRI              0x4000
#define IW_PROFILE_REDUCEDBITDEPTHS  0x8000
#define IW_PROFILE_PNG_BKGD          0x10000
#define IW_PROFILE_RGB8_BKGD         0x20000
#define IW_PROFILE_RGB16_BKGD        0x40000

/* ---- Resampling filter families (src/imagew.h:207-221) ---- */
#define IW_RESIZETYPE_AUTO       0x01
#define IW_RESIZETYPE_NULL       0x02
#define IW_RESIZETYPE_NEAREST    0x10
#define IW_RESIZETYPE_MIX        0x11
#define IW_RESIZETYPE_BOX        0x20
#define IW_RESIZETYPE_TRIANGLE   0x21
#define IW_RESIZETYPE_QUADRATIC  0x22
#define IW_RESIZETYPE_GAUSSIAN   0x23
#define IW_RESIZETYPE_HERMITE    0x24
#define IW_RESIZETYPE_CUBIC      0x25
#define IW_RESIZETYPE_BOXAVG     0x26
#define IW_RESIZETYPE_SINC       0x30
#define IW_RESIZETYPE_LANCZOS    0x31
#define IW_RESIZETYPE_HANNING    0x32
#define IW_RESIZETYPE_BLACKMAN   0x33

/* ---- Image types (src/imagew.h:223-230) ---- */
#define IW_IMGTYPE_GRAY    0x0001
#define IW_IMGTYPE_GRAYA   0x0101
#define IW_IMGTYPE_RGB     0x0010
#define IW_IMGTYPE_RGBA    0x0110
#define IW_IMGTYPE_PALETTE 0x1000
#define IW_IMGTYPE_IS_GRAY(x)   (((x)&0x001)?1:0)
#define IW_IMGTYPE_HAS_ALPHA(x) (((x)&0x100)?1:0)

#define IW_SAMPLETYPE_UINT          0
#define IW_SAMPLETYPE_FLOATINGPOINT 1

#define IW_COMPRESSION_AUTO     0
#define IW_COMPRESSION_NONE     1
#define IW_COMPRESSION_ZIP      2
#define IW_COMPRESSION_LZW      3
#define IW_COMPRESSION_JPEG     4
#define IW_COMPRESSION_RLE      5

#define IW_COLORTYPE_DEFAULT    0
#define IW_COLORTYPE_RGB        1
#define IW_COLORTYPE_YCBCR      2

/* Channel types; used as array indices (src/imagew.h:249-256). */
#define IW_CHANNELTYPE_RED      0
#define IW_CHANNELTYPE_GREEN    1
#define IW_CHANNELTYPE_BLUE     2
#define IW_CHANNELTYPE_ALPHA    3
#define IW_CHANNELTYPE_GRAY     4
#define IW_CHANNELTYPE_ALL      10
#define IW_CHANNELTYPE_NONALPHA 11

/* Colour-space families (src/imagew.h:258-262). */
#define IW_CSTYPE_SRGB      0
#define IW_CSTYPE_LINEAR    1
#define IW_CSTYPE_GAMMA     2
#define IW_CSTYPE_REC709    3

#define IW_SRGB_INTENT_PERCEPTUAL 0
#define IW_SRGB_INTENT_RELATIVE   1
#define IW_SRGB_INTENT_SATURATION 2
#define IW_SRGB_INTENT_ABSOLUTE   3

#define IW_INTENT_UNKNOWN    0
#define IW_INTENT_DEFAULT    1
#define IW_INTENT_NONE       2
#define IW_INTENT_PERCEPTUAL 10
#define IW_INTENT_RELATIVE   11
#define IW_INTENT_SATURATION 12
#define IW_INTENT_ABSOLUTE   13

#define IW_DIMENSION_H 0
#define IW_DIMENSION_V 1

/* Dither families and subtypes (src/imagew.h:282-298). */
#define IW_DITHERFAMILY_NONE         0
#define  IW_DITHERSUBTYPE_DEFAULT      0
#define IW_DITHERFAMILY_ORDERED      1
#define  IW_DITHERSUBTYPE_HALFTONE     1
#define IW_DITHERFAMILY_ERRDIFF      2
#define  IW_DITHERSUBTYPE_FS           0
#define  IW_DITHERSUBTYPE_JJN          1
#define  IW_DITHERSUBTYPE_STUCKI       2
#define  IW_DITHERSUBTYPE_BURKES       3
#define  IW_DITHERSUBTYPE_SIERRA3      4
#define  IW_DITHERSUBTYPE_SIERRA2      5
#define  IW_DITHERSUBTYPE_SIERRA42A    6
#define  IW_DITHERSUBTYPE_ATKINSON     7
#define IW_DITHERFAMILY_RANDOM       3
#define  IW_DITHERSUBTYPE_SAMEPATTERN  1

#define IW_DENSITY_UNKNOWN         0
#define IW_DENSITY_UNITS_UNKNOWN   1
#define IW_DENSITY_UNITS_PER_METER 2

#define IW_PREF_UNITS_DEFAULT    0
#define IW_PREF_UNITS_METRIC     1
#define IW_PREF_UNITS_IMPERIAL   2

#define IW_GSF_STANDARD      0
#define IW_GSF_COMPATIBLE    1
#define IW_GSF_WEIGHTED      2
#define IW_GSF_ORDERBYVALUE  3

#define IW_EDGE_POLICY_REPLICATE   1
#define IW_EDGE_POLICY_STANDARD    2
#define IW_EDGE_POLICY_TRANSPARENT 3

#define IW_REORIENT_NOCHANGE    0
#define IW_REORIENT_FLIP_H      1
#define IW_REORIENT_FLIP_V      2
#define IW_REORIENT_ROTATE_180  3
#define IW_REORIENT_TRANSPOSE   4
#define IW_REORIENT_ROTATE_90   5
#define IW_REORIENT_ROTATE_270  6
#define IW_REORIENT_TRANSVERSE  7

#define IW_OPT_GRAYSCALE    1
#define IW_OPT_PALETTE      2
#define IW_OPT_16_TO_8      3
#define IW_OPT_STRIP_ALPHA  4
#define IW_OPT_BINARY_TRNS  5

#define IW_TRANSLATEFLAG_FORMAT      0x0001
#define IW_TRANSLATEFLAG_POSTFORMAT  0x0002
#define IW_TRANSLATEFLAG_ERRORMSG    0x0010
#define IW_TRANSLATEFLAG_WARNINGMSG  0x0020

#define IW_MALLOCFLAG_ZEROMEM     0x01
#define IW_MALLOCFLAG_NOERRORS    0x02

#define iw_byte     uint8_t
#define iw_uint16   uint16_t
#define iw_int32    int32_t
#define iw_uint32   uint32_t
#define iw_int64    int64_t
#define iw_uint64   uint64_t
#define iw_float32  float
#define iw_float64  double

/* ---- Public structs: layouts fixed by the ABI (src/imagew.h:366-491) ---- */

struct iw_csdescr {
	int cstype;        /* IW_CSTYPE_* */
	int srgb_intent;   /* deprecated */
	double gamma;      /* for IW_CSTYPE_GAMMA */
};

struct iw_color {
	double c[4];       /* indexed by IW_CHANNELTYPE_RED..ALPHA */
};

/* An input or output image.  Integer samples wider than 8 bits are stored
 * big-endian; float samples use host byte order. */
struct iw_image {
	int imgtype;
	int bit_depth;
	int sampletype;
	int width, height;
	iw_byte *pixels;
	size_t bpr;
	unsigned int orient_transform;
	int native_grayscale;
	int density_code;
	double density_x, density_y;
	int has_colorkey_trns;
	unsigned int colorkey[3];
	int reduced_maxcolors;
	unsigned int maxcolorcode[5];
	int has_bkgdlabel;
	struct iw_color bkgdlabel;
	int rendering_intent;
};

struct iw_rgba8color {
	iw_byte r, g, b, a;
};

struct iw_palette {
	int num_entries;
	struct iw_rgba8color entry[256];
};

struct iw_context;

typedef void* (*iw_mallocfn_type)(void *userdata, unsigned int flags, size_t n);
typedef void  (*iw_freefn_type)(void *userdata, void *mem);

struct iw_init_params {
	int api_version;
	void *userdata;
	iw_mallocfn_type mallocfn;
	iw_freefn_type freefn;
};

typedef int  (*iw_translatefn_type)(struct iw_context *ctx,
	unsigned int flags, char *dst, size_t dstlen, const char *src);
typedef void (*iw_warningfn_type)(struct iw_context *ctx, const char *msg);

/* ---- Context lifetime and processing ---- */
IW_EXPORT(struct iw_context*) iw_create_context(struct iw_init_params *params);
IW_EXPORT(void) iw_destroy_context(struct iw_context *ctx);
IW_EXPORT(int)  iw_process_image(struct iw_context *ctx);
IW_EXPORT(void) iw_reorient_image(struct iw_context *ctx, unsigned int x);

/* ---- Errors, warnings, user data ---- */
IW_EXPORT(void) iw_set_translate_fn(struct iw_context *ctx, iw_translatefn_type xlatefn);
IW_EXPORT(int)  iw_get_errorflag(struct iw_context *ctx);
IW_EXPORT(const char*) iw_get_errormsg(struct iw_context *ctx, char *buf, int buflen);
IW_EXPORT(void) iw_set_userdata(struct iw_context *ctx, void *userdata);
IW_EXPORT(void*) iw_get_userdata(struct iw_context *ctx);
IW_EXPORT(void) iw_set_warning_fn(struct iw_context *ctx, iw_warningfn_type warnfn);
IW_EXPORT(void) iw_set_max_malloc(struct iw_context *ctx, size_t n);
IW_EXPORT(void) iw_set_error(struct iw_context *ctx, const char *s);
IW_EXPORT(void) iw_set_errorf(struct iw_context *ctx, const char *fmt, ...)
	iw_gnuc_attribute ((format (printf, 2, 3)));
IW_EXPORT(void) iw_warning(struct iw_context *ctx, const char *s);
IW_EXPORT(void) iw_warningf(struct iw_context *ctx, const char *fmt, ...)
	iw_gnuc_attribute ((format (printf, 2, 3)));

/* ---- Geometry ---- */
IW_EXPORT(void) iw_set_output_canvas_size(struct iw_context *ctx, int w, int h);
IW_EXPORT(void) iw_set_output_image_size(struct iw_context *ctx, double w, double h);
IW_EXPORT(void) iw_set_input_crop(struct iw_context *ctx, int x, int y, int w, int h);

/* ---- Output format, depth, dithering, colour counts ---- */
IW_EXPORT(void) iw_set_output_profile(struct iw_context *ctx, unsigned int n);
IW_EXPORT(void) iw_set_output_depth(struct iw_context *ctx, int bps);
IW_EXPORT(void) iw_set_output_max_color_code(struct iw_context *ctx, int channeltype, int n);
IW_EXPORT(void) iw_set_dither_type(struct iw_context *ctx, int channeltype, int family, int subtype);
IW_EXPORT(void) iw_set_color_count(struct iw_context *ctx, int channeltype, int c);

/* ---- Resampling ---- */
IW_EXPORT(void) iw_set_resize_alg(struct iw_context *ctx, int dimension, int family,
	double blur, double param1, double param2);
IW_EXPORT(void) iw_set_channel_offset(struct iw_context *ctx, int channeltype, int dimension, double offs);
IW_EXPORT(void) iw_set_grayscale_weights(struct iw_context *ctx, double r, double g, double b);

/* ---- Backgrounds ---- */
IW_EXPORT(void) iw_set_input_bkgd_label(struct iw_context *ctx, double r, double g, double b);
IW_EXPORT(void) iw_set_input_bkgd_label_2(struct iw_context *ctx, const struct iw_color *clr);
IW_EXPORT(void) iw_set_output_bkgd_label(struct iw_context *ctx, double r, double g, double b);
IW_EXPORT(void) iw_set_output_bkgd_label_2(struct iw_context *ctx, const struct iw_color *clr);
IW_EXPORT(void) iw_set_apply_bkgd(struct iw_context *ctx, double r, double g, double b);
IW_EXPORT(void) iw_set_apply_bkgd_2(struct iw_context *ctx, const struct iw_color *clr);
IW_EXPORT(void) iw_set_bkgd_checkerboard(struct iw_context *ctx, int checkersize, double r2, double g2, double b2);
IW_EXPORT(void) iw_set_bkgd_checkerboard_2(struct iw_context *ctx, int checkersize, const struct iw_color *clr);
IW_EXPORT(void) iw_set_bkgd_checkerboard_origin(struct iw_context *ctx, int x, int y);

/* ---- Colour spaces ---- */
IW_EXPORT(void) iw_set_output_colorspace(struct iw_context *ctx, const struct iw_csdescr *csdescr);
IW_EXPORT(void) iw_set_input_colorspace(struct iw_context *ctx, const struct iw_csdescr *csdescr);
IW_EXPORT(void) iw_make_linear_csdescr(struct iw_csdescr *cs);
IW_EXPORT(void) iw_make_srgb_csdescr(struct iw_csdescr *cs, int srgb_intent);
IW_EXPORT(void) iw_make_srgb_csdescr_2(struct iw_csdescr *cs);
IW_EXPORT(void) iw_make_rec709_csdescr(struct iw_csdescr *cs);
IW_EXPORT(void) iw_make_gamma_csdescr(struct iw_csdescr *cs, double gamma);

/* ---- Density, randomness, optimisations ---- */
IW_EXPORT(int)  iw_get_input_density(struct iw_context *ctx, double *px, double *py, int *pcode);
IW_EXPORT(void) iw_set_output_density(struct iw_context *ctx, double x, double y, int code);
IW_EXPORT(void) iw_set_random_seed(struct iw_context *ctx, int randomize, int rand_seed);
IW_EXPORT(void) iw_set_allow_opt(struct iw_context *ctx, int opt, int n);

/* ---- Images in and out ---- */
IW_EXPORT(void) iw_set_input_image(struct iw_context *ctx, const struct iw_image *img);
IW_EXPORT(void) iw_get_output_image(struct iw_context *ctx, struct iw_image *img);
IW_EXPORT(void) iw_get_output_colorspace(struct iw_context *ctx, struct iw_csdescr *csdescr);
IW_EXPORT(const struct iw_palette*) iw_get_output_palette(struct iw_context *ctx);

/* ---- Generic settings ---- */
IW_EXPORT(void)   iw_set_value(struct iw_context *ctx, int code, int n);
IW_EXPORT(int)    iw_get_value(struct iw_context *ctx, int code);
IW_EXPORT(void)   iw_set_value_dbl(struct iw_context *ctx, int code, double n);
IW_EXPORT(double) iw_get_value_dbl(struct iw_context *ctx, int code);
IW_EXPORT(void)   iw_set_option(struct iw_context *ctx, const char *name, const char *val);
IW_EXPORT(const char*) iw_get_option(struct iw_context *ctx, const char *name);

/* ---- Stateless helpers ---- */
IW_EXPORT(int)    iw_get_sample_size(void);
IW_EXPORT(double) iw_convert_sample_to_linear(double v, const struct iw_csdescr *csdescr);
IW_EXPORT(double) iw_convert_sample_from_linear(double v, const struct iw_csdescr *csdescr);
IW_EXPORT(unsigned int) iw_color_get_int_sample(struct iw_color *clr, int channel, unsigned int maxcolorcode);
IW_EXPORT(int)    iw_get_version_int(void);
IW_EXPORT(char*)  iw_get_version_string(struct iw_context *ctx, char *s, int s_len);
IW_EXPORT(char*)  iw_get_copyright_string(struct iw_context *ctx, char *s, int s_len);
IW_EXPORT(void)   iw_utf8_to_ascii(const char *src, char *dst, int dstlen);
IW_EXPORT(unsigned int) iw_get_profile_by_fmt(int fmt);
IW_EXPORT(int)    iw_detect_fmt_from_filename(const char *fn);
IW_EXPORT(const char*) iw_get_fmt_name(int fmt);
IW_EXPORT(int)    iw_detect_fmt_of_file(const iw_byte *buf, size_t buflen);
IW_EXPORT(int)    iw_is_input_fmt_supported(int fmt);
IW_EXPORT(int)    iw_is_output_fmt_supported(int fmt);

#ifdef IW_INCLUDE_UTIL_FUNCTIONS
/* Utility functions of the reference's IW_INCLUDE_UTIL_FUNCTIONS section. */
IW_EXPORT(void) iw_translate(struct iw_context *ctx, unsigned int flags,
	char *dst, size_t dstlen, const char *src);
IW_EXPORT(void) iw_translatev(struct iw_context *ctx, unsigned int flags,
	char *dst, size_t dstlen, const char *fmt, va_list ap);
IW_EXPORT(void) iw_translatef(struct iw_context *ctx, unsigned int flags,
	char *dst, size_t dstlen, const char *fmt, ...);
IW_EXPORT(void) iw_set_errorv(struct iw_context *ctx, const char *fmt, va_list ap);
IW_EXPORT(void) iw_warningv(struct iw_context *ctx, const char *fmt, va_list ap);
IW_EXPORT(void) iw_strlcpy(char *dst, const char *src, size_t dstlen);
IW_EXPORT(void) iw_vsnprintf(char *buf, size_t buflen, const char *fmt, va_list ap);
IW_EXPORT(void) iw_snprintf(char *buf, size_t buflen, const char *fmt, ...)
	iw_gnuc_attribute ((format (printf, 3, 4)));
IW_EXPORT(int)  iw_stricmp(const char *s1, const char *s2);
IW_EXPORT(void) iw_zeromem(void *mem, size_t n);
IW_EXPORT(void) iw_set_input_max_color_code(struct iw_context *ctx, int input_channel, int c);
IW_EXPORT(int)  iw_imgtype_num_channels(int t);
IW_EXPORT(size_t) iw_calc_bytesperrow(int num_pixels, int bits_per_pixel);
IW_EXPORT(int)  iw_check_image_dimensions(struct iw_context *ctx, int w, int h);
IW_EXPORT(int)  iw_is_valid_density(double density_x, double density_y, int density_code);
IW_EXPORT(void*) iw_malloc_ex(struct iw_context *ctx, unsigned int flags, size_t n);
IW_EXPORT(void*) iw_malloc(struct iw_context *ctx, size_t n);
IW_EXPORT(void*) iw_mallocz(struct iw_context *ctx, size_t n);
IW_EXPORT(void*) iw_malloc_large(struct iw_context *ctx, size_t n1, size_t n2);
IW_EXPORT(void*) iw_realloc_ex(struct iw_context *ctx, unsigned int flags, void *m, size_t oldn, size_t n);
IW_EXPORT(void*) iw_realloc(struct iw_context *ctx, void *m, size_t oldn, size_t n);
IW_EXPORT(char*) iw_strdup(struct iw_context *ctx, const char *s);
IW_EXPORT(void)  iw_free(struct iw_context *ctx, void *mem);
#define IW_ENDIAN_BIG    0
#define IW_ENDIAN_LITTLE 1
IW_EXPORT(int) iw_get_host_endianness(void);
IW_EXPORT(void) iw_set_ui16le(iw_byte *b, unsigned int n);
IW_EXPORT(void) iw_set_ui32le(iw_byte *b, unsigned int n);
IW_EXPORT(void) iw_set_ui16be(iw_byte *b, unsigned int n);
IW_EXPORT(void) iw_set_ui32be(iw_byte *b, unsigned int n);
IW_EXPORT(unsigned int) iw_get_ui16le(const iw_byte *b);
IW_EXPORT(int) iw_get_i32le(const iw_byte *b);
IW_EXPORT(unsigned int) iw_get_ui32le(const iw_byte *b);
IW_EXPORT(unsigned int) iw_get_ui16be(const iw_byte *b);
IW_EXPORT(unsigned int) iw_get_ui32be(const iw_byte *b);
IW_EXPORT(unsigned int) iw_get_ui16_e(const iw_byte *b, int endian);
IW_EXPORT(unsigned int) iw_get_ui32_e(const iw_byte *b, int endian);
IW_EXPORT(int) iw_max_color_to_bitdepth(unsigned int mc);
IW_EXPORT(int) iw_parse_number_list(const char *s, int max_numbers, double *results);
IW_EXPORT(double) iw_parse_number(const char *s);
IW_EXPORT(int) iw_parse_int(const char *s);
IW_EXPORT(int) iw_round_to_int(double x);
#endif /* IW_INCLUDE_UTIL_FUNCTIONS */

#ifdef __cplusplus
}
#endif

#endif /* IMAGEW_H */

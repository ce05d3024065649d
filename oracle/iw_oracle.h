/*
 * iw_oracle.h -- private state of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain-C restatement of the
 * ImageWorsener 1.3.5 pixel pipeline (iw_process_image and the settings API
 * around it).  It exists so that the GPU library can be checked, sample for
 * sample, against a CPU implementation that runs on any machine.  Only the
 * tests, __graft_entry__.smoke() and bench.py's CPU arm load it; the product
 * library never links or calls it.
 *
 * The oracle is pinned to the real reference: the CPU tests run it side by
 * side with the unmodified reference core (compiled from its own sources into
 * oracle/_ref/) over a grid of settings and require byte-identical output, and
 * against golden vectors generated from the reference (tests/golden/).
 */
#ifndef IW_ORACLE_H
#define IW_ORACLE_H

#define IW_INCLUDE_UTIL_FUNCTIONS
#include "imagew.h"

#define ORC_NCTYPES 5   /* R,G,B,A,Gray: indexable by IW_CHANNELTYPE_* */
#define ORC_MAXCH   4
#define ORC_MSG_MAX 200

/* Per-dimension resampling request (src/imagew-internals.h:38-51). */
struct orc_dim {
	int family;
	int edge;
	double blur;
	double p1, p2;
	double translate;
	double chan_offset[3];
	/* derived while planning */
	int use_offset;
	int no_cache;
	double true_size;
};

/* Post-processing state (src/imagew-internals.h:96-128). */
struct orc_opt {
	int width, height, imgtype, bit_depth;
	size_t bpr;
	const iw_byte *pix;
	iw_byte *tmp;
	int has_trns, has_partial_trns, has_16bit, has_color;
	int pal_is_gray;
	struct iw_palette *pal;
	int has_ckey;
	unsigned int ckey[3];
	int has_label;
	unsigned int label[4];
};

struct orc_option { char *name; char *val; };

struct iw_context {
	/* allocation, messages */
	iw_mallocfn_type mallocfn;
	iw_freefn_type freefn;
	void *userdata;
	size_t max_malloc;
	int max_w, max_h;
	int api_version;
	int error_flag;
	char *error_msg;
	iw_translatefn_type xlate;
	iw_warningfn_type warn;

	/* input */
	struct iw_image img1;
	struct iw_csdescr cs_in;
	int in_maxcc[ORC_MAXCH];

	/* request */
	unsigned int profile;
	int canvas_w, canvas_h;
	int crop_x, crop_y, crop_w, crop_h;
	int req_depth, req_sampletype;
	int req_maxcc[ORC_NCTYPES];
	int req_cc[ORC_NCTYPES];
	int dfam[ORC_NCTYPES], dsub[ORC_NCTYPES];
	int true_valid;
	double true_w, true_h;
	int req_intent;
	int cs_out_valid;
	struct iw_csdescr cs_out_req;
	int no_cslabel, negate;
	int bkgd_valid, bkgd_checker;
	struct iw_color bkgd, bkgd2;
	int check_size, check_origin[2];
	int outlabel_valid;
	struct iw_color outlabel;
	int use_file_label, no_outlabel;
	int inlabel_set;
	struct iw_color inlabel;
	int to_gray, gsf;
	double gsw[3];
	int no_gamma, intclamp, pref_units;
	int randomize, seed;
	iw_byte opt_gray, opt_pal, opt_16to8, opt_strip, opt_bintrns;
	struct orc_dim dim[2];
	int compression, page, include_screen, interlaced, bmp_nofh, out_fmt;
	struct orc_option *opts;
	int nopts;

	/* results */
	int use_count;
	struct iw_image img2;
	struct iw_csdescr cs_out;
	int reduced_out;
	int out_maxcc[ORC_MAXCH];
	struct orc_opt opt;
};

/* iw_oracle_opt.c: output post-pass (src/imagew-opt.c:1166-1314). */
void orc_optimize(struct iw_context *ctx);

#endif

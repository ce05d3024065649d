/* pnm.h -- PNM / PAM files for the imagew_gb300 command-line tool (pnm.c). */
#ifndef IWG_CLI_PNM_H
#define IWG_CLI_PNM_H

#include <stdio.h>
#ifndef IW_INCLUDE_UTIL_FUNCTIONS
#define IW_INCLUDE_UTIL_FUNCTIONS   /* iw_malloc_large, iw_parse_number_list, ... */
#endif
#include "imagew.h"

/* Reads a P4/P5/P6/P7 file and sets it as the context's input image.
 * Returns 1, or 0 with the context's error set. */
int pnm_read(struct iw_context *ctx, FILE *f);

/* Writes the context's output image as fmt (IW_FORMAT_PNM, _PPM, _PGM or
 * _PAM).  Returns 1, or 0 (with the context's error set where there is a
 * message). */
int pnm_write(struct iw_context *ctx, FILE *f, int fmt);

#endif

/*
 * mcx_json.h -- internal interface of the JSON input reader (mcx_json.c),
 * called by the public mcx_readconfig / mcx_parsejson in mcx_host.c.
 */
#ifndef MCX_JSON_H
#define MCX_JSON_H

#include <stddef.h>

#include "../../include/mcx_gb300.h"

/* Parse a JSON input text and fill cfg (positions as given, not yet
   converted to 0-based).  0 on success, else the reference's error id with
   a message in err. */
int mcxj_load(const char* text, Config* cfg, char* err, size_t errlen);
/* Parse only (syntax check): 0 when the text is one valid JSON value. */
int mcxj_check(const char* text, char* err, size_t errlen);

#endif

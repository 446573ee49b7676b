/*
 * mcx_json.c -- JSON input of the transport path.
 *
 * A small recursive-descent JSON parser (RFC 8259 values; object keys matched
 * case-insensitively, as the reference's lookups are) and the loader that
 * fills a Config from the sections the transport path reads: Session,
 * Forward, Optode (Source, Detector), Domain (Media, MieScatter, Dim, Step,
 * LengthUnit, MediaFormat, OriginType, InverseCDF, VolumeFile) and Shapes.
 * It follows the reference's mcx_loadjson (src/mcx_utils.c:2401-3287) and
 * its shape rasterisers (src/mcx_shapes.c:156-838): every key is looked up
 * in its section first and then as a dotted full name at the root
 * ("Session.Photons"), booleans read as 1/0 where an integer is expected,
 * and each shape tag writes its label into the voxels whose centres it
 * covers, in the order the tags appear.
 *
 * Positions are left as given (1-based unless Domain.OriginType or a
 * Config with issrcfrom0 says 0-based); mcx_validatecfg converts them, as
 * it does for every other input path.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "../../include/mcx_gb300.h"
#include "mcx_json.h"

#define J_MAXDEPTH 128
#define MAX_PROP_TOTAL 4000          /* media + detectors + 4 x extra sources (mcx_utils.c:3098-3100) */

enum { J_NULL, J_FALSE, J_TRUE, J_NUM, J_STR, J_ARR, J_OBJ };

typedef struct JNode {
    int type;
    char* key;                    /* member name inside an object */
    double num;
    char* str;
    struct JNode* child;          /* first element or member */
    struct JNode* next;
} JNode;

/* ----------------------------------------------------------------- parser */

typedef struct {
    const char* s;
    size_t pos, len;
    char* err;
    size_t errlen;
    int failed;
} JParser;

static void jfail(JParser* p, const char* what) {
    if (!p->failed) {
        size_t line = 1;
        for (size_t i = 0; i < p->pos && i < p->len; i++) {
            line += p->s[i] == '\n';
        }
        snprintf(p->err, p->errlen, "invalid JSON input: %s at line %zu (byte %zu)", what, line, p->pos);
        p->failed = 1;
    }
}

static void jfree(JNode* n) {
    while (n) {
        JNode* nx = n->next;
        jfree(n->child);
        free(n->key);
        free(n->str);
        free(n);
        n = nx;
    }
}

static void skipws(JParser* p) {
    while (p->pos < p->len) {
        char c = p->s[p->pos];
        if (c == ' ' || c == '\t' || c == '\n' || c == '\r') {
            p->pos++;
        } else {
            break;
        }
    }
}

static void put_utf8(char* out, size_t* n, unsigned int cp) {
    if (cp < 0x80) {
        out[(*n)++] = (char)cp;
    } else if (cp < 0x800) {
        out[(*n)++] = (char)(0xC0 | (cp >> 6));
        out[(*n)++] = (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
        out[(*n)++] = (char)(0xE0 | (cp >> 12));
        out[(*n)++] = (char)(0x80 | ((cp >> 6) & 0x3F));
        out[(*n)++] = (char)(0x80 | (cp & 0x3F));
    } else {
        out[(*n)++] = (char)(0xF0 | (cp >> 18));
        out[(*n)++] = (char)(0x80 | ((cp >> 12) & 0x3F));
        out[(*n)++] = (char)(0x80 | ((cp >> 6) & 0x3F));
        out[(*n)++] = (char)(0x80 | (cp & 0x3F));
    }
}

static int hex4(JParser* p, unsigned int* v) {
    *v = 0;
    for (int i = 0; i < 4; i++) {
        if (p->pos >= p->len) {
            return 0;
        }
        char c = p->s[p->pos++];
        *v <<= 4;
        if (c >= '0' && c <= '9') {
            *v |= (unsigned)(c - '0');
        } else if (c >= 'a' && c <= 'f') {
            *v |= (unsigned)(c - 'a' + 10);
        } else if (c >= 'A' && c <= 'F') {
            *v |= (unsigned)(c - 'A' + 10);
        } else {
            return 0;
        }
    }
    return 1;
}

/* a string starting at the opening quote; the decoded text is never longer
   than its escaped form */
static char* parse_string(JParser* p) {
    p->pos++;
    size_t start = p->pos;
    while (p->pos < p->len && p->s[p->pos] != '"') {
        p->pos += (p->s[p->pos] == '\\') ? 2 : 1;
    }
    if (p->pos >= p->len) {
        jfail(p, "unterminated string");
        return NULL;
    }
    size_t end = p->pos;
    char* out = (char*)malloc(end - start + 1);
    if (!out) {
        jfail(p, "out of memory");
        return NULL;
    }
    size_t n = 0;
    p->pos = start;
    while (p->pos < end) {
        char c = p->s[p->pos++];
        if ((unsigned char)c < 0x20) {
            free(out);
            jfail(p, "control character in a string");
            return NULL;
        }
        if (c != '\\') {
            out[n++] = c;
            continue;
        }
        char e = p->s[p->pos++];
        switch (e) {
            case '"': out[n++] = '"'; break;
            case '\\': out[n++] = '\\'; break;
            case '/': out[n++] = '/'; break;
            case 'b': out[n++] = '\b'; break;
            case 'f': out[n++] = '\f'; break;
            case 'n': out[n++] = '\n'; break;
            case 'r': out[n++] = '\r'; break;
            case 't': out[n++] = '\t'; break;
            case 'u': {
                unsigned int cp;
                if (!hex4(p, &cp)) {
                    free(out);
                    jfail(p, "bad \\u escape");
                    return NULL;
                }
                if (cp >= 0xD800 && cp <= 0xDBFF && p->pos + 6 <= end && p->s[p->pos] == '\\' &&
                        p->s[p->pos + 1] == 'u') {
                    unsigned int lo;
                    p->pos += 2;
                    if (hex4(p, &lo) && lo >= 0xDC00 && lo <= 0xDFFF) {
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                }
                put_utf8(out, &n, cp);
                break;
            }
            default:
                free(out);
                jfail(p, "bad escape in a string");
                return NULL;
        }
    }
    out[n] = '\0';
    p->pos = end + 1;
    return out;
}

static JNode* parse_value(JParser* p, int depth);

static JNode* newnode(JParser* p, int type) {
    JNode* n = (JNode*)calloc(1, sizeof(JNode));
    if (!n) {
        jfail(p, "out of memory");
        return NULL;
    }
    n->type = type;
    return n;
}

static JNode* parse_container(JParser* p, int depth, int isobj) {
    JNode* n = newnode(p, isobj ? J_OBJ : J_ARR);
    if (!n) {
        return NULL;
    }
    const char close = isobj ? '}' : ']';
    p->pos++;
    skipws(p);
    if (p->pos < p->len && p->s[p->pos] == close) {
        p->pos++;
        return n;
    }
    JNode** tail = &n->child;
    for (;;) {
        char* key = NULL;
        skipws(p);
        if (isobj) {
            if (p->pos >= p->len || p->s[p->pos] != '"') {
                jfail(p, "expected a member name");
                break;
            }
            key = parse_string(p);
            if (!key) {
                break;
            }
            skipws(p);
            if (p->pos >= p->len || p->s[p->pos] != ':') {
                free(key);
                jfail(p, "expected ':'");
                break;
            }
            p->pos++;
        }
        JNode* v = parse_value(p, depth + 1);
        if (!v) {
            free(key);
            break;
        }
        v->key = key;
        *tail = v;
        tail = &v->next;
        skipws(p);
        if (p->pos < p->len && p->s[p->pos] == ',') {
            p->pos++;
            continue;
        }
        if (p->pos < p->len && p->s[p->pos] == close) {
            p->pos++;
            return n;
        }
        jfail(p, isobj ? "expected ',' or '}'" : "expected ',' or ']'");
        break;
    }
    jfree(n);
    return NULL;
}

static JNode* parse_value(JParser* p, int depth) {
    if (depth > J_MAXDEPTH) {
        jfail(p, "nesting too deep");
        return NULL;
    }
    skipws(p);
    if (p->pos >= p->len) {
        jfail(p, "unexpected end of input");
        return NULL;
    }
    const char* s = p->s + p->pos;
    const size_t rest = p->len - p->pos;
    char c = *s;
    if (c == '{' || c == '[') {
        return parse_container(p, depth, c == '{');
    }
    if (c == '"') {
        char* str = parse_string(p);
        if (!str) {
            return NULL;
        }
        JNode* n = newnode(p, J_STR);
        if (!n) {
            free(str);
            return NULL;
        }
        n->str = str;
        return n;
    }
    if (rest >= 4 && !strncmp(s, "true", 4)) {
        p->pos += 4;
        return newnode(p, J_TRUE);
    }
    if (rest >= 5 && !strncmp(s, "false", 5)) {
        p->pos += 5;
        return newnode(p, J_FALSE);
    }
    if (rest >= 4 && !strncmp(s, "null", 4)) {
        p->pos += 4;
        return newnode(p, J_NULL);
    }
    if (c == '-' || (c >= '0' && c <= '9')) {
        /* strtod reads a superset of JSON numbers; bound it to the number's characters */
        size_t k = 0;
        while (k < rest && (isdigit((unsigned char)s[k]) || s[k] == '-' || s[k] == '+' || s[k] == '.' ||
                            s[k] == 'e' || s[k] == 'E')) {
            k++;
        }
        char buf[64];
        if (k == 0 || k >= sizeof(buf)) {
            jfail(p, "bad number");
            return NULL;
        }
        memcpy(buf, s, k);
        buf[k] = '\0';
        char* endp = NULL;
        double v = strtod(buf, &endp);
        if (endp != buf + k) {
            jfail(p, "bad number");
            return NULL;
        }
        JNode* n = newnode(p, J_NUM);
        if (!n) {
            return NULL;
        }
        n->num = v;
        p->pos += k;
        return n;
    }
    jfail(p, "unexpected character");
    return NULL;
}

static JNode* jparse(const char* text, char* err, size_t errlen) {
    JParser p = {text, 0, strlen(text), err, errlen, 0};
    JNode* root = parse_value(&p, 0);
    if (root) {
        skipws(&p);
        if (p.pos != p.len) {
            jfail(&p, "trailing characters after the top-level value");
            jfree(root);
            return NULL;
        }
    }
    return root;
}

/* ----------------------------------------------------------------- access */

static int jsize(const JNode* n) {
    int k = 0;
    for (const JNode* c = n ? n->child : NULL; c; c = c->next) {
        k++;
    }
    return k;
}

static JNode* jget(const JNode* obj, const char* key) {
    if (!obj || obj->type != J_OBJ) {
        return NULL;
    }
    for (JNode* c = obj->child; c; c = c->next) {
        if (c->key && !strcasecmp(c->key, key)) {
            return c;
        }
    }
    return NULL;
}

/* a key in its section, else its dotted full name at the root */
static JNode* jfind(const JNode* root, const JNode* parent, const char* key, const char* full) {
    JNode* v = jget(parent, key);
    return v ? v : (full ? jget(root, full) : NULL);
}

static double jnum(const JNode* n) {
    return (n && n->type == J_NUM) ? n->num : 0.0;
}

/* integer value: numbers truncated and clamped, true as 1 */
static int jint(const JNode* n) {
    if (!n) {
        return 0;
    }
    if (n->type == J_TRUE) {
        return 1;
    }
    if (n->type != J_NUM) {
        return 0;
    }
    if (n->num >= 2147483647.0) {
        return 2147483647;
    }
    if (n->num <= -2147483648.0) {
        return (-2147483647 - 1);
    }
    return (int)n->num;
}

static const JNode* jat(const JNode* arr, int i) {
    const JNode* c = arr ? arr->child : NULL;
    while (c && i-- > 0) {
        c = c->next;
    }
    return c;
}

/* the n numbers of an array into out (missing ones keep their value); the
   count of elements present */
static int jvec(const JNode* arr, float* out, int n) {
    int k = 0;
    for (const JNode* c = arr ? arr->child : NULL; c && k < n; c = c->next, k++) {
        out[k] = (float)jnum(c);
    }
    return k;
}

/* ------------------------------------------------------------- lookups */

static const char* k_srctypes[] = {"pencil", "isotropic", "cone", "gaussian", "planar", "pattern", "fourier",
                                   "arcsine", "disk", "fourierx", "fourierx2d", "zgaussian", "line", "slit",
                                   "pencilarray", "pattern3d", "hyperboloid", "ring", NULL};
static const char* k_mediaformats[] = {"byte", "short", "integer", "asgn_float", "svmc", "mixlabel", "labelplus",
                                       "muamus_float", "mua_float", "muamus_half", "asgn_byte", "muamus_short",
                                       NULL};
static const unsigned int k_mediaformatid[] = {1, 2, 4, 96, 97, 98, 99, 100, 101, 102, 103, 104};
static const char k_outputtype[] = "xfejpmrlstbaduvwq";
static const char k_debugflag[] = "RMPT";
static const char k_saveflag[] = "DSPMXVWI";

static int keylookup(const char* key, const char** table) {
    for (int i = 0; table[i]; i++) {
        if (!strcasecmp(key, table[i])) {
            return i;
        }
    }
    return -1;
}

/* letters of a flag string to bits (mcx_parsedebugopt, src/mcx_utils.c:5207) */
static unsigned int flagbits(const char* s, const char* table) {
    unsigned int v = 0;
    for (; *s; s++) {
        const char* q = strchr(table, toupper((unsigned char)*s));
        if (q && *q) {
            v |= 1u << (q - table);
        }
    }
    return v;
}

/* ----------------------------------------------------------------- shapes */

typedef struct {
    unsigned int** vol;
    mcx_uint4* dim;
    float orig[3];
} Grid;

#define VIDX(g, i, j, k) ((size_t)(k) * (g)->dim->x * (g)->dim->y + (size_t)(j) * (g)->dim->x + (size_t)(i))

static int shape_fail(char* err, size_t errlen, const char* msg) {
    snprintf(err, errlen, "%s", msg);
    return -1;
}

static int grid_ready(Grid* g, char* err, size_t errlen) {
    if (!*g->vol) {
        return shape_fail(err, errlen, "a shape comes before the grid is defined (Domain.Dim or a Grid tag)");
    }
    return 0;
}

/* every voxel centre inside the shape gets the tag (src/mcx_shapes.c:234-838) */
static int raster(const char* name, const JNode* obj, Grid* g, char* err, size_t errlen) {
    const JNode* tagn = jget(obj, "Tag");
    const unsigned int tag = (unsigned int)jint(tagn);
    const int nx = (int)g->dim->x, ny = (int)g->dim->y, nz = (int)g->dim->z;
    if (!strcasecmp(name, "Name")) {
        return 0;
    }
    if (!strcasecmp(name, "Origin")) {
        if (!obj || obj->type != J_ARR || jsize(obj) != 3) {
            return shape_fail(err, errlen, "An Origin record does not contain a triplet");
        }
        jvec(obj, g->orig, 3);
        return 0;
    }
    if (!strcasecmp(name, "Grid")) {
        const JNode* sz = jget(obj, "Size");
        if (!sz || jsize(sz) != 3) {
            return shape_fail(err, errlen, "A Grid command misses Size field");
        }
        g->dim->x = (unsigned int)jnum(jat(sz, 0));
        g->dim->y = (unsigned int)jnum(jat(sz, 1));
        g->dim->z = (unsigned int)jnum(jat(sz, 2));
        const size_t n = (size_t)g->dim->x * g->dim->y * g->dim->z;
        free(*g->vol);
        *g->vol = n ? (unsigned int*)calloc(n, sizeof(unsigned int)) : NULL;
        if (n && !*g->vol) {
            return shape_fail(err, errlen, "out of host memory for the grid");
        }
        if (tagn && *g->vol) {
            for (size_t i = 0; i < n; i++) {
                (*g->vol)[i] = tag;
            }
        }
        return 0;
    }
    if (grid_ready(g, err, errlen)) {
        return -1;
    }
    unsigned int* v = *g->vol;
    if (!strcasecmp(name, "Sphere")) {
        const JNode* o = jget(obj, "O");
        const JNode* r = jget(obj, "R");
        if (!o || jsize(o) != 3) {
            return shape_fail(err, errlen, "A Sphere command misses O field");
        }
        if (!r) {
            return shape_fail(err, errlen, "A Sphere command misses R field");
        }
        float O[3];
        jvec(o, O, 3);
        const float R = (float)jnum(r), R2 = R * R;
        /* the sphere's centre is in grid coordinates (the reference does not
           shift it by the origin) */
        for (int k = 0; k < nz; k++) {
            const float dz = (k + 0.5f) - O[2];
            for (int j = 0; j < ny; j++) {
                const float dy = (j + 0.5f) - O[1];
                for (int i = 0; i < nx; i++) {
                    const float dx = (i + 0.5f) - O[0];
                    if (dx * dx + dy * dy + dz * dz <= R2) {
                        v[VIDX(g, i, j, k)] = tag;
                    }
                }
            }
        }
        return 0;
    }
    if (!strcasecmp(name, "Box") || !strcasecmp(name, "Subgrid")) {
        const int sub = !strcasecmp(name, "Subgrid");
        const JNode* o = jget(obj, "O");
        const JNode* sz = jget(obj, "Size");
        if (!o || jsize(o) != 3) {
            return shape_fail(err, errlen, sub ? "A Subgrid command misses O field" : "A Box command misses O field");
        }
        if (!sz || jsize(sz) != 3) {
            return shape_fail(err, errlen, "A Box command misses Size field");
        }
        if (sub) {
            /* integer corners, 1-based, both ends inclusive */
            int O[3], S[3];
            for (int d = 0; d < 3; d++) {
                O[d] = (int)(jint(jat(o, d)) - 1 - g->orig[d]);
                S[d] = jint(jat(sz, d));
            }
            for (int k = 0; k < nz; k++) {
                if (k < O[2] || k > O[2] + S[2]) {
                    continue;
                }
                for (int j = 0; j < ny; j++) {
                    if (j < O[1] || j > O[1] + S[1]) {
                        continue;
                    }
                    for (int i = 0; i < nx; i++) {
                        if (i >= O[0] && i <= O[0] + S[0]) {
                            v[VIDX(g, i, j, k)] = tag;
                        }
                    }
                }
            }
        } else {
            float O[3], S[3];
            jvec(o, O, 3);
            jvec(sz, S, 3);
            for (int d = 0; d < 3; d++) {
                O[d] -= g->orig[d];
            }
            for (int k = 0; k < nz; k++) {
                const float dz = k + 0.5f;
                if (dz < O[2] || dz > O[2] + S[2]) {
                    continue;
                }
                for (int j = 0; j < ny; j++) {
                    const float dy = j + 0.5f;
                    if (dy < O[1] || dy > O[1] + S[1]) {
                        continue;
                    }
                    for (int i = 0; i < nx; i++) {
                        const float dx = i + 0.5f;
                        if (dx >= O[0] && dx <= O[0] + S[0]) {
                            v[VIDX(g, i, j, k)] = tag;
                        }
                    }
                }
            }
        }
        return 0;
    }
    if (!strcasecmp(name, "Cylinder")) {
        const JNode* c0 = jget(obj, "C0");
        const JNode* c1 = jget(obj, "C1");
        const JNode* r = jget(obj, "R");
        if (!c0 || jsize(c0) != 3) {
            return shape_fail(err, errlen, "A Cylinder command misses C0 field");
        }
        if (!c1 || jsize(c1) != 3) {
            return shape_fail(err, errlen, "A Cylinder command misses C1 field");
        }
        if (!r) {
            return shape_fail(err, errlen, "A Cylinder command misses R field");
        }
        float C0[3], C1[3], ax[3];
        jvec(c0, C0, 3);
        jvec(c1, C1, 3);
        for (int d = 0; d < 3; d++) {
            C0[d] -= g->orig[d];
            C1[d] -= g->orig[d];
            ax[d] = C1[d] - C0[d];
        }
        const float len = sqrtf(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
        if (len == 0.f) {
            return shape_fail(err, errlen, "Coincident end points in the definition of Cylinder command");
        }
        for (int d = 0; d < 3; d++) {
            ax[d] /= len;
        }
        const float R = (float)jnum(r), R2 = R * R;
        for (int k = 0; k < nz; k++) {
            const float dz = (k + 0.5f) - C0[2];
            for (int j = 0; j < ny; j++) {
                const float dy = (j + 0.5f) - C0[1];
                for (int i = 0; i < nx; i++) {
                    const float dx = (i + 0.5f) - C0[0];
                    float along = ax[0] * dx + ax[1] * dy + ax[2] * dz;
                    if (along > len || along < 0.f) {
                        continue;
                    }
                    if (dx * dx + dy * dy + dz * dz - along * along <= R2) {
                        v[VIDX(g, i, j, k)] = tag;
                    }
                }
            }
        }
        return 0;
    }
    if (!strcasecmp(name, "UpperSpace")) {
        const JNode* cf = jget(obj, "Coef");
        if (!cf || jsize(cf) != 4) {
            return shape_fail(err, errlen, "An UpperSpace command misses Coef field");
        }
        float C[4];
        jvec(cf, C, 4);
        for (int k = 0; k < nz; k++) {
            for (int j = 0; j < ny; j++) {
                for (int i = 0; i < nx; i++) {
                    if (C[0] * (i + 0.5f) + C[1] * (j + 0.5f) + C[2] * (k + 0.5f) > C[3]) {
                        v[VIDX(g, i, j, k)] = tag;
                    }
                }
            }
        }
        return 0;
    }
    const int slabs = (!strcasecmp(name, "XSlabs") || !strcasecmp(name, "YSlabs") || !strcasecmp(name, "ZSlabs"));
    const int layers = (!strcasecmp(name, "XLayers") || !strcasecmp(name, "YLayers") || !strcasecmp(name, "ZLayers"));
    if (slabs || layers) {
        const int dir = toupper((unsigned char)name[0]) - 'X';
        const int extent = (int)(&g->dim->x)[dir];
        /* slabs: {"Tag": t, "Bound": [a, b] or [[a, b], ...]} in voxel units,
           a rounded down by half a voxel; layers: [start, end, tag] triplets,
           1-based and inclusive */
        const JNode* list = slabs ? jget(obj, "Bound") : obj;
        if (!list || list->type != J_ARR) {
            snprintf(err, errlen, slabs ? "A %s command misses Bound field" : "A %s object must be an array", name);
            return -1;
        }
        const int width = slabs ? 2 : 3;
        const int single = (jsize(list) == width && list->child && list->child->type != J_ARR);
        for (const JNode* it = single ? list : list->child; it; it = single ? NULL : it->next) {
            if (jsize(it) != width) {
                snprintf(err, errlen, slabs ? "The Bound field must contain number pairs"
                                            : "The %s must contain integer triplets", name);
                return -1;
            }
            int lo, hi;
            unsigned int label = tag;
            if (slabs) {
                float a = (float)fmax(jnum(jat(it, 0)) - 0.5, 0.0);
                float b = (float)fmin(jnum(jat(it, 1)), (double)extent);
                if (b < a) {
                    float t = a;
                    a = b;
                    b = t;
                }
                lo = (int)a;
                hi = (int)b;
            } else {
                lo = (jint(jat(it, 0)) > 1 ? jint(jat(it, 0)) : 1) - 1;
                hi = jint(jat(it, 1)) < extent ? jint(jat(it, 1)) : extent;
                if (hi < lo) {
                    int t = lo;
                    lo = hi;
                    hi = t;
                }
                label = (unsigned int)jint(jat(it, 2));
            }
            for (int k = 0; k < nz; k++) {
                for (int j = 0; j < ny; j++) {
                    for (int i = 0; i < nx; i++) {
                        const int c = dir == 0 ? i : (dir == 1 ? j : k);
                        if (c >= lo && c < hi) {
                            v[VIDX(g, i, j, k)] = label;
                        }
                    }
                }
            }
        }
        return 0;
    }
    snprintf(err, errlen, "The Shapes section has an undefined tag %s", name);
    return -1;
}

/* --------------------------------------------------------------- sections */

static int fail(char* err, size_t errlen, int id, const char* msg) {
    snprintf(err, errlen, "%s", msg);
    return id;
}

/* Pos / Dir / Param1 / Param2 of the source: one vector, or an array of
   vectors whose first is the main source and the rest extra sources
   (src/mcx_utils.c:2694-2930) */
static int source_vectors(const JNode* item, Config* cfg, int which, char* err, size_t errlen) {
    if (!item || item->type != J_ARR) {
        return 0;
    }
    const JNode* first = item;
    int nextra = 0;
    if (item->child && item->child->type == J_ARR) {
        nextra = jsize(item) - 1;
        if (cfg->srcdata && (int)cfg->extrasrclen != nextra) {
            return fail(err, errlen, -1, "Length of sub-elements of Pos/Dir/Param1/Param2 must match");
        }
        first = item->child;
    }
    if (nextra > 0 && !cfg->srcdata) {
        cfg->extrasrclen = (unsigned int)nextra;
        cfg->srcdata = (ExtraSrc*)calloc((size_t)nextra, sizeof(ExtraSrc));
        if (!cfg->srcdata) {
            return fail(err, errlen, -2, "out of host memory");
        }
    }
    mcx_float4* mainv[4] = {&cfg->srcpos, &cfg->srcdir, &cfg->srcparam1, &cfg->srcparam2};
    const JNode* vec = first;
    for (int s = 0; vec && s <= nextra; s++, vec = vec->next) {
        mcx_float4* dst = s == 0 ? mainv[which]
                          : (which == 0 ? &cfg->srcdata[s - 1].srcpos
                             : which == 1 ? &cfg->srcdata[s - 1].srcdir
                             : which == 2 ? &cfg->srcdata[s - 1].srcparam1 : &cfg->srcdata[s - 1].srcparam2);
        float* f = &dst->x;
        int k = 0;
        for (const JNode* c = vec->child; c && k < 4; c = c->next, k++) {
            if (which == 1 && k == 3 && c->type == J_STR) {
                /* a direction's focal length may be written as "_NaN_" or "(-)_Inf_" */
                f[3] = !strcmp(c->str, "_NaN_") ? NAN : !strcmp(c->str, "_Inf_") ? INFINITY
                       : !strcmp(c->str, "-_Inf_") ? -INFINITY : f[3];
            } else {
                f[k] = (float)jnum(c);
            }
        }
        if (which < 2 && k < 3) {
            return fail(err, errlen, -1, which ? "Optode.Source.Dir needs three numbers"
                                               : "Optode.Source.Pos needs three numbers");
        }
    }
    return 0;
}

static int load_domain(const JNode* root, const JNode* dom, Config* cfg, char* volfile, size_t vflen, char* err,
                       size_t errlen) {
    const JNode* v = jfind(root, dom, "VolumeFile", "Domain.VolumeFile");
    if (v && v->type == J_STR) {
        snprintf(volfile, vflen, "%s", v->str);
    }
    v = jfind(root, dom, "MediaFormat", "Domain.MediaFormat");
    if (v) {
        int id = keylookup(v->type == J_STR ? v->str : "byte", k_mediaformats);
        if (id < 0) {
            return fail(err, errlen, -1, "Unsupported media format");
        }
        cfg->mediabyte = k_mediaformatid[id];
    }
    v = jfind(root, dom, "LengthUnit", "Domain.LengthUnit");
    cfg->unitinmm = v ? (float)jnum(v) : 1.f;
    const JNode* meds = jfind(root, dom, "Media", "Domain.Media");
    if (meds && meds->child) {
        const int n = jsize(meds);
        if (n > 255) {
            return fail(err, errlen, -4, "input media types exceed the maximum (255)");
        }
        free(cfg->prop);
        cfg->prop = (Medium*)calloc((size_t)n, sizeof(Medium));
        if (!cfg->prop) {
            return fail(err, errlen, -2, "out of host memory");
        }
        cfg->medianum = (unsigned int)n;
        int i = 0;
        for (const JNode* m = meds->child; m; m = m->next, i++) {
            Medium* q = &cfg->prop[i];
            if (m->type == J_OBJ) {
                const char* names[4] = {"mua", "mus", "g", "n"};
                const char* msgs[4] = {"You must specify absorption coeff, default in 1/mm",
                                       "You must specify scattering coeff, default in 1/mm",
                                       "You must specify anisotropy [0-1]", "You must specify refractive index"};
                float* f = &q->mua;
                for (int k = 0; k < 4; k++) {
                    const JNode* x = jget(m, names[k]);
                    if (!x) {
                        return fail(err, errlen, -1, msgs[k]);
                    }
                    f[k] = (float)jnum(x);
                }
            } else if (m->type == J_ARR && jsize(m) >= 4) {
                jvec(m, &q->mua, 4);
            } else {
                return fail(err, errlen, -1,
                            "Session.Media must be either an array of objects or array of 4-elem numerical arrays");
            }
        }
    }
    const JNode* mie = jfind(root, dom, "MieScatter", "Domain.MieScatter");
    if (mie && mie->child) {
        const int n = jsize(mie);
        free(cfg->polprop);
        cfg->polprop = (POLMedium*)calloc((size_t)n, sizeof(POLMedium));
        if (!cfg->polprop) {
            return fail(err, errlen, -2, "out of host memory");
        }
        cfg->polmedianum = (unsigned int)n;
        int i = 0;
        for (const JNode* m = mie->child; m; m = m->next, i++) {
            POLMedium* q = &cfg->polprop[i];
            if (m->type == J_OBJ) {
                q->mua = (float)jnum(jget(m, "mua"));
                q->r = (float)jnum(jget(m, "radius"));
                q->rho = (float)jnum(jget(m, "rho"));
                q->nsph = (float)jnum(jget(m, "nsph"));
                q->nmed = (float)jnum(jget(m, "nmed"));
            } else if (m->type == J_ARR) {
                jvec(m, &q->mua, 5);
            }
        }
    }
    v = jfind(root, dom, "Dim", "Domain.Dim");
    if (v && jsize(v) >= 3) {
        cfg->dim.x = (unsigned int)jint(jat(v, 0));
        cfg->dim.y = (unsigned int)jint(jat(v, 1));
        cfg->dim.z = (unsigned int)jint(jat(v, 2));
    } else if (!jget(root, "Shapes")) {
        return fail(err, errlen, -1, "You must specify the dimension of the volume");
    }
    v = jfind(root, dom, "Step", "Domain.Step");
    if (v) {
        if (jsize(v) < 3) {
            return fail(err, errlen, -1, "Domain::Step has incorrect element numbers");
        }
        jvec(v, &cfg->steps.x, 3);
    }
    if (cfg->steps.x != cfg->steps.y || cfg->steps.y != cfg->steps.z) {
        return fail(err, errlen, -9, "MCX currently does not support anisotropic voxels");
    }
    if (cfg->steps.x != 1.f && cfg->unitinmm == 1.f) {
        cfg->unitinmm = cfg->steps.x;
    }
    if (cfg->unitinmm != 1.f) {
        cfg->steps.x = cfg->steps.y = cfg->steps.z = cfg->unitinmm;
    }
    v = jfind(root, dom, "InverseCDF", "Domain.InverseCDF");
    if (v) {
        const int n = jsize(v);
        free(cfg->invcdf);
        cfg->nphase = (unsigned int)n + 2;
        cfg->invcdf = (float*)calloc(cfg->nphase, sizeof(float));
        if (!cfg->invcdf) {
            return fail(err, errlen, -2, "out of host memory");
        }
        cfg->invcdf[0] = -1.f;
        int i = 1;
        for (const JNode* c = v->child; c; c = c->next, i++) {
            cfg->invcdf[i] = (float)jnum(c);
            if (cfg->invcdf[i] < cfg->invcdf[i - 1] || cfg->invcdf[i] > 1.f || cfg->invcdf[i] < -1.f) {
                return fail(err, errlen, -1, "Domain.InverseCDF contains invalid data; it must be a monotonically "
                            "increasing vector with all values between -1 and 1");
            }
        }
        cfg->invcdf[cfg->nphase - 1] = 1.f;
    }
    v = jfind(root, dom, "OriginType", "Domain.OriginType");
    if (v && cfg->issrcfrom0 == 0) {
        cfg->issrcfrom0 = (char)jint(v);
    }
    return 0;
}

static int load_optode(const JNode* root, const JNode* opt, Config* cfg, char* err, size_t errlen) {
    const JNode* src = jfind(root, opt, "Source", "Optode.Source");
    if (src) {
        int rc = source_vectors(jfind(root, src, "Pos", "Optode.Source.Pos"), cfg, 0, err, errlen);
        const JNode* w = jfind(root, src, "Weight", "Optode.Source.Weight");
        if (!rc && w) {
            cfg->srcpos.w = (float)jnum(w);
        }
        if (!rc) {
            rc = source_vectors(jfind(root, src, "Dir", "Optode.Source.Dir"), cfg, 1, err, errlen);
        }
        const JNode* t = jfind(root, src, "Type", "Optode.Source.Type");
        if (!rc && t) {
            const int id = keylookup(t->type == J_STR ? t->str : "", k_srctypes);
            if (id < 0) {
                return fail(err, errlen, -1, "the specified source type is not supported");
            }
            cfg->srctype = (char)id;
        }
        if (!rc) {
            rc = source_vectors(jfind(root, src, "Param1", "Optode.Source.Param1"), cfg, 2, err, errlen);
        }
        if (!rc) {
            rc = source_vectors(jfind(root, src, "Param2", "Optode.Source.Param2"), cfg, 3, err, errlen);
        }
        if (rc) {
            return rc;
        }
        const JNode* x;
        if ((x = jfind(root, src, "Frequency", "Optode.Source.Frequency"))) {
            cfg->omega = (float)(jnum(x) * 6.28318530717959);
        }
        if ((x = jfind(root, src, "WaveLength", "Optode.Source.WaveLength"))) {
            cfg->lambda = (float)jnum(x);
        }
        if ((x = jfind(root, src, "SrcNum", "Optode.Source.SrcNum"))) {
            cfg->srcnum = (unsigned int)jint(x);
        }
        if ((x = jfind(root, src, "ID", "Optode.Source.ID"))) {
            cfg->srcid = jint(x);
        }
        const JNode* pat = jfind(root, src, "Pattern", "Optode.Source.Pattern");
        if (pat) {
            const int px = jint(jfind(root, pat, "Nx", "Optode.Source.Pattern.Nx"));
            const int py = jint(jfind(root, pat, "Ny", "Optode.Source.Pattern.Ny"));
            const JNode* pzn = jfind(root, pat, "Nz", "Optode.Source.Pattern.Nz");
            const int pz = pzn ? jint(pzn) : 1;
            const JNode* data = jfind(root, pat, "Data", "Optode.Source.Pattern.Data");
            if (px > 0 && py > 0 && pz > 0 && data) {
                const size_t n = (size_t)px * py * pz * (cfg->srcnum ? cfg->srcnum : 1);
                free(cfg->srcpattern);
                cfg->srcpattern = (float*)calloc(n, sizeof(float));
                if (!cfg->srcpattern) {
                    return fail(err, errlen, -2, "out of host memory");
                }
                if (data->type == J_ARR) {
                    const JNode* c = data->child;
                    for (size_t i = 0; i < n; i++, c = c->next) {
                        if (!c) {
                            return fail(err, errlen, -1, "Incomplete pattern data");
                        }
                        cfg->srcpattern[i] = (float)jnum(c);
                    }
                } else if (data->type == J_STR) {
                    FILE* fp = fopen(data->str, "rb");
                    if (!fp) {
                        return fail(err, errlen, -2, "can not read the source pattern file");
                    }
                    const size_t got = fread(cfg->srcpattern, sizeof(float), n, fp);
                    fclose(fp);
                    if (got != n) {
                        return fail(err, errlen, -2, "srcpattern file size does not match the specified data size");
                    }
                }
            }
        }
        const JNode* acdf = jfind(root, src, "AngleInverseCDF", "Optode.Source.AngleInverseCDF");
        if (acdf) {
            const int n = jsize(acdf);
            free(cfg->angleinvcdf);
            cfg->nangle = (unsigned int)n;
            cfg->angleinvcdf = (float*)calloc(n ? (size_t)n : 1, sizeof(float));
            if (!cfg->angleinvcdf) {
                return fail(err, errlen, -2, "out of host memory");
            }
            int i = 0;
            for (const JNode* c = acdf->child; c; c = c->next, i++) {
                cfg->angleinvcdf[i] = (float)jnum(c);
                if ((i > 0 && cfg->angleinvcdf[i] < cfg->angleinvcdf[i - 1]) || cfg->angleinvcdf[i] > 1.f ||
                        cfg->angleinvcdf[i] < 0.f) {
                    return fail(err, errlen, -1, "Optode.Source.AngleInverseCDF contains invalid data; it must be a "
                                "monotonically increasing vector with all values between 0 and 1");
                }
            }
        }
    }
    const JNode* dets = jfind(root, opt, "Detector", "Optode.Detector");
    if (dets && dets->child) {
        const int n = jsize(dets);
        free(cfg->detpos);
        cfg->detpos = (mcx_float4*)calloc((size_t)n, sizeof(mcx_float4));
        if (!cfg->detpos) {
            return fail(err, errlen, -2, "out of host memory");
        }
        cfg->detnum = (unsigned int)n;
        int i = 0;
        for (const JNode* d = dets->child; d; d = d->next, i++) {
            mcx_float4* q = &cfg->detpos[i];
            if (d->type == J_ARR) {
                /* [x, y, z, r] */
                jvec(d, &q->x, 4);
                continue;
            }
            const JNode* pos = jget(d, "Pos");
            const JNode* rad = jget(d, "R");
            const JNode* dir = jget(d, "Dir");
            if (!pos || jsize(pos) < 3) {
                return fail(err, errlen, -1, "a detector needs Pos, three numbers");
            }
            jvec(pos, &q->x, 3);
            if (rad) {
                q->w = (float)jnum(rad);
            }
            if (dir && dir->type == J_ARR) {
                if (!cfg->detdir) {
                    cfg->detdir = (mcx_float4*)calloc((size_t)n, sizeof(mcx_float4));
                    if (!cfg->detdir) {
                        return fail(err, errlen, -2, "out of host memory");
                    }
                }
                jvec(dir, &cfg->detdir[i].x, 4);
            }
        }
    }
    if (cfg->medianum + cfg->detnum + (cfg->extrasrclen << 2) > MAX_PROP_TOTAL) {
        return fail(err, errlen, -4, "input media types plus detector number plus additional sources exceeds the "
                    "maximum total (4000)");
    }
    return 0;
}

static int load_session(const JNode* root, const JNode* ses, Config* cfg, char* err, size_t errlen) {
    const JNode* v;
    v = jfind(root, ses, "RNGSeed", "Session.RNGSeed");
    cfg->seed = v ? jint(v) : -1;
    v = jfind(root, ses, "Photons", "Session.Photons");
    cfg->nphoton = v ? (size_t)jnum(v) : 0;
    if ((v = jfind(root, ses, "MaxDetPhoton", "Session.MaxDetPhoton"))) {
        cfg->maxdetphoton = (unsigned int)jnum(v);
    }
    if (cfg->session[0] == '\0') {
        v = jfind(root, ses, "ID", "Session.ID");
        snprintf(cfg->session, sizeof(cfg->session), "%s", (v && v->type == J_STR) ? v->str : "default");
    }
    if ((v = jfind(root, ses, "BCFlags", "Session.BCFlags")) && v->type == J_STR) {
        memset(cfg->bc, 0, sizeof(cfg->bc));
        strncpy(cfg->bc, v->str, 12);
    }
    struct {
        const char* key;
        const char* full;
        char* dst;
    } flags[] = {
        {"DoMismatch", "Session.DoMismatch", &cfg->isreflect}, {"DoSaveVolume", "Session.DoSaveVolume", &cfg->issave2pt},
        {"DoNormalize", "Session.DoNormalize", &cfg->isnormalized},
        {"DoPartialPath", "Session.DoPartialPath", &cfg->issavedet},
        {"DoSaveRef", "Session.DoSaveRef", &cfg->issaveref}, {"DoSaveExit", "Session.DoSaveExit", &cfg->issaveexit},
        {"DoSaveSeed", "Session.DoSaveSeed", &cfg->issaveseed},
        {"DoAutoThread", "Session.DoAutoThread", &cfg->autopilot}, {"DoDCS", "Session.DoDCS", &cfg->ismomentum},
        {"DoSpecular", "Session.DoSpecular", &cfg->isspecular},
    };
    for (size_t i = 0; i < sizeof(flags) / sizeof(flags[0]); i++) {
        if ((v = jfind(root, ses, flags[i].key, flags[i].full))) {
            *flags[i].dst = (char)jint(v);
        }
    }
    if ((v = jfind(root, ses, "DebugFlag", "Session.DebugFlag"))) {
        cfg->debuglevel = v->type == J_STR ? flagbits(v->str, k_debugflag) : (unsigned int)jint(v);
    }
    if ((v = jfind(root, ses, "SaveDataMask", "Session.SaveDataMask"))) {
        cfg->savedetflag = v->type == J_STR ? flagbits(v->str, k_saveflag) : (unsigned int)jint(v);
    }
    if ((v = jfind(root, ses, "OutputType", "Session.OutputType")) && v->type == J_STR) {
        const char* q = v->str[0] ? strchr(k_outputtype, tolower((unsigned char)v->str[0])) : NULL;
        if (!q) {
            return fail(err, errlen, -2, "the specified output data type is not recognized");
        }
        cfg->outputtype = (char)(q - k_outputtype);
    }
    if ((v = jfind(root, ses, "MinEnergy", "Session.MinEnergy"))) {
        cfg->minenergy = (float)jnum(v);
    }
    return 0;
}

static int load_forward(const JNode* root, const JNode* fwd, Config* cfg, char* err, size_t errlen) {
    cfg->tstart = (float)jnum(jfind(root, fwd, "T0", "Forward.T0"));
    cfg->tend = (float)jnum(jfind(root, fwd, "T1", "Forward.T1"));
    cfg->tstep = (float)jnum(jfind(root, fwd, "Dt", "Forward.Dt"));
    if (cfg->tstart > cfg->tend || cfg->tstep == 0.f) {
        return fail(err, errlen, -9, "incorrect time gate settings");
    }
    const unsigned int gates = (unsigned int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5f);
    if (cfg->maxgate == 0 || cfg->maxgate > gates) {
        cfg->maxgate = gates;
    }
    return 0;
}

/* a binary label volume: mediabyte 1, 2 or 4 bytes a voxel, x fastest
   (mcx_loadvolume, src/mcx_utils.c:3524-3600) */
static int load_volume_file(const char* path, Config* cfg, char* err, size_t errlen) {
    const unsigned int mb = cfg->mediabyte;
    if (mb != 1 && mb != 2 && mb != 4) {
        return fail(err, errlen, -6, "a volume file must hold byte, short or integer labels in this build");
    }
    const size_t n = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    if (!n) {
        return fail(err, errlen, -1, "You must specify the dimension of the volume");
    }
    FILE* fp = fopen(path, "rb");
    if (!fp) {
        return fail(err, errlen, -5, "the specified binary volume file does not exist");
    }
    unsigned char* raw = (unsigned char*)malloc(n * mb);
    free(cfg->vol);
    cfg->vol = (unsigned int*)malloc(n * sizeof(unsigned int));
    if (!raw || !cfg->vol) {
        fclose(fp);
        free(raw);
        return fail(err, errlen, -2, "out of host memory");
    }
    const size_t got = fread(raw, mb, n, fp);
    fclose(fp);
    if (got != n) {
        free(raw);
        return fail(err, errlen, -6, "file size does not match specified dimensions");
    }
    for (size_t i = 0; i < n; i++) {
        if (mb == 1) {
            cfg->vol[i] = raw[i];
        } else if (mb == 2) {
            unsigned short s;
            memcpy(&s, raw + 2 * i, 2);
            cfg->vol[i] = s;
        } else {
            memcpy(cfg->vol + i, raw + 4 * i, 4);
        }
    }
    free(raw);
    return 0;
}

/* A label volume given inline as a JData array in place of the Shapes list
   ({"_ArraySize_": [nx, ny, nz], "_ArrayType_": "uint8", "_ArrayData_":
   [...]}, row-major: mcx_jdatadecode, src/mcx_utils.c:4266-4360); the
   compressed form (_ArrayZipData_) is not read by this build. */
static int load_jdata_volume(const JNode* obj, Config* cfg, char* err, size_t errlen) {
    const JNode* size = jget(obj, "_ArraySize_");
    const JNode* type = jget(obj, "_ArrayType_");
    const JNode* data = jget(obj, "_ArrayData_");
    if (!data) {
        return fail(err, errlen, -1, jget(obj, "_ArrayZipData_") ? "compressed JData volumes are not read by this build"
                                                                 : "No _ArrayZipData_ or _ArrayData_ field is found");
    }
    if (type && type->type == J_STR) {
        if (strstr(type->str, "int8")) {
            cfg->mediabyte = 1;
        } else if (strstr(type->str, "int16")) {
            cfg->mediabyte = 2;
        } else if (strstr(type->str, "double") || strstr(type->str, "int64")) {
            return fail(err, errlen, -1, "8-byte volume array is not supported");
        } else {
            cfg->mediabyte = 4;
        }
    }
    if (data->type != J_ARR || (data->child && data->child->type != J_NUM)) {
        return fail(err, errlen, -1, "JData array constructs are not supported");
    }
    unsigned int dims[3] = {1, 1, 1};
    int k = 0;
    for (const JNode* c = size ? size->child : NULL; c && k < 3; c = c->next, k++) {
        dims[k] = (unsigned int)jint(c);
    }
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    if (n == 0 || (size_t)jsize(data) > n) {
        return fail(err, errlen, -1, "the JData volume's _ArrayData_ does not match its _ArraySize_");
    }
    free(cfg->vol);
    cfg->vol = (unsigned int*)calloc(n, sizeof(unsigned int));
    if (!cfg->vol) {
        return fail(err, errlen, -2, "out of host memory");
    }
    size_t i = 0;
    for (const JNode* c = data->child; c; c = c->next, i++) {
        const int v = jint(c);
        cfg->vol[i] = cfg->mediabyte == 1 ? (unsigned char)v : cfg->mediabyte == 2 ? (unsigned short)v : (unsigned int)v;
    }
    cfg->dim.x = dims[0];
    cfg->dim.y = dims[1];
    cfg->dim.z = dims[2];
    cfg->isrowmajor = 1;
    return 0;
}

int mcxj_load(const char* text, Config* cfg, char* err, size_t errlen) {
    err[0] = '\0';
    JNode* root = jparse(text, err, errlen);
    if (!root) {
        return -1;
    }
    if (root->type != J_OBJ) {
        jfree(root);
        return fail(err, errlen, -1, "the JSON input must be an object");
    }
    const JNode* dom = jget(root, "Domain");
    const JNode* opt = jget(root, "Optode");
    const JNode* ses = jget(root, "Session");
    const JNode* fwd = jget(root, "Forward");
    const JNode* shapes = jget(root, "Shapes");
    char volfile[MAX_PATH_LENGTH] = {0};
    int rc = 0;
    if (dom) {
        rc = load_domain(root, dom, cfg, volfile, sizeof(volfile), err, errlen);
    }
    if (!rc && opt) {
        rc = load_optode(root, opt, cfg, err, errlen);
    }
    if (!rc && ses) {
        rc = load_session(root, ses, cfg, err, errlen);
    }
    if (!rc && fwd) {
        rc = load_forward(root, fwd, cfg, err, errlen);
    }
    if (!rc) {
        if (volfile[0]) {
            rc = shapes ? fail(err, errlen, -1, "You can not specify both Domain.VolumeFile and Shapes sections")
                        : load_volume_file(volfile, cfg, err, errlen);
        } else if (shapes && jget(shapes, "_ArraySize_")) {
            rc = load_jdata_volume(shapes, cfg, err, errlen);
        } else if (shapes) {
            /* the background is label 1 over Domain.Dim, then each tag in turn
               (mcx_parse_jsonshapes, src/mcx_shapes.c:156-205); the origin is
               [1,1,1] unless positions are 0-based */
            Grid g = {&cfg->vol, &cfg->dim, {1.f, 1.f, 1.f}};
            if (cfg->issrcfrom0) {
                g.orig[0] = g.orig[1] = g.orig[2] = 0.f;
            }
            const size_t n = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
            free(cfg->vol);
            cfg->vol = NULL;
            if (n) {
                cfg->vol = (unsigned int*)malloc(n * sizeof(unsigned int));
                if (!cfg->vol) {
                    rc = fail(err, errlen, -2, "out of host memory");
                }
                for (size_t i = 0; !rc && i < n; i++) {
                    cfg->vol[i] = 1;
                }
            }
            int count = 1;
            for (const JNode* s = shapes->type == J_ARR ? shapes->child : NULL; !rc && s && s->child;
                    s = s->next, count++) {
                const JNode* obj = s->child;
                char sub[200];
                if (raster(obj->key ? obj->key : "", obj, &g, sub, sizeof(sub))) {
                    snprintf(err, errlen, "Shapes element #%d: %s", count, sub);
                    rc = -(count + 100);
                }
            }
        } else {
            rc = fail(err, errlen, -1, "You must either define Domain.VolumeFile, or define a Shapes section");
        }
    }
    jfree(root);
    return rc;
}

int mcxj_check(const char* text, char* err, size_t errlen) {
    JNode* root = jparse(text, err, errlen);
    if (!root) {
        return -1;
    }
    jfree(root);
    return 0;
}

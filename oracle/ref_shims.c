/*
 * ref_shims.c -- the libraries the EPREM reference links against, restated
 * for a one-process build in this repository's test harness.  TEST
 * INFRASTRUCTURE ONLY: it lets the reference's own sources (and its unchanged
 * driver src/eprem.c) run here, so that the CPU restatement and the drop-in
 * can be pinned against the reference and against its testsuite digests.
 *
 *   - MPI: MPI_COMM_WORLD of size 1.  Gathers and scatters are copies, sends
 *     to MPI_PROC_NULL do nothing, reductions copy, shared windows are
 *     calloc'd.  MPI_Abort calls a hook when one is set (the per-operator
 *     harness turns a panic into an error code), else exits.
 *   - libconfig: a reader for the libconfig file syntax (settings
 *     `name = value` or `name : value`, optional `;`/`,` terminators,
 *     integers, 64-bit integers, hex, floats, booleans, strings, arrays,
 *     lists, groups; `#`, `//` and C comments).  As in libconfig without
 *     auto-conversion, an integer setting does not satisfy a float lookup and
 *     a float setting does not satisfy an integer lookup.
 *   - netCDF: an in-memory capture.  Datasets are kept per path while the
 *     process lives (so nc_open finds what nc_create made); at process exit
 *     (normal or through MPI_Abort) every dataset that was closed at least
 *     once is written to `<path>.cap` in a small binary layout read by
 *     oracle/digest.py: every variable with its type, shape (the unlimited
 *     dimension at its current length), scale_factor / add_offset and values;
 *     unwritten values hold netCDF's default fill values.
 *   - HDF5: a read-only reader of the file-format subset the MAS slice files
 *     use (see the HDF5 section below).
 */
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpi.h"
#include "libconfig.h"
#include "netcdf.h"
#include "hdf5.h"

/* ======================================================================== */
/* MPI                                                                       */
/* ======================================================================== */
#define SHIM_MAX_TYPES 256
static size_t shim_type_size[SHIM_MAX_TYPES] = {0, 4, 8, 4, 8};
static int shim_ntypes = 5;
#define SHIM_MAX_WINS 4096
static void *shim_win_ptr[SHIM_MAX_WINS];
static int shim_nwins = 1;

void (*refshim_abort_hook)(int code) = NULL;

size_t refshim_type_size(MPI_Datatype t) {
  return (t > 0 && t < shim_ntypes) ? shim_type_size[t] : 0;
}
static int new_type(size_t size, MPI_Datatype *out) {
  if (shim_ntypes >= SHIM_MAX_TYPES) return 1;
  shim_type_size[shim_ntypes] = size;
  *out = shim_ntypes++;
  return 0;
}

double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
int MPI_Init_thread(int *a, char ***b, int req, int *prov) { (void)a; (void)b; *prov = req; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm c, int code) {
  (void)c;
  if (refshim_abort_hook) refshim_abort_hook(code ? code : 2);
  fflush(stdout);
  exit(code);
}
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
int MPI_Comm_split_type(MPI_Comm c, int t, int k, MPI_Info i, MPI_Comm *o) {
  (void)t; (void)k; (void)i; *o = c; return 0;
}
int MPI_Get_address(const void *p, MPI_Aint *a) { *a = (MPI_Aint)(ptrdiff_t)p; return 0; }
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *out) {
  return new_type((size_t)n * refshim_type_size(old), out);
}
int MPI_Type_create_struct(int n, const int bl[], const MPI_Aint disp[],
                           const MPI_Datatype types[], MPI_Datatype *out) {
  size_t ext = 0;
  for (int i = 0; i < n; i++) {
    size_t end = (size_t)disp[i] + (size_t)bl[i] * refshim_type_size(types[i]);
    if (end > ext) ext = end;
  }
  ext = (ext + 7) & ~(size_t)7;
  return new_type(ext, out);
}
int MPI_Type_create_hvector(int n, int bl, MPI_Aint stride, MPI_Datatype old,
                            MPI_Datatype *out) {
  size_t ext = n > 0 ? (size_t)(n - 1) * (size_t)stride + (size_t)bl * refshim_type_size(old) : 0;
  return new_type(ext, out);
}
int MPI_Igatherv(const void *sb, int sc, MPI_Datatype st, void *rb, const int rc[],
                 const int displs[], MPI_Datatype rt, int root, MPI_Comm c, MPI_Request *rq) {
  (void)rc; (void)root; (void)c;
  memmove((char *)rb + (size_t)displs[0] * refshim_type_size(rt), sb,
          (size_t)sc * refshim_type_size(st));
  *rq = 0;
  return 0;
}
int MPI_Iscatterv(const void *sb, const int sc[], const int displs[], MPI_Datatype st, void *rb,
                  int rc, MPI_Datatype rt, int root, MPI_Comm c, MPI_Request *rq) {
  (void)sc; (void)root; (void)c;
  memmove(rb, (const char *)sb + (size_t)displs[0] * refshim_type_size(st),
          (size_t)rc * refshim_type_size(rt));
  *rq = 0;
  return 0;
}
int MPI_Gatherv(const void *sb, int sc, MPI_Datatype st, void *rb, const int rc[],
                const int displs[], MPI_Datatype rt, int root, MPI_Comm c) {
  MPI_Request r;
  return MPI_Igatherv(sb, sc, st, rb, rc, displs, rt, root, c, &r);
}
int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; *r = 0; return 0;
}
int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; *r = 0; return 0;
}
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0;
}
int MPI_Waitall(int n, MPI_Request r[], MPI_Status s[]) { (void)n; (void)r; (void)s; return 0; }
int MPI_Reduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)op; (void)root; (void)c;
  memmove(rb, sb, (size_t)n * refshim_type_size(t));
  return 0;
}
int MPI_Allgather(const void *sb, int sc, MPI_Datatype st, void *rb, int rc, MPI_Datatype rt,
                  MPI_Comm c) {
  (void)rc; (void)rt; (void)c;
  memmove(rb, sb, (size_t)sc * refshim_type_size(st));
  return 0;
}
int MPI_Win_allocate_shared(MPI_Aint size, int du, MPI_Info i, MPI_Comm c, void *base, MPI_Win *w) {
  (void)du; (void)i; (void)c;
  if (shim_nwins >= SHIM_MAX_WINS) return 1;
  void *p = calloc(size > 0 ? (size_t)size : 1, 1);
  shim_win_ptr[shim_nwins] = p;
  *(void **)base = p;
  *w = shim_nwins++;
  return 0;
}
int MPI_Win_shared_query(MPI_Win w, int rank, MPI_Aint *size, int *du, void *base) {
  (void)rank;
  *size = 0;
  *du = 1;
  *(void **)base = (w > 0 && w < shim_nwins) ? shim_win_ptr[w] : NULL;
  return 0;
}
int MPI_Win_lock_all(int a, MPI_Win w) { (void)a; (void)w; return 0; }
int MPI_Win_unlock_all(MPI_Win w) { (void)w; return 0; }
int MPI_Win_sync(MPI_Win w) { (void)w; return 0; }
int MPI_Win_free(MPI_Win *w) {
  if (*w > 0 && *w < shim_nwins) { free(shim_win_ptr[*w]); shim_win_ptr[*w] = NULL; }
  return 0;
}

/* ======================================================================== */
/* libconfig file syntax                                                    */
/* ======================================================================== */
enum { CS_GROUP = 1, CS_INT, CS_INT64, CS_FLOAT, CS_STRING, CS_BOOL, CS_ARRAY, CS_LIST };

struct config_setting_t {
  char *name;      /* NULL for array / list elements */
  int type;
  long long ival;  /* CS_INT, CS_INT64, CS_BOOL */
  double fval;     /* CS_FLOAT */
  char *sval;      /* CS_STRING */
  int n, cap;      /* children of a group, array or list */
  struct config_setting_t **kids;
};

typedef struct {
  const char *s;
  size_t i, n;
  int line;
  const char *err;
} cfg_lex;

static config_setting_t *cs_new(int type) {
  config_setting_t *c = (config_setting_t *)calloc(1, sizeof(*c));
  c->type = type;
  return c;
}
static void cs_free(config_setting_t *c) {
  if (!c) return;
  for (int k = 0; k < c->n; k++) cs_free(c->kids[k]);
  free(c->kids);
  free(c->name);
  free(c->sval);
  free(c);
}
static void cs_add(config_setting_t *p, config_setting_t *c) {
  if (p->n == p->cap) {
    p->cap = p->cap ? 2 * p->cap : 8;
    p->kids = (config_setting_t **)realloc(p->kids, (size_t)p->cap * sizeof(*p->kids));
  }
  p->kids[p->n++] = c;
}

/* Skip white space and comments; returns the next character or 0 at end. */
static int lx_peek(cfg_lex *L) {
  for (;;) {
    while (L->i < L->n && (L->s[L->i] == ' ' || L->s[L->i] == '\t' || L->s[L->i] == '\r' ||
                           L->s[L->i] == '\n' || L->s[L->i] == '\f' || L->s[L->i] == '\v')) {
      if (L->s[L->i] == '\n') L->line++;
      L->i++;
    }
    if (L->i >= L->n) return 0;
    char c = L->s[L->i];
    if (c == '#' || (c == '/' && L->i + 1 < L->n && L->s[L->i + 1] == '/')) {
      while (L->i < L->n && L->s[L->i] != '\n') L->i++;
      continue;
    }
    if (c == '/' && L->i + 1 < L->n && L->s[L->i + 1] == '*') {
      L->i += 2;
      while (L->i + 1 < L->n && !(L->s[L->i] == '*' && L->s[L->i + 1] == '/')) {
        if (L->s[L->i] == '\n') L->line++;
        L->i++;
      }
      L->i = L->i + 2 <= L->n ? L->i + 2 : L->n;
      continue;
    }
    return (unsigned char)c;
  }
}

static int is_name_start(int c) {
  return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || c == '*';
}
static int is_name_char(int c) {
  return is_name_start(c) || (c >= '0' && c <= '9') || c == '-' || c == '_';
}
static int is_digit(int c) { return c >= '0' && c <= '9'; }

static int ci_word(const char *s, size_t len, const char *w) {
  if (strlen(w) != len) return 0;
  for (size_t k = 0; k < len; k++) {
    char a = s[k], b = w[k];
    if (a >= 'A' && a <= 'Z') a = (char)(a - 'A' + 'a');
    if (a != b) return 0;
  }
  return 1;
}

/* A number token: the longest run of characters that can belong to one,
 * then classified as libconfig's scanner does (integer, 64-bit integer with
 * an L suffix or out of int range, hexadecimal, or float when it has a
 * decimal point or an exponent). */
static config_setting_t *lx_number(cfg_lex *L) {
  size_t b = L->i, e = L->i;
  while (e < L->n) {
    char c = L->s[e];
    if (is_digit(c) || c == '.' || c == 'x' || c == 'X' || c == 'L' ||
        (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F') ||
        ((c == '+' || c == '-') && (e == b || L->s[e - 1] == 'e' || L->s[e - 1] == 'E')))
      e++;
    else
      break;
  }
  char tok[128];
  size_t len = e - b;
  if (len == 0 || len >= sizeof(tok)) { L->err = "syntax error"; return NULL; }
  memcpy(tok, L->s + b, len);
  tok[len] = 0;
  L->i = e;
  const char *p = tok;
  int neg = 0;
  if (*p == '+' || *p == '-') { neg = (*p == '-'); p++; }
  int nL = 0;
  while (len > 0 && tok[len - 1] == 'L') { tok[--len] = 0; nL++; }
  if (nL > 2) { L->err = "syntax error"; return NULL; }
  if (p[0] == '0' && (p[1] == 'x' || p[1] == 'X')) {
    if (!p[2]) { L->err = "syntax error"; return NULL; }
    for (const char *q = p + 2; *q; q++)
      if (!((*q >= '0' && *q <= '9') || (*q >= 'a' && *q <= 'f') || (*q >= 'A' && *q <= 'F'))) {
        L->err = "syntax error";
        return NULL;
      }
    unsigned long long u = strtoull(p + 2, NULL, 16);
    config_setting_t *c = cs_new(nL || u > 0xffffffffULL ? CS_INT64 : CS_INT);
    c->ival = nL || u > 0xffffffffULL ? (long long)u : (long long)(int)(unsigned)u;
    if (neg) c->ival = -c->ival;
    return c;
  }
  int digits = 0, dot = 0, expo = 0, bad = 0;
  for (const char *q = p; *q; q++) {
    if (is_digit(*q)) digits++;
    else if (*q == '.' && !dot && !expo) dot = 1;
    else if ((*q == 'e' || *q == 'E') && !expo && digits) {
      expo = 1;
      if (q[1] == '+' || q[1] == '-') q++;
      if (!is_digit(q[1])) bad = 1;
    } else bad = 1;
  }
  if (bad || !digits) { L->err = "syntax error"; return NULL; }
  if (dot || expo) {
    if (nL) { L->err = "syntax error"; return NULL; }
    config_setting_t *c = cs_new(CS_FLOAT);
    c->fval = strtod(tok, NULL);
    return c;
  }
  long long v = strtoll(tok, NULL, 10);
  config_setting_t *c = cs_new(nL || v > INT_MAX || v < INT_MIN ? CS_INT64 : CS_INT);
  c->ival = v;
  return c;
}

static config_setting_t *lx_string(cfg_lex *L) {
  size_t cap = 64, len = 0;
  char *out = (char *)malloc(cap);
  for (;;) { /* adjacent string literals concatenate */
    L->i++; /* opening quote */
    for (;;) {
      if (L->i >= L->n || L->s[L->i] == '\n') { free(out); L->err = "unterminated string"; return NULL; }
      char c = L->s[L->i++];
      if (c == '"') break;
      if (c == '\\' && L->i < L->n) {
        char d = L->s[L->i++];
        switch (d) {
          case 'n': c = '\n'; break;
          case 't': c = '\t'; break;
          case 'r': c = '\r'; break;
          case 'f': c = '\f'; break;
          case 'x': {
            unsigned v = 0;
            for (int k = 0; k < 2 && L->i < L->n; k++) {
              char h = L->s[L->i];
              int dv = is_digit(h) ? h - '0' : (h >= 'a' && h <= 'f') ? h - 'a' + 10
                     : (h >= 'A' && h <= 'F') ? h - 'A' + 10 : -1;
              if (dv < 0) break;
              v = 16 * v + (unsigned)dv;
              L->i++;
            }
            c = (char)v;
            break;
          }
          default: c = d; break;
        }
      }
      if (len + 2 > cap) { cap *= 2; out = (char *)realloc(out, cap); }
      out[len++] = c;
    }
    if (lx_peek(L) != '"') break;
  }
  out[len] = 0;
  config_setting_t *c = cs_new(CS_STRING);
  c->sval = out;
  return c;
}

static config_setting_t *lx_value(cfg_lex *L, int depth);

static int lx_settings(cfg_lex *L, config_setting_t *group, int closing, int depth) {
  for (;;) {
    int c = lx_peek(L);
    if (c == 0) {
      if (closing) { L->err = "syntax error"; return -1; }
      return 0;
    }
    if (closing && c == closing) { L->i++; return 0; }
    if (!is_name_start(c)) { L->err = "syntax error"; return -1; }
    size_t b = L->i;
    while (L->i < L->n && is_name_char((unsigned char)L->s[L->i])) L->i++;
    size_t len = L->i - b;
    c = lx_peek(L);
    if (c != '=' && c != ':') { L->err = "syntax error"; return -1; }
    L->i++;
    config_setting_t *v = lx_value(L, depth + 1);
    if (!v) return -1;
    v->name = (char *)malloc(len + 1);
    memcpy(v->name, L->s + b, len);
    v->name[len] = 0;
    for (int k = 0; k < group->n; k++)
      if (strcmp(group->kids[k]->name, v->name) == 0) {
        cs_free(v);
        L->err = "duplicate setting name";
        return -1;
      }
    cs_add(group, v);
    c = lx_peek(L);
    if (c == ';' || c == ',') L->i++;
  }
}

static config_setting_t *lx_value(cfg_lex *L, int depth) {
  if (depth > 64) { L->err = "nesting too deep"; return NULL; }
  int c = lx_peek(L);
  if (c == '"') return lx_string(L);
  if (c == '{') {
    L->i++;
    config_setting_t *g = cs_new(CS_GROUP);
    if (lx_settings(L, g, '}', depth) < 0) { cs_free(g); return NULL; }
    return g;
  }
  if (c == '[' || c == '(') {
    const int close = c == '[' ? ']' : ')';
    L->i++;
    config_setting_t *a = cs_new(c == '[' ? CS_ARRAY : CS_LIST);
    if (lx_peek(L) == close) { L->i++; return a; }
    for (;;) {
      config_setting_t *v = lx_value(L, depth + 1);
      if (!v) { cs_free(a); return NULL; }
      if (a->type == CS_ARRAY) {
        const int scalar = v->type == CS_INT || v->type == CS_INT64 || v->type == CS_FLOAT ||
                           v->type == CS_STRING || v->type == CS_BOOL;
        if (!scalar || (a->n > 0 && v->type != a->kids[0]->type)) {
          cs_free(v);
          cs_free(a);
          L->err = "mismatched element type in array";
          return NULL;
        }
      }
      cs_add(a, v);
      int d = lx_peek(L);
      if (d == ',') { L->i++; continue; }
      if (d == close) { L->i++; return a; }
      cs_free(a);
      L->err = "syntax error";
      return NULL;
    }
  }
  if (is_digit(c) || c == '.' || c == '+' || c == '-') return lx_number(L);
  if (is_name_start(c)) {
    size_t b = L->i;
    while (L->i < L->n && is_name_char((unsigned char)L->s[L->i])) L->i++;
    if (ci_word(L->s + b, L->i - b, "true") || ci_word(L->s + b, L->i - b, "false")) {
      config_setting_t *v = cs_new(CS_BOOL);
      v->ival = ci_word(L->s + b, L->i - b, "true");
      return v;
    }
  }
  L->err = "syntax error";
  return NULL;
}

typedef struct {
  config_setting_t *root;
  int line;
  char text[96];
} cfg_state;

static cfg_state *cfg_of(const config_t *c) { return (cfg_state *)c->impl; }

void config_init(config_t *c) {
  cfg_state *st = (cfg_state *)calloc(1, sizeof(cfg_state));
  c->impl = st;
}
void config_destroy(config_t *c) {
  cfg_state *st = cfg_of(c);
  if (!st) return;
  cs_free(st->root);
  free(st);
  c->impl = NULL;
}
int config_read_file(config_t *c, const char *path) {
  cfg_state *st = cfg_of(c);
  if (!st) { config_init(c); st = cfg_of(c); }
  cs_free(st->root);
  st->root = NULL;
  FILE *fp = fopen(path, "rb");
  if (!fp) { st->line = 0; snprintf(st->text, sizeof(st->text), "file I/O error"); return CONFIG_FALSE; }
  fseek(fp, 0, SEEK_END);
  long sz = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  char *buf = (char *)malloc(sz > 0 ? (size_t)sz + 1 : 1);
  size_t got = sz > 0 ? fread(buf, 1, (size_t)sz, fp) : 0;
  fclose(fp);
  buf[got] = 0;
  cfg_lex L = {buf, 0, got, 1, NULL};
  config_setting_t *root = cs_new(CS_GROUP);
  int rc = lx_settings(&L, root, 0, 0);
  free(buf);
  if (rc < 0) {
    cs_free(root);
    st->line = L.line;
    snprintf(st->text, sizeof(st->text), "%s", L.err ? L.err : "syntax error");
    return CONFIG_FALSE;
  }
  st->root = root;
  return CONFIG_TRUE;
}
int config_error_line(const config_t *c) { return cfg_of(c) ? cfg_of(c)->line : 0; }
const char *config_error_text(const config_t *c) { return cfg_of(c) ? cfg_of(c)->text : ""; }

/* Path lookup: names separated by '.', from the root group. */
config_setting_t *config_lookup(const config_t *c, const char *path) {
  cfg_state *st = cfg_of(c);
  if (!st || !st->root || !path) return NULL;
  config_setting_t *cur = st->root;
  const char *p = path;
  while (*p) {
    const char *q = p;
    while (*q && *q != '.') q++;
    size_t len = (size_t)(q - p);
    config_setting_t *next = NULL;
    if (cur->type == CS_GROUP)
      for (int k = 0; k < cur->n; k++)
        if (strlen(cur->kids[k]->name) == len && strncmp(cur->kids[k]->name, p, len) == 0) {
          next = cur->kids[k];
          break;
        }
    if (!next) return NULL;
    cur = next;
    p = *q ? q + 1 : q;
  }
  return cur == st->root ? NULL : cur;
}
int config_lookup_int(const config_t *c, const char *path, int *v) {
  const config_setting_t *s = config_lookup(c, path);
  if (!s) return CONFIG_FALSE;
  if (s->type == CS_INT || (s->type == CS_INT64 && s->ival >= INT_MIN && s->ival <= INT_MAX)) {
    *v = (int)s->ival;
    return CONFIG_TRUE;
  }
  return CONFIG_FALSE;
}
int config_lookup_float(const config_t *c, const char *path, double *v) {
  const config_setting_t *s = config_lookup(c, path);
  if (!s || s->type != CS_FLOAT) return CONFIG_FALSE;
  *v = s->fval;
  return CONFIG_TRUE;
}
int config_lookup_string(const config_t *c, const char *path, const char **v) {
  const config_setting_t *s = config_lookup(c, path);
  if (!s || s->type != CS_STRING) return CONFIG_FALSE;
  *v = s->sval;
  return CONFIG_TRUE;
}
int config_setting_length(const config_setting_t *s) {
  return (s && (s->type == CS_ARRAY || s->type == CS_LIST || s->type == CS_GROUP)) ? s->n : 0;
}
double config_setting_get_float_elem(const config_setting_t *s, int i) {
  if (!s || (s->type != CS_ARRAY && s->type != CS_LIST) || i < 0 || i >= s->n) return 0.0;
  const config_setting_t *e = s->kids[i];
  return e->type == CS_FLOAT ? e->fval : 0.0;
}

/* ======================================================================== */
/* netCDF capture                                                            */
/* ======================================================================== */
#define NCS_MAX_FILES 4096
#define NCS_MAX_DIMS 32
#define NCS_MAX_VARS 256
#define NCS_MAX_RANK 8
#define NCS_ERR (-33) /* NC_EBADID in netCDF's numbering */

typedef struct {
  char name[64];
  size_t len;    /* 0 for the unlimited dimension */
} ncs_dim;

typedef struct {
  char name[64];
  nc_type type;
  int ndims, dimids[NCS_MAX_RANK];
  int has_scale, has_offset;
  double scale, offset;
  double *vals;  /* values after conversion to the variable's type */
  size_t nrec;   /* records allocated (record variables) */
} ncs_var;

typedef struct {
  char *path;
  int ndims, nvars;
  ncs_dim dims[NCS_MAX_DIMS];
  ncs_var vars[NCS_MAX_VARS];
  size_t nrec;   /* current length of the unlimited dimension */
  int open, closed_once;
} ncs_file;

static ncs_file *ncs_files[NCS_MAX_FILES];
static int ncs_nfiles = 0;

static ncs_file *ncs_get(int id) {
  return (id >= 0 && id < ncs_nfiles && ncs_files[id] && ncs_files[id]->open) ? ncs_files[id] : NULL;
}
static ncs_var *ncs_getvar(ncs_file *f, int v) {
  return (f && v >= 0 && v < f->nvars) ? &f->vars[v] : NULL;
}
static int ncs_is_record(const ncs_file *f, const ncs_var *v) {
  return v->ndims > 0 && f->dims[v->dimids[0]].len == 0;
}
static size_t ncs_rec_size(const ncs_file *f, const ncs_var *v) {
  size_t n = 1;
  for (int k = ncs_is_record(f, v) ? 1 : 0; k < v->ndims; k++) n *= f->dims[v->dimids[k]].len;
  return n;
}
static double ncs_fill(nc_type t) {
  return t == NC_INT ? -2147483647.0 : 9.9692099683868690e+36;
}
static double ncs_convert(nc_type t, double x) {
  if (t == NC_FLOAT) return (double)(float)x;
  if (t == NC_INT) return (double)(int)x;
  return x;
}
static void ncs_free_file(ncs_file *f) {
  for (int v = 0; v < f->nvars; v++) free(f->vars[v].vals);
  free(f->path);
  free(f);
}

/* Make room for record r of every record variable of f, filling new records. */
static void ncs_grow(ncs_file *f, size_t nrec) {
  if (nrec <= f->nrec) return;
  f->nrec = nrec;
  for (int k = 0; k < f->nvars; k++) {
    ncs_var *v = &f->vars[k];
    if (!ncs_is_record(f, v) || v->nrec >= nrec) continue;
    const size_t rs = ncs_rec_size(f, v);
    v->vals = (double *)realloc(v->vals, nrec * rs * sizeof(double));
    for (size_t i = v->nrec * rs; i < nrec * rs; i++) v->vals[i] = ncs_fill(v->type);
    v->nrec = nrec;
  }
}

const char *nc_strerror(int e) { return e == 0 ? "No error" : "netCDF capture: invalid call"; }

int nc_create(const char *path, int mode, int *id) {
  (void)mode;
  for (int k = 0; k < ncs_nfiles; k++)
    if (ncs_files[k] && strcmp(ncs_files[k]->path, path) == 0) { /* clobber */
      ncs_free_file(ncs_files[k]);
      ncs_files[k] = NULL;
    }
  if (ncs_nfiles >= NCS_MAX_FILES) return NCS_ERR;
  ncs_file *f = (ncs_file *)calloc(1, sizeof(ncs_file));
  f->path = strdup(path);
  f->open = 1;
  ncs_files[ncs_nfiles] = f;
  *id = ncs_nfiles++;
  return NC_NOERR;
}
int nc_open(const char *path, int mode, int *id) {
  (void)mode;
  for (int k = ncs_nfiles - 1; k >= 0; k--)
    if (ncs_files[k] && strcmp(ncs_files[k]->path, path) == 0) {
      ncs_files[k]->open = 1;
      *id = k;
      return NC_NOERR;
    }
  return -2; /* NC_ENOENT-like: no such dataset */
}
int nc_enddef(int id) { return ncs_get(id) ? NC_NOERR : NCS_ERR; }
int nc_def_dim(int id, const char *name, size_t len, int *dimid) {
  ncs_file *f = ncs_get(id);
  if (!f || f->ndims >= NCS_MAX_DIMS) return NCS_ERR;
  snprintf(f->dims[f->ndims].name, sizeof(f->dims[0].name), "%s", name);
  f->dims[f->ndims].len = len;
  *dimid = f->ndims++;
  return NC_NOERR;
}
int nc_def_var(int id, const char *name, nc_type t, int nd, const int *dimids, int *varid) {
  ncs_file *f = ncs_get(id);
  if (!f || f->nvars >= NCS_MAX_VARS || nd < 0 || nd > NCS_MAX_RANK) return NCS_ERR;
  for (int k = 0; k < nd; k++)
    if (dimids[k] < 0 || dimids[k] >= f->ndims || (k > 0 && f->dims[dimids[k]].len == 0))
      return NCS_ERR;
  ncs_var *v = &f->vars[f->nvars];
  memset(v, 0, sizeof(*v));
  snprintf(v->name, sizeof(v->name), "%s", name);
  v->type = t;
  v->ndims = nd;
  for (int k = 0; k < nd; k++) v->dimids[k] = dimids[k];
  if (!ncs_is_record(f, v)) {
    const size_t n = ncs_rec_size(f, v);
    v->vals = (double *)malloc((n ? n : 1) * sizeof(double));
    for (size_t i = 0; i < n; i++) v->vals[i] = ncs_fill(t);
  } else {
    const size_t rs = ncs_rec_size(f, v);
    v->nrec = f->nrec;
    v->vals = (double *)malloc((f->nrec * rs > 0 ? f->nrec * rs : 1) * sizeof(double));
    for (size_t i = 0; i < f->nrec * rs; i++) v->vals[i] = ncs_fill(t);
  }
  *varid = f->nvars++;
  return NC_NOERR;
}
int nc_inq_varid(int id, const char *name, int *varid) {
  ncs_file *f = ncs_get(id);
  if (!f) return NCS_ERR;
  for (int k = 0; k < f->nvars; k++)
    if (strcmp(f->vars[k].name, name) == 0) { *varid = k; return NC_NOERR; }
  return -49; /* NC_ENOTVAR */
}
int nc_put_att_text(int id, int v, const char *name, size_t len, const char *text) {
  (void)v; (void)name; (void)len; (void)text;
  return ncs_get(id) ? NC_NOERR : NCS_ERR;
}
int nc_put_att_double(int id, int varid, const char *name, nc_type t, size_t len, const double *x) {
  ncs_file *f = ncs_get(id);
  if (!f) return NCS_ERR;
  ncs_var *v = ncs_getvar(f, varid);
  if (v && len >= 1) {
    if (strcmp(name, "scale_factor") == 0) { v->has_scale = 1; v->scale = ncs_convert(t, x[0]); }
    if (strcmp(name, "add_offset") == 0) { v->has_offset = 1; v->offset = ncs_convert(t, x[0]); }
  }
  return NC_NOERR;
}

/* Write one hyperslab: element (i_0..i_{n-1}) of the memory side sits at
 * mem[sum i_k imap_k] and goes to file index start_k + i_k stride_k. */
static int ncs_put(int id, int varid, const size_t *start, const size_t *count,
                   const ptrdiff_t *stride, const ptrdiff_t *imap, const void *mem, int memtype) {
  ncs_file *f = ncs_get(id);
  ncs_var *v = ncs_getvar(f, varid);
  if (!v) return NCS_ERR;
  const int nd = v->ndims;
  size_t shape[NCS_MAX_RANK], cnt[NCS_MAX_RANK], st[NCS_MAX_RANK];
  ptrdiff_t str[NCS_MAX_RANK], map[NCS_MAX_RANK];
  size_t total = 1;
  for (int k = 0; k < nd; k++) {
    shape[k] = f->dims[v->dimids[k]].len;
    cnt[k] = count ? count[k] : shape[k];
    if (k == 0 && ncs_is_record(f, v) && !count) cnt[k] = f->nrec;
    st[k] = start ? start[k] : 0;
    str[k] = stride ? stride[k] : 1;
    if (str[k] < 1) return -36; /* NC_ESTRIDE */
    total *= cnt[k];
  }
  if (imap) {
    for (int k = 0; k < nd; k++) map[k] = imap[k];
  } else {
    ptrdiff_t m = 1;
    for (int k = nd - 1; k >= 0; k--) { map[k] = m; m *= (ptrdiff_t)cnt[k]; }
  }
  if (total == 0) return NC_NOERR;
  /* bounds (record dimension grows) */
  for (int k = 0; k < nd; k++) {
    const size_t last = st[k] + (cnt[k] - 1) * (size_t)str[k];
    if (k == 0 && ncs_is_record(f, v)) {
      ncs_grow(f, last + 1);
    } else if (last >= shape[k]) {
      return -40; /* NC_EEDGE */
    }
  }
  size_t fstride[NCS_MAX_RANK];
  {
    size_t m = 1;
    for (int k = nd - 1; k >= 0; k--) {
      fstride[k] = m;
      m *= (k == 0 && ncs_is_record(f, v)) ? 1 : shape[k];
    }
  }
  size_t idx[NCS_MAX_RANK] = {0};
  for (size_t e = 0; e < total; e++) {
    size_t fo = 0;
    ptrdiff_t mo = 0;
    for (int k = 0; k < nd; k++) {
      fo += (st[k] + idx[k] * (size_t)str[k]) * fstride[k];
      mo += (ptrdiff_t)idx[k] * map[k];
    }
    double x;
    if (memtype == NC_INT) x = (double)((const int *)mem)[mo];
    else if (memtype == NC_FLOAT) x = (double)((const float *)mem)[mo];
    else x = ((const double *)mem)[mo];
    v->vals[fo] = ncs_convert(v->type, x);
    for (int k = nd - 1; k >= 0; k--) {
      if (++idx[k] < cnt[k]) break;
      idx[k] = 0;
    }
  }
  return NC_NOERR;
}

int nc_put_var(int id, int varid, const void *x) {
  ncs_var *v = ncs_getvar(ncs_get(id), varid);
  if (!v) return NCS_ERR;
  return ncs_put(id, varid, NULL, NULL, NULL, NULL, x, v->type);
}
int nc_put_var_double(int id, int varid, const double *x) {
  return ncs_put(id, varid, NULL, NULL, NULL, NULL, x, NC_DOUBLE);
}
int nc_put_var1_double(int id, int varid, const size_t *index, const double *x) {
  size_t one[NCS_MAX_RANK] = {1, 1, 1, 1, 1, 1, 1, 1};
  return ncs_put(id, varid, index, one, NULL, NULL, x, NC_DOUBLE);
}
int nc_put_vara_double(int id, int varid, const size_t *s, const size_t *c, const double *x) {
  return ncs_put(id, varid, s, c, NULL, NULL, x, NC_DOUBLE);
}
int nc_put_vara_int(int id, int varid, const size_t *s, const size_t *c, const int *x) {
  return ncs_put(id, varid, s, c, NULL, NULL, x, NC_INT);
}
int nc_put_varm_double(int id, int varid, const size_t *s, const size_t *c, const ptrdiff_t *st,
                       const ptrdiff_t *im, const double *x) {
  return ncs_put(id, varid, s, c, st, im, x, NC_DOUBLE);
}

/* <path>.cap: "EPCAP1\n\0", int32 nvars, then per variable
 *   int32 name length, name, int32 type (4 int, 5 float, 6 double),
 *   int32 rank, int64 shape[rank], int32 has_scale, float64 scale,
 *   int32 has_offset, float64 offset, values (int32 / float32 / float64). */
static int ncs_write(const ncs_file *f) {
  size_t plen = strlen(f->path);
  char *out = (char *)malloc(plen + 5);
  memcpy(out, f->path, plen);
  memcpy(out + plen, ".cap", 5);
  FILE *fp = fopen(out, "wb");
  free(out);
  if (!fp) return -1;
  fwrite("EPCAP1\n", 1, 8, fp);
  int32_t nv = f->nvars;
  fwrite(&nv, 4, 1, fp);
  for (int k = 0; k < f->nvars; k++) {
    const ncs_var *v = &f->vars[k];
    int32_t nl = (int32_t)strlen(v->name), t = v->type, nd = v->ndims;
    fwrite(&nl, 4, 1, fp);
    fwrite(v->name, 1, (size_t)nl, fp);
    fwrite(&t, 4, 1, fp);
    fwrite(&nd, 4, 1, fp);
    size_t n = 1;
    for (int d = 0; d < v->ndims; d++) {
      int64_t len = (d == 0 && ncs_is_record(f, v)) ? (int64_t)f->nrec
                                                    : (int64_t)f->dims[v->dimids[d]].len;
      fwrite(&len, 8, 1, fp);
      n *= (size_t)len;
    }
    int32_t hs = v->has_scale, ho = v->has_offset;
    fwrite(&hs, 4, 1, fp);
    fwrite(&v->scale, 8, 1, fp);
    fwrite(&ho, 4, 1, fp);
    fwrite(&v->offset, 8, 1, fp);
    for (size_t i = 0; i < n; i++) {
      const double x = (ncs_is_record(f, v) && i >= v->nrec * ncs_rec_size(f, v))
                           ? ncs_fill(v->type) : v->vals[i];
      if (v->type == NC_INT) { int32_t y = (int32_t)x; fwrite(&y, 4, 1, fp); }
      else if (v->type == NC_FLOAT) { float y = (float)x; fwrite(&y, 4, 1, fp); }
      else fwrite(&x, 8, 1, fp);
    }
  }
  fclose(fp);
  return 0;
}

static void ncs_flush_all(void) {
  for (int k = 0; k < ncs_nfiles; k++)
    if (ncs_files[k] && ncs_files[k]->closed_once && ncs_write(ncs_files[k]) != 0)
      fprintf(stderr, "netCDF capture: cannot write %s.cap\n", ncs_files[k]->path);
}

int nc_close(int id) {
  static int registered = 0;
  ncs_file *f = ncs_get(id);
  if (!f) return NCS_ERR;
  f->open = 0;
  f->closed_once = 1;
  if (!registered) registered = atexit(ncs_flush_all) == 0;
  return NC_NOERR;
}

/* ======================================================================== */
/* HDF5: the subset the MAS slice files use                                  */
/* ======================================================================== */
/* Read-only, whole file in memory.  Follows the published HDF5 file format:
 * superblock version 0 or 1; the root group's symbol table (version-1 B-tree
 * of group nodes, symbol table nodes "SNOD", local heap "HEAP" for names);
 * version-1 object headers with continuation blocks; dataspace, datatype and
 * data layout messages (layout versions 1-3, contiguous or compact storage).
 * Datasets must be IEEE floats or integers in little-endian order; chunked
 * or filtered storage, other superblock versions and nested groups are
 * refused (the open fails).  Handles: files, datasets, their dataspaces and
 * datatypes share one table; the datatype handle of a little-endian 4-byte
 * float is H5T_NATIVE_FLOAT and of an 8-byte one H5T_NATIVE_DOUBLE. */
#define H5S_MAX_OBJ 1024
#define H5S_MAX_RANK 8
typedef struct {
  int kind;            /* 0 free, 1 file, 2 dataset, 3 dataspace */
  unsigned char *buf;  /* file: contents */
  size_t size;
  int so, sl;          /* sizes of offsets and lengths */
  uint64_t root_btree, root_heap_data;
  int file;            /* dataset / dataspace: owning file handle */
  int rank;
  uint64_t dims[H5S_MAX_RANK];
  int tclass, tsize, tbig;  /* datatype class (0 int, 1 float), size, big-endian */
  int layout;          /* 0 compact, 1 contiguous */
  uint64_t addr, nbytes;
  size_t compact_at;   /* compact data offset in buf */
} h5s_obj;
static h5s_obj h5s_tab[H5S_MAX_OBJ];
#define H5S_BASE 100  /* handles are H5S_BASE + table index (small values are type constants) */

static int h5s_new(int kind) {
  for (int k = 0; k < H5S_MAX_OBJ; k++)
    if (h5s_tab[k].kind == 0) {
      memset(&h5s_tab[k], 0, sizeof(h5s_tab[k]));
      h5s_tab[k].kind = kind;
      return k;
    }
  return -1;
}
static h5s_obj *h5s_get(hid_t h, int kind) {
  const long long k = (long long)h - H5S_BASE;
  return (k >= 0 && k < H5S_MAX_OBJ && h5s_tab[k].kind == kind) ? &h5s_tab[k] : NULL;
}
static int h5s_rd(const h5s_obj *f, uint64_t at, int n, uint64_t *v) {
  if (at + (uint64_t)n > f->size) return -1;
  uint64_t x = 0;
  for (int i = n - 1; i >= 0; i--) x = (x << 8) | f->buf[at + (uint64_t)i];
  *v = x;
  return 0;
}
#define H5RD(f, at, n, v) do { if (h5s_rd((f), (at), (n), (v))) return -1; } while (0)

hid_t H5Fopen(const char *name, unsigned flags, hid_t plist) {
  (void)flags; (void)plist;
  FILE *fp = fopen(name, "rb");
  if (!fp) return -1;
  fseek(fp, 0, SEEK_END);
  long sz = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  if (sz < 96) { fclose(fp); return -1; }
  int k = h5s_new(1);
  if (k < 0) { fclose(fp); return -1; }
  h5s_obj *f = &h5s_tab[k];
  f->buf = (unsigned char *)malloc((size_t)sz);
  f->size = fread(f->buf, 1, (size_t)sz, fp);
  fclose(fp);
  static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  const int ver = f->size >= 16 ? f->buf[8] : -1;
  if (memcmp(f->buf, sig, 8) != 0 || (ver != 0 && ver != 1) || f->buf[13] != 8 ||
      f->buf[14] != 8) {
    free(f->buf);
    f->kind = 0;
    return -1;
  }
  f->so = f->buf[13];
  f->sl = f->buf[14];
  /* 24 fixed bytes (+4 in version 1), four addresses, then the root entry:
   * link name offset, object header address, cache type, reserved, scratch
   * pad holding the B-tree and local heap addresses (cache type 1). */
  const uint64_t root = 24 + (ver == 1 ? 4 : 0) + 4 * 8;
  uint64_t cache, heap, hdata;
  if (h5s_rd(f, root + 16, 4, &cache) || cache != 1 ||
      h5s_rd(f, root + 24, 8, &f->root_btree) || h5s_rd(f, root + 32, 8, &heap) ||
      heap + 32 > f->size || memcmp(f->buf + heap, "HEAP", 4) != 0 ||
      h5s_rd(f, heap + 24, 8, &hdata)) {
    free(f->buf);
    f->kind = 0;
    return -1;
  }
  f->root_heap_data = hdata;
  return H5S_BASE + k;
}
herr_t H5Fclose(hid_t h) {
  h5s_obj *f = h5s_get(h, 1);
  if (!f) return -1;
  free(f->buf);
  f->kind = 0;
  return 0;
}

/* Object header address of `name` under the B-tree node at `node`, or 0. */
static uint64_t h5s_find(const h5s_obj *f, uint64_t node, const char *name, int depth) {
  if (depth > 16 || node + 24 > f->size || memcmp(f->buf + node, "TREE", 4) != 0 ||
      f->buf[node + 4] != 0)
    return 0;
  const int level = f->buf[node + 5];
  uint64_t n;
  if (h5s_rd(f, node + 6, 2, &n)) return 0;
  uint64_t p = node + 8 + 16;  /* after the two sibling addresses */
  for (uint64_t i = 0; i < n; i++) {
    uint64_t child;
    p += 8;  /* key: heap offset */
    if (h5s_rd(f, p, 8, &child)) return 0;
    p += 8;
    if (level > 0) {
      const uint64_t r = h5s_find(f, child, name, depth + 1);
      if (r) return r;
      continue;
    }
    if (child + 8 > f->size || memcmp(f->buf + child, "SNOD", 4) != 0) return 0;
    uint64_t ns;
    if (h5s_rd(f, child + 6, 2, &ns)) return 0;
    for (uint64_t e = 0; e < ns; e++) {
      const uint64_t ent = child + 8 + 40 * e;
      uint64_t lno, oh;
      if (h5s_rd(f, ent, 8, &lno) || h5s_rd(f, ent + 8, 8, &oh)) return 0;
      const uint64_t at = f->root_heap_data + lno;
      if (at >= f->size) return 0;
      const size_t maxlen = f->size - at;
      if (strnlen((const char *)f->buf + at, maxlen) < maxlen &&
          strcmp((const char *)f->buf + at, name) == 0)
        return oh;
    }
  }
  return 0;
}

static int h5s_message(const h5s_obj *f, h5s_obj *d, int type, uint64_t at, uint64_t len) {
  if (at + len > f->size) return -1;
  uint64_t v;
  if (type == 0x0001) { /* dataspace */
    const int ver = f->buf[at], rank = f->buf[at + 1];
    if (rank > H5S_MAX_RANK || (ver != 1 && ver != 2)) return -1;
    const uint64_t dims_at = at + (ver == 1 ? 8 : 4);
    d->rank = rank;
    for (int k = 0; k < rank; k++) { H5RD(f, dims_at + 8 * (uint64_t)k, 8, &v); d->dims[k] = v; }
  } else if (type == 0x0003) { /* datatype */
    d->tclass = f->buf[at] & 0x0f;
    d->tbig = f->buf[at + 1] & 1;
    H5RD(f, at + 4, 4, &v);
    d->tsize = (int)v;
  } else if (type == 0x0008) { /* data layout */
    const int ver = f->buf[at];
    if (ver == 3) {
      const int cls = f->buf[at + 1];
      if (cls == 1) {
        d->layout = 1;
        H5RD(f, at + 2, 8, &d->addr);
        H5RD(f, at + 10, 8, &d->nbytes);
      } else if (cls == 0) {
        d->layout = 0;
        H5RD(f, at + 2, 2, &v);
        d->nbytes = v;
        d->compact_at = (size_t)(at + 4);
      } else {
        return -1; /* chunked */
      }
    } else if (ver == 1 || ver == 2) {
      const int nd = f->buf[at + 1], cls = f->buf[at + 2];
      if (cls == 1) {
        d->layout = 1;
        H5RD(f, at + 8, 8, &d->addr);
        d->nbytes = (uint64_t)-1; /* from the dataspace */
      } else if (cls == 0) {
        d->layout = 0;
        const uint64_t sz_at = at + 8 + 4 * (uint64_t)nd;
        H5RD(f, sz_at, 4, &v);
        d->nbytes = v;
        d->compact_at = (size_t)(sz_at + 4);
      } else {
        return -1;
      }
    } else {
      return -1;
    }
  } else if (type == 0x000B) { /* filter pipeline: not supported */
    return -1;
  }
  return 0;
}

hid_t H5Dopen2(hid_t file, const char *name, hid_t plist) {
  (void)plist;
  h5s_obj *f = h5s_get(file, 1);
  if (!f || !name) return -1;
  const uint64_t oh = h5s_find(f, f->root_btree, name, 0);
  if (!oh || oh + 16 > f->size || f->buf[oh] != 1) return -1;
  const int fk = (int)(f - h5s_tab);
  int k = h5s_new(2);
  if (k < 0) return -1;
  f = &h5s_tab[fk];
  h5s_obj *d = &h5s_tab[k];
  d->file = H5S_BASE + fk;
  d->tclass = -1;
  d->layout = -1;
  uint64_t nmsg, hsize;
  if (h5s_rd(f, oh + 2, 2, &nmsg) || h5s_rd(f, oh + 8, 4, &hsize)) { d->kind = 0; return -1; }
  /* message blocks: the header's own, then continuation blocks */
  uint64_t blk_at[64], blk_len[64];
  int nblk = 1, seen = 0;
  blk_at[0] = oh + 16;
  blk_len[0] = hsize;
  for (int b = 0; b < nblk && (uint64_t)seen < nmsg; b++) {
    uint64_t p = blk_at[b];
    const uint64_t end = blk_at[b] + blk_len[b];
    while (p + 8 <= end && (uint64_t)seen < nmsg) {
      uint64_t type, len;
      if (h5s_rd(f, p, 2, &type) || h5s_rd(f, p + 2, 2, &len)) { d->kind = 0; return -1; }
      if (type == 0x0010) {
        uint64_t ca, cl;
        if (nblk >= 64 || h5s_rd(f, p + 8, 8, &ca) || h5s_rd(f, p + 16, 8, &cl)) {
          d->kind = 0;
          return -1;
        }
        blk_at[nblk] = ca;
        blk_len[nblk++] = cl;
      } else if (h5s_message(f, d, (int)type, p + 8, len)) {
        d->kind = 0;
        return -1;
      }
      seen++;
      p += 8 + len;
    }
  }
  if (d->layout < 0 || d->tclass < 0 || d->tbig) { d->kind = 0; return -1; }
  uint64_t npts = 1;
  for (int r = 0; r < d->rank; r++) npts *= d->dims[r];
  const uint64_t need = npts * (uint64_t)d->tsize;
  if (d->nbytes == (uint64_t)-1) d->nbytes = need;
  const uint64_t start = d->layout == 1 ? d->addr : d->compact_at;
  if (d->nbytes < need || start + need > f->size) { d->kind = 0; return -1; }
  return H5S_BASE + k;
}
herr_t H5Dclose(hid_t h) {
  h5s_obj *d = h5s_get(h, 2);
  if (!d) return -1;
  d->kind = 0;
  return 0;
}
hid_t H5Dget_type(hid_t h) {
  h5s_obj *d = h5s_get(h, 2);
  if (!d) return -1;
  if (d->tclass == 1 && d->tsize == 4) return H5T_NATIVE_FLOAT;
  if (d->tclass == 1 && d->tsize == 8) return H5T_NATIVE_DOUBLE;
  return 3; /* some other type */
}
int H5Tequal(hid_t a, hid_t b) { return a >= 0 && a == b; }
herr_t H5Tclose(hid_t h) { return h >= 0 ? 0 : -1; }
hid_t H5Dget_space(hid_t h) {
  h5s_obj *d = h5s_get(h, 2);
  if (!d) return -1;
  int k = h5s_new(3);
  if (k < 0) return -1;
  d = h5s_get(h, 2);
  h5s_tab[k].rank = d->rank;
  memcpy(h5s_tab[k].dims, d->dims, sizeof(d->dims));
  return H5S_BASE + k;
}
herr_t H5Sclose(hid_t h) {
  h5s_obj *s = h5s_get(h, 3);
  if (!s) return -1;
  s->kind = 0;
  return 0;
}
hssize_t H5Sget_simple_extent_npoints(hid_t h) {
  h5s_obj *s = h5s_get(h, 3);
  if (!s) return -1;
  hssize_t n = 1;
  for (int r = 0; r < s->rank; r++) n *= (hssize_t)s->dims[r];
  return n;
}
/* Whole-dataset reads only (H5S_ALL selections) into a buffer of the file's
 * own type. */
herr_t H5Dread(hid_t dset, hid_t memtype, hid_t memspace, hid_t filespace, hid_t xfer, void *out) {
  (void)xfer;
  h5s_obj *d = h5s_get(dset, 2);
  if (!d || memspace != H5S_ALL || filespace != H5S_ALL || memtype != H5Dget_type(dset)) return -1;
  h5s_obj *f = h5s_get(d->file, 1);
  if (!f) return -1;
  uint64_t npts = 1;
  for (int r = 0; r < d->rank; r++) npts *= d->dims[r];
  const uint64_t start = d->layout == 1 ? d->addr : d->compact_at;
  memcpy(out, f->buf + start, (size_t)(npts * (uint64_t)d->tsize));
  return 0;
}

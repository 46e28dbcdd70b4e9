/*
 * fv3d_ini.c -- CPU restatement of the reference's .ini reader.
 *
 * TEST INFRASTRUCTURE ONLY: gives the oracle (and the reference arm of the
 * benchmark, which must not load the GPU library) the Params that the
 * reference's readInifile (SimInfo.h:169-306) builds from an .ini text.
 * Pinned by tests/test_ini.py against the Params the reference's own
 * readInifile produced for every golden case and for the INIReader edge
 * cases.
 *
 * INIReader semantics restated (jtilly/inih, the header SimInfo.h:5
 * includes; an empty, unpinned submodule of the reference): one
 * "[section]" or "name = value" / "name : value" per line, surrounding
 * whitespace stripped, ';' or '#' at the start of a line is a comment, ';'
 * after whitespace starts an inline comment, an indented line continues the
 * previous value, a UTF-8 BOM on the first line is skipped; section and key
 * names compare case-insensitively, values do not; a repeated key appends
 * "\n" + value.  Getters: integers by strtol(base 0), floats by strtof
 * (single precision), booleans true/yes/on/1 and false/no/off/0; a value
 * that does not parse yields the default.  Unknown enum strings map to 0
 * (std::map::operator[] in readInifile).
 */
#include "fv3d_oracle.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  char* key;   /* "section=name", lower case */
  char* value;
} ini_entry;

typedef struct {
  ini_entry* e;
  int n, cap;
} ini_table;

static char* dup_range(const char* b, size_t n) {
  char* s = (char*)malloc(n + 1);
  memcpy(s, b, n);
  s[n] = '\0';
  return s;
}

static char* make_key(const char* section, const char* name) {
  size_t a = strlen(section), b = strlen(name);
  char* k = (char*)malloc(a + b + 2);
  size_t i;
  for (i = 0; i < a; ++i) k[i] = (char)tolower((unsigned char)section[i]);
  k[a] = '=';
  for (i = 0; i < b; ++i) k[a + 1 + i] = (char)tolower((unsigned char)name[i]);
  k[a + b + 1] = '\0';
  return k;
}

static ini_entry* find(const ini_table* t, const char* key) {
  int i;
  for (i = 0; i < t->n; ++i)
    if (strcmp(t->e[i].key, key) == 0) return &t->e[i];
  return NULL;
}

/* INIReader::ValueHandler: repeated keys are joined with "\n". */
static void add(ini_table* t, const char* section, const char* name, const char* value) {
  char* key = make_key(section, name);
  ini_entry* e = find(t, key);
  if (!e) {
    if (t->n == t->cap) {
      t->cap = t->cap ? 2 * t->cap : 32;
      t->e = (ini_entry*)realloc(t->e, (size_t)t->cap * sizeof(ini_entry));
    }
    e = &t->e[t->n++];
    e->key = key;
    e->value = dup_range("", 0);
  } else {
    free(key);
  }
  if (e->value[0] != '\0') {
    size_t a = strlen(e->value), b = strlen(value);
    e->value = (char*)realloc(e->value, a + b + 2);
    e->value[a] = '\n';
    memcpy(e->value + a + 1, value, b + 1);
  } else {
    size_t b = strlen(value);
    e->value = (char*)realloc(e->value, b + 1);
    memcpy(e->value, value, b + 1);
  }
}

static int is_space(char c) { return isspace((unsigned char)c) != 0; }

/* Position in s[p..n) of the first char of `stops`, or of a ';' that
 * follows whitespace (an inline comment); n when there is none. */
static size_t scan(const char* s, size_t p, size_t n, const char* stops) {
  int prev_space = 0;
  for (; p < n; ++p) {
    char c = s[p];
    if (stops && c != '\0' && strchr(stops, c)) return p;
    if (prev_space && c == ';') return p;
    prev_space = is_space(c);
  }
  return n;
}

static char* trimmed(const char* s, size_t b, size_t e) {
  while (b < e && is_space(s[b])) ++b;
  while (e > b && is_space(s[e - 1])) --e;
  return dup_range(s + b, e - b);
}

static void parse(ini_table* t, const char* text) {
  char section[512] = "";
  char* last_name = NULL;
  size_t pos = 0, len = strlen(text);
  int first = 1;
  while (pos < len) {
    const char* nlp = strchr(text + pos, '\n');
    size_t nl = nlp ? (size_t)(nlp - text) : len;
    const char* line = text + pos;
    size_t n = nl - pos, b = 0, e;
    pos = nl + 1;
    if (first && n >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
        (unsigned char)line[2] == 0xBF) {
      line += 3;
      n -= 3;
    }
    first = 0;
    e = n;
    while (e > 0 && is_space(line[e - 1])) --e;
    while (b < e && is_space(line[b])) ++b;
    if (b == e) continue;
    if (line[b] == ';' || line[b] == '#') continue;
    if (b > 0 && last_name) { /* indented: continuation of the previous value */
      char* v = dup_range(line + b, e - b);
      add(t, section, last_name, v);
      free(v);
      continue;
    }
    if (line[b] == '[') {
      size_t close = scan(line, b + 1, e, "]");
      if (close < e && line[close] == ']') {
        size_t m = close - b - 1;
        if (m >= sizeof(section)) m = sizeof(section) - 1;
        memcpy(section, line + b + 1, m);
        section[m] = '\0';
        free(last_name);
        last_name = NULL;
      }
      continue;
    }
    {
      size_t sep = scan(line, b, e, "=:");
      if (sep < e && (line[sep] == '=' || line[sep] == ':')) {
        size_t vb = sep + 1, ve;
        char *name, *value;
        while (vb < e && is_space(line[vb])) ++vb;
        ve = scan(line, vb, e, NULL);
        name = trimmed(line, b, sep);
        value = trimmed(line, vb, ve);
        add(t, section, name, value);
        free(last_name);
        last_name = name;
        free(value);
      }
    }
  }
  free(last_name);
}

static void table_free(ini_table* t) {
  int i;
  for (i = 0; i < t->n; ++i) {
    free(t->e[i].key);
    free(t->e[i].value);
  }
  free(t->e);
}

static const char* get(const ini_table* t, const char* section, const char* name, const char* dflt) {
  char* key = make_key(section, name);
  const ini_entry* e = find(t, key);
  free(key);
  return e ? e->value : dflt;
}

static long get_integer(const ini_table* t, const char* section, const char* name, long dflt) {
  const char* v = get(t, section, name, "");
  char* end = NULL;
  long n = strtol(v, &end, 0);
  return end > v ? n : dflt;
}

static float get_float(const ini_table* t, const char* section, const char* name, float dflt) {
  const char* v = get(t, section, name, "");
  char* end = NULL;
  float n = strtof(v, &end);
  return end > v ? n : dflt;
}

static int get_boolean(const ini_table* t, const char* section, const char* name, int dflt) {
  const char* v = get(t, section, name, "");
  char low[16];
  size_t i, n = strlen(v);
  if (n >= sizeof(low)) return dflt;
  for (i = 0; i <= n; ++i) low[i] = (char)tolower((unsigned char)v[i]);
  if (!strcmp(low, "true") || !strcmp(low, "yes") || !strcmp(low, "on") || !strcmp(low, "1")) return 1;
  if (!strcmp(low, "false") || !strcmp(low, "no") || !strcmp(low, "off") || !strcmp(low, "0")) return 0;
  return dflt;
}

/* readInifile's std::map lookups: an unknown string gives enum value 0. */
static int lookup(const char* v, const char* const* names, const int* values, int n) {
  int i;
  for (i = 0; i < n; ++i)
    if (!strcmp(v, names[i])) return values[i];
  return 0;
}

static void copy_str(char* dst, size_t cap, const char* src) {
  strncpy(dst, src, cap - 1);
  dst[cap - 1] = '\0';
}

/* SimInfo.h:169-306 (field by field, same defaults and derived dx/dy/dz). */
static void fill_params(const ini_table* r, fv_params* o) {
  static const char* const bc_n[] = {"reflecting", "absorbing", "periodic", "C91"};
  static const int bc_v[] = {FV_BC_REFLECTING, FV_BC_ABSORBING, FV_BC_PERIODIC, FV_BC_C91};
  static const char* const rc_n[] = {"pcm", "pcm_wb", "plm"};
  static const int rc_v[] = {FV_PCM, FV_PCM_WB, FV_PLM};
  static const char* const rs_n[] = {"hll", "hllc"};
  static const int rs_v[] = {FV_HLL, FV_HLLC};
  static const char* const ts_n[] = {"euler", "RK2"};
  static const int ts_v[] = {FV_TS_EULER, FV_TS_RK2};
  static const char* const tcm_n[] = {"constant", "B02"};
  static const int tcm_v[] = {FV_TCM_CONSTANT, FV_TCM_B02};
  static const char* const bctc_n[] = {"none", "fixed_temperature", "fixed_gradient"};
  static const int bctc_v[] = {FV_BCTC_NONE, FV_BCTC_FIXED_TEMPERATURE, FV_BCTC_FIXED_GRADIENT};
  static const char* const vm_n[] = {"constant"};
  static const int vm_v[] = {FV_VSC_CONSTANT};
  static const char* const pr_n[] = {"fp64", "fp32_mixed"};
  static const int pr_v[] = {FV_PREC_FP64, FV_PREC_FP32_MIXED};
  static const char* const ph_n[] = {"reference", "corrected"};
  static const int ph_v[] = {FV_PHYS_REFERENCE, FV_PHYS_CORRECTED};

  memset(o, 0, sizeof(*o));
  o->Nx = (int)get_integer(r, "mesh", "Nx", 32);
  o->Ny = (int)get_integer(r, "mesh", "Ny", 32);
  o->Nz = (int)get_integer(r, "mesh", "Nz", 32);
  o->Ng = (int)get_integer(r, "mesh", "Nghosts", 2);
  o->xmin = get_float(r, "mesh", "xmin", 0.0f);
  o->xmax = get_float(r, "mesh", "xmax", 1.0f);
  o->ymin = get_float(r, "mesh", "ymin", 0.0f);
  o->ymax = get_float(r, "mesh", "ymax", 1.0f);
  o->zmin = get_float(r, "mesh", "zmin", 0.0f);
  o->zmax = get_float(r, "mesh", "zmax", 1.0f);
  o->dx = (o->xmax - o->xmin) / o->Nx;
  o->dy = (o->ymax - o->ymin) / o->Ny;
  o->dz = (o->zmax - o->zmin) / o->Nz;

  o->tend = get_float(r, "run", "tend", 1.0f);
  o->save_freq = get_float(r, "run", "save_freq", 1.0e-1f);
  copy_str(o->filename_out, sizeof(o->filename_out), get(r, "run", "output_filename", "run"));
  o->boundary_x = lookup(get(r, "run", "boundaries_x", "reflecting"), bc_n, bc_v, 4);
  o->boundary_y = lookup(get(r, "run", "boundaries_y", "reflecting"), bc_n, bc_v, 4);
  o->boundary_z = lookup(get(r, "run", "boundaries_z", "reflecting"), bc_n, bc_v, 4);

  o->reconstruction = lookup(get(r, "solvers", "reconstruction", "pcm"), rc_n, rc_v, 3);
  o->riemann_solver = lookup(get(r, "solvers", "riemann_solver", "hllc"), rs_n, rs_v, 2);
  o->time_stepping = lookup(get(r, "solvers", "time_stepping", "euler"), ts_n, ts_v, 2);
  o->CFL = get_float(r, "solvers", "CFL", 0.8f);

  o->epsilon = get_float(r, "misc", "epsilon", 1.0e-6f);
  o->gamma0 = get_float(r, "physics", "gamma0", (float)(5.0 / 3.0));
  o->gravity = get_boolean(r, "physics", "gravity", 0);
  o->g = get_float(r, "physics", "g", 0.0f);
  o->m1 = get_float(r, "polytrope", "m1", 1.0f);
  o->theta1 = get_float(r, "polytrope", "theta1", 10.0f);
  o->m2 = get_float(r, "polytrope", "m2", 1.0f);
  o->theta2 = get_float(r, "polytrope", "theta2", 10.0f);
  copy_str(o->problem, sizeof(o->problem), get(r, "physics", "problem", "blast"));
  o->well_balanced_flux_at_z_bc = get_boolean(r, "physics", "well_balanced_flux_at_z_bc", 0);

  o->thermal_conductivity_active = get_boolean(r, "thermal_conduction", "active", 0);
  o->thermal_conductivity_mode =
      lookup(get(r, "thermal_conduction", "conductivity_mode", "constant"), tcm_n, tcm_v, 2);
  o->kappa = get_float(r, "thermal_conduction", "kappa", 0.0f);
  o->bctc_zmin = lookup(get(r, "thermal_conduction", "bc_zmin", "none"), bctc_n, bctc_v, 3);
  o->bctc_zmax = lookup(get(r, "thermal_conduction", "bc_zmax", "none"), bctc_n, bctc_v, 3);
  o->bctc_zmin_value = get_float(r, "thermal_conduction", "bc_zmin_value", 1.0f);
  o->bctc_zmax_value = get_float(r, "thermal_conduction", "bc_zmax_value", 1.0f);

  o->viscosity_active = get_boolean(r, "viscosity", "active", 0);
  o->viscosity_mode = lookup(get(r, "viscosity", "viscosity_mode", "constant"), vm_n, vm_v, 1);
  o->mu = get_float(r, "viscosity", "mu", 0.0f);

  o->h84_pert = get_float(r, "H84", "perturbation", 1.0e-4f);
  o->c91_pert = get_float(r, "C91", "perturbation", 1.0e-3f);
  o->seed = (int)get_integer(r, "misc", "seed", 12345);
  o->log_frequency = (int)get_integer(r, "misc", "log_frequency", 10);

  /* keys of the GPU driver only (no reference counterpart) */
  o->precision = lookup(get(r, "gpu", "precision", "fp64"), pr_n, pr_v, 2);
  o->physics = lookup(get(r, "gpu", "physics", "reference"), ph_n, ph_v, 2);
}

int fvora_parse_ini(const char* text, fv_params* out) {
  ini_table t = {NULL, 0, 0};
  if (!text || !out) return FV_ERR_PARAM;
  parse(&t, text);
  fill_params(&t, out);
  table_free(&t);
  return FV_OK;
}

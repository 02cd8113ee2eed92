// Parameter-file reader with the reference's parsing rules
// (src/parameter.c:13-131), plus this library's extension keys.
//
// Rules kept from the reference: text from the first '#' is dropped; the line
// is split on spaces only (a tab stays inside its token); a token selects a key
// when it starts with the key's name (strncmp over the key's length); every key
// whose name prefixes the token is applied; atoi / atof / strdup convert the
// value, so a name followed directly by a newline keeps the newline (and then
// matches no special boundary condition, as in the reference).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

#include "nusif_internal.h"

namespace nusif {

Extras *extras_for(const Parameter *p, bool create)
{
  static std::unordered_map<const Parameter *, Extras> table;
  auto it = table.find(p);
  if (it != table.end()) return &it->second;
  if (!create) return nullptr;
  return &table[p];
}

namespace {

enum Kind { K_INT, K_REAL, K_STRING };
struct Key {
  const char *name;
  Kind kind;
  size_t offset;
};

#define NUSIF_KEY(member, kind) { #member, kind, offsetof(Parameter, member) }
// the reference's key list and conversion per key (src/parameter.c:65-95)
const Key kKeys[] = {
  NUSIF_KEY(xlength, K_REAL), NUSIF_KEY(ylength, K_REAL), NUSIF_KEY(zlength, K_REAL),
  NUSIF_KEY(imax, K_INT), NUSIF_KEY(jmax, K_INT), NUSIF_KEY(kmax, K_INT),
  NUSIF_KEY(itermax, K_INT), NUSIF_KEY(levels, K_INT), NUSIF_KEY(presmooth, K_INT),
  NUSIF_KEY(postsmooth, K_INT), NUSIF_KEY(eps, K_REAL), NUSIF_KEY(omg, K_REAL),
  NUSIF_KEY(re, K_REAL), NUSIF_KEY(tau, K_REAL), NUSIF_KEY(gamma, K_REAL),
  NUSIF_KEY(dt, K_REAL), NUSIF_KEY(te, K_REAL), NUSIF_KEY(gx, K_REAL), NUSIF_KEY(gy, K_REAL),
  NUSIF_KEY(gz, K_REAL), NUSIF_KEY(name, K_STRING), NUSIF_KEY(bcLeft, K_INT),
  NUSIF_KEY(bcRight, K_INT), NUSIF_KEY(bcBottom, K_INT), NUSIF_KEY(bcTop, K_INT),
  NUSIF_KEY(bcFront, K_INT), NUSIF_KEY(bcBack, K_INT), NUSIF_KEY(u_init, K_REAL),
  NUSIF_KEY(v_init, K_REAL), NUSIF_KEY(w_init, K_REAL), NUSIF_KEY(p_init, K_REAL),
};
#undef NUSIF_KEY

bool starts_with(const char *tok, const char *key) { return strncmp(tok, key, strlen(key)) == 0; }

// extension values are trimmed of trailing whitespace (the reference keys are not)
void trimmed(const char *val, char *out, size_t n)
{
  size_t len = strlen(val);
  while (len > 0 && (val[len - 1] == '\n' || val[len - 1] == '\r' || val[len - 1] == '\t' ||
                        val[len - 1] == ' '))
    len--;
  if (len >= n) len = n - 1;
  memcpy(out, val, len);
  out[len] = '\0';
}

int solver_from_name(const char *v)
{
  if (strcmp(v, "rb") == 0) return SOLVER_RB;
  if (strcmp(v, "mg-ref") == 0 || strcmp(v, "mgref") == 0) return SOLVER_MG_REF;
  if (strcmp(v, "mg") == 0) return SOLVER_MG;
  if (strcmp(v, "mg-mixed") == 0 || strcmp(v, "mixed") == 0) return SOLVER_MG_MIXED;
  return -1;
}

// extension keys; returns 1 if the token named one of them
int apply_extra(Parameter *param, const char *tok, const char *val)
{
  Extras *x = extras_for(param, true);
  char v[256];
  trimmed(val, v, sizeof(v));
  int hit = 0;
  if (starts_with(tok, "solver")) {
    int s = solver_from_name(v);
    if (s < 0) {
      fail(NUSIF_ERR_ARG, "unknown solver '%s' (rb, mg-ref, mg, mg-mixed)", v);
      return 1;
    }
    x->solver = s;
    hit = 1;
  }
  if (starts_with(tok, "lid")) { x->lid = atof(v); hit = 1; }
  if (starts_with(tok, "inflow")) { x->inflow = atof(v); hit = 1; }
  if (starts_with(tok, "rtol")) { x->rtol = atof(v); hit = 1; }
  if (starts_with(tok, "mg_levels")) { x->mg_levels = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_pre")) { x->mg_pre = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_post")) { x->mg_post = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_coarse")) { x->mg_coarse_sweeps = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_cycles")) { x->mg_maxcycles = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_inner")) { x->mg_inner = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_theta")) { x->mg_theta = atof(v); hit = 1; }
  if (starts_with(tok, "mg_omega")) { x->mg_omega = atof(v); hit = 1; }
  if (starts_with(tok, "mg_graph")) { x->mg_graph = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_tail")) { x->mg_tail = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_chunk")) { x->mg_chunk = atoi(v); hit = 1; }
  if (starts_with(tok, "host_fields")) { x->host_fields = atoi(v); hit = 1; }
  if (starts_with(tok, "mg_probe")) { x->mg_guess_probe = atoi(v); hit = 1; }
  if (starts_with(tok, "fuse_dt")) { x->fuse_dt = atoi(v); hit = 1; }
  if (starts_with(tok, "fg_arith")) {
    if (strcmp(v, "fp64") == 0) x->fg_fp64 = 1;
    else if (strcmp(v, "df32") == 0) x->fg_fp64 = 0;
    else {
      fail(NUSIF_ERR_ARG, "unknown fg_arith '%s' (df32, fp64)", v);
      return 1;
    }
    hit = 1;
  }
  if (starts_with(tok, "arith")) {
    if (strcmp(v, "fp64") == 0) x->arith_fp64 = x->fg_fp64 = 1;
    else if (strcmp(v, "df32") == 0) x->arith_fp64 = x->fg_fp64 = 0;
    else {
      fail(NUSIF_ERR_ARG, "unknown arith '%s' (df32, fp64)", v);
      return 1;
    }
    hit = 1;
  }
  if (starts_with(tok, "mg_guess")) {
    if (strcmp(v, "previous") == 0) x->mg_guess = 0;
    else if (strcmp(v, "extrapolate") == 0) x->mg_guess = 1;
    else if (strcmp(v, "quadratic") == 0) x->mg_guess = 2;
    else if (strcmp(v, "cubic") == 0) x->mg_guess = 3;
    else x->mg_guess = atoi(v);
    hit = 1;
  }
  return hit;
}

void apply_line(Parameter *param, char *line)
{
  char *hash = strchr(line, '#');
  if (hash) *hash = '\0';
  char *save = nullptr;
  char *tok = strtok_r(line, " ", &save);
  char *val = strtok_r(nullptr, " ", &save);
  if (tok == nullptr || val == nullptr) return;
  for (const Key &k : kKeys) {
    if (!starts_with(tok, k.name)) continue;
    char *slot = reinterpret_cast<char *>(param) + k.offset;
    switch (k.kind) {
    case K_INT: *reinterpret_cast<int *>(slot) = atoi(val); break;
    case K_REAL: *reinterpret_cast<double *>(slot) = atof(val); break;
    case K_STRING: *reinterpret_cast<char **>(slot) = strdup(val); break;
    }
  }
  apply_extra(param, tok, val);
}

}  // namespace
}  // namespace nusif

using namespace nusif;

extern "C" {

// initParameter, reference src/parameter.c:13-30 (same defaults; other members untouched)
void initParameter(Parameter *param)
{
  param->xlength = 1.0;
  param->ylength = 1.0;
  param->zlength = 1.0;
  param->imax = 100;
  param->jmax = 100;
  param->kmax = 100;
  param->itermax = 1000;
  param->eps = 0.0001;
  param->omg = 1.7;
  param->re = 100.0;
  param->gamma = 0.9;
  param->tau = 0.5;
  param->levels = 5;
  param->presmooth = 5;
  param->postsmooth = 5;
  *extras_for(param, true) = Extras();
}

// readParameter, reference src/parameter.c:32-98
void readParameter(Parameter *param, const char *filename)
{
  FILE *fp = fopen(filename, "r");
  if (!fp) {
    fail(NUSIF_ERR_IO, "Could not open parameter file: %s", filename);
    return;
  }
  char line[4096];
  while (!feof(fp)) {
    line[0] = '\0';
    if (fgets(line, sizeof(line), fp) == NULL && ferror(fp) != 0)
      fprintf(stderr, "Error in fgets function\n");
    apply_line(param, line);
  }
  fclose(fp);
}

// printParameter, reference src/parameter.c:100-131 (same text)
void printParameter(Parameter *param)
{
  printf("Parameters for %s\n", param->name);
  printf("Boundary conditions Left:%d Right:%d Bottom:%d Top:%d Front:%d "
         "Back:%d\n",
      param->bcLeft, param->bcRight, param->bcBottom, param->bcTop, param->bcFront,
      param->bcBack);
  printf("\tReynolds number: %.2f\n", param->re);
  printf("\tInit arrays: U:%.2f V:%.2f W:%.2f P:%.2f\n", param->u_init, param->v_init,
      param->w_init, param->p_init);
  printf("Geometry data:\n");
  printf("\tDomain box size (x, y, z): %.2f, %.2f, %.2f\n", param->xlength, param->ylength,
      param->zlength);
  printf("\tCells (x, y, z): %d, %d, %d\n", param->imax, param->jmax, param->kmax);
  printf("Timestep parameters:\n");
  printf("\tDefault stepsize: %.2f, Final time %.2f\n", param->dt, param->te);
  printf("\tTau factor: %.2f\n", param->tau);
  printf("Iterative solver parameters:\n");
  printf("\tMax iterations: %d\n", param->itermax);
  printf("\tepsilon (stopping tolerance) : %f\n", param->eps);
  printf("\tgamma (stopping tolerance) : %f\n", param->gamma);
  printf("\tomega (SOR relaxation): %f\n", param->omg);
}

int nusifParameterSet(Parameter *param, const char *key, const char *value)
{
  if (!param || !key || !value) {
    fail(NUSIF_ERR_ARG, "nusifParameterSet: null argument");
    return NUSIF_ERR_ARG;
  }
  char line[1024];
  snprintf(line, sizeof(line), "%s %s ", key, value);
  apply_line(param, line);
  return has_error() ? NUSIF_ERR_ARG : NUSIF_OK;
}

}  // extern "C"

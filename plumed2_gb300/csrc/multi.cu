// multi.cu -- many COORDINATION actions over one shared system in one launch.
#include "coordgpu.h"
#include "launch.h"

#include <string>
#include <vector>

struct coord_multi {
  std::vector<coord_ctx *> ctxs;
  int64_t n_atoms = 0;
  std::string err;
  bool graph = false;
};

extern "C" {

int coord_multi_create(coord_ctx *const *ctxs, int n_actions, int64_t n_atoms, coord_multi **out) {
  if (!ctxs || n_actions < 1 || !out) return COORD_ERR_ARG;
  coord_multi *m = new coord_multi();
  m->ctxs.assign(ctxs, ctxs + n_actions);
  m->n_atoms = n_atoms;
  *out = m;
  return COORD_OK;
}

int coord_multi_destroy(coord_multi *m) {
  delete m;
  return COORD_OK;
}

int coord_multi_deriv_offset(const coord_multi *m, int, int64_t *, int64_t *) {
  return m ? COORD_ERR_UNSUPPORTED : COORD_ERR_ARG;
}

int coord_multi_forward_device(coord_multi *m, int, const double *, const double *, unsigned, double *, double *,
                               double *, void *) {
  if (!m) return COORD_ERR_ARG;
  m->err = "multi-action batches are not built yet";
  return COORD_ERR_UNSUPPORTED;
}

int coord_multi_use_graph(coord_multi *m, int enable) {
  if (!m) return COORD_ERR_ARG;
  m->graph = enable != 0;
  return COORD_OK;
}

const char *coord_multi_last_error(const coord_multi *m) { return m ? m->err.c_str() : "null batch"; }
}

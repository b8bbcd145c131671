// C ABI of the Gaussian-atom Radon engine (declared in include/gauss_radon.h).
#include <new>
#include <vector>

#include "gr_kernels.cuh"
#include "gauss_radon.h"

namespace {

using namespace gr;

bool to_internal(const gr_atoms *a, const gr_geometry *g, Atoms &at, Geom &ge,
                 int *status) {
  *status = GR_ERR_ARG;
  if (!a || !g) return false;
  if (g->kdet != 1 && g->kdet != 2) return false;
  if (a->n_atoms < 0 || g->n_angles < 1 || !g->frames) return false;
  if (a->n_atoms > 0 && (!a->I || !a->x || !a->r)) return false;
  for (int k = 0; k < g->kdet; ++k) {
    if (g->n_det[k] < 1 || !g->det[k]) return false;
    if (!(g->det_inv_step[k] > 0.f)) {
      *status = GR_ERR_SHAPE;
      return false;
    }
  }
  at.n = a->n_atoms;
  at.I = a->I;
  at.x = a->x;
  at.r = a->r;
  at.r_iso = a->r_iso ? 1 : 0;
  at.order = a->order;
  ge.K = g->kdet;
  ge.n_angles = g->n_angles;
  ge.frames = g->frames;
  for (int k = 0; k < kMaxK; ++k) {
    const bool use = k < g->kdet;
    ge.ax[k].coords = use ? g->det[k] : nullptr;
    ge.ax[k].n = use ? g->n_det[k] : 1;
    ge.ax[k].first = use ? g->det_first[k] : 0.f;
    ge.ax[k].inv_step = use ? g->det_inv_step[k] : 1.f;
  }
  *status = GR_OK;
  return true;
}

// A batch member as the kernels' problem descriptor (buffers and atoms; the
// launch shapes are set by batch_create).
bool batch_member(const gr_batch_member &m, BatchProb &p) {
  int st;
  Geom g2;
  if (!to_internal(&m.cur, &m.geom, p.cur, p.g, &st)) return false;
  if (!to_internal(&m.trial, &m.geom, p.trial, g2, &st)) return false;
  if (p.g.K != 1 || p.cur.order || p.trial.order || !m.data || !m.fields || !m.loss_cur ||
      !m.loss_trial || !m.theta || !m.theta_trial || !m.lam || !m.step || !m.f || !m.g || !m.H ||
      !m.hist || !m.hist_acc || !m.counter || m.hist_len < 1 || m.max_iter < 1 ||
      !(m.tol >= 0.0))
    return false;
  p.out = ProjOut{nullptr, kEpiL2, m.data, 0.f, m.fields, nullptr, nullptr, 0};
  p.loss_cur = m.loss_cur;
  p.loss_trial = m.loss_trial;
  p.dout = DerivOut{m.f, m.g, m.H};
  p.theta = m.theta;
  p.theta_trial = m.theta_trial;
  p.lam = m.lam;
  p.step = m.step;
  p.hist = m.hist;
  p.hist_acc = m.hist_acc;
  p.counter = m.counter;
  p.hist_len = m.hist_len;
  p.max_iter = m.max_iter;
  p.tol = m.tol;
  p.lam_min = m.lam_min;
  p.lam_max = m.lam_max;
  return true;
}

}  // namespace

extern "C" {

size_t gr_batch_workspace_bytes(const gr_batch_member *members, int n) {
  if (!members || n < 1) return 0;
  std::vector<BatchProb> probs(n);
  for (int i = 0; i < n; ++i)
    if (!batch_member(members[i], probs[i])) return 0;
  return batch_workspace_bytes(probs.data(), n);
}

int gr_batch_create(const gr_batch_member *members, int n, void *ws, size_t ws_bytes,
                    int max_reject, void *stream, void **batch) {
  if (!members || n < 1 || !batch) return GR_ERR_ARG;
  *batch = nullptr;
  std::vector<BatchProb> probs(n);
  for (int i = 0; i < n; ++i)
    if (!batch_member(members[i], probs[i])) return GR_ERR_ARG;
  Batch *b = nullptr;
  const int rc = batch_create(probs.data(), n, ws, ws_bytes, max_reject,
                              static_cast<cudaStream_t>(stream), &b);
  *batch = b;
  return rc;
}

int gr_version(void) { return 10000; }

int gr_preload(void) {
  const int bad = preload_project() + preload_derivs() + preload_update() + preload_loop() +
                  preload_moments() + preload_reg() + preload_volume();
  return bad ? GR_ERR_LAUNCH : GR_OK;
}

const char *gr_status_string(int status) {
  switch (status) {
    case GR_OK: return "ok";
    case GR_ERR_ARG: return "invalid argument";
    case GR_ERR_WORKSPACE: return "workspace missing or too small";
    case GR_ERR_LAUNCH: return "CUDA launch or runtime error";
    case GR_ERR_SHAPE: return "unsupported geometry";
    case GR_ERR_TOO_LARGE: return "problem exceeds the 4 MiB built-in scratch of gr_radproj_noalloc";
    default: return "unknown status";
  }
}

static size_t workspace_bytes_impl(int op, const gr_atoms *atoms, const gr_geometry *geom,
                                   const Tuning &t) {
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return 0;
  const int D1 = g.K == 2 ? g.ax[1].n : 1;
  if (op == GR_OP_PROJECT)
    return project_workspace_bytes(g.K, at.n, g.n_angles, g.ax[0].n, D1, t);
  if (op == GR_OP_DERIVS_1 || op == GR_OP_DERIVS_2)
    return derivs_workspace_bytes(g.K, at.n, g.n_angles, op == GR_OP_DERIVS_1 ? 1 : 2, t);
  if (op == GR_OP_ATOM_STEP) return align_up((size_t)g.n_angles * sizeof(double));
  return 0;
}

size_t gr_workspace_bytes(int op, const gr_atoms *atoms, const gr_geometry *geom) {
  return workspace_bytes_impl(op, atoms, geom, g_tuning);
}

static int radproj_impl(const gr_atoms *atoms, const gr_geometry *geom, float *R,
                        void *workspace, size_t workspace_bytes, void *stream, int psf,
                        const Tuning &t = g_tuning) {
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return st;
  if (!R) return GR_ERR_ARG;
  ProjOut o{};
  o.R = R;
  o.epilogue = kEpiNone;
  o.psf = psf;
  return launch_project(at, g, o, nullptr, workspace, workspace_bytes,
                        static_cast<cudaStream_t>(stream), t);
}

int gr_radproj(const gr_atoms *atoms, const gr_geometry *geom, float *R,
               void *workspace, size_t workspace_bytes, void *stream) {
  return radproj_impl(atoms, geom, R, workspace, workspace_bytes, stream, 0);
}

int gr_psf_radproj(const gr_atoms *atoms, const gr_geometry *geom, float *R,
                   void *workspace, size_t workspace_bytes, void *stream) {
  return radproj_impl(atoms, geom, R, workspace, workspace_bytes, stream, 1);
}

static int fit_forward_impl(const gr_atoms *atoms, const gr_geometry *geom, int fit,
                            const float *data, float background, float *R, float *alpha,
                            float *beta, double *loss, void *workspace,
                            size_t workspace_bytes, void *stream, int psf,
                            const Tuning &t = g_tuning, int empty_mode = kEmptyNone,
                            double *empty_loss = nullptr) {
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return st;
  if (fit != GR_FIT_NONE && fit != GR_FIT_L2 && fit != GR_FIT_KL) return GR_ERR_ARG;
  if (fit != GR_FIT_NONE && !data) return GR_ERR_ARG;
  if (fit == GR_FIT_KL && !(background > 0.f)) return GR_ERR_ARG;
  if (fit == GR_FIT_NONE && (!R || loss)) return GR_ERR_ARG;
  ProjOut o{};
  o.R = R;
  o.epilogue = fit == GR_FIT_L2 ? kEpiL2 : fit == GR_FIT_KL ? kEpiKL : kEpiNone;
  o.data = data;
  o.bg = background;
  o.alpha = alpha;
  o.beta = beta;
  o.psf = psf;
  o.empty_mode = empty_mode;
  o.empty_loss = empty_loss;
  if (empty_mode != kEmptyNone && (g.K != 2 || psf || R || fit == GR_FIT_NONE || !empty_loss))
    return GR_ERR_ARG;
  return launch_project(at, g, o, loss, workspace, workspace_bytes,
                        static_cast<cudaStream_t>(stream), t);
}

int gr_fit_forward(const gr_atoms *atoms, const gr_geometry *geom, int fit,
                   const float *data, float background, float *R, float *alpha,
                   float *beta, double *loss, void *workspace,
                   size_t workspace_bytes, void *stream) {
  return fit_forward_impl(atoms, geom, fit, data, background, R, alpha, beta, loss,
                          workspace, workspace_bytes, stream, 0);
}

int gr_psf_fit_forward(const gr_atoms *atoms, const gr_geometry *geom, int fit,
                       const float *data, float background, float *R, float *alpha,
                       float *beta, double *loss, void *workspace,
                       size_t workspace_bytes, void *stream) {
  return fit_forward_impl(atoms, geom, fit, data, background, R, alpha, beta, loss,
                          workspace, workspace_bytes, stream, 1);
}

static int atom_derivs_impl(const gr_atoms *atoms, const gr_geometry *geom, int mode,
                            const float *field, const float *beta_field, float beta_const,
                            int order, double *f, double *g_out, double *H, void *workspace,
                            size_t workspace_bytes, void *stream, int psf,
                            const Tuning &t = g_tuning) {
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return st;
  if (mode != GR_MODE_FIELD && mode != GR_MODE_L2_ATOM && mode != GR_MODE_INNER)
    return GR_ERR_ARG;
  if (order != 1 && order != 2) return GR_ERR_ARG;
  if (!field || !f || !g_out || (order == 2 && !H)) return GR_ERR_ARG;
  DerivIn in{};
  in.mode = mode;
  in.order = order;
  in.alpha = field;
  in.beta = mode == GR_MODE_FIELD ? beta_field : nullptr;
  in.beta_const = mode == GR_MODE_FIELD ? beta_const : (mode == GR_MODE_L2_ATOM ? 1.f : 0.f);
  in.psf = psf;
  DerivOut out{f, g_out, H};
  return launch_derivs(at, g, in, out, workspace, workspace_bytes,
                       static_cast<cudaStream_t>(stream), t);
}

int gr_atom_derivs(const gr_atoms *atoms, const gr_geometry *geom, int mode,
                   const float *field, const float *beta_field, float beta_const,
                   int order, double *f, double *g_out, double *H, void *workspace,
                   size_t workspace_bytes, void *stream) {
  return atom_derivs_impl(atoms, geom, mode, field, beta_field, beta_const, order, f, g_out,
                          H, workspace, workspace_bytes, stream, 0);
}

int gr_psf_atom_derivs(const gr_atoms *atoms, const gr_geometry *geom, int mode,
                       const float *field, const float *beta_field, float beta_const,
                       int order, double *f, double *g_out, double *H, void *workspace,
                       size_t workspace_bytes, void *stream) {
  return atom_derivs_impl(atoms, geom, mode, field, beta_field, beta_const, order, f, g_out,
                          H, workspace, workspace_bytes, stream, 1);
}

int gr_atom_step(const gr_atoms *old_atom, const gr_atoms *new_atom,
                 const gr_geometry *geom, int fit, int apply, float *R,
                 const float *data, float background, float *alpha, float *beta,
                 double *dloss, void *workspace, size_t workspace_bytes, void *stream) {
  Atoms ao, an;
  Geom g;
  int st;
  if (!to_internal(old_atom, geom, ao, g, &st)) return st;
  if (!to_internal(new_atom, geom, an, g, &st)) return st;
  if (ao.n != 1 || an.n != 1 || ao.r_iso != an.r_iso) return GR_ERR_ARG;
  if (fit != GR_FIT_L2 && fit != GR_FIT_KL) return GR_ERR_ARG;
  if (!R || !alpha || !data || (!apply && !dloss)) return GR_ERR_ARG;
  if (fit == GR_FIT_KL && !(background > 0.f)) return GR_ERR_ARG;
  return launch_atom_update(ao, an, g, fit == GR_FIT_L2 ? kEpiL2 : kEpiKL, apply ? 1 : 0,
                            R, data, background, alpha, beta, dloss, workspace,
                            workspace_bytes, static_cast<cudaStream_t>(stream));
}

int gr_newton_solve(int dim, int iso, int n_atoms, const double *g, const double *H,
                    const double *lam, const double *theta, const unsigned char *mask,
                    double *theta_new, double *step_norm, int *fail, float *I_new,
                    float *x_new, float *r_new, void *stream) {
  if ((dim != 2 && dim != 3) || n_atoms < 0) return GR_ERR_ARG;
  if (n_atoms > 0 && (!g || !H || !lam || !theta || !theta_new || !step_norm))
    return GR_ERR_ARG;
  if ((I_new || x_new || r_new) && !(I_new && x_new && r_new)) return GR_ERR_ARG;
  AtomOut ao{I_new, x_new, r_new};
  return launch_newton_solve(dim, iso ? 1 : 0, n_atoms, g, H, lam, theta, mask, theta_new,
                             step_norm, fail, ao, static_cast<cudaStream_t>(stream));
}

static int newton_accept_impl(int dim, int iso, int n_atoms, double *loss_cur,
                              const double *loss_trial, double *theta,
                              const double *theta_trial, double *lam, double lam_min,
                              double lam_max, float *I, float *x, float *r,
                              const float *I_trial, const float *x_trial,
                              const float *r_trial, double *hist, int *hist_accepted,
                              int *counter, int hist_len, FieldCopy fc, void *stream) {
  if ((dim != 2 && dim != 3) || n_atoms < 0 || !loss_cur || !loss_trial || !counter)
    return GR_ERR_ARG;
  if (n_atoms > 0 && (!theta || !theta_trial || !lam || !I || !x || !r || !I_trial ||
                      !x_trial || !r_trial))
    return GR_ERR_ARG;
  if (hist_len > 0 && (!hist || !hist_accepted)) return GR_ERR_ARG;
  const int pr = iso ? 1 : (dim == 2 ? 3 : 6);
  const int P = 1 + dim + pr;
  return launch_newton_accept(n_atoms, P, pr, dim, loss_cur, loss_trial, theta, theta_trial,
                              lam, lam_min, lam_max, AtomOut{I, x, r},
                              AtomIn{I_trial, x_trial, r_trial}, hist, hist_accepted,
                              counter, hist_len, fc, static_cast<cudaStream_t>(stream));
}

int gr_newton_accept(int dim, int iso, int n_atoms, double *loss_cur,
                     const double *loss_trial, double *theta, const double *theta_trial,
                     double *lam, double lam_min, double lam_max, float *I, float *x,
                     float *r, const float *I_trial, const float *x_trial,
                     const float *r_trial, double *hist, int *hist_accepted,
                     int *counter, int hist_len, void *stream) {
  return newton_accept_impl(dim, iso, n_atoms, loss_cur, loss_trial, theta, theta_trial, lam,
                            lam_min, lam_max, I, x, r, I_trial, x_trial, r_trial, hist,
                            hist_accepted, counter, hist_len,
                            FieldCopy{nullptr, nullptr, nullptr, nullptr, 0}, stream);
}

int gr_newton_accept_fields(int dim, int iso, int n_atoms, double *loss_cur,
                            const double *loss_trial, double *theta,
                            const double *theta_trial, double *lam, double lam_min,
                            double lam_max, float *I, float *x, float *r,
                            const float *I_trial, const float *x_trial, const float *r_trial,
                            double *hist, int *hist_accepted, int *counter, int hist_len,
                            const float *alpha_trial, float *alpha, const float *beta_trial,
                            float *beta, size_t n_cells, void *stream) {
  if (!alpha_trial || !alpha || (beta && !beta_trial)) return GR_ERR_ARG;
  return newton_accept_impl(dim, iso, n_atoms, loss_cur, loss_trial, theta, theta_trial, lam,
                            lam_min, lam_max, I, x, r, I_trial, x_trial, r_trial, hist,
                            hist_accepted, counter, hist_len,
                            FieldCopy{alpha_trial, alpha, beta_trial, beta, n_cells}, stream);
}

static int volproj_impl(const gr_atoms *atoms, int dim, const int *n_vox,
                        const float *const *coords, float *u, void *stream, int psf,
                        float s) {
  if (!atoms || !n_vox || !coords || !u || (dim != 2 && dim != 3)) return GR_ERR_ARG;
  if (atoms->n_atoms < 0 || (atoms->n_atoms > 0 && (!atoms->I || !atoms->x || !atoms->r)))
    return GR_ERR_ARG;
  for (int k = 0; k < dim; ++k)
    if (n_vox[k] < 1 || !coords[k]) return GR_ERR_ARG;
  Atoms at;
  at.n = atoms->n_atoms;
  at.I = atoms->I;
  at.x = atoms->x;
  at.r = atoms->r;
  at.r_iso = atoms->r_iso ? 1 : 0;
  at.order = nullptr;
  return launch_volproj(at, dim, n_vox, coords, u, psf, s, static_cast<cudaStream_t>(stream));
}

int gr_volproj(const gr_atoms *atoms, int dim, const int *n_vox, const float *const *coords,
               float *u, void *stream) {
  return volproj_impl(atoms, dim, n_vox, coords, u, stream, 0, 0.f);
}

int gr_psf_volproj(const gr_atoms *atoms, int dim, const int *n_vox,
                   const float *const *coords, float voxel_half_width, float *u,
                   void *stream) {
  if (!(voxel_half_width > 0.f)) return GR_ERR_ARG;
  return volproj_impl(atoms, dim, n_vox, coords, u, stream, 1, voxel_half_width);
}

int gr_count_support(const gr_atoms *atoms, const gr_geometry *geom,
                     unsigned long long *count, void *stream) {
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return st;
  if (!count) return GR_ERR_ARG;
  return launch_count(at, g, count, static_cast<cudaStream_t>(stream));
}

int gr_probe_ex2(int blocks, int threads, int iters, float *sink, void *stream) {
  if (!sink) return GR_ERR_ARG;
  return launch_ex2_probe(blocks, threads, iters, sink,
                          static_cast<cudaStream_t>(stream));
}

unsigned long long gr_launch_count(void) { return g_launches.load(); }

int gr_sino_moments(const gr_geometry *geom, const float *res, const float *rr, float t,
                    float scale, double *S0, double *S1, double *S2, void *stream) {
  gr_atoms none = {};
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(&none, geom, at, g, &st)) return st;
  return launch_moments(g, res, rr, t, scale, S0, S1, S2, static_cast<cudaStream_t>(stream));
}

int gr_accept_fields(const double *loss_cur, const double *loss_trial, const float *alpha_trial,
                     float *alpha, const float *beta_trial, float *beta, size_t n_cells,
                     void *stream) {
  return launch_accept_fields(loss_cur, loss_trial, alpha_trial, alpha, beta_trial, beta, n_cells,
                              static_cast<cudaStream_t>(stream));
}

int gr_kernel_timer(int which, int enable) { return gr::timer_enable(which, enable); }

int gr_kernel_timer_read(int which, double *total_ms, int *launches) {
  return gr::timer_read(which, total_ms, launches);
}

int gr_set_tuning(int key, int value) { return tuning_set(g_tuning, key, value); }

int gr_get_tuning(int key) { return tuning_get(g_tuning, key); }

// ---- plans: a schedule (Tuning) owned by the caller ------------------------
struct gr_plan {
  gr::Tuning t;
  int op;
  int kdet, n_atoms, n_angles, n_det[2];
};

int gr_plan_create(int op, const gr_atoms *atoms, const gr_geometry *geom, gr_plan **plan) {
  if (!plan) return GR_ERR_ARG;
  *plan = nullptr;
  if (op != GR_OP_PROJECT && op != GR_OP_DERIVS_1 && op != GR_OP_DERIVS_2) return GR_ERR_ARG;
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(atoms, geom, at, g, &st)) return st;
  gr_plan *p = new (std::nothrow) gr_plan;
  if (!p) return GR_ERR_ARG;
  p->t = g_tuning;
  p->op = op;
  p->kdet = g.K;
  p->n_atoms = at.n;
  p->n_angles = g.n_angles;
  p->n_det[0] = g.ax[0].n;
  p->n_det[1] = g.K == 2 ? g.ax[1].n : 1;
  *plan = p;
  return GR_OK;
}

int gr_plan_destroy(gr_plan *plan) {
  delete plan;
  return GR_OK;
}

int gr_plan_set(gr_plan *plan, int key, int value) {
  return plan ? tuning_set(plan->t, key, value) : GR_ERR_ARG;
}

int gr_plan_get(const gr_plan *plan, int key) { return plan ? tuning_get(plan->t, key) : -1; }

size_t gr_plan_workspace_bytes(const gr_plan *plan, int op, const gr_atoms *atoms,
                               const gr_geometry *geom) {
  return plan ? workspace_bytes_impl(op, atoms, geom, plan->t) : 0;
}

int gr_radproj_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                    float *R, void *workspace, size_t workspace_bytes, void *stream) {
  if (!plan) return GR_ERR_ARG;
  return radproj_impl(atoms, geom, R, workspace, workspace_bytes, stream, 0, plan->t);
}

int gr_fit_forward_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int fit, const float *data, float background, float *R, float *alpha,
                        float *beta, double *loss, void *workspace, size_t workspace_bytes,
                        void *stream) {
  if (!plan) return GR_ERR_ARG;
  return fit_forward_impl(atoms, geom, fit, data, background, R, alpha, beta, loss, workspace,
                          workspace_bytes, stream, 0, plan->t);
}

int gr_fit_items(const gr_plan *plan, const gr_geometry *geom, size_t *n_items) {
  if (!n_items) return GR_ERR_ARG;
  *n_items = 0;
  gr_atoms none{};
  Atoms at;
  Geom g;
  int st;
  if (!to_internal(&none, geom, at, g, &st)) return st;
  *n_items = project_skip_items(g, 0, plan ? plan->t : g_tuning);
  return GR_OK;
}

// the record of empty items must have one entry per item of the forward's
// tiling: checked on the host, before any launch
static bool empty_record_fits(const gr_plan *plan, const gr_geometry *geom, size_t n_empty) {
  size_t n = 0;
  return gr_fit_items(plan, geom, &n) == GR_OK && n > 0 && n == n_empty;
}

int gr_fit_empty_loss(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                      int fit, const float *data, float background, double *empty_loss,
                      size_t n_empty, void *workspace, size_t workspace_bytes, void *stream) {
  if (!empty_record_fits(plan, geom, n_empty)) return GR_ERR_ARG;
  return fit_forward_impl(atoms, geom, fit, data, background, nullptr, nullptr, nullptr, nullptr,
                          workspace, workspace_bytes, stream, 0, plan ? plan->t : g_tuning,
                          kEmptyRecord, empty_loss);
}

int gr_fit_forward_skip(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int fit, const float *data, float background, float *alpha,
                        float *beta, double *loss, const double *empty_loss, size_t n_empty,
                        void *workspace, size_t workspace_bytes, void *stream) {
  if (!empty_record_fits(plan, geom, n_empty)) return GR_ERR_ARG;
  return fit_forward_impl(atoms, geom, fit, data, background, nullptr, alpha, beta, loss,
                          workspace, workspace_bytes, stream, 0, plan ? plan->t : g_tuning,
                          kEmptySkip, const_cast<double *>(empty_loss));
}

int gr_atom_derivs_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int mode, const float *field, const float *beta_field,
                        float beta_const, int order, double *f, double *g, double *H,
                        void *workspace, size_t workspace_bytes, void *stream) {
  if (!plan) return GR_ERR_ARG;
  return atom_derivs_impl(atoms, geom, mode, field, beta_field, beta_const, order, f, g, H,
                          workspace, workspace_bytes, stream, 0, plan->t);
}

}  // extern "C"

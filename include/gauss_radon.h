/*
 * gauss_radon.h -- C ABI of the GB300 Gaussian-atom Radon engine.
 *
 * Plain C types only: device pointers, sizes and a CUDA stream handle passed
 * as void* (a cudaStream_t; NULL is the legacy default stream).  Every entry
 * point is asynchronous on that stream, returns a status code (GR_OK = 0,
 * negative on error) and never aborts the process.
 *
 * The entry points replace the four callables of the reference's kernel
 * module, the plug-in point that GaussTomo._getOps returns
 * (GaussDictCode/atomFuncs.py:106-113):
 *   RadProj(atom, Rad, R)               -> gr_radproj
 *   L2derivs_RadProj(atom, Rad, C, ord) -> gr_atom_derivs(GR_MODE_L2_ATOM)
 *   derivs_RadProj(atom, Rad, C, ord)   -> gr_atom_derivs(GR_MODE_INNER)
 * and add the fused forms the fitting loops need (gr_fit_forward and
 * gr_atom_derivs(GR_MODE_FIELD)), which compute, for every atom at once, what
 * the reference obtains with one L2derivs_RadProj launch per atom
 * (NewtonGaussian.py:59-60).
 *
 * Conventions (reference GaussDictCode/bin/NewtonBases2D.py:17-72,
 * GaussDictCode/bin/NewtonBases.py:239-310):
 *   atom j = (I[j], x[j*d .. j*d+d-1], r[j*P_r ..]); d = kdet + 1;
 *   r packed upper-triangular: 2D [r00 r11 r01], 3D [r00 r11 r22 r01 r12 r02],
 *   or one radius per atom when r_iso != 0;
 *   derivative order [I, x_0..x_{d-1}, r_0..r_{P_r-1}] (isotropic: [I, x, s]).
 *   Sinograms are float32, C order, shape (n_angles, n_det[0]) for kdet = 1 or
 *   (n_angles, n_det[0], n_det[1]) for kdet = 2.
 */
#ifndef GAUSS_RADON_H
#define GAUSS_RADON_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GR_OK = 0,
    GR_ERR_ARG = -1,       /* invalid argument (null pointer, bad size) */
    GR_ERR_WORKSPACE = -2, /* workspace missing or too small */
    GR_ERR_LAUNCH = -3,    /* CUDA launch or runtime error */
    GR_ERR_SHAPE = -4,     /* geometry not supported (e.g. decreasing grid) */
    GR_ERR_TOO_LARGE = -5  /* problem needs more than the built-in scratch */
};

/* Atoms in device memory (float32).  order (nullable): a permutation of
 * 0..n_atoms-1 giving the order in which the derivative kernels visit the
 * atoms (spatially clustered orders read the weight fields with better cache
 * locality); outputs stay indexed by atom and do not depend on it. */
typedef struct {
    int n_atoms;
    const float *I;   /* (n_atoms) */
    const float *x;   /* (n_atoms, d) */
    const float *r;   /* (n_atoms, P_r) or (n_atoms) when r_iso */
    int r_iso;
    const int *order; /* (n_atoms) or NULL */
} gr_atoms;

/*
 * Projection geometry in device memory.  frames holds one record per angle:
 *   kdet = 1 (2D):  T(2) w0(2) wt0(2) wl0(2)                          -> 8 floats
 *   kdet = 2 (3D):  T(3) w0(3) w1(3) wt0(3) wt1(3) wl0(3) wl1(3) pad(3) -> 24 floats
 * T is the ray direction (ProjSpace.orientations), w0/w1 the detector axes
 * (ProjSpace.ortho), wt0/wt1 the first kdet rows of inverse([w0 w1 T])
 * rounded to float (equal to w0/w1 for orthonormal frames) and wl0/wl1 the
 * rounding residues (row - wt, in float), from which the kernels form each
 * atom's projection centre to ~1e-14.  The 2.5D single-axis tilt of the
 * reference (NewtonBases.py:685-688) is the 3D case with T = (T0, T1, 0),
 * w0 = (w00, w01, 0), w1 = (0, 0, 1).
 * det[k] are the detector cell centres (ProjSpace.detector), uniformly spaced
 * and increasing; det_first[k] = det[k][0], det_inv_step[k] = 1/spacing.
 */
typedef struct {
    int kdet;
    int n_angles;
    const float *frames;
    int n_det[2];
    const float *det[2];
    float det_first[2];
    float det_inv_step[2];
} gr_geometry;

enum { GR_FIT_NONE = 0, GR_FIT_L2 = 1, GR_FIT_KL = 2 };
enum { GR_MODE_FIELD = 0, GR_MODE_L2_ATOM = 1, GR_MODE_INNER = 2 };
enum { GR_OP_PROJECT = 0, GR_OP_DERIVS_1 = 1, GR_OP_DERIVS_2 = 2, GR_OP_ATOM_STEP = 3 };

/* Library version (major*10000 + minor*100 + patch). */
int gr_version(void);

/* Loads the code of every kernel of the library on the current device now.
 * CUDA loads modules lazily by default, so without this a kernel's first
 * launch, or the first instantiation of a graph that holds it, pays the load
 * while the caller's other work waits (a serving process calls it once at
 * start).  No reference counterpart: the reference compiles its kernels on
 * first call instead.  GR_ERR_LAUNCH if a kernel cannot be loaded. */
int gr_preload(void);

/* Static description of a status code. */
const char *gr_status_string(int status);

/*
 * Device workspace (bytes) an operation needs; the caller allocates it
 * (256-byte aligned) and may reuse it across calls on the same stream.
 */
size_t gr_workspace_bytes(int op, const gr_atoms *atoms, const gr_geometry *geom);

/*
 * Forward projection: R = sum over atoms of I / |r T| exp(-30 m), m <= 1.
 * Replaces RadProj (GaussDictCode/bin/NewtonBases2D.py:274-296,
 * GaussDictCode/bin/NewtonBases.py:714-756); R is written in full.
 */
int gr_radproj(const gr_atoms *atoms, const gr_geometry *geom, float *R,
               void *workspace, size_t workspace_bytes, void *stream);

/*
 * Forward projection fused with a data fit.
 *   GR_FIT_L2: alpha = R - data, *loss = 1/2 sum (R - data)^2
 *              (GaussDictCode/transport_loss.py:569-585).
 *   GR_FIT_KL: g = R + background, alpha = 1 - data/g, beta = data/g^2,
 *              *loss = sum data log(data/g) - data + g
 *              (KL_GaussRadon.py:52-54 with an explicit background).
 * R, alpha, beta and loss may each be NULL when not wanted; loss is one
 * double in device memory.
 */
int gr_fit_forward(const gr_atoms *atoms, const gr_geometry *geom, int fit,
                   const float *data, float background, float *R, float *alpha,
                   float *beta, double *loss, void *workspace,
                   size_t workspace_bytes, void *stream);

/*
 * Per-atom value, gradient and Hessian of a data fit, all atoms in one call.
 *   GR_MODE_INNER   (field = C): f = <R_j, C>, g = <dR_j, C>, H = <d2R_j, C>
 *                   (derivs_RadProj, NewtonBases2D.py:415-515,
 *                    NewtonBases.py:954-1069).
 *   GR_MODE_L2_ATOM (field = C): f = 1/2 |R_j - C|^2 with its gradient and
 *                   Hessian (L2derivs_RadProj, NewtonBases2D.py:299-401,
 *                   NewtonBases.py:759-870), each atom fitted alone to C.
 *   GR_MODE_FIELD   (field = alpha, beta_field or beta_const = beta):
 *                   g = sum alpha dR_j, H = sum beta dR_j dR_j^T + alpha d2R_j,
 *                   f = 0.  With alpha = R - data, beta = 1 this is the
 *                   reference's L2derivs_RadProj(atom_j, data + R_j - R) for
 *                   every j; with the KL fields of gr_fit_forward it is the
 *                   KL fit's gradient and Gauss-Newton-plus-curvature Hessian.
 * order 1: f and g; order 2: f, g and H.  Outputs are float64 in device
 * memory: f (n_atoms), g (n_atoms, P), H (n_atoms, P, P) with P = 1 + d + P_r
 * (isotropic: P = 2 + d, exact chain rule of r = (s, .., s, 0, ..)).
 */
int gr_atom_derivs(const gr_atoms *atoms, const gr_geometry *geom, int mode,
                   const float *field, const float *beta_field, float beta_const,
                   int order, double *f, double *g, double *H, void *workspace,
                   size_t workspace_bytes, void *stream);

/*
 * Render atoms on a voxel grid: u[i0, i1(, i2)] = sum_j I_j sqrt(30/pi)
 * exp(-30 |r_j (y - x_j)|^2) where |r_j (y - x_j)| <= 1, y = (coords[0][i0],
 * coords[1][i1](, coords[2][i2])).  Replaces VolProj / __VolProj
 * (GaussDictCode/bin/NewtonBases2D.py:252-271, NewtonBases.py:691-711).
 * dim 2 or 3; n_vox[k] voxels along axis k; coordinate vectors monotone;
 * u float32 C order, written in full.  No workspace.
 */
int gr_volproj(const gr_atoms *atoms, int dim, const int *n_vox, const float *const *coords,
               float *u, void *stream);

/*
 * Pixel-integrated ("point spread") operator: the same calls for the
 * single-particle kernel module (GaussDictCode/bin/point_spread_functions.py,
 * selected by SingleParticleGaussTomo._getOps, atomFuncs.py:168-172): RadProj
 * (:371), L2derivs_RadProj (:1077), derivs_RadProj (:1314), VolProj (:168).
 * A cell's value is the integral of the projection over the square cell
 * (half-width s = spacing/2 of detector axis 0) by the reference's 11-point
 * (2D) / 11 x 11 (3D) rule over the cell clipped to +-1/min(diag r) around the
 * atom; cells holding a whole atom get its total mass (with zero
 * derivatives, as the reference).  Arguments and outputs as gr_radproj,
 * gr_fit_forward and gr_atom_derivs.  gr_psf_volproj integrates over voxels
 * of half-width voxel_half_width (11^dim rule, __if2/__if3 :425-495).
 */
int gr_psf_radproj(const gr_atoms *atoms, const gr_geometry *geom, float *R,
                   void *workspace, size_t workspace_bytes, void *stream);
int gr_psf_fit_forward(const gr_atoms *atoms, const gr_geometry *geom, int fit,
                       const float *data, float background, float *R, float *alpha,
                       float *beta, double *loss, void *workspace,
                       size_t workspace_bytes, void *stream);
int gr_psf_atom_derivs(const gr_atoms *atoms, const gr_geometry *geom, int mode,
                       const float *field, const float *beta_field, float beta_const,
                       int order, double *f, double *g, double *H, void *workspace,
                       size_t workspace_bytes, void *stream);
int gr_psf_volproj(const gr_atoms *atoms, int dim, const int *n_vox,
                   const float *const *coords, float voxel_half_width, float *u,
                   void *stream);

/*
 * One atom of a fit moves from old_atom to new_atom (both n_atoms = 1, same
 * r_iso).  The sinogram R changes by R(new) - R(old) inside the union of the
 * two supports.  apply = 0 (trial): *dloss = change of the data fit (L2:
 * 1/2|R - data|^2, KL as in gr_fit_forward), nothing written.  apply = 1:
 * R, alpha (and beta for KL) are updated there.  This is the per-atom step
 * of the reference's fitting loops (GD_lib._step, GD_lib.py:492-536) without
 * its full re-projection and restore.
 */
int gr_atom_step(const gr_atoms *old_atom, const gr_atoms *new_atom,
                 const gr_geometry *geom, int fit, int apply, float *R,
                 const float *data, float background, float *alpha, float *beta,
                 double *dloss, void *workspace, size_t workspace_bytes, void *stream);

/*
 * Batched damped Newton step, float64, all atoms in one call: solve
 * (H_j + lam_j 1) d = -g_j (Cholesky; partial-pivoting LU when the damped
 * block is indefinite, as numpy.linalg.solve in NewtonGaussian.py:74), then
 * theta_new = theta + d with the reference's clamps: I >= 0 and sign flips
 * keeping diag(r) >= 0 (GD_lib.py:504-522).  theta (n, P) is [I, x, r] per
 * atom; mask (nullable) freezes atoms with mask[j] == 0; step_norm[j] = |d|;
 * fail (nullable) flags singular blocks (their parameters are kept).
 * I_new/x_new/r_new (all or none): the new parameters also as float32 atom
 * arrays, ready for gr_fit_forward.
 */
int gr_newton_solve(int dim, int iso, int n_atoms, const double *g, const double *H,
                    const double *lam, const double *theta, const unsigned char *mask,
                    double *theta_new, double *step_norm, int *fail, float *I_new,
                    float *x_new, float *r_new, void *stream);

/*
 * Device-side accept test of a batched Newton trial, so that a whole
 * iteration (gr_fit_forward, gr_atom_derivs, gr_newton_solve, gr_fit_forward
 * of the trial, gr_newton_accept) runs without a host round trip and can be
 * replayed as a CUDA graph.  If *loss_trial <= *loss_cur: theta, the float32
 * atoms and *loss_cur take the trial's values and lam halves; else lam grows
 * tenfold; lam is clamped to [lam_min, lam_max].  hist[*counter] = *loss_cur
 * and hist_accepted[*counter] = accepted (when *counter < hist_len), then
 * ++*counter.  The same backtracking rule as the reference's Newton loop
 * (NewtonGaussian.py:81-92), applied to all atoms at once.
 */
int gr_newton_accept(int dim, int iso, int n_atoms, double *loss_cur,
                     const double *loss_trial, double *theta, const double *theta_trial,
                     double *lam, double lam_min, double lam_max, float *I, float *x,
                     float *r, const float *I_trial, const float *x_trial,
                     const float *r_trial, double *hist, int *hist_accepted,
                     int *counter, int hist_len, void *stream);

/* gr_newton_accept plus, when the trial is accepted, the adoption of the
 * trial's fit fields (alpha_trial -> alpha and, for KL, beta_trial -> beta;
 * n_cells each), in one launch: the accept/reject step of the device-resident
 * fitting loop, where the trial's forward wrote its fields so that the next
 * iteration needs no projection of the current atoms.  Equivalent to
 * gr_newton_accept followed by gr_accept_fields.  GR_ERR_ARG as
 * gr_newton_accept, or for missing field pointers. */
int gr_newton_accept_fields(int dim, int iso, int n_atoms, double *loss_cur,
                            const double *loss_trial, double *theta,
                            const double *theta_trial, double *lam, double lam_min,
                            double lam_max, float *I, float *x, float *r,
                            const float *I_trial, const float *x_trial, const float *r_trial,
                            double *hist, int *hist_accepted, int *counter, int hist_len,
                            const float *alpha_trial, float *alpha, const float *beta_trial,
                            float *beta, size_t n_cells, void *stream);

/*
 * Measurement helpers (no counterpart in the reference, which has no
 * benchmarks).
 * gr_count_support: *count (device, one unsigned 64-bit integer) = number of
 *   (atom, angle, cell) triples inside the basis support m <= 1, the exact
 *   count of useful atom-cell evaluations of one projection.
 * gr_probe_ex2: runs blocks x threads x iters x 8 independent ex2.approx
 *   operations (sink: one device float, not written in practice); timing it
 *   gives the special-function-unit roofline of the GPU.
 * gr_launch_count: number of kernels this library has launched so far in
 *   the process (host-side counter).
 */
int gr_count_support(const gr_atoms *atoms, const gr_geometry *geom,
                     unsigned long long *count, void *stream);
int gr_probe_ex2(int blocks, int threads, int iters, float *sink, void *stream);
unsigned long long gr_launch_count(void);

/*
 * Work-split knobs of the kernels, process-wide (no counterpart
 * in the reference).  GR_TUNE_DERIV_WARPS: about this many warps per
 * derivative launch (atoms x angle chunks; default 131072);
 * GR_TUNE_DERIV_MIN_ANGLES: at least this many angles per lane group in a
 * chunk (default 1); GR_TUNE_DERIV_ATOMS_PER_WARP: atoms sharing a warp, a
 * power of two up to 32, the other lanes taking further angles of the same
 * atoms (default 0: automatic, one atom per warp for Hessians and for series
 * of 1024 or more angles, else four).  GR_TUNE_PROJ_TILING: tiles of the
 * point-sampled 3D projection, 1 = 16 x 32 cells (default, more resident
 * warps), 2 = 32 x 32 (fewer atoms cut by tile edges), 3 = as 1; of the 2D
 * projection, 32, 64 and 128 cells (one, two or four per lane: wide
 * footprints are listed and staged for fewer tiles).
 * GR_TUNE_PROJ_SPLIT_CELLS: 3D problems with fewer detector cells over all
 * angles than this (default 4194304; 0 = never) split each tile's atoms over
 * the four warps of a block, which shortens the slowest tile when there are
 * too few tiles to fill the GPU.  GR_TUNE_DERIV_SPLIT_LANES: problems with
 * fewer (atom, angle) pairs than this split each pair's cells over 2, 4 or 8
 * lanes of the point-sampled derivative kernel (the largest split with
 * pairs x lanes <= value; default 65536; 0 = never).  GR_TUNE_DERIV_ONE_MB:
 * take enough angle chunks that every lane has at most one angle whenever the
 * chunk partials then fit in this many MB of workspace (default 1024; 0 =
 * keep GR_TUNE_DERIV_WARPS).  GR_TUNE_DERIV_WIDE_ROWS: 1 walks the rows of
 * the 3D Hessian (order 2) kernels in chunks of 8 cells instead of 4, which
 * keeps more field loads in flight when supports are many cells wide and
 * idles lanes when they are narrow (default 0; the serving tuner picks it
 * per class of requests).  GR_TUNE_DERIV_BLOCK_WARPS: warps per block of
 * the derivative kernels that give each lane at most one angle, 1 (default)
 * or 4; with one-warp blocks a finished warp frees its slot at once instead
 * of waiting for the slowest warp of its block (3D Hessians of the largest
 * served requests 458 -> 415 us, config 4's gradient 5 % faster; results are
 * bitwise the same).  Set them before
 * gr_workspace_bytes and keep them fixed while launches that used the old
 * values are in flight.  Results do not depend on them beyond FP rounding of
 * the derivative chunk and lane sums and of a split tile's combined cell sums (the
 * tiling leaves projections bitwise equal).  gr_set_tuning returns
 * GR_ERR_ARG for an unknown key or out-of-range value; gr_get_tuning returns
 * the current value (-1 for an unknown key).
 */
enum {
  GR_TUNE_DERIV_WARPS = 0,
  GR_TUNE_DERIV_MIN_ANGLES = 1,
  GR_TUNE_DERIV_ATOMS_PER_WARP = 2,
  GR_TUNE_PROJ_TILING = 3,
  GR_TUNE_PROJ_SPLIT_CELLS = 4,
  GR_TUNE_DERIV_SPLIT_LANES = 6,
  GR_TUNE_DERIV_ONE_MB = 7,
  GR_TUNE_DERIV_WIDE_ROWS = 8,
  GR_TUNE_DERIV_BLOCK_WARPS = 9
};
int gr_set_tuning(int key, int value);
int gr_get_tuning(int key);

/*
 * Plans: a schedule of the same knobs held by the caller instead of the
 * process-wide one, so that concurrent streams (a serving process fitting
 * problems of different shapes at once) each run the split and tiling tuned
 * for their shape class.  No reference counterpart: the reference's kernel
 * modules derive their launch configuration from each call's sizes
 * (NewtonBases2D.py:302-316) and keep no schedule.
 *   gr_plan_create: a plan for op (GR_OP_PROJECT, GR_OP_DERIVS_1/2) on
 *     problems shaped like atoms/geom (only their sizes are read), holding a
 *     copy of the current process-wide values; GR_ERR_ARG / GR_ERR_SHAPE as
 *     gr_workspace_bytes' argument checks.
 *   gr_plan_set / gr_plan_get: as gr_set_tuning / gr_get_tuning on the plan.
 *   gr_plan_workspace_bytes: gr_workspace_bytes under the plan's schedule.
 *   gr_radproj_plan, gr_fit_forward_plan, gr_atom_derivs_plan: gr_radproj,
 *     gr_fit_forward and gr_atom_derivs under the plan's schedule (any
 *     problem size; the workspace must hold gr_plan_workspace_bytes of it).
 * Results do not depend on the schedule beyond the FP rounding stated for
 * gr_set_tuning.  A plan may be used by several streams at once; destroy it
 * only when no launch made with it is still to be enqueued (launches
 * already enqueued hold their own copy of the schedule).
 */
typedef struct gr_plan gr_plan;
int gr_plan_create(int op, const gr_atoms *atoms, const gr_geometry *geom, gr_plan **plan);
int gr_plan_destroy(gr_plan *plan);
int gr_plan_set(gr_plan *plan, int key, int value);
int gr_plan_get(const gr_plan *plan, int key);
size_t gr_plan_workspace_bytes(const gr_plan *plan, int op, const gr_atoms *atoms,
                               const gr_geometry *geom);
int gr_radproj_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                    float *R, void *workspace, size_t workspace_bytes, void *stream);
int gr_fit_forward_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int fit, const float *data, float background, float *R, float *alpha,
                        float *beta, double *loss, void *workspace, size_t workspace_bytes,
                        void *stream);
int gr_atom_derivs_plan(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int mode, const float *field, const float *beta_field,
                        float beta_const, int order, double *f, double *g, double *H,
                        void *workspace, size_t workspace_bytes, void *stream);

/*
 * Forwards of a fit that reads its fields only where atoms are (no
 * counterpart in the reference, whose loop re-reads the whole sinogram per
 * atom): a damped-Newton loop reads alpha / beta only inside its atoms'
 * supports, which lie in the (angle, tile) items the forward's binning marks.
 * For the point-sampled 3D forward (kdet 2):
 *   gr_fit_items: the forward's items under the plan's tiling (plan NULL:
 *     the process-wide schedule); 0 for 2D geometries, which do not skip.
 *   gr_fit_empty_loss: each item's loss with no atom in it (R = 0: the data
 *     term alone, L2 or KL) into empty_loss[n_empty], computed under the
 *     schedule a forward of these atoms takes (only n_atoms is read), so it
 *     equals bitwise what that forward computes for an item no atom meets.
 *     Once per data sinogram.
 *   gr_fit_forward_skip: gr_fit_forward_plan without R, where an item that no
 *     atom meets takes its loss from empty_loss and keeps whatever its fields
 *     held: the loss is bitwise that of gr_fit_forward_plan, and so are the
 *     fields in every item an atom meets.
 * n_empty must equal gr_fit_items under the same plan (a record made under
 * another tiling does not fit).  GR_ERR_ARG for a 2D geometry, a missing
 * pointer, fit GR_FIT_NONE or another n_empty.
 */
int gr_fit_items(const gr_plan *plan, const gr_geometry *geom, size_t *n_items);
int gr_fit_empty_loss(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                      int fit, const float *data, float background, double *empty_loss,
                      size_t n_empty, void *workspace, size_t workspace_bytes, void *stream);
int gr_fit_forward_skip(const gr_plan *plan, const gr_atoms *atoms, const gr_geometry *geom,
                        int fit, const float *data, float background, float *alpha,
                        float *beta, double *loss, const double *empty_loss, size_t n_empty,
                        void *workspace, size_t workspace_bytes, void *stream);

/*
 * Per-angle detector moments of a sinogram, for the moment-matching initial
 * guess of a new atom.  Replaces the reference's MOM0 / MOM1 / MOM2
 * (KL_GaussRadon.py:227-253, :347-368), CPU loops inside its guess
 * doKL_ProjGDStep_iso (:57-121).  Over the target
 *     f = max(0, res)                          (rr == NULL)
 *     f = max(0, t res + (1 - t) scale rr)     (otherwise; the blend of the
 *                                                reference's iteration)
 * (res, rr: sinograms of geom's shape) it writes, in FP64 and a fixed order,
 *     S0[a] = sum f,  S1[a][i] = sum f p_i,  S2[a][i] = sum f p_i^2
 * for every angle a and detector axis i < kdet (p_i the cell coordinate).
 * GR_ERR_ARG for missing pointers or an invalid geometry.
 */
int gr_sino_moments(const gr_geometry *geom, const float *res, const float *rr, float t,
                    float scale, double *S0, double *S1, double *S2, void *stream);

/*
 * Per-atom regularisers of the fitting loops.  Replaces the regulariser
 * classes of GaussDictCode/regularisation.py (Joubert :41-107, Mass :110-208,
 * Volume :211-297, Radius :300-366, Iso :369-442), whose value, gradient and
 * Hessian the Newton loop adds to each atom's block (NewtonGaussian.py:59-66).
 * For every atom: value f[j], gradient g[j, P] and Hessian H[j, P, P] in the
 * parameter order [I, x, r] (P = 1 + dim + 3|6, or 2 + dim for isotropic
 * atoms), in FP64; written, or added to the arrays when accumulate != 0 (so
 * the call can follow gr_atom_derivs on the same outputs).  f and H may be
 * NULL.  kind and params (n_params <= 8):
 *   GR_REG_JOUBERT  (a, b, c, d, e): -a log I + b/2|x|^2 + c R - d log R - e,
 *                   R = prod(diag r) or s^dim; the reference's
 *                   Joubert(dim, intensity, location, radius) has a =
 *                   intensity, b = location, c = radius[1], d = radius[1]
 *                   radius[0], e = radius[0] radius[1] (1 - log radius[0]);
 *   GR_REG_MASS     (m, k, w): w (I V - m)^k, V = 1/prod(diag r) or s^dim;
 *   GR_REG_VOLUME   (v0, k, w): w |R - v0|^k, R = prod(diag r) or s^-dim
 *                   (the reference's r0 gives v0 = |r0|^dim);
 *   GR_REG_RADIUS   (r0, w, k): w sum (r_ii - r0)^-k (isotropic: dim (s - r0)^-k);
 *   GR_REG_ISO      (w): w/2 |off-diagonal r|^2.
 * Values outside the domain (log or power of a non-positive number) are
 * +inf, as in the reference.  Hessians are exact (the reference's Joubert has
 * none, its Volume Hessian cannot run, its Mass Hessian misses mixed r-r
 * terms).  GR_ERR_ARG for an unknown kind, dim not 2 or 3, or missing
 * pointers.
 */
enum { GR_REG_NULL = 0, GR_REG_JOUBERT = 1, GR_REG_MASS = 2, GR_REG_VOLUME = 3,
       GR_REG_RADIUS = 4, GR_REG_ISO = 5 };
int gr_regulariser(int kind, const double *params, int n_params, const gr_atoms *atoms, int dim,
                   double *f, double *g, double *H, int accumulate, void *stream);

/*
 * After gr_newton_accept: if the trial was accepted (loss_cur == loss_trial),
 * copy the trial's fit fields (from gr_fit_forward of the trial atoms) over
 * the current ones; otherwise do nothing.  With it a Newton iteration needs
 * one projection (of the trial) instead of two: the current atoms' fields
 * are either the accepted trial's or unchanged.  No counterpart in the
 * reference, whose host loop re-projects (NewtonGaussian.py:59-75).
 * beta / beta_trial may be NULL (L2 fits).
 */
int gr_accept_fields(const double *loss_cur, const double *loss_trial, const float *alpha_trial,
                     float *alpha, const float *beta_trial, float *beta, size_t n_cells,
                     void *stream);

/*
 * Device-resident fitting loop.  Replaces the host-driven iteration of the
 * reference's Newton loop (GaussDictCode/NewtonGaussian.py:18-109: a Python
 * loop over sweeps with a host decision per step) by one CUDA graph per
 * fitting problem whose WHILE conditional node repeats a captured iteration.
 *
 *   gr_fit_loop_begin(stream, guard, &loop)  creates the graph (a memset of
 *       the caller's device int *guard, then the WHILE node) and starts
 *       capturing `stream` into the loop body (thread-local capture mode);
 *   the caller then issues ONE iteration on `stream` (gr_fit_forward,
 *       gr_atom_derivs, gr_newton_solve, gr_fit_forward of the trial atoms,
 *       gr_newton_accept; no other stream, no host synchronisation, no
 *       allocation);
 *   inside that iteration, gr_fit_loop_gate_begin(loop, stream, hist_acc,
 *       counter, hist_len) ... gr_fit_loop_gate_end(loop, stream) may
 *       bracket the derivative evaluation of the current atoms: the work
 *       issued between them goes into the body of an IF node that runs
 *       unless the previous trial was rejected (hist_acc[counter - 1] == 0),
 *       whose atoms, fit fields and derivatives are unchanged, so the
 *       previous outputs stand bit for bit.  At most one gated part per
 *       loop; an unclosed one makes gr_fit_loop_end fail with GR_ERR_ARG;
 *   gr_fit_loop_end(loop, stream, hist, hist_acc, counter, hist_len,
 *       max_iter, max_reject, tol, guard_max, stop_flag) appends the stop
 *       test and ends the capture;
 *   gr_fit_loop_instantiate(loop) instantiates the graph (touches no
 *       stream).  The body runs again unless: counter >= max_iter; the last
 *       max_reject entries of hist_acc are 0; the last accepted iteration
 *       i >= 1 changed the loss by at most tol * |hist[i - 1]|; or the body
 *       ran guard_max times (a bound that holds whatever the buffers
 *       contain).  The reason is written to *stop_flag (device int,
 *       nullable): 1 iterations or guard, 2 rejects, 3 converged;
 *   gr_fit_loop_launch(loop, stream)  runs the whole fit (one graph launch);
 *   gr_fit_loop_destroy(loop)  (waits until the device is idle: destroy
 *       finished loops when no fit is running).
 *
 * The buffers captured in the body are used by every launch; the caller
 * keeps them alive until gr_fit_loop_destroy.  On a capture or instantiation
 * failure gr_fit_loop_end / gr_fit_loop_instantiate return GR_ERR_LAUNCH (the
 * loop can only be destroyed); gr_fit_loop_launch before a successful
 * instantiation returns GR_ERR_ARG.
 */
int gr_fit_loop_begin(void *stream, int *guard, void **loop);
int gr_fit_loop_end(void *loop, void *stream, const double *hist, const int *hist_acc,
                    const int *counter, int hist_len, int max_iter, int max_reject,
                    double tol, int guard_max, int *stop_flag);
int gr_fit_loop_gate_begin(void *loop, void *stream, const int *hist_acc, const int *counter,
                           int hist_len);
int gr_fit_loop_gate_end(void *loop, void *stream);
int gr_fit_loop_instantiate(void *loop);
int gr_fit_loop_launch(void *loop, void *stream);
int gr_fit_loop_destroy(void *loop);

/* ---- batches of small 2D fits ------------------------------------------
 * Several 2D L2 damped-Newton fits run as one device loop in which every
 * kernel of an iteration is one launch over a table of the problems (each
 * kernel maps its blocks to (problem, block of that problem) and runs the
 * block body of the problem's own launch, so every problem gets the results
 * of its own loop): the launches and graph nodes an iteration costs are
 * shared by the batch.  A problem leaves the batch when its own stop test
 * (as gr_fit_loop_end's) says so; the loop ends when none is left.
 * Replaces, for small problems, one gr_fit_loop per problem; the reference
 * fits one problem at a time from the host (NewtonGaussian.py:18-109).
 *
 * A member is a 2D problem (geom.kdet 1) of n_atoms <= 224, every member of
 * a batch with the same r layout (isotropic: P = 4, else P = 6), at most 8192
 * (angle, 32-cell tile) items, whose derivative split gives every lane one
 * angle; gr_batch_workspace_bytes returns 0 for members that cannot be
 * batched.  Buffers as gr_newton_solve / gr_newton_accept use them; `fields`
 * holds the residual field of the latest projection (the current atoms' after
 * an accepted trial, which is when the derivatives read it).
 *
 *   gr_batch_create(members, n, ws, ws_bytes, max_reject, stream, &batch)
 *       lays the batch out in ws (gr_batch_workspace_bytes) and copies its
 *       tables (waits for that copy);
 *   gr_batch_prologue(batch, stream)  all members active, fields and
 *       loss_cur of their current atoms (before every launch of the loop);
 *   the loop: gr_fit_loop_begin(stream, guard, &loop),
 *       gr_batch_iterate(batch, loop, stream) (captured: derivatives, solves,
 *       trial projection, accept, batch stop test), gr_fit_loop_end_open(loop,
 *       stream) (no single-problem stop test), gr_fit_loop_instantiate,
 *       gr_fit_loop_launch;
 *   gr_batch_destroy(batch)  (the workspace stays the caller's). */
typedef struct gr_batch_member {
  gr_atoms cur;          /* current atoms (accepted steps update them) */
  gr_atoms trial;        /* trial atoms, same layout */
  gr_geometry geom;      /* 2D */
  const float *data;     /* data sinogram (n_angles, n_det) */
  float *fields;         /* residual field of the latest projection */
  double *loss_cur, *loss_trial;
  double *theta, *theta_trial;  /* (n, P) FP64 parameters [I, x, r] */
  double *lam, *step;           /* (n) damping, step norms */
  double *f, *g, *H;            /* (n), (n, P), (n, P, P) derivatives */
  double *hist;          /* (hist_len) loss after each iteration */
  int *hist_acc;         /* (hist_len) 1: accepted, 0: rejected */
  int *counter;          /* iterations done (zero before the first launch) */
  int hist_len, max_iter;
  double tol, lam_min, lam_max;
} gr_batch_member;
size_t gr_batch_workspace_bytes(const gr_batch_member *members, int n);
int gr_batch_create(const gr_batch_member *members, int n, void *ws, size_t ws_bytes,
                    int max_reject, void *stream, void **batch);
int gr_batch_prologue(void *batch, void *stream);
int gr_batch_iterate(void *batch, void *loop, void *stream);
int gr_fit_loop_end_open(void *loop, void *stream);
int gr_batch_destroy(void *batch);

/*
 * Kernel timers (no counterpart in the reference; measurement only).  While
 * enabled, CUDA events are recorded on the launching stream around each
 * launch of GR_TIMER_PROJECT (the projection kernel of gr_radproj /
 * gr_fit_forward and their pixel-integrated forms) or GR_TIMER_DERIVS (the
 * per-atom derivative kernel of gr_atom_derivs), up to 1024 launches.
 * gr_kernel_timer(which, 1) clears and starts, (which, 0) stops;
 * gr_kernel_timer_read waits for the recorded launches and returns their
 * summed duration in ms and their number.  Not for use while a stream is
 * being captured into a graph; not thread-safe against concurrent launches.
 */
enum { GR_TIMER_PROJECT = 1, GR_TIMER_DERIVS = 2 };
int gr_kernel_timer(int which, int enable);
int gr_kernel_timer_read(int which, double *total_ms, int *launches);

/*
 * gr_radproj without a caller-supplied workspace.  No counterpart in the
 * reference (its kernels are Numba launches that allocate as they please).
 *
 * For callers that cannot allocate device memory themselves: a host program
 * that owns the whole GPU memory budget and gives plug-ins only the buffers
 * they must fill, a binding that can pass device pointers but has no device
 * allocator, or a loop that must avoid cudaMalloc/cudaFree because they
 * synchronise the device.  The scratch is a 4 MiB array compiled into the
 * library; every GPU that loads the library keeps it until the process exits.
 * Problems whose projection workspace (gr_workspace_bytes(GR_OP_PROJECT, ..))
 * exceeds 4 MiB are rejected with GR_ERR_TOO_LARGE.  The call allocates
 * nothing.  The first call on a device looks up the scratch address on that
 * device (make it before any stream capture there); the address is kept per
 * CUDA context, so a call under another context of the device (one the
 * caller created, or the primary context re-created after cudaDeviceReset)
 * looks it up again, and the first call under that context should also come
 * before any capture.  All calls share the
 * scratch: calls whose GPU work overlaps in time race and must be serialised
 * by the caller.  Results equal gr_radproj's.
 */
int gr_radproj_noalloc(const gr_atoms *atoms, const gr_geometry *geom, float *R,
                       void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GAUSS_RADON_H */

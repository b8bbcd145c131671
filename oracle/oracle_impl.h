/*
 * Gaussian-atom Radon oracle: CPU restatement of the reference's dense
 * per-pixel kernels.  TEST INFRASTRUCTURE ONLY: tests/, the smoke check and
 * the CPU-baseline leg of bench.py may call it; the product path never does.
 *
 * This header is included twice by oracle.c, once with REAL=double
 * (SFX=_f64, the FP64 oracle) and once with REAL=float (SFX=_f32, a
 * single-precision twin that mirrors the reference's float32 arithmetic and
 * serves as the timed CPU baseline).  Every function evaluates every atom at
 * every detector cell, exactly as the reference's Numba kernels do (no
 * culling beyond the basis' own cutoff).
 *
 * Parameter conventions (reference GaussDictCode/bin/NewtonBases2D.py:17-72,
 * GaussDictCode/bin/NewtonBases.py:239-310):
 *   atom = (I, x[d], r[Pr]); r is the upper-triangular factor packed
 *   2D: [r00, r11, r01]; 3D: [r00, r11, r22, r01, r12, r02].
 *   derivative order: [I, x0..x_{d-1}, r0..r_{Pr-1}].
 * Geometry modes:
 *   GM_2D  : T[a] (2), w0[a] (2), y = p0*w0          (NewtonBases2D.py:247-249)
 *   GM_3D  : T[a] (3), w0[a], w1[a] (3), y = p0*w0 + p1*w1 (NewtonBases.py:677-680)
 *   GM_2P5D: T[a] (2), w0[a] (2), y = (p0*w0[0], p0*w0[1], p1), T padded
 *            with a zero third component (NewtonBases.py:685-688, :334-345)
 */
#ifndef REAL
#error "define REAL and SFX before including oracle_impl.h"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* radial basis of the projection, reference NewtonBases.py:50-71 */
static void FN(dRg)(REAL m, REAL *dg)
{
    if (m > 1) {
        dg[0] = 0; dg[1] = 0; dg[2] = 0;
    } else {
        dg[0] = RX_EXP(-30 * m);
        dg[1] = -30 * dg[0];
        dg[2] = 900 * dg[0];
    }
}

/* map packed r index -> (row, col) of the upper-triangular factor */
static void FN(rindex)(int dim, int p, int *a, int *b)
{
    static const int i2[3][2] = {{0, 0}, {1, 1}, {0, 1}};
    static const int i3[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {0, 2}};
    if (dim == 2) { *a = i2[p][0]; *b = i2[p][1]; }
    else { *a = i3[p][0]; *b = i3[p][1]; }
}

/* r as a dense dim x dim upper-triangular matrix */
static void FN(rmat)(int dim, const REAL *r, REAL M[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) M[i][j] = 0;
    int np = dim == 2 ? 3 : 6;
    for (int p = 0; p < np; p++) {
        int a, b;
        FN(rindex)(dim, p, &a, &b);
        M[a][b] = r[p];
    }
}

/* detector cell -> point y in the volume, for angle a */
static void FN(tovec)(int gm, int a, const REAL *w0, const REAL *w1, REAL p0,
                      REAL p1, REAL *y)
{
    if (gm == 2) {
        y[0] = p0 * w0[2 * a + 0];
        y[1] = p0 * w0[2 * a + 1];
    } else if (gm == 3) {
        for (int i = 0; i < 3; i++) y[i] = p0 * w0[3 * a + i] + p1 * w1[3 * a + i];
    } else {
        y[0] = p0 * w0[2 * a + 0];
        y[1] = p0 * w0[2 * a + 1];
        y[2] = p1;
    }
}

/*
 * Value of one atom at one detector point: I*Rg(|M r(y-x)|^2)/|rT|.
 * Follows NewtonBases2D.py:39-72 (dim 2) and NewtonBases.py:262-310 (dim 3,
 * lenT 2 or 3).
 */
static REAL FN(Rf_gen)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                       const REAL *y, const REAL *T, int cut)
{
    REAL M[3][3], Y[3] = {0, 0, 0}, rY[3] = {0, 0, 0}, rT[3] = {0, 0, 0},
                  T3[3] = {0, 0, 0};
    FN(rmat)(dim, r, M);
    for (int i = 0; i < dim; i++) Y[i] = y[i] - x[i];
    for (int i = 0; i < lenT; i++) T3[i] = T[i];
    for (int i = 0; i < dim; i++)
        for (int j = i; j < dim; j++) {
            rY[i] += M[i][j] * Y[j];
            rT[i] += M[i][j] * T3[j];
        }
    REAL n = 0;
    for (int i = 0; i < lenT; i++) n += rT[i] * rT[i];
    n = (REAL)1 / RX_SQRT(n);
    for (int i = 0; i < lenT; i++) rT[i] *= n;
    REAL IP = 0;
    for (int i = 0; i < lenT; i++) IP += rT[i] * rY[i];
    REAL m = 0;
    for (int i = 0; i < dim; i++) {
        REAL MY = rY[i] - rT[i] * IP;
        m += MY * MY;
    }
    if (cut && m > 1) return 0;
    return I * RX_EXP(-30 * m) * n;
}

static REAL FN(Rf)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                   const REAL *y, const REAL *T)
{
    return FN(Rf_gen)(dim, lenT, I, x, r, y, T, 1);
}

static REAL FN(Rf_nocut)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                         const REAL *y, const REAL *T)
{
    return FN(Rf_gen)(dim, lenT, I, x, r, y, T, 0);
}

/*
 * Value, gradient and Hessian of one atom at one detector point with respect
 * to (I, x, r).  Restates __dRf (NewtonBases2D.py:77-242) for dim 2 and
 * __dRf_aniso (NewtonBases.py:315-527) for dim 3, including the shared
 * intermediate quantities dJdy, dJdT, ddJdyy, ddJdyT, ddJdTT.  P = 1+dim+Pr.
 * ddR is P x P row-major.  With order 1 only R and dR are filled.
 */
static void FN(dRf_gen)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                        const REAL *y, const REAL *T, REAL *R, REAL *dR, REAL *ddR,
                        int order, int cut)
{
    const int Pr = dim == 2 ? 3 : 6, P = 1 + dim + Pr;
    REAL M[3][3], Y[3] = {0, 0, 0}, rY[3] = {0, 0, 0}, rT[3] = {0, 0, 0},
                  T3[3] = {0, 0, 0}, MY[3] = {0, 0, 0};
    FN(rmat)(dim, r, M);
    for (int i = 0; i < dim; i++) Y[i] = y[i] - x[i];
    for (int i = 0; i < lenT; i++) T3[i] = T[i];
    for (int i = 0; i < dim; i++)
        for (int j = i; j < dim; j++) {
            rY[i] += M[i][j] * Y[j];
            rT[i] += M[i][j] * T3[j];
        }
    REAL n = 0;
    for (int i = 0; i < lenT; i++) n += rT[i] * rT[i];
    n = (REAL)1 / RX_SQRT(n);
    for (int i = 0; i < lenT; i++) rT[i] *= n;
    REAL IP = 0;
    for (int i = 0; i < lenT; i++) IP += rT[i] * rY[i];
    REAL m = 0;
    for (int i = 0; i < dim; i++) {
        MY[i] = rY[i] - rT[i] * IP;
        m += MY[i] * MY[i];
    }
    REAL dMydT[3][3];
    for (int i = 0; i < dim; i++) {
        for (int j = 0; j < dim; j++) dMydT[i][j] = rT[i] * (IP * rT[j] - MY[j]);
        dMydT[i][i] -= IP;
    }
    REAL dg[3];
    if (cut) {
        FN(dRg)(m, dg);
    } else {
        dg[0] = RX_EXP(-30 * m);
        dg[1] = -30 * dg[0];
        dg[2] = 900 * dg[0];
    }
    for (int i = 0; i < P; i++) {
        dR[i] = 0;
        if (order > 1)
            for (int j = 0; j < P; j++) ddR[i * P + j] = 0;
    }
    *R = 0;
    if (dg[0] == 0 && dg[1] == 0 && dg[2] == 0) return;

    REAL dJdy[3], dJdT[3], ddJdyy[3][3], ddJdyT[3][3], ddJdTT[3][3];
    for (int i = 0; i < dim; i++) dJdy[i] = dg[1] * 2 * n * MY[i];
    for (int i = 0; i < dim; i++)
        dJdT[i] = -n * n * (2 * IP * MY[i] * dg[1] + rT[i] * dg[0]);
    if (order > 1) {
        for (int i = 0; i < dim; i++)
            for (int j = i; j < dim; j++) {
                REAL v;
                if (i == j)
                    v = 2 * n * (2 * MY[i] * MY[i] * dg[2] + (1 - rT[i] * rT[i]) * dg[1]);
                else
                    v = 2 * n * (2 * MY[i] * MY[j] * dg[2] - rT[i] * rT[j] * dg[1]);
                ddJdyy[i][j] = v;
                ddJdyy[j][i] = v;
            }
        for (int i = 0; i < dim; i++)
            for (int j = 0; j < dim; j++)
                ddJdyT[i][j] = 2 * n * n *
                               ((dMydT[i][j] - MY[i] * rT[j]) * dg[1] -
                                2 * IP * MY[i] * MY[j] * dg[2]);
        for (int i = 0; i < dim; i++)
            for (int j = i; j < dim; j++) {
                REAL v = 2 * n * n * n *
                         ((1.5 * rT[i] * rT[j] - (i == j ? 0.5 : 0.0)) * dg[0] +
                          (2 * IP * MY[i] * rT[j] + IP * rT[i] * MY[j] -
                           IP * dMydT[i][j] - MY[i] * MY[j]) * dg[1] +
                          2 * IP * IP * MY[i] * MY[j] * dg[2]);
                ddJdTT[i][j] = v;
                ddJdTT[j][i] = v;
            }
    }
    *R = I * dg[0] * n;
    /* first row of ddR: derivatives of dR/dI = R/I */
    REAL row0[10];
    row0[0] = 0;
    for (int c = 0; c < dim; c++) {
        REAL s = 0;
        for (int a = 0; a <= c; a++) s += M[a][c] * dJdy[a];
        row0[1 + c] = -s;
    }
    for (int p = 0; p < Pr; p++) {
        int a, b;
        FN(rindex)(dim, p, &a, &b);
        row0[1 + dim + p] = dJdy[a] * Y[b] + dJdT[a] * T3[b];
    }
    dR[0] = dg[0] * n;
    for (int i = 1; i < P; i++) dR[i] = I * row0[i];
    if (order <= 1) return;
    for (int i = 0; i < P; i++) ddR[i] = row0[i];
    /* r-r block */
    for (int p = 0; p < Pr; p++) {
        int a, b;
        FN(rindex)(dim, p, &a, &b);
        for (int q = p; q < Pr; q++) {
            int c, e;
            FN(rindex)(dim, q, &c, &e);
            ddR[(1 + dim + p) * P + 1 + dim + q] =
                I * (ddJdyy[a][c] * Y[b] * Y[e] + ddJdyT[a][c] * Y[b] * T3[e] +
                     ddJdyT[c][a] * Y[e] * T3[b] + ddJdTT[a][c] * T3[b] * T3[e]);
        }
    }
    /* x-r block */
    for (int p = 0; p < Pr; p++) {
        int a, b;
        FN(rindex)(dim, p, &a, &b);
        for (int cc = 0; cc < dim; cc++) {
            REAL s = 0;
            for (int k = 0; k <= cc; k++)
                s += (ddJdyy[a][k] * Y[b] + ddJdyT[k][a] * T3[b]) * M[k][cc];
            if (b == cc) s += dJdy[a];
            ddR[(1 + cc) * P + 1 + dim + p] = -I * s;
        }
    }
    /* x-x block */
    for (int c0 = 0; c0 < dim; c0++)
        for (int c1 = c0; c1 < dim; c1++) {
            REAL s = 0;
            for (int k = 0; k <= c0; k++)
                for (int l = 0; l <= c1; l++) s += ddJdyy[k][l] * M[k][c0] * M[l][c1];
            ddR[(1 + c0) * P + 1 + c1] = I * s;
        }
    for (int i = 0; i < P; i++)
        for (int j = 0; j < i; j++) ddR[i * P + j] = ddR[j * P + i];
}

static void FN(dRf)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                    const REAL *y, const REAL *T, REAL *R, REAL *dR, REAL *ddR,
                    int order)
{
    FN(dRf_gen)(dim, lenT, I, x, r, y, T, R, dR, ddR, order, 1);
}

static void FN(dRf_nocut)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                          const REAL *y, const REAL *T, REAL *R, REAL *dR, REAL *ddR,
                          int order)
{
    FN(dRf_gen)(dim, lenT, I, x, r, y, T, R, dR, ddR, order, 0);
}

static int FN(geom)(int gm, int *dim, int *lenT)
{
    if (gm == 2) { *dim = 2; *lenT = 2; }
    else if (gm == 3) { *dim = 3; *lenT = 3; }
    else if (gm == 25) { *dim = 3; *lenT = 2; }
    else return -1;
    return 0;
}

/*
 * Dense forward projection R[a, k0, k1] = sum_j Rf(atom j, y(a,k0,k1), T[a]).
 * Reference: __RadProj (NewtonBases2D.py:286-296), __RadProj_3D/_2p5D
 * (NewtonBases.py:731-756).  Atoms are summed in index order per cell.
 */
int FN(or_radproj)(int gm, int N, const REAL *I, const REAL *x, const REAL *r,
                   int A, const REAL *T, const REAL *w0, const REAL *w1, int D0,
                   const REAL *p0, int D1, const REAL *p1, REAL *R, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) D1 = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        REAL y[3] = {0, 0, 0};
        for (int k0 = 0; k0 < D0; k0++)
            for (int k1 = 0; k1 < D1; k1++) {
                FN(tovec)(gm, a, w0, w1, p0[k0], dim == 2 ? 0 : p1[k1], y);
                REAL acc = 0;
                for (int j = 0; j < N; j++)
                    acc += FN(Rf)(dim, lenT, I[j], x + dim * j, r + Pr * j, y,
                                  T + lenT * a);
                R[((size_t)a * D0 + k0) * D1 + k1] = acc;
            }
    }
    return 0;
}

/*
 * The same projection, visiting per (angle, atom) only the detector cells
 * whose coordinates fall inside the atom's shadow box.  The basis support
 * |r(z - x)| <= 1 is an ellipsoid; a cell's ray meets it exactly when the
 * cell's m <= 1 (m is the minimum of |r(z - x)|^2 along the ray), and the
 * ray's coordinate on a detector axis u (orthonormal to T) is u.z, so every
 * in-support cell lies within |u.x - p| <= |r^{-T} u| on each axis.  The box
 * is padded by one cell; Rf's own m <= 1 test still decides every visited
 * cell, and atoms are added in index order per cell, so the result equals
 * or_radproj's (cells outside every box receive exact zeros).  Used to build
 * the large benchmark workloads on the host.
 */
static void FN(cell_range)(const REAL *p, int n, double c, double h, int *lo, int *hi)
{
    int a = 0, b = n;                        /* first index with p >= c - h */
    while (a < b) {
        int m = (a + b) / 2;
        if ((double)p[m] < c - h) a = m + 1; else b = m;
    }
    int l = a - 1;
    a = 0; b = n;                            /* first index with p > c + h */
    while (a < b) {
        int m = (a + b) / 2;
        if ((double)p[m] <= c + h) a = m + 1; else b = m;
    }
    int u = a;
    *lo = l < 0 ? 0 : l;
    *hi = u > n - 1 ? n - 1 : u;
}

/* Cell index box [lo, hi] (per detector axis) of one atom's shadow at angle
 * a; returns 1 when the box is empty. */
static int FN(shadow_box)(int gm, int dim, int a, const REAL *w0, const REAL *w1,
                          const REAL *xj, const REAL *rj, int D0, const REAL *p0,
                          int D1, const REAL *p1, int *lo, int *hi)
{
    double u[2][3] = {{0, 0, 0}, {0, 0, 0}};
    if (gm == 2) {
        u[0][0] = w0[2 * a]; u[0][1] = w0[2 * a + 1];
    } else if (gm == 3) {
        for (int i = 0; i < 3; i++) { u[0][i] = w0[3 * a + i]; u[1][i] = w1[3 * a + i]; }
    } else {
        u[0][0] = w0[2 * a]; u[0][1] = w0[2 * a + 1]; u[1][2] = 1;
    }
    REAL M[3][3];
    FN(rmat)(dim, rj, M);
    lo[1] = hi[1] = 0;
    for (int c = 0; c < (dim == 2 ? 1 : 2); c++) {
        /* v = M^{-T} u_c: forward substitution, M^T lower triangular */
        double v[3], h2 = 0, ctr = 0;
        for (int i = 0; i < dim; i++) {
            double s = u[c][i];
            for (int k = 0; k < i; k++) s -= (double)M[k][i] * v[k];
            v[i] = s / (double)M[i][i];
            h2 += v[i] * v[i];
            ctr += u[c][i] * (double)xj[i];
        }
        double h = sqrt(h2) * (1 + 1e-6) + 1e-9;
        const REAL *pc = c == 0 ? p0 : p1;
        const int nc = c == 0 ? D0 : D1;
        FN(cell_range)(pc, nc, ctr, h, &lo[c], &hi[c]);
        if (!(h == h) || h > 1e30) { lo[c] = 0; hi[c] = nc - 1; }
        if (lo[c] > hi[c]) return 1;
    }
    return 0;
}

int FN(or_radproj_boxed)(int gm, int N, const REAL *I, const REAL *x, const REAL *r,
                         int A, const REAL *T, const REAL *w0, const REAL *w1, int D0,
                         const REAL *p0, int D1, const REAL *p1, REAL *R, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) D1 = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        REAL *Ra = R + (size_t)a * D0 * D1;
        for (size_t c = 0; c < (size_t)D0 * D1; c++) Ra[c] = 0;
        REAL y[3] = {0, 0, 0};
        for (int j = 0; j < N; j++) {
            const REAL *xj = x + dim * j, *rj = r + Pr * j;
            int lo[2], hi[2];
            if (FN(shadow_box)(gm, dim, a, w0, w1, xj, rj, D0, p0, D1, p1, lo, hi)) continue;
            for (int k0 = lo[0]; k0 <= hi[0]; k0++)
                for (int k1 = lo[1]; k1 <= hi[1]; k1++) {
                    FN(tovec)(gm, a, w0, w1, p0[k0], dim == 2 ? 0 : p1[k1], y);
                    Ra[(size_t)k0 * D1 + k1] += FN(Rf)(dim, lenT, I[j], xj, rj, y,
                                                       T + lenT * a);
                }
        }
    }
    return 0;
}

/*
 * Single-atom derivatives of a data fit, summed over every detector cell:
 *   kind 0 (L2):   f = 1/2 sum (R-C)^2, Df = sum (R-C) dR,
 *                  DDf = sum dR dR^T + (R-C) ddR
 *                  (__L2derivs_RadProj_aniso, NewtonBases2D.py:331-375;
 *                   __L2derivs_RadProj_aniso_3D, NewtonBases.py:794-844)
 *   kind 1 (inner product): f = sum R C, Df = sum C dR, DDf = sum C ddR
 *                  (__derivs_RadProj_aniso, NewtonBases2D.py:446-489;
 *                   __derivs_RadProj_aniso_3D, NewtonBases.py:995-1043)
 *   kind 2 (weight fields, C = alpha, Bf = beta): f = sum alpha R,
 *                  Df = sum alpha dR, DDf = sum beta dR dR^T + alpha ddR
 *                  (the all-atoms fit form: alpha = R_total - data, beta = 1
 *                   reproduces kind 0 with C = data + R_atom - R_total)
 * Per-angle partial sums are combined in angle order, so the result does not
 * depend on the thread count.  With order 1, DDf is left at zero.
 */
int FN(or_atom_derivs)(int kind, int gm, const REAL *I, const REAL *x,
                       const REAL *r, int A, const REAL *T, const REAL *w0,
                       const REAL *w1, int D0, const REAL *p0, int D1,
                       const REAL *p1, const REAL *C, const REAL *Bf, int order,
                       double *f, double *Df, double *DDf, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6, P = 1 + dim + Pr;
    if (dim == 2) D1 = 1;
    const int stride = 1 + P + P * P;
    double *part = (double *)calloc((size_t)A * stride, sizeof(double));
    if (!part) return -2;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        double *acc = part + (size_t)a * stride;
        REAL y[3] = {0, 0, 0}, Rv, dR[10], ddR[100];
        for (int k0 = 0; k0 < D0; k0++)
            for (int k1 = 0; k1 < D1; k1++) {
                FN(tovec)(gm, a, w0, w1, p0[k0], dim == 2 ? 0 : p1[k1], y);
                FN(dRf)(dim, lenT, I[0], x, r, y, T + lenT * a, &Rv, dR, ddR, order);
                REAL c = C[((size_t)a * D0 + k0) * D1 + k1];
                if (kind == 0) {
                    double res = (double)Rv - (double)c;
                    acc[0] += res * res;
                    for (int i = 0; i < P; i++) acc[1 + i] += res * dR[i];
                    if (order > 1)
                        for (int i = 0; i < P; i++)
                            for (int j = 0; j < P; j++)
                                acc[1 + P + i * P + j] +=
                                    (double)dR[i] * dR[j] + res * ddR[i * P + j];
                } else if (kind == 1) {
                    acc[0] += (double)Rv * c;
                    for (int i = 0; i < P; i++) acc[1 + i] += (double)c * dR[i];
                    if (order > 1)
                        for (int i = 0; i < P * P; i++)
                            acc[1 + P + i] += (double)c * ddR[i];
                } else {
                    double be = Bf[((size_t)a * D0 + k0) * D1 + k1];
                    acc[0] += (double)Rv * c;
                    for (int i = 0; i < P; i++) acc[1 + i] += (double)c * dR[i];
                    if (order > 1)
                        for (int i = 0; i < P; i++)
                            for (int j = 0; j < P; j++)
                                acc[1 + P + i * P + j] += be * dR[i] * dR[j] +
                                                          (double)c * ddR[i * P + j];
                }
            }
    }
    double tot[1 + 10 + 100];
    for (int i = 0; i < stride; i++) tot[i] = 0;
    for (int a = 0; a < A; a++)
        for (int i = 0; i < stride; i++) tot[i] += part[(size_t)a * stride + i];
    free(part);
    *f = kind == 0 ? 0.5 * tot[0] : tot[0];
    for (int i = 0; i < P; i++) Df[i] = tot[1 + i];
    for (int i = 0; i < P * P; i++) DDf[i] = order > 1 ? tot[1 + P + i] : 0.0;
    return 0;
}

/*
 * or_atom_derivs for kinds 1 (inner product) and 2 (weight fields) visiting
 * per angle only the atom's shadow box (or_radproj_boxed): every cell
 * outside it contributes exact zeros to those sums, and the box is walked in
 * the dense order, so the results are those of or_atom_derivs.  Kind 0 (whose
 * value also sums C^2 off the support) is not offered.
 */
int FN(or_atom_derivs_boxed)(int kind, int gm, const REAL *I, const REAL *x,
                             const REAL *r, int A, const REAL *T, const REAL *w0,
                             const REAL *w1, int D0, const REAL *p0, int D1,
                             const REAL *p1, const REAL *C, const REAL *Bf, int order,
                             double *f, double *Df, double *DDf, int nthreads)
{
    int dim, lenT;
    if (kind != 1 && kind != 2) return -1;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6, P = 1 + dim + Pr;
    if (dim == 2) D1 = 1;
    const int stride = 1 + P + P * P;
    double *part = (double *)calloc((size_t)A * stride, sizeof(double));
    if (!part) return -2;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        double *acc = part + (size_t)a * stride;
        int lo[2], hi[2];
        if (FN(shadow_box)(gm, dim, a, w0, w1, x, r, D0, p0, D1, p1, lo, hi)) continue;
        REAL y[3] = {0, 0, 0}, Rv, dR[10], ddR[100];
        for (int k0 = lo[0]; k0 <= hi[0]; k0++)
            for (int k1 = lo[1]; k1 <= hi[1]; k1++) {
                FN(tovec)(gm, a, w0, w1, p0[k0], dim == 2 ? 0 : p1[k1], y);
                FN(dRf)(dim, lenT, I[0], x, r, y, T + lenT * a, &Rv, dR, ddR, order);
                REAL c = C[((size_t)a * D0 + k0) * D1 + k1];
                acc[0] += (double)Rv * c;
                for (int i = 0; i < P; i++) acc[1 + i] += (double)c * dR[i];
                if (order > 1) {
                    if (kind == 1) {
                        for (int i = 0; i < P * P; i++) acc[1 + P + i] += (double)c * ddR[i];
                    } else {
                        double be = Bf[((size_t)a * D0 + k0) * D1 + k1];
                        for (int i = 0; i < P; i++)
                            for (int j = 0; j < P; j++)
                                acc[1 + P + i * P + j] += be * dR[i] * dR[j] +
                                                          (double)c * ddR[i * P + j];
                    }
                }
            }
    }
    double tot[1 + 10 + 100];
    for (int i = 0; i < stride; i++) tot[i] = 0;
    for (int a = 0; a < A; a++)
        for (int i = 0; i < stride; i++) tot[i] += part[(size_t)a * stride + i];
    free(part);
    *f = tot[0];
    for (int i = 0; i < P; i++) Df[i] = tot[1 + i];
    for (int i = 0; i < P * P; i++) DDf[i] = order > 1 ? tot[1 + P + i] : 0.0;
    return 0;
}

/*
 * Number of (atom, angle, cell) triples inside the basis support m <= 1,
 * counted densely (the useful work of one projection).
 */
long long FN(or_count_support)(int gm, int N, const REAL *I, const REAL *x,
                               const REAL *r, int A, const REAL *T, const REAL *w0,
                               const REAL *w1, int D0, const REAL *p0, int D1,
                               const REAL *p1, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) D1 = 1;
    long long total = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : total)
    for (int a = 0; a < A; a++) {
        REAL y[3] = {0, 0, 0};
        for (int k0 = 0; k0 < D0; k0++)
            for (int k1 = 0; k1 < D1; k1++) {
                FN(tovec)(gm, a, w0, w1, p0[k0], dim == 2 ? 0 : p1[k1], y);
                for (int j = 0; j < N; j++) {
                    /* unit intensity: Rf > 0 exactly when m <= 1 */
                    if (FN(Rf)(dim, lenT, 1, x + dim * j, r + Pr * j, y, T + lenT * a) > 0)
                        total++;
                }
            }
    }
    return total;
}

/*
 * Per-pixel value/gradient/Hessian at explicit points, for known-answer and
 * finite-difference checks of the restatement itself.
 */
int FN(or_point_derivs)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                        const REAL *y, const REAL *T, REAL *R, REAL *dR,
                        REAL *ddR, int order)
{
    FN(dRf)(dim, lenT, I, x, r, y, T, R, dR, ddR, order);
    return 0;
}

/*
 * Volume rendering u[v0, v1(, v2)] = sum_j I_j g(|r_j (y - x_j)|^2) with
 * g(n) = sqrt(30/pi) exp(-30 n) for n <= 1, else 0.
 * Reference: __f / __VolProj (NewtonBases2D.py:17-34, :261-271;
 * NewtonBases.py:239-257, :700-711).
 */
int FN(or_volproj)(int dim, int N, const REAL *I, const REAL *x, const REAL *r,
                   int V0, const REAL *y0, int V1, const REAL *y1, int V2,
                   const REAL *y2, REAL *u, int nthreads)
{
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) V2 = 1;
    const double c0 = sqrt(30.0 / 3.14159265358979323846);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int i0 = 0; i0 < V0; i0++)
        for (int i1 = 0; i1 < V1; i1++)
            for (int i2 = 0; i2 < V2; i2++) {
                REAL y[3] = {y0[i0], y1[i1], dim == 3 ? y2[i2] : 0};
                REAL acc = 0;
                for (int j = 0; j < N; j++) {
                    REAL M[3][3], Y[3] = {0, 0, 0}, rY[3] = {0, 0, 0};
                    FN(rmat)(dim, r + Pr * j, M);
                    for (int i = 0; i < dim; i++) Y[i] = y[i] - x[dim * j + i];
                    REAL nn = 0;
                    for (int i = 0; i < dim; i++) {
                        for (int k = i; k < dim; k++) rY[i] += M[i][k] * Y[k];
                        nn += rY[i] * rY[i];
                    }
                    if (nn <= 1)
                        acc += I[j] * RX_EXP(-30 * nn) * (REAL)c0;
                }
                u[((size_t)i0 * V1 + i1) * V2 + i2] = acc;
            }
    return 0;
}


/* ------------------------------------------------------------------------
 * Single-particle ("point spread") operator: pixel-integrated projections.
 * Restates GaussDictCode/bin/point_spread_functions.py: __Radius (:24),
 * __total (:60), __projnorm (:75), __Rf (:386, no m > 1 cut-off), __rf2 (:413),
 * __rf3 (:462), __dRf2/__dRf3 (:594, :738), __drf2 (:924), __drf3 (:1002),
 * the bin ranges of __RadProj_2D/_3D (:530-588) and the L2 / inner-product
 * accumulations (:1119-1313, :1354-1523).  Square pixels of half-width
 * s = |p0[1] - p0[0]| / 2, as the reference assumes.
 * ------------------------------------------------------------------------ */
static REAL FN(psf_radius)(int dim, const REAL *r)
{
    REAL R = r[0] < r[1] ? r[0] : r[1];
    if (dim == 3 && r[2] < R) R = r[2];
    return (REAL)1 / R;
}

static REAL FN(psf_total)(int dim, REAL I, const REAL *r)
{
    if (dim == 2) return I / (r[0] * r[1]) * RX_SQRT((REAL)(3.14159265358979323846 / 30));
    return I / (r[0] * r[1] * r[2]) * (REAL)(3.14159265358979323846 / 30);
}

/* value (and, with want_d, derivatives) of the pixel integral at pixel
 * centre y for one atom; T, W0, W1 padded to 3 components */
static void FN(psf_pixel)(int dim, int lenT, REAL I, const REAL *x, const REAL *r,
                          const REAL *y, const REAL *T, const REAL *W0, const REAL *W1,
                          REAL s, int want_d, int order, REAL *R, REAL *dR, REAL *ddR)
{
    const int Pr = dim == 2 ? 3 : 6, P = 1 + dim + Pr;
    REAL X[3] = {0, 0, 0};
    for (int i = 0; i < dim; i++) X[i] = x[i] - y[i];
    *R = 0;
    if (want_d)
        for (int i = 0; i < P; i++) {
            dR[i] = 0;
            for (int j = 0; j < P; j++) ddR[i * P + j] = 0;
        }
    REAL rr = FN(psf_radius)(dim, r);
    REAL t0 = 0, t1 = 0;
    for (int i = 0; i < dim; i++) t0 += X[i] * X[i];
    for (int i = 0; i < lenT; i++) t1 += X[i] * T[i];
    t0 = t0 - t1 * t1;
    REAL n = t0 > 0 ? RX_SQRT(t0) : 0;
    if (n + rr < s) {
        *R = FN(psf_total)(dim, I, r);
        return;
    } else if (n - rr > s) {
        return;
    }
    REAL lim[2][2];
    REAL Wv[2][3] = {{W0[0], W0[1], W0[2]}, {W1[0], W1[1], W1[2]}};
    const int K = dim - 1;
    for (int k = 0; k < K; k++) {
        REAL c = 0;
        for (int i = 0; i < dim; i++) c += X[i] * Wv[k][i];
        lim[k][1] = c + rr < s ? c + rr : s;
        lim[k][0] = c - rr > -s ? c - rr : -s;
    }
    REAL Ys[3] = {0, 0, 0};
    for (int i = 0; i < dim; i++) {
        Ys[i] = lim[0][0] * Wv[0][i];
        if (K == 2) Ys[i] += lim[1][0] * Wv[1][i];
    }
    REAL step[2];
    for (int k = 0; k < K; k++) step[k] = (REAL)0.1 * (lim[k][1] - lim[k][0]);
    REAL Rv, dRv[10], ddRv[100];
    int count = 0;
    REAL sum = 0;
    for (int a = 0; a < 11; a++) {
        for (int i = 0; i < dim; i++) Ys[i] += step[0] * Wv[0][i];
        int nb = K == 2 ? 11 : 1;
        for (int b = 0; b < nb; b++) {
            if (K == 2)
                for (int i = 0; i < dim; i++) Ys[i] += step[1] * Wv[1][i];
            /* point value at volume point y + Ys: the per-point basis has no
             * cut-off in this module */
            REAL Yp[3];
            for (int i = 0; i < dim; i++) Yp[i] = y[i] + Ys[i];
            if (want_d) {
                FN(dRf_nocut)(dim, lenT, I, x, r, Yp, T, &Rv, dRv, ddRv, order);
                sum += Rv;
                for (int i = 0; i < P; i++) {
                    dR[i] += dRv[i];
                    if (order > 1)
                        for (int j = 0; j < P; j++) ddR[i * P + j] += ddRv[i * P + j];
                }
            } else {
                sum += FN(Rf_nocut)(dim, lenT, I, x, r, Yp, T);
            }
            count++;
        }
        if (K == 2)
            for (int i = 0; i < dim; i++) Ys[i] -= 11 * step[1] * Wv[1][i];
    }
    REAL scale = K == 1 ? 10 * step[0] / count : 100 * step[0] * step[1] / count;
    *R = sum * scale;
    if (want_d)
        for (int i = 0; i < P; i++) {
            dR[i] *= scale;
            for (int j = 0; j < P; j++) ddR[i * P + j] *= scale;
        }
}

static void FN(psf_frame)(int gm, int a, const REAL *T, const REAL *w0, const REAL *w1,
                          REAL *T3, REAL *W0, REAL *W1, int *lenT)
{
    for (int i = 0; i < 3; i++) { T3[i] = 0; W0[i] = 0; W1[i] = 0; }
    if (gm == 2) {
        *lenT = 2;
        for (int i = 0; i < 2; i++) { T3[i] = T[2 * a + i]; W0[i] = w0[2 * a + i]; }
    } else if (gm == 3) {
        *lenT = 3;
        for (int i = 0; i < 3; i++) {
            T3[i] = T[3 * a + i]; W0[i] = w0[3 * a + i]; W1[i] = w1[3 * a + i];
        }
    } else {
        *lenT = 2;
        for (int i = 0; i < 2; i++) { T3[i] = T[2 * a + i]; W0[i] = w0[2 * a + i]; }
        W1[2] = 1;
    }
}

/* pixel-integrated forward projection (bin ranges of __RadProj_2D/_3D) */
int FN(or_psf_radproj)(int gm, int N, const REAL *I, const REAL *x, const REAL *r,
                       int A, const REAL *T, const REAL *w0, const REAL *w1, int D0,
                       const REAL *p0, int D1, const REAL *p1, REAL *R, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) D1 = 1;
    const REAL s = (REAL)fabs((double)(p0[1] - p0[0])) / 2;
    const REAL dp = 1 / (p0[1] - p0[0]);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        REAL T3[3], W0[3], W1[3], y[3];
        int lt;
        FN(psf_frame)(gm, a, T, w0, w1, T3, W0, W1, &lt);
        REAL *out = R + (size_t)a * D0 * D1;
        for (int k = 0; k < D0 * D1; k++) out[k] = 0;
        for (int j = 0; j < N; j++) {
            const REAL *xj = x + dim * j, *rj = r + Pr * j;
            REAL rr = FN(psf_radius)(dim, rj);
            REAL IP = 0;
            for (int i = 0; i < dim; i++) IP += xj[i] * W0[i];
            int b00 = (int)((IP - rr - p0[0]) * dp);
            if (b00 < 0) b00 = 0;
            int b01 = (int)((IP + rr - p0[0]) * dp) + 2;
            if (b01 > D0) b01 = D0;
            int b10 = 0, b11 = 1;
            if (dim == 3) {
                IP = 0;
                for (int i = 0; i < 3; i++) IP += xj[i] * W1[i];
                b10 = (int)((IP - rr - p1[0]) * dp);
                if (b10 < 0) b10 = 0;
                b11 = (int)((IP + rr - p1[0]) * dp) + 2;
                if (b11 > D1) b11 = D1;
            }
            for (int k0 = b00; k0 < b01; k0++)
                for (int k1 = b10; k1 < b11; k1++) {
                    for (int i = 0; i < 3; i++)
                        y[i] = p0[k0] * W0[i] + (dim == 3 ? p1[k1] * W1[i] : 0);
                    REAL v;
                    FN(psf_pixel)(dim, lt, I[j], xj, rj, y, T3, W0, W1, s, 0, 0, &v, 0, 0);
                    out[(size_t)k0 * D1 + k1] += v;
                }
        }
    }
    return 0;
}

/* single-atom derivatives of the pixel-integrated projection, summed over
 * all cells: kind 0 (L2, C^2 for cells outside the bins), kind 1 (inner) */
int FN(or_psf_atom_derivs)(int kind, int gm, const REAL *I, const REAL *x, const REAL *r,
                           int A, const REAL *T, const REAL *w0, const REAL *w1, int D0,
                           const REAL *p0, int D1, const REAL *p1, const REAL *C, int order,
                           double *f, double *Df, double *DDf, int nthreads)
{
    int dim, lenT;
    if (FN(geom)(gm, &dim, &lenT)) return -1;
    const int Pr = dim == 2 ? 3 : 6, P = 1 + dim + Pr;
    if (dim == 2) D1 = 1;
    const int stride = 1 + P + P * P;
    double *part = (double *)calloc((size_t)A * stride, sizeof(double));
    if (!part) return -2;
    const REAL s = (REAL)fabs((double)(p0[1] - p0[0])) / 2;
    const REAL dp = 1 / (p0[1] - p0[0]);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int a = 0; a < A; a++) {
        double *acc = part + (size_t)a * stride;
        REAL T3[3], W0[3], W1[3], y[3], Rv, dR[10], ddR[100];
        int lt;
        FN(psf_frame)(gm, a, T, w0, w1, T3, W0, W1, &lt);
        REAL rr = FN(psf_radius)(dim, r);
        REAL IP = 0;
        for (int i = 0; i < dim; i++) IP += x[i] * W0[i];
        int b00 = (int)((IP - rr - s - p0[0]) * dp);
        if (b00 < 0) b00 = 0;
        int b01 = (int)((IP + rr + s - p0[0]) * dp) + 1;
        if (b01 > D0) b01 = D0;
        int b10 = 0, b11 = 1;
        if (dim == 3) {
            IP = 0;
            for (int i = 0; i < 3; i++) IP += x[i] * W1[i];
            b10 = (int)((IP - rr - s - p1[0]) * dp) - 1;
            if (b10 < 0) b10 = 0;
            b11 = (int)((IP + rr + s - p1[0]) * dp) + 1;
            if (b11 > D1) b11 = D1;
        }
        for (int k0 = 0; k0 < D0; k0++)
            for (int k1 = 0; k1 < D1; k1++) {
                double c = C[((size_t)a * D0 + k0) * D1 + k1];
                int in = k0 >= b00 && k0 < b01 && k1 >= b10 && k1 < b11;
                if (!in) {
                    if (kind == 0) acc[0] += c * c;
                    continue;
                }
                for (int i = 0; i < 3; i++)
                    y[i] = p0[k0] * W0[i] + (dim == 3 ? p1[k1] * W1[i] : 0);
                FN(psf_pixel)(dim, lt, I[0], x, r, y, T3, W0, W1, s, 1, order, &Rv, dR, ddR);
                if (kind == 0) {
                    double res = (double)Rv - c;
                    acc[0] += res * res;
                    for (int i = 0; i < P; i++) acc[1 + i] += res * dR[i];
                    if (order > 1)
                        for (int i = 0; i < P; i++)
                            for (int j = 0; j < P; j++)
                                acc[1 + P + i * P + j] +=
                                    (double)dR[i] * dR[j] + res * ddR[i * P + j];
                } else {
                    acc[0] += (double)Rv * c;
                    for (int i = 0; i < P; i++) acc[1 + i] += c * dR[i];
                    if (order > 1)
                        for (int i = 0; i < P * P; i++) acc[1 + P + i] += c * ddR[i];
                }
            }
    }
    double tot[1 + 10 + 100];
    for (int i = 0; i < stride; i++) tot[i] = 0;
    for (int a = 0; a < A; a++)
        for (int i = 0; i < stride; i++) tot[i] += part[(size_t)a * stride + i];
    free(part);
    *f = kind == 0 ? 0.5 * tot[0] : tot[0];
    for (int i = 0; i < P; i++) Df[i] = tot[1 + i];
    for (int i = 0; i < P * P; i++) DDf[i] = order > 1 ? tot[1 + P + i] : 0.0;
    return 0;
}

/* voxel-integrated rendering (point_spread_functions.py __if2/__if3,
 * __dense_VolProj2/3): 11^dim rule, half-width s = |y1[1] - y1[0]| / 2 */
int FN(or_psf_volproj)(int dim, int N, const REAL *I, const REAL *x, const REAL *r,
                       int V0, const REAL *y0, int V1, const REAL *y1, int V2,
                       const REAL *y2, REAL *u, int nthreads)
{
    const int Pr = dim == 2 ? 3 : 6;
    if (dim == 2) V2 = 1;
    const REAL s = (REAL)fabs((double)(y1[1] - y1[0])) / 2;
    const REAL c0 = RX_SQRT((REAL)(30.0 / 3.14159265358979323846));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int i0 = 0; i0 < V0; i0++)
        for (int i1 = 0; i1 < V1; i1++)
            for (int i2 = 0; i2 < V2; i2++) {
                REAL y[3] = {y0[i0], y1[i1], dim == 3 ? y2[i2] : 0};
                REAL acc = 0;
                for (int j = 0; j < N; j++) {
                    REAL M[3][3], X[3] = {0, 0, 0};
                    FN(rmat)(dim, r + Pr * j, M);
                    const REAL *rj = r + Pr * j;
                    for (int i = 0; i < dim; i++) X[i] = x[dim * j + i] - y[i];
                    REAL rr = FN(psf_radius)(dim, rj), nn = 0;
                    for (int i = 0; i < dim; i++) nn += X[i] * X[i];
                    nn = RX_SQRT(nn);
                    if (nn + rr < s) { acc += FN(psf_total)(dim, I[j], rj); continue; }
                    if (nn - rr > s) continue;
                    REAL lo[3], st[3], Y[3];
                    for (int i = 0; i < dim; i++) {
                        REAL l = X[i] - rr > -s ? X[i] - rr : -s;
                        REAL h = X[i] + rr < s ? X[i] + rr : s;
                        lo[i] = l;
                        st[i] = (REAL)0.1 * (h - l);
                    }
                    REAL sum = 0;
                    int count = 0;
                    for (int a = 1; a <= 11; a++)
                        for (int b = 1; b <= 11; b++)
                            for (int c = 1; c <= (dim == 3 ? 11 : 1); c++) {
                                Y[0] = lo[0] + a * st[0] - X[0];
                                Y[1] = lo[1] + b * st[1] - X[1];
                                Y[2] = dim == 3 ? lo[2] + c * st[2] - X[2] : 0;
                                REAL n2 = 0;
                                for (int q = 0; q < dim; q++) {
                                    REAL v = 0;
                                    for (int k = q; k < dim; k++) v += M[q][k] * Y[k];
                                    n2 += v * v;
                                }
                                sum += RX_EXP(-30 * n2) * c0;
                                count++;
                            }
                    acc += I[j] * sum / count *
                           (dim == 2 ? 100 * st[0] * st[1] : 1000 * st[0] * st[1] * st[2]);
                }
                u[((size_t)i0 * V1 + i1) * V2 + i2] = acc;
            }
    return 0;
}

#undef FN

/*
 * FP64 CPU oracle for the MLS-MPM substep — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain serial C, the arithmetic of FEMFlow's MPM solver so that the
 * CUDA product path can be checked against it.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load it.  The product path never calls it.
 *
 * Parity pin: tests/golden/*.npz hold outputs of the unmodified reference functions (imported
 * in CPython behind a no-op numba stub by tests/golden/make_golden.py) together with the
 * reference's own known-answer vectors; tests/test_oracle_golden.py checks this file against
 * them.
 *
 * Reference files followed (paths inside the FEMFlow project):
 *   femflow/solvers/mpm/three_d/p2g.py:14-80       -> orc_p2g_3d
 *   femflow/solvers/mpm/three_d/grid_op.py:5-47    -> orc_grid_op_3d
 *   femflow/solvers/mpm/three_d/g2p.py:9-59        -> orc_g2p_3d
 *   femflow/solvers/mpm/two_d/p2g.py:11-76         -> orc_p2g_2d
 *   femflow/solvers/mpm/two_d/grid_op.py:5-24      -> orc_grid_op_2d
 *   femflow/solvers/mpm/two_d/g2p.py:5-47          -> orc_g2p_2d
 *   femflow/solvers/mpm/utils.py:7-135             -> hardening + fixed-corotated stress
 *   femflow/solvers/mpm/utils.py:138-150           -> oob rule
 *   femflow/numerics/linear_algebra.py:96-135      -> polar_2d / polar_3d
 *   femflow/solvers/mpm/mls_mpm.py:40-79           -> orc_substep_3d
 *
 * Grid layout follows the reference: grid_velocity[R][R](R)[dim] and grid_mass[R][R](R), R=res+1,
 * row-major, where the first index is the x node.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_OOB 1     /* reference raises RuntimeError (three_d) / IndexError (two_d) */
#define ORC_NOMEM 2
#define ORC_BADARG 3

#define MODEL_NEO_HOOKEAN 0 /* reference string "neo_hookean": fixed-corotated + constant hardening */
#define MODEL_SNOW 1
#define MODEL_FIXED_COROTATED 2 /* textbook stress: lam(J-1)J on the diagonal of PF only (not a reference model) */

/* ------------------------------------------------------------------ small 3x3 helpers */

static void mm3(const double *a, const double *b, double *c) { /* c = a @ b */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += a[i * 3 + k] * b[k * 3 + j];
            c[i * 3 + j] = s;
        }
}

static double det3(const double *m) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static double det2(const double *m) { return m[0] * m[3] - m[1] * m[2]; }

/*
 * Full 3x3 SVD F = U diag(s) V^T with s >= 0 sorted descending, by one-sided (Hestenes) Jacobi
 * rotations on the columns of F.  The reference calls LAPACK through np.linalg.svd
 * (linear_algebra.py:131); for a nonsingular F the polar factor U V^T is unique, so any accurate
 * SVD reproduces it to rounding.
 */
static void svd3(const double *F, double *U, double *s, double *V) {
    double A[9];
    memcpy(A, F, sizeof(A));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    static const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int pi = 0; pi < 3; ++pi) {
            int p = pairs[pi][0], q = pairs[pi][1];
            double alpha = 0, beta = 0, gamma = 0;
            for (int i = 0; i < 3; ++i) {
                alpha += A[i * 3 + p] * A[i * 3 + p];
                beta += A[i * 3 + q] * A[i * 3 + q];
                gamma += A[i * 3 + p] * A[i * 3 + q];
            }
            double nrm = sqrt(alpha * beta);
            if (gamma == 0.0 || nrm == 0.0) continue;
            double rel = fabs(gamma) / nrm;
            if (rel > off) off = rel;
            if (rel < 1e-17) continue;
            double zeta = (beta - alpha) / (2.0 * gamma);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
            for (int i = 0; i < 3; ++i) {
                double ap = A[i * 3 + p], aq = A[i * 3 + q];
                A[i * 3 + p] = c * ap - sn * aq;
                A[i * 3 + q] = sn * ap + c * aq;
                double vp = V[i * 3 + p], vq = V[i * 3 + q];
                V[i * 3 + p] = c * vp - sn * vq;
                V[i * 3 + q] = sn * vp + c * vq;
            }
        }
        if (off < 1e-16) break;
    }
    for (int j = 0; j < 3; ++j) {
        double n = sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
        s[j] = n;
    }
    /* sort descending */
    int idx[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (s[idx[b]] > s[idx[a]]) { int t = idx[a]; idx[a] = idx[b]; idx[b] = t; }
    double A2[9], V2[9], s2[3];
    for (int j = 0; j < 3; ++j) {
        s2[j] = s[idx[j]];
        for (int i = 0; i < 3; ++i) { A2[i * 3 + j] = A[i * 3 + idx[j]]; V2[i * 3 + j] = V[i * 3 + idx[j]]; }
    }
    memcpy(V, V2, sizeof(V2));
    memcpy(s, s2, sizeof(s2));
    double smax = s[0] > 0 ? s[0] : 1.0;
    for (int j = 0; j < 3; ++j) {
        if (s[j] > 1e-300 && s[j] > smax * 1e-15) {
            for (int i = 0; i < 3; ++i) U[i * 3 + j] = A2[i * 3 + j] / s[j];
        } else {
            /* rank-deficient column: complete an orthonormal basis */
            if (j == 2) {
                U[2] = U[3] * U[7] - U[6] * U[4];
                U[5] = U[6] * U[1] - U[0] * U[7];
                U[8] = U[0] * U[4] - U[3] * U[1];
            } else {
                /* pick any unit vector orthogonal to the previous columns */
                double e[3] = {1, 0, 0};
                if (j == 1 && fabs(U[0]) > 0.9) { e[0] = 0; e[1] = 1; }
                if (j == 1) {
                    double d = e[0] * U[0] + e[1] * U[3] + e[2] * U[6];
                    for (int i = 0; i < 3; ++i) e[i] -= d * U[i * 3];
                }
                double n = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                for (int i = 0; i < 3; ++i) U[i * 3 + j] = e[i] / n;
            }
        }
    }
}

/* linear_algebra.py:119-135: R = U @ Vh (no reflection fix-up). */
static void polar3(const double *F, double *R) {
    double U[9], s[3], V[9];
    svd3(F, U, s, V);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += U[i * 3 + k] * V[j * 3 + k];
            R[i * 3 + j] = acc;
        }
}

/* linear_algebra.py:96-116: closed form with the +1e-10 in the denominator. */
static void polar2(const double *m, double *r) {
    double x = m[0] + m[3];
    double y = m[2] - m[1];
    double denom = sqrt(x * x + y * y) + 1e-10;
    double scale = 1.0 / denom;
    double c = x * scale, s = y * scale;
    r[0] = c; r[1] = -s; r[2] = s; r[3] = c;
}

/* 2x2 SVD F = U diag(s) V^T with s >= 0 descending (closed form by the two-angle method). */
static void svd2(const double *F, double *U, double *s, double *V) {
    double a = F[0], b = F[1], c = F[2], d = F[3];
    double E = 0.5 * (a + d), Fh = 0.5 * (a - d), G = 0.5 * (c + b), H = 0.5 * (c - b);
    double Q = sqrt(E * E + H * H), Rr = sqrt(Fh * Fh + G * G);
    double s1 = Q + Rr, s2 = Q - Rr;
    double a1 = atan2(G, Fh), a2 = atan2(H, E);
    double th = 0.5 * (a2 - a1), ph = 0.5 * (a2 + a1);
    /* F = rot(ph) diag(s1, s2) rot(th), so U = rot(ph) and V = rot(th)^T = rot(-th). */
    double cu = cos(ph), su = sin(ph), cv = cos(th), sv = sin(th);
    U[0] = cu; U[1] = -su; U[2] = su; U[3] = cu;
    V[0] = cv; V[1] = sv; V[2] = -sv; V[3] = cv;
    if (s2 < 0) { s2 = -s2; U[1] = -U[1]; U[3] = -U[3]; }
    s[0] = s1; s[1] = s2;
}

/* utils.py:7-49 */
static void hardening_lame(int model, double mu0, double lam0, double h, double Jp, double *mu, double *lam) {
    double e = (model == MODEL_SNOW) ? exp(h * (1.0 - Jp)) : h;
    *mu = mu0 * e;
    *lam = lam0 * e;
}

/* utils.py:95-135: A = -(dt*vol)*(4*inv_dx^2*PF) + m*C,  PF = 2mu(F-R)F^T + lam(J-1)J (scalar on all 9). */
static void stress_affine_3d(const double *F, double inv_dx, double mu, double lam, double dt, double vol,
                             double mass, const double *C, double *A, int model) {
    double J = det3(F);
    double R[9];
    polar3(F, R);
    double Dinv = 4.0 * inv_dx * inv_dx;
    double FmR[9], Ft[9], PF[9];
    for (int i = 0; i < 9; ++i) FmR[i] = 2.0 * mu * (F[i] - R[i]);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Ft[i * 3 + j] = F[j * 3 + i];
    mm3(FmR, Ft, PF);
    double sc = lam * (J - 1.0) * J;
    for (int i = 0; i < 9; ++i) {
        if (model != MODEL_FIXED_COROTATED || i % 4 == 0) PF[i] += sc;
        A[i] = -(dt * vol) * (Dinv * PF[i]) + mass * C[i];
    }
}

/* utils.py:52-92 (2D). */
static void stress_affine_2d(const double *F, double inv_dx, double mu, double lam, double dt, double vol,
                             double mass, const double *C, double *A, int model) {
    double J = det2(F);
    double R[4];
    polar2(F, R);
    double Dinv = 4.0 * inv_dx * inv_dx;
    double FmR[4];
    for (int i = 0; i < 4; ++i) FmR[i] = 2.0 * mu * (F[i] - R[i]);
    double PF[4];
    PF[0] = FmR[0] * F[0] + FmR[1] * F[1];
    PF[1] = FmR[0] * F[2] + FmR[1] * F[3];
    PF[2] = FmR[2] * F[0] + FmR[3] * F[1];
    PF[3] = FmR[2] * F[2] + FmR[3] * F[3];
    double sc = lam * (J - 1.0) * J;
    for (int i = 0; i < 4; ++i)
        A[i] = -(dt * vol) * (Dinv * (PF[i] + ((model != MODEL_FIXED_COROTATED || i % 3 == 0) ? sc : 0.0))) + mass * C[i];
}

/* quadratic B-spline weights, p2g.py:55 */
static void bspline_w(double fx, double *w) {
    w[0] = 0.5 * (1.5 - fx) * (1.5 - fx);
    w[1] = 0.75 - (fx - 1.0) * (fx - 1.0);
    w[2] = 0.5 * (fx - 0.5) * (fx - 0.5);
}

/* base = int64(x*inv_dx - 0.5) truncating toward zero (numpy astype); valid iff base+2 <= res. */
static int base_of(double xs, int res, int64_t *base) {
    double t = xs - 0.5;
    if (!(t > -1.0 && t < (double)res)) return 0; /* also rejects NaN */
    int64_t b = (int64_t)t;
    if (b < 0 || b + 2 > res) return 0;
    *base = b;
    return 1;
}

/* ------------------------------------------------------------------ 3D */

int orc_p2g_3d(double inv_dx, double hardening, double dx, double dt, double volume, int res,
               double *gv, double *gm, int64_t n, const double *x, const double *mass,
               const double *mu0, const double *lam0, const double *v, const double *F,
               const double *C, const double *Jp, int model) {
    const int64_t R = res + 1;
    for (int64_t p = 0; p < n; ++p) {
        int64_t b[3];
        double fx[3], w[3][3];
        for (int d = 0; d < 3; ++d) {
            if (!base_of(x[p * 3 + d] * inv_dx, res, &b[d])) return ORC_OOB;
            fx[d] = x[p * 3 + d] * inv_dx - (double)b[d];
            double ww[3];
            bspline_w(fx[d], ww);
            for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
        }
        double mu, lam, A[9];
        hardening_lame(model, mu0[p], lam0[p], hardening, Jp[p], &mu, &lam);
        stress_affine_3d(&F[p * 9], inv_dx, mu, lam, dt, volume, mass[p], &C[p * 9], A, model);
        double m = mass[p];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    double dpos[3] = {((double)i - fx[0]) * dx, ((double)j - fx[1]) * dx, ((double)k - fx[2]) * dx};
                    double weight = w[i][0] * w[j][1] * w[k][2];
                    int64_t node = ((b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
                    for (int r = 0; r < 3; ++r) {
                        double ad = A[r * 3 + 0] * dpos[0] + A[r * 3 + 1] * dpos[1] + A[r * 3 + 2] * dpos[2];
                        gv[node * 3 + r] += weight * (v[p * 3 + r] * m + ad);
                    }
                    gm[node] += weight * m;
                }
    }
    return ORC_OK;
}

int orc_grid_op_3d(int res, double dx, double dt, double gravity, double *gv, const double *gm) {
    const int64_t R = res + 1;
    const double v_allowed = dx * 0.9 / dt;
    const int boundary = 1;
    for (int64_t i = 0; i < R; ++i)
        for (int64_t j = 0; j < R; ++j)
            for (int64_t k = 0; k < R; ++k) {
                int64_t node = (i * R + j) * R + k;
                double *g = &gv[node * 3];
                if (gm[node] > 0) {
                    for (int d = 0; d < 3; ++d) g[d] /= gm[node];
                    g[1] += dt * gravity;
                    for (int d = 0; d < 3; ++d) g[d] = g[d] < -v_allowed ? -v_allowed : (g[d] > v_allowed ? v_allowed : g[d]);
                }
                int64_t I[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    if (I[d] < boundary) g[d] = 0;
                    if (I[d] >= res - boundary) g[d] = 0;
                }
            }
    return ORC_OK;
}

int orc_g2p_3d(double inv_dx, double dt, int res, const double *gv, int64_t n, double *x, double *v,
               double *F, double *C, double *Jp, int model) {
    const int64_t R = res + 1;
    for (int64_t p = 0; p < n; ++p) {
        int64_t b[3];
        double fx[3], w[3][3];
        for (int d = 0; d < 3; ++d) {
            if (!base_of(x[p * 3 + d] * inv_dx, res, &b[d])) return ORC_OOB;
            fx[d] = x[p * 3 + d] * inv_dx - (double)b[d];
            double ww[3];
            bspline_w(fx[d], ww);
            for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
        }
        double vp[3] = {0, 0, 0}, Cp[9] = {0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    double dpos[3] = {(double)i - fx[0], (double)j - fx[1], (double)k - fx[2]};
                    int64_t node = ((b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
                    const double *g = &gv[node * 3];
                    double weight = w[i][0] * w[j][1] * w[k][2];
                    for (int r = 0; r < 3; ++r) vp[r] += weight * g[r];
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) Cp[r * 3 + c] += 4.0 * inv_dx * ((weight * g[r]) * dpos[c]);
                }
        for (int r = 0; r < 3; ++r) { v[p * 3 + r] = vp[r]; x[p * 3 + r] += dt * vp[r]; }
        memcpy(&C[p * 9], Cp, sizeof(Cp));
        double M[9], Fn[9];
        for (int i = 0; i < 9; ++i) M[i] = ((i % 4 == 0) ? 1.0 : 0.0) + dt * Cp[i];
        mm3(M, &F[p * 9], Fn);
        if (model == MODEL_SNOW) {
            /* g2p.py:48-58.  The clamp rebuilds F from the clamped singular values as U S V^T. */
            double U[9], s[3], V[9];
            svd3(Fn, U, s, V);
            for (int d = 0; d < 3; ++d) s[d] = s[d] < 1.0 - 2.5e-2 ? 1.0 - 2.5e-2 : (s[d] > 1.0 + 7.5e-3 ? 1.0 + 7.5e-3 : s[d]);
            double oldJ = det3(Fn);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double acc = 0;
                    for (int k = 0; k < 3; ++k) acc += U[i * 3 + k] * s[k] * V[j * 3 + k];
                    Fn[i * 3 + j] = acc;
                }
            double det = det3(Fn) + 1e-10;
            double jp = Jp[p] * oldJ / det;
            Jp[p] = jp < 0.6 ? 0.6 : (jp > 20.0 ? 20.0 : jp);
        }
        memcpy(&F[p * 9], Fn, sizeof(Fn));
    }
    return ORC_OK;
}

/* mls_mpm.py:40-79: fresh zero grid, p2g, grid_op, g2p, model fixed to neo_hookean. */
int orc_substep_3d(int res, double inv_dx, double hardening, double dx, double dt, double volume,
                   double gravity, int64_t n, double *x, const double *mass, const double *mu0,
                   const double *lam0, double *v, double *F, double *C, double *Jp, int model) {
    const int64_t R = res + 1;
    double *gv = (double *)calloc((size_t)(R * R * R * 3), sizeof(double));
    double *gm = (double *)calloc((size_t)(R * R * R), sizeof(double));
    if (!gv || !gm) { free(gv); free(gm); return ORC_NOMEM; }
    int st = orc_p2g_3d(inv_dx, hardening, dx, dt, volume, res, gv, gm, n, x, mass, mu0, lam0, v, F, C, Jp, model);
    if (st == ORC_OK) st = orc_grid_op_3d(res, dx, dt, gravity, gv, gm);
    if (st == ORC_OK) st = orc_g2p_3d(inv_dx, dt, res, gv, n, x, v, F, C, Jp, model);
    free(gv);
    free(gm);
    return st;
}

/* ------------------------------------------------------------------ 2D */

int orc_p2g_2d(double inv_dx, double hardening, double mu_0, double lambda_0, double mass, double dx,
               double dt, double volume, int res, double *gv, double *gm, int64_t n, const double *x,
               const double *v, const double *F, const double *C, const double *Jp, int model) {
    const int64_t R = res + 1;
    for (int64_t p = 0; p < n; ++p) {
        int64_t b[2];
        double fx[2], w[3][2];
        for (int d = 0; d < 2; ++d) {
            if (!base_of(x[p * 2 + d] * inv_dx, res, &b[d])) return ORC_OOB;
            fx[d] = x[p * 2 + d] * inv_dx - (double)b[d];
            double ww[3];
            bspline_w(fx[d], ww);
            for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
        }
        double mu, lam, A[4];
        hardening_lame(model, mu_0, lambda_0, hardening, Jp[p], &mu, &lam);
        stress_affine_2d(&F[p * 4], inv_dx, mu, lam, dt, volume, mass, &C[p * 4], A, model);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double dpos[2] = {((double)i - fx[0]) * dx, ((double)j - fx[1]) * dx};
                double weight = w[i][0] * w[j][1];
                int64_t node = (b[0] + i) * R + (b[1] + j);
                for (int r = 0; r < 2; ++r) {
                    double mv = v[p * 2 + r] * mass;
                    double ad = A[r * 2 + 0] * dpos[0] + A[r * 2 + 1] * dpos[1];
                    gv[node * 2 + r] += weight * (mv + ad);
                }
                gm[node] += weight * mass;
            }
    }
    return ORC_OK;
}

int orc_grid_op_2d(int res, double dt, double gravity, double *gv, const double *gm) {
    const int64_t R = res + 1;
    const double boundary = 0.05;
    for (int64_t i = 0; i < R; ++i)
        for (int64_t j = 0; j < R; ++j) {
            int64_t node = i * R + j;
            if (gm[node] > 0) {
                double *g = &gv[node * 2];
                g[0] /= gm[node];
                g[1] /= gm[node];
                g[1] += dt * gravity;
                double xx = (double)i / (double)res, yy = (double)j / (double)res;
                if (xx < boundary || xx > 1 - boundary || yy > 1 - boundary) { g[0] = 0; g[1] = 0; }
                if (yy < boundary) g[1] = g[1] > 0.0 ? g[1] : 0.0;
            }
        }
    return ORC_OK;
}

int orc_g2p_2d(double inv_dx, double dt, int res, const double *gv, int64_t n, double *x, double *v,
               double *F, double *C, double *Jp, int model) {
    const int64_t R = res + 1;
    for (int64_t p = 0; p < n; ++p) {
        int64_t b[2];
        double fx[2], w[3][2];
        for (int d = 0; d < 2; ++d) {
            if (!base_of(x[p * 2 + d] * inv_dx, res, &b[d])) return ORC_OOB;
            fx[d] = x[p * 2 + d] * inv_dx - (double)b[d];
            double ww[3];
            bspline_w(fx[d], ww);
            for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
        }
        double vp[2] = {0, 0}, Cp[4] = {0, 0, 0, 0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double dpos[2] = {(double)i - fx[0], (double)j - fx[1]};
                const double *g = &gv[((b[0] + i) * R + (b[1] + j)) * 2];
                double weight = w[i][0] * w[j][1];
                vp[0] += weight * g[0];
                vp[1] += weight * g[1];
                for (int r = 0; r < 2; ++r)
                    for (int c = 0; c < 2; ++c) Cp[r * 2 + c] += 4.0 * inv_dx * ((weight * g[r]) * dpos[c]);
            }
        v[p * 2 + 0] = vp[0];
        v[p * 2 + 1] = vp[1];
        x[p * 2 + 0] += dt * vp[0];
        x[p * 2 + 1] += dt * vp[1];
        memcpy(&C[p * 4], Cp, sizeof(Cp));
        const double *Fo = &F[p * 4];
        double M[4] = {1.0 + dt * Cp[0], dt * Cp[1], dt * Cp[2], 1.0 + dt * Cp[3]};
        double Fn[4] = {M[0] * Fo[0] + M[1] * Fo[2], M[0] * Fo[1] + M[1] * Fo[3],
                        M[2] * Fo[0] + M[3] * Fo[2], M[2] * Fo[1] + M[3] * Fo[3]};
        /* g2p.py:37-46: SVD always, clamp only for snow, rebuild, Jp update always. */
        double U[4], s[2], V[4];
        svd2(Fn, U, s, V);
        if (model == MODEL_SNOW)
            for (int d = 0; d < 2; ++d) s[d] = s[d] < 1.0 - 2.5e-2 ? 1.0 - 2.5e-2 : (s[d] > 1.0 + 7.5e-3 ? 1.0 + 7.5e-3 : s[d]);
        double oldJ = det2(Fn);
        double Fr[4];
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) Fr[i * 2 + j] = U[i * 2 + 0] * s[0] * V[j * 2 + 0] + U[i * 2 + 1] * s[1] * V[j * 2 + 1];
        double det = det2(Fr) + 1e-10;
        double jp = Jp[p] * oldJ / det;
        Jp[p] = jp < 0.6 ? 0.6 : (jp > 20.0 ? 20.0 : jp);
        memcpy(&F[p * 4], Fr, sizeof(Fr));
    }
    return ORC_OK;
}

int orc_substep_2d(int res, double inv_dx, double hardening, double mu_0, double lambda_0, double mass,
                   double dx, double dt, double volume, double gravity, int64_t n, double *x, double *v,
                   double *F, double *C, double *Jp, int model) {
    const int64_t R = res + 1;
    double *gv = (double *)calloc((size_t)(R * R * 2), sizeof(double));
    double *gm = (double *)calloc((size_t)(R * R), sizeof(double));
    if (!gv || !gm) { free(gv); free(gm); return ORC_NOMEM; }
    int st = orc_p2g_2d(inv_dx, hardening, mu_0, lambda_0, mass, dx, dt, volume, res, gv, gm, n, x, v, F, C, Jp, model);
    if (st == ORC_OK) st = orc_grid_op_2d(res, dt, gravity, gv, gm);
    if (st == ORC_OK) st = orc_g2p_2d(inv_dx, dt, res, gv, n, x, v, F, C, Jp, model);
    free(gv);
    free(gm);
    return st;
}

/* ------------------------------------------------------------------ helpers exposed for KATs */

void orc_bspline_weights(double fx, double *w3) { bspline_w(fx, w3); }
void orc_polar_3d(const double *F, double *R) { polar3(F, R); }
void orc_polar_2d(const double *F, double *R) { polar2(F, R); }
void orc_svd_3d(const double *F, double *U, double *s, double *V) { svd3(F, U, s, V); }
void orc_stress_affine_3d(const double *F, double inv_dx, double mu, double lam, double dt, double vol,
                          double mass, const double *C, double *A) {
    stress_affine_3d(F, inv_dx, mu, lam, dt, vol, mass, C, A, 0);
}
void orc_stress_affine_2d(const double *F, double inv_dx, double mu, double lam, double dt, double vol,
                          double mass, const double *C, double *A) {
    stress_affine_2d(F, inv_dx, mu, lam, dt, vol, mass, C, A, 0);
}

/* ------------------------------------------------------------------ multi-threaded timing variant
 * Same arithmetic as orc_substep_3d with the particle loops split across OpenMP threads and the
 * P2G scatter done with atomic adds.  Summation order differs from the serial oracle, so this
 * variant is only used to time the CPU path on all host cores, never as a parity reference. */
int orc_substep_3d_par(int res, double inv_dx, double hardening, double dx, double dt, double volume,
                       double gravity, int64_t n, double *x, const double *mass, const double *mu0,
                       const double *lam0, double *v, double *F, double *C, double *Jp, int model,
                       int nthreads, double *grid_scratch /* R^3*4 doubles, or NULL */) {
    const int64_t R = res + 1;
    const int64_t nn = R * R * R;
    double *g = grid_scratch ? grid_scratch : (double *)malloc((size_t)(nn * 4) * sizeof(double));
    if (!g) return ORC_NOMEM;
    double *gv = g, *gm = g + nn * 3;
    int st = ORC_OK;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nn * 4; ++i) g[i] = 0.0;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        int64_t b[3];
        double fx[3], w[3][3];
        int ok = 1;
        for (int d = 0; d < 3; ++d) {
            if (!base_of(x[p * 3 + d] * inv_dx, res, &b[d])) { ok = 0; break; }
            fx[d] = x[p * 3 + d] * inv_dx - (double)b[d];
            double ww[3];
            bspline_w(fx[d], ww);
            for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
        }
        if (!ok) {
#pragma omp atomic write
            st = ORC_OOB;
            continue;
        }
        double mu, lam, A[9];
        hardening_lame(model, mu0[p], lam0[p], hardening, Jp[p], &mu, &lam);
        stress_affine_3d(&F[p * 9], inv_dx, mu, lam, dt, volume, mass[p], &C[p * 9], A, model);
        double m = mass[p];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    double dpos[3] = {((double)i - fx[0]) * dx, ((double)j - fx[1]) * dx, ((double)k - fx[2]) * dx};
                    double weight = w[i][0] * w[j][1] * w[k][2];
                    int64_t node = ((b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
                    for (int r = 0; r < 3; ++r) {
                        double ad = A[r * 3 + 0] * dpos[0] + A[r * 3 + 1] * dpos[1] + A[r * 3 + 2] * dpos[2];
                        double add = weight * (v[p * 3 + r] * m + ad);
#pragma omp atomic update
                        gv[node * 3 + r] += add;
                    }
                    double addm = weight * m;
#pragma omp atomic update
                    gm[node] += addm;
                }
    }
    if (st == ORC_OK) {
        const double v_allowed = dx * 0.9 / dt;
#pragma omp parallel for schedule(static)
        for (int64_t node = 0; node < nn; ++node) {
            int64_t i = node / (R * R), j = (node / R) % R, k = node % R;
            double *gg = &gv[node * 3];
            if (gm[node] > 0) {
                for (int d = 0; d < 3; ++d) gg[d] /= gm[node];
                gg[1] += dt * gravity;
                for (int d = 0; d < 3; ++d) gg[d] = gg[d] < -v_allowed ? -v_allowed : (gg[d] > v_allowed ? v_allowed : gg[d]);
            }
            int64_t I[3] = {i, j, k};
            for (int d = 0; d < 3; ++d)
                if (I[d] < 1 || I[d] >= res - 1) gg[d] = 0;
        }
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; ++p) {
            int64_t b[3];
            double fx[3], w[3][3];
            for (int d = 0; d < 3; ++d) {
                base_of(x[p * 3 + d] * inv_dx, res, &b[d]);
                fx[d] = x[p * 3 + d] * inv_dx - (double)b[d];
                double ww[3];
                bspline_w(fx[d], ww);
                for (int i = 0; i < 3; ++i) w[i][d] = ww[i];
            }
            double vp[3] = {0, 0, 0}, Cp[9] = {0};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) {
                        double dpos[3] = {(double)i - fx[0], (double)j - fx[1], (double)k - fx[2]};
                        int64_t node = ((b[0] + i) * R + (b[1] + j)) * R + (b[2] + k);
                        const double *gg = &gv[node * 3];
                        double weight = w[i][0] * w[j][1] * w[k][2];
                        for (int r = 0; r < 3; ++r) vp[r] += weight * gg[r];
                        for (int r = 0; r < 3; ++r)
                            for (int c = 0; c < 3; ++c) Cp[r * 3 + c] += 4.0 * inv_dx * ((weight * gg[r]) * dpos[c]);
                    }
            for (int r = 0; r < 3; ++r) { v[p * 3 + r] = vp[r]; x[p * 3 + r] += dt * vp[r]; }
            memcpy(&C[p * 9], Cp, sizeof(Cp));
            double M[9], Fn[9];
            for (int i = 0; i < 9; ++i) M[i] = ((i % 4 == 0) ? 1.0 : 0.0) + dt * Cp[i];
            mm3(M, &F[p * 9], Fn);
            memcpy(&F[p * 9], Fn, sizeof(Fn));
        }
    }
    if (!grid_scratch) free(g);
    return st;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_svd_2d(const double *F, double *U, double *s, double *V) { svd2(F, U, s, V); }

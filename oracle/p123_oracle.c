/*
 * p123_oracle.c -- CPU restatement of ParaFEM's p123 (3-D Laplace, 8-node
 * bricks, Jacobi-preconditioned CG, element by element).
 *
 * TEST INFRASTRUCTURE ONLY, like p121_oracle.c: only the test suite, the
 * smoke check and the CPU baseline leg of the benchmark load it.
 *
 * Layouts follow the Fortran arrays of p123:
 *   coord(8,3)           coord[i + 8*d]
 *   g_coord(8,3,nels)    g_coord[i + 8*d + 24*e]
 *   g_num(8,nels)        g_num[i + 8*e]             (1-based node ids)
 *   g_g(8,nels)          g_g[i + 8*e]               (1-based eqs, 0 = fixed)
 *   storkc(8,8,nels)     storkc[i + 8*j + 64*e]
 *   rest(nr,2)           rest[r*2 + k]  (row-major here: node, flag)
 * and the file is compiled with -ffp-contract=off (Fortran evaluation order,
 * no fused multiply-add).
 *
 * Parity pin: the restatement reproduces the reference's recorded book run
 * (examples/5th_ed/p123/book/p123.res: 8,120,601 nodes, 120,601 restrained,
 * 8,000,000 equations, 180 iterations, total load 10, four potentials).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_sample(int nip, double *s, double *wt, int exact_weights);   /* p121_oracle.c */
double orc_determinant(const double *j);
void orc_invert3(double *m);

/* GEOMETRY_8BXZ (src/modules/shared/geometry.f90:70-166): boxes of 8-node
 * bricks counting x-z planes in the y-direction. */
void orc_geometry_8bxz(int iel, int nxe, int nze, double aa, double bb, double cc, double *coord, int *num)
{
    int iq = (iel - 1) / (nxe * nze) + 1;
    int iplane = iel - (iq - 1) * nxe * nze;
    int is = (iplane - 1) / nxe + 1;
    int ip = iplane - (is - 1) * nxe;
    num[0] = (iq - 1) * (nxe + 1) * (nze + 1) + is * (nxe + 1) + ip;
    num[1] = num[0] - nxe - 1;
    num[2] = num[1] + 1;
    num[3] = num[0] + 1;
    num[4] = num[0] + (nxe + 1) * (nze + 1);
    num[5] = num[4] - nxe - 1;
    num[6] = num[5] + 1;
    num[7] = num[4] + 1;
#define CO(i, d) coord[((i) - 1) + 8 * ((d) - 1)]
    CO(1, 1) = (ip - 1) * aa; CO(2, 1) = (ip - 1) * aa; CO(5, 1) = (ip - 1) * aa; CO(6, 1) = (ip - 1) * aa;
    CO(3, 1) = ip * aa; CO(4, 1) = ip * aa; CO(7, 1) = ip * aa; CO(8, 1) = ip * aa;
    CO(1, 2) = (iq - 1) * bb; CO(2, 2) = (iq - 1) * bb; CO(3, 2) = (iq - 1) * bb; CO(4, 2) = (iq - 1) * bb;
    CO(5, 2) = iq * bb; CO(6, 2) = iq * bb; CO(7, 2) = iq * bb; CO(8, 2) = iq * bb;
    CO(1, 3) = -is * cc; CO(4, 3) = -is * cc; CO(5, 3) = -is * cc; CO(8, 3) = -is * cc;
    CO(2, 3) = -(is - 1) * cc; CO(3, 3) = -(is - 1) * cc; CO(6, 3) = -(is - 1) * cc; CO(7, 3) = -(is - 1) * cc;
#undef CO
}

/* box_bc8 (src/modules/shared/geometry.f90:655-696): in every x-z plane but
 * the last, the nodes numbered a multiple of nxe+1 (the last x column) and
 * the first nxe (the top row); the whole last plane; flag 0 = fixed.
 * Returns the number of rows written. */
int orc_box_bc8(int nxe, int nye, int nze, int *rest)
{
    int face = (nxe + 1) * (nze + 1), count = 0;
    for (int i = 0; i <= nye - 1; ++i)
        for (int j = i * face + 1; j <= (i + 1) * face; ++j)
            if (j / (nxe + 1) * (nxe + 1) == j || j < i * face + nxe + 1) {
                rest[2 * count] = j;
                rest[2 * count + 1] = 0;
                ++count;
            }
    for (int j = nye * face + 1; j <= (nye + 1) * face; ++j) {
        rest[2 * count] = j;
        rest[2 * count + 1] = 0;
        ++count;
    }
    return count;
}

/* rearrange_2 (src/modules/shared/new_library.f90:3118-3124) */
void orc_rearrange_2(int nr, int *rest)
{
    for (int i = 1; i <= nr; ++i) rest[2 * (i - 1) + 1] = rest[2 * (i - 1)] - i;
    int m = 0;
    for (int i = 1; i <= nr; ++i)
        if (rest[2 * (i - 1) + 1] != 0) { m = i - 1; break; }
    for (int i = (m > 0 ? m : 1); i <= nr; ++i) rest[2 * (i - 1) + 1] += 1;
}

/* find_g4 (src/modules/shared/new_library.f90:3249-3271): one freedom per
 * node, binary search in the rearranged rest. */
void orc_find_g4(const int *num, int nod, int *g, int nr, const int *rest)
{
    for (int i = 0; i < nod; ++i) {
        int l = num[i], first = 1, last = nr;
        if (nr < 1) {   /* no restrained node (outside find_g4's domain): node = equation */
            g[i] = l;
            continue;
        }
        while (first != last) {
            int half = (first + last) / 2;
            if (l <= rest[2 * (half - 1)]) last = half;
            else first = half + 1;
        }
        int only = first;
        if (l == rest[2 * (only - 1)]) {
            g[i] = 0;
        } else {
            int s1 = only - 1;
            int s2 = rest[2 * (s1 - 1) + 1];
            int s3 = l - rest[2 * (s1 - 1)];
            g[i] = s2 + s3 - 1;
        }
    }
}

/* ABAQUS2SG, 8-node hexahedron (src/modules/shared/new_library.f90:3604-3618) */
void orc_abaqus2sg8(int nels, int *g_num)
{
    static const int map[8] = {1, 5, 6, 2, 4, 8, 7, 3};
    int t[8];
    for (int e = 0; e < nels; ++e) {
        int *g = &g_num[8 * e];
        memcpy(t, g, sizeof t);
        for (int i = 0; i < 8; ++i) g[i] = t[map[i] - 1];
    }
}

/* SHAPE_DER, 3-D 8-node brick (src/modules/shared/new_library.f90:769-793).  der(3,8). */
void orc_shape_der8(double *der, double xi, double eta, double zeta)
{
    double etam = 1.0 - eta, xim = 1.0 - xi, zetam = 1.0 - zeta;
    double etap = eta + 1.0, xip = xi + 1.0, zetap = zeta + 1.0;
#define D(a, b) der[((a) - 1) + 3 * ((b) - 1)]
    D(1, 1) = -0.125 * etam * zetam; D(1, 2) = -0.125 * etam * zetap;
    D(1, 3) = 0.125 * etam * zetap;  D(1, 4) = 0.125 * etam * zetam;
    D(1, 5) = -0.125 * etap * zetam; D(1, 6) = -0.125 * etap * zetap;
    D(1, 7) = 0.125 * etap * zetap;  D(1, 8) = 0.125 * etap * zetam;
    D(2, 1) = -0.125 * xim * zetam;  D(2, 2) = -0.125 * xim * zetap;
    D(2, 3) = -0.125 * xip * zetap;  D(2, 4) = -0.125 * xip * zetam;
    D(2, 5) = 0.125 * xim * zetam;   D(2, 6) = 0.125 * xim * zetap;
    D(2, 7) = 0.125 * xip * zetap;   D(2, 8) = 0.125 * xip * zetam;
    D(3, 1) = -0.125 * xim * etam;   D(3, 2) = 0.125 * xim * etam;
    D(3, 3) = 0.125 * xip * etam;    D(3, 4) = -0.125 * xip * etam;
    D(3, 5) = -0.125 * xim * etap;   D(3, 6) = 0.125 * xim * etap;
    D(3, 7) = 0.125 * xip * etap;    D(3, 8) = -0.125 * xip * etap;
#undef D
}

/* Element conductivity integration (src/programs/5th_ed/p123/p123.f90:70-85):
 * kcx += MATMUL(col,row)*det*weights(i) with col = row = deriv(1,:), likewise
 * kcy, kcz; storkc = kcx*kx + kcy*ky + kcz*kz. */
void orc_form_storkc(int nels, int nip, const double *g_coord, double kx, double ky, double kz, double *storkc)
{
    double *pts = (double *)malloc(sizeof(double) * nip * 3);
    double *wts = (double *)malloc(sizeof(double) * nip);
    orc_sample(nip, pts, wts, 0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nels; ++e) {
        const double *coord = &g_coord[(size_t)24 * e];
        double kc[3][64], der[24], jac[9], deriv[24];
        memset(kc, 0, sizeof kc);
        for (int i = 0; i < nip; ++i) {
            orc_shape_der8(der, pts[i], pts[i + nip], pts[i + 2 * nip]);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int k = 0; k < 8; ++k) s += der[a + 3 * k] * coord[k + 8 * b];
                    jac[a + 3 * b] = s;
                }
            double det = orc_determinant(jac);
            orc_invert3(jac);
            for (int l = 0; l < 8; ++l)
                for (int a = 0; a < 3; ++a) {
                    double s = 0.0;
                    for (int k = 0; k < 3; ++k) s += jac[a + 3 * k] * der[k + 3 * l];
                    deriv[a + 3 * l] = s;
                }
            for (int d = 0; d < 3; ++d)
                for (int c = 0; c < 8; ++c)
                    for (int r = 0; r < 8; ++r)
                        kc[d][r + 8 * c] = kc[d][r + 8 * c] + deriv[d + 3 * r] * deriv[d + 3 * c] * det * wts[i];
        }
        double *out = &storkc[(size_t)64 * e];
        for (int k = 0; k < 64; ++k) out[k] = kc[0][k] * kx + kc[1][k] * ky + kc[2][k] * kz;
    }
    free(pts);
    free(wts);
}

/* Jacobi diagonal (p123.f90:87-94): SCATTER of the element diagonals.
 * kc_stride 64: storkc per element; 0: one shared storkc. */
void orc_diag8(int nels, int neq, const int *g_g, const double *storkc, int kc_stride, double *diag)
{
    double *d0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    for (int e = 0; e < nels; ++e)
        for (int i = 0; i < 8; ++i) {
            int q = g_g[8 * e + i];
            d0[q] = d0[q] + storkc[(size_t)kc_stride * e + 9 * i];
        }
    memcpy(diag, d0 + 1, sizeof(double) * neq);
    free(d0);
}

/* The p123 PCG (p123.f90:121-148) with checon_par (src/modules/mpi/maths.f90:
 * 999-1069).  diag: assembled diagonal with the penalty of the fixed
 * freedoms already added (inverted here, :110); r: starting r (loads and
 * store*value of fixed freedoms).  Fixed freedoms fix_eq (1-based) get
 * u = p*store after the scatter (:127-131).  Returns iterations. */
int orc_pcg123(int nels, int neq, const int *g_g, const double *storkc, int kc_stride, const double *diag,
               const double *rhs, int nfix, const int *fix_eq, const double *fix_store, double tol, int limit,
               double *x_out, double *final_metric)
{
    size_t n1 = (size_t)neq + 1;
    double *dinv = (double *)malloc(sizeof(double) * n1);
    double *r = (double *)calloc(n1, sizeof(double));
    double *d = (double *)calloc(n1, sizeof(double));
    double *p = (double *)calloc(n1, sizeof(double));
    double *u = (double *)calloc(n1, sizeof(double));
    double *x = (double *)calloc(n1, sizeof(double));
    double *xnew = (double *)calloc(n1, sizeof(double));
    double *ut = (double *)malloc(sizeof(double) * 8 * (size_t)nels);
    dinv[0] = 0.0;
    for (int q = 1; q <= neq; ++q) { dinv[q] = 1.0 / diag[q - 1]; r[q] = rhs[q - 1]; }
    for (int q = 1; q <= neq; ++q) d[q] = dinv[q] * r[q];
    for (int q = 1; q <= neq; ++q) p[q] = d[q];
    int iters = 0;
    double metric = 0.0;
    for (;;) {
        ++iters;
        for (size_t q = 0; q < n1; ++q) u[q] = 0.0;
        p[0] = 0.0;
#pragma omp parallel for schedule(static)
        for (int e = 0; e < nels; ++e) {
            const double *kc = &storkc[(size_t)kc_stride * e];
            double pe[8], acc[8];
            for (int i = 0; i < 8; ++i) { pe[i] = p[g_g[8 * e + i]]; acc[i] = 0.0; }
            for (int j = 0; j < 8; ++j)
                for (int i = 0; i < 8; ++i) acc[i] = acc[i] + kc[i + 8 * j] * pe[j];
            memcpy(&ut[8 * (size_t)e], acc, sizeof acc);
        }
        for (int e = 0; e < nels; ++e)
            for (int i = 0; i < 8; ++i) {
                int q = g_g[8 * e + i];
                u[q] = u[q] + ut[8 * (size_t)e + i];
            }
        u[0] = 0.0;
        for (int i = 0; i < nfix; ++i) u[fix_eq[i]] = p[fix_eq[i]] * fix_store[i];
        double up = 0.0, pu = 0.0;
        for (int q = 1; q <= neq; ++q) up += r[q] * d[q];
        for (int q = 1; q <= neq; ++q) pu += p[q] * u[q];
        double alpha = up / pu;
        for (int q = 1; q <= neq; ++q) xnew[q] = x[q] + p[q] * alpha;
        for (int q = 1; q <= neq; ++q) r[q] = r[q] - u[q] * alpha;
        for (int q = 1; q <= neq; ++q) d[q] = dinv[q] * r[q];
        double rd = 0.0;
        for (int q = 1; q <= neq; ++q) rd += r[q] * d[q];
        double beta = rd / up;
        for (int q = 1; q <= neq; ++q) p[q] = d[q] + p[q] * beta;
        double maxl = 0.0, maxd = 0.0;
        for (int q = 1; q <= neq; ++q) {
            double a = fabs(xnew[q]);
            if (a > maxl) maxl = a;
            double b = fabs(xnew[q] - x[q]);
            if (b > maxd) maxd = b;
        }
        metric = maxd / maxl;
        int converged = metric <= tol;
        for (int q = 1; q <= neq; ++q) x[q] = xnew[q];
        if (converged || iters == limit) break;
    }
    memcpy(x_out, xnew + 1, sizeof(double) * neq);
    if (final_metric) *final_metric = metric;
    free(dinv); free(r); free(d); free(p); free(u); free(x); free(xnew); free(ut);
    return iters;
}

/* One product u = K p over equations (the loop body of p123.f90:124-131
 * without the fixed-freedom override). */
void orc_ebe_matvec8(int nels, int neq, const int *g_g, const double *storkc, int kc_stride, const double *p,
                     double *u)
{
    double *p0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    double *u0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    memcpy(p0 + 1, p, sizeof(double) * neq);
    for (int e = 0; e < nels; ++e) {
        const double *kc = &storkc[(size_t)kc_stride * e];
        double pe[8], acc[8];
        for (int i = 0; i < 8; ++i) { pe[i] = p0[g_g[8 * e + i]]; acc[i] = 0.0; }
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 8; ++i) acc[i] = acc[i] + kc[i + 8 * j] * pe[j];
        for (int i = 0; i < 8; ++i) {
            int q = g_g[8 * e + i];
            u0[q] = u0[q] + acc[i];
        }
    }
    memcpy(u, u0 + 1, sizeof(double) * neq);
    free(p0);
    free(u0);
}

/* Every element of the box (the p12meshgen p123 loop, p12meshgen.f90:698-701);
 * g_coord may be NULL. */
void orc_mesh_box8(int nxe, int nye, int nze, double aa, double bb, double cc, int *g_num, double *g_coord)
{
    long long nels = (long long)nxe * nye * nze;
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < nels; ++e) {
        double co[24];
        orc_geometry_8bxz((int)e + 1, nxe, nze, aa, bb, cc, co, &g_num[8 * e]);
        if (g_coord) memcpy(&g_coord[24 * e], co, sizeof co);
    }
}

/* find_g4 for every element (p123.f90:49-53) with the rearranged rest. */
void orc_steering8(int nels, const int *g_num, int nr, const int *rest, int *g_g)
{
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nels; ++e) orc_find_g4(&g_num[8 * (size_t)e], 8, &g_g[8 * (size_t)e], nr, rest);
}

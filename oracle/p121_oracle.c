/*
 * p121_oracle.c -- CPU restatement of ParaFEM's p121 solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * checked against.  Only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark may load it; the product library never
 * links or calls it.
 *
 * Every routine restates the algorithm of the Fortran routine it cites
 * (paths relative to the ParaFEM source tree).  Arrays follow the Fortran
 * column-major layouts of p121 so that the cited loops read the same:
 *   coord(20,3)          coord[i + 20*d]
 *   g_coord(20,3,nels)   g_coord[i + 20*d + 60*e]
 *   g_num(20,nels)       g_num[i + 20*e]            (1-based node ids)
 *   g_g(60,nels)         g_g[i + 60*e]              (1-based eqs, 0 = fixed)
 *   storkm(60,60,nels)   storkm[i + 60*j + 3600*e]
 *   rest(nr,4)           rest[r*4 + k]  (row-major here: node, fx, fy, fz)
 *
 * Floating-point expressions keep the Fortran evaluation order and the
 * file is compiled with -ffp-contract=off (no fused multiply-add), the
 * way gfortran evaluates them on x86-64 without -mfma.
 *
 * Parity pin: the restatement reproduces the reference's own golden run
 * (examples/5th_ed/p121/demo: p121_demo.res and p121_demo.ensi.DISPL-000001).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Mesh generation: geometry.f90 GEOMETRY_20BXZ (src/modules/shared/geometry.f90:172-290) */
void orc_geometry_20bxz(int iel, int nxe, int nze, double aa, double bb, double cc,
                        double *coord, int *num)
{
    int iq = (iel - 1) / (nxe * nze) + 1;
    int iplane = iel - (iq - 1) * nxe * nze;
    int is = (iplane - 1) / nxe + 1;
    int ip = iplane - (is - 1) * nxe;
    int fac1 = ((2 * nxe + 1) * (nze + 1) + (2 * nze + 1) * (nxe + 1)) * (iq - 1);
    int fac2 = ((2 * nxe + 1) * (nze + 1) + (2 * nze + 1) * (nxe + 1)) * iq;
#define NUM(k) num[(k) - 1]
#define CO(i, d) coord[((i) - 1) + 20 * ((d) - 1)]
    NUM(1) = fac1 + (3 * nxe + 2) * is + 2 * ip - 1;
    NUM(2) = fac1 + (3 * nxe + 2) * is - nxe + ip - 1;
    NUM(3) = NUM(1) - 3 * nxe - 2;
    NUM(4) = NUM(3) + 1;
    NUM(5) = NUM(4) + 1;
    NUM(6) = NUM(2) + 1;
    NUM(7) = NUM(1) + 2;
    NUM(8) = NUM(1) + 1;
    NUM(9) = fac2 - (nxe + 1) * (nze + 1) + (nxe + 1) * is + ip;
    NUM(10) = NUM(9) - nxe - 1;
    NUM(11) = NUM(10) + 1;
    NUM(12) = NUM(9) + 1;
    NUM(13) = fac2 + (3 * nxe + 2) * is + 2 * ip - 1;
    NUM(14) = fac2 + (3 * nxe + 2) * is - nxe + ip - 1;
    NUM(15) = NUM(13) - 3 * nxe - 2;
    NUM(16) = NUM(15) + 1;
    NUM(17) = NUM(16) + 1;
    NUM(18) = NUM(14) + 1;
    NUM(19) = NUM(13) + 2;
    NUM(20) = NUM(13) + 1;
    double x0 = (ip - 1) * aa, x1 = ip * aa;
    for (int i = 1; i <= 3; ++i) CO(i, 1) = x0;
    CO(9, 1) = x0; CO(10, 1) = x0;
    for (int i = 13; i <= 15; ++i) CO(i, 1) = x0;
    for (int i = 5; i <= 7; ++i) CO(i, 1) = x1;
    CO(11, 1) = x1; CO(12, 1) = x1;
    for (int i = 17; i <= 19; ++i) CO(i, 1) = x1;
    CO(4, 1) = .5 * (CO(3, 1) + CO(5, 1));
    CO(8, 1) = .5 * (CO(1, 1) + CO(7, 1));
    CO(16, 1) = .5 * (CO(15, 1) + CO(17, 1));
    CO(20, 1) = .5 * (CO(13, 1) + CO(19, 1));
    for (int i = 1; i <= 8; ++i) CO(i, 2) = (iq - 1) * bb;
    for (int i = 13; i <= 20; ++i) CO(i, 2) = iq * bb;
    CO(9, 2) = .5 * (CO(1, 2) + CO(13, 2));
    CO(10, 2) = .5 * (CO(3, 2) + CO(15, 2));
    CO(11, 2) = .5 * (CO(5, 2) + CO(17, 2));
    CO(12, 2) = .5 * (CO(7, 2) + CO(19, 2));
    double zb = -is * cc, zt = -(is - 1) * cc;
    CO(1, 3) = zb;
    for (int i = 7; i <= 9; ++i) CO(i, 3) = zb;
    CO(12, 3) = zb; CO(13, 3) = zb; CO(19, 3) = zb; CO(20, 3) = zb;
    for (int i = 3; i <= 5; ++i) CO(i, 3) = zt;
    CO(10, 3) = zt; CO(11, 3) = zt;
    for (int i = 15; i <= 17; ++i) CO(i, 3) = zt;
    CO(2, 3) = .5 * (CO(1, 3) + CO(3, 3));
    CO(6, 3) = .5 * (CO(5, 3) + CO(7, 3));
    CO(14, 3) = .5 * (CO(13, 3) + CO(15, 3));
    CO(18, 3) = .5 * (CO(17, 3) + CO(19, 3));
#undef NUM
#undef CO
}

/* cube_bc20 (src/modules/shared/geometry.f90:425-504).  rest row-major
 * (node, fx, fy, fz); returns the number of rows written. */
int orc_cube_bc20(int nxe, int nye, int nze, int *rest)
{
    int face1 = 3 * nxe * nze + 2 * (nxe + nze) + 1;
    int face2 = (nxe + 1) * (nze + 1);
    int face = face1 + face2;
    int l = nze * (nxe + 1);
    int m = 3 * nxe + 2;
    int n = 3 * nxe * nze + 2 * nze;
    int count = 0;
#define PUT(j, a, b, c) do { rest[count*4+0] = (j); rest[count*4+1] = (a); \
        rest[count*4+2] = (b); rest[count*4+3] = (c); ++count; } while (0)
    for (int i = 0; i <= nye; ++i) {
        for (int j = i * face + 1; j <= i * face + face1; ++j) {
            int k = j - i * face;
            if (i == 0 || i == nye) {
                if ((k + m - 1) / m * m == (k + m - 1) && k <= n) PUT(j, 0, 0, 1);
                else if ((k + nxe + 1) / m * m == (k + nxe + 1) && k <= n) PUT(j, 0, 0, 1);
                else if ((k + nxe) / m * m == (k + nxe) && k <= n) PUT(j, 0, 0, 1);
                else if (k / m * m == k && k <= n) PUT(j, 0, 0, 1);
                else if (k <= n) PUT(j, 1, 0, 1);
                else if (k > n) PUT(j, 0, 0, 0);
            } else {
                if ((k + m - 1) / m * m == (k + m - 1) && k <= n) PUT(j, 0, 1, 1);
                else if ((k + nxe + 1) / m * m == (k + nxe + 1) && k <= n) PUT(j, 0, 1, 1);
                else if ((k + nxe) / m * m == (k + nxe) && k <= n) PUT(j, 0, 1, 1);
                else if (k / m * m == k && k <= n) PUT(j, 0, 1, 1);
                else if (k > n) PUT(j, 0, 0, 0);
            }
        }
        if (i < nye) {
            for (int j = i * face + face1 + 1; j <= (i + 1) * face; ++j) {
                int k = j - (face1 + i * face);
                if ((k + nxe) / (nxe + 1) * (nxe + 1) == (k + nxe) && k <= l) PUT(j, 0, 1, 1);
                else if (k / (nxe + 1) * (nxe + 1) == k && k <= l) PUT(j, 0, 1, 1);
                else if (k > l) PUT(j, 0, 0, 0);
            }
        }
    }
#undef PUT
    return count;
}

/* load_p121, 20-node case (src/modules/mpi/loading.f90:386-480).  Writes
 * 3*nle*nle+4*nle+1 (node, value) pairs; returns the count. */
int orc_load_p121(int nle, int nxe, int nze, int *node, double *val)
{
    int f1 = (2 * nxe + 1) * (nze + 1) + (nxe + 1) * nze;
    int f2 = (nxe + 1) * (nze + 1);
    int c = 0;
    for (int i = 1; i <= 2 * nle + 1; ++i) {
        node[c] = i;
        if (i == 1 || i == 2 * nle + 1) val[c] = -1.0;
        else if (i % 2 == 0) val[c] = 4.0;
        else val[c] = -2.0;
        ++c;
    }
    for (int j = 0; j <= nle - 1; ++j) {
        for (int i = 1; i <= nle + 1; ++i) {
            node[c] = i + f1 + j * (f1 + f2);
            val[c] = (i == 1 || i == nle + 1) ? 4.0 : 8.0;
            ++c;
        }
        for (int i = 1; i <= 2 * nle + 1; ++i) {
            node[c] = i + f1 + (j + 1) * f2 + j * f1;
            if (j != nle - 1) {
                if (i == 1 || i == 2 * nle + 1) val[c] = -2.0;
                else if (i % 2 == 0) val[c] = 8.0;
                else val[c] = -4.0;
            } else {
                if (i == 1 || i == 2 * nle + 1) val[c] = -1.0;
                else if (i % 2 == 0) val[c] = 4.0;
                else val[c] = -2.0;
            }
            ++c;
        }
    }
    return c;
}

/* ------------------------------------------------------------------ */
/* Steering: REARRANGE (src/modules/shared/new_library.f90:3059-3112) */
void orc_rearrange(int nr, int *rest)
{
    int m = 0;
    for (int i = 0; i < nr; ++i)
        for (int k = 1; k <= 3; ++k)
            if (rest[i * 4 + k] != 0) rest[i * 4 + k] = ++m;
    for (int i = 0; i < nr; ++i) {
        int k = rest[i * 4];
        for (int mm = 1; mm <= 3; ++mm)
            if (rest[i * 4 + mm] != 0) rest[i * 4 + mm] += 3 * (k - (i + 1));
    }
}

/* find_g3 (src/modules/shared/new_library.f90:3130-3212).  The reference
 * reads rest(0,:) when a node precedes the first listed node; here that
 * case numbers the node as if every earlier node were free. */
void orc_find_g3(const int *num, int *g, int nr, const int *rest)
{
    for (int i = 1; i <= 20; ++i) {
        int l = num[i - 1];
        int first = 1, last = nr;
        if (nr < 1) {   /* no restrained node (outside find_g3's domain): all freedoms free */
            for (int j = 1; j <= 3; ++j) g[3 * i - 3 + j - 1] = 3 * (l - 1) + j;
            continue;
        }
        while (first != last) {
            int half = (first + last) / 2;
            if (l <= rest[(half - 1) * 4]) last = half;
            else first = half + 1;
        }
        int only = first;
        const int *ro = &rest[(only - 1) * 4];
        if (l == ro[0]) {
            for (int j = 1; j <= 3; ++j) g[3 * i - 3 + j - 1] = ro[j];
        } else {
            int k = (only == nr) ? 0 : 1;
            int s1;
            for (;;) {
                s1 = only - k;
                if (s1 < 1) break;
                const int *rs = &rest[(s1 - 1) * 4];
                if (rs[1] + rs[2] + rs[3] != 0 || s1 == 1) break;
                ++k;
            }
            if (s1 < 1) {
                for (int j = 1; j <= 3; ++j) g[3 * i - 3 + j - 1] = 3 * (l - 1) + j;
                continue;
            }
            const int *rs = &rest[(s1 - 1) * 4];
            int s2 = rs[1];
            if (rs[2] > s2) s2 = rs[2];
            if (rs[3] > s2) s2 = rs[3];
            int s3 = (only == nr) ? l - rs[0] - k : l - rs[0] - (k - 1);
            for (int j = 1; j <= 3; ++j) g[3 * i - 3 + j - 1] = s2 + 3 * s3 - (3 - j);
        }
    }
}

/* ABAQUS2SG, 20-node hexahedron (src/modules/shared/new_library.f90:3569-3597) */
void orc_abaqus2sg(int nels, int *g_num)
{
    static const int map[20] = {4, 12, 1, 9, 2, 10, 3, 11, 20, 17, 18, 19, 8, 16, 5, 13, 6, 14, 7, 15};
    int t[20];
    for (int e = 0; e < nels; ++e) {
        int *g = &g_num[20 * e];
        memcpy(t, g, sizeof t);
        for (int i = 0; i < 20; ++i) g[i] = t[map[i] - 1];
    }
}

/* ------------------------------------------------------------------ */
/* SAMPLE, hexahedron nip=8 and nip=27 (src/modules/shared/new_library.f90:1397-1514).
 * s(nip,3) column-major: s[i + nip*d].  With exact_weights==0 the 27-point
 * weights carry the default-REAL factors 5./9. and 8./9. of the reference
 * (wt = (/5./9.*v,8./9.*v,5./9.*v/) at :1493). */
int orc_sample(int nip, double *s, double *wt, int exact_weights)
{
    double root3 = 1.0 / sqrt(3.0);
    double r15 = 0.2 * sqrt(15.0);
    double w[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    double v[9];
    for (int i = 0; i < 3; ++i) {
        v[i] = 5.0 / 9.0 * w[i];
        v[3 + i] = 8.0 / 9.0 * w[i];
        v[6 + i] = 5.0 / 9.0 * w[i];
    }
#define S(i, d) s[((i) - 1) + nip * ((d) - 1)]
    if (nip == 1) {
        S(1, 1) = S(1, 2) = S(1, 3) = 0.0;
        wt[0] = 8.0;
    } else if (nip == 8) {
        static const int sg[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                     {-1, 1, 1}, {-1, -1, 1}, {-1, 1, -1}, {-1, -1, -1}};
        for (int i = 1; i <= 8; ++i)
            for (int d = 1; d <= 3; ++d) S(i, d) = sg[i - 1][d - 1] * root3;
        for (int i = 0; i < 8; ++i) wt[i] = 1.0;
    } else if (nip == 27) {
        double f59 = exact_weights ? 5.0 / 9.0 : (double)(5.0f / 9.0f);
        double f89 = exact_weights ? 8.0 / 9.0 : (double)(8.0f / 9.0f);
        for (int i = 0; i < 9; ++i) {
            wt[i] = f59 * v[i];
            wt[9 + i] = f89 * v[i];
            wt[18 + i] = f59 * v[i];
        }
        for (int blk = 0; blk < 3; ++blk) {      /* eta = -r15, 0, r15 */
            double eta = (blk == 0) ? -r15 : (blk == 1 ? 0.0 : r15);
            for (int i = 1; i <= 9; ++i) {
                int p = blk * 9 + i;
                int col = (i - 1) % 3;          /* xi  = -r15, 0, r15 */
                int row = (i - 1) / 3;          /* zeta = r15, 0, -r15 */
                S(p, 1) = (col == 0) ? -r15 : (col == 1 ? 0.0 : r15);
                S(p, 3) = (row == 0) ? r15 : (row == 1 ? 0.0 : -r15);
                S(p, 2) = eta;
            }
        }
    } else {
        return -1;
    }
#undef S
    return 0;
}

/* SHAPE_DER, 3-D 20-node brick (src/modules/shared/new_library.f90:865-896).
 * der(3,20) column-major: der[d + 3*l]. */
void orc_shape_der20(double *der, double xi, double eta, double zeta)
{
    static const int xii[20] = {-1, -1, -1, 0, 1, 1, 1, 0, -1, -1, 1, 1, -1, -1, -1, 0, 1, 1, 1, 0};
    static const int etai[20] = {-1, -1, -1, -1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1};
    static const int zetai[20] = {-1, 0, 1, 1, 1, 0, -1, -1, -1, 1, 1, -1, -1, 0, 1, 1, 1, 0, -1, -1};
    for (int l = 1; l <= 20; ++l) {
        double xi0 = xi * xii[l - 1];
        double eta0 = eta * etai[l - 1];
        double zeta0 = zeta * zetai[l - 1];
        double *d = &der[3 * (l - 1)];
        if (l == 4 || l == 8 || l == 16 || l == 20) {
            d[0] = -.5 * xi * (1. + eta0) * (1. + zeta0);
            d[1] = (.25 * etai[l - 1]) * (1. - xi * xi) * (1. + zeta0);
            d[2] = (.25 * zetai[l - 1]) * (1. - xi * xi) * (1. + eta0);
        } else if (l >= 9 && l <= 12) {
            d[0] = (.25 * xii[l - 1]) * (1. - eta * eta) * (1. + zeta0);
            d[1] = -.5 * eta * (1. + xi0) * (1. + zeta0);
            d[2] = (.25 * zetai[l - 1]) * (1. + xi0) * (1. - eta * eta);
        } else if (l == 2 || l == 6 || l == 14 || l == 18) {
            d[0] = (.25 * xii[l - 1]) * (1. + eta0) * (1. - zeta * zeta);
            d[1] = (.25 * etai[l - 1]) * (1. + xi0) * (1. - zeta * zeta);
            d[2] = -.5 * zeta * (1. + xi0) * (1. + eta0);
        } else {
            d[0] = (.125 * xii[l - 1]) * (1. + eta0) * (1. + zeta0) * (2. * xi0 + eta0 + zeta0 - 1.);
            d[1] = (.125 * etai[l - 1]) * (1. + xi0) * (1. + zeta0) * (xi0 + 2. * eta0 + zeta0 - 1.);
            d[2] = (.125 * zetai[l - 1]) * (1. + xi0) * (1. + eta0) * (xi0 + eta0 + 2. * zeta0 - 1.);
        }
    }
}

/* DEEMAT, nst=6 (src/modules/shared/new_library.f90:1604-1689).  dee(6,6) column-major. */
void orc_deemat(double *dee, double e, double v)
{
    double one = 1.0, two = 2.0, pt5 = 0.5;
    memset(dee, 0, 36 * sizeof(double));
    double v2 = v / (one - v);
    double vv = (one - two * v) / (one - v) * pt5;
    for (int i = 0; i < 3; ++i) dee[i + 6 * i] = one;
    for (int i = 3; i < 6; ++i) dee[i + 6 * i] = vv;
    dee[0 + 6 * 1] = v2; dee[1 + 6 * 0] = v2;
    dee[0 + 6 * 2] = v2; dee[2 + 6 * 0] = v2;
    dee[1 + 6 * 2] = v2; dee[2 + 6 * 1] = v2;
    double den = two * (one + v) * vv;       /* dee = dee*e/(two*(one+v)*vv) */
    for (int i = 0; i < 36; ++i) dee[i] = dee[i] * e / den;
}

/* DETERMINANT, 3x3 (src/modules/mpi/maths.f90:571-633).  jac(3,3) column-major. */
double orc_determinant(const double *j)
{
#define J(a, b) j[((a) - 1) + 3 * ((b) - 1)]
    double det = J(1, 1) * (J(2, 2) * J(3, 3) - J(3, 2) * J(2, 3));
    det = det - J(1, 2) * (J(2, 1) * J(3, 3) - J(3, 1) * J(2, 3));
    det = det + J(1, 3) * (J(2, 1) * J(3, 2) - J(3, 1) * J(2, 2));
    return det;
#undef J
}

/* INVERT, 3x3 cofactor form (src/modules/mpi/maths.f90:490-569) */
void orc_invert3(double *m)
{
#define M(a, b) m[((a) - 1) + 3 * ((b) - 1)]
    double det = M(1, 1) * (M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3));
    det = det - M(1, 2) * (M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3));
    det = det + M(1, 3) * (M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2));
    double j11 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    double j21 = -M(2, 1) * M(3, 3) + M(3, 1) * M(2, 3);
    double j31 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    double j12 = -M(1, 2) * M(3, 3) + M(3, 2) * M(1, 3);
    double j22 = M(1, 1) * M(3, 3) - M(3, 1) * M(1, 3);
    double j32 = -M(1, 1) * M(3, 2) + M(3, 1) * M(1, 2);
    double j13 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    double j23 = -M(1, 1) * M(2, 3) + M(2, 1) * M(1, 3);
    double j33 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    M(1, 1) = j11 / det; M(1, 2) = j12 / det; M(1, 3) = j13 / det;
    M(2, 1) = j21 / det; M(2, 2) = j22 / det; M(2, 3) = j23 / det;
    M(3, 1) = j31 / det; M(3, 2) = j32 / det; M(3, 3) = j33 / det;
#undef M
}

/* BEEMAT, nst=6 (src/modules/shared/new_library.f90:976-993).  bee(6,60) column-major. */
void orc_beemat(double *bee, const double *deriv)
{
    memset(bee, 0, 360 * sizeof(double));
#define B(r, c) bee[((r) - 1) + 6 * ((c) - 1)]
    for (int m = 1; m <= 20; ++m) {
        int n = 3 * m, k = n - 1, l = k - 1;
        double x = deriv[0 + 3 * (m - 1)], y = deriv[1 + 3 * (m - 1)], z = deriv[2 + 3 * (m - 1)];
        B(1, l) = x; B(4, k) = x; B(6, n) = x;
        B(2, k) = y; B(4, l) = y; B(5, n) = y;
        B(3, n) = z; B(5, k) = z; B(6, l) = z;
    }
#undef B
}

/* jac = MATMUL(der, coord): der(3,20) x coord(20,3) */
static void matmul_der_coord(const double *der, const double *coord, double *jac)
{
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int k = 0; k < 20; ++k) s += der[a + 3 * k] * coord[k + 20 * b];
            jac[a + 3 * b] = s;
        }
}

/* deriv = MATMUL(jac, der): jac(3,3) x der(3,20) */
static void matmul_jac_der(const double *jac, const double *der, double *deriv)
{
    for (int l = 0; l < 20; ++l)
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += jac[a + 3 * k] * der[k + 3 * l];
            deriv[a + 3 * l] = s;
        }
}

/* Element stiffness loop (src/programs/5th_ed/p121/p121.f90:54-64):
 * storkm(:,:,e) += MATMUL(MATMUL(TRANSPOSE(bee),dee),bee)*det*weights(i).
 * e_el / v_el: per-element E and nu when per_element != 0, else e_el[0], v_el[0]
 * (the per-element form follows src/programs/rfem/rfemsolve/rfemsolve.f90:217-221). */
void orc_form_storkm(int nels, int nip, int exact_weights, const double *g_coord,
                     const double *e_el, const double *v_el, int per_element,
                     double *storkm)
{
    double *pts = (double *)malloc(sizeof(double) * nip * 3);
    double *wts = (double *)malloc(sizeof(double) * nip);
    orc_sample(nip, pts, wts, exact_weights);
#pragma omp parallel
    {
        double dee[36], der[60], jac[9], deriv[60], bee[360], btd[360];
#pragma omp for schedule(static)
        for (int e = 0; e < nels; ++e) {
            double *km = &storkm[(size_t)3600 * e];
            const double *coord = &g_coord[(size_t)60 * e];
            memset(km, 0, 3600 * sizeof(double));
            orc_deemat(dee, per_element ? e_el[e] : e_el[0], per_element ? v_el[e] : v_el[0]);
            for (int i = 0; i < nip; ++i) {
                orc_shape_der20(der, pts[i], pts[i + nip], pts[i + 2 * nip]);
                matmul_der_coord(der, coord, jac);
                double det = orc_determinant(jac);
                orc_invert3(jac);
                matmul_jac_der(jac, der, deriv);
                orc_beemat(bee, deriv);
                /* btd(60,6) = TRANSPOSE(bee) . dee */
                for (int r = 0; r < 60; ++r)
                    for (int c = 0; c < 6; ++c) {
                        double s = 0.0;
                        for (int k = 0; k < 6; ++k) s += bee[k + 6 * r] * dee[k + 6 * c];
                        btd[r + 60 * c] = s;
                    }
                /* km += (btd . bee) * det * w */
                for (int c = 0; c < 60; ++c)
                    for (int r = 0; r < 60; ++r) {
                        double s = 0.0;
                        for (int k = 0; k < 6; ++k) s += btd[r + 60 * k] * bee[k + 6 * c];
                        km[r + 60 * c] = km[r + 60 * c] + s * det * wts[i];
                    }
            }
        }
    }
    free(pts);
    free(wts);
}

/* ------------------------------------------------------------------ */
/* Serial SCATTER (src/modules/mpi/gather_scatter.f90:694-854, one rank):
 * u(g(:,e)) += utemp(:,e) in element order; equation 0 is the dummy slot. */
static void scatter_add(int nels, const int *g_g, const double *utemp, double *u0 /*neq+1*/)
{
    for (int e = 0; e < nels; ++e)
        for (int i = 0; i < 60; ++i) {
            int q = g_g[60 * e + i];
            u0[q] = u0[q] + utemp[60 * e + i];
        }
}

/* Jacobi diagonal (src/programs/5th_ed/p121/p121.f90:65-69): scatter of
 * the element diagonals; returns diag (neq, not yet inverted). */
void orc_diag(int nels, int neq, const int *g_g, const double *storkm, double *diag)
{
    double *tmp = (double *)malloc(sizeof(double) * (size_t)60 * nels);
    double *d0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    for (int e = 0; e < nels; ++e)
        for (int i = 0; i < 60; ++i) tmp[60 * e + i] = storkm[(size_t)3600 * e + i + 60 * i];
    scatter_add(nels, g_g, tmp, d0);
    memcpy(diag, d0 + 1, sizeof(double) * neq);
    free(tmp);
    free(d0);
}

/* LOAD + SCATTER_NOADD (src/modules/mpi/loading.f90:36-146;
 * src/modules/mpi/gather_scatter.f90:856-993): r(g) = value, assignment. */
void orc_load(int nels, int neq, const int *g_num, const int *g_g, int loaded_nodes,
              const int *load_node, const double *load_value /*3 x loaded_nodes*/, double *r)
{
    double *r0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    /* node -> value lookup replaces the reference's triple loop; the result
     * is the same assignment because SCATTER_NOADD assigns, not sums. */
    int maxnode = 0;
    for (int i = 0; i < loaded_nodes; ++i) if (load_node[i] > maxnode) maxnode = load_node[i];
    int *slot = (int *)malloc(sizeof(int) * ((size_t)maxnode + 1));
    for (int i = 0; i <= maxnode; ++i) slot[i] = -1;
    for (int i = 0; i < loaded_nodes; ++i) slot[load_node[i]] = i;   /* last one wins */
    for (int e = 0; e < nels; ++e)
        for (int j = 0; j < 20; ++j) {
            int nd = g_num[20 * e + j];
            if (nd > maxnode || slot[nd] < 0) continue;
            for (int k = 0; k < 3; ++k) {
                int q = g_g[60 * e + 3 * j + k];
                if (q > 0) r0[q] = load_value[3 * slot[nd] + k];
            }
        }
    memcpy(r, r0 + 1, sizeof(double) * neq);
    free(slot);
    free(r0);
}

/* ------------------------------------------------------------------ */
/* The p121 PCG (src/programs/5th_ed/p121/p121.f90:86-104) with
 * checon_par (src/modules/mpi/maths.f90:999-1069) and DOT_PRODUCT_P
 * (src/modules/mpi/maths.f90:168-215, one rank: a sequential sum).
 *
 * diag: the assembled diagonal (inverted here, p121.f90:86).
 * stop_mode 0: checon_par test max|xnew-x|/max|xnew| <= tol (p121).
 * stop_mode 1: recomputed ||r||_2/||f||_2 <= tol (relative residual; the
 *              recursively updated r is used, checked every iteration).
 * Returns iterations; x receives xnew. */
int orc_pcg(int nels, int neq, const int *g_g, const double *storkm, const double *diag,
            const double *rhs, double tol, int limit, int stop_mode, double *x_out,
            double *final_metric, double *history /* limit entries or NULL */)
{
    size_t n1 = (size_t)neq + 1;
    double *dinv = (double *)malloc(sizeof(double) * n1);
    double *r = (double *)calloc(n1, sizeof(double));
    double *d = (double *)calloc(n1, sizeof(double));
    double *p = (double *)calloc(n1, sizeof(double));
    double *u = (double *)calloc(n1, sizeof(double));
    double *x = (double *)calloc(n1, sizeof(double));
    double *xnew = (double *)calloc(n1, sizeof(double));
    double *pmul = (double *)malloc(sizeof(double) * 60 * (size_t)nels);
    double *utemp = (double *)malloc(sizeof(double) * 60 * (size_t)nels);
    dinv[0] = 0.0;
    for (int q = 1; q <= neq; ++q) { dinv[q] = 1.0 / diag[q - 1]; r[q] = rhs[q - 1]; }
    for (int q = 1; q <= neq; ++q) d[q] = dinv[q] * r[q];
    for (int q = 1; q <= neq; ++q) p[q] = d[q];
    double ff = 0.0;
    for (int q = 1; q <= neq; ++q) ff += rhs[q - 1] * rhs[q - 1];
    int iters = 0;
    double metric = 0.0;
    for (;;) {
        ++iters;
        for (size_t q = 0; q < n1; ++q) u[q] = 0.0;
        /* GATHER (gather_scatter.f90:547-692): pmul(:,e) = p(g(:,e)), p(0)=0 */
        p[0] = 0.0;
        for (int e = 0; e < nels; ++e)
            for (int i = 0; i < 60; ++i) pmul[60 * (size_t)e + i] = p[g_g[60 * e + i]];
        /* element products utemp(:,e) = MATMUL(storkm(:,:,e), pmul(:,e)) */
#pragma omp parallel for schedule(static)
        for (int e = 0; e < nels; ++e) {
            const double *km = &storkm[(size_t)3600 * e];
            const double *pe = &pmul[60 * (size_t)e];
            double acc[60];
            for (int i = 0; i < 60; ++i) acc[i] = 0.0;
            for (int j = 0; j < 60; ++j) {
                double pj = pe[j];
                const double *col = &km[60 * j];
                for (int i = 0; i < 60; ++i) acc[i] = acc[i] + col[i] * pj;
            }
            memcpy(&utemp[60 * (size_t)e], acc, sizeof acc);
        }
        scatter_add(nels, g_g, utemp, u);
        u[0] = 0.0;
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
        int converged;
        if (stop_mode == 0) {
            double maxl = 0.0, maxd = 0.0;
            for (int q = 1; q <= neq; ++q) {
                double a = fabs(xnew[q]);
                if (a > maxl) maxl = a;
                double b = fabs(xnew[q] - x[q]);
                if (b > maxd) maxd = b;
            }
            metric = maxd / maxl;
            converged = metric <= tol;
        } else {
            double rr = 0.0;
            for (int q = 1; q <= neq; ++q) rr += r[q] * r[q];
            metric = sqrt(rr) / sqrt(ff);
            converged = metric <= tol;
        }
        if (history) history[iters - 1] = metric;
        for (int q = 1; q <= neq; ++q) x[q] = xnew[q];
        if (converged || iters == limit) break;
    }
    memcpy(x_out, xnew + 1, sizeof(double) * neq);
    if (final_metric) *final_metric = metric;
    free(dinv); free(r); free(d); free(p); free(u); free(x); free(xnew); free(pmul); free(utemp);
    return iters;
}

/* One element-by-element product u = K p over equations (GATHER, MATMUL,
 * SCATTER of p121.f90:92-97); p and u have neq entries. */
void orc_ebe_matvec(int nels, int neq, const int *g_g, const double *storkm,
                    const double *p, double *u)
{
    double *p0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    double *u0 = (double *)calloc((size_t)neq + 1, sizeof(double));
    double *ut = (double *)malloc(sizeof(double) * 60 * (size_t)nels);
    memcpy(p0 + 1, p, sizeof(double) * neq);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < nels; ++e) {
        const double *km = &storkm[(size_t)3600 * e];
        double pe[60], acc[60];
        for (int i = 0; i < 60; ++i) { pe[i] = p0[g_g[60 * e + i]]; acc[i] = 0.0; }
        for (int j = 0; j < 60; ++j)
            for (int i = 0; i < 60; ++i) acc[i] = acc[i] + km[i + 60 * j] * pe[j];
        memcpy(&ut[60 * (size_t)e], acc, sizeof acc);
    }
    scatter_add(nels, g_g, ut, u0);
    memcpy(u, u0 + 1, sizeof(double) * neq);
    free(p0); free(u0); free(ut);
}

/* Centroid stress of one element (src/programs/5th_ed/p121/p121.f90:112-123):
 * nip=1 at the origin, sigma = dee . bee . eld. */
void orc_centroid_stress(const double *coord /*20x3*/, const double *eld /*60*/,
                         double e, double v, double *sigma /*6*/)
{
    double der[60], jac[9], deriv[60], bee[360], dee[36], eps[6];
    orc_deemat(dee, e, v);
    orc_shape_der20(der, 0.0, 0.0, 0.0);
    matmul_der_coord(der, coord, jac);
    orc_invert3(jac);
    matmul_jac_der(jac, der, deriv);
    orc_beemat(bee, deriv);
    for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int k = 0; k < 60; ++k) s += bee[r + 6 * k] * eld[k];
        eps[r] = s;
    }
    for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int k = 0; k < 6; ++k) s += dee[r + 6 * k] * eps[k];
        sigma[r] = s;
    }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
